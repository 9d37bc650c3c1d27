// glsl_begin.hpp -- TEST INFRASTRUCTURE ONLY.  Included right before a
// reference shader source: maps the GLSL qualifiers and declarations that are
// not C++ onto C++ (layout(...) qualifiers vanish, `uniform` globals become
// TU-local statics the harness sets, a `buffer` block becomes a struct reached
// through a pointer the harness binds).  glsl_end.hpp undoes every macro.
#undef M_PI
#undef LOCAL_SIZE
#define layout(...)
#define in
#define uniform static
#define readonly
#define writeonly
#define buffer struct
#define indices indices_t : glsl::ssbo_base
#define bit_reversed (*ref_bit_reversed_ptr)
#define rgba rgba_()
#define rgbr rgbr_()
#define out
