// glsl_end.hpp -- TEST INFRASTRUCTURE ONLY.  Undoes glsl_begin.hpp.
#undef layout
#undef in
#undef uniform
#undef readonly
#undef writeonly
#undef buffer
#undef indices
#undef bit_reversed
#undef rgba
#undef LOCAL_SIZE
#undef M_PI
#undef rgbr
#undef out
