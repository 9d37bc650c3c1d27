// glsl_shim.hpp -- TEST INFRASTRUCTURE ONLY.
//
// The GLSL compute-shader vocabulary the reference's six hot-path shaders use
// (vec2/vec3/vec4/ivec2/uvec2/uvec3 with the swizzles they touch, the
// built-ins they call, image2D/sampler2D with imageLoad/imageStore/texture),
// so that those shader sources compile unchanged as C++ and run on the CPU.
// No graphics API is involved: images and samplers are plain float arrays and
// a dispatch is a loop over gl_GlobalInvocationID.
//
// Semantics chosen where GLSL leaves them to the implementation (they are the
// same pins the oracle documents):
//   - float arithmetic in FP32 (the harness is built with
//     -fsingle-precision-constant so unsuffixed literals are float, as in GLSL);
//   - pow(x, y) is C's powf, so pow(x, 2.0) is x*x for negative x;
//   - clamp(x, lo, hi) = min(max(x, lo), hi) with comparisons, NaN passes through;
//   - texture(): nearest filtering; the coordinate is converted to texels with
//     8 bits of sub-texel fixed point (rounded), then floored, then wrapped
//     (REPEAT) or clamped (CLAMP_TO_EDGE) per sampler;
//   - imageLoad outside the image returns 0, imageStore outside is dropped;
//     missing channels of a format read as (0, 0, 0, 1).
#pragma once
#include <stdint.h>

namespace glsl {

struct vec2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
    };
    vec2() = default;
    vec2(float a, float b) { x = a; y = b; }
    explicit vec2(float a) { x = a; y = a; }
};
// Two-component swizzle stored inside vec4's union (a member with
// constructors cannot live there); converts to vec2 wherever one is used.
struct sw2 {
    float x, y;
    operator vec2() const { return vec2(x, y); }
};
struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
    };
    vec3() = default;
    vec3(float a, float b, float c) { x = a; y = b; z = c; }
};
struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        struct { sw2 xy, zw; };
        struct { sw2 rg, ba; };
    };
    vec4() = default;
    vec4(float p, float q, float s, float t) { x = p; y = q; z = s; w = t; }
    vec4(vec2 v, float s, float t) { x = v.x; y = v.y; z = s; w = t; }
    vec4(vec3 v, float t) { x = v.x; y = v.y; z = v.z; w = t; }
    vec4 rgba_() const { return *this; }
};
struct uvec2 {
    unsigned x, y;
    operator vec2() const { return vec2((float)x, (float)y); }
};
struct uvec3 {
    union {
        struct { unsigned x, y, z; };
        struct { uvec2 xy; unsigned z_; };
    };
    uvec3() = default;
    uvec3(unsigned a, unsigned b, unsigned c) { x = a; y = b; z = c; }
};
struct ivec2 {
    int x, y;
    ivec2() = default;
    ivec2(int a, int b) : x(a), y(b) {}
    ivec2(uvec2 v) : x((int)v.x), y((int)v.y) {}
    ivec2(vec2 v) : x((int)v.x), y((int)v.y) {}
};

inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator-(vec2 a, vec2 b) { return vec2(a.x - b.x, a.y - b.y); }
inline vec2 operator-(vec2 a) { return vec2(-a.x, -a.y); }
inline vec2 operator-(vec2 a, float s) { return vec2(a.x - s, a.y - s); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(float s, vec2 a) { return vec2(a.x * s, a.y * s); }
inline vec2 operator/(vec2 a, float s) { return vec2(a.x / s, a.y / s); }
inline vec2 operator/(uvec2 a, float s) { return vec2((float)a.x / s, (float)a.y / s); }

inline float sqrt(float v) { return __builtin_sqrtf(v); }
inline float exp(float v) { return __builtin_expf(v); }
inline float log(float v) { return __builtin_logf(v); }
inline float cos(float v) { return __builtin_cosf(v); }
inline float sin(float v) { return __builtin_sinf(v); }
inline float pow(float a, float b) { return __builtin_powf(a, b); }
inline float floor(float v) { return __builtin_floorf(v); }
inline float mod(float a, float b) { return a - b * floor(a / b); }
inline float clamp(float v, float lo, float hi)
{
    float m = v < lo ? lo : v;
    return m > hi ? hi : m;
}
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float length(vec2 a) { return sqrt(dot(a, a)); }
inline vec2 normalize(vec2 a) { return a / length(a); }
inline vec3 normalize(vec3 a)
{
    float l = sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return vec3(a.x / l, a.y / l, a.z / l);
}

// Images: row-major float texels with `ch` channels (1 = r32f, 2 = rg32f, 4 = rgba32f).
struct image2D {
    float* data = nullptr;
    int    w = 0, h = 0, ch = 4;
};
inline vec4 imageLoad(const image2D& im, ivec2 p)
{
    vec4 v(0.0f, 0.0f, 0.0f, 1.0f);
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return vec4(0.0f, 0.0f, 0.0f, 0.0f);
    const float* t = im.data + ((size_t)p.y * im.w + p.x) * im.ch;
    v.x = t[0];
    if (im.ch > 1) v.y = t[1];
    if (im.ch > 2) v.z = t[2];
    if (im.ch > 3) v.w = t[3];
    return v;
}
inline void imageStore(image2D& im, ivec2 p, vec4 v)
{
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
    float* t = im.data + ((size_t)p.y * im.w + p.x) * im.ch;
    t[0] = v.x;
    if (im.ch > 1) t[1] = v.y;
    if (im.ch > 2) t[2] = v.z;
    if (im.ch > 3) t[3] = v.w;
}

struct sampler2D {
    const float* data = nullptr;
    int          w = 0, h = 0, ch = 1;
    bool         repeat = false;
};
inline int texel_index(float u, int n, bool repeat)
{
    // 8-bit sub-texel fixed point, then floor
    long long fx = (long long)__builtin_floorf(u * (float)n * 256.0f + 0.5f);
    long long i  = fx >= 0 ? fx / 256 : -((-fx + 255) / 256);
    if (repeat) {
        i %= n;
        if (i < 0) i += n;
    } else {
        if (i < 0) i = 0;
        if (i >= n) i = n - 1;
    }
    return (int)i;
}
inline vec4 texture(const sampler2D& s, vec2 uv)
{
    int          x = texel_index(uv.x, s.w, s.repeat), y = texel_index(uv.y, s.h, s.repeat);
    const float* t = s.data + ((size_t)y * s.w + x) * s.ch;
    vec4         v(t[0], 0.0f, 0.0f, 1.0f);
    if (s.ch > 1) v.y = t[1];
    if (s.ch > 2) v.z = t[2];
    if (s.ch > 3) v.w = t[3];
    return v;
}

// Base of the struct a `buffer` interface block becomes (see glsl_begin.hpp).
struct ssbo_base {
    int reserved_;
};

}  // namespace glsl
