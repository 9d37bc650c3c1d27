// glsl_shim.hpp -- TEST INFRASTRUCTURE ONLY.
//
// The GLSL vocabulary the reference's six hot-path compute shaders and its
// sky shaders (atmosphere.glsl, sky_envmap_fs.glsl) use (vec2/vec3/vec4/
// ivec2/uvec2/uvec3 with the swizzles and operators they touch, the built-ins
// they call, image2D/sampler2D/sampler3D with imageLoad/imageStore/texture),
// so that those shader sources compile as C++ and run on the CPU.
// No graphics API is involved: images and samplers are plain float arrays and
// a dispatch is a loop over gl_GlobalInvocationID.
//
// Semantics chosen where GLSL leaves them to the implementation (they are the
// same pins the oracle documents):
//   - float arithmetic in FP32 (the harness is built with
//     -fsingle-precision-constant so unsuffixed literals are float, as in GLSL);
//   - pow(x, y) is C's powf, so pow(x, 2.0) is x*x for negative x;
//   - clamp(x, lo, hi) = min(max(x, lo), hi) with comparisons, NaN passes through;
//   - texture() on a nearest sampler (the compute shaders' noise): the
//     coordinate is converted to texels with 8 bits of sub-texel fixed point
//     (rounded), then floored, then wrapped (REPEAT) or clamped
//     (CLAMP_TO_EDGE) per sampler;
//   - texture() on a linear sampler (the sky tables, GL_LINEAR +
//     CLAMP_TO_EDGE): texel coordinate u*W - 0.5, floor, FP32 weights
//     (hardware units quantise them), both texel indices clamped to the edge;
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
struct vec4;
struct vec3 {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
    };
    vec3() = default;
    vec3(float a, float b, float c) { x = a; y = b; z = c; }
    vec4 rgbr_() const;
};
// Three-component swizzle inside vec4's union; converts to vec3.
struct sw3 {
    float x, y, z;
    operator vec3() const { return vec3(x, y, z); }
};
struct vec4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        struct { sw2 xy, zw; };
        struct { sw2 rg, ba; };
        struct { sw3 rgb; float a_rgb_; };
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

inline vec4 vec3::rgbr_() const { return vec4(x, y, z, x); }

inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator-(vec3 a) { return vec3(-a.x, -a.y, -a.z); }
inline vec3 operator*(vec3 a, vec3 b) { return vec3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator/(vec3 a, vec3 b) { return vec3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline vec3 operator/(vec3 a, float s) { return vec3(a.x / s, a.y / s, a.z / s); }
inline vec3 operator/(float s, vec3 a) { return vec3(s / a.x, s / a.y, s / a.z); }
inline vec3& operator+=(vec3& a, vec3 b) { return a = a + b; }
inline vec3& operator-=(vec3& a, vec3 b) { return a = a - b; }
inline vec3& operator*=(vec3& a, float s) { return a = a * s; }
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline vec4 operator-(vec4 a, vec4 b) { return vec4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
inline vec4 operator*(vec4 a, vec4 b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator*(vec4 a, float s) { return vec4(a.x * s, a.y * s, a.z * s, a.w * s); }
inline vec4 operator*(float s, vec4 a) { return vec4(s * a.x, s * a.y, s * a.z, s * a.w); }

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
inline float atan(float v) { return __builtin_atanf(v); }
inline float tan(float v) { return __builtin_tanf(v); }
inline float abs(float v) { return __builtin_fabsf(v); }
inline float max(float a, float b) { return a < b ? b : a; }
inline float min(float a, float b) { return b < a ? b : a; }
inline vec4 max(vec4 a, float b) { return vec4(max(a.x, b), max(a.y, b), max(a.z, b), max(a.w, b)); }
inline vec3 min(vec3 a, float b) { return vec3(min(a.x, b), min(a.y, b), min(a.z, b)); }
inline float step(float edge, float x) { return x < edge ? 0.0f : 1.0f; }
inline float smoothstep(float e0, float e1, float x)
{
    float t = (x - e0) / (e1 - e0);
    t       = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
    return t * t * (3.0f - 2.0f * t);
}
inline vec4 mix(vec4 a, vec4 b, float t) { return a * (1.0f - t) + b * t; }
inline float mod(float a, float b) { return a - b * floor(a / b); }
inline float clamp(float v, float lo, float hi)
{
    float m = v < lo ? lo : v;
    return m > hi ? hi : m;
}
inline float dot(vec2 a, vec2 b) { return a.x * b.x + a.y * b.y; }
inline float dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float length(vec3 a) { return sqrt(dot(a, a)); }
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
    bool         linear = false;   // GL_LINEAR + CLAMP_TO_EDGE, 4 channels
};
struct sampler3D {   // GL_LINEAR + CLAMP_TO_EDGE, 4 channels, [d][h][w]
    const float* data = nullptr;
    int          w = 0, h = 0, d = 0;
};
inline void linear_axis(float u, int n, int& i0, int& i1, float& wt)
{
    float t = u * (float)n - 0.5f;
    float f = __builtin_floorf(t);
    int   i = (int)f;
    wt      = t - f;
    i0      = i < 0 ? 0 : (i > n - 1 ? n - 1 : i);
    i1      = i + 1 < 0 ? 0 : (i + 1 > n - 1 ? n - 1 : i + 1);
}
inline vec4 texel4(const float* t) { return vec4(t[0], t[1], t[2], t[3]); }
inline vec4 lerp4(vec4 a, vec4 b, float w)
{
    float v = 1.0f - w;
    return vec4(a.x * v + b.x * w, a.y * v + b.y * w, a.z * v + b.z * w, a.w * v + b.w * w);
}
inline vec4 texture(const sampler3D& s, vec3 p)
{
    int   x0, x1, y0, y1, z0, z1;
    float wx, wy, wz;
    linear_axis(p.x, s.w, x0, x1, wx);
    linear_axis(p.y, s.h, y0, y1, wy);
    linear_axis(p.z, s.d, z0, z1, wz);
    vec4 pl[2];
    for (int k = 0; k < 2; ++k) {
        const float* P = s.data + (size_t)4 * (k ? z1 : z0) * s.h * s.w;
        vec4 a = lerp4(texel4(P + 4 * ((size_t)y0 * s.w + x0)), texel4(P + 4 * ((size_t)y0 * s.w + x1)), wx);
        vec4 b = lerp4(texel4(P + 4 * ((size_t)y1 * s.w + x0)), texel4(P + 4 * ((size_t)y1 * s.w + x1)), wx);
        pl[k]  = lerp4(a, b, wy);
    }
    return lerp4(pl[0], pl[1], wz);
}
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
    if (s.linear) {
        int   x0, x1, y0, y1;
        float wx, wy;
        linear_axis(uv.x, s.w, x0, x1, wx);
        linear_axis(uv.y, s.h, y0, y1, wy);
        vec4 a = lerp4(texel4(s.data + 4 * ((size_t)y0 * s.w + x0)), texel4(s.data + 4 * ((size_t)y0 * s.w + x1)), wx);
        vec4 b = lerp4(texel4(s.data + 4 * ((size_t)y1 * s.w + x0)), texel4(s.data + 4 * ((size_t)y1 * s.w + x1)), wx);
        return lerp4(a, b, wy);
    }
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
