/*
 * glsl_compat.hpp — just enough of GLSL 4.60 in C++ to compile vtrace's fragment shader
 * (shaders/trace.frag) as a host function (TEST INFRASTRUCTURE ONLY).
 *
 * The build recipe (oracle/build.py, build_ref()) feeds the shader text, minus its `#version`
 * and `#extension` directives, to g++ with this header force-included, so the traversal that runs
 * is the reference's own source.  The header fixes the semantics GLSL leaves to the driver:
 *  - arithmetic is IEEE binary32, round to nearest, no contraction (-ffp-contract=off);
 *  - length(v) = sqrt((x*x + y*y) + z*z), normalize(v) = v / length(v), division correctly
 *    rounded; min(x, y) = (y < x) ? y : x as the GLSL specification defines it;
 *  - `vec3(bvec3) * v` is a select when VT_B2F_SELECT is 1 (the b2f-multiply rewrite shader
 *    compilers apply) and the literal IEEE product (0 * inf = NaN) when it is 0;
 *  - texture() on a sampler3D is NEAREST + CLAMP_TO_EDGE at level 0 (lib/descriptor.c:97-117):
 *    texel = clamp(floor(coord * size), 0, size - 1), RGBA8 with sRGB-decoded colour and linear
 *    alpha (VK_FORMAT_R8G8B8A8_SRGB, lib/memory.c:317).  It also records the texel it fetched
 *    and counts fetches, which is how the harness reads the hit voxel and the step count.
 */
#ifndef VT_GLSL_COMPAT_HPP
#define VT_GLSL_COMPAT_HPP

#include <math.h>
#include <stdint.h>

#ifndef VT_B2F_SELECT
#define VT_B2F_SELECT 1
#endif

typedef unsigned int uint;
struct vec3;
struct vec4;
struct ivec3;

template <int N, int A, int B, int C>
struct swz3 {
    float e[N];
    inline operator vec3() const;
};

struct bvec3 {
    bool x, y, z;
};

struct vec3 {
    union {
        float e[3];
        struct {
            float x, y, z;
        };
        swz3<3, 0, 1, 2> xyz;
        swz3<3, 1, 2, 0> yzx;
        swz3<3, 2, 0, 1> zxy;
    };
    bool from_bool;
    vec3() : e{0.f, 0.f, 0.f}, from_bool(false) {}
    explicit vec3(float s) : e{s, s, s}, from_bool(false) {}
    vec3(float a, float b, float c) : e{a, b, c}, from_bool(false) {}
    inline explicit vec3(const ivec3& v);
    explicit vec3(const bvec3& b)
        : e{b.x ? 1.f : 0.f, b.y ? 1.f : 0.f, b.z ? 1.f : 0.f}, from_bool(true) {}
    vec3(const vec3& o) : e{o.e[0], o.e[1], o.e[2]}, from_bool(o.from_bool) {}
    vec3& operator=(const vec3& o) {
        e[0] = o.e[0];
        e[1] = o.e[1];
        e[2] = o.e[2];
        from_bool = false;
        return *this;
    }
    float& operator[](int i) { return e[i]; }
    float operator[](int i) const { return e[i]; }
};

template <int N, int A, int B, int C>
inline swz3<N, A, B, C>::operator vec3() const {
    return vec3(e[A], e[B], e[C]);
}

struct vec4 {
    union {
        float e[4];
        struct {
            float x, y, z, w;
        };
        swz3<4, 0, 1, 2> xyz;
    };
    vec4() : e{0.f, 0.f, 0.f, 0.f} {}
    vec4(float a, float b, float c, float d) : e{a, b, c, d} {}
    vec4(const vec3& v, float d) : e{v.e[0], v.e[1], v.e[2], d} {}
    vec4(const vec4& o) : e{o.e[0], o.e[1], o.e[2], o.e[3]} {}
    vec4& operator=(const vec4& o) {
        for (int i = 0; i < 4; ++i) e[i] = o.e[i];
        return *this;
    }
    float& operator[](int i) { return e[i]; }
    float operator[](int i) const { return e[i]; }
};

struct ivec3 {
    int x, y, z;
    ivec3() : x(0), y(0), z(0) {}
    explicit ivec3(int s) : x(s), y(s), z(s) {}
    ivec3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit ivec3(const vec3& v) : x((int)v.e[0]), y((int)v.e[1]), z((int)v.e[2]) {}
    explicit ivec3(const bvec3& b) : x(b.x ? 1 : 0), y(b.y ? 1 : 0), z(b.z ? 1 : 0) {}
    ivec3& operator+=(const ivec3& o) {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
};

inline vec3::vec3(const ivec3& v) : e{(float)v.x, (float)v.y, (float)v.z}, from_bool(false) {}

/* column-major: m[c] is column c, m[c][r] row r */
struct mat4 {
    vec4 c[4];
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};

/* ---- vec3 arithmetic (component-wise, one rounding per operation) ---- */
inline vec3 operator+(const vec3& a, const vec3& b) { return vec3(a.e[0] + b.e[0], a.e[1] + b.e[1], a.e[2] + b.e[2]); }
inline vec3 operator-(const vec3& a, const vec3& b) { return vec3(a.e[0] - b.e[0], a.e[1] - b.e[1], a.e[2] - b.e[2]); }
inline vec3 operator/(const vec3& a, const vec3& b) { return vec3(a.e[0] / b.e[0], a.e[1] / b.e[1], a.e[2] / b.e[2]); }
inline vec3 operator*(const vec3& a, const vec3& b) {
#if VT_B2F_SELECT
    if (a.from_bool)
        return vec3(a.e[0] != 0.f ? b.e[0] : 0.f, a.e[1] != 0.f ? b.e[1] : 0.f, a.e[2] != 0.f ? b.e[2] : 0.f);
    if (b.from_bool)
        return vec3(b.e[0] != 0.f ? a.e[0] : 0.f, b.e[1] != 0.f ? a.e[1] : 0.f, b.e[2] != 0.f ? a.e[2] : 0.f);
#endif
    return vec3(a.e[0] * b.e[0], a.e[1] * b.e[1], a.e[2] * b.e[2]);
}
inline vec3 operator+(const vec3& a, float s) { return vec3(a.e[0] + s, a.e[1] + s, a.e[2] + s); }
inline vec3 operator-(const vec3& a, float s) { return vec3(a.e[0] - s, a.e[1] - s, a.e[2] - s); }
inline vec3 operator*(const vec3& a, float s) { return vec3(a.e[0] * s, a.e[1] * s, a.e[2] * s); }
inline vec3 operator/(const vec3& a, float s) { return vec3(a.e[0] / s, a.e[1] / s, a.e[2] / s); }
inline vec3& operator+=(vec3& a, const vec3& b) {
    a = a + b;
    return a;
}
inline vec3 operator/(const ivec3& a, const vec3& b) { return vec3(a) / b; }

inline ivec3 operator*(const ivec3& a, const ivec3& b) { return ivec3(a.x * b.x, a.y * b.y, a.z * b.z); }

/* ---- matrices ---- */
inline vec4 operator*(const mat4& m, const vec4& v) {
    vec4 r;
    for (int i = 0; i < 4; ++i)
        r.e[i] = ((m.c[0].e[i] * v.e[0] + m.c[1].e[i] * v.e[1]) + m.c[2].e[i] * v.e[2]) + m.c[3].e[i] * v.e[3];
    return r;
}
inline mat4 operator*(const mat4& a, const mat4& b) {
    mat4 r;
    for (int c = 0; c < 4; ++c) r.c[c] = a * b.c[c];
    return r;
}
/* cofactor expansion; exact for permutation and identity matrices */
inline mat4 inverse(const mat4& m) {
    float a[16], inv[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) a[c * 4 + r] = m.c[c].e[r];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    float det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    mat4 r;
    for (int c = 0; c < 4; ++c)
        for (int rr = 0; rr < 4; ++rr) r.c[c].e[rr] = inv[c * 4 + rr] / det;
    return r;
}

/* ---- built-in functions ---- */
inline float min(float x, float y) { return (y < x) ? y : x; }
inline int min(int x, int y) { return (y < x) ? y : x; }
inline vec3 min(const vec3& a, const vec3& b) { return vec3(min(a.e[0], b.e[0]), min(a.e[1], b.e[1]), min(a.e[2], b.e[2])); }
inline vec3 floor(const vec3& v) { return vec3(floorf(v.e[0]), floorf(v.e[1]), floorf(v.e[2])); }
inline float glsl_sign1(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
inline vec3 sign(const vec3& v) { return vec3(glsl_sign1(v.e[0]), glsl_sign1(v.e[1]), glsl_sign1(v.e[2])); }
inline vec3 abs(const vec3& v) { return vec3(fabsf(v.e[0]), fabsf(v.e[1]), fabsf(v.e[2])); }
inline float dot(const vec3& a, const vec3& b) { return (a.e[0] * b.e[0] + a.e[1] * b.e[1]) + a.e[2] * b.e[2]; }
inline float length(const vec3& v) { return sqrtf(dot(v, v)); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline bvec3 lessThanEqual(const vec3& a, const vec3& b) { return bvec3{a.e[0] <= b.e[0], a.e[1] <= b.e[1], a.e[2] <= b.e[2]}; }
inline bvec3 greaterThanEqual(const ivec3& a, const ivec3& b) { return bvec3{a.x >= b.x, a.y >= b.y, a.z >= b.z}; }
inline bvec3 lessThan(const ivec3& a, const ivec3& b) { return bvec3{a.x < b.x, a.y < b.y, a.z < b.z}; }
inline bool all(const bvec3& b) { return b.x && b.y && b.z; }
inline int floatBitsToInt(float f) {
    union {
        float f;
        int i;
    } u;
    u.f = f;
    return u.i;
}

/* ---- sampler3D: an RGBA8 grid, x-fastest ---- */
struct sampler3D_t {
    const uint8_t* texels;
    int nx, ny, nz;
    /* side channel for the harness */
    int last_x, last_y, last_z;
    uint32_t fetches;
};

inline ivec3 textureSize(const sampler3D_t& s, int lod) {
    (void)lod;
    return ivec3(s.nx, s.ny, s.nz);
}

inline float glsl_srgb_decode(uint8_t c) {
    float v = (float)c / 255.0f;
    return v <= 0.04045f ? v / 12.92f : powf((v + 0.055f) / 1.055f, 2.4f);
}

inline int glsl_nearest(float u, int n) {
    float f = floorf(u * (float)n);
    int i = (int)f;
    if (f < 0.f) i = 0;
    if (i > n - 1) i = n - 1;
    return i;
}

inline vec4 texture(sampler3D_t& s, const vec3& coord) {
    int x = glsl_nearest(coord.e[0], s.nx), y = glsl_nearest(coord.e[1], s.ny), z = glsl_nearest(coord.e[2], s.nz);
    s.last_x = x;
    s.last_y = y;
    s.last_z = z;
    s.fetches++;
    const uint8_t* p = s.texels + 4 * ((size_t)x + (size_t)s.nx * ((size_t)y + (size_t)s.ny * (size_t)z));
    return vec4(glsl_srgb_decode(p[0]), glsl_srgb_decode(p[1]), glsl_srgb_decode(p[2]), (float)p[3] / 255.0f);
}

extern bool glsl_discarded;

/* ---- GLSL declaration syntax ---- */
#define layout(...)
#define in
#define out
#define flat
#define uniform struct
/* `uniform sampler3D tex[];` becomes a forward declaration plus an extern array declaration */
#define sampler3D sampler3D_t; extern sampler3D_t
#define discard            \
    do {                   \
        glsl_discarded = true; \
        return;            \
    } while (0)
#define main trace_frag_main

#endif
