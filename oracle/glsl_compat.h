// ORACLE -- test infrastructure only.
//
// A small GLSL-to-C++ compatibility layer used to compile the reference's
// own GLSL function libraries (Shaders/DDGI/DDGICommon.glsl,
// Shaders/SDF/SDFCommon.glsl, Shaders/SDF/AtlasCommon.glsl and their
// includes) as C++ on the host, where they serve as a second CPU reference
// for the restatement in oracle.cpp.  Built by oracle/build_ref.py with
// -fsingle-precision-constant so unsuffixed literals are float as in GLSL.
//
// Provides: vec2/3/4, ivec2/3/4, uvec2/3/4 with swizzles (generated into
// glsl_swizzles.inc), mat3/mat4 (column-major), the GLSL built-ins the
// libraries call, and sampler2D/sampler3D with GL filtering rules
// (LINEAR + CLAMP_TO_EDGE for 3D, LINEAR + REPEAT or CLAMP for 2D,
// textureGather component order (i0,j1),(i1,j1),(i1,j0),(i0,j0)).
#pragma once

#include <cstdint>
#include <cstring>
#include <type_traits>

#include "packed_color.h"

typedef unsigned int uint;

#define in
#define highp
#define mediump
#define lowp

namespace glslc {
inline float f_sqrt(float x) { return __builtin_sqrtf(x); }
inline float f_floor(float x) { return __builtin_floorf(x); }
inline float f_abs(float x) { return __builtin_fabsf(x); }
inline float f_pow(float x, float y) { return __builtin_powf(x, y); }
inline float f_sin(float x) { return __builtin_sinf(x); }
inline float f_cos(float x) { return __builtin_cosf(x); }
inline float f_exp(float x) { return __builtin_expf(x); }
inline float f_log(float x) { return __builtin_logf(x); }
}  // namespace glslc

template <typename T, int N> struct gvec;

// Swizzle proxy over the parent's storage (union member of gvec).  Member
// bodies are instantiated on use, after gvec is complete.
template <typename T, int N, int... I> struct Swz {
    T e[N];
    static constexpr int L = sizeof...(I);
    operator gvec<T, L>() const {
        gvec<T, L> v;
        int k = 0;
        ((v.e[k++] = e[I]), ...);
        return v;
    }
    Swz& operator=(const gvec<T, L>& v) {
        int k = 0;
        ((e[I] = v.e[k++]), ...);
        return *this;
    }
    Swz& operator=(const Swz& o) { return *this = gvec<T, L>(o); }
    Swz& operator+=(const gvec<T, L>& v) { int k = 0; ((e[I] = e[I] + v.e[k++]), ...); return *this; }
    Swz& operator-=(const gvec<T, L>& v) { int k = 0; ((e[I] = e[I] - v.e[k++]), ...); return *this; }
    Swz& operator*=(const gvec<T, L>& v) { int k = 0; ((e[I] = e[I] * v.e[k++]), ...); return *this; }
    Swz& operator/=(const gvec<T, L>& v) { int k = 0; ((e[I] = e[I] / v.e[k++]), ...); return *this; }
    Swz& operator*=(T s) { ((e[I] = e[I] * s), ...); return *this; }
    Swz& operator/=(T s) { ((e[I] = e[I] / s), ...); return *this; }
};

#define SWZ(...) Swz<T, N, __VA_ARGS__>

template <typename T> struct gvec<T, 2> {
    static constexpr int N = 2;
    union {
        T e[2];
        struct { T x, y; };
        struct { T r, g; };
#include "glsl_swizzles_2.inc"
    };
    gvec() : e{T(0), T(0)} {}
    explicit gvec(T s) : e{s, s} {}
    gvec(T a, T b) : e{a, b} {}
    template <typename U> gvec(const gvec<U, 2>& o) : e{T(o.e[0]), T(o.e[1])} {}
    template <typename U> explicit gvec(const gvec<U, 3>& o) : e{T(o.e[0]), T(o.e[1])} {}
    template <typename U> explicit gvec(const gvec<U, 4>& o) : e{T(o.e[0]), T(o.e[1])} {}
    gvec(const gvec& o) { std::memcpy(e, o.e, sizeof(e)); }
    gvec& operator=(const gvec& o) { std::memcpy(e, o.e, sizeof(e)); return *this; }
    T& operator[](int i) { return e[i]; }
    const T& operator[](int i) const { return e[i]; }
};

template <typename T> struct gvec<T, 3> {
    static constexpr int N = 3;
    union {
        T e[3];
        struct { T x, y, z; };
        struct { T r, g, b; };
#include "glsl_swizzles_3.inc"
    };
    gvec() : e{T(0), T(0), T(0)} {}
    explicit gvec(T s) : e{s, s, s} {}
    gvec(T a, T b, T c) : e{a, b, c} {}
    gvec(const gvec<T, 2>& v, T c) : e{v.e[0], v.e[1], c} {}
    gvec(T a, const gvec<T, 2>& v) : e{a, v.e[0], v.e[1]} {}
    template <typename U> gvec(const gvec<U, 3>& o) : e{T(o.e[0]), T(o.e[1]), T(o.e[2])} {}
    template <typename U> explicit gvec(const gvec<U, 4>& o) : e{T(o.e[0]), T(o.e[1]), T(o.e[2])} {}
    gvec(const gvec& o) { std::memcpy(e, o.e, sizeof(e)); }
    gvec& operator=(const gvec& o) { std::memcpy(e, o.e, sizeof(e)); return *this; }
    T& operator[](int i) { return e[i]; }
    const T& operator[](int i) const { return e[i]; }
};

template <typename T> struct gvec<T, 4> {
    static constexpr int N = 4;
    union {
        T e[4];
        struct { T x, y, z, w; };
        struct { T r, g, b, a; };
#include "glsl_swizzles_4.inc"
    };
    gvec() : e{T(0), T(0), T(0), T(0)} {}
    explicit gvec(T s) : e{s, s, s, s} {}
    gvec(T a, T b, T c, T d) : e{a, b, c, d} {}
    gvec(const gvec<T, 3>& v, T d) : e{v.e[0], v.e[1], v.e[2], d} {}
    gvec(const gvec<T, 2>& v, T c, T d) : e{v.e[0], v.e[1], c, d} {}
    template <typename U> explicit gvec(const gvec<U, 4>& o) : e{T(o.e[0]), T(o.e[1]), T(o.e[2]), T(o.e[3])} {}
    gvec(const gvec& o) { std::memcpy(e, o.e, sizeof(e)); }
    gvec& operator=(const gvec& o) { std::memcpy(e, o.e, sizeof(e)); return *this; }
    T& operator[](int i) { return e[i]; }
    const T& operator[](int i) const { return e[i]; }
};

#undef SWZ

typedef gvec<float, 2> vec2;
typedef gvec<float, 3> vec3;
typedef gvec<float, 4> vec4;
typedef gvec<int, 2> ivec2;
typedef gvec<int, 3> ivec3;
typedef gvec<int, 4> ivec4;
typedef gvec<uint, 2> uvec2;
typedef gvec<uint, 3> uvec3;
typedef gvec<uint, 4> uvec4;
typedef gvec<bool, 3> bvec3;

// -------------------------------------------------- component-wise operators
// Non-template overloads per concrete type so swizzle proxies convert.
#define VEC_BINOP(V, S, N, OP)                                                                   \
    inline V operator OP(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] OP b.e[i]; return r; } \
    inline V operator OP(const V& a, S s) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] OP s; return r; }             \
    inline V operator OP(S s, const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = s OP a.e[i]; return r; }             \
    inline V& operator OP##=(V& a, const V& b) { for (int i = 0; i < N; ++i) a.e[i] = a.e[i] OP b.e[i]; return a; }        \
    inline V& operator OP##=(V& a, S s) { for (int i = 0; i < N; ++i) a.e[i] = a.e[i] OP s; return a; }
#define VEC_ARITH(V, S, N) VEC_BINOP(V, S, N, +) VEC_BINOP(V, S, N, -) VEC_BINOP(V, S, N, *) VEC_BINOP(V, S, N, /) \
    inline V operator-(const V& a) { V r; for (int i = 0; i < N; ++i) r.e[i] = -a.e[i]; return r; }
VEC_ARITH(vec2, float, 2)
VEC_ARITH(vec3, float, 3)
VEC_ARITH(vec4, float, 4)
VEC_ARITH(ivec2, int, 2)
VEC_ARITH(ivec3, int, 3)
VEC_ARITH(ivec4, int, 4)
#define IVEC_BIT(V, S, N, OP)                                                                   \
    inline V operator OP(const V& a, const V& b) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] OP b.e[i]; return r; } \
    inline V operator OP(const V& a, S s) { V r; for (int i = 0; i < N; ++i) r.e[i] = a.e[i] OP s; return r; }
IVEC_BIT(ivec3, int, 3, &)
IVEC_BIT(ivec3, int, 3, %)
IVEC_BIT(ivec2, int, 2, %)

// ------------------------------------------------------------- built-ins
#define F1(NAME, EXPR)                                                                            \
    inline float NAME(float x) { return EXPR; }                                                 \
    inline vec2 NAME(const vec2& v) { vec2 r; for (int i = 0; i < 2; ++i) { float x = v.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec3 NAME(const vec3& v) { vec3 r; for (int i = 0; i < 3; ++i) { float x = v.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec4 NAME(const vec4& v) { vec4 r; for (int i = 0; i < 4; ++i) { float x = v.e[i]; r.e[i] = EXPR; } return r; }
F1(abs, glslc::f_abs(x))
F1(floor, glslc::f_floor(x))
F1(fract, x - glslc::f_floor(x))
F1(sqrt, glslc::f_sqrt(x))
F1(inversesqrt, 1.0f / glslc::f_sqrt(x))
F1(sin, glslc::f_sin(x))
F1(cos, glslc::f_cos(x))
F1(exp, glslc::f_exp(x))
F1(log, glslc::f_log(x))
F1(sign, x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f))
// integer overloads only match integer arguments exactly, so that e.g.
// clamp(float, 0, 1) picks the float overload as GLSL does
template <typename I> using only_int = std::enable_if_t<std::is_same_v<I, int> || std::is_same_v<I, uint>, int>;
template <typename I, only_int<I> = 0> inline I abs(I x) { return x < 0 ? -x : x; }

#define F2(NAME, EXPR)                                                                            \
    inline float NAME(float x, float y) { return EXPR; }                                        \
    inline vec2 NAME(const vec2& a, const vec2& b) { vec2 r; for (int i = 0; i < 2; ++i) { float x = a.e[i], y = b.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec3 NAME(const vec3& a, const vec3& b) { vec3 r; for (int i = 0; i < 3; ++i) { float x = a.e[i], y = b.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec4 NAME(const vec4& a, const vec4& b) { vec4 r; for (int i = 0; i < 4; ++i) { float x = a.e[i], y = b.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec2 NAME(const vec2& a, float y) { vec2 r; for (int i = 0; i < 2; ++i) { float x = a.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec3 NAME(const vec3& a, float y) { vec3 r; for (int i = 0; i < 3; ++i) { float x = a.e[i]; r.e[i] = EXPR; } return r; } \
    inline vec4 NAME(const vec4& a, float y) { vec4 r; for (int i = 0; i < 4; ++i) { float x = a.e[i]; r.e[i] = EXPR; } return r; }
// GLSL: min(x, y) = y < x ? y : x; max(x, y) = x < y ? y : x
F2(min, y < x ? y : x)
F2(max, x < y ? y : x)
F2(pow, glslc::f_pow(x, y))
F2(mod, x - y * glslc::f_floor(x / y))
F2(step, x > y ? 0.0f : 1.0f)   // step(edge = x, v = y): 0 if v < edge
inline vec2 step(float edge, const vec2& v) { return vec2(v.e[0] < edge ? 0.0f : 1.0f, v.e[1] < edge ? 0.0f : 1.0f); }
inline vec3 step(float edge, const vec3& v) {
    return vec3(v.e[0] < edge ? 0.0f : 1.0f, v.e[1] < edge ? 0.0f : 1.0f, v.e[2] < edge ? 0.0f : 1.0f);
}
template <typename I, only_int<I> = 0> inline I min(I x, I y) { return y < x ? y : x; }
template <typename I, only_int<I> = 0> inline I max(I x, I y) { return x < y ? y : x; }

inline float clamp(float v, float lo, float hi) { return min(max(v, lo), hi); }
inline vec2 clamp(const vec2& v, float lo, float hi) { return min(max(v, lo), hi); }
inline vec3 clamp(const vec3& v, float lo, float hi) { return min(max(v, lo), hi); }
inline vec4 clamp(const vec4& v, float lo, float hi) { return min(max(v, lo), hi); }
inline vec2 clamp(const vec2& v, const vec2& lo, const vec2& hi) { return min(max(v, lo), hi); }
inline vec3 clamp(const vec3& v, const vec3& lo, const vec3& hi) { return min(max(v, lo), hi); }
template <typename I, only_int<I> = 0> inline I clamp(I v, I lo, I hi) { return min(max(v, lo), hi); }
inline ivec3 clamp(const ivec3& v, const ivec3& lo, const ivec3& hi) {
    ivec3 r;
    for (int i = 0; i < 3; ++i) r.e[i] = min(max(v.e[i], lo.e[i]), hi.e[i]);
    return r;
}

inline float mix(float x, float y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, const vec3& a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, float a) { return x * (1.0f - a) + y * a; }
inline vec3 mix(const vec3& x, const vec3& y, const ivec3& a) { return mix(x, y, vec3(a)); }

inline float dot(const vec2& a, const vec2& b) { return a.e[0] * b.e[0] + a.e[1] * b.e[1]; }
inline float dot(const vec3& a, const vec3& b) { return a.e[0] * b.e[0] + a.e[1] * b.e[1] + a.e[2] * b.e[2]; }
inline float dot(const vec4& a, const vec4& b) {
    return a.e[0] * b.e[0] + a.e[1] * b.e[1] + a.e[2] * b.e[2] + a.e[3] * b.e[3];
}
inline vec3 cross(const vec3& a, const vec3& b) {
    return vec3(a.e[1] * b.e[2] - a.e[2] * b.e[1], a.e[2] * b.e[0] - a.e[0] * b.e[2], a.e[0] * b.e[1] - a.e[1] * b.e[0]);
}
// reflect(I, N) = I - 2 dot(N, I) N
inline vec3 reflect(const vec3& i, const vec3& n) { return i - (2.0f * dot(n, i)) * n; }
inline float length(const vec2& v) { return glslc::f_sqrt(dot(v, v)); }
inline float length(const vec3& v) { return glslc::f_sqrt(dot(v, v)); }
inline float length(const ivec3& v) { return length(vec3(v)); }
inline float distance(const vec3& a, const vec3& b) { return length(a - b); }
// normalize(x) = x / length(x)
inline vec2 normalize(const vec2& v) { return v / length(v); }
inline vec3 normalize(const vec3& v) { return v / length(v); }
inline bvec3 greaterThan(const vec3& a, const vec3& b) {
    bvec3 r;
    for (int i = 0; i < 3; ++i) r.e[i] = a.e[i] > b.e[i];
    return r;
}
inline bool any(const bvec3& v) { return v.e[0] || v.e[1] || v.e[2]; }
inline float uintBitsToFloat(uint u) { float f; std::memcpy(&f, &u, 4); return f; }

// --------------------------------------------------------------- matrices
struct mat3 {
    vec3 c[3];
    mat3() {}
    mat3(const vec3& a, const vec3& b, const vec3& d) { c[0] = a; c[1] = b; c[2] = d; }
    explicit mat3(const struct mat4& m);
    vec3& operator[](int i) { return c[i]; }
    const vec3& operator[](int i) const { return c[i]; }
};
struct mat4 {
    vec4 c[4];
    mat4() {}
    vec4& operator[](int i) { return c[i]; }
    const vec4& operator[](int i) const { return c[i]; }
};
inline mat3::mat3(const mat4& m) {
    for (int i = 0; i < 3; ++i) c[i] = vec3(m.c[i].e[0], m.c[i].e[1], m.c[i].e[2]);
}
inline vec3 operator*(const mat3& m, const vec3& v) {
    return m.c[0] * v.e[0] + m.c[1] * v.e[1] + m.c[2] * v.e[2];
}
inline vec4 operator*(const mat4& m, const vec4& v) {
    return m.c[0] * v.e[0] + m.c[1] * v.e[1] + m.c[2] * v.e[2] + m.c[3] * v.e[3];
}
// inverse of a 4x4 matrix by Gauss-Jordan elimination with partial pivoting
inline mat4 inverse(const mat4& m) {
    float a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) {
            a[r][k] = m.c[k].e[r];
            a[r][k + 4] = (r == k) ? 1.0f : 0.0f;
        }
    for (int col = 0; col < 4; ++col) {
        int piv = col;
        for (int r = col + 1; r < 4; ++r)
            if (glslc::f_abs(a[r][col]) > glslc::f_abs(a[piv][col])) piv = r;
        if (piv != col)
            for (int k = 0; k < 8; ++k) { float t = a[col][k]; a[col][k] = a[piv][k]; a[piv][k] = t; }
        float inv = 1.0f / a[col][col];
        for (int k = 0; k < 8; ++k) a[col][k] *= inv;
        for (int r = 0; r < 4; ++r) {
            if (r == col) continue;
            float f = a[r][col];
            for (int k = 0; k < 8; ++k) a[r][k] -= f * a[col][k];
        }
    }
    mat4 o;
    for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) o.c[k].e[r] = a[r][k + 4];
    return o;
}

// --------------------------------------------------------------- samplers
struct sampler3D {
    const float* f32 = nullptr;
    const uint16_t* f16 = nullptr;
    int W = 0, H = 0, D = 0;
    // mip levels (FP16) with REPEAT wrap for textureLod: the mesh SDF
    // volumes (Texture3D with their default sampler); levels == 0 = none
    int levels = 0;
    const uint16_t* lv[3] = {nullptr, nullptr, nullptr};
    int lw[3] = {0, 0, 0}, lh[3] = {0, 0, 0}, ld[3] = {0, 0, 0};
    float at(int x, int y, int z) const {
        size_t i = size_t(x) + size_t(W) * (size_t(y) + size_t(H) * size_t(z));
        if (f16) { _Float16 h; std::memcpy(&h, f16 + i, 2); return float(h); }
        return f32[i];
    }
};
struct sampler2D {
    const float* f32 = nullptr;
    const uint16_t* f16 = nullptr;
    const uint8_t* u8 = nullptr;
    const uint32_t* r11 = nullptr;   // packed R11G11B10F (oracle/packed_color.h)
    int W = 0, H = 0, C = 4;
    bool repeat = false;
    float at(int x, int y, int ch) const {
        if (r11) return packed_color::channel(r11[size_t(y) * size_t(W) + size_t(x)], ch);
        if (ch >= C) return ch == 3 ? 1.0f : 0.0f;
        size_t i = (size_t(y) * size_t(W) + size_t(x)) * size_t(C) + size_t(ch);
        if (f16) { _Float16 h; std::memcpy(&h, f16 + i, 2); return float(h); }
        if (u8) return float(u8[i]) / 255.0f;
        return f32[i];
    }
    int wrap(int i, int n) const {
        if (repeat) { int r = i % n; return r < 0 ? r + n : r; }
        return i < 0 ? 0 : (i >= n ? n - 1 : i);
    }
};
struct samplerCube { vec3 color; };

inline vec4 texture(const sampler3D& t, const vec3& uvw) {
    float x = uvw.e[0] * float(t.W) - 0.5f, y = uvw.e[1] * float(t.H) - 0.5f, z = uvw.e[2] * float(t.D) - 0.5f;
    float fx = glslc::f_floor(x), fy = glslc::f_floor(y), fz = glslc::f_floor(z);
    float a = x - fx, b = y - fy, c = z - fz;
    auto cl = [](int i, int n) { return i < 0 ? 0 : (i >= n ? n - 1 : i); };
    int x0 = cl(int(fx), t.W), x1 = cl(int(fx) + 1, t.W), y0 = cl(int(fy), t.H), y1 = cl(int(fy) + 1, t.H);
    int z0 = cl(int(fz), t.D), z1 = cl(int(fz) + 1, t.D);
    float v = (1 - a) * (1 - b) * (1 - c) * t.at(x0, y0, z0) + a * (1 - b) * (1 - c) * t.at(x1, y0, z0) +
              (1 - a) * b * (1 - c) * t.at(x0, y1, z0) + a * b * (1 - c) * t.at(x1, y1, z0) +
              (1 - a) * (1 - b) * c * t.at(x0, y0, z1) + a * (1 - b) * c * t.at(x1, y0, z1) +
              (1 - a) * b * c * t.at(x0, y1, z1) + a * b * c * t.at(x1, y1, z1);
    return vec4(v, 0.0f, 0.0f, 1.0f);
}
inline vec4 textureLod(const sampler3D& t, const vec3& uvw, float lod) {
    if (t.levels == 0) return texture(t, uvw);
    int L = int(lod);
    L = L < 0 ? 0 : (L >= t.levels ? t.levels - 1 : L);
    const int W = t.lw[L], H = t.lh[L], D = t.ld[L];
    float x = uvw.e[0] * float(W) - 0.5f, y = uvw.e[1] * float(H) - 0.5f, z = uvw.e[2] * float(D) - 0.5f;
    float fx = glslc::f_floor(x), fy = glslc::f_floor(y), fz = glslc::f_floor(z);
    float a = x - fx, b = y - fy, c = z - fz;
    auto wr = [](int i, int n) { int r = i % n; return r < 0 ? r + n : r; };
    int x0 = wr(int(fx), W), x1 = wr(int(fx) + 1, W), y0 = wr(int(fy), H), y1 = wr(int(fy) + 1, H);
    int z0 = wr(int(fz), D), z1 = wr(int(fz) + 1, D);
    auto at = [&](int i, int j, int k) {
        _Float16 h;
        std::memcpy(&h, t.lv[L] + size_t(i) + size_t(W) * (size_t(j) + size_t(H) * size_t(k)), 2);
        return float(h);
    };
    float v = (1 - a) * (1 - b) * (1 - c) * at(x0, y0, z0) + a * (1 - b) * (1 - c) * at(x1, y0, z0) +
              (1 - a) * b * (1 - c) * at(x0, y1, z0) + a * b * (1 - c) * at(x1, y1, z0) +
              (1 - a) * (1 - b) * c * at(x0, y0, z1) + a * (1 - b) * c * at(x1, y0, z1) +
              (1 - a) * b * c * at(x0, y1, z1) + a * b * c * at(x1, y1, z1);
    return vec4(v, 0.0f, 0.0f, 1.0f);
}
inline vec4 texture(const sampler2D& t, const vec2& uv) {
    float x = uv.e[0] * float(t.W) - 0.5f, y = uv.e[1] * float(t.H) - 0.5f;
    float fx = glslc::f_floor(x), fy = glslc::f_floor(y);
    float a = x - fx, b = y - fy;
    int i0 = t.wrap(int(fx), t.W), i1 = t.wrap(int(fx) + 1, t.W), j0 = t.wrap(int(fy), t.H), j1 = t.wrap(int(fy) + 1, t.H);
    vec4 r;
    for (int ch = 0; ch < 4; ++ch)
        r.e[ch] = (1 - a) * (1 - b) * t.at(i0, j0, ch) + a * (1 - b) * t.at(i1, j0, ch) + (1 - a) * b * t.at(i0, j1, ch) +
                  a * b * t.at(i1, j1, ch);
    return r;
}
inline vec4 textureLod(const sampler2D& t, const vec2& uv, float) { return texture(t, uv); }
inline vec4 textureGather(const sampler2D& t, const vec2& uv, int ch) {
    float x = uv.e[0] * float(t.W) - 0.5f, y = uv.e[1] * float(t.H) - 0.5f;
    int i0 = int(glslc::f_floor(x)), j0 = int(glslc::f_floor(y));
    int i1 = t.wrap(i0 + 1, t.W), j1 = t.wrap(j0 + 1, t.H);
    i0 = t.wrap(i0, t.W);
    j0 = t.wrap(j0, t.H);
    return vec4(t.at(i0, j1, ch), t.at(i1, j1, ch), t.at(i1, j0, ch), t.at(i0, j0, ch));
}
inline vec4 texture(const samplerCube& t, const vec3&) { return vec4(t.color, 1.0f); }
