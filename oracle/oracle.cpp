// ORACLE -- test infrastructure only.  Not part of the product path.
//
// A CPU restatement (C++17, OpenMP over probes) of LuxGI's non-raytracing
// DDGI probe update, written from the reference GLSL.  Every function cites
// the reference lines it follows (paths relative to Code/Maple/src/Shaders/
// unless stated).  Templated on the arithmetic type: R = float is the FP32
// transcription (same operation order as the CUDA kernels, no FP
// contraction, so the SDF march matches them bit for bit), R = double is the
// FP64 error reference.  The FP16-storage switch rounds at the points where
// the reference stores RGBA16F / RG16F (Engine/DDGI/DDGIRenderer.cpp:173-204).
//
// Parity pins: the reference ships no tests or golden data.  This oracle is
// pinned against the reference's own GLSL function libraries compiled as
// C++ (oracle/build_ref.py, oracle/ref_harness.cpp), by the border tables
// read from the reference source (tests/golden/) and by analytic
// known-answer tests.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// this library.
#include "../include/luxgi_ddgi.h"
#include "packed_color.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <array>
#include <limits>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- vectors
template <typename R> struct V2 { R x, y; };
template <typename R> struct V3 { R x, y, z; };
template <typename R> struct V4 { R x, y, z, w; };

template <typename R> inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <typename R> inline V3<R> add(V3<R> a, V3<R> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <typename R> inline V3<R> sub(V3<R> a, V3<R> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <typename R> inline V3<R> mul(V3<R> a, R s) { return {a.x * s, a.y * s, a.z * s}; }
template <typename R> inline V3<R> mulv(V3<R> a, V3<R> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
// GLSL dot: left-to-right sum of products
template <typename R> inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <typename R> inline R length(V3<R> a) { return std::sqrt(dot(a, a)); }
// normalize(v) = v * (1 / sqrt(dot(v, v))) -- the form the kernels use too
template <typename R> inline V3<R> normalize(V3<R> a) { R inv = R(1) / std::sqrt(dot(a, a)); return mul(a, inv); }
template <typename R> inline R clampr(R v, R lo, R hi) { return std::min(std::max(v, lo), hi); }
template <typename R> inline R fractr(R v) { return v - std::floor(v); }
template <typename R> inline R mixr(R x, R y, R a) { return x * (R(1) - a) + y * a; }

// column-major 4x4: m[col*4 + row]
template <typename R> struct M4 { R m[16]; };
template <typename R> inline M4<R> load_m4(const float* f) { M4<R> r; for (int i = 0; i < 16; ++i) r.m[i] = R(f[i]); return r; }
template <typename R> inline V4<R> mul_m4(const M4<R>& M, V4<R> v) {
    const R* m = M.m;
    return {m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * v.w,
            m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * v.w,
            m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * v.w,
            m[3] * v.x + m[7] * v.y + m[11] * v.z + m[15] * v.w};
}
// mat3(M) * v
template <typename R> inline V3<R> mul_m3of4(const M4<R>& M, V3<R> v) {
    const R* m = M.m;
    return {m[0] * v.x + m[4] * v.y + m[8] * v.z,
            m[1] * v.x + m[5] * v.y + m[9] * v.z,
            m[2] * v.x + m[6] * v.y + m[10] * v.z};
}
// inverse(M): adjugate / determinant, cofactors from 2x2 sub-determinants of
// the lower and upper row pairs (Laplace expansion).
template <typename R> inline M4<R> inverse(const M4<R>& A) {
    // a[r][c]
    R a[4][4];
    for (int c = 0; c < 4; ++c) for (int r = 0; r < 4; ++r) a[r][c] = A.m[c * 4 + r];
    R s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    R s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    R s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    R s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    R s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    R s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    R c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    R c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    R c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    R c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    R c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    R c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    R det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    R id = R(1) / det;
    R b[4][4];
    b[0][0] = ( a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3) * id;
    b[0][1] = (-a[0][1] * c5 + a[0][2] * c4 - a[0][3] * c3) * id;
    b[0][2] = ( a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3) * id;
    b[0][3] = (-a[2][1] * s5 + a[2][2] * s4 - a[2][3] * s3) * id;
    b[1][0] = (-a[1][0] * c5 + a[1][2] * c2 - a[1][3] * c1) * id;
    b[1][1] = ( a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1) * id;
    b[1][2] = (-a[3][0] * s5 + a[3][2] * s2 - a[3][3] * s1) * id;
    b[1][3] = ( a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1) * id;
    b[2][0] = ( a[1][0] * c4 - a[1][1] * c2 + a[1][3] * c0) * id;
    b[2][1] = (-a[0][0] * c4 + a[0][1] * c2 - a[0][3] * c0) * id;
    b[2][2] = ( a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0) * id;
    b[2][3] = (-a[2][0] * s4 + a[2][1] * s2 - a[2][3] * s0) * id;
    b[3][0] = (-a[1][0] * c3 + a[1][1] * c1 - a[1][2] * c0) * id;
    b[3][1] = ( a[0][0] * c3 - a[0][1] * c1 + a[0][2] * c0) * id;
    b[3][2] = (-a[3][0] * s3 + a[3][1] * s1 - a[3][2] * s0) * id;
    b[3][3] = ( a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0) * id;
    M4<R> out;
    for (int c = 0; c < 4; ++c) for (int r = 0; r < 4; ++r) out.m[c * 4 + r] = b[r][c];
    return out;
}

inline float h2f(uint16_t h) { _Float16 v; std::memcpy(&v, &h, 2); return float(v); }

inline uint32_t pack_r11g11b10(const float* v) { return packed_color::pack(v); }
inline float r11g11b10_channel(uint32_t v, int ch) { return packed_color::channel(v, ch); }
// One texel of a surface colour texture (luxgi_color_format) into rgba.
inline void color_load(const void* p, int fmt, size_t texel, float* out) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        const uint32_t v = static_cast<const uint32_t*>(p)[texel];
        for (int c = 0; c < 4; ++c) out[c] = r11g11b10_channel(v, c);
    } else {
        for (int c = 0; c < 4; ++c) out[c] = h2f(static_cast<const uint16_t*>(p)[texel * 4 + size_t(c)]);
    }
}
// The value a render target of format `fmt` keeps of v.
inline void color_round(int fmt, float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        const uint32_t q = pack_r11g11b10(v);
        for (int c = 0; c < 4; ++c) v[c] = r11g11b10_channel(q, c);
    } else {
        for (int c = 0; c < 4; ++c) v[c] = float(_Float16(v[c]));
    }
}
inline float round_half(float f) { return float(_Float16(f)); }

// ---------------------------------------------------------- sin / cos
// FP32: Cody-Waite reduction by pi/2 and Taylor polynomials of degree 9/8 on
// [-pi/4, pi/4]; the CUDA ray generator evaluates the same sequence.  FP64:
// the C library.  (GLSL leaves sin/cos precision to the implementation.)
inline void sincos_r(float x, float* s, float* c) {
    const float k = std::floor(x * 0.63661977f + 0.5f);
    const float r = (x - k * 1.57079637f) - k * -4.37113883e-8f;
    const float r2 = r * r;
    const float sp = r + r * r2 * (-0.166666672f + r2 * (0.00833333377f + r2 * (-0.000198412701f + r2 * 2.75573188e-6f)));
    const float cp = 1.0f + r2 * (-0.5f + r2 * (0.0416666679f + r2 * (-0.00138888892f + r2 * 2.48015876e-5f)));
    const int q = int(k) & 3;
    if (q == 0) { *s = sp; *c = cp; }
    else if (q == 1) { *s = cp; *c = -sp; }
    else if (q == 2) { *s = -sp; *c = -cp; }
    else { *s = -cp; *c = sp; }
}
inline void sincos_r(double x, double* s, double* c) { *s = std::sin(x); *c = std::cos(x); }

template <typename R> inline R pi_r();
template <> inline float pi_r<float>() { return 3.14159265f; }
template <> inline double pi_r<double>() { return 3.14159265358979323846; }

// ------------------------------------------------ DDGICommon.glsl
// madfrac(i, PHI - 1) (DDGICommon.glsl:46-47).  FP64: direct.  FP32:
// compensated -- PHI - 1 as a hi + lo float pair, the product i * hi split
// exactly by one FMA -- so FP32 directions stay within ~1e-7 of FP64 at any
// ray index (the plain FP32 product loses ~2^-24 * i turns).
inline double fib_frac(double i) {
    const double PHI = std::sqrt(5.0) * 0.5 + 0.5;
    double t = i * (PHI - 1.0);
    return t - std::floor(t);
}
inline float fib_frac(float i) {
    const float c_hi = 0.618034005165100098f;
    const float c_lo = -1.64152047e-8f;
    const float p = i * c_hi;
    const float e = std::fmaf(i, c_hi, -p);
    float m = (p - std::floor(p)) + (e + i * c_lo);
    if (m >= 1.0f) m = m - 1.0f;
    if (m < 0.0f) m = m + 1.0f;
    return m;
}

// sphericalFibonacci (DDGICommon.glsl:42-52)
template <typename R> V3<R> spherical_fibonacci(R i, R n) {
    R mf = fib_frac(i);
    R phi = (R(2) * pi_r<R>()) * mf;
    R cos_t = R(1) - (R(2) * i + R(1)) * (R(1) / n);
    R sin_t = std::sqrt(clampr(R(1) - cos_t * cos_t, R(0), R(1)));
    R sp, cp;
    sincos_r(phi, &sp, &cp);
    return {cp * sin_t, sp * sin_t, cos_t};
}

template <typename R> inline R sign_not_zero(R k) { return k >= R(0) ? R(1) : R(-1); }

// octEncode (DDGICommon.glsl:65-72)
template <typename R> V2<R> oct_encode(V3<R> v) {
    R l1 = std::fabs(v.x) + std::fabs(v.y) + std::fabs(v.z);
    R inv = R(1) / l1;
    V2<R> r{v.x * inv, v.y * inv};
    if (v.z < R(0)) {
        V2<R> t{(R(1) - std::fabs(r.y)) * sign_not_zero(r.x), (R(1) - std::fabs(r.x)) * sign_not_zero(r.y)};
        r = t;
    }
    return r;
}
// octDecode (DDGICommon.glsl:74-82)
template <typename R> V3<R> oct_decode(V2<R> o) {
    V3<R> v{o.x, o.y, R(1) - std::fabs(o.x) - std::fabs(o.y)};
    if (v.z < R(0)) {
        R nx = (R(1) - std::fabs(v.y)) * sign_not_zero(v.x);
        R ny = (R(1) - std::fabs(v.x)) * sign_not_zero(v.y);
        v.x = nx; v.y = ny;
    }
    return normalize(v);
}
// normalizedOctCoord (DDGICommon.glsl:85-92) for interior texel (tx, ty)
template <typename R> V2<R> normalized_oct_coord(int tx, int ty, int side) {
    R s = R(2) / R(side);
    return {(R(tx) + R(0.5)) * s - R(1), (R(ty) + R(0.5)) * s - R(1)};
}
// textureCoordFromDirection (DDGICommon.glsl:141-158)
template <typename R> V2<R> tex_coord_from_dir(V3<R> dir, int probe, int width, int height, int side) {
    V2<R> o = oct_encode(normalize(dir));
    V2<R> zo{(o.x + R(1)) * R(0.5), (o.y + R(1)) * R(0.5)};
    R pwb = R(side) + R(2);
    V2<R> octn{(zo.x * R(side)) / R(width), (zo.y * R(side)) / R(height)};
    int ppr = (width - 2) / int(pwb);
    V2<R> tl{R(probe % ppr) * pwb + R(2), R(probe / ppr) * pwb + R(2)};
    V2<R> tln{tl.x / R(width), tl.y / R(height)};
    return {tln.x + octn.x, tln.y + octn.y};
}

// ------------------------------------------------ texture emulation
// GL LINEAR filtering, CLAMP_TO_EDGE, on the packed SDF (x fastest).
struct Vol {
    const float* f32 = nullptr;
    const uint16_t* f16 = nullptr;
    int W = 0, H = 0, D = 0;
    float at(int x, int y, int z) const {
        size_t i = size_t(x) + size_t(W) * (size_t(y) + size_t(H) * size_t(z));
        return f16 ? h2f(f16[i]) : f32[i];
    }
};
template <typename R> R sample3d(const Vol& v, V3<R> uvw) {
    R x = uvw.x * R(v.W) - R(0.5), y = uvw.y * R(v.H) - R(0.5), z = uvw.z * R(v.D) - R(0.5);
    R fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    R a = x - fx, b = y - fy, c = z - fz;
    int x0 = int(fx), y0 = int(fy), z0 = int(fz);
    int x1 = std::min(std::max(x0 + 1, 0), v.W - 1), y1 = std::min(std::max(y0 + 1, 0), v.H - 1),
        z1 = std::min(std::max(z0 + 1, 0), v.D - 1);
    x0 = std::min(std::max(x0, 0), v.W - 1); y0 = std::min(std::max(y0, 0), v.H - 1);
    z0 = std::min(std::max(z0, 0), v.D - 1);
    R t000 = R(v.at(x0, y0, z0)), t100 = R(v.at(x1, y0, z0));
    R t010 = R(v.at(x0, y1, z0)), t110 = R(v.at(x1, y1, z0));
    R t001 = R(v.at(x0, y0, z1)), t101 = R(v.at(x1, y0, z1));
    R t011 = R(v.at(x0, y1, z1)), t111 = R(v.at(x1, y1, z1));
    R ia = R(1) - a, ib = R(1) - b, ic = R(1) - c;
    R c00 = t000 * ia + t100 * a, c10 = t010 * ia + t110 * a;
    R c01 = t001 * ia + t101 * a, c11 = t011 * ia + t111 * a;
    R c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// 2D atlas texel access
struct Tex2 {
    const float* f32 = nullptr;      // interleaved channels
    const uint16_t* f16 = nullptr;
    const uint8_t* u8 = nullptr;     // UNORM
    const uint32_t* r11 = nullptr;   // packed R11G11B10F (alpha reads 1)
    int W = 0, H = 0, C = 4;
    float at(int x, int y, int ch) const {
        const size_t texel = size_t(y) * size_t(W) + size_t(x);
        if (r11) return r11g11b10_channel(r11[texel], ch);
        size_t i = texel * size_t(C) + size_t(ch);
        if (f16) return h2f(f16[i]);
        if (u8) return float(u8[i]) / 255.0f;
        return f32[i];
    }
    // a colour texture of luxgi_color_format `fmt`
    void set_color(const void* p, int fmt) {
        if (fmt == LUXGI_COLOR_R11G11B10F) r11 = static_cast<const uint32_t*>(p);
        else f16 = static_cast<const uint16_t*>(p);
        C = 4;
    }
    // a G-buffer of luxgi_gbuffer_format `fmt`
    void set_gbuffer(const void* p, int fmt) {
        if (fmt == LUXGI_GBUFFER_RGBA16F) f16 = static_cast<const uint16_t*>(p);
        else f32 = static_cast<const float*>(p);
        C = 4;
    }
};
// textureGather component order: (i0,j1), (i1,j1), (i1,j0), (i0,j0); clamp to edge
template <typename R> V4<R> gather(const Tex2& t, V2<R> uv, int ch) {
    R x = uv.x * R(t.W) - R(0.5), y = uv.y * R(t.H) - R(0.5);
    int i0 = int(std::floor(x)), j0 = int(std::floor(y));
    int i1 = std::min(std::max(i0 + 1, 0), t.W - 1), j1 = std::min(std::max(j0 + 1, 0), t.H - 1);
    i0 = std::min(std::max(i0, 0), t.W - 1); j0 = std::min(std::max(j0, 0), t.H - 1);
    return {R(t.at(i0, j1, ch)), R(t.at(i1, j1, ch)), R(t.at(i1, j0, ch)), R(t.at(i0, j0, ch))};
}
// textureLod(..., 0) bilinear with REPEAT (default sampler of the probe atlases)
template <typename R> R bilinear_repeat(const Tex2& t, V2<R> uv, int ch) {
    R x = uv.x * R(t.W) - R(0.5), y = uv.y * R(t.H) - R(0.5);
    R fx = std::floor(x), fy = std::floor(y);
    R a = x - fx, b = y - fy;
    auto wrap = [](int i, int n) { int r = i % n; return r < 0 ? r + n : r; };
    int i0 = wrap(int(fx), t.W), i1 = wrap(int(fx) + 1, t.W);
    int j0 = wrap(int(fy), t.H), j1 = wrap(int(fy) + 1, t.H);
    R t00 = R(t.at(i0, j0, ch)), t10 = R(t.at(i1, j0, ch)), t01 = R(t.at(i0, j1, ch)), t11 = R(t.at(i1, j1, ch));
    R r0 = t00 * (R(1) - a) + t10 * a, r1 = t01 * (R(1) - a) + t11 * a;
    return r0 * (R(1) - b) + r1 * b;
}

// ------------------------------------------------ SDFCommon.glsl
template <typename R> struct Hit {
    V3<R> normal{R(0), R(0), R(0)};
    R time = R(-1);
    int cascade = 0;
    int steps = 0;
    int fine = 0;
    R sdf = R(0);
};

// lineHitAABB (SDFCommon.glsl:84-95)
template <typename R> V2<R> line_hit_aabb(V3<R> s, V3<R> e, V3<R> bmin, V3<R> bmax) {
    V3<R> d = sub(e, s);
    V3<R> inv{R(1) / d.x, R(1) / d.y, R(1) / d.z};
    V3<R> en{(bmin.x - s.x) * inv.x, (bmin.y - s.y) * inv.y, (bmin.z - s.z) * inv.z};
    V3<R> ex{(bmax.x - s.x) * inv.x, (bmax.y - s.y) * inv.y, (bmax.z - s.z) * inv.z};
    V3<R> mn{std::min(en.x, ex.x), std::min(en.y, ex.y), std::min(en.z, ex.z)};
    V3<R> mx{std::max(en.x, ex.x), std::max(en.y, ex.y), std::max(en.z, ex.z)};
    V2<R> r{std::max(mn.x, std::max(mn.y, mn.z)), std::min(mx.x, std::min(mx.y, mx.z))};
    return {clampr(r.x, R(0), R(1)), clampr(r.y, R(0), R(1))};
}

// getGlobalSDFCascadeUV (SDFCommon.glsl:64-71)
template <typename R> V3<R> cascade_texture_uv(const luxgi_sdf_data& d, int cascade, V3<R> p, R* max_dist) {
    V3<R> c{R(d.cascade_pos_distance[cascade][0]), R(d.cascade_pos_distance[cascade][1]), R(d.cascade_pos_distance[cascade][2])};
    R w = R(d.cascade_pos_distance[cascade][3]);
    V3<R> pic = sub(p, c);
    R md = w * R(2);
    *max_dist = md;
    V3<R> cuv{clampr(pic.x / md + R(0.5), R(0), R(1)), clampr(pic.y / md + R(0.5), R(0), R(1)),
              clampr(pic.z / md + R(0.5), R(0), R(1))};
    return {(R(cascade) + cuv.x) / R(d.cascades_count), cuv.y, cuv.z};
}

// tracyGlobalSDF (SDFCommon.glsl:98-194) with stepScale = 1.  The probe
// rays use start bias 0 and want the hit normal (GISDFRays.comp:79-87); the
// surface-cache shadow rays start 2 voxels along and skip the normal
// (SDFDeferredLight.frag:104-111).
// Optional record of a march's sample points: per step the packed texture
// coordinates (u, v, w) and 1 when the full-resolution SDF was sampled.
struct MarchTrail {
    float* out;
    int cap, n;
};

template <typename R> Hit<R> trace_sdf(const luxgi_sdf_data& d, const Vol& tex, const Vol& mip,
                                       V3<R> origin, V3<R> dir, R trace_max, int max_steps,
                                       R start_bias = R(0), bool want_normal = true, MarchTrail* trail = nullptr) {
    Hit<R> hit;
    const int C = int(d.cascades_count);
    R tmax = std::min(trace_max, R(d.cascade_pos_distance[C - 1][3]) * R(2));
    R chunk = R(32) / R(d.resolution);
    R margin = R(4) / R(d.resolution);
    R next_start = R(0);
    V3<R> end = add(origin, mul(dir, tmax));
    for (int cascade = 0; cascade < C && hit.time < R(0); ++cascade) {
        V3<R> cpos{R(d.cascade_pos_distance[cascade][0]), R(d.cascade_pos_distance[cascade][1]), R(d.cascade_pos_distance[cascade][2])};
        R cw = R(d.cascade_pos_distance[cascade][3]);
        R voxel = R(d.cascade_voxel_size[cascade]);
        R voxel_half = voxel * R(0.5);
        V3<R> wpos = add(origin, mul(dir, voxel * start_bias));
        V2<R> is = line_hit_aabb(wpos, end, v3(cpos.x - cw, cpos.y - cw, cpos.z - cw), v3(cpos.x + cw, cpos.y + cw, cpos.z + cw));
        is.x = is.x * tmax;
        is.y = is.y * tmax;
        is.x = std::max(is.x, next_start);
        R t = is.x;
        if (is.x >= is.y) t = is.y;
        else next_start = is.y;
        int step = 0;
        for (; step < max_steps && t < is.y; ++step) {
            V3<R> sp = add(wpos, mul(dir, t));
            R cmd;
            V3<R> uv = cascade_texture_uv(d, cascade, sp, &cmd);
            R sd = sample3d(mip, uv);
            if (trail && trail->n < trail->cap) {
                float* o = trail->out + 4 * trail->n++;
                o[0] = float(uv.x); o[1] = float(uv.y); o[2] = float(uv.z); o[3] = sd < chunk ? 1.0f : 0.0f;
            }
            if (sd < chunk) {
                R sdt = sample3d(tex, uv);
                ++hit.fine;
                if (sdt < margin * R(2)) sd = sdt;
            } else {
                sd = chunk;
            }
            sd = sd * cmd;
            R thick = voxel_half * clampr(t / voxel, R(0), R(1));
            if (sd < thick) {
                hit.time = std::max(t + sd - thick, R(0));
                hit.cascade = cascade;
                hit.sdf = sd;
                if (!want_normal) break;
                R off = R(1) / R(d.resolution);
                R xp = sample3d(tex, v3(uv.x + off, uv.y, uv.z));
                R xn = sample3d(tex, v3(uv.x - off, uv.y, uv.z));
                R yp = sample3d(tex, v3(uv.x, uv.y + off, uv.z));
                R yn = sample3d(tex, v3(uv.x, uv.y - off, uv.z));
                R zp = sample3d(tex, v3(uv.x, uv.y, uv.z + off));
                R zn = sample3d(tex, v3(uv.x, uv.y, uv.z - off));
                hit.normal = normalize(v3(xp - xn, yp - yn, zp - zn));
                break;
            }
            t = t + std::max(sd * R(1), voxel);
        }
        hit.steps += step;
    }
    return hit;
}

// ------------------------------------------------ AtlasCommon.glsl
struct Surface {
    const luxgi_surface_desc* d;
    Tex2 depth, c0, c1;     // c1 used for the second (albedo) atlas in mode B
    bool two = false;
};

// sampleGlobalSurfaceAtlasTile, both overloads (AtlasCommon.glsl:58-112).
// Accumulates colour * weight into acc0 (and acc1 for the second atlas).
template <typename R> void sample_tile(const Surface& S, const luxgi_surface_tile& tile, V3<R> local,
                                       V3<R> nrm_local, R thr, V3<R>& acc0, V3<R>& acc1, R& accw) {
    M4<R> T = load_m4<R>(tile.transform);
    V4<R> n4 = mul_m4(T, V4<R>{nrm_local.x, nrm_local.y, nrm_local.z, R(1)});
    V3<R> n = normalize(V3<R>{n4.x, n4.y, n4.z});
    R nw = clampr(R(0) * n.x + R(0) * n.y + R(1) * n.z, R(0), R(1));
    nw = (nw - R(0.05f)) / (R(1) - R(0.05f));
    if (nw <= R(0)) return;
    V4<R> tp = mul_m4(T, V4<R>{local.x, local.y, local.z, R(1)});
    R bx = R(tile.object_bounds[0]), by = R(tile.object_bounds[1]), bz = R(tile.object_bounds[2]);
    R tdepth = tp.z / bz;
    V2<R> tuv{clampr(tp.x / bx + R(0.5), R(0), R(1)), clampr(tp.y / by + R(0.5), R(0), R(1))};
    V2<R> auv{tuv.x * R(tile.extends[2]) + R(tile.extends[0]), tuv.y * R(tile.extends[3]) + R(tile.extends[1])};
    R res = R(S.d->data.resolution);
    V2<R> bwu{fractr(auv.x * res + R(0.5)), fractr(auv.y * res + R(0.5))};
    V4<R> bw{(R(1) - bwu.x) * bwu.y, bwu.x * bwu.y, bwu.x * (R(1) - bwu.y), (R(1) - bwu.x) * (R(1) - bwu.y)};
    V4<R> tz = gather(S.depth, auv, 0);
    R dthr = R(2) * thr / bz;
    R dv[4];
    R tzs[4] = {tz.x, tz.y, tz.z, tz.w};
    for (int i = 0; i < 4; ++i) {
        dv[i] = R(1) - clampr((std::fabs(tdepth - tzs[i]) - dthr) / (R(0.5) * dthr), R(0), R(1));
        if (tzs[i] >= R(1)) dv[i] = R(0);
    }
    R sw = dv[0] * bw.x + dv[1] * bw.y + dv[2] * bw.z + dv[3] * bw.w;
    sw = sw * nw;
    if (sw <= R(0)) return;
    V4<R> w{bw.x * dv[0], bw.y * dv[1], bw.z * dv[2], bw.w * dv[3]};
    auto color = [&](const Tex2& tex) {
        V4<R> gx = gather(tex, auv, 0), gy = gather(tex, auv, 1), gz = gather(tex, auv, 2);
        return V3<R>{gx.x * w.x + gx.y * w.y + gx.z * w.z + gx.w * w.w,
                     gy.x * w.x + gy.y * w.y + gy.z * w.z + gy.w * w.w,
                     gz.x * w.x + gz.y * w.y + gz.z * w.z + gz.w * w.w};
    };
    V3<R> c0 = color(S.c0);
    acc0 = add(acc0, mul(c0, sw));
    if (S.two) {
        V3<R> c1 = color(S.c1);
        acc1 = add(acc1, mul(c1, sw));
    }
    accw = accw + sw;
}

// sampleGlobalSurfaceAtlas macro (AtlasCommon.glsl:115-157), debug = false.
template <typename R> R sample_surface(const Surface& S, V3<R> pos, V3<R> wn, R thr, V3<R>& out0, V3<R>& out1) {
    const luxgi_surface_desc* d = S.d;
    V3<R> acc0{R(0), R(0), R(0)}, acc1{R(0), R(0), R(0)};
    R accw = R(0);
    R cs = R(d->data.chunk_size);
    int cc[3];
    R pc[3] = {pos.x, pos.y, pos.z};
    for (int k = 0; k < 3; ++k) {
        int v = int(std::floor(pc[k] / cs + R(40 * 0.5f)));
        cc[k] = std::min(std::max(v, 0), 39);
    }
    uint32_t addr = uint32_t(cc[2] * 40 * 40 + cc[1] * 40 + cc[0]);
    uint32_t start = d->chunks[addr];
    out0 = acc0; out1 = acc1;
    if (start == 0) return R(0);
    uint32_t count = d->culled_objects[start];
    if (count > d->data.objects_count) return R(0);
    ++start;
    for (uint32_t oi = 0; oi < count; ++oi) {
        uint32_t oaddr = d->culled_objects[start++];
        const luxgi_surface_object& ob = d->objects[oaddr];
        V3<R> bc{R(ob.object_bounds[0]), R(ob.object_bounds[1]), R(ob.object_bounds[2])};
        if (length(sub(bc, pos)) > R(ob.object_bounds[3])) continue;
        M4<R> w2l = inverse(load_m4<R>(ob.transform));
        V4<R> lp4 = mul_m4(w2l, V4<R>{pos.x, pos.y, pos.z, R(1)});
        V3<R> lp{lp4.x, lp4.y, lp4.z};
        V3<R> ext{R(ob.extends[0]) + thr, R(ob.extends[1]) + thr, R(ob.extends[2]) + thr};
        if (std::fabs(lp.x) > ext.x || std::fabs(lp.y) > ext.y || std::fabs(lp.z) > ext.z) continue;
        V3<R> ln = normalize(mul_m3of4(w2l, wn));
        for (int i = 0; i < 6; ++i) {
            uint32_t to = ob.tile_offset[i];
            if (to != 0) sample_tile(S, d->tiles[to], lp, ln, thr, acc0, acc1, accw);
        }
    }
    R den = std::max(accw, R(0.0001f));
    out0 = V3<R>{acc0.x / den, acc0.y / den, acc0.z / den};
    out1 = V3<R>{acc1.x / den, acc1.y / den, acc1.z / den};
    return accw;
}

// ------------------------------------------------ sampleIrradiance
struct Atlases {
    Tex2 irr, dist;
};
// sampleIrradiance (DDGICommon.glsl:163-233)
template <typename R> V3<R> sample_irradiance(const luxgi_ddgi_uniform& u, const Atlases& A, V3<R> P, V3<R> N, V3<R> Wo) {
    V3<R> start{R(u.start_position[0]), R(u.start_position[1]), R(u.start_position[2])};
    V3<R> stp{R(u.step[0]), R(u.step[1]), R(u.step[2])};
    int cnt[3] = {u.probe_counts[0], u.probe_counts[1], u.probe_counts[2]};
    V3<R> rel{(P.x - start.x) / stp.x, (P.y - start.y) / stp.y, (P.z - start.z) / stp.z};
    int base[3] = {int(rel.x), int(rel.y), int(rel.z)};
    for (int k = 0; k < 3; ++k) base[k] = std::min(std::max(base[k], 0), cnt[k] - 1);
    V3<R> bpos{stp.x * R(base[0]) + start.x, stp.y * R(base[1]) + start.y, stp.z * R(base[2]) + start.z};
    V3<R> alpha{clampr((P.x - bpos.x) / stp.x, R(0), R(1)), clampr((P.y - bpos.y) / stp.y, R(0), R(1)),
                clampr((P.z - bpos.z) / stp.z, R(0), R(1))};
    V3<R> sum{R(0), R(0), R(0)};
    R sumw = R(0);
    for (int i = 0; i < 8; ++i) {
        int off[3] = {i & 1, (i >> 1) & 1, (i >> 2) & 1};
        int g[3];
        for (int k = 0; k < 3; ++k) g[k] = std::min(std::max(base[k] + off[k], 0), cnt[k] - 1);
        V3<R> ppos{stp.x * R(g[0]) + start.x, stp.y * R(g[1]) + start.y, stp.z * R(g[2]) + start.z};
        V3<R> tri{off[0] ? alpha.x : R(1) - alpha.x, off[1] ? alpha.y : R(1) - alpha.y, off[2] ? alpha.z : R(1) - alpha.z};
        R weight = R(1);
        V3<R> dtp = normalize(sub(ppos, P));
        R bf = std::max(R(0.0001f), (dot(dtp, N) + R(1)) * R(0.5));
        weight = weight * (bf * bf + R(0.2f));
        int pidx = g[0] + g[1] * cnt[0] + g[2] * cnt[0] * cnt[1];
        V3<R> vb = mul(add(N, mul(Wo, R(3))), R(u.normal_bias));
        V3<R> ptp = add(sub(P, ppos), vb);
        V3<R> dir = normalize(mul(ptp, R(-1)));
        V2<R> tc = tex_coord_from_dir(mul(dir, R(-1)), pidx, u.depth_width, u.depth_height, u.depth_probe_side);
        R dist = length(ptp);
        R mean = bilinear_repeat(A.dist, tc, 0);
        R mean2 = bilinear_repeat(A.dist, tc, 1);
        R variance = std::fabs(mean * mean - mean2);
        R dm = std::max(dist - mean, R(0));
        R cheb = variance / (variance + dm * dm);
        cheb = std::max(cheb * cheb * cheb, R(0));
        weight = weight * ((dist <= mean) ? R(1) : cheb);
        weight = std::max(R(0.000001f), weight);
        tc = tex_coord_from_dir(normalize(N), pidx, u.irradiance_width, u.irradiance_height, u.irradiance_probe_side);
        R ge = R(u.ddgi_gamma) * R(0.5);
        V3<R> pir{std::pow(bilinear_repeat(A.irr, tc, 0), ge), std::pow(bilinear_repeat(A.irr, tc, 1), ge),
                  std::pow(bilinear_repeat(A.irr, tc, 2), ge)};
        const R crush = R(0.2f);
        if (weight < crush) weight = weight * (weight * weight * (R(1) / (crush * crush)));
        weight = weight * (tri.x * tri.y * tri.z);
        sum = add(sum, mul(pir, weight));
        sumw = sumw + weight;
    }
    V3<R> net{sum.x / sumw, sum.y / sumw, sum.z / sumw};
    net = mulv(net, net);
    return mul(net, R(2) * pi_r<R>());
}

// ------------------------------------------------ probe location
template <typename R> V3<R> probe_location(const luxgi_ddgi_uniform& u, int index) {
    int X = u.probe_counts[0], Y = u.probe_counts[1];
    int gx = index % X, gy = (index % (X * Y)) / X, gz = index / (X * Y);
    return {R(u.step[0]) * R(gx) + R(u.start_position[0]), R(u.step[1]) * R(gy) + R(u.start_position[1]),
            R(u.step[2]) * R(gz) + R(u.start_position[2])};
}

template <typename R> V3<R> ray_direction(const float rot[9], int r, int nrays) {
    V3<R> f = spherical_fibonacci<R>(R(r), R(nrays));
    // mat3(randomOrientation) * f, column-major
    V3<R> m{R(rot[0]) * f.x + R(rot[3]) * f.y + R(rot[6]) * f.z,
            R(rot[1]) * f.x + R(rot[4]) * f.y + R(rot[7]) * f.z,
            R(rot[2]) * f.x + R(rot[5]) * f.y + R(rot[8]) * f.z};
    return normalize(m);
}

struct TraceCtx {
    const luxgi_ddgi_volume_desc* vd;
    const luxgi_sdf_desc* sdf;
    const luxgi_surface_desc* surf;
    Vol tex, mip;
    Surface S;
    Atlases prev;
    bool bounce;   // infinite bounce active this frame (mode B)
};

// GISDFRays.comp main (GISDFRays.comp:63-128) for one (probe, ray).
// out: rgb radiance, distance; info: steps, hit cascade (-1 = miss).
template <typename R> void trace_one(const TraceCtx& c, const float rot[9], int probe, int ray, float out[4], int32_t info[4]) {
    const luxgi_ddgi_uniform& u = c.vd->uniform;
    const luxgi_sdf_data& sd = c.sdf->data;
    const R WORLD = R(60000.0f);
    V3<R> origin = probe_location<R>(u, probe);
    V3<R> dir = ray_direction<R>(rot, ray, u.rays_per_probe);
    Hit<R> hit = trace_sdf<R>(sd, c.tex, c.mip, origin, dir, WORLD, c.vd->max_steps);
    V3<R> rad{R(0), R(0), R(0)};
    R dist;
    info[0] = hit.steps;
    info[1] = -1;
    info[2] = hit.fine;
    info[3] = 0;
    if (hit.time >= R(0)) {
        info[1] = hit.cascade;
        if (hit.sdf <= R(0) && hit.time <= R(sd.cascade_voxel_size[0])) {
            dist = WORLD;
        } else {
            V3<R> hp = add(origin, mul(dir, hit.time));
            R thr = R(sd.cascade_voxel_size[hit.cascade]) * R(1.05f);
            V3<R> s0, s1;
            sample_surface(c.S, hp, hit.normal, thr, s0, s1);
            if (c.vd->light_mode == LUXGI_LIGHT_PER_HIT) {
                rad = s0;
                if (c.bounce) {
                    // intensity * albedo / pi * E (Raytraced/Lighting.glsl:79-84, with the
                    // volume intensity SDFAtlasIndirectLight.frag:47 applies)
                    V3<R> e = sample_irradiance<R>(u, c.prev, hp, hit.normal, mul(dir, R(-1)));
                    V3<R> diff{s1.x / pi_r<R>(), s1.y / pi_r<R>(), s1.z / pi_r<R>()};
                    rad = add(rad, mulv(mul(diff, R(c.vd->intensity)), e));
                }
            } else {
                rad = s0;
            }
            dist = std::max(hit.time + R(sd.cascade_voxel_size[hit.cascade]) * R(0.5), R(0));
        }
    } else {
        rad = V3<R>{R(c.vd->sky_radiance[0]), R(c.vd->sky_radiance[1]), R(c.vd->sky_radiance[2])};
        dist = WORLD;
    }
    out[0] = float(rad.x); out[1] = float(rad.y); out[2] = float(rad.z); out[3] = float(dist);
    if (c.vd->storage == LUXGI_STORAGE_FP16)
        for (int k = 0; k < 4; ++k) out[k] = round_half(out[k]);
}

// ------------------------------------------------ ProbeUpdate.glsl
// One probe of the irradiance or distance blend (ProbeUpdate.glsl:66-152).
// dirs: float4 [R] (already storage-rounded), rays: float4 [P][R].
template <typename R> void blend_probe(const luxgi_ddgi_volume_desc* vd, const float* dirs, const float* rays,
                                       const float* prev, float* out, int probe, bool depth, bool first, int p0) {
    const luxgi_ddgi_uniform& u = vd->uniform;
    const int n = depth ? u.depth_probe_side : u.irradiance_probe_side;
    const int W = depth ? u.depth_width : u.irradiance_width;
    const int nc = depth ? 2 : 4;
    const int XY = u.probe_counts[0] * u.probe_counts[1];
    const int cx = probe % XY, cy = probe / XY;
    const int Rn = u.rays_per_probe;
    const R FLT_EPS = R(0.00000001f);
    for (int ty = 0; ty < n; ++ty) {
        for (int tx = 0; tx < n; ++tx) {
            V3<R> td = oct_decode(normalized_oct_coord<R>(tx, ty, n));
            R res[3] = {R(0), R(0), R(0)};
            R tw = R(0);
            for (int r = 0; r < Rn; ++r) {
                const float* dd = dirs + 4 * r;
                const float* ry = rays + (size_t(probe - p0) * Rn + r) * 4;
                V3<R> rd{R(dd[0]), R(dd[1]), R(dd[2])};
                R cosv = std::max(R(0), dot(td, rd));
                if (depth) {
                    R d = std::min(R(u.max_distance), R(ry[3]) - R(0.01f));
                    if (d == R(-1)) d = R(u.max_distance);
                    R w = std::pow(cosv, R(u.sharpness));
                    if (w >= FLT_EPS) {
                        res[0] = res[0] + d * w;
                        res[1] = res[1] + (d * d) * w;
                        tw = tw + w;
                    }
                } else {
                    R w = cosv;
                    if (w >= FLT_EPS) {
                        res[0] = res[0] + R(ry[0]) * w;
                        res[1] = res[1] + R(ry[1]) * w;
                        res[2] = res[2] + R(ry[2]) * w;
                        tw = tw + w;
                    }
                }
            }
            if (tw > FLT_EPS) {
                R s = R(1) / (R(2) * tw);
                for (int k = 0; k < 3; ++k) res[k] = res[k] * s;
            }
            if (!depth) {
                R ig = R(1) / R(u.ddgi_gamma);
                for (int k = 0; k < 3; ++k) res[k] = std::pow(res[k], ig);
            }
            const int x = cx * (n + 2) + tx + 2, y = cy * (n + 2) + ty + 2;
            const size_t ti = (size_t(y) * size_t(W) + size_t(x)) * size_t(nc);
            R h = R(u.hysteresis);
            int nch = depth ? 2 : 3;
            for (int k = 0; k < nch; ++k) {
                R v = res[k];
                if (!first) v = mixr(v, R(prev[ti + size_t(k)]), h);
                float f = float(v);
                if (vd->storage == LUXGI_STORAGE_FP16) f = round_half(f);
                out[ti + size_t(k)] = f;
            }
            if (!depth) out[ti + 3] = 1.0f;
        }
    }
}

// BorderUpdate.glsl:136-156 for side n, generalised from its 36/68-entry
// offset tables: (dst, src) pairs relative to the cell origin.
int border_pairs(int n, int (*pairs)[4]) {
    int k = 0;
    for (int x = 1; x <= n; ++x) { pairs[k][0] = x; pairs[k][1] = 0; pairs[k][2] = n + 1 - x; pairs[k][3] = 1; ++k; }
    for (int x = 1; x <= n; ++x) { pairs[k][0] = x; pairs[k][1] = n + 1; pairs[k][2] = n + 1 - x; pairs[k][3] = n; ++k; }
    for (int y = 1; y <= n; ++y) { pairs[k][0] = 0; pairs[k][1] = y; pairs[k][2] = 1; pairs[k][3] = n + 1 - y; ++k; }
    for (int y = 1; y <= n; ++y) { pairs[k][0] = n + 1; pairs[k][1] = y; pairs[k][2] = n; pairs[k][3] = n + 1 - y; ++k; }
    int corners[4][4] = {{0, 0, n, n}, {n + 1, 0, 1, n}, {0, n + 1, n, 1}, {n + 1, n + 1, 1, 1}};
    for (auto& c : corners) { for (int q = 0; q < 4; ++q) pairs[k][q] = c[q]; ++k; }
    return k;
}

void border_atlas(float* atlas, int W, int nc, int n, int cells_x, int cells_y) {
    std::vector<int> buf(size_t(4 * (4 * n + 4)));
    int (*pairs)[4] = reinterpret_cast<int (*)[4]>(buf.data());
    int np = border_pairs(n, pairs);
#pragma omp parallel for
    for (int cy = 0; cy < cells_y; ++cy) {
        for (int cx = 0; cx < cells_x; ++cx) {
            int ox = cx * (n + 2) + 1, oy = cy * (n + 2) + 1;
            for (int i = 0; i < np; ++i) {
                size_t dst = (size_t(oy + pairs[i][1]) * size_t(W) + size_t(ox + pairs[i][0])) * size_t(nc);
                size_t src = (size_t(oy + pairs[i][3]) * size_t(W) + size_t(ox + pairs[i][2])) * size_t(nc);
                for (int c = 0; c < nc; ++c) atlas[dst + size_t(c)] = atlas[src + size_t(c)];
            }
        }
    }
}

// GlobalSDFMipmap.comp sampleSDF/main (GlobalSDFMipmap.comp:32-67) and
// combineDistanceToSDF (SDFCommon.glsl:18-36).
inline float combine(float sdf, float dist) {
    if (sdf <= 0.0f && dist <= 0.0f) return sdf;
    float m = std::max(sdf, 0.0f);
    return std::sqrt(m * m + dist * dist);
}

void mip_pass(const std::vector<float>& src, int src_w, int src_res, int src_off_x, std::vector<float>& dst, int dst_w,
              int dst_off_x, int mres, int coord_scale, float max_dist, bool fp16) {
    static const int off[7][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
#pragma omp parallel for
    for (int z = 0; z < mres; ++z)
        for (int y = 0; y < mres; ++y)
            for (int x = 0; x < mres; ++x) {
                float mn = 0.0f;
                for (int i = 0; i < 7; ++i) {
                    int c[3] = {x * coord_scale + off[i][0], y * coord_scale + off[i][1], z * coord_scale + off[i][2]};
                    for (int k = 0; k < 3; ++k) c[k] = std::min(std::max(c[k], 0), src_res - 1);
                    c[0] += src_off_x;
                    float v = src[size_t(c[0]) + size_t(src_w) * (size_t(c[1]) + size_t(src_res) * size_t(c[2]))];
                    float len = std::sqrt(float(off[i][0] * off[i][0] + off[i][1] * off[i][1] + off[i][2] * off[i][2]));
                    float dv = len * (max_dist / float(src_res));
                    float r = combine(v, dv);
                    mn = (i == 0) ? r : std::min(mn, r);
                }
                if (fp16) mn = round_half(mn);
                dst[size_t(x + dst_off_x) + size_t(dst_w) * (size_t(y) + size_t(mres) * size_t(z))] = mn;
            }
}

// ------------------------------------------------ surface-cache raster passes
// The tile quads of addTiles2 (Engine/DDGI/GlobalSurfaceAtlas.cpp:554-574)
// cover the pixels [x, x + w] x [y, y + h], (x, y, w, h) = round(extends *
// res): the TileBuffer extends hold the tile size less one texel of padding
// (:272-279) while the quad spans the whole tile.  The fragment at pixel
// (x + i, y + j) has inTileUV = ((i + 0.5) / (w + 1), (j + 0.5) / (h + 1))
// and samples the surface textures at atlasUV = inTileUV * extends.zw +
// extends.xy (SDFDeferredLight.frag:82, SDFAtlasIndirectLight.frag:55,
// CopyEmissive.frag:25) with their default LINEAR + REPEAT sampler
// (RHI/Definitions.h:152-159).
struct Footprint {
    int x0, y0, w, h;   // w, h: pixels of the quad
};
inline Footprint footprint(const luxgi_surface_tile& tl, int res) {
    Footprint f;
    f.x0 = int(std::lround(tl.extends[0] * float(res)));
    f.y0 = int(std::lround(tl.extends[1] * float(res)));
    f.w = int(std::lround(tl.extends[2] * float(res))) + 1;
    f.h = int(std::lround(tl.extends[3] * float(res))) + 1;
    return f;
}
template <typename R> V2<R> fragment_uv(const luxgi_surface_tile& tl, const Footprint& f, int i, int j) {
    const R tu = (R(i) + R(0.5)) / R(f.w), tv = (R(j) + R(0.5)) / R(f.h);
    return {tu * R(tl.extends[2]) + R(tl.extends[0]), tv * R(tl.extends[3]) + R(tl.extends[1])};
}

// The surface G-buffer at a fragment: albedo, world position and normal
// (SDFDeferredLight.frag:83-87), metallic and roughness (:120-121; no PBR
// texture reads as metallic 0, roughness 1).
template <typename R> struct SurfaceFragment {
    V3<R> albedo, pos, normal;
    R metallic, roughness;
};
struct SurfaceTextures {
    Tex2 g0, g1, pbr, emissive;
    bool has_pbr = false, has_emissive = false;
    explicit SurfaceTextures(const luxgi_surface_desc* s) {
        const int res = int(s->data.resolution);
        g0.set_gbuffer(s->gbuffer0, s->gbuffer_format); g0.W = res; g0.H = res;
        g1.set_gbuffer(s->gbuffer1, s->gbuffer_format); g1.W = res; g1.H = res;
        pbr.u8 = s->pbr; pbr.W = res; pbr.H = res; pbr.C = 4;
        emissive.set_color(s->emissive, s->light_format); emissive.W = res; emissive.H = res;
        has_pbr = s->pbr != nullptr;
        has_emissive = s->emissive != nullptr;
    }
};
template <typename R> SurfaceFragment<R> surface_fragment(const SurfaceTextures& T, V2<R> uv) {
    SurfaceFragment<R> f;
    f.albedo = {bilinear_repeat(T.g0, uv, 0), bilinear_repeat(T.g0, uv, 1), bilinear_repeat(T.g0, uv, 2)};
    const R wx = bilinear_repeat(T.g0, uv, 3);
    const V2<R> oct{bilinear_repeat(T.g1, uv, 0), bilinear_repeat(T.g1, uv, 1)};
    f.pos = {wx, bilinear_repeat(T.g1, uv, 2), bilinear_repeat(T.g1, uv, 3)};
    f.normal = oct_decode(oct);                  // octohedralToDirection, Math.glsl:26-32
    f.metallic = T.has_pbr ? bilinear_repeat(T.pbr, uv, 0) : R(0);
    f.roughness = T.has_pbr ? bilinear_repeat(T.pbr, uv, 1) : R(1);
    return f;
}

inline uint16_t f2h_bits(float v) {
    _Float16 h = _Float16(v);
    uint16_t b;
    std::memcpy(&b, &h, 2);
    return b;
}

// Stores rgba rounded to a surface colour format (alpha dropped for
// R11G11B10F).
inline void color_store(void* p, int fmt, size_t texel, const float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        static_cast<uint32_t*>(p)[texel] = pack_r11g11b10(v);
    } else {
        for (int c = 0; c < 4; ++c) static_cast<uint16_t*>(p)[texel * 4 + size_t(c)] = f2h_bits(v[c]);
    }
}

// Raytraced/BRDF.glsl:14-41 and :65-81 (Cook-Torrance: GGX distribution,
// Schlick-GGX geometry with k = (r + 1)^2 / 8, Schlick Fresnel).
template <typename R> R ndf_ggx(R cos_lh, R roughness) {
    const R alpha = roughness * roughness;
    const R alpha_sq = alpha * alpha;
    const R denom = (cos_lh * cos_lh) * (alpha_sq - R(1)) + R(1);
    return alpha_sq / (pi_r<R>() * denom * denom);
}
template <typename R> R ga_schlick_g1(R cos_theta, R k) { return cos_theta / (cos_theta * (R(1) - k) + k); }
template <typename R> R ga_schlick_ggx(R cos_li, R n_dot_v, R roughness) {
    const R r = roughness + R(1);
    const R k = (r * r) / R(8);
    return ga_schlick_g1(cos_li, k) * ga_schlick_g1(n_dot_v, k);
}
template <typename R> V3<R> brdf(V3<R> albedo, V3<R> n, R roughness, R metallic, V3<R> view, V3<R> half_v, V3<R> l) {
    const V3<R> f0{mixr(R(0.04f), albedo.x, metallic), mixr(R(0.04f), albedo.y, metallic),
                   mixr(R(0.04f), albedo.z, metallic)};
    const R cos_li = std::max(R(0), dot(n, l));
    const R cos_lh = std::max(R(0), dot(n, half_v));
    const R n_dot_v = std::max(R(0), dot(n, view));
    const R fw = std::pow(clampr(R(1) - std::max(dot(half_v, view), R(0)), R(0), R(1)), R(5));
    const V3<R> F{f0.x + (R(1) - f0.x) * fw, f0.y + (R(1) - f0.y) * fw, f0.z + (R(1) - f0.z) * fw};
    const R D = ndf_ggx(cos_lh, roughness);
    const R G = ga_schlick_ggx(cos_li, n_dot_v, roughness);
    const R den = std::max(R(0.00001f), R(4) * cos_li * n_dot_v);
    const R km = R(1) - metallic;
    const R Fv[3] = {F.x, F.y, F.z}, av[3] = {albedo.x, albedo.y, albedo.z};
    R out[3];
    for (int c = 0; c < 3; ++c) {
        const R kd = (R(1) - Fv[c]) * km;
        const R diffuse = kd * av[c] / pi_r<R>();
        const R specular = (Fv[c] * D * G) / den;
        out[c] = diffuse + specular;
    }
    return {out[0], out[1], out[2]};
}

// fetchLight (SDFDeferredLight.frag:41-76): direction to the light, trace
// distance and attenuation.  Types other than directional, spot and point
// leave the outputs unset in the shader; the entry point rejects them.
template <typename R> void fetch_light(const luxgi_light& L, V3<R> wp, V3<R>& wi, R& tmax, R& atten) {
    const R WORLD = R(60000.0f);
    if (L.type == 0.0f) {
        wi = {-R(L.direction[0]), -R(L.direction[1]), -R(L.direction[2])};
        tmax = WORLD;
        atten = R(1);
    } else if (L.type == 2.0f) {
        const V3<R> d = sub(V3<R>{R(L.position[0]), R(L.position[1]), R(L.position[2])}, wp);
        const R dist = length(d);
        wi = normalize(d);
        atten = R(L.radius) / (std::pow(dist, R(2)) + R(1));
        tmax = dist;
    } else {
        const V3<R> lv = sub(V3<R>{R(L.position[0]), R(L.position[1]), R(L.position[2])}, wp);
        const R cutoff = R(1) - R(L.angle);
        wi = normalize(lv);
        const R dist = length(lv);
        const R theta = dot(wi, V3<R>{R(L.direction[0]), R(L.direction[1]), R(L.direction[2])});
        const R eps = cutoff - cutoff * R(0.9f);
        R a = (theta - cutoff) / eps;
        a = a * (R(L.radius) / (std::pow(dist, R(2)) + R(1)));
        atten = clampr(a, R(0), R(1));
        tmax = dist;
    }
}

// SDFDeferredLight.frag:79-129 for one fragment and one light: the light's
// contribution (rgb) to the light cache.  `shadowed` reports the SDF shadow.
template <typename R> V3<R> direct_light(const luxgi_sdf_desc* sdf, const Vol& tex, const Vol& mip,
                                         const SurfaceFragment<R>& f, const luxgi_light& L, const float cam[3],
                                         float shadow_bias, int max_steps, bool* shadowed) {
    V3<R> wi{R(0), R(0), R(0)};
    R dist = R(60000.0f), atten = R(1);
    fetch_light<R>(L, f.pos, wi, dist, atten);
    R shadow = R(1);
    const R sb = R(shadow_bias);
    const R nol = dot(f.normal, wi);
    const R bias = R(2) * sb * clampr(R(1) - nol, R(0), R(1)) + sb;
    if (nol > R(0)) {
        if (atten > R(0)) {
            const V3<R> origin = add(f.pos, mul(f.normal, sb));
            const Hit<R> hit = trace_sdf<R>(sdf->data, tex, mip, origin, wi, dist - bias, max_steps, R(2), false);
            shadow = hit.time >= R(0) ? R(0) : R(1);
        }
    } else {
        shadow = R(0);
    }
    *shadowed = shadow == R(0);
    const V3<R> c{R(cam[0]), R(cam[1]), R(cam[2])};
    const V3<R> view = normalize(sub(c, f.pos));
    const R intensity = std::pow(R(L.intensity), R(1.4f)) + R(0.1f);
    const V3<R> lrad{R(L.color[0]) * intensity, R(L.color[1]) * intensity, R(L.color[2]) * intensity};
    const V3<R> lh = normalize(add(wi, view));
    const R cos_li = std::max(R(0), dot(f.normal, wi));
    const V3<R> b = brdf<R>(f.albedo, f.normal, f.roughness, f.metallic, view, lh, wi);
    const R s = cos_li * shadow * atten;
    return {b.x * lrad.x * s, b.y * lrad.y * s, b.z * lrad.z * s};
}

// ------------------------------------------------ global SDF from objects
// merge_sdf::system (Engine/DDGI/GlobalDistanceField.cpp:576-842, first
// build), chunkCalculate (:465-535), getChunkId (:193-210), the cascade
// placement (:592-626), SDFRasterizeModel.glsl:42-63 and distanceToModelSDF
// (SDFCommon.glsl:38-62).  FP32 with glm's association of matrix-vector
// products; matrices column-major.
namespace sdfb {

struct Mat {
    float m[16];
};
struct Vec4 {
    float x, y, z, w;
};

inline Vec4 mv(const Mat& M, float x, float y, float z, float w) {
    const float* m = M.m;
    return {(m[0] * x + m[4] * y) + (m[8] * z + m[12] * w), (m[1] * x + m[5] * y) + (m[9] * z + m[13] * w),
            (m[2] * x + m[6] * y) + (m[10] * z + m[14] * w), (m[3] * x + m[7] * y) + (m[11] * z + m[15] * w)};
}
inline Mat mm(const Mat& A, const Mat& B) {
    Mat r;
    for (int c = 0; c < 4; ++c) {
        Vec4 v = mv(A, B.m[c * 4], B.m[c * 4 + 1], B.m[c * 4 + 2], B.m[c * 4 + 3]);
        r.m[c * 4] = v.x; r.m[c * 4 + 1] = v.y; r.m[c * 4 + 2] = v.z; r.m[c * 4 + 3] = v.w;
    }
    return r;
}
inline Mat inv(const Mat& A) {
    M4<float> a;
    std::memcpy(a.m, A.m, sizeof(a.m));
    M4<float> b = inverse(a);
    Mat r;
    std::memcpy(r.m, b.m, sizeof(r.m));
    return r;
}
inline float fmin_g(float a, float b) { return b < a ? b : a; }   // GLSL / glm min
inline float fmax_g(float a, float b) { return a < b ? b : a; }

constexpr float kScales[4] = {1.0f, 2.5f, 5.0f, 10.0f};

struct Cascade {
    float center[3], distance, voxel;
};

// cascade placement: a fixed view point on +z from math::lineHitsAABB of the
// segment 0 -> FORWARD * 2 c0 against [-c0, c0]^3, snapped to the chunk grid
inline Cascade cascade(const luxgi_sdf_build_desc& d, int c) {
    const float dist = fmin_g(15000.0f, d.gi_distance) * d.global_scale;
    const float extent = dist / kScales[d.cascades - 1];
    const float c0 = extent * kScales[0];
    const float inv_z = 1.0f / ((0.0f + 1.0f * (c0 * 2.0f)) - 0.0f);
    const float inf = INFINITY;
    const float ex_x = (c0 - 0.0f) * inf, en_x = (-c0 - 0.0f) * inf;
    const float ex_z = (c0 - 0.0f) * inv_z, en_z = (-c0 - 0.0f) * inv_z;
    const float far = fmin_g(fmax_g(en_x, ex_x), fmin_g(fmax_g(en_x, ex_x), fmax_g(en_z, ex_z)));
    const float y = fmin_g(fmax_g(far, 0.0f), 1.0f);
    const float offset = y * c0 * 0.6f;
    const float view[3] = {0.0f * offset, 0.0f * offset, 0.0f + 1.0f * offset};
    Cascade k;
    k.distance = extent * kScales[c];
    k.voxel = (k.distance * 2.0f) / float(d.resolution);
    const float chunk = k.voxel * 32.0f;
    for (int i = 0; i < 3; ++i) k.center[i] = std::floor(view[i] / chunk) * chunk;
    return k;
}

struct Plan {
    std::vector<luxgi_sdf_raster_object> recs;
    std::vector<int> mesh;
    std::vector<luxgi_sdf_chunk> chunks;
};

inline int plan(const luxgi_sdf_build_desc& d, const luxgi_mesh_sdf* meshes, int nm, const luxgi_sdf_object* objs,
                int no, int c, Plan& P) {
    const Cascade K = cascade(d, c);
    float bmin[3], bmax[3];
    for (int i = 0; i < 3; ++i) {
        bmin[i] = K.center[i] - K.distance;
        bmax[i] = K.center[i] + K.distance;
    }
    const float min_radius = d.min_object_radius * d.global_scale;
    std::map<std::array<int, 3>, size_t> table;
    for (int o = 0; o < no; ++o) {
        const int mi = objs[o].mesh;
        if (mi < 0 || mi >= nm) return LUXGI_EINVAL;
        const luxgi_mesh_sdf& m = meshes[mi];
        Mat W;
        std::memcpy(W.m, objs[o].world, sizeof(W.m));
        // sdf.aabb.transform(world) (Math/BoundingBox.cpp:10-22)
        const float cen[3] = {(m.aabb_max[0] + m.aabb_min[0]) * 0.5f, (m.aabb_max[1] + m.aabb_min[1]) * 0.5f,
                              (m.aabb_max[2] + m.aabb_min[2]) * 0.5f};
        const Vec4 nc = mv(W, cen[0], cen[1], cen[2], 1.0f);
        const float oe[3] = {(m.aabb_max[0] - m.aabb_min[0]) * 0.5f, (m.aabb_max[1] - m.aabb_min[1]) * 0.5f,
                             (m.aabb_max[2] - m.aabb_min[2]) * 0.5f};
        const float* w = W.m;
        float ne[3];
        for (int r = 0; r < 3; ++r)
            ne[r] = std::fabs(w[r]) * oe[0] + std::fabs(w[4 + r]) * oe[1] + std::fabs(w[8 + r] * oe[2]);
        const float ncv[3] = {nc.x, nc.y, nc.z};
        float omin[3], omax[3];
        for (int i = 0; i < 3; ++i) {
            omin[i] = ncv[i] - ne[i];
            omax[i] = ncv[i] + ne[i];
        }
        // BoundingSphere(box), BoundingBox::intersectsWithSphere
        float sc[3], q[3], dd[3];
        for (int i = 0; i < 3; ++i) {
            sc[i] = (omax[i] + omin[i]) * 0.5f;
            dd[i] = omax[i] - omin[i];
        }
        const float radius = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) / 2.0f;
        for (int i = 0; i < 3; ++i) q[i] = sc[i] - fmin_g(fmax_g(sc[i], bmin[i]), bmax[i]);
        const float d2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        if (!(d2 <= radius * radius && radius >= min_radius)) continue;
        // getChunkId, unclamped as in the reference
        const float margin = K.voxel * 4.0f, chunk = K.voxel * 32.0f;
        int cmin[3], cmax[3];
        for (int i = 0; i < 3; ++i) {
            const float base = bmin[i] + 0.1f;
            cmin[i] = int(((omin[i] - margin) - base) / chunk);
            cmax[i] = int(((omax[i] + margin) - base) / chunk);
        }
        // ObjectRasterizeData
        Mat T;
        for (int i = 0; i < 16; ++i) T.m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
        T.m[12] = -cen[0];
        T.m[13] = -cen[1];
        T.m[14] = -cen[2];
        const Mat w2v = mm(inv(W), T);
        const Mat v2w = inv(w2v);
        luxgi_sdf_raster_object r{};
        std::memcpy(r.world_to_volume, w2v.m, sizeof(w2v.m));
        std::memcpy(r.volume_to_world, v2w.m, sizeof(v2w.m));
        for (int i = 0; i < 3; ++i) {
            r.volume_to_uvw_mul[i] = m.local_to_uvw_mul[i];
            r.volume_to_uvw_add[i] = m.local_to_uvw_add[i] + cen[i] * m.local_to_uvw_mul[i];
            r.volume_local_bounds_extent[i] = (m.aabb_max[i] - m.aabb_min[i]) / 2.0f;
        }
        r.mip_offset = float(std::min(c, 2));
        r.decode_mul = m.max_distance;
        r.decode_add = -m.max_distance;
        const uint32_t id = uint32_t(P.recs.size());
        P.recs.push_back(r);
        P.mesh.push_back(mi);
        for (int z = cmin[2]; z <= cmax[2]; ++z)
            for (int y = cmin[1]; y <= cmax[1]; ++y)
                for (int x = cmin[0]; x <= cmax[0]; ++x) {
                    auto it = table.find({x, y, z});
                    if (it == table.end()) {
                        luxgi_sdf_chunk ck{};
                        ck.coord[0] = x; ck.coord[1] = y; ck.coord[2] = z;
                        it = table.emplace(std::array<int, 3>{x, y, z}, P.chunks.size()).first;
                        P.chunks.push_back(ck);
                    }
                    luxgi_sdf_chunk& ck = P.chunks[it->second];
                    // a full layer-0 entry is overwritten by the (empty) next
                    // layer before the object is appended (:516-523)
                    if (ck.count == 28) ck.count = 0;
                    ck.models[ck.count++] = id;
                }
    }
    return 0;
}

// textureLod on a mesh SDF level: trilinear, REPEAT
inline float sample_level(const uint16_t* v, int W, int H, int D, float u, float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    const float a = x - fx, b = y - fy, c = z - fz;
    auto wr = [](int i, int n) { int r = i % n; return r < 0 ? r + n : r; };
    const int x0 = wr(int(fx), W), x1 = wr(int(fx) + 1, W), y0 = wr(int(fy), H), y1 = wr(int(fy) + 1, H);
    const int z0 = wr(int(fz), D), z1 = wr(int(fz) + 1, D);
    auto at = [&](int i, int j, int k) { return h2f(v[size_t(i) + size_t(W) * (size_t(j) + size_t(H) * size_t(k))]); };
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = at(x0, y0, z0) * ia + at(x1, y0, z0) * a, c10 = at(x0, y1, z0) * ia + at(x1, y1, z0) * a;
    const float c01 = at(x0, y0, z1) * ia + at(x1, y0, z1) * a, c11 = at(x0, y1, z1) * ia + at(x1, y1, z1) * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

inline void xf(const float* m, const float p[3], float o[3]) {
    o[0] = (m[0] * p[0] + m[4] * p[1]) + (m[8] * p[2] + m[12]);
    o[1] = (m[1] * p[0] + m[5] * p[1]) + (m[9] * p[2] + m[13]);
    o[2] = (m[2] * p[0] + m[6] * p[1]) + (m[10] * p[2] + m[14]);
}

// distanceToModelSDF (SDFCommon.glsl:38-62)
inline float distance_to_model(float min_distance, const luxgi_sdf_raster_object& r, const uint16_t* vol, int W,
                               int H, int D, const float wp[3]) {
    float vp[3], uvw[3], vc[3], wc[3];
    xf(r.world_to_volume, wp, vp);
    for (int i = 0; i < 3; ++i) {
        uvw[i] = vp[i] * r.volume_to_uvw_mul[i] + r.volume_to_uvw_add[i];
        const float e = r.volume_local_bounds_extent[i];
        vc[i] = fmin_g(fmax_g(vp[i], -e), e);
    }
    xf(r.volume_to_world, vc, wc);
    const float q[3] = {wp[0] - wc[0], wp[1] - wc[1], wp[2] - wc[2]};
    float dtv = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    if (dtv < 0.01f) {
        const float s[3] = {vp[0] - vc[0], vp[1] - vc[1], vp[2] - vc[2]};
        dtv = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    }
    dtv = fmax_g(dtv, 0.0f);
    if (min_distance <= dtv) return dtv;
    const float vd = (sample_level(vol, W, H, D, uvw[0], uvw[1], uvw[2]) * 2.0f - 1.0f) * r.decode_mul;
    float result = combine(vd, dtv);
    if (dtv > 0.0f) result = fmax_g(dtv, result);
    return result;
}

}  // namespace sdfb

}  // namespace

// ===================================================================== C API
extern "C" {

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

// Rotated Fibonacci directions, float4 [R] (w = 0); storage rounding as the
// blend sees them when fp16_round != 0.
int oracle_ray_dirs(const float rot[9], int nrays, int precision, int fp16_round, float* out) {
    for (int r = 0; r < nrays; ++r) {
        float v[3];
        if (precision == 1) {
            V3<double> d = ray_direction<double>(rot, r, nrays);
            v[0] = float(d.x); v[1] = float(d.y); v[2] = float(d.z);
        } else {
            V3<float> d = ray_direction<float>(rot, r, nrays);
            v[0] = d.x; v[1] = d.y; v[2] = d.z;
        }
        for (int k = 0; k < 3; ++k) out[4 * r + k] = fp16_round ? round_half(v[k]) : v[k];
        out[4 * r + 3] = 0.0f;
    }
    return 0;
}

// Rotation of glm::angleAxis(angle, axis) cast to a matrix (DDGIRenderer.cpp:
// 267-272), column-major; the quaternion-to-matrix identity.
int oracle_rotation(const float axis[3], float angle, float out[9]) {
    double half = double(angle) * 0.5, s = std::sin(half);
    double x = axis[0] * s, y = axis[1] * s, z = axis[2] * s, w = std::cos(half);
    double m[9] = {1 - 2 * (y * y + z * z), 2 * (x * y + w * z), 2 * (x * z - w * y),
                   2 * (x * y - w * z), 1 - 2 * (x * x + z * z), 2 * (y * z + w * x),
                   2 * (x * z + w * y), 2 * (y * z - w * x), 1 - 2 * (x * x + y * y)};
    for (int i = 0; i < 9; ++i) out[i] = float(m[i]);
    return 0;
}

// The synthetic workloads' per-frame rotation, which replaces the
// reference's std::random_device draw (DDGIRenderer.cpp:267-272): a
// xoshiro256** stream (Blackman & Vigna) seeded through splitmix64 from
// seed ^ (0xD1B54A32D192ED03 * (frame + 1)); axis = normalize of three
// U(-1, 1) draws, angle = U(0, 1) * 2pi, each draw the top 24 bits of a
// 64-bit output; the matrix of the unit quaternion in FP32.  Restated so
// that a CPU-only run derives the same rotations as the library.
int oracle_frame_rotation(uint64_t seed, uint32_t frame, float out[9]) {
    uint64_t st = seed ^ (0xD1B54A32D192ED03ull * (uint64_t(frame) + 1ull));
    uint64_t s[4];
    for (uint64_t& w : s) {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        w = z ^ (z >> 31);
    }
    auto rol = [](uint64_t v, int k) { return (v << k) | (v >> (64 - k)); };
    auto draw = [&](float lo, float hi) {
        const uint64_t r = rol(s[1] * 5, 7) * 9, t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rol(s[3], 45);
        return lo + (hi - lo) * (float(r >> 40) * (1.0f / 16777216.0f));
    };
    float a[3];
    for (float& c : a) c = draw(-1.0f, 1.0f);
    const float n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    if (n > 0.0f) { a[0] /= n; a[1] /= n; a[2] /= n; } else { a[0] = 0.0f; a[1] = 0.0f; a[2] = 1.0f; }
    const float half = draw(0.0f, 1.0f) * 3.14159265f * 2.0f * 0.5f, sh = std::sin(half);
    const float qx = a[0] * sh, qy = a[1] * sh, qz = a[2] * sh, qw = std::cos(half);
    out[0] = 1.0f - 2.0f * (qy * qy + qz * qz); out[1] = 2.0f * (qx * qy + qw * qz); out[2] = 2.0f * (qx * qz - qw * qy);
    out[3] = 2.0f * (qx * qy - qw * qz); out[4] = 1.0f - 2.0f * (qx * qx + qz * qz); out[5] = 2.0f * (qy * qz + qw * qx);
    out[6] = 2.0f * (qx * qz + qw * qy); out[7] = 2.0f * (qy * qz - qw * qx); out[8] = 1.0f - 2.0f * (qx * qx + qy * qy);
    return 0;
}

// n texels of float rgba into a surface colour format (luxgi_color_format):
// RGBA16F (4 x u16) or R11G11B10F (u32), rounded as a render target would.
int oracle_pack_colors(const float* rgba, int64_t n, int fmt, void* out) {
    for (int64_t i = 0; i < n; ++i) color_store(out, fmt, size_t(i), rgba + 4 * i);
    return 0;
}
// n texels of a surface colour format back to float rgba (alpha 1 for
// R11G11B10F).
int oracle_unpack_colors(const void* in, int64_t n, int fmt, float* rgba) {
    for (int64_t i = 0; i < n; ++i) color_load(in, fmt, size_t(i), rgba + 4 * i);
    return 0;
}

// The FP32 march's sample points of n rays (probes[i], rays[i]) under
// `rot`: out [n][cap][4] = (u, v, w, full-resolution sampled) per step, -1
// past the end of a ray's march.  Analysis aid of the march's memory
// locality (which texels a group of rays reads at each step).
int oracle_march_trails(const luxgi_ddgi_volume_desc* vd, const luxgi_sdf_desc* sdf, const float rot[9],
                        const int32_t* probes, const int32_t* rays, int n, int cap, float* out) {
    const int res = sdf->resolution, mres = sdf->mip_resolution, C = int(sdf->data.cascades_count);
    Vol tex, mip;
    tex.W = res * C; tex.H = res; tex.D = res;
    mip.W = mres * C; mip.H = mres; mip.D = mres;
    if (sdf->format == LUXGI_STORAGE_FP16) {
        tex.f16 = static_cast<const uint16_t*>(sdf->sdf);
        mip.f16 = static_cast<const uint16_t*>(sdf->mip);
    } else {
        tex.f32 = static_cast<const float*>(sdf->sdf);
        mip.f32 = static_cast<const float*>(sdf->mip);
    }
    const luxgi_ddgi_uniform& u = vd->uniform;
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < n; ++i) {
        float* o = out + size_t(i) * cap * 4;
        for (int k = 0; k < cap * 4; ++k) o[k] = -1.0f;
        MarchTrail tr{o, cap, 0};
        const V3<float> origin = probe_location<float>(u, probes[i]);
        const V3<float> dir = ray_direction<float>(rot, rays[i], u.rays_per_probe);
        trace_sdf<float>(sdf->data, tex, mip, origin, dir, 60000.0f, vd->max_steps, 0.0f, false, &tr);
    }
    return 0;
}

// Atlas sizes of DDGIRenderer.cpp:182-185: a cell of side + 2 texels per
// probe, probes (x + y X) along the width and z along the height, plus a
// 1-texel pad around the whole atlas.
int oracle_derive_uniform(luxgi_ddgi_uniform* u) {
    const int XY = u->probe_counts[0] * u->probe_counts[1], Z = u->probe_counts[2];
    u->irradiance_width = (u->irradiance_probe_side + 2) * XY + 2;
    u->irradiance_height = (u->irradiance_probe_side + 2) * Z + 2;
    u->depth_width = (u->depth_probe_side + 2) * XY + 2;
    u->depth_height = (u->depth_probe_side + 2) * Z + 2;
    u->probe_counts[3] = 0;
    return 0;
}

// Trace probes [p0, p1): out float4 [P][R] (rgb, distance), info int4 [P][R]
// (steps, cascade, full-resolution samples, 0) or NULL.  sdf/surface descriptors hold HOST pointers;
// prev_irr / prev_dist are float atlases (mode B when frames > 0).
int oracle_trace(const luxgi_ddgi_volume_desc* vd, const luxgi_sdf_desc* sdf, const luxgi_surface_desc* surf,
                 const float* prev_irr, const float* prev_dist, int frames, const float rot[9], int precision,
                 int p0, int p1, float* out, int32_t* info) {
    const luxgi_ddgi_uniform& u = vd->uniform;
    TraceCtx c;
    c.vd = vd; c.sdf = sdf; c.surf = surf;
    const int res = sdf->resolution, mres = sdf->mip_resolution, C = int(sdf->data.cascades_count);
    c.tex.W = res * C; c.tex.H = res; c.tex.D = res;
    c.mip.W = mres * C; c.mip.H = mres; c.mip.D = mres;
    if (sdf->format == LUXGI_STORAGE_FP16) {
        c.tex.f16 = static_cast<const uint16_t*>(sdf->sdf);
        c.mip.f16 = static_cast<const uint16_t*>(sdf->mip);
    } else {
        c.tex.f32 = static_cast<const float*>(sdf->sdf);
        c.mip.f32 = static_cast<const float*>(sdf->mip);
    }
    const int ares = int(surf->data.resolution);
    c.S.d = surf;
    c.S.depth.f32 = surf->depth; c.S.depth.W = ares; c.S.depth.H = ares; c.S.depth.C = 1;
    if (vd->light_mode == LUXGI_LIGHT_PER_HIT) {
        c.S.c0.set_color(surf->direct_light, surf->light_format);
        c.S.c1.u8 = surf->albedo;
        c.S.c1.W = ares; c.S.c1.H = ares; c.S.c1.C = 4;
        c.S.two = true;
    } else {
        c.S.c0.set_color(surf->light_cache, surf->light_format);
    }
    c.S.c0.W = ares; c.S.c0.H = ares; c.S.c0.C = 4;
    c.prev.irr.f32 = prev_irr; c.prev.irr.W = u.irradiance_width; c.prev.irr.H = u.irradiance_height; c.prev.irr.C = 4;
    c.prev.dist.f32 = prev_dist; c.prev.dist.W = u.depth_width; c.prev.dist.H = u.depth_height; c.prev.dist.C = 2;
    c.bounce = vd->infinite_bounce && frames != 0 && prev_irr && prev_dist;
    const int Rn = u.rays_per_probe;
#pragma omp parallel for schedule(dynamic, 1)
    for (int p = p0; p < p1; ++p) {
        for (int r = 0; r < Rn; ++r) {
            size_t i = size_t(p - p0) * Rn + r;
            int32_t inf[4];
            if (precision == 1) trace_one<double>(c, rot, p, r, out + 4 * i, inf);
            else trace_one<float>(c, rot, p, r, out + 4 * i, inf);
            if (info) for (int k = 0; k < 4; ++k) info[4 * i + k] = inf[k];
        }
    }
    return 0;
}

// Irradiance + distance blend of probes [p0, p1) (ProbeUpdate.glsl; p1 <= 0
// means all) followed by the border copy of every cell when `border` != 0.
// rays holds probes [p0, p1).  Atlases are float arrays; prev may be NULL
// when first != 0.
int oracle_blend(const luxgi_ddgi_volume_desc* vd, const float* dirs, const float* rays, const float* prev_irr,
                 const float* prev_dist, float* out_irr, float* out_dist, int first, int precision, int border,
                 int p0, int p1) {
    const luxgi_ddgi_uniform& u = vd->uniform;
    const int P = u.probe_counts[0] * u.probe_counts[1] * u.probe_counts[2];
    if (p1 <= 0 || p1 > P) p1 = P;
    if (p0 < 0) p0 = 0;
#pragma omp parallel for schedule(dynamic, 4)
    for (int p = p0; p < p1; ++p) {
        if (precision == 1) {
            blend_probe<double>(vd, dirs, rays, prev_irr, out_irr, p, false, first != 0, p0);
            blend_probe<double>(vd, dirs, rays, prev_dist, out_dist, p, true, first != 0, p0);
        } else {
            blend_probe<float>(vd, dirs, rays, prev_irr, out_irr, p, false, first != 0, p0);
            blend_probe<float>(vd, dirs, rays, prev_dist, out_dist, p, true, first != 0, p0);
        }
    }
    if (border) {
        const int XY = u.probe_counts[0] * u.probe_counts[1], Z = u.probe_counts[2];
        border_atlas(out_irr, u.irradiance_width, 4, u.irradiance_probe_side, XY, Z);
        border_atlas(out_dist, u.depth_width, 2, u.depth_probe_side, XY, Z);
    }
    return 0;
}

int oracle_border(const luxgi_ddgi_uniform* u, float* irr, float* dist) {
    const int XY = u->probe_counts[0] * u->probe_counts[1], Z = u->probe_counts[2];
    if (irr) border_atlas(irr, u->irradiance_width, 4, u->irradiance_probe_side, XY, Z);
    if (dist) border_atlas(dist, u->depth_width, 2, u->depth_probe_side, XY, Z);
    return 0;
}

// (dst, src) offset pairs of the border rule for side n: int4 [4n+4].
int oracle_border_pairs(int n, int32_t* out) {
    std::vector<int> buf(size_t(4 * (4 * n + 4)));
    int (*pairs)[4] = reinterpret_cast<int (*)[4]>(buf.data());
    int np = border_pairs(n, pairs);
    for (int i = 0; i < np * 4; ++i) out[i] = buf[size_t(i)];
    return np;
}

// SDF mip + 4 flood passes for every cascade.  sdf_f32: the SDF as float
// values (FP16 SDFs converted by the caller); mip_out float [(mres*C)*mres^3].
int oracle_build_mip(const luxgi_sdf_desc* sdf, const float* sdf_f32, float* mip_out) {
    const int res = sdf->resolution, mres = sdf->mip_resolution, C = int(sdf->data.cascades_count);
    const bool fp16 = sdf->format == LUXGI_STORAGE_FP16;
    std::vector<float> src(sdf_f32, sdf_f32 + size_t(res) * C * res * res);
    std::vector<float> mip(size_t(mres) * C * mres * mres, 0.0f), tmp(size_t(mres) * mres * mres, 0.0f);
    for (int k = 0; k < C; ++k) {
        float maxd = sdf->data.cascade_pos_distance[k][3] * 2.0f;
        mip_pass(src, res * C, res, k * res, mip, mres * C, k * mres, mres, 4, maxd, fp16);
        for (int i = 1; i < 5; ++i) {
            if (i & 1) mip_pass(mip, mres * C, mres, k * mres, tmp, mres, 0, mres, 1, maxd, fp16);
            else mip_pass(tmp, mres, mres, 0, mip, mres * C, k * mres, mres, 1, maxd, fp16);
        }
    }
    std::memcpy(mip_out, mip.data(), mip.size() * sizeof(float));
    return 0;
}

// SDFCulling.comp (SDFCulling.comp:36-101) with a deterministic layout:
// chunks in flattened order at prefix-sum offsets starting at word 1, each
// list = [count, ids ascending]; [0] = words the full layout needs.  Chunks
// whose list would pass `capacity` stay empty (entry 0) and the call
// reports LUXGI_ENOMEM.
int oracle_cull(const luxgi_surface_desc* s, uint32_t* chunks, uint32_t* culled, uint32_t capacity) {
    const int N = 40;
    std::memset(chunks, 0, sizeof(uint32_t) * N * N * N);
    uint32_t used = 1;
    for (int z = 0; z < N; ++z)
        for (int y = 0; y < N; ++y)
            for (int x = 0; x < N; ++x) {
                float cs = s->data.chunk_size;
                float mn[3] = {(float(x) - N * 0.5f) * cs, (float(y) - N * 0.5f) * cs, (float(z) - N * 0.5f) * cs};
                float mx[3] = {mn[0] + cs, mn[1] + cs, mn[2] + cs};
                std::vector<uint32_t> ids;
                for (uint32_t o = 0; o < s->data.objects_count; ++o) {
                    const float* b = s->objects[o].object_bounds;
                    float cc[3], d2[3];
                    for (int k = 0; k < 3; ++k) { cc[k] = std::min(std::max(b[k], mn[k]), mx[k]); d2[k] = b[k] - cc[k]; }
                    float dist = std::sqrt(d2[0] * d2[0] + d2[1] * d2[1] + d2[2] * d2[2]);
                    if (dist <= b[3]) ids.push_back(o);
                }
                if (ids.empty()) continue;
                uint32_t need = uint32_t(ids.size()) + 1;
                uint32_t st = used;
                used += need;
                if (st + need > capacity) continue;
                culled[st] = uint32_t(ids.size());
                for (size_t i = 0; i < ids.size(); ++i) culled[st + 1 + i] = ids[i];
                chunks[z * N * N + y * N + x] = st;
            }
    if (capacity > 0) culled[0] = used;
    return used > capacity ? LUXGI_ENOMEM : 0;
}

// SDFAtlasIndirectLight.frag:44-67 over the footprint of every tile;
// light_out [res^2] of the surface's light format holds the light cache on
// entry (texels outside every footprint keep it); each footprint texel
// becomes direct_light + the bounce, rounded to that format (the additive
// draw into SurfaceLightCache).
int oracle_inject(const luxgi_ddgi_volume_desc* vd, const luxgi_surface_desc* s, const float* irr, const float* dist,
                  int frames, int precision, void* light_out) {
    const int res = int(s->data.resolution);
    const bool bounce = vd->infinite_bounce && frames != 0;
    Atlases A;
    const luxgi_ddgi_uniform& u = vd->uniform;
    A.irr.f32 = irr; A.irr.W = u.irradiance_width; A.irr.H = u.irradiance_height; A.irr.C = 4;
    A.dist.f32 = dist; A.dist.W = u.depth_width; A.dist.H = u.depth_height; A.dist.C = 2;
    const SurfaceTextures T(s);
    for (int t = 1; t < s->num_tiles; ++t) {
        const luxgi_surface_tile& tl = s->tiles[t];
        const Footprint fp = footprint(tl, res);
#pragma omp parallel for
        for (int j = 0; j < fp.h; ++j)
            for (int i = 0; i < fp.w; ++i) {
                const size_t ti = size_t(fp.y0 + j) * size_t(res) + size_t(fp.x0 + i);
                float add[3] = {0.0f, 0.0f, 0.0f};
                if (bounce) {
                    auto shade = [&](auto zero) {
                        using R = decltype(zero);
                        const SurfaceFragment<R> f = surface_fragment<R>(T, fragment_uv<R>(tl, fp, i, j));
                        const V3<R> cam{R(s->data.camera_pos[0]), R(s->data.camera_pos[1]), R(s->data.camera_pos[2])};
                        const V3<R> wo = normalize(sub(cam, f.pos));
                        const V3<R> e = sample_irradiance<R>(u, A, f.pos, f.normal, wo);
                        const R alb[3] = {std::min(f.albedo.x, R(0.9f)), std::min(f.albedo.y, R(0.9f)),
                                          std::min(f.albedo.z, R(0.9f))};
                        const R ev[3] = {e.x, e.y, e.z};
                        for (int k = 0; k < 3; ++k) {
                            const R diff = (alb[k] - alb[k] * f.metallic) / pi_r<R>();
                            add[k] = float(R(vd->intensity) * diff * ev[k]);
                        }
                    };
                    if (precision == 1) shade(0.0);
                    else shade(0.0f);
                }
                float v[4];
                color_load(s->direct_light, s->light_format, ti, v);
                for (int k = 0; k < 3; ++k) v[k] = v[k] + add[k];
                color_store(light_out, s->light_format, ti, v);
            }
    }
    return 0;
}

// One surface-lighting pass (the CopyEmissive draw, then one
// SDFDeferredLight draw per light with additive blending into the light
// cache, GlobalSurfaceAtlas.cpp:886-996) over tiles[0 .. n): out [res^2] of
// the surface's light format in/out, every draw's result rounded to that
// format.  masks[k] bit l: light l draws tile k (NULL: all).
// shadow_out (optional, u32 per texel) collects bit l for each light whose
// SDF shadow test blocked the fragment.
int oracle_surface_light(const luxgi_sdf_desc* sdf, const luxgi_surface_desc* s, const luxgi_light* lights,
                         int num_lights, const uint32_t* tiles, const uint32_t* masks, int num_tiles,
                         const float cam[3], float shadow_bias, int copy_emissive, int max_steps, int precision,
                         void* out, uint32_t* shadow_out) {
    const int fmt = s->light_format;
    const int res = int(s->data.resolution), mres = sdf->mip_resolution, C = int(sdf->data.cascades_count);
    Vol tex, mip;
    tex.W = sdf->resolution * C; tex.H = sdf->resolution; tex.D = sdf->resolution;
    mip.W = mres * C; mip.H = mres; mip.D = mres;
    if (sdf->format == LUXGI_STORAGE_FP16) {
        tex.f16 = static_cast<const uint16_t*>(sdf->sdf);
        mip.f16 = static_cast<const uint16_t*>(sdf->mip);
    } else {
        tex.f32 = static_cast<const float*>(sdf->sdf);
        mip.f32 = static_cast<const float*>(sdf->mip);
    }
    const SurfaceTextures T(s);
    for (int k = 0; k < num_tiles; ++k) {
        const uint32_t t = tiles[k];
        if (t < 1 || int(t) >= s->num_tiles) return LUXGI_EINVAL;
        const luxgi_surface_tile& tl = s->tiles[t];
        const Footprint fp = footprint(tl, res);
        const uint32_t mask = masks ? masks[k] : (num_lights >= 32 ? 0xFFFFFFFFu : ((1u << num_lights) - 1u));
#pragma omp parallel for schedule(dynamic)
        for (int j = 0; j < fp.h; ++j)
            for (int i = 0; i < fp.w; ++i) {
                const size_t ti = size_t(fp.y0 + j) * size_t(res) + size_t(fp.x0 + i);
                float acc[4];
                if (copy_emissive) {
                    const V2<float> uv = fragment_uv<float>(tl, fp, i, j);
                    for (int c = 0; c < 4; ++c)
                        acc[c] = T.has_emissive ? bilinear_repeat(T.emissive, uv, c) : (c == 3 ? 1.0f : 0.0f);
                    if (T.has_emissive) color_round(fmt, acc);
                } else {
                    color_load(out, fmt, ti, acc);
                }
                uint32_t blocked = 0;
                for (int l = 0; l < num_lights; ++l) {
                    if (!(mask >> l & 1u)) continue;
                    float d[3];
                    bool sh = false;
                    if (precision == 1) {
                        const SurfaceFragment<double> f = surface_fragment<double>(T, fragment_uv<double>(tl, fp, i, j));
                        const V3<double> v = direct_light<double>(sdf, tex, mip, f, lights[l], cam, shadow_bias,
                                                                  max_steps, &sh);
                        d[0] = float(v.x); d[1] = float(v.y); d[2] = float(v.z);
                    } else {
                        const SurfaceFragment<float> f = surface_fragment<float>(T, fragment_uv<float>(tl, fp, i, j));
                        const V3<float> v = direct_light<float>(sdf, tex, mip, f, lights[l], cam, shadow_bias,
                                                                max_steps, &sh);
                        d[0] = v.x; d[1] = v.y; d[2] = v.z;
                    }
                    if (sh) blocked |= 1u << l;
                    for (int c = 0; c < 3; ++c) acc[c] = acc[c] + d[c];
                    acc[3] = acc[3] + 1.0f;
                    color_round(fmt, acc);
                }
                color_store(out, fmt, ti, acc);
                if (shadow_out) shadow_out[ti] = blocked;
            }
    }
    return 0;
}

// SampleProbe.comp:36-60 over a W x H G-buffer (depth R32F, nch floats of
// normal a pixel, octahedral xy first), float atlases; out RGBA16F bits:
// (irradiance, 1), or 0 where depth == 1.  worldPositionFromDepth
// (Common/Math.glsl:35-42) with glm's association of the matrix product.
int oracle_sample_probe_image(const luxgi_ddgi_uniform* u, const float* irr, const float* dist, const float* depth,
                              const float* normal, int nch, int W, int H, const float cam[3], const float vpi[16],
                              uint16_t* out) {
    Atlases A;
    A.irr.f32 = irr; A.irr.W = u->irradiance_width; A.irr.H = u->irradiance_height; A.irr.C = 4;
    A.dist.f32 = dist; A.dist.W = u->depth_width; A.dist.H = u->depth_height; A.dist.C = 2;
#pragma omp parallel for
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t i = size_t(y) * W + x;
            const float d = depth[i];
            float o[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (d != 1.0f) {
                const float tx = (float(x) + 0.5f) / float(W), ty = (float(y) + 0.5f) / float(H);
                const float sx = tx * 2.0f - 1.0f, sy = ty * 2.0f - 1.0f;
                const float* m = vpi;
                const float wx = (m[0] * sx + m[4] * sy) + (m[8] * d + m[12]);
                const float wy = (m[1] * sx + m[5] * sy) + (m[9] * d + m[13]);
                const float wz = (m[2] * sx + m[6] * sy) + (m[10] * d + m[14]);
                const float ww = (m[3] * sx + m[7] * sy) + (m[11] * d + m[15]);
                const V3<float> P{wx / ww, wy / ww, wz / ww};
                const V3<float> N = oct_decode(V2<float>{normal[i * nch], normal[i * nch + 1]});
                const V3<float> Wo = normalize(sub(V3<float>{cam[0], cam[1], cam[2]}, P));
                const V3<float> e = sample_irradiance<float>(*u, A, P, N, Wo);
                o[0] = e.x; o[1] = e.y; o[2] = e.z; o[3] = 1.0f;
            }
            for (int c = 0; c < 4; ++c) out[i * 4 + size_t(c)] = f2h_bits(o[c]);
        }
    return 0;
}

// sampleIrradiance for n points (float3 arrays), float atlases.
int oracle_sample_irradiance(const luxgi_ddgi_uniform* u, const float* irr, const float* dist, const float* pos,
                             const float* nrm, const float* wo, float* out, int n, int precision) {
    Atlases A;
    A.irr.f32 = irr; A.irr.W = u->irradiance_width; A.irr.H = u->irradiance_height; A.irr.C = 4;
    A.dist.f32 = dist; A.dist.W = u->depth_width; A.dist.H = u->depth_height; A.dist.C = 2;
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        if (precision == 1) {
            V3<double> e = sample_irradiance<double>(*u, A, V3<double>{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]},
                                                     V3<double>{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]},
                                                     V3<double>{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]});
            out[3 * i] = float(e.x); out[3 * i + 1] = float(e.y); out[3 * i + 2] = float(e.z);
        } else {
            V3<float> e = sample_irradiance<float>(*u, A, V3<float>{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]},
                                                   V3<float>{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]},
                                                   V3<float>{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]});
            out[3 * i] = e.x; out[3 * i + 1] = e.y; out[3 * i + 2] = e.z;
        }
    }
    return 0;
}

// Texel directions octDecode(normalizedOctCoord) for side n: float3 [n*n].
int oracle_texel_dirs(int n, int precision, float* out) {
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            int i = ty * n + tx;
            if (precision == 1) {
                V3<double> d = oct_decode(normalized_oct_coord<double>(tx, ty, n));
                out[3 * i] = float(d.x); out[3 * i + 1] = float(d.y); out[3 * i + 2] = float(d.z);
            } else {
                V3<float> d = oct_decode(normalized_oct_coord<float>(tx, ty, n));
                out[3 * i] = d.x; out[3 * i + 1] = d.y; out[3 * i + 2] = d.z;
            }
        }
    return 0;
}

// octEncode for n float3 directions (test aid).
int oracle_oct_encode(const float* dirs, int n, float* out) {
    for (int i = 0; i < n; ++i) {
        V2<double> o = oct_encode(V3<double>{dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]});
        out[2 * i] = float(o.x); out[2 * i + 1] = float(o.y);
    }
    return 0;
}

// The global SDF from objects (first build): every voxel 1, then per
// cascade its chunks rasterised and its mip built (flood passes only when
// the cascade has chunks).  Mesh volumes are host FP16 arrays.  sdf_out
// (res*C) x res x res and mip_out (mres*C) x mres^2 as float; fp16 rounds
// every stored value to half as the R16F textures do.
int oracle_sdf_build(const luxgi_sdf_build_desc* d, const luxgi_mesh_sdf* meshes, int nm,
                     const luxgi_sdf_object* objs, int no, float* sdf_out, float* mip_out, luxgi_sdf_data* data_out) {
    const int res = d->resolution, C = d->cascades, mres = res / 4;
    const bool fp16 = d->format == LUXGI_STORAGE_FP16;
    const int TW = res * C;
    std::vector<float> sdf(size_t(TW) * res * res, 1.0f);
    std::vector<float> mip(size_t(mres) * C * mres * mres, 1.0f), tmp(size_t(mres) * mres * mres, 1.0f);
    luxgi_sdf_data data{};
    for (int c = 0; c < C; ++c) {
        sdfb::Plan P;
        const int st = sdfb::plan(*d, meshes, nm, objs, no, c, P);
        if (st != 0) return st;
        const sdfb::Cascade K = sdfb::cascade(*d, c);
        data.cascade_pos_distance[c][0] = K.center[0];
        data.cascade_pos_distance[c][1] = K.center[1];
        data.cascade_pos_distance[c][2] = K.center[2];
        data.cascade_pos_distance[c][3] = K.distance;
        data.cascade_voxel_size[c] = K.voxel;
        const float maxd = K.distance * 2.0f;
        float mul[3], add[3];
        for (int i = 0; i < 3; ++i) {
            const float lo = K.center[i] - K.distance, hi = K.center[i] + K.distance;
            mul[i] = (hi - lo) / float(res);
            add[i] = lo + K.voxel * 0.5f;
        }
        const int level = std::min(c, 2);
#pragma omp parallel for schedule(dynamic)
        for (int k = 0; k < int(P.chunks.size()); ++k) {
            const luxgi_sdf_chunk& ck = P.chunks[size_t(k)];
            for (int lz = 0; lz < 32; ++lz)
                for (int ly = 0; ly < 32; ++ly)
                    for (int lx = 0; lx < 32; ++lx) {
                        const int vx = ck.coord[0] * 32 + lx, vy = ck.coord[1] * 32 + ly, vz = ck.coord[2] * 32 + lz;
                        const int gx = vx + c * res;
                        if (gx < 0 || gx >= TW || vy < 0 || vy >= res || vz < 0 || vz >= res) continue;
                        const float wp[3] = {float(vx) * mul[0] + add[0], float(vy) * mul[1] + add[1],
                                             float(vz) * mul[2] + add[2]};
                        float md = maxd;
                        for (int i = 0; i < ck.count; ++i) {
                            const uint32_t id = ck.models[i];
                            const luxgi_mesh_sdf& m = meshes[P.mesh[id]];
                            const int L = std::min(level, m.mip_count - 1);
                            const int W = std::max(m.size[0] >> L, 1), H = std::max(m.size[1] >> L, 1),
                                      D = std::max(m.size[2] >> L, 1);
                            const float od = sdfb::distance_to_model(md, P.recs[id], m.mips[L], W, H, D, wp);
                            md = sdfb::fmin_g(md, od);
                        }
                        float v = sdfb::fmin_g(sdfb::fmax_g(md / maxd, -1.0f), 1.0f);
                        if (fp16) v = round_half(v);
                        sdf[size_t(gx) + size_t(TW) * (size_t(vy) + size_t(res) * size_t(vz))] = v;
                    }
        }
        mip_pass(sdf, TW, res, c * res, mip, mres * C, c * mres, mres, 4, maxd, fp16);
        if (!P.chunks.empty())
            for (int i = 1; i < 5; ++i) {
                if (i & 1) mip_pass(mip, mres * C, mres, c * mres, tmp, mres, 0, mres, 1, maxd, fp16);
                else mip_pass(tmp, mres, mres, 0, mip, mres * C, c * mres, mres, 1, maxd, fp16);
            }
    }
    data.cascades_count = uint32_t(C);
    data.resolution = float(res);
    data.near_plane = d->near_plane;
    data.far_plane = d->far_plane;
    std::memcpy(sdf_out, sdf.data(), sdf.size() * sizeof(float));
    std::memcpy(mip_out, mip.data(), mip.size() * sizeof(float));
    if (data_out) *data_out = data;
    return 0;
}

// The plan of one cascade: records, their meshes and chunks (capacities as
// luxgi_sdf_build_plan).
int oracle_sdf_plan(const luxgi_sdf_build_desc* d, const luxgi_mesh_sdf* meshes, int nm, const luxgi_sdf_object* objs,
                    int no, int cascade, luxgi_sdf_raster_object* recs, int rec_cap, int* n_recs, int32_t* rec_mesh,
                    luxgi_sdf_chunk* chunks, int chunk_cap, int* n_chunks) {
    sdfb::Plan P;
    const int st = sdfb::plan(*d, meshes, nm, objs, no, cascade, P);
    if (st != 0) return st;
    *n_recs = int(P.recs.size());
    *n_chunks = int(P.chunks.size());
    if (int(P.recs.size()) > rec_cap || int(P.chunks.size()) > chunk_cap) return LUXGI_ENOMEM;
    for (size_t i = 0; i < P.recs.size(); ++i) {
        recs[i] = P.recs[i];
        rec_mesh[i] = P.mesh[i];
    }
    for (size_t i = 0; i < P.chunks.size(); ++i) chunks[i] = P.chunks[i];
    return 0;
}

}  // extern "C"
