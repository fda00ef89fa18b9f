// Device-side math shared by the DDGI kernels (sm_103a).
//
// The SDF march is evaluated in FP32 with a fixed operation order and no
// fused multiply-add (the translation units that include the march build
// with -fmad=false), so its hit times equal those of an FP32 CPU evaluation
// of the same expressions bit for bit.  min/max follow the C++ std::min /
// std::max convention ((b < a) ? b : a), not fminf/fmaxf.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_fp16.h>

#include "luxgi_ddgi.h"

namespace luxgi {

constexpr float kWorldSize = 60000.0f;          // GLOBAL_SDF_WORLD_SIZE (SDFCommon.glsl:8)
constexpr int kChunksRes = 40;                  // GLOBAL_SURFACE_ATLAS_CHUNKS_RESOLUTION
constexpr float kPi = 3.14159265f;

struct f3 { float x, y, z; };

__host__ __device__ __forceinline__ float mn(float a, float b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ float mx(float a, float b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ int imn(int a, int b) { return (b < a) ? b : a; }
__host__ __device__ __forceinline__ int imx(int a, int b) { return (a < b) ? b : a; }
__host__ __device__ __forceinline__ float clampf(float v, float lo, float hi) { return mn(mx(v, lo), hi); }
__device__ __forceinline__ f3 make3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 mul3(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 mulv3(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float len3(f3 a) { return sqrtf(dot3(a, a)); }
__device__ __forceinline__ f3 norm3(f3 a) { float inv = 1.0f / sqrtf(dot3(a, a)); return mul3(a, inv); }

// x / d for a divisor d > 0 fixed over a loop, bit for bit the IEEE quotient
// RN(x / d), without a division per call.  y = RN(1 / d) is computed once
// (for the march's divisors on the host, with the SDF's view).
// q0 = RN(x y) lies within 1.5 ulp of x / d; one correction with the
// remainder, q1 = RN(q0 + RN(x - d q0) y), brings it within 1 ulp (the
// error left is |x - d q0| |y - 1/d|, a few 2^-24 ulp); a second, whose
// remainder x - d q1 an FMA computes exactly, rounds to RN(x / d) by
// Markstein's theorem (y within 1/2 ulp of 1/d, q1 within 1 ulp of x / d;
// P. Markstein, IBM J. Res. Dev. 34(1), 1990), as long as no intermediate
// leaves the normal range, which holds for |x| in [2^-100, 2^100] and the
// march's divisors (cascade extents, voxel sizes, the cascade count).  The
// remainder is kept negated (d q - x) so that x = -0 gives -0 like the
// division.  For a power of two d both corrections add zero.
// tests/exact_div_check.c checks the sequence against IEEE division over
// every significand of x (both signs, several binades, signed zeros) for
// the engine's default cascade divisors and significands at the edges.
struct ExactDiv {
    float d, y;
    bool pow2;   // d a power of two with a normal reciprocal: x y is exact
};

__device__ __forceinline__ ExactDiv exact_div(float d) {
    const uint32_t b = __float_as_uint(d);
    const uint32_t ex = (b >> 23) & 0xFFu;
    return ExactDiv{d, 1.0f / d, (b & 0x7FFFFFu) == 0u && ex >= 2u && ex <= 252u};
}

// POW2: every divisor of the loop is a power of two (the corrections would
// add zero), chosen outside the loop so the steps carry no test for it.
template <bool POW2>
__device__ __forceinline__ float xdiv(float x, const ExactDiv& e) {
    float q = x * e.y;
    if (POW2) return q;
    float r = fmaf(e.d, q, -x);
    q = fmaf(-r, e.y, q);
    r = fmaf(e.d, q, -x);
    return fmaf(-r, e.y, q);
}

// How a march step loop forms its quotients: kStepPow2 multiplies alone
// (every divisor a power of two), kStepExact the corrected quotient,
// kStepSelect either per call by the divisor's flag.
enum StepDiv { kStepExact = 0, kStepPow2 = 1, kStepSelect = 2 };
template <int M>
__device__ __forceinline__ float qdiv(float x, const ExactDiv& e) {
    if (M == kStepPow2) return xdiv<true>(x, e);
    if (M == kStepSelect) return e.pow2 ? xdiv<true>(x, e) : xdiv<false>(x, e);
    return xdiv<false>(x, e);
}
// How march_run compiles its step loop: twice, a power-of-two copy and an
// exact one, chosen per cascade (kDivSplit); once with exact quotients
// (kDivExact); once choosing per quotient (kDivSelect).
enum MarchDiv { kDivSplit = 0, kDivExact = 1, kDivSelect = 2 };

// sin/cos for the Fibonacci azimuth: Cody-Waite reduction by pi/2 and Taylor
// polynomials of degree 9 (sin) and 8 (cos) on [-pi/4, pi/4].
__device__ __forceinline__ void fib_sincos(float x, float* s, float* c) {
    const float k = floorf(x * 0.63661977f + 0.5f);
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

// madfrac(i, PHI - 1) of sphericalFibonacci in compensated FP32: PHI - 1 as
// a hi + lo pair and the product i * hi split exactly with one FMA, so the
// azimuth keeps ~1e-7 rad at any ray index (plain FP32 loses ~2^-24 * i turns).
__host__ __device__ __forceinline__ float fib_frac(float i) {
    const float c_hi = 0.618034005165100098f;      // float(PHI - 1)
    const float c_lo = -1.64152047e-8f;            // (PHI - 1) - c_hi
    const float p = i * c_hi;
    const float e = fmaf(i, c_hi, -p);             // exact low part of i * c_hi
    float m = (p - floorf(p)) + (e + i * c_lo);
    if (m >= 1.0f) m = m - 1.0f;
    if (m < 0.0f) m = m + 1.0f;
    return m;
}

// sphericalFibonacci (DDGICommon.glsl:42-52) rotated by mat3(rot), normalised.
__device__ __forceinline__ f3 ray_direction(const float* rot, int r, int nrays) {
    const float i = float(r);
    const float mf = fib_frac(i);
    const float phi = (2.0f * kPi) * mf;
    const float cos_t = 1.0f - (2.0f * i + 1.0f) * (1.0f / float(nrays));
    const float sin_t = sqrtf(clampf(1.0f - cos_t * cos_t, 0.0f, 1.0f));
    float sp, cp;
    fib_sincos(phi, &sp, &cp);
    const f3 f{cp * sin_t, sp * sin_t, cos_t};
    const f3 m{rot[0] * f.x + rot[3] * f.y + rot[6] * f.z,
               rot[1] * f.x + rot[4] * f.y + rot[7] * f.z,
               rot[2] * f.x + rot[5] * f.y + rot[8] * f.z};
    return norm3(m);
}

// probeLocation (DDGICommon.glsl:101-114)
// Division by a run-time invariant d >= 1 as multiply-high and shift
// (Granlund and Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994, theorem 4.2): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1, n / d = (mulhi(n, m) + n) >> l for
// every 32-bit n.  Exact, so it replaces '/' and '%' without changing results.
struct FastDiv {
    uint32_t d, m, s;
};

inline FastDiv make_fastdiv(uint32_t d) {
    FastDiv f;
    f.d = d;
    uint32_t l = 0;
    while ((uint64_t(1) << l) < d) ++l;
    f.s = l;
    f.m = uint32_t(((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d + 1);
    return f;
}

__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return uint32_t((uint64_t(__umulhi(n, f.m)) + n) >> f.s);
}

// probeLocation with the grid index split by precomputed divisors of X and X*Y.
__device__ __forceinline__ f3 probe_location(const luxgi_ddgi_uniform& u, uint32_t index, const FastDiv& div_x,
                                             const FastDiv& div_xy) {
    const uint32_t gz = fdiv(index, div_xy);
    const uint32_t rem = index - gz * div_xy.d;
    const uint32_t gy = fdiv(rem, div_x);
    const uint32_t gx = rem - gy * div_x.d;
    return f3{__fadd_rn(__fmul_rn(u.step[0], float(int(gx))), u.start_position[0]),
              __fadd_rn(__fmul_rn(u.step[1], float(int(gy))), u.start_position[1]),
              __fadd_rn(__fmul_rn(u.step[2], float(int(gz))), u.start_position[2])};
}

__device__ __forceinline__ f3 probe_location(const luxgi_ddgi_uniform& u, int index) {
    const int X = u.probe_counts[0], Y = u.probe_counts[1];
    const int gx = index % X, gy = (index % (X * Y)) / X, gz = index / (X * Y);
    return f3{u.step[0] * float(gx) + u.start_position[0], u.step[1] * float(gy) + u.start_position[1],
              u.step[2] * float(gz) + u.start_position[2]};
}

__device__ __forceinline__ float load_val(const float* p, size_t i) { return __ldg(p + i); }
__device__ __forceinline__ float load_val(const __half* p, size_t i) { return __half2float(__ldg(p + i)); }

// GL LINEAR + CLAMP_TO_EDGE trilinear sample of a W x H x D volume.
template <typename T>
__device__ __forceinline__ float sample3d(const T* __restrict__ v, int W, int H, int D, float u, float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const float a = x - fx, b = y - fy, c = z - fz;
    int x0 = int(fx), y0 = int(fy), z0 = int(fz);
    const int x1 = imn(imx(x0 + 1, 0), W - 1), y1 = imn(imx(y0 + 1, 0), H - 1), z1 = imn(imx(z0 + 1, 0), D - 1);
    x0 = imn(imx(x0, 0), W - 1); y0 = imn(imx(y0, 0), H - 1); z0 = imn(imx(z0, 0), D - 1);
    const size_t WH = size_t(W) * size_t(H);
    const size_t r00 = size_t(y0) * W + z0 * WH, r10 = size_t(y1) * W + z0 * WH;
    const size_t r01 = size_t(y0) * W + z1 * WH, r11 = size_t(y1) * W + z1 * WH;
    const float t000 = load_val(v, r00 + x0), t100 = load_val(v, r00 + x1);
    const float t010 = load_val(v, r10 + x0), t110 = load_val(v, r10 + x1);
    const float t001 = load_val(v, r01 + x0), t101 = load_val(v, r01 + x1);
    const float t011 = load_val(v, r11 + x0), t111 = load_val(v, r11 + x1);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = t000 * ia + t100 * a, c10 = t010 * ia + t110 * a;
    const float c01 = t001 * ia + t101 * a, c11 = t011 * ia + t111 * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// sample3d for coordinates u, v, w in [0, 1] (or NaN): the floors of u W -
// 0.5 ... lie in [-1, W - 1] (a NaN converts to 0), so each corner index
// needs one side of its clamp, and texel indices are 32-bit (volumes of
// fewer than 2^32 texels, checked when the SDF is bound).  Same texels,
// same arithmetic.
template <typename T>
__device__ __forceinline__ float sample3d_unit(const T* __restrict__ v, int W, int H, int D, float u, float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const float a = x - fx, b = y - fy, c = z - fz;
    const int ix = int(fx), iy = int(fy), iz = int(fz);
    const uint32_t x0 = uint32_t(imx(ix, 0)), x1 = uint32_t(imn(ix + 1, W - 1));
    const uint32_t y0 = uint32_t(imx(iy, 0)), y1 = uint32_t(imn(iy + 1, H - 1));
    const uint32_t z0 = uint32_t(imx(iz, 0)), z1 = uint32_t(imn(iz + 1, D - 1));
    const uint32_t Wu = uint32_t(W), WH = Wu * uint32_t(H);
    const uint32_t r00 = y0 * Wu + z0 * WH, r10 = y1 * Wu + z0 * WH;
    const uint32_t r01 = y0 * Wu + z1 * WH, r11 = y1 * Wu + z1 * WH;
    const float t000 = load_val(v, r00 + x0), t100 = load_val(v, r00 + x1);
    const float t010 = load_val(v, r10 + x0), t110 = load_val(v, r10 + x1);
    const float t001 = load_val(v, r01 + x0), t101 = load_val(v, r01 + x1);
    const float t011 = load_val(v, r11 + x0), t111 = load_val(v, r11 + x1);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = t000 * ia + t100 * a, c10 = t010 * ia + t110 * a;
    const float c01 = t001 * ia + t101 * a, c11 = t011 * ia + t111 * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// Quad-packed volume: texel (x, y, z) for x in [-1, W-1], y in [-1, H-1]
// holds (v[x, y], v[x+1, y], v[x, y+1], v[x+1, y+1]) of plane z with the
// indices clamped to the volume, at [z][y + 1][x + 1] of a (W+1) x (H+1) x D
// array.  A GL trilinear sample with clamp-to-edge needs two of them (planes
// z0 and z1) and reads exactly the values of the eight-tap form.
template <typename T> struct Quad;
template <> struct Quad<float> { using type = float4; };
template <> struct Quad<__half> { using type = uint2; };

__device__ __forceinline__ void quad_vals(const float4& q, float* o) { o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.w; }
__device__ __forceinline__ void quad_vals(const uint2& q, float* o) {
    const __half2 a = *reinterpret_cast<const __half2*>(&q.x);
    const __half2 b = *reinterpret_cast<const __half2*>(&q.y);
    o[0] = __low2float(a); o[1] = __high2float(a); o[2] = __low2float(b); o[3] = __high2float(b);
}

// The quad-packed sample from its integer corner (ix, iy, iz) = the floors
// of the texel coordinates and the fractions (a, b, c).  Texel indices are
// 32-bit: the volume holds fewer than 2^32 quad texels (checked when the
// packed copy is made).
template <typename T>
__device__ __forceinline__ float quad_lerp(const typename Quad<T>::type* __restrict__ q, int W, int H, int D, float a,
                                           float b, float c, int ix, int iy, int iz) {
    const int qx = imn(imx(ix, -1), W - 1) + 1, qy = imn(imx(iy, -1), H - 1) + 1;
    const int z0 = imn(imx(iz, 0), D - 1), z1 = imn(imx(iz + 1, 0), D - 1);
    const uint32_t QW = uint32_t(W) + 1u, QWH = QW * (uint32_t(H) + 1u);
    const uint32_t row = uint32_t(qy) * QW + uint32_t(qx);
    float p0[4], p1[4];
    quad_vals(__ldg(q + (uint32_t(z0) * QWH + row)), p0);
    quad_vals(__ldg(q + (uint32_t(z1) * QWH + row)), p1);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = p0[0] * ia + p0[1] * a, c10 = p0[2] * ia + p0[3] * a;
    const float c01 = p1[0] * ia + p1[1] * a, c11 = p1[2] * ia + p1[3] * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// quad_lerp for coordinates u, v, w in [0, 1] (or NaN): the floors of u W -
// 0.5 ... then lie in [-1, W - 1] (a NaN converts to 0), so the x and y
// clamps of quad_lerp never bind and only the z planes are clamped.  Same
// texels, same arithmetic.
template <typename T>
__device__ __forceinline__ float quad_lerp_unit(const typename Quad<T>::type* __restrict__ q, int W, int H, int D,
                                                float a, float b, float c, int ix, int iy, int iz) {
    const int z0 = imx(iz, 0), z1 = imn(iz + 1, D - 1);
    const uint32_t QW = uint32_t(W) + 1u, QWH = QW * (uint32_t(H) + 1u);
    const uint32_t row = uint32_t(iy + 1) * QW + uint32_t(ix + 1);
    float p0[4], p1[4];
    quad_vals(__ldg(q + (uint32_t(z0) * QWH + row)), p0);
    quad_vals(__ldg(q + (uint32_t(z1) * QWH + row)), p1);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = p0[0] * ia + p0[1] * a, c10 = p0[2] * ia + p0[3] * a;
    const float c01 = p1[0] * ia + p1[1] * a, c11 = p1[2] * ia + p1[3] * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

template <typename T>
__device__ __forceinline__ float sample3d_quad_unit(const typename Quad<T>::type* __restrict__ q, int W, int H, int D,
                                                    float u, float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    return quad_lerp_unit<T>(q, W, H, D, x - fx, y - fy, z - fz, int(fx), int(fy), int(fz));
}

template <typename T>
__device__ __forceinline__ float sample3d_quad(const typename Quad<T>::type* __restrict__ q, int W, int H, int D, float u,
                                               float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    return quad_lerp<T>(q, W, H, D, x - fx, y - fy, z - fz, int(fx), int(fy), int(fz));
}

// Pair-packed volume: texel (x, y, z) for x in [-1, W-1] holds
// (v[x, y, z], v[x+1, y, z]) with x clamped, at [z][y][x + 1] of a
// (W+1) x H x D array: a trilinear sample is four paired loads.
template <typename T> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<__half> { using type = __half2; };
__device__ __forceinline__ void pair_vals(const float2& q, float* o) { o[0] = q.x; o[1] = q.y; }
__device__ __forceinline__ void pair_vals(const __half2& q, float* o) { o[0] = __low2float(q); o[1] = __high2float(q); }

template <typename T>
__device__ __forceinline__ float sample3d_pair(const typename Pair<T>::type* __restrict__ q, int W, int H, int D, float u,
                                               float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const float a = x - fx, b = y - fy, c = z - fz;
    const int px = imn(imx(int(fx), -1), W - 1) + 1;
    const int y0 = imn(imx(int(fy), 0), H - 1), y1 = imn(imx(int(fy) + 1, 0), H - 1);
    const int z0 = imn(imx(int(fz), 0), D - 1), z1 = imn(imx(int(fz) + 1, 0), D - 1);
    const size_t PW = size_t(W) + 1, PWH = PW * size_t(H);
    float r00[2], r10[2], r01[2], r11[2];
    pair_vals(__ldg(q + size_t(z0) * PWH + size_t(y0) * PW + px), r00);
    pair_vals(__ldg(q + size_t(z0) * PWH + size_t(y1) * PW + px), r10);
    pair_vals(__ldg(q + size_t(z1) * PWH + size_t(y0) * PW + px), r01);
    pair_vals(__ldg(q + size_t(z1) * PWH + size_t(y1) * PW + px), r11);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = r00[0] * ia + r00[1] * a, c10 = r10[0] * ia + r10[1] * a;
    const float c01 = r01[0] * ia + r01[1] * a, c11 = r11[0] * ia + r11[1] * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// Gather-texture volume: the z planes of a W x H x D volume tiled into one
// 2D texture (CUDA array, block-linear), gx = 2^lg planes a row, each plane
// (W + 2) x (H + 2) texels with a 1-texel apron that repeats its edge
// (clamp-to-edge inside the tile).  Volume texel (x, y, z) sits at texture
// texel (ox + x + 1, oy + y + 1), (ox, oy) = ((z mod gx) (W + 2),
// (z div gx) (H + 2)).  One textureGather at the unnormalised point
// (ox + ix + 2, oy + iy + 2) -- the centre of a 2x2 block, so the texture
// unit's sub-texel rounding cannot move the footprint -- returns the four
// texels (ix .. ix+1) x (iy .. iy+1) of plane z, clamped; a trilinear sample
// is two gathers (planes z0, z1) and the same FP32 lerps as the eight-tap
// form.  One copy of the volume (+1.6 % of apron at 256^2 planes) where the
// quad-packed copy holds four.
struct GatherVol {
    unsigned long long tex;   // cudaTextureObject_t
    int lg;                   // planes per texture row = 2^lg
};

template <typename T>
__device__ __forceinline__ float gather_lerp(const GatherVol& g, int W, int H, int D, float a, float b, float c, int ix,
                                             int iy, int iz) {
    const int z0 = imx(iz, 0), z1 = imn(iz + 1, D - 1);
    const int m = (1 << g.lg) - 1;
    const int ox0 = (z0 & m) * (W + 2), oy0 = (z0 >> g.lg) * (H + 2);
    const int ox1 = (z1 & m) * (W + 2), oy1 = (z1 >> g.lg) * (H + 2);
    // (texel x, y) + 1 for the apron, + 1 for the block centre
    const float4 q0 = tex2Dgather<float4>(g.tex, float(ox0 + ix + 2), float(oy0 + iy + 2), 0);
    const float4 q1 = tex2Dgather<float4>(g.tex, float(ox1 + ix + 2), float(oy1 + iy + 2), 0);
    // gather order (i0, j1), (i1, j1), (i1, j0), (i0, j0)
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = q0.w * ia + q0.z * a, c10 = q0.x * ia + q0.y * a;
    const float c01 = q1.w * ia + q1.z * a, c11 = q1.x * ia + q1.y * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// A sample anywhere (the hit normal's taps reach one texel past [0, 1]):
// the corner clamped to [-1, W - 1] per axis, so that the x and y taps read
// the apron (the edge value) and the planes z0 = max(iz, 0), z1 = min(iz + 1,
// D - 1) are those of the two-sided clamp; the fractions stay those of the
// unclamped corner, as in sample3d (equal taps then mix to the same value).
template <typename T>
__device__ __forceinline__ float sample3d_gather(const GatherVol& g, int W, int H, int D, float u, float vv, float w) {
    const float x = u * float(W) - 0.5f, y = vv * float(H) - 0.5f, z = w * float(D) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const int ix = imn(imx(int(fx), -1), W - 1), iy = imn(imx(int(fy), -1), H - 1);
    const int iz = imn(imx(int(fz), -1), D - 1);
    return gather_lerp<T>(g, W, H, D, x - fx, y - fy, z - fz, ix, iy, iz);
}

// Volume layouts a march variant reads
enum VolLayout { kPlain = 0, kQuad = 1, kPair = 2, kGather = 3 };

struct SdfView {
    luxgi_sdf_data data;
    const void* sdf;
    const void* mip;
    const void* sdf_quad;   // packed copy of the full-resolution volume (quad or
                            // pair layout, march variants 4 / 5) or nullptr
    const void* mip_quad;   // quad-packed mip (variants 3-5) or nullptr
    GatherVol sdf_g;        // gather textures (variant 10), tex 0 otherwise
    GatherVol mip_g;
    // One bit per cell (i, j, k) of the full-resolution volume, 32 cells a
    // word: set unless the minimum texel over [4i, 4i+4] x [4j, 4j+4] x
    // [4k, 4k+4] (clamped; every texel a trilinear footprint whose lower
    // corner lies in the cell can read) is at or above the march's skip
    // threshold.  nullptr: not built.
    const uint32_t* cell_near;
    int cw, ch;             // cells along x (packed cascades) and y
    int res, mres, C;
    int format;   // luxgi_storage of the sdf/mip texels
    // the march's loop-fixed divisors with their reciprocals, made once on
    // the host (IEEE division there as here): per cascade 2 x its half
    // extent and its voxel size, and the cascade count
    ExactDiv div_ext[4], div_voxel[4], div_count;
    // 32 / resolution, 4 / resolution and 1 / resolution (SDFCommon.glsl's
    // chunk and margin in texture coordinates, the normal's offset), also
    // divided once on the host
    float chunk, margin, texel;
};

constexpr int kCellSide = 4;

// False when the trilinear full-resolution sample at packed texture
// coordinates (u, v, w) is certainly >= the skip threshold 2 margin (1.001):
// every texel it interpolates is >= the cell minimum, and a convex
// combination of values >= m > 0 computed in FP32 is >= m (1 - 2^-20), so
// such a sample is never used (SDFCommon.glsl:150-158).  The 32 KB a
// cascade of bits stay in L1, unlike the cell minima they are made from.
// The same from the floors (ix, iy, iz) of the full-resolution texel
// coordinates u W - 0.5 ... of coordinates in [0, 1] (or NaN): the floors
// lie in [-1, W - 1] (NaN converts to 0), so only the lower clamp binds.
__device__ __forceinline__ bool fine_needed_at(const SdfView& s, int ix, int iy, int iz) {
    if (!s.cell_near) return true;
    const uint32_t x0 = uint32_t(imx(ix, 0)), y0 = uint32_t(imx(iy, 0)), z0 = uint32_t(imx(iz, 0));
    const uint32_t c = ((z0 / kCellSide) * uint32_t(s.ch) + (y0 / kCellSide)) * uint32_t(s.cw) + x0 / kCellSide;
    return (__ldg(s.cell_near + (c >> 5)) >> (c & 31u)) & 1u;
}

__device__ __forceinline__ bool fine_needed(const SdfView& s, float u, float v, float w) {
    const int W = s.res * s.C, H = s.res, D = s.res;
    return fine_needed_at(s, int(floorf(u * float(W) - 0.5f)), int(floorf(v * float(H) - 0.5f)),
                          int(floorf(w * float(D) - 0.5f)));
}

// One GL trilinear sample of the full-resolution or mip volume, from the
// plain layout or from its quad-packed copy (same values either way).
template <typename T, int LAYOUT>
__device__ __forceinline__ float sample_vol(const void* plain, const void* packed, const GatherVol& g, int W, int H,
                                            int D, float u, float v, float w) {
    if (LAYOUT == kGather) return sample3d_gather<T>(g, W, H, D, u, v, w);
    if (LAYOUT == kQuad) return sample3d_quad<T>(static_cast<const typename Quad<T>::type*>(packed), W, H, D, u, v, w);
    if (LAYOUT == kPair) return sample3d_pair<T>(static_cast<const typename Pair<T>::type*>(packed), W, H, D, u, v, w);
    return sample3d(static_cast<const T*>(plain), W, H, D, u, v, w);
}

// Hit normal: central differences of the full-resolution SDF at +-1/res in
// packed texture coordinates (SDFCommon.glsl:174-183).  Kept out of line so
// the march loop's register budget does not carry its taps.
template <typename T, int LAYOUT>
__device__ __noinline__ f3 sdf_normal(const void* tex, const void* texq, const GatherVol g, int TW, int res, float tu,
                                      float uy, float uz, float off) {
    const float xp = sample_vol<T, LAYOUT>(tex, texq, g, TW, res, res, tu + off, uy, uz);
    const float xn = sample_vol<T, LAYOUT>(tex, texq, g, TW, res, res, tu - off, uy, uz);
    const float yp = sample_vol<T, LAYOUT>(tex, texq, g, TW, res, res, tu, uy + off, uz);
    const float yn = sample_vol<T, LAYOUT>(tex, texq, g, TW, res, res, tu, uy - off, uz);
    const float zp = sample_vol<T, LAYOUT>(tex, texq, g, TW, res, res, tu, uy, uz + off);
    const float zn = sample_vol<T, LAYOUT>(tex, texq, g, TW, res, res, tu, uy, uz - off);
    return norm3(f3{xp - xn, yp - yn, zp - zn});
}

struct MarchHit {
    f3 normal;     // filled by march_hit_normal
    float time;
    int cascade;
    int steps;
    int fine;      // full-resolution SDF samples taken (for byte accounting)
    float sdf;
    float u, v, w; // packed texture coordinates of the hit sample
};

// Where a ray's march stands between calls of march_run: the cascade (and
// whether its entry was computed), the step within it, the march distance
// t, the cascade's exit distance, the next cascade's start, and the step and
// full-resolution sample totals.  Everything else is recomputed from the
// ray's origin and direction.
struct MarchState {
    int cascade;
    int in_cascade;
    int step;
    float t, is_y, next_start;
    int steps, fine;
};

__device__ __forceinline__ void march_state_init(MarchState& m) {
    m.cascade = 0;
    m.in_cascade = 0;
    m.step = 0;
    m.t = 0.0f;
    m.is_y = 0.0f;
    m.next_start = 0.0f;
    m.steps = 0;
    m.fine = 0;
}

// tracyGlobalSDF (SDFCommon.glsl:98-194) with stepScale 1, run for at most
// `budget` steps: returns true with `hit` filled when the march ended (hit,
// or every cascade left), false when the budget ran out first (m holds the
// state to resume from).  Resuming performs exactly the arithmetic of an
// unbroken march.  QMIP / QTEX select the layouts (VolLayout) read for the
// mip / full-resolution volume.  The probe rays use start bias 0 and want
// the hit normal (GISDFRays.comp:79-87): march_hit_normal computes it once
// the march is over, outside the step loop, so that the lanes of a warp
// whose rays hit at different steps fetch their normal taps together.  The
// surface-cache shadow rays start 2 voxels along and skip it
// (SDFDeferredLight.frag:104-111).
template <typename T, int QMIP = kPlain, int QTEX = kPlain, int DIV = kDivSplit>
__device__ __forceinline__ bool march_run(const SdfView& s, f3 origin, f3 dir, float trace_max, int max_steps,
                                          MarchState& m, int budget, MarchHit& hit, float start_bias = 0.0f) {
    const int C = s.C;
    const int TW = s.res * C, MW = s.mres * C;
    const float tmax = mn(trace_max, s.data.cascade_pos_distance[C - 1][3] * 2.0f);
    const float chunk = s.chunk;
    const float margin = s.margin;
    const f3 end = add3(origin, mul3(dir, tmax));
    for (; m.cascade < C; ++m.cascade) {
        const int cascade = m.cascade;
        const float cx = s.data.cascade_pos_distance[cascade][0], cy = s.data.cascade_pos_distance[cascade][1],
                    cz = s.data.cascade_pos_distance[cascade][2], cw = s.data.cascade_pos_distance[cascade][3];
        const float voxel = s.data.cascade_voxel_size[cascade];
        const float voxel_half = voxel * 0.5f;
        const f3 wpos = add3(origin, mul3(dir, voxel * start_bias));
        if (!m.in_cascade) {
            // lineHitAABB (SDFCommon.glsl:84-95)
            const f3 d = sub3(end, wpos);
            const f3 inv{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
            const f3 en{((cx - cw) - wpos.x) * inv.x, ((cy - cw) - wpos.y) * inv.y, ((cz - cw) - wpos.z) * inv.z};
            const f3 ex{((cx + cw) - wpos.x) * inv.x, ((cy + cw) - wpos.y) * inv.y, ((cz + cw) - wpos.z) * inv.z};
            const float i0 = mx(mn(en.x, ex.x), mx(mn(en.y, ex.y), mn(en.z, ex.z)));
            const float i1 = mn(mx(en.x, ex.x), mn(mx(en.y, ex.y), mx(en.z, ex.z)));
            float is_x = clampf(i0, 0.0f, 1.0f) * tmax;
            m.is_y = clampf(i1, 0.0f, 1.0f) * tmax;
            is_x = mx(is_x, m.next_start);
            m.t = is_x;
            if (is_x >= m.is_y) m.t = m.is_y;
            else m.next_start = m.is_y;
            m.step = 0;
            m.in_cascade = 1;
        }
        const float md = cw * 2.0f;
        // the host's reciprocals (kDivSplit, kDivExact: parameters in the
        // constant bank), or computed here (kDivSelect, the batched kernels,
        // whose parameters sit in shared or global memory: batch48 4.61 ->
        // 4.55 ms a frame against the copies)
        ExactDiv div_md, div_c, div_voxel;
        if constexpr (DIV == kDivSelect) {
            div_md = exact_div(md);
            div_c = exact_div(float(C));
            div_voxel = exact_div(voxel);
        } else {
            div_md = s.div_ext[cascade];
            div_c = s.div_count;
            div_voxel = s.div_voxel[cascade];
        }
        float t = m.t;
        int step = m.step;
        // steps this call may take in the cascade: up to the cap, and no
        // more than the budget (a march that would step past the budget is
        // suspended where it stands)
        const int room = max_steps - step;
        const int last = step + (budget < room ? budget : room);
        // the step loop (MarchDiv): with kDivSplit compiled twice, with
        // multiplies alone when the cascade's divisors and the volume sizes
        // are all powers of two and with the corrected quotients otherwise
        // (the choice is the cascade's, outside the loop); once for kernels
        // whose registers cannot hold two copies without spilling
        auto steps = [&](auto mode) -> bool {
            constexpr int M = decltype(mode)::value;
            constexpr bool P2 = M == kStepPow2;
            for (; step < last && t < m.is_y; ++step) {
                const f3 sp = add3(wpos, mul3(dir, t));
                // getGlobalSDFCascadeUV (SDFCommon.glsl:64-71)
                // (with a power-of-two extent the quotient is an exact
                // scaling, so one FMA rounds like the multiply and the add)
                const float ux = clampf(P2 ? fmaf(sp.x - cx, div_md.y, 0.5f) : qdiv<M>(sp.x - cx, div_md) + 0.5f,
                                        0.0f, 1.0f);
                const float uy = clampf(P2 ? fmaf(sp.y - cy, div_md.y, 0.5f) : qdiv<M>(sp.y - cy, div_md) + 0.5f,
                                        0.0f, 1.0f);
                const float uz = clampf(P2 ? fmaf(sp.z - cz, div_md.y, 0.5f) : qdiv<M>(sp.z - cz, div_md) + 0.5f,
                                        0.0f, 1.0f);
                const float cu = float(cascade) + ux;
                const float tu = qdiv<M>(cu, div_c);
                // the full-resolution taps are issued together with the mip taps
                // (one memory round trip per step) unless the cell minima show
                // their value cannot be used; it is used only where
                // SDFCommon.glsl:150-158 samples the full-resolution SDF
                float sd, sdt;
                if (QTEX == kQuad || QTEX == kGather) {
                    // texel coordinates u W - 0.5 of the full-resolution (f)
                    // and mip (g) volumes.  With power-of-two sizes and
                    // divisors tu W = cu res exactly (tu = cu / C, W = res C),
                    // so one FMA rounds like the multiply and the subtraction.
                    float fx, fy, fz, gx, gy, gz;
                    if constexpr (P2) {
                        const float r = float(s.res), mr = float(s.mres);
                        fx = fmaf(cu, r, -0.5f); fy = fmaf(uy, r, -0.5f); fz = fmaf(uz, r, -0.5f);
                        gx = fmaf(cu, mr, -0.5f); gy = fmaf(uy, mr, -0.5f); gz = fmaf(uz, mr, -0.5f);
                    } else {
                        fx = tu * float(TW) - 0.5f; fy = uy * float(s.res) - 0.5f; fz = uz * float(s.res) - 0.5f;
                        gx = tu * float(MW) - 0.5f; gy = uy * float(s.mres) - 0.5f; gz = uz * float(s.mres) - 0.5f;
                    }
                    // the cell test and the quad / gather sample share the floors
                    // of the full-resolution texel coordinates
                    const float lx = floorf(fx), ly = floorf(fy), lz = floorf(fz);
                    const int ix = int(lx), iy = int(ly), iz = int(lz);
                    const bool need_fine = fine_needed_at(s, ix, iy, iz);
                    // tu, uy, uz lie in [0, 1] (clamped above; tu = (cascade + ux) / C),
                    // so the floors lie in [-1, W - 1] (a NaN converts to 0)
                    const float mlx = floorf(gx), mly = floorf(gy), mlz = floorf(gz);
                    if (QMIP == kQuad)
                        sd = quad_lerp_unit<T>(static_cast<const typename Quad<T>::type*>(s.mip_quad), MW, s.mres, s.mres,
                                               gx - mlx, gy - mly, gz - mlz, int(mlx), int(mly), int(mlz));
                    else if (QMIP == kGather)
                        sd = gather_lerp<T>(s.mip_g, MW, s.mres, s.mres, gx - mlx, gy - mly, gz - mlz, int(mlx), int(mly),
                                            int(mlz));
                    else
                        sd = sample_vol<T, QMIP>(s.mip, s.mip_quad, s.mip_g, MW, s.mres, s.mres, tu, uy, uz);
                    if (!need_fine)
                        sdt = 1.0f;
                    else if (QTEX == kGather)
                        sdt = gather_lerp<T>(s.sdf_g, TW, s.res, s.res, fx - lx, fy - ly, fz - lz, ix, iy, iz);
                    else
                        sdt = quad_lerp_unit<T>(static_cast<const typename Quad<T>::type*>(s.sdf_quad), TW, s.res, s.res,
                                                fx - lx, fy - ly, fz - lz, ix, iy, iz);
                } else {
                    const bool need_fine = fine_needed(s, tu, uy, uz);
                    if (QMIP == kPlain)
                        sd = sample3d_unit<T>(static_cast<const T*>(s.mip), MW, s.mres, s.mres, tu, uy, uz);
                    else if (QMIP == kQuad)
                        sd = sample3d_quad_unit<T>(static_cast<const typename Quad<T>::type*>(s.mip_quad), MW, s.mres,
                                                   s.mres, tu, uy, uz);
                    else
                        sd = sample_vol<T, QMIP>(s.mip, s.mip_quad, s.mip_g, MW, s.mres, s.mres, tu, uy, uz);
                    if (!need_fine)
                        sdt = 1.0f;
                    else if (QTEX == kPlain)
                        sdt = sample3d_unit<T>(static_cast<const T*>(s.sdf), TW, s.res, s.res, tu, uy, uz);
                    else
                        sdt = sample_vol<T, QTEX>(s.sdf, s.sdf_quad, s.sdf_g, TW, s.res, s.res, tu, uy, uz);
                }
                if (sd < chunk) {
                    ++m.fine;
                    if (sdt < margin * 2.0f) sd = sdt;
                } else {
                    sd = chunk;
                }
                sd = sd * md;
                const float thick = voxel_half * clampf(qdiv<M>(t, div_voxel), 0.0f, 1.0f);
                if (sd < thick) {
                    hit.time = mx(t + sd - thick, 0.0f);
                    hit.cascade = cascade;
                    hit.sdf = sd;
                    hit.normal = f3{0.0f, 0.0f, 0.0f};
                    hit.u = tu;
                    hit.v = uy;
                    hit.w = uz;
                    hit.steps = m.steps + step;
                    hit.fine = m.fine;
                    return true;
                }
                t = t + mx(sd * 1.0f, voxel);
            }
            return false;
        };
        if constexpr (DIV == kDivSplit) {
            const bool pow2 = div_md.pow2 && div_c.pow2 && div_voxel.pow2 && (s.res & (s.res - 1)) == 0 &&
                              (s.mres & (s.mres - 1)) == 0;
            if (pow2 ? steps(std::integral_constant<int, kStepPow2>{})
                     : steps(std::integral_constant<int, kStepExact>{}))
                return true;
        } else if constexpr (DIV == kDivSelect) {
            if (steps(std::integral_constant<int, kStepSelect>{})) return true;
        } else {
            if (steps(std::integral_constant<int, kStepExact>{})) return true;
        }
        if (step < max_steps && t < m.is_y) {
            // the budget ran out first
            m.t = t;
            m.step = step;
            return false;
        }
        budget -= step - m.step;
        m.steps += step;
        m.in_cascade = 0;
    }
    hit.normal = f3{0.0f, 0.0f, 0.0f};
    hit.time = -1.0f;
    hit.cascade = 0;
    hit.sdf = 0.0f;
    hit.steps = m.steps;
    hit.fine = m.fine;
    hit.u = hit.v = hit.w = 0.0f;
    return true;
}

// Hit normal of an ended march (SDFCommon.glsl:174-183): central
// differences at the hit sample's texture coordinates; zero for a miss.
template <typename T, int QTEX>
__device__ __forceinline__ void march_hit_normal(const SdfView& s, MarchHit& hit) {
    if (hit.time >= 0.0f)
        hit.normal = sdf_normal<T, QTEX>(s.sdf, s.sdf_quad, s.sdf_g, s.res * s.C, s.res, hit.u, hit.v, hit.w,
                                         s.texel);
}

// The whole march in one call.
template <typename T, int QMIP = kPlain, int QTEX = kPlain>
__device__ __forceinline__ MarchHit march_sdf(const SdfView& s, f3 origin, f3 dir, float trace_max, int max_steps) {
    MarchState m;
    march_state_init(m);
    MarchHit hit;
    march_run<T, QMIP, QTEX>(s, origin, dir, trace_max, max_steps, m, 0x7FFFFFFF, hit);
    march_hit_normal<T, QTEX>(s, hit);
    return hit;
}

// ------------------------------------------------ surface atlas sampling
// ------------------------------------------------ packed R11G11B10F colour
// The unsigned small floats of the R11G11B10F format, written from the
// format's definition: a 5-bit exponent with bias 15 and an M-bit mantissa
// (M = 6 for R and G, 5 for B), no sign.  Exponent 0 holds the denormals
// m * 2^-(14 + M), exponent 31 Inf (m = 0) or NaN.  Encoding rounds to
// nearest, ties to even; negative values and -0 become 0, NaN stays NaN, a
// finite value that rounds past the largest finite one becomes Inf.
template <int M>
__device__ __forceinline__ float ufloat_decode(uint32_t v) {
    const uint32_t e = v >> M, m = v & ((1u << M) - 1u);
    if (e == 0u) return float(m) * __uint_as_float(uint32_t(127 - 14 - M) << 23);   // m * 2^-(14+M), exact
    if (e == 31u) return __uint_as_float(m ? 0x7FC00000u : 0x7F800000u);
    return __uint_as_float(((e + 112u) << 23) | (m << (23 - M)));
}
template <int M>
__device__ __forceinline__ uint32_t ufloat_encode(float x) {
    if (x != x) return (31u << M) | ((1u << M) - 1u);
    if (!(x > 0.0f)) return 0u;
    const uint32_t b = __float_as_uint(x);
    if (b >= 0x7F800000u) return 31u << M;
    if (b < (113u << 23)) {
        // below 2^-14: a multiple of 2^-(14+M) (the power-of-two scale is
        // exact); a result of 2^M is the smallest normal's code
        return uint32_t(rintf(__fmul_rn(x, __uint_as_float(uint32_t(127 + 14 + M) << 23))));
    }
    constexpr uint32_t sh = 23 - M;
    const uint32_t r = (b + ((1u << (sh - 1)) - 1u) + ((b >> sh) & 1u)) >> sh;   // (exponent << M) | mantissa
    const uint32_t e = (r >> M) - 112u;                                             // rebias 127 -> 15
    return e >= 31u ? (31u << M) : ((e << M) | (r & ((1u << M) - 1u)));
}
__device__ __forceinline__ uint32_t pack_r11g11b10(float r, float g, float b) {
    return ufloat_encode<6>(r) | (ufloat_encode<6>(g) << 11) | (ufloat_encode<5>(b) << 22);
}
__device__ __forceinline__ void unpack_r11g11b10(uint32_t v, float* out) {
    out[0] = ufloat_decode<6>(v & 0x7FFu);
    out[1] = ufloat_decode<6>((v >> 11) & 0x7FFu);
    out[2] = ufloat_decode<5>(v >> 22);
}

// One texel of a surface colour texture (luxgi_color_format): rgba, alpha 1
// for R11G11B10F.  color_texel_ro reads through the read-only cache.
__device__ __forceinline__ void color_texel_ro(const void* p, int fmt, size_t texel, float* out) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        unpack_r11g11b10(__ldg(static_cast<const uint32_t*>(p) + texel), out);
        out[3] = 1.0f;
    } else {
        const uint2 raw = __ldg(static_cast<const uint2*>(p) + texel);
        const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
        const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
        out[0] = __low2float(a); out[1] = __high2float(a); out[2] = __low2float(b); out[3] = __high2float(b);
    }
}
__device__ __forceinline__ void color_texel(const void* p, int fmt, size_t texel, float* out) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        unpack_r11g11b10(static_cast<const uint32_t*>(p)[texel], out);
        out[3] = 1.0f;
    } else {
        const uint2 raw = static_cast<const uint2*>(p)[texel];
        const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
        const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
        out[0] = __low2float(a); out[1] = __high2float(a); out[2] = __low2float(b); out[3] = __high2float(b);
    }
}
// Stores rgba (alpha dropped for R11G11B10F), rounded to the format.
__device__ __forceinline__ void color_store(void* p, int fmt, size_t texel, const float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        static_cast<uint32_t*>(p)[texel] = pack_r11g11b10(v[0], v[1], v[2]);
    } else {
        const __half2 a = __floats2half2_rn(v[0], v[1]);
        const __half2 b = __floats2half2_rn(v[2], v[3]);
        uint2 raw;
        raw.x = *reinterpret_cast<const uint32_t*>(&a);
        raw.y = *reinterpret_cast<const uint32_t*>(&b);
        static_cast<uint2*>(p)[texel] = raw;
    }
}
// The value a render target of format `fmt` keeps of v (each channel).
__device__ __forceinline__ void color_round(int fmt, float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        v[0] = ufloat_decode<6>(ufloat_encode<6>(v[0]));
        v[1] = ufloat_decode<6>(ufloat_encode<6>(v[1]));
        v[2] = ufloat_decode<5>(ufloat_encode<5>(v[2]));
        v[3] = 1.0f;
    } else {
#pragma unroll
        for (int c = 0; c < 4; ++c) v[c] = __half2float(__float2half_rn(v[c]));
    }
}

struct SurfaceView {
    luxgi_surface_data data;
    const luxgi_surface_object* objects;
    const float* w2l;         // [objects][16] inverse(object.transform), precomputed; or nullptr
    const luxgi_surface_tile* tiles;
    const uint32_t* chunks;
    const uint32_t* culled;
    const void* color0;       // light cache (mode A) or direct light (mode B)
    int color0_format;        // luxgi_color_format of color0
    const uint8_t* color1;    // albedo RGBA8 (mode B)
    const float* depth;
    float inv_chunk;          // 1 / data.chunk_size (the march's shading bins)
};

// Exact FP32 arithmetic (round to nearest, never contracted into an FMA,
// IEEE division and square root) whatever the translation unit's flags.
// The hard cut-offs of the surface sampler (chunk of the hit point, object
// bounding sphere, OBB margin) are computed with these, like the CPU
// restatement computes them, so that a hit point lying within an ulp of a
// cut-off is classified the same way; the continuous weights around them
// may use the fast forms.
__device__ __forceinline__ f3 mat4_mul_pt_rn(const float* m, f3 v, float w) {
    return f3{__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[4], v.y)), __fmul_rn(m[8], v.z)),
                        __fmul_rn(m[12], w)),
              __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[1], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[9], v.z)),
                        __fmul_rn(m[13], w)),
              __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[2], v.x), __fmul_rn(m[6], v.y)), __fmul_rn(m[10], v.z)),
                        __fmul_rn(m[14], w))};
}
__device__ __forceinline__ float len3_rn(f3 a) {
    return __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)), __fmul_rn(a.z, a.z)));
}
// a + d * t per component, exact (the hit point of a march record)
__device__ __forceinline__ f3 ray_point_rn(f3 a, f3 d, float t) {
    return f3{__fadd_rn(a.x, __fmul_rn(d.x, t)), __fadd_rn(a.y, __fmul_rn(d.y, t)), __fadd_rn(a.z, __fmul_rn(d.z, t))};
}

__device__ __forceinline__ f3 mat4_mul_pt(const float* m, f3 v, float w) {
    return f3{m[0] * v.x + m[4] * v.y + m[8] * v.z + m[12] * w,
              m[1] * v.x + m[5] * v.y + m[9] * v.z + m[13] * w,
              m[2] * v.x + m[6] * v.y + m[10] * v.z + m[14] * w};
}

// 4x4 inverse by adjugate (same cofactor sequence as the CPU restatement).
__device__ __forceinline__ void mat4_inverse(const float* A, float* out) {
    float a[4][4];
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int r = 0; r < 4; ++r) a[r][c] = A[c * 4 + r];
    const float s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    const float s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const float s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    const float s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const float s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    const float s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const float c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    const float c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const float c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    const float c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const float c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    const float c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const float id = 1.0f / det;
    float b[4][4];
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
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = b[r][c];
}

// textureGather texel indices (clamp to edge): (i0,j1),(i1,j1),(i1,j0),(i0,j0)
struct Gather4 { int i0, i1, j0, j1; };
__device__ __forceinline__ Gather4 gather_idx(float u, float v, int W, int H) {
    const float x = __fadd_rn(__fmul_rn(u, float(W)), -0.5f), y = __fadd_rn(__fmul_rn(v, float(H)), -0.5f);
    int i0 = int(floorf(x)), j0 = int(floorf(y));
    Gather4 g;
    g.i1 = imn(imx(i0 + 1, 0), W - 1);
    g.j1 = imn(imx(j0 + 1, 0), H - 1);
    g.i0 = imn(imx(i0, 0), W - 1);
    g.j0 = imn(imx(j0, 0), H - 1);
    return g;
}

// sampleGlobalSurfaceAtlasTile, both overloads (AtlasCommon.glsl:58-112);
// accumulates colour*weight of one or two atlases.
template <bool TWO>
__device__ __forceinline__ void sample_tile(const SurfaceView& S, const luxgi_surface_tile* __restrict__ tl, f3 local,
                                            f3 nrm_local, float thr, f3& acc0, f3& acc1, float& accw) {
    float T[16];
    {
        // 96-byte tile records: the matrix sits at a 16-byte-aligned offset
        const float4* src = reinterpret_cast<const float4*>(tl->transform);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float4 c = __ldg(src + k);
            T[4 * k] = c.x; T[4 * k + 1] = c.y; T[4 * k + 2] = c.z; T[4 * k + 3] = c.w;
        }
    }
    const f3 n = norm3(mat4_mul_pt(T, nrm_local, 1.0f));
    float nw = clampf(0.0f * n.x + 0.0f * n.y + 1.0f * n.z, 0.0f, 1.0f);
    nw = (nw - 0.05f) * (1.0f / (1.0f - 0.05f));
    if (nw <= 0.0f) return;
    // The atlas coordinate (au, av) exactly: the reference takes the
    // bilinear fractions from fract(au * res + 0.5) but the gathered texels
    // from textureGather's own floor(au * res - 0.5), so at a texel boundary
    // an ulp of au can pair the fractions with the neighbouring texels; au is
    // computed like the restatement computes it (tile-space x / y, IEEE
    // division by the bounds, no contraction), so both sides pair them alike.
    // The depth (continuous through the visibility ramp) may round freely.
    const float bx = __ldg(&tl->object_bounds[0]), by = __ldg(&tl->object_bounds[1]), bz = __ldg(&tl->object_bounds[2]);
    const float tpx = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[0], local.x), __fmul_rn(T[4], local.y)),
                                          __fmul_rn(T[8], local.z)), T[12]);
    const float tpy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[1], local.x), __fmul_rn(T[5], local.y)),
                                          __fmul_rn(T[9], local.z)), T[13]);
    const float tpz = T[2] * local.x + T[6] * local.y + T[10] * local.z + T[14];
    const float ibz = 1.0f / bz;
    const float tdepth = tpz * ibz;
    const float tu = clampf(__fadd_rn(__fdiv_rn(tpx, bx), 0.5f), 0.0f, 1.0f);
    const float tv = clampf(__fadd_rn(__fdiv_rn(tpy, by), 0.5f), 0.0f, 1.0f);
    const float au = __fadd_rn(__fmul_rn(tu, __ldg(&tl->extends[2])), __ldg(&tl->extends[0]));
    const float av = __fadd_rn(__fmul_rn(tv, __ldg(&tl->extends[3])), __ldg(&tl->extends[1]));
    const float res = float(S.data.resolution);
    float bu = __fadd_rn(__fmul_rn(au, res), 0.5f); bu = bu - floorf(bu);
    float bv = __fadd_rn(__fmul_rn(av, res), 0.5f); bv = bv - floorf(bv);
    const float bw0 = (1.0f - bu) * bv, bw1 = bu * bv, bw2 = bu * (1.0f - bv), bw3 = (1.0f - bu) * (1.0f - bv);
    const int R = int(S.data.resolution);
    const Gather4 g = gather_idx(au, av, R, R);
    const size_t o0 = size_t(g.j1) * R + g.i0, o1 = size_t(g.j1) * R + g.i1;
    const size_t o2 = size_t(g.j0) * R + g.i1, o3 = size_t(g.j0) * R + g.i0;
    const float tz[4] = {__ldg(S.depth + o0), __ldg(S.depth + o1), __ldg(S.depth + o2), __ldg(S.depth + o3)};
    // the visibility ramp (|depth difference| - dthr) / (dthr / 2), with the
    // reciprocals taken once a tile (shading compares by tolerance)
    const float dthr = 2.0f * thr * ibz, idr = 1.0f / (thr * ibz);
    float dv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        dv[i] = 1.0f - clampf((fabsf(tdepth - tz[i]) - dthr) * idr, 0.0f, 1.0f);
        if (tz[i] >= 1.0f) dv[i] = 0.0f;
    }
    float sw = dv[0] * bw0 + dv[1] * bw1 + dv[2] * bw2 + dv[3] * bw3;
    sw = sw * nw;
    if (sw <= 0.0f) return;
    const float w0 = bw0 * dv[0], w1 = bw1 * dv[1], w2 = bw2 * dv[2], w3 = bw3 * dv[3];
    const size_t offs[4] = {o0, o1, o2, o3};
    float ch[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i) color_texel_ro(S.color0, S.color0_format, offs[i], ch[i]);
    const f3 c0{ch[0][0] * w0 + ch[1][0] * w1 + ch[2][0] * w2 + ch[3][0] * w3,
                ch[0][1] * w0 + ch[1][1] * w1 + ch[2][1] * w2 + ch[3][1] * w3,
                ch[0][2] * w0 + ch[1][2] * w1 + ch[2][2] * w2 + ch[3][2] * w3};
    acc0 = add3(acc0, mul3(c0, sw));
    if (TWO) {
        // RGBA8 albedo: the bytes weighted, the 1/255 applied once
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uchar4 a = __ldg(reinterpret_cast<const uchar4*>(S.color1) + offs[i]);
            ch[i][0] = float(a.x); ch[i][1] = float(a.y); ch[i][2] = float(a.z);
        }
        const f3 c1{ch[0][0] * w0 + ch[1][0] * w1 + ch[2][0] * w2 + ch[3][0] * w3,
                    ch[0][1] * w0 + ch[1][1] * w1 + ch[2][1] * w2 + ch[3][1] * w3,
                    ch[0][2] * w0 + ch[1][2] * w1 + ch[2][2] * w2 + ch[3][2] * w3};
        acc1 = add3(acc1, mul3(c1, sw * (1.0f / 255.0f)));
    }
    accw = accw + sw;
}

// sampleGlobalSurfaceAtlas (AtlasCommon.glsl:115-157), debug off.
template <bool TWO>
__device__ __forceinline__ float sample_surface(const SurfaceView& S, f3 pos, f3 wn, float thr, f3& out0, f3& out1) {
    f3 acc0{0.0f, 0.0f, 0.0f}, acc1{0.0f, 0.0f, 0.0f};
    float accw = 0.0f;
    out0 = acc0;
    out1 = acc1;
    const float cs = S.data.chunk_size;
    const float half_res = float(kChunksRes * 0.5f);
    const int cx = imn(imx(int(floorf(__fadd_rn(__fdiv_rn(pos.x, cs), half_res))), 0), kChunksRes - 1);
    const int cy = imn(imx(int(floorf(__fadd_rn(__fdiv_rn(pos.y, cs), half_res))), 0), kChunksRes - 1);
    const int cz = imn(imx(int(floorf(__fadd_rn(__fdiv_rn(pos.z, cs), half_res))), 0), kChunksRes - 1);
    const uint32_t addr = uint32_t(cz * kChunksRes * kChunksRes + cy * kChunksRes + cx);
    uint32_t start = __ldg(S.chunks + addr);
    if (start == 0) return 0.0f;
    const uint32_t count = __ldg(S.culled + start);
    if (count > S.data.objects_count) return 0.0f;
    ++start;
    for (uint32_t oi = 0; oi < count; ++oi) {
        const uint32_t oaddr = __ldg(S.culled + start++);
        const luxgi_surface_object* ob = S.objects + oaddr;
        const float4 bnd = __ldg(reinterpret_cast<const float4*>(ob->object_bounds));
        if (len3_rn(sub3(f3{bnd.x, bnd.y, bnd.z}, pos)) > bnd.w) continue;
        float w2l[16];
        if (S.w2l) {
            // inverse(object.transform), computed once per scene by the same
            // mat4_inverse (AtlasCommon.glsl:134 recomputes it per ray)
            const float4* src = reinterpret_cast<const float4*>(S.w2l + size_t(oaddr) * 16);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float4 c = __ldg(src + k);
                w2l[4 * k] = c.x; w2l[4 * k + 1] = c.y; w2l[4 * k + 2] = c.z; w2l[4 * k + 3] = c.w;
            }
        } else {
            float M[16];
#pragma unroll
            for (int k = 0; k < 16; ++k) M[k] = __ldg(&ob->transform[k]);
            mat4_inverse(M, w2l);
        }
        const f3 lp = mat4_mul_pt_rn(w2l, pos, 1.0f);
        const float4 e = __ldg(reinterpret_cast<const float4*>(ob->extends));
        if (fabsf(lp.x) > __fadd_rn(e.x, thr) || fabsf(lp.y) > __fadd_rn(e.y, thr) || fabsf(lp.z) > __fadd_rn(e.z, thr))
            continue;
        const f3 ln = norm3(f3{w2l[0] * wn.x + w2l[4] * wn.y + w2l[8] * wn.z,
                               w2l[1] * wn.x + w2l[5] * wn.y + w2l[9] * wn.z,
                               w2l[2] * wn.x + w2l[6] * wn.y + w2l[10] * wn.z});
        for (int i = 0; i < 6; ++i) {
            const uint32_t to = __ldg(&ob->tile_offset[i]);
            if (to != 0) sample_tile<TWO>(S, S.tiles + to, lp, ln, thr, acc0, acc1, accw);
        }
    }
    const float iden = 1.0f / mx(accw, 0.0001f);
    out0 = mul3(acc0, iden);
    out1 = mul3(acc1, iden);
    return accw;
}

// ------------------------------------------------ probe atlas sampling
struct AtlasView {
    const void* irr;
    const void* dist;
    int storage;   // luxgi_storage
};

__device__ __forceinline__ float atlas_load(const void* p, int storage, size_t i) {
    if (storage == LUXGI_STORAGE_FP16) return __half2float(__ldg(static_cast<const __half*>(p) + i));
    return __ldg(static_cast<const float*>(p) + i);
}

// GL REPEAT of texel index i over n texels: i mod n in [0, n).  The texel
// coordinates of the probe atlases stay within one period of the atlas, so
// the remainder is almost never needed.
__device__ __forceinline__ int wrap_repeat(int i, int n) {
    if (i >= 0 && i < n) return i;
    if (i < 0 && i >= -n) return i + n;
    if (i >= n && i < 2 * n) return i - n;
    const int r = i % n;
    return r < 0 ? r + n : r;
}

// textureLod bilinear with REPEAT of channel ch (nc channels per texel).
__device__ __forceinline__ float bilinear_repeat(const void* p, int storage, int W, int H, int nc, float u, float v, int ch) {
    const float x = u * float(W) - 0.5f, y = v * float(H) - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const int i0 = wrap_repeat(int(fx), W), i1 = wrap_repeat(int(fx) + 1, W);
    const int j0 = wrap_repeat(int(fy), H), j1 = wrap_repeat(int(fy) + 1, H);
    const float t00 = atlas_load(p, storage, (size_t(j0) * W + i0) * nc + ch);
    const float t10 = atlas_load(p, storage, (size_t(j0) * W + i1) * nc + ch);
    const float t01 = atlas_load(p, storage, (size_t(j1) * W + i0) * nc + ch);
    const float t11 = atlas_load(p, storage, (size_t(j1) * W + i1) * nc + ch);
    const float r0 = t00 * (1.0f - a) + t10 * a, r1 = t01 * (1.0f - a) + t11 * a;
    return r0 * (1.0f - b) + r1 * b;
}

// All NC channels of one atlas texel in one load (NC = 4 irradiance, 2 distance).
template <int NC>
__device__ __forceinline__ void atlas_texel(const void* p, int storage, size_t texel, float* out) {
    if (storage == LUXGI_STORAGE_FP16) {
        if (NC == 4) {
            const uint2 raw = __ldg(static_cast<const uint2*>(p) + texel);
            const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
            const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
            out[0] = __low2float(a); out[1] = __high2float(a); out[2] = __low2float(b); out[3] = __high2float(b);
        } else {
            const __half2 a = __ldg(static_cast<const __half2*>(p) + texel);
            out[0] = __low2float(a); out[1] = __high2float(a);
        }
    } else {
        if (NC == 4) {
            const float4 v = __ldg(static_cast<const float4*>(p) + texel);
            out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
        } else {
            const float2 v = __ldg(static_cast<const float2*>(p) + texel);
            out[0] = v.x; out[1] = v.y;
        }
    }
}

// textureLod bilinear with REPEAT, all NC channels (same per-channel
// arithmetic as bilinear_repeat).
template <int NC>
__device__ __forceinline__ void bilinear_repeat_v(const void* p, int storage, int W, int H, float u, float v, float* out) {
    const float x = u * float(W) - 0.5f, y = v * float(H) - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const int i0 = wrap_repeat(int(fx), W), i1 = wrap_repeat(int(fx) + 1, W);
    const int j0 = wrap_repeat(int(fy), H), j1 = wrap_repeat(int(fy) + 1, H);
    float t00[NC], t10[NC], t01[NC], t11[NC];
    atlas_texel<NC>(p, storage, size_t(j0) * W + i0, t00);
    atlas_texel<NC>(p, storage, size_t(j0) * W + i1, t10);
    atlas_texel<NC>(p, storage, size_t(j1) * W + i0, t01);
    atlas_texel<NC>(p, storage, size_t(j1) * W + i1, t11);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const float r0 = t00[c] * (1.0f - a) + t10[c] * a, r1 = t01[c] * (1.0f - a) + t11[c] * a;
        out[c] = r0 * (1.0f - b) + r1 * b;
    }
}


// textureCoordFromDirection (DDGICommon.glsl:141-158) in texel units: the
// shader forms a UV normalised by the atlas size, (cell corner + octEncode
// offset) / W, and the sampler turns it back into texels, u * W - 0.5, which
// FP32 resolves only to W x 6e-8 texel (2e-3 texel in a 32,770-texel-wide
// atlas).  Here the cell corner (an integer) and the offset inside the cell
// are kept apart: oct_cell_point gives the sample point inside the cell,
// (octEncode(d) + 1) / 2 * side - 0.5 per axis, and bilinear_at_t adds the
// corner after the floor, so the bilinear fractions keep FP32's precision
// (~1e-7 texel).  The texels and weights are those of the shader's formula
// evaluated exactly.
__device__ __forceinline__ float sign_nz(float k) { return k >= 0.0f ? 1.0f : -1.0f; }

__device__ __forceinline__ void oct_cell_point(f3 d, int side, float& rx, float& ry) {
    const float l1 = fabsf(d.x) + fabsf(d.y) + fabsf(d.z);
    const float inv = 1.0f / l1;
    float ox = d.x * inv, oy = d.y * inv;
    if (d.z < 0.0f) {
        const float tx = (1.0f - fabsf(oy)) * sign_nz(ox);
        const float ty = (1.0f - fabsf(ox)) * sign_nz(oy);
        ox = tx; oy = ty;
    }
    rx = (ox + 1.0f) * 0.5f * float(side) - 0.5f;
    ry = (oy + 1.0f) * 0.5f * float(side) - 0.5f;
}

// A bilinear tap at texel (x0 + rx, y0 + ry) of an atlas, (x0, y0) the
// interior corner of a probe cell (cell * (side + 2) + 2) and (rx, ry) from
// oct_cell_point.  rx lies in [-0.5, side - 0.5], so the four texels stay
// inside the cell and its 1-texel border (the clamp only guards a NaN
// direction, which converts to the cell's first texel).  tap_frac splits the
// point into its texel corner and fractions, which a direction shared by
// several cells (sampleIrradiance's normal) computes once.
struct TapFrac {
    int ix, iy;   // texel corner relative to the cell's interior corner
    float a, b;   // fractions
};

__device__ __forceinline__ TapFrac tap_frac(int side, float rx, float ry) {
    const float fx = fminf(fmaxf(floorf(rx), -1.0f), float(side - 1));
    const float fy = fminf(fmaxf(floorf(ry), -1.0f), float(side - 1));
    TapFrac f;
    f.ix = int(fx);
    f.iy = int(fy);
    f.a = rx - fx;
    f.b = ry - fy;
    return f;
}

// One texel's NC channels (NC = 4 irradiance, 2 distance) at p, one load.
template <int NC>
__device__ __forceinline__ void texel_ld(const float* p, float* out) {
    if (NC == 4) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(p));
        out[0] = v.x; out[1] = v.y; out[2] = v.z; out[3] = v.w;
    } else {
        const float2 v = __ldg(reinterpret_cast<const float2*>(p));
        out[0] = v.x; out[1] = v.y;
    }
}
template <int NC>
__device__ __forceinline__ void texel_ld(const __half* p, float* out) {
    if (NC == 4) {
        const uint2 raw = __ldg(reinterpret_cast<const uint2*>(p));
        const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
        const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
        out[0] = __low2float(a); out[1] = __high2float(a); out[2] = __low2float(b); out[3] = __high2float(b);
    } else {
        const __half2 a = __ldg(reinterpret_cast<const __half2*>(p));
        out[0] = __low2float(a); out[1] = __high2float(a);
    }
}

// Bilinear tap of NC channels at texel (x0 + f.ix, y0 + f.iy) .. + 1 of an
// atlas of element ST with `row` elements a texel row.  Both texel indices
// are >= 0 (x0, y0 >= 2, f.ix, f.iy >= -1), so the two row pointers come
// from unsigned 32 x 64-bit products and the second texel of a row is the
// next one: four loads off two pointers.
template <int NC, typename ST>
__device__ __forceinline__ void bilinear_at_t(const ST* __restrict__ base, size_t row, uint32_t x0, uint32_t y0,
                                              const TapFrac& f, float* out) {
    const ST* r0 = base + size_t(y0 + uint32_t(f.iy)) * row + size_t(x0 + uint32_t(f.ix)) * NC;
    const ST* r1 = r0 + row;
    const float a = f.a, b = f.b;
    float t00[NC], t10[NC], t01[NC], t11[NC];
    texel_ld<NC>(r0, t00);
    texel_ld<NC>(r0 + NC, t10);
    texel_ld<NC>(r1, t01);
    texel_ld<NC>(r1 + NC, t11);
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        const float r0c = t00[c] * (1.0f - a) + t10[c] * a, r1c = t01[c] * (1.0f - a) + t11[c] * a;
        out[c] = r0c * (1.0f - b) + r1c * b;
    }
}

// pow(x, e) of the irradiance decode; x*x*sqrt(x) for the default gamma
// (e = 2.5), within 1.5 ulp of powf
__device__ __forceinline__ float pow_decode(float x, float e) {
    return (e == 2.5f) ? x * x * sqrtf(x) : powf(x, e);
}

// sampleIrradiance (DDGICommon.glsl:163-233) over atlases of element ST.
// The normal-bias vector and the octahedral coordinate of N (its texel
// corner and fractions in every irradiance cell) are the same for the 8
// cage probes and are computed once, and so are, per axis, the two
// candidate grid coordinates, their positions and their trilinear weights
// (the same expressions the shader evaluates per probe).
// FAST (hit shading, compared by tolerance): the probe-to-point direction is
// normalised once and the distance taken from the same reciprocal root.
template <int UNROLL, bool FAST, typename ST>
__device__ __forceinline__ f3 sample_irradiance_t(const luxgi_ddgi_uniform& u, const ST* __restrict__ irr,
                                                  const ST* __restrict__ dist_atlas, f3 P, f3 N, f3 Wo) {
    const float start[3] = {u.start_position[0], u.start_position[1], u.start_position[2]};
    const float stp[3] = {u.step[0], u.step[1], u.step[2]};
    const float pk[3] = {P.x, P.y, P.z};
    float plo[3], phi[3], wlo[3], whi[3];
    int glo[3], ghi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int cnt = u.probe_counts[k];
        const int base = imn(imx(int((pk[k] - start[k]) / stp[k]), 0), cnt - 1);
        const float bpos = stp[k] * float(base) + start[k];
        const float alpha = clampf((pk[k] - bpos) / stp[k], 0.0f, 1.0f);
        // probe coordinate base + off, off in {0, 1}, clamped to the grid
        glo[k] = base;
        ghi[k] = imn(base + 1, cnt - 1);
        plo[k] = bpos;
        phi[k] = stp[k] * float(ghi[k]) + start[k];
        wlo[k] = 1.0f - alpha;
        whi[k] = alpha;
    }
    f3 sum{0.0f, 0.0f, 0.0f};
    float sumw = 0.0f;
    const float ge = u.ddgi_gamma * 0.5f;
    const f3 vb = mul3(add3(N, mul3(Wo, 3.0f)), u.normal_bias);
    // textureCoordFromDirection(normalize(N), ...) (DDGICommon.glsl:213): the
    // point inside every cage probe's irradiance cell
    float nrx, nry;
    oct_cell_point(norm3(N), u.irradiance_probe_side, nrx, nry);
    const TapFrac nf = tap_frac(u.irradiance_probe_side, nrx, nry);
    const int ni = u.irradiance_probe_side, nd = u.depth_probe_side;
    const size_t irow = size_t(u.irradiance_width) * 4, drow = size_t(u.depth_width) * 2;
    const int cnt0 = u.probe_counts[0];
    // UNROLL cage probes per iteration overlap their texel fetches; the sums
    // still accumulate in probe order 0..7
#pragma unroll UNROLL
    for (int i = 0; i < 8; ++i) {
        const bool ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
        const int g0 = ox ? ghi[0] : glo[0], g1 = oy ? ghi[1] : glo[1], g2 = oz ? ghi[2] : glo[2];
        const f3 ppos{ox ? phi[0] : plo[0], oy ? phi[1] : plo[1], oz ? phi[2] : plo[2]};
        const f3 tri{ox ? whi[0] : wlo[0], oy ? whi[1] : wlo[1], oz ? whi[2] : wlo[2]};
        float weight = 1.0f;
        const f3 pd = sub3(ppos, P);
        const f3 dtp = FAST ? mul3(pd, rsqrtf(dot3(pd, pd))) : norm3(pd);
        const float bf = mx(0.0001f, (dot3(dtp, N) + 1.0f) * 0.5f);
        weight = weight * (bf * bf + 0.2f);
        // probe index g0 + g1 X + g2 X Y sits in atlas cell (g0 + g1 X, g2)
        const uint32_t cell_x = uint32_t(g0 + g1 * cnt0), cell_y = uint32_t(g2);
        const f3 ptp = add3(sub3(P, ppos), vb);
        float rx, ry, dist;
        if (FAST) {
            // textureCoordFromDirection(-normalize(-ptp)) normalises ptp once
            // more; here the unit vector and the distance share one
            // reciprocal square root
            const float d2 = dot3(ptp, ptp);
            const float rl = rsqrtf(d2);
            oct_cell_point(mul3(ptp, rl), nd, rx, ry);
            dist = d2 * rl;
        } else {
            const f3 dir = norm3(mul3(ptp, -1.0f));
            oct_cell_point(norm3(mul3(dir, -1.0f)), nd, rx, ry);
            dist = len3(ptp);
        }
        float mm[2];
        bilinear_at_t<2>(dist_atlas, drow, cell_x * uint32_t(nd + 2) + 2u, cell_y * uint32_t(nd + 2) + 2u,
                         tap_frac(nd, rx, ry), mm);
        const float mean = mm[0];
        const float mean2 = mm[1];
        const float variance = fabsf(mean * mean - mean2);
        const float dm = mx(dist - mean, 0.0f);
        float cheb = variance / (variance + dm * dm);
        cheb = mx(cheb * cheb * cheb, 0.0f);
        weight = weight * ((dist <= mean) ? 1.0f : cheb);
        weight = mx(0.000001f, weight);
        float ir[4];
        bilinear_at_t<4>(irr, irow, cell_x * uint32_t(ni + 2) + 2u, cell_y * uint32_t(ni + 2) + 2u, nf, ir);
        const f3 pir{pow_decode(ir[0], ge), pow_decode(ir[1], ge), pow_decode(ir[2], ge)};
        const float crush = 0.2f;
        if (weight < crush) weight = weight * (weight * weight * (1.0f / (crush * crush)));
        weight = weight * (tri.x * tri.y * tri.z);
        sum = add3(sum, mul3(pir, weight));
        sumw = sumw + weight;
    }
    f3 net{sum.x / sumw, sum.y / sumw, sum.z / sumw};
    net = mulv3(net, net);
    return mul3(net, 2.0f * kPi);
}

// sampleIrradiance over the atlases of a volume (FP32 or FP16 texels).
template <int UNROLL = 1, bool FAST = false>
__device__ __forceinline__ f3 sample_irradiance(const luxgi_ddgi_uniform& u, const AtlasView& A, f3 P, f3 N, f3 Wo) {
    if (A.storage == LUXGI_STORAGE_FP16)
        return sample_irradiance_t<UNROLL, FAST>(u, static_cast<const __half*>(A.irr),
                                                 static_cast<const __half*>(A.dist), P, N, Wo);
    return sample_irradiance_t<UNROLL, FAST>(u, static_cast<const float*>(A.irr), static_cast<const float*>(A.dist),
                                             P, N, Wo);
}

}  // namespace luxgi
