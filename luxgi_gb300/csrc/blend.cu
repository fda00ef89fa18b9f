// Probe blend (ProbeUpdate.glsl) as a contraction, and the border copy
// (BorderUpdate.glsl).
//
// Every probe of a volume traces the same R directions in a frame (one
// rotation per frame, DDGIRenderer.cpp:267-272), so the texel x ray weights
//   irradiance  W[t][r] = max(0, D_t . dir_r)                 (ProbeUpdate.glsl:90)
//   distance    W[t][r] = pow(max(0, D_t . dir_r), sharpness) (ProbeUpdate.glsl:88)
// (zeroed below 1e-8, ProbeUpdate.glsl:93) and the normalisers
// 1 / (2 sum_r W[t][r]) are shared by all probes.  The blend is then
//   out[p][t][c] = n[t] * sum_r W[t][r] * ray[p][r][c]
// followed by the gamma encode, the hysteresis mix and the store; the
// border copy is fused into the store (each interior texel writes its
// border mirrors too).
#include <algorithm>

#include <cuda_fp16.h>

#include "atlas_io.cuh"
#include "luxgi_internal.h"

namespace luxgi {


// ------------------------------------------------------------- weights
// One block per texel row, threads over rays: octDecode(normalizedOctCoord)
// (DDGICommon.glsl:74-92) against every ray direction.  The row sum is a
// fixed-order tree reduction (deterministic).  Also writes the FP16 K-major
// weight operands of the tensor-core blend (rows padded with zeros) and
// their own normalisers.
constexpr int kWeightThreads = 128;

__device__ __forceinline__ void weights_row(const BlendParams& p, int row, float (*red)[kWeightThreads]) {
    const luxgi_ddgi_uniform& u = p.u;
    const int ni = u.irradiance_probe_side, nd = u.depth_probe_side;
    const int Ti = ni * ni, Td = nd * nd;
    const int R = p.R;
    const bool tc = p.tcw_irr != nullptr;
    const int rows_i = tc ? p.tc_ni : Ti;       // tensor-core rows are padded (>= T)
    const bool depth = row >= rows_i;
    const int t = depth ? row - rows_i : row;
    const int n = depth ? nd : ni;
    const int T = depth ? Td : Ti;
    __half* tcw = depth ? p.tcw_dist : p.tcw_irr;
    if (t >= T) {                                  // tensor-core padding row
        for (int r = threadIdx.x; r < R; r += blockDim.x) tcw[size_t(t) * R + r] = __float2half_rn(0.0f);
        return;
    }
    const int tx = t % n, ty = t / n;
    const float s = 2.0f / float(n);
    const float ox = (float(tx) + 0.5f) * s - 1.0f, oy = (float(ty) + 0.5f) * s - 1.0f;
    f3 v{ox, oy, 1.0f - fabsf(ox) - fabsf(oy)};
    if (v.z < 0.0f) {
        const float nx = (1.0f - fabsf(v.y)) * sign_nz(v.x);
        const float ny = (1.0f - fabsf(v.x)) * sign_nz(v.y);
        v.x = nx; v.y = ny;
    }
    const f3 td = norm3(v);
    float* w = depth ? p.w_dist : p.w_irr;
    const int Tp = blend_row_pitch(T);          // ray-major rows, padded to whole texel tiles
    const float4* dirs = p.dirs;
    float sum = 0.0f, sum_h = 0.0f;
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const float4 d = __ldg(dirs + r);
        const float c = mx(0.0f, td.x * d.x + td.y * d.y + td.z * d.z);
        float wt = depth ? powf(c, u.sharpness) : c;
        if (!(wt >= 1e-8f)) wt = 0.0f;
        w[size_t(r) * Tp + t] = wt;
        sum = sum + wt;
        if (tc) {
            const __half h = __float2half_rn(wt);
            tcw[size_t(t) * R + r] = h;
            sum_h = sum_h + __half2float(h);
        }
    }
    red[0][threadIdx.x] = sum;
    red[1][threadIdx.x] = sum_h;
    __syncthreads();
    for (int k = kWeightThreads / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) {
            red[0][threadIdx.x] += red[0][threadIdx.x + k];
            red[1][threadIdx.x] += red[1][threadIdx.x + k];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        float* nrm = depth ? p.n_dist : p.n_irr;
        sum = red[0][0];
        sum_h = red[1][0];
        nrm[t] = (sum > 1e-8f) ? 1.0f / (2.0f * sum) : 1.0f;
        if (tc) nrm[T + t] = (sum_h > 1e-8f) ? 1.0f / (2.0f * sum_h) : 1.0f;   // tensor-core normaliser
    }
}

__global__ void __launch_bounds__(kWeightThreads) weights_kernel(const BlendParams p) {
    __shared__ float red[2][kWeightThreads];
    weights_row(p, int(blockIdx.x), red);
}

__global__ void __launch_bounds__(kWeightThreads)
    weights_batch_kernel(const BlendParams* __restrict__ vp, const int* __restrict__ starts, int n) {
    __shared__ float red[2][kWeightThreads];
    const int v = batch_volume(starts, n, int(blockIdx.x));
    weights_row(vp[v], int(blockIdx.x) - __ldg(starts + v), red);
}

// Rows of the weights launch of one volume (texels, or padded tensor-core rows).
int weight_rows(const BlendParams& p) {
    const int Ti = p.u.irradiance_probe_side * p.u.irradiance_probe_side;
    const int Td = p.u.depth_probe_side * p.u.depth_probe_side;
    return p.tcw_irr ? p.tc_ni + p.tc_nd : Ti + Td;
}

cudaError_t launch_weights(const BlendParams& p, cudaStream_t st) {
    weights_kernel<<<weight_rows(p), kWeightThreads, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_weights_batch(const BlendParams* vp, const int* starts, int n, int blocks, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    weights_batch_kernel<<<blocks, kWeightThreads, 0, st>>>(vp, starts, n);
    note_launch();
    return cudaGetLastError();
}

// --------------------------------------------------------------- blend
// Register-tiled contraction: a block takes PB probes and every texel of
// one atlas; each thread owns a tile of kTexelTile consecutive texels x PP
// probes (x 3 or 2 channels) in registers.  Rays go through shared memory
// in chunks of kRayChunk: the weights chunk [r][texel] (copied as float4 from
// the ray-major weight rows) and the ray chunk [r][probe] (rgb, or the
// clamped distance and its square).  Per ray a thread loads one float4 of
// weights and PP ray values and issues kTexelTile x PP x channels FMAs.  Each
// accumulator sums its rays in ascending order with fmaf, as the
// restatement does.
constexpr int kBlendThreads = 256;
constexpr int kRayChunk = 32;
constexpr int kMaxProbesPerBlock = 128;

struct BlendShape {
    int TG;   // texel groups (threads along texels)
    int PG;   // probe groups (threads along probes)
    int PB;   // probes per block
};

__host__ __device__ __forceinline__ BlendShape blend_shape(int T, int PP) {
    BlendShape s;
    s.TG = (T + kTexelTile - 1) / kTexelTile;
    int pg = kBlendThreads / s.TG;
    const int cap = kMaxProbesPerBlock / PP;
    s.PG = pg < 1 ? 1 : (pg > cap ? cap : pg);
    s.PB = s.PG * PP;
    return s;
}

// FP32 rays take the pipelined path: chunks of kPipeChunk rays, two buffers,
// the next chunk's weights and rays copied with cp.async while the current
// chunk's FMAs run (the same shared memory as one 32-ray buffer).
#ifndef LUXGI_BLEND_PIPE_CHUNK
#define LUXGI_BLEND_PIPE_CHUNK 16
#endif
constexpr int kPipeChunk = LUXGI_BLEND_PIPE_CHUNK;

__host__ __device__ __forceinline__ size_t blend_smem_bytes(int T, int PP, bool depth, bool pipelined) {
    const BlendShape s = blend_shape(T, PP);
    const int Tp = s.TG * kTexelTile;
    if (pipelined)
        return 2 * sizeof(float) * kPipeChunk * Tp +
               (depth ? 2 * sizeof(float) * kPipeChunk * s.PB + sizeof(float2) * kPipeChunk * s.PB
                      : 2 * sizeof(float4) * kPipeChunk * s.PB);
    return sizeof(float) * kRayChunk * Tp + size_t(depth ? 8 : 16) * kRayChunk * s.PB;
}

// cp.async of 16 (or 4) bytes global -> shared; src_bytes 0 fills zeros
__device__ __forceinline__ void cp_async16(void* dst, const void* src, int src_bytes) {
    const unsigned d = unsigned(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src, int src_bytes) {
    const unsigned d = unsigned(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(src), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <bool DEPTH> struct RayVal;
template <> struct RayVal<false> { using type = float4; };
template <> struct RayVal<true> { using type = float2; };

// The epilogue of a block: normalise, gamma, hysteresis, store + border
// mirrors (ProbeUpdate.glsl:105-152, BorderUpdate.glsl:136-156).
template <int DEPTH, typename AT, int PP, int NC_ACC>
__device__ __forceinline__ void blend_epilogue(const BlendParams& p, int p0, int tg, int pg, int T, int n, int W,
                                               float (&acc)[PP][kTexelTile][NC_ACC]) {
    const luxgi_ddgi_uniform& u = p.u;
    const int XY = u.probe_counts[0] * u.probe_counts[1];
    const float* nrm = DEPTH ? p.n_dist : p.n_irr;
    const void* prev = DEPTH ? p.prev_dist : p.prev_irr;
    void* out = DEPTH ? p.out_dist : p.out_irr;
    constexpr int NC = DEPTH ? 2 : 4;
    const float h = u.hysteresis;
    const float ig = 1.0f / u.ddgi_gamma;
#pragma unroll
    for (int j = 0; j < PP; ++j) {
        const int pr = p0 + pg * PP + j;
        if (pr >= p.P) continue;
        const int cx = pr % XY, cy = pr / XY;
#pragma unroll
        for (int k = 0; k < kTexelTile; ++k) {
            const int t = tg * kTexelTile + k;
            if (t >= T) continue;
            const int tx = t % n, ty = t / n;
            const float s = __ldg(nrm + t);
            float v[4];
            v[0] = acc[j][k][0] * s;
            v[1] = acc[j][k][1] * s;
            v[2] = DEPTH ? 0.0f : acc[j][k][NC_ACC - 1] * s;
            v[3] = 1.0f;
            if (!DEPTH) {
#pragma unroll
                for (int c = 0; c < 3; ++c) v[c] = powf(v[c], ig);
            }
            const size_t texel = size_t(cy * (n + 2) + ty + 2) * W + (cx * (n + 2) + tx + 2);
            constexpr int nch = DEPTH ? 2 : 3;
            float pv[NC];
            if (!p.first) AtlasIO<AT>::template ld_texel<NC>(prev, texel, pv);
#pragma unroll
            for (int c = 0; c < nch; ++c) {
                float x = v[c];
                if (!p.first) x = x * (1.0f - h) + pv[c] * h;
                v[c] = AtlasIO<AT>::rnd(x);
            }
            store_texel<AT, NC>(out, W, n, cx, cy, tx, ty, v);
        }
    }
}

// FP32 rays: the chunk loop with cp.async double buffering.  Chunk c+1's
// weight rows and rays (rgb+distance float4s, or the distances alone) are in
// flight while chunk c's FMAs run; the distance blend turns the raw
// distances into (d, d^2) in shared memory once a chunk has landed.  The
// accumulation order per accumulator is the single-buffer kernel's.
template <int DEPTH, typename AT, int PP>
__device__ __forceinline__ void blend_block_pipelined(const BlendParams& p, int block, float* smem) {
    using RV = typename RayVal<DEPTH != 0>::type;
    constexpr int NC_ACC = DEPTH ? 2 : 3;
    constexpr int KC = kPipeChunk;
    const luxgi_ddgi_uniform& u = p.u;
    const int n = DEPTH ? u.depth_probe_side : u.irradiance_probe_side;
    const int T = n * n;
    const int W = DEPTH ? u.depth_width : u.irradiance_width;
    const int R = p.R;
    const BlendShape sh = blend_shape(T, PP);
    const int Tp = sh.TG * kTexelTile;
    const int PB = sh.PB;
    const int p0 = block * PB;
    float* Ws = smem;                                               // [2][KC][Tp]
    float* rbuf = smem + 2 * KC * Tp;                               // irr: float4 [2][KC][PB]; dist: float [2][KC][PB]
    RV* Rd = reinterpret_cast<RV*>(rbuf + 2 * KC * PB);             // dist only: float2 [KC][PB]
    const float* Wg = DEPTH ? p.w_dist : p.w_irr;                   // [R][Tp]
    const float4* rays = static_cast<const float4*>(p.rays);
    const int tg = int(threadIdx.x) % sh.TG, pg = int(threadIdx.x) / sh.TG;
    const bool active = pg < sh.PG;
    float acc[PP][kTexelTile][NC_ACC];
#pragma unroll
    for (int j = 0; j < PP; ++j)
#pragma unroll
        for (int k = 0; k < kTexelTile; ++k)
#pragma unroll
            for (int c = 0; c < NC_ACC; ++c) acc[j][k][c] = 0.0f;
    const int nchunks = (R + KC - 1) / KC;
    auto issue = [&](int c) {
        const int r0 = c * KC, kc = min(KC, R - r0), b = c & 1;
        const float4* src = reinterpret_cast<const float4*>(Wg + size_t(r0) * Tp);
        float4* dst = reinterpret_cast<float4*>(Ws + b * KC * Tp);
        for (int i = threadIdx.x; i < kc * Tp / 4; i += blockDim.x) cp_async16(dst + i, src + i, 16);
        for (int i = threadIdx.x; i < PB * kc; i += blockDim.x) {
            const int pb = i / kc, r = i % kc;
            const int pr = p0 + pb;
            const bool ok = pr < p.P;
            const float4* g = rays + (ok ? size_t(pr) * R + r0 + r : 0);
            if constexpr (DEPTH)
                cp_async4(rbuf + b * KC * PB + r * PB + pb, reinterpret_cast<const float*>(g) + 3, ok ? 4 : 0);
            else
                cp_async16(reinterpret_cast<float4*>(rbuf) + b * KC * PB + r * PB + pb, g, ok ? 16 : 0);
        }
        cp_async_commit();
    };
    issue(0);
    for (int c = 0; c < nchunks; ++c) {
        const int kc = min(KC, R - c * KC), b = c & 1;
        if (c + 1 < nchunks) {
            issue(c + 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const RV* rs;
        if constexpr (DEPTH) {
            const float* raw = rbuf + b * KC * PB;
            for (int i = threadIdx.x; i < PB * kc; i += blockDim.x) {
                const int pb = i / kc, r = i % kc;
                const bool ok = p0 + pb < p.P;
                float d = mn(u.max_distance, raw[r * PB + pb] - 0.01f);
                if (d == -1.0f) d = u.max_distance;
                Rd[r * PB + pb] = ok ? make_float2(d, d * d) : make_float2(0.0f, 0.0f);
            }
            __syncthreads();
            rs = Rd;
        } else {
            rs = reinterpret_cast<const RV*>(rbuf) + b * KC * PB;
        }
        if (active) {
            const float* wrow = Ws + b * KC * Tp + tg * kTexelTile;
            const RV* rrow = rs + pg * PP;
#pragma unroll 2
            for (int r = 0; r < kc; ++r) {
                float w[kTexelTile];
#pragma unroll
                for (int q = 0; q < kTexelTile / 4; ++q) {
                    const float4 w4 = *reinterpret_cast<const float4*>(wrow + r * Tp + 4 * q);
                    w[4 * q] = w4.x;
                    w[4 * q + 1] = w4.y;
                    w[4 * q + 2] = w4.z;
                    w[4 * q + 3] = w4.w;
                }
#pragma unroll
                for (int j = 0; j < PP; ++j) {
                    const RV v = rrow[r * PB + j];
#pragma unroll
                    for (int k = 0; k < kTexelTile; ++k) {
                        acc[j][k][0] = fmaf(v.x, w[k], acc[j][k][0]);
                        acc[j][k][1] = fmaf(v.y, w[k], acc[j][k][1]);
                        if constexpr (!DEPTH) acc[j][k][2] = fmaf(v.z, w[k], acc[j][k][2]);
                    }
                }
            }
        }
        // the buffer just read is the target of the copies issued next
        __syncthreads();
    }
    if (!active) return;
    blend_epilogue<DEPTH, AT, PP, NC_ACC>(p, p0, tg, pg, T, n, W, acc);
}

template <int DEPTH, typename RT, typename AT, int PP>
__device__ __forceinline__ void blend_block(const BlendParams& p, int block, float* smem) {
    if constexpr (sizeof(RT) == 16) {
        blend_block_pipelined<DEPTH, AT, PP>(p, block, smem);
        return;
    }
    using RV = typename RayVal<DEPTH != 0>::type;
    constexpr int NC_ACC = DEPTH ? 2 : 3;
    const luxgi_ddgi_uniform& u = p.u;
    const int n = DEPTH ? u.depth_probe_side : u.irradiance_probe_side;
    const int T = n * n;
    const int W = DEPTH ? u.depth_width : u.irradiance_width;
    const int R = p.R;
    const BlendShape sh = blend_shape(T, PP);
    const int Tp = sh.TG * kTexelTile;
    const int PB = sh.PB;
    const int p0 = block * PB;
    float* Ws = smem;                                               // [kRayChunk][Tp]
    RV* Rs = reinterpret_cast<RV*>(smem + kRayChunk * Tp);          // [kRayChunk][PB]
    const float* Wg = DEPTH ? p.w_dist : p.w_irr;                   // [R][Tp]
    const int tg = int(threadIdx.x) % sh.TG, pg = int(threadIdx.x) / sh.TG;
    const bool active = pg < sh.PG;
    float acc[PP][kTexelTile][NC_ACC];
#pragma unroll
    for (int j = 0; j < PP; ++j)
#pragma unroll
        for (int k = 0; k < kTexelTile; ++k)
#pragma unroll
            for (int c = 0; c < NC_ACC; ++c) acc[j][k][c] = 0.0f;
    for (int r0 = 0; r0 < R; r0 += kRayChunk) {
        const int kc = min(kRayChunk, R - r0);
        {
            const float4* src = reinterpret_cast<const float4*>(Wg + size_t(r0) * Tp);
            float4* dst = reinterpret_cast<float4*>(Ws);
            for (int i = threadIdx.x; i < kc * Tp / 4; i += blockDim.x) dst[i] = __ldg(src + i);
        }
        for (int i = threadIdx.x; i < PB * kc; i += blockDim.x) {
            const int pb = i / kc, r = i % kc;
            const int pr = p0 + pb;
            float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (pr < p.P) {
                const size_t o = size_t(pr) * R + r0 + r;
                if (sizeof(RT) == 16) {
                    v = __ldg(static_cast<const float4*>(p.rays) + o);
                } else {
                    const uint2 raw = __ldg(static_cast<const uint2*>(p.rays) + o);
                    const __half2 a = *reinterpret_cast<const __half2*>(&raw.x);
                    const __half2 b = *reinterpret_cast<const __half2*>(&raw.y);
                    v = make_float4(__low2float(a), __high2float(a), __low2float(b), __high2float(b));
                }
            }
            if constexpr (DEPTH) {
                float d = mn(u.max_distance, v.w - 0.01f);
                if (d == -1.0f) d = u.max_distance;
                Rs[r * PB + pb] = make_float2(d, d * d);
            } else {
                Rs[r * PB + pb] = v;
            }
        }
        __syncthreads();
        if (active) {
            const float* wrow = Ws + tg * kTexelTile;
            const RV* rrow = Rs + pg * PP;
#pragma unroll 2
            for (int r = 0; r < kc; ++r) {
                float w[kTexelTile];
#pragma unroll
                for (int q = 0; q < kTexelTile / 4; ++q) {
                    const float4 w4 = *reinterpret_cast<const float4*>(wrow + r * Tp + 4 * q);
                    w[4 * q] = w4.x;
                    w[4 * q + 1] = w4.y;
                    w[4 * q + 2] = w4.z;
                    w[4 * q + 3] = w4.w;
                }
#pragma unroll
                for (int j = 0; j < PP; ++j) {
                    const RV v = rrow[r * PB + j];
#pragma unroll
                    for (int k = 0; k < kTexelTile; ++k) {
                        acc[j][k][0] = fmaf(v.x, w[k], acc[j][k][0]);
                        acc[j][k][1] = fmaf(v.y, w[k], acc[j][k][1]);
                        if constexpr (!DEPTH) acc[j][k][2] = fmaf(v.z, w[k], acc[j][k][2]);
                    }
                }
            }
        }
        __syncthreads();
    }
    if (!active) return;
    blend_epilogue<DEPTH, AT, PP, NC_ACC>(p, p0, tg, pg, T, n, W, acc);
}

template <int DEPTH, typename RT, typename AT, int PP>
__global__ void __launch_bounds__(kBlendThreads) blend_kernel(const BlendParams p) {
    extern __shared__ __align__(16) float smem[];
    blend_block<DEPTH, RT, AT, PP>(p, int(blockIdx.x), smem);
}

// Batched: every volume of the launch uses the same probes-per-thread PP;
// its probes per block follow from its texel count.  Parameters staged in
// shared memory once per block.
template <int DEPTH, typename RT, typename AT, int PP>
__global__ void __launch_bounds__(kBlendThreads)
    blend_batch_kernel(const BlendParams* __restrict__ vp, const int* __restrict__ starts, int n) {
    extern __shared__ __align__(16) float smem[];
    __shared__ __align__(16) uint32_t sp[sizeof(BlendParams) / 4];
    const int v = batch_volume(starts, n, int(blockIdx.x));
    const BlendParams& p = stage_params(vp + v, sp);
    blend_block<DEPTH, RT, AT, PP>(p, int(blockIdx.x) - __ldg(starts + v), smem);
}

// Both kinds of a volume in one launch: the distance blocks first (the
// longer ones), then the irradiance blocks, which fill the last partial
// wave of the distance blocks instead of starting after it.
template <typename RT, typename AT, int PPI, int PPD>
__global__ void __launch_bounds__(kBlendThreads) blend_pair_kernel(const BlendParams p, int blocks_dist) {
    extern __shared__ __align__(16) float smem[];
    const int b = int(blockIdx.x);
    if (b < blocks_dist) blend_block<1, RT, AT, PPD>(p, b, smem);
    else blend_block<0, RT, AT, PPI>(p, b - blocks_dist, smem);
}

static int blend_side(const BlendParams& p, bool depth) {
    return depth ? p.u.depth_probe_side : p.u.irradiance_probe_side;
}

int blend_blocks(const BlendParams& p, bool depth, int pp) {
    const int side = blend_side(p, depth);
    const int PB = blend_shape(side * side, pp).PB;
    return (p.P + PB - 1) / PB;
}

size_t blend_smem(const BlendParams& p, bool depth, int pp) {
    const int side = blend_side(p, depth);
    return blend_smem_bytes(side * side, pp, depth, p.storage != LUXGI_STORAGE_FP16);
}

// Probes per thread of a single-volume launch: the largest tile that still
// gives every SM two blocks.
static int auto_pp(const BlendParams& p, bool depth) {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    for (int pp : {4, 2})
        if (blend_blocks(p, depth, pp) >= 2 * sms) return pp;
    return 1;
}

template <int DEPTH, typename RT, typename AT, int PP>
static cudaError_t launch_kind_pp(const void* vp, const int* starts, int n, int blocks, size_t sm, bool batch,
                                  cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    if (batch) {
        auto k = blend_batch_kernel<DEPTH, RT, AT, PP>;
        if (sm > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
            if (e != cudaSuccess) return e;
        }
        k<<<blocks, kBlendThreads, sm, st>>>(static_cast<const BlendParams*>(vp), starts, n);
    } else {
        auto k = blend_kernel<DEPTH, RT, AT, PP>;
        if (sm > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
            if (e != cudaSuccess) return e;
        }
        k<<<blocks, kBlendThreads, sm, st>>>(*static_cast<const BlendParams*>(vp));
    }
    note_launch();
    return cudaGetLastError();
}

template <int DEPTH, typename RT, typename AT>
static cudaError_t launch_kind(const void* vp, const int* starts, int n, int blocks, size_t sm, int pp, bool batch,
                               cudaStream_t st) {
    switch (pp) {
        case 1: return launch_kind_pp<DEPTH, RT, AT, 1>(vp, starts, n, blocks, sm, batch, st);
        case 2: return launch_kind_pp<DEPTH, RT, AT, 2>(vp, starts, n, blocks, sm, batch, st);
        case 4: return launch_kind_pp<DEPTH, RT, AT, 4>(vp, starts, n, blocks, sm, batch, st);
        default: return cudaErrorInvalidValue;
    }
}

template <typename RT, typename AT, int PPI, int PPD>
static cudaError_t launch_pair_pp(const BlendParams& p, int bi, int bd, size_t sm, cudaStream_t st) {
    auto k = blend_pair_kernel<RT, AT, PPI, PPD>;
    if (sm > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        if (e != cudaSuccess) return e;
    }
    k<<<bi + bd, kBlendThreads, sm, st>>>(p, bd);
    note_launch();
    return cudaGetLastError();
}

// The irradiance kind has more probes per block than the distance kind at
// equal probes per thread, so auto_pp never gives it the larger tile: the
// pairs below are all that occur.
template <typename RT, typename AT>
static cudaError_t launch_pair(const BlendParams& p, int ppi, int ppd, int bi, int bd, size_t sm, cudaStream_t st) {
    switch (ppi * 8 + ppd) {
        case 1 * 8 + 1: return launch_pair_pp<RT, AT, 1, 1>(p, bi, bd, sm, st);
        case 1 * 8 + 2: return launch_pair_pp<RT, AT, 1, 2>(p, bi, bd, sm, st);
        case 1 * 8 + 4: return launch_pair_pp<RT, AT, 1, 4>(p, bi, bd, sm, st);
        case 2 * 8 + 2: return launch_pair_pp<RT, AT, 2, 2>(p, bi, bd, sm, st);
        case 2 * 8 + 4: return launch_pair_pp<RT, AT, 2, 4>(p, bi, bd, sm, st);
        case 4 * 8 + 4: return launch_pair_pp<RT, AT, 4, 4>(p, bi, bd, sm, st);
        default: return cudaErrorNotSupported;
    }
}

// ------------------------------------------------ sparse distance blend
// The distance weights are pow(cos, sharpness) cut below 1e-8: with the
// default sharpness of 50 a texel takes ~15 % of the rays and a group of
// four consecutive texels (one register tile) ~26 % (66 of 256).  Every
// probe of a frame shares the directions, so the rays that carry weight for
// a group are the same for all probes: ray_list_kernel lists them once a
// frame, and the distance blend walks only those, in ascending order.  The
// rays left out add fmaf(v, 0, acc) = acc in the dense blend (distances are
// finite), so the sums are those of the dense blend, bit for bit.
constexpr int kListThreads = 256;

// One block per 4-texel group of the distance atlas: the rays whose cut
// weight is nonzero for any of the group's texels, ascending, with the four
// weights (a block-wide stream compaction, kListThreads rays at a time).
__global__ void __launch_bounds__(kListThreads) ray_list_kernel(const BlendParams p) {
    __shared__ int wsum[kListThreads / 32 + 1];
    const int n = p.u.depth_probe_side;
    const int Tp = blend_row_pitch(n * n);
    const int g = int(blockIdx.x);
    const int warp = int(threadIdx.x) / 32, lane = int(threadIdx.x) & 31;
    const int R = p.R;
    const float4* W4 = reinterpret_cast<const float4*>(p.w_dist);   // [R][Tp / 4]
    int base = 0;
    for (int r0 = 0; r0 < R; r0 += kListThreads) {
        const int r = r0 + int(threadIdx.x);
        float4 w = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (r < R) w = __ldg(W4 + size_t(r) * (Tp / 4) + g);
        const bool nz = w.x != 0.0f || w.y != 0.0f || w.z != 0.0f || w.w != 0.0f;
        const unsigned m = __ballot_sync(0xffffffffu, nz);
        if (lane == 0) wsum[warp] = __popc(m);
        __syncthreads();
        if (threadIdx.x == 0) {
            int s = 0;
            for (int k = 0; k < kListThreads / 32; ++k) {
                const int c = wsum[k];
                wsum[k] = s;
                s += c;
            }
            wsum[kListThreads / 32] = s;
        }
        __syncthreads();
        if (nz) {
            const int i = base + wsum[warp] + __popc(m & ((1u << lane) - 1u));
            p.sp_ray[size_t(g) * R + i] = r;
            p.sp_w[size_t(g) * R + i] = w;
        }
        base += wsum[kListThreads / 32];
        __syncthreads();
    }
    if (threadIdx.x == 0) p.sp_count[g] = base;
}

// The distance blend over the listed rays: a block takes 32 probes (a lane
// each) and every texel group (a warp each in turn).  The probes' clamped
// distances are staged in shared memory ray-major, [R][33] (the odd pitch
// keeps the transposing stores free of bank conflicts).  A warp copies its
// group's list to shared memory 32 entries at a time; each lane then reads
// the entry (a broadcast) and its probe's distance of that ray (conflict
// free), squares it as the dense blend does, and accumulates its four
// texels.
constexpr int kSparseWarps = 8;
constexpr int kSparsePitch = 33;

static_assert(32 * kSparseWarps == kBlendThreads, "the sparse and dense blocks share a launch");

template <typename RT, typename AT>
__device__ __forceinline__ void blend_dist_sparse_block(const BlendParams& p, int block, float* dsm) {
    // dsm: [R][kSparsePitch]
    __shared__ float4 lw[kSparseWarps][32];
    __shared__ int lr[kSparseWarps][32];
    const luxgi_ddgi_uniform& u = p.u;
    const int n = u.depth_probe_side, T = n * n, W = u.depth_width;
    const int TG = blend_row_pitch(T) / 4;
    const int R = p.R;
    const int p0 = block * 32;
    for (int i = int(threadIdx.x); i < 32 * R; i += int(blockDim.x)) {
        const int pb = i / R, r = i - pb * R;
        const int pr = p0 + pb;
        float d = 0.0f;
        if (pr < p.P) {
            const size_t o = size_t(pr) * R + r;
            float raw;
            if (sizeof(RT) == 16) {
                raw = __ldg(reinterpret_cast<const float*>(static_cast<const float4*>(p.rays) + o) + 3);
            } else {
                const uint2 q = __ldg(static_cast<const uint2*>(p.rays) + o);
                raw = __high2float(*reinterpret_cast<const __half2*>(&q.y));
            }
            d = mn(u.max_distance, raw - 0.01f);
            if (d == -1.0f) d = u.max_distance;
        }
        dsm[r * kSparsePitch + pb] = d;
    }
    __syncthreads();
    const int warp = int(threadIdx.x) / 32, lane = int(threadIdx.x) & 31;
    for (int g = warp; g < TG; g += kSparseWarps) {
        float acc[1][kTexelTile][2];
#pragma unroll
        for (int k = 0; k < kTexelTile; ++k) acc[0][k][0] = acc[0][k][1] = 0.0f;
        const int cnt = __ldg(p.sp_count + g);
        const int* rl = p.sp_ray + size_t(g) * R;
        const float4* wl = p.sp_w + size_t(g) * R;
        for (int c0 = 0; c0 < cnt; c0 += 32) {
            if (c0 + lane < cnt) {
                lr[warp][lane] = __ldg(rl + c0 + lane) * kSparsePitch;   // the ray's row of distances
                lw[warp][lane] = __ldg(wl + c0 + lane);
            }
            __syncwarp();
            const int m = min(32, cnt - c0);
#pragma unroll 8
            for (int j = 0; j < m; ++j) {
                const float4 w4 = lw[warp][j];
                const float d = dsm[lr[warp][j] + lane];
                const float d2 = d * d;
                const float w[4] = {w4.x, w4.y, w4.z, w4.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    acc[0][k][0] = fmaf(d, w[k], acc[0][k][0]);
                    acc[0][k][1] = fmaf(d2, w[k], acc[0][k][1]);
                }
            }
            __syncwarp();
        }
        blend_epilogue<1, AT, 1, 2>(p, p0, g, lane, T, n, W, acc);
    }
}

// Both kinds in one launch: the sparse distance blocks first, then the
// dense irradiance blocks, which fill the distance blocks' last wave.
template <typename RT, typename AT, int PPI>
__global__ void __launch_bounds__(kBlendThreads) blend_sparse_pair_kernel(const BlendParams p, int blocks_dist) {
    extern __shared__ __align__(16) float smem[];
    const int b = int(blockIdx.x);
    if (b < blocks_dist) blend_dist_sparse_block<RT, AT>(p, b, smem);
    else blend_block<0, RT, AT, PPI>(p, b - blocks_dist, smem);
}

template <typename RT, typename AT, int PPI>
static cudaError_t launch_sparse_pair_pp(const BlendParams& p, int bi, int bd, size_t sm, cudaStream_t st) {
    auto k = blend_sparse_pair_kernel<RT, AT, PPI>;
    if (sm > 48 * 1024) {
        const cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm));
        if (e != cudaSuccess) return e;
    }
    k<<<bi + bd, kBlendThreads, sm, st>>>(p, bd);
    note_launch();
    return cudaGetLastError();
}

template <typename RT, typename AT>
static cudaError_t launch_sparse_pair(const BlendParams& p, int ppi, int bi, int bd, size_t sm, cudaStream_t st) {
    switch (ppi) {
        case 1: return launch_sparse_pair_pp<RT, AT, 1>(p, bi, bd, sm, st);
        case 2: return launch_sparse_pair_pp<RT, AT, 2>(p, bi, bd, sm, st);
        case 4: return launch_sparse_pair_pp<RT, AT, 4>(p, bi, bd, sm, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_blend(const BlendParams& p, cudaStream_t st) {
    if (p.P <= 0) return cudaSuccess;
    if (kTexelTile == 4 && p.sp_count && p.R <= kSparseMaxRays) {
        // the distance kind over the listed rays and the irradiance kind, one launch
        const int TG = blend_row_pitch(p.u.depth_probe_side * p.u.depth_probe_side) / 4;
        ray_list_kernel<<<TG, kListThreads, 0, st>>>(p);
        note_launch();
        const int ppi = auto_pp(p, false);
        const int bi = blend_blocks(p, false, ppi), bd = (p.P + 31) / 32;
        const size_t sm = std::max(sizeof(float) * size_t(p.R) * kSparsePitch, blend_smem(p, false, ppi));
        return p.storage == LUXGI_STORAGE_FP16 ? launch_sparse_pair<uint2, __half>(p, ppi, bi, bd, sm, st)
                                               : launch_sparse_pair<float4, float>(p, ppi, bi, bd, sm, st);
    }
    const int ppi = auto_pp(p, false), ppd = auto_pp(p, true);
    const int bi = blend_blocks(p, false, ppi), bd = blend_blocks(p, true, ppd);
    const size_t si = blend_smem(p, false, ppi), sd = blend_smem(p, true, ppd);
    if (ppi <= ppd) {
        const size_t sm = si > sd ? si : sd;
        return p.storage == LUXGI_STORAGE_FP16 ? launch_pair<uint2, __half>(p, ppi, ppd, bi, bd, sm, st)
                                               : launch_pair<float4, float>(p, ppi, ppd, bi, bd, sm, st);
    }
    cudaError_t e;
    if (p.storage == LUXGI_STORAGE_FP16) {
        e = launch_kind<0, uint2, __half>(&p, nullptr, 1, bi, si, ppi, false, st);
        if (e == cudaSuccess) e = launch_kind<1, uint2, __half>(&p, nullptr, 1, bd, sd, ppd, false, st);
    } else {
        e = launch_kind<0, float4, float>(&p, nullptr, 1, bi, si, ppi, false, st);
        if (e == cudaSuccess) e = launch_kind<1, float4, float>(&p, nullptr, 1, bd, sd, ppd, false, st);
    }
    return e;
}

cudaError_t launch_blend_batch(const BlendParams* vp, const int* starts_irr, int blocks_irr, size_t smem_irr,
                               const int* starts_dist, int blocks_dist, size_t smem_dist, int n, int pp,
                               int storage, cudaStream_t st) {
    if (pp != 1 && pp != 2 && pp != 4) return cudaErrorInvalidValue;
    cudaError_t e;
    if (storage == LUXGI_STORAGE_FP16) {
        e = launch_kind<0, uint2, __half>(vp, starts_irr, n, blocks_irr, smem_irr, pp, true, st);
        if (e == cudaSuccess) e = launch_kind<1, uint2, __half>(vp, starts_dist, n, blocks_dist, smem_dist, pp, true, st);
    } else {
        e = launch_kind<0, float4, float>(vp, starts_irr, n, blocks_irr, smem_irr, pp, true, st);
        if (e == cudaSuccess) e = launch_kind<1, float4, float>(vp, starts_dist, n, blocks_dist, smem_dist, pp, true, st);
    }
    return e;
}

// --------------------------------------------------------------- border
// Standalone BorderUpdate.glsl: one block per probe cell, one thread per
// (dst, src) pair; sources are interior texels, destinations border texels.
template <typename AT, int NC>
__global__ void border_kernel(void* atlas, int W, int n, int XY, int P) {
    const int p = blockIdx.x;
    if (p >= P) return;
    const int cx = p % XY, cy = p / XY;
    const int ox = cx * (n + 2) + 1, oy = cy * (n + 2) + 1;
    for (int i = threadIdx.x; i < 4 * n + 4; i += blockDim.x) {
        int dx, dy, sx, sy;
        const int side = i / n, k = i % n + 1;
        if (i < 4 * n) {
            if (side == 0) { dx = k; dy = 0; sx = n + 1 - k; sy = 1; }
            else if (side == 1) { dx = k; dy = n + 1; sx = n + 1 - k; sy = n; }
            else if (side == 2) { dx = 0; dy = k; sx = 1; sy = n + 1 - k; }
            else { dx = n + 1; dy = k; sx = n; sy = n + 1 - k; }
        } else {
            const int c = i - 4 * n;
            if (c == 0) { dx = 0; dy = 0; sx = n; sy = n; }
            else if (c == 1) { dx = n + 1; dy = 0; sx = 1; sy = n; }
            else if (c == 2) { dx = 0; dy = n + 1; sx = n; sy = 1; }
            else { dx = n + 1; dy = n + 1; sx = 1; sy = 1; }
        }
        const size_t d = (size_t(oy + dy) * W + ox + dx) * NC, s = (size_t(oy + sy) * W + ox + sx) * NC;
#pragma unroll
        for (int c = 0; c < NC; ++c) AtlasIO<AT>::st(atlas, d + c, AtlasIO<AT>::ld(atlas, s + c));
    }
}

cudaError_t launch_border(const luxgi_ddgi_uniform& u, void* irr, void* dist, int storage, cudaStream_t st) {
    const int XY = u.probe_counts[0] * u.probe_counts[1];
    const int P = XY * u.probe_counts[2];
    if (P <= 0) return cudaSuccess;
    if (storage == LUXGI_STORAGE_FP16) {
        border_kernel<__half, 4><<<P, 128, 0, st>>>(irr, u.irradiance_width, u.irradiance_probe_side, XY, P);
        border_kernel<__half, 2><<<P, 128, 0, st>>>(dist, u.depth_width, u.depth_probe_side, XY, P);
    } else {
        border_kernel<float, 4><<<P, 128, 0, st>>>(irr, u.irradiance_width, u.irradiance_probe_side, XY, P);
        border_kernel<float, 2><<<P, 128, 0, st>>>(dist, u.depth_width, u.depth_probe_side, XY, P);
    }
    note_launch(2);
    return cudaGetLastError();
}

}  // namespace luxgi
