// Tensor-core probe blend (tcgen05, sm_103a).
//
// The blend of ProbeUpdate.glsl is a contraction with a weight matrix shared
// by every probe of a volume (see blend.cu):
//     D[(p,c)][t] = sum_k A[(p,c)][k] * B[t][k]
// A = per-ray data of 128 (probe, channel) rows, FP16, K-major:
//     irradiance  rows (p, r|g|b|0), K = R rays
//     distance    rows (p, d|d^2),   K = 2R: the value split hi + lo
//                 (FP16 hi, FP16 residual) so the sums keep ~FP32 accuracy
// B = weights W[t][r] in FP16, K-major, N = texels padded to 16; for the
//     distance the same B block multiplies the hi and the lo half of A.
// D accumulates in TMEM (FP32).  A launch runs a list of jobs, a job being
// one blend kind of one volume (its two operand maps and its arguments):
// both kinds of one volume, or every volume of a batch.  The jobs' 128-row
// tiles form one list; one CTA per SM, persistent over a contiguous range
// of it (ranges split by the bytes a tile moves), loads a job's B into
// shared memory once and reloads it where its range crosses into the next
// job:
//   warp 0      TMA producer (cp.async.bulk.tensor, 128B swizzle, 16 KB stages)
//   warp 1      TMEM allocator + single-thread tcgen05.mma issuer
//   warps 2..17 epilogue: tcgen05.ld, normalise, gamma, hysteresis, store
//               (four warps per TMEM lane quadrant, each a quarter of the
//               column chunks) with the border mirrors
// The accumulator is double buffered in TMEM so the epilogue of one tile
// overlaps the MMAs of the next.  Every mbarrier wait is bounded by a clock
// budget; on expiry the kernel raises the status word of every job it had
// tiles of, stops issuing work, drains what it issued and frees its TMEM.
#include <algorithm>
#include <climits>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "atlas_io.cuh"
#include "luxgi_internal.h"

namespace luxgi {

namespace {

constexpr int kStages = 5;
constexpr int kKBlock = 64;                 // halves per 128-byte swizzle row
constexpr int kStageBytes = 128 * 128;      // 128 rows x 128 bytes
constexpr int kEpilogueWarps = 16;          // 4 per TMEM lane quadrant
constexpr int kThreads = 64 + 32 * kEpilogueWarps;
constexpr int kEpilogueThreads = kThreads - 64;
constexpr long long kWaitCycles = 4000000000LL;   // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait: false when the clock budget ran out or another role gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, volatile int* abort_flag, long long budget) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort_flag) return false;
        if (clock64() - t0 > budget) {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (stride byte offset), descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= uint64_t((addr & 0x3FFFF) >> 4);
    d |= uint64_t(1) << 16;                 // leading byte offset (unused with 128B swizzle)
    d |= uint64_t(1024 >> 4) << 32;         // stride byte offset
    d |= uint64_t(1) << 46;                 // version
    d |= uint64_t(2) << 61;                 // SWIZZLE_128B
    return d;
}

// Instruction descriptor of kind::f16: D = F32, A = B = F16, both K-major.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4) | (0u << 7) | (0u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
    uint32_t r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
    luxgi_ddgi_uniform u;
    const float* norm;        // [N] tensor-core normalisers (1 / (2 sum w_fp16))
    const void* prev;
    void* out;
    uint32_t* status;
    int dist;                             // 1: distance kind, 0: irradiance
    int first, P, R, N, T, side, W, nc;   // nc: atlas channels (4 irradiance, 2 distance)
    int rows_per_probe;                   // 4 irradiance, 2 distance
    int kb_a;                             // K blocks of A per tile
    int kb_b;                             // K blocks of B (ceil(R / 64))
    int lo_offset;                        // column of the lo half in A (distance), 0 otherwise
    int tiles;                            // 128-row tiles of this job
    int tile0;                            // its first tile in the launch's tile list
    long long wait_cycles;                // this job's bound of an mbarrier wait, SM clock cycles (a launch
                                          // takes the smallest of its jobs')
    int withhold;                         // test aid: block 0 skips the first A load of its first tile
};

// One blend kind of one volume: its operand maps and its arguments.
struct TcJob {
    CUtensorMap ma;   // A, the per-ray operands: 64 x 128 boxes
    CUtensorMap mb;   // B, the weights: 64 x N boxes
    TcArgs g;
};
static_assert(alignof(TcJob) == 128 && sizeof(TcJob) % 128 == 0, "tensor maps are 128-byte aligned");

// Kernel parameters: the jobs (in the parameter space for one volume, in
// device memory for a batch) and the split of the tile list between CTAs.
struct TcLaunchArgs {
    TcJob local[2];
    const TcJob* jobs;        // null: `local`
    long long wait_cycles;
    int njobs, nmax, b_bytes;
    int split[kTcMaxGrid + 1];   // CTA b takes tiles [split[b], split[b + 1])
};
static_assert(sizeof(TcLaunchArgs) <= 4096, "kernel parameter block");

// Lane-group transposes of the epilogue.  The lanes of one probe each hold
// one channel over C accumulator columns (texels); afterwards each lane
// holds every channel of its own texels, so that a texel is loaded (the
// hysteresis history) and stored (with its border mirrors) in one vector
// access instead of one scalar access per channel.
// Irradiance, 4 lanes (r, g, b, zero row) and C / 4 4x4 blocks: lane m ends
// with texels 4k + m as v[4k .. 4k+3].
template <int C>
__device__ __forceinline__ void transpose_quad(float* v, int lane) {
    const bool b1 = (lane & 2) != 0, b0 = (lane & 1) != 0;
#pragma unroll
    for (int k = 0; k < C / 4; ++k) {
        float* a = v + 4 * k;
        // swap the off-diagonal 2x2 blocks with lane ^ 2 ...
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const float x = __shfl_xor_sync(0xffffffffu, b1 ? a[i] : a[i + 2], 2);
            if (b1) a[i] = x;
            else a[i + 2] = x;
        }
        // ... then transpose each 2x2 block with lane ^ 1
        const float x0 = __shfl_xor_sync(0xffffffffu, b0 ? a[0] : a[1], 1);
        const float x1 = __shfl_xor_sync(0xffffffffu, b0 ? a[2] : a[3], 1);
        if (b0) {
            a[0] = x0;
            a[2] = x1;
        } else {
            a[1] = x0;
            a[3] = x1;
        }
    }
}

// Distance, 2 lanes (d, d^2) and C / 2 2x2 blocks: lane m ends with texels
// 2k + m as v[2k .. 2k+1].
template <int C>
__device__ __forceinline__ void transpose_pair(float* v, int lane) {
    const bool b0 = (lane & 1) != 0;
#pragma unroll
    for (int k = 0; k < C / 2; ++k) {
        float* a = v + 2 * k;
        const float x = __shfl_xor_sync(0xffffffffu, b0 ? a[0] : a[1], 1);
        if (b0) a[0] = x;
        else a[1] = x;
    }
}


// The job holding tile t, from job j onwards (jobs in tile order).
__device__ __forceinline__ int job_from(const TcJob* J, int njobs, int j, int t) {
    while (j + 1 < njobs && t >= J[j + 1].g.tile0) ++j;
    return j;
}

// Epilogue of one tile for the 16 epilogue warps: tcgen05.ld, normalise,
// gamma, hysteresis, store with the border mirrors (four warps per TMEM lane
// quadrant, each a quarter of the column chunks).  False when the wait for
// the accumulator gave up.
template <bool DIST, typename AT>
__device__ __forceinline__ bool epilogue_tile(const TcArgs& g, int lt, uint32_t taddr, int q, int part, int lane,
                                              uint64_t* tfull, uint32_t parity, volatile int* abort_flag,
                                              long long budget) {
    constexpr int G = DIST ? 2 : 4;         // lanes (accumulator rows) of one probe = atlas channels
    constexpr int kParts = kEpilogueWarps / 4;
    // the job's fields in registers (the atlas stores may alias the job list)
    const int T = g.T, W = g.W, n = g.side;
    const bool first = g.first != 0;
    const float* norm = g.norm;
    const void* prev = g.prev;
    void* out = g.out;
    const int XY = g.u.probe_counts[0] * g.u.probe_counts[1];
    const float h = g.u.hysteresis;
    const float ig = 1.0f / g.u.ddgi_gamma;
    const int row = q * 32 + lane;          // accumulator row = (probe, channel)
    const int m = lane & (G - 1);           // after the transpose: texels G k + m of each chunk
    const int chunks = g.N / 16;
    const int c_begin = (chunks * part / kParts) * 16, c_end = (chunks * (part + 1) / kParts) * 16;
    const int p = lt * (128 / G) + row / G;
    const bool live = p < g.P;
    const int cx = p % XY, cy = p / XY;
    const bool hyst = !first && live;
    // the columns go in 8-wide chunks; the previous texels (hysteresis) of
    // this lane in a chunk are loaded one chunk ahead: the first chunk's
    // before the wait for the accumulator, each next chunk's while the
    // current one is stored (8-wide chunks keep the accumulator values, the
    // history and the history in flight within the 96 registers a thread
    // that 576 threads leave)
    constexpr int CW = 8;
    auto load_prev = [&](int c0, float* pv) {
        int ty = (c0 + m) / n, tx = c0 + m - ty * n;
#pragma unroll
        for (int k = 0; k < CW / G; ++k) {
            if (c0 + G * k + m < T) {
                AtlasIO<AT>::template ld_texel<G>(prev, size_t(cy * (n + 2) + ty + 2) * W + (cx * (n + 2) + tx + 2),
                                                  pv + G * k);
            }
            tx += G;
            while (tx >= n) {
                tx -= n;
                ++ty;
            }
        }
    };
    float pv[CW], pn[CW];
    if (hyst && c_begin < c_end) load_prev(c_begin, pv);
    if (!mbar_wait(tfull, parity, abort_flag, budget)) return false;
    tc_fence_after();
    for (int c0 = c_begin; c0 < c_end; c0 += CW) {
        float v[CW];
        tmem_ld8(taddr + uint32_t(c0), v);
        if (DIST) transpose_pair<CW>(v, lane);   // every lane: the shuffles span the warp
        else transpose_quad<CW>(v, lane);
        if (!live) continue;
        if (hyst && c0 + CW < c_end) load_prev(c0 + CW, pn);
        int ty = (c0 + m) / n, tx = c0 + m - ty * n;
#pragma unroll
        for (int k = 0; k < CW / G; ++k) {
            const int t = c0 + G * k + m;
            if (t < T) {
                const float nt = __ldg(norm + t);
                float x[G];
#pragma unroll
                for (int ch = 0; ch < G; ++ch) {
                    if (!DIST && ch == 3) {
                        x[ch] = 1.0f;   // alpha (ProbeUpdate.glsl:150)
                        continue;
                    }
                    float y = v[G * k + ch] * nt;
                    if (!DIST) y = __powf(y, ig);   // within the tensor path's 2e-3
                    if (!first) y = y * (1.0f - h) + pv[G * k + ch] * h;
                    x[ch] = y;
                }
                store_texel<AT, G>(out, W, n, cx, cy, tx, ty, x);
            }
            tx += G;
            while (tx >= n) {
                tx -= n;
                ++ty;
            }
        }
        if (hyst) {
#pragma unroll
            for (int j = 0; j < CW; ++j) pv[j] = pn[j];
        }
    }
    return true;
}

template <typename AT>
__global__ void __launch_bounds__(kThreads, 1) tc_blend_kernel(const __grid_constant__ TcLaunchArgs L) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    const TcJob* J = L.jobs ? L.jobs : L.local;
    const int njobs = L.njobs;
    // 1024-byte aligned carve-out: B blocks (the widest job's), A stages, then barriers
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint8_t* smem_b = base;
    uint8_t* smem_a = smem_b + L.b_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_a + kStages * kStageBytes);
    uint64_t* full = bars;                       // [kStages]
    uint64_t* empty = bars + kStages;            // [kStages]
    uint64_t* bfull = bars + 2 * kStages;        // [1] B loaded
    uint64_t* bempty = bars + 2 * kStages + 1;   // [1] the multiplies reading B done
    uint64_t* tfull = bars + 2 * kStages + 2;    // [2]
    uint64_t* tempty = bars + 2 * kStages + 4;   // [2]
    uint64_t* mdrain = bars + 2 * kStages + 6;   // [1] MMAs issued before an abort
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 7);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const long long budget = L.wait_cycles > 0 ? L.wait_cycles : kWaitCycles;
    const int t_begin = L.split[blockIdx.x], t_end = L.split[blockIdx.x + 1];
    const int j_begin = job_from(J, njobs, 0, t_begin);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int cols = 2 * L.nmax;
    const uint32_t tmem_cols = (cols <= 32) ? 32 : (cols <= 64) ? 64 : (cols <= 128) ? 128 : (cols <= 256) ? 256 : 512;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(bfull, 1);
        mbar_init(bempty, 1);
        mbar_init(&tfull[0], 1);
        mbar_init(&tfull[1], 1);
        mbar_init(&tempty[0], kEpilogueThreads);
        mbar_init(&tempty[1], kEpilogueThreads);
        mbar_init(mdrain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(tmem_cols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;
    // phase of the last A load issued into each stage, and of the last B
    // load (producer thread)
    uint32_t pending[kStages];
    for (int s = 0; s < kStages; ++s) pending[s] = 0xFFFFFFFFu;
    uint32_t b_pending = 0xFFFFFFFFu;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            int j = j_begin, jb = -1, nb = 0;
            for (int t = t_begin; t < t_end && ok; ++t) {
                j = job_from(J, njobs, j, t);
                const TcArgs& g = J[j].g;
                if (j != jb) {
                    // the job's weights, once the multiplies of the last job are done with B
                    if (nb > 0) {
                        ok = mbar_wait(bempty, uint32_t(nb - 1) & 1u, abort_flag, budget);
                        if (!ok) break;
                    }
                    const int bb = g.N * 128;
                    mbar_expect_tx(bfull, uint32_t(g.kb_b * bb));
                    for (int kb = 0; kb < g.kb_b; ++kb) tma_load_2d(smem_b + kb * bb, &J[j].mb, bfull, kb * kKBlock, 0);
                    b_pending = uint32_t(nb) & 1u;
                    ++nb;
                    jb = j;
                }
                const int lt = t - g.tile0;
                for (int kb = 0; kb < g.kb_a && ok; ++kb) {
                    ok = mbar_wait(&empty[stage], phase ^ 1u, abort_flag, budget);
                    if (!ok) break;
                    if (g.withhold && blockIdx.x == 0 && t == t_begin && kb == 0) {
                        // test aid: this stage's load is never issued, so the
                        // MMA issuer's bounded wait on it runs out
                        if (++stage == kStages) { stage = 0; phase ^= 1u; }
                        continue;
                    }
                    const int x = (kb < g.kb_b) ? kb * kKBlock : g.lo_offset + (kb - g.kb_b) * kKBlock;
                    mbar_expect_tx(&full[stage], kStageBytes);
                    tma_load_2d(smem_a + stage * kStageBytes, &J[j].ma, &full[stage], x, lt * 128);
                    pending[stage] = phase;
                    if (++stage == kStages) { stage = 0; phase ^= 1u; }
                }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            int it = 0;
            int j = j_begin, jb = -1, nb = 0;
            for (int t = t_begin; t < t_end && ok; ++t, ++it) {
                j = job_from(J, njobs, j, t);
                const TcArgs& g = J[j].g;
                if (j != jb) {
                    ok = mbar_wait(bfull, uint32_t(nb) & 1u, abort_flag, budget);
                    if (!ok) break;
                    ++nb;
                    jb = j;
                }
                const int acc = it & 1;
                const uint32_t use = uint32_t(it >> 1);
                ok = mbar_wait(&tempty[acc], (use & 1u) ^ 1u, abort_flag, budget);
                if (!ok) break;
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + uint32_t(acc * L.nmax);
                const uint32_t idesc = idesc_f16(128, g.N);
                const int bb = g.N * 128;
                for (int kb = 0; kb < g.kb_a && ok; ++kb) {
                    ok = mbar_wait(&full[stage], phase, abort_flag, budget);
                    if (!ok) break;
                    tc_fence_after();
                    const int bk = (kb < g.kb_b) ? kb : kb - g.kb_b;
                    const uint32_t a_addr = smem_u32(smem_a + stage * kStageBytes);
                    const uint32_t b_addr = smem_u32(smem_b + bk * bb);
#pragma unroll
                    for (int k = 0; k < kKBlock / 16; ++k) {
                        mma_f16(d_tmem, smem_desc(a_addr + k * 32), smem_desc(b_addr + k * 32), idesc,
                                (kb > 0 || k > 0) ? 1u : 0u);
                    }
                    mma_commit(&empty[stage]);
                    if (++stage == kStages) { stage = 0; phase ^= 1u; }
                }
                if (!ok) break;
                mma_commit(&tfull[acc]);
                // B is free for the next job once this job's last multiplies are done
                if (t + 1 < t_end && t + 1 >= g.tile0 + g.tiles) mma_commit(bempty);
            }
        }
    } else {
        // ------------------------------------------------ epilogue
        const int q = warp & 3;                 // TMEM lane quadrant of this warp
        const int part = (warp - 2) >> 2;       // which share of the column chunks
        int it = 0;
        int j = j_begin;
        for (int t = t_begin; t < t_end; ++t, ++it) {
            j = job_from(J, njobs, j, t);
            const TcArgs& g = J[j].g;
            const int acc = it & 1;
            const uint32_t parity = uint32_t(it >> 1) & 1u;
            const uint32_t taddr = tmem_base + (uint32_t(q * 32) << 16) + uint32_t(acc * L.nmax);
            const bool ok = g.dist ? epilogue_tile<true, AT>(g, t - g.tile0, taddr, q, part, lane, &tfull[acc], parity,
                                                             abort_flag, budget)
                                   : epilogue_tile<false, AT>(g, t - g.tile0, taddr, q, part, lane, &tfull[acc], parity,
                                                              abort_flag, budget);
            if (!ok) break;
            tc_fence_before();
            mbar_arrive(&tempty[acc]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (*abort_flag) {
        // A role gave up (every role has left its loop by now): the loads and
        // multiplies already issued are drained, each wait bounded, before the
        // shared memory and the tensor memory they target are released.
        if (warp == 0 && lane == 0) {
            for (int s = 0; s < kStages; ++s) {
                if (pending[s] == 0xFFFFFFFFu) continue;
                const long long t0 = clock64();
                while (!mbar_try_wait(&full[s], pending[s]) && clock64() - t0 < budget) {}
            }
            if (b_pending != 0xFFFFFFFFu) {
                const long long t0 = clock64();
                while (!mbar_try_wait(bfull, b_pending) && clock64() - t0 < budget) {}
            }
        } else if (warp == 1 && lane == 0) {
            // one commit tracks every multiply this thread issued
            mma_commit(mdrain);
            const long long t0 = clock64();
            while (!mbar_try_wait(mdrain, 0) && clock64() - t0 < budget) {}
        }
        tc_fence_before();
        __syncthreads();
    }
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(tmem_cols));
    }
    if (threadIdx.x == 0 && *abort_flag && t_begin < t_end) {
        // every job this CTA had tiles of
        const int j_end = job_from(J, njobs, j_begin, t_end - 1);
        for (int j = j_begin; j <= j_end; ++j) atomicOr(J[j].g.status, 1u);
    }
}

// ------------------------------------------------------------ host side
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

bool make_map(CUtensorMap* m, const void* ptr, uint64_t inner, uint64_t rows, uint32_t box_inner, uint32_t box_rows) {
    EncodeTiled fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[2] = {inner, rows};
    cuuint64_t strides[1] = {inner * 2};
    cuuint32_t box[2] = {box_inner, box_rows};
    cuuint32_t estr[2] = {1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <bool DIST>
void fill_args(const TcBlendParams& p, TcArgs& g) {
    const luxgi_ddgi_uniform& u = p.u;
    std::memset(&g, 0, sizeof(g));
    g.u = u;
    g.dist = DIST ? 1 : 0;
    g.first = p.first;
    g.P = p.P;
    g.R = p.R;
    g.side = DIST ? u.depth_probe_side : u.irradiance_probe_side;
    g.T = g.side * g.side;
    g.N = DIST ? p.Nd : p.Ni;
    g.W = DIST ? u.depth_width : u.irradiance_width;
    g.nc = DIST ? 2 : 4;
    g.rows_per_probe = DIST ? 2 : 4;
    g.kb_b = (p.R + kKBlock - 1) / kKBlock;
    g.kb_a = DIST ? 2 * g.kb_b : g.kb_b;
    g.lo_offset = DIST ? p.R : 0;
    g.norm = DIST ? p.n_dist : p.n_irr;
    g.prev = DIST ? p.prev_dist : p.prev_irr;
    g.out = DIST ? p.out_dist : p.out_irr;
    g.status = p.status;
    const int64_t rows = int64_t(p.P) * g.rows_per_probe;
    g.tiles = int((rows + 127) / 128);
    g.wait_cycles = p.wait_cycles > 0 ? p.wait_cycles : kWaitCycles;
    g.withhold = p.withhold;
}

// Tensor maps of one blend kind of one volume.
template <bool DIST>
bool make_maps(const TcBlendParams& p, CUtensorMap& ma, CUtensorMap& mb) {
    TcArgs g;
    fill_args<DIST>(p, g);
    const int64_t rows = int64_t(p.P) * g.rows_per_probe;
    const uint64_t a_inner = DIST ? uint64_t(2) * p.R : uint64_t(p.R);
    if (!make_map(&ma, DIST ? static_cast<const void*>(p.a_dist) : static_cast<const void*>(p.a_irr), a_inner,
                  uint64_t(rows), kKBlock, 128))
        return false;
    return make_map(&mb, DIST ? static_cast<const void*>(p.w_dist) : static_cast<const void*>(p.w_irr),
                    uint64_t(p.R), uint64_t(g.N), kKBlock, uint32_t(g.N));
}

void fill_job(const TcBlendParams& p, const TcPlan& plan, int k, TcJob& J) {
    std::memset(&J, 0, sizeof(J));
    J.ma = plan.ma[k];
    J.mb = plan.mb[k];
    if (k) fill_args<true>(p, J.g);
    else fill_args<false>(p, J.g);
    J.g.tile0 = plan.tile0[k];
}

template <typename AT>
cudaError_t launch_kernel(const TcLaunchArgs& a, const TcLaunch& L, cudaStream_t st) {
    auto kern = tc_blend_kernel<AT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(L.smem));
    if (e != cudaSuccess) return e;
    kern<<<L.grid, kThreads, L.smem, st>>>(a);
    note_launch();
    return cudaGetLastError();
}

// One launch over the jobs: `local` (two jobs, passed as parameters) or
// d_jobs (device memory).
cudaError_t launch_args(const TcLaunch& L, int storage, const TcJob* local, const void* d_jobs, cudaStream_t st) {
    if (L.grid <= 0) return cudaSuccess;
    TcLaunchArgs a;
    std::memset(&a, 0, sizeof(a));
    if (local) {
        a.local[0] = local[0];
        a.local[1] = local[1];
    }
    a.jobs = local ? nullptr : static_cast<const TcJob*>(d_jobs);
    a.wait_cycles = L.wait_cycles;
    a.njobs = L.njobs;
    a.nmax = L.nmax;
    a.b_bytes = int(L.b_bytes);
    std::memcpy(a.split, L.split, sizeof(a.split));
    return storage == LUXGI_STORAGE_FP16 ? launch_kernel<__half>(a, L, st) : launch_kernel<float>(a, L, st);
}

}  // namespace

bool tc_blend_supported(const luxgi_ddgi_uniform& u) {
    const int R = u.rays_per_probe;
    if (R % 16 != 0 || R < 16) return false;
    const int ni = u.irradiance_probe_side * u.irradiance_probe_side;
    const int nd = u.depth_probe_side * u.depth_probe_side;
    const int Ni = (ni + 15) / 16 * 16, Nd = (nd + 15) / 16 * 16;
    if (Ni > 256 || Nd > 256) return false;      // one UMMA N, one TMA box
    const int kb = (R + kKBlock - 1) / kKBlock;
    const size_t smem = 1024 + size_t(kb) * (Nd > Ni ? Nd : Ni) * 128 + size_t(kStages) * kStageBytes + 256;
    return smem <= 227 * 1024 && encode_fn() != nullptr;
}

bool tc_plan(const TcBlendParams& p, TcPlan& plan) {
    if (p.P <= 0 || !tc_blend_supported(p.u)) return false;
    plan.tile0[0] = plan.tile0[1] = 0;
    return make_maps<false>(p, plan.ma[0], plan.mb[0]) && make_maps<true>(p, plan.ma[1], plan.mb[1]);
}

bool tc_launch_shape(const TcBlendParams* ps, TcPlan* plans, int n, int storage, TcLaunch& L) {
    L = TcLaunch();
    if (n <= 0) return true;
    L.njobs = 2 * n;
    std::vector<int64_t> cost(size_t(L.njobs)), tiles(size_t(L.njobs));
    const int64_t texel_bytes = storage == LUXGI_STORAGE_FP16 ? 2 : 4;
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < 2; ++k) {
            TcArgs g;
            if (k) fill_args<true>(ps[i], g);
            else fill_args<false>(ps[i], g);
            const size_t jk = size_t(2 * i + k);
            plans[i].tile0[k] = int(total);
            tiles[jk] = g.tiles;
            total += g.tiles;
            if (total > INT_MAX) return false;
            L.nmax = std::max(L.nmax, g.N);
            L.b_bytes = std::max(L.b_bytes, size_t(g.kb_b) * size_t(g.N) * 128);
            // bytes a tile moves: its A operand, the history read and the
            // texels written with their borders
            const int64_t cell = int64_t(g.side + 2) * (g.side + 2) * g.nc * texel_bytes;
            cost[jk] = int64_t(g.kb_a) * kStageBytes + 2 * int64_t(128 / g.rows_per_probe) * cell;
            L.wait_cycles = (jk == 0) ? g.wait_cycles : std::min(L.wait_cycles, g.wait_cycles);
        }
    }
    L.total = int(total);
    L.grid = int(std::min<int64_t>(total, std::min(num_sms(), kTcMaxGrid)));
    L.smem = 1024 + L.b_bytes + size_t(kStages) * kStageBytes + 256;
    if (L.smem > 227 * 1024) return false;
    // CTA b starts at the first tile whose cost prefix reaches b / grid of the total
    int64_t C = 0;
    for (int j = 0; j < L.njobs; ++j) C += cost[size_t(j)] * tiles[size_t(j)];
    int j = 0;
    int64_t before = 0;
    for (int b = 0; b <= L.grid; ++b) {
        const int64_t target = L.grid > 0 ? C * b / L.grid : 0;
        while (j < L.njobs && before + cost[size_t(j)] * tiles[size_t(j)] < target) {
            before += cost[size_t(j)] * tiles[size_t(j)];
            ++j;
        }
        if (j == L.njobs) {
            L.split[b] = L.total;
        } else {
            const int64_t c = cost[size_t(j)];
            const int64_t i = std::min<int64_t>((target - before + c - 1) / c, tiles[size_t(j)]);
            const int tile0 = plans[j / 2].tile0[j % 2];
            L.split[b] = int(tile0 + i);
        }
    }
    L.split[L.grid] = L.total;
    return true;
}

size_t tc_job_bytes() { return 2 * sizeof(TcJob); }

void tc_fill_jobs(const TcBlendParams& p, const TcPlan& plan, void* out) {
    TcJob J[2];
    fill_job(p, plan, 0, J[0]);
    fill_job(p, plan, 1, J[1]);
    std::memcpy(out, J, sizeof(J));
}

cudaError_t launch_tc_blend_jobs(const TcLaunch& L, int storage, const void* d_jobs, cudaStream_t st) {
    return launch_args(L, storage, nullptr, d_jobs, st);
}

cudaError_t launch_tc_blend(const TcBlendParams& p, cudaStream_t st) {
    if (p.P <= 0) return cudaSuccess;
    if (!tc_blend_supported(p.u)) return cudaErrorNotSupported;
    TcPlan plan;
    TcLaunch L;
    if (!tc_plan(p, plan) || !tc_launch_shape(&p, &plan, 1, p.storage, L)) return cudaErrorNotSupported;
    TcJob J[2];
    fill_job(p, plan, 0, J[0]);
    fill_job(p, plan, 1, J[1]);
    return launch_args(L, p.storage, J, nullptr, st);
}

}  // namespace luxgi
