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
// D accumulates in TMEM (FP32).  One CTA per SM, persistent over M tiles:
//   warp 0      TMA producer (cp.async.bulk.tensor, 128B swizzle, 16 KB stages)
//   warp 1      TMEM allocator + single-thread tcgen05.mma issuer
//   warps 2..17 epilogue: tcgen05.ld, normalise, gamma, hysteresis, store
//               (four warps per TMEM lane quadrant, each a quarter of the
//               column chunks) with the border mirrors
// The accumulator is double buffered in TMEM so the epilogue of one tile
// overlaps the MMAs of the next.  Every mbarrier wait is bounded by a clock
// budget; on expiry the kernel raises *status, stops issuing work, drains
// what it issued and frees its TMEM.
#include <cstring>

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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

struct TcArgs {
    luxgi_ddgi_uniform u;
    const float* norm;        // [N] tensor-core normalisers (1 / (2 sum w_fp16))
    const void* prev;
    void* out;
    uint32_t* status;
    int first, P, R, N, T, side, W, nc;   // nc: atlas channels (4 irradiance, 2 distance)
    int rows_per_probe;                   // 4 irradiance, 2 distance
    int kb_a;                             // K blocks of A per tile
    int kb_b;                             // K blocks of B (ceil(R / 64))
    int lo_offset;                        // column of the lo half in A (distance), 0 otherwise
    int tiles;
    long long wait_cycles;                // bound of every mbarrier wait, SM clock cycles
    int withhold;                         // test aid: block 0 skips the first A load of its first tile
};

// Lane-group transposes of the epilogue.  The lanes of one probe each hold
// one channel over 16 accumulator columns (texels); afterwards each lane
// holds every channel of its own texels, so that a texel is loaded (the
// hysteresis history) and stored (with its border mirrors) in one vector
// access instead of one scalar access per channel.
// Irradiance, 4 lanes (r, g, b, zero row) and four 4x4 blocks: lane m ends
// with texels 4k + m as v[4k .. 4k+3].
__device__ __forceinline__ void transpose_quad(float* v, int lane) {
    const bool b1 = (lane & 2) != 0, b0 = (lane & 1) != 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
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

// Distance, 2 lanes (d, d^2) and eight 2x2 blocks: lane m ends with texels
// 2k + m as v[2k .. 2k+1].
__device__ __forceinline__ void transpose_pair(float* v, int lane) {
    const bool b0 = (lane & 1) != 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        float* a = v + 2 * k;
        const float x = __shfl_xor_sync(0xffffffffu, b0 ? a[0] : a[1], 1);
        if (b0) a[0] = x;
        else a[1] = x;
    }
}

template <bool DIST, typename AT>
__device__ __forceinline__ void tc_blend_body(const CUtensorMap& map_a, const CUtensorMap& map_b, const TcArgs& g) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // 1024-byte aligned carve-out: B blocks, A stages, then barriers
    uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int b_block_bytes = g.N * 128;
    uint8_t* smem_b = base;
    uint8_t* smem_a = smem_b + g.kb_b * b_block_bytes;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_a + kStages * kStageBytes);
    uint64_t* full = bars;                       // [kStages]
    uint64_t* empty = bars + kStages;            // [kStages]
    uint64_t* bfull = bars + 2 * kStages;        // [1]
    uint64_t* tfull = bars + 2 * kStages + 1;    // [2]
    uint64_t* tempty = bars + 2 * kStages + 3;   // [2]
    uint64_t* mdrain = bars + 2 * kStages + 5;   // [1] MMAs issued before an abort
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * kStages + 6);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const long long budget = g.wait_cycles > 0 ? g.wait_cycles : kWaitCycles;

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint32_t tmem_cols = (2 * g.N <= 32) ? 32 : (2 * g.N <= 64) ? 64 : (2 * g.N <= 128) ? 128 : (2 * g.N <= 256) ? 256 : 512;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(bfull, 1);
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
    const uint32_t idesc = idesc_f16(128, g.N);
    // phase of the last A load issued into each stage (producer thread)
    uint32_t pending[kStages];
    for (int s = 0; s < kStages; ++s) pending[s] = 0xFFFFFFFFu;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            mbar_expect_tx(bfull, uint32_t(g.kb_b * b_block_bytes));
            for (int kb = 0; kb < g.kb_b; ++kb) tma_load_2d(smem_b + kb * b_block_bytes, &map_b, bfull, kb * kKBlock, 0);
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int tile = blockIdx.x; tile < g.tiles && ok; tile += gridDim.x) {
                for (int kb = 0; kb < g.kb_a && ok; ++kb) {
                    ok = mbar_wait(&empty[stage], phase ^ 1u, abort_flag, budget);
                    if (!ok) break;
                    if (g.withhold && blockIdx.x == 0 && tile == 0 && kb == 0) {
                        // test aid: this stage's load is never issued, so the
                        // MMA issuer's bounded wait on it runs out
                        if (++stage == kStages) { stage = 0; phase ^= 1u; }
                        continue;
                    }
                    const int x = (kb < g.kb_b) ? kb * kKBlock : g.lo_offset + (kb - g.kb_b) * kKBlock;
                    mbar_expect_tx(&full[stage], kStageBytes);
                    tma_load_2d(smem_a + stage * kStageBytes, &map_a, &full[stage], x, tile * 128);
                    pending[stage] = phase;
                    if (++stage == kStages) { stage = 0; phase ^= 1u; }
                }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer
        if (lane == 0) {
            bool ok = mbar_wait(bfull, 0, abort_flag, budget);
            int stage = 0;
            uint32_t phase = 0;
            int it = 0;
            for (int tile = blockIdx.x; tile < g.tiles && ok; tile += gridDim.x, ++it) {
                const int acc = it & 1;
                const uint32_t use = uint32_t(it >> 1);
                ok = mbar_wait(&tempty[acc], (use & 1u) ^ 1u, abort_flag, budget);
                if (!ok) break;
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + uint32_t(acc * g.N);
                for (int kb = 0; kb < g.kb_a && ok; ++kb) {
                    ok = mbar_wait(&full[stage], phase, abort_flag, budget);
                    if (!ok) break;
                    tc_fence_after();
                    const int bk = (kb < g.kb_b) ? kb : kb - g.kb_b;
                    const uint32_t a_addr = smem_u32(smem_a + stage * kStageBytes);
                    const uint32_t b_addr = smem_u32(smem_b + bk * b_block_bytes);
#pragma unroll
                    for (int k = 0; k < kKBlock / 16; ++k) {
                        mma_f16(d_tmem, smem_desc(a_addr + k * 32), smem_desc(b_addr + k * 32), idesc,
                                (kb > 0 || k > 0) ? 1u : 0u);
                    }
                    mma_commit(&empty[stage]);
                    if (++stage == kStages) { stage = 0; phase ^= 1u; }
                }
                if (ok) mma_commit(&tfull[acc]);
            }
        }
    } else {
        // ------------------------------------------------ epilogue
        constexpr int G = DIST ? 2 : 4;         // lanes (accumulator rows) of one probe = atlas channels
        const int q = warp & 3;                 // TMEM lane quadrant of this warp
        const int row = q * 32 + lane;          // accumulator row = (probe, channel)
        const int m = lane & (G - 1);           // after the transpose: texels G k + m of each chunk
        constexpr int kParts = kEpilogueWarps / 4;
        const int part = (warp - 2) >> 2;       // which share of the column chunks
        const int chunks = g.N / 16;
        const int c_begin = (chunks * part / kParts) * 16, c_end = (chunks * (part + 1) / kParts) * 16;
        const luxgi_ddgi_uniform& u = g.u;
        const int XY = u.probe_counts[0] * u.probe_counts[1];
        const int n = g.side;
        const float h = u.hysteresis;
        const float ig = 1.0f / u.ddgi_gamma;
        constexpr int probes_per_tile = 128 / G;
        int it = 0;
        bool ok = true;
        // the previous texels (hysteresis) of this lane in a 16-column chunk:
        // the first chunk's before the wait for the accumulator, each next
        // chunk's while the current one is stored
        auto load_prev = [&](int c0, int cx, int cy, float* pv) {
            int ty = (c0 + m) / n, tx = c0 + m - ty * n;
#pragma unroll
            for (int k = 0; k < 16 / G; ++k) {
                if (c0 + G * k + m < g.T) {
                    AtlasIO<AT>::template ld_texel<G>(
                        g.prev, size_t(cy * (n + 2) + ty + 2) * g.W + (cx * (n + 2) + tx + 2), pv + G * k);
                }
                tx += G;
                while (tx >= n) {
                    tx -= n;
                    ++ty;
                }
            }
        };
        for (int tile = blockIdx.x; tile < g.tiles; tile += gridDim.x, ++it) {
            const int acc = it & 1;
            const uint32_t use = uint32_t(it >> 1);
            const int p = tile * probes_per_tile + row / G;
            const bool live = p < g.P;
            const int cx = p % XY, cy = p / XY;
            const bool hyst = !g.first && live;
            float pv[16], pn[16];
            if (hyst && c_begin < c_end) load_prev(c_begin, cx, cy, pv);
            ok = mbar_wait(&tfull[acc], use & 1u, abort_flag, budget);
            if (!ok) break;
            tc_fence_after();
            for (int c0 = c_begin; c0 < c_end; c0 += 16) {
                float v[16];
                tmem_ld16(tmem_base + (uint32_t(q * 32) << 16) + uint32_t(acc * g.N + c0), v);
                if (DIST) transpose_pair(v, lane);   // every lane: the shuffles span the warp
                else transpose_quad(v, lane);
                if (!live) continue;
                if (hyst && c0 + 16 < c_end) load_prev(c0 + 16, cx, cy, pn);
                int ty = (c0 + m) / n, tx = c0 + m - ty * n;
#pragma unroll
                for (int k = 0; k < 16 / G; ++k) {
                    const int t = c0 + G * k + m;
                    if (t < g.T) {
                        const float nt = __ldg(g.norm + t);
                        float x[G];
#pragma unroll
                        for (int ch = 0; ch < G; ++ch) {
                            if (!DIST && ch == 3) {
                                x[ch] = 1.0f;   // alpha (ProbeUpdate.glsl:150)
                                continue;
                            }
                            float y = v[G * k + ch] * nt;
                            if (!DIST) y = __powf(y, ig);   // within the tensor path's 2e-3
                            if (!g.first) y = y * (1.0f - h) + pv[G * k + ch] * h;
                            x[ch] = y;
                        }
                        store_texel<AT, G>(g.out, g.W, n, cx, cy, tx, ty, x);
                    }
                    tx += G;
                    while (tx >= n) {
                        tx -= n;
                        ++ty;
                    }
                }
                if (hyst) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) pv[j] = pn[j];
                }
            }
            tc_fence_before();
            mbar_arrive(&tempty[acc]);
        }
        (void)ok;
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
            const long long t0 = clock64();
            while (!mbar_try_wait(bfull, 0) && clock64() - t0 < budget) {}
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
    if (threadIdx.x == 0 && *abort_flag) atomicOr(g.status, 1u);
}

template <bool DIST, typename AT>
__global__ void __launch_bounds__(kThreads, 1)
tc_blend_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, const TcArgs g) {
    tc_blend_body<DIST, AT>(map_a, map_b, g);
}

// Same kernel with the per-frame arguments (ping-pong atlases, first-frame
// flag) read from device memory, so that a captured graph replays it frame
// after frame while the host rewrites the arguments.
template <bool DIST, typename AT>
__global__ void __launch_bounds__(kThreads, 1)
tc_blend_dyn_kernel(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b,
                    const TcArgs* __restrict__ gd) {
    tc_blend_body<DIST, AT>(map_a, map_b, *gd);
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

// Tensor maps, shared memory and grid of one blend kind of one volume.
template <bool DIST>
bool plan_kind(const TcBlendParams& p, CUtensorMap& ma, CUtensorMap& mb, size_t& smem, int& grid) {
    TcArgs g;
    fill_args<DIST>(p, g);
    const int64_t rows = int64_t(p.P) * g.rows_per_probe;
    const uint64_t a_inner = DIST ? uint64_t(2) * p.R : uint64_t(p.R);
    if (!make_map(&ma, DIST ? static_cast<const void*>(p.a_dist) : static_cast<const void*>(p.a_irr), a_inner,
                  uint64_t(rows), kKBlock, 128))
        return false;
    if (!make_map(&mb, DIST ? static_cast<const void*>(p.w_dist) : static_cast<const void*>(p.w_irr), uint64_t(p.R),
                  uint64_t(g.N), kKBlock, uint32_t(g.N)))
        return false;
    smem = 1024 + size_t(g.kb_b) * g.N * 128 + size_t(kStages) * kStageBytes + 256;
    grid = g.tiles < num_sms() ? g.tiles : num_sms();
    return true;
}

template <bool DIST, typename AT>
cudaError_t launch_one(const TcBlendParams& p, cudaStream_t st) {
    TcArgs g;
    fill_args<DIST>(p, g);
    CUtensorMap ma, mb;
    size_t smem = 0;
    int grid = 0;
    if (!plan_kind<DIST>(p, ma, mb, smem, grid)) return cudaErrorNotSupported;
    auto kern = tc_blend_kernel<DIST, AT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    kern<<<grid, kThreads, smem, st>>>(ma, mb, g);
    note_launch();
    return cudaGetLastError();
}

template <bool DIST, typename AT>
cudaError_t launch_dyn(const TcPlan& plan, const void* d_args, cudaStream_t st) {
    const int k = DIST ? 1 : 0;
    auto kern = tc_blend_dyn_kernel<DIST, AT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(plan.smem[k]));
    if (e != cudaSuccess) return e;
    kern<<<plan.grid[k], kThreads, plan.smem[k], st>>>(plan.ma[k], plan.mb[k],
                                                      static_cast<const TcArgs*>(d_args) + k);
    note_launch();
    return cudaGetLastError();
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

size_t tc_args_bytes() { return sizeof(TcArgs); }

void tc_fill_args(const TcBlendParams& p, void* out) {
    TcArgs* g = static_cast<TcArgs*>(out);
    fill_args<false>(p, g[0]);
    fill_args<true>(p, g[1]);
}

bool tc_plan(const TcBlendParams& p, TcPlan& plan) {
    if (p.P <= 0 || !tc_blend_supported(p.u)) return false;
    return plan_kind<false>(p, plan.ma[0], plan.mb[0], plan.smem[0], plan.grid[0]) &&
           plan_kind<true>(p, plan.ma[1], plan.mb[1], plan.smem[1], plan.grid[1]);
}

cudaError_t launch_tc_blend_dyn(const TcPlan& plan, int storage, const void* d_args, cudaStream_t st) {
    cudaError_t e;
    if (storage == LUXGI_STORAGE_FP16) {
        e = launch_dyn<false, __half>(plan, d_args, st);
        if (e == cudaSuccess) e = launch_dyn<true, __half>(plan, d_args, st);
    } else {
        e = launch_dyn<false, float>(plan, d_args, st);
        if (e == cudaSuccess) e = launch_dyn<true, float>(plan, d_args, st);
    }
    return e;
}

cudaError_t launch_tc_blend(const TcBlendParams& p, cudaStream_t st) {
    if (p.P <= 0) return cudaSuccess;
    if (!tc_blend_supported(p.u)) return cudaErrorNotSupported;
    cudaError_t e;
    if (p.storage == LUXGI_STORAGE_FP16) {
        e = launch_one<false, __half>(p, st);
        if (e == cudaSuccess) e = launch_one<true, __half>(p, st);
    } else {
        e = launch_one<false, float>(p, st);
        if (e == cudaSuccess) e = launch_one<true, float>(p, st);
    }
    return e;
}

}  // namespace luxgi
