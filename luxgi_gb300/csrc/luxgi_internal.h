// Internal launch interface between the C ABI (capi.cu) and the kernels.
#pragma once

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "luxgi_ddgi.h"
#include "luxgi_common.cuh"

namespace luxgi {

// March variants 6-9 are the pooled march (warps refill finished lanes
// from a ray pool); 1-5, 10 and 11 run one ray per thread.
inline bool pooled_variant(int mv) { return mv >= 6 && mv <= 9; }
inline bool per_ray_variant(int mv) { return (mv >= 1 && mv <= 5) || mv == 10 || mv == 11; }
// The SDF copies a march layout (variant, or a pooled variant's per-ray
// twin) reads: the quad-packed mip (3-5, 11), the gather texture of the
// full-resolution volume (10, 11) and of the mip (10).
inline bool layout_mip_quad(int layout) { return (layout >= 3 && layout <= 5) || layout == 11; }
inline bool layout_sdf_gather(int layout) { return layout == 10 || layout == 11; }
inline bool layout_mip_gather(int layout) { return layout == 10; }

// Texels per thread of the FP32 blend tile; the FP32 weight rows are stored
// ray-major, [R][Tp] with Tp = T rounded up to whole tiles (padding zero).
#ifndef LUXGI_BLEND_TEXEL_TILE
#define LUXGI_BLEND_TEXEL_TILE 4
#endif
constexpr int kTexelTile = LUXGI_BLEND_TEXEL_TILE;   // a multiple of 4
__host__ __device__ inline int blend_row_pitch(int T) { return (T + kTexelTile - 1) / kTexelTile * kTexelTile; }

// Count of kernel launches issued by the library (luxgi_launch_count).
void note_launch(int n = 1);

struct Rot { float m[9]; };

struct TraceParams {
    Rot rot;                 // frame rotation of the ray directions
    luxgi_ddgi_uniform u;
    SdfView sdf;
    SurfaceView surf;
    AtlasView prev;          // previous-frame atlases (mode B bounce)
    const float4* dirs;      // [R] exact FP32 directions
    float4* dirs_blend;      // [R] directions as the blend reads them (raygen output)
    float4* hit_t;           // [P][R] march result: hit time, normal xyz
    int* hit_c;              // [P][R] hit cascade, -1 miss, -2 inside (GISDFRays.comp:93)
    void* out;               // [P][R] x4 radiance rgb + distance (FP32 or FP16)
    int4* info;              // [P][R] steps, cascade (-1 miss), fine samples, 0; or nullptr
    // tensor-core blend operands (nullptr unless the tensor blend is on)
    __half* tc_irr;          // [P][4][R]  r, g, b, 0
    __half* tc_dist;         // [P][2][2R] (d_hi | d_lo), (d2_hi | d2_lo)
    float sky[3];
    float intensity;
    int storage, light_mode, max_steps, bounce;
    int march_variant;
    int shade_variant;
    int P, R;
    int order;               // ray order: 0 ray-major over all probes, 1 probe tiles (kProbeTile)
    int index32;             // work < 2^32: (probe, ray) from a 32-bit index
    int64_t work;            // march / shade work items (P * R, or whole tiles x R)
    FastDiv div_p, div_r, div_x, div_xy;   // divisors P, R, X, X * Y
    // march compaction: pass 1 marches every ray for at most budget1 steps
    // and queues the unfinished ones (qa); pass 2 resumes them for budget2
    // more (unfinished into qb); pass 3 finishes qb.  budget1 == 0: one pass.
    int4* qa;                // [qa_cap][2] suspended marches
    int4* qb;                // [qb_cap][2]
    uint32_t* qcount;        // [0] entries pushed to qa, [1] to qb
    uint32_t qa_cap, qb_cap;
    int budget1, budget2;
    int vol;                 // this volume's index in a batched launch (queue entries)
    // shading order by hit chunk (shade_order 1): the march counts its hits
    // per bin and records each work item's bin and its rank there; a scan
    // of the counts and a placement give `shade_seq`, the work items bin by
    // bin, which the shade kernel walks.
    uint32_t* bin_count;     // [2][kShadeBins]: per-bin counts, then the bin starts
    uint2* bin_key;          // [work] (bin, rank within the bin) of each work item
    uint32_t* shade_seq;     // [work] work items sorted by bin
    uint32_t bin_base;       // this volume's bins: bin_base + (chunk mod bin_span),
    uint32_t bin_span;       // the last one for misses (alone: 0, kShadeBins)
    // split shading (single volume, compacted march): the rays that finish
    // in pass 1 are sorted and shaded while passes 2 and 3 run.  Pass 1
    // marks the rays it queues with kDeferredBin; passes 2 and 3 record
    // theirs in a second histogram and slot array.
    int split;
    int shade_part;          // the shade launch covers: 0 every work item,
                             // 1 the pass-1 finishers, 2 the queued rays (qa)
};

// Slot bin of a ray that pass 1 queued when the shading is split.
constexpr uint32_t kDeferredBin = 0xFFFFFFFFu;

// Shading bins: the 40^3 surface-cache chunks of the hits, then one bin for
// misses, rays inside geometry and padding.
constexpr int kShadeBins = 40 * 40 * 40 + 1;
constexpr int kBatchShadeBins = 1 << 17;

constexpr int kProbeTile = 256;

// Work items of the march and shade launches of a volume in ray order `order`.
inline int64_t trace_work(int P, int R, int order) {
    if (order == 1) return (int64_t(P) + kProbeTile - 1) / kProbeTile * kProbeTile * R;
    return int64_t(P) * R;
}

// (probe, ray) of work item idx; false for the padding of the last tile.
//   order 0: idx = ray * P + probe
//   order 1: idx = (tile * R + ray) * kProbeTile + j, probe = tile * kProbeTile + j
__device__ __forceinline__ bool probe_ray(const TraceParams& p, int64_t idx, int& probe, int& ray) {
    if (p.order == 1) {
        const int64_t tr = idx / kProbeTile;
        const int j = int(idx % kProbeTile);
        int64_t tile;
        if (p.index32) {
            tile = fdiv(uint32_t(tr), p.div_r);
        } else {
            tile = tr / p.R;
        }
        ray = int(tr - tile * p.R);
        const int64_t pr = tile * kProbeTile + j;
        probe = int(pr);
        return pr < p.P;
    }
    if (p.index32) {
        const uint32_t r = fdiv(uint32_t(idx), p.div_p);
        ray = int(r);
        probe = int(uint32_t(idx) - r * p.div_p.d);
    } else {
        ray = int(idx / p.P);
        probe = int(idx - int64_t(ray) * p.P);
    }
    return true;
}

struct BlendParams {
    luxgi_ddgi_uniform u;
    const float4* dirs;      // [R] directions as the blend sees them
    const void* rays;        // [P][R] x4
    const void* prev_irr;
    const void* prev_dist;
    void* out_irr;
    void* out_dist;
    float* w_irr;            // [R][blend_row_pitch(Ti)] cut weights, ray-major
    float* w_dist;           // [R][blend_row_pitch(Td)]
    float* n_irr;            // [Ti] 1/(2 sum w) or 1 (then the tensor-core normalisers)
    float* n_dist;           // [Td]
    __half* tcw_irr;         // [tc_ni][R] FP16 tensor-core weights, or nullptr
    __half* tcw_dist;        // [tc_nd][R]
    int tc_ni, tc_nd;        // tensor-core weight rows (texels padded to 16)
    int storage, first, P, R;
    // the distance blend's contributing rays (blend.cu, sparse distance
    // blend), or nullptr: per 4-texel group g, sp_count[g] rays, their
    // indices sp_ray[g * R + i] ascending and their four weights sp_w[g * R + i]
    int* sp_count;
    int* sp_ray;
    float4* sp_w;
};
// Rays a volume may have for the sparse distance blend (its shared-memory
// column of distances, 33 floats a ray, within a 227 KB block).
constexpr int kSparseMaxRays = 1536;

cudaError_t launch_raygen(const Rot& rot, int R, int storage, float4* dirs_trace, float4* dirs_blend,
                          cudaStream_t st);

// ------------------------------------------------------- batched launches
// One launch covers many volumes: block b belongs to volume v when
// starts[v] <= b < starts[v + 1] (starts has n + 1 entries, starts[0] = 0),
// and the volume's parameters are vp[v] in device memory.
__device__ __forceinline__ int batch_volume(const int* __restrict__ starts, int n, int b) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(starts + mid) <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Copies one parameter block to shared memory (all threads of the block
// take part) and returns it there.
template <typename T>
__device__ __forceinline__ const T& stage_params(const T* __restrict__ src, uint32_t* dst) {
    static_assert(sizeof(T) % 4 == 0, "parameter blocks are word multiples");
    const uint32_t* s = reinterpret_cast<const uint32_t*>(src);
    for (int i = threadIdx.x; i < int(sizeof(T) / 4); i += blockDim.x) dst[i] = __ldg(s + i);
    __syncthreads();
    return *reinterpret_cast<const T*>(dst);
}

cudaError_t launch_raygen_batch(const TraceParams* vp, const int* starts, int n, int blocks, cudaStream_t st);
// Suspended-march queue capacities for `work` work items (entries of 32 B).
inline uint32_t march_qa_cap(int64_t work) { return uint32_t((work * 3 + 4) / 5); }
inline uint32_t march_qb_cap(int64_t work) { return uint32_t((work + 4) / 5); }
// variant 1-5 as TraceParams::march_variant; tpb 128 or 256 rays a block.
// With compaction (budget1 > 0 in the parameter blocks) the batch shares the
// queues q (two int4 per entry, capacities qa_cap / qb_cap, counters qcount)
// and the resume passes follow the first.
cudaError_t launch_march_batch(const TraceParams* vp, const int* starts, int n, int blocks, int variant, int tpb,
                               int sdf_format, int compact, uint32_t* qcount, cudaStream_t st);
cudaError_t launch_shade_batch(const TraceParams* vp, const int* starts, int n, int blocks, int light_mode,
                               int shade_variant, cudaStream_t st);
cudaError_t launch_march(const TraceParams& p, cudaStream_t st);
// The compacted march with split shading: pass 1 with p, `after_first`
// recorded on st, passes 2 and 3 with `resume` (its own histogram and slots).
cudaError_t launch_march_split(const TraceParams& p, const TraceParams& resume, cudaEvent_t after_first,
                               cudaStream_t st);
cudaError_t launch_shade(const TraceParams& p, cudaStream_t st);
// tensor-core blend operands from the shaded rays (coalesced, after shading)
cudaError_t launch_tc_pack(const TraceParams& p, cudaStream_t st);
cudaError_t launch_tc_pack_batch(const TraceParams* vp, const int* starts, int n, int blocks, cudaStream_t st);
// Scan of the shading bins and placement of the work items into `shade_seq`
// (shade_part 2: of the queued rays, read from qa).
cudaError_t launch_shade_sort(const TraceParams& p, cudaStream_t st);
// The same over raw arrays: bins [2][nb] (counts, starts), (bin, rank)
// slots and seq [work].
cudaError_t launch_bin_sort(uint32_t* bins, int nb, const uint2* slots, uint32_t* seq, int64_t work,
                            cudaStream_t st);
// Batched shading in bin order: seq holds batch-wide work indices; work_off
// [n + 1] the first batch-wide index of each volume.
cudaError_t launch_shade_batch_sorted(const TraceParams* vp, const int* work_off, int n, const uint32_t* seq,
                                      int64_t work, int light_mode, int shade_variant, cudaStream_t st);
cudaError_t launch_world_to_local(const luxgi_surface_object* objs, int n, float* w2l, cudaStream_t st);
size_t quad_bytes(int W, int H, int D, int format);
size_t cell_min_bytes(int W, int H, int D);
// The one-bit-per-cell table that follows the cell minima in their buffer.
const uint32_t* cell_bits(const float* cmin, int W, int H, int D);
cudaError_t launch_cell_min(const void* src, int W, int H, int D, int format, float resolution, float* dst,
                            cudaStream_t st);
cudaError_t launch_quad_pack(const void* src, int W, int H, int D, int format, void* dst, cudaStream_t st);
cudaError_t launch_gather_pack(const void* src, int W, int H, int D, int gx, int tw, int th, int format, void* dst,
                               cudaStream_t st);
size_t pair_bytes(int W, int H, int D, int format);
cudaError_t launch_pair_pack(const void* src, int W, int H, int D, int format, void* dst, cudaStream_t st);
cudaError_t launch_shade_lists(const luxgi_surface_data& d, const luxgi_surface_object* objects,
                               const uint32_t* ref_chunks, const uint32_t* ref_culled, float thr, uint32_t* chunks,
                               uint32_t* culled, uint32_t capacity, uint32_t* d_counts, uint32_t* d_status,
                               cudaStream_t st);
cudaError_t launch_weights(const BlendParams& p, cudaStream_t st);
cudaError_t launch_blend(const BlendParams& p, cudaStream_t st);
// batched weights / blend (block-to-volume maps as above); pp = probes per
// thread of the FP32 blend tile (1, 2 or 4)
int weight_rows(const BlendParams& p);
int blend_blocks(const BlendParams& p, bool depth, int pp);
size_t blend_smem(const BlendParams& p, bool depth, int pp);
cudaError_t launch_weights_batch(const BlendParams* vp, const int* starts, int n, int blocks, cudaStream_t st);
cudaError_t launch_blend_batch(const BlendParams* vp, const int* starts_irr, int blocks_irr, size_t smem_irr,
                               const int* starts_dist, int blocks_dist, size_t smem_dist, int n, int pp,
                               int storage, cudaStream_t st);
cudaError_t launch_border(const luxgi_ddgi_uniform& u, void* irr, void* dist, int storage, cudaStream_t st);
cudaError_t launch_inject(const luxgi_ddgi_uniform& u, const SurfaceView& s, const void* gb0, const void* gb1,
                          int gbuffer_format, const uint8_t* pbr, const void* direct, void* light, int light_format,
                          const AtlasView& A, int num_tiles, float intensity, int bounce, cudaStream_t st);
cudaError_t launch_surface_light(const SdfView& sdf, const luxgi_surface_desc& s, const luxgi_surface_lighting& L,
                                 void* out, cudaStream_t st);
cudaError_t launch_sample_irradiance(const luxgi_ddgi_uniform& u, const AtlasView& A, const float* pos,
                                     const float* nrm, const float* wo, float* out, int n, cudaStream_t st);
struct Mat4 {
    float m[16];   // column-major
};
cudaError_t launch_sample_probe(const luxgi_ddgi_uniform& u, const AtlasView& A, const float* depth,
                                const float* normal, int nch, int W, int H, const float cam[3], const float vpi[16],
                                void* out, cudaStream_t st);
cudaError_t launch_mip(const luxgi_sdf_desc& s, void* mip, void* tmp, cudaStream_t st);
cudaError_t launch_mip_cascade(const luxgi_sdf_desc& s, int k, bool flood, void* mip, void* tmp, cudaStream_t st);
cudaError_t launch_cull(const luxgi_surface_data& d, const luxgi_surface_object* objects, uint32_t* chunks,
                        uint32_t* culled, uint32_t capacity, uint32_t* d_counts, uint32_t* d_status,
                        cudaStream_t st);

// Tensor-core blend (tcgen05).  One launch runs a list of jobs, a job
// being one blend kind (irradiance or distance) of one volume: both kinds of
// one volume (launch_tc_blend), or of every volume of a batch
// (launch_tc_blend_jobs).  Returns cudaErrorNotSupported when a shape is
// outside what the kernel handles.
struct TcBlendParams {
    luxgi_ddgi_uniform u;
    const __half* a_irr;     // [P*4][R]
    const __half* a_dist;    // [P*2][2R]
    const __half* w_irr;     // [Ni][R]  (Ni = Ti padded to 16), K-major
    const __half* w_dist;    // [Nd][R]
    const float* n_irr;
    const float* n_dist;
    const void* prev_irr;
    const void* prev_dist;
    void* out_irr;
    void* out_dist;
    uint32_t* status;        // device word: nonzero = a bounded wait gave up
    int storage, first, P, R, Ni, Nd;
    long long wait_cycles;   // bound of each device wait in SM cycles (0 = ~2 s)
    int withhold;            // test aid: one operand load withheld (see blend_tc.cu)
};
cudaError_t launch_tc_blend(const TcBlendParams& p, cudaStream_t st);
bool tc_blend_supported(const luxgi_ddgi_uniform& u);

// Graph-replayable batched form.  The tensor maps of a volume's two jobs
// (index 0 irradiance, 1 distance) and their place in the launch's tile
// list are fixed per plan; the jobs themselves (maps + per-frame
// arguments, tc_job_bytes() per volume, filled by tc_fill_jobs) live in
// device memory, 128-byte aligned, volume after volume.
struct TcPlan {
    CUtensorMap ma[2], mb[2];
    int tile0[2];            // first tile of each job in the launch's tile list
};
constexpr int kTcMaxGrid = 256;
// Shape of one launch: shared memory, grid, the widest job (TMEM columns)
// and the split of the tile list between the CTAs (by estimated cost).
struct TcLaunch {
    size_t smem = 0, b_bytes = 0;
    int grid = 0, njobs = 0, nmax = 0, total = 0;
    long long wait_cycles = 0;
    int split[kTcMaxGrid + 1] = {};
};
bool tc_plan(const TcBlendParams& p, TcPlan& plan);
// Places the n volumes' jobs in one tile list (plans[i].tile0) and sizes the launch.
bool tc_launch_shape(const TcBlendParams* ps, TcPlan* plans, int n, int storage, TcLaunch& L);
size_t tc_job_bytes();
void tc_fill_jobs(const TcBlendParams& p, const TcPlan& plan, void* out);
cudaError_t launch_tc_blend_jobs(const TcLaunch& L, int storage, const void* d_jobs, cudaStream_t st);

}  // namespace luxgi
