// The volume object behind luxgi_ddgi_volume* (C ABI) and the helpers the
// single-volume and batched entry points share.
#pragma once

#include <cuda_runtime.h>

#include "luxgi_internal.h"

// Everything the reference keeps in DDGIPipelineInternal + DDGIUniform
// (Engine/DDGI/DDGIRenderer.cpp:85-97) plus the scene-derived caches.
struct luxgi_ddgi_volume {
    luxgi_ddgi_volume_desc desc;
    int device = 0;
    int P = 0, R = 0, Ti = 0, Td = 0;
    int frames = 0, ping_pong = 0;
    int debug_rays = 0;
    bool bound = false;
    bool tc = false;
    bool auto_variant = false;     // march variant left to the library: chosen at bind by the SDF format
    long long tc_wait_cycles = 0;  // bound of the tensor-core blend's waits (0: ~2 s)
    int tc_withhold = 0;           // test aid, one probe update: withhold one operand load
    int tc_ni = 0, tc_nd = 0;      // padded weight rows (multiples of 16)
    size_t irr_bytes = 0, dist_bytes = 0;
    void* irr[2] = {nullptr, nullptr};
    void* dist[2] = {nullptr, nullptr};
    float4* dirs_trace = nullptr;
    float4* dirs_blend = nullptr;
    void* rays = nullptr;
    int4* info = nullptr;
    float* w_irr = nullptr;
    float* w_dist = nullptr;
    float* n_irr = nullptr;
    float* n_dist = nullptr;
    int* sp_count = nullptr;           // sparse distance blend: contributing rays per texel group
    int* sp_ray = nullptr;
    float4* sp_w = nullptr;
    __half* tc_irr = nullptr;
    __half* tc_dist = nullptr;
    __half* tcw_irr = nullptr;
    __half* tcw_dist = nullptr;
    uint32_t* status = nullptr;
    float4* hit_t = nullptr;       // march records: time, normal
    int* hit_c = nullptr;          // march records: cascade / -1 miss / -2 inside
    float* w2l = nullptr;          // per-object inverse transforms of the bound scene
    int w2l_cap = 0;
    bool w2l_dirty = true;
    uint32_t* shade_chunks = nullptr;   // shading lists (subset of the reference lists)
    uint32_t* shade_culled = nullptr;
    uint32_t* shade_scratch = nullptr;  // 40^3 counts + status
    uint32_t shade_cap = 0;
    void* sdf_quad = nullptr;           // quad-packed copies for march variants 3, 4
    void* mip_quad = nullptr;
    size_t sdf_quad_bytes = 0, mip_quad_bytes = 0;
    // gather textures of the full-resolution SDF and the mip (march variant
    // 10): a 2D CUDA array each, planes tiled gx to a row
    struct GatherTex {
        cudaArray_t arr = nullptr;
        cudaTextureObject_t tex = 0;
        int gx = 0, tw = 0, th = 0, W = 0, H = 0, D = 0, format = -1;
    };
    GatherTex sdf_gt, mip_gt;
    luxgi_sdf_desc sdf{};
    luxgi_surface_desc surf{};
    float* cell_min = nullptr;          // conservative cell minima of the full-resolution SDF
    size_t cell_min_bytes = 0;
    // per-stage CUDA events of the last frame (luxgi_ddgi_set_stage_timing):
    // [0] trace start, [1] march start, [2] shade start, [3] trace end,
    // [4] probe update end
    cudaEvent_t stage_ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool stage_timing = false;
    bool stage_blend_recorded = false;
    uint32_t* shade_bins = nullptr;     // shading order: [2][kShadeBins] counts + cursors
    uint2* shade_key = nullptr;         // [work] (bin, rank within the bin) of each work item
    uint32_t* shade_order = nullptr;    // [work] work items by bin
    int4* mq = nullptr;                 // suspended-march queues (march compaction)
    uint32_t* mq_count = nullptr;
    uint32_t mqa_cap = 0, mqb_cap = 0;
    // split shading: the second stream, its fork / join events, and the
    // resumed rays' histogram [2][kShadeBins], slots [work], order [qa_cap]
    cudaStream_t side = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    uint32_t* split_bins = nullptr;
    uint2* split_key = nullptr;
    uint32_t* split_order = nullptr;
};


namespace luxgi {

int cuda_status(cudaError_t e);
// Scene-derived caches (world-to-local, shading lists, packed SDF copies)
// for the first trace after a bind or a variant change.
int volume_prepare(luxgi_ddgi_volume* v, cudaStream_t st);
// Per-frame kernel parameters of a volume in its current state.
void volume_trace_params(const luxgi_ddgi_volume* v, const float rot[9], TraceParams& p);
void volume_blend_params(const luxgi_ddgi_volume* v, BlendParams& p);
void volume_tc_params(const luxgi_ddgi_volume* v, TcBlendParams& p);
// (Re)allocates the packed SDF copies the volume's march variant reads.
int volume_alloc_packs(luxgi_ddgi_volume* v);
// The march variant a volume that leaves it to the library (march_variant
// 0) runs over this SDF: the gather textures (10) for an FP32 SDF whose
// planes fit the device's gather limits, else the quad-packed copies (4).
int default_march_variant(const luxgi_sdf_desc& sdf);
// Steps of the first march pass with compaction for a volume whose work is
// `work` items and whose march variant / budget / step cap are those of d;
// 0 when the march runs in one pass.
int march_budget_for(const luxgi_ddgi_volume_desc& d, int64_t work, int cascades);
// Launches of at least this many march work items take the compacted march
// and the binned shading by default.
constexpr int64_t kLargeWork = int64_t(1) << 20;
// Steps of the first and second compacted march passes when the volume
// leaves them to the library (march_budget 0); a volume that sets a budget
// runs it in both.
constexpr int kDefaultMarchBudget = 12;
constexpr int kDefaultMarchBudget2 = 8;
inline int march_budget2(int requested, int budget1) {
    return (requested == 0 && budget1 > kDefaultMarchBudget2) ? kDefaultMarchBudget2 : budget1;
}
// Whether a volume's hits are shaded in bin order (shade_order and size).
bool shade_binned(const luxgi_ddgi_volume_desc& d, int64_t work);
// Whether the shading of a binned, compacted march of `work` items is split
// (shade_split).  By default only below 2^24 items: the split hides the
// resume passes' latency tail, which does not grow with the ray count, while
// the contention between the concurrent march and shading does (GB300: +1.7 %
// at 2^22 rays, -0.7 % at 2^25).
constexpr int64_t kSplitMaxWork = int64_t(1) << 24;
inline bool shade_split(const luxgi_ddgi_volume_desc& d, int64_t work) {
    return d.shade_split == 1 || (d.shade_split == 0 && work < kSplitMaxWork);
}
// Device bytes a volume of description d allocates once bound to the scene
// (luxgi_ddgi_create + luxgi_ddgi_bind_scene; debug ray records excluded).
uint64_t volume_device_bytes(const luxgi_ddgi_volume_desc& d, const luxgi_sdf_desc& sdf,
                             const luxgi_surface_desc& surf);

}  // namespace luxgi
