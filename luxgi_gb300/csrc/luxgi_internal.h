// Internal launch interface between the C ABI (capi.cu) and the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "luxgi_ddgi.h"
#include "luxgi_common.cuh"

namespace luxgi {

// Count of kernel launches issued by the library (luxgi_launch_count).
void note_launch(int n = 1);

struct Rot { float m[9]; };

struct TraceParams {
    luxgi_ddgi_uniform u;
    SdfView sdf;
    SurfaceView surf;
    AtlasView prev;          // previous-frame atlases (mode B bounce)
    const float4* dirs;      // [R] exact FP32 directions
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
};

struct BlendParams {
    luxgi_ddgi_uniform u;
    const float4* dirs;      // [R] directions as the blend sees them
    const void* rays;        // [P][R] x4
    const void* prev_irr;
    const void* prev_dist;
    void* out_irr;
    void* out_dist;
    const float* w_irr;      // [Ti][R] cut weights
    const float* w_dist;     // [Td][R]
    const float* n_irr;      // [Ti] 1/(2 sum w) or 1
    const float* n_dist;     // [Td]
    int storage, first, P, R;
};

cudaError_t launch_raygen(const Rot& rot, int R, int storage, float4* dirs_trace, float4* dirs_blend,
                          cudaStream_t st);
cudaError_t launch_trace(const TraceParams& p, cudaStream_t st);
cudaError_t launch_shade(const TraceParams& p, cudaStream_t st);
cudaError_t launch_world_to_local(const luxgi_surface_object* objs, int n, float* w2l, cudaStream_t st);
size_t quad_bytes(int W, int H, int D, int format);
cudaError_t launch_quad_pack(const void* src, int W, int H, int D, int format, void* dst, cudaStream_t st);
size_t pair_bytes(int W, int H, int D, int format);
cudaError_t launch_pair_pack(const void* src, int W, int H, int D, int format, void* dst, cudaStream_t st);
cudaError_t launch_shade_lists(const luxgi_surface_data& d, const luxgi_surface_object* objects,
                               const uint32_t* ref_chunks, const uint32_t* ref_culled, float thr, uint32_t* chunks,
                               uint32_t* culled, uint32_t capacity, uint32_t* d_counts, uint32_t* d_status,
                               cudaStream_t st);
cudaError_t launch_weights(const luxgi_ddgi_uniform& u, const float4* dirs, float* w_irr, float* w_dist,
                           float* n_irr, float* n_dist, __half* tc_w_irr, __half* tc_w_dist, int tc_n_irr,
                           int tc_n_dist, cudaStream_t st);
cudaError_t launch_blend(const BlendParams& p, cudaStream_t st);
cudaError_t launch_border(const luxgi_ddgi_uniform& u, void* irr, void* dist, int storage, cudaStream_t st);
cudaError_t launch_inject(const luxgi_ddgi_uniform& u, const SurfaceView& s, const float* gb0, const float* gb1,
                          const __half* direct, __half* light, const AtlasView& A, int num_tiles, float intensity,
                          int bounce, cudaStream_t st);
cudaError_t launch_sample_irradiance(const luxgi_ddgi_uniform& u, const AtlasView& A, const float* pos,
                                     const float* nrm, const float* wo, float* out, int n, cudaStream_t st);
cudaError_t launch_mip(const luxgi_sdf_desc& s, void* mip, void* tmp, cudaStream_t st);
cudaError_t launch_cull(const luxgi_surface_data& d, const luxgi_surface_object* objects, uint32_t* chunks,
                        uint32_t* culled, uint32_t capacity, uint32_t* d_counts, uint32_t* d_status,
                        cudaStream_t st);

// Tensor-core blend (tcgen05).  Returns cudaErrorNotSupported when the
// shape is outside what the kernel handles.
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
};
cudaError_t launch_tc_blend(const TcBlendParams& p, cudaStream_t st);
bool tc_blend_supported(const luxgi_ddgi_uniform& u);

}  // namespace luxgi
