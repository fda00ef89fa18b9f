// C ABI of the DDGI probe-update path (include/luxgi_ddgi.h).
//
// Replaces the bodies of the three ECS systems of Engine/DDGI/DDGIRenderer.cpp
// (trace_rays :217-330, probe_update :347-413, border_update :418-464) and
// end_frame (:335-342); the volume object owns what DDGIPipelineInternal and
// the DDGIUniform hold there (:85-97).
#include <atomic>
#include <cmath>
#include <cstring>
#include <new>

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "luxgi_volume.h"

namespace luxgi {
static std::atomic<uint64_t> g_launches{0};
void note_launch(int n) { g_launches.fetch_add(uint64_t(n), std::memory_order_relaxed); }
}  // namespace luxgi

using namespace luxgi;


int luxgi::cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return LUXGI_OK;
    if (e == cudaErrorMemoryAllocation) return LUXGI_ENOMEM;
    if (e == cudaErrorNotSupported) return LUXGI_EUNSUPPORTED;
    return LUXGI_ECUDA;
}

namespace {

int check_uniform(const luxgi_ddgi_uniform& u) {
    for (int k = 0; k < 3; ++k)
        if (u.probe_counts[k] <= 0) return LUXGI_EINVAL;
    if (u.irradiance_probe_side < 1 || u.irradiance_probe_side > 32) return LUXGI_EINVAL;
    if (u.depth_probe_side < 1 || u.depth_probe_side > 32) return LUXGI_EINVAL;
    if (u.rays_per_probe < 1 || u.rays_per_probe > 4096) return LUXGI_EINVAL;
    if (!(u.step[0] > 0.0f) || !(u.step[1] > 0.0f) || !(u.step[2] > 0.0f)) return LUXGI_EINVAL;
    if (!(u.ddgi_gamma > 0.0f)) return LUXGI_EINVAL;
    const int64_t P = int64_t(u.probe_counts[0]) * u.probe_counts[1] * u.probe_counts[2];
    if (P > (int64_t(1) << 26)) return LUXGI_EINVAL;
    const int64_t XY = int64_t(u.probe_counts[0]) * u.probe_counts[1];
    if (u.irradiance_width != (u.irradiance_probe_side + 2) * XY + 2) return LUXGI_EINVAL;
    if (u.irradiance_height != (u.irradiance_probe_side + 2) * u.probe_counts[2] + 2) return LUXGI_EINVAL;
    if (u.depth_width != (u.depth_probe_side + 2) * XY + 2) return LUXGI_EINVAL;
    if (u.depth_height != (u.depth_probe_side + 2) * u.probe_counts[2] + 2) return LUXGI_EINVAL;
    return LUXGI_OK;
}

template <typename T> cudaError_t dmalloc(T** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(p), bytes);
}

using GatherTex = luxgi_ddgi_volume::GatherTex;

void gather_free(GatherTex& g) {
    if (g.tex) cudaDestroyTextureObject(g.tex);
    if (g.arr) cudaFreeArray(g.arr);
    g = GatherTex{};
}

// The gather texture of a W x H x D volume (march variants 10, 11): planes of
// (W + 2) x (H + 2) texels tiled gx to a row within the device's texture
// gather limits, in a CUDA array made for gathers; point sampling,
// unnormalised coordinates.  Reuses the array when the shape is unchanged.
// Planes a row of the gather texture of a W x H x D volume: the largest
// power of two within the device's gather width (and no more than the
// planes need), so a plane's tile is a shift and a mask; 0 when the tiled
// planes exceed the gather limits, -1 when the limits cannot be read.
int gather_planes_per_row(int W, int H, int D) {
    int dev = 0, maxw = 0, maxh = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&maxw, cudaDevAttrMaxTexture2DGatherWidth, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&maxh, cudaDevAttrMaxTexture2DGatherHeight, dev);
    if (e != cudaSuccess) return -1;
    const int pw = W + 2, ph = H + 2;
    int gx = 1;
    while (gx * 2 * pw <= maxw && gx < D) gx *= 2;
    const int gy = (D + gx - 1) / gx;
    if (gx * pw > maxw || int64_t(gy) * ph > int64_t(maxh)) return 0;
    return gx;
}

int gather_alloc(GatherTex& g, int W, int H, int D, int format) {
    if (g.arr && g.W == W && g.H == H && g.D == D && g.format == format) return LUXGI_OK;
    gather_free(g);
    const int gx = gather_planes_per_row(W, H, D);
    if (gx < 0) return LUXGI_ECUDA;
    if (gx == 0) return LUXGI_EUNSUPPORTED;
    const int pw = W + 2, ph = H + 2;
    const int gy = (D + gx - 1) / gx;
    cudaError_t e;
    const cudaChannelFormatDesc cd =
        format == LUXGI_STORAGE_FP16 ? cudaCreateChannelDescHalf() : cudaCreateChannelDesc<float>();
    e = cudaMallocArray(&g.arr, &cd, size_t(gx * pw), size_t(gy * ph), cudaArrayTextureGather);
    if (e != cudaSuccess) {
        g.arr = nullptr;
        return e == cudaErrorMemoryAllocation ? LUXGI_ENOMEM : cuda_status(e);
    }
    cudaResourceDesc rd{};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = g.arr;
    cudaTextureDesc td{};
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    e = cudaCreateTextureObject(&g.tex, &rd, &td, nullptr);
    if (e != cudaSuccess) {
        g.tex = 0;
        gather_free(g);
        return cuda_status(e);
    }
    g.gx = gx;
    g.tw = gx * pw;
    g.th = gy * ph;
    g.W = W;
    g.H = H;
    g.D = D;
    g.format = format;
    return LUXGI_OK;
}

// Fills a gather texture from the linear volume `src` through a staging
// image (allocated for the copy).
cudaError_t gather_fill(const GatherTex& g, const void* src, cudaStream_t st) {
    const size_t esz = g.format == LUXGI_STORAGE_FP16 ? 2 : 4;
    void* stage = nullptr;
    cudaError_t e = cudaMallocAsync(&stage, esz * size_t(g.tw) * size_t(g.th), st);
    if (e != cudaSuccess) return e;
    e = launch_gather_pack(src, g.W, g.H, g.D, g.gx, g.tw, g.th, g.format, stage, st);
    if (e == cudaSuccess)
        e = cudaMemcpy2DToArrayAsync(g.arr, 0, 0, stage, esz * size_t(g.tw), esz * size_t(g.tw), size_t(g.th),
                                     cudaMemcpyDeviceToDevice, st);
    const cudaError_t f = cudaFreeAsync(stage, st);
    return e != cudaSuccess ? e : f;
}

GatherVol gather_view(const GatherTex& g) {
    GatherVol v{};
    v.tex = g.tex;
    v.lg = 0;
    while ((1 << (v.lg + 1)) <= g.gx) ++v.lg;
    return v;
}

void free_volume(luxgi_ddgi_volume* v) {
    void* ptrs[] = {v->irr[0], v->irr[1], v->dist[0], v->dist[1], v->dirs_trace, v->dirs_blend, v->rays, v->info,
                    v->w_irr, v->w_dist, v->n_irr, v->n_dist, v->tc_irr, v->tc_dist, v->tcw_irr, v->tcw_dist,
                    v->status, v->hit_t, v->hit_c, v->w2l, v->shade_chunks, v->shade_culled, v->shade_scratch,
                    v->sdf_quad, v->mip_quad, v->mq, v->mq_count, v->cell_min, v->shade_bins, v->shade_key,
                    v->shade_order, v->split_bins, v->split_key, v->split_order, v->sp_count, v->sp_ray,
                    v->sp_w};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    gather_free(v->sdf_gt);
    gather_free(v->mip_gt);
    if (v->fork_ev) cudaEventDestroy(v->fork_ev);
    if (v->join_ev) cudaEventDestroy(v->join_ev);
    if (v->side) cudaStreamDestroy(v->side);
}

// Second stream, events and buffers of the split shading, made on the
// first trace that uses it.
int alloc_split(luxgi_ddgi_volume* v, int64_t work) {
    if (v->side) return LUXGI_OK;
    cudaError_t e = dmalloc(&v->split_bins, sizeof(uint32_t) * 2 * kShadeBins);
    if (e == cudaSuccess) e = dmalloc(&v->split_key, sizeof(uint2) * size_t(work));
    if (e == cudaSuccess) e = dmalloc(&v->split_order, sizeof(uint32_t) * size_t(v->mqa_cap));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->fork_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v->join_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&v->side, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        void* ptrs[] = {v->split_bins, v->split_key, v->split_order};
        for (void* q : ptrs)
            if (q) cudaFree(q);
        if (v->fork_ev) cudaEventDestroy(v->fork_ev);
        if (v->join_ev) cudaEventDestroy(v->join_ev);
        v->split_bins = nullptr;
        v->split_key = nullptr;
        v->split_order = nullptr;
        v->fork_ev = v->join_ev = nullptr;
        v->side = nullptr;
        return cuda_status(e);
    }
    return LUXGI_OK;
}

// The march samples the SDF and its mip with 32-bit texel indices: fewer
// than 2^32 texels in each packed volume.
bool sdf_texels_fit(const luxgi_sdf_desc& s) {
    const uint64_t r = uint64_t(s.resolution > 0 ? s.resolution : 0);
    const uint64_t m = uint64_t(s.mip_resolution > 0 ? s.mip_resolution : 0);
    const uint64_t C = uint64_t(s.data.cascades_count);
    return r * C * r * r < (uint64_t(1) << 32) && m * C * m * m < (uint64_t(1) << 32);
}

// exact_div on the host: the same reciprocal (IEEE single division) and
// power-of-two flag
ExactDiv host_exact_div(float d) {
    uint32_t b;
    std::memcpy(&b, &d, sizeof(b));
    const uint32_t ex = (b >> 23) & 0xFFu;
    return ExactDiv{d, 1.0f / d, (b & 0x7FFFFFu) == 0u && ex >= 2u && ex <= 252u};
}

SdfView sdf_view(const luxgi_sdf_desc& s) {
    SdfView v{};
    v.data = s.data;
    v.sdf = s.sdf;
    v.mip = s.mip;
    v.res = s.resolution;
    v.mres = s.mip_resolution;
    v.C = int(s.data.cascades_count);
    v.format = s.format;
    for (int k = 0; k < 4; ++k) {
        v.div_ext[k] = host_exact_div(s.data.cascade_pos_distance[k][3] * 2.0f);
        v.div_voxel[k] = host_exact_div(s.data.cascade_voxel_size[k]);
    }
    v.div_count = host_exact_div(float(v.C));
    v.chunk = 32.0f / s.data.resolution;
    v.margin = 4.0f / s.data.resolution;
    v.texel = 1.0f / s.data.resolution;
    return v;
}

SurfaceView surface_view(const luxgi_surface_desc& s, int light_mode, const float* w2l = nullptr) {
    SurfaceView v;
    v.data = s.data;
    v.objects = s.objects;
    v.w2l = w2l;
    v.tiles = s.tiles;
    v.chunks = s.chunks;
    v.culled = s.culled_objects;
    v.depth = s.depth;
    v.color0_format = s.light_format;
    if (light_mode == LUXGI_LIGHT_PER_HIT) {
        v.color0 = s.direct_light;
        v.color1 = s.albedo;
    } else {
        v.color0 = s.light_cache;
        v.color1 = nullptr;
    }
    v.inv_chunk = s.data.chunk_size > 0.0f ? 1.0f / s.data.chunk_size : 0.0f;
    return v;
}

// The surface formats the library reads and writes.
bool surface_formats_valid(const luxgi_surface_desc& s) {
    return (s.light_format == LUXGI_COLOR_RGBA16F || s.light_format == LUXGI_COLOR_R11G11B10F) &&
           (s.gbuffer_format == LUXGI_GBUFFER_RGBA32F || s.gbuffer_format == LUXGI_GBUFFER_RGBA16F);
}

size_t ray_elem_bytes(int storage) { return storage == LUXGI_STORAGE_FP16 ? 8 : 16; }
size_t atlas_elem_bytes(int storage) { return storage == LUXGI_STORAGE_FP16 ? 2 : 4; }

}  // namespace

bool luxgi::shade_binned(const luxgi_ddgi_volume_desc& d, int64_t work) {
    if (pooled_variant(d.march_variant) || work >= (int64_t(1) << 32) || d.shade_order < 0) return false;
    return d.shade_order == 1 || work >= kLargeWork;     // default: large launches
}

int luxgi::march_budget_for(const luxgi_ddgi_volume_desc& d, int64_t work, int cascades) {
    const int mv = d.march_variant == 0 ? 4 : d.march_variant;
    if (d.march_budget < 0 || pooled_variant(mv)) return 0;
    // queue entries hold 32-bit work indices and 16-bit step totals
    if (work >= (int64_t(1) << 32) || int64_t(cascades) * d.max_steps >= 65536) return 0;
    // default: compacted passes after 12 steps (then 8) for large launches
    // (first-pass budgets 8 and 16 measured slower on GB300); small ones
    // cannot amortise the two extra passes
    if (d.march_budget == 0) return work >= kLargeWork ? kDefaultMarchBudget : 0;
    return d.march_budget;
}

int luxgi::default_march_variant(const luxgi_sdf_desc& sdf) {
    // FP32 SDFs: the gather textures of both volumes (one copy; production
    // march 0.847 -> 0.812 ms against the quad-packed copies; the quad mip
    // with the full-resolution gathers, variant 11, runs the same).  FP16
    // SDFs: the quad-packed mip and the full-resolution gathers (precision
    // scene, 131,072 probes: march 4.63 ms against 4.79 ms with both
    // gathers and 4.88 ms with both quad copies).
    const int C = int(sdf.data.cascades_count);
    if (gather_planes_per_row(sdf.resolution * C, sdf.resolution, sdf.resolution) <= 0) return 4;
    if (sdf.format != LUXGI_STORAGE_FP32) return 11;
    if (gather_planes_per_row(sdf.mip_resolution * C, sdf.mip_resolution, sdf.mip_resolution) <= 0) return 11;
    return 10;
}

uint64_t luxgi::volume_device_bytes(const luxgi_ddgi_volume_desc& d, const luxgi_sdf_desc& sdf,
                                    const luxgi_surface_desc& surf) {
    // mirrors the allocations of luxgi_ddgi_create and luxgi_ddgi_bind_scene
    const luxgi_ddgi_uniform& u = d.uniform;
    const uint64_t P = uint64_t(u.probe_counts[0]) * u.probe_counts[1] * u.probe_counts[2];
    const uint64_t R = uint64_t(u.rays_per_probe), PR = P * R;
    const uint64_t Ti = uint64_t(u.irradiance_probe_side) * u.irradiance_probe_side;
    const uint64_t Td = uint64_t(u.depth_probe_side) * u.depth_probe_side;
    const uint64_t ae = atlas_elem_bytes(d.storage);
    uint64_t b = 2 * (uint64_t(u.irradiance_width) * u.irradiance_height * 4 * ae +
                      uint64_t(u.depth_width) * u.depth_height * 2 * ae);
    b += 2 * 16 * R + PR * ray_elem_bytes(d.storage) + 4 * uint64_t(blend_row_pitch(int(Ti)) + blend_row_pitch(int(Td))) * R + 8 * (Ti + Td) + 16 +
         PR * (16 + 4);
    if (d.blend == LUXGI_BLEND_TENSOR) b += PR * 16 + 2 * ((Ti + 15) / 16 * 16 + (Td + 15) / 16 * 16) * R;
    else if (R <= uint64_t(kSparseMaxRays)) b += uint64_t(blend_row_pitch(int(Td)) / 4) * (4 + 20 * R);
    const uint64_t nobj = surf.data.objects_count;
    uint64_t cap = surf.data.culled_objects_capacity;
    if (cap == 0) cap = 1 + 40ull * 40 * 40 * (nobj + 1);
    b += 64 * nobj + 4 * cap + 4 * (2 * 40ull * 40 * 40 + 1);
    const int C = int(sdf.data.cascades_count);
    const int mv = d.march_variant == 0 ? default_march_variant(sdf) : d.march_variant;
    const int layout = pooled_variant(mv) ? mv - 4 : mv;
    if (layout_mip_quad(layout))
        b += quad_bytes(sdf.mip_resolution * C, sdf.mip_resolution, sdf.mip_resolution, sdf.format);
    if (layout == 4) b += quad_bytes(sdf.resolution * C, sdf.resolution, sdf.resolution, sdf.format);
    if (layout == 5) b += pair_bytes(sdf.resolution * C, sdf.resolution, sdf.resolution, sdf.format);
    {
        // the gather textures: planes with a 1-texel apron
        const uint64_t esz = sdf.format == LUXGI_STORAGE_FP16 ? 2 : 4;
        const uint64_t r = uint64_t(sdf.resolution), m = uint64_t(sdf.mip_resolution);
        if (layout_sdf_gather(layout)) b += esz * (r * C + 2) * (r + 2) * r;
        if (layout_mip_gather(layout)) b += esz * (m * C + 2) * (m + 2) * m;
    }
    if (!pooled_variant(mv)) b += cell_min_bytes(sdf.resolution * C, sdf.resolution, sdf.resolution);
    return b;
}

int luxgi::volume_alloc_packs(luxgi_ddgi_volume* v) {
    // quad-packed SDF copies for the march variants that read them
    // (variants 3-5 and 11 per-ray threads, 7-9 the pooled march with the
    // layouts of 3-5)
    const luxgi_sdf_desc& sdf = v->sdf;
    const int C = int(sdf.data.cascades_count);
    const int mv = v->desc.march_variant;
    const int layout = pooled_variant(mv) ? mv - 4 : mv;   // 6..9 -> 2..5
    // the quad samplers index texels with 32-bit arithmetic
    auto quad_texels = [](int W, int H, int D) { return uint64_t(W + 1) * uint64_t(H + 1) * uint64_t(D); };
    if (layout_mip_quad(layout) && quad_texels(sdf.mip_resolution * C, sdf.mip_resolution, sdf.mip_resolution) >> 32)
        return LUXGI_EUNSUPPORTED;
    if (layout == 4 && quad_texels(sdf.resolution * C, sdf.resolution, sdf.resolution) >> 32)
        return LUXGI_EUNSUPPORTED;
    const size_t mq = layout_mip_quad(layout) ? quad_bytes(sdf.mip_resolution * C, sdf.mip_resolution,
                                                           sdf.mip_resolution, sdf.format)
                                              : 0;
    const size_t sq = (layout == 4)   ? quad_bytes(sdf.resolution * C, sdf.resolution, sdf.resolution, sdf.format)
                      : (layout == 5) ? pair_bytes(sdf.resolution * C, sdf.resolution, sdf.resolution, sdf.format)
                                      : 0;
    if (mq != v->mip_quad_bytes) {
        if (v->mip_quad) cudaFree(v->mip_quad);
        v->mip_quad = nullptr;
        v->mip_quad_bytes = 0;
        if (mq) {
            const cudaError_t e = dmalloc(&v->mip_quad, mq);
            if (e != cudaSuccess) return cuda_status(e);
            v->mip_quad_bytes = mq;
        }
    }
    if (sq != v->sdf_quad_bytes) {
        if (v->sdf_quad) cudaFree(v->sdf_quad);
        v->sdf_quad = nullptr;
        v->sdf_quad_bytes = 0;
        if (sq) {
            const cudaError_t e = dmalloc(&v->sdf_quad, sq);
            if (e != cudaSuccess) return cuda_status(e);
            v->sdf_quad_bytes = sq;
        }
    }
    // gather textures for variants 10 (both volumes) and 11 (the
    // full-resolution volume)
    if (layout_sdf_gather(layout)) {
        const int s = gather_alloc(v->sdf_gt, sdf.resolution * C, sdf.resolution, sdf.resolution, sdf.format);
        if (s != LUXGI_OK) return s;
    } else {
        gather_free(v->sdf_gt);
    }
    if (layout_mip_gather(layout)) {
        const int s =
            gather_alloc(v->mip_gt, sdf.mip_resolution * C, sdf.mip_resolution, sdf.mip_resolution, sdf.format);
        if (s != LUXGI_OK) return s;
    } else {
        gather_free(v->mip_gt);
    }
    // cell minima for every per-ray march variant (the pooled march reads none)
    const size_t cb = pooled_variant(mv) ? 0 : cell_min_bytes(sdf.resolution * C, sdf.resolution, sdf.resolution);
    if (cb != v->cell_min_bytes) {
        if (v->cell_min) cudaFree(v->cell_min);
        v->cell_min = nullptr;
        v->cell_min_bytes = 0;
        if (cb) {
            const cudaError_t e = dmalloc(&v->cell_min, cb);
            if (e != cudaSuccess) return cuda_status(e);
            v->cell_min_bytes = cb;
        }
    }
    v->w2l_dirty = true;
    return LUXGI_OK;
}

int luxgi::volume_prepare(luxgi_ddgi_volume* v, cudaStream_t st) {
    if (!v->bound) return LUXGI_ENOTBOUND;
    if (!v->w2l_dirty) return LUXGI_OK;
    cudaError_t e = launch_world_to_local(v->surf.objects, int(v->surf.data.objects_count), v->w2l, st);
    if (e != cudaSuccess) return cuda_status(e);
    float thr = 0.0f;   // largest surface threshold (SDFCommon.glsl:196-199)
    for (int k = 0; k < int(v->sdf.data.cascades_count); ++k)
        thr = std::fmax(thr, v->sdf.data.cascade_voxel_size[k] * 1.05f);
    e = launch_shade_lists(v->surf.data, v->surf.objects, v->surf.chunks, v->surf.culled_objects, thr,
                           v->shade_chunks, v->shade_culled, v->shade_cap, v->shade_scratch,
                           v->shade_scratch + 40 * 40 * 40, st);
    if (e != cudaSuccess) return cuda_status(e);
    const int C = int(v->sdf.data.cascades_count), res = v->sdf.resolution, mres = v->sdf.mip_resolution;
    if (v->mip_quad) {
        e = launch_quad_pack(v->sdf.mip, mres * C, mres, mres, v->sdf.format, v->mip_quad, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (v->cell_min) {
        e = launch_cell_min(v->sdf.sdf, res * C, res, res, v->sdf.format, v->sdf.data.resolution, v->cell_min, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (v->sdf_gt.arr) {
        e = gather_fill(v->sdf_gt, v->sdf.sdf, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (v->mip_gt.arr) {
        e = gather_fill(v->mip_gt, v->sdf.mip, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (v->sdf_quad) {
        e = (v->desc.march_variant == 5 || v->desc.march_variant == 9)
                ? launch_pair_pack(v->sdf.sdf, res * C, res, res, v->sdf.format, v->sdf_quad, st)
                : launch_quad_pack(v->sdf.sdf, res * C, res, res, v->sdf.format, v->sdf_quad, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    v->w2l_dirty = false;
    return LUXGI_OK;
}

void luxgi::volume_trace_params(const luxgi_ddgi_volume* v, const float rot[9], TraceParams& p) {
    const luxgi_ddgi_volume_desc& d = v->desc;
    std::memset(&p, 0, sizeof(p));
    for (int i = 0; i < 9; ++i) p.rot.m[i] = rot[i];
    p.u = d.uniform;
    p.sdf = sdf_view(v->sdf);
    p.surf = surface_view(v->surf, d.light_mode, v->w2l);
    p.surf.chunks = v->shade_chunks;
    p.surf.culled = v->shade_culled;
    p.sdf.sdf_quad = v->sdf_quad;
    p.sdf.mip_quad = v->mip_quad;
    p.sdf.sdf_g = gather_view(v->sdf_gt);
    p.sdf.mip_g = gather_view(v->mip_gt);
    p.sdf.cell_near =
        v->cell_min ? cell_bits(v->cell_min, v->sdf.resolution * int(v->sdf.data.cascades_count), v->sdf.resolution,
                                v->sdf.resolution)
                    : nullptr;
    p.sdf.cw = (v->sdf.resolution * int(v->sdf.data.cascades_count) + kCellSide - 1) / kCellSide;
    p.sdf.ch = (v->sdf.resolution + kCellSide - 1) / kCellSide;
    p.hit_t = v->hit_t;
    p.hit_c = v->hit_c;
    p.prev.irr = v->irr[v->ping_pong];
    p.prev.dist = v->dist[v->ping_pong];
    p.prev.storage = d.storage;
    p.dirs = v->dirs_trace;
    p.dirs_blend = v->dirs_blend;
    p.out = v->rays;
    p.info = v->debug_rays ? v->info : nullptr;
    p.tc_irr = v->tc ? v->tc_irr : nullptr;
    p.tc_dist = v->tc ? v->tc_dist : nullptr;
    for (int k = 0; k < 3; ++k) p.sky[k] = d.sky_radiance[k];
    p.intensity = d.intensity;
    p.storage = d.storage;
    p.light_mode = d.light_mode;
    p.max_steps = d.max_steps;
    p.march_variant = d.march_variant;
    p.shade_variant = d.shade_variant;
    p.bounce = (d.infinite_bounce && v->frames != 0) ? 1 : 0;
    p.P = v->P;
    p.R = v->R;
    p.order = (d.ray_order == 1 && !pooled_variant(d.march_variant)) ? 1 : 0;
    p.work = trace_work(v->P, v->R, p.order);
    p.index32 = p.work < (int64_t(1) << 32) ? 1 : 0;
    p.div_p = make_fastdiv(uint32_t(v->P));
    p.div_r = make_fastdiv(uint32_t(v->R));
    const int budget = v->mq ? march_budget_for(d, p.work, int(v->sdf.data.cascades_count)) : 0;
    p.budget1 = budget;
    p.budget2 = march_budget2(d.march_budget, budget);
    p.qa = v->mq;
    p.qb = v->mq ? v->mq + 2 * size_t(v->mqa_cap) : nullptr;
    p.qcount = v->mq_count;
    p.qa_cap = v->mqa_cap;
    p.qb_cap = v->mqb_cap;
    p.vol = 0;
    const bool sorted = v->shade_bins && shade_binned(d, p.work);
    p.bin_count = sorted ? v->shade_bins : nullptr;
    p.bin_key = sorted ? v->shade_key : nullptr;
    p.shade_seq = sorted ? v->shade_order : nullptr;
    p.bin_base = 0;
    p.bin_span = kShadeBins;
    p.div_x = make_fastdiv(uint32_t(d.uniform.probe_counts[0]));
    p.div_xy = make_fastdiv(uint32_t(d.uniform.probe_counts[0]) * uint32_t(d.uniform.probe_counts[1]));
}

void luxgi::volume_tc_params(const luxgi_ddgi_volume* v, TcBlendParams& p) {
    const luxgi_ddgi_volume_desc& d = v->desc;
    const int rd = v->ping_pong, wr = 1 - v->ping_pong;
    std::memset(&p, 0, sizeof(p));
    p.u = d.uniform;
    p.a_irr = v->tc_irr;
    p.a_dist = v->tc_dist;
    p.w_irr = v->tcw_irr;
    p.w_dist = v->tcw_dist;
    p.n_irr = v->n_irr + v->Ti;
    p.n_dist = v->n_dist + v->Td;
    p.prev_irr = v->irr[rd];
    p.prev_dist = v->dist[rd];
    p.out_irr = v->irr[wr];
    p.out_dist = v->dist[wr];
    p.status = v->status;
    p.wait_cycles = v->tc_wait_cycles;
    p.storage = d.storage;
    p.first = v->frames == 0;
    p.P = v->P;
    p.R = v->R;
    p.Ni = v->tc_ni;
    p.Nd = v->tc_nd;
}

void luxgi::volume_blend_params(const luxgi_ddgi_volume* v, BlendParams& p) {
    const luxgi_ddgi_volume_desc& d = v->desc;
    const int rd = v->ping_pong, wr = 1 - v->ping_pong;
    std::memset(&p, 0, sizeof(p));
    p.u = d.uniform;
    p.dirs = v->dirs_blend;
    p.rays = v->rays;
    p.prev_irr = v->irr[rd];
    p.prev_dist = v->dist[rd];
    p.out_irr = v->irr[wr];
    p.out_dist = v->dist[wr];
    p.w_irr = v->w_irr;
    p.w_dist = v->w_dist;
    p.n_irr = v->n_irr;
    p.n_dist = v->n_dist;
    p.tcw_irr = v->tc ? v->tcw_irr : nullptr;
    p.tcw_dist = v->tc ? v->tcw_dist : nullptr;
    p.tc_ni = v->tc_ni;
    p.tc_nd = v->tc_nd;
    p.storage = d.storage;
    p.first = v->frames == 0;
    p.P = v->P;
    p.R = v->R;
    p.sp_count = v->sp_count;
    p.sp_ray = v->sp_ray;
    p.sp_w = v->sp_w;
}

namespace {

int do_trace(luxgi_ddgi_volume* v, const float rot[9], cudaStream_t st) {
    if (!v->bound) return LUXGI_ENOTBOUND;
    const int order = (v->desc.ray_order == 1 && !pooled_variant(v->desc.march_variant)) ? 1 : 0;
    const int64_t work = trace_work(v->P, v->R, order);
    if (!v->mq && march_budget_for(v->desc, work, int(v->sdf.data.cascades_count)) > 0) {
        // queues of the compacted march, made on the first trace that needs them
        const uint32_t ca = march_qa_cap(work), cb = march_qb_cap(work);
        cudaError_t e = dmalloc(&v->mq, sizeof(int4) * 2 * (size_t(ca) + cb));
        if (e == cudaSuccess) e = dmalloc(&v->mq_count, 2 * sizeof(uint32_t));
        if (e != cudaSuccess) {
            if (v->mq) cudaFree(v->mq);
            v->mq = nullptr;
            return cuda_status(e);
        }
        v->mqa_cap = ca;
        v->mqb_cap = cb;
    }
    if (!v->shade_bins && shade_binned(v->desc, work)) {
        // shading-order buffers, made on the first trace that needs them
        cudaError_t e = dmalloc(&v->shade_bins, sizeof(uint32_t) * 2 * kShadeBins);
        if (e == cudaSuccess) e = dmalloc(&v->shade_key, sizeof(uint2) * size_t(work));
        if (e == cudaSuccess) e = dmalloc(&v->shade_order, sizeof(uint32_t) * size_t(work));
        if (e != cudaSuccess) {
            void* ptrs[] = {v->shade_bins, v->shade_key, v->shade_order};
            for (void* q : ptrs)
                if (q) cudaFree(q);
            v->shade_bins = nullptr;
            v->shade_key = nullptr;
            v->shade_order = nullptr;
            return cuda_status(e);
        }
    }
    TraceParams p;
    volume_trace_params(v, rot, p);
    BlendParams b;
    volume_blend_params(v, b);
    nvtxRangePushA("luxgi_ddgi_trace");
    auto mark = [&](int i) { if (v->stage_timing) cudaEventRecord(v->stage_ev[i], st); };
    mark(0);
    v->stage_blend_recorded = false;
    cudaError_t e = launch_raygen(p.rot, v->R, v->desc.storage, v->dirs_trace, v->dirs_blend, st);
    if (e == cudaSuccess) e = launch_weights(b, st);
    int s = e == cudaSuccess ? volume_prepare(v, st) : cuda_status(e);
    const bool split =
        s == LUXGI_OK && p.bin_count && p.budget1 > 0 && !pooled_variant(p.march_variant) &&
        shade_split(v->desc, p.work);
    if (split) s = alloc_split(v, p.work);
    if (s == LUXGI_OK && split) {
        // pass 1 on st; its finishers sorted and shaded on the side stream
        // while passes 2 and 3 run on st; the queued rays sorted and shaded
        // on st after them; st then waits for the side stream
        TraceParams pa = p, pb = p;
        pa.split = 1;
        pa.shade_part = 1;
        pb.bin_count = v->split_bins;
        pb.bin_key = v->split_key;
        pb.shade_seq = v->split_order;
        pb.shade_part = 2;
        mark(1);
        cudaError_t e2 = cudaMemsetAsync(pa.bin_count, 0, sizeof(uint32_t) * kShadeBins, st);
        if (e2 == cudaSuccess) e2 = cudaMemsetAsync(pb.bin_count, 0, sizeof(uint32_t) * kShadeBins, st);
        if (e2 == cudaSuccess) e2 = launch_march_split(pa, pb, v->fork_ev, st);
        if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(v->side, v->fork_ev, 0);
        if (e2 == cudaSuccess) e2 = launch_shade_sort(pa, v->side);
        if (e2 == cudaSuccess) e2 = launch_shade(pa, v->side);
        if (e2 == cudaSuccess) e2 = cudaEventRecord(v->join_ev, v->side);
        if (e2 == cudaSuccess) {
            mark(2);
            e2 = launch_shade_sort(pb, st);
        }
        if (e2 == cudaSuccess) e2 = launch_shade(pb, st);
        if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(st, v->join_ev, 0);
        if (e2 == cudaSuccess) e2 = launch_tc_pack(p, st);
        s = cuda_status(e2);
        mark(3);
        nvtxRangePop();
        return s;
    }
    if (s == LUXGI_OK) {
        mark(1);
        cudaError_t em = p.bin_count ? cudaMemsetAsync(p.bin_count, 0, sizeof(uint32_t) * kShadeBins, st)
                                     : cudaSuccess;
        if (em == cudaSuccess) em = launch_march(p, st);
        s = cuda_status(em);
    }
    if (s == LUXGI_OK) {
        mark(2);
        cudaError_t es = p.bin_count ? launch_shade_sort(p, st) : cudaSuccess;
        if (es == cudaSuccess) es = launch_shade(p, st);
        if (es == cudaSuccess) es = launch_tc_pack(p, st);
        s = cuda_status(es);
        mark(3);
    }
    nvtxRangePop();
    return s;
}

int do_probe_update(luxgi_ddgi_volume* v, cudaStream_t st) {
    nvtxRangePushA("luxgi_ddgi_probe_update");
    cudaError_t e;
    if (v->tc) {
        TcBlendParams p;
        volume_tc_params(v, p);
        p.withhold = v->tc_withhold;
        v->tc_withhold = 0;
        e = launch_tc_blend(p, st);
    } else {
        BlendParams p;
        volume_blend_params(v, p);
        e = launch_blend(p, st);
    }
    if (e == cudaSuccess && v->stage_timing) {
        e = cudaEventRecord(v->stage_ev[4], st);
        v->stage_blend_recorded = true;
    }
    nvtxRangePop();
    return cuda_status(e);
}

}  // namespace

extern "C" {

const char* luxgi_strerror(int s) {
    switch (s) {
        case LUXGI_OK: return "ok";
        case LUXGI_EINVAL: return "invalid argument";
        case LUXGI_ENOMEM: return "out of device memory or capacity";
        case LUXGI_ECUDA: return "CUDA runtime error";
        case LUXGI_ETIMEOUT: return "bounded device wait timed out";
        case LUXGI_ENOTBOUND: return "scene not bound";
        case LUXGI_EUNSUPPORTED: return "unsupported option";
        case LUXGI_ESCRATCH: return "input exceeds the 1 MiB static scratch of luxgi_sdf_build_mip_noalloc";
        default: return "unknown status";
    }
}

uint64_t luxgi_launch_count(void) { return g_launches.load(); }

int luxgi_ddgi_derive_uniform(luxgi_ddgi_uniform* u) {
    if (!u) return LUXGI_EINVAL;
    for (int k = 0; k < 3; ++k)
        if (u->probe_counts[k] <= 0) return LUXGI_EINVAL;
    const int XY = u->probe_counts[0] * u->probe_counts[1], Z = u->probe_counts[2];
    if (u->irradiance_probe_side <= 0 || u->depth_probe_side <= 0) return LUXGI_EINVAL;
    // 1-texel border per probe plus a 1-texel pad around the atlas
    // (DDGIRenderer.cpp:181-185)
    u->irradiance_width = (u->irradiance_probe_side + 2) * XY + 2;
    u->irradiance_height = (u->irradiance_probe_side + 2) * Z + 2;
    u->depth_width = (u->depth_probe_side + 2) * XY + 2;
    u->depth_height = (u->depth_probe_side + 2) * Z + 2;
    u->probe_counts[3] = 0;
    return check_uniform(*u);
}

int luxgi_ddgi_rotation(const float axis[3], float angle, float out[9]) {
    if (!axis || !out) return LUXGI_EINVAL;
    // glm::angleAxis then mat4_cast: the unit quaternion (axis sin(a/2),
    // cos(a/2)) turned into its rotation matrix, column-major.
    const float h = angle * 0.5f, s = std::sin(h);
    const float x = axis[0] * s, y = axis[1] * s, z = axis[2] * s, w = std::cos(h);
    const float xx = x * x, yy = y * y, zz = z * z, xy = x * y, xz = x * z, yz = y * z, wx = w * x, wy = w * y,
                wz = w * z;
    out[0] = 1.0f - 2.0f * (yy + zz); out[1] = 2.0f * (xy + wz);        out[2] = 2.0f * (xz - wy);
    out[3] = 2.0f * (xy - wz);        out[4] = 1.0f - 2.0f * (xx + zz); out[5] = 2.0f * (yz + wx);
    out[6] = 2.0f * (xz + wy);        out[7] = 2.0f * (yz - wx);        out[8] = 1.0f - 2.0f * (xx + yy);
    return LUXGI_OK;
}

int luxgi_ddgi_frame_rotation(uint64_t seed, uint32_t frame, float out[9]) {
    if (!out) return LUXGI_EINVAL;
    // splitmix64 -> xoshiro256**, one fresh stream per (seed, frame)
    uint64_t x = seed ^ (0xD1B54A32D192ED03ull * (uint64_t(frame) + 1ull));
    uint64_t s[4];
    for (int i = 0; i < 4; ++i) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        s[i] = z ^ (z >> 31);
    }
    auto rotl = [](uint64_t v, int k) { return (v << k) | (v >> (64 - k)); };
    auto next = [&]() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    };
    auto uni = [&](float a, float b) { return a + (b - a) * (float(next() >> 40) * (1.0f / 16777216.0f)); };
    float ax[3] = {uni(-1.0f, 1.0f), uni(-1.0f, 1.0f), uni(-1.0f, 1.0f)};
    const float len = std::sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    if (len > 0.0f) for (float& a : ax) a /= len;
    else { ax[0] = 0.0f; ax[1] = 0.0f; ax[2] = 1.0f; }
    const float angle = uni(0.0f, 1.0f) * 3.14159265f * 2.0f;
    return luxgi_ddgi_rotation(ax, angle, out);
}

int luxgi_ddgi_create(const luxgi_ddgi_volume_desc* desc, luxgi_ddgi_volume** out) {
    if (!desc || !out) return LUXGI_EINVAL;
    *out = nullptr;
    int st = check_uniform(desc->uniform);
    if (st != LUXGI_OK) return st;
    if (desc->storage != LUXGI_STORAGE_FP32 && desc->storage != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    if (desc->light_mode != LUXGI_LIGHT_CACHE && desc->light_mode != LUXGI_LIGHT_PER_HIT) return LUXGI_EINVAL;
    if (desc->blend != LUXGI_BLEND_FP32 && desc->blend != LUXGI_BLEND_TENSOR) return LUXGI_EINVAL;
    if (desc->max_steps < 1) return LUXGI_EINVAL;
    if (desc->march_variant < 0 || desc->march_variant > 11) return LUXGI_EINVAL;
    if (desc->ray_order != 0 && desc->ray_order != 1) return LUXGI_EINVAL;
    if (desc->march_budget < -1) return LUXGI_EINVAL;
    if (desc->shade_split < -1 || desc->shade_split > 1) return LUXGI_EINVAL;
    if (desc->shade_order < -1 || desc->shade_order > 1) return LUXGI_EINVAL;
    if (desc->shade_variant != 0 && desc->shade_variant != 1 && desc->shade_variant != 2 &&
        desc->shade_variant != 4 && desc->shade_variant != 8)
        return LUXGI_EINVAL;
    if (desc->blend == LUXGI_BLEND_TENSOR && !tc_blend_supported(desc->uniform)) return LUXGI_EUNSUPPORTED;
    luxgi_ddgi_volume* v = new (std::nothrow) luxgi_ddgi_volume();
    if (!v) return LUXGI_ENOMEM;
    v->desc = *desc;
    // defaults: the variants measured fastest on the production workload;
    // the march variant is settled when the SDF (its format) is bound
    if (v->desc.march_variant == 0) {
        v->auto_variant = true;
        v->desc.march_variant = 4;
    }
    if (v->desc.shade_variant == 0) v->desc.shade_variant = 1;
    cudaGetDevice(&v->device);
    const luxgi_ddgi_uniform& u = desc->uniform;
    v->P = u.probe_counts[0] * u.probe_counts[1] * u.probe_counts[2];
    v->R = u.rays_per_probe;
    v->Ti = u.irradiance_probe_side * u.irradiance_probe_side;
    v->Td = u.depth_probe_side * u.depth_probe_side;
    v->tc = desc->blend == LUXGI_BLEND_TENSOR;
    v->tc_ni = (v->Ti + 15) / 16 * 16;
    v->tc_nd = (v->Td + 15) / 16 * 16;
    const size_t ae = atlas_elem_bytes(desc->storage);
    v->irr_bytes = size_t(u.irradiance_width) * u.irradiance_height * 4 * ae;
    v->dist_bytes = size_t(u.depth_width) * u.depth_height * 2 * ae;
    const size_t PR = size_t(v->P) * v->R;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = dmalloc(&v->irr[i], v->irr_bytes);
        if (e == cudaSuccess) e = dmalloc(&v->dist[i], v->dist_bytes);
    }
    if (e == cudaSuccess) e = dmalloc(&v->dirs_trace, sizeof(float4) * v->R);
    if (e == cudaSuccess) e = dmalloc(&v->dirs_blend, sizeof(float4) * v->R);
    if (e == cudaSuccess) e = dmalloc(&v->rays, PR * ray_elem_bytes(desc->storage));
    // FP32 weights: ray-major rows padded to whole texel tiles, padding zero
    const size_t wi_bytes = sizeof(float) * size_t(blend_row_pitch(v->Ti)) * v->R;
    const size_t wd_bytes = sizeof(float) * size_t(blend_row_pitch(v->Td)) * v->R;
    if (e == cudaSuccess) e = dmalloc(&v->w_irr, wi_bytes);
    if (e == cudaSuccess) e = dmalloc(&v->w_dist, wd_bytes);
    if (e == cudaSuccess) e = cudaMemset(v->w_irr, 0, wi_bytes);
    if (e == cudaSuccess) e = cudaMemset(v->w_dist, 0, wd_bytes);
    if (e == cudaSuccess) e = dmalloc(&v->n_irr, sizeof(float) * 2 * v->Ti);
    if (e == cudaSuccess) e = dmalloc(&v->n_dist, sizeof(float) * 2 * v->Td);
    if (e == cudaSuccess) e = dmalloc(&v->status, sizeof(uint32_t) * 4);
    if (e == cudaSuccess) e = dmalloc(&v->hit_t, sizeof(float4) * PR);
    if (e == cudaSuccess) e = dmalloc(&v->hit_c, sizeof(int) * PR);
    if (!v->tc && v->R <= kSparseMaxRays) {
        // the sparse distance blend's ray lists: per 4-texel group, up to R
        // ray indices and their weights
        const size_t groups = size_t(blend_row_pitch(v->Td) / 4);
        if (e == cudaSuccess) e = dmalloc(&v->sp_count, sizeof(int) * groups);
        if (e == cudaSuccess) e = dmalloc(&v->sp_ray, sizeof(int) * groups * v->R);
        if (e == cudaSuccess) e = dmalloc(&v->sp_w, sizeof(float4) * groups * v->R);
    }
    if (v->tc) {
        if (e == cudaSuccess) e = dmalloc(&v->tc_irr, sizeof(__half) * PR * 4);
        if (e == cudaSuccess) e = dmalloc(&v->tc_dist, sizeof(__half) * PR * 4);
        if (e == cudaSuccess) e = dmalloc(&v->tcw_irr, sizeof(__half) * v->tc_ni * v->R);
        if (e == cudaSuccess) e = dmalloc(&v->tcw_dist, sizeof(__half) * v->tc_nd * v->R);
    }
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        e = cudaMemset(v->irr[i], 0, v->irr_bytes);
        if (e == cudaSuccess) e = cudaMemset(v->dist[i], 0, v->dist_bytes);
    }
    if (e == cudaSuccess) e = cudaMemset(v->status, 0, sizeof(uint32_t) * 4);
    if (e != cudaSuccess) {
        free_volume(v);
        delete v;
        return cuda_status(e);
    }
    *out = v;
    return LUXGI_OK;
}

int luxgi_ddgi_destroy(luxgi_ddgi_volume* v) {
    if (!v) return LUXGI_EINVAL;
    for (cudaEvent_t& ev : v->stage_ev)
        if (ev) cudaEventDestroy(ev);
    free_volume(v);
    delete v;
    return LUXGI_OK;
}

int luxgi_ddgi_bind_scene(luxgi_ddgi_volume* v, const luxgi_sdf_desc* sdf, const luxgi_surface_desc* surf) {
    if (!v || !sdf || !surf) return LUXGI_EINVAL;
    const int C = int(sdf->data.cascades_count);
    if (C < 1 || C > 4 || sdf->resolution < 4 || sdf->mip_resolution < 1 || !sdf->sdf || !sdf->mip) return LUXGI_EINVAL;
    if (sdf->resolution != int(sdf->data.resolution)) return LUXGI_EINVAL;
    if (sdf->format != LUXGI_STORAGE_FP32 && sdf->format != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    if (!sdf_texels_fit(*sdf)) return LUXGI_EUNSUPPORTED;
    if (!surf->objects || !surf->tiles || !surf->chunks || !surf->culled_objects || !surf->depth) return LUXGI_EINVAL;
    if (surf->data.resolution == 0) return LUXGI_EINVAL;
    if (!surface_formats_valid(*surf)) return LUXGI_EINVAL;
    if (v->desc.light_mode == LUXGI_LIGHT_PER_HIT && (!surf->direct_light || !surf->albedo)) return LUXGI_EINVAL;
    if (v->desc.light_mode == LUXGI_LIGHT_CACHE && !surf->light_cache) return LUXGI_EINVAL;
    const int nobj = int(surf->data.objects_count);
    if (nobj > v->w2l_cap) {
        if (v->w2l) cudaFree(v->w2l);
        v->w2l = nullptr;
        v->w2l_cap = 0;
        const cudaError_t e = dmalloc(&v->w2l, sizeof(float) * 16 * size_t(nobj));
        if (e != cudaSuccess) return cuda_status(e);
        v->w2l_cap = nobj;
    }
    // shading lists are a subset of the reference lists: the same capacity
    // (or the worst case when the descriptor does not state it) always fits
    uint32_t cap = surf->data.culled_objects_capacity;
    if (cap == 0) cap = 1u + 40u * 40u * 40u * uint32_t(nobj + 1);
    if (cap > v->shade_cap) {
        if (v->shade_culled) cudaFree(v->shade_culled);
        v->shade_culled = nullptr;
        v->shade_cap = 0;
        const cudaError_t e = dmalloc(&v->shade_culled, sizeof(uint32_t) * size_t(cap));
        if (e != cudaSuccess) return cuda_status(e);
        v->shade_cap = cap;
    }
    if (!v->shade_chunks) {
        cudaError_t e = dmalloc(&v->shade_chunks, sizeof(uint32_t) * 40 * 40 * 40);
        if (e == cudaSuccess) e = dmalloc(&v->shade_scratch, sizeof(uint32_t) * (40 * 40 * 40 + 1));
        if (e != cudaSuccess) return cuda_status(e);
    }
    v->sdf = *sdf;
    v->surf = *surf;
    if (v->auto_variant) v->desc.march_variant = default_march_variant(*sdf);
    int st = volume_alloc_packs(v);
    if (st == LUXGI_EUNSUPPORTED && v->auto_variant && v->desc.march_variant != 4) {
        v->desc.march_variant = 4;
        st = volume_alloc_packs(v);
    }
    if (st != LUXGI_OK) return st;
    v->w2l_dirty = true;
    v->bound = true;
    return LUXGI_OK;
}

int luxgi_ddgi_trace(luxgi_ddgi_volume* v, const float rot[9], void* stream) {
    if (!v || !rot) return LUXGI_EINVAL;
    return do_trace(v, rot, static_cast<cudaStream_t>(stream));
}

int luxgi_ddgi_probe_update(luxgi_ddgi_volume* v, void* stream) {
    if (!v) return LUXGI_EINVAL;
    return do_probe_update(v, static_cast<cudaStream_t>(stream));
}

int luxgi_ddgi_border_update(luxgi_ddgi_volume* v, void* stream) {
    if (!v) return LUXGI_EINVAL;
    const int wr = 1 - v->ping_pong;
    return cuda_status(launch_border(v->desc.uniform, v->irr[wr], v->dist[wr], v->desc.storage,
                                     static_cast<cudaStream_t>(stream)));
}

int luxgi_ddgi_end_frame(luxgi_ddgi_volume* v) {
    if (!v) return LUXGI_EINVAL;
    v->ping_pong = 1 - v->ping_pong;
    v->frames += 1;
    return LUXGI_OK;
}

int luxgi_ddgi_update(luxgi_ddgi_volume* v, const float rot[9], void* stream) {
    if (!v || !rot) return LUXGI_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int s = do_trace(v, rot, st);
    if (s != LUXGI_OK) return s;
    s = do_probe_update(v, st);
    if (s != LUXGI_OK) return s;
    return luxgi_ddgi_end_frame(v);
}

int luxgi_ddgi_get_atlases(const luxgi_ddgi_volume* v, luxgi_ddgi_atlases* out) {
    if (!v || !out) return LUXGI_EINVAL;
    const luxgi_ddgi_uniform& u = v->desc.uniform;
    out->irradiance = v->irr[v->ping_pong];
    out->distance = v->dist[v->ping_pong];
    out->prev_irradiance = v->irr[1 - v->ping_pong];
    out->prev_distance = v->dist[1 - v->ping_pong];
    out->irradiance_width = u.irradiance_width;
    out->irradiance_height = u.irradiance_height;
    out->depth_width = u.depth_width;
    out->depth_height = u.depth_height;
    out->storage = v->desc.storage;
    out->frames = v->frames;
    return LUXGI_OK;
}

int luxgi_ddgi_get_rays(const luxgi_ddgi_volume* v, luxgi_ddgi_rays* out) {
    if (!v || !out) return LUXGI_EINVAL;
    out->directions = reinterpret_cast<const float*>(v->dirs_trace);
    out->radiance = v->rays;
    out->hit_info = v->debug_rays ? reinterpret_cast<const int32_t*>(v->info) : nullptr;
    out->probes = v->P;
    out->rays = v->R;
    out->storage = v->desc.storage;
    return LUXGI_OK;
}

int luxgi_ddgi_check_status(luxgi_ddgi_volume* v, void* stream) {
    if (!v) return LUXGI_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t word = 0;
    cudaError_t e = cudaMemcpyAsync(&word, v->status, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    if (word == 0) return LUXGI_OK;
    e = cudaMemsetAsync(v->status, 0, sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? LUXGI_ETIMEOUT : cuda_status(e);
}

int luxgi_ddgi_set_blend_wait_test(luxgi_ddgi_volume* v, int64_t wait_cycles, int withhold) {
    if (!v || wait_cycles < 0) return LUXGI_EINVAL;
    if (withhold && !v->tc) return LUXGI_EUNSUPPORTED;
    v->tc_wait_cycles = wait_cycles;
    v->tc_withhold = withhold ? 1 : 0;
    return LUXGI_OK;
}

int luxgi_ddgi_set_stage_timing(luxgi_ddgi_volume* v, int enable) {
    if (!v) return LUXGI_EINVAL;
    if (enable && !v->stage_ev[0]) {
        for (cudaEvent_t& ev : v->stage_ev) {
            const cudaError_t e = cudaEventCreate(&ev);
            if (e != cudaSuccess) return cuda_status(e);
        }
    }
    v->stage_timing = enable != 0;
    return LUXGI_OK;
}

int luxgi_ddgi_stage_times(luxgi_ddgi_volume* v, float out[4]) {
    if (!v || !out) return LUXGI_EINVAL;
    if (!v->stage_timing) return LUXGI_EINVAL;
    cudaError_t e = cudaEventSynchronize(v->stage_blend_recorded ? v->stage_ev[4] : v->stage_ev[3]);
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) e = cudaEventElapsedTime(&out[i], v->stage_ev[i], v->stage_ev[i + 1]);
    out[3] = 0.0f;
    if (e == cudaSuccess && v->stage_blend_recorded) e = cudaEventElapsedTime(&out[3], v->stage_ev[3], v->stage_ev[4]);
    return cuda_status(e);
}

int luxgi_ddgi_set_debug_rays(luxgi_ddgi_volume* v, int enable) {
    if (!v) return LUXGI_EINVAL;
    if (enable && !v->info) {
        cudaError_t e = dmalloc(&v->info, sizeof(int4) * size_t(v->P) * v->R);
        if (e != cudaSuccess) return cuda_status(e);
    }
    v->debug_rays = enable ? 1 : 0;
    return LUXGI_OK;
}

int luxgi_ddgi_load_atlases(luxgi_ddgi_volume* v, const void* irr, const void* dist, int32_t frames, void* stream) {
    if (!v || !irr || !dist || frames < 0) return LUXGI_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    for (int i = 0; i < 2; ++i) {
        cudaError_t e = cudaMemcpyAsync(v->irr[i], irr, v->irr_bytes, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(v->dist[i], dist, v->dist_bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return cuda_status(e);
    }
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    v->frames = frames;
    return LUXGI_OK;
}

int luxgi_ddgi_save_atlases(const luxgi_ddgi_volume* v, void* irr, void* dist, int32_t* frames, void* stream) {
    if (!v || !irr || !dist) return LUXGI_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(irr, v->irr[v->ping_pong], v->irr_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dist, v->dist[v->ping_pong], v->dist_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    if (frames) *frames = v->frames;
    return LUXGI_OK;
}

int luxgi_ddgi_inject_indirect(luxgi_ddgi_volume* v, void* stream) {
    if (!v) return LUXGI_EINVAL;
    if (!v->bound) return LUXGI_ENOTBOUND;
    const luxgi_surface_desc& s = v->surf;
    if (!s.light_cache || !s.direct_light || !s.gbuffer0 || !s.gbuffer1 || !s.tiles) return LUXGI_EINVAL;
    AtlasView A;
    A.irr = v->irr[v->ping_pong];
    A.dist = v->dist[v->ping_pong];
    A.storage = v->desc.storage;
    const int bounce = (v->desc.infinite_bounce && v->frames != 0) ? 1 : 0;
    return cuda_status(launch_inject(v->desc.uniform, surface_view(s, LUXGI_LIGHT_CACHE), s.gbuffer0, s.gbuffer1,
                                     s.gbuffer_format, s.pbr, s.direct_light, s.light_cache, s.light_format, A,
                                     s.num_tiles, v->desc.intensity, bounce, static_cast<cudaStream_t>(stream)));
}

int luxgi_ddgi_sample_irradiance(const luxgi_ddgi_volume* v, const float* pos, const float* nrm, const float* wo,
                                 float* out, int n, void* stream) {
    if (!v || n < 0 || (n > 0 && (!pos || !nrm || !wo || !out))) return LUXGI_EINVAL;
    AtlasView A;
    A.irr = v->irr[v->ping_pong];
    A.dist = v->dist[v->ping_pong];
    A.storage = v->desc.storage;
    return cuda_status(launch_sample_irradiance(v->desc.uniform, A, pos, nrm, wo, out, n,
                                                static_cast<cudaStream_t>(stream)));
}

int luxgi_ddgi_sample_probe_image(const luxgi_ddgi_volume* v, const float* depth, const float* normal,
                                  int normal_channels, int width, int height, const float camera_pos[3],
                                  const float view_proj_inv[16], void* out, void* stream) {
    if (!v || width < 0 || height < 0 || !camera_pos || !view_proj_inv) return LUXGI_EINVAL;
    if (normal_channels < 2 || normal_channels > 4) return LUXGI_EINVAL;
    if (width > 0 && height > 0 && (!depth || !normal || !out)) return LUXGI_EINVAL;
    AtlasView A;
    A.irr = v->irr[v->ping_pong];
    A.dist = v->dist[v->ping_pong];
    A.storage = v->desc.storage;
    return cuda_status(launch_sample_probe(v->desc.uniform, A, depth, normal, normal_channels, width, height,
                                           camera_pos, view_proj_inv, out, static_cast<cudaStream_t>(stream)));
}

int luxgi_sdf_build_mip(const luxgi_sdf_desc* sdf, void* mip, void* tmp, void* stream) {
    if (!sdf || !mip || !tmp || !sdf->sdf) return LUXGI_EINVAL;
    const int C = int(sdf->data.cascades_count);
    if (C < 1 || C > 4 || sdf->resolution < 4 || sdf->resolution % 4 != 0 ||
        sdf->mip_resolution != sdf->resolution / 4)
        return LUXGI_EINVAL;
    if (sdf->format != LUXGI_STORAGE_FP32 && sdf->format != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    return cuda_status(launch_mip(*sdf, mip, tmp, static_cast<cudaStream_t>(stream)));
}

int luxgi_surface_cull(const luxgi_surface_desc* s, uint32_t* chunks, uint32_t* culled, uint32_t capacity,
                       void* stream) {
    if (!s || !chunks || !culled || !s->objects || capacity < 1) return LUXGI_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* scratch = nullptr;   // 40^3 counts + status word
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&scratch), sizeof(uint32_t) * (40 * 40 * 40 + 1), st);
    if (e != cudaSuccess) return cuda_status(e);
    e = launch_cull(s->data, s->objects, chunks, culled, capacity, scratch, scratch + 40 * 40 * 40, st);
    uint32_t status = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, scratch + 40 * 40 * 40, sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    cudaError_t e2 = cudaFreeAsync(scratch, st);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    return status ? LUXGI_ENOMEM : LUXGI_OK;
}

int luxgi_surface_light(const luxgi_sdf_desc* sdf, const luxgi_surface_desc* s, const luxgi_surface_lighting* L,
                        void* out, void* stream) {
    if (!sdf || !s || !L || !out) return LUXGI_EINVAL;
    if (L->num_lights < 0 || L->num_lights > LUXGI_MAX_LIGHTS || (L->num_lights > 0 && !L->lights)) return LUXGI_EINVAL;
    if (L->num_tiles < 0 || L->num_tiles > 65535 || (L->num_tiles > 0 && !L->tiles)) return LUXGI_EINVAL;
    if (!(L->shadow_bias >= 0.0f) || L->max_steps < 1) return LUXGI_EINVAL;
    if (!s->tiles || !s->gbuffer0 || !s->gbuffer1 || s->data.resolution < 1) return LUXGI_EINVAL;
    if (!surface_formats_valid(*s)) return LUXGI_EINVAL;
    if (L->num_lights > 0 && (!sdf->sdf || !sdf->mip || sdf->data.cascades_count < 1)) return LUXGI_EINVAL;
    if (sdf->format != LUXGI_STORAGE_FP32 && sdf->format != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    if (L->num_lights > 0 && !sdf_texels_fit(*sdf)) return LUXGI_EUNSUPPORTED;
    for (int i = 0; i < L->num_lights; ++i) {
        const float t = L->lights[i].type;
        if (t != float(LUXGI_LIGHT_DIRECTIONAL) && t != float(LUXGI_LIGHT_SPOT) && t != float(LUXGI_LIGHT_POINT))
            return LUXGI_EINVAL;
    }
    return cuda_status(launch_surface_light(sdf_view(*sdf), *s, *L, out,
                                            static_cast<cudaStream_t>(stream)));
}

}  // extern "C"
