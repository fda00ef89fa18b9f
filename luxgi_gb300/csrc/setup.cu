// Scene set-up stages of the path: the SDF mip (GlobalSDFMipmap.comp plus
// the four flood passes of GlobalDistanceField.cpp:537-573) and the surface
// chunk culling (SDFCulling.comp).  Built with -fmad=false so the mip and
// the sphere-vs-chunk tests equal their FP32 CPU restatement bit for bit.
#include <mutex>

#include <cuda_fp16.h>

#include "luxgi_internal.h"

namespace luxgi {

// combineDistanceToSDF (SDFCommon.glsl:18-36)
__device__ __forceinline__ float combine_sdf(float sdf, float dist) {
    if (sdf <= 0.0f && dist <= 0.0f) return sdf;
    const float m = mx(sdf, 0.0f);
    return sqrtf(m * m + dist * dist);
}

template <typename T> __device__ __forceinline__ float ldv(const T* p, size_t i);
template <> __device__ __forceinline__ float ldv<float>(const float* p, size_t i) { return p[i]; }
template <> __device__ __forceinline__ float ldv<__half>(const __half* p, size_t i) { return __half2float(p[i]); }
template <typename T> __device__ __forceinline__ void stv(T* p, size_t i, float v);
template <> __device__ __forceinline__ void stv<float>(float* p, size_t i, float v) { p[i] = v; }
template <> __device__ __forceinline__ void stv<__half>(__half* p, size_t i, float v) { p[i] = __float2half_rn(v); }

// One mip voxel per thread: min over self and the 6 face neighbours of
// combine(src[scale*v + o], |o| * maxDistance / srcRes) (GlobalSDFMipmap.comp:32-67).
template <typename T>
__global__ void mip_kernel(const T* __restrict__ src, int src_w, int src_res, int src_off_x, T* __restrict__ dst,
                           int dst_w, int dst_off_x, int mres, int scale, float max_dist) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int z = blockIdx.z * blockDim.z + threadIdx.z;
    if (x >= mres || y >= mres || z >= mres) return;
    const int off[7][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}};
    float m = 0.0f;
#pragma unroll
    for (int i = 0; i < 7; ++i) {
        const int cx = imn(imx(x * scale + off[i][0], 0), src_res - 1) + src_off_x;
        const int cy = imn(imx(y * scale + off[i][1], 0), src_res - 1);
        const int cz = imn(imx(z * scale + off[i][2], 0), src_res - 1);
        const float v = ldv(src, size_t(cx) + size_t(src_w) * (size_t(cy) + size_t(src_res) * cz));
        const float len = sqrtf(float(off[i][0] * off[i][0] + off[i][1] * off[i][1] + off[i][2] * off[i][2]));
        const float r = combine_sdf(v, len * (max_dist / float(src_res)));
        m = (i == 0) ? r : mn(m, r);
    }
    stv(dst, size_t(x + dst_off_x) + size_t(dst_w) * (size_t(y) + size_t(mres) * z), m);
}

// Cascade k's mip: the downsampling pass, then (flood) the four flood passes
// through tmp (GlobalDistanceField.cpp:537-573, 821-835).
template <typename T>
static cudaError_t mip_cascade_t(const luxgi_sdf_desc& s, int k, bool flood, T* mip, T* tmp, cudaStream_t st) {
    const int res = s.resolution, mres = s.mip_resolution, C = int(s.data.cascades_count);
    const T* sdf = static_cast<const T*>(s.sdf);
    dim3 blk(8, 8, 4);
    dim3 grd((mres + 7) / 8, (mres + 7) / 8, (mres + 3) / 4);
    const float maxd = s.data.cascade_pos_distance[k][3] * 2.0f;
    mip_kernel<T><<<grd, blk, 0, st>>>(sdf, res * C, res, k * res, mip, mres * C, k * mres, mres, 4, maxd);
    note_launch();
    if (!flood) return cudaGetLastError();
    for (int i = 1; i < 5; ++i) {
        if (i & 1) mip_kernel<T><<<grd, blk, 0, st>>>(mip, mres * C, mres, k * mres, tmp, mres, 0, mres, 1, maxd);
        else mip_kernel<T><<<grd, blk, 0, st>>>(tmp, mres, mres, 0, mip, mres * C, k * mres, mres, 1, maxd);
    }
    note_launch(4);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t mip_t(const luxgi_sdf_desc& s, T* mip, T* tmp, cudaStream_t st) {
    for (int k = 0; k < int(s.data.cascades_count); ++k) {
        const cudaError_t e = mip_cascade_t<T>(s, k, true, mip, tmp, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_mip_cascade(const luxgi_sdf_desc& s, int k, bool flood, void* mip, void* tmp, cudaStream_t st) {
    if (s.format == LUXGI_STORAGE_FP16)
        return mip_cascade_t<__half>(s, k, flood, static_cast<__half*>(mip), static_cast<__half*>(tmp), st);
    return mip_cascade_t<float>(s, k, flood, static_cast<float*>(mip), static_cast<float*>(tmp), st);
}

cudaError_t launch_mip(const luxgi_sdf_desc& s, void* mip, void* tmp, cudaStream_t st) {
    if (s.format == LUXGI_STORAGE_FP16)
        return mip_t<__half>(s, static_cast<__half*>(mip), static_cast<__half*>(tmp), st);
    return mip_t<float>(s, static_cast<float*>(mip), static_cast<float*>(tmp), st);
}

// ---------------------------------------------------------------- culling
constexpr int kChunks = kChunksRes * kChunksRes * kChunksRes;

// boxIntersectsSphere (AtlasCommon.glsl:34-38) for chunk c and object o.
__device__ __forceinline__ bool chunk_hits(const luxgi_surface_data& d, const luxgi_surface_object* objs, int c, uint32_t o) {
    const int x = c % kChunksRes, y = (c / kChunksRes) % kChunksRes, z = c / (kChunksRes * kChunksRes);
    const float cs = d.chunk_size;
    const float mnx = (float(x) - kChunksRes * 0.5f) * cs, mny = (float(y) - kChunksRes * 0.5f) * cs,
                mnz = (float(z) - kChunksRes * 0.5f) * cs;
    const float mxx = mnx + cs, mxy = mny + cs, mxz = mnz + cs;
    const float4 b = __ldg(reinterpret_cast<const float4*>(objs[o].object_bounds));
    const float dx = b.x - clampf(b.x, mnx, mxx), dy = b.y - clampf(b.y, mny, mxy), dz = b.z - clampf(b.z, mnz, mxz);
    return sqrtf(dx * dx + dy * dy + dz * dz) <= b.w;
}

// pass 1: words each chunk needs (0 or count + 1)
__global__ void cull_count_kernel(const luxgi_surface_data d, const luxgi_surface_object* __restrict__ objs,
                                  uint32_t* __restrict__ need) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kChunks) return;
    uint32_t n = 0;
    for (uint32_t o = 0; o < d.objects_count; ++o) n += chunk_hits(d, objs, c, o) ? 1u : 0u;
    need[c] = n ? n + 1 : 0;
}

// pass 2: exclusive scan of the needs (one block); offsets start at word 1
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) cull_scan_kernel(uint32_t* __restrict__ need, uint32_t* __restrict__ culled,
                                                                  uint32_t capacity, uint32_t* __restrict__ status) {
    __shared__ uint32_t part[kScanThreads];
    const int per = (kChunks + kScanThreads - 1) / kScanThreads;
    const int b = threadIdx.x * per, e = min(b + per, kChunks);
    uint32_t s = 0;
    for (int i = b; i < e; ++i) s += need[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < kScanThreads; off <<= 1) {     // Hillis-Steele inclusive scan
        const uint32_t v = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = 1 + (threadIdx.x ? part[threadIdx.x - 1] : 0u);
    for (int i = b; i < e; ++i) {
        const uint32_t n = need[i];
        need[i] = run;           // becomes the chunk's start offset
        run += n;
    }
    if (threadIdx.x == kScanThreads - 1) {
        const uint32_t used = 1 + part[kScanThreads - 1];
        if (capacity > 0) culled[0] = used;
        *status = used > capacity ? 1u : 0u;
    }
}

// pass 3: write [count, ids ascending] and the chunk table
__global__ void cull_fill_kernel(const luxgi_surface_data d, const luxgi_surface_object* __restrict__ objs,
                                 const uint32_t* __restrict__ start, uint32_t* __restrict__ chunks,
                                 uint32_t* __restrict__ culled, uint32_t capacity) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kChunks) return;
    const uint32_t st = start[c];
    const uint32_t nx = (c + 1 < kChunks) ? start[c + 1] : 0u;
    uint32_t n = 0;
    for (uint32_t o = 0; o < d.objects_count; ++o) n += chunk_hits(d, objs, c, o) ? 1u : 0u;
    (void)nx;
    if (n == 0 || st + n + 1 > capacity) {
        chunks[c] = 0;
        return;
    }
    culled[st] = n;
    uint32_t k = st + 1;
    for (uint32_t o = 0; o < d.objects_count; ++o)
        if (chunk_hits(d, objs, c, o)) culled[k++] = o;
    chunks[c] = st;
}

cudaError_t launch_cull(const luxgi_surface_data& d, const luxgi_surface_object* objects, uint32_t* chunks,
                        uint32_t* culled, uint32_t capacity, uint32_t* d_counts, uint32_t* d_status,
                        cudaStream_t st) {
    const int threads = 128, blocks = (kChunks + threads - 1) / threads;
    cull_count_kernel<<<blocks, threads, 0, st>>>(d, objects, d_counts);
    cull_scan_kernel<<<1, kScanThreads, 0, st>>>(d_counts, culled, capacity, d_status);
    cull_fill_kernel<<<blocks, threads, 0, st>>>(d, objects, d_counts, chunks, culled, capacity);
    note_launch(3);
    return cudaGetLastError();
}

// ------------------------------------------------------- shading lists
// Per chunk, the objects of the reference list (SDFCulling.comp) that a
// surface-atlas lookup from inside the chunk can actually accept: the
// sampler (AtlasCommon.glsl:132-138) skips an object unless the point lies
// within its box grown by the surface threshold, so an object whose grown
// box misses the chunk contributes nothing there and is left out.  Edge
// chunks extend to infinity outwards (lookups clamp into them).  Same
// layout as the reference lists; the contributions summed in the sampler
// are unchanged, only fewer objects are visited.
__device__ __forceinline__ bool shade_candidate(const luxgi_surface_data& d, const luxgi_surface_object* objs, int c,
                                                uint32_t o, float thr) {
    const int x = c % kChunksRes, y = (c / kChunksRes) % kChunksRes, z = c / (kChunksRes * kChunksRes);
    const float cs = d.chunk_size;
    const int cc[3] = {x, y, z};
    const float* M = objs[o].transform;
    const float* e = objs[o].extends;
    const float slack = 1e-3f * cs;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        // world AABB of the object box [-(e+thr), e+thr] (column-major M)
        const float h = fabsf(M[0 * 4 + k]) * (e[0] + thr) + fabsf(M[1 * 4 + k]) * (e[1] + thr) +
                        fabsf(M[2 * 4 + k]) * (e[2] + thr) + slack;
        const float lo = M[12 + k] - h, hi = M[12 + k] + h;
        const float cmin = (cc[k] == 0) ? -INFINITY : (float(cc[k]) - kChunksRes * 0.5f) * cs - slack;
        const float cmax = (cc[k] == kChunksRes - 1) ? INFINITY : (float(cc[k]) - kChunksRes * 0.5f + 1.0f) * cs + slack;
        if (hi < cmin || lo > cmax) return false;
    }
    return true;
}

__global__ void shade_list_count_kernel(const luxgi_surface_data d, const luxgi_surface_object* __restrict__ objs,
                                        const uint32_t* __restrict__ ref_chunks, const uint32_t* __restrict__ ref_culled,
                                        float thr, uint32_t* __restrict__ need) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kChunks) return;
    const uint32_t st = ref_chunks[c];
    uint32_t n = 0;
    if (st != 0) {
        const uint32_t cnt = ref_culled[st];
        if (cnt <= d.objects_count)
            for (uint32_t i = 0; i < cnt; ++i) n += shade_candidate(d, objs, c, ref_culled[st + 1 + i], thr) ? 1u : 0u;
    }
    need[c] = n ? n + 1 : 0;
}

__global__ void shade_list_fill_kernel(const luxgi_surface_data d, const luxgi_surface_object* __restrict__ objs,
                                       const uint32_t* __restrict__ ref_chunks, const uint32_t* __restrict__ ref_culled,
                                       float thr, const uint32_t* __restrict__ start, uint32_t* __restrict__ chunks,
                                       uint32_t* __restrict__ culled, uint32_t capacity) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= kChunks) return;
    const uint32_t rs = ref_chunks[c];
    const uint32_t at = start[c];
    uint32_t n = 0;
    if (rs != 0) {
        const uint32_t cnt = ref_culled[rs];
        if (cnt <= d.objects_count)
            for (uint32_t i = 0; i < cnt; ++i) n += shade_candidate(d, objs, c, ref_culled[rs + 1 + i], thr) ? 1u : 0u;
    }
    if (n == 0 || at + n + 1 > capacity) {
        chunks[c] = 0;
        return;
    }
    culled[at] = n;
    uint32_t k = at + 1;
    const uint32_t cnt = ref_culled[rs];
    for (uint32_t i = 0; i < cnt; ++i) {
        const uint32_t o = ref_culled[rs + 1 + i];
        if (shade_candidate(d, objs, c, o, thr)) culled[k++] = o;
    }
    chunks[c] = at;
}

cudaError_t launch_shade_lists(const luxgi_surface_data& d, const luxgi_surface_object* objects,
                               const uint32_t* ref_chunks, const uint32_t* ref_culled, float thr, uint32_t* chunks,
                               uint32_t* culled, uint32_t capacity, uint32_t* d_counts, uint32_t* d_status,
                               cudaStream_t st) {
    const int threads = 128, blocks = (kChunks + threads - 1) / threads;
    shade_list_count_kernel<<<blocks, threads, 0, st>>>(d, objects, ref_chunks, ref_culled, thr, d_counts);
    cull_scan_kernel<<<1, kScanThreads, 0, st>>>(d_counts, culled, capacity, d_status);
    shade_list_fill_kernel<<<blocks, threads, 0, st>>>(d, objects, ref_chunks, ref_culled, thr, d_counts, chunks, culled,
                                                       capacity);
    note_launch(3);
    return cudaGetLastError();
}

// ------------------------------------------------------- no-alloc mip build
// Scratch of luxgi_sdf_build_mip_noalloc: the flood-fill ping-pong plane
// (mres^3 texels) in a static device array, so the call allocates nothing.
// 1 MiB holds a 64^3 FP32 or an 80^3 FP16 plane.  Every GPU that loads the
// library holds it until the process exits.
static constexpr size_t kMipScratchBytes = size_t(1) << 20;
static __device__ __align__(256) unsigned char g_mip_scratch[kMipScratchBytes];

namespace {
constexpr int kMaxScratchDevices = 128;
std::mutex g_mip_scratch_mu;
void* g_mip_scratch_addr[kMaxScratchDevices] = {};

// Device address of g_mip_scratch on the current device.  Host code cannot
// name the array directly (its host symbol is only a stand-in), so the first
// call on each device looks the address up with that device current and
// caches it.
cudaError_t mip_scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxScratchDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mip_scratch_mu);
    if (!g_mip_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_mip_scratch);
        if (e != cudaSuccess) return e;
        g_mip_scratch_addr[dev] = p;
    }
    *out = g_mip_scratch_addr[dev];
    return cudaSuccess;
}
}  // namespace

}  // namespace luxgi

extern "C" int luxgi_sdf_build_mip_noalloc(const luxgi_sdf_desc* sdf, void* mip, void* stream) {
    using namespace luxgi;
    if (!sdf || !mip || !sdf->sdf) return LUXGI_EINVAL;
    const int C = int(sdf->data.cascades_count);
    if (C < 1 || C > 4 || sdf->resolution < 4 || sdf->resolution % 4 != 0 ||
        sdf->mip_resolution != sdf->resolution / 4)
        return LUXGI_EINVAL;
    if (sdf->format != LUXGI_STORAGE_FP32 && sdf->format != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    const size_t m = size_t(sdf->mip_resolution);
    const size_t need = m * m * m * (sdf->format == LUXGI_STORAGE_FP16 ? 2 : 4);
    if (need > kMipScratchBytes) return LUXGI_ESCRATCH;
    void* tmp = nullptr;
    cudaError_t e = mip_scratch_address(&tmp);
    if (e == cudaSuccess) e = launch_mip(*sdf, mip, tmp, static_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) return LUXGI_OK;
    return e == cudaErrorMemoryAllocation ? LUXGI_ENOMEM : LUXGI_ECUDA;
}

