// Ray generation, SDF sphere tracing and hit shading (GISDFRays.comp), the
// mode-A light-cache injection (SDFAtlasIndirectLight.frag) and batched
// sampleIrradiance.  Built with -fmad=false: the march must reproduce the
// FP32 CPU restatement bit for bit.
#include <algorithm>

#include <cuda_fp16.h>

#include "luxgi_internal.h"

namespace luxgi {

// --------------------------------------------------------------- raygen
// sphericalFibonacci under the frame rotation (GISDFRays.comp:73); one
// direction per ray index, shared by every probe of the volume.
__global__ void raygen_kernel(Rot rot, int R, int storage, float4* __restrict__ dirs_trace,
                              float4* __restrict__ dirs_blend) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const f3 d = ray_direction(rot.m, r, R);
    dirs_trace[r] = make_float4(d.x, d.y, d.z, 0.0f);
    if (storage == LUXGI_STORAGE_FP16) {
        // the reference's blend reads directions back from an RGBA16F texture
        dirs_blend[r] = make_float4(__half2float(__float2half_rn(d.x)), __half2float(__float2half_rn(d.y)),
                                    __half2float(__float2half_rn(d.z)), 0.0f);
    } else {
        dirs_blend[r] = make_float4(d.x, d.y, d.z, 0.0f);
    }
}

cudaError_t launch_raygen(const Rot& rot, int R, int storage, float4* dirs_trace, float4* dirs_blend,
                          cudaStream_t st) {
    raygen_kernel<<<(R + 127) / 128, 128, 0, st>>>(rot, R, storage, dirs_trace, dirs_blend);
    note_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------- march
// One thread per (probe, ray); consecutive threads take consecutive probes
// with the same ray index, so a warp marches 32 parallel rays from
// neighbouring probes through nearby SDF texels.  The march is the whole
// kernel (no shading code): small, low register count, high occupancy.
template <typename SdfT, int MIN_BLOCKS, int QMIP, int QTEX>
__global__ void __launch_bounds__(256, MIN_BLOCKS) march_kernel(const TraceParams p) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = int64_t(p.P) * p.R;
    if (idx >= total) return;
    const int probe = int(idx % p.P);
    const int ray = int(idx / p.P);
    const float4 d4 = __ldg(p.dirs + ray);
    const f3 dir{d4.x, d4.y, d4.z};
    const f3 origin = probe_location(p.u, probe);
    const MarchHit hit = march_sdf<SdfT, QMIP, QTEX>(p.sdf, origin, dir, kWorldSize, p.max_steps);
    int cls = -1;                                          // miss
    if (hit.time >= 0.0f) {
        // GISDFRays.comp:93: a hit at the probe from inside a surface
        cls = (hit.sdf <= 0.0f && hit.time <= p.sdf.data.cascade_voxel_size[0]) ? -2 : hit.cascade;
    }
    const size_t o = size_t(probe) * p.R + ray;
    p.hit_t[o] = make_float4(hit.time, hit.normal.x, hit.normal.y, hit.normal.z);
    p.hit_c[o] = cls;
    if (p.info) p.info[o] = make_int4(hit.steps, hit.time >= 0.0f ? hit.cascade : -1, hit.fine, 0);
}

// ---------------------------------------------------------------- shade
// Hit classification and shading of GISDFRays.comp:89-127 from the march
// records: sky for misses, zero for rays starting inside geometry, the
// surface-cache sample (and, per hit, the previous frame's irradiance) for
// hits; writes the per-ray radiance + distance and the tensor-core operands.
template <int MODE, int UNROLL>
__global__ void __launch_bounds__(128) shade_kernel(const TraceParams p) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t total = int64_t(p.P) * p.R;
    if (idx >= total) return;
    const int probe = int(idx % p.P);
    const int ray = int(idx / p.P);
    const size_t o = size_t(probe) * p.R + ray;
    const float4 h = p.hit_t[o];
    const int cls = p.hit_c[o];
    f3 rad{0.0f, 0.0f, 0.0f};
    float dist = kWorldSize;
    if (cls == -1) {
        rad = f3{p.sky[0], p.sky[1], p.sky[2]};
    } else if (cls >= 0) {
        const float4 d4 = __ldg(p.dirs + ray);
        const f3 dir{d4.x, d4.y, d4.z};
        const f3 origin = probe_location(p.u, probe);
        const f3 nrm{h.y, h.z, h.w};
        const f3 hp = add3(origin, mul3(dir, h.x));
        const float vs = p.sdf.data.cascade_voxel_size[cls];
        const float thr = vs * 1.05f;
        f3 s0, s1;
        if (MODE == LUXGI_LIGHT_PER_HIT) {
            sample_surface<true>(p.surf, hp, nrm, thr, s0, s1);
            rad = s0;
            if (p.bounce) {
                const f3 e = sample_irradiance<UNROLL>(p.u, p.prev, hp, nrm, mul3(dir, -1.0f));
                const f3 diff{s1.x / kPi, s1.y / kPi, s1.z / kPi};
                rad = add3(rad, mulv3(mul3(diff, p.intensity), e));
            }
        } else {
            sample_surface<false>(p.surf, hp, nrm, thr, s0, s1);
            rad = s0;
        }
        dist = mx(h.x + vs * 0.5f, 0.0f);
    }
    if (p.storage == LUXGI_STORAGE_FP16) {
        const __half2 rg = __floats2half2_rn(rad.x, rad.y);
        const __half2 bd = __floats2half2_rn(rad.z, dist);
        uint2 raw;
        raw.x = *reinterpret_cast<const uint32_t*>(&rg);
        raw.y = *reinterpret_cast<const uint32_t*>(&bd);
        reinterpret_cast<uint2*>(p.out)[o] = raw;
        rad = f3{__low2float(rg), __high2float(rg), __low2float(bd)};
        dist = __high2float(bd);
    } else {
        reinterpret_cast<float4*>(p.out)[o] = make_float4(rad.x, rad.y, rad.z, dist);
    }
    if (p.tc_irr) {
        // tensor-core operands: radiance rows and the blend's per-ray depth
        // split into FP16 hi + lo (ProbeUpdate.glsl:204-207)
        __half* a = p.tc_irr + size_t(probe) * 4 * p.R + ray;
        a[0] = __float2half_rn(rad.x);
        a[p.R] = __float2half_rn(rad.y);
        a[2 * p.R] = __float2half_rn(rad.z);
        a[3 * p.R] = __float2half_rn(0.0f);
        float dd = mn(p.u.max_distance, dist - 0.01f);
        if (dd == -1.0f) dd = p.u.max_distance;
        const float d2 = dd * dd;
        const __half dh = __float2half_rn(dd), d2h = __float2half_rn(d2);
        const __half dl = __float2half_rn(dd - __half2float(dh));
        const __half d2l = __float2half_rn(d2 - __half2float(d2h));
        __half* b = p.tc_dist + size_t(probe) * 4 * p.R;
        b[ray] = dh;
        b[p.R + ray] = dl;
        b[2 * p.R + ray] = d2h;
        b[3 * p.R + ray] = d2l;
    }
}

cudaError_t launch_trace(const TraceParams& p, cudaStream_t st) {
    const int64_t total = int64_t(p.P) * p.R;
    if (total <= 0) return cudaSuccess;
    const unsigned mblocks = unsigned((total + 255) / 256);
    // variants: 1 plain layout, 64 registers (4 blocks of 256 per SM);
    // 2 plain layout, no register bound; 3 quad-packed mip; 4 quad-packed
    // mip and full-resolution volume; 5 quad-packed mip, pair-packed
    // full-resolution volume.  All produce identical results.
    const bool h = p.sdf.format == LUXGI_STORAGE_FP16;
    switch (p.march_variant) {
        case 2:
            if (h) march_kernel<__half, 1, kPlain, kPlain><<<mblocks, 256, 0, st>>>(p);
            else march_kernel<float, 1, kPlain, kPlain><<<mblocks, 256, 0, st>>>(p);
            break;
        case 3:
            if (h) march_kernel<__half, 4, kQuad, kPlain><<<mblocks, 256, 0, st>>>(p);
            else march_kernel<float, 4, kQuad, kPlain><<<mblocks, 256, 0, st>>>(p);
            break;
        case 4:
            if (h) march_kernel<__half, 4, kQuad, kQuad><<<mblocks, 256, 0, st>>>(p);
            else march_kernel<float, 4, kQuad, kQuad><<<mblocks, 256, 0, st>>>(p);
            break;
        case 5:
            if (h) march_kernel<__half, 4, kQuad, kPair><<<mblocks, 256, 0, st>>>(p);
            else march_kernel<float, 4, kQuad, kPair><<<mblocks, 256, 0, st>>>(p);
            break;
        default:
            if (h) march_kernel<__half, 4, kPlain, kPlain><<<mblocks, 256, 0, st>>>(p);
            else march_kernel<float, 4, kPlain, kPlain><<<mblocks, 256, 0, st>>>(p);
            break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const unsigned sblocks = unsigned((total + 127) / 128);
    if (p.light_mode == LUXGI_LIGHT_PER_HIT) {
        switch (p.shade_variant) {
            case 2: shade_kernel<LUXGI_LIGHT_PER_HIT, 2><<<sblocks, 128, 0, st>>>(p); break;
            case 4: shade_kernel<LUXGI_LIGHT_PER_HIT, 4><<<sblocks, 128, 0, st>>>(p); break;
            case 8: shade_kernel<LUXGI_LIGHT_PER_HIT, 8><<<sblocks, 128, 0, st>>>(p); break;
            default: shade_kernel<LUXGI_LIGHT_PER_HIT, 1><<<sblocks, 128, 0, st>>>(p); break;
        }
    } else {
        shade_kernel<LUXGI_LIGHT_CACHE, 1><<<sblocks, 128, 0, st>>>(p);   // no per-hit bounce
    }
    note_launch(2);
    return cudaGetLastError();
}

// ------------------------------------------------------- world-to-local
// inverse(object.transform) for every object (AtlasCommon.glsl:134), once
// per bound scene instead of once per ray and object.
__global__ void world_to_local_kernel(const luxgi_surface_object* __restrict__ objs, int n, float* __restrict__ w2l) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float M[16], inv[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) M[k] = objs[i].transform[k];
    mat4_inverse(M, inv);
#pragma unroll
    for (int k = 0; k < 16; ++k) w2l[size_t(i) * 16 + k] = inv[k];
}

cudaError_t launch_world_to_local(const luxgi_surface_object* objs, int n, float* w2l, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    world_to_local_kernel<<<(n + 127) / 128, 128, 0, st>>>(objs, n, w2l);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------------ quad pack
// Quad-packed copy of a W x H x D volume (see Quad / sample3d_quad).
template <typename T>
__global__ void quad_pack_kernel(const T* __restrict__ src, int W, int H, int D, typename Quad<T>::type* __restrict__ dst) {
    const int64_t QW = int64_t(W) + 1, QH = int64_t(H) + 1;
    const int64_t n = QW * QH * D;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int qx = int(i % QW), qy = int((i / QW) % QH), z = int(i / (QW * QH));
        const int x0 = imn(imx(qx - 1, 0), W - 1), x1 = imn(imx(qx, 0), W - 1);
        const int y0 = imn(imx(qy - 1, 0), H - 1), y1 = imn(imx(qy, 0), H - 1);
        const size_t pz = size_t(z) * W * H;
        const T a = src[pz + size_t(y0) * W + x0], b = src[pz + size_t(y0) * W + x1];
        const T c = src[pz + size_t(y1) * W + x0], d = src[pz + size_t(y1) * W + x1];
        if constexpr (sizeof(T) == 4) {
            dst[i] = make_float4(a, b, c, d);
        } else {
            __half2 ab = __halves2half2(a, b), cd = __halves2half2(c, d);
            uint2 q;
            q.x = *reinterpret_cast<const uint32_t*>(&ab);
            q.y = *reinterpret_cast<const uint32_t*>(&cd);
            dst[i] = q;
        }
    }
}

size_t quad_bytes(int W, int H, int D, int format) {
    return (size_t(W) + 1) * (size_t(H) + 1) * size_t(D) * (format == LUXGI_STORAGE_FP16 ? 8 : 16);
}

cudaError_t launch_quad_pack(const void* src, int W, int H, int D, int format, void* dst, cudaStream_t st) {
    const int64_t n = (int64_t(W) + 1) * (int64_t(H) + 1) * D;
    const unsigned blocks = unsigned(std::min<int64_t>((n + 255) / 256, 65535));
    if (format == LUXGI_STORAGE_FP16)
        quad_pack_kernel<__half><<<blocks, 256, 0, st>>>(static_cast<const __half*>(src), W, H, D, static_cast<uint2*>(dst));
    else
        quad_pack_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(src), W, H, D, static_cast<float4*>(dst));
    note_launch();
    return cudaGetLastError();
}

// Pair-packed copy of a W x H x D volume (see Pair / sample3d_pair).
template <typename T>
__global__ void pair_pack_kernel(const T* __restrict__ src, int W, int H, int D, typename Pair<T>::type* __restrict__ dst) {
    const int64_t PW = int64_t(W) + 1;
    const int64_t n = PW * H * D;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int px = int(i % PW);
        const int64_t row = i / PW;                      // y + H * z
        const int x0 = imn(imx(px - 1, 0), W - 1), x1 = imn(imx(px, 0), W - 1);
        const T a = src[size_t(row) * W + x0], b = src[size_t(row) * W + x1];
        if constexpr (sizeof(T) == 4) dst[i] = make_float2(a, b);
        else dst[i] = __halves2half2(a, b);
    }
}

size_t pair_bytes(int W, int H, int D, int format) {
    return (size_t(W) + 1) * size_t(H) * size_t(D) * (format == LUXGI_STORAGE_FP16 ? 4 : 8);
}

cudaError_t launch_pair_pack(const void* src, int W, int H, int D, int format, void* dst, cudaStream_t st) {
    const int64_t n = (int64_t(W) + 1) * H * D;
    const unsigned blocks = unsigned(std::min<int64_t>((n + 255) / 256, 65535));
    if (format == LUXGI_STORAGE_FP16)
        pair_pack_kernel<__half><<<blocks, 256, 0, st>>>(static_cast<const __half*>(src), W, H, D, static_cast<__half2*>(dst));
    else
        pair_pack_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(src), W, H, D, static_cast<float2*>(dst));
    note_launch();
    return cudaGetLastError();
}

// --------------------------------------------------------------- inject
// SDFAtlasIndirectLight.frag:44-67 over every texel of every tile rect
// (the raster pass draws each tile's (w-1) x (h-1) viewport): the light
// cache becomes direct light plus intensity * min(albedo, 0.9)/pi *
// sampleIrradiance(previous atlases).  One block row per tile.
__global__ void inject_kernel(const luxgi_ddgi_uniform u, const SurfaceView s, const float* __restrict__ gb0,
                              const float* __restrict__ gb1, const __half* __restrict__ direct,
                              __half* __restrict__ light, const AtlasView A, float intensity, int bounce) {
    const int t = blockIdx.y + 1;                 // tile slot 0 is "no tile"
    const luxgi_surface_tile* tl = s.tiles + t;
    const int res = int(s.data.resolution);
    const int x0 = int(lrintf(__ldg(&tl->extends[0]) * float(res)));
    const int y0 = int(lrintf(__ldg(&tl->extends[1]) * float(res)));
    const int w = int(lrintf(__ldg(&tl->extends[2]) * float(res)));
    const int h = int(lrintf(__ldg(&tl->extends[3]) * float(res)));
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w * h; k += gridDim.x * blockDim.x) {
        const int i = k % w, j = k / w;
        const size_t ti = size_t(y0 + j) * res + (x0 + i);
        float add[3] = {0.0f, 0.0f, 0.0f};
        if (bounce) {
            const float4 g0 = __ldg(reinterpret_cast<const float4*>(gb0) + ti);
            const float4 g1 = __ldg(reinterpret_cast<const float4*>(gb1) + ti);
            // octohedralToDirection (Math.glsl:27-33)
            f3 v{g1.x, g1.y, 1.0f - fabsf(g1.x) - fabsf(g1.y)};
            if (v.z < 0.0f) {
                const float nx = (1.0f - fabsf(v.y)) * (v.x >= 0.0f ? 1.0f : -1.0f);
                const float ny = (1.0f - fabsf(v.x)) * (v.y >= 0.0f ? 1.0f : -1.0f);
                v.x = nx; v.y = ny;
            }
            const f3 n = norm3(v);
            const f3 wp{g0.w, g1.z, g1.w};
            const f3 cam{s.data.camera_pos[0], s.data.camera_pos[1], s.data.camera_pos[2]};
            const f3 wo = norm3(sub3(cam, wp));
            const f3 e = sample_irradiance(u, A, wp, n, wo);
            const float alb[3] = {mn(g0.x, 0.9f), mn(g0.y, 0.9f), mn(g0.z, 0.9f)};
            const float ev[3] = {e.x, e.y, e.z};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float diff = (alb[c] - alb[c] * 0.0f) / kPi;
                add[c] = intensity * diff * ev[c];
            }
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) light[ti * 4 + c] = __float2half_rn(__half2float(direct[ti * 4 + c]) + add[c]);
        light[ti * 4 + 3] = direct[ti * 4 + 3];
    }
}

cudaError_t launch_inject(const luxgi_ddgi_uniform& u, const SurfaceView& s, const float* gb0, const float* gb1,
                          const __half* direct, __half* light, const AtlasView& A, int num_tiles, float intensity,
                          int bounce, cudaStream_t st) {
    if (num_tiles <= 1) return cudaSuccess;
    dim3 grid(8, unsigned(num_tiles - 1));
    inject_kernel<<<grid, 256, 0, st>>>(u, s, gb0, gb1, direct, light, A, intensity, bounce);
    note_launch();
    return cudaGetLastError();
}

// ------------------------------------------------------- sampleIrradiance
__global__ void sample_irradiance_kernel(const luxgi_ddgi_uniform u, const AtlasView A, const float* __restrict__ pos,
                                         const float* __restrict__ nrm, const float* __restrict__ wo,
                                         float* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 P{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    const f3 N{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
    const f3 W{wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]};
    const f3 e = sample_irradiance(u, A, P, N, W);
    out[3 * i] = e.x;
    out[3 * i + 1] = e.y;
    out[3 * i + 2] = e.z;
}

cudaError_t launch_sample_irradiance(const luxgi_ddgi_uniform& u, const AtlasView& A, const float* pos,
                                     const float* nrm, const float* wo, float* out, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    sample_irradiance_kernel<<<(n + 127) / 128, 128, 0, st>>>(u, A, pos, nrm, wo, out, n);
    note_launch();
    return cudaGetLastError();
}

}  // namespace luxgi
