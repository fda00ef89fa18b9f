// Hit shading of the march records (GISDFRays.comp:89-127): the
// surface-cache sample and the per-hit infinite bounce.  This translation
// unit builds with approximate division and square root, FMA contraction
// and denormals flushed to zero (-prec-div=false -prec-sqrt=false -fmad=true
// -ftz=true; no quantity of the shading lies near 1e-38): shading is
// compared with the CPU restatement by tolerance (1e-4 relative), while the
// march, whose hit test must reproduce the restatement's branches bit for
// bit, stays in trace.cu with IEEE arithmetic.  The hit point and the
// surface sampler's cut-offs (chunk, bounding sphere, OBB margin) use the
// exact *_rn forms, so every hit is sorted into the same objects and tiles
// as in the restatement and only continuous weights carry rounding.
#include <algorithm>
#include <cuda_fp16.h>

#include "luxgi_internal.h"

namespace luxgi {

// ---------------------------------------------------------------- shade
// Hit classification and shading of GISDFRays.comp:89-127 from the march
// records: sky for misses, zero for rays starting inside geometry, the
// surface-cache sample (and, per hit, the previous frame's irradiance) for
// hits; writes the per-ray radiance + distance and the tensor-core operands.
template <int MODE, int UNROLL>
__device__ __forceinline__ void shade_ray(const TraceParams& p, int64_t idx) {
    int probe, ray;
    if (!probe_ray(p, idx, probe, ray)) return;
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
        const f3 origin = probe_location(p.u, uint32_t(probe), p.div_x, p.div_xy);
        const f3 nrm{h.y, h.z, h.w};
        const f3 hp = ray_point_rn(origin, dir, h.x);
        const float vs = p.sdf.data.cascade_voxel_size[cls];
        const float thr = vs * 1.05f;
        f3 s0, s1;
        if (MODE == LUXGI_LIGHT_PER_HIT) {
            sample_surface<true>(p.surf, hp, nrm, thr, s0, s1);
            rad = s0;
            if (p.bounce) {
                const f3 e = sample_irradiance<UNROLL, true>(p.u, p.prev, hp, nrm, mul3(dir, -1.0f));
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
}

// 8 blocks of 128 a SM (64 registers): the shading waits on its gathers, so
// the warps of the eighth block pay for the few spilled bytes (production
// shading 0.450 -> 0.420 ms against the 72 registers the compiler takes).
template <int MODE, int UNROLL>
__global__ void __launch_bounds__(128, 8) shade_kernel(const TraceParams p) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t n = p.work;
    if (p.shade_part) {
        // split shading: the queued rays are qa's entries (its counter may
        // run past the capacity; rays beyond it finished in pass 1)
        const int64_t q = min(__ldg(p.qcount), p.qa_cap);
        n = p.shade_part == 1 ? p.work - q : q;
    }
    if (i >= n) return;
    shade_ray<MODE, UNROLL>(p, p.shade_seq ? int64_t(__ldg(p.shade_seq + i)) : i);
}

// ------------------------------------------------------ shading order
// Exclusive scan of the bin counts into the bin starts, one block of 32
// warps: warp w owns a contiguous segment of the bins.  Pass 1 sums each
// segment (32-bin coalesced slices, kScanAhead loads in flight per lane),
// warp 0 scans the 32 segment totals, pass 2 rescans each segment from its
// base (warp shuffles, the slices' loads again issued kScanAhead ahead).
constexpr int kScanThreads = 1024;
constexpr int kScanWarps = kScanThreads / 32;
constexpr int kScanAhead = 16;

__global__ void __launch_bounds__(kScanThreads) bin_scan_kernel(const uint32_t* __restrict__ count,
                                                               uint32_t* __restrict__ start, int nb) {
    __shared__ uint32_t seg_base[kScanWarps];
    const int lane = int(threadIdx.x) & 31, warp = int(threadIdx.x) >> 5;
    const int seg = ((nb + kScanWarps - 1) / kScanWarps + 31) & ~31;
    const int b0 = warp * seg, b1 = min(b0 + seg, nb);
    uint32_t total = 0;
    for (int b = b0; b < b1; b += kScanAhead * 32) {
        uint32_t v[kScanAhead];
#pragma unroll
        for (int k = 0; k < kScanAhead; ++k) {
            const int i = b + k * 32 + lane;
            v[k] = (b + k * 32 < b1 && i < b1) ? __ldg(count + i) : 0u;
        }
#pragma unroll
        for (int k = 0; k < kScanAhead; ++k) total += __reduce_add_sync(0xffffffffu, v[k]);
    }
    if (lane == 0) seg_base[warp] = total;
    __syncthreads();
    if (warp == 0) {
        const uint32_t t = seg_base[lane];
        uint32_t x = t;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
            if (lane >= off) x += y;
        }
        seg_base[lane] = x - t;
    }
    __syncthreads();
    uint32_t running = seg_base[warp];
    for (int b = b0; b < b1; b += kScanAhead * 32) {
        uint32_t v[kScanAhead];
#pragma unroll
        for (int k = 0; k < kScanAhead; ++k) {
            const int i = b + k * 32 + lane;
            v[k] = i < b1 ? __ldg(count + i) : 0u;
        }
#pragma unroll
        for (int k = 0; k < kScanAhead; ++k) {
            uint32_t x = v[k];                              // inclusive scan of the slice
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
                if (lane >= off) x += y;
            }
            const int i = b + k * 32 + lane;
            if (i < b1) start[i] = running + x - v[k];
            running += __shfl_sync(0xffffffffu, x, 31);
        }
    }
}

// Work items into `order` bin by bin: item idx goes to its bin's start plus
// the rank it drew from the bin's count when the march recorded it (the
// order within a bin is arbitrary; each item is shaded the same wherever
// it lands).
__global__ void __launch_bounds__(256) bin_place_kernel(const uint2* __restrict__ slot,
                                                        const uint32_t* __restrict__ start, uint32_t* __restrict__ order,
                                                        int64_t work) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= work) return;
    const uint2 s = __ldg(slot + idx);
    if (s.x == kDeferredBin) return;              // queued by pass 1, placed with the queue
    const uint32_t pos = __ldg(start + s.x) + s.y;
    if (pos < work) order[pos] = uint32_t(idx);   // the counts cover every work item once
}

// The same for the rays pass 1 queued (split shading): entry i of qa names
// its work item, whose slot passes 2 and 3 recorded.
__global__ void __launch_bounds__(256) bin_place_queue_kernel(const int4* __restrict__ qa,
                                                              const uint32_t* __restrict__ qcount, uint32_t cap,
                                                              const uint2* __restrict__ slot,
                                                              const uint32_t* __restrict__ start,
                                                              uint32_t* __restrict__ order) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = min(__ldg(qcount), cap);
    if (i >= n) return;
    const uint32_t idx = uint32_t(__ldg(qa + 2 * size_t(i)).x);
    const uint2 s = __ldg(slot + idx);
    const uint32_t pos = __ldg(start + s.x) + s.y;
    if (pos < n) order[pos] = idx;
}

cudaError_t launch_bin_sort(uint32_t* bins, int nb, const uint2* slots, uint32_t* seq, int64_t work,
                            cudaStream_t st) {
    if (work <= 0) return cudaSuccess;
    uint32_t* start = bins + nb;
    bin_scan_kernel<<<1, kScanThreads, 0, st>>>(bins, start, nb);
    bin_place_kernel<<<unsigned((work + 255) / 256), 256, 0, st>>>(slots, start, seq, work);
    note_launch(2);
    return cudaGetLastError();
}

cudaError_t launch_shade_sort(const TraceParams& p, cudaStream_t st) {
    if (p.shade_part != 2) return launch_bin_sort(p.bin_count, kShadeBins, p.bin_key, p.shade_seq, p.work, st);
    if (p.qa_cap == 0) return cudaSuccess;
    uint32_t* start = p.bin_count + kShadeBins;
    bin_scan_kernel<<<1, kScanThreads, 0, st>>>(p.bin_count, start, kShadeBins);
    bin_place_queue_kernel<<<(p.qa_cap + 255) / 256, 256, 0, st>>>(p.qa, p.qcount, p.qa_cap, p.bin_key, start,
                                                                  p.shade_seq);
    note_launch(2);
    return cudaGetLastError();
}

// Batched shading in bin order.  Every volume owns a contiguous run of
// bins, so the order groups the volumes and a block's 128 work items come
// from the volumes between those of its first and last item: up to
// kStagedVolumes of them are staged in shared memory, more are read from
// device memory.
constexpr int kStagedVolumes = 4;

// Resident blocks of 128 threads a SM the batched shading is compiled for
// (8: 64 registers, 6: 80); without a bound the compiler takes 96
// registers and the SM keeps 28 % of its warp slots busy.
#ifndef LUXGI_SHADE_BATCH_MIN_BLOCKS
#define LUXGI_SHADE_BATCH_MIN_BLOCKS 8
#endif
template <int MODE, int UNROLL>
__global__ void __launch_bounds__(128, LUXGI_SHADE_BATCH_MIN_BLOCKS)
    shade_batch_sorted_kernel(const TraceParams* __restrict__ vp, const int* __restrict__ work_off, int n,
                              const uint32_t* __restrict__ seq, int64_t work) {
    constexpr int kWords = int(sizeof(TraceParams) / 4);
    __shared__ __align__(16) uint32_t sp[kStagedVolumes][kWords];
    __shared__ int vrange[2];
    const int64_t i0 = int64_t(blockIdx.x) * blockDim.x;
    if (threadIdx.x == 0) {
        const int64_t last = min(i0 + int64_t(blockDim.x) - 1, work - 1);
        vrange[0] = batch_volume(work_off, n, int(__ldg(seq + i0)));
        vrange[1] = batch_volume(work_off, n, int(__ldg(seq + last)));
    }
    __syncthreads();
    const int vlo = vrange[0], vhi = vrange[1];
    const bool staged = vhi - vlo < kStagedVolumes;
    if (staged) {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(vp + vlo);
        for (int k = threadIdx.x; k < (vhi - vlo + 1) * kWords; k += blockDim.x) sp[k / kWords][k % kWords] = __ldg(src + k);
    }
    __syncthreads();
    const int64_t i = i0 + threadIdx.x;
    if (i >= work) return;
    const int g = int(__ldg(seq + i));
    const int v = batch_volume(work_off, n, g);
    const int64_t idx = int64_t(g - __ldg(work_off + v));
    if (staged) shade_ray<MODE, UNROLL>(*reinterpret_cast<const TraceParams*>(sp[v - vlo]), idx);
    else shade_ray<MODE, UNROLL>(vp[v], idx);
}

cudaError_t launch_shade_batch_sorted(const TraceParams* vp, const int* work_off, int n, const uint32_t* seq,
                                      int64_t work, int light_mode, int shade_variant, cudaStream_t st) {
    if (work <= 0) return cudaSuccess;
    const unsigned b = unsigned((work + 127) / 128);
    if (light_mode == LUXGI_LIGHT_PER_HIT) {
        switch (shade_variant) {
            case 2: shade_batch_sorted_kernel<LUXGI_LIGHT_PER_HIT, 2><<<b, 128, 0, st>>>(vp, work_off, n, seq, work); break;
            case 4: shade_batch_sorted_kernel<LUXGI_LIGHT_PER_HIT, 4><<<b, 128, 0, st>>>(vp, work_off, n, seq, work); break;
            case 8: shade_batch_sorted_kernel<LUXGI_LIGHT_PER_HIT, 8><<<b, 128, 0, st>>>(vp, work_off, n, seq, work); break;
            default: shade_batch_sorted_kernel<LUXGI_LIGHT_PER_HIT, 1><<<b, 128, 0, st>>>(vp, work_off, n, seq, work); break;
        }
    } else {
        shade_batch_sorted_kernel<LUXGI_LIGHT_CACHE, 1><<<b, 128, 0, st>>>(vp, work_off, n, seq, work);
    }
    note_launch();
    return cudaGetLastError();
}

// Batched over many volumes (128 rays a block), parameters staged in
// shared memory once per block.
template <int MODE, int UNROLL>
__global__ void __launch_bounds__(128, LUXGI_SHADE_BATCH_MIN_BLOCKS)
    shade_batch_kernel(const TraceParams* __restrict__ vp, const int* __restrict__ starts, int n) {
    __shared__ __align__(16) uint32_t sp[sizeof(TraceParams) / 4];
    const int v = batch_volume(starts, n, int(blockIdx.x));
    const TraceParams& p = stage_params(vp + v, sp);
    const int64_t idx = int64_t(int(blockIdx.x) - __ldg(starts + v)) * 128 + threadIdx.x;
    if (idx >= p.work) return;
    shade_ray<MODE, UNROLL>(p, idx);
}

// ------------------------------------------------ tensor-core operands
// The tensor-core blend's operands from the shaded rays: radiance rows and
// the blend's per-ray depth split into FP16 hi + lo (ProbeUpdate.glsl:
// 204-207), K-major [P][4][R].  One thread per (probe, ray), ray fastest, so
// that the ray reads and the operand writes both coalesce; the shading runs
// in hit-chunk order, where these 2-byte stores scattered one sector each.
__device__ __forceinline__ void tc_pack_one(const TraceParams& p, int64_t local) {
    const int probe = int(p.index32 ? fdiv(uint32_t(local), p.div_r) : uint32_t(local / p.R));
    const int ray = int(local - int64_t(probe) * p.R);
    const size_t o = size_t(probe) * p.R + ray;
    float r, g, b, dist;
    if (p.storage == LUXGI_STORAGE_FP16) {
        const uint2 raw = __ldg(static_cast<const uint2*>(p.out) + o);
        const __half2 rg = *reinterpret_cast<const __half2*>(&raw.x);
        const __half2 bd = *reinterpret_cast<const __half2*>(&raw.y);
        r = __low2float(rg); g = __high2float(rg); b = __low2float(bd); dist = __high2float(bd);
    } else {
        const float4 v = __ldg(static_cast<const float4*>(p.out) + o);
        r = v.x; g = v.y; b = v.z; dist = v.w;
    }
    __half* a = p.tc_irr + size_t(probe) * 4 * p.R + ray;
    a[0] = __float2half_rn(r);
    a[p.R] = __float2half_rn(g);
    a[2 * p.R] = __float2half_rn(b);
    a[3 * p.R] = __float2half_rn(0.0f);
    float dd = mn(p.u.max_distance, dist - 0.01f);
    if (dd == -1.0f) dd = p.u.max_distance;
    const float d2 = dd * dd;
    const __half dh = __float2half_rn(dd), d2h = __float2half_rn(d2);
    const __half dl = __float2half_rn(dd - __half2float(dh));
    const __half d2l = __float2half_rn(d2 - __half2float(d2h));
    __half* bq = p.tc_dist + size_t(probe) * 4 * p.R + ray;
    bq[0] = dh;
    bq[p.R] = dl;
    bq[2 * p.R] = d2h;
    bq[3 * p.R] = d2l;
}

__global__ void __launch_bounds__(256) tc_pack_kernel(const TraceParams p) {
    const int64_t n = int64_t(p.P) * p.R;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
        tc_pack_one(p, i);
}

// Batched: block b belongs to the volume whose block range holds it.
__global__ void __launch_bounds__(256) tc_pack_batch_kernel(const TraceParams* __restrict__ vp,
                                                            const int* __restrict__ starts, int n) {
    const int v = batch_volume(starts, n, int(blockIdx.x));
    const TraceParams& p = vp[v];
    const int64_t local = int64_t(int(blockIdx.x) - __ldg(starts + v)) * 256 + threadIdx.x;
    if (local >= int64_t(p.P) * p.R) return;
    tc_pack_one(p, local);
}

cudaError_t launch_tc_pack(const TraceParams& p, cudaStream_t st) {
    const int64_t n = int64_t(p.P) * p.R;
    if (n <= 0 || !p.tc_irr) return cudaSuccess;
    const unsigned blocks = unsigned(std::min<int64_t>((n + 255) / 256, 65535));
    tc_pack_kernel<<<blocks, 256, 0, st>>>(p);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_tc_pack_batch(const TraceParams* vp, const int* starts, int n, int blocks, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    tc_pack_batch_kernel<<<unsigned(blocks), 256, 0, st>>>(vp, starts, n);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_shade(const TraceParams& p, cudaStream_t st) {
    const int64_t total = p.shade_part == 2 ? int64_t(p.qa_cap) : p.work;
    if (total <= 0) return cudaSuccess;
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
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_shade_batch(const TraceParams* vp, const int* starts, int n, int blocks, int light_mode,
                               int shade_variant, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    const unsigned b = unsigned(blocks);
    if (light_mode == LUXGI_LIGHT_PER_HIT) {
        switch (shade_variant) {
            case 2: shade_batch_kernel<LUXGI_LIGHT_PER_HIT, 2><<<b, 128, 0, st>>>(vp, starts, n); break;
            case 4: shade_batch_kernel<LUXGI_LIGHT_PER_HIT, 4><<<b, 128, 0, st>>>(vp, starts, n); break;
            case 8: shade_batch_kernel<LUXGI_LIGHT_PER_HIT, 8><<<b, 128, 0, st>>>(vp, starts, n); break;
            default: shade_batch_kernel<LUXGI_LIGHT_PER_HIT, 1><<<b, 128, 0, st>>>(vp, starts, n); break;
        }
    } else {
        shade_batch_kernel<LUXGI_LIGHT_CACHE, 1><<<b, 128, 0, st>>>(vp, starts, n);
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace luxgi
