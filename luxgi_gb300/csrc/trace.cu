// Ray generation and SDF sphere tracing (GISDFRays.comp), their batched
// launches, and sampleIrradiance for caller points.  Built with
// -fmad=false: the march must reproduce the FP32 CPU restatement bit for
// bit.
#include <algorithm>

#include <cuda_fp16.h>

#include "luxgi_internal.h"

namespace luxgi {

// --------------------------------------------------------------- raygen
// sphericalFibonacci under the frame rotation (GISDFRays.comp:73); one
// direction per ray index, shared by every probe of the volume.
__device__ __forceinline__ void raygen_ray(const Rot& rot, int R, int storage, float4* __restrict__ dirs_trace,
                                           float4* __restrict__ dirs_blend, int r) {
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

__global__ void raygen_kernel(Rot rot, int R, int storage, float4* __restrict__ dirs_trace,
                              float4* __restrict__ dirs_blend) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    raygen_ray(rot, R, storage, dirs_trace, dirs_blend, r);
}

// Batched: blocks of 128 rays, volume found from the block index.
__global__ void __launch_bounds__(128) raygen_batch_kernel(const TraceParams* __restrict__ vp,
                                                          const int* __restrict__ starts, int n) {
    const int v = batch_volume(starts, n, int(blockIdx.x));
    const TraceParams& p = vp[v];
    const int r = (int(blockIdx.x) - __ldg(starts + v)) * 128 + int(threadIdx.x);
    if (r >= p.R) return;
    raygen_ray(p.rot, p.R, p.storage, const_cast<float4*>(p.dirs), p.dirs_blend, r);
}

cudaError_t launch_raygen(const Rot& rot, int R, int storage, float4* dirs_trace, float4* dirs_blend,
                          cudaStream_t st) {
    raygen_kernel<<<(R + 127) / 128, 128, 0, st>>>(rot, R, storage, dirs_trace, dirs_blend);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_raygen_batch(const TraceParams* vp, const int* starts, int n, int blocks, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    raygen_batch_kernel<<<blocks, 128, 0, st>>>(vp, starts, n);
    note_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------- march
// One thread per (probe, ray); consecutive threads take consecutive probes
// with the same ray index, so a warp marches 32 parallel rays from
// neighbouring probes through nearby SDF texels.  The march is the whole
// kernel (no shading code): small, low register count, high occupancy.
// Counts work item idx into shading bin `key` (one atomic per group of
// converged lanes with the same bin) and records its bin.
__device__ __forceinline__ void record_bin(const TraceParams& p, int64_t idx, uint32_t key) {
    const unsigned act = __activemask();
    const unsigned same = __match_any_sync(act, key);
    const int lane = int(threadIdx.x) & 31;
    const int leader = __ffs(same) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(p.bin_count + key, uint32_t(__popc(same)));
    base = __shfl_sync(same, base, leader);
    p.bin_key[idx] = make_uint2(key, base + uint32_t(__popc(same & ((1u << lane) - 1u))));
}

// Shading bin of a march result: the surface-cache chunk of the hit point
// (the chunk grid of sampleGlobalSurfaceAtlas), or the last bin.
__device__ __forceinline__ uint32_t shade_bin(const TraceParams& p, int cls, f3 origin, f3 dir, float time) {
    if (cls < 0) return p.bin_base + p.bin_span - 1;
    // the bin only groups hits for the shading (any bin gives the same
    // results), so the chunk comes from a multiply by the reciprocal
    const f3 hp = add3(origin, mul3(dir, time));
    const float ics = p.surf.inv_chunk;
    const int cx = imn(imx(int(floorf(hp.x * ics + float(kChunksRes * 0.5f))), 0), kChunksRes - 1);
    const int cy = imn(imx(int(floorf(hp.y * ics + float(kChunksRes * 0.5f))), 0), kChunksRes - 1);
    const int cz = imn(imx(int(floorf(hp.z * ics + float(kChunksRes * 0.5f))), 0), kChunksRes - 1);
    const uint32_t key = uint32_t((cz * kChunksRes + cy) * kChunksRes + cx);
    return p.bin_base + (p.bin_span == uint32_t(kShadeBins) ? key : key % p.bin_span);
}

__device__ __forceinline__ void write_march(const TraceParams& p, int64_t idx, int probe, int ray, f3 origin, f3 dir,
                                            const MarchHit& hit) {
    int cls = -1;                                          // miss
    if (hit.time >= 0.0f) {
        // GISDFRays.comp:93: a hit at the probe from inside a surface
        cls = (hit.sdf <= 0.0f && hit.time <= p.sdf.data.cascade_voxel_size[0]) ? -2 : hit.cascade;
    }
    const size_t o = size_t(probe) * p.R + ray;
    p.hit_t[o] = make_float4(hit.time, hit.normal.x, hit.normal.y, hit.normal.z);
    p.hit_c[o] = cls;
    if (p.info) p.info[o] = make_int4(hit.steps, hit.time >= 0.0f ? hit.cascade : -1, hit.fine, 0);
    if (p.bin_count) record_bin(p, idx, shade_bin(p, cls, origin, dir, hit.time));
}

// Suspended-march queue entry: (work item, volume, cascade | in-cascade << 7
// | step << 8, steps | fine << 16), (t, exit, next start, 0).
__device__ __forceinline__ void encode_march(int64_t idx, int vol, const MarchState& m, int4& a, float4& b) {
    a = make_int4(int(uint32_t(idx)), vol, m.cascade | (m.in_cascade << 7) | (m.step << 8), m.steps | (m.fine << 16));
    b = make_float4(m.t, m.is_y, m.next_start, 0.0f);
}

__device__ __forceinline__ void decode_march(const int4& a, const float4& b, int64_t& idx, int& vol, MarchState& m) {
    idx = int64_t(uint32_t(a.x));
    vol = a.y;
    m.cascade = a.z & 0x7F;
    m.in_cascade = (a.z >> 7) & 1;
    m.step = int(uint32_t(a.z) >> 8);
    m.steps = a.w & 0xFFFF;
    m.fine = int(uint32_t(a.w) >> 16);
    m.t = b.x;
    m.is_y = b.y;
    m.next_start = b.z;
}

// Appends the suspended marches of the calling lanes that want it, one
// atomic per group of converged lanes.  False where the queue is full (the
// lane then finishes its march in place).
__device__ __forceinline__ bool enqueue_march(int4* q, uint32_t* count, uint32_t cap, bool want, int64_t idx, int vol,
                                              const MarchState& m) {
    const unsigned act = __activemask();
    const unsigned ball = __ballot_sync(act, want);
    if (!ball) return false;
    const int lane = int(threadIdx.x) & 31;
    const int leader = __ffs(ball) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, uint32_t(__popc(ball)));
    base = __shfl_sync(act, base, leader);
    if (!want) return false;
    const uint32_t slot = base + uint32_t(__popc(ball & ((1u << lane) - 1u)));
    if (slot >= cap) return false;
    int4 ea;
    float4 eb;
    encode_march(idx, vol, m, ea, eb);
    q[2 * size_t(slot)] = ea;
    reinterpret_cast<float4*>(q)[2 * size_t(slot) + 1] = eb;
    return true;
}

// One work item: the whole march, or (compaction) at most budget1 steps
// with the rest queued.
template <typename SdfT, int QMIP, int QTEX, int DIV = kDivSplit>
__device__ __forceinline__ void march_ray(const TraceParams& p, int64_t idx) {
    int probe, ray;
    const bool valid = probe_ray(p, idx, probe, ray);
    MarchState m;
    march_state_init(m);
    MarchHit hit;
    bool done = true;
    if (!valid && p.bin_count) record_bin(p, idx, p.bin_base + p.bin_span - 1);   // tile padding
    if (valid) {
        const float4 d4 = __ldg(p.dirs + ray);
        const f3 dir{d4.x, d4.y, d4.z};
        const f3 origin = probe_location(p.u, uint32_t(probe), p.div_x, p.div_xy);
        done = march_run<SdfT, QMIP, QTEX, DIV>(p.sdf, origin, dir, kWorldSize, p.max_steps, m,
                                                  p.budget1 > 0 ? p.budget1 : 0x7FFFFFFF, hit);
        if (p.budget1 > 0 && enqueue_march(p.qa, p.qcount, p.qa_cap, !done, idx, p.vol, m)) {
            if (p.split) p.bin_key[idx] = make_uint2(kDeferredBin, 0u);
            return;
        }
        if (!done)
            march_run<SdfT, QMIP, QTEX, DIV>(p.sdf, origin, dir, kWorldSize, p.max_steps, m, 0x7FFFFFFF, hit);
        march_hit_normal<SdfT, QTEX>(p.sdf, hit);
        write_march(p, idx, probe, ray, origin, dir, hit);
    }
}

// Resumes queued marches: pass 2 (FINAL false) reads qa, runs budget2 more
// steps and queues the unfinished into qb; pass 3 (FINAL) finishes qb.
// Persistent blocks walk the queue.  vp: batched parameter blocks indexed
// by each entry's volume, or nullptr (then p).
template <typename SdfT, int QMIP, int QTEX, bool FINAL, int DIV = kDivSplit>
__device__ __forceinline__ void march_resume(const TraceParams& p0, const TraceParams* __restrict__ vp) {
    const int4* in = FINAL ? p0.qb : p0.qa;
    const uint32_t n = min(__ldg(p0.qcount + (FINAL ? 1 : 0)), FINAL ? p0.qb_cap : p0.qa_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int64_t idx;
        int vol;
        MarchState m;
        decode_march(__ldg(in + 2 * size_t(i)), __ldg(reinterpret_cast<const float4*>(in) + 2 * size_t(i) + 1), idx,
                     vol, m);
        const TraceParams& p = vp ? vp[vol] : p0;
        int probe, ray;
        probe_ray(p, idx, probe, ray);
        const float4 d4 = __ldg(p.dirs + ray);
        const f3 dir{d4.x, d4.y, d4.z};
        const f3 origin = probe_location(p.u, uint32_t(probe), p.div_x, p.div_xy);
        MarchHit hit;
        bool done = march_run<SdfT, QMIP, QTEX, DIV>(p.sdf, origin, dir, kWorldSize, p.max_steps, m,
                                                       FINAL ? 0x7FFFFFFF : p.budget2, hit);
        if (!FINAL && enqueue_march(p0.qb, p0.qcount + 1, p0.qb_cap, !done, idx, vol, m)) continue;
        if (!done)
            march_run<SdfT, QMIP, QTEX, DIV>(p.sdf, origin, dir, kWorldSize, p.max_steps, m, 0x7FFFFFFF, hit);
        march_hit_normal<SdfT, QTEX>(p.sdf, hit);
        write_march(p, idx, probe, ray, origin, dir, hit);
    }
}

// Pass 1 keeps 9 blocks of 128 a SM (56 registers; 36 warps where 64
// registers leave 32): the march waits on its taps, so more resident rays
// pay for the few spilled bytes (production march 0.851 -> 0.841 ms).  The
// gather textures of both volumes (variant 10) run best at 8 (64
// registers: production march 0.800 -> 0.796 ms; variant 11 loses at 8).
// MIN_BLOCKS 1 (variant 2) leaves the registers unbounded.
template <typename SdfT, int MIN_BLOCKS, int QMIP, int QTEX>
__global__ void __launch_bounds__(128, MIN_BLOCKS == 1 ? 2 : (QMIP == kGather && QTEX == kGather ? 8 : 9))
    march_kernel(const TraceParams p) {
    const int64_t idx = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (idx >= p.work) return;
    march_ray<SdfT, QMIP, QTEX>(p, idx);
}

template <typename SdfT, int MIN_BLOCKS, int QMIP, int QTEX, bool FINAL>
__global__ void __launch_bounds__(256, MIN_BLOCKS) march_resume_kernel(const TraceParams p) {
    march_resume<SdfT, QMIP, QTEX, FINAL>(p, nullptr);
}

// Batched march over many volumes: TPB rays per block, the volume's
// parameters staged in shared memory once per block.  Same per-ray code as
// march_kernel, hence the same results.
template <typename SdfT, int TPB, int MIN_BLOCKS, int QMIP, int QTEX>
__global__ void __launch_bounds__(TPB, MIN_BLOCKS)
    march_batch_kernel(const TraceParams* __restrict__ vp, const int* __restrict__ starts, int n) {
    __shared__ __align__(16) uint32_t sp[sizeof(TraceParams) / 4];
    const int v = batch_volume(starts, n, int(blockIdx.x));
    const TraceParams& p = stage_params(vp + v, sp);
    const int64_t idx = int64_t(int(blockIdx.x) - __ldg(starts + v)) * TPB + threadIdx.x;
    if (idx >= p.work) return;
    // one step loop choosing each quotient's form (two copies spill here:
    // batch48 2.52e9 -> 2.30e9 probe-rays/s; exact quotients alone 2.93e9,
    // chosen per quotient 2.97e9)
    march_ray<SdfT, QMIP, QTEX, kDivSelect>(p, idx);
}

// Resume passes of a batch: every volume's parameter block names the same
// queues; entries carry their volume.
template <typename SdfT, int MIN_BLOCKS, int QMIP, int QTEX, bool FINAL>
__global__ void __launch_bounds__(256, MIN_BLOCKS) march_resume_batch_kernel(const TraceParams* __restrict__ vp) {
    march_resume<SdfT, QMIP, QTEX, FINAL, kDivSelect>(vp[0], vp);
}

// ------------------------------------------------------- pooled march
// Warp-cooperative step scheduling: each warp owns a pool of 32 * POOL
// consecutive rays; a lane whose ray ends takes the next one from the pool
// at once, so lanes do not idle while the warp's longest ray finishes.  The
// per-ray arithmetic is exactly march_sdf's (SDFCommon.glsl:98-194), kept
// as a small state machine: a cascade set-up phase and a step phase.
template <typename SdfT, int QMIP, int QTEX, int POOL>
__global__ void __launch_bounds__(256, 4) march_pool_kernel(const TraceParams p) {
    const SdfView& s = p.sdf;
    const int lane = threadIdx.x & 31;
    const int64_t total = int64_t(p.P) * p.R;
    const int64_t wbase = ((int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5) * (32 * POOL);
    const int64_t wend = wbase + 32 * POOL < total ? wbase + 32 * POOL : total;
    const int C = s.C;
    const int TW = s.res * C, MW = s.mres * C;
    const float tmax = mn(kWorldSize, s.data.cascade_pos_distance[C - 1][3] * 2.0f);
    const float chunk = 32.0f / s.data.resolution;
    const float margin = 4.0f / s.data.resolution;
    // lane state
    int64_t cur = wbase + lane;
    bool has = cur < wend;
    f3 origin{0.0f, 0.0f, 0.0f}, dir{0.0f, 0.0f, 0.0f}, end{0.0f, 0.0f, 0.0f};
    float t = 0.0f, is_y = 0.0f, next_start = 0.0f;
    int cascade = 0, step = 0, steps = 0, fine = 0;
    bool setup = true;
    auto begin_ray = [&](int64_t idx) {
        int probe, ray;
        probe_ray(p, idx, probe, ray);
        const float4 d4 = __ldg(p.dirs + ray);
        dir = f3{d4.x, d4.y, d4.z};
        origin = probe_location(p.u, uint32_t(probe), p.div_x, p.div_xy);
        end = add3(origin, mul3(dir, tmax));
        next_start = 0.0f;
        cascade = 0;
        steps = 0;
        fine = 0;
        setup = true;
    };
    auto finish_ray = [&](int64_t idx, float time, int hc, float hsdf, f3 nrm) {
        int probe, ray;
        probe_ray(p, idx, probe, ray);
        int cls = -1;
        if (time >= 0.0f) cls = (hsdf <= 0.0f && time <= s.data.cascade_voxel_size[0]) ? -2 : hc;
        const size_t o = size_t(probe) * p.R + ray;
        p.hit_t[o] = make_float4(time, nrm.x, nrm.y, nrm.z);
        p.hit_c[o] = cls;
        if (p.info) p.info[o] = make_int4(steps, time >= 0.0f ? hc : -1, fine, 0);
    };
    if (has) begin_ray(cur);
    int handed = 32;                                  // rays of the pool taken so far (warp-uniform)
    while (__any_sync(0xffffffffu, has)) {
        if (has) {
            const float cx = s.data.cascade_pos_distance[cascade < C ? cascade : 0][0];
            const float cy = s.data.cascade_pos_distance[cascade < C ? cascade : 0][1];
            const float cz = s.data.cascade_pos_distance[cascade < C ? cascade : 0][2];
            const float cw = s.data.cascade_pos_distance[cascade < C ? cascade : 0][3];
            const float voxel = s.data.cascade_voxel_size[cascade < C ? cascade : 0];
            const f3 wpos = add3(origin, mul3(dir, voxel * 0.0f));
            if (setup) {
                if (cascade >= C) {
                    finish_ray(cur, -1.0f, 0, 0.0f, f3{0.0f, 0.0f, 0.0f});     // left every cascade: miss
                    has = false;
                } else {
                    // lineHitAABB (SDFCommon.glsl:84-95) and the cascade entry
                    const f3 d = sub3(end, wpos);
                    const f3 inv{1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
                    const f3 en{((cx - cw) - wpos.x) * inv.x, ((cy - cw) - wpos.y) * inv.y, ((cz - cw) - wpos.z) * inv.z};
                    const f3 ex{((cx + cw) - wpos.x) * inv.x, ((cy + cw) - wpos.y) * inv.y, ((cz + cw) - wpos.z) * inv.z};
                    const float i0 = mx(mn(en.x, ex.x), mx(mn(en.y, ex.y), mn(en.z, ex.z)));
                    const float i1 = mn(mx(en.x, ex.x), mn(mx(en.y, ex.y), mx(en.z, ex.z)));
                    float is_x = clampf(i0, 0.0f, 1.0f) * tmax;
                    is_y = clampf(i1, 0.0f, 1.0f) * tmax;
                    is_x = mx(is_x, next_start);
                    t = is_x;
                    if (is_x >= is_y) t = is_y;
                    else next_start = is_y;
                    step = 0;
                    setup = false;
                }
            }
            if (has && !setup) {
                if (step < p.max_steps && t < is_y) {
                    const float md = cw * 2.0f;
                    const f3 sp = add3(wpos, mul3(dir, t));
                    const float ux = clampf((sp.x - cx) / md + 0.5f, 0.0f, 1.0f);
                    const float uy = clampf((sp.y - cy) / md + 0.5f, 0.0f, 1.0f);
                    const float uz = clampf((sp.z - cz) / md + 0.5f, 0.0f, 1.0f);
                    const float tu = (float(cascade) + ux) / float(C);
                    float sd = sample_vol<SdfT, QMIP>(s.mip, s.mip_quad, s.mip_g, MW, s.mres, s.mres, tu, uy, uz);
                    const float sdt = sample_vol<SdfT, QTEX>(s.sdf, s.sdf_quad, s.sdf_g, TW, s.res, s.res, tu, uy, uz);
                    if (sd < chunk) {
                        ++fine;
                        if (sdt < margin * 2.0f) sd = sdt;
                    } else {
                        sd = chunk;
                    }
                    sd = sd * md;
                    const float thick = (voxel * 0.5f) * clampf(t / voxel, 0.0f, 1.0f);
                    if (sd < thick) {
                        const float time = mx(t + sd - thick, 0.0f);
                        const f3 nrm = sdf_normal<SdfT, QTEX>(s.sdf, s.sdf_quad, s.sdf_g, TW, s.res, tu, uy, uz,
                                                             1.0f / s.data.resolution);
                        steps += step;
                        finish_ray(cur, time, cascade, sd, nrm);
                        has = false;
                    } else {
                        t = t + mx(sd * 1.0f, voxel);
                        ++step;
                    }
                } else {
                    steps += step;                     // this cascade is done
                    ++cascade;
                    setup = true;
                }
            }
        }
        // refill finished lanes from the warp's pool
        const unsigned need = __ballot_sync(0xffffffffu, !has);
        const int avail = 32 * POOL - handed;
        if (need && avail > 0) {
            const int rank = __popc(need & ((1u << lane) - 1u));
            if (!has && rank < avail) {
                cur = wbase + handed + rank;
                has = cur < wend;
                if (has) begin_ray(cur);
            }
            const int taken = __popc(need);
            handed += taken < avail ? taken : avail;
        }
    }
}

static unsigned resume_blocks() {
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    return unsigned(sms * 4);
}

// One march variant: pass 1 over every work item, then (compaction) the two
// resume passes over the queued rays, with the parameters `rp` (those of
// pass 1 unless the shading is split) and `after_first` (or nullptr)
// recorded between.
template <typename SdfT, int MINB, int QMIP, int QTEX>
static cudaError_t launch_march_variant(const TraceParams& p, cudaStream_t st, const TraceParams& rp,
                                        cudaEvent_t after_first) {
    const unsigned mblocks = unsigned((p.work + 127) / 128);
    if (p.budget1 > 0) {
        const cudaError_t e = cudaMemsetAsync(p.qcount, 0, 2 * sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
    }
    march_kernel<SdfT, MINB, QMIP, QTEX><<<mblocks, 128, 0, st>>>(p);
    note_launch();
    if (after_first) {
        const cudaError_t e = cudaEventRecord(after_first, st);
        if (e != cudaSuccess) return e;
    }
    if (p.budget1 > 0) {
        const unsigned rb = resume_blocks();
        march_resume_kernel<SdfT, MINB, QMIP, QTEX, false><<<rb, 256, 0, st>>>(rp);
        march_resume_kernel<SdfT, MINB, QMIP, QTEX, true><<<rb, 256, 0, st>>>(rp);
        note_launch(2);
    }
    return cudaGetLastError();
}

static cudaError_t launch_march_passes(const TraceParams& p, cudaStream_t st, const TraceParams& rp,
                                       cudaEvent_t after_first);

cudaError_t launch_march(const TraceParams& p, cudaStream_t st) { return launch_march_passes(p, st, p, nullptr); }

cudaError_t launch_march_split(const TraceParams& p, const TraceParams& resume, cudaEvent_t after_first,
                               cudaStream_t st) {
    if (pooled_variant(p.march_variant) || p.budget1 <= 0 || !after_first) return cudaErrorInvalidValue;
    return launch_march_passes(p, st, resume, after_first);
}

static cudaError_t launch_march_passes(const TraceParams& p, cudaStream_t st, const TraceParams& rp,
                                       cudaEvent_t after_first) {
    const int64_t total = p.work;
    if (total <= 0) return cudaSuccess;
    if (pooled_variant(p.march_variant)) {
        // pooled march: 8 rays per lane, 8 warps per block
        constexpr int POOL = 8;
        const int64_t warps = (total + 32 * POOL - 1) / (32 * POOL);
        const unsigned pblocks = unsigned((warps + 7) / 8);
        const bool h = p.sdf.format == LUXGI_STORAGE_FP16;
        switch (p.march_variant) {
            case 7:
                if (h) march_pool_kernel<__half, kQuad, kPlain, POOL><<<pblocks, 256, 0, st>>>(p);
                else march_pool_kernel<float, kQuad, kPlain, POOL><<<pblocks, 256, 0, st>>>(p);
                break;
            case 8:
                if (h) march_pool_kernel<__half, kQuad, kQuad, POOL><<<pblocks, 256, 0, st>>>(p);
                else march_pool_kernel<float, kQuad, kQuad, POOL><<<pblocks, 256, 0, st>>>(p);
                break;
            case 9:
                if (h) march_pool_kernel<__half, kQuad, kPair, POOL><<<pblocks, 256, 0, st>>>(p);
                else march_pool_kernel<float, kQuad, kPair, POOL><<<pblocks, 256, 0, st>>>(p);
                break;
            default:
                if (h) march_pool_kernel<__half, kPlain, kPlain, POOL><<<pblocks, 256, 0, st>>>(p);
                else march_pool_kernel<float, kPlain, kPlain, POOL><<<pblocks, 256, 0, st>>>(p);
                break;
        }
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        note_launch();
        return cudaSuccess;
    }
    // variants: 1 plain layout, 64 registers (4 blocks of 256 per SM);
    // 2 plain layout, no register bound; 3 quad-packed mip; 4 quad-packed
    // mip and full-resolution volume; 5 quad-packed mip, pair-packed
    // full-resolution volume; 10 gather textures of the mip and the
    // full-resolution volume; 11 quad-packed mip, gather texture of the
    // full-resolution volume (the mip's loads on the LSU path, the fine
    // samples on the texture path).  All produce identical results.
    const bool h = p.sdf.format == LUXGI_STORAGE_FP16;
    cudaError_t e;
    const TraceParams& r = rp;
    cudaEvent_t a = after_first;
    switch (p.march_variant) {
        case 2: e = h ? launch_march_variant<__half, 1, kPlain, kPlain>(p, st, r, a) : launch_march_variant<float, 1, kPlain, kPlain>(p, st, r, a); break;
        case 3: e = h ? launch_march_variant<__half, 4, kQuad, kPlain>(p, st, r, a) : launch_march_variant<float, 4, kQuad, kPlain>(p, st, r, a); break;
        case 4: e = h ? launch_march_variant<__half, 4, kQuad, kQuad>(p, st, r, a) : launch_march_variant<float, 4, kQuad, kQuad>(p, st, r, a); break;
        case 5: e = h ? launch_march_variant<__half, 4, kQuad, kPair>(p, st, r, a) : launch_march_variant<float, 4, kQuad, kPair>(p, st, r, a); break;
        case 10: e = h ? launch_march_variant<__half, 4, kGather, kGather>(p, st, r, a) : launch_march_variant<float, 4, kGather, kGather>(p, st, r, a); break;
        case 11: e = h ? launch_march_variant<__half, 4, kQuad, kGather>(p, st, r, a) : launch_march_variant<float, 4, kQuad, kGather>(p, st, r, a); break;
        default: e = h ? launch_march_variant<__half, 4, kPlain, kPlain>(p, st, r, a) : launch_march_variant<float, 4, kPlain, kPlain>(p, st, r, a); break;
    }
    return e;
}

template <typename SdfT, int TPB, int MINB, int QMIP, int QTEX>
static void march_batch_launch(unsigned blocks, const TraceParams* vp, const int* starts, int n, bool compact,
                               cudaStream_t st) {
    march_batch_kernel<SdfT, TPB, MINB, QMIP, QTEX><<<blocks, TPB, 0, st>>>(vp, starts, n);
    if (compact) {
        constexpr int RMINB = MINB == 1 ? 1 : 4;   // resume kernels run 256-thread blocks
        const unsigned rb = resume_blocks();
        march_resume_batch_kernel<SdfT, RMINB, QMIP, QTEX, false><<<rb, 256, 0, st>>>(vp);
        march_resume_batch_kernel<SdfT, RMINB, QMIP, QTEX, true><<<rb, 256, 0, st>>>(vp);
    }
}

template <typename SdfT, int TPB, int MINB>
static void march_batch_variant(int variant, unsigned blocks, const TraceParams* vp, const int* starts, int n,
                                bool compact, cudaStream_t st) {
    switch (variant) {
        case 2: march_batch_launch<SdfT, TPB, 1, kPlain, kPlain>(blocks, vp, starts, n, compact, st); break;
        case 3: march_batch_launch<SdfT, TPB, MINB, kQuad, kPlain>(blocks, vp, starts, n, compact, st); break;
        case 4: march_batch_launch<SdfT, TPB, MINB, kQuad, kQuad>(blocks, vp, starts, n, compact, st); break;
        case 5: march_batch_launch<SdfT, TPB, MINB, kQuad, kPair>(blocks, vp, starts, n, compact, st); break;
        case 10: march_batch_launch<SdfT, TPB, MINB, kGather, kGather>(blocks, vp, starts, n, compact, st); break;
        case 11: march_batch_launch<SdfT, TPB, MINB, kQuad, kGather>(blocks, vp, starts, n, compact, st); break;
        default: march_batch_launch<SdfT, TPB, MINB, kPlain, kPlain>(blocks, vp, starts, n, compact, st); break;
    }
}

cudaError_t launch_march_batch(const TraceParams* vp, const int* starts, int n, int blocks, int variant, int tpb,
                               int sdf_format, int compact, uint32_t* qcount, cudaStream_t st) {
    if (blocks <= 0) return cudaSuccess;
    if (!per_ray_variant(variant)) return cudaErrorInvalidValue;
    if (tpb != 128 && tpb != 256) return cudaErrorInvalidValue;
    if (compact) {
        const cudaError_t e = cudaMemsetAsync(qcount, 0, 2 * sizeof(uint32_t), st);
        if (e != cudaSuccess) return e;
    }
    const bool h = sdf_format == LUXGI_STORAGE_FP16;
    // bounded variants keep 56 registers a thread in 128-ray blocks (9 blocks
    // a SM: batch48 frame 4.84 -> 4.80 ms against 8 at 64 registers) and 64
    // in 256-ray blocks
    if (tpb == 128) {
        if (h) march_batch_variant<__half, 128, 9>(variant, unsigned(blocks), vp, starts, n, compact != 0, st);
        else march_batch_variant<float, 128, 9>(variant, unsigned(blocks), vp, starts, n, compact != 0, st);
    } else {
        if (h) march_batch_variant<__half, 256, 4>(variant, unsigned(blocks), vp, starts, n, compact != 0, st);
        else march_batch_variant<float, 256, 4>(variant, unsigned(blocks), vp, starts, n, compact != 0, st);
    }
    note_launch(compact ? 3 : 1);
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

// ------------------------------------------------------------ cell minima
// Cell (i, j, k) of a W x H x D volume: min over texels [4i, 4i+4] x
// [4j, 4j+4] x [4k, 4k+4] clamped to the volume (every texel of a trilinear
// footprint whose clamped lower corner lies in the cell).
template <typename T>
__global__ void cell_min_kernel(const T* __restrict__ src, int W, int H, int D, int cw, int ch, int cd,
                                float* __restrict__ dst) {
    const int64_t n = int64_t(cw) * ch * cd;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int cx = int(i % cw), cy = int((i / cw) % ch), cz = int(i / (int64_t(cw) * ch));
        float m = 3.0e38f;
        for (int z = cz * kCellSide; z <= imn(cz * kCellSide + kCellSide, D - 1); ++z)
            for (int y = cy * kCellSide; y <= imn(cy * kCellSide + kCellSide, H - 1); ++y)
                for (int x = cx * kCellSide; x <= imn(cx * kCellSide + kCellSide, W - 1); ++x)
                    m = mn(m, load_val(src, (size_t(z) * H + y) * W + x));
        dst[i] = m;
    }
}

// One bit per cell, 32 cells a word: set where the cell minimum is below the
// march's skip threshold, i.e. where the full-resolution taps may be used.
// The threshold is march_run's, computed by the same expression.
__global__ void cell_bits_kernel(const float* __restrict__ cmin, int64_t n, float resolution,
                                 uint32_t* __restrict__ bits) {
    const float margin = 4.0f / resolution;
    const float thr = (margin * 2.0f) * 1.001f;
    const int64_t words = (n + 31) / 32;
    for (int64_t w = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; w < words; w += int64_t(gridDim.x) * blockDim.x) {
        uint32_t b = 0;
        for (int k = 0; k < 32; ++k) {
            const int64_t i = w * 32 + k;
            if (i < n && !(cmin[i] >= thr)) b |= 1u << k;
        }
        bits[w] = b;
    }
}

static int64_t cell_count(int W, int H, int D) {
    return int64_t((W + kCellSide - 1) / kCellSide) * ((H + kCellSide - 1) / kCellSide) *
           ((D + kCellSide - 1) / kCellSide);
}

// The cell minima (FP32), then the bits, 16-byte aligned.
static size_t cell_bits_offset(int64_t n) { return (sizeof(float) * size_t(n) + 15) / 16 * 16; }

size_t cell_min_bytes(int W, int H, int D) {
    const int64_t n = cell_count(W, H, D);
    return cell_bits_offset(n) + sizeof(uint32_t) * size_t((n + 31) / 32);
}

const uint32_t* cell_bits(const float* cmin, int W, int H, int D) {
    return reinterpret_cast<const uint32_t*>(reinterpret_cast<const uint8_t*>(cmin) +
                                             cell_bits_offset(cell_count(W, H, D)));
}

cudaError_t launch_cell_min(const void* src, int W, int H, int D, int format, float resolution, float* dst,
                            cudaStream_t st) {
    const int cw = (W + kCellSide - 1) / kCellSide, ch = (H + kCellSide - 1) / kCellSide;
    const int cd = (D + kCellSide - 1) / kCellSide;
    const int64_t n = int64_t(cw) * ch * cd;
    const unsigned blocks = unsigned(std::min<int64_t>((n + 255) / 256, 4096));
    if (format == LUXGI_STORAGE_FP16)
        cell_min_kernel<__half><<<blocks, 256, 0, st>>>(static_cast<const __half*>(src), W, H, D, cw, ch, cd, dst);
    else
        cell_min_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(src), W, H, D, cw, ch, cd, dst);
    const int64_t words = (n + 31) / 32;
    cell_bits_kernel<<<unsigned(std::min<int64_t>((words + 255) / 256, 4096)), 256, 0, st>>>(
        dst, n, resolution, const_cast<uint32_t*>(cell_bits(dst, W, H, D)));
    note_launch(2);
    return cudaGetLastError();
}

// ------------------------------------------------------------ gather pack
// The gather-texture image of a W x H x D volume (GatherVol): planes of
// (W + 2) x (H + 2) texels, gx to a row, each with a 1-texel apron that
// repeats its edge; texels past the last plane are 0.  Written to a linear
// staging image of tw x th elements, copied into the texture's array.
template <typename T>
__global__ void gather_pack_kernel(const T* __restrict__ src, int W, int H, int D, int gx, int tw, int th,
                                   T* __restrict__ dst) {
    const int pw = W + 2, ph = H + 2;
    const int64_t n = int64_t(tw) * th;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const int tx = int(i % tw), ty = int(i / tw);
        const int z = (ty / ph) * gx + tx / pw;
        T v = T(0.0f);
        if (z < D) {
            const int x = imn(imx(tx % pw - 1, 0), W - 1), y = imn(imx(ty % ph - 1, 0), H - 1);
            v = src[(size_t(z) * H + y) * W + x];
        }
        dst[i] = v;
    }
}

cudaError_t launch_gather_pack(const void* src, int W, int H, int D, int gx, int tw, int th, int format, void* dst,
                               cudaStream_t st) {
    const int64_t n = int64_t(tw) * th;
    const unsigned blocks = unsigned(std::min<int64_t>((n + 255) / 256, 8192));
    if (format == LUXGI_STORAGE_FP16)
        gather_pack_kernel<__half><<<blocks, 256, 0, st>>>(static_cast<const __half*>(src), W, H, D, gx, tw, th,
                                                           static_cast<__half*>(dst));
    else
        gather_pack_kernel<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(src), W, H, D, gx, tw, th,
                                                          static_cast<float*>(dst));
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

// SampleProbe.comp:36-60: one thread per pixel of a screen G-buffer.  The
// world position comes back from the depth through the inverse
// view-projection (worldPositionFromDepth, Common/Math.glsl:35-42), the
// normal from the octahedral normal target (octohedralToDirection,
// Math.glsl:26-32); background pixels (depth 1) get 0.
__global__ void sample_probe_kernel(const luxgi_ddgi_uniform u, const AtlasView A, const float* __restrict__ depth,
                                    const float* __restrict__ normal, int nch, int W, int H, const float3 cam,
                                    const Mat4 vpi, __half* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t i = size_t(y) * W + x;
    const float d = __ldg(depth + i);
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (d != 1.0f) {
        const float tx = (float(x) + 0.5f) / float(W), ty = (float(y) + 0.5f) / float(H);
        const float sx = tx * 2.0f - 1.0f, sy = ty * 2.0f - 1.0f;
        const float* m = vpi.m;
        const float wx = (m[0] * sx + m[4] * sy) + (m[8] * d + m[12]);
        const float wy = (m[1] * sx + m[5] * sy) + (m[9] * d + m[13]);
        const float wz = (m[2] * sx + m[6] * sy) + (m[10] * d + m[14]);
        const float ww = (m[3] * sx + m[7] * sy) + (m[11] * d + m[15]);
        const f3 P{wx / ww, wy / ww, wz / ww};
        const float ex = __ldg(normal + i * nch), ey = __ldg(normal + i * nch + 1);
        f3 v{ex, ey, 1.0f - fabsf(ex) - fabsf(ey)};
        if (v.z < 0.0f) {
            const float nx = (1.0f - fabsf(v.y)) * sign_nz(v.x);
            const float ny = (1.0f - fabsf(v.x)) * sign_nz(v.y);
            v.x = nx;
            v.y = ny;
        }
        const f3 N = norm3(v);
        const f3 Wo = norm3(sub3(f3{cam.x, cam.y, cam.z}, P));
        const f3 e = sample_irradiance(u, A, P, N, Wo);
        o = make_float4(e.x, e.y, e.z, 1.0f);
    }
    const __half2 a = __floats2half2_rn(o.x, o.y), b = __floats2half2_rn(o.z, o.w);
    uint2 raw;
    raw.x = *reinterpret_cast<const uint32_t*>(&a);
    raw.y = *reinterpret_cast<const uint32_t*>(&b);
    reinterpret_cast<uint2*>(out)[i] = raw;
}

cudaError_t launch_sample_probe(const luxgi_ddgi_uniform& u, const AtlasView& A, const float* depth,
                                const float* normal, int nch, int W, int H, const float cam[3], const float vpi[16],
                                void* out, cudaStream_t st) {
    if (W <= 0 || H <= 0) return cudaSuccess;
    Mat4 m;
    for (int k = 0; k < 16; ++k) m.m[k] = vpi[k];
    const dim3 blk(32, 8), grd(unsigned((W + 31) / 32), unsigned((H + 7) / 8));
    sample_probe_kernel<<<grd, blk, 0, st>>>(u, A, depth, normal, nch, W, H, make_float3(cam[0], cam[1], cam[2]), m,
                                             static_cast<__half*>(out));
    note_launch();
    return cudaGetLastError();
}

}  // namespace luxgi
