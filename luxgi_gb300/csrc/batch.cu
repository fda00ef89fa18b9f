// Batched updates of many volumes: luxgi_ddgi_update_batch and the
// luxgi_ddgi_batch_* objects (graph capture and replay, autotuning).
//
// The reference dispatches the DDGI compute passes once per volume
// (Engine/DDGI/DDGIRenderer.cpp:217-464).  Here a frame of a whole set of
// volumes is one launch per stage: every batched kernel finds the volume of
// its block in a block-offset table and reads that volume's parameters from
// a per-frame argument block in device memory.  The kernels run the same
// per-ray and per-texel code as the single-volume launches, so each
// volume's results equal its own luxgi_ddgi_update.
#include <algorithm>
#include <climits>
#include <cstring>
#include <new>
#include <vector>

#include <cuda_runtime.h>

#include "luxgi_batch.h"

using namespace luxgi;

namespace luxgi {


static size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

int compat_check(luxgi_ddgi_volume* const* vols, int n) {
    if (n < 1 || !vols) return LUXGI_EINVAL;
    for (int i = 0; i < n; ++i) {
        const luxgi_ddgi_volume* v = vols[i];
        if (!v) return LUXGI_EINVAL;
        if (!v->bound) return LUXGI_ENOTBOUND;
        const luxgi_ddgi_volume* a = vols[0];
        if (v->desc.storage != a->desc.storage || v->desc.light_mode != a->desc.light_mode || v->tc != a->tc ||
            v->sdf.format != a->sdf.format || v->device != a->device)
            return LUXGI_EINVAL;
        for (int j = 0; j < i; ++j)
            if (vols[j] == v) return LUXGI_EINVAL;
    }
    return LUXGI_OK;
}

bool tuning_valid(const luxgi_ddgi_batch_tuning& t) {
    return per_ray_variant(t.march_variant) &&
           (t.march_threads == 128 || t.march_threads == 256) &&
           (t.shade_variant == 1 || t.shade_variant == 2 || t.shade_variant == 4 || t.shade_variant == 8) &&
           (t.blend_probes == 1 || t.blend_probes == 2 || t.blend_probes == 4) && (t.use_graph == 0 || t.use_graph == 1) &&
           t.march_budget >= -1 && t.shade_order >= -1 && t.shade_order <= 1;
}

luxgi_ddgi_batch_tuning default_tuning() {
    luxgi_ddgi_batch_tuning t;
    std::memset(&t, 0, sizeof(t));
    t.march_variant = 4;
    t.march_threads = 256;
    t.shade_variant = 1;
    t.blend_probes = 2;
    t.use_graph = 1;
    t.march_budget = 0;
    return t;
}

static size_t queue_bytes(const Plan& P) {
    return P.budget > 0 ? sizeof(int4) * 2 * (size_t(P.qa_cap) + P.qb_cap) + 16 : 0;
}

size_t plan_aux_bytes(const Plan& P) {
    size_t b = queue_bytes(P);
    if (P.sorted) b += sizeof(uint32_t) * (2 * size_t(kBatchShadeBins) + 3 * size_t(P.work)) + 16;
    return b;
}

void plan_set_aux(Plan& P, void* dev) {
    P.q = nullptr;
    P.qcount = nullptr;
    P.sbins = P.sseq = nullptr;
    P.skeys = nullptr;
    if (!dev) return;
    uint8_t* base = static_cast<uint8_t*>(dev);
    if (P.budget > 0) {
        P.q = reinterpret_cast<int4*>(base);
        P.qcount = reinterpret_cast<uint32_t*>(P.q + 2 * (size_t(P.qa_cap) + P.qb_cap));
        base += queue_bytes(P);
    }
    if (P.sorted) {
        P.sbins = reinterpret_cast<uint32_t*>(base);
        P.skeys = reinterpret_cast<uint2*>(P.sbins + 2 * size_t(kBatchShadeBins));
        P.sseq = reinterpret_cast<uint32_t*>(P.skeys + size_t(P.work));
    }
}

// Gives every volume the plan's march and shade variant (the packed SDF
// copies follow the march variant).
int apply_variants(luxgi_ddgi_volume* const* vols, int n, const luxgi_ddgi_batch_tuning& t) {
    for (int i = 0; i < n; ++i) {
        luxgi_ddgi_volume* v = vols[i];
        v->desc.shade_variant = t.shade_variant;
        if (v->desc.march_variant != t.march_variant) {
            v->desc.march_variant = t.march_variant;
            const int s = volume_alloc_packs(v);
            if (s != LUXGI_OK) return s;
        }
    }
    return LUXGI_OK;
}

int plan_build(Plan& P, luxgi_ddgi_volume* const* vols, int n, const luxgi_ddgi_batch_tuning& t) {
    P = Plan();
    P.vols.assign(vols, vols + n);
    P.n = n;
    P.t = t;
    P.storage = vols[0]->desc.storage;
    P.light_mode = vols[0]->desc.light_mode;
    P.sdf_format = vols[0]->sdf.format;
    P.tc = vols[0]->tc;
    P.tc_bytes = tc_job_bytes();
    P.off_trace = 0;
    P.off_blend = align16(sizeof(TraceParams) * n);
    // the tensor-core jobs hold tensor maps: 128-byte aligned
    P.off_tc = (P.off_blend + align16(sizeof(BlendParams) * n) + 127) / 128 * 128;
    P.arg_bytes = P.off_tc + (P.tc ? P.tc_bytes * n : 0);
    P.starts.assign(size_t(kNumStages) * (n + 1), 0);
    int64_t acc[kNumStages] = {};
    std::vector<TcBlendParams> tps;
    if (P.tc) P.tcp.resize(n);
    P.budget = 1 << 30;
    for (int i = 0; i < n; ++i) {
        const luxgi_ddgi_volume* v = vols[i];
        BlendParams b;
        volume_blend_params(v, b);
        const int64_t PR = trace_work(v->P, v->R, (v->desc.ray_order == 1 && !pooled_variant(v->desc.march_variant)) ? 1 : 0);
        luxgi_ddgi_volume_desc vd = v->desc;
        vd.march_budget = t.march_budget == 0 ? kDefaultMarchBudget : t.march_budget;
        P.budget = std::min(P.budget, march_budget_for(vd, PR, int(v->sdf.data.cascades_count)));
        P.work += PR;
        int64_t cnt[kNumStages];
        cnt[kRaygen] = (v->R + 127) / 128;
        cnt[kWeights] = weight_rows(b);
        cnt[kMarch] = (PR + t.march_threads - 1) / t.march_threads;
        cnt[kShade] = (PR + 127) / 128;
        cnt[kBlendI] = P.tc ? 0 : blend_blocks(b, false, t.blend_probes);
        cnt[kBlendD] = P.tc ? 0 : blend_blocks(b, true, t.blend_probes);
        cnt[kWork] = PR;
        cnt[kPack] = P.tc ? (int64_t(v->P) * v->R + 255) / 256 : 0;
        for (int s = 0; s < kNumStages; ++s) {
            P.starts[size_t(s) * (n + 1) + i] = int(acc[s]);
            acc[s] += cnt[s];
            if (acc[s] > INT_MAX) return LUXGI_EINVAL;
        }
        if (!P.tc) {
            P.smem_i = std::max(P.smem_i, blend_smem(b, false, t.blend_probes));
            P.smem_d = std::max(P.smem_d, blend_smem(b, true, t.blend_probes));
        } else {
            TcBlendParams tp;
            volume_tc_params(v, tp);
            if (!tc_plan(tp, P.tcp[i])) return LUXGI_EUNSUPPORTED;
            tps.push_back(tp);
        }
    }
    // every volume's two blend kinds in one tensor-core launch
    if (P.tc && !tc_launch_shape(tps.data(), P.tcp.data(), n, P.storage, P.tcl)) return LUXGI_EUNSUPPORTED;
    for (int s = 0; s < kNumStages; ++s) {
        P.starts[size_t(s) * (n + 1) + n] = int(acc[s]);
        P.blocks[s] = int(acc[s]);
    }
    // the batch's queue entries hold 32-bit work indices per volume; the
    // counters hold the whole batch's
    if (P.work >= (int64_t(1) << 32)) P.budget = 0;
    if (t.march_budget == 0 && P.work < kLargeWork) P.budget = 0;   // default: large batches only
    if (P.budget > 0) {
        P.qa_cap = march_qa_cap(P.work);
        P.qb_cap = march_qb_cap(P.work);
    }
    // batch-wide work indices are ints in the work-offset table (INT_MAX checked above)
    P.sorted = t.shade_order == 1 && !pooled_variant(t.march_variant) && n <= kBatchShadeBins / 2;
    return LUXGI_OK;
}

// Per-frame arguments of every volume in its current state.
void plan_fill(const Plan& P, const float* rots, uint8_t* host) {
    TraceParams* tp = reinterpret_cast<TraceParams*>(host + P.off_trace);
    BlendParams* bp = reinterpret_cast<BlendParams*>(host + P.off_blend);
    for (int i = 0; i < P.n; ++i) {
        const luxgi_ddgi_volume* v = P.vols[i];
        volume_trace_params(v, rots + 9 * i, tp[i]);
        tp[i].budget1 = P.q ? P.budget : 0;
        tp[i].budget2 = march_budget2(P.t.march_budget, P.budget);
        tp[i].qa = P.q;
        tp[i].qb = P.q ? P.q + 2 * size_t(P.qa_cap) : nullptr;
        tp[i].qcount = P.qcount;
        tp[i].qa_cap = P.qa_cap;
        tp[i].qb_cap = P.qb_cap;
        tp[i].vol = i;
        // shading bins shared by the batch; keys at the volume's batch-wide offset
        tp[i].bin_count = P.sbins;
        tp[i].bin_key = P.sbins ? P.skeys + P.starts[size_t(kWork) * (P.n + 1) + i] : nullptr;
        tp[i].shade_seq = nullptr;
        // each volume its own run of bins, so the shading order groups volumes
        const uint32_t span = uint32_t(std::max(2, kBatchShadeBins / P.n));
        tp[i].bin_base = P.sbins ? uint32_t(i) * span : 0u;
        tp[i].bin_span = span;
        volume_blend_params(v, bp[i]);
        if (P.tc) {
            TcBlendParams t;
            volume_tc_params(v, t);
            tc_fill_jobs(t, P.tcp[i], host + P.off_tc + size_t(i) * P.tc_bytes);
        }
    }
}

// Launches one frame.
cudaError_t plan_launch(const Plan& P, uint8_t* d_args, const int* d_starts, cudaStream_t st) {
    const TraceParams* tp = reinterpret_cast<const TraceParams*>(d_args + P.off_trace);
    const BlendParams* bp = reinterpret_cast<const BlendParams*>(d_args + P.off_blend);
    const int n = P.n, n1 = P.n + 1;
    cudaError_t e = launch_raygen_batch(tp, d_starts + kRaygen * n1, n, P.blocks[kRaygen], st);
    if (e == cudaSuccess) e = launch_weights_batch(bp, d_starts + kWeights * n1, n, P.blocks[kWeights], st);
    if (e == cudaSuccess && P.sbins)
        e = cudaMemsetAsync(P.sbins, 0, sizeof(uint32_t) * kBatchShadeBins, st);
    if (e == cudaSuccess)
        e = launch_march_batch(tp, d_starts + kMarch * n1, n, P.blocks[kMarch], P.t.march_variant,
                               P.t.march_threads, P.sdf_format, P.q ? 1 : 0, P.qcount, st);
    if (P.sbins) {
        const int nb = std::max(2, kBatchShadeBins / n) * n;
        if (e == cudaSuccess) e = launch_bin_sort(P.sbins, nb, P.skeys, P.sseq, P.work, st);
        if (e == cudaSuccess)
            e = launch_shade_batch_sorted(tp, d_starts + kWork * n1, n, P.sseq, P.work, P.light_mode,
                                          P.t.shade_variant, st);
    } else if (e == cudaSuccess) {
        e = launch_shade_batch(tp, d_starts + kShade * n1, n, P.blocks[kShade], P.light_mode, P.t.shade_variant, st);
    }
    if (e == cudaSuccess && P.tc) e = launch_tc_pack_batch(tp, d_starts + kPack * n1, n, P.blocks[kPack], st);
    if (e != cudaSuccess) return e;
    if (!P.tc)
        return launch_blend_batch(bp, d_starts + kBlendI * n1, P.blocks[kBlendI], P.smem_i, d_starts + kBlendD * n1,
                                  P.blocks[kBlendD], P.smem_d, n, P.t.blend_probes, P.storage, st);
    // every volume's irradiance and distance blends: one persistent launch
    return launch_tc_blend_jobs(P.tcl, P.storage, d_args + P.off_tc, st);
}

int prepare_all(const Plan& P, cudaStream_t st) {
    for (luxgi_ddgi_volume* v : P.vols) {
        const int s = volume_prepare(v, st);
        if (s != LUXGI_OK) return s;
    }
    return LUXGI_OK;
}

void end_frame_all(const Plan& P) {
    for (luxgi_ddgi_volume* v : P.vols) {
        v->ping_pong = 1 - v->ping_pong;
        v->frames += 1;
    }
}

}  // namespace luxgi

namespace {

// One frame of a compatible group through direct batched launches, with
// transient stream-ordered device buffers.
int run_group(luxgi_ddgi_volume* const* vols, int n, const float* rots, cudaStream_t st) {
    luxgi_ddgi_batch_tuning t = default_tuning();
    t.march_variant = vols[0]->desc.march_variant;
    t.shade_variant = vols[0]->desc.shade_variant;
    t.march_budget = vols[0]->desc.march_budget;
    t.shade_order = vols[0]->desc.shade_order;
    t.use_graph = 0;
    Plan P;
    int s = plan_build(P, vols, n, t);
    if (s != LUXGI_OK) return s;
    s = prepare_all(P, st);
    if (s != LUXGI_OK) return s;
    std::vector<uint8_t> host(P.arg_bytes + P.starts.size() * sizeof(int));
    const size_t qoff = align16(host.size());
    uint8_t* dev = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&dev), qoff + plan_aux_bytes(P), st);
    if (e != cudaSuccess) return cuda_status(e);
    plan_set_aux(P, dev + qoff);
    plan_fill(P, rots, host.data());
    std::memcpy(host.data() + P.arg_bytes, P.starts.data(), P.starts.size() * sizeof(int));
    // pageable source: the copy has taken the bytes when the call returns
    e = cudaMemcpyAsync(dev, host.data(), host.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = plan_launch(P, dev, reinterpret_cast<const int*>(dev + P.arg_bytes), st);
    const cudaError_t e2 = cudaFreeAsync(dev, st);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return cuda_status(e);
    end_frame_all(P);
    return LUXGI_OK;
}

}  // namespace

struct luxgi_ddgi_batch {
    Plan plan;
    int device = 0;
    uint8_t* host[2] = {nullptr, nullptr};   // pinned per-frame argument blocks (double buffered)
    uint8_t* dev_args = nullptr;
    int* dev_starts = nullptr;
    void* dev_q = nullptr;                   // march compaction queues
    size_t dev_args_cap = 0, dev_starts_cap = 0, host_cap = 0, dev_q_cap = 0;
    cudaStream_t cap = nullptr;              // capture stream
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    uint64_t kernels_per_frame = 0;
    cudaEvent_t done[2] = {nullptr, nullptr};
    bool pending[2] = {false, false};
    uint64_t frame = 0;
};

namespace {

void drop_graphs(luxgi_ddgi_batch* b) {
    for (int k = 0; k < 2; ++k) {
        if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
        b->exec[k] = nullptr;
    }
}

// Waits for the frames still reading the pinned argument blocks.
cudaError_t drain(luxgi_ddgi_batch* b) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2; ++k) {
        if (b->pending[k]) {
            const cudaError_t e2 = cudaEventSynchronize(b->done[k]);
            if (e == cudaSuccess) e = e2;
            b->pending[k] = false;
        }
    }
    return e;
}

void release(luxgi_ddgi_batch* b) {
    drain(b);
    drop_graphs(b);
    for (int k = 0; k < 2; ++k) {
        if (b->host[k]) cudaFreeHost(b->host[k]);
        if (b->done[k]) cudaEventDestroy(b->done[k]);
    }
    if (b->dev_args) cudaFree(b->dev_args);
    if (b->dev_starts) cudaFree(b->dev_starts);
    if (b->dev_q) cudaFree(b->dev_q);
    if (b->cap) cudaStreamDestroy(b->cap);
}

// (Re)plans for tuning t: variants applied to the volumes, buffers grown,
// block tables uploaded, graphs dropped (captured again on next use).
int replan(luxgi_ddgi_batch* b, const luxgi_ddgi_batch_tuning& t) {
    cudaError_t e = drain(b);
    if (e != cudaSuccess) return cuda_status(e);
    drop_graphs(b);
    std::vector<luxgi_ddgi_volume*> vols = b->plan.vols;
    int s = apply_variants(vols.data(), int(vols.size()), t);
    if (s != LUXGI_OK) return s;
    s = plan_build(b->plan, vols.data(), int(vols.size()), t);
    if (s != LUXGI_OK) return s;
    const size_t qb = plan_aux_bytes(b->plan);
    if (qb > b->dev_q_cap) {
        if (b->dev_q) cudaFree(b->dev_q);
        b->dev_q = nullptr;
        b->dev_q_cap = 0;
        e = cudaMalloc(&b->dev_q, qb);
        if (e != cudaSuccess) return cuda_status(e);
        b->dev_q_cap = qb;
    }
    plan_set_aux(b->plan, b->dev_q);
    const Plan& P = b->plan;
    if (P.arg_bytes > b->host_cap) {
        for (int k = 0; k < 2; ++k) {
            if (b->host[k]) cudaFreeHost(b->host[k]);
            b->host[k] = nullptr;
        }
        b->host_cap = 0;
        for (int k = 0; k < 2; ++k) {
            e = cudaHostAlloc(reinterpret_cast<void**>(&b->host[k]), P.arg_bytes, cudaHostAllocDefault);
            if (e != cudaSuccess) return cuda_status(e);
        }
        b->host_cap = P.arg_bytes;
    }
    if (P.arg_bytes > b->dev_args_cap) {
        if (b->dev_args) cudaFree(b->dev_args);
        b->dev_args = nullptr;
        b->dev_args_cap = 0;
        e = cudaMalloc(reinterpret_cast<void**>(&b->dev_args), P.arg_bytes);
        if (e != cudaSuccess) return cuda_status(e);
        b->dev_args_cap = P.arg_bytes;
    }
    const size_t sb = P.starts.size() * sizeof(int);
    if (sb > b->dev_starts_cap) {
        if (b->dev_starts) cudaFree(b->dev_starts);
        b->dev_starts = nullptr;
        b->dev_starts_cap = 0;
        e = cudaMalloc(reinterpret_cast<void**>(&b->dev_starts), sb);
        if (e != cudaSuccess) return cuda_status(e);
        b->dev_starts_cap = sb;
    }
    e = cudaMemcpy(b->dev_starts, P.starts.data(), sb, cudaMemcpyHostToDevice);
    return cuda_status(e);
}

// Captures the frame that reads argument block k.
int capture(luxgi_ddgi_batch* b, int k) {
    const Plan& P = b->plan;
    const uint64_t before = luxgi_launch_count();
    cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_status(e);
    cudaError_t el = cudaMemcpyAsync(b->dev_args, b->host[k], P.arg_bytes, cudaMemcpyHostToDevice, b->cap);
    if (el == cudaSuccess) el = plan_launch(P, b->dev_args, b->dev_starts, b->cap);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->cap, &g);
    const uint64_t captured = luxgi_launch_count() - before;
    note_launch(-int(captured));                // counted again at every replay
    if (el != cudaSuccess || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_status(el != cudaSuccess ? el : e);
    }
    e = cudaGraphInstantiate(&b->exec[k], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        b->exec[k] = nullptr;
        return cuda_status(e);
    }
    b->kernels_per_frame = captured;
    return LUXGI_OK;
}

int batch_frame(luxgi_ddgi_batch* b, const float* rots, cudaStream_t st) {
    const Plan& P = b->plan;
    int s = compat_check(P.vols.data(), P.n);
    if (s != LUXGI_OK) return s;
    for (luxgi_ddgi_volume* v : P.vols)
        if (v->desc.march_variant != P.t.march_variant || v->desc.shade_variant != P.t.shade_variant)
            return LUXGI_EINVAL;   // a volume was retuned outside the batch
    s = prepare_all(P, st);
    if (s != LUXGI_OK) return s;
    const int k = int(b->frame & 1);
    cudaError_t e = cudaSuccess;
    if (b->pending[k]) {
        e = cudaEventSynchronize(b->done[k]);
        b->pending[k] = false;
        if (e != cudaSuccess) return cuda_status(e);
    }
    plan_fill(P, rots, b->host[k]);
    if (P.t.use_graph) {
        if (!b->exec[k]) {
            s = capture(b, k);
            if (s != LUXGI_OK) return s;
        }
        e = cudaGraphLaunch(b->exec[k], st);
        if (e == cudaSuccess) note_launch(int(b->kernels_per_frame));
    } else {
        e = cudaMemcpyAsync(b->dev_args, b->host[k], P.arg_bytes, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = plan_launch(P, b->dev_args, b->dev_starts, st);
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->done[k], st);
    if (e != cudaSuccess) return cuda_status(e);
    b->pending[k] = true;
    end_frame_all(P);
    b->frame += 1;
    return LUXGI_OK;
}

// Atlases, frame counts and ping-pong of every volume, kept on the device
// while the autotuner runs frames.
struct Snapshot {
    uint8_t* dev = nullptr;
    std::vector<int> frames, ping;
};

int snapshot_take(const Plan& P, Snapshot& S, cudaStream_t st) {
    size_t total = 0;
    for (const luxgi_ddgi_volume* v : P.vols) total += 2 * (v->irr_bytes + v->dist_bytes);
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&S.dev), total);
    if (e != cudaSuccess) return cuda_status(e);
    size_t o = 0;
    for (const luxgi_ddgi_volume* v : P.vols) {
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = cudaMemcpyAsync(S.dev + o, v->irr[k], v->irr_bytes, cudaMemcpyDeviceToDevice, st);
            o += v->irr_bytes;
            if (e == cudaSuccess) e = cudaMemcpyAsync(S.dev + o, v->dist[k], v->dist_bytes, cudaMemcpyDeviceToDevice, st);
            o += v->dist_bytes;
        }
        S.frames.push_back(v->frames);
        S.ping.push_back(v->ping_pong);
    }
    return cuda_status(e);
}

int snapshot_restore(const Plan& P, Snapshot& S, cudaStream_t st) {
    size_t o = 0;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < P.n; ++i) {
        luxgi_ddgi_volume* v = P.vols[i];
        for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
            e = cudaMemcpyAsync(v->irr[k], S.dev + o, v->irr_bytes, cudaMemcpyDeviceToDevice, st);
            o += v->irr_bytes;
            if (e == cudaSuccess) e = cudaMemcpyAsync(v->dist[k], S.dev + o, v->dist_bytes, cudaMemcpyDeviceToDevice, st);
            o += v->dist_bytes;
        }
        v->frames = S.frames[i];
        v->ping_pong = S.ping[i];
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(S.dev);
    S.dev = nullptr;
    return cuda_status(e);
}

// Mean frame time of `frames` frames after 2 warm-up frames, or a negative
// status when the candidate cannot run.
float time_candidate(luxgi_ddgi_batch* b, const luxgi_ddgi_batch_tuning& t, int frames, cudaStream_t st,
                     std::vector<float>& rots, int* status) {
    *status = replan(b, t);
    if (*status != LUXGI_OK) return -1.0f;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float ms = -1.0f;
    for (int f = 0; f < frames + 2; ++f) {
        for (int i = 0; i < b->plan.n; ++i) luxgi_ddgi_frame_rotation(0, uint32_t(f), rots.data() + 9 * i);
        if (f == 2) cudaEventRecord(t0, st);
        *status = batch_frame(b, rots.data(), st);
        if (*status != LUXGI_OK) break;
    }
    if (*status == LUXGI_OK) {
        cudaEventRecord(t1, st);
        const cudaError_t e = cudaEventSynchronize(t1);
        if (e == cudaSuccess && cudaEventElapsedTime(&ms, t0, t1) == cudaSuccess) ms /= float(frames);
        else *status = cuda_status(e);
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return *status == LUXGI_OK ? ms : -1.0f;
}

}  // namespace

extern "C" {

int luxgi_ddgi_update_batch(luxgi_ddgi_volume* const* vols, int n, const float* rots, void* stream) {
    if ((!vols && n > 0) || n < 0 || (!rots && n > 0)) return LUXGI_EINVAL;
    for (int i = 0; i < n; ++i) {
        if (!vols[i]) return LUXGI_EINVAL;
        for (int j = 0; j < i; ++j)
            if (vols[j] == vols[i]) return LUXGI_EINVAL;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // group volumes that can share launches (per-ray march variants 1-5,
    // 10 and 11); the pooled march variants and lone volumes take the
    // single-volume path
    std::vector<bool> done(size_t(n), false);
    for (int i = 0; i < n; ++i) {
        if (done[i]) continue;
        luxgi_ddgi_volume* a = vols[i];
        std::vector<luxgi_ddgi_volume*> grp{a};
        std::vector<float> grots(rots + 9 * i, rots + 9 * i + 9);
        done[i] = true;
        const int mv = a->desc.march_variant;
        if (a->bound && per_ray_variant(mv)) {
            for (int j = i + 1; j < n; ++j) {
                const luxgi_ddgi_volume* c = vols[j];
                if (done[j] || !c->bound || c->desc.march_variant != mv ||
                    c->desc.shade_variant != a->desc.shade_variant || c->desc.march_budget != a->desc.march_budget ||
                    c->desc.shade_order != a->desc.shade_order ||
                    c->desc.storage != a->desc.storage ||
                    c->desc.light_mode != a->desc.light_mode || c->tc != a->tc || c->sdf.format != a->sdf.format ||
                    c->device != a->device)
                    continue;
                grp.push_back(vols[j]);
                grots.insert(grots.end(), rots + 9 * j, rots + 9 * j + 9);
                done[j] = true;
            }
        }
        const int s = grp.size() > 1 ? run_group(grp.data(), int(grp.size()), grots.data(), st)
                                     : luxgi_ddgi_update(a, rots + 9 * i, stream);
        if (s != LUXGI_OK) return s;
    }
    return LUXGI_OK;
}

int luxgi_ddgi_batch_create(luxgi_ddgi_volume* const* vols, int n, const luxgi_ddgi_batch_tuning* tuning,
                            luxgi_ddgi_batch** out) {
    if (!out) return LUXGI_EINVAL;
    *out = nullptr;
    int s = compat_check(vols, n);
    if (s != LUXGI_OK) return s;
    const luxgi_ddgi_batch_tuning t = tuning ? *tuning : default_tuning();
    if (!tuning_valid(t)) return LUXGI_EINVAL;
    luxgi_ddgi_batch* b = new (std::nothrow) luxgi_ddgi_batch();
    if (!b) return LUXGI_ENOMEM;
    cudaGetDevice(&b->device);
    b->plan.vols.assign(vols, vols + n);
    cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaEventCreateWithFlags(&b->done[k], cudaEventDisableTiming);
    s = e == cudaSuccess ? replan(b, t) : cuda_status(e);
    if (s != LUXGI_OK) {
        release(b);
        delete b;
        return s;
    }
    *out = b;
    return LUXGI_OK;
}

int luxgi_ddgi_batch_update(luxgi_ddgi_batch* b, const float* rots, void* stream) {
    if (!b || !rots) return LUXGI_EINVAL;
    return batch_frame(b, rots, static_cast<cudaStream_t>(stream));
}

int luxgi_ddgi_batch_autotune(luxgi_ddgi_batch* b, int frames, void* stream, luxgi_ddgi_batch_tuning* best_out) {
    if (!b || frames < 1) return LUXGI_EINVAL;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = drain(b);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_status(e);
    const luxgi_ddgi_batch_tuning start = b->plan.t;
    Snapshot snap;
    int s = snapshot_take(b->plan, snap, st);
    if (s != LUXGI_OK) {
        if (snap.dev) cudaFree(snap.dev);
        return s;
    }
    std::vector<float> rots(size_t(9) * b->plan.n);
    luxgi_ddgi_batch_tuning best = start;
    float best_ms = -1.0f;
    auto consider = [&](const luxgi_ddgi_batch_tuning& c) {
        int cs = LUXGI_OK;
        const float ms = time_candidate(b, c, frames, st, rots, &cs);
        if (cs == LUXGI_OK && ms > 0.0f && (best_ms < 0.0f || ms < best_ms)) {
            best_ms = ms;
            best = c;
        }
        return cs;
    };
    // coordinate descent: march variant x rays per block, then the march
    // compaction budget, then shade variant, then the FP32 blend's probes
    // per thread
    for (int mv : {1, 2, 3, 4, 5, 10, 11}) {
        for (int tpb : {128, 256}) {
            luxgi_ddgi_batch_tuning c = best;
            c.march_variant = mv;
            c.march_threads = tpb;
            c.use_graph = 1;
            consider(c);
        }
    }
    for (int mb : {-1, 8, 12, 16}) {
        luxgi_ddgi_batch_tuning c = best;
        c.march_budget = mb;
        const int cur = best.march_budget == 0 ? kDefaultMarchBudget : best.march_budget;
        if (mb != cur) consider(c);
    }
    {
        luxgi_ddgi_batch_tuning c = best;
        c.shade_order = best.shade_order == 1 ? -1 : 1;
        consider(c);
    }
    for (int sv : {1, 2, 4}) {
        luxgi_ddgi_batch_tuning c = best;
        c.shade_variant = sv;
        if (c.shade_variant != best.shade_variant) consider(c);
    }
    if (!b->plan.tc) {
        for (int pb : {1, 2, 4}) {
            luxgi_ddgi_batch_tuning c = best;
            c.blend_probes = pb;
            if (c.blend_probes != best.blend_probes) consider(c);
        }
    }
    e = drain(b);
    s = snapshot_restore(b->plan, snap, st);
    if (e != cudaSuccess && s == LUXGI_OK) s = cuda_status(e);
    if (s != LUXGI_OK) return s;
    if (best_ms < 0.0f) {
        replan(b, start);
        return LUXGI_EUNSUPPORTED;
    }
    best.frame_ms = best_ms;
    s = replan(b, best);
    if (s != LUXGI_OK) return s;
    b->plan.t.frame_ms = best_ms;
    if (best_out) *best_out = best;
    return LUXGI_OK;
}

int luxgi_ddgi_batch_get_tuning(const luxgi_ddgi_batch* b, luxgi_ddgi_batch_tuning* out) {
    if (!b || !out) return LUXGI_EINVAL;
    *out = b->plan.t;
    return LUXGI_OK;
}

int luxgi_ddgi_batch_set_tuning(luxgi_ddgi_batch* b, const luxgi_ddgi_batch_tuning* t) {
    if (!b || !t || !tuning_valid(*t)) return LUXGI_EINVAL;
    return replan(b, *t);
}

int luxgi_ddgi_batch_destroy(luxgi_ddgi_batch* b) {
    if (!b) return LUXGI_EINVAL;
    release(b);
    delete b;
    return LUXGI_OK;
}

}  // extern "C"
