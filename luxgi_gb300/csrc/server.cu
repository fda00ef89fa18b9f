// Serving loop over many DDGI volumes (include/luxgi_serve.h).
//
// One scheduler thread per server owns every CUDA call of the serving
// path.  Callers only queue requests (under the server mutex) and read
// counters.  Each scheduler pass
//   1. retires launch groups whose completion event fired (latency is taken
//      here, on the host clock, against the request's submit time);
//   2. while a stream slot is free: picks the sessions whose oldest pending
//      request is oldest (at most one request per session in flight, all of
//      one kind so they share batched launches), admitting sessions that
//      are not resident -- evicting least recently used idle sessions while
//      the budget is short -- and issues the group on the free slot;
//   3. sleeps until a submission or a short poll interval.
// The policy (steps 1-2) is the same for both executors; only admit /
// evict / launch / poll differ.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <random>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "luxgi_batch.h"
#include "luxgi_serve.h"

using namespace luxgi;

namespace {

using Clock = std::chrono::steady_clock;

double seconds_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

struct Request {
    uint64_t ticket = 0;
    int32_t session = 0;
    float rot[9] = {};
    Clock::time_point t_submit;
};

struct Session {
    int32_t id = 0;
    luxgi_ddgi_volume_desc vdesc{};
    luxgi_session_scene scene{};
    uint64_t bytes = 0;            // resident footprint
    uint64_t key = 0;              // launch-compatibility class
    bool resident = false;
    bool busy = false;             // a request of this session is in flight
    bool transit = false;          // being admitted or evicted while the lock
                                   // is released: no other thread schedules,
                                   // evicts or admits it meanwhile
    uint64_t lru = 0;
    int32_t frames = 0;
    uint64_t submitted = 0;        // requests submitted (rotation index of run_poisson)
    std::deque<Request> queue;
    // CUDA executor state
    luxgi_ddgi_volume* vol = nullptr;
    void* d_sdf = nullptr;
    void* d_mip = nullptr;
    luxgi_surface_object* d_objects = nullptr;
    luxgi_surface_tile* d_tiles = nullptr;
    uint32_t* d_chunks = nullptr;
    uint32_t* d_culled = nullptr;
    float* d_depth = nullptr;
    void* d_direct = nullptr;
    uint8_t* d_albedo = nullptr;
    void* d_light = nullptr;
    luxgi_sdf_desc sdf_dev{};
    luxgi_surface_desc surf_dev{};
    // state saved at eviction
    std::vector<uint8_t> saved_irr, saved_dist;
    bool saved = false;
};

struct Slot {
    bool busy = false;
    // CUDA executor
    cudaStream_t st = nullptr;
    cudaEvent_t ev = nullptr;
    uint8_t* host = nullptr;       // pinned staging of the launch arguments
    size_t hcap = 0;
    uint8_t* dev = nullptr;        // device arguments and per-ray buffers
    size_t cap = 0;
    // group in flight
    std::vector<Request> reqs;
    uint64_t probe_rays = 0;
    double sim_done = 0.0;         // SIM: completion time (s since server start)
};

uint64_t sdf_elems(const luxgi_sdf_desc& s, bool mip) {
    const uint64_t r = uint64_t(mip ? s.mip_resolution : s.resolution);
    return r * r * r * s.data.cascades_count;
}

uint64_t cull_capacity(const luxgi_surface_desc& s) {
    return s.data.culled_objects_capacity ? s.data.culled_objects_capacity
                                          : 1 + 40ull * 40 * 40 * (uint64_t(s.data.objects_count) + 1);
}

// bytes a texel of the scene's surface colour textures
uint64_t color_bytes(const luxgi_session_scene& sc) {
    return sc.surface.light_format == LUXGI_COLOR_R11G11B10F ? 4 : 8;
}

uint64_t scene_bytes(const luxgi_session_scene& sc, int light_mode) {
    const uint64_t esz = sc.sdf.format == LUXGI_STORAGE_FP16 ? 2 : 4;
    const uint64_t A2 = uint64_t(sc.atlas_resolution) * sc.atlas_resolution;
    const uint64_t cb = color_bytes(sc);
    uint64_t b = esz * (sdf_elems(sc.sdf, false) + sdf_elems(sc.sdf, true));
    b += sizeof(luxgi_surface_object) * uint64_t(sc.surface.num_objects);
    b += sizeof(luxgi_surface_tile) * uint64_t(sc.surface.num_tiles);
    b += 4 * (40ull * 40 * 40 + cull_capacity(sc.surface));
    b += A2 * (4 + cb + 4);                         // depth, direct light, albedo
    if (light_mode == LUXGI_LIGHT_CACHE) b += A2 * cb;
    return b;
}

luxgi_ddgi_batch_tuning server_tuning(const luxgi_server_desc& d) {
    luxgi_ddgi_batch_tuning t = default_tuning();
    if (d.tuning.march_variant) t.march_variant = d.tuning.march_variant;
    if (d.tuning.march_threads) t.march_threads = d.tuning.march_threads;
    if (d.tuning.shade_variant) t.shade_variant = d.tuning.shade_variant;
    if (d.tuning.blend_probes) t.blend_probes = d.tuning.blend_probes;
    t.march_budget = d.tuning.march_budget;
    t.shade_order = d.tuning.shade_order;
    t.use_graph = 0;
    return t;
}

}  // namespace

struct luxgi_server {
    luxgi_server_desc desc{};
    luxgi_ddgi_batch_tuning tuning{};
    bool sim = false;
    int device = 0;
    Clock::time_point t0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    std::thread worker;
    std::vector<std::unique_ptr<Session>> sessions;
    std::vector<Slot> slots;
    cudaStream_t adm = nullptr;                // admission copies and set-up
    int first_error = LUXGI_OK;
    uint64_t next_ticket = 1, lru_clock = 0;
    // counters (under mu)
    uint64_t submitted = 0, completed = 0, pending = 0, inflight = 0;
    uint64_t admissions = 0, evictions = 0, rejected = 0;
    uint64_t resident_sessions = 0, resident_bytes = 0, peak_resident_bytes = 0;
    uint64_t groups = 0, probe_rays = 0, max_overlap = 0, grouped_requests = 0;
    std::vector<double> latencies_ms;
    bool have_first = false;
    Clock::time_point t_first_submit, t_last_done;
};

namespace {

double now_s(const luxgi_server* s) { return seconds_since(s->t0, Clock::now()); }

// ------------------------------------------------------------ CUDA executor
template <typename T> cudaError_t dalloc(T** p, uint64_t bytes) {
    *p = nullptr;
    return bytes ? cudaMalloc(reinterpret_cast<void**>(p), bytes) : cudaSuccess;
}

void free_device(Session& ss) {
    if (ss.vol) luxgi_ddgi_destroy(ss.vol);
    ss.vol = nullptr;
    void* ptrs[] = {ss.d_sdf, ss.d_mip, ss.d_objects, ss.d_tiles, ss.d_chunks, ss.d_culled,
                    ss.d_depth, ss.d_direct, ss.d_albedo, ss.d_light};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    ss.d_sdf = ss.d_mip = ss.d_light = nullptr;
    ss.d_objects = nullptr;
    ss.d_tiles = nullptr;
    ss.d_chunks = ss.d_culled = nullptr;
    ss.d_depth = nullptr;
    ss.d_direct = nullptr;
    ss.d_albedo = nullptr;
}

int cuda_admit(luxgi_server* S, Session& ss) {
    const luxgi_session_scene& sc = ss.scene;
    const uint64_t esz = sc.sdf.format == LUXGI_STORAGE_FP16 ? 2 : 4;
    const uint64_t A2 = uint64_t(sc.atlas_resolution) * sc.atlas_resolution;
    const uint64_t cap = cull_capacity(sc.surface);
    cudaStream_t st = S->adm;
    cudaError_t e = dalloc(&ss.d_sdf, esz * sdf_elems(sc.sdf, false));
    if (e == cudaSuccess) e = dalloc(&ss.d_mip, esz * sdf_elems(sc.sdf, true));
    if (e == cudaSuccess) e = dalloc(&ss.d_objects, sizeof(luxgi_surface_object) * uint64_t(sc.surface.num_objects));
    if (e == cudaSuccess) e = dalloc(&ss.d_tiles, sizeof(luxgi_surface_tile) * uint64_t(sc.surface.num_tiles));
    if (e == cudaSuccess) e = dalloc(&ss.d_chunks, 4ull * 40 * 40 * 40);
    if (e == cudaSuccess) e = dalloc(&ss.d_culled, 4 * cap);
    if (e == cudaSuccess) e = dalloc(&ss.d_depth, 4 * A2);
    const uint64_t cb = color_bytes(sc);
    if (e == cudaSuccess) e = dalloc(&ss.d_direct, cb * A2);
    if (e == cudaSuccess) e = dalloc(&ss.d_albedo, 4 * A2);
    if (e == cudaSuccess && ss.vdesc.light_mode == LUXGI_LIGHT_CACHE) e = dalloc(&ss.d_light, cb * A2);
    auto up = [&](void* dst, const void* src, uint64_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st);
    };
    up(ss.d_sdf, sc.sdf.sdf, esz * sdf_elems(sc.sdf, false));
    up(ss.d_objects, sc.surface.objects, sizeof(luxgi_surface_object) * uint64_t(sc.surface.num_objects));
    up(ss.d_tiles, sc.surface.tiles, sizeof(luxgi_surface_tile) * uint64_t(sc.surface.num_tiles));
    up(ss.d_depth, sc.surface.depth, 4 * A2);
    up(ss.d_direct, sc.surface.direct_light, cb * A2);
    up(ss.d_albedo, sc.surface.albedo, 4 * A2);
    if (ss.d_light) up(ss.d_light, sc.surface.light_cache ? sc.surface.light_cache : sc.surface.direct_light, cb * A2);
    if (e != cudaSuccess) {
        free_device(ss);
        return cuda_status(e);
    }
    ss.sdf_dev = sc.sdf;
    ss.sdf_dev.sdf = ss.d_sdf;
    ss.sdf_dev.mip = ss.d_mip;
    void* tmp = nullptr;
    e = dalloc(&tmp, esz * uint64_t(sc.sdf.mip_resolution) * sc.sdf.mip_resolution * sc.sdf.mip_resolution);
    int s = e == cudaSuccess ? luxgi_sdf_build_mip(&ss.sdf_dev, ss.d_mip, tmp, st) : cuda_status(e);
    if (s == LUXGI_OK) s = cuda_status(cudaStreamSynchronize(st));
    if (tmp) cudaFree(tmp);
    ss.surf_dev = sc.surface;
    ss.surf_dev.data.culled_objects_capacity = uint32_t(cap);
    ss.surf_dev.objects = ss.d_objects;
    ss.surf_dev.tiles = ss.d_tiles;
    ss.surf_dev.chunks = ss.d_chunks;
    ss.surf_dev.culled_objects = ss.d_culled;
    ss.surf_dev.depth = ss.d_depth;
    ss.surf_dev.direct_light = ss.d_direct;
    ss.surf_dev.albedo = ss.d_albedo;
    ss.surf_dev.light_cache = ss.d_light;
    ss.surf_dev.gbuffer0 = nullptr;
    ss.surf_dev.gbuffer1 = nullptr;
    ss.surf_dev.gbuffer_format = LUXGI_GBUFFER_RGBA32F;    // G-buffers are not used by sessions
    if (s == LUXGI_OK) s = luxgi_surface_cull(&ss.surf_dev, ss.d_chunks, ss.d_culled, uint32_t(cap), st);
    luxgi_ddgi_volume_desc vd = ss.vdesc;
    vd.march_variant = S->tuning.march_variant;
    vd.shade_variant = S->tuning.shade_variant;
    if (s == LUXGI_OK) s = luxgi_ddgi_create(&vd, &ss.vol);
    if (s == LUXGI_OK) s = luxgi_ddgi_bind_scene(ss.vol, &ss.sdf_dev, &ss.surf_dev);
    if (s == LUXGI_OK && ss.saved)
        s = luxgi_ddgi_load_atlases(ss.vol, ss.saved_irr.data(), ss.saved_dist.data(), ss.frames, st);
    if (s == LUXGI_OK) s = volume_prepare(ss.vol, st);
    if (s == LUXGI_OK) s = cuda_status(cudaStreamSynchronize(st));
    if (s != LUXGI_OK) {
        free_device(ss);
        return s;
    }
    ss.saved = false;
    std::vector<uint8_t>().swap(ss.saved_irr);
    std::vector<uint8_t>().swap(ss.saved_dist);
    return LUXGI_OK;
}

int cuda_evict(luxgi_server* S, Session& ss) {
    luxgi_ddgi_atlases a;
    int s = luxgi_ddgi_get_atlases(ss.vol, &a);
    if (s != LUXGI_OK) return s;
    const uint64_t ae = a.storage == LUXGI_STORAGE_FP16 ? 2 : 4;
    ss.saved_irr.resize(uint64_t(a.irradiance_width) * a.irradiance_height * 4 * ae);
    ss.saved_dist.resize(uint64_t(a.depth_width) * a.depth_height * 2 * ae);
    cudaError_t e = cudaMemcpyAsync(ss.saved_irr.data(), a.irradiance, ss.saved_irr.size(), cudaMemcpyDeviceToHost,
                                    S->adm);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ss.saved_dist.data(), a.distance, ss.saved_dist.size(), cudaMemcpyDeviceToHost, S->adm);
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->adm);
    if (e != cudaSuccess) return cuda_status(e);
    ss.frames = a.frames;
    ss.saved = true;
    free_device(ss);
    return LUXGI_OK;
}

int cuda_launch(luxgi_server* S, Slot& sl, const std::vector<Session*>& members) {
    std::vector<luxgi_ddgi_volume*> vols;
    std::vector<float> rots;
    for (size_t i = 0; i < members.size(); ++i) {
        vols.push_back(members[i]->vol);
        rots.insert(rots.end(), sl.reqs[i].rot, sl.reqs[i].rot + 9);
    }
    Plan P;
    int s = plan_build(P, vols.data(), int(vols.size()), S->tuning);
    if (s != LUXGI_OK) return s;
    const size_t sb = P.starts.size() * sizeof(int);
    const size_t qoff = (P.arg_bytes + sb + 15) & ~size_t(15);
    const size_t need = qoff + plan_aux_bytes(P);
    // The slot's buffers grow geometrically.  The pinned staging holds the
    // arguments alone (a few KB a volume); the device buffer, which also
    // holds the per-ray buffers (hundreds of MB for a group of large
    // volumes), is stream-ordered on the slot's stream, so growing it
    // neither waits for the other slots' groups nor synchronises the device
    // (a pinned allocation of that size stalled the whole server for
    // ~0.2 s).  The slot is reused only after its previous group retired.
    const size_t hneed = P.arg_bytes + sb;
    if (hneed > sl.hcap) {
        if (sl.host) cudaFreeHost(sl.host);
        sl.host = nullptr;
        sl.hcap = 0;
        const cudaError_t e = cudaHostAlloc(reinterpret_cast<void**>(&sl.host), hneed * 2, cudaHostAllocDefault);
        if (e != cudaSuccess) return cuda_status(e);
        sl.hcap = hneed * 2;
    }
    if (need > sl.cap) {
        if (sl.dev) cudaFreeAsync(sl.dev, sl.st);
        sl.dev = nullptr;
        sl.cap = 0;
        const cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&sl.dev), need * 2, sl.st);
        if (e != cudaSuccess) return cuda_status(e);
        sl.cap = need * 2;
    }
    s = prepare_all(P, sl.st);
    if (s != LUXGI_OK) return s;
    plan_set_aux(P, sl.dev + qoff);
    plan_fill(P, rots.data(), sl.host);
    std::memcpy(sl.host + P.arg_bytes, P.starts.data(), sb);
    cudaError_t e = cudaMemcpyAsync(sl.dev, sl.host, P.arg_bytes + sb, cudaMemcpyHostToDevice, sl.st);
    if (e == cudaSuccess) e = plan_launch(P, sl.dev, reinterpret_cast<const int*>(sl.dev + P.arg_bytes), sl.st);
    if (e == cudaSuccess) e = cudaEventRecord(sl.ev, sl.st);
    if (e != cudaSuccess) return cuda_status(e);
    end_frame_all(P);
    return LUXGI_OK;
}

// ------------------------------------------------------------------ policy
// Frees budget for `need` bytes by evicting idle resident sessions, those
// with nothing pending first, least recently used first.  Caller holds mu.
// The eviction copy runs with mu released; the victim is marked in transit
// first, so that meanwhile no group is issued on it and no other caller
// picks it again.  An eviction that fails leaves the victim resident (its
// device state intact, its bytes still counted) and returns false.
bool make_room(luxgi_server* S, uint64_t need, const std::vector<Session*>& keep, std::unique_lock<std::mutex>& lk) {
    while (S->resident_bytes + need > S->desc.memory_budget) {
        Session* victim = nullptr;
        for (auto& up : S->sessions) {
            Session* c = up.get();
            if (!c->resident || c->busy || c->transit) continue;
            if (std::find(keep.begin(), keep.end(), c) != keep.end()) continue;
            if (!victim || std::make_pair(!c->queue.empty(), c->lru) < std::make_pair(!victim->queue.empty(), victim->lru))
                victim = c;
        }
        if (!victim) return false;
        int s = LUXGI_OK;
        victim->transit = true;
        if (!S->sim) {
            lk.unlock();
            s = cuda_evict(S, *victim);
            lk.lock();
        } else {
            if (S->desc.sim_evict_s > 0.0f) {
                // the modelled eviction copy, with the lock released like
                // the device copy above
                lk.unlock();
                std::this_thread::sleep_for(std::chrono::duration<double>(S->desc.sim_evict_s));
                lk.lock();
            }
            victim->saved = true;
        }
        victim->transit = false;
        S->cv_done.notify_all();
        if (s != LUXGI_OK) {
            if (S->first_error == LUXGI_OK) S->first_error = s;
            return false;
        }
        victim->resident = false;
        S->resident_bytes -= victim->bytes;
        S->resident_sessions -= 1;
        S->evictions += 1;
    }
    return true;
}

void retire(luxgi_server* S, Slot& sl, int status) {
    // caller holds mu
    const Clock::time_point t = Clock::now();
    for (const Request& r : sl.reqs) {
        Session* ss = S->sessions[size_t(r.session)].get();
        ss->busy = false;
        ss->lru = ++S->lru_clock;
        S->latencies_ms.push_back(std::chrono::duration<double, std::milli>(t - r.t_submit).count());
        S->completed += 1;
    }
    if (status != LUXGI_OK && S->first_error == LUXGI_OK) S->first_error = status;
    S->probe_rays += sl.probe_rays;
    S->t_last_done = t;
    S->inflight -= 1;
    sl.reqs.clear();
    sl.busy = false;
}

void scheduler(luxgi_server* S) {
    if (!S->sim) cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    for (;;) {
        // 1. retire finished groups
        bool progressed = false;
        for (Slot& sl : S->slots) {
            if (!sl.busy) continue;
            bool done;
            int status = LUXGI_OK;
            if (S->sim) {
                done = S->stop || now_s(S) >= sl.sim_done;   // modelled work ends at once on stop
            } else {
                const cudaError_t q = cudaEventQuery(sl.ev);
                done = q != cudaErrorNotReady;
                if (done && q != cudaSuccess) status = cuda_status(q);
            }
            if (done) {
                retire(S, sl, status);
                progressed = true;
            }
        }
        if (progressed) S->cv_done.notify_all();
        if (S->stop && S->inflight == 0) break;
        // 2. issue groups on free slots
        for (Slot& sl : S->slots) {
            if (sl.busy || S->stop) continue;
            std::vector<Session*> cand;
            for (auto& up : S->sessions)
                if (!up->busy && !up->transit && !up->queue.empty()) cand.push_back(up.get());
            if (cand.empty()) break;
            std::sort(cand.begin(), cand.end(),
                      [](const Session* a, const Session* b) { return a->queue.front().ticket < b->queue.front().ticket; });
            const uint64_t key = cand.front()->key;
            std::vector<Session*> members;
            double admit_s = 0.0;
            const size_t max_group = size_t(S->desc.max_group);
            for (Session* c : cand) {
                if (members.size() >= max_group) break;
                // (transit re-checked: admissions above release the lock, and
                // a touch that started earlier may have claimed c meanwhile)
                if (c->key != key || c->transit) continue;
                if (!c->resident) {
                    if (!make_room(S, c->bytes, members, lk)) continue;   // wait for memory
                    int s = LUXGI_OK;
                    if (!S->sim) {
                        c->transit = true;
                        lk.unlock();
                        s = cuda_admit(S, *c);
                        lk.lock();
                        c->transit = false;
                        S->cv_done.notify_all();
                    } else {
                        admit_s += S->desc.sim_admit_s;
                    }
                    if (s != LUXGI_OK) {
                        if (S->first_error == LUXGI_OK) S->first_error = s;
                        // drop the session's requests so that drain ends
                        S->completed += c->queue.size();
                        S->pending -= c->queue.size();
                        c->queue.clear();
                        continue;
                    }
                    c->resident = true;
                    S->resident_bytes += c->bytes;
                    S->resident_sessions += 1;
                    S->peak_resident_bytes = std::max(S->peak_resident_bytes, S->resident_bytes);
                    S->admissions += 1;
                }
                members.push_back(c);
            }
            if (members.empty()) break;
            sl.reqs.clear();
            sl.probe_rays = 0;
            for (Session* c : members) {
                sl.reqs.push_back(c->queue.front());
                c->queue.pop_front();
                c->busy = true;
                c->lru = ++S->lru_clock;
                c->frames += 1;
                const luxgi_ddgi_uniform& u = c->vdesc.uniform;
                sl.probe_rays += uint64_t(u.probe_counts[0]) * u.probe_counts[1] * u.probe_counts[2] * u.rays_per_probe;
            }
            S->pending -= members.size();
            sl.busy = true;
            S->inflight += 1;
            S->groups += 1;
            S->grouped_requests += members.size();
            S->max_overlap = std::max(S->max_overlap, S->inflight);
            int s = LUXGI_OK;
            if (S->sim) {
                sl.sim_done = now_s(S) + admit_s + double(sl.probe_rays) / S->desc.sim_rate;
            } else {
                lk.unlock();
                s = cuda_launch(S, sl, members);
                lk.lock();
            }
            if (s != LUXGI_OK) {
                if (!S->sim) cudaStreamSynchronize(sl.st);
                retire(S, sl, s);
                S->cv_done.notify_all();
            }
        }
        // 3. wait for work
        if (S->inflight == 0 && S->pending == 0 && !S->stop) {
            S->cv_work.wait(lk);
        } else {
            S->cv_work.wait_for(lk, std::chrono::microseconds(40));
        }
    }
}

int check_scene(const luxgi_session_scene* sc, int light_mode) {
    if (!sc || !sc->sdf.sdf || !sc->surface.objects || !sc->surface.tiles || !sc->surface.depth ||
        !sc->surface.direct_light || !sc->surface.albedo || sc->atlas_resolution <= 0)
        return LUXGI_EINVAL;
    const int C = int(sc->sdf.data.cascades_count);
    if (C < 1 || C > 4 || sc->sdf.resolution < 4 || sc->sdf.resolution % 4 != 0 ||
        sc->sdf.mip_resolution != sc->sdf.resolution / 4 || sc->sdf.resolution != int(sc->sdf.data.resolution))
        return LUXGI_EINVAL;
    if (sc->sdf.format != LUXGI_STORAGE_FP32 && sc->sdf.format != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    if (sc->surface.light_format != LUXGI_COLOR_RGBA16F && sc->surface.light_format != LUXGI_COLOR_R11G11B10F)
        return LUXGI_EINVAL;
    if (sc->surface.num_objects < 0 || sc->surface.num_tiles < 1 ||
        uint32_t(sc->surface.num_objects) != sc->surface.data.objects_count)
        return LUXGI_EINVAL;
    (void)light_mode;
    return LUXGI_OK;
}

int check_volume(const luxgi_ddgi_volume_desc* d) {
    if (!d) return LUXGI_EINVAL;
    luxgi_ddgi_uniform u = d->uniform;
    const int s = luxgi_ddgi_derive_uniform(&u);
    if (s != LUXGI_OK) return s;
    if (u.irradiance_width != d->uniform.irradiance_width || u.depth_height != d->uniform.depth_height)
        return LUXGI_EINVAL;
    if (d->storage != LUXGI_STORAGE_FP32 && d->storage != LUXGI_STORAGE_FP16) return LUXGI_EINVAL;
    if (d->light_mode != LUXGI_LIGHT_CACHE && d->light_mode != LUXGI_LIGHT_PER_HIT) return LUXGI_EINVAL;
    if (d->blend != LUXGI_BLEND_FP32 && d->blend != LUXGI_BLEND_TENSOR) return LUXGI_EINVAL;
    if (d->max_steps < 1) return LUXGI_EINVAL;
    return LUXGI_OK;
}

}  // namespace

extern "C" {

int luxgi_server_create(const luxgi_server_desc* desc, luxgi_server** out) {
    if (!desc || !out) return LUXGI_EINVAL;
    *out = nullptr;
    if (desc->executor != LUXGI_SERVE_EXEC_CUDA && desc->executor != LUXGI_SERVE_EXEC_SIM) return LUXGI_EINVAL;
    if (desc->max_group < 0 || desc->max_inflight < 0 || desc->max_inflight > 16 || desc->sim_rate < 0.0 ||
        desc->sim_admit_s < 0.0 || !(desc->sim_evict_s >= 0.0f) || desc->sim_evict_s > 60.0f)
        return LUXGI_EINVAL;
    luxgi_server* S = new (std::nothrow) luxgi_server();
    if (!S) return LUXGI_ENOMEM;
    S->desc = *desc;
    if (S->desc.max_group == 0) S->desc.max_group = 64;
    if (S->desc.max_inflight == 0) S->desc.max_inflight = 3;
    if (S->desc.sim_rate == 0.0) S->desc.sim_rate = 1e9;
    S->tuning = server_tuning(S->desc);
    if (!tuning_valid(S->tuning)) {
        delete S;
        return LUXGI_EINVAL;
    }
    S->sim = desc->executor == LUXGI_SERVE_EXEC_SIM;
    S->t0 = Clock::now();
    S->slots.resize(size_t(S->desc.max_inflight));
    if (!S->sim) {
        cudaGetDevice(&S->device);
        cudaError_t e = cudaStreamCreateWithFlags(&S->adm, cudaStreamNonBlocking);
        for (Slot& sl : S->slots) {
            if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming);
        }
        if (e != cudaSuccess) {
            for (Slot& sl : S->slots) {
                if (sl.st) cudaStreamDestroy(sl.st);
                if (sl.ev) cudaEventDestroy(sl.ev);
            }
            if (S->adm) cudaStreamDestroy(S->adm);
            delete S;
            return cuda_status(e);
        }
    }
    S->worker = std::thread(scheduler, S);
    *out = S;
    return LUXGI_OK;
}

int luxgi_server_destroy(luxgi_server* S) {
    if (!S) return LUXGI_EINVAL;
    {
        std::lock_guard<std::mutex> g(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    S->worker.join();
    if (!S->sim) {
        for (auto& up : S->sessions) free_device(*up);
        for (Slot& sl : S->slots) {
            if (sl.host) cudaFreeHost(sl.host);
            if (sl.dev) cudaFree(sl.dev);
            cudaStreamDestroy(sl.st);
            cudaEventDestroy(sl.ev);
        }
        cudaStreamDestroy(S->adm);
    }
    delete S;
    return LUXGI_OK;
}

int luxgi_server_add_session(luxgi_server* S, const luxgi_ddgi_volume_desc* volume, const luxgi_session_scene* scene,
                             int32_t* session_id) {
    if (!S || !session_id) return LUXGI_EINVAL;
    int s = check_volume(volume);
    if (s == LUXGI_OK) s = check_scene(scene, volume->light_mode);
    if (s != LUXGI_OK) return s;
    std::unique_ptr<Session> ss(new (std::nothrow) Session());
    if (!ss) return LUXGI_ENOMEM;
    ss->vdesc = *volume;
    ss->vdesc.march_variant = S->tuning.march_variant;
    ss->vdesc.shade_variant = S->tuning.shade_variant;
    ss->scene = *scene;
    luxgi_surface_desc surf = scene->surface;
    surf.data.culled_objects_capacity = uint32_t(cull_capacity(scene->surface));
    ss->bytes = scene_bytes(*scene, volume->light_mode) + volume_device_bytes(ss->vdesc, scene->sdf, surf);
    ss->key = uint64_t(volume->storage) | uint64_t(volume->light_mode) << 8 | uint64_t(volume->blend) << 16 |
              uint64_t(scene->sdf.format) << 24;
    std::lock_guard<std::mutex> g(S->mu);
    if (ss->bytes > S->desc.memory_budget) {
        S->rejected += 1;
        return LUXGI_ENOMEM;
    }
    ss->id = int32_t(S->sessions.size());
    *session_id = ss->id;
    S->sessions.push_back(std::move(ss));
    return LUXGI_OK;
}

int luxgi_server_session_bytes(luxgi_server* S, int32_t id, uint64_t* bytes) {
    if (!S || !bytes) return LUXGI_EINVAL;
    std::lock_guard<std::mutex> g(S->mu);
    if (id < 0 || size_t(id) >= S->sessions.size()) return LUXGI_EINVAL;
    *bytes = S->sessions[size_t(id)]->bytes;
    return LUXGI_OK;
}

int luxgi_server_submit(luxgi_server* S, int32_t id, const float rot[9], uint64_t* ticket) {
    if (!S || !rot) return LUXGI_EINVAL;
    {
        std::lock_guard<std::mutex> g(S->mu);
        if (id < 0 || size_t(id) >= S->sessions.size() || S->stop) return LUXGI_EINVAL;
        Request r;
        r.ticket = S->next_ticket++;
        r.session = id;
        std::memcpy(r.rot, rot, sizeof(r.rot));
        r.t_submit = Clock::now();
        if (!S->have_first) {
            S->have_first = true;
            S->t_first_submit = r.t_submit;
        }
        Session* ss = S->sessions[size_t(id)].get();
        ss->queue.push_back(r);
        ss->submitted += 1;
        S->submitted += 1;
        S->pending += 1;
        if (ticket) *ticket = r.ticket;
    }
    S->cv_work.notify_one();
    return LUXGI_OK;
}

int luxgi_server_drain(luxgi_server* S, double timeout_s) {
    if (!S) return LUXGI_EINVAL;
    std::unique_lock<std::mutex> lk(S->mu);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(
                                          timeout_s > 0.0 ? timeout_s : 1e9));
    while (S->completed < S->submitted) {
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout && S->completed < S->submitted)
            return LUXGI_ETIMEOUT;
    }
    return S->first_error;
}

int luxgi_server_run_poisson(luxgi_server* S, const int32_t* ids, int n, double rate, double seconds,
                             uint64_t seed) {
    if (!S || !ids || n < 1 || !(rate > 0.0) || !(seconds > 0.0)) return LUXGI_EINVAL;
    std::mt19937_64 rng(seed);
    std::exponential_distribution<double> gap(rate);
    std::uniform_int_distribution<int> pick(0, n - 1);
    const Clock::time_point start = Clock::now();
    double t = 0.0;
    for (;;) {
        t += gap(rng);
        if (t >= seconds) break;
        const Clock::time_point due = start + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t));
        for (;;) {
            const auto left = due - Clock::now();
            if (left <= Clock::duration::zero()) break;
            if (left > std::chrono::microseconds(300)) std::this_thread::sleep_for(left - std::chrono::microseconds(200));
            else std::this_thread::yield();
        }
        const int32_t id = ids[pick(rng)];
        uint64_t k = 0;
        {
            std::lock_guard<std::mutex> g(S->mu);
            if (id < 0 || size_t(id) >= S->sessions.size()) return LUXGI_EINVAL;
            k = S->sessions[size_t(id)]->submitted;
        }
        float rot[9];
        luxgi_ddgi_frame_rotation(uint64_t(id), uint32_t(k), rot);
        const int s = luxgi_server_submit(S, id, rot, nullptr);
        if (s != LUXGI_OK) return s;
    }
    return luxgi_server_drain(S, 0.0);
}

int luxgi_server_stats_get(luxgi_server* S, luxgi_server_stats* out, int reset) {
    if (!S || !out) return LUXGI_EINVAL;
    std::lock_guard<std::mutex> g(S->mu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->pending = S->pending;
    out->inflight_groups = S->inflight;
    out->admissions = S->admissions;
    out->evictions = S->evictions;
    out->rejected = S->rejected;
    out->resident_sessions = S->resident_sessions;
    out->resident_bytes = S->resident_bytes;
    out->peak_resident_bytes = S->peak_resident_bytes;
    out->groups = S->groups;
    out->probe_rays = S->probe_rays;
    out->max_overlap = S->max_overlap;
    out->mean_group = S->groups ? double(S->grouped_requests) / double(S->groups) : 0.0;
    std::vector<double> v = S->latencies_ms;
    if (!v.empty()) {
        auto q = [&](double f) {
            const size_t k = std::min(v.size() - 1, size_t(std::ceil(f * double(v.size())) - 1));
            std::nth_element(v.begin(), v.begin() + std::ptrdiff_t(k), v.end());
            return v[k];
        };
        double sum = 0.0, mx = 0.0;
        for (double x : v) {
            sum += x;
            mx = std::max(mx, x);
        }
        out->latency_ms_mean = sum / double(v.size());
        out->latency_ms_max = mx;
        out->latency_ms_p50 = q(0.50);
        out->latency_ms_p95 = q(0.95);
        out->latency_ms_p99 = q(0.99);
    }
    if (S->have_first && S->completed > 0) out->wall_s = seconds_since(S->t_first_submit, S->t_last_done);
    if (reset) {
        S->latencies_ms.clear();
        S->submitted -= S->completed;   // keep requests in flight counted
        S->completed = 0;
        S->admissions = S->evictions = S->rejected = 0;
        S->groups = S->grouped_requests = S->probe_rays = 0;
        S->max_overlap = S->inflight;
        S->peak_resident_bytes = S->resident_bytes;
        S->have_first = false;
    }
    return LUXGI_OK;
}

int luxgi_server_touch(luxgi_server* S, int32_t id) {
    if (!S) return LUXGI_EINVAL;
    std::unique_lock<std::mutex> lk(S->mu);
    if (id < 0 || size_t(id) >= S->sessions.size()) return LUXGI_EINVAL;
    Session* ss = S->sessions[size_t(id)].get();
    // a session another caller is admitting or evicting: wait for the outcome
    S->cv_done.wait(lk, [&] { return !ss->transit; });
    if (ss->resident) return LUXGI_OK;
    if (ss->busy || !ss->queue.empty()) return LUXGI_EINVAL;
    // admission from the caller's thread: only while the scheduler is idle
    if (S->inflight != 0 || S->pending != 0) return LUXGI_EINVAL;
    if (!S->sim) cudaSetDevice(S->device);
    // in transit until admitted: requests submitted while make_room runs
    // with the lock released wait for it rather than admit it twice
    ss->transit = true;
    const bool room = make_room(S, ss->bytes, {}, lk);
    int s = room ? LUXGI_OK : LUXGI_ENOMEM;
    if (room && !S->sim) s = cuda_admit(S, *ss);
    ss->transit = false;
    if (s == LUXGI_OK) {
        ss->resident = true;
        ss->lru = ++S->lru_clock;
        S->resident_bytes += ss->bytes;
        S->resident_sessions += 1;
        S->peak_resident_bytes = std::max(S->peak_resident_bytes, S->resident_bytes);
        S->admissions += 1;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
    return s;
}

int luxgi_server_session_atlases(luxgi_server* S, int32_t id, luxgi_ddgi_atlases* out) {
    if (!S || !out) return LUXGI_EINVAL;
    std::lock_guard<std::mutex> g(S->mu);
    if (id < 0 || size_t(id) >= S->sessions.size()) return LUXGI_EINVAL;
    Session* ss = S->sessions[size_t(id)].get();
    if (S->sim || !ss->resident || !ss->vol) return LUXGI_ENOTBOUND;
    if (ss->busy || !ss->queue.empty()) return LUXGI_EINVAL;
    return luxgi_ddgi_get_atlases(ss->vol, out);
}

int luxgi_server_session_state(luxgi_server* S, int32_t id, int32_t* resident, int32_t* frames) {
    if (!S) return LUXGI_EINVAL;
    std::lock_guard<std::mutex> g(S->mu);
    if (id < 0 || size_t(id) >= S->sessions.size()) return LUXGI_EINVAL;
    const Session* ss = S->sessions[size_t(id)].get();
    if (resident) *resident = ss->resident ? 1 : 0;
    if (frames) *frames = ss->frames;
    return LUXGI_OK;
}

}  // extern "C"
