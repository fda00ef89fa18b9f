/* luxgi_serve.h -- serving loop over many DDGI probe volumes (sessions).
 *
 * No reference counterpart: LuxGI updates the volumes of one scene inside
 * its frame loop (Engine/DDGI/DDGIRenderer.cpp:217-464).  Here independent
 * sessions submit volume-update requests (one frame each) at any time; a
 * scheduler thread owned by the server
 *   - admits sessions to the device by a memory budget: a session's scene
 *     (SDF + mip, surface cache, culling lists) and volume (atlases and
 *     per-frame buffers) are made resident on first use and stay resident;
 *   - evicts the least recently used idle session when the budget is full
 *     (its current atlases and frame count are saved to host memory and
 *     restored on re-admission, so its results do not change);
 *   - forms launch groups from whatever requests are pending (continuous
 *     batching: at most one request per session in flight, oldest first)
 *     and issues each group as batched launches (one per stage over all
 *     volumes of the group) on one of several streams, so groups overlap on
 *     the device;
 *   - records per-request latency (submit to completion seen by the host).
 * Each request's result equals the same session's frames run alone.
 *
 * The scheduling policy is the same host code for both executors: the CUDA
 * executor runs the path on the current device, the host-simulated executor
 * (LUXGI_SERVE_EXEC_SIM) allocates nothing and completes a group after a
 * modelled time, for tests of admission, rejection and eviction without a
 * GPU.
 *
 * Conventions as luxgi_ddgi.h: int status (LUXGI_OK = 0, negative error). */
#ifndef LUXGI_SERVE_H
#define LUXGI_SERVE_H

#include <stdint.h>

#include "luxgi_ddgi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct luxgi_server luxgi_server;

typedef enum luxgi_serve_executor {
    LUXGI_SERVE_EXEC_CUDA = 0,
    LUXGI_SERVE_EXEC_SIM = 1
} luxgi_serve_executor;

typedef struct luxgi_server_desc {
    uint64_t memory_budget;        /* device bytes for resident sessions      */
    int32_t  executor;             /* luxgi_serve_executor                    */
    int32_t  max_group;            /* requests per launch group (0 = 64)      */
    int32_t  max_inflight;         /* groups on the device at once, one stream
                                      each (0 = 3)                            */
    int32_t  reserved0;
    luxgi_ddgi_batch_tuning tuning;/* variants of the batched launches
                                      (use_graph ignored); zeros = defaults   */
    double   sim_rate;             /* SIM: modelled probe-rays per second
                                      (0 = 1e9)                               */
    double   sim_admit_s;          /* SIM: modelled admission time (s)        */
    float    sim_evict_s;          /* SIM: modelled eviction copy (s, <= 60),
                                      run with the server's lock released as
                                      the device copy is                      */
    int32_t  reserved[3];
} luxgi_server_desc;

/* A session's scene, HOST memory owned by the caller (valid until the
 * server is destroyed).  sdf.sdf: (res*C) x res x res texels of sdf.format;
 * sdf.mip ignored (built at admission).  surface.objects, tiles, depth,
 * direct_light, albedo: host arrays; light_cache: host RGBA16F (light-cache
 * mode, NULL = copy of direct_light); chunks, culled_objects, gbuffer*:
 * ignored (the culling lists are built at admission). */
typedef struct luxgi_session_scene {
    luxgi_sdf_desc     sdf;
    luxgi_surface_desc surface;
    int32_t            atlas_resolution;   /* surface atlas side (texels)      */
    int32_t            reserved[3];
} luxgi_session_scene;

typedef struct luxgi_server_stats {
    uint64_t submitted, completed, pending, inflight_groups;
    uint64_t admissions, evictions, rejected;
    uint64_t resident_sessions, resident_bytes, peak_resident_bytes;
    uint64_t groups, probe_rays;           /* groups issued, probe-rays done   */
    uint64_t max_overlap;                  /* most groups in flight at once    */
    double   mean_group;                   /* requests per group               */
    double   latency_ms_p50, latency_ms_p95, latency_ms_p99;
    double   latency_ms_mean, latency_ms_max;
    double   wall_s;                       /* first submit to last completion  */
} luxgi_server_stats;

int luxgi_server_create(const luxgi_server_desc* desc, luxgi_server** out);
/* Stops the scheduler after the work in flight and frees every session. */
int luxgi_server_destroy(luxgi_server* server);

/* Registers a session (not yet resident).  Returns LUXGI_ENOMEM when the
 * session alone exceeds the memory budget (rejected; counted), LUXGI_EINVAL
 * for a bad volume or scene description. */
int luxgi_server_add_session(luxgi_server* server, const luxgi_ddgi_volume_desc* volume,
                             const luxgi_session_scene* scene, int32_t* session_id);
/* Device bytes the session holds while resident (scene + volume). */
int luxgi_server_session_bytes(luxgi_server* server, int32_t session_id, uint64_t* bytes);

/* Queues one frame of the session (rotation: column-major 3x3, host).
 * Returns at once with the request's ticket. */
int luxgi_server_submit(luxgi_server* server, int32_t session_id, const float rot[9],
                        uint64_t* ticket);
/* Blocks until every submitted request completed (or timeout_s passed:
 * LUXGI_ETIMEOUT).  Returns the first error a group met, if any. */
int luxgi_server_drain(luxgi_server* server, double timeout_s);

/* Open-loop load: for `seconds`, submits requests to sessions drawn
 * uniformly from ids[0..n) with exponential inter-arrival times of total
 * rate `rate` per second (seeded); each request's rotation is
 * luxgi_ddgi_frame_rotation(session id, its request index).  Then drains. */
int luxgi_server_run_poisson(luxgi_server* server, const int32_t* ids, int n, double rate,
                             double seconds, uint64_t seed);

/* Counters and latency percentiles over the requests completed since the
 * last reset (reset != 0 clears them after reading). */
int luxgi_server_stats_get(luxgi_server* server, luxgi_server_stats* out, int reset);

/* Makes an idle session resident (admitting, evicting as needed) without
 * running a frame: warm-up before timed runs. */
int luxgi_server_touch(luxgi_server* server, int32_t session_id);
/* Device views of an idle resident session's atlases (drain first);
 * LUXGI_ENOTBOUND when the session is not resident. */
int luxgi_server_session_atlases(luxgi_server* server, int32_t session_id,
                                 luxgi_ddgi_atlases* out);
/* Resident flag and frames done of a session. */
int luxgi_server_session_state(luxgi_server* server, int32_t session_id, int32_t* resident,
                               int32_t* frames);

#ifdef __cplusplus
}
#endif
#endif /* LUXGI_SERVE_H */
