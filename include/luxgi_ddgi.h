/*
 * luxgi_ddgi.h -- C ABI of the GB300 (sm_103a) DDGI probe-update path.
 *
 * This library replaces the non-raytracing ("SoftTrace") DDGI probe update of
 * LuxGI/Maple: the three ECS systems
 *     trace_rays::system    Code/Maple/src/Engine/DDGI/DDGIRenderer.cpp:217-330
 *     probe_update::system  Code/Maple/src/Engine/DDGI/DDGIRenderer.cpp:347-413
 *     border_update::system Code/Maple/src/Engine/DDGI/DDGIRenderer.cpp:418-464
 *     end_frame::system     Code/Maple/src/Engine/DDGI/DDGIRenderer.cpp:335-342
 * and the shaders they dispatch (Shaders/DDGI/GISDFRays.comp,
 * Shaders/DDGI/ProbeUpdate.glsl, Shaders/DDGI/BorderUpdate.glsl).
 *
 * Conventions
 *   - every entry point returns an int status: 0 = LUXGI_OK, negative = error;
 *     no exceptions cross the ABI;
 *   - all buffer arguments are plain pointers; "device" pointers must be CUDA
 *     device (or managed) memory, "host" pointers ordinary host memory;
 *   - a `stream` argument is a cudaStream_t passed as void* (NULL = legacy
 *     default stream);
 *   - the library never frees memory it did not allocate; scene inputs bound
 *     with luxgi_ddgi_bind_scene stay owned by the caller and must outlive the
 *     volume's use of them;
 *   - a volume is not thread-safe; use one volume per caller thread, or
 *     serialise calls on it.
 *
 * Texel/array layouts (all "x fastest"):
 *   SDF volume       (res*C) x res x res, cascades packed along x
 *                    (GlobalDistanceField.cpp:615, SDFRasterizeModel.glsl:47)
 *   SDF mip          (mres*C) x mres x mres, mres = res/4
 *   probe atlases    width x height texels, width  = (n+2)*X*Y + 2,
 *                    height = (n+2)*Z + 2   (DDGIRenderer.cpp:182-185);
 *                    irradiance = 4 channels (RGBA), distance = 2 (RG);
 *                    element type FP32 or FP16 (luxgi_storage)
 *   surface atlases  res x res texels (GlobalSurfaceAtlas.cpp:91)
 */
#ifndef LUXGI_DDGI_H
#define LUXGI_DDGI_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define LUXGI_OK            0
#define LUXGI_EINVAL       -1   /* bad argument (null pointer, bad dims ...)  */
#define LUXGI_ENOMEM       -2   /* device allocation or capacity exhausted    */
#define LUXGI_ECUDA        -3   /* a CUDA runtime call failed                 */
#define LUXGI_ETIMEOUT     -4   /* a bounded device-side wait gave up         */
#define LUXGI_ENOTBOUND    -5   /* luxgi_ddgi_bind_scene was not called       */
#define LUXGI_EUNSUPPORTED -6   /* option not available on this device/build  */
#define LUXGI_ESCRATCH     -7   /* input too large for the static scratch of
                                   luxgi_sdf_build_mip_noalloc               */

/* ---------------------------------------------------------------- enums */
enum luxgi_storage {           /* element type of ray buffers and atlases      */
    LUXGI_STORAGE_FP32 = 0,    /* FP32 atlases (meets 1e-4 rel vs FP64)        */
    LUXGI_STORAGE_FP16 = 1     /* RGBA16F/RG16F like the reference (F4)        */
};
enum luxgi_light_mode {
    LUXGI_LIGHT_CACHE   = 0,   /* hits sample the light-cache atlas; infinite
                                  bounce is injected into that atlas by
                                  luxgi_ddgi_inject_indirect
                                  (GISDFRays.comp:104-118,
                                   SDFAtlasIndirectLight.frag:44-67)           */
    LUXGI_LIGHT_PER_HIT = 1    /* hits sample the direct-light and albedo
                                  atlases and add albedo/pi * E_prev(hit)
                                  (Raytraced/Lighting.glsl:79-84)              */
};
enum luxgi_color_format {      /* the surface cache's colour textures       */
    LUXGI_COLOR_RGBA16F    = 0,  /* 4 x FP16, 8 bytes a texel                  */
    LUXGI_COLOR_R11G11B10F = 1   /* packed unsigned floats, 4 bytes a texel:
                                    R bits 0-10 and G bits 11-21 (5-bit
                                    exponent, 6-bit mantissa), B bits 22-31
                                    (5-bit exponent, 5-bit mantissa), bias 15,
                                    no sign; alpha reads as 1.  The engine's
                                    SurfaceEmissive and SurfaceLightCache
                                    (TextureFormat::R11G11B10,
                                    GlobalSurfaceAtlas.cpp:410-411)           */
};
enum luxgi_gbuffer_format {     /* the surface cache's G-buffers              */
    LUXGI_GBUFFER_RGBA32F = 0,   /* float4 a texel                             */
    LUXGI_GBUFFER_RGBA16F = 1    /* 4 x FP16 a texel: the engine's
                                    SurfaceGBuffer-Color / -Normal
                                    (TextureFormat::RGBA16,
                                    GlobalSurfaceAtlas.cpp:407-408)           */
};
enum luxgi_blend {
    LUXGI_BLEND_FP32   = 0,    /* FP32 SIMT contraction                        */
    LUXGI_BLEND_TENSOR = 1     /* tcgen05 FP16 operands, FP32 accumulation;
                                  distance data split hi+lo                    */
};

/* ------------------------------------------------------- parameter blocks */

/* DDGIUniform (Shaders/DDGI/DDGICommon.glsl:11-31, host copy
 * Engine/DDGI/DDGIRenderer.h:22-42), scalar layout, 96 bytes.  Width and
 * height fields left at 0 are derived by luxgi_ddgi_derive_uniform. */
typedef struct luxgi_ddgi_uniform {
    float   start_position[4];
    float   step[4];
    int32_t probe_counts[4];
    float   max_distance;
    float   sharpness;
    float   hysteresis;
    float   normal_bias;
    float   ddgi_gamma;
    int32_t irradiance_probe_side;
    int32_t irradiance_width;
    int32_t irradiance_height;
    int32_t depth_probe_side;
    int32_t depth_width;
    int32_t depth_height;
    int32_t rays_per_probe;
} luxgi_ddgi_uniform;

/* GlobalSDFData (Shaders/SDF/GlobalSDFData.glsl), 96 bytes. */
typedef struct luxgi_sdf_data {
    float    cascade_pos_distance[4][4];  /* center.xyz, half extent w      */
    float    cascade_voxel_size[4];
    uint32_t cascades_count;
    float    resolution;
    float    near_plane;
    float    far_plane;
} luxgi_sdf_data;

/* GlobalSurfaceAtlasData (Shaders/SDF/AtlasCommon.glsl:8-16), 32 bytes. */
typedef struct luxgi_surface_data {
    float    camera_pos[3];
    float    chunk_size;
    uint32_t culled_objects_capacity;
    uint32_t resolution;
    uint32_t objects_count;
    uint32_t padding;
} luxgi_surface_data;

/* ObjectBuffer (AtlasCommon.glsl:18-25, std430), 128 bytes.  Matrices are
 * column-major.  tile_offset[i] == 0 means "no tile" (AtlasCommon.glsl:143),
 * so tile slot 0 is never a real tile. */
typedef struct luxgi_surface_object {
    float    object_bounds[4];     /* bounding sphere center.xyz, radius     */
    uint32_t tile_offset[6];
    int32_t  padding[2];
    float    transform[16];        /* object(OBB) -> world                   */
    float    extends[4];           /* OBB half extents                       */
} luxgi_surface_object;

/* TileBuffer (AtlasCommon.glsl:27-32), 96 bytes. */
typedef struct luxgi_surface_tile {
    float extends[4];              /* (x, y, w-1, h-1) / atlas resolution    */
    float transform[16];           /* tile view rotation, translation zeroed */
    float object_bounds[4];        /* tile-space bounds size (x, y, z, 0)    */
} luxgi_surface_tile;

/* Scene inputs produced upstream of the path: the global SDF and its mip
 * (GlobalDistanceFieldPublic, GlobalDistanceField.h:31-42). */
typedef struct luxgi_sdf_desc {
    luxgi_sdf_data data;
    int32_t     format;            /* luxgi_storage: element type of sdf/mip  */
    int32_t     resolution;        /* res  (texels per cascade side)          */
    int32_t     mip_resolution;    /* mres (res / 4)                          */
    int32_t     reserved;
    const void* sdf;               /* device, (res*C) x res x res             */
    const void* mip;               /* device, (mres*C) x mres x mres          */
} luxgi_sdf_desc;

/* The surface cache (GlobalSurfacePublic, GlobalSurfaceAtlas.h:31-44).
 * The colour textures (light_cache, direct_light, emissive) are all of
 * `light_format`, the G-buffers of `gbuffer_format`; the engine's own
 * textures are R11G11B10F and RGBA16F (GlobalSurfaceAtlas.cpp:407-411). */
typedef struct luxgi_surface_desc {
    luxgi_surface_data          data;
    int32_t                     num_objects;
    int32_t                     num_tiles;      /* including dummy slot 0     */
    const luxgi_surface_object* objects;        /* device                     */
    const luxgi_surface_tile*   tiles;          /* device                     */
    const uint32_t*             chunks;         /* device, 40^3 u32           */
    const uint32_t*             culled_objects; /* device, [0] = used words   */
    void*                       light_cache;    /* device res^2 (mode A
                                                   sampled; written by inject) */
    const float*                depth;          /* device R32F res^2, 1 = empty*/
    const void*                 direct_light;   /* device res^2               */
    const uint8_t*              albedo;         /* device RGBA8 UNORM res^2   */
    const void*                 gbuffer0;       /* device res^2: albedo.rgb,
                                                   world.x (SDFDeferredColor
                                                   .frag:114)                 */
    const void*                 gbuffer1;       /* device res^2: oct normal.xy,
                                                   world.yz (:115)            */
    const uint8_t*              pbr;            /* device RGBA8 UNORM res^2
                                                   (SurfaceGBufferPRB): r
                                                   metallic, g roughness; NULL
                                                   = metallic 0, roughness 1  */
    const void*                 emissive;       /* device res^2
                                                   (SurfaceEmissive), or NULL */
    int32_t                     light_format;   /* luxgi_color_format of
                                                   light_cache, direct_light,
                                                   emissive and the lit atlas
                                                   of luxgi_surface_light     */
    int32_t                     gbuffer_format; /* luxgi_gbuffer_format       */
} luxgi_surface_desc;

/* Volume configuration: DDGIUniform plus the IrradianceVolume fields the
 * path reads (DDGIRenderer.h:44-60) and the build's own switches. */
typedef struct luxgi_ddgi_volume_desc {
    luxgi_ddgi_uniform uniform;
    int32_t storage;               /* luxgi_storage                           */
    int32_t light_mode;            /* luxgi_light_mode                        */
    int32_t blend;                 /* luxgi_blend                             */
    int32_t max_steps;             /* march step cap per cascade; 250 in the
                                      reference (SDFCommon.glsl:143)          */
    int32_t infinite_bounce;       /* IrradianceVolume::infiniteBounce        */
    float   intensity;             /* IrradianceVolume::intensity             */
    float   sky_radiance[3];       /* constant sky for misses                 */
    int32_t march_variant;         /* tuning, results identical, speed differs:
                                      0 default, settled at bind: 10 for an
                                      FP32 SDF, 11 for an FP16 SDF (4 where
                                      the SDF's planes exceed the texture
                                      gather limits); 1 plain SDF layout,
                                      64-register march; 2 plain, no register
                                      bound; 3 quad-packed mip; 4 quad-packed
                                      mip + SDF (4x SDF memory); 5 quad-packed
                                      mip + pair-packed SDF (2x SDF memory);
                                      6-9 as 2-5 with the pooled march (warps
                                      refill finished lanes from a ray pool);
                                      10 gather textures: one copy of the mip
                                      and of the SDF in 2D texture arrays,
                                      a trilinear sample two textureGathers
                                      (1x SDF memory); 11 quad-packed mip +
                                      gather texture of the SDF             */
    int32_t shade_variant;         /* tuning, results identical: cage probes of
                                      sampleIrradiance per loop iteration
                                      (0 default = 1; 1, 2, 4 or 8)          */
    int32_t ray_order;             /* tuning, results identical: order of the
                                      (probe, ray) work of march and shade.
                                      0 every probe for ray 0, then ray 1 ...;
                                      1 tiles of 256 consecutive probes, all
                                      rays of a tile before the next (a warp
                                      is 32 probes with one ray either way).
                                      The pooled march variants use 0.       */
    int32_t march_budget;          /* tuning, results identical: > 0 the march
                                      runs every ray for at most this many
                                      steps, queues the unfinished ones and
                                      resumes them with full warps (twice,
                                      then to the end); 0 default (12, then 8
                                      in the second pass, when the volume has
                                      >= 2^20 probe-rays, else one pass); -1
                                      one pass.  Per-ray variants
                                      1-5, 10 and 11.                        */
    int32_t shade_order;           /* tuning, results identical: 1 bin the
                                      hits by their surface-cache chunk first
                                      (histogram, scan, scatter) so a warp
                                      shades nearby hits; -1 shade in march
                                      order; 0 default (1 when the volume has
                                      >= 2^20 probe-rays, else -1).  Per-ray
                                      march variants 1-5, 10 and 11.         */
    int32_t shade_split;           /* tuning, results identical: 1 the rays
                                      that end in the compacted march's first
                                      pass are sorted and shaded on a second
                                      stream while the resume passes run, the
                                      others after them; -1 off; 0 default
                                      (on when the march is compacted, the
                                      shading binned and the volume has
                                      < 2^24 probe-rays).  The call keeps its
                                      stream semantics.                      */
    int32_t reserved[2];
} luxgi_ddgi_volume_desc;

/* Device views of a volume's probe atlases. */
typedef struct luxgi_ddgi_atlases {
    void*   irradiance;            /* current (last written) irradiance       */
    void*   distance;              /* current distance                        */
    void*   prev_irradiance;       /* the other ping-pong copy                */
    void*   prev_distance;
    int32_t irradiance_width, irradiance_height;
    int32_t depth_width, depth_height;
    int32_t storage;               /* luxgi_storage                           */
    int32_t frames;                /* frames completed                        */
} luxgi_ddgi_atlases;

/* Device views of the last trace's per-ray results (the reference's
 * "DDGI Raytrace Radiance" / "Direction Depth" textures, DDGIRenderer.cpp:173-177). */
typedef struct luxgi_ddgi_rays {
    const float* directions;       /* float4 [R]: rotated ray directions      */
    const void*  radiance;         /* [P][R] x4: rgb radiance, hit distance;
                                      FP32 or FP16 per storage                */
    const int32_t* hit_info;       /* int4 [P][R]: march steps, hit cascade
                                      (-1 miss), full-resolution SDF samples,
                                      0; NULL unless debug rays are on       */
    int32_t probes, rays, storage;
} luxgi_ddgi_rays;

typedef struct luxgi_ddgi_volume luxgi_ddgi_volume;

/* ------------------------------------------------------------ volumes */

/* Fill width/height fields of `u` from probe counts and sides
 * (DDGIRenderer.cpp:182-185) and validate it.  Host only. */
int luxgi_ddgi_derive_uniform(luxgi_ddgi_uniform* u);

/* Rotation matrix of angleAxis(angle, axis) as a column-major 3x3
 * (DDGIRenderer.cpp:267-272: glm::mat4_cast(glm::angleAxis(...))). Host only. */
int luxgi_ddgi_rotation(const float axis[3], float angle, float out_mat3[9]);

/* The seeded per-frame rotation used in place of std::random_device (F5):
 * xoshiro256** seeded by splitmix64(seed); axis = normalize(U(-1,1)^3),
 * angle = U(0,1) * 2pi, drawn in that order for each frame. Host only. */
int luxgi_ddgi_frame_rotation(uint64_t seed, uint32_t frame, float out_mat3[9]);

/* Allocate a volume (both atlas copies, per-ray buffers, weight tables) on
 * the current device.  Replaces ddgi::on_game_start + initializeProbeGrid
 * (DDGIRenderer.cpp:163-211, 565-683).  Atlases start zeroed. */
int luxgi_ddgi_create(const luxgi_ddgi_volume_desc* desc, luxgi_ddgi_volume** out);
int luxgi_ddgi_destroy(luxgi_ddgi_volume* vol);

/* Bind scene inputs (device pointers, caller-owned). */
int luxgi_ddgi_bind_scene(luxgi_ddgi_volume* vol, const luxgi_sdf_desc* sdf,
                          const luxgi_surface_desc* surface);

/* trace_rays::system: ray generation under `rot` (column-major 3x3) plus
 * SDF march and hit shading into the per-ray buffers. */
int luxgi_ddgi_trace(luxgi_ddgi_volume* vol, const float rot[9], void* stream);
/* probe_update::system: irradiance and distance blend into the write copy
 * (1 - pingPong), reading the previous copy; the border copy is fused in. */
int luxgi_ddgi_probe_update(luxgi_ddgi_volume* vol, void* stream);
/* border_update::system, standalone (in place on the write copy). */
int luxgi_ddgi_border_update(luxgi_ddgi_volume* vol, void* stream);
/* end_frame::system: flip ping-pong, frames++.  Host only. */
int luxgi_ddgi_end_frame(luxgi_ddgi_volume* vol);

/* One whole frame: trace + probe update (fused border) + end_frame. */
int luxgi_ddgi_update(luxgi_ddgi_volume* vol, const float rot[9], void* stream);

/* Many volumes, one frame each.  rots = n consecutive column-major 3x3
 * matrices (host).  Volumes that share storage, light mode, blend kind, SDF
 * format and a per-ray march variant (1-5, 10, 11) run together, one launch per
 * stage for the group; the rest run one after another.  A volume may appear
 * once.  The reference dispatches every volume separately
 * (DDGIRenderer.cpp:217-464); this call replaces a loop over those
 * dispatches.  For repeated frames of the same volumes luxgi_ddgi_batch_*
 * below adds graph replay and tuning. */
int luxgi_ddgi_update_batch(luxgi_ddgi_volume* const* vols, int n,
                            const float* rots, void* stream);

/* ------------------------------------------------ batched volume sets
 * A fixed set of volumes (uneven probe grids and ray counts) updated
 * together, frame after frame: raygen, weights, march, shade and the FP32
 * blend are each one launch over all volumes (blocks find their volume by
 * a block-offset table); the tensor-core blend is one persistent launch
 * over every volume's irradiance and distance jobs.  The frame is
 * captured once as a CUDA graph and replayed; the per-frame arguments
 * (rotations, ping-pong atlases, first-frame and bounce flags) are
 * written to pinned host memory and copied in by the graph.  Results
 * equal luxgi_ddgi_update of each volume alone.  No reference
 * counterpart. */
typedef struct luxgi_ddgi_batch luxgi_ddgi_batch;

typedef struct luxgi_ddgi_batch_tuning {
    int32_t march_variant;   /* 1-5, 10 or 11, as luxgi_ddgi_volume_desc.march_variant */
    int32_t march_threads;   /* rays per march block: 128 or 256              */
    int32_t shade_variant;   /* 1, 2, 4 or 8                                  */
    int32_t blend_probes;    /* probes per thread of the FP32-blend register
                                tile (x 4 texels): 1, 2 or 4                 */
    int32_t use_graph;       /* 1 capture + replay a CUDA graph, 0 launch     */
    int32_t march_budget;    /* as luxgi_ddgi_volume_desc.march_budget        */
    int32_t shade_order;     /* 1 shade in bin order (bins shared by the
                                batch's volumes), 0 or -1 march order        */
    int32_t reserved[1];
    float frame_ms;          /* frame time measured by the autotuner, else 0  */
} luxgi_ddgi_batch_tuning;

/* All volumes bound, on the current device, with the same storage, light
 * mode, blend kind and SDF format; none twice.  tuning may be NULL (march
 * variant 4, 256 rays a block, shade variant 1, 2 blend probes, graph on).  The
 * batch sets every volume's march and shade variant to its own (reallocating
 * the packed SDF copies the variant reads).  Volumes must outlive the batch
 * and must not be destroyed, re-created or updated concurrently with it. */
int luxgi_ddgi_batch_create(luxgi_ddgi_volume* const* vols, int n,
                            const luxgi_ddgi_batch_tuning* tuning,
                            luxgi_ddgi_batch** out);
/* One frame of every volume; rots = n column-major 3x3 matrices (host).
 * Consecutive frames of one batch must be ordered on the GPU (same stream,
 * or synchronised).  Host-side end_frame of every volume included. */
int luxgi_ddgi_batch_update(luxgi_ddgi_batch* batch, const float* rots, void* stream);
/* Times `frames` frames (after 2 warm-up frames) of each candidate tuning
 * (march variant x rays per block, then shade variant, then blend tile)
 * with CUDA events on `stream`, applies the fastest and writes it to *best
 * (may be NULL).  Every volume's atlases, frame count and ping-pong are saved
 * before and restored after, so results are unchanged by tuning.  Rotations
 * of the timed frames come from luxgi_ddgi_frame_rotation(seed 0). */
int luxgi_ddgi_batch_autotune(luxgi_ddgi_batch* batch, int frames, void* stream,
                              luxgi_ddgi_batch_tuning* best);
int luxgi_ddgi_batch_get_tuning(const luxgi_ddgi_batch* batch, luxgi_ddgi_batch_tuning* out);
int luxgi_ddgi_batch_set_tuning(luxgi_ddgi_batch* batch, const luxgi_ddgi_batch_tuning* tuning);
int luxgi_ddgi_batch_destroy(luxgi_ddgi_batch* batch);

/* Per-stage timing: with timing on, every trace / probe update records CUDA
 * events on its stream between its stages; luxgi_ddgi_stage_times waits for
 * the last frame's events and writes its milliseconds: [0] ray generation,
 * weights and scene set-up, [1] march (all passes), [2] hit shading,
 * [3] probe update (0 when none followed the trace).  Entry points also
 * push NVTX ranges (no cost without a profiler attached). */
int luxgi_ddgi_set_stage_timing(luxgi_ddgi_volume* vol, int enable);
int luxgi_ddgi_stage_times(luxgi_ddgi_volume* vol, float out[4]);

int luxgi_ddgi_get_atlases(const luxgi_ddgi_volume* vol, luxgi_ddgi_atlases* out);
int luxgi_ddgi_get_rays(const luxgi_ddgi_volume* vol, luxgi_ddgi_rays* out);
/* Synchronise `stream` and read the volume's device status word: returns
 * LUXGI_ETIMEOUT (and clears the word) when a bounded device-side wait of
 * the tensor-core blend gave up since the last check, else LUXGI_OK. */
int luxgi_ddgi_check_status(luxgi_ddgi_volume* vol, void* stream);
/* Test aid for the bounded device waits of the tensor-core blend (no
 * reference counterpart).  wait_cycles > 0 bounds each of its mbarrier waits
 * at that many SM clock cycles on this volume's later probe updates (0
 * restores the default, about 2 s).  withhold != 0 makes the next probe
 * update -- that one only -- skip one operand load in its first CTA, so the
 * matrix-multiply issuer's wait for it runs out: the kernel then stops
 * issuing work, drains the loads and multiplies it issued, frees its tensor
 * memory, returns, and raises the volume's status word, which
 * luxgi_ddgi_check_status reports as LUXGI_ETIMEOUT.  That frame's atlases
 * are incomplete; the device and the volume stay usable.  LUXGI_EUNSUPPORTED
 * for a volume without the tensor-core blend. */
int luxgi_ddgi_set_blend_wait_test(luxgi_ddgi_volume* vol, int64_t wait_cycles, int withhold);
/* Record per-ray march steps / hit cascade on the next traces (test aid). */
int luxgi_ddgi_set_debug_rays(luxgi_ddgi_volume* vol, int enable);
/* Copy the current atlases (the copy the next frame reads) to host buffers
 * of the volume's storage type and report the frame counter; waits for the
 * copies.  With luxgi_ddgi_load_atlases this checkpoints a volume: frames
 * run after a load equal the frames the saved volume would have run. */
int luxgi_ddgi_save_atlases(const luxgi_ddgi_volume* vol, void* irradiance_host, void* distance_host,
                            int32_t* frames, void* stream);
/* Overwrite both atlas copies from host buffers of the volume's storage type
 * and set the frame counter (atlas persistence / restore). */
int luxgi_ddgi_load_atlases(luxgi_ddgi_volume* vol, const void* irradiance_host,
                            const void* distance_host, int32_t frames, void* stream);

/* Mode A infinite bounce (SDFAtlasIndirectLight.frag:44-67) over the
 * raster footprint of every tile (see luxgi_surface_light): light_cache =
 * direct_light + intensity * (a - a * metallic)/pi * sampleIrradiance(prev
 * atlases), rounded to the light format (direct_light and light_cache may be
 * the same texture, as the engine's additive draw into SurfaceLightCache
 * is), a = min(albedo, 0.9), albedo, normal, position and metallic
 * sampled bilinearly at the fragment's atlas coordinate.  Texels outside
 * every tile keep their light_cache value.  When infinite bounce is off or
 * no frame is done yet the footprint gets direct_light unchanged. */
int luxgi_ddgi_inject_indirect(luxgi_ddgi_volume* vol, void* stream);

/* sampleIrradiance (DDGICommon.glsl:163-233) for n points against the
 * volume's current atlases: positions, normals, view vectors float3 [n]
 * (device), out float3 [n] (device). */
int luxgi_ddgi_sample_irradiance(const luxgi_ddgi_volume* vol, const float* pos,
                                 const float* nrm, const float* wo, float* out,
                                 int n, void* stream);

/* sample_probe::system + SampleProbe.comp:36-60 (DDGIRenderer.cpp:466-500):
 * the indirect-lighting image of a screen G-buffer from the volume's
 * current atlases.  depth: device R32F width x height (1 = background);
 * normal: device, normal_channels (2..4) floats a pixel, the first two the
 * octahedral normal; view_proj_inv: inverse(projView), column-major (host);
 * out: device RGBA16F, (irradiance, 1), or 0 at background pixels. */
int luxgi_ddgi_sample_probe_image(const luxgi_ddgi_volume* vol, const float* depth, const float* normal,
                                  int normal_channels, int width, int height, const float camera_pos[3],
                                  const float view_proj_inv[16], void* out, void* stream);

/* ------------------------------------------------------- scene set-up */

/* GlobalSDFMipmap.comp + 4 flood passes (GlobalDistanceField.cpp:537-573,
 * 823-841): mip (device) from sdf (device), for every cascade.  `tmp` is a
 * device buffer of mres^3 elements. */
int luxgi_sdf_build_mip(const luxgi_sdf_desc* sdf, void* mip, void* tmp, void* stream);

/* luxgi_sdf_build_mip for callers that cannot allocate device memory: an
 * engine that hands every byte of device memory out of its own fixed-budget
 * pool, or a frame loop that must not call cudaMalloc (it can synchronise
 * the device and stall the render thread).  No counterpart in the
 * reference: there the mip build's scratch is an engine-owned texture.
 * The flood-fill scratch plane lives in a 1 MiB static device array inside
 * the library (held by every GPU that loads the library until the process
 * exits), so the caller passes only the SDF and the mip.  Limit: mres^3
 * texels of the SDF's element type must fit in 1 MiB -- a mip of up to 64^3
 * FP32 texels (SDF resolution <= 256) or 80^3 FP16 texels; larger inputs
 * return LUXGI_ESCRATCH before anything runs.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture.  All
 * calls share the one array, so calls that overlap on the GPU (e.g. on two
 * streams) race; every scratch texel is written before it is read, so no
 * state carries over between calls.  Allocates nothing. */
int luxgi_sdf_build_mip_noalloc(const luxgi_sdf_desc* sdf, void* mip, void* stream);

/* ------------------------------------------- global SDF from objects */

/* A baked mesh SDF: the MeshDistanceField component (Engine/DDGI/
 * MeshDistanceField.h:15-26) and its FP16 volume with up to 3 mips
 * (SDFBaker.cpp:96-205).  Texel (x, y, z) of mip m sits at
 * x + y*w + z*w*h, (w, h, d) = max(size >> m, 1) per axis; a texel holds
 * (distance / max_distance + 1) / 2. */
typedef struct luxgi_mesh_sdf {
    float           aabb_min[3];        /* padded local bounds (paddingSDFBox)  */
    float           aabb_max[3];
    float           local_to_uvw_add[3];/* -min / size                          */
    float           local_to_uvw_mul[3];/* 1 / size                             */
    float           max_distance;       /* max3(size)                           */
    int32_t         size[3];            /* mip-0 texels                         */
    int32_t         mip_count;          /* 1 .. 3                               */
    int32_t         reserved;
    const uint16_t* mips[3];            /* device FP16 volumes                  */
} luxgi_mesh_sdf;

/* One placed object: an entity with MeshRenderer, Transform and
 * MeshDistanceField (GlobalDistanceField.cpp:672-693). */
typedef struct luxgi_sdf_object {
    float   world[16];                  /* Transform::getWorldMatrix, column-major */
    int32_t mesh;                       /* index into the mesh array            */
    int32_t reserved[3];
} luxgi_sdf_object;

/* The global SDF's parameters (GlobalDistanceFieldPublic and
 * GlobalDistanceField, GlobalDistanceField.h:29-45 and :590-604). */
typedef struct luxgi_sdf_build_desc {
    float   gi_distance;                /* giDistance, 4000 in the reference    */
    float   global_scale;               /* gloalScale, 0.1                      */
    float   min_object_radius;          /* minObjectRadius, 10 (times the scale) */
    int32_t resolution;                 /* voxels per cascade side, 192 (Quality::Test) */
    int32_t cascades;                   /* 1 .. 4, 2 (Quality::Test)            */
    int32_t format;                     /* luxgi_storage of the SDF and mip: FP16 is
                                           the reference's R16F                 */
    float   near_plane, far_plane;      /* copied into luxgi_sdf_data           */
} luxgi_sdf_build_desc;

/* ObjectRasterizeData (ObjectRasterizeData.glsl:8-18), 176 bytes: one per
 * object a cascade rasterises, in object order. */
typedef struct luxgi_sdf_raster_object {
    float   world_to_volume[16];
    float   volume_to_world[16];
    float   volume_to_uvw_mul[3];
    float   mip_offset;                 /* min(cascade, 2)                      */
    float   volume_to_uvw_add[3];
    float   decode_mul;                 /* max_distance                         */
    float   volume_local_bounds_extent[3];
    float   decode_add;                 /* -max_distance                        */
} luxgi_sdf_raster_object;

#define LUXGI_SDF_CHUNK 32              /* CONSTS_SDF_RASTERIZE_CHUNK_SIZE      */
#define LUXGI_SDF_CHUNK_MODELS 28       /* CONSTS_SDF_RASTERIZE_MODEL_MAX_COUNT */

/* A rasterised chunk: 32^3 voxels from coord * 32 of its cascade, the
 * objects (indices into the cascade's raster objects) it lists. */
typedef struct luxgi_sdf_chunk {
    int32_t  coord[3];
    int32_t  count;
    uint32_t models[LUXGI_SDF_CHUNK_MODELS];
} luxgi_sdf_chunk;

/* Host only: the cascade layout (centres, half extents, voxel sizes) of
 * GlobalDistanceField.cpp:590-626 and :837-841 into `out`. */
int luxgi_sdf_cascade_layout(const luxgi_sdf_build_desc* desc, luxgi_sdf_data* out);

/* Host only: the objects and chunks cascade `cascade` rasterises
 * (GlobalDistanceField.cpp:465-535, 672-700): objects whose bounding sphere
 * meets the cascade and is at least min_object_radius, each with the chunks
 * its margin-grown bounds cover, at most 28 per chunk as the reference's
 * chunk table keeps them.  `meshes` may carry null volume pointers.
 * Writes up to the capacities and returns the counts in *num_objects_out /
 * *num_chunks_out (LUXGI_ENOMEM when a capacity is short). */
int luxgi_sdf_build_plan(const luxgi_sdf_build_desc* desc, const luxgi_mesh_sdf* meshes, int num_meshes,
                         const luxgi_sdf_object* objects, int num_objects, int cascade,
                         luxgi_sdf_raster_object* raster_out, int raster_capacity, int* num_objects_out,
                         int32_t* object_mesh_out, luxgi_sdf_chunk* chunks_out, int chunk_capacity,
                         int* num_chunks_out);

/* The global SDF from objects (merge_sdf::system, GlobalDistanceField.cpp:
 * 576-842, first build): every voxel of every cascade set to 1, then per
 * cascade its chunks rasterised (SDFRasterizeModel.glsl: the minimum over
 * the chunk's objects of distanceToModelSDF, SDFCommon.glsl:38-62, stored
 * as clamp(d / (2 extent), -1, 1)) and its mip built (luxgi_sdf_build_mip's
 * passes; the flood passes only when the cascade has chunks).  sdf: device
 * (res*C) x res x res, mip (mres*C) x mres x mres, mres = res/4, tmp mres^3
 * elements, all of desc->format.  `data_out` gets the cascade layout.  A
 * chunk lying partly outside its cascade writes the voxels that fall inside
 * the packed texture, as the reference's image stores do. */
int luxgi_sdf_build(const luxgi_sdf_build_desc* desc, const luxgi_mesh_sdf* meshes, int num_meshes,
                    const luxgi_sdf_object* objects, int num_objects, void* sdf, void* mip, void* tmp,
                    luxgi_sdf_data* data_out, void* stream);

/* Host only: the layout of a baked .sdf file (SDFBaker.cpp:158-205, cereal
 * binary: uvec3 size, int32 mip count, then per mip a u64 byte count and the
 * FP16 texels).  Fills size, mip_count and, per mip, the byte offset of its
 * texels in `bytes` and their count; checks every length against n. */
typedef struct luxgi_mesh_sdf_file {
    int32_t  size[3];
    int32_t  mip_count;
    uint64_t mip_offset[3];
    uint64_t mip_bytes[3];
} luxgi_mesh_sdf_file;
int luxgi_mesh_sdf_parse(const void* bytes, uint64_t n, luxgi_mesh_sdf_file* out);

/* SDFCulling.comp: chunk table (40^3 u32, device) and culled-object lists
 * (device, `capacity` u32) for the objects of `surface`.  Layout is
 * deterministic: chunks in flattened order, objects in index order; entry
 * [0] of the list holds the number of words used.  Returns LUXGI_ENOMEM
 * when the lists do not fit (chunks that do not fit stay empty). */
int luxgi_surface_cull(const luxgi_surface_desc* surface, uint32_t* chunks,
                       uint32_t* culled, uint32_t capacity, void* stream);

/* Light (Common/Light.glsl:19-28, std140), 64 bytes. */
typedef struct luxgi_light {
    float color[4];                /* rgb                                     */
    float position[4];             /* xyz: point and spot lights              */
    float direction[4];            /* xyz, unit: directional and spot lights  */
    float intensity;
    float radius;                  /* attenuation radius (point, spot)        */
    float type;                    /* luxgi_light_type, a float as in GLSL    */
    float angle;                   /* spot: cut-off cosine is 1 - angle       */
} luxgi_light;

enum luxgi_light_type {            /* Light.glsl:13-15 */
    LUXGI_LIGHT_DIRECTIONAL = 0,
    LUXGI_LIGHT_SPOT        = 1,
    LUXGI_LIGHT_POINT       = 2
};
#define LUXGI_MAX_LIGHTS 32        /* MAX_LIGHTS, Light.glsl:30 */

/* One surface-cache lighting pass: the CopyEmissive draw followed by one
 * SDFDeferredLight draw per light (GlobalSurfaceAtlas.cpp:886-996), over a
 * list of tiles.  A tile covers the atlas pixels [x, x + w] x [y, y + h],
 * (x, y, w, h) = round(extends * resolution): the tile quad of addTiles2
 * (GlobalSurfaceAtlas.cpp:554-574) spans w + 1 pixels, the TileBuffer
 * extends holding the width less one texel of padding (:272-279).  The
 * fragment at pixel (x + i, y + j) samples every surface texture bilinearly
 * with REPEAT (the textures' default sampler, RHI/Definitions.h:152-159)
 * at atlasUV = ((i + 0.5) / (w + 1), (j + 0.5) / (h + 1)) * extends.zw +
 * extends.xy. */
typedef struct luxgi_surface_lighting {
    const luxgi_light* lights;     /* HOST, num_lights entries (copied into
                                      the launch's parameters)                */
    int32_t         num_lights;    /* 0 .. LUXGI_MAX_LIGHTS                   */
    int32_t         num_tiles;     /* entries of tiles and light_masks        */
    const uint32_t* tiles;         /* device: tile addresses, 1 .. surface
                                      num_tiles - 1, each at most once (others
                                      are skipped)                            */
    const uint32_t* light_masks;   /* device: bit l set = light l draws tile k
                                      (the per-light tile selection of
                                      GlobalSurfaceAtlas.cpp:912-944); NULL =
                                      every light draws every tile            */
    float           camera_pos[3]; /* UniformBufferObject.cameraPos.xyz       */
    float           shadow_bias;   /* cameraPos.w = GlobalSurface::shadowBias
                                      (1 in the reference)                    */
    int32_t         copy_emissive; /* 1: the footprint first gets the sampled
                                      surface emissive (alpha 1 where the
                                      surface has none); 0: lights add onto
                                      `out` as it is                          */
    int32_t         max_steps;     /* shadow march step cap per cascade; 250
                                      in the reference (SDFCommon.glsl:143)   */
    int32_t         reserved[2];
} luxgi_surface_lighting;

/* SDF-shadowed direct lighting of the surface cache: per footprint pixel,
 * for each light of its tile in index order, `out` (device res^2 of the
 * surface's light_format) += (BRDF * radiance * cos * shadow * attenuation,
 * 1), rounded to the target's format after each light like the additive
 * blend into the render target: FP16 per channel (RGBA16F) or the 11/11/10-
 * bit unsigned floats, nearest even, negative to 0 (R11G11B10F, no alpha)
 * (SDFDeferredLight.frag:41-129, Raytraced/BRDF.glsl:65-81).  The emissive
 * copy rounds the same way.  The shadow is a global-SDF march towards the
 * light from position + normal * bias with start bias 2 voxels and no hit
 * normal (SDFDeferredLight.frag:95-118). */
int luxgi_surface_light(const luxgi_sdf_desc* sdf, const luxgi_surface_desc* surface,
                        const luxgi_surface_lighting* lighting, void* out, void* stream);

/* ------------------------------------------------------------ misc */
const char* luxgi_strerror(int status);
/* Kernel launches issued by this library since load (all entry points). */
uint64_t luxgi_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* LUXGI_DDGI_H */
