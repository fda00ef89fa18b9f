/*
 * luxgi_scene.h -- seeded synthetic scene inputs for the DDGI probe-update path.
 *
 * LuxGI builds the path's inputs in other engine systems (the global SDF in
 * GlobalDistanceField.cpp, the surface cache in GlobalSurfaceAtlas.cpp).  This
 * host library builds equivalent inputs from analytic primitives:
 *   - the global SDF: per-voxel exact distance to seeded spheres, axis-aligned
 *     boxes and the room walls, normalised like SDFRasterizeModel.glsl:46-62
 *     (value = clamp(d / cascadeMaxDistance, -1, 1), voxel centres at
 *     bounds.min + (i + 0.5) * voxel);
 *   - the surface cache: one object per primitive and per wall slab with six
 *     axis-aligned cards whose tile matrices follow cacheToSurface
 *     (GlobalSurfaceAtlas.cpp:226-280: lookAt from the face towards the
 *     centre, translation zeroed), a depth atlas holding the tile-space depth
 *     AtlasCommon.glsl:63 compares against (1.0 = empty texel), an RGBA8 albedo
 *     atlas, an RGBA16F direct-light atlas (Lambert sun, no shadow) and the
 *     two G-buffer atlases SDFAtlasIndirectLight.frag reads.
 * The SDF mip and chunk culling are NOT built here: they are stages of the
 * path (luxgi_sdf_build_mip, luxgi_surface_cull).
 * Host only, deterministic for a given config (compiled without FP
 * contraction so x86-64 and aarch64 produce identical bits).
 */
#ifndef LUXGI_SCENE_H
#define LUXGI_SCENE_H

#include <stdint.h>
#include "luxgi_ddgi.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct luxgi_scene_config {
    uint64_t seed;
    float    room_size;            /* scene spans [-L/2, L/2]^3                 */
    float    wall_thickness;
    int32_t  num_primitives;       /* each a sphere or a box, seeded           */
    float    sphere_radius[2];     /* U[min, max]                              */
    float    box_half_extent[2];   /* U[min, max] per axis                     */
    int32_t  sdf_resolution;       /* texels per cascade side                  */
    int32_t  cascades;             /* 1..4                                     */
    int32_t  sdf_format;           /* luxgi_storage                            */
    int32_t  atlas_resolution;
    float    albedo_range[2];      /* U[min, max] per channel                  */
    float    sun_direction[3];     /* towards the sun; all 0 = seeded on the
                                      upper hemisphere                          */
    float    sun_color[3];
    int32_t  tile_resolution;      /* 0 = derived from atlas size and count    */
    int32_t  reserved[4];
} luxgi_scene_config;

typedef struct luxgi_scene_primitive {
    int32_t kind;                  /* 0 sphere, 1 box, 2 wall slab             */
    float   center[3];
    float   half_extent[3];        /* sphere: (r, r, r)                        */
    float   albedo[3];
} luxgi_scene_primitive;

typedef struct luxgi_scene_view {
    luxgi_sdf_data              sdf_data;
    int32_t                     sdf_format;
    int32_t                     sdf_resolution;
    int32_t                     mip_resolution;
    int32_t                     cascades;
    const void*                 sdf;           /* host, (res*C)*res*res      */
    int64_t                     sdf_bytes;
    luxgi_surface_data          surface_data;
    int32_t                     num_objects;
    int32_t                     num_tiles;     /* including dummy slot 0     */
    const luxgi_surface_object* objects;
    const luxgi_surface_tile*   tiles;
    int32_t                     atlas_resolution;
    const uint16_t*             direct_light;  /* RGBA16F res^2              */
    const float*                depth;         /* R32F res^2                 */
    const uint8_t*              albedo;        /* RGBA8 res^2                */
    const float*                gbuffer0;      /* float4 res^2               */
    const float*                gbuffer1;      /* float4 res^2               */
    int32_t                     num_primitives;
    const luxgi_scene_primitive* primitives;   /* spheres/boxes, then walls  */
    float                       sun_direction[3];
    float                       sun_color[3];
    const uint8_t*              pbr;           /* RGBA8 res^2: metallic,
                                                  roughness, 0, 1            */
    const uint16_t*             emissive;      /* RGBA16F res^2              */
} luxgi_scene_view;

typedef struct luxgi_scene luxgi_scene;

int luxgi_scene_build(const luxgi_scene_config* cfg, luxgi_scene** out);
int luxgi_scene_view_get(const luxgi_scene* scene, luxgi_scene_view* out);
int luxgi_scene_destroy(luxgi_scene* scene);

/* Exact analytic distance of the scene at a world point (test aid). */
float luxgi_scene_distance(const luxgi_scene* scene, const float p[3]);

/* IEEE binary16 <-> binary32, round to nearest even (host). */
uint16_t luxgi_float_to_half(float f);
float    luxgi_half_to_float(uint16_t h);

#ifdef __cplusplus
}
#endif
#endif /* LUXGI_SCENE_H */
