// ORACLE -- test infrastructure only.
//
// Host harness around the reference's own GLSL function libraries, compiled
// as C++ (see oracle/build_ref.py).  Every computation below is a call into
// the reference functions -- sphericalFibonacci, probeLocation,
// tracyGlobalSDF, getHitPosition, getGlobalSurfaceAtlasThreshold, the
// sampleGlobalSurfaceAtlas macro, sampleIrradiance, octDecode,
// normalizedOctCoord, getProbeId, combineDistanceToSDF, boxIntersectsSphere,
// flattenId -- glued together the way the shader entry points do:
//   ref_trace  GISDFRays.comp:63-128
//   ref_blend  ProbeUpdate.glsl:66-152
//   ref_mip    GlobalSDFMipmap.comp:32-67 and GlobalDistanceField.cpp:537-573
//   ref_cull   SDFCulling.comp:36-101 (deterministic list placement)
//   ref_surface_light  CopyEmissive.frag:22-26, SDFDeferredLight.frag:41-129
//                      (BRDF from Raytraced/BRDF.glsl:65-81)
//   ref_inject SDFAtlasIndirectLight.frag:44-67
//   ref_sample_probe_image SampleProbe.comp:36-60 (worldPositionFromDepth,
//              Common/Math.glsl:35-42)
//   ref_sdf_raster SDFRasterizeModel.glsl:42-63 (distanceToModelSDF,
//              SDFCommon.glsl:38-62) over a cascade's chunks
// The two raster passes run over the pixels of the tile quads of addTiles2
// (Engine/DDGI/GlobalSurfaceAtlas.cpp:554-574).
// The entry-point bodies are restated because they declare Vulkan
// resources (images, SSBOs, push constants) that do not compile as C++.
#include "glsl_compat.h"

#include "DDGI/DDGICommon.glsl"
#include "SDF/SDFCommon.glsl"
#include "SDF/AtlasCommon.glsl"
#include "Raytraced/BRDF.glsl"
#include "Common/Light.glsl"

#include <vector>

#include "luxgi_ddgi.h"

static_assert(sizeof(DDGIUniform) == sizeof(luxgi_ddgi_uniform), "DDGIUniform layout");
static_assert(sizeof(GlobalSDFData) == sizeof(luxgi_sdf_data), "GlobalSDFData layout");
static_assert(sizeof(GlobalSurfaceAtlasData) == sizeof(luxgi_surface_data), "GlobalSurfaceAtlasData layout");
static_assert(sizeof(ObjectBuffer) == sizeof(luxgi_surface_object), "ObjectBuffer layout");
static_assert(sizeof(TileBuffer) == sizeof(luxgi_surface_tile), "TileBuffer layout");
static_assert(sizeof(Light) == sizeof(luxgi_light), "Light layout");
static_assert(sizeof(ObjectRasterizeData) == sizeof(luxgi_sdf_raster_object), "ObjectRasterizeData layout");

namespace {

template <typename T, typename S> T as(const S& s) {
    T t;
    std::memcpy(static_cast<void*>(&t), &s, sizeof(T));
    return t;
}

sampler3D volume(const void* p, int fmt, int W, int H, int D) {
    sampler3D s;
    if (fmt == LUXGI_STORAGE_FP16) s.f16 = static_cast<const uint16_t*>(p);
    else s.f32 = static_cast<const float*>(p);
    s.W = W; s.H = H; s.D = D;
    return s;
}

sampler2D tex2d(const float* f32, const uint16_t* f16, const uint8_t* u8, int W, int H, int C, bool repeat) {
    sampler2D s;
    s.f32 = f32; s.f16 = f16; s.u8 = u8;
    s.W = W; s.H = H; s.C = C;
    s.repeat = repeat;
    return s;
}

// A surface colour texture of luxgi_color_format `fmt` (RGBA16F, or packed
// R11G11B10F sampled as rgb + alpha 1).
sampler2D color_tex(const void* p, int fmt, int W, int H, bool repeat) {
    sampler2D s = tex2d(nullptr, fmt == LUXGI_COLOR_R11G11B10F ? nullptr : static_cast<const uint16_t*>(p), nullptr,
                        W, H, 4, repeat);
    if (fmt == LUXGI_COLOR_R11G11B10F) s.r11 = static_cast<const uint32_t*>(p);
    return s;
}
// A surface G-buffer of luxgi_gbuffer_format `fmt`.
sampler2D gbuffer_tex(const void* p, int fmt, int W, int H) {
    if (fmt == LUXGI_GBUFFER_RGBA16F) return tex2d(nullptr, static_cast<const uint16_t*>(p), nullptr, W, H, 4, true);
    return tex2d(static_cast<const float*>(p), nullptr, nullptr, W, H, 4, true);
}
// The render target's rounding of a colour (what an RGBA16F or R11G11B10F
// attachment stores), and its texel load and store.
void target_round(int fmt, float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        const uint32_t q = packed_color::pack(v);
        for (int c = 0; c < 4; ++c) v[c] = packed_color::channel(q, c);
    } else {
        for (int c = 0; c < 4; ++c) v[c] = float(_Float16(v[c]));
    }
}
void target_load(const void* p, int fmt, size_t ti, float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        const uint32_t q = static_cast<const uint32_t*>(p)[ti];
        for (int c = 0; c < 4; ++c) v[c] = packed_color::channel(q, c);
    } else {
        for (int c = 0; c < 4; ++c) {
            _Float16 h;
            std::memcpy(&h, static_cast<const uint16_t*>(p) + ti * 4 + size_t(c), 2);
            v[c] = float(h);
        }
    }
}
void target_store(void* p, int fmt, size_t ti, const float* v) {
    if (fmt == LUXGI_COLOR_R11G11B10F) {
        static_cast<uint32_t*>(p)[ti] = packed_color::pack(v);
    } else {
        for (int c = 0; c < 4; ++c) {
            const _Float16 h = _Float16(v[c]);
            std::memcpy(static_cast<uint16_t*>(p) + ti * 4 + size_t(c), &h, 2);
        }
    }
}

// The pixels a tile quad of addTiles2 covers (Engine/DDGI/
// GlobalSurfaceAtlas.cpp:554-574): tile->x .. x + width - 1, with
// extends.z = (width - 1) / resolution (:272-279), and the fragment's
// interpolated inTileUV at pixel centres.
struct Quad {
    int x, y, width, height;
};
Quad tile_quad(const TileBuffer& t, int res) {
    Quad q;
    q.x = int(__builtin_lroundf(t.extends.x * float(res)));
    q.y = int(__builtin_lroundf(t.extends.y * float(res)));
    q.width = int(__builtin_lroundf(t.extends.z * float(res))) + 1;
    q.height = int(__builtin_lroundf(t.extends.w * float(res))) + 1;
    return q;
}
vec2 tile_uv(const Quad& q, int i, int j) {
    return vec2((float(i) + 0.5f) / float(q.width), (float(j) + 0.5f) / float(q.height));
}
float h16(uint16_t b) { _Float16 h; std::memcpy(&h, &b, 2); return float(h); }
uint16_t to16(float f) { _Float16 h = _Float16(f); uint16_t b; std::memcpy(&b, &h, 2); return b; }

// fetchLight, SDFDeferredLight.frag:41-76 (a function of the entry-point
// file, restated here).
void fetchLight(const Light& light, vec3 worldPos, vec3 normal, vec3& Wi, float& tmax, float& attenuation) {
    vec3 lightDir = vec3(0, 0, 0);
    if (light.type == LIGHT_DIRECTIONAL) {
        lightDir = -vec3(light.direction.xyz);
        tmax = GLOBAL_SDF_WORLD_SIZE;
        Wi = lightDir;
        attenuation = 1.0;
    } else if (light.type == LIGHT_POINT) {
        vec3 dir = vec3(light.position.xyz) - worldPos;
        float dist = length(dir);
        lightDir = normalize(dir);
        attenuation = light.radius / (pow(dist, 2.0) + 1.0);
        Wi = lightDir;
        tmax = dist;
    } else if (light.type == LIGHT_SPOT) {
        vec3 L = vec3(light.position.xyz) - worldPos;
        float cutoffAngle = 1.0f - light.angle;
        lightDir = normalize(L);
        float dist = length(L);
        float theta = dot(lightDir, vec3(light.direction.xyz));
        float epsilon = cutoffAngle - cutoffAngle * 0.9f;
        attenuation = ((theta - cutoffAngle) / epsilon);
        attenuation *= light.radius / (pow(dist, 2.0) + 1.0);
        attenuation = clamp(attenuation, 0.0, 1.0);
        Wi = lightDir;
        tmax = dist;
    }
    (void)normal;
}

}  // namespace

extern "C" {

// GISDFRays.comp main for probes [p0, p1): out float4 [n][R] (rgb, distance),
// info int2 [n][R] (steps, hit cascade or -1).  Mode B adds
// intensity * albedo/pi * sampleIrradiance(previous atlases) at hits
// (Raytraced/Lighting.glsl:79-84 with the volume intensity).
// `dirs` (float4 [R], optional) replaces the rotated sphericalFibonacci
// directions, so march and shading can be compared on identical rays.
int ref_trace(const luxgi_ddgi_volume_desc* vd, const luxgi_sdf_desc* sdf, const luxgi_surface_desc* surf,
              const float* prev_irr, const float* prev_dist, int frames, const float rot9[9], int p0, int p1,
              float* out, int32_t* info, const float* dirs) {
    const DDGIUniform ddgi = as<DDGIUniform>(vd->uniform);
    const GlobalSDFData sd = as<GlobalSDFData>(sdf->data);
    const GlobalSurfaceAtlasData ad = as<GlobalSurfaceAtlasData>(surf->data);
    const int C = int(sdf->data.cascades_count), res = sdf->resolution, mres = sdf->mip_resolution;
    const sampler3D tex = volume(sdf->sdf, sdf->format, res * C, res, res);
    const sampler3D mip = volume(sdf->mip, sdf->format, mres * C, mres, mres);
    const int A = int(surf->data.resolution);
    const sampler2D depthS = tex2d(surf->depth, nullptr, nullptr, A, A, 1, false);
    const bool per_hit = vd->light_mode == LUXGI_LIGHT_PER_HIT;
    const sampler2D colorS = color_tex(per_hit ? surf->direct_light : surf->light_cache, surf->light_format, A, A,
                                       false);
    const sampler2D albedoS = tex2d(nullptr, nullptr, surf->albedo, A, A, 4, false);
    const sampler2D irrS = tex2d(prev_irr, nullptr, nullptr, ddgi.irradianceTextureWidth, ddgi.irradianceTextureHeight, 4, true);
    const sampler2D distS = tex2d(prev_dist, nullptr, nullptr, ddgi.depthTextureWidth, ddgi.depthTextureHeight, 2, true);
    const ObjectBuffer* objects = reinterpret_cast<const ObjectBuffer*>(surf->objects);
    const TileBuffer* tiles = reinterpret_cast<const TileBuffer*>(surf->tiles);
    const uint* chunks = surf->chunks;
    const uint* cull = surf->culled_objects;
    const bool bounce = per_hit && vd->infinite_bounce && frames != 0 && prev_irr && prev_dist;
    mat3 orientation(vec3(rot9[0], rot9[1], rot9[2]), vec3(rot9[3], rot9[4], rot9[5]), vec3(rot9[6], rot9[7], rot9[8]));
    const int R = ddgi.raysPerProbe;
#pragma omp parallel for schedule(dynamic, 1)
    for (int probeId = p0; probeId < p1; ++probeId) {
        for (int rayId = 0; rayId < R; ++rayId) {
            vec3 rayOrigin = probeLocation(ddgi, probeId);
            vec3 direction = dirs ? vec3(dirs[4 * rayId], dirs[4 * rayId + 1], dirs[4 * rayId + 2])
                                  : normalize(orientation * sphericalFibonacci(float(rayId), float(ddgi.raysPerProbe)));
            GlobalSDFTrace trace;
            trace.worldPosition = rayOrigin;
            trace.worldDirection = direction;
            trace.minDistance = 0;
            trace.maxDistance = GLOBAL_SDF_WORLD_SIZE;
            trace.stepScale = 1.f;
            trace.needsHitNormal = true;
            GlobalSDFHit hit = tracyGlobalSDF(sd, tex, mip, trace, 0);
            vec4 radiance = vec4(0);
            if (isHit(hit)) {
                if (hit.hitSDF <= 0.0f && hit.hitTime <= sd.cascadeVoxelSize[0]) {
                    radiance = vec4(0, 0, 0, GLOBAL_SDF_WORLD_SIZE);
                } else {
                    vec3 hitPosition = getHitPosition(hit, trace);
                    float surfaceThreshold = getGlobalSurfaceAtlasThreshold(sd, hit);
                    vec4 surfaceColor;
                    sampleGlobalSurfaceAtlas(surfaceColor, ad, chunks, cull, objects, tiles, depthS, colorS,
                                             getHitPosition(hit, trace), hit.hitNormal, surfaceThreshold, false);
                    radiance = vec4(vec3(surfaceColor.rgb), hit.hitTime);
                    if (bounce) {
                        vec4 albedo;
                        sampleGlobalSurfaceAtlas(albedo, ad, chunks, cull, objects, tiles, depthS, albedoS,
                                                 hitPosition, hit.hitNormal, surfaceThreshold, false);
                        vec3 diffuseColor = (vec3(albedo.rgb) - vec3(albedo.rgb) * 0.0f) / PI;
                        vec3 e = sampleIrradiance(ddgi, hitPosition, hit.hitNormal, -direction, irrS, distS);
                        radiance.rgb += vd->intensity * diffuseColor * e;
                    }
                    radiance.w = max(radiance.w + sd.cascadeVoxelSize[hit.hitCascade] * 0.5f, 0);
                }
            } else {
                radiance = vec4(vd->sky_radiance[0], vd->sky_radiance[1], vd->sky_radiance[2], GLOBAL_SDF_WORLD_SIZE);
            }
            const size_t i = size_t(probeId - p0) * R + rayId;
            out[4 * i + 0] = radiance.x;
            out[4 * i + 1] = radiance.y;
            out[4 * i + 2] = radiance.z;
            out[4 * i + 3] = radiance.w;
            if (info) {
                info[2 * i] = int32_t(hit.stepsCount);
                info[2 * i + 1] = isHit(hit) ? int32_t(hit.hitCascade) : -1;
            }
        }
    }
    return 0;
}

// ProbeUpdate.glsl main for both atlases.  dirs float4 [R], rays float4
// [P][R] (rgb, distance); atlases float, prev may be NULL when first.
int ref_blend(const luxgi_ddgi_volume_desc* vd, const float* dirs, const float* rays, const float* prev_irr,
              const float* prev_dist, float* out_irr, float* out_dist, int first) {
    const DDGIUniform ddgi = as<DDGIUniform>(vd->uniform);
    const int XY = ddgi.probeCounts.x * ddgi.probeCounts.y, Z = ddgi.probeCounts.z;
    const float FLT_EPS = 0.00000001;
    for (int depth = 0; depth < 2; ++depth) {
        const int n = depth ? ddgi.depthProbeSideLength : ddgi.irradianceProbeSideLength;
        const int W = depth ? ddgi.depthTextureWidth : ddgi.irradianceTextureWidth;
        const int nc = depth ? 2 : 4;
        const float* prev = depth ? prev_dist : prev_irr;
        float* outp = depth ? out_dist : out_irr;
#pragma omp parallel for collapse(2)
        for (int gy = 0; gy < Z; ++gy)
            for (int gx = 0; gx < XY; ++gx)
                for (int ly = 0; ly < n; ++ly)
                    for (int lx = 0; lx < n; ++lx) {
                        // gl_GlobalInvocationID = workgroup * local size + local id
                        const ivec2 currentCoord = ivec2(gx * n + lx, gy * n + ly) + (ivec2(gx, gy) * ivec2(2)) + ivec2(2);
                        const int relativeProbeId = getProbeId(vec2(currentCoord), W, n);
                        vec3 result = vec3(0.0f);
                        float totalWeight = 0.0f;
                        vec3 texelDirection = octDecode(normalizedOctCoord(currentCoord, n));
                        for (int r = 0; r < ddgi.raysPerProbe; ++r) {
                            const float* dd = dirs + 4 * r;
                            const float* ry = rays + (size_t(relativeProbeId) * ddgi.raysPerProbe + r) * 4;
                            vec3 rayDirection = vec3(dd[0], dd[1], dd[2]);
                            float weight = 0.0f;
                            if (depth) {
                                float rayProbeDistance = min(ddgi.maxDistance, ry[3] - 0.01f);
                                if (rayProbeDistance == -1.0f) rayProbeDistance = ddgi.maxDistance;
                                weight = pow(max(0.0, dot(texelDirection, rayDirection)), ddgi.sharpness);
                                if (weight >= FLT_EPS) {
                                    result += vec3(rayProbeDistance * weight, square(rayProbeDistance) * weight, 0.0);
                                    totalWeight += weight;
                                }
                            } else {
                                vec3 rayHitRadiance = vec3(ry[0], ry[1], ry[2]);
                                weight = max(0.0, dot(texelDirection, rayDirection));
                                if (weight >= FLT_EPS) {
                                    result += vec3(rayHitRadiance * weight);
                                    totalWeight += weight;
                                }
                            }
                        }
                        if (totalWeight > FLT_EPS) result *= 1.f / (2 * totalWeight);
                        const size_t ti = (size_t(currentCoord.y) * W + size_t(currentCoord.x)) * nc;
                        vec3 prevResult = vec3(0.0f);
                        if (!first) {
                            prevResult.x = prev[ti];
                            prevResult.y = prev[ti + 1];
                            if (!depth) prevResult.z = prev[ti + 2];
                        }
                        if (!depth) result.rgb = pow(vec3(result.rgb), vec3(1.0f / ddgi.ddgiGamma));
                        if (!first) result = mix(result, prevResult, ddgi.hysteresis);
                        outp[ti] = result.x;
                        outp[ti + 1] = result.y;
                        if (!depth) {
                            outp[ti + 2] = result.z;
                            outp[ti + 3] = 1.0f;
                        }
                    }
    }
    return 0;
}

// GlobalSDFMipmap.comp main + the four fillFlood passes, every cascade.
int ref_mip(const luxgi_sdf_desc* s, const float* sdf, float* mip_out) {
    const int res = s->resolution, mres = s->mip_resolution, C = int(s->data.cascades_count);
    std::vector<float> mip(size_t(mres) * C * mres * mres, 1.0f), tmp(size_t(mres) * mres * mres, 1.0f);
    const ivec3 coords[6] = {ivec3(1, 0, 0), ivec3(0, 1, 0), ivec3(0, 0, 1), ivec3(-1, 0, 0), ivec3(0, -1, 0), ivec3(0, 0, -1)};
    auto pass = [&](const float* src, int srcW, int srcRes, int scale, int offX, float* dst, int dstW, int dstOffX,
                    float maxDistance) {
        auto sampleSDF = [&](ivec3 voxelCoordMip, ivec3 offset) {
            voxelCoordMip = clamp(voxelCoordMip * scale + offset, ivec3(0), ivec3(srcRes - 1));
            voxelCoordMip.x += offX;
            float result = src[size_t(voxelCoordMip.x) + size_t(srcW) * (size_t(voxelCoordMip.y) + size_t(srcRes) * voxelCoordMip.z)];
            float distanceToVoxel = length(offset) * (maxDistance / float(srcRes));
            return combineDistanceToSDF(result, distanceToVoxel);
        };
        for (int z = 0; z < mres; ++z)
            for (int y = 0; y < mres; ++y)
                for (int x = 0; x < mres; ++x) {
                    ivec3 uvw = ivec3(x, y, z);
                    float minDistance = sampleSDF(uvw, ivec3(0, 0, 0));
                    for (int i = 0; i < 6; i++) minDistance = min(minDistance, sampleSDF(uvw, coords[i]));
                    if (s->format == LUXGI_STORAGE_FP16) minDistance = float(_Float16(minDistance));
                    dst[size_t(x + dstOffX) + size_t(dstW) * (size_t(y) + size_t(mres) * z)] = minDistance;
                }
    };
    for (int k = 0; k < C; ++k) {
        const float maxd = s->data.cascade_pos_distance[k][3] * 2.0f;
        pass(sdf, res * C, res, 4, k * res, mip.data(), mres * C, k * mres, maxd);
        for (int i = 1; i < 5; ++i) {
            if (i & 1) pass(mip.data(), mres * C, mres, 1, k * mres, tmp.data(), mres, 0, maxd);
            else pass(tmp.data(), mres, mres, 1, 0, mip.data(), mres * C, k * mres, maxd);
        }
    }
    std::memcpy(mip_out, mip.data(), mip.size() * sizeof(float));
    return 0;
}

// SDFCulling.comp main: for every chunk, the objects whose bounding sphere
// touches the chunk box.  Lists are written in flattened chunk order at
// prefix-sum offsets from word 1 (the reference appends them with an
// atomic counter in arbitrary order; the per-chunk contents are the same).
int ref_cull(const luxgi_surface_desc* s, uint32_t* chunks, uint32_t* culled, uint32_t capacity) {
    const GlobalSurfaceAtlasData data = as<GlobalSurfaceAtlasData>(s->data);
    const ObjectBuffer* objects = reinterpret_cast<const ObjectBuffer*>(s->objects);
    const int NC = GLOBAL_SURFACE_ATLAS_CHUNKS_RESOLUTION;
    std::memset(chunks, 0, sizeof(uint32_t) * NC * NC * NC);
    uint32_t used = 1;
    for (int z = 0; z < NC; ++z)
        for (int y = 0; y < NC; ++y)
            for (int x = 0; x < NC; ++x) {
                ivec3 chunkCoord = ivec3(x, y, z);
                uint chunkAddress = flattenId(chunkCoord);
                vec3 chunkMin = (vec3(chunkCoord) - (GLOBAL_SURFACE_ATLAS_CHUNKS_RESOLUTION * 0.5f)) * data.chunkSize;
                vec3 chunkMax = chunkMin + data.chunkSize;
                std::vector<uint32_t> ids;
                for (uint objectIndex = 0; objectIndex < data.objectsCount; objectIndex++) {
                    ObjectBuffer obj = objects[objectIndex];
                    if (boxIntersectsSphere(chunkMin, chunkMax, vec3(obj.objectBounds.xyz), obj.objectBounds.w))
                        ids.push_back(objectIndex);
                }
                if (ids.empty()) continue;
                const uint32_t need = uint32_t(ids.size()) + 1, st = used;
                used += need;
                if (st + need > capacity) continue;
                culled[st] = uint32_t(ids.size());
                for (size_t i = 0; i < ids.size(); ++i) culled[st + 1 + i] = ids[i];
                chunks[chunkAddress] = st;
            }
    if (capacity > 0) culled[0] = used;
    return used > capacity ? LUXGI_ENOMEM : 0;
}

// sampleIrradiance for n points (float3) against float atlases.
int ref_sample_irradiance(const luxgi_ddgi_uniform* u, const float* irr, const float* dist, const float* pos,
                          const float* nrm, const float* wo, float* out, int n) {
    const DDGIUniform ddgi = as<DDGIUniform>(*u);
    const sampler2D irrS = tex2d(irr, nullptr, nullptr, ddgi.irradianceTextureWidth, ddgi.irradianceTextureHeight, 4, true);
    const sampler2D distS = tex2d(dist, nullptr, nullptr, ddgi.depthTextureWidth, ddgi.depthTextureHeight, 2, true);
#pragma omp parallel for
    for (int i = 0; i < n; ++i) {
        vec3 e = sampleIrradiance(ddgi, vec3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                                  vec3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]),
                                  vec3(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), irrS, distS);
        out[3 * i] = e.x;
        out[3 * i + 1] = e.y;
        out[3 * i + 2] = e.z;
    }
    return 0;
}

// CopyEmissive.frag main, then SDFDeferredLight.frag main (:79-129) for each
// light whose bit is set in masks[k] (NULL: all), blended additively into
// the target `out` of the surface's light format (rounded after each draw),
// over tiles[0 .. n).  copy_emissive = 0 skips the CopyEmissive draw.
int ref_surface_light(const luxgi_sdf_desc* sdf, const luxgi_surface_desc* surf, const luxgi_light* lights,
                      int num_lights, const uint32_t* tile_ids, const uint32_t* masks, int n, const float cam[3],
                      float shadow_bias, int copy_emissive, void* out) {
    const int fmt = surf->light_format;
    const GlobalSDFData sd = as<GlobalSDFData>(sdf->data);
    const int C = int(sdf->data.cascades_count), res = sdf->resolution, mres = sdf->mip_resolution;
    const sampler3D tex = volume(sdf->sdf, sdf->format, res * C, res, res);
    const sampler3D mip = volume(sdf->mip, sdf->format, mres * C, mres, mres);
    const int A = int(surf->data.resolution);
    const sampler2D colorS = gbuffer_tex(surf->gbuffer0, surf->gbuffer_format, A, A);
    const sampler2D normalS = gbuffer_tex(surf->gbuffer1, surf->gbuffer_format, A, A);
    const sampler2D pbrS = tex2d(nullptr, nullptr, surf->pbr, A, A, 4, true);
    const sampler2D emissiveS = color_tex(surf->emissive, fmt, A, A, true);
    const TileBuffer* tiles = reinterpret_cast<const TileBuffer*>(surf->tiles);
    for (int k = 0; k < n; ++k) {
        const TileBuffer tile = tiles[tile_ids[k]];
        const Quad q = tile_quad(tile, A);
        const uint32_t mask = masks ? masks[k] : 0xFFFFFFFFu;
#pragma omp parallel for schedule(dynamic)
        for (int j = 0; j < q.height; ++j)
            for (int i = 0; i < q.width; ++i) {
                const size_t ti = size_t(q.y + j) * size_t(A) + size_t(q.x + i);
                const vec2 inTileUV = tile_uv(q, i, j);
                const vec2 atlasUV = inTileUV * vec2(tile.extends.zw) + vec2(tile.extends.xy);
                float dst[4];
                if (copy_emissive) {
                    const vec4 e = surf->emissive ? texture(emissiveS, atlasUV) : vec4(0, 0, 0, 1);
                    dst[0] = e.x; dst[1] = e.y; dst[2] = e.z; dst[3] = e.w;
                    target_round(fmt, dst);
                } else {
                    target_load(out, fmt, ti, dst);
                }
                for (int l = 0; l < num_lights; ++l) {
                    if (!(mask >> l & 1u)) continue;
                    const Light light = as<Light>(lights[l]);
                    vec4 albedo = texture(colorS, atlasUV);
                    vec4 normalTex = texture(normalS, atlasUV);
                    vec4 pbr = surf->pbr ? texture(pbrS, atlasUV) : vec4(0, 1, 0, 1);
                    vec3 normal = octohedralToDirection(vec2(normalTex.xy));
                    vec3 worldPos = vec3(albedo.w, normalTex.z, normalTex.w);
                    vec3 L = vec3(0);
                    float dist = GLOBAL_SDF_WORLD_SIZE;
                    float atten = 1;
                    fetchLight(light, worldPos, normal, L, dist, atten);
                    float shadowMask = 1.0;
                    float NoL = dot(normal, L);
                    float shadowBias = shadow_bias;
                    float bias = 2 * shadowBias * clamp(1 - NoL, 0, 1) + shadowBias;
                    if (NoL > 0) {
                        if (atten > 0) {
                            GlobalSDFTrace trace;
                            trace.worldPosition = worldPos + normal * shadowBias;
                            trace.worldDirection = L;
                            trace.minDistance = bias;
                            trace.maxDistance = dist - bias;
                            trace.stepScale = 1;
                            trace.needsHitNormal = false;
                            GlobalSDFHit hit = tracyGlobalSDF(sd, tex, mip, trace, 2);
                            shadowMask = isHit(hit) ? 0.0 : 1;
                        }
                    } else {
                        shadowMask = 0;
                    }
                    float metallic = pbr.r;
                    float roughness = pbr.g;
                    vec3 view = normalize(vec3(cam[0], cam[1], cam[2]) - worldPos);
                    float intensity = pow(light.intensity, 1.4) + 0.1;
                    vec3 Lradiance = vec3(light.color.xyz) * intensity;
                    vec3 Lh = normalize(L + view);
                    float cosLi = max(0.0, dot(normal, L));
                    vec3 directShading = BRDF(vec3(albedo.rgb), normal, roughness, metallic, view, Lh, L) * Lradiance *
                                         cosLi * shadowMask * atten;
                    dst[0] = dst[0] + directShading.x;
                    dst[1] = dst[1] + directShading.y;
                    dst[2] = dst[2] + directShading.z;
                    dst[3] = dst[3] + 1.0f;
                    target_round(fmt, dst);
                }
                target_store(out, fmt, ti, dst);
            }
    }
    return 0;
}

// SDFAtlasIndirectLight.frag main (:51-67, indirectLighting :44-48) over
// every tile's quad: out = direct_light + the fragment's indirect light,
// rounded to the surface's light format, the additive draw into the light
// cache (texels outside the quads are left as they are).
int ref_inject(const luxgi_ddgi_volume_desc* vd, const luxgi_surface_desc* surf, const float* irr, const float* dist,
               void* out) {
    const DDGIUniform ddgi = as<DDGIUniform>(vd->uniform);
    const int A = int(surf->data.resolution);
    const int fmt = surf->light_format;
    const sampler2D colorS = gbuffer_tex(surf->gbuffer0, surf->gbuffer_format, A, A);
    const sampler2D normalS = gbuffer_tex(surf->gbuffer1, surf->gbuffer_format, A, A);
    const sampler2D pbrS = tex2d(nullptr, nullptr, surf->pbr, A, A, 4, true);
    const sampler2D irrS = tex2d(irr, nullptr, nullptr, ddgi.irradianceTextureWidth, ddgi.irradianceTextureHeight, 4, true);
    const sampler2D distS = tex2d(dist, nullptr, nullptr, ddgi.depthTextureWidth, ddgi.depthTextureHeight, 2, true);
    const TileBuffer* tiles = reinterpret_cast<const TileBuffer*>(surf->tiles);
    const vec3 cam(surf->data.camera_pos[0], surf->data.camera_pos[1], surf->data.camera_pos[2]);
    for (int t = 1; t < surf->num_tiles; ++t) {
        const TileBuffer tile = tiles[t];
        const Quad q = tile_quad(tile, A);
#pragma omp parallel for
        for (int j = 0; j < q.height; ++j)
            for (int i = 0; i < q.width; ++i) {
                const size_t ti = size_t(q.y + j) * size_t(A) + size_t(q.x + i);
                const vec2 atlasUV = tile_uv(q, i, j) * vec2(tile.extends.zw) + vec2(tile.extends.xy);
                SurfaceMaterial p;
                vec4 albedo = texture(colorS, atlasUV);
                vec4 normalTex = texture(normalS, atlasUV);
                vec4 pbr = surf->pbr ? texture(pbrS, atlasUV) : vec4(0, 1, 0, 1);
                p.normal = octohedralToDirection(vec2(normalTex.xy));
                p.albedo = vec4(min(vec3(albedo.xyz), 0.9), 1);
                p.metallic = pbr.r;
                p.roughness = pbr.g;
                vec3 worldPos = vec3(albedo.w, normalTex.z, normalTex.w);
                const vec3 Wo = normalize(cam - worldPos);
                vec3 diffuseColor = (vec3(p.albedo.rgb) - vec3(p.albedo.rgb) * p.metallic) / PI;
                vec3 e = vd->intensity * diffuseColor * sampleIrradiance(ddgi, worldPos, p.normal, Wo, irrS, distS);
                float v[4];
                target_load(surf->direct_light, fmt, ti, v);
                v[0] = v[0] + e.x;
                v[1] = v[1] + e.y;
                v[2] = v[2] + e.z;
                target_store(out, fmt, ti, v);
            }
    }
    return 0;
}

// SDFRasterizeModel.glsl main without READ_DISTANCE (:42-63) for every
// voxel of the given chunks of cascade `cascade`: the ubo (cascadeCoordTo
// PosMul / Add, maxDistance) as GlobalDistanceField.cpp:755-760 fills it,
// the records and mesh volumes as the plan binds them.  sdf (float,
// (res*C) x res x res) is written where the voxel lands in the texture.
int ref_sdf_raster(const luxgi_sdf_build_desc* d, const luxgi_sdf_data* data, int cascade,
                   const luxgi_sdf_raster_object* recs, const int32_t* rec_mesh, const luxgi_sdf_chunk* chunks,
                   int n_chunks, const luxgi_mesh_sdf* meshes, float* sdf) {
    const int res = d->resolution, C = d->cascades;
    const float cd = data->cascade_pos_distance[cascade][3], voxel = data->cascade_voxel_size[cascade];
    vec3 center(data->cascade_pos_distance[cascade][0], data->cascade_pos_distance[cascade][1],
                data->cascade_pos_distance[cascade][2]);
    const vec3 bmin = center - cd, bmax = center + cd;
    const vec3 cascadeCoordToPosMul = (bmax - bmin) / float(res);
    const vec3 cascadeCoordToPosAdd = bmin + voxel * 0.5f;
    const float maxDistance = cd * 2.0f;
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < n_chunks; ++k) {
        const luxgi_sdf_chunk& ch = chunks[k];
        std::vector<sampler3D> tex(size_t(ch.count));
        for (int i = 0; i < ch.count; ++i) {
            const luxgi_mesh_sdf& m = meshes[rec_mesh[ch.models[i]]];
            sampler3D& t = tex[size_t(i)];
            t.levels = m.mip_count;
            for (int L = 0; L < m.mip_count; ++L) {
                t.lv[L] = m.mips[L];
                t.lw[L] = m.size[0] >> L > 0 ? m.size[0] >> L : 1;
                t.lh[L] = m.size[1] >> L > 0 ? m.size[1] >> L : 1;
                t.ld[L] = m.size[2] >> L > 0 ? m.size[2] >> L : 1;
            }
        }
        for (int lz = 0; lz < 32; ++lz)
            for (int ly = 0; ly < 32; ++ly)
                for (int lx = 0; lx < 32; ++lx) {
                    ivec3 voxelCoord = ivec3(ch.coord[0] * 32, ch.coord[1] * 32, ch.coord[2] * 32) + ivec3(lx, ly, lz);
                    vec3 voxelWorldPos = vec3(voxelCoord) * cascadeCoordToPosMul + cascadeCoordToPosAdd;
                    voxelCoord.x += cascade * res;
                    float minDistance = maxDistance;
                    for (int i = 0; i < ch.count; ++i) {
                        const ObjectRasterizeData objectData = as<ObjectRasterizeData>(recs[ch.models[i]]);
                        float objectDistance = distanceToModelSDF(minDistance, objectData, tex[size_t(i)], voxelWorldPos);
                        minDistance = min(minDistance, objectDistance);
                    }
                    const float v = clamp(minDistance / maxDistance, -1, 1);
                    if (voxelCoord.x < 0 || voxelCoord.x >= res * C || voxelCoord.y < 0 || voxelCoord.y >= res ||
                        voxelCoord.z < 0 || voxelCoord.z >= res)
                        continue;
                    sdf[size_t(voxelCoord.x) + size_t(res * C) * (size_t(voxelCoord.y) + size_t(res) * size_t(voxelCoord.z))] = v;
                }
    }
    return 0;
}

// SampleProbe.comp main (:36-60) over a W x H G-buffer: out float4 per pixel.
int ref_sample_probe_image(const luxgi_ddgi_uniform* u, const float* irr, const float* dist, const float* depth,
                           const float* normal, int nch, int W, int H, const float cam[3], const float vpi[16],
                           float* out) {
    const DDGIUniform ddgi = as<DDGIUniform>(*u);
    const sampler2D irrS = tex2d(irr, nullptr, nullptr, ddgi.irradianceTextureWidth, ddgi.irradianceTextureHeight, 4, true);
    const sampler2D distS = tex2d(dist, nullptr, nullptr, ddgi.depthTextureWidth, ddgi.depthTextureHeight, 2, true);
    mat4 viewProjInv;
    for (int c = 0; c < 4; ++c) viewProjInv[c] = vec4(vpi[4 * c], vpi[4 * c + 1], vpi[4 * c + 2], vpi[4 * c + 3]);
    const vec3 cameraPosition(cam[0], cam[1], cam[2]);
#pragma omp parallel for
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t i = size_t(y) * W + x;
            const ivec2 size = ivec2(W, H);
            const ivec2 currentCoord = ivec2(x, y);
            const vec2 pixelCenter = vec2(currentCoord) + vec2(0.5);
            const vec2 texCoord = pixelCenter / vec2(size);
            float d = depth[i];
            vec4 result(0.0f);
            if (d != 1.0f) {
                const vec3 P = worldPositionFromDepth(texCoord, d, viewProjInv);
                const vec3 N = octohedralToDirection(vec2(normal[i * nch], normal[i * nch + 1]));
                const vec3 Wo = normalize(cameraPosition - P);
                vec3 irradiance = sampleIrradiance(ddgi, P, N, Wo, irrS, distS);
                result = vec4(irradiance, 1.0f);
            }
            out[4 * i] = result.x;
            out[4 * i + 1] = result.y;
            out[4 * i + 2] = result.z;
            out[4 * i + 3] = result.w;
        }
    return 0;
}

// sphericalFibonacci under a rotation (GISDFRays.comp:73), float4 [R].
int ref_ray_dirs(const float rot9[9], int R, float* out) {
    mat3 orientation(vec3(rot9[0], rot9[1], rot9[2]), vec3(rot9[3], rot9[4], rot9[5]), vec3(rot9[6], rot9[7], rot9[8]));
    for (int r = 0; r < R; ++r) {
        vec3 d = normalize(orientation * sphericalFibonacci(float(r), float(R)));
        out[4 * r] = d.x; out[4 * r + 1] = d.y; out[4 * r + 2] = d.z; out[4 * r + 3] = 0.0f;
    }
    return 0;
}

}  // extern "C"
