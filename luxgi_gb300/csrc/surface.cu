// Surface-cache raster passes over the pixel footprints of atlas tiles:
// light-cache injection of the probe irradiance (SDFAtlasIndirectLight.frag)
// and SDF-shadowed direct lighting (CopyEmissive.frag, then
// SDFDeferredLight.frag once per light).
//
// The reference draws each tile as a quad (addTiles2,
// Engine/DDGI/GlobalSurfaceAtlas.cpp:554-574) spanning the pixels
// [x, x + w] x [y, y + h], (x, y, w, h) = round(extends * resolution); the
// fragment at pixel (x + i, y + j) samples the surface textures bilinearly
// with REPEAT at ((i + 0.5) / (w + 1), (j + 0.5) / (h + 1)) * extends.zw +
// extends.xy.  Here one thread shades one footprint pixel: there is no
// rasteriser, and the light loop of the per-light draws runs inside the
// thread, rounding the FP16 target after each light as the blend unit does.
//
// Compiled without FMA contraction: the shadow march then takes exactly the
// oracle's steps and the blocked / lit decision of every fragment matches.
#include <cmath>

#include "luxgi_internal.h"

#include "luxgi_common.cuh"

namespace luxgi {

namespace {

struct Footprint {
    int x0, y0, w, h;   // w, h: pixels of the quad
};

__device__ __forceinline__ Footprint footprint(const luxgi_surface_tile* tl, int res) {
    Footprint f;
    f.x0 = int(lrintf(__ldg(&tl->extends[0]) * float(res)));
    f.y0 = int(lrintf(__ldg(&tl->extends[1]) * float(res)));
    f.w = int(lrintf(__ldg(&tl->extends[2]) * float(res))) + 1;
    f.h = int(lrintf(__ldg(&tl->extends[3]) * float(res))) + 1;
    return f;
}

// atlasUV of the fragment at footprint pixel (i, j)
__device__ __forceinline__ void fragment_uv(const luxgi_surface_tile* tl, const Footprint& f, int i, int j, float& u,
                                            float& v) {
    const float tu = (float(i) + 0.5f) / float(f.w), tv = (float(j) + 0.5f) / float(f.h);
    u = tu * __ldg(&tl->extends[2]) + __ldg(&tl->extends[0]);
    v = tv * __ldg(&tl->extends[3]) + __ldg(&tl->extends[1]);
}

// RGBA8 UNORM texel, channels 0 and 1 (metallic, roughness)
__device__ __forceinline__ void unorm_rg(const uint8_t* p, size_t texel, float* out) {
    const uchar4 q = __ldg(reinterpret_cast<const uchar4*>(p) + texel);
    out[0] = float(q.x) / 255.0f;
    out[1] = float(q.y) / 255.0f;
}

// Bilinear REPEAT sample of the PBR texture's metallic and roughness (the
// per-channel arithmetic of bilinear_repeat).
__device__ __forceinline__ void sample_pbr(const uint8_t* p, int W, int H, float u, float v, float& metallic,
                                           float& roughness) {
    const float x = u * float(W) - 0.5f, y = v * float(H) - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const int i0 = wrap_repeat(int(fx), W), i1 = wrap_repeat(int(fx) + 1, W);
    const int j0 = wrap_repeat(int(fy), H), j1 = wrap_repeat(int(fy) + 1, H);
    float t00[2], t10[2], t01[2], t11[2], o[2];
    unorm_rg(p, size_t(j0) * W + i0, t00);
    unorm_rg(p, size_t(j0) * W + i1, t10);
    unorm_rg(p, size_t(j1) * W + i0, t01);
    unorm_rg(p, size_t(j1) * W + i1, t11);
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const float r0 = t00[c] * (1.0f - a) + t10[c] * a, r1 = t01[c] * (1.0f - a) + t11[c] * a;
        o[c] = r0 * (1.0f - b) + r1 * b;
    }
    metallic = o[0];
    roughness = o[1];
}

// octohedralToDirection (Common/Math.glsl:26-32)
__device__ __forceinline__ f3 oct_to_dir(float ex, float ey) {
    f3 v{ex, ey, 1.0f - fabsf(ex) - fabsf(ey)};
    if (v.z < 0.0f) {
        const float nx = (1.0f - fabsf(v.y)) * sign_nz(v.x);
        const float ny = (1.0f - fabsf(v.x)) * sign_nz(v.y);
        v.x = nx;
        v.y = ny;
    }
    return norm3(v);
}

// The surface G-buffer at a fragment (SDFDeferredLight.frag:83-87, :120-121;
// no PBR texture reads as metallic 0, roughness 1).
struct Fragment {
    f3 albedo, pos, normal;
    float metallic, roughness;
};

// gb_storage: LUXGI_STORAGE_FP32 for RGBA32F G-buffers, LUXGI_STORAGE_FP16
// for RGBA16F ones (the texels are widened to FP32 before the filter).
__device__ __forceinline__ Fragment surface_fragment(const void* gb0, const void* gb1, int gb_storage,
                                                     const uint8_t* pbr, int res, float u, float v) {
    float g0[4], g1[4];
    bilinear_repeat_v<4>(gb0, gb_storage, res, res, u, v, g0);
    bilinear_repeat_v<4>(gb1, gb_storage, res, res, u, v, g1);
    Fragment f;
    f.albedo = f3{g0[0], g0[1], g0[2]};
    f.pos = f3{g0[3], g1[2], g1[3]};
    f.normal = oct_to_dir(g1[0], g1[1]);
    if (pbr) {
        sample_pbr(pbr, res, res, u, v, f.metallic, f.roughness);
    } else {
        f.metallic = 0.0f;
        f.roughness = 1.0f;
    }
    return f;
}

// textureLod bilinear with REPEAT of a surface colour texture, rgba (the
// per-channel arithmetic of bilinear_repeat; alpha 1 for R11G11B10F).
__device__ __forceinline__ void bilinear_color_repeat(const void* p, int fmt, int W, int H, float u, float v,
                                                      float* out) {
    const float x = u * float(W) - 0.5f, y = v * float(H) - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const int i0 = wrap_repeat(int(fx), W), i1 = wrap_repeat(int(fx) + 1, W);
    const int j0 = wrap_repeat(int(fy), H), j1 = wrap_repeat(int(fy) + 1, H);
    float t00[4], t10[4], t01[4], t11[4];
    color_texel_ro(p, fmt, size_t(j0) * W + i0, t00);
    color_texel_ro(p, fmt, size_t(j0) * W + i1, t10);
    color_texel_ro(p, fmt, size_t(j1) * W + i0, t01);
    color_texel_ro(p, fmt, size_t(j1) * W + i1, t11);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float r0 = t00[c] * (1.0f - a) + t10[c] * a, r1 = t01[c] * (1.0f - a) + t11[c] * a;
        out[c] = r0 * (1.0f - b) + r1 * b;
    }
}

// ------------------------------------------------------------- inject
// SDFAtlasIndirectLight.frag:44-67 over the footprint of every tile: the
// light cache becomes direct light plus intensity * (a - a * metallic)/pi *
// sampleIrradiance(previous atlases), a = min(albedo, 0.9).  One block row
// per tile.
// `direct` and `light` may be one texture: each texel is read and written by
// the one thread of its footprint pixel (tiles do not overlap).
__global__ void inject_kernel(const luxgi_ddgi_uniform u, const SurfaceView s, const void* __restrict__ gb0,
                              const void* __restrict__ gb1, int gb_storage, const uint8_t* __restrict__ pbr,
                              const void* direct, void* light, int light_format, const AtlasView A, float intensity,
                              int bounce) {
    const luxgi_surface_tile* tl = s.tiles + (blockIdx.y + 1);   // tile slot 0 is "no tile"
    const int res = int(s.data.resolution);
    const Footprint fp = footprint(tl, res);
    const int n = fp.w * fp.h;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k % fp.w, j = k / fp.w;
        const int px = fp.x0 + i, py = fp.y0 + j;
        if (px < 0 || px >= res || py < 0 || py >= res) continue;
        const size_t ti = size_t(py) * res + px;
        float add[3] = {0.0f, 0.0f, 0.0f};
        if (bounce) {
            float uu, vv;
            fragment_uv(tl, fp, i, j, uu, vv);
            const Fragment f = surface_fragment(gb0, gb1, gb_storage, pbr, res, uu, vv);
            const f3 cam{s.data.camera_pos[0], s.data.camera_pos[1], s.data.camera_pos[2]};
            const f3 wo = norm3(sub3(cam, f.pos));
            const f3 e = sample_irradiance(u, A, f.pos, f.normal, wo);
            const float alb[3] = {mn(f.albedo.x, 0.9f), mn(f.albedo.y, 0.9f), mn(f.albedo.z, 0.9f)};
            const float ev[3] = {e.x, e.y, e.z};
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const float diff = (alb[c] - alb[c] * f.metallic) / kPi;
                add[c] = intensity * diff * ev[c];
            }
        }
        float v[4];
        color_texel(direct, light_format, ti, v);
#pragma unroll
        for (int c = 0; c < 3; ++c) v[c] = v[c] + add[c];
        color_store(light, light_format, ti, v);
    }
}

// ---------------------------------------------------- direct lighting
// Raytraced/BRDF.glsl:65-81 (GGX distribution :14-21, Schlick-GGX geometry
// with k = (r + 1)^2 / 8 :24-35, Schlick Fresnel :38-41).
__device__ __forceinline__ f3 brdf(f3 albedo, f3 n, float roughness, float metallic, f3 view, f3 half_v, f3 l) {
    const float f0[3] = {0.04f * (1.0f - metallic) + albedo.x * metallic,
                         0.04f * (1.0f - metallic) + albedo.y * metallic,
                         0.04f * (1.0f - metallic) + albedo.z * metallic};
    const float cos_li = mx(0.0f, dot3(n, l));
    const float cos_lh = mx(0.0f, dot3(n, half_v));
    const float n_dot_v = mx(0.0f, dot3(n, view));
    // pow(x, 5) of fresnelSchlick as (x^2)^2 x: within 3 ulps of the exact power
    const float fx = clampf(1.0f - mx(dot3(half_v, view), 0.0f), 0.0f, 1.0f);
    const float fx2 = fx * fx;
    const float fw = fx2 * fx2 * fx;
    const float alpha = roughness * roughness;
    const float alpha_sq = alpha * alpha;
    const float denom = (cos_lh * cos_lh) * (alpha_sq - 1.0f) + 1.0f;
    const float D = alpha_sq / (kPi * denom * denom);
    const float r = roughness + 1.0f;
    const float k = (r * r) / 8.0f;
    const float G = (cos_li / (cos_li * (1.0f - k) + k)) * (n_dot_v / (n_dot_v * (1.0f - k) + k));
    const float den = mx(0.00001f, 4.0f * cos_li * n_dot_v);
    const float km = 1.0f - metallic;
    const float av[3] = {albedo.x, albedo.y, albedo.z};
    float out[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float F = f0[c] + (1.0f - f0[c]) * fw;
        const float kd = (1.0f - F) * km;
        const float diffuse = kd * av[c] / kPi;
        const float specular = (F * D * G) / den;
        out[c] = diffuse + specular;
    }
    return f3{out[0], out[1], out[2]};
}

// The launch's copy of the lights; color[3] (unused by the shader) carries
// the per-light radiance factor pow(intensity, 1.4) + 0.1
// (SDFDeferredLight.frag:124), evaluated once on the host.
struct LightSet {
    luxgi_light l[LUXGI_MAX_LIGHTS];
};

// SDFDeferredLight.frag:41-129 for one fragment and one light: the light's
// contribution (rgb) to the light cache.
template <typename T>
__device__ __forceinline__ f3 direct_light(const SdfView& sdf, const Fragment& f, const luxgi_light& L, f3 cam,
                                           float sb, int max_steps) {
    // fetchLight (:41-76)
    f3 wi{0.0f, 0.0f, 0.0f};
    float dist = kWorldSize, atten = 1.0f;
    if (L.type == 0.0f) {
        wi = f3{-L.direction[0], -L.direction[1], -L.direction[2]};
    } else if (L.type == 2.0f) {
        const f3 d = sub3(f3{L.position[0], L.position[1], L.position[2]}, f.pos);
        dist = len3(d);
        wi = norm3(d);
        atten = L.radius / (dist * dist + 1.0f);
    } else {
        const f3 lv = sub3(f3{L.position[0], L.position[1], L.position[2]}, f.pos);
        const float cutoff = 1.0f - L.angle;
        wi = norm3(lv);
        dist = len3(lv);
        const float theta = dot3(wi, f3{L.direction[0], L.direction[1], L.direction[2]});
        const float eps = cutoff - cutoff * 0.9f;
        float a = (theta - cutoff) / eps;
        a = a * (L.radius / (dist * dist + 1.0f));
        atten = clampf(a, 0.0f, 1.0f);
    }
    // SDF shadow (:95-118)
    float shadow = 1.0f;
    const float nol = dot3(f.normal, wi);
    const float bias = 2.0f * sb * clampf(1.0f - nol, 0.0f, 1.0f) + sb;
    if (nol > 0.0f) {
        if (atten > 0.0f) {
            MarchState m;
            march_state_init(m);
            MarchHit hit;
            // one step loop with the corrected quotients: the pass ran 1.10 ms
            // with an IEEE division a step and 1.12 ms with the loop compiled
            // twice (registers), 1.03 ms so
            march_run<T, kPlain, kPlain, kDivExact>(sdf, add3(f.pos, mul3(f.normal, sb)), wi, dist - bias, max_steps,
                                                    m, 0x7FFFFFFF, hit, 2.0f);
            shadow = hit.time >= 0.0f ? 0.0f : 1.0f;
        }
    } else {
        shadow = 0.0f;
    }
    // shading (:120-128)
    const f3 view = norm3(sub3(cam, f.pos));
    const float intensity = L.color[3];
    const f3 lrad{L.color[0] * intensity, L.color[1] * intensity, L.color[2] * intensity};
    const f3 lh = norm3(add3(wi, view));
    const float cos_li = mx(0.0f, dot3(f.normal, wi));
    const f3 b = brdf(f.albedo, f.normal, f.roughness, f.metallic, view, lh, wi);
    const float s = cos_li * shadow * atten;
    return f3{b.x * lrad.x * s, b.y * lrad.y * s, b.z * lrad.z * s};
}

struct LightPass {
    SdfView sdf;
    const luxgi_surface_tile* tiles;
    int num_surface_tiles;
    int res;
    const void* gb0;
    const void* gb1;
    int gb_storage;            // LUXGI_STORAGE_FP32 / FP16 G-buffer texels
    int light_format;          // luxgi_color_format of emissive and out
    const uint8_t* pbr;
    const void* emissive;
    const uint32_t* list;      // tile addresses
    const uint32_t* masks;     // per listed tile, or nullptr
    void* out;
    float cam[3];
    float shadow_bias;
    int num_lights;
    int copy_emissive;
    int max_steps;
};

// One block row per listed tile; the block's threads stride over the tile's
// footprint.  The light set arrives in the launch parameters and is staged
// in shared memory.
template <typename T>
__global__ void __launch_bounds__(128) surface_light_kernel(const LightPass p, const LightSet ls) {
    __shared__ luxgi_light sl[LUXGI_MAX_LIGHTS];
    for (int i = threadIdx.x; i < p.num_lights; i += blockDim.x) sl[i] = ls.l[i];
    __syncthreads();
    const uint32_t t = __ldg(p.list + blockIdx.y);
    if (t < 1u || t >= uint32_t(p.num_surface_tiles)) return;
    const uint32_t all = p.num_lights >= 32 ? 0xFFFFFFFFu : ((1u << p.num_lights) - 1u);
    const uint32_t mask = (p.masks ? __ldg(p.masks + blockIdx.y) : 0xFFFFFFFFu) & all;
    const luxgi_surface_tile* tl = p.tiles + t;
    const Footprint fp = footprint(tl, p.res);
    const int n = fp.w * fp.h;
    const f3 cam{p.cam[0], p.cam[1], p.cam[2]};
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const int i = k % fp.w, j = k / fp.w;
        const int px = fp.x0 + i, py = fp.y0 + j;
        if (px < 0 || px >= p.res || py < 0 || py >= p.res) continue;
        const size_t ti = size_t(py) * p.res + px;
        float uu, vv;
        fragment_uv(tl, fp, i, j, uu, vv);
        float acc[4];
        if (p.copy_emissive) {
            if (p.emissive) {
                bilinear_color_repeat(p.emissive, p.light_format, p.res, p.res, uu, vv, acc);
                color_round(p.light_format, acc);
            } else {
                acc[0] = acc[1] = acc[2] = 0.0f;
                acc[3] = 1.0f;
            }
        } else {
            color_texel(p.out, p.light_format, ti, acc);
        }
        if (mask) {
            const Fragment f = surface_fragment(p.gb0, p.gb1, p.gb_storage, p.pbr, p.res, uu, vv);
            for (uint32_t m = mask; m; m &= m - 1u) {
                const int l = __ffs(int(m)) - 1;
                const f3 d = direct_light<T>(p.sdf, f, sl[l], cam, p.shadow_bias, p.max_steps);
                acc[0] = acc[0] + d.x;
                acc[1] = acc[1] + d.y;
                acc[2] = acc[2] + d.z;
                acc[3] = acc[3] + 1.0f;
                color_round(p.light_format, acc);
            }
        }
        color_store(p.out, p.light_format, ti, acc);
    }
}

}  // namespace

int gbuffer_storage(int gbuffer_format) {
    return gbuffer_format == LUXGI_GBUFFER_RGBA16F ? LUXGI_STORAGE_FP16 : LUXGI_STORAGE_FP32;
}

cudaError_t launch_inject(const luxgi_ddgi_uniform& u, const SurfaceView& s, const void* gb0, const void* gb1,
                          int gbuffer_format, const uint8_t* pbr, const void* direct, void* light, int light_format,
                          const AtlasView& A, int num_tiles, float intensity, int bounce, cudaStream_t st) {
    if (num_tiles <= 1) return cudaSuccess;
    dim3 grid(8, unsigned(num_tiles - 1));
    inject_kernel<<<grid, 256, 0, st>>>(u, s, gb0, gb1, gbuffer_storage(gbuffer_format), pbr, direct, light,
                                        light_format, A, intensity, bounce);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_surface_light(const SdfView& sdf, const luxgi_surface_desc& s, const luxgi_surface_lighting& L,
                                 void* out, cudaStream_t st) {
    if (L.num_tiles <= 0) return cudaSuccess;
    LightPass p;
    p.sdf = sdf;
    p.tiles = s.tiles;
    p.num_surface_tiles = s.num_tiles;
    p.res = int(s.data.resolution);
    p.gb0 = s.gbuffer0;
    p.gb1 = s.gbuffer1;
    p.gb_storage = gbuffer_storage(s.gbuffer_format);
    p.light_format = s.light_format;
    p.pbr = s.pbr;
    p.emissive = s.emissive;
    p.list = L.tiles;
    p.masks = L.light_masks;
    p.out = out;
    p.cam[0] = L.camera_pos[0];
    p.cam[1] = L.camera_pos[1];
    p.cam[2] = L.camera_pos[2];
    p.shadow_bias = L.shadow_bias;
    p.num_lights = L.num_lights;
    p.copy_emissive = L.copy_emissive;
    p.max_steps = L.max_steps;
    LightSet ls;
    for (int i = 0; i < LUXGI_MAX_LIGHTS; ++i) {
        ls.l[i] = i < L.num_lights ? L.lights[i] : luxgi_light{};
        ls.l[i].color[3] = std::pow(ls.l[i].intensity, 1.4f) + 0.1f;
    }
    // a tile of the reference's atlas is at most 128 x 128 pixels: 8 blocks of
    // 128 threads give every thread ~16 pixels there and one on an 32 x 32 tile
    const dim3 grid(8, unsigned(L.num_tiles));
    if (sdf.format == LUXGI_STORAGE_FP16)
        surface_light_kernel<__half><<<grid, 128, 0, st>>>(p, ls);
    else
        surface_light_kernel<float><<<grid, 128, 0, st>>>(p, ls);
    note_launch();
    return cudaGetLastError();
}

}  // namespace luxgi
