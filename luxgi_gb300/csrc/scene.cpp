// Seeded synthetic scene inputs for the DDGI probe-update path (host, C++17).
//
// See include/luxgi_scene.h for what is built and which reference passes the
// layouts follow.  Compiled with -ffp-contract=off: the SDF voxels and atlas
// texels are bit-identical on x86-64 and aarch64.
#include "luxgi_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

namespace {

// ------------------------------------------------------------------ RNG
// splitmix64 seeding a xoshiro256** generator (Vigna & Blackman).
struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) s[i] = splitmix(x);
    }
    static uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
    uint64_t next() {
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return r;
    }
    float uniform() { return float(next() >> 40) * (1.0f / 16777216.0f); }   // [0,1)
    float uniform(float a, float b) { return a + (b - a) * uniform(); }
};

struct V3 { float x, y, z; };
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) { float inv = 1.0f / length(a); return a * inv; }
inline V3 vabs(V3 a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
inline V3 vmax(V3 a, float m) { return {std::max(a.x, m), std::max(a.y, m), std::max(a.z, m)}; }

// Exact signed distance to an axis-aligned box (centre c, half extents h).
inline float sd_box(V3 p, V3 c, V3 h) {
    V3 q = vabs(p - c) - h;
    V3 qp = vmax(q, 0.0f);
    float outside = length(qp);
    float inside = std::min(std::max(q.x, std::max(q.y, q.z)), 0.0f);
    return outside + inside;
}

inline float sd_prim(const luxgi_scene_primitive& pr, V3 p) {
    V3 c{pr.center[0], pr.center[1], pr.center[2]};
    if (pr.kind == 0) return length(p - c) - pr.half_extent[0];
    return sd_box(p, c, {pr.half_extent[0], pr.half_extent[1], pr.half_extent[2]});
}

// Math.glsl:21-25 directionToOctohedral (G-buffer normal encoding).
inline void dir_to_oct(V3 n, float out[2]) {
    float inv = 1.0f / (std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z));
    float px = n.x * inv, py = n.y * inv;
    if (n.z > 0.0f) { out[0] = px; out[1] = py; return; }
    float sx = px >= 0.0f ? 1.0f : -1.0f;   // step(0,p)*2-1
    float sy = py >= 0.0f ? 1.0f : -1.0f;
    out[0] = (1.0f - std::fabs(py)) * sx;
    out[1] = (1.0f - std::fabs(px)) * sy;
}

}  // namespace

// -------------------------------------------------------- half conversion
extern "C" uint16_t luxgi_float_to_half(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t absx = x & 0x7FFFFFFFu;
    if (absx >= 0x7F800000u) {                       // inf / nan
        return uint16_t(sign | 0x7C00u | (absx > 0x7F800000u ? 0x200u : 0u));
    }
    if (absx >= 0x477FF000u) return uint16_t(sign | 0x7C00u);   // overflow -> inf
    if (absx < 0x38800000u) {                        // subnormal half or zero
        if (absx < 0x33000000u) return uint16_t(sign);          // < 2^-25 -> 0
        uint32_t e = absx >> 23;
        uint32_t m = (absx & 0x7FFFFFu) | 0x800000u;
        uint32_t shift = 126u - e;                   // 14..24
        uint32_t h = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (h & 1u))) ++h;
        return uint16_t(sign | h);
    }
    uint32_t h = ((absx - 0x38000000u) >> 13);
    uint32_t rem = absx & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return uint16_t(sign | h);
}

extern "C" float luxgi_half_to_float(uint16_t h) {
    uint32_t sign = uint32_t(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1Fu;
    uint32_t m = h & 0x3FFu;
    uint32_t x;
    if (e == 0) {
        if (m == 0) {
            x = sign;
        } else {
            int sh = 0;
            while (!(m & 0x400u)) { m <<= 1; ++sh; }
            m &= 0x3FFu;
            x = sign | (uint32_t(113 - sh) << 23) | (m << 13);
        }
    } else if (e == 31) {
        x = sign | 0x7F800000u | (m << 13);
    } else {
        x = sign | ((e + 112u) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &x, 4);
    return f;
}

// ------------------------------------------------------------------ scene
struct luxgi_scene {
    luxgi_scene_config cfg;
    luxgi_sdf_data sdf_data;
    int res = 0, mres = 0, C = 1;
    std::vector<float> sdf32;
    std::vector<uint16_t> sdf16;
    luxgi_surface_data surface_data;
    std::vector<luxgi_surface_object> objects;
    std::vector<luxgi_surface_tile> tiles;
    int atlas = 0;
    std::vector<uint16_t> direct;
    std::vector<float> depth;
    std::vector<uint8_t> albedo;
    std::vector<float> gb0, gb1;
    std::vector<uint8_t> pbr;                   // RGBA8: metallic, roughness, 0, 1
    std::vector<uint16_t> emissive;             // RGBA16F
    std::vector<luxgi_scene_primitive> prims;   // spheres/boxes then walls
    int n_solid = 0;                            // spheres + boxes
    float wall_half_inner = 0.0f;
    V3 sun{0, 1, 0}, sun_color{1, 1, 1};
};

namespace {

float scene_distance(const luxgi_scene& s, V3 p) {
    // walls: positive inside the room interior box
    float a = s.wall_half_inner;
    float d = -sd_box(p, {0, 0, 0}, {a, a, a});
    for (int i = 0; i < s.n_solid; ++i) {
        const auto& pr = s.prims[size_t(i)];
        V3 c{pr.center[0], pr.center[1], pr.center[2]};
        V3 dd = p - c;
        float rho = std::max(pr.half_extent[0], std::max(pr.half_extent[1], pr.half_extent[2]));
        if (pr.kind == 1) rho = length({pr.half_extent[0], pr.half_extent[1], pr.half_extent[2]});
        float bound = d + rho;                       // prim distance >= |p-c| - rho
        if (bound > 0.0f && dot(dd, dd) >= bound * bound) continue;
        d = std::min(d, sd_prim(pr, p));
    }
    return d;
}

void build_sdf(luxgi_scene& s) {
    const float scales[4] = {1.0f, 2.5f, 5.0f, 10.0f};
    const int C = s.C, res = s.res;
    const float outer_half = 0.5f * s.cfg.room_size;
    std::memset(&s.sdf_data, 0, sizeof(s.sdf_data));
    s.sdf_data.cascades_count = uint32_t(C);
    s.sdf_data.resolution = float(res);
    for (int k = 0; k < C; ++k) {
        float half = outer_half * (scales[k] / scales[C - 1]);
        s.sdf_data.cascade_pos_distance[k][0] = 0.0f;
        s.sdf_data.cascade_pos_distance[k][1] = 0.0f;
        s.sdf_data.cascade_pos_distance[k][2] = 0.0f;
        s.sdf_data.cascade_pos_distance[k][3] = half;
        s.sdf_data.cascade_voxel_size[k] = (2.0f * half) / float(res);
    }
    const int64_t W = int64_t(res) * C;
    const int64_t n = W * res * res;
    const bool fp16 = s.cfg.sdf_format == LUXGI_STORAGE_FP16;
    if (fp16) s.sdf16.assign(size_t(n), 0); else s.sdf32.assign(size_t(n), 0.0f);
    for (int k = 0; k < C; ++k) {
        const float half = s.sdf_data.cascade_pos_distance[k][3];
        const float voxel = s.sdf_data.cascade_voxel_size[k];
        const float maxd = 2.0f * half;              // cascadeMaxDistance
        const float mn = -half;
#pragma omp parallel for schedule(dynamic, 1)
        for (int z = 0; z < res; ++z) {
            for (int y = 0; y < res; ++y) {
                for (int x = 0; x < res; ++x) {
                    V3 p{mn + (float(x) + 0.5f) * voxel, mn + (float(y) + 0.5f) * voxel,
                         mn + (float(z) + 0.5f) * voxel};
                    float d = std::min(scene_distance(s, p), maxd);
                    float v = std::min(std::max(d / maxd, -1.0f), 1.0f);
                    int64_t idx = (int64_t(k) * res + x) + W * (int64_t(y) + int64_t(res) * z);
                    if (fp16) s.sdf16[size_t(idx)] = luxgi_float_to_half(v);
                    else s.sdf32[size_t(idx)] = v;
                }
            }
        }
    }
}

// Tile view rotation for card `i` (GlobalSurfaceAtlas.cpp:252-279): a
// lookAt from the face towards the object centre; rows s, u, -f.
void tile_axes(int i, V3& s, V3& u, V3& f) {
    V3 z{0, 0, 0};
    float sign = (i & 1) ? 1.0f : -1.0f;
    if (i / 2 == 0) z.x = sign; else if (i / 2 == 1) z.y = sign; else z.z = sign;
    V3 up = (i == 2 || i == 3) ? V3{1, 0, 0} : V3{0, 1, 0};
    f = normalize(z);
    s = normalize(cross(f, up));
    u = cross(s, f);
}

int build_surface(luxgi_scene& s) {
    const int nobj = int(s.prims.size());
    const int ntiles = 6 * nobj;
    const int res = s.cfg.atlas_resolution;
    int per_row = int(std::ceil(std::sqrt(double(ntiles))));
    int tr = s.cfg.tile_resolution;
    if (tr <= 0) {
        tr = ((res - 2) / per_row) / 8 * 8;
        tr = std::min(tr, 128);
    }
    if (tr < 8 || per_row * tr + 2 > res) return LUXGI_EINVAL;
    s.atlas = res;
    const size_t texels = size_t(res) * size_t(res);
    s.direct.assign(texels * 4, 0);
    s.depth.assign(texels, 1.0f);
    s.albedo.assign(texels * 4, 0);
    s.gb0.assign(texels * 4, 0.0f);
    s.gb1.assign(texels * 4, 0.0f);
    s.pbr.assign(texels * 4, 0);
    s.emissive.assign(texels * 4, 0);
    for (size_t i = 0; i < texels; ++i) s.emissive[i * 4 + 3] = luxgi_float_to_half(1.0f);   // R11G11B10 reads a = 1
    // materials from a stream of their own, so that the geometry and albedo
    // draws stay those of scenes built without them: solids get metallic in
    // [0, 0.6) and roughness in [0.25, 1); every seventh solid (3, 10, ...)
    // emits 1.5 x its albedo; walls are rough dielectrics
    Rng mrng(s.cfg.seed ^ 0x6D6174657269616Cull);
    std::vector<float> metal(size_t(nobj), 0.0f), rough(size_t(nobj), 0.9f), emit(size_t(nobj), 0.0f);
    for (int o = 0; o < nobj; ++o) {
        const float m = mrng.uniform(0.0f, 0.6f), r = mrng.uniform(0.25f, 1.0f);
        if (s.prims[size_t(o)].kind == 2) continue;
        metal[size_t(o)] = m;
        rough[size_t(o)] = r;
        if (o % 7 == 3) emit[size_t(o)] = 1.5f;
    }

    s.objects.assign(size_t(nobj), luxgi_surface_object{});
    s.tiles.assign(size_t(ntiles + 1), luxgi_surface_tile{});   // slot 0 = no tile
    for (int o = 0; o < nobj; ++o) {
        const auto& pr = s.prims[size_t(o)];
        V3 c{pr.center[0], pr.center[1], pr.center[2]};
        V3 e{pr.half_extent[0], pr.half_extent[1], pr.half_extent[2]};
        luxgi_surface_object& ob = s.objects[size_t(o)];
        std::memset(&ob, 0, sizeof(ob));
        ob.object_bounds[0] = c.x; ob.object_bounds[1] = c.y; ob.object_bounds[2] = c.z;
        ob.object_bounds[3] = length(e);             // sphere around the AABB
        for (int k = 0; k < 16; ++k) ob.transform[k] = (k % 5 == 0) ? 1.0f : 0.0f;
        ob.transform[12] = c.x; ob.transform[13] = c.y; ob.transform[14] = c.z;
        ob.extends[0] = e.x; ob.extends[1] = e.y; ob.extends[2] = e.z; ob.extends[3] = 1.0f;
        V3 ext = vmax(e, 0.05f);
        for (int i = 0; i < 6; ++i) {
            const int t = o * 6 + i;
            const int addr = t + 1;
            ob.tile_offset[i] = uint32_t(addr);
            V3 sx, uy, f;
            tile_axes(i, sx, uy, f);
            luxgi_surface_tile& tl = s.tiles[size_t(addr)];
            // column-major rotation with rows s, u, -f; translation zeroed
            float R[3][3] = {{sx.x, sx.y, sx.z}, {uy.x, uy.y, uy.z}, {-f.x, -f.y, -f.z}};
            for (int col = 0; col < 4; ++col)
                for (int row = 0; row < 4; ++row)
                    tl.transform[col * 4 + row] =
                        (col < 3 && row < 3) ? R[row][col] : (col == 3 && row == 3 ? 1.0f : 0.0f);
            V3 b{std::fabs(dot(sx, ext)) * 2.0f, std::fabs(dot(uy, ext)) * 2.0f,
                 std::fabs(dot(f, ext)) * 2.0f};
            tl.object_bounds[0] = b.x; tl.object_bounds[1] = b.y; tl.object_bounds[2] = b.z;
            tl.object_bounds[3] = 0.0f;
            const int tx0 = 1 + (t % per_row) * tr;
            const int ty0 = 1 + (t / per_row) * tr;
            tl.extends[0] = float(tx0) / float(res);
            tl.extends[1] = float(ty0) / float(res);
            tl.extends[2] = float(tr - 1) / float(res);
            tl.extends[3] = float(tr - 1) / float(res);
            // card texels
            for (int j = 0; j < tr; ++j) {
                for (int ii = 0; ii < tr; ++ii) {
                    float ut = (float(ii) + 0.5f) / float(tr - 1);
                    float vt = (float(j) + 0.5f) / float(tr - 1);
                    float px = (ut - 0.5f) * b.x, py = (vt - 0.5f) * b.y;
                    bool hit = false;
                    float tz = 0.0f;
                    V3 nrm{0, 0, 0};
                    if (pr.kind == 0) {
                        float r = e.x;
                        float rho2 = px * px + py * py;
                        if (rho2 <= r * r) {
                            tz = std::sqrt(r * r - rho2);
                            hit = true;
                        }
                    } else if (std::fabs(px) <= 0.5f * b.x && std::fabs(py) <= 0.5f * b.y) {
                        tz = 0.5f * b.z;
                        hit = true;
                    }
                    const size_t ti = size_t(ty0 + j) * size_t(res) + size_t(tx0 + ii);
                    if (!hit) continue;
                    V3 local = sx * px + uy * py - f * tz;
                    if (pr.kind == 0) nrm = normalize(local);
                    else nrm = f * -1.0f;
                    V3 w = c + local;
                    s.depth[ti] = tz / b.z;
                    float alb[3];
                    for (int q = 0; q < 3; ++q) {
                        int a8 = int(std::lround(std::min(std::max(pr.albedo[q], 0.0f), 1.0f) * 255.0f));
                        s.albedo[ti * 4 + size_t(q)] = uint8_t(a8);
                        alb[q] = float(a8) / 255.0f;
                    }
                    s.albedo[ti * 4 + 3] = 255;
                    s.pbr[ti * 4 + 0] = uint8_t(std::lround(metal[size_t(o)] * 255.0f));
                    s.pbr[ti * 4 + 1] = uint8_t(std::lround(rough[size_t(o)] * 255.0f));
                    s.pbr[ti * 4 + 3] = 255;
                    for (int q = 0; q < 3; ++q)
                        s.emissive[ti * 4 + size_t(q)] = luxgi_float_to_half(alb[q] * emit[size_t(o)]);
                    s.emissive[ti * 4 + 3] = luxgi_float_to_half(1.0f);
                    float ndl = std::max(dot(nrm, s.sun), 0.0f);
                    float sc[3] = {s.sun_color.x, s.sun_color.y, s.sun_color.z};
                    for (int q = 0; q < 3; ++q)
                        s.direct[ti * 4 + size_t(q)] = luxgi_float_to_half(alb[q] * sc[q] * ndl);
                    s.direct[ti * 4 + 3] = luxgi_float_to_half(1.0f);
                    float oct[2];
                    dir_to_oct(nrm, oct);
                    s.gb0[ti * 4 + 0] = alb[0]; s.gb0[ti * 4 + 1] = alb[1];
                    s.gb0[ti * 4 + 2] = alb[2]; s.gb0[ti * 4 + 3] = w.x;
                    s.gb1[ti * 4 + 0] = oct[0]; s.gb1[ti * 4 + 1] = oct[1];
                    s.gb1[ti * 4 + 2] = w.y;    s.gb1[ti * 4 + 3] = w.z;
                }
            }
        }
    }
    std::memset(&s.surface_data, 0, sizeof(s.surface_data));
    s.surface_data.chunk_size = s.cfg.room_size / 40.0f;   // giDistance / 40
    s.surface_data.resolution = uint32_t(res);
    s.surface_data.objects_count = uint32_t(nobj);
    s.surface_data.culled_objects_capacity = 0;              // set by caller
    return LUXGI_OK;
}

}  // namespace

extern "C" int luxgi_scene_build(const luxgi_scene_config* cfg, luxgi_scene** out) {
    if (!cfg || !out) return LUXGI_EINVAL;
    *out = nullptr;
    if (cfg->room_size <= 0.0f || cfg->wall_thickness < 0.0f || cfg->num_primitives < 0 ||
        cfg->sdf_resolution < 4 || (cfg->sdf_resolution % 4) != 0 || cfg->cascades < 1 ||
        cfg->cascades > 4 || cfg->atlas_resolution < 16 ||
        (cfg->sdf_format != LUXGI_STORAGE_FP32 && cfg->sdf_format != LUXGI_STORAGE_FP16))
        return LUXGI_EINVAL;
    luxgi_scene* s = new (std::nothrow) luxgi_scene();
    if (!s) return LUXGI_ENOMEM;
    s->cfg = *cfg;
    s->res = cfg->sdf_resolution;
    s->mres = cfg->sdf_resolution / 4;
    s->C = cfg->cascades;
    Rng rng(cfg->seed);
    const float L = cfg->room_size, t = cfg->wall_thickness;
    const float a = 0.5f * L - t;
    s->wall_half_inner = a;
    // sun
    V3 sd{cfg->sun_direction[0], cfg->sun_direction[1], cfg->sun_direction[2]};
    if (sd.x == 0.0f && sd.y == 0.0f && sd.z == 0.0f) {
        float cy = rng.uniform(0.2f, 1.0f);
        float phi = rng.uniform() * 6.2831853f;
        float sxz = std::sqrt(1.0f - cy * cy);
        sd = {sxz * std::cos(phi), cy, sxz * std::sin(phi)};
    }
    s->sun = normalize(sd);
    s->sun_color = {cfg->sun_color[0], cfg->sun_color[1], cfg->sun_color[2]};
    // primitives
    for (int i = 0; i < cfg->num_primitives; ++i) {
        luxgi_scene_primitive p{};
        p.kind = rng.uniform() < 0.5f ? 0 : 1;
        if (p.kind == 0) {
            float r = rng.uniform(cfg->sphere_radius[0], cfg->sphere_radius[1]);
            p.half_extent[0] = p.half_extent[1] = p.half_extent[2] = r;
        } else {
            for (int q = 0; q < 3; ++q)
                p.half_extent[q] = rng.uniform(cfg->box_half_extent[0], cfg->box_half_extent[1]);
        }
        for (int q = 0; q < 3; ++q) {
            float m = std::max(a - p.half_extent[q], 0.0f);
            p.center[q] = rng.uniform(-m, m);
        }
        for (int q = 0; q < 3; ++q) p.albedo[q] = rng.uniform(cfg->albedo_range[0], cfg->albedo_range[1]);
        s->prims.push_back(p);
    }
    s->n_solid = int(s->prims.size());
    // six wall slabs: -X,+X,-Y,+Y,-Z,+Z (only their cards are used; the SDF
    // uses the exact complement of the interior box)
    for (int w = 0; w < 6; ++w) {
        luxgi_scene_primitive p{};
        p.kind = 2;
        int ax = w / 2;
        float sg = (w & 1) ? 1.0f : -1.0f;
        for (int q = 0; q < 3; ++q) { p.center[q] = 0.0f; p.half_extent[q] = 0.5f * L; }
        p.center[ax] = sg * 0.5f * (0.5f * L + a);
        p.half_extent[ax] = std::max(0.5f * (0.5f * L - a), 0.05f);
        for (int q = 0; q < 3; ++q) p.albedo[q] = rng.uniform(cfg->albedo_range[0], cfg->albedo_range[1]);
        s->prims.push_back(p);
    }
    build_sdf(*s);
    int st = build_surface(*s);
    if (st != LUXGI_OK) { delete s; return st; }
    *out = s;
    return LUXGI_OK;
}

extern "C" int luxgi_scene_view_get(const luxgi_scene* s, luxgi_scene_view* v) {
    if (!s || !v) return LUXGI_EINVAL;
    std::memset(v, 0, sizeof(*v));
    v->sdf_data = s->sdf_data;
    v->sdf_format = s->cfg.sdf_format;
    v->sdf_resolution = s->res;
    v->mip_resolution = s->mres;
    v->cascades = s->C;
    if (s->cfg.sdf_format == LUXGI_STORAGE_FP16) {
        v->sdf = s->sdf16.data();
        v->sdf_bytes = int64_t(s->sdf16.size() * 2);
    } else {
        v->sdf = s->sdf32.data();
        v->sdf_bytes = int64_t(s->sdf32.size() * 4);
    }
    v->surface_data = s->surface_data;
    v->num_objects = int32_t(s->objects.size());
    v->num_tiles = int32_t(s->tiles.size());
    v->objects = s->objects.data();
    v->tiles = s->tiles.data();
    v->atlas_resolution = s->atlas;
    v->direct_light = s->direct.data();
    v->depth = s->depth.data();
    v->albedo = s->albedo.data();
    v->gbuffer0 = s->gb0.data();
    v->gbuffer1 = s->gb1.data();
    v->num_primitives = int32_t(s->prims.size());
    v->primitives = s->prims.data();
    v->sun_direction[0] = s->sun.x; v->sun_direction[1] = s->sun.y; v->sun_direction[2] = s->sun.z;
    v->sun_color[0] = s->sun_color.x; v->sun_color[1] = s->sun_color.y; v->sun_color[2] = s->sun_color.z;
    v->pbr = s->pbr.data();
    v->emissive = s->emissive.data();
    return LUXGI_OK;
}

extern "C" int luxgi_scene_destroy(luxgi_scene* s) {
    delete s;
    return LUXGI_OK;
}

extern "C" float luxgi_scene_distance(const luxgi_scene* s, const float p[3]) {
    if (!s || !p) return 0.0f;
    return scene_distance(*s, {p[0], p[1], p[2]});
}
