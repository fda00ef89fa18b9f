// The global SDF built from placed mesh SDFs (merge_sdf::system,
// Engine/DDGI/GlobalDistanceField.cpp:465-842; SDFRasterizeModel.glsl;
// distanceToModelSDF, SDFCommon.glsl:38-62), and the parser of baked .sdf
// files (SDFBaker.cpp:158-240).
//
// The host plans each cascade the way the reference's system does -- object
// selection, ObjectRasterizeData records and the 32^3-voxel chunk table with
// at most 28 objects a chunk -- and the device rasterises: one block per
// plane (or 8-row band) of a chunk, the chunk's records and mesh volumes
// staged in shared memory.  Cascade by cascade: rasterise, then that
// cascade's mip, as the reference orders its dispatches.
//
// Built with -fmad=false (and the host part without contraction): the
// rasterised voxels equal the FP32 CPU restatement bit for bit.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <unordered_map>
#include <vector>

#include <cuda_fp16.h>

#include "luxgi_internal.h"

namespace luxgi {

namespace {

// ------------------------------------------------------------ host maths
struct M4 {
    float m[16];   // column-major: m[col * 4 + row]
};
struct V4 {
    float x, y, z, w;
};

M4 identity() {
    M4 r{};
    r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.0f;
    return r;
}

// M * v with glm's association: (c0 x + c1 y) + (c2 z + c3 w)
V4 mulv(const M4& M, float x, float y, float z, float w) {
    const float* m = M.m;
    V4 r;
    r.x = (m[0] * x + m[4] * y) + (m[8] * z + m[12] * w);
    r.y = (m[1] * x + m[5] * y) + (m[9] * z + m[13] * w);
    r.z = (m[2] * x + m[6] * y) + (m[10] * z + m[14] * w);
    r.w = (m[3] * x + m[7] * y) + (m[11] * z + m[15] * w);
    return r;
}

M4 mul(const M4& A, const M4& B) {
    M4 r;
    for (int c = 0; c < 4; ++c) {
        const V4 v = mulv(A, B.m[c * 4], B.m[c * 4 + 1], B.m[c * 4 + 2], B.m[c * 4 + 3]);
        r.m[c * 4] = v.x; r.m[c * 4 + 1] = v.y; r.m[c * 4 + 2] = v.z; r.m[c * 4 + 3] = v.w;
    }
    return r;
}

// Inverse by cofactors: 2x2 sub-determinants of the upper and lower row
// pairs (Laplace expansion), adjugate times 1/det.
M4 inverse(const M4& A) {
    float a[4][4];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) a[r][c] = A.m[c * 4 + r];
    const float s0 = a[0][0] * a[1][1] - a[1][0] * a[0][1];
    const float s1 = a[0][0] * a[1][2] - a[1][0] * a[0][2];
    const float s2 = a[0][0] * a[1][3] - a[1][0] * a[0][3];
    const float s3 = a[0][1] * a[1][2] - a[1][1] * a[0][2];
    const float s4 = a[0][1] * a[1][3] - a[1][1] * a[0][3];
    const float s5 = a[0][2] * a[1][3] - a[1][2] * a[0][3];
    const float c5 = a[2][2] * a[3][3] - a[3][2] * a[2][3];
    const float c4 = a[2][1] * a[3][3] - a[3][1] * a[2][3];
    const float c3 = a[2][1] * a[3][2] - a[3][1] * a[2][2];
    const float c2 = a[2][0] * a[3][3] - a[3][0] * a[2][3];
    const float c1 = a[2][0] * a[3][2] - a[3][0] * a[2][2];
    const float c0 = a[2][0] * a[3][1] - a[3][0] * a[2][1];
    const float det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    const float id = 1.0f / det;
    float b[4][4];
    b[0][0] = ( a[1][1] * c5 - a[1][2] * c4 + a[1][3] * c3) * id;
    b[0][1] = (-a[0][1] * c5 + a[0][2] * c4 - a[0][3] * c3) * id;
    b[0][2] = ( a[3][1] * s5 - a[3][2] * s4 + a[3][3] * s3) * id;
    b[0][3] = (-a[2][1] * s5 + a[2][2] * s4 - a[2][3] * s3) * id;
    b[1][0] = (-a[1][0] * c5 + a[1][2] * c2 - a[1][3] * c1) * id;
    b[1][1] = ( a[0][0] * c5 - a[0][2] * c2 + a[0][3] * c1) * id;
    b[1][2] = (-a[3][0] * s5 + a[3][2] * s2 - a[3][3] * s1) * id;
    b[1][3] = ( a[2][0] * s5 - a[2][2] * s2 + a[2][3] * s1) * id;
    b[2][0] = ( a[1][0] * c4 - a[1][1] * c2 + a[1][3] * c0) * id;
    b[2][1] = (-a[0][0] * c4 + a[0][1] * c2 - a[0][3] * c0) * id;
    b[2][2] = ( a[3][0] * s4 - a[3][1] * s2 + a[3][3] * s0) * id;
    b[2][3] = (-a[2][0] * s4 + a[2][1] * s2 - a[2][3] * s0) * id;
    b[3][0] = (-a[1][0] * c3 + a[1][1] * c1 - a[1][2] * c0) * id;
    b[3][1] = ( a[0][0] * c3 - a[0][1] * c1 + a[0][2] * c0) * id;
    b[3][2] = (-a[3][0] * s3 + a[3][1] * s1 - a[3][2] * s0) * id;
    b[3][3] = ( a[2][0] * s3 - a[2][1] * s1 + a[2][2] * s0) * id;
    M4 out;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out.m[c * 4 + r] = b[r][c];
    return out;
}

float hmin(float a, float b) { return b < a ? b : a; }
float hmax(float a, float b) { return a < b ? b : a; }
float saturate(float v) { return hmin(hmax(v, 0.0f), 1.0f); }

constexpr float kCascadeScales[4] = {1.0f, 2.5f, 5.0f, 10.0f};   // GlobalDistanceField.cpp:594

// The cascade's centre, half extent and voxel size (GlobalDistanceField.cpp:
// 592-626): the cascades sit around a fixed view point 0.3 cascade-0 extents
// along +z (the camera-relative placement is commented out in the
// reference), snapped to the cascade's chunk grid.
void cascade_geometry(const luxgi_sdf_build_desc& d, int c, float center[3], float* distance, float* voxel) {
    const float dist = hmin(15000.0f, d.gi_distance) * d.global_scale;
    const float extent = dist / kCascadeScales[d.cascades - 1];
    const float c0 = extent * kCascadeScales[0];
    // math::lineHitsAABB (Math/MathUtils.h:162-170) from the origin to
    // FORWARD * 2 c0 against [-c0, c0]^3; x and y of the segment are 0
    const float dz = (0.0f + 1.0f * (c0 * 2.0f)) - 0.0f;
    const float inv_z = 1.0f / dz;
    const float inf = INFINITY;
    const float en[3] = {(-c0 - 0.0f) * inf, (-c0 - 0.0f) * inf, (-c0 - 0.0f) * inv_z};
    const float ex[3] = {(c0 - 0.0f) * inf, (c0 - 0.0f) * inf, (c0 - 0.0f) * inv_z};
    const float mx3 = hmin(hmax(en[0], ex[0]), hmin(hmax(en[1], ex[1]), hmax(en[2], ex[2])));
    const float hit_y = saturate(mx3);
    const float offset = hit_y * c0 * 0.6f;
    const float view[3] = {0.0f * offset, 0.0f * offset, 0.0f + 1.0f * offset};
    const float cd = extent * kCascadeScales[c];
    const float maxd = cd * 2.0f;
    const float vox = maxd / float(d.resolution);
    const float chunk = vox * float(LUXGI_SDF_CHUNK);
    for (int i = 0; i < 3; ++i) center[i] = std::floor(view[i] / chunk) * chunk;
    *distance = cd;
    *voxel = vox;
}

// BoundingBox::transform (Math/BoundingBox.cpp:10-22)
void transform_box(const float mn[3], const float mxv[3], const M4& T, float omin[3], float omax[3]) {
    const float ctr[3] = {(mxv[0] + mn[0]) * 0.5f, (mxv[1] + mn[1]) * 0.5f, (mxv[2] + mn[2]) * 0.5f};
    const V4 nc = mulv(T, ctr[0], ctr[1], ctr[2], 1.0f);
    const float e[3] = {(mxv[0] - mn[0]) * 0.5f, (mxv[1] - mn[1]) * 0.5f, (mxv[2] - mn[2]) * 0.5f};
    const float* m = T.m;
    const float ne[3] = {
        std::fabs(m[0]) * e[0] + std::fabs(m[4]) * e[1] + std::fabs(m[8] * e[2]),
        std::fabs(m[1]) * e[0] + std::fabs(m[5]) * e[1] + std::fabs(m[9] * e[2]),
        std::fabs(m[2]) * e[0] + std::fabs(m[6]) * e[1] + std::fabs(m[10] * e[2])};
    const float c[3] = {nc.x, nc.y, nc.z};
    for (int i = 0; i < 3; ++i) {
        omin[i] = c[i] - ne[i];
        omax[i] = c[i] + ne[i];
    }
}

struct ChunkSlot {
    int32_t coord[3];
    int count;
    uint32_t models[LUXGI_SDF_CHUNK_MODELS];
};

struct CascadePlan {
    std::vector<luxgi_sdf_raster_object> records;
    std::vector<int32_t> mesh_of;
    std::vector<ChunkSlot> chunks;
};

bool mesh_ok(const luxgi_mesh_sdf& m) {
    return m.size[0] > 0 && m.size[1] > 0 && m.size[2] > 0 && m.mip_count >= 1 && m.mip_count <= 3;
}

// Cascade c's objects and chunk table (GlobalDistanceField.cpp:465-535 and
// 672-693).
int plan_cascade(const luxgi_sdf_build_desc& d, const luxgi_mesh_sdf* meshes, int nm, const luxgi_sdf_object* objs,
                 int no, int c, CascadePlan& out) {
    float center[3], cd, vox;
    cascade_geometry(d, c, center, &cd, &vox);
    const float bmin[3] = {center[0] - cd, center[1] - cd, center[2] - cd};
    const float bmax[3] = {center[0] + cd, center[1] + cd, center[2] + cd};
    const float min_radius = d.min_object_radius * d.global_scale;
    // chunk table keyed by coordinate; layers beyond 0 only ever hold an
    // empty entry (see below), so one slot per coordinate suffices
    std::unordered_map<uint64_t, int> slot_of;
    auto key = [](int x, int y, int z) -> uint64_t {
        return (uint64_t(uint32_t(x) & 0x1FFFFFu) << 42) | (uint64_t(uint32_t(y) & 0x1FFFFFu) << 21) |
               uint64_t(uint32_t(z) & 0x1FFFFFu);
    };
    for (int o = 0; o < no; ++o) {
        const luxgi_sdf_object& ob = objs[o];
        if (ob.mesh < 0 || ob.mesh >= nm || !mesh_ok(meshes[ob.mesh])) return LUXGI_EINVAL;
        const luxgi_mesh_sdf& ms = meshes[ob.mesh];
        M4 W;
        std::memcpy(W.m, ob.world, sizeof(W.m));
        float omin[3], omax[3];
        transform_box(ms.aabb_min, ms.aabb_max, W, omin, omax);
        // BoundingSphere(box) (Math/BoundingSphere.cpp:9-13) against the
        // cascade box (BoundingBox::intersectsWithSphere, BoundingBox.cpp:31-36)
        const float sc[3] = {(omax[0] + omin[0]) * 0.5f, (omax[1] + omin[1]) * 0.5f, (omax[2] + omin[2]) * 0.5f};
        const float dd[3] = {omax[0] - omin[0], omax[1] - omin[1], omax[2] - omin[2]};
        const float radius = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]) / 2.0f;
        float d2 = 0.0f;
        {
            float q[3];
            for (int i = 0; i < 3; ++i) q[i] = sc[i] - hmin(hmax(sc[i], bmin[i]), bmax[i]);
            d2 = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
        }
        if (!(d2 <= radius * radius && radius >= min_radius)) continue;
        // chunkCalculate (:465-535)
        const float margin = vox * 4.0f;                       // CONSTS_SDF_RASTERIZE_CHUNK_MARGIN
        const float bias_min[3] = {bmin[0] + 0.1f, bmin[1] + 0.1f, bmin[2] + 0.1f};
        const float chunk_size = vox * float(LUXGI_SDF_CHUNK);
        int cmin[3], cmax[3];
        for (int i = 0; i < 3; ++i) {
            // the reference's glm::clamp results are discarded (:202-203),
            // so object bounds are not clamped to the cascade
            const float lo = (omin[i] - margin) - bias_min[i];
            const float hi = (omax[i] + margin) - bias_min[i];
            cmin[i] = int(lo / chunk_size);                       // ivec3(vec3): truncation
            cmax[i] = int(hi / chunk_size);
        }
        const float vc[3] = {(ms.aabb_max[0] + ms.aabb_min[0]) * 0.5f, (ms.aabb_max[1] + ms.aabb_min[1]) * 0.5f,
                             (ms.aabb_max[2] + ms.aabb_min[2]) * 0.5f};
        const M4 world_to_local = inverse(W);
        M4 T = identity();
        T.m[12] = -vc[0];
        T.m[13] = -vc[1];
        T.m[14] = -vc[2];
        const M4 w2v = mul(world_to_local, T);
        const M4 v2w = inverse(w2v);
        luxgi_sdf_raster_object r{};
        std::memcpy(r.world_to_volume, w2v.m, sizeof(w2v.m));
        std::memcpy(r.volume_to_world, v2w.m, sizeof(v2w.m));
        for (int i = 0; i < 3; ++i) {
            r.volume_local_bounds_extent[i] = (ms.aabb_max[i] - ms.aabb_min[i]) / 2.0f;
            r.volume_to_uvw_mul[i] = ms.local_to_uvw_mul[i];
            r.volume_to_uvw_add[i] = ms.local_to_uvw_add[i] + vc[i] * ms.local_to_uvw_mul[i];
        }
        r.mip_offset = float(c < 2 ? c : 2);
        r.decode_mul = ms.max_distance;
        r.decode_add = -ms.max_distance;
        const uint32_t index = uint32_t(out.records.size());
        out.records.push_back(r);
        out.mesh_of.push_back(ob.mesh);
        for (int z = cmin[2]; z <= cmax[2]; ++z)
            for (int y = cmin[1]; y <= cmax[1]; ++y)
                for (int x = cmin[0]; x <= cmax[0]; ++x) {
                    const auto it = slot_of.find(key(x, y, z));
                    int k = it == slot_of.end() ? -1 : it->second;
                    if (k < 0) {
                        k = int(out.chunks.size());
                        slot_of.emplace(key(x, y, z), k);
                        ChunkSlot sl{};
                        sl.coord[0] = x; sl.coord[1] = y; sl.coord[2] = z;
                        sl.count = 0;
                        out.chunks.push_back(sl);
                    }
                    ChunkSlot& sl = out.chunks[size_t(k)];
                    // :516-523: a full chunk makes the loop copy the empty
                    // next-layer entry over the layer-0 entry it holds by
                    // reference, so the chunk restarts with this object
                    if (sl.count == LUXGI_SDF_CHUNK_MODELS) sl.count = 0;
                    sl.models[sl.count++] = index;
                }
    }
    return LUXGI_OK;
}

bool layout_ok(const luxgi_sdf_build_desc& d) {
    return d.cascades >= 1 && d.cascades <= 4 && d.resolution >= 4 && d.resolution % 4 == 0 &&
           d.gi_distance > 0.0f && d.global_scale > 0.0f &&
           (d.format == LUXGI_STORAGE_FP32 || d.format == LUXGI_STORAGE_FP16);
}

void layout_data(const luxgi_sdf_build_desc& d, luxgi_sdf_data& out) {
    std::memset(&out, 0, sizeof(out));
    for (int c = 0; c < d.cascades; ++c) {
        float center[3], cd, vox;
        cascade_geometry(d, c, center, &cd, &vox);
        out.cascade_pos_distance[c][0] = center[0];
        out.cascade_pos_distance[c][1] = center[1];
        out.cascade_pos_distance[c][2] = center[2];
        out.cascade_pos_distance[c][3] = cd;
        out.cascade_voxel_size[c] = vox;
    }
    out.cascades_count = uint32_t(d.cascades);
    out.resolution = float(d.resolution);
    out.near_plane = d.near_plane;
    out.far_plane = d.far_plane;
}

// ------------------------------------------------------------ device side
struct RasterMesh {
    const __half* vol;   // the level sampled in this cascade
    int w, h, d;
    // a world-space sphere around the object's volume box: centre (the
    // volume origin) and a radius bounding every box point's distance
    float cx, cy, cz, radius;
};

struct RasterParams {
    float mul[3], add[3];   // cascadeCoordToPosMul / Add (GlobalDistanceField.cpp:756-757)
    float max_dist;         // 2 x half extent
    int res, C, cascade;
};

__device__ __forceinline__ float ld_half(const __half* p, size_t i) { return __half2float(__ldg(p + i)); }

// textureLod of a mesh SDF: trilinear with REPEAT (its sampler's default
// wrap, RHI/Definitions.h:169-171) on one mip level
__device__ __forceinline__ float sample_mesh(const RasterMesh& m, float u, float v, float w) {
    const float x = u * float(m.w) - 0.5f, y = v * float(m.h) - 0.5f, z = w * float(m.d) - 0.5f;
    const float fx = floorf(x), fy = floorf(y), fz = floorf(z);
    const float a = x - fx, b = y - fy, c = z - fz;
    const int x0 = wrap_repeat(int(fx), m.w), x1 = wrap_repeat(int(fx) + 1, m.w);
    const int y0 = wrap_repeat(int(fy), m.h), y1 = wrap_repeat(int(fy) + 1, m.h);
    const int z0 = wrap_repeat(int(fz), m.d), z1 = wrap_repeat(int(fz) + 1, m.d);
    const size_t sw = size_t(m.w), sp = size_t(m.w) * size_t(m.h);
    const float t000 = ld_half(m.vol, x0 + sw * y0 + sp * z0), t100 = ld_half(m.vol, x1 + sw * y0 + sp * z0);
    const float t010 = ld_half(m.vol, x0 + sw * y1 + sp * z0), t110 = ld_half(m.vol, x1 + sw * y1 + sp * z0);
    const float t001 = ld_half(m.vol, x0 + sw * y0 + sp * z1), t101 = ld_half(m.vol, x1 + sw * y0 + sp * z1);
    const float t011 = ld_half(m.vol, x0 + sw * y1 + sp * z1), t111 = ld_half(m.vol, x1 + sw * y1 + sp * z1);
    const float ia = 1.0f - a, ib = 1.0f - b, ic = 1.0f - c;
    const float c00 = t000 * ia + t100 * a, c10 = t010 * ia + t110 * a;
    const float c01 = t001 * ia + t101 * a, c11 = t011 * ia + t111 * a;
    const float c0 = c00 * ib + c10 * b, c1 = c01 * ib + c11 * b;
    return c0 * ic + c1 * c;
}

// combineDistanceToSDF (SDFCommon.glsl:18-36)
__device__ __forceinline__ float combine_to_sdf(float sdf, float dist) {
    if (sdf <= 0.0f && dist <= 0.0f) return sdf;
    const float m = mx(sdf, 0.0f);
    return sqrtf(m * m + dist * dist);
}

__device__ __forceinline__ f3 xform(const float* m, f3 p) {
    return f3{(m[0] * p.x + m[4] * p.y) + (m[8] * p.z + m[12]), (m[1] * p.x + m[5] * p.y) + (m[9] * p.z + m[13]),
              (m[2] * p.x + m[6] * p.y) + (m[10] * p.z + m[14])};
}

// distanceToModelSDF (SDFCommon.glsl:38-62)
__device__ __forceinline__ float distance_to_model(float min_distance, const luxgi_sdf_raster_object& r,
                                                   const RasterMesh& m, f3 wp) {
    const f3 vp = xform(r.world_to_volume, wp);
    const f3 uvw{vp.x * r.volume_to_uvw_mul[0] + r.volume_to_uvw_add[0],
                 vp.y * r.volume_to_uvw_mul[1] + r.volume_to_uvw_add[1],
                 vp.z * r.volume_to_uvw_mul[2] + r.volume_to_uvw_add[2]};
    const float* e = r.volume_local_bounds_extent;
    const f3 vc{clampf(vp.x, -e[0], e[0]), clampf(vp.y, -e[1], e[1]), clampf(vp.z, -e[2], e[2])};
    const f3 wc = xform(r.volume_to_world, vc);
    float dtv = len3(sub3(wp, wc));
    if (dtv < 0.01f) dtv = len3(sub3(vp, vc));
    dtv = mx(dtv, 0.0f);
    if (min_distance <= dtv) return dtv;
    const float vd = (sample_mesh(m, uvw.x, uvw.y, uvw.z) * 2.0f - 1.0f) * r.decode_mul;
    float result = combine_to_sdf(vd, dtv);
    if (dtv > 0.0f) result = mx(dtv, result);
    return result;
}

template <typename T> __device__ __forceinline__ void store_sdf(T* p, size_t i, float v);
template <> __device__ __forceinline__ void store_sdf<float>(float* p, size_t i, float v) { p[i] = v; }
template <> __device__ __forceinline__ void store_sdf<__half>(__half* p, size_t i, float v) { p[i] = __float2half_rn(v); }

__global__ void fill_kernel(__half* h, float* f, size_t n) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        if (h) h[i] = __float2half_rn(1.0f);
        else f[i] = 1.0f;
    }
}

// SDFRasterizeModel.glsl main (no READ_DISTANCE: the reference's chunks
// never reach a second layer): blockIdx.x = chunk, blockIdx.y = z plane,
// blockIdx.z = band of 32 / gridDim.z rows of the plane.  Cascades with
// many chunks take whole planes (4 voxels a thread, the records staged
// once a plane); the coarse cascades' few chunks take 8-row bands so that
// they still fill the GPU.
template <typename T>
__global__ void __launch_bounds__(256) sdf_raster_kernel(const luxgi_sdf_chunk* __restrict__ chunks,
                                                         const luxgi_sdf_raster_object* __restrict__ recs,
                                                         const RasterMesh* __restrict__ mesh_of,
                                                         const RasterParams p, T* __restrict__ out) {
    __shared__ luxgi_sdf_raster_object srec[LUXGI_SDF_CHUNK_MODELS];
    __shared__ RasterMesh smesh[LUXGI_SDF_CHUNK_MODELS];
    const luxgi_sdf_chunk* ch = chunks + blockIdx.x;
    const int n = imn(imx(__ldg(&ch->count), 0), LUXGI_SDF_CHUNK_MODELS);
    constexpr int kWords = int(sizeof(luxgi_sdf_raster_object) / 4);
    for (int i = threadIdx.x; i < n * kWords; i += blockDim.x) {
        const int k = i / kWords, w = i % kWords;
        const uint32_t id = __ldg(&ch->models[k]);
        reinterpret_cast<float*>(&srec[k])[w] = __ldg(reinterpret_cast<const float*>(recs + id) + w);
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) smesh[k] = mesh_of[__ldg(&ch->models[k])];
    __syncthreads();
    const int ox = __ldg(&ch->coord[0]) * LUXGI_SDF_CHUNK, oy = __ldg(&ch->coord[1]) * LUXGI_SDF_CHUNK,
              oz = __ldg(&ch->coord[2]) * LUXGI_SDF_CHUNK;
    const int TW = p.res * p.C;
    const int vz = oz + int(blockIdx.y);
    const int rows = LUXGI_SDF_CHUNK / int(gridDim.z);
    for (int v = threadIdx.x; v < LUXGI_SDF_CHUNK * rows; v += blockDim.x) {
        const int vx = ox + (v & 31), vy = oy + int(blockIdx.z) * rows + (v >> 5);
        const int gx = vx + p.cascade * p.res;
        // image stores outside the packed texture are discarded; x past the
        // cascade lands in its neighbour, as in the reference
        if (gx < 0 || gx >= TW || vy < 0 || vy >= p.res || vz < 0 || vz >= p.res) continue;
        const f3 wp{float(vx) * p.mul[0] + p.add[0], float(vy) * p.mul[1] + p.add[1], float(vz) * p.mul[2] + p.add[2]};
        float md = p.max_dist;
        for (int k = 0; k < n; ++k) {
            // an object whose box is certainly farther than max(md, 0.01)
            // (distanceToModelSDF's world-space branch) returns a distance
            // >= md, which leaves md unchanged: skip it.  The margin covers
            // the rounding of the transforms.
            const RasterMesh& m = smesh[k];
            const float dx = wp.x - m.cx, dy = wp.y - m.cy, dz = wp.z - m.cz;
            const float dc = sqrtf(dx * dx + dy * dy + dz * dz);
            const float lim = mx(md, 0.01f);
            if (dc - m.radius > lim + 1e-4f * (dc + m.radius + lim) + 1e-3f) continue;
            const float od = distance_to_model(md, srec[k], m, wp);
            md = mn(md, od);
        }
        store_sdf<T>(out, size_t(gx) + size_t(TW) * (size_t(vy) + size_t(p.res) * size_t(vz)),
                     clampf(md / p.max_dist, -1.0f, 1.0f));
    }
}

template <typename T> T* as_t(void* p) { return static_cast<T*>(p); }

}  // namespace

}  // namespace luxgi

using namespace luxgi;

extern "C" {

int luxgi_sdf_cascade_layout(const luxgi_sdf_build_desc* d, luxgi_sdf_data* out) {
    if (!d || !out || !layout_ok(*d)) return LUXGI_EINVAL;
    layout_data(*d, *out);
    return LUXGI_OK;
}

int luxgi_sdf_build_plan(const luxgi_sdf_build_desc* d, const luxgi_mesh_sdf* meshes, int nm,
                         const luxgi_sdf_object* objs, int no, int cascade, luxgi_sdf_raster_object* raster_out,
                         int raster_capacity, int* num_objects_out, int32_t* object_mesh_out,
                         luxgi_sdf_chunk* chunks_out, int chunk_capacity, int* num_chunks_out) {
    if (!d || !layout_ok(*d) || cascade < 0 || cascade >= d->cascades || nm < 0 || no < 0 ||
        (nm > 0 && !meshes) || (no > 0 && !objs) || !num_objects_out || !num_chunks_out)
        return LUXGI_EINVAL;
    CascadePlan plan;
    const int st = plan_cascade(*d, meshes, nm, objs, no, cascade, plan);
    if (st != LUXGI_OK) return st;
    *num_objects_out = int(plan.records.size());
    *num_chunks_out = int(plan.chunks.size());
    if ((raster_out || object_mesh_out) && int(plan.records.size()) > raster_capacity) return LUXGI_ENOMEM;
    if (chunks_out && int(plan.chunks.size()) > chunk_capacity) return LUXGI_ENOMEM;
    for (size_t i = 0; i < plan.records.size(); ++i) {
        if (raster_out) raster_out[i] = plan.records[i];
        if (object_mesh_out) object_mesh_out[i] = plan.mesh_of[i];
    }
    if (chunks_out)
        for (size_t i = 0; i < plan.chunks.size(); ++i) {
            luxgi_sdf_chunk c{};
            std::memcpy(c.coord, plan.chunks[i].coord, sizeof(c.coord));
            c.count = plan.chunks[i].count;
            std::memcpy(c.models, plan.chunks[i].models, sizeof(c.models));
            chunks_out[i] = c;
        }
    return LUXGI_OK;
}

int luxgi_sdf_build(const luxgi_sdf_build_desc* d, const luxgi_mesh_sdf* meshes, int nm, const luxgi_sdf_object* objs,
                    int no, void* sdf, void* mip, void* tmp, luxgi_sdf_data* data_out, void* stream) {
    if (!d || !layout_ok(*d) || !sdf || !mip || !tmp || nm < 0 || no < 0 || (nm > 0 && !meshes) ||
        (no > 0 && !objs))
        return LUXGI_EINVAL;
    for (int i = 0; i < no; ++i) {
        if (objs[i].mesh < 0 || objs[i].mesh >= nm) return LUXGI_EINVAL;
        const luxgi_mesh_sdf& m = meshes[objs[i].mesh];
        // merge_sdf::system returns before rasterising anything when a mesh
        // SDF is not loaded (:690-691)
        if (!mesh_ok(m)) return LUXGI_EINVAL;
        for (int k = 0; k < m.mip_count; ++k)
            if (!m.mips[k]) return LUXGI_EINVAL;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int res = d->resolution, C = d->cascades;
    int ordinal = 0, sms = 0;
    cudaGetDevice(&ordinal);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ordinal);
    if (sms <= 0) sms = 1;
    luxgi_sdf_desc sd{};
    layout_data(*d, sd.data);
    sd.format = d->format;
    sd.resolution = res;
    sd.mip_resolution = res / 4;
    sd.sdf = sdf;
    sd.mip = mip;
    const size_t n = size_t(res) * C * res * res;
    const bool h = d->format == LUXGI_STORAGE_FP16;
    fill_kernel<<<1024, 256, 0, st>>>(h ? as_t<__half>(sdf) : nullptr, h ? nullptr : as_t<float>(sdf), n);
    note_launch();
    cudaError_t e = cudaGetLastError();
    std::vector<CascadePlan> plans(static_cast<size_t>(C));
    for (int c = 0; c < C && e == cudaSuccess; ++c) {
        const int s = plan_cascade(*d, meshes, nm, objs, no, c, plans[size_t(c)]);
        if (s != LUXGI_OK) return s;
    }
    // one device staging area for every cascade's lists (cascades run in
    // stream order, each after its lists' upload)
    size_t tot_chunks = 0, tot_recs = 0;
    for (const CascadePlan& pl : plans) {
        tot_chunks += pl.chunks.size();
        tot_recs += pl.records.size();
    }
    const size_t bytes = tot_chunks * sizeof(luxgi_sdf_chunk) + tot_recs * (sizeof(luxgi_sdf_raster_object) +
                                                                         sizeof(RasterMesh));
    std::vector<unsigned char> host(bytes > 0 ? bytes : 1);
    void* dev = nullptr;
    if (e == cudaSuccess && bytes > 0) e = cudaMallocAsync(&dev, bytes, st);
    size_t off = 0;
    std::vector<size_t> chunk_off(static_cast<size_t>(C)), rec_off(chunk_off), mesh_off(chunk_off);
    for (int c = 0; c < C; ++c) {
        const CascadePlan& pl = plans[size_t(c)];
        chunk_off[size_t(c)] = off;
        for (const ChunkSlot& sl : pl.chunks) {
            luxgi_sdf_chunk ck{};
            std::memcpy(ck.coord, sl.coord, sizeof(ck.coord));
            ck.count = sl.count;
            std::memcpy(ck.models, sl.models, sizeof(ck.models));
            std::memcpy(host.data() + off, &ck, sizeof(ck));
            off += sizeof(ck);
        }
        rec_off[size_t(c)] = off;
        std::memcpy(host.data() + off, pl.records.data(), pl.records.size() * sizeof(luxgi_sdf_raster_object));
        off += pl.records.size() * sizeof(luxgi_sdf_raster_object);
        mesh_off[size_t(c)] = off;
        const int level = c < 2 ? c : 2;
        for (size_t i = 0; i < pl.records.size(); ++i) {
            const luxgi_mesh_sdf& m = meshes[pl.mesh_of[i]];
            // textureLod past the last level reads the last level
            const int L = level < m.mip_count - 1 ? level : m.mip_count - 1;
            RasterMesh rm;
            rm.vol = reinterpret_cast<const __half*>(m.mips[L]);
            rm.w = std::max(m.size[0] >> L, 1);
            rm.h = std::max(m.size[1] >> L, 1);
            rm.d = std::max(m.size[2] >> L, 1);
            const luxgi_sdf_raster_object& r = pl.records[i];
            const float* v2w = r.volume_to_world;
            rm.cx = v2w[12];
            rm.cy = v2w[13];
            rm.cz = v2w[14];
            double rad = 0.0;
            for (int a = 0; a < 3; ++a) {
                const double cn = std::sqrt(double(v2w[a * 4]) * v2w[a * 4] + double(v2w[a * 4 + 1]) * v2w[a * 4 + 1] +
                                            double(v2w[a * 4 + 2]) * v2w[a * 4 + 2]);
                rad += cn * double(r.volume_local_bounds_extent[a]);
            }
            rm.radius = float(rad * 1.0001);
            std::memcpy(host.data() + off, &rm, sizeof(rm));
            off += sizeof(rm);
        }
    }
    // the upload is staged through pageable memory: the copy is complete when
    // cudaMemcpyAsync returns, so `host` may go out of scope afterwards
    if (e == cudaSuccess && bytes > 0) e = cudaMemcpyAsync(dev, host.data(), bytes, cudaMemcpyHostToDevice, st);
    for (int c = 0; c < C && e == cudaSuccess; ++c) {
        const CascadePlan& pl = plans[size_t(c)];
        float center[3], cd, vox;
        cascade_geometry(*d, c, center, &cd, &vox);
        RasterParams p;
        for (int i = 0; i < 3; ++i) {
            const float bmin = center[i] - cd, bmax = center[i] + cd;
            p.mul[i] = (bmax - bmin) / float(res);
            p.add[i] = bmin + vox * 0.5f;
        }
        p.max_dist = cd * 2.0f;
        p.res = res;
        p.C = C;
        p.cascade = c;
        if (!pl.chunks.empty()) {
            unsigned char* base = static_cast<unsigned char*>(dev);
            const auto* ck = reinterpret_cast<const luxgi_sdf_chunk*>(base + chunk_off[size_t(c)]);
            const auto* rc = reinterpret_cast<const luxgi_sdf_raster_object*>(base + rec_off[size_t(c)]);
            const auto* rm = reinterpret_cast<const RasterMesh*>(base + mesh_off[size_t(c)]);
            // whole planes once there are 8 blocks an SM, else 8-row bands
            const unsigned bands = pl.chunks.size() * LUXGI_SDF_CHUNK >= size_t(sms) * 8 ? 1u : 4u;
            const dim3 grid(unsigned(pl.chunks.size()), LUXGI_SDF_CHUNK, bands);
            if (h) sdf_raster_kernel<__half><<<grid, 256, 0, st>>>(ck, rc, rm, p, as_t<__half>(sdf));
            else sdf_raster_kernel<float><<<grid, 256, 0, st>>>(ck, rc, rm, p, as_t<float>(sdf));
            note_launch();
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = launch_mip_cascade(sd, c, !pl.chunks.empty(), mip, tmp, st);
    }
    if (dev) {
        const cudaError_t e2 = cudaFreeAsync(dev, st);
        if (e == cudaSuccess) e = e2;
    }
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? LUXGI_ENOMEM : LUXGI_ECUDA;
    if (data_out) *data_out = sd.data;
    return LUXGI_OK;
}

int luxgi_mesh_sdf_parse(const void* bytes, uint64_t n, luxgi_mesh_sdf_file* out) {
    if (!bytes || !out) return LUXGI_EINVAL;
    const unsigned char* b = static_cast<const unsigned char*>(bytes);
    std::memset(out, 0, sizeof(*out));
    if (n < 16) return LUXGI_EINVAL;
    uint32_t size[3];
    int32_t mips;
    std::memcpy(size, b, 12);
    std::memcpy(&mips, b + 12, 4);
    if (mips < 1 || mips > 3) return LUXGI_EINVAL;
    for (int i = 0; i < 3; ++i)
        if (size[i] < 1 || size[i] > 4096) return LUXGI_EINVAL;
    uint64_t off = 16;
    int32_t dims[3] = {int32_t(size[0]), int32_t(size[1]), int32_t(size[2])};
    for (int m = 0; m < mips; ++m) {
        if (n - off < 8) return LUXGI_EINVAL;
        uint64_t len;
        std::memcpy(&len, b + off, 8);
        off += 8;
        const uint64_t want = uint64_t(dims[0]) * uint64_t(dims[1]) * uint64_t(dims[2]) * 2u;
        if (len != want || n - off < len) return LUXGI_EINVAL;
        out->mip_offset[m] = off;
        out->mip_bytes[m] = len;
        off += len;
        for (int i = 0; i < 3; ++i) dims[i] = std::max(dims[i] / 2, 1);   // SDFBaker.cpp:168
    }
    out->size[0] = int32_t(size[0]);
    out->size[1] = int32_t(size[1]);
    out->size[2] = int32_t(size[2]);
    out->mip_count = mips;
    return LUXGI_OK;
}

}  // extern "C"
