// Texel loads and stores of the FP32 / FP16 probe atlases, shared by the
// SIMT blend (blend.cu) and the tensor-core blend (blend_tc.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_fp16.h>

namespace luxgi {

template <typename AT> struct AtlasIO;
template <> struct AtlasIO<float> {
    __device__ static float ld(const void* p, size_t i) { return static_cast<const float*>(p)[i]; }
    __device__ static float rnd(float v) { return v; }
    __device__ static void st(void* p, size_t i, float v) { static_cast<float*>(p)[i] = v; }
    // all NC channels of texel `texel` in one access (atlases are 16-byte aligned)
    template <int NC> __device__ static void ld_texel(const void* p, size_t texel, float* v) {
        if constexpr (NC == 4) {
            const float4 q = static_cast<const float4*>(p)[texel];
            v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
        } else {
            const float2 q = static_cast<const float2*>(p)[texel];
            v[0] = q.x; v[1] = q.y;
        }
    }
    template <int NC> __device__ static void st_texel(void* p, size_t texel, const float* v) {
        if constexpr (NC == 4) static_cast<float4*>(p)[texel] = make_float4(v[0], v[1], v[2], v[3]);
        else static_cast<float2*>(p)[texel] = make_float2(v[0], v[1]);
    }
};
template <> struct AtlasIO<__half> {
    __device__ static float ld(const void* p, size_t i) { return __half2float(static_cast<const __half*>(p)[i]); }
    __device__ static float rnd(float v) { return __half2float(__float2half_rn(v)); }
    __device__ static void st(void* p, size_t i, float v) { static_cast<__half*>(p)[i] = __float2half_rn(v); }
    template <int NC> __device__ static void ld_texel(const void* p, size_t texel, float* v) {
        if constexpr (NC == 4) {
            const uint2 q = static_cast<const uint2*>(p)[texel];
            const __half2 a = *reinterpret_cast<const __half2*>(&q.x);
            const __half2 b = *reinterpret_cast<const __half2*>(&q.y);
            v[0] = __low2float(a); v[1] = __high2float(a); v[2] = __low2float(b); v[3] = __high2float(b);
        } else {
            const __half2 a = static_cast<const __half2*>(p)[texel];
            v[0] = __low2float(a); v[1] = __high2float(a);
        }
    }
    template <int NC> __device__ static void st_texel(void* p, size_t texel, const float* v) {
        if constexpr (NC == 4) {
            const __half2 a = __floats2half2_rn(v[0], v[1]), b = __floats2half2_rn(v[2], v[3]);
            uint2 q;
            q.x = *reinterpret_cast<const uint32_t*>(&a);
            q.y = *reinterpret_cast<const uint32_t*>(&b);
            static_cast<uint2*>(p)[texel] = q;
        } else {
            static_cast<__half2*>(p)[texel] = __floats2half2_rn(v[0], v[1]);
        }
    }
};

// Writes channel values v[0..nc) of interior texel (tx, ty) of cell
// (cx, cy) and its border mirrors (BorderUpdate.glsl:136-156, rule
// generalised from the 8/16 tables at :25-133).
template <typename AT, int NC>
__device__ __forceinline__ void store_texel(void* atlas, int W, int n, int cx, int cy, int tx, int ty, const float* v) {
    const int ox = cx * (n + 2) + 1, oy = cy * (n + 2) + 1;   // cell origin (border corner)
    const int X = tx + 1, Y = ty + 1;                        // cell-relative interior coords
    auto put = [&](int x, int y) { AtlasIO<AT>::template st_texel<NC>(atlas, size_t(oy + y) * W + (ox + x), v); };
    put(X, Y);
    if (Y == 1) put(n + 1 - X, 0);
    if (Y == n) put(n + 1 - X, n + 1);
    if (X == 1) put(0, n + 1 - Y);
    if (X == n) put(n + 1, n + 1 - Y);
    // corners: (0,0)<-(n,n), (n+1,0)<-(1,n), (0,n+1)<-(n,1), (n+1,n+1)<-(1,1)
    if (X == n && Y == n) put(0, 0);
    if (X == 1 && Y == n) put(n + 1, 0);
    if (X == n && Y == 1) put(0, n + 1);
    if (X == 1 && Y == 1) put(n + 1, n + 1);
}

}  // namespace luxgi
