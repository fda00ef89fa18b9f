// ORACLE -- test infrastructure only.
//
// The packed R11G11B10F colour format of the surface cache's emissive and
// light-cache textures (TextureFormat::R11G11B10, Engine/DDGI/
// GlobalSurfaceAtlas.cpp:410-411), restated from the format's definition
// for the CPU restatement (oracle.cpp) and the reference harness
// (ref_harness.cpp), which model what the texture unit and the render target
// do with it.  Bits 0-10 R and 11-21 G (5-bit exponent, 6-bit mantissa),
// bits 22-31 B (5-bit exponent, 5-bit mantissa); exponent bias 15, no sign;
// exponent 0 holds the denormals m * 2^-(14 + M), exponent 31 Inf (m = 0)
// or NaN.  Decoding is exact (ldexp); encoding rounds the scaled mantissa
// to nearest, ties to even (frexp + nearbyint); negative values and -0
// become 0, NaN stays NaN, values rounding past the largest finite become
// Inf.  Sampling an R11G11B10F texture reads alpha 1.
#ifndef LUXGI_ORACLE_PACKED_COLOR_H
#define LUXGI_ORACLE_PACKED_COLOR_H

#include <cstdint>

// (compiler builtins rather than <cmath>: the reference harness defines the
// GLSL built-ins of the same names at global scope)

namespace packed_color {

inline float uf_decode(uint32_t v, int M) {
    const uint32_t e = v >> M, m = v & ((1u << M) - 1u);
    if (e == 0) return __builtin_ldexpf(float(m), -(14 + M));
    if (e == 31) return m ? __builtin_nanf("") : __builtin_inff();
    return __builtin_ldexpf(1.0f + float(m) / float(1u << M), int(e) - 15);
}

inline uint32_t uf_encode(float x, int M) {
    if (x != x) return (31u << M) | ((1u << M) - 1u);
    if (!(x > 0.0f)) return 0u;
    if (__builtin_isinf(x)) return 31u << M;
    int k = 0;
    const float f = __builtin_frexpf(x, &k);           // x = f 2^k, f in [0.5, 1)
    int E = k - 1;                                     // x = (2f) 2^E
    if (E < -14) return uint32_t(__builtin_nearbyintf(__builtin_ldexpf(x, 14 + M)));   // 2^M: the smallest normal
    float q = __builtin_nearbyintf(__builtin_ldexpf(2.0f * f, M));                        // in [2^M, 2^(M+1)]
    if (q == float(1u << (M + 1))) { q = float(1u << M); ++E; }
    if (E + 15 >= 31) return 31u << M;
    return (uint32_t(E + 15) << M) | (uint32_t(q) - (1u << M));
}

inline uint32_t pack(const float* rgb) {
    return uf_encode(rgb[0], 6) | (uf_encode(rgb[1], 6) << 11) | (uf_encode(rgb[2], 5) << 22);
}

// channel ch (0-3) of a packed texel; alpha reads 1
inline float channel(uint32_t v, int ch) {
    if (ch == 0) return uf_decode(v & 0x7FFu, 6);
    if (ch == 1) return uf_decode((v >> 11) & 0x7FFu, 6);
    if (ch == 2) return uf_decode(v >> 22, 5);
    return 1.0f;
}

}  // namespace packed_color

#endif
