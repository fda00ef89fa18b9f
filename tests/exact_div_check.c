/* Host check of the march's exact quotient (xdiv in luxgi_common.cuh): for
 * a divisor d > 0 and y = RN(1 / d),
 *     q = RN(x y); r = RN(d q - x); q = RN(q - r y); r = RN(d q - x); q = RN(q - r y)
 * (each RN(a b + c) one fused multiply-add) must equal the IEEE quotient
 * RN(x / d) bit for bit, signed zeros included.  Away from the ends of the
 * normal range every intermediate scales exactly with x and with d, so the
 * sequence is checked over every significand of x (both signs, one binade)
 * for each divisor given, at a few exponent offsets of x, plus x = +-0.
 *
 * usage: exact_div_check d1 d2 ...   prints "ok N", or the divisor and
 * the count of mismatches and exits 1. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float from_bits(uint32_t b) { float x; memcpy(&x, &b, 4); return x; }
static uint32_t to_bits(float x) { uint32_t b; memcpy(&b, &x, 4); return b; }

static float xdiv(float x, float d, float y) {
    float q = x * y;
    float r = fmaf(d, q, -x);
    q = fmaf(-r, y, q);
    r = fmaf(d, q, -x);
    return fmaf(-r, y, q);
}

int main(int argc, char** argv) {
    static const int exps[] = {-40, 0, 1, 40};   /* exponent of x (unbiased) */
    long long checked = 0;
    for (int k = 1; k < argc; ++k) {
        const float d = strtof(argv[k], NULL);
        const float y = 1.0f / d;
        for (int s = 0; s < 2; ++s) {
            const float z = s ? -0.0f : 0.0f;
            if (to_bits(xdiv(z, d, y)) != to_bits(z / d)) {
                printf("mismatch d=%a x=%a\n", d, z);
                return 1;
            }
        }
        for (size_t e = 0; e < sizeof(exps) / sizeof(exps[0]); ++e) {
            long long bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
            for (int m = 0; m < (1 << 23); ++m) {
                for (uint32_t s = 0; s < 2; ++s) {
                    const float x = from_bits((s << 31) | ((uint32_t)(exps[e] + 127) << 23) | (uint32_t)m);
                    if (to_bits(xdiv(x, d, y)) != to_bits(x / d)) ++bad;
                }
            }
            if (bad) {
                printf("mismatch d=%a: %lld dividends of exponent %d\n", d, bad, exps[e]);
                return 1;
            }
            checked += 2ll << 23;
        }
    }
    printf("ok %lld\n", checked);
    return 0;
}
