/* Host check of the fixed-divisor division sequence of the neighbour passes
 * (q0 = RN(a*y), r = fma(-q0, b, a), q = fma(r, y, q0), y = RN(1/b)): a divisor that
 * passes on every significand of the binade [1, 2) must give the IEEE quotient for every
 * dividend of magnitude in [2^-100, 2^100] (the scaling argument of xdiv_fixed_nz), and
 * the sign fix must return -0 for -0.  Prints "ok <divisors verified> <dividends tested>"
 * or the first counterexample.  Built with -ffp-contract=off. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

static float seq(float a, float b, float y) {
    const float q0 = a * y;
    const float r = fmaf(-q0, b, a);
    return fmaf(r, y, q0);
}

static int verified(float b, float y) {
    for (uint32_t m = 0; m < (1u << 23); ++m) {
        const float a = f_of(0x3f800000u | m);
        if (seq(a, b, y) != a / b) return 0;
    }
    return 1;
}

static uint64_t state = 0x243F6A8885A308D3ull;
static uint64_t next(void) {  /* splitmix64 */
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main(void) {
    const float hs[] = {0.02f, 0.01f, 0.015f, 0.0123f, 0.05f, 1.0f, 3.7f, 1e-3f, 250.0f};
    int nver = 0;
    long tested = 0;
    for (unsigned k = 0; k < sizeof(hs) / sizeof(hs[0]); ++k) {
        for (int sq = 0; sq < 2; ++sq) {
            const float b = sq ? hs[k] * hs[k] : hs[k];
            const float y = 1.0f / b;
            if (!verified(b, y)) continue;
            ++nver;
            for (int i = 0; i < (1 << 19); ++i) {
                const uint64_t z = next();
                const int e = (int)(z % 201) - 100;                 /* 2^-100 .. 2^100 */
                const uint32_t sig = (uint32_t)(z >> 20) & 0x7fffffu;
                const uint32_t sgn = (uint32_t)(z >> 63) << 31;
                const float a = f_of(sgn | ((uint32_t)(127 + e) << 23) | sig);
                const float q = seq(a, b, y), ref = a / b;
                ++tested;
                if (u_of(q) != u_of(ref)) {
                    printf("mismatch b=%a a=%a seq=%a ieee=%a\n", b, a, q, ref);
                    return 1;
                }
            }
            /* signed zeros: the sequence gives +0, the sign fix restores -0 */
            const float nz = -0.0f;
            const float q = seq(nz, b, y);
            const float fixed = f_of((u_of(q) & 0x7fffffffu) | (u_of(nz) & 0x80000000u));
            if (u_of(fixed) != u_of(nz / b) || u_of(seq(0.0f, b, y)) != u_of(0.0f / b)) {
                printf("zero sign b=%a\n", b);
                return 1;
            }
        }
    }
    printf("ok %d %ld\n", nver, tested);
    return nver > 0 ? 0 : 1;
}
