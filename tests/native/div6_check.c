/* Exhaustive check of the division by 6 in the smoothers' interior path
 * (div6_rn, flub_gb300/csrc/smooth8.cuh): Markstein's FMA correction of a * RN(1/6)
 * against IEEE single-precision a / 6.0f, bit for bit, for every float32 a
 * with |a| in [2^-100, 2^100] (the range the kernel sends through it), and
 * the two zeros, for which the kernel returns the product a * RN(1/6).
 * Prints the number of mismatches and exits 1 if there is any. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

int main(void) {
    const float y = 0x1.555556p-3f; /* 1/6 rounded to nearest */
    long long checked = 0, bad = 0;
#pragma omp parallel for reduction(+ : checked, bad) schedule(static)
    for (int64_t u = 0; u < (1LL << 32); u++) {
        const uint32_t bits = (uint32_t)u;
        float a;
        memcpy(&a, &bits, 4);
        const float m = fabsf(a);
        const int zero = m == 0.0f;
        if (!(m >= 0x1p-100f && m <= 0x1p100f) && !zero) continue;
        const float ref = a / 6.0f;
        const float q0 = a * y;
        const float q = zero ? q0 : fmaf(fmaf(-q0, 6.0f, a), y, q0);
        uint32_t b1, b2;
        memcpy(&b1, &ref, 4);
        memcpy(&b2, &q, 4);
        checked++;
        bad += b1 != b2;
    }
    printf("checked %lld, mismatches %lld\n", checked, bad);
    return bad != 0;
}
