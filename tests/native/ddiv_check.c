/* Randomised check of the FP64 bottom's division by the diagonal count d
 * (1..6) in flub_gb300/csrc/tail.cuh: Markstein's FMA correction of
 * a * RN(1/d) against IEEE double a / d, bit for bit, for 2^28 random
 * doubles per d with |a| in [2^-900, 2^900] (uniform exponent, random
 * mantissa and sign), and the zeros, for which the kernel returns the
 * product a * RN(1/d).  Exits 1 on any mismatch. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static uint64_t splitmix(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main(void) {
    long long bad = 0, checked = 0;
    for (int d = 1; d <= 6; d++) {
        const double y = 1.0 / (double)d;
#pragma omp parallel for reduction(+ : bad, checked) schedule(static)
        for (int64_t t = 0; t < (1LL << 28); t++) {
            uint64_t s = (uint64_t)t * 6 + (uint64_t)d;
            const uint64_t r1 = splitmix(&s);
            const int e = (int)(r1 % 1801) - 900;
            const uint64_t mant = splitmix(&s) & ((1ull << 52) - 1);
            uint64_t bits = ((uint64_t)(e + 1023) << 52) | mant | ((r1 >> 63) << 63);
            double a;
            memcpy(&a, &bits, 8);
            const double ref = a / (double)d;
            const double q0 = a * y;
            const double q = fma(fma(-q0, (double)d, a), y, q0);
            uint64_t b1, b2;
            memcpy(&b1, &ref, 8);
            memcpy(&b2, &q, 8);
            checked++;
            bad += b1 != b2;
        }
    }
    /* the zeros return the product a * RN(1/d), a zero of a's sign */
    for (int d = 1; d <= 6; d++)
        for (int sg = 0; sg < 2; sg++) {
            const double a = sg ? -0.0 : 0.0, ref = a / (double)d, q = a * (1.0 / (double)d);
            uint64_t b1, b2;
            memcpy(&b1, &ref, 8);
            memcpy(&b2, &q, 8);
            bad += b1 != b2;
        }
    printf("checked %lld, mismatches %lld\n", checked, bad);
    return bad != 0;
}
