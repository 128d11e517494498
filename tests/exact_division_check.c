/* Exhaustive check of the library's division by the map resolution (div_res in
 * supereight2_gb300/csrc/se_gpu_internal.cuh): for every float x in [lo, hi) the sequence
 * q = RN(x r), e = RN(fma(-q, res, x)), q' = RN(fma(e, r, q)) with r = RN(1 / res) must equal the
 * IEEE quotient RN(x / res). Usage: exact_division_check res lo_bits hi_bits; prints the number
 * of mismatches. Built with -ffp-contract=off; fmaf is the C library's correctly rounded fma. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static float bits_to_float(uint32_t u)
{
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}

int main(int argc, char** argv)
{
    if (argc != 4)
        return 2;
    volatile float res = strtof(argv[1], NULL);
    const uint32_t lo = (uint32_t) strtoul(argv[2], NULL, 0), hi = (uint32_t) strtoul(argv[3], NULL, 0);
    const float r = 1.0f / res;
    unsigned long long bad = 0, n = 0;
    for (uint32_t u = lo; u < hi; ++u) {
        const float x = bits_to_float(u);
        const float q = x * r;
        const float q2 = fmaf(fmaf(-q, res, x), r, q);
        if (q2 != x / res || bits_to_float(u | 0x80000000u) / res != -q2)
            ++bad;
        ++n;
    }
    printf("%llu %llu\n", bad, n);
    return 0;
}
