/* exact_arith_check.c -- the truncation of recon_gb300/csrc/exact_arith.cuh
 * restated in C and compared with the C conversion on the host (gcc -O2
 * -ffp-contract=off): x + 2^23 rounded toward zero, minus the bits of 2^23,
 * for every float x in [2^22, 2^23) and every 97th float below.  The device
 * code itself is compared on the GPU by recon_selftest_exact_arith.  Prints
 * the mismatch count and exits 0 when it is zero. */
#include <fenv.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

static float f_of(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static uint32_t b_of(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

int main(void) {
    long long bad = 0, n = 0;
    fesetround(FE_TOWARDZERO);
    for (uint32_t k = 0; k < 0x4B000000u; k += (k < 0x4A800000u ? 97u : 1u)) {
        float x = f_of(k);
        volatile float s = x + 8388608.0f;
        int t = (int)(b_of(s) - 0x4B000000u);
        bad += t != (int)x;
        n++;
    }
    fesetround(FE_TONEAREST);
    printf("trunc %lld/%lld\n", bad, n);
    return bad ? 1 : 0;
}
