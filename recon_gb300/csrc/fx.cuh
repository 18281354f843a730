// fx.cuh -- exact fixed-point accumulation of FP32 values on the GPU.
//
// A value is the integer sum_k L[k] * 2^(32k) in units of 2^-64, held as four
// 64-bit limb sums.  An FP32 input is truncated toward zero at 2^-64 and splits
// into at most two adjacent 32-bit pieces, so limb sums never carry and can be
// added with plain integer atomics in any order: the total is the exact sum of
// the inputs.  It is rounded once to FP64 (nearest, ties to even) with integer
// arithmetic only.  Inputs must satisfy |v| < 2^48; Inf, NaN and larger values
// set a flag instead.  The oracle's orc_fx_add / orc_fx_to_double are the same
// definition.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "track_kernels.cuh"

namespace rt {

// v -> (limb index k0, piece for limb k0, piece for limb k0+1); sets bad when
// v is out of range.  Zero pieces mean nothing to add.
__device__ __forceinline__ void fx_split(float v, int &k0, long long &lo, long long &hi, int &bad) {
    uint32_t bits = __float_as_uint(v);
    uint32_t E = (bits >> 23) & 0xffu, M = bits & 0x7fffffu;
    k0 = 0;
    lo = 0;
    hi = 0;
    if (E == 0xffu) { bad = 1; return; }
    uint64_t m = (E == 0) ? (uint64_t)M : (uint64_t)(M | 0x800000u);
    int e = (E == 0) ? -149 : (int)E - 150;
    if (m == 0) return;
    if (e >= 25) { bad = 1; return; }
    int s = e + 64;
    if (s < 0) {
        m = (-s >= 24) ? 0 : (m >> -s);
        s = 0;
    }
    uint64_t t = m << (s & 31);
    k0 = s >> 5;
    lo = (long long)(t & 0xffffffffu);
    hi = (long long)(t >> 32);
    if (bits >> 31) { lo = -lo; hi = -hi; }
}

__device__ __forceinline__ double fx_to_double(const long long *L) {
    unsigned __int128 Q = 0;
#pragma unroll
    for (int k = kFxLimbs - 1; k >= 0; k--) Q = (Q << 32) + (unsigned __int128)(__int128)L[k];
    bool neg = (uint64_t)(Q >> 127) != 0;
    unsigned __int128 U = neg ? (unsigned __int128)0 - Q : Q;
    if (U == 0) return 0.0;
    uint64_t hi = (uint64_t)(U >> 64), lo = (uint64_t)U;
    int n = hi ? 127 - __clzll((long long)hi) : 63 - __clzll((long long)lo);
    uint64_t mant;
    int e2;
    if (n <= 52) {
        mant = (uint64_t)U << (52 - n);
        e2 = -64 - (52 - n);
    } else {
        int sh = n - 52;
        mant = (uint64_t)(U >> sh);
        unsigned __int128 rem = U - ((unsigned __int128)mant << sh);
        unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        if (rem > half || (rem == half && (mant & 1))) mant++;
        if (mant >> 53) {
            mant >>= 1;
            sh++;
        }
        e2 = sh - 64;
    }
    uint64_t out = ((uint64_t)(e2 + 52 + 1023) << 52) | (mant & ((1ull << 52) - 1));
    if (neg) out |= 1ull << 63;
    return __longlong_as_double((long long)out);
}

}  // namespace rt
