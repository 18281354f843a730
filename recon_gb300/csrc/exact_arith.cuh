// exact_arith.cuh -- the int truncation of the Student-t variance sums in two
// instructions instead of a bit-field extraction.
//
// trunc_small(x) = (int)x for 0 <= x < 2^23: x + 2^23 rounded toward zero is
// 2^23 + trunc(x) exactly (the ulp of [2^23, 2^24) is 1), so the integer is the
// sum's bits minus those of 2^23.  recon_selftest_exact_arith compares it with
// the conversion for every float in that range on the GPU.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rt {

__device__ __forceinline__ int trunc_small(float x) {
    return (int)(__float_as_uint(__fadd_rz(x, 8388608.0f)) - 0x4B000000u);
}

}  // namespace rt
