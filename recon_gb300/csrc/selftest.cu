// selftest.cu -- compares the truncation of the Student-t variance sums
// (exact_arith.cuh) with the conversion it replaces, on the GPU the library
// runs on.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/recon_track.h"
#include "exact_arith.cuh"

namespace rt {

void set_last_error(const char *msg);

namespace {

__device__ __forceinline__ void add_count(unsigned long long *dst, unsigned long long c) {
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(dst, c);
}

// every float x in [0, 2^23): trunc_small(x) against (int)x
__global__ void k_check_trunc(unsigned long long *bad) {
    unsigned long long c = 0;
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < 0x4B000000u; b += stride) {
        float x = __uint_as_float(b);
        c += trunc_small(x) != (int)x;
    }
    add_count(bad, c);
}

}  // namespace
}  // namespace rt

extern "C" int recon_selftest_exact_arith(int64_t *mismatches) {
    using namespace rt;
    if (!mismatches) {
        set_last_error("recon_selftest_exact_arith: null argument");
        return RECON_ERR_INVALID_ARG;
    }
    unsigned long long *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        k_check_trunc<<<152 * 8, 256>>>(d);
        e = cudaGetLastError();
    }
    unsigned long long h = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    if (d) cudaFree(d);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return RECON_ERR_CUDA;
    }
    *mismatches = (int64_t)h;
    return RECON_OK;
}
