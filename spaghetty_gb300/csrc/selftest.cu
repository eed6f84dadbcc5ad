// selftest.cu -- on-device check of the integer-pipe double addition
// (arith.cuh) against the FP64 pipe's __dadd_rn.
#include "../../include/spaghetty_gb300.h"
#include "arith.cuh"

#include <cuda_runtime.h>

#include <cstring>

namespace {

__device__ __forceinline__ uint64_t spg_mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Operand i of the test: exponent gaps of every size, equal, all-ones and
// single-bit significands, powers of two (exact ties), both signs, and
// every IEEE class (zero, subnormal, inf, NaN) now and then.
__device__ void spg_operands(uint64_t i, uint64_t seed, double *a, double *b) {
    const uint64_t r1 = spg_mix64(seed + 3 * i), r2 = spg_mix64(seed + 3 * i + 1), r3 = spg_mix64(seed + 3 * i + 2);
    const uint64_t cls = (r3 >> 56) & 31;
    uint64_t ea = 1 + r3 % 2046;
    const int64_t gap = ((r3 >> 50) & 1) ? (int64_t)((r3 >> 12) % 8) + 50 - (int64_t)((r3 >> 51) & 1) * 100
                                         : (int64_t)((r3 >> 12) % 140) - 70;
    int64_t eb = (int64_t)ea + gap;
    eb = eb < 0 ? 0 : (eb > 2047 ? 2047 : eb);
    uint64_t ma = r1, mb = r2;
    switch ((r3 >> 20) % 8) {
        case 0: mb = ma; break;
        case 1: mb = ma ^ 1; break;
        case 2: ma |= 0xFFFFFFFFFFFFFull; break;
        case 3: mb &= 0xFFF0000000000ull; break;
        case 4: ma &= ~0xFFFull; mb |= 0x7FFull; break;
        case 5: mb = 0; break;
        case 6: mb = 1; ma = (r1 & 1) ? 0 : ~0ull; break;
        default: break;
    }
    if (cls == 0) ea = 0;                          // zero or subnormal
    if (cls == 1) ea = 0x7FF;                      // inf or NaN
    if (cls == 2) { ea = 0; ma = 0; }              // signed zero
    const uint64_t M = (1ull << 52) - 1;
    const uint64_t ua = (((r3 >> 40) & 1) << 63) | (ea << 52) | (ma & M);
    const uint64_t ub = (((r3 >> 41) & 1) << 63) | ((uint64_t)eb << 52) | (mb & M);
    *a = __longlong_as_double((long long)ua);
    *b = __longlong_as_double((long long)ub);
}

__global__ void spg_selftest_add_kernel(uint64_t n, uint64_t seed, unsigned long long *bad) {
    unsigned long long mine = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        double a, b;
        spg_operands(i, seed, &a, &b);
        const double want = __dadd_rn(a, b);
        const double got = spg_dadd_int(a, b);
        const long long w = __double_as_longlong(want), g = __double_as_longlong(got);
        // NaN results: any NaN matches (the payload is not part of the contract)
        const bool nan_w = (w & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll;
        const bool nan_g = (g & 0x7FFFFFFFFFFFFFFFll) > 0x7FF0000000000000ll;
        if (w != g && !(nan_w && nan_g)) ++mine;
    }
    if (mine) atomicAdd(bad, mine);
}

}  // namespace

extern "C" long long spaghetty_selftest_device(long long n) {
    if (n <= 0) return 0;
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) {
        cudaGetLastError();
        return -SPAGHETTY_ERR_CUDA;
    }
    unsigned long long h = 0;
    long long rc = -SPAGHETTY_ERR_CUDA;
    if (cudaMemset(d, 0, sizeof(*d)) == cudaSuccess) {
        spg_selftest_add_kernel<<<1216, 256>>>((uint64_t)n, 0x5EEDull, d);
        if (cudaGetLastError() == cudaSuccess && cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess)
            rc = (long long)h;
    }
    cudaGetLastError();
    cudaFree(d);
    return rc;
}
