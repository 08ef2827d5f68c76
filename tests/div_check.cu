// Test-only: compares fwi::div_by_const (fwi_gb300/csrc/fwi_div.cuh) bit for
// bit with CUDA's IEEE division over all 2^32 single-precision values of the
// dividend, for one divisor b and its host reciprocal y = RN(1/b).
#include <cstdint>

#include "fwi_div.cuh"

namespace {

__global__ void k_check(float b, float y, unsigned long long* bad, unsigned* first) {
    const uint64_t n = 1ull << 32;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned u = (unsigned)i;
        const float a = __uint_as_float(u);
        const float ref = __fdiv_rn(a, b);
        const float got = fwi::div_by_const(a, b, y);
        const bool same = (__float_as_uint(ref) == __float_as_uint(got)) || (ref != ref && got != got);
        if (!same) {
            atomicAdd(bad, 1ull);
            atomicMin(first, u);
        }
    }
}

}  // namespace

extern "C" int div_check(float b, float y, unsigned long long* mismatches, unsigned* first_bad) {
    unsigned long long* d_bad = nullptr;
    unsigned* d_first = nullptr;
    if (cudaMalloc(&d_bad, sizeof *d_bad) != cudaSuccess) return 1;
    if (cudaMalloc(&d_first, sizeof *d_first) != cudaSuccess) return 1;
    const unsigned init = 0xffffffffu;
    cudaMemset(d_bad, 0, sizeof *d_bad);
    cudaMemcpy(d_first, &init, sizeof init, cudaMemcpyHostToDevice);
    k_check<<<152 * 16, 256>>>(b, y, d_bad, d_first);
    cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(mismatches, d_bad, sizeof *d_bad, cudaMemcpyDeviceToHost);
    cudaMemcpy(first_bad, d_first, sizeof *d_first, cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    cudaFree(d_first);
    return e == cudaSuccess ? 0 : 2;
}
