// Diagnostics: exhaustive error measurement of the approximate square root
// that the sweep's filter relies on (logo_diag_sqrt_error).
#include <cstring>

#include "../../include/logo_gpu.h"
#include "logo_device.cuh"

namespace {

// One thread per input bit pattern in [lo, hi): relative error of
// sqrt.approx.ftz.f32 against the correctly rounded root, as a double; the
// maximum is kept as ordered bits (non-negative doubles order like their
// bit patterns).
__global__ void sqrt_error_kernel(uint32_t lo, uint32_t hi,
                                  unsigned long long* max_bits) {
    double worst = 0.0;
    for (uint64_t b = (uint64_t)lo + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
         b < hi; b += (uint64_t)gridDim.x * blockDim.x) {
        const float s = __uint_as_float((uint32_t)b);
        float a;
        asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(s));
        const float e = __fsqrt_rn(s);
        const double rel = fabs((double)a - (double)e) / (double)e;
        worst = rel > worst ? rel : worst;
    }
    unsigned long long w = (unsigned long long)__double_as_longlong(worst);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long v = __shfl_xor_sync(0xffffffffu, w, o);
        w = v > w ? v : w;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(max_bits, w);
}

}  // namespace

extern "C" logo_status logo_diag_sqrt_error(int device, double* max_rel_err) {
    if (!max_rel_err) return LOGO_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return LOGO_ERR_NO_DEVICE;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return LOGO_ERR_OOM;
    cudaMemset(d, 0, sizeof(*d));
    // positive normal floats: 0x00800000 .. 0x7F7FFFFF
    sqrt_error_kernel<<<152 * 16, 256>>>(0x00800000u, 0x7F800000u, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return LOGO_ERR_CUDA;
    double v;
    std::memcpy(&v, &h, sizeof(v));
    *max_rel_err = v;
    return LOGO_OK;
}
