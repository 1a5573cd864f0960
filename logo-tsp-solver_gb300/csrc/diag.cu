// Diagnostics: exhaustive error measurement of the approximate square root
// that the sweep's filter relies on (logo_diag_sqrt_error), and a check that
// the device-side waits give up (logo_diag_wait_limits).
#include <cstring>

#include <chrono>

#include "../../include/logo_gpu.h"
#include "logo_device.cuh"
#include "logo_internal.h"

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

// An mbarrier that is told to expect 16 bytes which no copy will deliver:
// the bounded wait of the sweep kernels gives up after its budget and sets
// kErrTimeout.  No copy is in flight when the CTA exits.
__global__ void mbar_probe_kernel(unsigned int* status) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        logo::mbar_init(&bar, 1);
        logo::fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) logo::mbar_arrive_expect_tx(&bar, 16);
    __syncthreads();
    logo::mbar_wait_bounded(&bar, 0, status);
}

}  // namespace

extern "C" logo_status logo_diag_wait_limits(int device, uint32_t* mbarrier_status,
                                             uint32_t* barrier_status, double* waited_ms) {
    if (!mbarrier_status || !barrier_status) return LOGO_ERR_INVALID_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return LOGO_ERR_NO_DEVICE;
    unsigned int* d_status = nullptr;
    logo::CoopSync* cs = nullptr;
    logo::DevState* st = nullptr;
    logo_status rc = LOGO_OK;
    if (cudaMalloc(&d_status, sizeof(unsigned int)) != cudaSuccess ||
        cudaMalloc(&cs, sizeof(logo::CoopSync)) != cudaSuccess ||
        cudaMalloc(&st, sizeof(logo::DevState)) != cudaSuccess) {
        rc = LOGO_ERR_OOM;
    } else {
        cudaMemset(d_status, 0, sizeof(unsigned int));
        cudaMemset(cs, 0, sizeof(logo::CoopSync));
        cudaMemset(st, 0, sizeof(logo::DevState));
        const auto t0 = std::chrono::steady_clock::now();
        mbar_probe_kernel<<<1, 32>>>(d_status);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) e = logo::launch_barrier_probe(cs, st, nullptr);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        const auto t1 = std::chrono::steady_clock::now();
        unsigned int a = 0, b = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&a, d_status, sizeof(a), cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(&b, &st->status, sizeof(b), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            rc = LOGO_ERR_CUDA;
        } else {
            *mbarrier_status = a;
            *barrier_status = b;
            if (waited_ms)
                *waited_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
        }
    }
    cudaFree(d_status);
    cudaFree(cs);
    cudaFree(st);
    return rc;
}

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
