// Peak arithmetic throughput of the non-tensor FP pipes (FP64 / FP32 FMA),
// used as the roofline denominator of the FP64-bound WENO kernels: the
// measured HBM and bf16-tensor peaks do not bound this path.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/shocks.h"

namespace {

template <class T, int CHAINS>
__global__ void __launch_bounds__(256) fma_chains(T* out, int iters, T a, T b) {
    T x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = T(threadIdx.x + c) * T(1e-3);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
    }
    T s = T(0);
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    if (s == T(12345.678)) out[threadIdx.x] = s;  // keeps the chains alive
}

template <class T>
int run(double* flops_per_s, int iters) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    T* out = nullptr;
    if (cudaMalloc(&out, 256 * sizeof(T)) != cudaSuccess) return SHK_ENOMEM;
    constexpr int kChains = 8;
    const int blocks = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T, kChains><<<blocks, 256>>>(out, iters / 10 + 1, T(0.999999), T(1e-7));
    cudaEventRecord(e0);
    fma_chains<T, kChains><<<blocks, 256>>>(out, iters, T(0.999999), T(1e-7));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return SHK_ECUDA;
    const double fmas = double(blocks) * 256.0 * kChains * double(iters);
    *flops_per_s = 2.0 * fmas / (double(ms) * 1e-3);
    return SHK_OK;
}

}  // namespace

extern "C" int shk_measure_fp_peak(int32_t dtype, int32_t iters, double* flops_per_s) {
    if (!flops_per_s || iters <= 0) return SHK_EINVAL;
    return dtype == SHK_F64 ? run<double>(flops_per_s, iters) : run<float>(flops_per_s, iters);
}
