// Measured arithmetic peaks of the current device, for the compute side of the roofline figures
// (instrumentation only; no reference counterpart).  Each thread runs 8 independent fused
// multiply-add chains in a loop (enough independent work to cover the pipe latency), on a grid of
// 8 blocks of 256 threads per SM; the rate is FMA lane operations per second (x2 for flops).
#include <cuda_runtime.h>

#include "../../include/intfadv.h"
#include "capi_internal.cuh"

namespace {

constexpr int kIters = 2048;

template <class T>
__global__ void __launch_bounds__(256) fma_chains_k(T* out, T b, T c) {
    T a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = T(threadIdx.x + k) * T(1e-3);
#pragma unroll 16
    for (int it = 0; it < kIters; ++it) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
    if (s == T(12345.678)) out[0] = s;   // never true for these inputs; keeps the chains live
}

template <class T>
double fma_rate(void* scratch, int sms, cudaStream_t st) {
    const dim3 grid(sms * 8), block(256);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains_k<T><<<grid, block, 0, st>>>(static_cast<T*>(scratch), T(0.999999), T(1e-6));   // warm-up
    ia::note_launch();
    cudaEventRecord(e0, st);
    const int reps = 5;
    for (int r = 0; r < reps; ++r) {
        fma_chains_k<T><<<grid, block, 0, st>>>(static_cast<T*>(scratch), T(0.999999), T(1e-6));
        ia::note_launch();
    }
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double ops = double(grid.x) * block.x * kIters * 8.0 * reps;
    return ms > 0.f ? ops / (ms * 1e-3) : 0.0;
}

}  // namespace

extern "C" int ia_probe_fma_rates(double* fp64_fma_per_s, double* fp32_fma_per_s) {
    if (!fp64_fma_per_s || !fp32_fma_per_s) return IA_ERR_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return IA_ERR_NO_DEVICE;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    void* scratch = nullptr;
    if (cudaMalloc(&scratch, 64) != cudaSuccess) return IA_ERR_CUDA;
    *fp64_fma_per_s = fma_rate<double>(scratch, sms, nullptr);
    *fp32_fma_per_s = fma_rate<float>(scratch, sms, nullptr);
    const cudaError_t e = cudaGetLastError();
    cudaFree(scratch);
    return e == cudaSuccess ? IA_OK : IA_ERR_CUDA;
}
