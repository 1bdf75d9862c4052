// FMA-throughput probe (mpgos_probe_fma_peak in mpgos.h): the measured FP64
// and FP32 peaks the per-thread kernels are measured against.
#include "mpgos.h"

#include <cuda_runtime.h>

#include <string>

#define MPGOS_EXPORT extern "C" __attribute__((visibility("default")))

namespace {

constexpr int kChains = 8;
constexpr int kIters  = 2048;

// kChains independent FMA chains per thread; the result is stored only if a
// runtime flag says so, which keeps the chains live without memory traffic.
template <class T>
__global__ void fma_chains(T seed, T mul, int store, T* out)
{
    T a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = seed + static_cast<T>(threadIdx.x + c);
    for (int i = 0; i < kIters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) a[c] = fma(a[c], mul, seed);
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += a[c];
    if (store) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T>
cudaError_t run(int sms, double* flops)
{
    const int block = 256, grid = sms * 8;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_chains<T><<<grid, block>>>(static_cast<T>(1.0), static_cast<T>(0.999999), 0, nullptr);  // warm-up
    cudaEventRecord(e0);
    const int reps = 5;
    for (int r = 0; r < reps; r++)
        fma_chains<T><<<grid, block>>>(static_cast<T>(1.0), static_cast<T>(0.999999), 0, nullptr);
    cudaEventRecord(e1);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double fmas = static_cast<double>(reps) * grid * block * kChains * kIters;
    *flops = 2.0 * fmas / (static_cast<double>(ms) * 1e-3);
    return e;
}

}  // namespace

MPGOS_EXPORT int mpgos_probe_fma_peak(int device, int32_t precision_bytes, double* flops_per_second)
{
    if (flops_per_second == nullptr || (precision_bytes != 4 && precision_bytes != 8)) return MPGOS_ERR_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return MPGOS_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MPGOS_ERR_CUDA;
    cudaError_t e = precision_bytes == 8 ? run<double>(sms, flops_per_second) : run<float>(sms, flops_per_second);
    return e == cudaSuccess ? MPGOS_OK : MPGOS_ERR_CUDA;
}
