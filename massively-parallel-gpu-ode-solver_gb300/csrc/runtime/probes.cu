// FMA-throughput probe (mpgos_probe_fma_peak in mpgos.h): the measured FP64
// and FP32 peaks the per-thread kernels are measured against; and the
// double-float math probe (mpgos_probe_df_math): the device build of the
// DF_STAGE arithmetic evaluated on given arguments.
#include "mpgos.h"
#include "df_convert.cuh"

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

// one double-float operation per element; out[2i], out[2i+1] = hi, lo
__global__ void df_math(int32_t op, long long n, const double* a, const double* b, double* out)
{
    using mpgos::df::dfloat;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        if (op >= MPGOS_DF_SPLIT) {
            // SPLIT-mode operations on the doubles themselves
            if (op == MPGOS_DF_SPLIT) {
                const dfloat r = mpgos::df::split(a[i]);
                out[2 * i]     = static_cast<double>(r.hi);
                out[2 * i + 1] = static_cast<double>(r.lo);
            } else {
                const bool fifth = op == MPGOS_DF_ROOT5;
                const float l    = mpgos::df::log2_estimate(a[i]) - mpgos::df::log2_estimate(b[i]);
                out[2 * i]       = mpgos::df::root_refine(mpgos::df::root_estimate(l, fifth), a[i], b[i], fifth);
                out[2 * i + 1]   = 0.0;
            }
            continue;
        }
        const dfloat x(a[i]), y(b[i]);
        dfloat r;
        switch (op) {
            case MPGOS_DF_EXP: r = mpgos::df::exp(x); break;
            case MPGOS_DF_LOG: r = mpgos::df::log(x); break;
            case MPGOS_DF_POW: r = mpgos::df::pow(x, y); break;
            case MPGOS_DF_SIN: r = mpgos::df::sin(x); break;
            case MPGOS_DF_COS: r = mpgos::df::cos(x); break;
            case MPGOS_DF_SQRT: r = mpgos::df::sqrt(x); break;
            case MPGOS_DF_DIV: r = x / y; break;
            case MPGOS_DF_MUL: r = x * y; break;
            case MPGOS_DF_ADD: r = x + y; break;
            case MPGOS_DF_SINPI: { dfloat c; mpgos::df::sincospi(x, &r, &c); break; }
            case MPGOS_DF_COSPI: { dfloat s; mpgos::df::sincospi(x, &s, &r); break; }
            default: r = mpgos::df::pow(x, static_cast<int>(b[i])); break;
        }
        out[2 * i]     = static_cast<double>(r.hi);
        out[2 * i + 1] = static_cast<double>(r.lo);
    }
}

}  // namespace

MPGOS_EXPORT int mpgos_probe_df_math(int device, int32_t op, int64_t n, const double* a, const double* b,
                                     double* out)
{
    if (n < 0 || op < MPGOS_DF_EXP || op > MPGOS_DF_ROOT4 || (n > 0 && (a == nullptr || b == nullptr || out == nullptr)))
        return MPGOS_ERR_ARGUMENT;
    if (n == 0) return MPGOS_OK;
    if (cudaSetDevice(device) != cudaSuccess) return MPGOS_ERR_CUDA;
    const size_t bytes = static_cast<size_t>(n) * sizeof(double);
    double *da = nullptr, *db = nullptr, *dout = nullptr;
    cudaError_t e = cudaMalloc(&da, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&db, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&dout, 2 * bytes);
    if (e == cudaSuccess) e = cudaMemcpy(da, a, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(db, b, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const int blocks = static_cast<int>(n / 256 + 1 < 4096 ? n / 256 + 1 : 4096);
        df_math<<<blocks, 256>>>(op, n, da, db, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, 2 * bytes, cudaMemcpyDeviceToHost);
    for (double* p : {da, db, dout})
        if (p) cudaFree(p);
    return e == cudaSuccess ? MPGOS_OK : MPGOS_ERR_CUDA;
}

MPGOS_EXPORT int mpgos_probe_fma_peak(int device, int32_t precision_bytes, double* flops_per_second)
{
    if (flops_per_second == nullptr || (precision_bytes != 4 && precision_bytes != 8)) return MPGOS_ERR_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return MPGOS_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return MPGOS_ERR_CUDA;
    cudaError_t e = precision_bytes == 8 ? run<double>(sms, flops_per_second) : run<float>(sms, flops_per_second);
    return e == cudaSuccess ? MPGOS_OK : MPGOS_ERR_CUDA;
}
