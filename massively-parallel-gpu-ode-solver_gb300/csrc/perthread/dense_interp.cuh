// Dense-output interpolation (extension; the reference stores the accepted
// (t, x) points only, SingleSystem_PerThread_DenseOutput.cuh:5-58).
//
// For each requested time tau and instance, the stored points bracketing tau,
// (t_k, x_k) and (t_k+1, x_k+1), are joined by the cubic Hermite polynomial
// whose end slopes are the user's right-hand side at the two points:
//     h = t_k+1 - t_k,  s = (tau - t_k) / h,
//     x(tau) = (1+2s)(1-s)^2 x_k + s(1-s)^2 h f_k + s^2(3-2s) x_k+1 + s^2(s-1) h f_k+1,
// fourth-order accurate in h between consecutive accepted steps. The
// right-hand side is evaluated with the instance's control parameters, the
// shared parameters and the accessories as they are at the call. tau outside
// [t_0, t_last] of an instance (or an instance with no stored point) gives NaN.
// The polynomial assumes the solution is smooth between the two points: across
// a discontinuity made by an event action the value is meaningless.
#pragma once

namespace mpgos {
namespace pt {

// Index k of the last stored time <= tau among t_0..t_{n-1} (ascending), -1
// when tau < t_0. Binary search over the instance's column of DenseTime.
template <class P>
__device__ __forceinline__ int dense_bracket(const P* dtime, long long i, long long nt, int n, double tau)
{
    int lo = 0, hi = n - 1;
    if (!(static_cast<double>(dtime[i]) <= tau)) return -1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (static_cast<double>(dtime[i + static_cast<long long>(mid) * nt]) <= tau) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// One thread per instance, every requested time: out[j][c][i] (FP64).
template <class S, class P>
__global__ void __launch_bounds__(MPGOS_MAX_BLOCK) dense_interp_kernel(Args<P> a, const double* times, int n_times,
                                                                       double* out)
{
    constexpr int SD = S::SD, NCP = S::NCP, NSP = S::NSP, NISP = S::NISP, NA = S::NA, NIA = S::NIA;
    extern __shared__ __align__(16) unsigned char mpgos_dyn_smem[];
    P* sp    = reinterpret_cast<P*>(mpgos_dyn_smem);
    int* spi = reinterpret_cast<int*>(mpgos_dyn_smem + sizeof(P) * NSP);
    for (int k = threadIdx.x; k < NSP; k += blockDim.x) sp[k] = a.sp[k];
    for (int k = threadIdx.x; k < NISP; k += blockDim.x) spi[k] = a.spi[k];
    __syncthreads();

    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= a.n_active) return;
    const long long nt = a.nt;
    const int ti = static_cast<int>(i), nti = static_cast<int>(nt);
    P cp[AtLeastOne<NCP>::value];
    P acc[AtLeastOne<NA>::value];
    int acci[AtLeastOne<NIA>::value];
#pragma unroll
    for (int k = 0; k < NCP; k++) cp[k] = a.cp[i + k * nt];
#pragma unroll
    for (int k = 0; k < NA; k++) acc[k] = a.acc[i + k * nt];
#pragma unroll
    for (int k = 0; k < NIA; k++) acci[k] = a.acci[i + k * nt];
    const int n = min(a.didx[i], a.o.ndo);
    const long long step = nt * SD;  // stride of one stored point in DenseState

    int kc = -2;  // bracket whose end slopes are held in f0 / f1
    P x0[SD], x1[SD], f0[SD], f1[SD];
    double t0 = 0.0, t1 = 0.0;
    for (int j = 0; j < n_times; j++) {
        const double tau = times[j];
        double* o = out + static_cast<long long>(j) * step + i;
        const int k = (n > 0) ? dense_bracket(a.dtime, i, nt, n, tau) : -1;
        const bool inside = k >= 0 && (k < n - 1 || static_cast<double>(a.dtime[i + static_cast<long long>(k) * nt]) == tau);
        if (!inside) {
#pragma unroll
            for (int c = 0; c < SD; c++) o[c * nt] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        if (k == n - 1) {  // tau is the last stored time
#pragma unroll
            for (int c = 0; c < SD; c++) o[c * nt] = static_cast<double>(a.dstate[i + c * nt + k * step]);
            continue;
        }
        if (k != kc) {
            t0 = static_cast<double>(a.dtime[i + static_cast<long long>(k) * nt]);
            t1 = static_cast<double>(a.dtime[i + static_cast<long long>(k + 1) * nt]);
#pragma unroll
            for (int c = 0; c < SD; c++) {
                x0[c] = a.dstate[i + c * nt + k * step];
                x1[c] = a.dstate[i + c * nt + (k + 1) * step];
            }
            PerThread_OdeFunction(ti, nti, f0, x0, static_cast<P>(t0), cp, sp, spi, acc, acci);
            PerThread_OdeFunction(ti, nti, f1, x1, static_cast<P>(t1), cp, sp, spi, acc, acci);
            kc = k;
        }
        const double h = t1 - t0;
        if (!(h > 0.0)) {  // repeated time stamp: the later point
#pragma unroll
            for (int c = 0; c < SD; c++) o[c * nt] = static_cast<double>(x1[c]);
            continue;
        }
        const double s = (tau - t0) / h, r = 1.0 - s;
        const double h00 = (1.0 + 2.0 * s) * r * r, h10 = s * r * r * h;
        const double h01 = s * s * (3.0 - 2.0 * s), h11 = s * s * (s - 1.0) * h;
#pragma unroll
        for (int c = 0; c < SD; c++)
            o[c * nt] = h00 * static_cast<double>(x0[c]) + h10 * static_cast<double>(f0[c]) +
                        h01 * static_cast<double>(x1[c]) + h11 * static_cast<double>(f1[c]);
    }
}

template <class S, class P>
struct DenseInterpTable {
    static int launch(const mpgos_pt_launch* L, const double* times, int32_t n_times, double* out, int grid,
                      int block, size_t smem, void* stream)
    {
        Args<P> a = make_args<P>(*L);
        int n = n_times;
        void* params[] = {&a, &times, &n, &out};
        return static_cast<int>(cudaLaunchKernel(reinterpret_cast<void*>(&dense_interp_kernel<S, P>), dim3(grid),
                                                 dim3(block), params, smem, static_cast<cudaStream_t>(stream)));
    }
};

}  // namespace pt
}  // namespace mpgos
