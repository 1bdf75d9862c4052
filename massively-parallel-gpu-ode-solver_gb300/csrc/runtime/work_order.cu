// Work order of the per-thread instances (MPGOS_WORK_ORDER).
//
// Before a launch, the instances 0 .. n-1 are ordered longest first by the
// step attempts (accepted + rejected) each took in the previous launch, so
// that the persistent queue and the static lanes start the instances that
// will run longest first and the last wave of the launch is short (the
// longest-processing-time-first rule), and the lanes of a warp hold instances
// of similar length. On the uneven Keller-Miksis grid (47 .. 2018 steps per
// instance and period) this order cut the persistent SPLIT form from 1745 to
// 1145 ms for 16 periods.
//
// A counting sort on a logarithmic key: 16 buckets per octave of the attempt
// count (instances in one bucket differ by less than 4.5 %), buckets in
// decreasing order. Three launches on the solver's stream (so a CUDA graph of
// phases captures them): a histogram (per block in shared memory, then one
// atomic per bucket and block), an exclusive scan of the 512 counts in one
// block, and a scatter in which every block reserves its range per bucket with
// one atomic. The order inside a bucket is whatever the atomics give; no
// instance's result depends on it.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

constexpr int kOrderBuckets = 512;  // 16 per octave, attempt counts below 2^31
constexpr int kOrderBlock = 256;

__device__ __forceinline__ int order_bucket(const int32_t* nacc, const int32_t* nrej, long long i)
{
    const int a = max(nacc[i], 0) + max(nrej[i], 0);
    const int b = static_cast<int>(__log2f(static_cast<float>(a) + 1.0f) * 16.0f);
    return kOrderBuckets - 1 - min(max(b, 0), kOrderBuckets - 1);  // longest first
}

__global__ void order_count(const int32_t* nacc, const int32_t* nrej, long long n, unsigned* counts)
{
    __shared__ unsigned s[kOrderBuckets];
    for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x) s[k] = 0u;
    __syncthreads();
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<long long>(gridDim.x) * blockDim.x)
        atomicAdd(&s[order_bucket(nacc, nrej, i)], 1u);
    __syncthreads();
    for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x)
        if (s[k] != 0u) atomicAdd(&counts[k], s[k]);
}

// counts -> exclusive offsets, one block of kOrderBuckets threads
__global__ void order_scan(unsigned* counts)
{
    __shared__ unsigned s[kOrderBuckets];
    const int t = threadIdx.x;
    const unsigned own = counts[t];
    s[t] = own;
    __syncthreads();
    for (int off = 1; off < kOrderBuckets; off <<= 1) {
        const unsigned v = t >= off ? s[t - off] : 0u;
        __syncthreads();
        s[t] += v;
        __syncthreads();
    }
    counts[t] = s[t] - own;
}

__global__ void order_scatter(const int32_t* nacc, const int32_t* nrej, long long n, unsigned* offsets,
                              int32_t* order)
{
    __shared__ unsigned s_count[kOrderBuckets];
    __shared__ unsigned s_base[kOrderBuckets];
    for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x) s_count[k] = 0u;
    __syncthreads();
    const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
    int b = 0;
    unsigned rank = 0u;
    if (i < n) {
        b = order_bucket(nacc, nrej, i);
        rank = atomicAdd(&s_count[b], 1u);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kOrderBuckets; k += blockDim.x)
        if (s_count[k] != 0u) s_base[k] = atomicAdd(&offsets[k], s_count[k]);
    __syncthreads();
    if (i < n) order[s_base[b] + rank] = static_cast<int32_t>(i);
}

}  // namespace

// Writes the longest-first order of instances 0 .. n-1 into `order` from the
// last launch's per-instance accepted and rejected steps; `scratch` holds
// kOrderBuckets unsigned counters. Enqueued on `stream`; returns a CUDA error
// code.
int mpgos_internal_order_instances(cudaStream_t stream, const int32_t* nacc, const int32_t* nrej, long long n,
                                   unsigned* scratch, int32_t* order, int sm_count)
{
    if (n <= 0) return 0;
    cudaError_t e = cudaMemsetAsync(scratch, 0, kOrderBuckets * sizeof(unsigned), stream);
    if (e != cudaSuccess) return static_cast<int>(e);
    const long long blocks = (n + kOrderBlock - 1) / kOrderBlock;
    const int count_grid = static_cast<int>(blocks < 4LL * sm_count ? blocks : 4LL * sm_count);
    order_count<<<count_grid, kOrderBlock, 0, stream>>>(nacc, nrej, n, scratch);
    order_scan<<<1, kOrderBuckets, 0, stream>>>(scratch);
    order_scatter<<<static_cast<unsigned>(blocks), kOrderBlock, 0, stream>>>(nacc, nrej, n, scratch, order);
    return static_cast<int>(cudaGetLastError());
}

// Size of the scratch the function above needs, in unsigned counters.
int mpgos_internal_order_scratch_counters() { return kOrderBuckets; }
