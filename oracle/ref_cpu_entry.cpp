// CPU build of the reference's own per-thread solver kernel, used to pin the
// oracle.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_oracle.py compiles this file with
// g++ against the reference's unmodified SourceCodes/SingleSystem_PerThread_Solver.cuh
// (and the headers it includes) where they lie in the reference checkout,
// into oracle/_ref/libref_cpu_<system>.so (git-ignored). Nothing from the
// reference is copied into the repository's history; on a machine without the
// checkout the same headers come from the git-ignored baseline/_ref staging
// copy (build_oracle.stage_reference_sources).
//
// The kernel template SingleSystem_PerThread<NT,...> is executed on the CPU
// by calling it once per instance with a one-thread block (blockDim.x = 1,
// threadIdx.x = 0, blockIdx.x = instance): with one thread per block every
// block-shared load loop of the kernel loads all entries itself. Instances
// are spread over host threads with OpenMP (the CPU baseline of the
// benchmark): the CUDA index variables, the kernel's __shared__ arrays and
// the backing store of its dynamic shared memory are thread_local, so every
// host thread runs its own one-thread "blocks". NT is a template argument of
// the reference kernel, so the entry point is compiled for a fixed list of
// ensemble sizes (MPGOS_REF_NT_LIST, plus MPGOS_REF_NT_EXTRA for RKCK45
// without dense output).
//
// Compile: -DMPGOS_SYSTEM_HEADER="<hooks>.cuh" -I<reference>/SourceCodes -fopenmp
//          -fno-extern-tls-init.
#include "host_shim.hpp"

#include <cstdint>

#include <omp.h>

// CUDA spellings the reference kernel uses; a block-shared array becomes a
// per-host-thread static.
#define __global__
#define __shared__ thread_local
struct MpgosHostDim3 {
    unsigned x, y, z;
};
static thread_local MpgosHostDim3 threadIdx{0, 0, 0};
static thread_local MpgosHostDim3 blockIdx{0, 0, 0};
static thread_local MpgosHostDim3 blockDim{1, 1, 1};
static inline int max(int a, int b) { return a > b ? a : b; }
static inline int min(int a, int b) { return a < b ? a : b; }
static inline int __float_as_int(float f) { int i; std::memcpy(&i, &f, 4); return i; }
static inline float __int_as_float(int i) { float f; std::memcpy(&f, &i, 4); return f; }
static inline long long __double_as_longlong(double d) { long long i; std::memcpy(&i, &d, 8); return i; }
static inline double __longlong_as_double(long long i) { double d; std::memcpy(&d, &i, 8); return d; }
static inline int atomicCAS(int* a, int c, int v) { int o = *a; if (o == c) *a = v; return o; }
static inline unsigned long long atomicCAS(unsigned long long* a, unsigned long long c, unsigned long long v)
{
    unsigned long long o = *a;
    if (o == c) *a = v;
    return o;
}
// Backing store of the kernel's `extern __shared__ int DynamicSharedMemory[]`.
thread_local int DynamicSharedMemory[1 << 14];

#include "ref_types.hpp"

#include MPGOS_SYSTEM_HEADER

#include "SingleSystem_PerThread_Solver.cuh"

#ifndef MPGOS_REF_NT_LIST
#define MPGOS_REF_NT_LIST X(64) X(256) X(1024)
#endif
#ifndef MPGOS_REF_NT_EXTRA
#define MPGOS_REF_NT_EXTRA
#endif

namespace {
constexpr int SD = MPGOS_SYS_SD, NCP = MPGOS_SYS_NCP, NSP = MPGOS_SYS_NSP, NISP = MPGOS_SYS_NISP;
constexpr int NE = MPGOS_SYS_NE, NA = MPGOS_SYS_NA, NIA = MPGOS_SYS_NIA;

int g_threads = 1;

template <int NT, int NDO, Algorithms ALG>
void run(long long n_active, const Struct_GlobalVariables<double>& g, const Struct_SolverOptions<double>& o)
{
    Struct_ThreadConfiguration tc{(int)NT, 1, (int)n_active};
    Struct_SharedMemoryUsage sm{1, ALG == RK4 ? 0 : 1};
#pragma omp parallel for schedule(dynamic, 64) num_threads(g_threads)
    for (long long i = 0; i < n_active; i++) {
        blockDim.x  = 1;
        threadIdx.x = 0;
        blockIdx.x  = (unsigned)i;
        SingleSystem_PerThread<NT, SD, NCP, NSP, NISP, NE, NA, NIA, NDO, ALG, double>(tc, g, sm, o);
    }
}
}  // namespace

extern "C" {

// Host threads the next ref_cpu_solve calls use (0: all the machine has);
// returns the count in effect. Results do not depend on it.
int ref_cpu_set_threads(int threads)
{
    g_threads = threads > 0 ? threads : omp_get_num_procs();
    return g_threads;
}

// Returns 0 on success, 2 if (nt, ndo) is not in the compiled list.
// ndo must be 0 or 16 (the NDO template argument of the compiled kernels).
int ref_cpu_solve(int algorithm, long long nt, long long n_active, int ndo, double* td, double* x, double* t,
                  double* cp, double* sp, int* spi, double* acc, int* acci, double* rtol, double* atol, double* etol,
                  int* edir, int* didx, double* dtime, double* dstate, const double* opt6, int dense_freq)
{
    Struct_GlobalVariables<double> g{td, x, t, cp, sp, spi, acc, acci, rtol, atol, etol, edir, didx, dtime, dstate};
    Struct_SolverOptions<double> o{opt6[0], opt6[1], opt6[2], opt6[3], opt6[4], dense_freq, opt6[5]};
#define X(N)                                                                  \
    if (nt == N) {                                                            \
        if (ndo == 0 && algorithm == 0) { run<N, 0, RK4>(n_active, g, o); return 0; }     \
        if (ndo == 0 && algorithm == 1) { run<N, 0, RKCK45>(n_active, g, o); return 0; }  \
        if (ndo == 16 && algorithm == 0) { run<N, 16, RK4>(n_active, g, o); return 0; }   \
        if (ndo == 16 && algorithm == 1) { run<N, 16, RKCK45>(n_active, g, o); return 0; } \
    }
    MPGOS_REF_NT_LIST
#undef X
#define X(N)                                                                  \
    if (nt == N && ndo == 0 && algorithm == 1) { run<N, 0, RKCK45>(n_active, g, o); return 0; }
    MPGOS_REF_NT_EXTRA
#undef X
    return 2;
}

}  // extern "C"
