// sm_103a build of the reference's own per-thread solver kernel, one template
// instantiation per cubin.
//
// TEST INFRASTRUCTURE ONLY. oracle/build_oracle.py compiles this file with
// nvcc -cubin against the reference's unmodified
// SourceCodes/SingleSystem_PerThread_Solver.cuh where it lies in the reference
// checkout, into oracle/_ref/ref_gpu_<system>_<alg>_nt<NT>_ndo<NDO>[_rr64].cubin
// (git-ignored; device code only, so it runs on any GB300 host). oracle/ref_gpu.py
// loads it with the CUDA driver API and launches it on the device buffers of
// a GB300 solver object, to check the GB300 kernels against the reference
// kernel bit for bit and to time the reference kernel on the same GPU.
//
// Compile: -DMPGOS_SYSTEM_HEADER="<hooks>.cuh" -DREF_NT=<NT> -DREF_ALG=<RK4|RKCK45>
//          -DREF_NDO=<NDO> -I<reference>/SourceCodes
#include "ref_types.hpp"

#include MPGOS_SYSTEM_HEADER

#include "SingleSystem_PerThread_Solver.cuh"

template __global__ void SingleSystem_PerThread<REF_NT, MPGOS_SYS_SD, MPGOS_SYS_NCP, MPGOS_SYS_NSP, MPGOS_SYS_NISP,
                                                MPGOS_SYS_NE, MPGOS_SYS_NA, MPGOS_SYS_NIA, REF_NDO, REF_ALG, double>(
    Struct_ThreadConfiguration, Struct_GlobalVariables<double>, Struct_SharedMemoryUsage, Struct_SolverOptions<double>);
