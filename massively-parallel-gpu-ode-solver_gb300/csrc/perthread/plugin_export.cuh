// Turns one hook file into a system plugin: include it after the hook file
// (which defines MPGOS_SYS_NAME and MPGOS_SYS_SD/NCP/NSP/NISP/NE/NA/NIA) to
// export mpgos_pt_system_kernels(), the entry point of libmpgos_<system>.so
// declared in mpgos.h.
//
// Instantiated tables: RKCK45 and RK4 in double, plus float when
// MPGOS_PLUGIN_FLOAT is defined (the reference's Precision=float build), plus
// the discrete-adjoint kernels when MPGOS_PLUGIN_ADJOINT is defined. The
// user's own translation units get the same tables through the C++ drop-in
// header instead.
//
// Parallel build (MPGOS_PLUGIN_PARTS): the same source is compiled once as the
// main unit (the tables, the FP64 and float kernels, the adjoint) and once per
// double-float kernel set with MPGOS_PART_ARITH (16 = DF_STAGE, 128 = SPLIT)
// and MPGOS_PART_ALG (0 = RK4, 1 = RKCK45) defined; each part unit defines
// only its set's getter, and the objects are linked into one library.
#pragma once

#include "kernel.cuh"
#if defined(MPGOS_PLUGIN_ADJOINT) && !defined(MPGOS_PART_ARITH)
#include "adjoint.cuh"
#endif

namespace mpgos_plugin {
using SysShape = mpgos::pt::Shape<MPGOS_SYS_SD, MPGOS_SYS_NCP, MPGOS_SYS_NSP, MPGOS_SYS_NISP, MPGOS_SYS_NE,
                                  MPGOS_SYS_NA, MPGOS_SYS_NIA>;

#define MPGOS_PART_CAT(a, b, c, d) a##b##c##d
#define MPGOS_PART_NAME(arith, alg) MPGOS_PART_CAT(part_kernel_, arith, _, alg)

#ifdef MPGOS_PLUGIN_PARTS
void* MPGOS_PART_NAME(16, 0)(int mode);
void* MPGOS_PART_NAME(16, 1)(int mode);
void* MPGOS_PART_NAME(128, 0)(int mode);
void* MPGOS_PART_NAME(128, 1)(int mode);
#endif
}  // namespace mpgos_plugin

#ifdef MPGOS_PART_ARITH

// ---- one double-float kernel set (a part unit) --------------------------------
void* mpgos_plugin::MPGOS_PART_NAME(MPGOS_PART_ARITH, MPGOS_PART_ALG)(int mode)
{
    return mpgos::pt::DfKernelSet<SysShape, MPGOS_PART_ALG, MPGOS_PART_ARITH>::get(mode);
}

#else

#ifdef MPGOS_PLUGIN_PARTS
void* mpgos::pt::plugin_part_kernel(int arith, int alg, int mode)
{
    using namespace mpgos_plugin;
    if (arith == MPGOS_MODE_DF_STAGE) return alg == MPGOS_RK4 ? MPGOS_PART_NAME(16, 0)(mode) : MPGOS_PART_NAME(16, 1)(mode);
    if (arith == MPGOS_MODE_SPLIT) return alg == MPGOS_RK4 ? MPGOS_PART_NAME(128, 0)(mode) : MPGOS_PART_NAME(128, 1)(mode);
    return nullptr;
}
#endif

extern "C" __attribute__((visibility("default"))) const mpgos_pt_kernels* mpgos_pt_system_kernels(
    int32_t algorithm, int32_t precision_bytes)
{
    using namespace mpgos::pt;
    using S = mpgos_plugin::SysShape;
    if (precision_bytes == 8) {
#ifdef MPGOS_PLUGIN_ADJOINT
        if (algorithm == MPGOS_RKCK45)
            return KernelTable<S, MPGOS_RKCK45, double>::get(MPGOS_SYS_NAME, &AdjointTable<S, MPGOS_RKCK45>::launch_record,
                                                             &AdjointTable<S, MPGOS_RKCK45>::launch_adjoint);
        if (algorithm == MPGOS_RK4)
            return KernelTable<S, MPGOS_RK4, double>::get(MPGOS_SYS_NAME, &AdjointTable<S, MPGOS_RK4>::launch_record,
                                                          &AdjointTable<S, MPGOS_RK4>::launch_adjoint);
#else
        if (algorithm == MPGOS_RKCK45) return KernelTable<S, MPGOS_RKCK45, double>::get(MPGOS_SYS_NAME);
        if (algorithm == MPGOS_RK4) return KernelTable<S, MPGOS_RK4, double>::get(MPGOS_SYS_NAME);
#endif
    }
#ifdef MPGOS_PLUGIN_FLOAT
    if (precision_bytes == 4) {
        if (algorithm == MPGOS_RKCK45) return KernelTable<S, MPGOS_RKCK45, float>::get(MPGOS_SYS_NAME);
        if (algorithm == MPGOS_RK4) return KernelTable<S, MPGOS_RK4, float>::get(MPGOS_SYS_NAME);
    }
#endif
    return nullptr;
}

#endif
