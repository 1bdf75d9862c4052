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
#pragma once

#include "kernel.cuh"
#ifdef MPGOS_PLUGIN_ADJOINT
#include "adjoint.cuh"
#endif

namespace mpgos_plugin {
using SysShape = mpgos::pt::Shape<MPGOS_SYS_SD, MPGOS_SYS_NCP, MPGOS_SYS_NSP, MPGOS_SYS_NISP, MPGOS_SYS_NE,
                                  MPGOS_SYS_NA, MPGOS_SYS_NIA>;
}

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
