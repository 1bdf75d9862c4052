// Turns one coupled-system hook file into a plugin: include it after the hook
// file (which defines MPGOS_SYS_UPS/UD/NC/NUP/NSP/NGP/NIGP/NUA/NIUA/NSA/NISA/NE)
// and after defining MPGOS_SYS_NAME, MPGOS_SYS_CBW and MPGOS_SYS_CCI (coupling
// storage), to export mpgos_cb_system_kernels() of mpgos.h. Instantiated:
// RKCK45 and RK4 in double (with DF_STAGE variants and the discrete adjoint
// with respect to the system parameters, unless MPGOS_PLUGIN_NO_ADJOINT is
// defined: the reverse kernels of large systems dominate the compile time).
#pragma once

#include "coupled_kernel.cuh"
#ifndef MPGOS_PLUGIN_NO_ADJOINT
#include "coupled_adjoint.cuh"
#endif

namespace mpgos_cb_plugin {
using SysShape = mpgos::cb::Shape<MPGOS_SYS_UPS, MPGOS_SYS_UD, MPGOS_SYS_NC, MPGOS_SYS_CBW, MPGOS_SYS_CCI, MPGOS_SYS_NUP,
                                  MPGOS_SYS_NSP, MPGOS_SYS_NGP, MPGOS_SYS_NIGP, MPGOS_SYS_NUA, MPGOS_SYS_NIUA,
                                  MPGOS_SYS_NSA, MPGOS_SYS_NISA, MPGOS_SYS_NE>;
}

extern "C" __attribute__((visibility("default"))) const mpgos_cb_kernels* mpgos_cb_system_kernels(
    int32_t algorithm, int32_t precision_bytes)
{
    using namespace mpgos::cb;
    using S = mpgos_cb_plugin::SysShape;
    if (precision_bytes == 8) {
#ifdef MPGOS_PLUGIN_NO_ADJOINT
        if (algorithm == MPGOS_RKCK45) return KernelTable<S, MPGOS_RKCK45, double>::get(MPGOS_SYS_NAME);
        if (algorithm == MPGOS_RK4) return KernelTable<S, MPGOS_RK4, double>::get(MPGOS_SYS_NAME);
#else
        if (algorithm == MPGOS_RKCK45) {
            using A = CoupledAdjointTable<S, MPGOS_RKCK45>;
            return KernelTable<S, MPGOS_RKCK45, double>::get(MPGOS_SYS_NAME, &A::launch_record, &A::launch_adjoint,
                                                             &A::smem, &A::occupancy);
        }
        if (algorithm == MPGOS_RK4) {
            using A = CoupledAdjointTable<S, MPGOS_RK4>;
            return KernelTable<S, MPGOS_RK4, double>::get(MPGOS_SYS_NAME, &A::launch_record, &A::launch_adjoint,
                                                          &A::smem, &A::occupancy);
        }
#endif
    }
    return nullptr;
}
