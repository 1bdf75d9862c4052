// System plugin libmpgos_duffing_param.so: the hooks of duffing_param.cuh compiled into the
// per-thread solver kernels.
//
// cos(T) with T in [TD0, TD1] (Initialization restarts every launch at TD0):
// below 2^14 for up to 2607 forcing periods from 0, so the branch-free
// double-float cosine applies (MPGOS_DF_TRIG_BOUNDED; beyond the bound the
// double-float steps report non-finite). 2^18 instances, 64 periods, GB300:
// SPLIT forward 164 -> 156 ms, DF_STAGE 119 -> 108 ms, double-float reverse
// 443 -> 434 ms, gradients unchanged.
#define MPGOS_DF_TRIG_BOUNDED
#include "duffing_param.cuh"
#define MPGOS_PLUGIN_ADJOINT 1
#include "plugin_export.cuh"
