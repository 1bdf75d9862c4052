// System plugin libmpgos_duffing_param.so: the hooks of duffing_param.cuh compiled into the
// per-thread solver kernels.
#include "duffing_param.cuh"
#define MPGOS_PLUGIN_ADJOINT 1
#include "plugin_export.cuh"
