// System plugin libmpgos_duffing_param.so: the hooks of duffing_param.cuh compiled into the
// per-thread solver kernels.
#include "duffing_param.cuh"
#include "plugin_export.cuh"
