// System plugin libmpgos_duffing_param_sens.so: the forward-sensitivity system
// of duffing_param.cuh compiled into the per-thread solver kernels.
#include "duffing_param_sens.cuh"
#include "plugin_export.cuh"
