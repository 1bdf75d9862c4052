// System plugin libmpgos_duffing.so: the hooks of duffing.cuh compiled into the
// per-thread solver kernels.
#include "duffing.cuh"
#include "plugin_export.cuh"
