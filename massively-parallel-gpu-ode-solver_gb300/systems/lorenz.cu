// System plugin libmpgos_lorenz.so: the Lorenz hooks compiled into the
// per-thread solver kernels (double and float tables).
#include "lorenz.cuh"
#define MPGOS_PLUGIN_ADJOINT 1
#define MPGOS_PLUGIN_FLOAT 1
#include "plugin_export.cuh"
