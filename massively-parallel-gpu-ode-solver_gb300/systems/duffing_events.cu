// System plugin libmpgos_duffing_events.so: the hooks of duffing_events.cuh compiled into the
// per-thread solver kernels.
#include "duffing_events.cuh"
#include "plugin_export.cuh"
