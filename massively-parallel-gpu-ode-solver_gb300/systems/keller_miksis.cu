// System plugin libmpgos_keller_miksis.so: the hooks of keller_miksis.cuh compiled into the
// per-thread solver kernels.
#include "keller_miksis.cuh"
#include "plugin_export.cuh"
