// System plugin libmpgos_bouncing_ball.so: the hooks of bouncing_ball.cuh compiled into the
// per-thread solver kernels.
#include "bouncing_ball.cuh"
#include "plugin_export.cuh"
