// System plugin libmpgos_keller_miksis.so: the hooks of keller_miksis.cuh compiled into the
// per-thread solver kernels.
//
// The SPLIT kernels run the six Cash-Karp stages as one loop: this right-hand
// side (double-float pow, sincospi, sin, cos, two divisions) inlined six times
// overflows the instruction cache. On the 512 x 512 grid over 16 periods
// (persistent, work order): inlined 2360 -> 1210 ms, out of line 1152 ->
// 1128 ms on GB300, results bit-identical. (Lorenz, whose right-hand side is
// small, runs 19 % slower with the loop and keeps the straight-line step.)
#define MPGOS_SPLIT_STAGE_LOOP
#include "keller_miksis.cuh"
#include "plugin_export.cuh"
