// System plugin libmpgos_duffing.so: the hooks of duffing.cuh compiled into the
// per-thread solver kernels.
//
// The fixed-step ensemble this system serves (8192 instances) leaves each busy
// scheduler one warp, so occupancy does not matter and the step time is its
// dependent-instruction chain: letting ptxas use registers for one resident
// block (80 instead of 72 for SPLIT RK4) shortens it (180 -> 166 ms for 256
// periods on GB300; double-float 153 -> 151 ms).
#define MPGOS_SPLIT_MIN_BLOCKS 1
#define MPGOS_DF_MIN_BLOCKS 1
#include "duffing.cuh"
#include "plugin_export.cuh"
