// System plugin libmpgos_duffing.so: the hooks of duffing.cuh compiled into the
// per-thread solver kernels.
//
// The fixed-step ensemble this system serves (8192 instances) leaves each busy
// scheduler one warp, so occupancy does not matter and the step time is its
// dependent-instruction chain: letting ptxas use registers for one resident
// block (80 instead of 72 for SPLIT RK4) shortens it (180 -> 166 ms for 256
// periods on GB300; double-float 153 -> 151 ms).
//
// Every launch restarts the time at TD0 (Initialization), so the argument of
// cos stays in [TD0, TD1], one forcing period [0, 2 pi] in this system's
// ensembles: far below the 2^14 bound of the branch-free double-float cosine
// (MPGOS_DF_TRIG_BOUNDED). Without the branch to its wide-range path the
// compiler interleaves the stages' cos(t) with the state arithmetic (one
// period, 8192 instances: SPLIT 0.65 -> 0.50 ms, DF_STAGE 0.60 -> 0.41 ms on
// GB300, results bit-identical). A TD1 at or beyond 2^14 makes the double-
// float steps there non-finite (reported as MPGOS_INSTANCE_NONFINITE); the
// FP64 modes have no bound.
#define MPGOS_SPLIT_MIN_BLOCKS 1
#define MPGOS_DF_MIN_BLOCKS 1
#define MPGOS_DF_TRIG_BOUNDED
#include "duffing.cuh"
#include "plugin_export.cuh"
