// System plugin libmpgos_lorenz.so: the Lorenz hooks compiled into the
// per-thread solver kernels (double and float tables).
//
// SPLIT kernels capped for three resident 256-thread blocks (85 registers,
// a few bytes of spills): 24 instead of 16 resident warps per SM hide more of
// the FP64 latency; 2^20 instances, block 64, persistent: 80.2 -> 76.9 ms on
// GB300 (a two-block cap, 128 registers, ran 82.2 ms; a four-block cap, 64
// registers and ~300 bytes of spills, 80.0 ms against 78.3 ms).
#define MPGOS_SPLIT_MIN_BLOCKS 3
#include "lorenz.cuh"
#define MPGOS_PLUGIN_ADJOINT 1
#define MPGOS_PLUGIN_FLOAT 1
#include "plugin_export.cuh"
