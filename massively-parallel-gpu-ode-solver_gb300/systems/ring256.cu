// Coupled-system plugin libmpgos_ring256.so: rings of 256 forced Duffing units
// (ring_duffing.cuh) with full 256x256 coupling matrix: eight units per lane
// of the warp that integrates a system (the reference launches such systems
// through its MultipleBlockLaunches kernels, UPS > threads per block).
#define MPGOS_SYS_NAME "ring256"
#define MPGOS_SYS_UPS  256
#define MPGOS_SYS_CBW  0
#define MPGOS_SYS_CCI  0
#define MPGOS_PLUGIN_NO_ADJOINT 1
// Every unit of a system evaluates cos(T) at the same stage time, so the
// double-float cosine's table lookup saves no divergence here; the series
// path is ~3 % faster on these kernels (GB300, 16384 rings of 64).
#define MPGOS_DF_TRIG_SERIES
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
