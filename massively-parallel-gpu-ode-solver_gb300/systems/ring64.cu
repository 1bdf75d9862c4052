// Coupled-system plugin libmpgos_ring64.so: rings of 64 forced Duffing units
// (ring_duffing.cuh) with full 64x64 coupling matrix
// (CouplingBandwidthRadius 0, CouplingCircularity 0).
#define MPGOS_SYS_NAME "ring64"
#define MPGOS_SYS_UPS  64
#define MPGOS_SYS_CBW  0
#define MPGOS_SYS_CCI  0
// Every unit of a system evaluates cos(T) at the same stage time, so the
// double-float cosine's table lookup saves no divergence here; the series
// path is ~3 % faster on these kernels (GB300, 16384 rings of 64).
#define MPGOS_DF_TRIG_SERIES
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
