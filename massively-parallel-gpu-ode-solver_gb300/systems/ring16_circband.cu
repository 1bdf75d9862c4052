// Coupled-system plugin libmpgos_ring16_circband.so: rings of 16 forced Duffing units
// (ring_duffing.cuh) with circular banded coupling, bandwidth radius 1
// (CouplingBandwidthRadius 1, CouplingCircularity 1).
#define MPGOS_SYS_NAME "ring16_circband"
#define MPGOS_SYS_UPS  16
#define MPGOS_SYS_CBW  1
#define MPGOS_SYS_CCI  1
// Every unit of a system evaluates cos(T) at the same stage time, so the
// double-float cosine's table lookup saves no divergence here; the series
// path is ~3 % faster on these kernels (GB300, 16384 rings of 64).
#define MPGOS_DF_TRIG_SERIES
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
