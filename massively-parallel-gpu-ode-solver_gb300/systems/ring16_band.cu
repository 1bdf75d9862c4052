// Coupled-system plugin libmpgos_ring16_band.so: rings of 16 forced Duffing units
// (ring_duffing.cuh) with banded coupling, bandwidth radius 1
// (CouplingBandwidthRadius 1, CouplingCircularity 0).
#define MPGOS_SYS_NAME "ring16_band"
#define MPGOS_SYS_UPS  16
#define MPGOS_SYS_CBW  1
#define MPGOS_SYS_CCI  0
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
