// Coupled-system plugin libmpgos_ring16_full.so: rings of 16 forced Duffing units
// (ring_duffing.cuh) with full 16x16 coupling matrix
// (CouplingBandwidthRadius 0, CouplingCircularity 0).
#define MPGOS_SYS_NAME "ring16_full"
#define MPGOS_SYS_UPS  16
#define MPGOS_SYS_CBW  0
#define MPGOS_SYS_CCI  0
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
