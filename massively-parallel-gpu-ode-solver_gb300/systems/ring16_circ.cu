// Coupled-system plugin libmpgos_ring16_circ.so: rings of 16 forced Duffing units
// (ring_duffing.cuh) with full circular coupling
// (CouplingBandwidthRadius 0, CouplingCircularity 1).
#define MPGOS_SYS_NAME "ring16_circ"
#define MPGOS_SYS_UPS  16
#define MPGOS_SYS_CBW  0
#define MPGOS_SYS_CCI  1
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
