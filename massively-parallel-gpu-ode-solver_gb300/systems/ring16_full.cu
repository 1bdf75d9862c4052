// Coupled-system plugin libmpgos_ring16_full.so: rings of 16 forced Duffing units
// (ring_duffing.cuh) with full 16x16 coupling matrix
// (CouplingBandwidthRadius 0, CouplingCircularity 0).
#define MPGOS_SYS_NAME "ring16_full"
#define MPGOS_SYS_UPS  16
#define MPGOS_SYS_CBW  0
#define MPGOS_SYS_CCI  0
// The forcing cos(T) takes T in [TD0, TD1] (Initialization restarts every
// launch at TD0), below 2^14 for up to 2607 forcing periods from 0: the
// branch-free double-float cosine (MPGOS_DF_TRIG_BOUNDED; beyond the bound
// the double-float steps report non-finite) ran 16384 rings of 64 over four
// periods in 870 ms SPLIT / 819 ms DF_STAGE on GB300, against 974 / 852 ms
// with the series path and 1019 / 901 ms with the table path behind its
// range branch.
#define MPGOS_DF_TRIG_BOUNDED
#include "ring_duffing.cuh"
#include "../csrc/coupled/coupled_plugin_export.cuh"
