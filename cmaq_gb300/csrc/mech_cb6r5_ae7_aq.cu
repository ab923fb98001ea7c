// Grid kernels of the chemistry operator instantiated for mechanism cb6r5_ae7_aq
// (device code generated from CCTM/src/MECHS/cb6r5_ae7_aq by cmaq_gb300.mechgen).
#include "gen/cb6r5_ae7_aq_mech.cuh"
#include "mech_ops.cuh"

DEFINE_MECH_OPS(mech_cb6r5_ae7_aq, mech_ops_cb6r5_ae7_aq)
