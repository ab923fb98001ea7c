// Grid kernels of the chemistry operator instantiated for mechanism cracmm2
// (device code generated from CCTM/src/MECHS/cracmm2 by cmaq_gb300.mechgen).
#include "gen/cracmm2_mech.cuh"
#include "mech_ops.cuh"

DEFINE_MECH_OPS(mech_cracmm2, mech_ops_cracmm2)
