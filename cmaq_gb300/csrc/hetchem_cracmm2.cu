// HETCHEM_RATES for cracmm2 (its 9 KHETERO labels, CRACMM's IEPOX pair table; tables
// gen/cracmm2_hetchem.cuh).
#define HET_NS het_cracmm2
#define HET_GEN "gen/cracmm2_hetchem.cuh"
#include "../../include/cmaqchem.h"
#include "hetchem_mech.cuh"

static_assert(het_cracmm2::NAE == CMAQCHEM_HET_CRACMM2_NAE && het_cracmm2::NHET == CMAQCHEM_HET_CRACMM2_NHETERO &&
                  het_cracmm2::AE_FIRST == CMAQCHEM_HET_CRACMM2_AE_FIRST,
              "HETCHEM layout");

HetMech hetchem_mech_cracmm2() { return het_cracmm2::entry("cracmm2"); }
