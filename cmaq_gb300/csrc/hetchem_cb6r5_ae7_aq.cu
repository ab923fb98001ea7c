// HETCHEM_RATES for cb6r5_ae7_aq (its 17 KHETERO labels; tables gen/cb6r5_ae7_aq_hetchem.cuh).
#include "../../include/cmaqchem.h"
#include "hetchem_mech.cuh"

static_assert(het::NAE == CMAQCHEM_HET_CB6R5_NAE && het::NHET == CMAQCHEM_HET_CB6R5_NHETERO &&
                  het::AE_FIRST == CMAQCHEM_HET_CB6R5_AE_FIRST,
              "HETCHEM layout");

HetMech hetchem_mech_cb6r5_ae7_aq() { return het::entry("cb6r5_ae7_aq"); }
