// The mechanisms the HETCHEM_RATES entries of the C ABI know (hetchem.cu): each one's
// aerosol-block layout and kernel launcher, defined by its translation unit
// hetchem_<mech>.cu.
#pragma once

#include <cuda_runtime.h>

struct HetMech {
    const char* name;   // the mechanism's name in the C ABI
    int nae;            // rows of its CGRID aerosol block
    int ae_first;       // the block's first row in its CGRID (0-based)
    int nhet;           // KHETERO rows
    cudaError_t (*launch)(long long ncell, const float* ae, const float* ta, const float* pres, const float* qv,
                          const float* dens, double* khetero, cudaStream_t stream);
};

__attribute__((visibility("hidden"))) HetMech hetchem_mech_cb6r5_ae7_aq();
__attribute__((visibility("hidden"))) HetMech hetchem_mech_cracmm2();
