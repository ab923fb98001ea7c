// One mechanism's HETCHEM_RATES kernel: hetchem.cuh for the mechanism that HET_NS / HET_GEN
// name (a translation unit per mechanism, hetchem_<mech>.cu), its tables in constant
// memory, and its entry in the table that the C ABI (hetchem.cu) looks mechanisms up in.
#pragma once

#include <cuda_runtime.h>

#include "hetchem.cuh"
#include "hetchem_table.h"

namespace HET_NS {

__constant__ HetTables c_het = HET_TABLES_INIT;

constexpr int HET_THREADS = 128;

// One cell per thread, grid-stride: KHETERO(:, c) from row r of the aerosol block at
// ae[r * ncell + c] and the cell's met fields
__global__ void __launch_bounds__(HET_THREADS) k_hetchem_rates(const float* ae, long long ncell, const float* ta,
                                                               const float* pres, const float* qv, const float* dens,
                                                               double* khetero)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
        double k[NHET];
        het_cell(c_het, ae + c, ncell, ta[c], pres[c], qv[c], dens[c], k);
        for (int j = 0; j < NHET; ++j) khetero[c * NHET + j] = k[j];
    }
}

// ncell >= 1; 16 blocks of 128 threads per SM at most, grid-stride beyond
inline cudaError_t launch(long long ncell, const float* ae, const float* ta, const float* pres, const float* qv,
                          const float* dens, double* khetero, cudaStream_t stream)
{
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (ncell + HET_THREADS - 1) / HET_THREADS;
    const long long cap = (long long)(nsm > 0 ? nsm : 1) * 16;
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    k_hetchem_rates<<<blocks, HET_THREADS, 0, stream>>>(ae, ncell, ta, pres, qv, dens, khetero);
    return cudaGetLastError();
}

inline HetMech entry(const char* name) { return HetMech{name, NAE, AE_FIRST, NHET, &launch}; }

}  // namespace HET_NS
