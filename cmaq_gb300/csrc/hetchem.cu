// C ABI of the heterogeneous rate constants (include/cmaqchem.h: cmaqchem_hetchem_*):
// HETCHEM_RATES (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:282-1535) for every cell of a
// grid, one cell per thread (hetchem.cuh).
//
// The reference calls HETCHEM_RATES from the chemistry driver once per synchronisation
// step before CHEM (rbdriver.F:409); KHETERO then feeds CALC_RCONST.  Here the kernel
// reads the aerosol block of the caller's CGRID (CONC(:,:,:,AE_STRT:), REAL) and the met
// fields in place and writes KHETERO(NHETERO, NCOLS, NROWS, NLAYS) (REAL(8)), the layout
// the CHEM entries take.  Each thread holds its cell's aerosol state (54 species x 3
// modes) in local memory; the work per cell is a few thousand float and double
// operations, so the kernel is bound by instruction issue, not by its 0.5 KB per cell
// of DRAM traffic.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/cmaqchem.h"
#include "hetchem.cuh"

__attribute__((visibility("hidden"))) void cmaqchem_set_error(const std::string& msg);

static_assert(het::NAE == CMAQCHEM_HET_CB6R5_NAE && het::NHET == CMAQCHEM_HET_CB6R5_NHETERO, "HETCHEM layout");
static_assert(het::AE_FIRST == CMAQCHEM_HET_CB6R5_AE_FIRST, "HETCHEM layout");

namespace het {
__constant__ HetTables c_het = HET_TABLES_INIT;
}

namespace {

constexpr int HET_THREADS = 128;

__global__ void __launch_bounds__(HET_THREADS) k_hetchem_rates(const float* ae, long long ncell, const float* ta,
                                                               const float* pres, const float* qv, const float* dens,
                                                               double* khetero)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
        double k[het::NHET];
        het::het_cell(het::c_het, ae + c, ncell, ta[c], pres[c], qv[c], dens[c], k);
        for (int j = 0; j < het::NHET; ++j) khetero[c * het::NHET + j] = k[j];
    }
}

int fail(const std::string& msg)
{
    cmaqchem_set_error(msg);
    return -1;
}

int check_mechanism(const char* mechanism)
{
    if (!mechanism || std::strcmp(mechanism, "cb6r5_ae7_aq") != 0)
        return fail(std::string("HETCHEM_RATES: mechanism '") + (mechanism ? mechanism : "(null)") +
                    "' is not built (cb6r5_ae7_aq only)");
    return 0;
}

}  // namespace

extern "C" int cmaqchem_hetchem_layout(const char* mechanism, int* nae, int* ae_first, int* nhetero)
{
    if (check_mechanism(mechanism) != 0) return -1;
    if (nae) *nae = het::NAE;
    if (ae_first) *ae_first = het::AE_FIRST;
    if (nhetero) *nhetero = het::NHET;
    return 0;
}

extern "C" int cmaqchem_hetchem_rates_device(const char* mechanism, long long ncell, const float* ae,
                                             const float* ta, const float* pres, const float* qv, const float* dens,
                                             double* khetero, void* stream)
{
    if (check_mechanism(mechanism) != 0) return -1;
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!ae || !ta || !pres || !qv || !dens || !khetero) return fail("null array argument");
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (ncell + HET_THREADS - 1) / HET_THREADS;
    const long long cap = (long long)(nsm > 0 ? nsm : 1) * 16;   // 16 blocks of 128 per SM, grid-stride beyond
    const unsigned blocks = (unsigned)(want < cap ? want : cap);
    cudaStream_t s = (cudaStream_t)stream;
    k_hetchem_rates<<<blocks, HET_THREADS, 0, s>>>(ae, ncell, ta, pres, qv, dens, khetero);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(std::string("k_hetchem_rates: ") + cudaGetErrorString(e));
    return 0;
}

// Host-array form: the same layouts in host memory, device buffers for the call,
// synchronous copies.
extern "C" int cmaqchem_hetchem_rates(const char* mechanism, long long ncell, const float* ae, const float* ta,
                                      const float* pres, const float* qv, const float* dens, double* khetero,
                                      int device)
{
    if (check_mechanism(mechanism) != 0) return -1;
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!ae || !ta || !pres || !qv || !dens || !khetero) return fail("null array argument");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    const size_t n = (size_t)ncell;
    const size_t bytes[6] = {sizeof(float) * het::NAE * n, sizeof(float) * n, sizeof(float) * n, sizeof(float) * n,
                             sizeof(float) * n, sizeof(double) * het::NHET * n};
    const void* src[5] = {ae, ta, pres, qv, dens};
    void* d[6] = {};
    int rc = 0;
    for (int i = 0; i < 6 && rc == 0; ++i)
        if ((e = cudaMalloc(&d[i], bytes[i])) != cudaSuccess) rc = fail(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    for (int i = 0; i < 5 && rc == 0; ++i)
        if ((e = cudaMemcpy(d[i], src[i], bytes[i], cudaMemcpyHostToDevice)) != cudaSuccess)
            rc = fail(std::string("copy to the device: ") + cudaGetErrorString(e));
    if (rc == 0)
        rc = cmaqchem_hetchem_rates_device(mechanism, ncell, (const float*)d[0], (const float*)d[1],
                                           (const float*)d[2], (const float*)d[3], (const float*)d[4], (double*)d[5],
                                           nullptr);
    if (rc == 0 && (e = cudaMemcpy(khetero, d[5], bytes[5], cudaMemcpyDeviceToHost)) != cudaSuccess)
        rc = fail(std::string("copy to the host: ") + cudaGetErrorString(e));
    for (void* q : d)
        if (q) cudaFree(q);
    return rc;
}
