// C ABI of the heterogeneous rate constants (include/cmaqchem.h: cmaqchem_hetchem_*):
// HETCHEM_RATES (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:282-1535) for every cell of a
// grid, one cell per thread (hetchem.cuh), for the mechanisms of hetchem_table.h.
//
// The reference calls HETCHEM_RATES from the chemistry driver once per synchronisation
// step before CHEM (rbdriver.F:409); KHETERO then feeds CALC_RCONST.  Here the kernel
// reads the aerosol block of the caller's CGRID (CONC(:,:,:,AE_STRT:), REAL) and the met
// fields in place and writes KHETERO(NHETERO, NCOLS, NROWS, NLAYS) (REAL(8)), the layout
// the CHEM entries take.  Each thread holds its cell's aerosol state (about 54 species x 3
// modes) in local memory; the work per cell is a few thousand float and double
// operations, so the kernel is bound by instruction issue, not by its 0.5 KB per cell
// of DRAM traffic.
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "../../include/cmaqchem.h"
#include "hetchem_table.h"

__attribute__((visibility("hidden"))) void cmaqchem_set_error(const std::string& msg);

namespace {

int fail(const std::string& msg)
{
    cmaqchem_set_error(msg);
    return -1;
}

// the mechanism's entry, or null with the error set
const HetMech* find_mechanism(const char* mechanism)
{
    static const HetMech table[] = {hetchem_mech_cb6r5_ae7_aq(), hetchem_mech_cracmm2()};
    if (mechanism)
        for (const HetMech& m : table)
            if (std::strcmp(mechanism, m.name) == 0) return &m;
    fail(std::string("HETCHEM_RATES: mechanism '") + (mechanism ? mechanism : "(null)") +
         "' is not built (cb6r5_ae7_aq, cracmm2)");
    return nullptr;
}

}  // namespace

extern "C" int cmaqchem_hetchem_layout(const char* mechanism, int* nae, int* ae_first, int* nhetero)
{
    const HetMech* m = find_mechanism(mechanism);
    if (!m) return -1;
    if (nae) *nae = m->nae;
    if (ae_first) *ae_first = m->ae_first;
    if (nhetero) *nhetero = m->nhet;
    return 0;
}

extern "C" int cmaqchem_hetchem_rates_device(const char* mechanism, long long ncell, const float* ae,
                                             const float* ta, const float* pres, const float* qv, const float* dens,
                                             double* khetero, void* stream)
{
    const HetMech* m = find_mechanism(mechanism);
    if (!m) return -1;
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!ae || !ta || !pres || !qv || !dens || !khetero) return fail("null array argument");
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = m->launch(ncell, ae, ta, pres, qv, dens, khetero, s);
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
    const HetMech* m = find_mechanism(mechanism);
    if (!m) return -1;
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!ae || !ta || !pres || !qv || !dens || !khetero) return fail("null array argument");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    const size_t n = (size_t)ncell;
    const size_t bytes[6] = {sizeof(float) * m->nae * n, sizeof(float) * n, sizeof(float) * n, sizeof(float) * n,
                             sizeof(float) * n, sizeof(double) * m->nhet * n};
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
