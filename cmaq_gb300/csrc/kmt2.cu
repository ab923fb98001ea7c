// C ABI of the KMT2 aqueous cloud chemistry kernel (include/cmaqchem.h:
// cmaqchem_kmt2_*): the kinetic core of AQCHEM (CCTM/src/cloud/acm_ae7_kmt2/aqchem_kmt.F90:
// 371-543) for a batch of cloudy cells, one cell per thread.
//
// Each thread is a lane with its own slice of the caller's workspace (element i at
// ws[lane + i * nlanes], so a warp's 32 lanes read consecutive doubles) and integrates
// cells lane, lane + nlanes, ...; inputs and outputs are [element][cell].  The loops of
// the integrator are bounded (200,000 Rodas3 steps per pass, 5 step halvings per
// singular factorisation, 16 passes), so every thread ends.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "../../include/cmaqchem.h"
#include "kmt2.cuh"

__attribute__((visibility("hidden"))) void cmaqchem_set_error(const std::string& msg);

static_assert(kmt2::NVAR == CMAQCHEM_KMT2_NVAR && kmt2::NFIX == CMAQCHEM_KMT2_NFIX, "KMT2 sizes");
static_assert(kmt2::NPARAM == CMAQCHEM_KMT2_NPARAM && kmt2::NSTAT == CMAQCHEM_KMT2_NSTAT, "KMT2 layout");
static_assert(kmt2::KG_NGAS == CMAQCHEM_AQ_NGAS && kmt2::KA_NIDX == CMAQCHEM_AQ_NSURROGATE, "AQCHEM layout");
static_assert(kmt2::KF_N == CMAQCHEM_AQ_NFACTOR && kmt2::KO_N == CMAQCHEM_AQ_NOUT, "AQCHEM layout");

namespace {

constexpr int KMT2_THREADS = 128;
constexpr long long KMT2_LANES_PER_SM = 256;   // two 128-thread blocks per SM

struct Kmt2Args {
    const double* params;
    const double* var_mix;
    double* var_out;
    double* fix_out;
    int* stats;
    double* ws;
    long long ncell;
    long long nlanes;
};

__global__ void __launch_bounds__(KMT2_THREADS) k_kmt2_cells(Kmt2Args a)
{
    const long long lane = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (lane >= a.nlanes) return;
    double* ws = a.ws + lane;
    for (long long c = lane; c < a.ncell; c += a.nlanes)
        kmt2::kq_cell(a.params + c, a.var_mix + c, a.var_out + c, a.fix_out ? a.fix_out + c : nullptr, a.stats + c,
                      a.ncell, ws, a.nlanes);
}

struct AqchemArgs {
    const double* params;
    double* gas;
    double* aer;
    double* gas_wdep;
    double* aer_wdep;
    double* out;
    int* stats;
    double* ws;
    long long ncell;
    long long nlanes;
    int naer;
    int ai[kmt2::KA_NIDX];
    double fac[kmt2::KF_N];
};

__global__ void __launch_bounds__(KMT2_THREADS) k_aqchem_cells(AqchemArgs a)
{
    const long long lane = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (lane >= a.nlanes) return;
    double* ws = a.ws + lane;
    for (long long c = lane; c < a.ncell; c += a.nlanes)
        kmt2::kq_aqchem_cell(a.params + c, a.gas + c, a.aer + c, a.naer, a.ai, a.fac, a.gas_wdep + c, a.aer_wdep + c,
                             a.out + c, a.stats + c, a.ncell, ws, a.nlanes);
}

int fail(const std::string& msg)
{
    cmaqchem_set_error(msg);
    return -1;
}

}  // namespace

extern "C" long long cmaqchem_kmt2_workspace_doubles(long long nlanes)
{
    return nlanes > 0 ? nlanes * (long long)kmt2::WS_ELEMS : 0;
}

extern "C" int cmaqchem_kmt2_solve_device(long long ncell, const double* params, const double* var_mix,
                                          double* var_out, double* fix_out, int* stats, double* workspace,
                                          long long workspace_doubles, void* stream)
{
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!params || !var_mix || !var_out || !stats || !workspace) return fail("null array argument");
    long long nlanes = workspace_doubles / kmt2::WS_ELEMS;
    if (nlanes < 1) return fail("workspace smaller than one lane (cmaqchem_kmt2_workspace_doubles(1) doubles)");
    if (nlanes > ncell) nlanes = ncell;
    const long long blocks = (nlanes + KMT2_THREADS - 1) / KMT2_THREADS;
    if (blocks > 0x7fffffffLL) return fail("too many lanes");
    Kmt2Args a{params, var_mix, var_out, fix_out, stats, workspace, ncell, nlanes};
    cudaStream_t s = (cudaStream_t)stream;
    k_kmt2_cells<<<(unsigned)blocks, KMT2_THREADS, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(std::string("k_kmt2_cells: ") + cudaGetErrorString(e));
    return 0;
}

// Host-array form for callers without device arrays (a Fortran cloud module): the same
// [element][cell] layouts in host memory; device buffers are allocated for the call and
// freed before it returns, the copies are synchronous.
extern "C" int cmaqchem_kmt2_solve(long long ncell, const double* params, const double* var_mix, double* var_out,
                                   double* fix_out, int* stats, int device)
{
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!params || !var_mix || !var_out || !stats) return fail("null array argument");
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    const long long lanes = std::min<long long>(ncell, (long long)(nsm > 0 ? nsm : 1) * KMT2_LANES_PER_SM);
    const size_t n = (size_t)ncell;
    const size_t bytes[6] = {sizeof(double) * kmt2::NPARAM * n, sizeof(double) * kmt2::NVAR * n,
                             sizeof(double) * kmt2::NVAR * n, fix_out ? sizeof(double) * kmt2::NFIX * n : 0,
                             sizeof(int) * kmt2::NSTAT * n,
                             sizeof(double) * (size_t)cmaqchem_kmt2_workspace_doubles(lanes)};
    void* d[6] = {};
    int rc = 0;
    for (int i = 0; i < 6 && rc == 0; ++i)
        if (bytes[i] && (e = cudaMalloc(&d[i], bytes[i])) != cudaSuccess)
            rc = fail(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    if (rc == 0 && ((e = cudaMemcpy(d[0], params, bytes[0], cudaMemcpyHostToDevice)) != cudaSuccess ||
                    (e = cudaMemcpy(d[1], var_mix, bytes[1], cudaMemcpyHostToDevice)) != cudaSuccess))
        rc = fail(std::string("copy to the device: ") + cudaGetErrorString(e));
    if (rc == 0)
        rc = cmaqchem_kmt2_solve_device(ncell, (const double*)d[0], (const double*)d[1], (double*)d[2],
                                        (double*)d[3], (int*)d[4], (double*)d[5], (long long)(bytes[5] / sizeof(double)),
                                        nullptr);
    if (rc == 0 && ((e = cudaMemcpy(var_out, d[2], bytes[2], cudaMemcpyDeviceToHost)) != cudaSuccess ||
                    (e = cudaMemcpy(stats, d[4], bytes[4], cudaMemcpyDeviceToHost)) != cudaSuccess ||
                    (fix_out && (e = cudaMemcpy(fix_out, d[3], bytes[3], cudaMemcpyDeviceToHost)) != cudaSuccess)))
        rc = fail(std::string("copy to the host: ") + cudaGetErrorString(e));
    for (void* q : d)
        if (q) cudaFree(q);
    return rc;
}

// The whole AQCHEM for a batch of cloudy cells: GAS / AEROSOL in, the KPP state, the kinetic
// core, GAS / AEROSOL / wet deposition out (include/cmaqchem.h: cmaqchem_aqchem_device).
extern "C" int cmaqchem_aqchem_device(long long ncell, const double* params, double* gas, double* aerosol, int naer,
                                      const int* aer_index, const double* factors, double* gas_wdep,
                                      double* aer_wdep, double* out, int* stats, double* workspace,
                                      long long workspace_doubles, void* stream)
{
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!params || !gas || !aerosol || !aer_index || !factors || !gas_wdep || !aer_wdep || !out || !stats ||
        !workspace)
        return fail("null array argument");
    if (naer < 1) return fail("naer must be >= 1");
    AqchemArgs a{};
    for (int i = 0; i < kmt2::KA_NIDX; ++i) {
        if (aer_index[i] < 0 || aer_index[i] >= naer) return fail("aer_index entry outside [0, naer)");
        a.ai[i] = aer_index[i];
    }
    for (int i = 0; i < kmt2::KF_N; ++i) a.fac[i] = factors[i];
    long long nlanes = workspace_doubles / kmt2::WS_ELEMS;
    if (nlanes < 1) return fail("workspace smaller than one lane (cmaqchem_kmt2_workspace_doubles(1) doubles)");
    if (nlanes > ncell) nlanes = ncell;
    const long long blocks = (nlanes + KMT2_THREADS - 1) / KMT2_THREADS;
    if (blocks > 0x7fffffffLL) return fail("too many lanes");
    a.params = params;
    a.gas = gas;
    a.aer = aerosol;
    a.gas_wdep = gas_wdep;
    a.aer_wdep = aer_wdep;
    a.out = out;
    a.stats = stats;
    a.ws = workspace;
    a.ncell = ncell;
    a.nlanes = nlanes;
    a.naer = naer;
    cudaStream_t s = (cudaStream_t)stream;
    k_aqchem_cells<<<(unsigned)blocks, KMT2_THREADS, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(std::string("k_aqchem_cells: ") + cudaGetErrorString(e));
    return 0;
}
