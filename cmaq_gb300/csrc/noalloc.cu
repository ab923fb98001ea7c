// Allocation-free ROS3 solver entry point (include/cmaqchem.h: cmaqchem_ros3_solve_noalloc).
//
// Some callers cannot allocate device memory at the point where they integrate the
// chemistry: host models that own the whole device footprint through their own
// pool and forbid other allocations, callers running under a fixed device-memory
// budget, and loops in which the implicit device-wide synchronisation of
// cudaMalloc / cudaFree is not acceptable.  For them this entry point runs the same
// solver kernel as cmaqchem_ros3_solve_device, but without a handle: its per-warp
// workspace lives in the file-scope device array below, and the call itself
// allocates nothing (no cudaMalloc, cudaFree or allocating library routine).
//
// The array (CMAQCHEM_NOALLOC_SCRATCH_BYTES) exists on every GPU that loads the
// library until the process exits.  It bounds how many warps integrate at once, not
// the number of cells: the kernel strides over all cells with the warps that fit.
// Every call shares the array and it keeps the last call's contents; no element has
// to start at zero, because the integrator writes every workspace element of a cell
// before it reads it.  Calls whose kernels overlap on the GPU (different streams, or
// host threads) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>
#include <string>
#include <string.h>

#include "../../include/cmaqchem.h"
#include "mech_ops.cuh"

extern const MechOps mech_ops_cb6r5_ae7_aq;
extern const MechOps mech_ops_cracmm2;
// error text of the calling thread, shared with the other entry points (chem_capi.cu)
__attribute__((visibility("hidden"))) void cmaqchem_set_error(const std::string& msg);

namespace {

constexpr size_t SCRATCH_DOUBLES = CMAQCHEM_NOALLOC_SCRATCH_BYTES / sizeof(double);
constexpr int MAX_DEVICES = 64;

// the scratch workspace; host code may only use its address from cudaGetSymbolAddress
static __device__ __align__(256) double g_noalloc_ws[SCRATCH_DOUBLES];

std::mutex g_setup_mutex;
void* g_scratch_ptr[MAX_DEVICES] = {};

int noalloc_fail(const std::string& msg)
{
    cmaqchem_set_error(msg);   // read back through cmaqchem_last_error
    return -1;
}

// Device address of the scratch array on `device` (current), looked up once per device
// and kept until the process exits (a cudaDeviceReset would leave it stale; the header
// tells callers not to call again after one).
cudaError_t scratch_on(int device, double** out)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_ws);
        if (e != cudaSuccess) return e;
        g_scratch_ptr[device] = p;
    }
    *out = static_cast<double*>(g_scratch_ptr[device]);
    return cudaSuccess;
}

const MechOps* lookup(const char* name)
{
    if (!name) return nullptr;
    const MechOps* all[] = {&mech_ops_cb6r5_ae7_aq, &mech_ops_cracmm2};
    for (const MechOps* m : all)
        if (strcmp(m->name, name) == 0) return m;
    return nullptr;
}

}  // namespace

extern "C" int cmaqchem_ros3_solve_noalloc(const char* mechanism, long long ncell, double* y, const double* rki,
                                           const unsigned char* night, double chemstep_min, double rtol,
                                           double atol, int* status, void* stream)
{
    const MechOps* m = lookup(mechanism);
    if (!m) return noalloc_fail(std::string("unknown mechanism ") + (mechanism ? mechanism : "(null)"));
    if (ncell < 0 || ncell > CMAQCHEM_NOALLOC_MAX_CELLS)
        return noalloc_fail("ncell must be in [0, " + std::to_string((long long)CMAQCHEM_NOALLOC_MAX_CELLS) + "]");
    if (ncell == 0) return 0;
    if (!y || !rki || !night) return noalloc_fail("null array argument");
    if (!(chemstep_min > 0.0) || !(rtol > 0.0) || !(atol > 0.0))
        return noalloc_fail("chemstep, rtol and atol must be positive");
    // warps whose workspaces fit in the scratch array, in whole blocks
    const size_t per_warp = (size_t)m->ws_elems * 32;
    const long long warps = (long long)(SCRATCH_DOUBLES / per_warp);
    const int nblocks = (int)(warps / chem::WARPS_PER_BLOCK);
    if (nblocks < 1)
        return noalloc_fail(std::string("mechanism ") + m->name + " needs " +
                            std::to_string(per_warp * sizeof(double) * chem::WARPS_PER_BLOCK) +
                            " bytes of scratch per block; the array holds " +
                            std::to_string((long long)CMAQCHEM_NOALLOC_SCRATCH_BYTES));
    int device = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return noalloc_fail(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (device < 0 || device >= MAX_DEVICES) return noalloc_fail("device ordinal out of range");
    double* ws = nullptr;
    e = scratch_on(device, &ws);
    if (e != cudaSuccess) return noalloc_fail(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    chem::SolveArgs a{};
    a.y = y;
    a.rki = rki;
    a.night = night;
    a.ncell = ncell;
    a.chemstep = chemstep_min;
    a.tol = ros3::Tol{rtol, atol, (double)(1.0f / (float)m->nspec)};
    a.ws = ws;
    a.max_iter = 100000;
    a.cell_status = status;
    a.cell_nsteps = nullptr;
    a.cell_nfails = nullptr;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    e = m->solve(a, nblocks, s);
    if (e != cudaSuccess) return noalloc_fail(std::string("launch: ") + cudaGetErrorString(e));
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return noalloc_fail(std::string("kernel: ") + cudaGetErrorString(e));
    return 0;
}
