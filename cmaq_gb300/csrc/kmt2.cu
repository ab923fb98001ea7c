// C ABI of the KMT2 aqueous cloud chemistry kernels (include/cmaqchem.h: cmaqchem_kmt2_*,
// cmaqchem_aqchem_device): the kinetic core of AQCHEM (CCTM/src/cloud/acm_ae7_kmt2/
// aqchem_kmt.F90:371-543), or the whole AQCHEM, for a batch of cloudy cells.
//
// Each thread is a lane with its own slice of the caller's workspace, a warp's slices
// together ([warp][element][32 lanes]: a warp's access to one element reads 256
// consecutive bytes, and a warp's workspace is one contiguous block).  The cells form a
// queue: a lane takes the next cell from a counter at the end of the workspace, advances it
// one Rodas3 attempt per pass of the kernel's loop (the phases of kmt2.cuh, with a block
// barrier between them), and takes a new cell when its cell ends, so the lanes of a warp
// stay busy while the cells' step counts differ.  A block leaves the loop when the queue is
// empty and all its lanes are idle.  The integrator's loops are bounded (200,000 Rodas3
// steps per pass, 5 step halvings per singular factorisation, 16 passes; a run of rejected
// attempts shrinks h by 0.9 or more each until it is accepted or reaches 0, whose NaN error
// norm is accepted as 1e-10), so every cell ends and so does every thread.
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

// resident 128-thread blocks per SM the kernels are built for (registers: 65536 / (128 x
// blocks), at most 255)
#ifndef KMT2_MIN_BLOCKS
#define KMT2_MIN_BLOCKS 4
#endif
constexpr int KMT2_THREADS = 128;
constexpr long long KMT2_LANES_PER_SM = KMT2_THREADS * KMT2_MIN_BLOCKS;
constexpr long long KMT2_WS_TAIL = 16;          // doubles after the lanes' slices: the queue counter

struct Kmt2Args {
    const double* params;
    const double* var_mix;
    double* var_out;
    double* fix_out;
    int* stats;
    double* ws;
    unsigned long long* next;   // the queue: cells handed out so far
    long long ncell;
    long long nlanes;           // a multiple of 32
};

// One pass of the warp's refill: the lanes with no cell (need) take consecutive cells of
// the queue with one atomic per warp.  Returns the lane's new cell, or -1 when the queue is
// empty.  Called by all 32 lanes of the warp.
__device__ __forceinline__ long long take_cell(bool need, unsigned long long* next, long long ncell)
{
    const unsigned want = __ballot_sync(0xffffffffu, need);
    if (want == 0) return -1;
    const int me = threadIdx.x & 31, leader = __ffs(want) - 1;
    unsigned long long base = 0;
    if (me == leader) base = atomicAdd(next, (unsigned long long)__popc(want));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (!need) return -1;
    const long long c = (long long)(base + (unsigned long long)__popc(want & ((1u << me) - 1u)));
    return c < ncell ? c : -1;
}

// The queue loop of a block, each pass: the warps' refill (begin(cell, c, L, st) sets a
// new cell up), then the phases of one Rodas3 attempt (kmt2.cuh: kq_next ... kq_decide)
// with a block barrier between phases (KMT2_LOCKSTEP), so that the block's warps run the
// same generated routine at the same time and share its instruction-cache lines; finish
// (cell, c, L, st) writes a finished cell.  The block leaves the loop when, after a
// refill, none of its lanes holds a cell (the queue is empty); a refill pass runs only
// when KMT2_REFILL_MIN of the block's lanes are idle or none is busy.
#ifndef KMT2_LOCKSTEP
#define KMT2_LOCKSTEP 1
#endif
#ifndef KMT2_REFILL_MIN
#define KMT2_REFILL_MIN 16
#endif
#if KMT2_LOCKSTEP
#define KMT2_PHASE_BARRIER() __syncthreads()
#else
#define KMT2_PHASE_BARRIER() ((void)0)
#endif
template <class Begin, class Finish>
__device__ __forceinline__ void kmt2_queue_loop(bool has_ws, double* ws, unsigned long long* next, long long ncell,
                                                Begin begin, Finish finish)
{
    kmt2::Cell c;
    kmt2::Lane L;
    long long st[kmt2::NSTAT];
    long long cell = -1;
    bool drained = !has_ws;
    for (;;) {
        // refill when KMT2_REFILL_MIN lanes of the block are idle (or none is busy), so that
        // the set-up of new cells runs for several lanes at once
        const int nidle = __syncthreads_count(cell < 0 && !drained);
        const int nbusy = __syncthreads_count(cell >= 0);
        const bool need = cell < 0 && !drained && (nidle >= KMT2_REFILL_MIN || nbusy == 0);
        const long long got = take_cell(need, next, ncell);
        if (need) {
            if (got < 0) {
                drained = true;
            } else {
                cell = got;
                begin(cell, c, L, st);
            }
        }
        if (!__syncthreads_or(cell >= 0)) break;
        bool att = false;
        if (cell >= 0) {
            if (kmt2::kq_next(c, L, ws, st)) {
                finish(cell, c, L, st);
                cell = -1;
            } else {
                att = true;
            }
        }
        KMT2_PHASE_BARRIER();
        if (att) att = kmt2::kq_prepare(L, ws, st);
        KMT2_PHASE_BARRIER();
        if (att) kmt2::kq_stages12(L, ws);
        KMT2_PHASE_BARRIER();
        if (att) kmt2::kq_stage_f(ws, 3, st);
        KMT2_PHASE_BARRIER();
        if (att) kmt2::kq_stage3s(L, ws);
        KMT2_PHASE_BARRIER();
        if (att) kmt2::kq_stage_f(ws, 4, st);
        KMT2_PHASE_BARRIER();
        if (att) {
            kmt2::kq_stage4s(L, ws, st);
            kmt2::kq_decide(L, ws, st);
        }
    }
}

__global__ void __launch_bounds__(KMT2_THREADS, KMT2_MIN_BLOCKS) k_kmt2_queue(Kmt2Args a)
{
    const long long lane = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double* ws = a.ws + (lane >> 5) * (kmt2::KQ_S * kmt2::WS_ELEMS) + (lane & 31);
    const long long n = a.ncell;
    constexpr long long s = kmt2::KQ_S;
    kmt2_queue_loop(
        lane < a.nlanes, ws, a.next, n,
        [&](long long cell, kmt2::Cell& c, kmt2::Lane& L, long long* st) {
            kmt2::kq_begin(c, L, a.params + cell, n, a.var_mix + cell, n, a.params[kmt2::P_HO * n + cell], ws, st);
        },
        [&](long long cell, kmt2::Cell&, kmt2::Lane& L, long long* st) {
            const double* y = ws + kmt2::W_Y * s;
            const double* f = ws + kmt2::W_F * s;
            const bool nan = L.ierr <= -101;   // failed set-up: no state to return
            for (int i = 0; i < kmt2::NVAR; ++i) a.var_out[i * n + cell] = nan ? (double)NAN : y[i * s];
            if (a.fix_out)
                for (int i = 0; i < kmt2::NFIX; ++i) a.fix_out[i * n + cell] = nan ? (double)NAN : f[i * s];
            for (int i = 0; i < kmt2::NSTAT; ++i) a.stats[i * n + cell] = (int)st[i];
        });
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
    unsigned long long* next;
    long long ncell;
    long long nlanes;
    int naer;
    int ai[kmt2::KA_NIDX];
    double fac[kmt2::KF_N];
};

// the whole AQCHEM: a new cell is mapped into the KPP state (kq_aq_map) before its set-up, a
// finished one redistributed (kq_aq_finish)
__global__ void __launch_bounds__(KMT2_THREADS, KMT2_MIN_BLOCKS) k_aqchem_queue(AqchemArgs a)
{
    const long long lane = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double* ws = a.ws + (lane >> 5) * (kmt2::KQ_S * kmt2::WS_ELEMS) + (lane & 31);
    const long long n = a.ncell;
    kmt2_queue_loop(
        lane < a.nlanes, ws, a.next, n,
        [&](long long cell, kmt2::Cell& c, kmt2::Lane& L, long long* st) {
            kmt2::kq_aq_map(a.params + cell, a.gas + cell, a.aer + cell, a.naer, a.ai, a.fac, n, ws);
            kmt2::kq_begin(c, L, a.params + cell, n, ws + kmt2::W_YNEW * kmt2::KQ_S, kmt2::KQ_S,
                           a.gas[kmt2::KG_HO * n + cell], ws, st);
        },
        [&](long long cell, kmt2::Cell& c, kmt2::Lane& L, long long* st) {
            kmt2::kq_aq_finish(c, L.ierr, st, a.params + cell, a.gas + cell, a.aer + cell, a.naer, a.ai, a.fac,
                               a.gas_wdep + cell, a.aer_wdep + cell, a.out + cell, a.stats + cell, n, ws);
        });
}

int fail(const std::string& msg)
{
    cmaqchem_set_error(msg);
    return -1;
}

// Lanes of a call: whole warps of the workspace (at most enough for ncell), the queue
// counter after the last warp's slices; returns the blocks to launch, or -1.
long long kmt2_lanes(long long ncell, double* workspace, long long workspace_doubles, long long* nlanes,
                     unsigned long long** next)
{
    const long long warp_doubles = kmt2::KQ_S * kmt2::WS_ELEMS;
    long long warps = workspace_doubles >= KMT2_WS_TAIL ? (workspace_doubles - KMT2_WS_TAIL) / warp_doubles : 0;
    if (warps < 1) return fail("workspace smaller than one warp of lanes (cmaqchem_kmt2_workspace_doubles(1) doubles)");
    warps = std::min(warps, (ncell + 31) / 32);
    const long long blocks = (warps * 32 + KMT2_THREADS - 1) / KMT2_THREADS;
    if (blocks > 0x7fffffffLL) return fail("too many lanes");
    *nlanes = warps * 32;
    *next = (unsigned long long*)(workspace + warps * warp_doubles);
    return blocks;
}

}  // namespace

extern "C" long long cmaqchem_kmt2_default_lanes(int device)
{
    int nsm = 0;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || nsm < 1) {
        cudaGetLastError();
        return fail("cmaqchem_kmt2_default_lanes: no such device");
    }
    return (long long)nsm * KMT2_LANES_PER_SM;
}

extern "C" long long cmaqchem_kmt2_workspace_doubles(long long nlanes)
{
    return nlanes > 0 ? (nlanes + 31) / 32 * 32 * (long long)kmt2::WS_ELEMS + KMT2_WS_TAIL : 0;
}

extern "C" int cmaqchem_kmt2_solve_device(long long ncell, const double* params, const double* var_mix,
                                          double* var_out, double* fix_out, int* stats, double* workspace,
                                          long long workspace_doubles, void* stream)
{
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!params || !var_mix || !var_out || !stats || !workspace) return fail("null array argument");
    long long nlanes = 0;
    unsigned long long* next = nullptr;
    const long long blocks = kmt2_lanes(ncell, workspace, workspace_doubles, &nlanes, &next);
    if (blocks < 0) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(next, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return fail(std::string("queue counter: ") + cudaGetErrorString(e));
    Kmt2Args a{params, var_mix, var_out, fix_out, stats, workspace, next, ncell, nlanes};
    k_kmt2_queue<<<(unsigned)blocks, KMT2_THREADS, 0, s>>>(a);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(std::string("k_kmt2_queue: ") + cudaGetErrorString(e));
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
    long long nlanes = 0;
    unsigned long long* next = nullptr;
    const long long blocks = kmt2_lanes(ncell, workspace, workspace_doubles, &nlanes, &next);
    if (blocks < 0) return -1;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(next, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return fail(std::string("queue counter: ") + cudaGetErrorString(e));
    a.params = params;
    a.gas = gas;
    a.aer = aerosol;
    a.gas_wdep = gas_wdep;
    a.aer_wdep = aer_wdep;
    a.out = out;
    a.stats = stats;
    a.ws = workspace;
    a.next = next;
    a.ncell = ncell;
    a.nlanes = nlanes;
    a.naer = naer;
    k_aqchem_queue<<<(unsigned)blocks, KMT2_THREADS, 0, s>>>(a);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(std::string("k_aqchem_queue: ") + cudaGetErrorString(e));
    return 0;
}
