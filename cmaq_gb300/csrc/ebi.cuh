// EBI (Euler Backward Iterative) integration of one grid cell per thread, FP64.
//
// Restates CMAQ's HRSOLVER (CCTM/src/gas/ebi_<mech>/hrsolver.F:212-440) for one cell.
// The reference nests three loops (EBI time steps, sub-steps, iterations) and leaves them
// with EXIT / CYCLE; here the same control flow is a state machine advanced by one
// Backward-Euler iteration per call, so the lanes of a warp execute the same iteration
// code together and a lane whose cell is done can take a new cell at once.
// Mechanism routines HRRATES, HRG1-4, HRPRODLOSS are translated from the reference
// (generated <mech>_ebi.cu); the EBI arrays YC, YC0, YCP, PROD, LOSS, PNEG of the cell
// live in the per-warp workspace next to RKI and RXRAT.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace ebi {

// hrsolver.F:70-74
constexpr double DTMIN = 1.0e-08;
constexpr double EPSLON = 1.0e-30;
constexpr double MAXPRED = 1.0e+03;
constexpr double ZERO = 1.0e-40;
constexpr double FLOOR = 1.0e-08;

constexpr int ST_OK = 0;
constexpr int ST_DT_UNDERFLOW = 1;   // sub-step fell to DTMIN (the reference stops the run)
constexpr int ST_MAXITER = 2;        // iteration cap reached (no counterpart; guards the loop)

struct State {
    double dtc, tmstep;
    int n_ebi_steps, nebi, ninr, n_inr_steps, nbkups, iter;
    int total_iter;
    bool lebi_conv, substep_start, done;
    int status;
    uint32_t notmax[8];   // NOTMAX flags of up to 256 species
};

// EBI step count and length for a sync step of itmstep seconds (hrdriver.F:296-308)
__host__ __device__ inline void steps_for(int itmstep, double deltat, int* n, double* len)
{
    const double chemstep = (double)itmstep / 60.0;
    const int delt_sec = (int)(deltat * 60.0 + 0.1);
    if (delt_sec >= itmstep) {
        *n = 2;
        *len = 0.5 * chemstep;
    } else {
        *n = (itmstep % delt_sec == 0) ? itmstep / delt_sec : itmstep / delt_sec + 1;
        *len = chemstep / (double)(*n);
    }
}

template <class M>
__device__ void start(double* __restrict__ ws, State& s, int n_ebi_steps, double tmstep)
{
    static_assert(M::NSPEC <= 32 * 8, "NOTMAX flags hold 256 species");
    s.tmstep = tmstep;
    s.dtc = tmstep;
    s.n_ebi_steps = n_ebi_steps;
    s.nebi = 1;
    s.ninr = 1;
    s.n_inr_steps = 1;
    s.nbkups = 0;
    s.iter = 0;
    s.total_iter = 0;
    s.lebi_conv = true;
    s.substep_start = true;
    s.done = false;
    s.status = ST_OK;
    for (int k = 0; k < 8; ++k) s.notmax[k] = 0u;
    for (int i = 0; i < M::NSPEC; ++i)
        if (ws[(M::EBI_OFF_YC + i) * 32] <= MAXPRED) s.notmax[i >> 5] |= 1u << (i & 31);
}

// One Backward-Euler iteration of the current sub-step and the bookkeeping that follows it.
// yv (nullptr: off): the cell's YCDDM in the caller's YAVE array (solver species order,
// stride ystride), YCDDM += (0.5 DTC) (YC + YC0) at every converged sub-step
// (hrsolver.F:372-376)
template <class M>
__device__ void iterate(double* __restrict__ ws, State& s, int max_iter, double* yv = nullptr,
                        long long ystride = 0)
{
    if (s.total_iter >= max_iter) {
        s.status |= ST_MAXITER;
        s.done = true;
        return;
    }
    if (s.substep_start) {             // IF( LEBI_CONV ) YC0 = YC
        if (s.lebi_conv)
            for (int i = 0; i < M::NSPEC; ++i) ws[(M::EBI_OFF_YC0 + i) * 32] = ws[(M::EBI_OFF_YC + i) * 32];
        s.substep_start = false;
        s.iter = 0;
    }
    s.iter++;
    s.total_iter++;
    const double dtc = s.dtc;
    M::ebi_hrrates(ws);
    M::ebi_hrg1(ws, dtc);
    M::ebi_hrg2(ws, dtc);
    M::ebi_hrg3(ws, dtc);
    M::ebi_hrg4(ws, dtc);
    M::ebi_hrprodloss(ws);
    for (int e = 0; e < M::EBI_N_EBISP; ++e) {
        const int sp = M::ebi_ebisp(e);
        const double yc = ws[(M::EBI_OFF_YC + sp) * 32];
        ws[(M::EBI_OFF_YCP + sp) * 32] =
            yc * ((ws[(M::EBI_OFF_YC0 + sp) * 32] + ws[(M::EBI_OFF_PROD + sp) * 32] * dtc) /
                  (yc + ws[(M::EBI_OFF_LOSS + sp) * 32] * dtc));
    }
    for (int k = 0; k < M::EBI_NPNEG; ++k) {   // negative product stoichiometry (hrsolver.F:294-304)
        const int p = M::ebi_pneg(k);
        const double pneg = ws[(M::EBI_OFF_PNEG + p) * 32];
        if (pneg > 0.0) {
            const double fxdloss = pneg * dtc;
            const double yc0 = ws[(M::EBI_OFF_YC0 + p) * 32], prod = ws[(M::EBI_OFF_PROD + p) * 32];
            if (fxdloss >= yc0 + prod * dtc) {
                ws[(M::EBI_OFF_YCP + p) * 32] = 0.0;
            } else {
                const double varloss = fmax(ws[(M::EBI_OFF_LOSS + p) * 32] - pneg, ZERO);
                ws[(M::EBI_OFF_YCP + p) * 32] =
                    (yc0 + prod * dtc - fxdloss) / (1.0 + varloss * dtc / ws[(M::EBI_OFF_YC + p) * 32]);
            }
        }
    }
    bool conv = true, mxfl = false;
    for (int i = 0; i < M::NSPEC; ++i) {
        const double ycp = fmax(ZERO, ws[(M::EBI_OFF_YCP + i) * 32]);
        const double yc = ws[(M::EBI_OFF_YC + i) * 32];
        const double aerror = fmax(fabs(yc - ycp), EPSLON);
        const double rerror = aerror / fmax(FLOOR, fabs(yc + ycp));
        if (rerror > M::ebi_rtol(i) || aerror > 1.0e-5) conv = false;
        if (ycp > MAXPRED && (s.notmax[i >> 5] >> (i & 31) & 1u)) {
            mxfl = true;
            conv = false;
        }
        ws[(M::EBI_OFF_YCP + i) * 32] = ycp;
        ws[(M::EBI_OFF_YC + i) * 32] = ycp;
    }
    s.lebi_conv = conv;
    if (conv) {                               // CYCLE SUBSTEP_EBI
        if (yv) {
            static_assert(M::ISCHAN == M::NSPEC, "YCDDM is stored in the solver's species order");
            for (int i = 0; i < M::NSPEC; ++i) {
                double& a = yv[(size_t)M::iold2new(i) * ystride];
                a = fma(0.5 * dtc, ws[(M::EBI_OFF_YC + i) * 32] + ws[(M::EBI_OFF_YC0 + i) * 32], a);
            }
        }
        s.ninr++;
        s.substep_start = true;
        if (s.ninr <= s.n_inr_steps) return;
        s.nebi++;                             // sub-steps of this EBI step done
        if (s.nebi > s.n_ebi_steps) {
            s.done = true;
            return;
        }
        if (s.nbkups != 0) {
            s.nbkups = 0;
            s.n_inr_steps = 1;
            s.dtc = s.tmstep;
        }
        s.ninr = 1;
        return;
    }
    if (mxfl || s.iter >= M::EBI_NEBITER) {   // iterating for the sub-step failed
        s.nbkups++;
        if (s.dtc > DTMIN) {
            for (int i = 0; i < M::NSPEC; ++i) ws[(M::EBI_OFF_YC + i) * 32] = ws[(M::EBI_OFF_YC0 + i) * 32];
            s.dtc = 0.5 * s.dtc;
            s.n_inr_steps = 1 << (s.nbkups < 30 ? s.nbkups : 30);
            s.ninr = 1;
            s.substep_start = true;
            return;
        }
        s.status |= ST_DT_UNDERFLOW;
        s.done = true;
    }
}

}  // namespace ebi

// EBI_CELL_ONLY: the per-cell state machine above without the kernels below (the host
// build of the CPU tests)
#ifndef EBI_CELL_ONLY
#include "chem_kernels.cuh"
#include "queue_kernels.cuh"

namespace chem {

struct EbiArgs {
    int n_ebi_steps;      // EBI time steps in the sync step
    double tmstep;        // EBI_TMSTEP [min]
    const float* fwd;     // [nspec] FORWARD_CONV of the EBI driver (hrinit.F:90)
    const float* rev;     // [nspec] REVERSE_CONV (hrinit.F:91)
    // one-cell-per-lane kernel: a cell still running after defer_after iterations (> 0) is
    // dropped and its index appended to deferred[*ndeferred]; the one-cell-per-warp kernel
    // then integrates it from its gathered inputs (the same result)
    int defer_after;
    int* deferred;
    unsigned long long* ndeferred;
};

// Gather one cell as hrdriver.F:372-415 does (REAL(4) conc and met, REAL(8) pressure factor).
template <class M>
__device__ bool gather_cell_ebi(const GridArgs& a, const EbiArgs& e, long long c, double* __restrict__ ws)
{
    const float inv_dens = __fdiv_rn(1.0f, a.dens[c]);
    for (int s = 0; s < M::NSPEC; ++s) {
        const float cv = a.cgrid[(size_t)a.cgrid_index[s] * a.ncell + c];
        const float v = a.convert[s] ? fmaxf(CONCMIN_F, __fmul_rn(__fmul_rn(inv_dens, e.fwd[s]), cv))
                                     : fmaxf(cv, CONCMIN_F);
        ws[(M::EBI_OFF_YC + s) * 32] = (double)v;
    }
    const double temp = (double)a.ta[c];
    const double atmpres = (double)(1.0f / 101325.0f) * (double)a.pres[c];
    const float maomv = 1.0e6f * 28.9628f / 18.0153f;
    const double h2o = (double)fmaxf(__fmul_rn(maomv, a.qv[c]), 0.0f);
    const int col = (int)(c % a.ncolrow);
    const double seawater = fmax(0.0, (double)__fsub_rn(a.ocean_szone[col], a.seaice[col]));
    double rjv[M::NPHOTAB];
    bool sun = false;
#pragma unroll
    for (int k = 0; k < M::NPHOTAB; ++k) {
        rjv[k] = (double)a.rj[(size_t)k * a.ncell + c];
        sun = sun || (rjv[k] > 0.0);
    }
    double hetv[M::NHETERO];
#pragma unroll
    for (int k = 0; k < M::NHETERO; ++k) hetv[k] = a.khet[(size_t)c * M::NHETERO + k];
    M::rconst(ws, temp, atmpres, h2o, seawater, sun ? 1 : 0, rjv, hetv);
    return sun;
}

// Write-back of hrdriver.F:446-454.
template <class M>
__device__ void scatter_cell_ebi(const GridArgs& a, const EbiArgs& e, long long c, const double* __restrict__ ws)
{
    const float dens = a.dens[c];
    for (int s = 0; s < M::NSPEC; ++s) {
        const double y = fmax(ws[(M::EBI_OFF_YC + s) * 32], 1.0e-30);
        const float v = a.convert[s] ? (float)((double)__fmul_rn(e.rev[s], dens) * y) : (float)y;
        a.cgrid[(size_t)a.cgrid_index[s] * a.ncell + c] = v;
    }
}

// One EBI CHEM call; lanes pull cells from the work queue (ordered by previous iterations).
// DDM-3D: YCDDM of a cell zeroed when the cell starts (hrsolver.F:169-171) and divided by
// CHEMSTEP, values below 1e-25 set to zero, when it ends (:443-447); lanes first..., step
template <class M>
__device__ __forceinline__ void ycddm_zero(double* yv, long long stride, int first, int step)
{
    for (int i = first; i < M::NSPEC; i += step) yv[(size_t)i * stride] = 0.0;
}
template <class M>
__device__ __forceinline__ void ycddm_finish(double* yv, long long stride, double chemstep, int first, int step)
{
    for (int i = first; i < M::NSPEC; i += step) {
        double& a = yv[(size_t)i * stride];
        a = a / chemstep;
        if (a < 1.0e-25) a = 0.0;
    }
}

template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK, 1) k_chem_ebi_queue(GridArgs a, QueueArgs q, EbiArgs e)
{
    const int lane = threadIdx.x & 31;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    ebi::State s;
    long long cell = -1;
    bool sun = false, drained = false;
    unsigned long long iters = 0, failed = 0, sunlit = 0;
    for (;;) {
        if (!drained) {
            const unsigned need = __ballot_sync(0xffffffffu, cell < 0);
            if (need) {
                const int leader = __ffs(need) - 1;
                unsigned long long base = 0;
                if (lane == leader) base = atomicAdd(q.head, (unsigned long long)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (cell < 0) {
                    const unsigned long long pos = base + __popc(need & ((1u << lane) - 1u));
                    if (pos < queue_len(q, a.ncell)) {
                        cell = q.cell0 + (q.order ? q.order[pos] : (long long)pos);
                        sun = gather_cell_ebi<M>(a, e, cell, ws);
                        ebi::start<M>(ws, s, e.n_ebi_steps, e.tmstep);
                        if (a.yave) ycddm_zero<M>(a.yave + cell, a.ncell, 0, 1);
                    }
                }
                drained = __any_sync(0xffffffffu, base + __popc(need) >= queue_len(q, a.ncell));
            }
        }
        const bool busy = cell >= 0;
        if (!__any_sync(0xffffffffu, busy)) break;
        if (busy) {
            ebi::iterate<M>(ws, s, a.max_iter, a.yave ? a.yave + cell : nullptr, a.ncell);
            if (!s.done && e.defer_after > 0 && s.total_iter >= e.defer_after) {
                e.deferred[atomicAdd(e.ndeferred, 1ull)] = (int)cell;
                cell = -1;
            } else if (s.done) {
                scatter_cell_ebi<M>(a, e, cell, ws);
                if (a.yave) ycddm_finish<M>(a.yave + cell, a.ncell, a.chemstep, 0, 1);
                iters += s.total_iter;
                failed += s.status != ebi::ST_OK;
                sunlit += sun;
                if (a.cell_status) a.cell_status[cell] = s.status;
                if (a.cell_steps) a.cell_steps[cell] = s.total_iter;
                cell = -1;
            }
        }
    }
    if (a.counters) {
        for (int o = 16; o > 0; o >>= 1) {
            iters += __shfl_down_sync(0xffffffffu, iters, o);
            failed += __shfl_down_sync(0xffffffffu, failed, o);
            sunlit += __shfl_down_sync(0xffffffffu, sunlit, o);
        }
        if (lane == 0) {
            atomicAdd(&a.counters[0], iters);
            atomicAdd(&a.counters[2], failed);
            atomicAdd(&a.counters[3], sunlit);
        }
    }
}

struct EbiSolveArgs {
    double* yc;            // [nspec][ncell] mechanism order, updated in place
    const double* rki;     // [nrxns][ncell]
    long long ncell;
    int n_ebi_steps;
    double tmstep;
    double* ws;
    int max_iter;
    int* cell_status;
    int* cell_iters;
};

// HRSOLVER for cells with given concentrations and rate constants.
template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK, 1) k_ebi_solve(EbiSolveArgs a)
{
    const long long nwarps = (long long)gridDim.x * WARPS_PER_BLOCK;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    for (long long base = warp * 32; base < a.ncell; base += nwarps * 32) {
        const long long c = base + (threadIdx.x & 31);
        if (c >= a.ncell) continue;
        for (int i = 0; i < M::NSPEC; ++i) ws[(M::EBI_OFF_YC + i) * 32] = a.yc[(size_t)i * a.ncell + c];
        for (int r = 0; r < M::NRXNS; ++r) ws[(M::OFF_RKI + r) * 32] = a.rki[(size_t)r * a.ncell + c];
        ebi::State s;
        ebi::start<M>(ws, s, a.n_ebi_steps, a.tmstep);
        while (!s.done) ebi::iterate<M>(ws, s, a.max_iter);
        for (int i = 0; i < M::NSPEC; ++i) a.yc[(size_t)i * a.ncell + c] = ws[(M::EBI_OFF_YC + i) * 32];
        if (a.cell_status) a.cell_status[c] = s.status;
        if (a.cell_iters) a.cell_iters[c] = s.total_iter;
    }
}

}  // namespace chem

namespace chem {

// Warp-cooperative EBI: one cell per warp, its EBI state (YC, YC0, YCP, PROD, LOSS, PNEG,
// NOTMAX, RKI, RXRAT) in shared memory.  HRRATES and HRPRODLOSS run from tables, their
// statements spread over the lanes; HRG1-HRG4 (short, sequential) run on lane 0; the
// per-species loops of HRSOLVER are split over the lanes and their convergence flags
// combined by warp votes.  Every value is computed with the same operations in the same
// order as the per-lane kernel and the oracle, so results are bit-identical; what
// changes is that a cell's iteration runs on 32 lanes from shared memory instead of on
// one lane from the (DRAM-resident) workspace, which shortens the long cells that set
// the call time.
constexpr int EBIW_WPB = 4;

template <class M>
__device__ void ebiw_gather(const GridArgs& a, const EbiArgs& e, long long c, double* __restrict__ sm,
                            double* __restrict__ ws0, int lane, bool& sun)
{
    const float inv_dens = __fdiv_rn(1.0f, a.dens[c]);
    for (int s = lane; s < M::NSPEC; s += 32) {
        const float cv = a.cgrid[(size_t)a.cgrid_index[s] * a.ncell + c];
        const float v = a.convert[s] ? fmaxf(CONCMIN_F, __fmul_rn(__fmul_rn(inv_dens, e.fwd[s]), cv))
                                     : fmaxf(cv, CONCMIN_F);
        sm[M::EBIW_YC + s] = (double)v;
    }
    int lsun = 0;
    if (lane == 0) {   // met, rate constants of the cell into lane 0's workspace column
        const double temp = (double)a.ta[c];
        const double atmpres = (double)(1.0f / 101325.0f) * (double)a.pres[c];
        const float maomv = 1.0e6f * 28.9628f / 18.0153f;
        const double h2o = (double)fmaxf(__fmul_rn(maomv, a.qv[c]), 0.0f);
        const int col = (int)(c % a.ncolrow);
        const double seawater = fmax(0.0, (double)__fsub_rn(a.ocean_szone[col], a.seaice[col]));
        double rjv[M::NPHOTAB];
        for (int k = 0; k < M::NPHOTAB; ++k) {
            rjv[k] = (double)a.rj[(size_t)k * a.ncell + c];
            lsun |= rjv[k] > 0.0;
        }
        double hetv[M::NHETERO];
        for (int k = 0; k < M::NHETERO; ++k) hetv[k] = a.khet[(size_t)c * M::NHETERO + k];
        M::rconst(ws0, temp, atmpres, h2o, seawater, lsun, rjv, hetv);
    }
    sun = __shfl_sync(0xffffffffu, lsun, 0) != 0;
    __syncwarp();
    for (int r = lane; r < M::NRXNS; r += 32) {
        sm[M::EBIW_RKI + r] = ws0[(M::OFF_RKI + r) * 32];
        sm[M::EBIW_RXRAT + r] = 0.0;
    }
    for (int s = lane; s < M::NSPEC; s += 32) {
        sm[M::EBIW_PROD + s] = 0.0;
        sm[M::EBIW_LOSS + s] = 0.0;
        sm[M::EBIW_PNEG + s] = 0.0;
        sm[M::EBIW_YCP + s] = 0.0;
        sm[M::EBIW_YC0 + s] = 0.0;
        sm[M::EBIW_NOTMAX + s] = sm[M::EBIW_YC + s] <= ebi::MAXPRED ? 1.0 : 0.0;
    }
    __syncwarp();
}

// One Backward-Euler iteration of the warp's cell plus HRSOLVER's bookkeeping (the same
// control flow as ebi::iterate; the scalar state is kept identically by every lane).
template <class M>
__device__ void ebiw_iterate(double* __restrict__ sm, ebi::State& s, int max_iter, int lane, double* yv = nullptr,
                             long long ystride = 0)
{
    using namespace ebi;
    if (s.total_iter >= max_iter) {
        s.status |= ST_MAXITER;
        s.done = true;
        return;
    }
    if (s.substep_start) {
        if (s.lebi_conv)
            for (int i = lane; i < M::NSPEC; i += 32) sm[M::EBIW_YC0 + i] = sm[M::EBIW_YC + i];
        s.substep_start = false;
        s.iter = 0;
    }
    s.iter++;
    s.total_iter++;
    const double dtc = s.dtc;
    __syncwarp();
    {   // HRRATES
        const int* rr = M::ebiw_rate_r();
        const int* nf = M::ebiw_rate_nf();
        const int* sp = M::ebiw_rate_sp();
        for (int q = lane; q < M::EBIW_NRATE; q += 32) {
            const int r = rr[q];
            double acc = sm[M::EBIW_RKI + r];
            for (int j = 0; j < nf[q]; ++j) acc = acc * sm[M::EBIW_YC + sp[3 * q + j]];
            sm[M::EBIW_RXRAT + r] = acc;
        }
    }
    __syncwarp();
    if (lane == 0) {
        M::ebiw_hrg1(sm, dtc);
        M::ebiw_hrg2(sm, dtc);
        M::ebiw_hrg3(sm, dtc);
        M::ebiw_hrg4(sm, dtc);
    }
    __syncwarp();
    {   // HRPRODLOSS
        const int* ptr = M::ebiw_pl_ptr();
        const int* kind = M::ebiw_pl_kind();
        const int* spc = M::ebiw_pl_sp();
        const int* t0 = M::ebiw_pl_t0();
        const int* tr = M::ebiw_term_r();
        const double* tc = M::ebiw_term_c();
        for (int q = ptr[lane]; q < ptr[lane + 1]; ++q) {
            double acc = 0.0;
            const int a0 = t0[q], a1 = t0[q + 1];
            if (a1 > a0) {
                acc = tc[a0] * sm[M::EBIW_RXRAT + tr[a0]];
                for (int t = a0 + 1; t < a1; ++t) acc = acc + tc[t] * sm[M::EBIW_RXRAT + tr[t]];
            }
            const int base = kind[q] == 0 ? M::EBIW_PROD : (kind[q] == 1 ? M::EBIW_LOSS : M::EBIW_PNEG);
            sm[base + spc[q]] = acc;
        }
    }
    __syncwarp();
    for (int e = lane; e < M::EBI_N_EBISP; e += 32) {
        const int sp = M::ebi_ebisp(e);
        const double yc = sm[M::EBIW_YC + sp];
        sm[M::EBIW_YCP + sp] = yc * ((sm[M::EBIW_YC0 + sp] + sm[M::EBIW_PROD + sp] * dtc) /
                                     (yc + sm[M::EBIW_LOSS + sp] * dtc));
    }
    __syncwarp();
    if (lane == 0) {
        for (int k = 0; k < M::EBI_NPNEG; ++k) {
            const int p = M::ebi_pneg(k);
            const double pneg = sm[M::EBIW_PNEG + p];
            if (pneg > 0.0) {
                const double fxdloss = pneg * dtc;
                const double yc0 = sm[M::EBIW_YC0 + p], prod = sm[M::EBIW_PROD + p];
                if (fxdloss >= yc0 + prod * dtc) {
                    sm[M::EBIW_YCP + p] = 0.0;
                } else {
                    const double varloss = fmax(sm[M::EBIW_LOSS + p] - pneg, ZERO);
                    sm[M::EBIW_YCP + p] = (yc0 + prod * dtc - fxdloss) / (1.0 + varloss * dtc / sm[M::EBIW_YC + p]);
                }
            }
        }
    }
    __syncwarp();
    bool conv = true, mxfl = false;
    for (int i = lane; i < M::NSPEC; i += 32) {
        const double ycp = fmax(ZERO, sm[M::EBIW_YCP + i]);
        const double yc = sm[M::EBIW_YC + i];
        const double aerror = fmax(fabs(yc - ycp), EPSLON);
        const double rerror = aerror / fmax(FLOOR, fabs(yc + ycp));
        if (rerror > M::ebi_rtol(i) || aerror > 1.0e-5) conv = false;
        if (ycp > MAXPRED && sm[M::EBIW_NOTMAX + i] != 0.0) {
            mxfl = true;
            conv = false;
        }
        sm[M::EBIW_YCP + i] = ycp;
        sm[M::EBIW_YC + i] = ycp;
    }
    conv = __all_sync(0xffffffffu, conv);
    mxfl = __any_sync(0xffffffffu, mxfl);
    s.lebi_conv = conv;
    if (conv) {
        if (yv)   // each lane its own species, whose YC and YC0 it wrote itself
            for (int i = lane; i < M::NSPEC; i += 32) {
                double& a = yv[(size_t)M::iold2new(i) * ystride];
                a = fma(0.5 * dtc, sm[M::EBIW_YC + i] + sm[M::EBIW_YC0 + i], a);
            }
        s.ninr++;
        s.substep_start = true;
        if (s.ninr <= s.n_inr_steps) return;
        s.nebi++;
        if (s.nebi > s.n_ebi_steps) {
            s.done = true;
            return;
        }
        if (s.nbkups != 0) {
            s.nbkups = 0;
            s.n_inr_steps = 1;
            s.dtc = s.tmstep;
        }
        s.ninr = 1;
        return;
    }
    if (mxfl || s.iter >= M::EBI_NEBITER) {
        s.nbkups++;
        if (s.dtc > DTMIN) {
            __syncwarp();
            for (int i = lane; i < M::NSPEC; i += 32) sm[M::EBIW_YC + i] = sm[M::EBIW_YC0 + i];
            s.dtc = 0.5 * s.dtc;
            s.n_inr_steps = 1 << (s.nbkups < 30 ? s.nbkups : 30);
            s.ninr = 1;
            s.substep_start = true;
            return;
        }
        s.status |= ST_DT_UNDERFLOW;
        s.done = true;
    }
}

// One EBI CHEM call, a cell per warp from the work queue.  Dynamic shared memory:
// EBIW_WPB * EBIW_ELEMS doubles.
template <class M>
__global__ void __launch_bounds__(EBIW_WPB * 32) k_chem_ebi_warp(GridArgs a, QueueArgs q, EbiArgs e)
{
    extern __shared__ double smem_all[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    double* sm = smem_all + (size_t)wib * M::EBIW_ELEMS;
    const long long warp = (long long)blockIdx.x * EBIW_WPB + wib;
    double* ws0 = a.ws + (size_t)warp * ((size_t)M::WS_ELEMS * 32);   // lane 0's workspace column
    const unsigned long long qlen = queue_len(q, a.ncell);
    unsigned long long iters = 0, failed = 0, sunlit = 0;
    for (;;) {
        unsigned long long pos = 0;
        if (lane == 0) pos = atomicAdd(q.head, 1ull);
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (pos >= qlen) break;
        const long long cell = q.cell0 + (q.order ? q.order[pos] : (long long)pos);
        bool sun = false;
        ebiw_gather<M>(a, e, cell, sm, ws0, lane, sun);
        ebi::State s;
        s.tmstep = e.tmstep;
        s.dtc = e.tmstep;
        s.n_ebi_steps = e.n_ebi_steps;
        s.nebi = 1;
        s.ninr = 1;
        s.n_inr_steps = 1;
        s.nbkups = 0;
        s.iter = 0;
        s.total_iter = 0;
        s.lebi_conv = true;
        s.substep_start = true;
        s.done = false;
        s.status = ebi::ST_OK;
        double* yv = a.yave ? a.yave + cell : nullptr;
        if (yv) ycddm_zero<M>(yv, a.ncell, lane, 32);
        __syncwarp();
        while (!s.done) ebiw_iterate<M>(sm, s, a.max_iter, lane, yv, a.ncell);
        __syncwarp();
        if (yv) ycddm_finish<M>(yv, a.ncell, a.chemstep, lane, 32);
        const float dens = a.dens[cell];
        for (int sp = lane; sp < M::NSPEC; sp += 32) {   // write-back (hrdriver.F:446-454)
            const double y = fmax(sm[M::EBIW_YC + sp], 1.0e-30);
            const float v = a.convert[sp] ? (float)((double)__fmul_rn(e.rev[sp], dens) * y) : (float)y;
            a.cgrid[(size_t)a.cgrid_index[sp] * a.ncell + cell] = v;
        }
        if (lane == 0) {
            iters += s.total_iter;
            failed += s.status != ebi::ST_OK;
            sunlit += sun;
            if (a.cell_status) a.cell_status[cell] = s.status;
            if (a.cell_steps) a.cell_steps[cell] = s.total_iter;
        }
        __syncwarp();
    }
    if (a.counters && lane == 0) {
        atomicAdd(&a.counters[0], iters);
        atomicAdd(&a.counters[2], failed);
        atomicAdd(&a.counters[3], sunlit);
    }
}

}  // namespace chem
#endif  // EBI_CELL_ONLY
