// ROS3 integration of one grid cell per thread, FP64.
//
// Restates the time loop of CMAQ's ROS3 solver (CCTM/src/gas/ros3/rbsolver.F:344-589)
// for a single cell, i.e. the reference with BLKSIZE = 1: the step size, error norm
// and accept / reject decision belong to the cell alone.  Method coefficients are the
// KPP ROS3 set of rbsolver.F:85-113 (Sandu et al., Atm. Env. 31, 1997).
//
// Per-cell state lives in a per-warp workspace block [element][lane] (see the
// generated mechanism header): element k of this thread's cell is ws[k * 32].
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#ifdef CHEM_PHASE_TIMING
extern __device__ unsigned long long g_chem_phase_cycles[8];
#endif

namespace ros3 {

constexpr double GAM = 0.43586652150845899941601945119356;
constexpr double C21 = -0.10156171083877702091975600115545e+01;
constexpr double C31 = 0.40759956452537699824805835358067e+01;
constexpr double C32 = 0.92076794298330791242156818474003e+01;
constexpr double B1 = 0.10000000000000000000000000000000e+01;
constexpr double B2 = 0.61697947043828245592553615689730e+01;
constexpr double B3 = -0.42772256543218573326238373806514e+00;
constexpr double D1 = 0.50000000000000000000000000000000e+00;
constexpr double D2 = -0.29079558716805469821718236208017e+01;
constexpr double D3 = 0.22354069897811569627360909276199e+00;
constexpr double GROW = 1.0 / 3.00;
constexpr double RGAM = 1.0 / GAM;
constexpr double DTSTART = 0.5e-01;
constexpr double DTMIN = 1.0e-08;
constexpr double DTMAX = 1.0e+01;
constexpr double UROUND = 1.0e-18;
constexpr double FACMAX = 1.0e+01;
constexpr double FACMIN = 1.0e-01;
constexpr double FACONE = 1.0e+00;
constexpr double CONMIN = 1.0e-30;

// per-cell status codes (bit flags)
constexpr int ST_OK = 0;
constexpr int ST_DT_UNDERFLOW = 1;   // step size fell below DTMIN (the reference stops the run)
constexpr int ST_MAXITER = 2;        // iteration cap reached (no counterpart; guards the loop)
constexpr int ST_NONFINITE = 4;      // an accepted solution held a non-finite value

struct Tol {
    double rtol, atol, rnspec;
    double dtmin = DTMIN;   // the reference's DTMIN; lowered only for tight accuracy runs
};

struct CellStats {
    int nsteps, nfails, nbad_starts, status;
};

// Fortran MAX/MIN of finite values; NaN in the error norm is kept so that the step is rejected.
__device__ __forceinline__ double fmax_keepnan(double a, double b) { return (b != b) ? b : fmax(a, b); }

// Integrator state of one cell between step attempts.
struct CellState {
    double tnow, dt;
    int iter;
    bool lpass, have_f0;
    bool yave;          // accumulate the time integral of Y in ws[OFF_YAVE] (DDM-3D)
    CellStats st;
    long long tmark;    // phase-timing builds: clock at the last phase barrier (thread 0)
};

#ifdef CHEM_PHASE_TIMING
// Diagnostic build: thread 0 of each block adds the clock cycles between consecutive
// phase barriers of the lock-stepped attempt to g_chem_phase_cycles[phase] (diag.cu,
// global namespace); slot 7 counts the block's attempts.
#define CHEM_PHASE_MARK(s, i)                                                                  \
    do {                                                                                       \
        if (threadIdx.x == 0) {                                                                \
            const long long t_ = clock64();                                                    \
            atomicAdd(&::g_chem_phase_cycles[i], (unsigned long long)(t_ - (s).tmark));        \
            (s).tmark = t_;                                                                    \
            if ((i) == 0) atomicAdd(&::g_chem_phase_cycles[7], 1ull);                           \
        }                                                                                      \
    } while (0)
#else
#define CHEM_PHASE_MARK(s, i) ((void)0)
#endif

__device__ __forceinline__ void start(CellState& s)
{
    s.tnow = 0.0;
    s.dt = fmax(DTMIN, DTSTART);
    s.iter = 0;
    s.lpass = false;
    s.have_f0 = false;
    s.yave = false;
    s.st = CellStats{0, 0, 0, ST_OK};
}

__device__ __forceinline__ bool finished(const CellState& s, double chemstep)
{
    return !(s.tnow < chemstep) || s.st.status != ST_OK;
}

// f += E (emission tendency of the cell, ppm/min)
template <class M>
__device__ __forceinline__ void add_emis(double* __restrict__ ws, int off)
{
    for (int n = 0; n < M::ISCHAN; ++n) ws[(off + n) * 32] = ws[(off + n) * 32] + ws[(M::ADJ_EMIS + n) * 32];
}

// One linear solve of a stage; SYNC as in attempt_phased.
template <class M, int SYNC>
__device__ __forceinline__ void solve_phase(double* __restrict__ ws, int rhs, bool night, bool go)
{
    if (SYNC == 2) {
        if (night) M::solve_1_sync(ws, rhs, go); else M::solve_0_sync(ws, rhs, go);
    } else {
        if (go) {
            if (night) M::solve_1(ws, rhs); else M::solve_0(ws, rhs);
        }
        if (SYNC) __syncthreads();
    }
}

// One pass of the DO WHILE body of rbsolver.F:344-589 for one cell: stages, error
// estimate, accept or reject, new step size.  Requires Y and RKI in ws.  `night` must be
// warp-uniform: it selects the night reaction list and LU pattern, which give the same
// numbers as the day pattern for a dark cell (the dropped reactions have zero rates)
// with fewer operations.  Every thread of the warp (of the block when SYNC > 0) calls
// this; lanes with active == false do no work.  SYNC = 1: the block's warps pass a
// barrier between phases; SYNC = 2: also after every generated chunk of the LU and the
// solves.  Walking the (large) generated code together lets the warps share the
// instruction cache.  EMIS: f(y) + E with the emission tendency E at ws[ADJ_EMIS] (only
// the adjoint kernels, whose workspaces hold the adjoint arrays, set it).
template <class M, int SYNC, bool EMIS = false>
__device__ void attempt_phased(double* __restrict__ ws, CellState& s, double chemstep, Tol tol, bool night,
                               int max_iter, bool active)
{
    bool go = active;
    if (go && s.iter >= max_iter) { s.st.status |= ST_MAXITER; go = false; }
    double dt = 0.0, tend = 0.0, dtinv = 0.0, gdtinv = 0.0;
    if (go) {
        s.iter++;
        // f(Y) is unchanged after a rejected step; it is kept in F0
        if (!s.have_f0) {
            if (night) M::feval_1(ws, M::OFF_Y, M::OFF_F0); else M::feval_0(ws, M::OFF_Y, M::OFF_F0);
            if (EMIS) add_emis<M>(ws, M::OFF_F0);
            s.have_f0 = true;
        }
        dt = s.dt;
        tend = s.tnow + dt;
        if (tend > chemstep) { dt = chemstep - s.tnow; tend = chemstep; }
        dtinv = 1.0 / dt;
        gdtinv = dtinv * RGAM;
        if (night) M::explic_1(ws); else M::explic_0(ws);
    }
    if (SYNC) __syncthreads();
    if (SYNC) CHEM_PHASE_MARK(s, 0);
    if (SYNC == 2) {
        if (night) M::jacdecomp_1_sync(ws, gdtinv, go); else M::jacdecomp_0_sync(ws, gdtinv, go);
    } else {
        if (go) {
            if (night) M::jacdecomp_1(ws, gdtinv); else M::jacdecomp_0(ws, gdtinv);
        }
        if (SYNC) __syncthreads();
    }
    if (SYNC) CHEM_PHASE_MARK(s, 1);
    if (go) {   // stage 1
        for (int n = 0; n < M::NSPEC; ++n) ws[(M::OFF_K1 + n) * 32] = -ws[(M::OFF_F0 + n) * 32];
    }
    solve_phase<M, SYNC>(ws, M::OFF_K1, night, go);
    if (SYNC) CHEM_PHASE_MARK(s, 2);
    if (go) {   // stage 2
        for (int n = 0; n < M::NSPEC; ++n)
            ws[(M::OFF_YP + n) * 32] = ws[(M::OFF_Y + n) * 32] + ws[(M::OFF_K1 + n) * 32];
        if (night) M::feval_1(ws, M::OFF_YP, M::OFF_YDOT); else M::feval_0(ws, M::OFF_YP, M::OFF_YDOT);
        if (EMIS) add_emis<M>(ws, M::OFF_YDOT);
        const double x1 = C21 * dtinv;
        for (int n = 0; n < M::NSPEC; ++n)
            ws[(M::OFF_K2 + n) * 32] = fma(-x1, ws[(M::OFF_K1 + n) * 32], -ws[(M::OFF_YDOT + n) * 32]);
    }
    if (SYNC) __syncthreads();
    if (SYNC) CHEM_PHASE_MARK(s, 3);
    solve_phase<M, SYNC>(ws, M::OFF_K2, night, go);
    if (SYNC) CHEM_PHASE_MARK(s, 4);
    if (go) {   // stage 3
        const double x1 = C31 * dtinv;
        const double x2 = C32 * dtinv;
        for (int n = 0; n < M::NSPEC; ++n) {
            const double t = fma(-x1, ws[(M::OFF_K1 + n) * 32], -ws[(M::OFF_YDOT + n) * 32]);
            ws[(M::OFF_K3 + n) * 32] = fma(-x2, ws[(M::OFF_K2 + n) * 32], t);
        }
    }
    solve_phase<M, SYNC>(ws, M::OFF_K3, night, go);
    if (SYNC) CHEM_PHASE_MARK(s, 5);
    if (!go) return;
    // solution and error estimate
    double err = 0.0;
    bool finite = true;
    for (int n = 0; n < M::NSPEC; ++n) {
        const double k1 = ws[(M::OFF_K1 + n) * 32];
        const double k2 = ws[(M::OFF_K2 + n) * 32];
        const double k3 = ws[(M::OFF_K3 + n) * 32];
        double yp = fma(B1, k1, ws[(M::OFF_Y + n) * 32]);
        yp = fma(B2, k2, yp);
        yp = fma(B3, k3, yp);
        ws[(M::OFF_YP + n) * 32] = yp;
        const double ytol = fma(tol.rtol, fabs(yp), tol.atol);
        double e = D1 * k1;
        e = fma(D2, k2, e);
        e = fma(D3, k3, e);
        const double q = e / ytol;
        err = fma(q, q, err);
        finite = finite && isfinite(yp);
    }
    const double maxerr = fmax_keepnan(fmax(0.0, UROUND), sqrt(err * tol.rnspec));
    double dtfac = 0.9 / pow(maxerr, GROW);
    if (maxerr <= 1.0) {
        s.st.nsteps++;
        if (s.yave) {   // YAVE += (Y + Y') / 2 * DT (rbsolver.F:468-475)
            for (int n = 0; n < M::NSPEC; ++n) {
                const double yn = fmax(ws[(M::OFF_YP + n) * 32], CONMIN);
                ws[(M::OFF_YAVE + n) * 32] = ws[(M::OFF_YAVE + n) * 32] + 0.5 * (ws[(M::OFF_Y + n) * 32] + yn) * dt;
                ws[(M::OFF_Y + n) * 32] = yn;
            }
        } else {
            for (int n = 0; n < M::NSPEC; ++n)
                ws[(M::OFF_Y + n) * 32] = fmax(ws[(M::OFF_YP + n) * 32], CONMIN);
        }
        if (!finite) s.st.status |= ST_NONFINITE;
        s.have_f0 = false;
        s.tnow = tend;
        dtfac = s.lpass ? fmax(FACMIN, fmin(dtfac, FACMAX)) : fmax(FACMIN, fmin(dtfac, FACONE));
        s.dt = fmin(DTMAX, fmax(tol.dtmin, dtfac * dt));
        s.lpass = true;
    } else {
        if (s.st.nfails == 0 && s.tnow == 0.0) s.st.nbad_starts++;
        s.st.nfails++;
        s.dt = FACMIN * dt;
        s.lpass = false;
        if (s.dt < tol.dtmin) s.st.status |= ST_DT_UNDERFLOW;
    }
}

template <class M>
__device__ __forceinline__ void attempt(double* __restrict__ ws, CellState& s, double chemstep, Tol tol,
                                        bool night, int max_iter)
{
    attempt_phased<M, 0>(ws, s, chemstep, tol, night, max_iter, true);
}

// Integrate the cell in ws over chemstep minutes (the whole DO WHILE loop).
template <class M>
__device__ CellStats integrate(double* __restrict__ ws, double chemstep, Tol tol, bool night, int max_iter,
                               bool yave = false)
{
    CellState s;
    start(s);
    if (yave) {
        s.yave = true;
        for (int n = 0; n < M::NSPEC; ++n) ws[(M::OFF_YAVE + n) * 32] = 0.0;
    }
    while (!finished(s, chemstep)) attempt<M>(ws, s, chemstep, tol, night, max_iter);
    return s.st;
}

}  // namespace ros3
