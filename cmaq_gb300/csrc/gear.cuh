// SMVGEAR (CCTM/src/gas/smvgear): variable-order, variable-step Gear (BDF) integration of
// each cell, BLKSIZE = 1 semantics, on the GPU.
//
// The reference integrates a block of cells with one shared step size and order
// (grsmvgear.F:230-1007).  Here every lane integrates its own cell: the control flow of
// SMVGEAR (restarts, order and step selection, Jacobian reuse, Newton corrector) runs
// per lane as a state machine (`advance`) that returns whenever the cell needs its next
// right-hand side (SUBFUN).  The kernel's loop then gives every busy lane of the warp
// one f evaluation together, preceded by the predictor matrix P = I - ASN1*DELT*J and
// its LU factors for the lanes whose Jacobian is due (PDERIV + DECOMP) and followed by
// the corrector solve (BACKSUB) for lanes in a Newton iteration, so the generated
// routines run with the warp converged.  Cells come from the same work queue as the ROS3
// kernel; a lane that finishes takes the next cell at once.
//
// Numbers: the symbolic structure (JSPARSE) is ROS3's (grsprse.F is rbsparse.F), and the
// generated feval/solve are ROS3's (SUBFUN's derivative sums and BACKSUB are RBFEVAL's
// and RBSOLVE's); PDERIV has its own generated assembly.  The LU pattern is the day one
// for every cell: a dark cell's photolysis rate constants are zero, so its extra entries
// are zeros and the results equal the night pattern's; unlike a ROS3 attempt, a Gear LU
// lives for many steps, so a per-warp choice could not follow the warp's changing cells.
// Floating point follows the oracle's rule (every x +/- a*b of the reference one fma),
// REAL(4) literals keep their REAL(4) values; see oracle/gear_oracle.c.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math_constants.h>
// GEAR_CELL_ONLY: the per-cell SMVGEAR code without the kernels at the end (the host
// build of the CPU tests)
#ifndef GEAR_CELL_ONLY
#include "queue_kernels.cuh"
#endif

namespace gear {

constexpr int MAXORD = 5;
constexpr int MSTEP = 3;
constexpr int MBETWEEN = 50;
constexpr int MXLOWRED = 20;
constexpr int NBINS = 5;
constexpr double HMAXDAY = 15.0, HMAXNIT = 5.0, HMIN = 1.0e-10, FRACDEC = 0.25;
constexpr double CONCMIN = 1.0e-30, ZBOUND = 1.0e-30;
constexpr double PT2 = 0.2, PT003 = 0.003, OMIC = 0.000001, OPT2MIC = 0.0000012, OPT3MIC = 0.0000013,
                 OPT4MIC = 0.0000014, HRMAX = 0.3;

// Gear coefficients (GRINIT, JSPARSE: grinit.F:163-171, grsprse.F:682-720) and tolerances
// (OPTIMAL_ATOL_PPM levels, GRVARS.F:640-668), formed on the host.
struct Coef {
    double aset[10][8];           // ASET(10, 8): [nqq-1][j-1]
    double pertst[7][3];          // PERTST**2
    double enqq1[7], enqq2[7], enqq3[7], conpst[7], conp15[7];
    double errmax;                // ERRMAX = REAL(GEAR_RTOL, 8)
    double ylow;                  // YLOW = REAL(GEAR_MIN_ATOL, 8)
    double atol_level[NBINS + 1];
    double atol_floor;            // REAL(GEAR_CONC_FLOOR, 8)
    int max_iter;                 // cap on SUBFUN calls per cell and call (0: none)
};

// Gear coefficients and tolerances: GRINIT / JSPARSE constants (grinit.F:163-171,
// grsprse.F:682-720) and the OPTIMAL_ATOL_PPM levels (GRVARS.F:640-668); the same numbers
// as the oracle's (REAL(4) expressions in REAL(4)).
inline void coefficients(double rtol, float max_atol, float min_atol, float conc_floor, int max_iter, Coef* g)
{
    static const double pertst[3][7] = {{2.0, 4.5, 7.333, 10.42, 13.7, 17.15, 1.0},
                                        {3.0, 6.0, 9.167, 12.5, 15.98, 1.0, 1.0},
                                        {1.0, 1.0, 0.5, 0.1667, 0.04133, 0.008267, 1.0}};
    *g = Coef{};
    for (int q = 0; q < 7; ++q) {
        const int nqq = q + 1;
        g->enqq1[q] = (double)(0.5f / (float)nqq);
        g->enqq2[q] = (double)(0.5f / (float)(nqq + 1));
        g->enqq3[q] = (double)(0.5f / (float)(nqq + 2));
        g->conpst[q] = 1.0 / (pertst[0][q] * g->enqq3[q]);
        g->conp15[q] = 1.5 * g->conpst[q];
        for (int k = 0; k < 3; ++k) g->pertst[q][k] = pertst[k][q] * pertst[k][q];
    }
    // Nordsieck coefficients of the BDF formulas of order 1-6 (grsprse.F:698-720)
    const double rows[6][7] = {{1.0, 1.0},
                               {2.0 / 3.0, 1.0, 1.0 / 3.0},
                               {6.0 / 11.0, 1.0, 6.0 / 11.0, 1.0 / 11.0},
                               {12.0 / 25.0, 1.0, 0.70, 0.20, 0.02},
                               {60.0 / 137.0, 1.0, 225.0 / 274.0, 85.0 / 274.0, 15.0 / 274.0, 1.0 / 274.0},
                               {180.0 / 441.0, 1.0, 406.0 / 441.0, 735.0 / 1764.0, 175.0 / 1764.0, 21.0 / 1764.0,
                                1.0 / 1764.0}};
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 7; ++j) g->aset[i][j] = rows[i][j];
    g->errmax = rtol;
    g->ylow = (double)min_atol;
    const double abhi = log10((double)max_atol), ablo = log10((double)min_atol);
    g->atol_level[0] = pow(10.0, abhi);
    g->atol_level[NBINS] = pow(10.0, ablo);
    for (int i = 2; i <= NBINS; ++i) {
        const double t = (abhi - ablo) * (double)(NBINS - i + 1) / (double)NBINS;
        g->atol_level[i - 1] = pow(10.0, ablo + t);
    }
    g->atol_floor = (double)conc_floor;
    g->max_iter = max_iter;
}

enum { ST_OK = 0, ST_DT_UNDERFLOW = 1, ST_MAXITER = 2, ST_NONFINITE = 4 };
enum { L_BEGIN = 0, L_INIT_POST = 1, L_ITER_POST = 2, L_DONE = 3 };
enum { NEED_F = 0, DONE = 1 };

struct Stats {
    int nsteps, ncfail, nefail, npderiv, nsubfun, nnewt, maxord, status;
};

struct State {
    int label;
    bool need_jac;       // the next f evaluation is preceded by P and its LU factors
    bool lsun;
    bool yave;           // DDM-3D: accumulate CAVEG (grsmvgear.F, sens blocks)
    int ifsuccess, idoub, nslp, jrestar, nqq, nqqold, kstep, jeval, l3, nqqisc, jfail, nylowred;
    bool higher_order;
    double xelaps, told, rdelmax, hratio, asn1, delt, rdelt, enqq, eup, edwn, drate, rmserr, der2max, rdeltup;
    double ylowa, r1delt;
    Stats st;
};

__device__ __forceinline__ double min2(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double max2(double a, double b) { return b > a ? b : a; }

// x**y of SMVGEAR's step-size estimates (grsmvgear.F:939, 955, 972) for x >= 0, y > 0,
// as exp(y log x) from series, with IEEE +, -, *, /, fma, frexp/ldexp and rint only, so
// that the device and the oracle (oracle/gear_oracle.c: gear_pow, the same operations)
// give the same bits.  libm's pow differs by ulps between platforms, and a single ulp
// changes the step sequence of stiff cells (measured: 830 vs 823 and 913 step attempts).
// log: x = m 2^k, m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(s), s = (m-1)/(m+1), series
// to s^23; exp: t = n ln2 + r with a Cody-Waite split of ln2, |r| <= ln2/2, Taylor series
// to r^13.  Relative error below 4e-16 x max(1, |y log x|) (about 4e-15 at x = 1e-30).
static __device__ double gpow(double x, double y)
{
    if (!(x > 0.0)) return x == 0.0 ? 0.0 : x;
    if (isinf(x)) return x;
    int k;
    double m = frexp(x, &k);
    if (m < 0x1.6a09e667f3bcdp-1) {
        m = m * 2.0;
        k = k - 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double z = s * s;
    double p = 0x1.642c8590b2164p-5;        // 1/23
    p = fma(p, z, 0x1.8618618618618p-5);    // 1/21
    p = fma(p, z, 0x1.af286bca1af28p-5);    // 1/19
    p = fma(p, z, 0x1.e1e1e1e1e1e1ep-5);    // 1/17
    p = fma(p, z, 0x1.1111111111111p-4);    // 1/15
    p = fma(p, z, 0x1.3b13b13b13b14p-4);    // 1/13
    p = fma(p, z, 0x1.745d1745d1746p-4);    // 1/11
    p = fma(p, z, 0x1.c71c71c71c71cp-4);    // 1/9
    p = fma(p, z, 0x1.2492492492492p-3);    // 1/7
    p = fma(p, z, 0x1.999999999999ap-3);    // 1/5
    p = fma(p, z, 0x1.5555555555555p-2);    // 1/3
    p = fma(p, z, 1.0);
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    const double lx = fma((double)k, ln2_hi, fma((double)k, ln2_lo, (2.0 * s) * p));
    const double t = y * lx;
    if (t > 709.0) return CUDART_INF;
    if (t < -745.0) return 0.0;
    const double n = rint(t * 0x1.71547652b82fep+0);   // t / ln2
    const double r = fma(-n, ln2_lo, fma(-n, ln2_hi, t));
    double e = 0x1.6124613a86d09p-33;       // 1/13!
    e = fma(e, r, 0x1.1eed8eff8d898p-29);   // 1/12!
    e = fma(e, r, 0x1.ae64567f544e4p-26);   // 1/11!
    e = fma(e, r, 0x1.27e4fb7789f5cp-22);   // 1/10!
    e = fma(e, r, 0x1.71de3a556c734p-19);   // 1/9!
    e = fma(e, r, 0x1.a01a01a01a01ap-16);   // 1/8!
    e = fma(e, r, 0x1.a01a01a01a01ap-13);   // 1/7!
    e = fma(e, r, 0x1.6c16c16c16c17p-10);   // 1/6!
    e = fma(e, r, 0x1.1111111111111p-7);    // 1/5!
    e = fma(e, r, 0x1.5555555555555p-5);    // 1/4!
    e = fma(e, r, 0x1.5555555555555p-3);    // 1/3!
    e = fma(e, r, 0.5);
    e = fma(e, r, 1.0);
    e = fma(e, r, 1.0);
    return ldexp(e, (int)n);
}

// The state machine below runs in two forms.  S = 32, COOP = false: one cell per lane on
// the per-warp workspace ([element][lane]), calling the generated routines.  S = 1,
// COOP = true: one cell per warp on the warp's shared-memory copy of the cell's workspace;
// element-wise species loops are spread over the lanes (LOOP, then SYNC) and the f
// evaluation, P and its LU and the solves run in table-driven cooperative forms
// (coop_feval, coop_pdecomp, coop_solve), while every lane runs the control flow and the
// reductions (in the reference's order) itself, so all lanes hold the same state.  Both
// forms perform the same operations in the same order on every element.
#define GW(off) ws[(off) * S]
#define LOOP(i, n) for (int i = (COOP ? (int)(threadIdx.x & 31) : 0); i < (n); i += (COOP ? 32 : 1))
#define SYNC()                 \
    do {                       \
        if (COOP) __syncwarp(); \
    } while (0)

// Sum over species of e_j * e_j in species order (fma chain), e_j = EXPR(j).  Cooperative
// form: the lanes form the e_j into the scratch array GEAR_E first, then every lane runs
// the chain; the same products and the same order either way.
#define REDUCE_SQ(result, EXPR)                                                              \
    do {                                                                                     \
        double dely_ = 0.0;                                                                  \
        if (COOP) {                                                                          \
            SYNC();                                                                          \
            LOOP(j, isc) GW(M::GEAR_E + j) = (EXPR);                                         \
            SYNC();                                                                          \
            for (int j = 0; j < isc; ++j) {                                                  \
                const double e_ = GW(M::GEAR_E + j);                                         \
                dely_ = fma(e_, e_, dely_);                                                  \
            }                                                                                \
        } else {                                                                             \
            for (int j = 0; j < isc; ++j) {                                                  \
                const double e_ = (EXPR);                                                    \
                dely_ = fma(e_, e_, dely_);                                                  \
            }                                                                                \
        }                                                                                    \
        result = dely_;                                                                      \
    } while (0)

// OPTIMAL_ATOL_PPM (GRVARS.F:670-706) for one cell
template <class M, int S>
__device__ double optimal_atol(const double* __restrict__ ws, const Coef* __restrict__ K)
{
    const double l0 = K->atol_level[0], l1 = K->atol_level[1], l2 = K->atol_level[2], l3 = K->atol_level[3],
                 l4 = K->atol_level[4], l5 = K->atol_level[5], fl = K->atol_floor;
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0, b5 = 0;
    for (int s = 0; s < M::NSPEC; ++s) {
        const double v = GW(M::GEAR_CNEW + s);
        if (v >= l0) ++b0;
        else if (v >= l1) ++b1;
        else if (v >= l2) ++b2;
        else if (v >= l3) ++b3;
        else if (v >= l4) ++b4;
        else if (v >= fl) ++b5;
    }
    const int c0 = b0, c1 = b1 + c0, c2 = b2 + c1, c3 = b3 + c2, c4 = b4 + c3, c5 = b5 + c4;
    const int cutoff = (int)__fmul_rn(0.4f, (float)c5);
    return c0 > cutoff ? l0 : c1 > cutoff ? l1 : c2 > cutoff ? l2 : c3 > cutoff ? l3 : c4 > cutoff ? l4 : l5;
}

// Pascal-triangle prediction of the history (sign +1) or its undoing (-1).  The reference's
// loop runs I upwards, so each column reads the next column's old values: columns go in
// order, the species of one column in parallel.
template <class M, int S, bool COOP>
__device__ __forceinline__ void predict(double* __restrict__ ws, int nqq, int nqqisc, double sign)
{
    constexpr int isc = M::ISCHAN;
    int i1 = nqqisc;
    for (int jb = 1; jb <= nqq; ++jb) {
        i1 -= isc;
        for (int c0 = i1; c0 < nqqisc; c0 += isc) {
            LOOP(j, isc) {
                double& z = GW(M::GEAR_CONC + c0 + j);
                const double zn = GW(M::GEAR_CONC + c0 + j + isc);
                z = sign > 0.0 ? z + zn : z - zn;
            }
            SYNC();
        }
    }
}

template <class M, int S, bool COOP>
__device__ void start(State& s, double* __restrict__ ws, bool lsun, const Coef* __restrict__ K, bool yave = false)
{
    s = State{};
    s.label = L_BEGIN;
    s.lsun = lsun;
    s.yave = yave;
    s.rmserr = 0.0;
    s.drate = 0.7;
    LOOP(i, M::NSPEC) {
        GW(M::GEAR_BLKCONC + i) = GW(M::GEAR_CNEW + i);
        if (yave) GW(M::GEAR_CAVEG + i) = 0.0;   // CAVEG = 0 (grsmvgear.F:273-274)
    }
    SYNC();
    s.ylowa = optimal_atol<M, S>(ws, K);
}

// grsmvgear.F:1002-1005 (and CAVEG / CHEMSTEP floored at CONCMIN, :1007-1013), plus the
// status checks of this build
template <class M, int S, bool COOP>
__device__ int finish(State& s, double* __restrict__ ws, bool failed, double chemstep)
{
    constexpr int isc = M::ISCHAN;
    const double rchem = 1.0 / chemstep;
    bool bad = false;
    LOOP(i, isc) {
        double& c = GW(M::GEAR_CNEW + i);
        if (failed) c = GW(M::GEAR_CONC + i);   // last accepted state
        if (c <= ZBOUND) c = CONCMIN;
        bad = bad || !isfinite(c);
        if (s.yave) GW(M::GEAR_CAVEG + i) = max2(GW(M::GEAR_CAVEG + i) * rchem, CONCMIN);
    }
    SYNC();
    if (COOP) bad = __any_sync(0xffffffffu, bad);
    if (bad) s.st.status |= ST_NONFINITE;
    s.label = L_DONE;
    return DONE;
}

// Run SMVGEAR's control flow (grsmvgear.F:326-1000) from s.label until the cell needs
// SUBFUN (returns NEED_F; s.label says where to resume, s.need_jac whether P and its LU
// are due first) or is done (DONE).  On entry at L_ITER_POST, GLOSS holds the corrector
// solve's result; at L_INIT_POST, SUBFUN's.
template <class M, int S, bool COOP>
__device__ int advance(double* __restrict__ ws, State& s, const Coef* __restrict__ K, double chemstep)
{
    constexpr int isc = M::ISCHAN;
#define CN(i) GW(M::GEAR_CNEW + (i))
#define GL(i) GW(M::GEAR_GLOSS + (i))
#define DT(i) GW(M::GEAR_DTLOS + (i))
#define CH(i) GW(M::GEAR_CHOLD + (i))
#define CE(i) GW(M::GEAR_CEST + (i))
#define CO(i) GW(M::GEAR_CONC + (i))
#define ASET(i, j) K->aset[(i) - 1][(j) - 1]
    const double order = (double)isc;
    const double eps = K->errmax, eps1 = 1.0 / eps, epslow = min2(eps, PT003);
    const double h0fac = s.lsun ? 0.0625 : 1.0;
    const double hmax = s.lsun ? HMAXDAY : HMAXNIT;
    const double abst2 = 1.0 / (chemstep * chemstep);
    switch (s.label) {
    case L_BEGIN: goto loop_begin;
    case L_INIT_POST: goto init_post;
    case L_ITER_POST: goto iter_post;
    default: return DONE;
    }

loop_begin:
    s.ifsuccess = 1;
    s.idoub = 2;
    s.xelaps = 0.0;
    s.told = s.xelaps;
    s.rdelmax = 10000.0;
    s.nslp = MBETWEEN;
    s.jrestar = 0;
    s.hratio = 0.0;
    s.asn1 = 1.0;

loop_initialize:
    s.need_jac = false;
    s.label = L_INIT_POST;
    s.st.nsubfun++;
    return NEED_F;

init_post:
    {
        const double yloweps = s.ylowa / epslow;
        double dely;
        REDUCE_SQ(dely, GL(j) / (CN(j) + yloweps));
        const double rmstop = dely > 0.0 ? dely : 0.0;
        double delt = sqrt(epslow / (abst2 + rmstop / order)) * h0fac;
        delt = min2(delt, chemstep);
        delt = min2(delt, hmax);
        s.delt = max2(delt, HMIN);
        s.nqq = 1;
        const double dl = s.delt;
        LOOP(j, isc) {
            CO(j) = CN(j);
            CO(isc + j) = dl * GL(j);
            if (s.yave) GW(M::GEAR_CFINI + j) = GW(M::GEAR_BLKCONC + j);   // CFINI = BLKCONC (grsmvgear.F:427-431)
        }
        SYNC();
        s.nqqold = 0;
        s.rdelt = 1.0;
        s.jeval = 1;
    }

loop_order:
    s.higher_order = true;
    {
        const double timremain = chemstep - s.xelaps;
        if (timremain <= OMIC) return finish<M, S, COOP>(s, ws, false, chemstep);
        if (s.nqq != s.nqqold) {
            s.nqqold = s.nqq;
            s.kstep = s.nqq + 1;
            s.hratio = s.hratio * ASET(s.nqq, 1) / s.asn1;
            s.asn1 = ASET(s.nqq, 1);
            s.enqq = K->pertst[s.nqq - 1][0] * order;
            s.eup = K->pertst[s.nqq - 1][1] * order;
            s.edwn = K->pertst[s.nqq - 1][2] * order;
            s.nqqisc = s.nqq * isc;
        }
        s.rdelt = min2(min2(min2(s.rdelt, s.rdelmax), hmax / s.delt), timremain / s.delt);
    }
    s.delt = s.delt * s.rdelt;
    s.hratio = s.hratio * s.rdelt;
    if (s.delt < HMIN) {
        s.ylowa = s.ylowa * (double)0.1f;
        s.nylowred++;
        if (s.nylowred < MXLOWRED) {
            LOOP(i, isc) CN(i) = GW(M::GEAR_BLKCONC + i);
            SYNC();
            goto loop_begin;
        }
        s.st.status |= ST_DT_UNDERFLOW;
        return finish<M, S, COOP>(s, ws, true, chemstep);
    }
    if (s.rdelt != 1.0) {
        double rdelta = 1.0;
        int i1 = 0;
        for (int j = 2; j <= s.kstep; ++j) {
            rdelta = rdelta * s.rdelt;
            i1 += isc;
            const double rd = rdelta;
            LOOP(i, isc) CO(i1 + i) = CO(i1 + i) * rd;
        }
        SYNC();
    }
    if (s.ifsuccess == 1) {
        s.rdelmax = 10.0;
        if (s.st.nsteps % 3 == 2) s.ylowa = optimal_atol<M, S>(ws, K);
        const double yloweps1 = s.ylowa * eps1;
        LOOP(j, isc) CH(j) = eps1 / (fabs(CN(j)) + yloweps1);
        SYNC();
    }
    if (fabs(s.hratio - 1.0) > HRMAX || s.st.nsteps >= s.nslp) s.jeval = 1;
    s.xelaps = s.xelaps + s.delt;
    predict<M, S, COOP>(ws, s.nqq, s.nqqisc, 1.0);

newton_start:
    s.l3 = 0;
    s.st.nnewt++;
    LOOP(i, isc) {
        CN(i) = CO(i);
        DT(i) = 0.0;
    }
    SYNC();
    s.need_jac = false;
    if (s.jeval == 1) {
        s.r1delt = -s.asn1 * s.delt;
        s.need_jac = true;
        s.st.npderiv++;
        s.jeval = -1;
        s.hratio = 1.0;
        s.nslp = s.st.nsteps + MBETWEEN;
        s.drate = 0.70;
    }

newton_iter:
    if (K->max_iter > 0 && s.st.nsubfun >= K->max_iter) {
        predict<M, S, COOP>(ws, s.nqq, s.nqqisc, -1.0);
        s.st.status |= ST_MAXITER;
        return finish<M, S, COOP>(s, ws, true, chemstep);
    }
    s.st.nsubfun++;
    s.label = L_ITER_POST;
    return NEED_F;

iter_post:
    s.need_jac = false;
    {
        const double asn1 = s.asn1;
        LOOP(i, isc) {
            const double d = DT(i) + GL(i);
            DT(i) = d;
            CN(i) = fma(asn1, d, CO(i));
        }
        SYNC();
        double dely;
        REDUCE_SQ(dely, GL(j) * CH(j));
        const double rmserrp = s.rmserr;
        s.der2max = dely > 0.0 ? dely : 0.0;
        s.rmserr = sqrt(s.der2max / order);
        s.l3++;
        if (s.l3 > 1) {
            const double rmsrat = s.rmserr / rmserrp;
            s.drate = max2((double)0.2f * s.drate, rmsrat);
        }
        const double dcon = s.rmserr * min2(K->conpst[s.nqq - 1], K->conp15[s.nqq - 1] * s.drate);
        if (dcon <= 1.0) goto converged;
    }
    if (s.l3 < MSTEP) goto newton_iter;
    s.st.ncfail++;
    if (s.jeval == 0) {
        s.jeval = 1;
        goto newton_start;
    }
    s.rdelmax = 2.0;
    s.xelaps = s.told;
    s.rdelt = FRACDEC;
    s.jeval = 1;
    s.ifsuccess = 0;
    predict<M, S, COOP>(ws, s.nqq, s.nqqisc, -1.0);
    goto loop_order;

converged:
    s.jeval = 0;
    if (s.l3 > 1) {
        double dely;
        REDUCE_SQ(dely, DT(j) * CH(j));
        s.der2max = dely > 0.0 ? dely : 0.0;
    }
    if (s.der2max > s.enqq) {
        s.st.nefail++;
        s.xelaps = s.told;
        s.jfail++;
        predict<M, S, COOP>(ws, s.nqq, s.nqqisc, -1.0);
        s.rdelmax = 2.0;
        if (s.jfail <= 6) {
            s.ifsuccess = 0;
            s.rdeltup = 0.0;
            s.higher_order = false;
        } else if (s.jfail <= 20) {
            s.ifsuccess = 0;
            s.rdelt = FRACDEC;
            goto loop_order;
        } else {
            s.ifsuccess = 1;
            s.delt = s.delt * 0.1;
            s.rdelt = 1.0;
            s.jfail = 0;
            s.jrestar++;
            s.idoub = 5;
            LOOP(i, isc) CN(i) = CO(i);
            SYNC();
            if (s.jrestar == 100) {
                s.st.status |= ST_MAXITER;
                return finish<M, S, COOP>(s, ws, true, chemstep);
            }
            goto loop_initialize;
        }
    } else {
        s.jfail = 0;
        s.ifsuccess = 1;
        s.told = s.xelaps;
        s.st.nsteps++;
        if (s.nqq > s.st.maxord) s.st.maxord = s.nqq;
        int i1 = -isc;
        for (int j = 1; j <= s.kstep; ++j) {
            i1 += isc;
            const double a = ASET(s.nqq, j);
            LOOP(i, isc) CO(i1 + i) = fma(a, DT(i), CO(i1 + i));
        }
        SYNC();
        LOOP(i, isc) {
            if (CO(i) <= CONCMIN) {
                CO(i) = ZBOUND;
                CN(i) = ZBOUND;
                for (int k = 1; k <= 5; ++k) CO(i + k * isc) = 0.0;
            }
            if (s.yave) {   // CAVEG += 0.5 (CFINI + CONC) DELT; CFINI = CONC (grsmvgear.F:841-849)
                const double c = CO(i);
                GW(M::GEAR_CAVEG + i) = fma(0.5 * (GW(M::GEAR_CFINI + i) + c), s.delt, GW(M::GEAR_CAVEG + i));
                GW(M::GEAR_CFINI + i) = c;
            }
        }
        SYNC();
        if (s.idoub > 1) {
            s.idoub--;
            if (s.idoub == 1) {
                LOOP(j, isc) CE(j) = DT(j);
                SYNC();
            }
            s.rdelt = 1.0;
            goto loop_order;
        }
    }

    // step size and order of the next step (grsmvgear.F:893-995)
    if (s.higher_order) {
        if (s.nqq < MAXORD) {
            double dely;
            REDUCE_SQ(dely, (DT(j) - CE(j)) * CH(j));
            const double der3max = dely > 0.0 ? dely : 0.0;
            const double pr3 = (double)1.4f * gpow(der3max / s.eup, K->enqq3[s.nqq - 1]);
            s.rdeltup = 1.0 / (pr3 + OPT4MIC);
        } else {
            s.rdeltup = 0.0;
        }
    }
    s.higher_order = true;
    {
        const double pr2 = 1.2 * gpow(s.der2max / s.enqq, K->enqq2[s.nqq - 1]);
        const double rdeltsm = 1.0 / (pr2 + OPT2MIC);
        double rdeltdn = 0.0;
        if (s.nqq > 1) {
            double dely;
            const int col = (s.kstep - 1) * isc;
            REDUCE_SQ(dely, CO(col + j) * CH(j));
            const double der1max = dely > 0.0 ? dely : 0.0;
            const double pr1 = 1.3 * gpow(der1max / s.edwn, K->enqq1[s.nqq - 1]);
            rdeltdn = 1.0 / (pr1 + OPT3MIC);
        }
        s.rdelt = max2(max2(rdeltsm, s.rdeltup), rdeltdn);
        if (s.rdelt < (double)1.1f && s.ifsuccess == 1) {
            s.idoub = 3;
            goto loop_order;
        }
        if (s.rdelt == rdeltdn) {
            s.nqq = s.nqq - 1;
            if (s.ifsuccess == 0) s.rdelt = min2(s.rdelt, 1.0);
        } else if (s.rdelt == s.rdeltup) {
            const double consmult = ASET(s.nqq, s.kstep) / (double)s.kstep;
            s.nqq = s.kstep;
            const int nqisc = s.nqq * isc;
            LOOP(j, isc) CO(j + nqisc) = DT(j) * consmult;
            SYNC();
        }
    }
    if (s.jfail >= 2) s.rdelt = min2(s.rdelt, PT2);
    s.idoub = s.nqq + 1;
    goto loop_order;
#undef CN
#undef GL
#undef DT
#undef CH
#undef CE
#undef CO
#undef ASET
}

// ---- warp-cooperative forms of the generated routines (one cell per warp, workspace in
// shared memory with stride 1), driven by the generator's gw tables.  Each element gets
// the same operations in the same order as in the generated sequential code.

// GLOSS = f(CNEW): rates over the lanes, then each species' terms in RBFEVAL's order by
// the lane the species is assigned to
template <class M>
__device__ void coop_feval(double* __restrict__ ws)
{
    const int lane = threadIdx.x & 31;
    const int* ar = M::gw_act_r();
    const int* asp = M::gw_act_sp();
    for (int t = lane; t < M::GW_NACT; t += 32) {
        double x = ws[M::OFF_RKI + ar[t]];
        const int s0 = asp[3 * t], s1 = asp[3 * t + 1], s2 = asp[3 * t + 2];
        if (s0 >= 0) x = x * ws[M::GEAR_CNEW + s0];
        if (s1 >= 0) x = x * ws[M::GEAR_CNEW + s1];
        if (s2 >= 0) x = x * ws[M::GEAR_CNEW + s2];
        ws[M::OFF_RXRAT + ar[t]] = x;
    }
    __syncwarp();
    const int* lp = M::gw_lane_ptr();
    const int* ls = M::gw_lane_sp();
    const int* sptr = M::gw_sum_ptr();
    const int* sr = M::gw_sum_r();
    const int* sk = M::gw_sum_k();
    const double* sc = M::gw_sum_c();
    for (int u = lp[lane]; u < lp[lane + 1]; ++u) {
        const int sp = ls[u];
        const int t0 = sptr[sp], t1 = sptr[sp + 1];
        double a = 0.0;
        if (t0 < t1) {
            const double r0 = ws[M::OFF_RXRAT + sr[t0]];
            a = sk[t0] ? sc[t0] * r0 : -r0;
            for (int t = t0 + 1; t < t1; ++t) {
                const double rr = ws[M::OFF_RXRAT + sr[t]];
                a = sk[t] ? fma(sc[t], rr, a) : a - rr;
            }
        }
        ws[M::GEAR_GLOSS + sp] = a;
    }
    __syncwarp();
}

// P = I - ASN1*DELT*J at CNEW and its LU factors: EXPLIC and the assembly over the lanes,
// then the elimination pivot by pivot (L entries of the pivot's column scaled, then its
// updates, each over the lanes)
template <class M>
__device__ void coop_pdecomp(double* __restrict__ ws, double r1delt)
{
    const int lane = threadIdx.x & 31;
    const int* xr = M::gw_ex_r();
    const int* xs = M::gw_ex_sp();
    const int* xo = M::gw_ex_off();
#define CEFF_(v) ((v) <= 1.0e-30 ? 0.0 : (v))
    for (int t = lane; t < M::GW_NEX; t += 32) {
        const double kk = ws[M::OFF_RKI + xr[t]];
        const double y1 = CEFF_(ws[M::GEAR_CNEW + xs[3 * t]]);
        const double y2 = CEFF_(ws[M::GEAR_CNEW + xs[3 * t + 1]]);
        const int o = xo[t];
        if (xs[3 * t + 2] < 0) {
            ws[o] = kk * y2;
            ws[o + 1] = kk * y1;
        } else {
            const double y3 = CEFF_(ws[M::GEAR_CNEW + xs[3 * t + 2]]);
            const double cr2 = kk * y2;
            ws[o] = cr2 * y3;
            ws[o + 1] = (kk * y1) * y3;
            ws[o + 2] = cr2 * y1;
        }
    }
#undef CEFF_
    __syncwarp();
    double* __restrict__ lu = ws + M::OFF_LU;
    double* __restrict__ vd = ws + M::OFF_VDIAG;
    const int* ap = M::gw_asm_ptr();
    const int* asrc = M::gw_asm_src();
    const int* ak = M::gw_asm_kind();
    const double* ac = M::gw_asm_c();
    constexpr int NST = M::IARRAY_DAY;
    for (int st = lane + 1; st <= NST; st += 32) {
        double a = st > NST - M::ISCHAN ? 1.0 : 0.0;   // the diagonal is stored last
        for (int t = ap[st]; t < ap[st + 1]; ++t) {
            const double ex = ws[asrc[t]];
            const int k = ak[t];
            a = k < 0 ? fma(-r1delt, ex, a) : (k == 0 ? fma(r1delt, ex, a) : fma(ac[t] * r1delt, ex, a));
        }
        lu[st] = a;
    }
    __syncwarp();
    const int* pd = M::gw_piv_diag();
    const int* lsp = M::gw_lsc_ptr();
    const int* lst = M::gw_lsc_st();
    const int* upp = M::gw_up_ptr();
    const int* uij = M::gw_up_ij();
    const int* uik = M::gw_up_ik();
    const int* ukj = M::gw_up_kj();
    for (int k = 0; k < M::ISCHAN; ++k) {
        const double v = 1.0 / lu[pd[k]];
        vd[k] = v;
        for (int t = lsp[k] + lane; t < lsp[k + 1]; t += 32) lu[lst[t]] = lu[lst[t]] * v;
        __syncwarp();
        for (int t = upp[k] + lane; t < upp[k + 1]; t += 32) lu[uij[t]] = fma(-lu[uik[t]], lu[ukj[t]], lu[uij[t]]);
        __syncwarp();
    }
}

// forward then backward substitution in place at ws[rhs], rows of a dependency level over
// the lanes, each row's terms in RBSOLVE's order
template <class M>
__device__ void coop_solve(double* __restrict__ ws, int rhs)
{
    const int lane = threadIdx.x & 31;
    const double* __restrict__ lu = ws + M::OFF_LU;
    const double* __restrict__ vd = ws + M::OFF_VDIAG;
    double* __restrict__ b = ws + rhs;
    const int* flp = M::gw_fl_ptr();
    const int* flr = M::gw_fl_row();
    const int* frp = M::gw_fr_ptr();
    const int* frs = M::gw_fr_st();
    const int* frc = M::gw_fr_col();
    for (int l = 0; l < M::GW_NFL; ++l) {
        for (int u = flp[l] + lane; u < flp[l + 1]; u += 32) {
            const int i = flr[u];
            double x = b[i];
            for (int t = frp[i]; t < frp[i + 1]; ++t) x = fma(-lu[frs[t]], b[frc[t]], x);
            b[i] = x;
        }
        __syncwarp();
    }
    const int* blp = M::gw_bl_ptr();
    const int* blr = M::gw_bl_row();
    const int* brp = M::gw_br_ptr();
    const int* brs = M::gw_br_st();
    const int* brc = M::gw_br_col();
    for (int l = 0; l < M::GW_NBL; ++l) {
        for (int u = blp[l] + lane; u < blp[l + 1]; u += 32) {
            const int i = blr[u];
            double x = b[i];
            for (int t = brp[i]; t < brp[i + 1]; ++t) x = fma(-lu[brs[t]], b[brc[t]], x);
            b[i] = x * vd[i];
        }
        __syncwarp();
    }
}

// The f evaluation a cell asked for, with its predictor matrix first and its corrector
// solve after (day pattern, see the file comment).
template <class M, int S, bool COOP>
__device__ __forceinline__ void evaluate(double* __restrict__ ws, const State& s, bool go)
{
    if (go && s.need_jac) {
        if (COOP) {
            coop_pdecomp<M>(ws, s.r1delt);
        } else {
            M::gear_explic_0(ws);
            M::gear_pdecomp_0(ws, s.r1delt);
        }
    }
    if (go) {
        if (COOP) coop_feval<M>(ws);
        else M::feval_0(ws, M::GEAR_CNEW, M::GEAR_GLOSS);
        SYNC();
        LOOP(i, M::ISCHAN) {   // SUBFUN's floor (grsubfun.F:164-171)
            double& g = GW(M::GEAR_GLOSS + i);
            if (GW(M::GEAR_CNEW + i) <= ZBOUND && g < 0.0) g = 0.0;
        }
        SYNC();
    }
    if (go && s.label == L_ITER_POST) {
        const double delt = s.delt;
        LOOP(i, M::ISCHAN) {   // grsmvgear.F:616-620
            double& g = GW(M::GEAR_GLOSS + i);
            g = fma(delt, g, -(GW(M::GEAR_CONC + M::ISCHAN + i) + GW(M::GEAR_DTLOS + i)));
        }
        SYNC();
        if (COOP) coop_solve<M>(ws, M::GEAR_GLOSS);
        else M::solve_0(ws, M::GEAR_GLOSS);
        SYNC();
    }
}
#undef REDUCE_SQ
#undef LOOP
#undef SYNC
#undef GW

}  // namespace gear

#ifndef GEAR_CELL_ONLY
namespace chem {

#ifndef GEAR_WARPS_PER_SM
#define GEAR_WARPS_PER_SM 16
#endif
constexpr int GEAR_WPB = 4;   // warps per block

struct GearArgs {
    const gear::Coef* coef;
    // solver level (k_gear with GRID = false): cells given in the solver's species order
    double* y;              // [nspec][ncell], updated in place
    const double* rk;       // [nrxns][ncell]
    const uint8_t* night;   // [ncell] 1: dark cell (HMAXNIT, H0FAC 1)
    int* cell_stats;        // [ncell][8] (nsteps, ncfail, nefail, npderiv, nsubfun, nnewt, maxord, status) or nullptr
};

template <class M>
__device__ __forceinline__ double* gear_ws(double* ws_all, long long warp_global)
{
    return ws_all + (size_t)warp_global * ((size_t)M::GEAR_WS_ELEMS * 32) + (threadIdx.x & 31);
}

// GRID: one Gear CHEM call on the grid (gather with the SMVGEAR driver's REAL(8)
// concentration floor, grdriver.F:398-459; write-back grdriver.F:577-596).  Otherwise the
// solver-level entry on given concentrations and rate constants.  Persistent grid, cells
// from the work queue q (of a.ncell cells at the solver level).
template <class M, bool GRID>
__global__ void __launch_bounds__(GEAR_WPB * 32, GEAR_WARPS_PER_SM / GEAR_WPB) k_gear(GridArgs a, QueueArgs q, GearArgs g)
{
    const int lane = threadIdx.x & 31;
    const long long warp = (long long)blockIdx.x * GEAR_WPB + (threadIdx.x >> 5);
    double* ws = gear_ws<M>(a.ws, warp);
    const gear::Coef* K = g.coef;
    gear::State s;
    long long cell = -1;
    bool drained = false;
    unsigned long long acc = 0, rej = 0, failed = 0, sunlit = 0, sun_att = 0;
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
                        bool sun;
                        if (GRID) {
                            sun = gather_cell<M>(a, cell, ws, true);
                        } else {
                            for (int i = 0; i < M::NSPEC; ++i)
                                ws[(M::GEAR_CNEW + i) * 32] = g.y[(size_t)i * a.ncell + cell];
                            for (int r = 0; r < M::NRXNS; ++r)
                                ws[(M::OFF_RKI + r) * 32] = g.rk[(size_t)r * a.ncell + cell];
                            sun = g.night[cell] == 0;
                        }
                        gear::start<M, 32, false>(s, ws, sun, K, a.yave != nullptr);
                    }
                }
                drained = __any_sync(0xffffffffu, base + __popc(need) >= queue_len(q, a.ncell));
            }
        }
        bool busy = cell >= 0;
        if (!__any_sync(0xffffffffu, busy)) break;
        if (busy && gear::advance<M, 32, false>(ws, s, K, a.chemstep) == gear::DONE) {
            if (GRID) {
                scatter_cell<M>(a, cell, ws);
                if (a.yave)
                    for (int i = 0; i < M::ISCHAN; ++i)
                        a.yave[(size_t)i * a.ncell + cell] = ws[(M::GEAR_CAVEG + i) * 32];
            } else {
                for (int i = 0; i < M::NSPEC; ++i) g.y[(size_t)i * a.ncell + cell] = ws[(M::GEAR_CNEW + i) * 32];
                if (g.cell_stats) {
                    int* o = g.cell_stats + (size_t)8 * cell;
                    o[0] = s.st.nsteps; o[1] = s.st.ncfail; o[2] = s.st.nefail; o[3] = s.st.npderiv;
                    o[4] = s.st.nsubfun; o[5] = s.st.nnewt; o[6] = s.st.maxord; o[7] = s.st.status;
                }
            }
            const int att = s.st.nsteps + s.st.ncfail + s.st.nefail;
            acc += s.st.nsteps;
            rej += s.st.ncfail + s.st.nefail;
            failed += s.st.status != gear::ST_OK;
            sunlit += s.lsun;
            if (s.lsun) sun_att += att;
            if (a.cell_status) a.cell_status[cell] = s.st.status;
            if (a.cell_steps) a.cell_steps[cell] = att;
            cell = -1;
            busy = false;
        }
        gear::evaluate<M, 32, false>(ws, s, busy);
    }
    if (a.counters) {
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_down_sync(0xffffffffu, acc, o);
            rej += __shfl_down_sync(0xffffffffu, rej, o);
            failed += __shfl_down_sync(0xffffffffu, failed, o);
            sunlit += __shfl_down_sync(0xffffffffu, sunlit, o);
            sun_att += __shfl_down_sync(0xffffffffu, sun_att, o);
        }
        if (lane == 0) {
            atomicAdd(&a.counters[0], acc);
            atomicAdd(&a.counters[1], rej);
            atomicAdd(&a.counters[2], failed);
            atomicAdd(&a.counters[3], sunlit);
            atomicAdd(&a.counters[4], sun_att);
        }
    }
}

// One cell per warp, the cell's workspace in shared memory (GEAR_WS_ELEMS doubles,
// stride 1; dynamic shared memory of that size per one-warp block): the lanes share the
// cell's element-wise work, f evaluation, LU and solves.  SMVGEAR's stiffest cells need
// tens of thousands of Newton iterations in one call, a call lasts as long as its slowest
// cell, and on this GPU one FP64 warp instruction takes 64 cycles whatever its number of
// active lanes, so a lone cell must spread its FP64 work over the lanes to advance.
// Cells come from the work queue; results equal k_gear's bit for bit.
template <class M, bool GRID>
__global__ void __launch_bounds__(32) k_gear_warp(GridArgs a, QueueArgs q, GearArgs g)
{
    extern __shared__ double sm[];
    const int lane = threadIdx.x & 31;
    // lane 0's slot of this warp's global workspace, for the gather (stride 32)
    double* wsg = a.ws + (size_t)blockIdx.x * ((size_t)M::WS_ELEMS * 32);
    const gear::Coef* K = g.coef;
    const unsigned long long qlen = queue_len(q, a.ncell);
    unsigned long long acc = 0, rej = 0, failed = 0, sunlit = 0, sun_att = 0;
    for (;;) {
        unsigned long long pos = 0;
        if (lane == 0) pos = atomicAdd(q.head, 1ull);
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (pos >= qlen) break;
        const long long cell = q.cell0 + (q.order ? q.order[pos] : (long long)pos);
        bool sun;
        if (GRID) {
            int sflag = 0;
            if (lane == 0) sflag = gather_cell<M>(a, cell, wsg, true) ? 1 : 0;
            sun = __shfl_sync(0xffffffffu, sflag, 0) != 0;
            __syncwarp();
            for (int i = lane; i < M::NSPEC; i += 32) sm[M::GEAR_CNEW + i] = wsg[(M::OFF_Y + i) * 32];
            for (int r = lane; r < M::NRXNS; r += 32) sm[M::OFF_RKI + r] = wsg[(M::OFF_RKI + r) * 32];
        } else {
            for (int i = lane; i < M::NSPEC; i += 32) sm[M::GEAR_CNEW + i] = g.y[(size_t)i * a.ncell + cell];
            for (int r = lane; r < M::NRXNS; r += 32) sm[M::OFF_RKI + r] = g.rk[(size_t)r * a.ncell + cell];
            sun = g.night[cell] == 0;
        }
        __syncwarp();
        gear::State s;
        gear::start<M, 1, true>(s, sm, sun, K, GRID && a.yave != nullptr);
        while (gear::advance<M, 1, true>(sm, s, K, a.chemstep) == gear::NEED_F)
            gear::evaluate<M, 1, true>(sm, s, true);
        if (GRID) {   // write-back as scatter_cell
            const double densd = (double)a.dens[cell];
            for (int i = lane; i < M::ISCHAN; i += 32) {
                const int old = M::inew2old(i);
                const double y = sm[M::GEAR_CNEW + i];
                const float v = a.convert[old] ? (float)((a.rev_conv[old] * densd) * y) : (float)y;
                a.cgrid[(size_t)a.cgrid_index[old] * a.ncell + cell] = v;
                if (a.yave) a.yave[(size_t)i * a.ncell + cell] = sm[M::GEAR_CAVEG + i];
            }
        } else {
            for (int i = lane; i < M::NSPEC; i += 32) g.y[(size_t)i * a.ncell + cell] = sm[M::GEAR_CNEW + i];
            if (g.cell_stats && lane == 0) {
                int* o = g.cell_stats + (size_t)8 * cell;
                o[0] = s.st.nsteps; o[1] = s.st.ncfail; o[2] = s.st.nefail; o[3] = s.st.npderiv;
                o[4] = s.st.nsubfun; o[5] = s.st.nnewt; o[6] = s.st.maxord; o[7] = s.st.status;
            }
        }
        __syncwarp();   // the next cell overwrites the shared workspace
        if (lane == 0) {
            const int att = s.st.nsteps + s.st.ncfail + s.st.nefail;
            acc += s.st.nsteps;
            rej += s.st.ncfail + s.st.nefail;
            failed += s.st.status != gear::ST_OK;
            sunlit += s.lsun;
            if (s.lsun) sun_att += att;
            if (a.cell_status) a.cell_status[cell] = s.st.status;
            if (a.cell_steps) a.cell_steps[cell] = att;
        }
    }
    if (a.counters && lane == 0) {
        atomicAdd(&a.counters[0], acc);
        atomicAdd(&a.counters[1], rej);
        atomicAdd(&a.counters[2], failed);
        atomicAdd(&a.counters[3], sunlit);
        atomicAdd(&a.counters[4], sun_att);
    }
}

}  // namespace chem
#endif  // GEAR_CELL_ONLY
