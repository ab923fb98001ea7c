// KMT2 aqueous cloud chemistry: the kinetic core of AQCHEM (CCTM/src/cloud/acm_ae7_kmt2)
// for one cloudy cell, as host/device code.
//
//   set-up      aqchem_kmt.F90:371-396, 511 (Henry's law constants, cloud thickness) and
//               aqchem_Initialize.F90:252-288, 425-485, 491-636 (units, tolerances, fixed
//               species, pH by charge balance, the rate constants set once)
//   rates       aqchem_Rates.F90:146-362 (DISF, DISB, KRXN, KIEPOX), :415-581
//               (Update_RCONST: ionic strength, activity coefficients), refreshed from the
//               accepted state before every step, as the reference's Fun / Jac templates
//               do (aqchem_Integrator.F90:1318-1388: Update_RCONST reads the module's VAR,
//               which is the integrator's Y)
//   f, J, LU    generated straight-line Fun, Jac_SP, KppDecomp, KppSolve (gen/kmt2_aq.cuh)
//   integrator  KPP Rosenbrock with Rodas3, autonomous, vector tolerances and the
//               reference's defaults (aqchem_Integrator.F90:79-132, 300-425, 485-831,
//               1070-1134); AQCHEM's DO WHILE (T < TEND) loop (aqchem_kmt.F90:530-543)
//               with at most 16 passes
//
// The same operations in the same order as the reference's Fortran (REAL(4) literals
// and REAL(4) intermediates kept, no contraction of a*b+c: the library is compiled with
// -fmad=false), with exp and x**y by portable series routines (kq_exp, kq_pow) that
// give the same bits on the host and on the device.  One cell's arrays live in a
// lane-interleaved FP64 workspace (element i of a lane at ws[i * KQ_S]); inputs and
// outputs are [element][cell] with stride n.  The header compiles as plain C++ too, so
// the host can run exactly this code.
#pragma once

#include <float.h>
#include <math.h>

#ifdef __CUDACC__
#define KQ_HD __host__ __device__
#define KQ_NOINLINE __noinline__
#else
#define KQ_HD
#define KQ_NOINLINE
#endif

namespace kmt2 {

#include "gen/kmt2_aq_consts.cuh"

// The workspace holds a warp's 32 lanes side by side: element i of a lane at ws[i * KQ_S]
// (ws pointing at the lane's first element), so a warp's access to one element reads 256
// consecutive bytes and every offset is a constant.
constexpr long long KQ_S = 32;

// per-cell parameters, [KQ_NPARAM][ncell] (include/cmaqchem.h: CMAQCHEM_KMT2_*)
enum { P_TEMP2 = 0, P_PRES_PA, P_TAUCLD, P_PRCRATE, P_WCAVG, P_WTAVG, P_AIRM, P_ALFA0, P_ALFA3, P_COSZEN,
       P_JH2O2, P_HO, P_ISPC8, P_MTPYRAC, P_PHOTO, NPARAM };
// per-cell statistics, [NSTAT][ncell]
enum { S_NSTP = 0, S_NACC, S_NREJ, S_NFUN, S_NJAC, S_NDEC, S_NSOL, S_NSNG, S_IERR, S_NKRON, NSTAT };
// workspace layout of one lane (elements): Y, YNEW, FCN0, K1-K4, JAC0, GHIMJ, the rates, FIX
constexpr int W_Y = 0, W_YNEW = NVAR, W_FCN0 = 2 * NVAR, W_K = 3 * NVAR, W_JAC0 = 7 * NVAR,
              W_GHIMJ = W_JAC0 + LU_NONZERO, W_R = W_GHIMJ + LU_NONZERO, W_F = W_R + NREACT, WS_ELEMS = W_F + NFIX;

struct Cell {   // aqchem_Global of one cell
    double temp_kpp, press, lwc, lwcfrac, delinvt, phi2, invphi2, ddiam;
    double czen, photo, jh2o2, alfa3, alfa0, wetfac, cfactor, tend, dt;
    double stion, gm1, gm2;
    int ispc8, mtpyrac;
    double henry[NHENRY];
};

// ----------------------------------------------------------------------------- portable exp and pow
// Every exp and x**y of the kinetic core goes through these two routines, on the host
// and on the device alike, so that the GPU reproduces the oracle bit for bit (CUDA's
// double exp and pow differ from libm's by ulps, and Rodas3's accept / reject decisions
// amplify one ulp in a rate constant to 1e-5 in the final state).

// exp(t) by t = n ln2 + r (Cody-Waite split of ln 2, |r| <= ln2/2) and a Taylor series to
// r^13, with IEEE operations, fma, rint and ldexp only: the same bits on host and device.
KQ_HD inline double kq_exp(double t)
{
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    if (t > 709.0) return INFINITY;
    if (t < -745.0) return 0.0;
    const double n = rint(t * 0x1.71547652b82fep+0);
    const double r = fma(-n, ln2_lo, fma(-n, ln2_hi, t));
    double e = 0x1.6124613a86d09p-33;
    e = fma(e, r, 0x1.1eed8eff8d898p-29);
    e = fma(e, r, 0x1.ae64567f544e4p-26);
    e = fma(e, r, 0x1.27e4fb7789f5cp-22);
    e = fma(e, r, 0x1.71de3a556c734p-19);
    e = fma(e, r, 0x1.a01a01a01a01ap-16);
    e = fma(e, r, 0x1.a01a01a01a01ap-13);
    e = fma(e, r, 0x1.6c16c16c16c17p-10);
    e = fma(e, r, 0x1.1111111111111p-7);
    e = fma(e, r, 0x1.5555555555555p-5);
    e = fma(e, r, 0x1.5555555555555p-3);
    e = fma(e, r, 0.5);
    e = fma(e, r, 1.0);
    e = fma(e, r, 1.0);
    return ldexp(e, (int)n);
}

// x**y for x >= 0, y > 0 from series with IEEE +, -, *, /, fma, frexp/ldexp and rint only,
// identical on host and device (the routine of the Gear kernels, gear.cuh: gpow; libm
// and CUDA pow differ by ulps, which move step-size decisions): log by 2 atanh(s) to
// s^23 after x = m 2^k, exp by Taylor to r^13 after a Cody-Waite reduction by ln 2.
KQ_HD inline double kq_pow(double x, double y)
{
    if (!(x > 0.0)) return x == 0.0 ? 0.0 : x;
    if (isinf(x)) return x;
    int k;
    double m = frexp(x, &k);
    if (m < 0x1.6a09e667f3bcdp-1) {
        m = m * 2.0;
        k = k - 1;
    }
    const double u = (m - 1.0) / (m + 1.0);
    const double z = u * u;
    double p = 0x1.642c8590b2164p-5;
    p = fma(p, z, 0x1.8618618618618p-5);
    p = fma(p, z, 0x1.af286bca1af28p-5);
    p = fma(p, z, 0x1.e1e1e1e1e1e1ep-5);
    p = fma(p, z, 0x1.1111111111111p-4);
    p = fma(p, z, 0x1.3b13b13b13b14p-4);
    p = fma(p, z, 0x1.745d1745d1746p-4);
    p = fma(p, z, 0x1.c71c71c71c71cp-4);
    p = fma(p, z, 0x1.2492492492492p-3);
    p = fma(p, z, 0x1.999999999999ap-3);
    p = fma(p, z, 0x1.5555555555555p-2);
    p = fma(p, z, 1.0);
    const double ln2_hi = 0x1.62e42fee00000p-1, ln2_lo = 0x1.a39ef35793c76p-33;
    const double lx = fma((double)k, ln2_hi, fma((double)k, ln2_lo, (2.0 * u) * p));
    return kq_exp(y * lx);
}

// x**y of the rate laws (metal inhibition, activity coefficients): the portable pow, NaN
// for x < 0 as Fortran's real power of a negative base gives
KQ_HD inline double kq_rpow(double x, double y)
{
    return x < 0.0 ? NAN : kq_pow(x, y);
}

// ----------------------------------------------------------------------------- rate laws

// Schwartz (1986) mass-transfer coefficient of KMTF / KMTB (aqchem_Initialize.F90:53-104);
// PI is a REAL(4) literal there
KQ_HD inline double kq_kmt(const Cell& c, double accom, double dg, double mw)
{
    const double rad = c.ddiam * 0.5;
    const double v = sqrt(8.0 * 8.3145 * c.temp_kpp * 1000.0 / (double)3.1415926536f / mw);
    double kmt = (rad * rad) / (3.0 * dg);
    kmt = kmt + (4.0 * rad / (3.0 * v * accom));
    return 1.0 / kmt;
}
KQ_HD inline double kq_kmtf(const Cell& c, double accom, double dg, double mw)
{
    return kq_kmt(c, accom, dg, mw) * c.lwc / 1000.0;
}
KQ_HD inline double kq_kmtb(const Cell& c, double hl, double accom, double dg, double mw)
{
    return kq_kmt(c, accom, dg, mw) / (0.08206 * c.temp_kpp * hl);
}
// aqchem_Initialize.F90:106-117
KQ_HD inline double kq_hydf(const Cell& c, double kf, double dh)
{
    const double k = kf * kq_exp(dh * c.delinvt);
    return k * c.phi2;
}
// aqchem_Initialize.F90:132-152 (a negative J: the COSZEN estimate scaled by PHOTO)
KQ_HD inline double kq_kphot(const Cell& c, double maxc, double jval)
{
    if (!(jval < 0.0)) return jval;
    return c.czen > 0.001 ? c.photo * 2.718281828 * maxc * kq_exp(-1.0 / c.czen) : 0.0;
}
// aqchem_Rates.F90:146-158
KQ_HD inline double kq_disf(const Cell& c, double keq, double dh, double kb, int g1)
{
    const double k = kb * (keq * kq_exp(dh * c.delinvt));
    return g1 == 1 ? k * c.gm1 : k;
}
// aqchem_Rates.F90:160-174
KQ_HD inline double kq_disb(const Cell& c, double kb, int g1)
{
    double k = kb;
    if (g1 == 1) k = k * c.gm1 * c.gm2;
    else if (g1 == 2) k = k * c.gm1 * c.gm1;
    return k * c.phi2;
}
// Q of the aqueous diffusion limitation for a first-order rate krate (aqchem_Rates.F90:
// 225-242, 300-316, 338-354)
KQ_HD inline double kq_diffusion_factor(const Cell& c, double krate)
{
    const double q1 = krate < 0.0 ? 0.0 : c.ddiam / 2.0 * sqrt(krate / 1.0e-9);
    if (!(q1 > 1.0e-3)) return 1.0;
    if (q1 > 100.0) return 3.0 / q1;
    const double e2 = kq_exp(2.0 * q1);
    const double coth = (e2 + 1.0) / (e2 - 1.0);
    const double q = 3.0 * ((coth / q1) - (1.0 / (q1 * q1)));
    return q > 1.0 ? 1.0 : q;
}
// aqchem_Rates.F90:176-249
KQ_HD inline double kq_krxn(const Cell& c, const double* v, double kr, double dh, int rtype, int qy,
                            int metal)
{
    const double phi2 = c.phi2;
    double k = kr * kq_exp(dh * c.delinvt);
    if (rtype == 1) k = (k / (1.0 + 13.0 * v[L_HPLUS * KQ_S] * phi2)) * phi2;
    else if (rtype == 3) k = k * phi2;
    else if (rtype == 4) k = k / phi2;
    if (metal > 0) {
        const double s6 = (v[L_H2SO4 * KQ_S] + v[L_HSO4MIN * KQ_S] + v[L_SO4MIN2 * KQ_S]) * phi2;
        k = k / (1.0 + 75.0 * kq_rpow(s6, 0.67));
    }
    if (qy >= 1) {
        const double k1 = 2.4e+4 * kq_exp(0.0 * c.delinvt);
        const double k2 = 3.7e+5 * kq_exp(-5530.88 * c.delinvt);
        const double k3 = 1.5e+9 * kq_exp(-5280.56 * c.delinvt);
        const double kt = (k1 * v[L_SO2 * KQ_S] + k2 * v[L_HSO3MIN * KQ_S] + k3 * v[L_SO3MIN2 * KQ_S]) * phi2;
        k = k * kq_diffusion_factor(c, kt);
    }
    return k * phi2;
}
// aqchem_Rates.F90:251-362
KQ_HD inline double kq_kiepox(const Cell& c, const double* v, const double* f, double kh, double khso4,
                              int type)
{
    const double phi2 = c.phi2;
    if (c.ispc8 <= 0 ? type > 0 : type < 1) return 0.0;
    const double h = v[L_HPLUS * KQ_S], hso4 = v[L_HSO4MIN * KQ_S], so4 = v[L_SO4MIN2 * KQ_S];
    double kiepox = kh * h * phi2 + khso4 * hso4 * phi2;
    double kt = (9.0e-4 * h * phi2 + 1.31e-5 * hso4 * phi2) * f[L_H2O * KQ_S] * phi2;
    if (type <= 1) {
        kt = kt + (8.83e-3 * h * phi2 + 2.92e-6 * hso4 * phi2) * so4 * phi2;
        const double kn = 2.0e-4 * h * phi2 + 2.92e-6 * hso4 * phi2;
        if (c.ispc8 <= 0) {
            kt = kt + kn * v[L_NO3MIN * KQ_S] * phi2;
        } else {
            kt = kt + kn * v[L_IETET * KQ_S] * phi2;
            kt = kt + kn * v[L_IEOS * KQ_S] * phi2;
        }
    } else {
        kt = kt + (2.0e-4 * h * phi2 + 2.92e-6 * hso4 * phi2) * so4 * phi2;
    }
    kiepox = kiepox * kq_diffusion_factor(c, kt);
    return kiepox * phi2;
}

// ionic strength and activity coefficients (aqchem_Rates.F90:423-452), terms in the
// reference's order (L_HMSMIN twice, as there)
KQ_HD KQ_NOINLINE void kq_ionic(Cell& c, const double* v)
{
#define V(n) v[(n) * KQ_S]
    const double sum = V(L_HPLUS) + V(L_NH4PLUS) + V(L_OHMIN) + V(L_HCO3MIN) + V(L_O2MIN) + V(L_NO2MIN)
                     + V(L_NO4MIN) + V(L_GLYACMIN) + V(L_OXLACMIN) + V(L_PYRACMIN) + V(L_GCOLACMIN) + V(L_CCOOHMIN)
                     + V(L_HSO3MIN) + V(L_HCOOMIN) + V(L_NO3MIN) + V(L_HSO4MIN) + V(L_HMSMIN) + V(L_NAPLUS)
                     + V(L_KPLUS) + V(L_CLMIN) + V(L_SO4MIN) + V(L_SO3MIN) + V(L_HMSMIN) + V(L_SO5MIN)
                     + V(L_HSO5MIN) + V(L_CO2MIN) + 3.0 * V(L_FEPLUS3) + 2.0 * V(L_MNPLUS2)
                     + 4.0 * (V(L_SO4MIN2) + V(L_CO3MIN2) + V(L_OXLACMIN2) + V(L_SO3MIN2) + V(L_MNPLUS2)
                              + V(L_CAPLUS2) + V(L_MGPLUS2))
                     + 9.0 * V(L_FEPLUS3);
#undef V
    c.stion = 0.5 * sum * c.phi2;
    const double lg1 = -0.509 * (sqrt(c.stion) / (1.0 + sqrt(c.stion)) - 0.2 * c.stion);
    c.gm1 = kq_rpow(10.0, lg1);
    const double gm2 = kq_rpow(10.0, lg1 * 4.0);
    c.gm2 = gm2 > 1.0e-30 ? gm2 : 1.0e-30;
}

// HLCONST with EFFECTIVE = .FALSE. (hlconst.F:509-511), REAL(4) throughout; its EXP is
// kq_exp rounded to float (libm's and CUDA's expf differ by up to 2 float ulps, 1e-7
// relative, which would move the gas / aqueous partitioning by as much)
KQ_HD inline float kq_hlconst(float a, float e, float temp)
{
    const float tfac = (298.0f - temp) / (298.0f * temp);
    return a * (float)kq_exp((double)(e * tfac));
}

#include "gen/kmt2_aq.cuh"

// ----------------------------------------------------------------------------- set-up
// AQCHEM before the integration; y, f, r are the lane's workspace arrays, vmix (stride vn)
// the KPP state as Initialize maps it, ho the gas-phase OH.  Returns 0, or -1 for the
// reference's MET DATA ERROR (aqchem_kmt.F90:427-431), -2 for its initial pH error
// (aqchem_Initialize.F90:476-481).
KQ_HD KQ_NOINLINE int kq_setup(Cell& c, const double* p, long long n, const double* vmix, long long vn, double ho,
                               double* y, double* f, double* r)
{
    const float temp2 = (float)p[P_TEMP2 * n], pres_pa = (float)p[P_PRES_PA * n];
    const float taucld = (float)p[P_TAUCLD * n], prcrate = (float)p[P_PRCRATE * n];
    const float wcavg = (float)p[P_WCAVG * n], wtavg = (float)p[P_WTAVG * n], airm = (float)p[P_AIRM * n];
    if (temp2 <= 0.0f || airm <= 0.0f || pres_pa <= 0.0f) return -1;
    kq_henry(c, temp2);
    c.jh2o2 = p[P_JH2O2 * n];
    c.ispc8 = (int)p[P_ISPC8 * n];
    c.mtpyrac = (int)p[P_MTPYRAC * n];
    c.photo = p[P_PHOTO * n];
    const double cthk1 = (double)(airm * temp2) * 0.08206 / ((double)pres_pa / 101325.0 * 1000.0);
    c.dt = (double)taucld;
    c.tend = 0.0 + c.dt;
    c.ddiam = 1.6e-5;
    c.temp_kpp = (double)temp2;
    c.press = (double)pres_pa / 101325.0;
    c.lwc = (double)wcavg;
    c.lwcfrac = c.lwc * 1.0e-3;
    c.delinvt = (298.0 - c.temp_kpp) / (298.0 * c.temp_kpp);
    const double prc = (double)prcrate > 1.0e-20 ? (double)prcrate : 1.0e-20;
    const double twash = (double)wtavg * 1000.0 * cthk1 * 3600.0 / (1000.0 * prc);
    c.wetfac = prcrate > 0.0f ? 1.0 / twash : 0.0;
    c.alfa3 = (double)(float)p[P_ALFA3 * n];
    c.alfa0 = (double)(float)p[P_ALFA0 * n];
    c.phi2 = 1000.0 / 6.022e23 / c.lwcfrac;
    c.invphi2 = 1.0 / c.phi2;
    c.czen = (double)(float)p[P_COSZEN * n];
    c.cfactor = (double)pres_pa / (c.temp_kpp * (double)8.314510f) * 6.0221413e17;
    for (int i = 0; i < NVAR; ++i) y[i * KQ_S] = c.cfactor * vmix[i * vn];
    for (int i = 0; i < NFIX; ++i) f[i * KQ_S] = c.cfactor * 0.0;
    f[L_H2O * KQ_S] = 55.5 * c.invphi2;
    f[G_HO * KQ_S] = ho * c.cfactor;
    f[L_O2 * KQ_S] = (double)0.21f * c.press * 1.3e-3 * kq_exp(1500.0 * c.delinvt) * c.invphi2;
    const double kw = 1.00e-14 * kq_exp(-6.955e+03 * c.delinvt);
    double pos = 2.0 * (y[L_CAPLUS2 * KQ_S] + y[L_MGPLUS2 * KQ_S]) + y[L_NAPLUS * KQ_S] + y[L_KPLUS * KQ_S] + y[L_NH4PLUS * KQ_S];
    double neg = 2.0 * (y[L_SO4MIN2 * KQ_S] + y[L_OXLACMIN2 * KQ_S]) + y[L_NO3MIN * KQ_S] + y[L_CLMIN * KQ_S];
    pos = pos * c.phi2;
    neg = neg * c.phi2;
    const double chg = pos - neg;
    const double oh = (chg + sqrt(chg * chg + 4.0 * kw)) * 0.5;
    if (!(oh > 0.0)) return -2;
    y[L_OHMIN * KQ_S] = oh * c.invphi2;
    y[L_HPLUS * KQ_S] = (kw / oh) * c.invphi2;
    kq_rates_once(c, y, f, r);
    return 0;
}

// ros_ErrorNorm (aqchem_Integrator.F90:694-724) of Rodas3's error estimate, which is K4
// (E = 0, 0, 0, 1: YERR = 0 + 1 * K4)
KQ_HD inline double kq_error_norm(const double* y, const double* ynew, const double* k4)
{
    double err = 0.0;
    for (int i = 0; i < NVAR; ++i) {
        const double ymax = fmax(fabs(y[i * KQ_S]), fabs(ynew[i * KQ_S]));
        const double q = (0.0 + k4[i * KQ_S]) / (kq_atol(i) + kq_rtol(i) * ymax);
        err = err + q * q;
    }
    err = sqrt(err / (double)NVAR);
    return err > 1.0e-10 ? err : 1.0e-10;
}

// AQCHEM's integration loop (aqchem_kmt.F90:529-543: INTEGRATE called while T < TEND, at
// most 16 times) around KPP's ros_Integrator with Rodas3 (aqchem_Integrator.F90:485-690,
// 1070-1134), unrolled into one Rodas3 attempt per call of kq_advance.  A lane keeps its
// cell's loop variables in a Lane between calls, so that a warp's lanes can each be at a
// different step of a different cell and a lane whose cell ends takes the next one; the
// operations of a cell, and their order, are those of the two nested loops.  Rodas3's four
// stages are written out with its coefficients (A = 2, 0, 2, 0, 1; C = 4, 1, -1, 1, -1,
// -8/3; M = 2, 0, 1, 1; E = 0, 0, 0, 1; gamma_1 = 1/2; new f at stages 3 and 4).
enum { KL_PASS = 0, KL_STEP, KL_ATTEMPT, KL_DONE };
struct Lane {
    double tc;                       // AQCHEM's T: where the next INTEGRATE call starts
    double t, tend, hmax, h, texit;  // ros_Integrator's T, Tend, Hmax, H and the last accepted T
    long long nstp, nacc;            // its step counters (per INTEGRATE call)
    int phase, ierr;
    bool reject_last, reject_more;
};

// A cell's kinetic core is kq_begin, then kq_advance until it returns true; the state stays
// in the workspace (Y, F).
//
// kq_begin: statistics cleared, the set-up, the first INTEGRATE call pending.  A failed set-up
// (-1, -2) leaves the lane done with IERR -101 / -102.  Returns the set-up's status.
KQ_HD inline int kq_begin(Cell& c, Lane& L, const double* p, long long n, const double* vmix, long long vn, double ho,
                          double* ws, long long* st)
{
    for (int i = 0; i < NSTAT; ++i) st[i] = 0;
    const int e = kq_setup(c, p, n, vmix, vn, ho, ws + W_Y * KQ_S, ws + W_F * KQ_S, ws + W_R * KQ_S);
    L.tc = 0.0;
    L.ierr = e != 0 ? e - 100 : 1;
    L.phase = e != 0 ? KL_DONE : KL_PASS;
    return e;
}

// the return of an INTEGRATE call with status ierr: AQCHEM's T becomes the last accepted time,
// and a call that failed without an accepted step ends the loop
KQ_HD inline void kq_return(Lane& L, int ierr)
{
    L.ierr = ierr;
    L.tc = L.texit;
    L.phase = (ierr < 0 && L.texit <= 0.0) ? KL_DONE : KL_PASS;
}

// The phases of one pass of a lane, in order: kq_next (the INTEGRATE calls' and steps'
// transitions up to the next attempt: a new step's rates, f and J), kq_prepare (ros_
// PrepareMatrix), kq_stages12, kq_stage3f, kq_stage3s, kq_stage4f, kq_stage4s (Rodas3's
// stages, solves apart from the f evaluations so that each phase runs one routine) and
// kq_decide (error norm, accept or reject).  A kernel may put a block barrier between
// phases, so that its warps run the same routine at the same time; kq_advance runs them
// back to back.  Rodas3's stages, each vector formed in one pass (ros_Integrator's stage
// loop and WAXPY calls, a zero multiplier skipped as WAXPY does): K1 = FCN0; K2 = FCN0 +
// (4/h) K1; YNEW = Y + 2 K1 -> K3 = f(YNEW) + (1/h) K1 - (1/h) K2; YNEW + K3 -> K4 =
// f(YNEW) + (1/h) K1 - (1/h) K2 - (8/3/h) K3; YNEW + K4 is the new state (M = 2, 0, 1, 1:
// stage 4's Y + 2 K1 + K3 is stage 3's YNEW + K3, bit for bit).

// Moves the lane to its next attempt.  Returns true when the cell is finished: L.ierr is
// IERR (1 = success, -6 / -7 / -8 from ros_Integrator, -100 for 16 calls, -101 / -102 for a
// failed set-up), also in st[S_IERR].  Each pass of the loop moves the lane on by one
// phase, at most 16 INTEGRATE calls.
KQ_HD inline bool kq_next(Cell& c, Lane& L, double* ws, long long* st)
{
    double* y = ws + W_Y * KQ_S;
    const double roundoff = DBL_EPSILON;
    for (;;) {
        if (L.phase == KL_DONE) {
            st[S_IERR] = L.ierr;
            return true;
        }
        if (L.phase == KL_ATTEMPT) return false;
        if (L.phase == KL_PASS) {        // AQCHEM's loop head, then ros_Integrator's entry
            if (!(L.tc < c.tend)) {
                L.phase = KL_DONE;
                continue;
            }
            if (st[S_NKRON] >= 16) {
                L.ierr = -100;
                L.phase = KL_DONE;
                continue;
            }
            st[S_NKRON]++;
            const double tstart = L.tc;
            L.tend = tstart + c.dt;
            L.hmax = fabs(L.tend - tstart);
            L.nstp = L.nacc = 0;
            L.t = tstart;
            L.h = fmin(1.0e-5, L.hmax);
            L.texit = 0.0;
            if (fabs(L.h) <= 10.0 * roundoff) L.h = 1.0e-5;
            L.reject_last = L.reject_more = false;
            L.phase = KL_STEP;
        }
        // KL_STEP: a new step, rates, f and J at the accepted state
        if (!(fabs(L.t - L.tend) >= roundoff)) {
            kq_return(L, 1);
            continue;
        }
        if (L.nstp > 200000) {
            kq_return(L, -6);
            continue;
        }
        if ((L.t + 0.1 * L.h) == L.t || L.h <= roundoff) {
            kq_return(L, -7);
            continue;
        }
        L.h = fmin(L.h, fabs(L.tend - L.t));
        double* r = ws + W_R * KQ_S;
        const double* f = ws + W_F * KQ_S;
        kq_ionic(c, y);
        kq_rates_update(c, y, f, r);
        kqu_fun(y, f, r, ws + W_FCN0 * KQ_S);
        st[S_NFUN]++;
        kqu_jac(y, f, r, ws + W_JAC0 * KQ_S);
        st[S_NJAC]++;
        L.phase = KL_ATTEMPT;
        return false;
    }
}

// ros_PrepareMatrix: GHIMJ = 1/(h gamma) - JAC0 factorised, h halved after a singular
// factorisation; after 5 halvings the INTEGRATE call returns -8 and this returns false
// (the lane's next pass starts at kq_next)
KQ_HD inline bool kq_prepare(Lane& L, double* ws, long long* st)
{
    const double* jac0 = ws + W_JAC0 * KQ_S;
    double* ghimj = ws + W_GHIMJ * KQ_S;
    int nsing = 0;
    for (;;) {
        for (int i = 0; i < LU_NONZERO; ++i) ghimj[i * KQ_S] = -jac0[i * KQ_S];
        const double ghinv = 1.0 / (L.h * 0.5);
        kq_add_diagonal(ghimj, ghinv);
        const int ising = kqu_decomp(ghimj);
        st[S_NDEC]++;
        if (ising == 0) return true;
        st[S_NSNG]++;
        if (++nsing > 5) {
            kq_return(L, -8);
            return false;
        }
        L.h = L.h * 0.5;
    }
}

// stages 1 and 2: K1, K2 and stage 3's YNEW
KQ_HD inline void kq_stages12(const Lane& L, double* ws)
{
    const double* y = ws + W_Y * KQ_S;
    double* ynew = ws + W_YNEW * KQ_S;
    const double* fcn0 = ws + W_FCN0 * KQ_S;
    double* k1 = ws + W_K * KQ_S;
    double* k2 = k1 + NVAR * KQ_S;
    const double* ghimj = ws + W_GHIMJ * KQ_S;
    const double c21 = 4.0 / L.h;
    for (int i = 0; i < NVAR; ++i) k1[i * KQ_S] = fcn0[i * KQ_S];
    kqu_solve(ghimj, k1);
    for (int i = 0; i < NVAR; ++i) {
        double t = fcn0[i * KQ_S];
        if (c21 != 0.0) t = t + c21 * k1[i * KQ_S];
        k2[i * KQ_S] = t;
    }
    kqu_solve(ghimj, k2);
    for (int i = 0; i < NVAR; ++i) ynew[i * KQ_S] = y[i * KQ_S] + 2.0 * k1[i * KQ_S];
}

// stage 3 (k = 3) or 4 (k = 4): f(YNEW) into Kk
KQ_HD inline void kq_stage_f(double* ws, int k, long long* st)
{
    const double* r = ws + W_R * KQ_S;
    const double* f = ws + W_F * KQ_S;
    kqu_fun(ws + W_YNEW * KQ_S, f, r, ws + (W_K + (k - 1) * NVAR) * KQ_S);
    st[S_NFUN]++;
}

// stage 3's K3 from f(YNEW), solved, and stage 4's YNEW
KQ_HD inline void kq_stage3s(const Lane& L, double* ws)
{
    double* ynew = ws + W_YNEW * KQ_S;
    const double* k1 = ws + W_K * KQ_S;
    const double* k2 = k1 + NVAR * KQ_S;
    double* k3 = ws + (W_K + 2 * NVAR) * KQ_S;
    const double c31 = 1.0 / L.h, c32 = -1.0 / L.h;
    for (int i = 0; i < NVAR; ++i) {
        double t = k3[i * KQ_S];
        if (c31 != 0.0) t = t + c31 * k1[i * KQ_S];
        if (c32 != 0.0) t = t + c32 * k2[i * KQ_S];
        k3[i * KQ_S] = t;
    }
    kqu_solve(ws + W_GHIMJ * KQ_S, k3);
    for (int i = 0; i < NVAR; ++i) ynew[i * KQ_S] = ynew[i * KQ_S] + k3[i * KQ_S];
}

// stage 4's K4 from f(YNEW), solved, and the new state
KQ_HD inline void kq_stage4s(const Lane& L, double* ws, long long* st)
{
    double* ynew = ws + W_YNEW * KQ_S;
    const double* k1 = ws + W_K * KQ_S;
    const double* k2 = k1 + NVAR * KQ_S;
    const double* k3 = k2 + NVAR * KQ_S;
    double* k4 = ws + (W_K + 3 * NVAR) * KQ_S;
    const double c31 = 1.0 / L.h, c32 = -1.0 / L.h, c43 = -(8.0 / 3.0) / L.h;
    for (int i = 0; i < NVAR; ++i) {
        double t = k4[i * KQ_S];
        if (c31 != 0.0) t = t + c31 * k1[i * KQ_S];
        if (c32 != 0.0) t = t + c32 * k2[i * KQ_S];
        if (c43 != 0.0) t = t + c43 * k3[i * KQ_S];
        k4[i * KQ_S] = t;
    }
    kqu_solve(ws + W_GHIMJ * KQ_S, k4);
    st[S_NSOL] += 4;
    for (int i = 0; i < NVAR; ++i) ynew[i * KQ_S] = ynew[i * KQ_S] + k4[i * KQ_S];
}

// the error norm and ros_Integrator's accept / reject decision (Hmin = 0)
KQ_HD inline void kq_decide(Lane& L, double* ws, long long* st)
{
    double* y = ws + W_Y * KQ_S;
    const double* ynew = ws + W_YNEW * KQ_S;
    const double h = L.h;
    const double err = kq_error_norm(y, ynew, ws + (W_K + 3 * NVAR) * KQ_S);
    double hnew = h * fmin(6.0, fmax(0.2, 0.9 / kq_pow(err, 1.0 / 3.0)));
    L.nstp++;
    st[S_NSTP]++;
    if (err <= 1.0) {                    // accept
        L.nacc++;
        st[S_NACC]++;
        for (int i = 0; i < NVAR; ++i) y[i * KQ_S] = ynew[i * KQ_S];
        L.t = L.t + h;
        hnew = fmax(0.0, fmin(hnew, L.hmax));
        if (L.reject_last) hnew = fmin(hnew, h);
        L.texit = L.t;
        L.reject_last = L.reject_more = false;
        L.h = hnew;
        L.phase = KL_STEP;
        return;
    }
    if (L.reject_more) hnew = h * 0.1;   // reject: the next attempt reuses f and J
    L.reject_more = L.reject_last;
    L.reject_last = true;
    L.h = hnew;
    if (L.nacc >= 1) st[S_NREJ]++;
}

// Runs the cell up to the end of its next Rodas3 attempt (the phases back to back).
// Returns true when the cell is finished (as kq_next).
KQ_HD inline bool kq_advance(Cell& c, Lane& L, double* ws, long long* st)
{
    for (;;) {
        if (kq_next(c, L, ws, st)) return true;
        if (!kq_prepare(L, ws, st)) continue;
        kq_stages12(L, ws);
        kq_stage_f(ws, 3, st);
        kq_stage3s(L, ws);
        kq_stage_f(ws, 4, st);
        kq_stage4s(L, ws, st);
        kq_decide(L, ws, st);
        return false;
    }
}

// ----------------------------------------------------------------------------- the whole AQCHEM
// AQCHEM's GAS array in AQ_DATA.F's srggas order (29 species, mol/molV)
enum { KG_SO2 = 0, KG_HNO3, KG_N2O5, KG_CO2, KG_NH3, KG_H2O2, KG_O3, KG_FOA, KG_MHP, KG_PAA, KG_H2SO4, KG_HCL,
       KG_GLY, KG_MGLY, KG_HO, KG_IEPOX, KG_IMAE, KG_IHMML, KG_HO2, KG_NO2, KG_HONO, KG_HNO4, KG_GCOL, KG_CCOOH,
       KG_HCHO, KG_NO3RAD, KG_CH3O2, KG_HCHOP, KG_PYRUV, KG_NGAS };
// positions (in the caller's AEROSOL(NAER, NMODES) list) of the surrogates AQCHEM reads or
// writes: AQ_DATA.F's LSO4, LNH4, ...; element (i, mode) is aer[(i + naer * mode) * n]
enum { KA_SO4 = 0, KA_NH4, KA_NO3, KA_CL, KA_NA, KA_EC, KA_POA, KA_PRI, KA_SOA, KA_NUM, KA_SOILC, KA_SEASC,
       KA_ANTHC, KA_CAACC, KA_MGACC, KA_KACC, KA_FEACC, KA_MNACC, KA_ORGC, KA_TRACER_AKN, KA_TRACER_ACC,
       KA_TRACER_COR, KA_PHG_AKN, KA_PHG_ACC, KA_PHG_COR, KA_IETET, KA_IEOS, KA_DIMER, KA_IMGA, KA_IMOS,
       KA_ISO3, KA_NIDX };
enum { KM_AKN = 0, KM_ACC, KM_COR };
// coarse crustal factors of aqchem_kmt.F90:329-365 (computed once by the caller)
enum { KF_SOIL_FE = 0, KF_CORS_FE, KF_SOIL_MN, KF_CORS_MN, KF_SEAS_NA, KF_SOIL_NA, KF_CORS_NA, KF_SEAS_MG,
       KF_SOIL_MG, KF_CORS_MG, KF_SEAS_CA, KF_SOIL_CA, KF_CORS_CA, KF_SEAS_K, KF_SOIL_K, KF_CORS_K, KF_N };
// per-cell scalar outputs: HPWDEP, BETASO4, FRACTR, FRACPOA, FRACPRI, FRACSOA and the four
// mass-balance percentages AQCHEM checks (S, N without NH3, NH3 / NH4, Cl)
enum { KO_HPWDEP = 0, KO_BETASO4, KO_FRACTR, KO_FRACPOA, KO_FRACPRI, KO_FRACSOA, KO_MBAL, KO_N = KO_MBAL + 4 };

// REAL(4) EXP of the redistribution (EXP of a REAL product): the portable exp rounded to float
KQ_HD inline double kq_fexp(float x) { return (double)(float)kq_exp((double)x); }

#define AER(k, m) aer[(long long)(ai[k] + naer * (m)) * n]
#define AWD(k, m) awd[(long long)(ai[k] + naer * (m)) * n]

// Initialize's mapping of AQCHEM's GAS / AEROSOL into the KPP state in mol/molV
// (aqchem_Initialize.F90:290-421), into the workspace's YNEW, which the set-up reads
KQ_HD inline void kq_aq_map(const double* p, const double* gas, const double* aer, int naer, const int* ai,
                            const double* fac, long long n, double* ws)
{
    const float coszen = (float)p[P_COSZEN * n];
    const int ispc8 = (int)p[P_ISPC8 * n], mtpyrac = (int)p[P_MTPYRAC * n];
    const int dark = coszen <= 0.0f;
    const double fe_iii = dark ? 0.9 : 0.1, mn_ii = 1.0, fe_sol = 0.1, mn_sol = 0.5;
    double* v = ws + W_YNEW * KQ_S;   // Initialize's VAR before the unit conversion
    for (int i = 0; i < NVAR; ++i) v[i * KQ_S] = 0.0;
    v[G_SO2 * KQ_S] = gas[KG_SO2 * n];
    v[G_HNO3 * KQ_S] = gas[KG_HNO3 * n] + 2.0 * gas[KG_N2O5 * n];
    v[G_CO2 * KQ_S] = gas[KG_CO2 * n];
    v[G_NH3 * KQ_S] = gas[KG_NH3 * n];
    v[G_H2O2 * KQ_S] = gas[KG_H2O2 * n];
    v[G_O3 * KQ_S] = gas[KG_O3 * n];
    v[G_HCOOH * KQ_S] = gas[KG_FOA * n];
    v[G_MHP * KQ_S] = gas[KG_MHP * n];
    v[G_PAA * KQ_S] = gas[KG_PAA * n];
    v[G_HCL * KQ_S] = gas[KG_HCL * n];
    v[G_GLY * KQ_S] = gas[KG_GLY * n];
    v[G_MGLY * KQ_S] = gas[KG_MGLY * n];
    v[G_IEPOX * KQ_S] = gas[KG_IEPOX * n];
    if (ispc8 > 0) {
        v[G_IMAE * KQ_S] = gas[KG_IMAE * n];
        v[G_IHMML * KQ_S] = gas[KG_IHMML * n];
    }
    v[G_NO2 * KQ_S] = gas[KG_NO2 * n];
    v[G_HONO * KQ_S] = gas[KG_HONO * n];
    v[G_HNO4 * KQ_S] = gas[KG_HNO4 * n];
    v[G_NO3 * KQ_S] = gas[KG_NO3RAD * n];
    v[G_CH3O2 * KQ_S] = gas[KG_CH3O2 * n];
    v[G_GCOL * KQ_S] = gas[KG_GCOL * n];
    v[G_CCOOH * KQ_S] = gas[KG_CCOOH * n];
    v[G_HCHO * KQ_S] = gas[KG_HCHO * n];
    v[G_HO2 * KQ_S] = gas[KG_HO2 * n];
    v[G_HCHOP * KQ_S] = gas[KG_HCHOP * n];
    if (mtpyrac > 0) v[G_PYRAC * KQ_S] = gas[KG_PYRUV * n];
    v[A_NO3AKN * KQ_S] = AER(KA_NO3, KM_AKN);
    v[A_NH4AKN * KQ_S] = AER(KA_NH4, KM_AKN);
    v[A_CLAKN * KQ_S] = AER(KA_CL, KM_AKN);
    v[A_NAAKN * KQ_S] = AER(KA_NA, KM_AKN);
    v[A_SO4AKN * KQ_S] = AER(KA_SO4, KM_AKN);
    v[A_PECAKN * KQ_S] = AER(KA_EC, KM_AKN);
    v[A_POAAKN * KQ_S] = AER(KA_POA, KM_AKN);
    v[A_PRIAKN * KQ_S] = AER(KA_PRI, KM_AKN);
    v[L_SO4MIN2 * KQ_S] = AER(KA_SO4, KM_ACC) + AER(KA_SO4, KM_COR);
    v[L_NO3MIN * KQ_S] = AER(KA_NO3, KM_ACC) + AER(KA_NO3, KM_COR);
    v[L_NH4PLUS * KQ_S] = AER(KA_NH4, KM_ACC) + AER(KA_NH4, KM_COR);
    v[L_CLMIN * KQ_S] = AER(KA_CL, KM_ACC) + AER(KA_CL, KM_COR);
    v[L_PRIACC * KQ_S] = AER(KA_PRI, KM_ACC);
    v[L_NAPLUS * KQ_S] = AER(KA_NA, KM_ACC);
    v[L_CAPLUS2 * KQ_S] = AER(KA_CAACC, KM_ACC);
    v[L_MGPLUS2 * KQ_S] = AER(KA_MGACC, KM_ACC);
    v[L_KPLUS * KQ_S] = AER(KA_KACC, KM_ACC);
    v[L_PECACC * KQ_S] = AER(KA_EC, KM_ACC);
    v[L_ORGC * KQ_S] = (double)0.2f * AER(KA_ORGC, KM_ACC);
    v[L_OXLACMIN2 * KQ_S] = (double)0.8f * AER(KA_ORGC, KM_ACC) / (double)(90.03f / 177.0f);
    v[L_POAACC * KQ_S] = AER(KA_POA, KM_ACC);
    if (ispc8 > 0) {
        v[L_IETET * KQ_S] = AER(KA_IETET, KM_ACC);
        v[L_IEOS * KQ_S] = AER(KA_IEOS, KM_ACC);
        v[L_DIMER * KQ_S] = AER(KA_DIMER, KM_ACC);
        v[L_IMGA * KQ_S] = AER(KA_IMGA, KM_ACC);
        v[L_IMOS * KQ_S] = AER(KA_IMOS, KM_ACC);
    } else {
        v[L_ISO3 * KQ_S] = AER(KA_ISO3, KM_ACC);
    }
    v[L_SO4MIN2 * KQ_S] = v[L_SO4MIN2 * KQ_S] + gas[KG_H2SO4 * n];
    const double soilc = AER(KA_SOILC, KM_COR), anthc = AER(KA_ANTHC, KM_COR), seasc = AER(KA_SEASC, KM_COR);
    double fecor = fac[KF_SOIL_FE] * soilc + fac[KF_CORS_FE] * anthc;
    double mncor = fac[KF_SOIL_MN] * soilc + fac[KF_CORS_MN] * anthc;
    double nacor = fac[KF_SEAS_NA] * seasc + fac[KF_SOIL_NA] * soilc + fac[KF_CORS_NA] * anthc;
    double mgcor = fac[KF_SEAS_MG] * seasc + fac[KF_SOIL_MG] * soilc + fac[KF_CORS_MG] * anthc;
    double cacor = fac[KF_SEAS_CA] * seasc + fac[KF_SOIL_CA] * soilc + fac[KF_CORS_CA] * anthc;
    double kcor = fac[KF_SEAS_K] * seasc + fac[KF_SOIL_K] * soilc + fac[KF_CORS_K] * anthc;
    v[L_NAPLUS * KQ_S] = v[L_NAPLUS * KQ_S] + nacor;
    v[L_CAPLUS2 * KQ_S] = v[L_CAPLUS2 * KQ_S] + cacor;
    v[L_MGPLUS2 * KQ_S] = v[L_MGPLUS2 * KQ_S] + mgcor;
    v[L_KPLUS * KQ_S] = v[L_KPLUS * KQ_S] + kcor;
    v[L_FEPLUS3 * KQ_S] = fe_sol * fe_iii * (AER(KA_FEACC, KM_ACC) + fecor);
    v[L_MNPLUS2 * KQ_S] = mn_sol * mn_ii * (AER(KA_MNACC, KM_ACC) + mncor);
}

// AQCHEM after the kinetic core (c, ierr, st: the lane's at the end): the fractional weights and the
// mass-balance start (aqchem_kmt.F90:434-507) from gas / aer as they came in, then the
// redistribution into GAS, AEROSOL, GASWDEP, AERWDEP (:546-976).  A failed set-up (IERR
// -101, -102) gives NaN in every output, where the reference stops the run.  Returns 0, or
// 1 when the integration or the set-up failed.
KQ_HD inline int kq_aq_finish(const Cell& c, int ierr, const long long* st, const double* p, double* gas, double* aer,
                              int naer, const int* ai, const double* fac, double* gwd, double* awd, double* out,
                              int* st_out, long long n, const double* ws)
{
    const float taucld = (float)p[P_TAUCLD * n], alfa0 = (float)p[P_ALFA0 * n], alfa3 = (float)p[P_ALFA3 * n];
    const float coszen = (float)p[P_COSZEN * n];
    const int ispc8 = (int)p[P_ISPC8 * n], mtpyrac = (int)p[P_MTPYRAC * n];
    /* aqchem_kmt.F90:434-477: fractional weights */
    double totnit = gas[KG_HNO3 * n] + AER(KA_NO3, KM_ACC);
    const double fhno3 = totnit > 0.0 ? gas[KG_HNO3 * n] / totnit : 1.0;
    const double fno3acc = AER(KA_NO3, KM_ACC) + AER(KA_NO3, KM_COR) > 0.0
                               ? AER(KA_NO3, KM_ACC) / (AER(KA_NO3, KM_ACC) + AER(KA_NO3, KM_COR)) : 1.0;
    double totamm = gas[KG_NH3 * n] + AER(KA_NH4, KM_ACC);
    const double fnh3 = totamm > 0.0 ? gas[KG_NH3 * n] / totamm : 1.0;
    const double fnh4acc = AER(KA_NH4, KM_ACC) + AER(KA_NH4, KM_COR) > 0.0
                               ? AER(KA_NH4, KM_ACC) / (AER(KA_NH4, KM_ACC) + AER(KA_NH4, KM_COR)) : 1.0;
    const double totcl = gas[KG_HCL * n] + AER(KA_CL, KM_ACC);
    const double fhcl = totcl > 0.0 ? gas[KG_HCL * n] / totcl : 1.0;
    const double fclacc = AER(KA_CL, KM_ACC) + AER(KA_CL, KM_COR) > 0.0
                              ? AER(KA_CL, KM_ACC) / (AER(KA_CL, KM_ACC) + AER(KA_CL, KM_COR)) : 1.0;
    (void)fhcl;
    const int dark = coszen <= 0.0f;
    /* :486-498: mass balance at the start */
    const double w_s = (double)32.06f, w_n = (double)14.007f, w_cl = (double)35.5f;
    double startm[4];
    startm[0] = (gas[KG_SO2 * n] + gas[KG_H2SO4 * n]) * w_s;
    startm[1] = (gas[KG_HNO3 * n] + 2 * gas[KG_N2O5 * n] + gas[KG_NO2 * n] + gas[KG_HONO * n] + gas[KG_HNO4 * n] + gas[KG_NO3RAD * n]) * w_n;
    startm[2] = gas[KG_NH3 * n] * w_n;
    startm[3] = gas[KG_HCL * n] * w_cl;
    for (int m = 0; m < 3; ++m) {
        startm[0] = startm[0] + AER(KA_SO4, m) * w_s;
        startm[1] = startm[1] + AER(KA_NO3, m) * w_n;
        startm[2] = startm[2] + AER(KA_NH4, m) * w_n;
        startm[3] = startm[3] + AER(KA_CL, m) * w_cl;
    }
    const double poaiinit = AER(KA_POA, KM_AKN), priiinit = AER(KA_PRI, KM_AKN);
    const double traciinit = AER(KA_TRACER_AKN, KM_AKN), soaiinit = AER(KA_SOA, KM_AKN);
    const double fe_iii = dark ? 0.9 : 0.1, mn_ii = 1.0, fe_sol = 0.1, mn_sol = 0.5;
    for (int i = 0; i < NSTAT; ++i) st_out[i * n] = (int)st[i];
    if (ierr <= -101) {   /* set-up failed: the reference stops the run */
        for (int i = 0; i < KG_NGAS; ++i) gas[i * n] = gwd[i * n] = NAN;
        for (int i = 0; i < naer * 3; ++i) aer[i * n] = awd[i * n] = NAN;
        for (int i = 0; i < KO_N; ++i) out[i * n] = NAN;
        return 1;
    }
    const double* y = ws + W_Y * KQ_S;
    const double* f = ws + W_F * KQ_S;
    /* :546-976: redistribution */
    for (int i = 0; i < KG_NGAS; ++i) gwd[i * n] = 0.0;
    for (int i = 0; i < naer * 3; ++i) awd[i * n] = 0.0;
    const float temp2 = (float)p[P_TEMP2 * n], airm = (float)p[P_AIRM * n], pres_pa = (float)p[P_PRES_PA * n];
    const double cthk1 = (double)(airm * temp2) * 0.08206 / ((double)pres_pa / 101325.0 * 1000.0);
    const double cfactor = c.cfactor, invcfac = 1.0 / cfactor;
    const double wfactor = (double)(float)p[P_WCAVG * n] * cthk1 * c.phi2;
    const double expwet = kq_exp(-c.wetfac * (double)taucld);
    const double ex0 = kq_fexp(-alfa0 * taucld), ex3 = kq_fexp(-alfa3 * taucld);
    AER(KA_NO3, KM_AKN) = y[A_NO3AKN * KQ_S] * invcfac;
    AER(KA_NH4, KM_AKN) = y[A_NH4AKN * KQ_S] * invcfac;
    AER(KA_CL, KM_AKN) = y[A_CLAKN * KQ_S] * invcfac;
    AER(KA_NA, KM_AKN) = y[A_NAAKN * KQ_S] * invcfac;
    AER(KA_SO4, KM_AKN) = y[A_SO4AKN * KQ_S] * invcfac;
    AER(KA_EC, KM_AKN) = y[A_PECAKN * KQ_S] * invcfac;
    AER(KA_POA, KM_AKN) = y[A_POAAKN * KQ_S] * invcfac;
    AER(KA_PRI, KM_AKN) = y[A_PRIAKN * KQ_S] * invcfac;
    AER(KA_NUM, KM_AKN) = AER(KA_NUM, KM_AKN) * ex0;
    AER(KA_TRACER_ACC, KM_ACC) = AER(KA_TRACER_ACC, KM_ACC) + AER(KA_TRACER_AKN, KM_AKN) * (1.0 - ex3);
    AER(KA_PHG_ACC, KM_ACC) = AER(KA_PHG_ACC, KM_ACC) + AER(KA_PHG_AKN, KM_AKN) * (1.0 - ex3);
    AER(KA_TRACER_AKN, KM_AKN) = AER(KA_TRACER_AKN, KM_AKN) * ex3;
    AER(KA_PHG_AKN, KM_AKN) = AER(KA_PHG_AKN, KM_AKN) * ex3;
    AWD(KA_TRACER_ACC, KM_ACC) = AER(KA_TRACER_ACC, KM_ACC) * (1.0 - expwet) * cfactor;
    AWD(KA_PHG_ACC, KM_ACC) = AER(KA_PHG_ACC, KM_ACC) * (1.0 - expwet) * cfactor;
    AWD(KA_TRACER_COR, KM_COR) = AER(KA_TRACER_COR, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_PHG_COR, KM_COR) = AER(KA_PHG_COR, KM_COR) * (1.0 - expwet) * cfactor;
    AER(KA_TRACER_ACC, KM_ACC) = AER(KA_TRACER_ACC, KM_ACC) * expwet;
    AER(KA_PHG_ACC, KM_ACC) = AER(KA_PHG_ACC, KM_ACC) * expwet;
    AER(KA_TRACER_COR, KM_COR) = AER(KA_TRACER_COR, KM_COR) * expwet;
    AER(KA_PHG_COR, KM_COR) = AER(KA_PHG_COR, KM_COR) * expwet;
    AER(KA_SOA, KM_ACC) = AER(KA_SOA, KM_ACC) + AER(KA_SOA, KM_AKN) * (1.0 - ex3);
    AER(KA_SOA, KM_AKN) = AER(KA_SOA, KM_AKN) * ex3;
    AWD(KA_SOA, KM_ACC) = AER(KA_SOA, KM_ACC) * (1.0 - expwet) * cfactor;
    AER(KA_SOA, KM_ACC) = AER(KA_SOA, KM_ACC) * expwet;
    AWD(KA_SOILC, KM_COR) = AER(KA_SOILC, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_SEASC, KM_COR) = AER(KA_SEASC, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_ANTHC, KM_COR) = AER(KA_ANTHC, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_SO4, KM_COR) = AER(KA_SO4, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_NH4, KM_COR) = AER(KA_NH4, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_NO3, KM_COR) = AER(KA_NO3, KM_COR) * (1.0 - expwet) * cfactor;
    AWD(KA_CL, KM_COR) = AER(KA_CL, KM_COR) * (1.0 - expwet) * cfactor;
    AER(KA_NUM, KM_COR) = AER(KA_NUM, KM_COR) * expwet;
    AER(KA_SOILC, KM_COR) = AER(KA_SOILC, KM_COR) * expwet;
    AER(KA_SEASC, KM_COR) = AER(KA_SEASC, KM_COR) * expwet;
    AER(KA_ANTHC, KM_COR) = AER(KA_ANTHC, KM_COR) * expwet;
    AER(KA_SO4, KM_COR) = AER(KA_SO4, KM_COR) * expwet;
    AER(KA_NH4, KM_COR) = AER(KA_NH4, KM_COR) * expwet;
    AER(KA_NO3, KM_COR) = AER(KA_NO3, KM_COR) * expwet;
    AER(KA_CL, KM_COR) = AER(KA_CL, KM_COR) * expwet;
    const double wsoil = AWD(KA_SOILC, KM_COR), wanth = AWD(KA_ANTHC, KM_COR), wseas = AWD(KA_SEASC, KM_COR);
    const double wdfecor = fac[KF_SOIL_FE] * wsoil + fac[KF_CORS_FE] * wanth;
    const double wdmncor = fac[KF_SOIL_MN] * wsoil + fac[KF_CORS_MN] * wanth;
    const double wdnacor = fac[KF_SEAS_NA] * wseas + fac[KF_SOIL_NA] * wsoil + fac[KF_CORS_NA] * wanth;
    const double wdmgcor = fac[KF_SEAS_MG] * wseas + fac[KF_SOIL_MG] * wsoil + fac[KF_CORS_MG] * wanth;
    const double wdcacor = fac[KF_SEAS_CA] * wseas + fac[KF_SOIL_CA] * wsoil + fac[KF_CORS_CA] * wanth;
    const double wdkcor = fac[KF_SEAS_K] * wseas + fac[KF_SOIL_K] * wsoil + fac[KF_CORS_K] * wanth;
    AWD(KA_FEACC, KM_ACC) = fmax((y[WD_FEPLUS3 * KQ_S] / fe_iii / fe_sol) - wdfecor, 0.0);
    AWD(KA_MNACC, KM_ACC) = fmax((y[WD_MNPLUS2 * KQ_S] / mn_ii / mn_sol) - wdmncor, 0.0);
    AWD(KA_NA, KM_ACC) = fmax(y[WD_NAPLUS * KQ_S] - wdnacor, 0.0);
    AWD(KA_CAACC, KM_ACC) = fmax(y[WD_CAPLUS2 * KQ_S] - wdcacor, 0.0);
    AWD(KA_MGACC, KM_ACC) = fmax(y[WD_MGPLUS2 * KQ_S] - wdmgcor, 0.0);
    AWD(KA_KACC, KM_ACC) = fmax(y[WD_KPLUS * KQ_S] - wdkcor, 0.0);
    AWD(KA_SO4, KM_ACC) = fmax(y[WD_H2SO4 * KQ_S] - AWD(KA_SO4, KM_COR), 0.0);
    AWD(KA_NH4, KM_ACC) = fmax(y[WD_NH4PLUS * KQ_S] - AWD(KA_NH4, KM_COR), 0.0);
    AWD(KA_NO3, KM_ACC) = fmax(y[WD_NO3MIN * KQ_S] - AWD(KA_NO3, KM_COR), 0.0);
    AWD(KA_CL, KM_ACC) = fmax(y[WD_CLMIN * KQ_S] - AWD(KA_CL, KM_COR), 0.0);
    AWD(KA_PRI, KM_ACC) = y[WD_PRIACC * KQ_S];
    AWD(KA_EC, KM_ACC) = y[WD_PECACC * KQ_S];
    AWD(KA_ORGC, KM_ACC) = y[WD_ORGC * KQ_S];
    AWD(KA_POA, KM_ACC) = y[WD_POAACC * KQ_S];
    if (ispc8 > 0) {
        AWD(KA_IETET, KM_ACC) = y[WD_IETET * KQ_S];
        AWD(KA_IEOS, KM_ACC) = y[WD_IEOS * KQ_S];
        AWD(KA_DIMER, KM_ACC) = y[WD_DIMER * KQ_S];
        AWD(KA_IMGA, KM_ACC) = y[WD_IMGA * KQ_S];
        AWD(KA_IMOS, KM_ACC) = y[WD_IMOS * KQ_S];
    } else {
        AWD(KA_ISO3, KM_ACC) = y[WD_IETET * KQ_S];
    }
    if (AWD(KA_NH4, KM_COR) > y[WD_NH4PLUS * KQ_S]) {
        AWD(KA_NH4, KM_COR) = (1.0 - fnh4acc) * y[WD_NH4PLUS * KQ_S];
        AWD(KA_NH4, KM_ACC) = fnh4acc * y[WD_NH4PLUS * KQ_S];
        AER(KA_NH4, KM_COR) = (1.0 - fnh4acc) * (y[L_NH4OH * KQ_S] + y[L_NH4PLUS * KQ_S]) * invcfac;
    }
    if (AWD(KA_NO3, KM_COR) > y[WD_NO3MIN * KQ_S]) {
        AWD(KA_NO3, KM_COR) = (1.0 - fno3acc) * y[WD_NO3MIN * KQ_S];
        AWD(KA_NO3, KM_ACC) = fno3acc * y[WD_NO3MIN * KQ_S];
        AER(KA_NO3, KM_COR) = (1.0 - fno3acc) * (y[L_HNO3 * KQ_S] + y[L_NO3MIN * KQ_S]) * invcfac;
    }
    if (AWD(KA_CL, KM_COR) > y[WD_CLMIN * KQ_S]) {
        AWD(KA_CL, KM_COR) = (1.0 - fclacc) * y[WD_CLMIN * KQ_S];
        AWD(KA_CL, KM_ACC) = fclacc * y[WD_CLMIN * KQ_S];
        AER(KA_CL, KM_COR) = (1.0 - fclacc) * y[L_CLMIN * KQ_S] * invcfac;
    }
    AER(KA_PRI, KM_ACC) = y[L_PRIACC * KQ_S] * invcfac;
    AER(KA_EC, KM_ACC) = y[L_PECACC * KQ_S] * invcfac;
    AER(KA_ORGC, KM_ACC) = y[L_ORGC * KQ_S] * invcfac;
    AER(KA_POA, KM_ACC) = y[L_POAACC * KQ_S] * invcfac;
    out[(KO_FRACTR) * n] = AER(KA_TRACER_ACC, KM_ACC) > 0.0
        ? fmin(((traciinit - AER(KA_TRACER_AKN, KM_AKN)) * expwet) / AER(KA_TRACER_ACC, KM_ACC), 1.0) : 0.0;
    out[(KO_FRACPOA) * n] = AER(KA_POA, KM_ACC) > 0.0
        ? fmin(((poaiinit - AER(KA_POA, KM_AKN)) * expwet) / AER(KA_POA, KM_ACC), 1.0) : 0.0;
    out[(KO_FRACPRI) * n] = AER(KA_PRI, KM_ACC) > 0.0
        ? fmin(((priiinit - AER(KA_PRI, KM_AKN)) * expwet) / AER(KA_PRI, KM_ACC), 1.0) : 0.0;
    out[(KO_FRACSOA) * n] = AER(KA_SOA, KM_ACC) > 0.0
        ? fmin(((soaiinit - AER(KA_SOA, KM_AKN)) * expwet) / AER(KA_SOA, KM_ACC), 1.0) : 0.0;
    if (ispc8 > 0) {
        AER(KA_IETET, KM_ACC) = y[L_IETET * KQ_S] * invcfac;
        AER(KA_IEOS, KM_ACC) = y[L_IEOS * KQ_S] * invcfac;
        AER(KA_DIMER, KM_ACC) = y[L_DIMER * KQ_S] * invcfac;
        AER(KA_IMGA, KM_ACC) = y[L_IMGA * KQ_S] * invcfac;
        AER(KA_IMOS, KM_ACC) = y[L_IMOS * KQ_S] * invcfac;
    } else {
        AER(KA_ISO3, KM_ACC) = (y[L_ISO3 * KQ_S]) * invcfac;
    }
    const double soilc2 = AER(KA_SOILC, KM_COR), anthc2 = AER(KA_ANTHC, KM_COR), seasc2 = AER(KA_SEASC, KM_COR);
    const double fecor = fac[KF_SOIL_FE] * soilc2 + fac[KF_CORS_FE] * anthc2;
    const double mncor = fac[KF_SOIL_MN] * soilc2 + fac[KF_CORS_MN] * anthc2;
    const double nacor = fac[KF_SEAS_NA] * seasc2 + fac[KF_SOIL_NA] * soilc2 + fac[KF_CORS_NA] * anthc2;
    const double mgcor = fac[KF_SEAS_MG] * seasc2 + fac[KF_SOIL_MG] * soilc2 + fac[KF_CORS_MG] * anthc2;
    const double cacor = fac[KF_SEAS_CA] * seasc2 + fac[KF_SOIL_CA] * soilc2 + fac[KF_CORS_CA] * anthc2;
    const double kcor = fac[KF_SEAS_K] * seasc2 + fac[KF_SOIL_K] * soilc2 + fac[KF_CORS_K] * anthc2;
    AER(KA_FEACC, KM_ACC) = fmax((y[L_FEPLUS3 * KQ_S] / fe_iii / fe_sol - fecor * cfactor) * invcfac, 0.0);
    AER(KA_MNACC, KM_ACC) = fmax((y[L_MNPLUS2 * KQ_S] / mn_ii / mn_sol - mncor * cfactor) * invcfac, 0.0);
    AER(KA_NA, KM_ACC) = fmax((y[L_NAPLUS * KQ_S] - nacor * cfactor) * invcfac, 0.0);
    AER(KA_CAACC, KM_ACC) = fmax((y[L_CAPLUS2 * KQ_S] - cacor * cfactor) * invcfac, 0.0);
    AER(KA_MGACC, KM_ACC) = fmax((y[L_MGPLUS2 * KQ_S] - mgcor * cfactor) * invcfac, 0.0);
    AER(KA_KACC, KM_ACC) = fmax((y[L_KPLUS * KQ_S] - kcor * cfactor) * invcfac, 0.0);
    AER(KA_SO4, KM_ACC) = fmax(((y[L_H2SO4 * KQ_S] + y[L_SO4MIN2 * KQ_S] + y[L_HSO4MIN * KQ_S]) * invcfac)
                               - AER(KA_SO4, KM_COR), 0.0);
    AER(KA_CL, KM_ACC) = fmax((y[L_CLMIN * KQ_S] * invcfac) - AER(KA_CL, KM_COR), 0.0);
    totamm = y[G_NH3 * KQ_S] + y[L_NH4OH * KQ_S] + y[L_NH4PLUS * KQ_S] - AER(KA_NH4, KM_COR) * cfactor;
    totnit = y[G_HNO3 * KQ_S] + y[L_HNO3 * KQ_S] + y[L_NO3MIN * KQ_S] - AER(KA_NO3, KM_COR) * cfactor;
    totamm = fmax(totamm, 0.0);
    totnit = fmax(totnit, 0.0);
    AER(KA_NO3, KM_ACC) = ((1.0 - fhno3) * totnit) * invcfac;
    AER(KA_NH4, KM_ACC) = ((1.0 - fnh3) * totamm) * invcfac;
    const double oliggly = 0.0 * 3.3e-1, oligmgly = 0.0 * 1.9e-1;   /* OLIG = 0 (aqchem_kmt.F90:412) */
    gas[KG_SO2 * n] = (y[G_SO2 * KQ_S] + y[L_SO2 * KQ_S] + y[L_HSO3MIN * KQ_S] + y[L_SO3MIN2 * KQ_S] + y[L_HMSMIN * KQ_S]
                   + y[L_SO3MIN * KQ_S] + y[L_SO5MIN * KQ_S] + y[L_HSO5MIN * KQ_S] + y[L_SO4MIN * KQ_S]) * invcfac;
    gas[KG_N2O5 * n] = 0.0;
    gas[KG_CO2 * n] = (y[G_CO2 * KQ_S] + y[L_H2CO3 * KQ_S] + y[L_HCO3MIN * KQ_S] + y[L_CO3MIN2 * KQ_S] + y[L_CO2MIN * KQ_S])
                  * invcfac;
    gas[KG_H2O2 * n] = (y[G_H2O2 * KQ_S] + y[L_H2O2 * KQ_S]) * invcfac;
    gas[KG_O3 * n] = (y[G_O3 * KQ_S] + y[L_O3 * KQ_S]) * invcfac;
    gas[KG_FOA * n] = (y[G_HCOOH * KQ_S] + y[L_HCOOH * KQ_S] + y[L_HCOOMIN * KQ_S]) * invcfac;
    gas[KG_MHP * n] = (y[G_MHP * KQ_S] + y[L_MHP * KQ_S]) * invcfac;
    gas[KG_PAA * n] = (y[G_PAA * KQ_S] + y[L_PAA * KQ_S]) * invcfac;
    gas[KG_H2SO4 * n] = 0.0;
    gas[KG_HCL * n] = (y[G_HCL * KQ_S] + y[L_HCL * KQ_S]) * invcfac;
    gas[KG_GLY * n] = (y[G_GLY * KQ_S] + y[L_GLY * KQ_S] * (1.0 - oliggly)) * invcfac;
    gas[KG_MGLY * n] = (y[G_MGLY * KQ_S] + y[L_MGLY * KQ_S] * (1.0 - oligmgly)) * invcfac;
    gas[KG_HNO3 * n] = (fhno3 * totnit) * invcfac;
    gas[KG_NH3 * n] = (fnh3 * totamm) * invcfac;
    gas[KG_HO * n] = (f[G_HO * KQ_S]) * invcfac;
    gas[KG_IEPOX * n] = (y[G_IEPOX * KQ_S] + y[L_IEPOX * KQ_S]) * invcfac;
    if (ispc8 > 0) {
        gas[KG_IMAE * n] = (y[G_IMAE * KQ_S] + y[L_IMAE * KQ_S]) * invcfac;
        gas[KG_IHMML * n] = (y[G_IHMML * KQ_S] + y[L_IHMML * KQ_S]) * invcfac;
    }
    gas[KG_HO2 * n] = (y[G_HO2 * KQ_S] + y[L_HO2 * KQ_S] + y[L_O2MIN * KQ_S]) * invcfac;
    gas[KG_NO2 * n] = (y[G_NO2 * KQ_S] + y[L_NO2 * KQ_S]) * invcfac;
    gas[KG_HONO * n] = (y[G_HONO * KQ_S] + y[L_HONO * KQ_S] + y[L_NO2MIN * KQ_S]) * invcfac;
    gas[KG_HNO4 * n] = (y[G_HNO4 * KQ_S] + y[L_HNO4 * KQ_S] + y[L_NO4MIN * KQ_S]) * invcfac;
    gas[KG_NO3RAD * n] = (y[G_NO3 * KQ_S] + y[L_NO3 * KQ_S]) * invcfac;
    gas[KG_CH3O2 * n] = (y[G_CH3O2 * KQ_S] + y[L_CH3O2 * KQ_S]) * invcfac;
    gas[KG_CCOOH * n] = (y[G_CCOOH * KQ_S] + y[L_CCOOH * KQ_S] + y[L_CCOOHMIN * KQ_S]) * invcfac;
    gas[KG_HCHO * n] = (y[G_HCHO * KQ_S] + y[L_CH2OHYD * KQ_S] + y[L_HCHO * KQ_S] + y[L_HMSMIN * KQ_S]) * invcfac;
    gas[KG_GCOL * n] = (y[G_GCOL * KQ_S] + y[L_GCOL * KQ_S]) * invcfac;
    gas[KG_HCHOP * n] = (y[G_HCHOP * KQ_S] + y[L_CH2OHYDP * KQ_S] + y[L_HCHOP * KQ_S] + y[L_HMSMINP * KQ_S]) * invcfac;
    gwd[KG_SO2 * n] = y[WD_SO2 * KQ_S];
    gwd[KG_HNO3 * n] = y[WD_HNO3 * KQ_S];
    gwd[KG_N2O5 * n] = 0.0;
    gwd[KG_CO2 * n] = y[WD_CO2 * KQ_S];
    gwd[KG_NH3 * n] = y[WD_NH4OH * KQ_S];
    gwd[KG_H2O2 * n] = y[WD_H2O2 * KQ_S];
    gwd[KG_O3 * n] = y[WD_O3 * KQ_S];
    gwd[KG_FOA * n] = y[WD_HCOOH * KQ_S];
    gwd[KG_MHP * n] = y[WD_MHP * KQ_S];
    gwd[KG_PAA * n] = y[WD_PAA * KQ_S];
    gwd[KG_H2SO4 * n] = 0.0;
    gwd[KG_HCL * n] = y[WD_HCL * KQ_S];
    gwd[KG_GLY * n] = y[WD_GLY * KQ_S] * (1.0 - oliggly);
    gwd[KG_MGLY * n] = y[WD_MGLY * KQ_S] * (1.0 - oligmgly);
    gwd[KG_HO * n] = y[WD_HO * KQ_S];
    gwd[KG_IEPOX * n] = y[WD_IEPOX * KQ_S];
    if (ispc8 > 0) {
        gwd[KG_IMAE * n] = y[WD_IMAE * KQ_S];
        gwd[KG_IHMML * n] = y[WD_IHMML * KQ_S];
    }
    gwd[KG_NO2 * n] = y[WD_NO2 * KQ_S];
    gwd[KG_HONO * n] = y[WD_HONO * KQ_S];
    gwd[KG_HNO4 * n] = y[WD_HNO4 * KQ_S];
    gwd[KG_NO3RAD * n] = y[WD_NO3 * KQ_S];
    gwd[KG_CH3O2 * n] = y[WD_CH3O2 * KQ_S];
    gwd[KG_GCOL * n] = y[WD_GCOL * KQ_S];
    gwd[KG_CCOOH * n] = y[WD_CCOOH * KQ_S];
    gwd[KG_HCHO * n] = y[WD_CH2OHYD * KQ_S];
    gwd[KG_HO2 * n] = y[WD_HO2 * KQ_S];
    gwd[KG_HCHOP * n] = y[WD_CH2OHYDP * KQ_S];
    double apyrac = 0.0, wdpyrac = 0.0;
    if (mtpyrac > 0) {
        gas[KG_PYRUV * n] = (y[G_PYRAC * KQ_S] + y[L_PYRAC * KQ_S]) * invcfac;
        gwd[KG_PYRUV * n] = y[WD_PYRAC * KQ_S];
        wdpyrac = 0.0;
        apyrac = y[L_PYRACMIN * KQ_S];
    } else {
        wdpyrac = y[WD_PYRAC * KQ_S];
        apyrac = y[L_PYRAC * KQ_S] + y[L_PYRACMIN * KQ_S];
    }
    const double r7404 = (double)(74.04f / 177.0f), r9003 = (double)(90.03f / 177.0f);
    const double r8806 = (double)(88.06f / 177.0f), r7605 = (double)(76.05f / 177.0f);
    const double r5804 = (double)(58.04f / 177.0f), r7206 = (double)(72.06f / 177.0f);
    AER(KA_ORGC, KM_ACC) = (y[L_ORGC * KQ_S] + (r7404 * y[L_GLYAC * KQ_S]) + (r9003 * y[L_OXLAC * KQ_S])
                            + (r9003 * y[L_OXLACMIN * KQ_S]) + (r9003 * y[L_OXLACMIN2 * KQ_S]) + (r8806 * apyrac)
                            + (r7605 * y[L_GCOLAC * KQ_S]) + (r7404 * y[L_GLYACMIN * KQ_S])
                            + (r7605 * y[L_GCOLACMIN * KQ_S])
                            + r5804 * oliggly * y[L_GLY * KQ_S] + r7206 * oligmgly * y[L_MGLY * KQ_S]) * invcfac;
    AWD(KA_ORGC, KM_ACC) = y[WD_ORGC * KQ_S] + (r7404 * y[WD_GLYAC * KQ_S]) + (r9003 * y[WD_OXLAC * KQ_S])
                           + (r8806 * wdpyrac) + (r7605 * y[WD_GCOLAC * KQ_S])
                           + r5804 * oliggly * y[WD_GLY * KQ_S] + r7206 * oligmgly * y[WD_MGLY * KQ_S];
    for (int i = 0; i < KG_NGAS; ++i) gwd[i * n] = gwd[i * n] * wfactor;
    for (int i = 0; i < naer * 3; ++i) awd[i * n] = awd[i * n] * wfactor;
    for (int i = 0; i < KG_NGAS; ++i) {
        if (gas[i * n] < 0.0) gas[i * n] = 0.0;
        if (gwd[i * n] < 0.0) gwd[i * n] = 0.0;
    }
    for (int i = 0; i < naer * 3; ++i) {
        if (aer[i * n] < 0.0) aer[i * n] = 0.0;
        if (awd[i * n] < 0.0) awd[i * n] = 0.0;
    }
    out[(KO_HPWDEP) * n] = (double)(float)(y[WD_HPLUS * KQ_S] * wfactor);   /* HPWDEP is REAL */
    const double depsum = AWD(KA_SO4, KM_ACC) / wfactor;
    const double betaso4 = AER(KA_SO4, KM_ACC) * cfactor + depsum > 0.0
                               ? depsum / (AER(KA_SO4, KM_ACC) * cfactor + depsum) / (double)taucld : 0.0;
    out[(KO_BETASO4) * n] = betaso4;
    AER(KA_NUM, KM_ACC) = AER(KA_NUM, KM_ACC) * kq_exp(-betaso4 * (double)taucld);
    /* :919-973: mass balance at the end */
    double endm[4];
    endm[0] = (gas[KG_SO2 * n] + gas[KG_H2SO4 * n] + (gwd[KG_SO2 * n] + gwd[KG_H2SO4 * n]) / wfactor / cfactor) * w_s;
    endm[1] = (gas[KG_HNO3 * n] + 2 * gas[KG_N2O5 * n] + gas[KG_NO2 * n] + gas[KG_HONO * n] + gas[KG_HNO4 * n] + gas[KG_NO3RAD * n]
               + (gwd[KG_HNO3 * n] + gwd[KG_NO2 * n] + gwd[KG_HONO * n] + gwd[KG_HNO4 * n] + gwd[KG_NO3RAD * n]) / wfactor / cfactor)
              * w_n;
    endm[2] = (gas[KG_NH3 * n] + gwd[KG_NH3 * n] / wfactor / cfactor) * w_n;
    endm[3] = (gas[KG_HCL * n] + gwd[KG_HCL * n] / wfactor / cfactor) * w_cl;
    for (int m = 0; m < 3; ++m) {
        endm[0] = endm[0] + AER(KA_SO4, m) * w_s;
        endm[1] = endm[1] + AER(KA_NO3, m) * w_n;
        endm[2] = endm[2] + AER(KA_NH4, m) * w_n;
        endm[3] = endm[3] + AER(KA_CL, m) * w_cl;
    }
    for (int m = 0; m < 3; ++m) {
        endm[0] = endm[0] + (AWD(KA_SO4, m) / wfactor / cfactor) * w_s;
        endm[1] = endm[1] + (AWD(KA_NO3, m) / wfactor / cfactor) * w_n;
        endm[2] = endm[2] + (AWD(KA_NH4, m) / wfactor / cfactor) * w_n;
        endm[3] = endm[3] + (AWD(KA_CL, m) / wfactor / cfactor) * w_cl;
    }
    for (int i = 0; i < 4; ++i) out[(KO_MBAL + i) * n] = startm[i] > 0.0 ? 100 * (startm[i] - endm[i]) / startm[i] : 0.0;
    return ierr == 1 ? 0 : 1;
}

#undef AER
#undef AWD

}  // namespace kmt2
