/* CPU oracle of CMAQ's KMT2 aqueous cloud chemistry kinetics (test infrastructure).
 *
 * Restates, per cloudy cell, the kinetic core of AQCHEM in CCTM/src/cloud/acm_ae7_kmt2:
 *
 *   set-up        aqchem_Initialize.F90:163-638 (units, tolerances, pH by charge
 *                 balance, fixed species) and the Henry's law constants of
 *                 aqchem_kmt.F90:371-396 (hlconst.F:491-511 for the table entries)
 *   rate laws     aqchem_Initialize.F90:53-152, 491-636 (KMTF, KMTB, HYDF, KPHOT; set
 *                 once) and aqchem_Rates.F90:146-362, 415-581 (ionic strength, activity
 *                 coefficients, DISF, DISB, KRXN, KIEPOX; refreshed from the state at the
 *                 start of every step)
 *   f, J          aqchem_Function.F90 (Fun), aqchem_Jacobian.F90 (Jac_SP): walked from the
 *                 generated tables of gen/kmt2_aq.c (reaction factors, tendencies,
 *                 derivative terms); gen/kmt2_aq_unrolled.c holds the same routines as
 *                 straight-line code
 *   LU, solve     aqchem_LinearAlgebra.F90:57-94 (KppDecomp), :655-916 (KppSolve)
 *   integrator    aqchem_Integrator.F90:79-132 (INTEGRATE), :135-425 (Rosenbrock
 *                 parameters), :485-690 (ros_Integrator), :694-724 (ros_ErrorNorm),
 *                 :753-831 (ros_PrepareMatrix), :1070-1134 (Rodas3)
 *   driver loop   aqchem_kmt.F90:511-543 (the call sequence and the DO WHILE (T < TEND) loop)
 *
 * Input is the state vector as the reference's Initialize maps it from the gas and
 * aerosol arrays (mixing ratios, mol/molV, before the unit conversion), so the mapping
 * of CGRID to GAS / AEROSOL (aq_map.F, AQCHEM's set-up) and the redistribution of the
 * result (aqchem_kmt.F90:546-976) are outside this file.
 *
 * Arithmetic follows the reference's Fortran: the same operation order, REAL(4)
 * literals and REAL(4) intermediates where the reference has them, no contraction of
 * a*b+c (built with -ffp-contract=off; the reference's build flags decide that for
 * the Fortran, which cannot be compiled here).  Every EXP and ** (the rate laws,
 * HLCONST's REAL(4) EXP, the activity coefficients, the step-size factor Err**(1/3))
 * uses the portable exp and pow of portable_pow.h, which the device code restates
 * operation for operation: libm's and CUDA's exp and pow differ by ulps, and Rodas3's
 * accept / reject decisions amplify one ulp in a rate constant to 1e-5 in the state.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include "gen/kmt2_aq.c"
#include "gen/kmt2_aq_unrolled.c"
#include "portable_pow.h"

/* x**y of the rate laws: the portable pow, NaN for x < 0 (Fortran's real power of a
 * negative base) */
static double kq_rpow(double x, double y) { return x < 0.0 ? NAN : portable_pow(x, y); }

/* per-cell parameters: the AQCHEM arguments the kinetic core reads */
enum {
    KQP_TEMP2 = 0,   /* K (REAL) */
    KQP_PRES_PA,     /* Pa (REAL) */
    KQP_TAUCLD,      /* s (REAL) */
    KQP_PRCRATE,     /* mm/h (REAL) */
    KQP_WCAVG,       /* kg/m3 liquid water (REAL) */
    KQP_WTAVG,       /* kg/m3 total water (REAL) */
    KQP_AIRM,        /* mol/m2 air in the cloudy layers (REAL) */
    KQP_ALFA0,       /* Aitken number scavenging coefficient (REAL) */
    KQP_ALFA3,       /* Aitken mass scavenging coefficient (REAL) */
    KQP_COSZEN,      /* cosine of the solar zenith angle (REAL) */
    KQP_JH2O2,       /* H2O2 photolysis rate from the gas-phase photolysis (REAL(dp)) */
    KQP_HO,          /* gas-phase OH, mol/molV (REAL(8)) */
    KQP_ISPC8,       /* 1 with the IEPOX-SOA species of AE6I/AE7I, else 0 */
    KQP_MTPYRAC,     /* 1 when pyruvic acid partitions, else 0 */
    KQP_PHOTO,       /* PHOTO (aqchem_kmt.F90:423): 0 in the reference */
    KQ_NPARAM
};

enum { KQS_NSTP = 0, KQS_NACC, KQS_NREJ, KQS_NFUN, KQS_NJAC, KQS_NDEC, KQS_NSOL, KQS_NSNG, KQS_IERR, KQS_NKRON,
       KQ_NSTAT };

typedef struct {   /* aqchem_Global of one cell */
    double temp_kpp, press, lwc, lwcfrac, inv_temp, delinvt, phi2, invphi2, ddiam;
    double czen, photo, jh2o2, alfa3, alfa0, wetfac, cfactor, tend, dt;
    int ispc8, mtpyrac;
    double henry[KQ_NHENRY];
    double fix[KQ_NFIX];
    double rconst[KQ_NREACT];
    double stion, gm1, gm2;
} KqState;

static const double KQ_PHI = 6.0221413e17;   /* aqchem_Global.F90: PHI */
static const double KQ_DAQ = 1.0e-9;         /* aqchem_Global.F90: DAQ */

/* ------------------------------------------------------------------ Henry's law */
/* hlconst.F:509-511 with EFFECTIVE = .FALSE.: REAL(4) throughout.  The REAL(4) EXP is
 * the portable exp rounded to float: libm's and CUDA's expf differ by up to 2 float ulps
 * (1e-7 relative, which moves the gas / aqueous partitioning by as much), so oracle and
 * device share this routine; it is within one float ulp of the exact value. */
static float kq_hlconst(float a, float e, float temp)
{
    const float tfac = (298.0f - temp) / (298.0f * temp);
    return a * (float)portable_exp((double)(e * tfac));
}

/* ------------------------------------------------------------------ rate laws */
/* aqchem_Initialize.F90:53-77 (KMTF) and :79-104 (KMTB): the mass-transfer coefficient of
 * Schwartz (1986); PI is a REAL(4) literal there. */
static double kq_kmt(const KqState* s, double accom, double dg, double mw)
{
    const double rad = s->ddiam * 0.5;
    const double r = 8.3145;
    const double pi = (double)3.1415926536f;
    const double v = sqrt(8.0 * r * s->temp_kpp * 1000.0 / pi / mw);
    double kmt = (rad * rad) / (3.0 * dg);
    kmt = kmt + (4.0 * rad / (3.0 * v * accom));
    return 1.0 / kmt;
}
static double kq_kmtf(const KqState* s, double accom, double dg, double mw)
{
    return kq_kmt(s, accom, dg, mw) * s->lwc / 1000.0;
}
static double kq_kmtb(const KqState* s, double hl, double accom, double dg, double mw)
{
    const double r2 = 0.08206;
    return kq_kmt(s, accom, dg, mw) / (r2 * s->temp_kpp * hl);
}
/* aqchem_Initialize.F90:106-117 */
static double kq_hydf(const KqState* s, double kf, double dh)
{
    double v = kf * portable_exp(dh * s->delinvt);
    return v * s->phi2;
}
/* aqchem_Initialize.F90:132-152 */
static double kq_kphot(const KqState* s, double maxc, double jval)
{
    if (jval < 0.0) {
        if (s->czen > 0.001) return s->photo * 2.718281828 * maxc * portable_exp(-1.0 / s->czen);
        return 0.0;
    }
    return jval;
}

/* aqchem_Rates.F90:146-158 */
static double kq_disf(const KqState* s, double keq, double dh, double kb, int g1)
{
    double v = kb * (keq * portable_exp(dh * s->delinvt));
    if (g1 == 1) v = v * s->gm1;
    return v;
}
/* aqchem_Rates.F90:160-174 */
static double kq_disb(const KqState* s, double kb, int g1)
{
    double v = kb;
    if (g1 == 1) v = v * s->gm1 * s->gm2;
    if (g1 == 2) v = v * s->gm1 * s->gm1;
    return v * s->phi2;
}
/* Aqueous diffusion limitation: the diffuso-reactive parameter q1 and the factor Q
 * (aqchem_Rates.F90:225-242, 300-316, 338-354). */
static double kq_diffusion_q(const KqState* s, double krate)
{
    double q1 = 0.0;
    if (krate < 0.0) q1 = 0.0;
    else q1 = s->ddiam / 2.0 * sqrt(krate / KQ_DAQ);
    double q;
    if (q1 > 1.0e-3) {
        if (q1 <= 100.0) {
            const double e2 = portable_exp(2.0 * q1);
            const double cothq = (e2 + 1.0) / (e2 - 1.0);
            q = 3.0 * ((cothq / q1) - (1.0 / (q1 * q1)));
            if (q > 1.0) q = 1.0;
        } else {
            q = 3.0 / q1;
        }
    } else {
        q = 1.0;
    }
    return q;
}
/* aqchem_Rates.F90:176-249 */
static double kq_krxn(const KqState* s, const double* var, double kr, double dh, int rtype, int qy, int metal)
{
    const double phi2 = s->phi2;
    const double sviinh = 1.0 + 75.0 * kq_rpow((var[KQ_L_H2SO4] + var[KQ_L_HSO4MIN] + var[KQ_L_SO4MIN2]) * phi2, 0.67);
    double k = kr * portable_exp(dh * s->delinvt);
    if (rtype == 1) k = (k / (1.0 + 13.0 * var[KQ_L_HPLUS] * phi2)) * phi2;
    else if (rtype == 3) k = k * phi2;
    else if (rtype == 4) k = k / phi2;
    if (metal > 0) k = k / sviinh;
    if (qy >= 1) {
        const double ko31 = 2.4e+4 * portable_exp(0.0 * s->delinvt);
        const double ko32 = 3.7e+5 * portable_exp(-5530.88 * s->delinvt);
        const double ko33 = 1.5e+9 * portable_exp(-5280.56 * s->delinvt);
        const double ko3t = (ko31 * var[KQ_L_SO2] + ko32 * var[KQ_L_HSO3MIN] + ko33 * var[KQ_L_SO3MIN2]) * phi2;
        k = k * kq_diffusion_q(s, ko3t);
    }
    return k * phi2;
}
/* aqchem_Rates.F90:251-362 */
static double kq_kiepox(const KqState* s, const double* var, double kh, double khso4, int type)
{
    const double phi2 = s->phi2;
    if (s->ispc8 <= 0) {
        if (type > 0) return 0.0;
    } else {
        if (type < 1) return 0.0;
    }
    double k1 = kh * var[KQ_L_HPLUS] * phi2;
    double k2 = khso4 * var[KQ_L_HSO4MIN] * phi2;
    double kiepox = k1 + k2;
    double q;
    if (type <= 1) {
        k1 = 9.0e-4 * var[KQ_L_HPLUS] * phi2;
        k2 = 1.31e-5 * var[KQ_L_HSO4MIN] * phi2;
        double kt = (k1 + k2) * s->fix[KQ_L_H2O] * phi2;
        k1 = 8.83e-3 * var[KQ_L_HPLUS] * phi2;
        k2 = 2.92e-6 * var[KQ_L_HSO4MIN] * phi2;
        kt = kt + (k1 + k2) * var[KQ_L_SO4MIN2] * phi2;
        k1 = 2.0e-4 * var[KQ_L_HPLUS] * phi2;
        k2 = 2.92e-6 * var[KQ_L_HSO4MIN] * phi2;
        if (s->ispc8 <= 0) {
            kt = kt + (k1 + k2) * var[KQ_L_NO3MIN] * phi2;
        } else {
            kt = kt + (k1 + k2) * var[KQ_L_IETET] * phi2;
            kt = kt + (k1 + k2) * var[KQ_L_IEOS] * phi2;
        }
        q = kq_diffusion_q(s, kt);
    } else {
        k1 = 9.0e-4 * var[KQ_L_HPLUS] * phi2;
        k2 = 1.31e-5 * var[KQ_L_HSO4MIN] * phi2;
        double kt = (k1 + k2) * s->fix[KQ_L_H2O] * phi2;
        k1 = 2.0e-4 * var[KQ_L_HPLUS] * phi2;
        k2 = 2.92e-6 * var[KQ_L_HSO4MIN] * phi2;
        kt = kt + (k1 + k2) * var[KQ_L_SO4MIN2] * phi2;
        q = kq_diffusion_q(s, kt);
    }
    kiepox = kiepox * q;
    return kiepox * phi2;
}

/* Ionic strength and activity coefficients, aqchem_Rates.F90:423-452: the terms in the
 * reference's order (L_HMSMIN appears twice there and twice here). */
static void kq_ionic(KqState* s, const double* v)
{
    double sum = v[KQ_L_HPLUS] + v[KQ_L_NH4PLUS] + v[KQ_L_OHMIN] + v[KQ_L_HCO3MIN] + v[KQ_L_O2MIN]
               + v[KQ_L_NO2MIN] + v[KQ_L_NO4MIN] + v[KQ_L_GLYACMIN] + v[KQ_L_OXLACMIN] + v[KQ_L_PYRACMIN]
               + v[KQ_L_GCOLACMIN] + v[KQ_L_CCOOHMIN] + v[KQ_L_HSO3MIN] + v[KQ_L_HCOOMIN] + v[KQ_L_NO3MIN]
               + v[KQ_L_HSO4MIN] + v[KQ_L_HMSMIN] + v[KQ_L_NAPLUS] + v[KQ_L_KPLUS] + v[KQ_L_CLMIN]
               + v[KQ_L_SO4MIN] + v[KQ_L_SO3MIN] + v[KQ_L_HMSMIN] + v[KQ_L_SO5MIN] + v[KQ_L_HSO5MIN]
               + v[KQ_L_CO2MIN] + 3.0 * v[KQ_L_FEPLUS3] + 2.0 * v[KQ_L_MNPLUS2]
               + 4.0 * (v[KQ_L_SO4MIN2] + v[KQ_L_CO3MIN2] + v[KQ_L_OXLACMIN2] + v[KQ_L_SO3MIN2]
                        + v[KQ_L_MNPLUS2] + v[KQ_L_CAPLUS2] + v[KQ_L_MGPLUS2])
               + 9.0 * v[KQ_L_FEPLUS3];
    s->stion = 0.5 * sum * s->phi2;
    const double rs = sqrt(s->stion);
    const double gm1log = -0.509 * (rs / (1.0 + sqrt(s->stion)) - 0.2 * s->stion);
    const double gm2log = gm1log * 4.0;
    s->gm1 = kq_rpow(10.0, gm1log);
    const double gm2 = kq_rpow(10.0, gm2log);
    s->gm2 = gm2 > 1.0e-30 ? gm2 : 1.0e-30;
}

static double kq_rate(const KqState* s, const double* var, int r)
{
    const double* a = &kq_rate_arg[r * 5];
    double v;
    switch (kq_rate_kind[r]) {
    case KQ_RATE_DISF: v = kq_disf(s, a[0], a[1], a[2], (int)a[3]); break;
    case KQ_RATE_DISB: v = kq_disb(s, a[0], (int)a[1]); break;
    case KQ_RATE_KRXN: v = kq_krxn(s, var, a[0], a[1], (int)a[2], (int)a[3], (int)a[4]); break;
    case KQ_RATE_KIEPOX: v = kq_kiepox(s, var, a[0], a[1], (int)a[2]); break;
    case KQ_RATE_KMTF: v = kq_kmtf(s, a[0], a[1], a[2]); break;
    case KQ_RATE_KMTB: v = kq_kmtb(s, s->henry[(int)a[0]], a[1], a[2], a[3]); break;
    case KQ_RATE_HYDF: v = kq_hydf(s, a[0], a[1]); break;
    case KQ_RATE_KPHOT: v = kq_kphot(s, a[0], a[1] == -2.0 ? s->jh2o2 : a[1]); break;
    case KQ_RATE_ALFA3: v = s->alfa3; break;
    case KQ_RATE_WETFAC: v = s->wetfac; break;
    default: v = a[0]; break;
    }
    if (kq_rate_mtpyrac[r]) v = (double)s->mtpyrac * v;
    return v;
}

/* Update_RCONST (aqchem_Rates.F90:415-581) from the state var. */
static void kq_update_rconst(KqState* s, const double* var)
{
    kq_ionic(s, var);
    for (int r = 0; r < KQ_NREACT; ++r)
        if (kq_rate_update[r]) s->rconst[r] = kq_rate(s, var, r);
}

/* ------------------------------------------------------------------ set-up */
/* AQCHEM's Henry's law constants, Initialize and the first Update_RCONST.  var_mix: the
 * 161 species as Initialize maps them (mol/molV); var: the state in molec/cm3. */
static int kq_setup(const double* p, const double* var_mix, KqState* s, double* var)
{
    memset(s, 0, sizeof(*s));
    const float temp2 = (float)p[KQP_TEMP2];
    const float pres_pa = (float)p[KQP_PRES_PA];
    const float taucld = (float)p[KQP_TAUCLD];
    const float prcrate = (float)p[KQP_PRCRATE];
    const float wcavg = (float)p[KQP_WCAVG];
    const float wtavg = (float)p[KQP_WTAVG];
    const float airm = (float)p[KQP_AIRM];
    if (temp2 <= 0.0f || airm <= 0.0f || pres_pa <= 0.0f) return -1;    /* aqchem_kmt.F90:427-431 */

    /* aqchem_kmt.F90:371-396 */
    for (int h = 0; h < KQ_NHENRY; ++h) {
        if (kq_henry_kind[h] == 0)
            s->henry[h] = (double)kq_hlconst((float)kq_henry_a[h], (float)kq_henry_e[h], temp2);
        else if (kq_henry_kind[h] == 1)
            s->henry[h] = kq_henry_a[h] * portable_exp(kq_henry_e[h] * ((298.0 - (double)temp2) / (298.0 * (double)temp2)));
        else
            s->henry[h] = kq_henry_a[h];
    }
    s->jh2o2 = p[KQP_JH2O2];
    s->ispc8 = (int)p[KQP_ISPC8];
    s->mtpyrac = (int)p[KQP_MTPYRAC];
    s->photo = p[KQP_PHOTO];
    /* aqchem_kmt.F90:511: cloud thickness; AIRM * TEMP2 is a REAL(4) product */
    const double cthk1 = (double)(airm * temp2) * 0.08206 / ((double)pres_pa / 101325.0 * 1000.0);

    /* aqchem_Initialize.F90:252-288 */
    s->dt = (double)taucld;
    s->tend = 0.0 + s->dt;
    s->ddiam = 1.6e-5;
    s->temp_kpp = (double)temp2;
    s->press = (double)pres_pa / 101325.0;
    s->lwc = (double)wcavg;
    s->lwcfrac = s->lwc * 1.0e-3;
    s->inv_temp = 1.0 / s->temp_kpp;
    s->delinvt = (298.0 - s->temp_kpp) / (298.0 * s->temp_kpp);
    const double max_prc = (double)prcrate > 1.0e-20 ? (double)prcrate : 1.0e-20;
    const double twash = (double)wtavg * 1000.0 * cthk1 * 3600.0 / (1000.0 * max_prc);
    s->wetfac = prcrate > 0.0f ? 1.0 / twash : 0.0;
    s->alfa3 = (double)(float)p[KQP_ALFA3];
    s->alfa0 = (double)(float)p[KQP_ALFA0];
    s->phi2 = 1000.0 / 6.022e23 / s->lwcfrac;
    s->invphi2 = 1.0 / s->phi2;
    s->czen = (double)(float)p[KQP_COSZEN];

    /* aqchem_Initialize.F90:425-485 */
    s->cfactor = (double)pres_pa / (s->temp_kpp * (double)8.314510f) * KQ_PHI;
    for (int i = 0; i < KQ_NVAR; ++i) var[i] = s->cfactor * var_mix[i];
    for (int i = 0; i < KQ_NFIX; ++i) s->fix[i] = s->cfactor * 0.0;
    s->fix[KQ_L_H2O] = 55.5 * s->invphi2;
    s->fix[KQ_G_HO] = p[KQP_HO] * s->cfactor;
    s->fix[KQ_L_O2] = (double)0.21f * s->press * 1.3e-3 * portable_exp(1500.0 * s->delinvt) * s->invphi2;
    const double kw = 1.00e-14 * portable_exp(-6.955e+03 * s->delinvt);
    double sumpos = 2.0 * (var[KQ_L_CAPLUS2] + var[KQ_L_MGPLUS2]) + var[KQ_L_NAPLUS] + var[KQ_L_KPLUS]
                  + var[KQ_L_NH4PLUS];
    double sumneg = 2.0 * (var[KQ_L_SO4MIN2] + var[KQ_L_OXLACMIN2]) + var[KQ_L_NO3MIN] + var[KQ_L_CLMIN];
    sumpos = sumpos * s->phi2;
    sumneg = sumneg * s->phi2;
    const double chgbal = sumpos - sumneg;
    var[KQ_L_OHMIN] = (chgbal + sqrt(chgbal * chgbal + 4.0 * kw)) * 0.5;
    if (!(var[KQ_L_OHMIN] > 0.0)) return -2;                               /* ERROR IN INITIAL PH CALC */
    var[KQ_L_HPLUS] = kw / var[KQ_L_OHMIN];
    var[KQ_L_OHMIN] = var[KQ_L_OHMIN] * s->invphi2;
    var[KQ_L_HPLUS] = var[KQ_L_HPLUS] * s->invphi2;

    /* aqchem_Initialize.F90:491-636: the rate constants set once */
    for (int r = 0; r < KQ_NREACT; ++r)
        if (!kq_rate_update[r]) s->rconst[r] = kq_rate(s, var, r);
    return 0;
}

/* ------------------------------------------------------------------ f, J, LU */
/* Fun (aqchem_Function.F90): A(i) = RCT(i) * factors in order; Vdot(k) = sum of c * A(i)
 * in the order of the generated statement. */
static void kq_fun(const double* var, const double* fix, const double* rct, double* a, double* vdot)
{
    for (int r = 0; r < KQ_NREACT; ++r) {
        double x = rct[r];
        for (int t = kq_fac_ptr[r]; t < kq_fac_ptr[r + 1]; ++t) {
            const int f = kq_fac[t];
            x = x * (f < KQ_NVAR ? var[f] : fix[f - KQ_NVAR]);
        }
        a[r] = x;
    }
    for (int k = 0; k < KQ_NVAR; ++k) {
        double s = 0.0;
        for (int t = kq_f_ptr[k]; t < kq_f_ptr[k + 1]; ++t) s = s + kq_f_coef[t] * a[kq_f_rxn[t]];
        vdot[k] = s;
    }
}

/* Jac_SP (aqchem_Jacobian.F90:59-2286): B = RCT * multiplicity * other factors, then each
 * stored LU entry as the sum of its coefficient * B terms (0 for fill-in). */
static void kq_jac(const double* var, const double* fix, const double* rct, double* b, double* jvs)
{
    for (int i = 0; i < KQ_NB; ++i) {
        double x = rct[kq_b_rxn[i]];
        if (kq_b_mult[i] > 1) x = x * (double)kq_b_mult[i];
        for (int t = kq_b_ptr[i]; t < kq_b_ptr[i + 1]; ++t) {
            const int f = kq_b_fac[t];
            x = x * (f < KQ_NVAR ? var[f] : fix[f - KQ_NVAR]);
        }
        b[i] = x;
    }
    for (int k = 0; k < KQ_LU_NONZERO; ++k) {
        double s = 0.0;
        for (int t = kq_j_ptr[k]; t < kq_j_ptr[k + 1]; ++t) s = s + kq_j_coef[t] * b[kq_j_b[t]];
        jvs[k] = s;
    }
}

/* KppDecomp (aqchem_LinearAlgebra.F90:57-94): row-wise elimination through a dense
 * work row; returns the 1-based row of a pivot below TINY, else 0. */
static int kq_decomp(double* jvs)
{
    double w[KQ_NVAR];
    for (int k = 0; k < KQ_NVAR; ++k) {
        if (fabs(jvs[kq_lu_diag[k]]) < DBL_MIN) return k + 1;
        for (int kk = kq_lu_crow[k]; kk < kq_lu_crow[k + 1]; ++kk) w[kq_lu_icol[kk]] = jvs[kk];
        for (int kk = kq_lu_crow[k]; kk < kq_lu_diag[k]; ++kk) {
            const int j = kq_lu_icol[kk];
            const double a = -w[j] / jvs[kq_lu_diag[j]];
            w[j] = -a;
            for (int jj = kq_lu_diag[j] + 1; jj < kq_lu_crow[j + 1]; ++jj)
                w[kq_lu_icol[jj]] = w[kq_lu_icol[jj]] + a * jvs[jj];
        }
        for (int kk = kq_lu_crow[k]; kk < kq_lu_crow[k + 1]; ++kk) jvs[kk] = w[kq_lu_icol[kk]];
    }
    return 0;
}

/* KppSolve (aqchem_LinearAlgebra.F90:655-916): forward substitution with the unit lower
 * factor row by row, then backward substitution, each in increasing column order. */
static void kq_solve(const double* jvs, double* x)
{
    for (int i = 0; i < KQ_NVAR; ++i) {
        double v = x[i];
        for (int kk = kq_lu_crow[i]; kk < kq_lu_diag[i]; ++kk) v = v - jvs[kk] * x[kq_lu_icol[kk]];
        x[i] = v;
    }
    for (int i = KQ_NVAR - 1; i >= 0; --i) {
        double v = x[i];
        for (int kk = kq_lu_diag[i] + 1; kk < kq_lu_crow[i + 1]; ++kk) v = v - jvs[kk] * x[kq_lu_icol[kk]];
        x[i] = v / jvs[kq_lu_diag[i]];
    }
}

/* ------------------------------------------------------------------ Rodas3 */
/* Rodas3 coefficients (aqchem_Integrator.F90:1070-1134; Sandu et al. 1997). */
static const double RD3_A[6] = {0.0, 2.0, 0.0, 2.0, 0.0, 1.0};
static const double RD3_C[6] = {4.0, 1.0, -1.0, 1.0, -1.0, -(8.0 / 3.0)};
static const int RD3_NEWF[4] = {1, 0, 1, 1};
static const double RD3_M[4] = {2.0, 0.0, 1.0, 1.0};
static const double RD3_E[4] = {0.0, 0.0, 0.0, 1.0};
static const double RD3_ELO = 3.0;
static const double RD3_GAMMA[4] = {0.5, 1.5, 0.0, 0.0};

/* WAXPY (aqchem_LinearAlgebra.F90:1361-1395): y += alpha x, nothing for alpha = 0 */
static void kq_waxpy(double alpha, const double* x, double* y)
{
    if (alpha == 0.0) return;
    for (int i = 0; i < KQ_NVAR; ++i) y[i] = y[i] + alpha * x[i];
}

/* Multiplier of RTOL for convergence tests (1 = the reference's tolerances, which it
 * leaves bit for bit unchanged). */
static double kq_rtol_scale = 1.0;

/* ros_ErrorNorm (aqchem_Integrator.F90:694-724) with vector tolerances */
static double kq_error_norm(const double* y, const double* ynew, const double* yerr)
{
    double err = 0.0;
    for (int i = 0; i < KQ_NVAR; ++i) {
        const double ymax = fabs(y[i]) > fabs(ynew[i]) ? fabs(y[i]) : fabs(ynew[i]);
        const double scale = kq_atol[i] + (kq_rtol[i] * kq_rtol_scale) * ymax;
        const double q = yerr[i] / scale;
        err = err + q * q;
    }
    err = sqrt(err / (double)KQ_NVAR);
    return err > 1.0e-10 ? err : 1.0e-10;
}

typedef struct {
    double jac0[KQ_LU_NONZERO], ghimj[KQ_LU_NONZERO];
    double ynew[KQ_NVAR], fcn0[KQ_NVAR], fcn[KQ_NVAR], k[4][KQ_NVAR], yerr[KQ_NVAR];
} KqWork;

/* ros_Integrator with Rodas3, autonomous (ICNTRL(1) = 1), vector tolerances, the
 * straight-line f, J, LU and solve (the form of the reference's KPP-generated code, and
 * bit for bit the table-driven routines' results; tests hold them equal), the
 * reference's defaults: Hmin = 0, Hmax = |Tend - Tstart|, Hstart = 1e-5, FacMin 0.2,
 * FacMax 6, FacRej 0.1, FacSafe 0.9, 200000 steps.  The rate constants follow the
 * accepted state: Fun and Jac call Update_RCONST, which reads the module's VAR, the
 * integrator's Y (aqchem_Integrator.F90:1318-1388).  Returns IERR (1 = success) and the
 * time reached in *texit. */
static int kq_ros_integrator(KqState* s, double* y, double tstart, double tend, double* texit, int* st, KqWork* w)
{
    const double roundoff = DBL_EPSILON;           /* WLAMCH('E') */
    const double hmin = 0.0, hmax = fabs(tend - tstart), hstart = 1.0e-5;
    const double facmin = 0.2, facmax = 6.0, facrej = 0.1, facsafe = 0.9;
    const int max_steps = 200000;
    int nstp = 0, nacc = 0;
    double t = tstart;
    *texit = 0.0;                                  /* RSTATUS(Ntexit) before the first accepted step */
    double h = fmin(fmax(fabs(hmin), fabs(hstart)), fabs(hmax));
    if (fabs(h) <= 10.0 * roundoff) h = 1.0e-5;
    int reject_last = 0, reject_more = 0;
    while (fabs(t - tend) >= roundoff) {
        if (nstp > max_steps) return -6;
        if ((t + 0.1 * h) == t || h <= roundoff) return -7;
        h = fmin(h, fabs(tend - t));
        kq_update_rconst(s, y);
        kqu_fun(y, s->fix, s->rconst, w->fcn0);
        st[KQS_NFUN]++;
        kqu_jac(y, s->fix, s->rconst, w->jac0);
        st[KQS_NJAC]++;
        for (;;) {
            /* ros_PrepareMatrix */
            int nconsecutive = 0;
            for (;;) {
                for (int i = 0; i < KQ_LU_NONZERO; ++i) w->ghimj[i] = -w->jac0[i];
                const double ghinv = 1.0 / (h * RD3_GAMMA[0]);
                for (int i = 0; i < KQ_NVAR; ++i) w->ghimj[kq_lu_diag[i]] = w->ghimj[kq_lu_diag[i]] + ghinv;
                const int ising = kqu_decomp(w->ghimj);
                st[KQS_NDEC]++;
                if (ising == 0) break;
                st[KQS_NSNG]++;
                if (++nconsecutive <= 5) h = h * 0.5;
                else return -8;
            }
            for (int s_ = 0; s_ < 4; ++s_) {
                if (s_ == 0) {
                    memcpy(w->fcn, w->fcn0, sizeof(w->fcn));
                } else if (RD3_NEWF[s_]) {
                    memcpy(w->ynew, y, sizeof(w->ynew));
                    for (int j = 0; j < s_; ++j) kq_waxpy(RD3_A[s_ * (s_ - 1) / 2 + j], w->k[j], w->ynew);
                    kqu_fun(w->ynew, s->fix, s->rconst, w->fcn);
                    st[KQS_NFUN]++;
                }
                memcpy(w->k[s_], w->fcn, sizeof(w->fcn));
                for (int j = 0; j < s_; ++j) kq_waxpy(RD3_C[s_ * (s_ - 1) / 2 + j] / h, w->k[j], w->k[s_]);
                kqu_solve(w->ghimj, w->k[s_]);
                st[KQS_NSOL]++;
            }
            memcpy(w->ynew, y, sizeof(w->ynew));
            for (int j = 0; j < 4; ++j) kq_waxpy(RD3_M[j], w->k[j], w->ynew);
            memset(w->yerr, 0, sizeof(w->yerr));
            for (int j = 0; j < 4; ++j) kq_waxpy(RD3_E[j], w->k[j], w->yerr);
            const double err = kq_error_norm(y, w->ynew, w->yerr);
            const double fac = fmin(facmax, fmax(facmin, facsafe / portable_pow(err, 1.0 / RD3_ELO)));
            double hnew = h * fac;
            nstp++;
            st[KQS_NSTP]++;
            if (err <= 1.0 || h <= hmin) {
                nacc++;
                st[KQS_NACC]++;
                memcpy(y, w->ynew, sizeof(w->ynew));
                t = t + h;
                hnew = fmax(hmin, fmin(hnew, hmax));
                if (reject_last) hnew = fmin(hnew, h);
                *texit = t;
                reject_last = 0;
                reject_more = 0;
                h = hnew;
                break;
            }
            if (reject_more) hnew = h * facrej;
            reject_more = reject_last;
            reject_last = 1;
            h = hnew;
            if (nacc >= 1) st[KQS_NREJ]++;
        }
    }
    return 1;
}

/* One cell: set-up, then aqchem_kmt.F90:531-543 (INTEGRATE from T to T + DT while
 * T < TEND; at most 16 passes where the reference would loop on).  var_out gets the
 * state in molec/cm3, fix_out the fixed species. */
static int kq_cell_state(const double* p, const double* var_mix, double* var_out, double* fix_out, int* st,
                         KqWork* w, KqState* sp)
{
    KqState s;
    memset(st, 0, sizeof(int) * KQ_NSTAT);
    int rc = kq_setup(p, var_mix, &s, var_out);
    if (rc != 0) {   /* no state to return: NaN marks the cell's outputs */
        for (int i = 0; i < KQ_NVAR; ++i) var_out[i] = NAN;
        if (fix_out)
            for (int i = 0; i < KQ_NFIX; ++i) fix_out[i] = NAN;
        st[KQS_IERR] = rc - 100;
        return 1;
    }
    double t = 0.0;
    int ierr = 1;
    while (t < s.tend) {
        if (st[KQS_NKRON] >= 16) {
            ierr = -100;
            break;
        }
        st[KQS_NKRON]++;
        kq_update_rconst(&s, var_out);
        double texit = 0.0;
        ierr = kq_ros_integrator(&s, var_out, t, t + s.dt, &texit, st, w);
        t = texit;
        if (ierr < 0 && texit <= 0.0) break;
    }
    if (fix_out) memcpy(fix_out, s.fix, sizeof(s.fix));
    st[KQS_IERR] = ierr;
    if (sp) *sp = s;
    return ierr == 1 ? 0 : 1;
}

static int kq_cell(const double* p, const double* var_mix, double* var_out, double* fix_out, int* st, KqWork* w)
{
    return kq_cell_state(p, var_mix, var_out, fix_out, st, w, NULL);
}

/* ------------------------------------------------------------------ the whole AQCHEM */
/* AQCHEM's GAS array in AQ_DATA.F's srggas order (29 species, mol/molV) */
enum { KG_SO2 = 0, KG_HNO3, KG_N2O5, KG_CO2, KG_NH3, KG_H2O2, KG_O3, KG_FOA, KG_MHP, KG_PAA, KG_H2SO4, KG_HCL,
       KG_GLY, KG_MGLY, KG_HO, KG_IEPOX, KG_IMAE, KG_IHMML, KG_HO2, KG_NO2, KG_HONO, KG_HNO4, KG_GCOL, KG_CCOOH,
       KG_HCHO, KG_NO3RAD, KG_CH3O2, KG_HCHOP, KG_PYRUV, KG_NGAS };
/* positions of the aerosol surrogates AQCHEM reads or writes in the caller's AEROSOL(NAER,
 * NMODES) list (AQ_DATA.F's LSO4, LNH4, ...); element (i, mode) is aer[i + naer * mode] */
enum { KA_SO4 = 0, KA_NH4, KA_NO3, KA_CL, KA_NA, KA_EC, KA_POA, KA_PRI, KA_SOA, KA_NUM, KA_SOILC, KA_SEASC,
       KA_ANTHC, KA_CAACC, KA_MGACC, KA_KACC, KA_FEACC, KA_MNACC, KA_ORGC, KA_TRACER_AKN, KA_TRACER_ACC,
       KA_TRACER_COR, KA_PHG_AKN, KA_PHG_ACC, KA_PHG_COR, KA_IETET, KA_IEOS, KA_DIMER, KA_IMGA, KA_IMOS,
       KA_ISO3, KA_NIDX };
enum { KM_AKN = 0, KM_ACC, KM_COR };
/* coarse crustal factors of aqchem_kmt.F90:329-365 (computed once by the caller) */
enum { KF_SOIL_FE = 0, KF_CORS_FE, KF_SOIL_MN, KF_CORS_MN, KF_SEAS_NA, KF_SOIL_NA, KF_CORS_NA, KF_SEAS_MG,
       KF_SOIL_MG, KF_CORS_MG, KF_SEAS_CA, KF_SOIL_CA, KF_CORS_CA, KF_SEAS_K, KF_SOIL_K, KF_CORS_K, KF_N };
/* per-cell scalar outputs: HPWDEP, BETASO4, FRACTR, FRACPOA, FRACPRI, FRACSOA, and the four
 * mass-balance percentages AQCHEM checks (S, N without NH3, NH3/NH4, Cl) */
enum { KO_HPWDEP = 0, KO_BETASO4, KO_FRACTR, KO_FRACPOA, KO_FRACPRI, KO_FRACSOA, KO_MBAL, KO_N = KO_MBAL + 4 };

/* REAL(4) EXP of the redistribution (EXP of a REAL product): the portable exp rounded to float */
static double kq_fexp(float x) { return (double)(float)portable_exp((double)x); }

/* AQCHEM (aqchem_kmt.F90:21-978) for one cloudy cell: the fractions and mass-balance start
 * (:434-507), Initialize's mapping of GAS / AEROSOL into the KPP state (aqchem_Initialize.F90:
 * 290-421), the set-up and integration of the kinetic core (kq_cell_state), and the
 * redistribution into GAS, AEROSOL, GASWDEP, AERWDEP (:546-976).  gas [KG_NGAS], aer
 * [naer * 3] in and out; gwd [KG_NGAS], awd [naer * 3], out [KO_N] out.  The GAS value of HO
 * replaces the HO parameter.  Returns 0, or 1 when the integration or the set-up failed
 * (set-up: every output NaN, where the reference stops the run). */
static int kq_aqchem_cell(const double* p, double* gas, double* aer, int naer, const int* ai, const double* fac,
                          double* gwd, double* awd, double* out, int* st, KqWork* w)
{
#define AER(k, m) aer[ai[k] + naer * (m)]
#define AWD(k, m) awd[ai[k] + naer * (m)]
    double pp[KQ_NPARAM];
    memcpy(pp, p, sizeof(pp));
    pp[KQP_HO] = gas[KG_HO];
    const float taucld = (float)p[KQP_TAUCLD], alfa0 = (float)p[KQP_ALFA0], alfa3 = (float)p[KQP_ALFA3];
    const float coszen = (float)p[KQP_COSZEN];
    const int ispc8 = (int)p[KQP_ISPC8], mtpyrac = (int)p[KQP_MTPYRAC];
    /* aqchem_kmt.F90:434-477: fractional weights */
    double totnit = gas[KG_HNO3] + AER(KA_NO3, KM_ACC);
    const double fhno3 = totnit > 0.0 ? gas[KG_HNO3] / totnit : 1.0;
    const double fno3acc = AER(KA_NO3, KM_ACC) + AER(KA_NO3, KM_COR) > 0.0
                               ? AER(KA_NO3, KM_ACC) / (AER(KA_NO3, KM_ACC) + AER(KA_NO3, KM_COR)) : 1.0;
    double totamm = gas[KG_NH3] + AER(KA_NH4, KM_ACC);
    const double fnh3 = totamm > 0.0 ? gas[KG_NH3] / totamm : 1.0;
    const double fnh4acc = AER(KA_NH4, KM_ACC) + AER(KA_NH4, KM_COR) > 0.0
                               ? AER(KA_NH4, KM_ACC) / (AER(KA_NH4, KM_ACC) + AER(KA_NH4, KM_COR)) : 1.0;
    const double totcl = gas[KG_HCL] + AER(KA_CL, KM_ACC);
    const double fhcl = totcl > 0.0 ? gas[KG_HCL] / totcl : 1.0;
    const double fclacc = AER(KA_CL, KM_ACC) + AER(KA_CL, KM_COR) > 0.0
                              ? AER(KA_CL, KM_ACC) / (AER(KA_CL, KM_ACC) + AER(KA_CL, KM_COR)) : 1.0;
    (void)fhcl;
    const int dark = coszen <= 0.0f;
    /* :486-498: mass balance at the start */
    const double w_s = (double)32.06f, w_n = (double)14.007f, w_cl = (double)35.5f;
    double startm[4];
    startm[0] = (gas[KG_SO2] + gas[KG_H2SO4]) * w_s;
    startm[1] = (gas[KG_HNO3] + 2 * gas[KG_N2O5] + gas[KG_NO2] + gas[KG_HONO] + gas[KG_HNO4] + gas[KG_NO3RAD]) * w_n;
    startm[2] = gas[KG_NH3] * w_n;
    startm[3] = gas[KG_HCL] * w_cl;
    for (int m = 0; m < 3; ++m) {
        startm[0] = startm[0] + AER(KA_SO4, m) * w_s;
        startm[1] = startm[1] + AER(KA_NO3, m) * w_n;
        startm[2] = startm[2] + AER(KA_NH4, m) * w_n;
        startm[3] = startm[3] + AER(KA_CL, m) * w_cl;
    }
    const double poaiinit = AER(KA_POA, KM_AKN), priiinit = AER(KA_PRI, KM_AKN);
    const double traciinit = AER(KA_TRACER_AKN, KM_AKN), soaiinit = AER(KA_SOA, KM_AKN);
    /* aqchem_Initialize.F90:290-421: the KPP state in mol/molV */
    const double fe_iii = dark ? 0.9 : 0.1, mn_ii = 1.0, fe_sol = 0.1, mn_sol = 0.5;
    double v[KQ_NVAR];
    for (int i = 0; i < KQ_NVAR; ++i) v[i] = 0.0;
    v[KQ_G_SO2] = gas[KG_SO2];
    v[KQ_G_HNO3] = gas[KG_HNO3] + 2.0 * gas[KG_N2O5];
    v[KQ_G_CO2] = gas[KG_CO2];
    v[KQ_G_NH3] = gas[KG_NH3];
    v[KQ_G_H2O2] = gas[KG_H2O2];
    v[KQ_G_O3] = gas[KG_O3];
    v[KQ_G_HCOOH] = gas[KG_FOA];
    v[KQ_G_MHP] = gas[KG_MHP];
    v[KQ_G_PAA] = gas[KG_PAA];
    v[KQ_G_HCL] = gas[KG_HCL];
    v[KQ_G_GLY] = gas[KG_GLY];
    v[KQ_G_MGLY] = gas[KG_MGLY];
    v[KQ_G_IEPOX] = gas[KG_IEPOX];
    if (ispc8 > 0) {
        v[KQ_G_IMAE] = gas[KG_IMAE];
        v[KQ_G_IHMML] = gas[KG_IHMML];
    }
    v[KQ_G_NO2] = gas[KG_NO2];
    v[KQ_G_HONO] = gas[KG_HONO];
    v[KQ_G_HNO4] = gas[KG_HNO4];
    v[KQ_G_NO3] = gas[KG_NO3RAD];
    v[KQ_G_CH3O2] = gas[KG_CH3O2];
    v[KQ_G_GCOL] = gas[KG_GCOL];
    v[KQ_G_CCOOH] = gas[KG_CCOOH];
    v[KQ_G_HCHO] = gas[KG_HCHO];
    v[KQ_G_HO2] = gas[KG_HO2];
    v[KQ_G_HCHOP] = gas[KG_HCHOP];
    if (mtpyrac > 0) v[KQ_G_PYRAC] = gas[KG_PYRUV];
    v[KQ_A_NO3AKN] = AER(KA_NO3, KM_AKN);
    v[KQ_A_NH4AKN] = AER(KA_NH4, KM_AKN);
    v[KQ_A_CLAKN] = AER(KA_CL, KM_AKN);
    v[KQ_A_NAAKN] = AER(KA_NA, KM_AKN);
    v[KQ_A_SO4AKN] = AER(KA_SO4, KM_AKN);
    v[KQ_A_PECAKN] = AER(KA_EC, KM_AKN);
    v[KQ_A_POAAKN] = AER(KA_POA, KM_AKN);
    v[KQ_A_PRIAKN] = AER(KA_PRI, KM_AKN);
    v[KQ_L_SO4MIN2] = AER(KA_SO4, KM_ACC) + AER(KA_SO4, KM_COR);
    v[KQ_L_NO3MIN] = AER(KA_NO3, KM_ACC) + AER(KA_NO3, KM_COR);
    v[KQ_L_NH4PLUS] = AER(KA_NH4, KM_ACC) + AER(KA_NH4, KM_COR);
    v[KQ_L_CLMIN] = AER(KA_CL, KM_ACC) + AER(KA_CL, KM_COR);
    v[KQ_L_PRIACC] = AER(KA_PRI, KM_ACC);
    v[KQ_L_NAPLUS] = AER(KA_NA, KM_ACC);
    v[KQ_L_CAPLUS2] = AER(KA_CAACC, KM_ACC);
    v[KQ_L_MGPLUS2] = AER(KA_MGACC, KM_ACC);
    v[KQ_L_KPLUS] = AER(KA_KACC, KM_ACC);
    v[KQ_L_PECACC] = AER(KA_EC, KM_ACC);
    v[KQ_L_ORGC] = (double)0.2f * AER(KA_ORGC, KM_ACC);
    v[KQ_L_OXLACMIN2] = (double)0.8f * AER(KA_ORGC, KM_ACC) / (double)(90.03f / 177.0f);
    v[KQ_L_POAACC] = AER(KA_POA, KM_ACC);
    if (ispc8 > 0) {
        v[KQ_L_IETET] = AER(KA_IETET, KM_ACC);
        v[KQ_L_IEOS] = AER(KA_IEOS, KM_ACC);
        v[KQ_L_DIMER] = AER(KA_DIMER, KM_ACC);
        v[KQ_L_IMGA] = AER(KA_IMGA, KM_ACC);
        v[KQ_L_IMOS] = AER(KA_IMOS, KM_ACC);
    } else {
        v[KQ_L_ISO3] = AER(KA_ISO3, KM_ACC);
    }
    v[KQ_L_SO4MIN2] = v[KQ_L_SO4MIN2] + gas[KG_H2SO4];
    const double soilc = AER(KA_SOILC, KM_COR), anthc = AER(KA_ANTHC, KM_COR), seasc = AER(KA_SEASC, KM_COR);
    double fecor = fac[KF_SOIL_FE] * soilc + fac[KF_CORS_FE] * anthc;
    double mncor = fac[KF_SOIL_MN] * soilc + fac[KF_CORS_MN] * anthc;
    double nacor = fac[KF_SEAS_NA] * seasc + fac[KF_SOIL_NA] * soilc + fac[KF_CORS_NA] * anthc;
    double mgcor = fac[KF_SEAS_MG] * seasc + fac[KF_SOIL_MG] * soilc + fac[KF_CORS_MG] * anthc;
    double cacor = fac[KF_SEAS_CA] * seasc + fac[KF_SOIL_CA] * soilc + fac[KF_CORS_CA] * anthc;
    double kcor = fac[KF_SEAS_K] * seasc + fac[KF_SOIL_K] * soilc + fac[KF_CORS_K] * anthc;
    v[KQ_L_NAPLUS] = v[KQ_L_NAPLUS] + nacor;
    v[KQ_L_CAPLUS2] = v[KQ_L_CAPLUS2] + cacor;
    v[KQ_L_MGPLUS2] = v[KQ_L_MGPLUS2] + mgcor;
    v[KQ_L_KPLUS] = v[KQ_L_KPLUS] + kcor;
    v[KQ_L_FEPLUS3] = fe_sol * fe_iii * (AER(KA_FEACC, KM_ACC) + fecor);
    v[KQ_L_MNPLUS2] = mn_sol * mn_ii * (AER(KA_MNACC, KM_ACC) + mncor);
    /* the kinetic core */
    double var[KQ_NVAR];
    KqState s;
    const int fail = kq_cell_state(pp, v, var, NULL, st, w, &s);
    if (st[KQS_IERR] <= -101) {   /* set-up failed: the reference stops the run */
        for (int i = 0; i < KG_NGAS; ++i) gas[i] = gwd[i] = NAN;
        for (int i = 0; i < naer * 3; ++i) aer[i] = awd[i] = NAN;
        for (int i = 0; i < KO_N; ++i) out[i] = NAN;
        return 1;
    }
    const double* fixv = s.fix;
    /* :546-976: redistribution */
    for (int i = 0; i < KG_NGAS; ++i) gwd[i] = 0.0;
    for (int i = 0; i < naer * 3; ++i) awd[i] = 0.0;
    const float temp2 = (float)p[KQP_TEMP2], airm = (float)p[KQP_AIRM], pres_pa = (float)p[KQP_PRES_PA];
    const double cthk1 = (double)(airm * temp2) * 0.08206 / ((double)pres_pa / 101325.0 * 1000.0);
    const double cfactor = s.cfactor, invcfac = 1.0 / cfactor;
    const double wfactor = (double)(float)p[KQP_WCAVG] * cthk1 * s.phi2;
    const double expwet = portable_exp(-s.wetfac * (double)taucld);
    const double ex0 = kq_fexp(-alfa0 * taucld), ex3 = kq_fexp(-alfa3 * taucld);
    AER(KA_NO3, KM_AKN) = var[KQ_A_NO3AKN] * invcfac;
    AER(KA_NH4, KM_AKN) = var[KQ_A_NH4AKN] * invcfac;
    AER(KA_CL, KM_AKN) = var[KQ_A_CLAKN] * invcfac;
    AER(KA_NA, KM_AKN) = var[KQ_A_NAAKN] * invcfac;
    AER(KA_SO4, KM_AKN) = var[KQ_A_SO4AKN] * invcfac;
    AER(KA_EC, KM_AKN) = var[KQ_A_PECAKN] * invcfac;
    AER(KA_POA, KM_AKN) = var[KQ_A_POAAKN] * invcfac;
    AER(KA_PRI, KM_AKN) = var[KQ_A_PRIAKN] * invcfac;
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
    AWD(KA_FEACC, KM_ACC) = fmax((var[KQ_WD_FEPLUS3] / fe_iii / fe_sol) - wdfecor, 0.0);
    AWD(KA_MNACC, KM_ACC) = fmax((var[KQ_WD_MNPLUS2] / mn_ii / mn_sol) - wdmncor, 0.0);
    AWD(KA_NA, KM_ACC) = fmax(var[KQ_WD_NAPLUS] - wdnacor, 0.0);
    AWD(KA_CAACC, KM_ACC) = fmax(var[KQ_WD_CAPLUS2] - wdcacor, 0.0);
    AWD(KA_MGACC, KM_ACC) = fmax(var[KQ_WD_MGPLUS2] - wdmgcor, 0.0);
    AWD(KA_KACC, KM_ACC) = fmax(var[KQ_WD_KPLUS] - wdkcor, 0.0);
    AWD(KA_SO4, KM_ACC) = fmax(var[KQ_WD_H2SO4] - AWD(KA_SO4, KM_COR), 0.0);
    AWD(KA_NH4, KM_ACC) = fmax(var[KQ_WD_NH4PLUS] - AWD(KA_NH4, KM_COR), 0.0);
    AWD(KA_NO3, KM_ACC) = fmax(var[KQ_WD_NO3MIN] - AWD(KA_NO3, KM_COR), 0.0);
    AWD(KA_CL, KM_ACC) = fmax(var[KQ_WD_CLMIN] - AWD(KA_CL, KM_COR), 0.0);
    AWD(KA_PRI, KM_ACC) = var[KQ_WD_PRIACC];
    AWD(KA_EC, KM_ACC) = var[KQ_WD_PECACC];
    AWD(KA_ORGC, KM_ACC) = var[KQ_WD_ORGC];
    AWD(KA_POA, KM_ACC) = var[KQ_WD_POAACC];
    if (ispc8 > 0) {
        AWD(KA_IETET, KM_ACC) = var[KQ_WD_IETET];
        AWD(KA_IEOS, KM_ACC) = var[KQ_WD_IEOS];
        AWD(KA_DIMER, KM_ACC) = var[KQ_WD_DIMER];
        AWD(KA_IMGA, KM_ACC) = var[KQ_WD_IMGA];
        AWD(KA_IMOS, KM_ACC) = var[KQ_WD_IMOS];
    } else {
        AWD(KA_ISO3, KM_ACC) = var[KQ_WD_IETET];
    }
    if (AWD(KA_NH4, KM_COR) > var[KQ_WD_NH4PLUS]) {
        AWD(KA_NH4, KM_COR) = (1.0 - fnh4acc) * var[KQ_WD_NH4PLUS];
        AWD(KA_NH4, KM_ACC) = fnh4acc * var[KQ_WD_NH4PLUS];
        AER(KA_NH4, KM_COR) = (1.0 - fnh4acc) * (var[KQ_L_NH4OH] + var[KQ_L_NH4PLUS]) * invcfac;
    }
    if (AWD(KA_NO3, KM_COR) > var[KQ_WD_NO3MIN]) {
        AWD(KA_NO3, KM_COR) = (1.0 - fno3acc) * var[KQ_WD_NO3MIN];
        AWD(KA_NO3, KM_ACC) = fno3acc * var[KQ_WD_NO3MIN];
        AER(KA_NO3, KM_COR) = (1.0 - fno3acc) * (var[KQ_L_HNO3] + var[KQ_L_NO3MIN]) * invcfac;
    }
    if (AWD(KA_CL, KM_COR) > var[KQ_WD_CLMIN]) {
        AWD(KA_CL, KM_COR) = (1.0 - fclacc) * var[KQ_WD_CLMIN];
        AWD(KA_CL, KM_ACC) = fclacc * var[KQ_WD_CLMIN];
        AER(KA_CL, KM_COR) = (1.0 - fclacc) * var[KQ_L_CLMIN] * invcfac;
    }
    AER(KA_PRI, KM_ACC) = var[KQ_L_PRIACC] * invcfac;
    AER(KA_EC, KM_ACC) = var[KQ_L_PECACC] * invcfac;
    AER(KA_ORGC, KM_ACC) = var[KQ_L_ORGC] * invcfac;
    AER(KA_POA, KM_ACC) = var[KQ_L_POAACC] * invcfac;
    out[KO_FRACTR] = AER(KA_TRACER_ACC, KM_ACC) > 0.0
        ? fmin(((traciinit - AER(KA_TRACER_AKN, KM_AKN)) * expwet) / AER(KA_TRACER_ACC, KM_ACC), 1.0) : 0.0;
    out[KO_FRACPOA] = AER(KA_POA, KM_ACC) > 0.0
        ? fmin(((poaiinit - AER(KA_POA, KM_AKN)) * expwet) / AER(KA_POA, KM_ACC), 1.0) : 0.0;
    out[KO_FRACPRI] = AER(KA_PRI, KM_ACC) > 0.0
        ? fmin(((priiinit - AER(KA_PRI, KM_AKN)) * expwet) / AER(KA_PRI, KM_ACC), 1.0) : 0.0;
    out[KO_FRACSOA] = AER(KA_SOA, KM_ACC) > 0.0
        ? fmin(((soaiinit - AER(KA_SOA, KM_AKN)) * expwet) / AER(KA_SOA, KM_ACC), 1.0) : 0.0;
    if (ispc8 > 0) {
        AER(KA_IETET, KM_ACC) = var[KQ_L_IETET] * invcfac;
        AER(KA_IEOS, KM_ACC) = var[KQ_L_IEOS] * invcfac;
        AER(KA_DIMER, KM_ACC) = var[KQ_L_DIMER] * invcfac;
        AER(KA_IMGA, KM_ACC) = var[KQ_L_IMGA] * invcfac;
        AER(KA_IMOS, KM_ACC) = var[KQ_L_IMOS] * invcfac;
    } else {
        AER(KA_ISO3, KM_ACC) = (var[KQ_L_ISO3]) * invcfac;
    }
    const double soilc2 = AER(KA_SOILC, KM_COR), anthc2 = AER(KA_ANTHC, KM_COR), seasc2 = AER(KA_SEASC, KM_COR);
    fecor = fac[KF_SOIL_FE] * soilc2 + fac[KF_CORS_FE] * anthc2;
    mncor = fac[KF_SOIL_MN] * soilc2 + fac[KF_CORS_MN] * anthc2;
    nacor = fac[KF_SEAS_NA] * seasc2 + fac[KF_SOIL_NA] * soilc2 + fac[KF_CORS_NA] * anthc2;
    mgcor = fac[KF_SEAS_MG] * seasc2 + fac[KF_SOIL_MG] * soilc2 + fac[KF_CORS_MG] * anthc2;
    cacor = fac[KF_SEAS_CA] * seasc2 + fac[KF_SOIL_CA] * soilc2 + fac[KF_CORS_CA] * anthc2;
    kcor = fac[KF_SEAS_K] * seasc2 + fac[KF_SOIL_K] * soilc2 + fac[KF_CORS_K] * anthc2;
    AER(KA_FEACC, KM_ACC) = fmax((var[KQ_L_FEPLUS3] / fe_iii / fe_sol - fecor * cfactor) * invcfac, 0.0);
    AER(KA_MNACC, KM_ACC) = fmax((var[KQ_L_MNPLUS2] / mn_ii / mn_sol - mncor * cfactor) * invcfac, 0.0);
    AER(KA_NA, KM_ACC) = fmax((var[KQ_L_NAPLUS] - nacor * cfactor) * invcfac, 0.0);
    AER(KA_CAACC, KM_ACC) = fmax((var[KQ_L_CAPLUS2] - cacor * cfactor) * invcfac, 0.0);
    AER(KA_MGACC, KM_ACC) = fmax((var[KQ_L_MGPLUS2] - mgcor * cfactor) * invcfac, 0.0);
    AER(KA_KACC, KM_ACC) = fmax((var[KQ_L_KPLUS] - kcor * cfactor) * invcfac, 0.0);
    AER(KA_SO4, KM_ACC) = fmax(((var[KQ_L_H2SO4] + var[KQ_L_SO4MIN2] + var[KQ_L_HSO4MIN]) * invcfac)
                               - AER(KA_SO4, KM_COR), 0.0);
    AER(KA_CL, KM_ACC) = fmax((var[KQ_L_CLMIN] * invcfac) - AER(KA_CL, KM_COR), 0.0);
    totamm = var[KQ_G_NH3] + var[KQ_L_NH4OH] + var[KQ_L_NH4PLUS] - AER(KA_NH4, KM_COR) * cfactor;
    totnit = var[KQ_G_HNO3] + var[KQ_L_HNO3] + var[KQ_L_NO3MIN] - AER(KA_NO3, KM_COR) * cfactor;
    totamm = fmax(totamm, 0.0);
    totnit = fmax(totnit, 0.0);
    AER(KA_NO3, KM_ACC) = ((1.0 - fhno3) * totnit) * invcfac;
    AER(KA_NH4, KM_ACC) = ((1.0 - fnh3) * totamm) * invcfac;
    const double oliggly = 0.0 * 3.3e-1, oligmgly = 0.0 * 1.9e-1;   /* OLIG = 0 (aqchem_kmt.F90:412) */
    gas[KG_SO2] = (var[KQ_G_SO2] + var[KQ_L_SO2] + var[KQ_L_HSO3MIN] + var[KQ_L_SO3MIN2] + var[KQ_L_HMSMIN]
                   + var[KQ_L_SO3MIN] + var[KQ_L_SO5MIN] + var[KQ_L_HSO5MIN] + var[KQ_L_SO4MIN]) * invcfac;
    gas[KG_N2O5] = 0.0;
    gas[KG_CO2] = (var[KQ_G_CO2] + var[KQ_L_H2CO3] + var[KQ_L_HCO3MIN] + var[KQ_L_CO3MIN2] + var[KQ_L_CO2MIN])
                  * invcfac;
    gas[KG_H2O2] = (var[KQ_G_H2O2] + var[KQ_L_H2O2]) * invcfac;
    gas[KG_O3] = (var[KQ_G_O3] + var[KQ_L_O3]) * invcfac;
    gas[KG_FOA] = (var[KQ_G_HCOOH] + var[KQ_L_HCOOH] + var[KQ_L_HCOOMIN]) * invcfac;
    gas[KG_MHP] = (var[KQ_G_MHP] + var[KQ_L_MHP]) * invcfac;
    gas[KG_PAA] = (var[KQ_G_PAA] + var[KQ_L_PAA]) * invcfac;
    gas[KG_H2SO4] = 0.0;
    gas[KG_HCL] = (var[KQ_G_HCL] + var[KQ_L_HCL]) * invcfac;
    gas[KG_GLY] = (var[KQ_G_GLY] + var[KQ_L_GLY] * (1.0 - oliggly)) * invcfac;
    gas[KG_MGLY] = (var[KQ_G_MGLY] + var[KQ_L_MGLY] * (1.0 - oligmgly)) * invcfac;
    gas[KG_HNO3] = (fhno3 * totnit) * invcfac;
    gas[KG_NH3] = (fnh3 * totamm) * invcfac;
    gas[KG_HO] = (fixv[KQ_G_HO]) * invcfac;
    gas[KG_IEPOX] = (var[KQ_G_IEPOX] + var[KQ_L_IEPOX]) * invcfac;
    if (ispc8 > 0) {
        gas[KG_IMAE] = (var[KQ_G_IMAE] + var[KQ_L_IMAE]) * invcfac;
        gas[KG_IHMML] = (var[KQ_G_IHMML] + var[KQ_L_IHMML]) * invcfac;
    }
    gas[KG_HO2] = (var[KQ_G_HO2] + var[KQ_L_HO2] + var[KQ_L_O2MIN]) * invcfac;
    gas[KG_NO2] = (var[KQ_G_NO2] + var[KQ_L_NO2]) * invcfac;
    gas[KG_HONO] = (var[KQ_G_HONO] + var[KQ_L_HONO] + var[KQ_L_NO2MIN]) * invcfac;
    gas[KG_HNO4] = (var[KQ_G_HNO4] + var[KQ_L_HNO4] + var[KQ_L_NO4MIN]) * invcfac;
    gas[KG_NO3RAD] = (var[KQ_G_NO3] + var[KQ_L_NO3]) * invcfac;
    gas[KG_CH3O2] = (var[KQ_G_CH3O2] + var[KQ_L_CH3O2]) * invcfac;
    gas[KG_CCOOH] = (var[KQ_G_CCOOH] + var[KQ_L_CCOOH] + var[KQ_L_CCOOHMIN]) * invcfac;
    gas[KG_HCHO] = (var[KQ_G_HCHO] + var[KQ_L_CH2OHYD] + var[KQ_L_HCHO] + var[KQ_L_HMSMIN]) * invcfac;
    gas[KG_GCOL] = (var[KQ_G_GCOL] + var[KQ_L_GCOL]) * invcfac;
    gas[KG_HCHOP] = (var[KQ_G_HCHOP] + var[KQ_L_CH2OHYDP] + var[KQ_L_HCHOP] + var[KQ_L_HMSMINP]) * invcfac;
    gwd[KG_SO2] = var[KQ_WD_SO2];
    gwd[KG_HNO3] = var[KQ_WD_HNO3];
    gwd[KG_N2O5] = 0.0;
    gwd[KG_CO2] = var[KQ_WD_CO2];
    gwd[KG_NH3] = var[KQ_WD_NH4OH];
    gwd[KG_H2O2] = var[KQ_WD_H2O2];
    gwd[KG_O3] = var[KQ_WD_O3];
    gwd[KG_FOA] = var[KQ_WD_HCOOH];
    gwd[KG_MHP] = var[KQ_WD_MHP];
    gwd[KG_PAA] = var[KQ_WD_PAA];
    gwd[KG_H2SO4] = 0.0;
    gwd[KG_HCL] = var[KQ_WD_HCL];
    gwd[KG_GLY] = var[KQ_WD_GLY] * (1.0 - oliggly);
    gwd[KG_MGLY] = var[KQ_WD_MGLY] * (1.0 - oligmgly);
    gwd[KG_HO] = var[KQ_WD_HO];
    gwd[KG_IEPOX] = var[KQ_WD_IEPOX];
    if (ispc8 > 0) {
        gwd[KG_IMAE] = var[KQ_WD_IMAE];
        gwd[KG_IHMML] = var[KQ_WD_IHMML];
    }
    gwd[KG_NO2] = var[KQ_WD_NO2];
    gwd[KG_HONO] = var[KQ_WD_HONO];
    gwd[KG_HNO4] = var[KQ_WD_HNO4];
    gwd[KG_NO3RAD] = var[KQ_WD_NO3];
    gwd[KG_CH3O2] = var[KQ_WD_CH3O2];
    gwd[KG_GCOL] = var[KQ_WD_GCOL];
    gwd[KG_CCOOH] = var[KQ_WD_CCOOH];
    gwd[KG_HCHO] = var[KQ_WD_CH2OHYD];
    gwd[KG_HO2] = var[KQ_WD_HO2];
    gwd[KG_HCHOP] = var[KQ_WD_CH2OHYDP];
    double apyrac = 0.0, wdpyrac = 0.0;
    if (mtpyrac > 0) {
        gas[KG_PYRUV] = (var[KQ_G_PYRAC] + var[KQ_L_PYRAC]) * invcfac;
        gwd[KG_PYRUV] = var[KQ_WD_PYRAC];
        wdpyrac = 0.0;
        apyrac = var[KQ_L_PYRACMIN];
    } else {
        wdpyrac = var[KQ_WD_PYRAC];
        apyrac = var[KQ_L_PYRAC] + var[KQ_L_PYRACMIN];
    }
    const double r7404 = (double)(74.04f / 177.0f), r9003 = (double)(90.03f / 177.0f);
    const double r8806 = (double)(88.06f / 177.0f), r7605 = (double)(76.05f / 177.0f);
    const double r5804 = (double)(58.04f / 177.0f), r7206 = (double)(72.06f / 177.0f);
    AER(KA_ORGC, KM_ACC) = (var[KQ_L_ORGC] + (r7404 * var[KQ_L_GLYAC]) + (r9003 * var[KQ_L_OXLAC])
                            + (r9003 * var[KQ_L_OXLACMIN]) + (r9003 * var[KQ_L_OXLACMIN2]) + (r8806 * apyrac)
                            + (r7605 * var[KQ_L_GCOLAC]) + (r7404 * var[KQ_L_GLYACMIN])
                            + (r7605 * var[KQ_L_GCOLACMIN])
                            + r5804 * oliggly * var[KQ_L_GLY] + r7206 * oligmgly * var[KQ_L_MGLY]) * invcfac;
    AWD(KA_ORGC, KM_ACC) = var[KQ_WD_ORGC] + (r7404 * var[KQ_WD_GLYAC]) + (r9003 * var[KQ_WD_OXLAC])
                           + (r8806 * wdpyrac) + (r7605 * var[KQ_WD_GCOLAC])
                           + r5804 * oliggly * var[KQ_WD_GLY] + r7206 * oligmgly * var[KQ_WD_MGLY];
    for (int i = 0; i < KG_NGAS; ++i) gwd[i] = gwd[i] * wfactor;
    for (int i = 0; i < naer * 3; ++i) awd[i] = awd[i] * wfactor;
    for (int i = 0; i < KG_NGAS; ++i) {
        if (gas[i] < 0.0) gas[i] = 0.0;
        if (gwd[i] < 0.0) gwd[i] = 0.0;
    }
    for (int i = 0; i < naer * 3; ++i) {
        if (aer[i] < 0.0) aer[i] = 0.0;
        if (awd[i] < 0.0) awd[i] = 0.0;
    }
    out[KO_HPWDEP] = (double)(float)(var[KQ_WD_HPLUS] * wfactor);   /* HPWDEP is REAL */
    const double depsum = AWD(KA_SO4, KM_ACC) / wfactor;
    const double betaso4 = AER(KA_SO4, KM_ACC) * cfactor + depsum > 0.0
                               ? depsum / (AER(KA_SO4, KM_ACC) * cfactor + depsum) / (double)taucld : 0.0;
    out[KO_BETASO4] = betaso4;
    AER(KA_NUM, KM_ACC) = AER(KA_NUM, KM_ACC) * portable_exp(-betaso4 * (double)taucld);
    /* :919-973: mass balance at the end */
    double endm[4];
    endm[0] = (gas[KG_SO2] + gas[KG_H2SO4] + (gwd[KG_SO2] + gwd[KG_H2SO4]) / wfactor / cfactor) * w_s;
    endm[1] = (gas[KG_HNO3] + 2 * gas[KG_N2O5] + gas[KG_NO2] + gas[KG_HONO] + gas[KG_HNO4] + gas[KG_NO3RAD]
               + (gwd[KG_HNO3] + gwd[KG_NO2] + gwd[KG_HONO] + gwd[KG_HNO4] + gwd[KG_NO3RAD]) / wfactor / cfactor)
              * w_n;
    endm[2] = (gas[KG_NH3] + gwd[KG_NH3] / wfactor / cfactor) * w_n;
    endm[3] = (gas[KG_HCL] + gwd[KG_HCL] / wfactor / cfactor) * w_cl;
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
    for (int i = 0; i < 4; ++i) out[KO_MBAL + i] = startm[i] > 0.0 ? 100 * (startm[i] - endm[i]) / startm[i] : 0.0;
    return fail;
#undef AER
#undef AWD
}

/* ------------------------------------------------------------------ exports */
int oracle_kq_sizes(int* out)
{
    out[0] = KQ_NVAR;
    out[1] = KQ_NFIX;
    out[2] = KQ_NREACT;
    out[3] = KQ_LU_NONZERO;
    out[4] = KQ_NB;
    out[5] = KQ_NHENRY;
    out[6] = KQ_NPARAM;
    out[7] = KQ_NSTAT;
    return 0;
}

const char* oracle_kq_name(int i) { return (i >= 0 && i < KQ_NVAR + KQ_NFIX) ? kq_names[i] : ""; }

int oracle_kq_lu_structure(int* icol, int* crow, int* diag)
{
    memcpy(icol, kq_lu_icol, sizeof(kq_lu_icol));
    memcpy(crow, kq_lu_crow, sizeof(kq_lu_crow));
    memcpy(diag, kq_lu_diag, sizeof(kq_lu_diag));
    return 0;
}

/* Set-up of one cell: var (molec/cm3), fix, rconst after Initialize and one
 * Update_RCONST, henry[KQ_NHENRY]; scalars = {phi2, cfactor, stion, gm1, gm2, wetfac,
 * delinvt, tend}. */
int oracle_kq_setup(const double* p, const double* var_mix, double* var, double* fix, double* rconst, double* henry,
                    double* scalars)
{
    KqState s;
    const int rc = kq_setup(p, var_mix, &s, var);
    if (rc != 0) return rc;
    kq_update_rconst(&s, var);
    memcpy(fix, s.fix, sizeof(s.fix));
    memcpy(rconst, s.rconst, sizeof(s.rconst));
    memcpy(henry, s.henry, sizeof(s.henry));
    const double sc[8] = {s.phi2, s.cfactor, s.stion, s.gm1, s.gm2, s.wetfac, s.delinvt, s.tend};
    memcpy(scalars, sc, sizeof(sc));
    return 0;
}

/* Update_RCONST for a given state after the set-up of p / var_mix (for the rate tests). */
int oracle_kq_rconst_at(const double* p, const double* var_mix, const double* var, double* rconst)
{
    KqState s;
    double v0[KQ_NVAR];
    const int rc = kq_setup(p, var_mix, &s, v0);
    if (rc != 0) return rc;
    kq_update_rconst(&s, var);
    memcpy(rconst, s.rconst, sizeof(s.rconst));
    return 0;
}

void oracle_kq_fun(const double* var, const double* fix, const double* rconst, double* vdot)
{
    double a[KQ_NREACT];
    kq_fun(var, fix, rconst, a, vdot);
}

void oracle_kq_jac(const double* var, const double* fix, const double* rconst, double* jvs)
{
    double b[KQ_NB];
    kq_jac(var, fix, rconst, b, jvs);
}

int oracle_kq_decomp(double* jvs) { return kq_decomp(jvs); }

void oracle_kq_set_rtol_scale(double scale) { kq_rtol_scale = scale; }

/* The generated straight-line routines (gen/kmt2_aq_unrolled.c), the form of the device
 * code, for the tests that hold them to the table-driven ones bit for bit. */
void oracle_kq_fun_unrolled(const double* var, const double* fix, const double* rconst, double* vdot)
{
    kqu_fun(var, fix, rconst, vdot);
}
void oracle_kq_jac_unrolled(const double* var, const double* fix, const double* rconst, double* jvs)
{
    kqu_jac(var, fix, rconst, jvs);
}
int oracle_kq_decomp_unrolled(double* jvs) { return kqu_decomp(jvs); }
void oracle_kq_solve_unrolled(const double* jvs, double* x) { kqu_solve(jvs, x); }

void oracle_kq_solve(const double* jvs, double* x) { kq_solve(jvs, x); }

/* Integrate ncell cells: params[ncell][KQ_NPARAM], var_mix[ncell][KQ_NVAR] in; var_out
 * [ncell][KQ_NVAR], fix_out [ncell][KQ_NFIX] (may be NULL), stats [ncell][KQ_NSTAT].
 * Returns the number of cells that did not finish. */
int oracle_kq_cells(long long ncell, const double* params, const double* var_mix, double* var_out, double* fix_out,
                    int* stats, int threads)
{
    int nfail = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : 1) reduction(+ : nfail)
    {
        static __thread KqWork w;
#pragma omp for schedule(dynamic, 1)
        for (long long c = 0; c < ncell; ++c)
            nfail += kq_cell(&params[c * KQ_NPARAM], &var_mix[c * KQ_NVAR], &var_out[c * KQ_NVAR],
                             fix_out ? &fix_out[c * KQ_NFIX] : NULL, &stats[c * KQ_NSTAT], &w);
    }
    return nfail;
}

/* AQCHEM for ncell cells: params [ncell][KQ_NPARAM]; gas [ncell][29] and aer [ncell][naer * 3]
 * in and out; aer_index [31] positions of the surrogates in the caller's aerosol list;
 * factors [16]; gas_wdep [ncell][29], aer_wdep [ncell][naer * 3], out [ncell][10], stats
 * [ncell][KQ_NSTAT] out.  Returns the number of cells that did not finish. */
int oracle_kq_aqchem_cells(long long ncell, const double* params, double* gas, double* aer, int naer,
                           const int* aer_index, const double* factors, double* gas_wdep, double* aer_wdep,
                           double* out, int* stats, int threads)
{
    int nfail = 0;
#pragma omp parallel num_threads(threads > 0 ? threads : 1) reduction(+ : nfail)
    {
        static __thread KqWork w;
#pragma omp for schedule(dynamic, 1)
        for (long long c = 0; c < ncell; ++c)
            nfail += kq_aqchem_cell(&params[c * KQ_NPARAM], &gas[c * KG_NGAS], &aer[c * naer * 3], naer, aer_index,
                                    factors, &gas_wdep[c * KG_NGAS], &aer_wdep[c * naer * 3], &out[c * KO_N],
                                    &stats[c * KQ_NSTAT], &w);
    }
    return nfail;
}
