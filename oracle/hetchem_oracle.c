/* CPU oracle of CMAQ's heterogeneous rate constants KHETERO (test infrastructure).
 *
 * Restates, per grid cell, HETCHEM_RATES (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:282-1535)
 * for the mechanism of gen/<mech>_hetchem.h (cb6r5_ae7_aq, cracmm2), with the aerosol-state
 * routines it calls, each as a function of the same name over a per-cell copy of the
 * AERO_DATA module state:
 *
 *   extract_aero     AERO_DATA.F:1296-1420 (minchk = .TRUE.)
 *   calcmoments      AERO_DATA.F:1575-1699 (both branches)
 *   getpar           getpar.f (FIXED_sg of AERO_DATA, .FALSE.)
 *   hetchem_extract_aero  aero_subs.F:3052-3135 (the wet moments and diameters)
 *   n2o5_gamma       AEROSOL_CHEMISTRY.F:1649-2044 (every GPARAM; HETCHEM_RATES uses 0, 5)
 *   crystalized, freezes  :2047-2179, :2182-2282
 *   pncom_loss       :1539-1646
 *   calcisopgammas   :2285-2555
 *   hetchem_rates    :862-1302, the cell loop, for the KHETERO labels of the mechanism
 *
 * Arithmetic follows the reference's Fortran: REAL(4) variables, literals and
 * intermediates as float, REAL(8) as double, the same operation order; the C math
 * library's functions of the matching kind for the intrinsics (logf / expf / powf /
 * sqrtf for REAL, log / exp / pow / sqrt / tanh / log10 for REAL(8)).  No reference
 * outputs exist here for this routine (no Fortran compiler); tests/test_oracle_hetchem.py
 * pins its pieces against the reference's formulas restated independently in Python.
 */
#include <math.h>
#include <string.h>

/* the mechanism's tables: HO_TABLES names gen/<mech>_hetchem.h (oracle/build.py builds one
 * library per mechanism) */
#ifndef HO_TABLES
#define HO_TABLES "gen/cb6r5_ae7_aq_hetchem.h"
#endif
#include HO_TABLES

/* CONST.EXT, AEROMET_DATA, AERO_DATA parameters */
static const float PI_F = 3.14159265f;
static const double DPI_D = 3.14159265358979324;
static const float RGASUNIV_F = 8.314510f, STDATMPA_F = 101325.0f, STDTEMP_F = 273.15f, MWAIR_F = 28.9628f,
                   MWWAT_F = 18.0153f;
static const float MIN_SIGMA_G_F = 1.05f, MAX_SIGMA_G_F = 2.5001f;
static const float AEROMODE_MIN_F = 1.0e-23f;   /* min_numconc = min_m2conc = min_m3conc = conmin */

/* per-cell copy of the AERO_DATA module variables HETCHEM touches */
typedef struct {
    float aerospc_conc[HO_NSPC][3];
    float moment0_conc[3], moment2_conc[3], moment3_conc[3];
    float aeromode_diam[3], aeromode_lnsg[3], aeromode_mass[3], aeromode_dens[3];
    int wet_moments_flag;
    double wet_m2[3], wet_m3[3], de_wet[3];   /* AEROSOL_CHEMISTRY's WET_M2, WET_M3, DE_WET */
} HoState;

static int ho_missing(int spc, int m) { return ho_row[spc * 3 + m] < 0; }
static float f6pi(void) { return 6.0f / PI_F; }

static void extract_aero(HoState* s, const float* conc, long long stride)
{
    for (int spc = 0; spc < HO_NSPC; ++spc)
        for (int m = 0; m < 3; ++m) s->aerospc_conc[spc][m] = 0.0f;
    for (int m = 0; m < 3; ++m)
        for (int spc = 0; spc < HO_NSPC; ++spc) {
            const int n = ho_row[spc * 3 + m];
            if (n >= 0) {
                const float c = conc[n * stride], lo = ho_min_conc[spc * 3 + m];
                s->aerospc_conc[spc][m] = c > lo ? c : lo;
            }
        }
    for (int m = 0; m < 3; ++m) {   /* dry third moment */
        float sum = 0.0f;
        for (int spc = 0; spc < HO_NSPC; ++spc)
            if (!ho_no_m2wet[spc] && !ho_tracer[spc]) sum += s->aerospc_conc[spc][m] / ho_density[spc];
        const float v = sum * 1.0e-9f * f6pi();
        s->moment3_conc[m] = v > AEROMODE_MIN_F ? v : AEROMODE_MIN_F;
    }
    for (int m = 0; m < 3; ++m) {
        const float n0 = conc[ho_num_row[m] * stride], n2 = conc[ho_srf_row[m] * stride] / PI_F;
        s->moment0_conc[m] = n0 > AEROMODE_MIN_F ? n0 : AEROMODE_MIN_F;
        s->moment2_conc[m] = n2 > AEROMODE_MIN_F ? n2 : AEROMODE_MIN_F;
    }
    s->wet_moments_flag = 0;
}

static void calcmoments(HoState* s, int addwet)
{
    const double two3rds = 2.0 / 3.0;
    float m2[3], m3[3];
    for (int n = 0; n < 3; ++n) {
        const float initial_m2 = s->moment2_conc[n];
        const float initial_m3 = s->moment3_conc[n] > AEROMODE_MIN_F ? s->moment3_conc[n] : AEROMODE_MIN_F;
        double summ3 = 0.0;
        for (int spc = 0; spc < HO_NSPC; ++spc) {
            if (ho_tracer[spc] || ho_missing(spc, n)) continue;
            if (!addwet && ho_no_m2wet[spc]) continue;
            const double factor = (double)(1.0e-9f * f6pi() / ho_density[spc]);
            summ3 = summ3 + factor * (double)s->aerospc_conc[spc][n];
        }
        m3[n] = (float)summ3 > AEROMODE_MIN_F ? (float)summ3 : AEROMODE_MIN_F;
        const int rescale = addwet ? !s->wet_moments_flag : s->wet_moments_flag;
        m2[n] = rescale ? initial_m2 * powf((float)summ3 / initial_m3, (float)two3rds) : initial_m2;
    }
    for (int n = 0; n < 3; ++n) {
        s->moment2_conc[n] = m2[n];
        s->moment3_conc[n] = m3[n];
    }
    s->wet_moments_flag = addwet;
}

static void getpar(HoState* s, int fixed_sg)
{
    const double one3d = 1.0 / 3.0, two3d = 2.0 / 3.0;
    const float one3 = 1.0f / 3.0f, densmin = 1.0e03f;
    const double minl2sg = (double)(logf(MIN_SIGMA_G_F) * logf(MIN_SIGMA_G_F));
    const double maxl2sg = (double)(logf(MAX_SIGMA_G_F) * logf(MAX_SIGMA_G_F));
    for (int n = 0; n < 3; ++n) {
        double sum_m3 = 0.0, sum_mass = 0.0;
        for (int spc = 0; spc < HO_NSPC; ++spc) {
            if (ho_tracer[spc] || ho_missing(spc, n) || (ho_no_m2wet[spc] && !s->wet_moments_flag)) continue;
            const double factor = (double)(1.0e-9f * f6pi() / ho_density[spc]);
            const double mass = (double)s->aerospc_conc[spc][n];
            sum_m3 = sum_m3 + factor * mass;
            sum_mass = sum_mass + mass;
        }
        s->moment3_conc[n] = (float)sum_m3 > AEROMODE_MIN_F ? (float)sum_m3 : AEROMODE_MIN_F;
        s->aeromode_mass[n] = (float)sum_mass;
    }
    for (int n = 0; n < 3; ++n) {
        const float d = 1.0e-9f * f6pi() * s->aeromode_mass[n] / s->moment3_conc[n];
        s->aeromode_dens[n] = d < densmin ? densmin : d;
    }
    for (int n = 0; n < 3; ++n) {
        const double xxm0 = (double)s->moment0_conc[n], xxm3 = (double)s->moment3_conc[n];
        const double xfsum = one3d * log(xxm0) + two3d * log(xxm3);
        double l2sg;
        if (fixed_sg) {
            l2sg = (double)(s->aeromode_lnsg[n] * s->aeromode_lnsg[n]);
        } else {
            const double lxfm2 = log((double)s->moment2_conc[n]);
            l2sg = xfsum - lxfm2;
            if (l2sg < minl2sg) l2sg = minl2sg;
            if (l2sg > maxl2sg) l2sg = maxl2sg;
        }
        const double lxfm2 = xfsum - l2sg;
        s->moment2_conc[n] = (float)exp(lxfm2);
        s->aeromode_lnsg[n] = (float)sqrt(l2sg);
        const float es36 = (float)exp(4.5 * l2sg);
        const float lim = s->moment3_conc[n] / (1.0e-12f * es36);
        if (lim > s->moment0_conc[n]) s->moment0_conc[n] = lim;
        s->aeromode_diam[n] = powf(s->moment3_conc[n] / (s->moment0_conc[n] * es36), one3);
    }
}

static void hetchem_extract_aero(HoState* s, const float* conc, long long stride)
{
    extract_aero(s, conc, stride);
    calcmoments(s, 1);
    getpar(s, 0);
    for (int n = 0; n < 3; ++n) {
        s->wet_m3[n] = (double)s->moment3_conc[n];
        s->wet_m2[n] = (double)s->moment2_conc[n];
        const float lnsg2 = s->aeromode_lnsg[n] * s->aeromode_lnsg[n];
        s->de_wet[n] = (double)(s->aeromode_diam[n] * expf(1.5f * lnsg2));
    }
}

static int crystalized(const HoState* s, double rh, int complete)
{
    if (rh <= 0.01) return 1;
    if (rh > 0.351) return 0;
    const float nno3 = (s->aerospc_conc[HO_ANO3][0] + s->aerospc_conc[HO_ANO3][1]) / ho_molwt[HO_ANO3];
    const float nso4 = (s->aerospc_conc[HO_ASO4][0] + s->aerospc_conc[HO_ASO4][1]) / ho_molwt[HO_ASO4];
    const float nnh4 = (s->aerospc_conc[HO_ANH4][0] + s->aerospc_conc[HO_ANH4][1]) / ho_molwt[HO_ANH4];
    const float other = 2.0f * nso4 + nno3;
    const float ncat = nnh4 > other ? nnh4 : other;
    const float nani = nno3 + nso4;
    const float x = nnh4 / ncat, y = nso4 / nani;
    if (x < 0.50f || y < 0.22f) return 0;
    const float x2 = x * x, xy = x * y, x2y = x2 * y, y2 = y * y, xy2 = x * y2;
    const float rden = 1.0f / (25.0f + (x - 0.7f) * (y - 0.5f));
    float crh;
    if (complete)
        crh = 3143.44f + (63.07f * x) + (0.114f * x2) + (87.97f * y) - (125.73f * xy) + (0.586f * x2y)
            + (0.95f * y2) - (1.384f * xy2) - (79692.5f * rden);
    else
        crh = -697.908f - (15.351f * x) + (0.43f * x2) - (22.11f * y) + (33.882f * xy) - (1.818f * x2y)
            + (0.772f * y2) - (1.636f * xy2) + (17707.6f * rden);
    return rh <= (double)crh;
}

static int freezes(double temp, double rh)
{
    const double tst = 373.16, t0 = 273.16, logpst = 3.0057149, logp0 = 0.78583503;
    if (!(temp < t0)) return 0;
    const double eirh = 1.61299 + temp * (4.4117437e-5 * temp - 1.4293888e-2);
    const double lirh = eirh - 0.005, uirh = eirh + 0.005;
    if (rh > uirh) return 1;
    if (rh < lirh) return 0;
    const double tsdt = tst / temp, tdts = temp / tst, t0dt = t0 / temp, tdt0 = temp / t0;
    const double logpw = -7.90298 * (tsdt - 1.0) + 5.02808 * log10(tsdt)
                       - 1.3816e-7 * (pow(10.0, 11.344 * (1.0 - tdts)) - 1.0)
                       + 8.1328e-3 * (pow(10.0, -3.49149 * (tsdt - 1.0)) - 1.0) + logpst;
    const double logpi = -9.09718 * (t0dt - 1.0) - 3.56654 * log10(t0dt) + .876793 * (1.0 - tdt0) + logp0;
    return rh > pow(10.0, logpi - logpw);
}

static float logitinv(float xx) { return 1.0f / (1.0f + expf(-xx)); }
static float minf_(float a, float b) { return a < b ? a : b; }
static float maxf_(float a, float b) { return a > b ? a : b; }

static double n2o5_gamma(const HoState* s, double temp, double rh, int gparam)
{
    const float anh4 = s->aerospc_conc[HO_ANH4][0] + s->aerospc_conc[HO_ANH4][1];
    const float ano3 = s->aerospc_conc[HO_ANO3][0] + s->aerospc_conc[HO_ANO3][1];
    const float aso4 = s->aerospc_conc[HO_ASO4][0] + s->aerospc_conc[HO_ASO4][1];
    const float ah2of = s->aerospc_conc[HO_AH2O][0] + s->aerospc_conc[HO_AH2O][1];
    const float aclf = s->aerospc_conc[HO_ACL][0] + s->aerospc_conc[HO_ACL][1];
    const float ano3f = ano3;
    const float ah2ok = s->aerospc_conc[HO_AH2O][2], aclk = s->aerospc_conc[HO_ACL][2];
    const float ano3k = s->aerospc_conc[HO_ANO3][2];
    const float A = 3.2e-08f, BETA_BT = 1.15e06f, DELTA = 1.3e-01f, K3OK2B = 6.0e-02f, K4OK2B = 29.0f;
    if (gparam == 1) return 0.1;
    if (gparam == 2 || gparam == 3) {
        float gamma1;
        if (gparam == 2) {
            gamma1 = 0.02f;
        } else {
            const float alpha = 2.79e-04f + (float)(rh * (1.3e-02 + rh * (-3.43e-02 + 7.52e-02 * rh)));
            if (temp < 282.0) gamma1 = 3.0199517f * alpha;
            else gamma1 = alpha * powf(10.0f, 0.04f * (294.0f - (float)temp));
        }
        const float fracso4 = ano3 > 0.0f ? aso4 / (aso4 + ano3) : 1.0f;
        const float gamma2 = 0.1f * gamma1;
        return (double)(gamma2 + fracso4 * (gamma1 - gamma2));
    }
    if (gparam == 4 || gparam == 5) {
        const float inv_vol = gparam == 4 ? 1.0e-9f * f6pi() / (float)(s->wet_m3[0] + s->wet_m3[1])
                                          : 1.0e-9f * f6pi() / (float)s->wet_m3[2];
        const float h2o = gparam == 4 ? ah2of : ah2ok, cl = gparam == 4 ? aclf : aclk;
        const float no3 = gparam == 4 ? ano3f : ano3k;
        const float ah2om = h2o * inv_vol / ho_molwt[HO_AH2O];
        const float aclm = cl * inv_vol / ho_molwt[HO_ACL];
        const float ano3m = no3 * inv_vol / ho_molwt[HO_ANO3];
        const float k2fp = BETA_BT - BETA_BT * expf(-DELTA * ah2om);
        const float den1 = K3OK2B * (ah2om / ano3m);
        const float den2 = K4OK2B * (aclm / ano3m);
        const float den = den1 + 1.0f + den2;
        return (double)(A * k2fp * (1.0f - 1.0f / den));
    }
    const int crystal = crystalized(s, rh, 1);
    const int frozen = freezes(temp, rh);
    if (frozen) return 0.02;
    const float nno3 = ano3 / ho_molwt[HO_ANO3], nso4 = aso4 / ho_molwt[HO_ASO4], nnh4 = anh4 / ho_molwt[HO_ANH4];
    const float nani = nno3 + nso4;
    const float x3 = nno3 / nani;
    const float x2 = maxf_(0.0f, minf_(1.0f - x3, nnh4 / nani - 1.0f));
    const float x1 = 1.0f - (x2 + x3);
    const float lam3 = -8.10774f + 4.902f * (float)rh;
    const float gam3 = minf_(logitinv(lam3), 0.0154f);
    if (crystal) {
        const float t293 = maxf_(0.0f, (float)temp - 293.0f);
        const float lamd = -6.13376f + 3.592f * (float)rh - 0.19688f * t293;
        const float gamd = minf_(logitinv(lamd), 0.0124f);
        return (double)((x1 + x2) * gamd + x3 * minf_(gamd, gam3));
    }
    const float t291 = maxf_(0.0f, (float)temp - 291.0f);
    const float rh46 = minf_(0.0f, (float)rh - 0.46f);   /* APNDX = .TRUE. */
    const float lam2 = -3.64849f + 9.553f * rh46;
    const float lam1 = lam2 + 0.97579f - 0.20427f * t291;
    const float gam1 = minf_(logitinv(lam1), 0.08585f);
    const float gam2 = minf_(logitinv(lam2), 0.053f);
    return (double)((x1 * gam1) + (x2 * gam2) + (x3 * gam3));
}

static double pncom_loss(float poc, float pncom)
{
    const double KOHEFF = 2.5e-12, MAX_RATE = 15.0 / 16.0 * KOHEFF;
    const float LOWER = 7.0f / 6.0f, UPPER = 11.0f / 3.0f;
    if (poc <= 1.0e-30) return 0.0;
    const double ratio = (double)((poc + pncom) / poc);
    if (ratio > LOWER && ratio < UPPER) return 15.0 * KOHEFF / (16.0 + (UPPER - ratio) / (ratio - LOWER));
    if (ratio >= UPPER) return MAX_RATE;
    return 0.0;
}

/* CALCISOPGAMMAS for the IEPOX parent (NUMVOC = 1 for this mechanism's pair table); *q_out
 * (if given) receives the diffuso-reactive parameter q */
static void calcisopgammas_q(const HoState* s, double radius, double temperature, double cfactor_iepox,
                             double* gammaiepox, double* kpiepox, double* ftet, double* fos, double* q_out);
static void calcisopgammas(const HoState* s, double radius, double temperature, double cfactor_iepox,
                           double* gammaiepox, double* kpiepox, double* ftet, double* fos)
{
    calcisopgammas_q(s, radius, temperature, cfactor_iepox, gammaiepox, kpiepox, ftet, fos, NULL);
}
static void calcisopgammas_q(const HoState* s, double radius, double temperature, double cfactor_iepox,
                             double* gammaiepox, double* kpiepox, double* ftet, double* fos, double* q_out)
{
    const double inv_alpha = 1.0 / 0.02, diffusivity = 1.0e-9, RgasLatmmolK = 0.08206;
    double acidmolconc[2];
    const double eqlbh = s->aerospc_conc[HO_AH3OP][1] / ho_molwt[HO_AH3OP] * 1.0e-6;
    acidmolconc[0] = eqlbh > 0.0 ? eqlbh : 0.0;
    double charge = 0.0;
    for (int i = 0; i < HO_NSPC; ++i) {
        if (ho_tracer[i] || ho_missing(i, 1)) continue;
        charge = charge - (float)ho_charge[i] * s->aerospc_conc[i][1] / ho_molwt[i];
    }
    const double h = charge * 1.0e-6 - acidmolconc[0];
    acidmolconc[1] = h > 0.0 ? h : 0.0;
    double inv_volume = 0.0;
    for (int i = 0; i < HO_NSPC; ++i) {
        if (ho_tracer[i] || ho_missing(i, 1)) continue;
        inv_volume = inv_volume + (double)(s->aerospc_conc[i][1] / ho_density[i]);
    }
    inv_volume = 1.0e6 / inv_volume;
    double kparticle = 0.0, kchemos = 0.0, kchemtet = 0.0;
    for (int i = 0; i < HO_NNUC; ++i) {
        const int nm = ho_nuc_spc[i];
        double nuc = s->aerospc_conc[nm][1] / ho_molwt[nm] * 1.0e-6;
        const double acid = acidmolconc[ho_nuc_acid[i] - 1];
        if (ho_nuc_remove[i] >= 1) {
            nuc = nuc - acidmolconc[ho_nuc_remove[i] - 1];
            if (nuc < 0.0) nuc = 0.0;
        }
        const double kchem = ho_nuc_kchem[i] * nuc * acid * (inv_volume * inv_volume);
        kparticle = kparticle + kchem;
        if (ho_nuc_os[i]) kchemos = kchemos + kchem;
        else kchemtet = kchemtet + kchem;
    }
    const float temp = (float)temperature;
    const float tfac = (298.0f - temp) / (298.0f * temp);   /* HLCONST, EFFECTIVE = .FALSE. */
    const double heff = (double)(ho_hl_iepox_a * expf(ho_hl_iepox_e * tfac));
    const double q = radius * sqrt(kparticle / diffusivity);
    if (q_out) *q_out = q;
    if (q / tanh(q) > 1.0) {
        const double nu = cfactor_iepox * sqrt(temperature);
        const double denom = (inv_alpha + nu * radius
                              / (4.0 * heff * RgasLatmmolK * temperature * diffusivity * (q / tanh(q) - 1.0)));
        *gammaiepox = 1.0 / denom;
        *ftet = kchemtet / kparticle;
        *fos = kchemos / kparticle;
    } else {
        *gammaiepox = 0.0;
        *ftet = 0.0;
        *fos = 0.0;
    }
    *kpiepox = kparticle;
}

static int label_is(int irate, const char* name) { return strcmp(ho_hetero[irate], name) == 0; }

/* HETCHEM_RATES for one cell: conc[r * stride] is row r of the CGRID aerosol block */
static void hetchem_rates_cell(const float* conc, long long stride, float temp, float press, float wvapor, float dens,
                               double* khetero)
{
    const double AQUEOUS_FREQUENCY = 1.0e+9, INV_SQRT_MWN2O5 = 9.62161363758323e-2;
    const double INV_SQRT_MWCLNO3 = 1.012739360000e-1, COEF1 = 7.24382926227485e10;
    const double GAMMA_GLY = 2.9e-3, GAMMA_NO3 = 1.0e-3, GAMMA_HO2 = 0.2;
    const double STD_DIFF_N2O5 = 0.0855e-4, STD_DIFF_CLNO3 = 0.1014e-4;
    const float GPKG = 1.0e+03f;
    const float CFACTOR = 8.0f * GPKG * RGASUNIV_F / PI_F;
    const float INV_STDTEMP = 1.0f / STDTEMP_F, EPSWATER = MWWAT_F / MWAIR_F;
    const float ON_ALPHA1 = 0.34f, ON_ALPHA2 = 0.66f, ON_CSTAR1 = 0.73f, ON_CSTAR2 = 1000.0f;
    const float MIN_TOA = 0.0001f, KHON = 2.7778E-03f;
    const double INV_GAMMA_CLNO3_H2O = 1.0 / 0.024;
    const double AL = 610.94, BL = 17.625, CL = 243.04, DL = 1.0 / AL;
    /* first-pass constants (AEROSOL_CHEMISTRY.F:722-800) */
    const double inv_mwcl = (double)(1.0f / ho_molwt[HO_ACL]);
    const float mwclh2o = ho_molwt[HO_ACL] / ho_molwt[HO_AH2O];
    const float mwh2ocl = 1.0f / mwclh2o;
    const double cfactor_iepox = sqrt(8.0e3 * (double)RGASUNIV_F / (ho_mw_iepox * DPI_D));
    const double inv_mwaso4 = (double)(1.0f / ho_molwt[HO_ASO4]);
    const double cfactor_gly = sqrt(8.0e3 * (double)RGASUNIV_F / (ho_mw_gly * DPI_D));
    const double cfactor_mgly = sqrt(8.0e3 * (double)RGASUNIV_F / (ho_mw_mgly * DPI_D));
    const double cfactor_no3 = sqrt(8.0e3 * (double)RGASUNIV_F / (ho_mw_no3 * DPI_D));
    const double cfactor_ho2 = sqrt(8.0e3 * (double)RGASUNIV_F / (ho_mw_ho2 * DPI_D));

    HoState st;
    HoState* s = &st;
    hetchem_extract_aero(s, conc, stride);
    const double airtemp = (double)temp;
    const double h2ovp = (double)(press * wvapor / (EPSWATER + wvapor));
    double airrh = h2ovp * (DL * exp(BL * (273.15 - airtemp) / (airtemp - 273.15 + CL)));
    if (airrh > 0.99) airrh = 0.99;
    if (airrh < 0.005) airrh = 0.005;
    const double cbar_coeff = (double)sqrtf(CFACTOR * temp);
    const double adjust_diff = (double)(powf(temp * INV_STDTEMP, 1.75f) * (STDATMPA_F / press));
    const double ppm_factor = 1.0e-3 * (double)(MWAIR_F / dens);
    const double rfactor = 60.0 * COEF1 * (double)(press / temp);
    const double cbar = cbar_coeff * INV_SQRT_MWN2O5;
    const double cbargly = cfactor_gly * sqrt(airtemp);
    const double cbarmgly = cfactor_mgly * sqrt(airtemp);
    const double cbarno3 = cfactor_no3 * sqrt(airtemp);
    const double cbarho2 = cfactor_ho2 * sqrt(airtemp);
    const double cbar_clno3 = cbar_coeff * INV_SQRT_MWCLNO3;
    const double inv_diffusivity = 1.0 / (STD_DIFF_N2O5 * adjust_diff);
    const double inv_diff_clno3 = 1.0 / (STD_DIFF_CLNO3 * adjust_diff);
    double kn2o5[3], kno3[3], kgly[3], kmgly[3], kho2[3], cl_ppm[3], yield_clno2[3] = {0.0, 0.0, 0.0};
    double yieldij = 0.0;
    for (int n = 0; n < 3; ++n) {
        double gamma;
        if (n <= 1) gamma = n2o5_gamma(s, airtemp, airrh, 0);
        else gamma = n2o5_gamma(s, airtemp, airrh, 5);
        const double xxf = s->wet_m2[n] / (4.0 + 0.5 * s->de_wet[n] * gamma * cbar * inv_diffusivity);
        kn2o5[n] = gamma * xxf;
        kno3[n] = GAMMA_NO3 * s->wet_m2[n] / (4.0 + 0.5 * s->de_wet[n] * GAMMA_NO3 * cbarno3 * inv_diffusivity)
                * cbarno3 * DPI_D;
        kgly[n] = GAMMA_GLY * s->wet_m2[n] / (4.0 + 0.5 * s->de_wet[n] * GAMMA_GLY * cbargly * inv_diffusivity)
                * cbargly * DPI_D;
        kmgly[n] = 0.09f * GAMMA_GLY * s->wet_m2[n]
                 / (4.0 + 0.5 * s->de_wet[n] * 0.09f * GAMMA_GLY * cbarmgly * inv_diffusivity) * cbarmgly * DPI_D;
        kho2[n] = GAMMA_HO2 * s->wet_m2[n] / (4.0 + 0.5 * s->de_wet[n] * GAMMA_HO2 * cbarho2 * inv_diffusivity)
                * cbarho2 * DPI_D;
        const float ah2o = s->aerospc_conc[HO_AH2O][n], acl = s->aerospc_conc[HO_ACL][n];
        cl_ppm[n] = ppm_factor * (acl * inv_mwcl);
        if (ah2o > 5.0e-01f && acl > 1.0e-04f) {
            if (mwh2ocl * acl > 1.0e-4f * ah2o)
                yield_clno2[n] = 1.0 / (1.0 + (1.0 / 483.0) * (ah2o / acl) * mwclh2o);
        }
    }
    {
        const float ah2o = s->aerospc_conc[HO_AH2O][0] + s->aerospc_conc[HO_AH2O][1];
        const float acl = s->aerospc_conc[HO_ACL][0] + s->aerospc_conc[HO_ACL][1];
        if (ah2o > 5.0e-01f && acl > 1.0e-04f) {
            if (mwh2ocl * acl > 1.0e-4f * ah2o) yieldij = 1.0 / (1.0 + (1.0 / 483.0) * (double)((ah2o / acl) * mwclh2o));
        }
    }
    for (int n = 0; n < 3; ++n) kn2o5[n] = cbar * DPI_D * kn2o5[n];
    const double totsurfa = (s->wet_m2[0] + s->wet_m2[1]) * DPI_D;
    const double radius_i = 0.5 * s->de_wet[0], radius = 0.5 * s->de_wet[1];
    const double clno3_h2o_rxn_time = 4.0 * INV_GAMMA_CLNO3_H2O / cbar_clno3;
    const double cbariepox = cfactor_iepox * sqrt(airtemp);
    double gammaiepox, kpiepox, fh2o, fos;
    calcisopgammas(s, radius, airtemp, cfactor_iepox, &gammaiepox, &kpiepox, &fh2o, &fos);
    double kiepox, aso4j_ppm;
    if (gammaiepox > 1.0e-72) {
        kiepox = s->wet_m2[1] * DPI_D / (radius * inv_diffusivity + 4.0 / (cbariepox * gammaiepox));
        aso4j_ppm = ppm_factor * (double)s->aerospc_conc[HO_ASO4][1] * inv_mwaso4;
    } else {
        kiepox = 0.0;
        aso4j_ppm = 0.0;
    }
    for (int irate = 0; irate < HO_NHET; ++irate) {
        double k = 0.0;
        if (label_is(irate, "HETERO_N2O5IJ")) {
            k = 60.0 * (kn2o5[0] + kn2o5[1]);
        } else if (label_is(irate, "HETERO_N2O5K")) {
            k = 60.0 * kn2o5[2];
        } else if (label_is(irate, "HETERO_H2NO3PAIJ")) {
            const double y = 1.0 - yieldij;
            k = 60.0 * AQUEOUS_FREQUENCY * (y > 0.0 ? y : 0.0);
        } else if (label_is(irate, "HETERO_H2NO3PBIJ")) {
            k = yieldij > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * yieldij / (cl_ppm[0] + cl_ppm[1]) : 0.0;
        } else if (label_is(irate, "HETERO_H2NO3PAK")) {
            const double y = 1.0 - yield_clno2[2];
            k = 60.0 * AQUEOUS_FREQUENCY * (y > 0.0 ? y : 0.0);
        } else if (label_is(irate, "HETERO_H2NO3PBK")) {
            k = yield_clno2[2] > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * yield_clno2[2] / cl_ppm[2] : 0.0;
        } else if (label_is(irate, "HETERO_PNCOMLI")) {
            k = rfactor * pncom_loss(s->aerospc_conc[HO_APOC][0], s->aerospc_conc[HO_APNCOM][0]);
        } else if (label_is(irate, "HETERO_PNCOMLJ")) {
            k = rfactor * pncom_loss(s->aerospc_conc[HO_APOC][1], s->aerospc_conc[HO_APNCOM][1]);
        } else if (label_is(irate, "HETERO_NO2")) {
            const double kno2 = 1.0e-04 * totsurfa;
            k = 60.0 * (kno2 > 0.0 ? kno2 : 0.0);
        } else if (label_is(irate, "HETERO_IEPOX")) {
            k = 60.0 * kiepox;
        } else if (label_is(irate, "HETERO_TETROL")) {
            k = 60.0 * AQUEOUS_FREQUENCY * fh2o;
        } else if (label_is(irate, "HETERO_IEPOXOS")) {
            k = aso4j_ppm > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * fos / aso4j_ppm : 0.0;
        } else if (label_is(irate, "HETERO_ISO3NOSJ")) {   /* CRACMM's IEPOX SOA */
            k = 60.0 * AQUEOUS_FREQUENCY * fh2o;
        } else if (label_is(irate, "HETERO_ISO3OSJ")) {
            k = aso4j_ppm > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * fos / aso4j_ppm : 0.0;
        } else if (label_is(irate, "HETERO_NO3")) {
            k = 60.0 * (kno3[0] + kno3[1]);
        } else if (label_is(irate, "HETERO_HO2")) {
            k = 60.0 * kho2[1];
        } else if (label_is(irate, "HETERO_GLY")) {
            k = 60.0 * kgly[1];
        } else if (label_is(irate, "HETERO_MGLY")) {
            k = 60.0 * kmgly[1];
        } else if (label_is(irate, "HETERO_NTR2")) {
            float con_toa = 0.0f;
            for (int spc = 0; spc < HO_NSPC; ++spc)
                if (ho_om[spc] && !ho_tracer[spc]) con_toa += s->aerospc_conc[spc][0] + s->aerospc_conc[spc][1];
            float f_part_ntr2 = 0.0f;
            if (con_toa >= MIN_TOA)
                f_part_ntr2 = ON_ALPHA1 / (1.0f + ON_CSTAR1 / con_toa) + ON_ALPHA2 / (1.0f + ON_CSTAR2 / con_toa);
            if (airrh <= 0.2 || f_part_ntr2 <= 0.0f) k = 0.0;
            else if (airrh >= 0.4) k = (double)(f_part_ntr2 * KHON);
            else k = (double)(f_part_ntr2 * KHON) * (5.0 * airrh - 1.0);
        } else if (label_is(irate, "HETERO_CLNO3_WAI")) {
            k = 60.0 * s->wet_m2[0] * DPI_D / (radius_i * inv_diff_clno3 + clno3_h2o_rxn_time);
        } else if (label_is(irate, "HETERO_CLNO3_WAJ")) {
            k = 60.0 * s->wet_m2[1] * DPI_D / (radius * inv_diff_clno3 + clno3_h2o_rxn_time);
        } else {
            k = NAN;   /* a label this oracle does not restate */
        }
        khetero[irate] = k;
    }
}

/* KHETERO for ncell cells: conc [HO_NAE][ncell] (the CGRID aerosol block, cell index
 * fastest), temp / press / wvapor / dens [ncell], khetero [ncell][HO_NHET] out. */
void oracle_hetchem_rates(long long ncell, const float* conc, const float* temp, const float* press,
                          const float* wvapor, const float* dens, double* khetero, int threads)
{
#pragma omp parallel for num_threads(threads > 0 ? threads : 1) schedule(static)
    for (long long c = 0; c < ncell; ++c)
        hetchem_rates_cell(conc + c, ncell, temp[c], press[c], wvapor[c], dens[c], khetero + c * HO_NHET);
}

/* pieces for the pinning tests: N2O5_GAMMA, CRYSTALIZED, FREEZES and PNCOM_LOSS of one
 * cell (the aerosol state extracted from its block), and its wet moments and diameters */
double oracle_het_n2o5_gamma(const float* conc, long long stride, double temp, double rh, int gparam)
{
    HoState s;
    hetchem_extract_aero(&s, conc, stride);
    return n2o5_gamma(&s, temp, rh, gparam);
}
int oracle_het_crystalized(const float* conc, long long stride, double rh, int complete)
{
    HoState s;
    hetchem_extract_aero(&s, conc, stride);
    return crystalized(&s, rh, complete);
}
int oracle_het_freezes(double temp, double rh) { return freezes(temp, rh); }
double oracle_het_pncom_loss(float poc, float pncom) { return pncom_loss(poc, pncom); }
void oracle_het_moments(const float* conc, long long stride, double* wet_m2, double* wet_m3, double* de_wet)
{
    HoState s;
    hetchem_extract_aero(&s, conc, stride);
    for (int n = 0; n < 3; ++n) {
        wet_m2[n] = s.wet_m2[n];
        wet_m3[n] = s.wet_m3[n];
        de_wet[n] = s.de_wet[n];
    }
}
/* CALCISOPGAMMAS' diffuso-reactive parameter q of one cell (its switch q / TANH( q ) > 1
 * decides whether the epoxide uptake is on) */
double oracle_het_isop_q(const float* conc, long long stride, double temp)
{
    HoState s;
    hetchem_extract_aero(&s, conc, stride);
    double g, kp, ft, fo, q = 0.0;
    calcisopgammas_q(&s, 0.5 * s.de_wet[1], temp, sqrt(8.0e3 * (double)RGASUNIV_F / (ho_mw_iepox * DPI_D)), &g,
                     &kp, &ft, &fo, &q);
    return q;
}
