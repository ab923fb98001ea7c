// HETCHEM_RATES (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:282-1535): the heterogeneous rate
// constants KHETERO of one grid cell from its aerosol block of CGRID and the met fields, as
// host/device code.
//
//   aerosol state  HETCHEM_EXTRACT_AERO (aero_subs.F:3052-3135): extract_aero with the
//                  minimum concentrations (AERO_DATA.F:1296-1420), calcmoments' wet moments
//                  (AERO_DATA.F:1575-1699), getpar's modal parameters (getpar.f), the wet
//                  second and third moments and effective diameters of the three modes
//   rates          HETCHEM_RATES' cell loop (AEROSOL_CHEMISTRY.F:862-1302): molecular
//                  speeds, diffusivities, N2O5_GAMMA (:1649-2044, with CRYSTALIZED and
//                  FREEZES), the ClNO2 yields, CALCISOPGAMMAS (:2285-2555), PNCOM_LOSS
//                  (:1539-1646), the NTR2 partitioning, and the rate of each KHETERO label
//
// The reference's REAL(4) and REAL(8) variables and literals are kept as float and double,
// operation by operation, with the C math library's functions in place of Fortran's
// intrinsics of the same kind.  The mechanism's tables (aerosol species, CGRID rows,
// KHETERO labels, epoxide pairs) come from gen/<mech>_hetchem.cuh: a translation unit
// includes this file for one mechanism, HET_NS naming the namespace that holds the code
// and HET_GEN the generated header (CB6r5's, in namespace het, unless both are defined).
// The sea-salt surface area of HETCHEM_RATES feeds only the bromine and iodine rates of
// CB6R5M_AE7_AQ; the mechanisms here have none, so it is not formed.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define HC_HD __host__ __device__
#else
#define HC_HD
#endif

#ifndef HET_NS
#define HET_NS het
#define HET_GEN "gen/cb6r5_ae7_aq_hetchem.cuh"
#endif

namespace HET_NS {

#include HET_GEN

// CONST.EXT and AEROMET_DATA (REAL(4) unless noted)
constexpr float PI = 3.14159265f;
constexpr double DPI = 3.14159265358979324;
constexpr float RGASUNIV = 8.314510f, STDATMPA = 101325.0f, STDTEMP = 273.15f, MWAIR = 28.9628f, MWWAT = 18.0153f;
constexpr float GPKG = 1.0e3f;
constexpr float F6PI = 6.0f / PI;
constexpr float CONMIN = 1.0e-23f;   // aeromode's min_numconc, min_m2conc, min_m3conc
constexpr float MIN_SIGMA_G = 1.05f, MAX_SIGMA_G = 2.5001f;
// HETCHEM_RATES' parameters (AEROSOL_CHEMISTRY.F:424-470)
constexpr double AQUEOUS_FREQUENCY = 1.0e9;
constexpr double INV_SQRT_MWN2O5 = 9.62161363758323e-2, INV_SQRT_MWCLNO3 = 1.012739360000e-1;
constexpr double COEF1 = 7.24382926227485e10;
constexpr double GAMMA_NO3 = 1.0e-3, GAMMA_GLY = 2.9e-3, GAMMA_HO2 = 0.2;
constexpr double STD_DIFF_N2O5 = 0.0855e-4, STD_DIFF_CLNO3 = 0.1014e-4;
constexpr float CFACTOR = 8.0f * GPKG * RGASUNIV / PI;
constexpr float INV_STDTEMP = 1.0f / STDTEMP;
constexpr float EPSWATER = MWWAT / MWAIR;
constexpr float ON_ALPHA1 = 0.34f, ON_ALPHA2 = 0.66f, ON_CSTAR1 = 0.73f, ON_CSTAR2 = 1000.0f;
constexpr float MIN_TOA = 0.0001f, KHON = 2.7778e-03f;
constexpr double INV_GAMMA_CLNO3_H2O = 1.0 / 0.024;
constexpr double AL = 610.94, BL = 17.625, CL = 243.04, DL = 1.0 / AL;

// the cell's aerosol state after HETCHEM_EXTRACT_AERO
struct Aero {
    float conc[NSPC][3];            // aerospc_conc [ug/m3], 0 where a mode is missing
    double wet_m2[3], wet_m3[3], de_wet[3];
};

HC_HD inline bool missing(const HetTables& T, int s, int m) { return T.row[s][m] < 0; }

// HETCHEM_EXTRACT_AERO for one cell: ae[r * n] is row r of the CGRID aerosol block
HC_HD inline void het_extract(const HetTables& T, const float* ae, long long n, Aero& a)
{
    float m0[3], m2[3], m3[3], lnsg[3], diam[3];
    for (int m = 0; m < 3; ++m)                                         // extract_aero
        for (int s = 0; s < NSPC; ++s)
            a.conc[s][m] = missing(T, s, m) ? 0.0f : fmaxf(ae[T.row[s][m] * n], T.min_conc[s][m]);
    for (int m = 0; m < 3; ++m) {
        float sum = 0.0f;
        for (int s = 0; s < NSPC; ++s)
            if (!T.no_m2wet[s] && !T.tracer[s]) sum = sum + a.conc[s][m] / T.density[s];
        m3[m] = fmaxf(sum * 1.0e-9f * F6PI, CONMIN);
        m0[m] = fmaxf(ae[T.num_row[m] * n], CONMIN);
        m2[m] = fmaxf(ae[T.srf_row[m] * n] / PI, CONMIN);
    }
    // calcmoments( .true. ), then getpar( FIXED_sg = F ): both sum the mode's wet third
    // moment over the same species in the same order (the species' factor REAL( 1.0E-9 *
    // f6pi / density, 8 ) from the tables), so the sum is formed once
    for (int m = 0; m < 3; ++m) {
        const float initial_m2 = m2[m];
        const float initial_m3 = fmaxf(m3[m], CONMIN);
        double wetsum = 0.0;
        for (int s = 0; s < NSPC; ++s) {
            if (T.tracer[s] || missing(T, s, m)) continue;
            wetsum = wetsum + T.m3fac[s] * (double)a.conc[s][m];
        }
        m3[m] = fmaxf((float)wetsum, CONMIN);
        m2[m] = initial_m2 * powf((float)wetsum / initial_m3, (float)(2.0 / 3.0));
    }
    const double minl2sg = (double)(logf(MIN_SIGMA_G) * logf(MIN_SIGMA_G));
    const double maxl2sg = (double)(logf(MAX_SIGMA_G) * logf(MAX_SIGMA_G));
    for (int m = 0; m < 3; ++m) {
        const double xfsum = (1.0 / 3.0) * log((double)m0[m]) + (2.0 / 3.0) * log((double)m3[m]);
        double l2sg = xfsum - log((double)m2[m]);
        l2sg = fmax(l2sg, minl2sg);
        l2sg = fmin(l2sg, maxl2sg);
        m2[m] = (float)exp(xfsum - l2sg);
        lnsg[m] = (float)sqrt(l2sg);
        const float es36 = (float)exp(4.5 * l2sg);
        m0[m] = fmaxf(m0[m], m3[m] / (1.0e-12f * es36));
        diam[m] = powf(m3[m] / (m0[m] * es36), 1.0f / 3.0f);
    }
    for (int m = 0; m < 3; ++m) {
        a.wet_m3[m] = (double)m3[m];
        a.wet_m2[m] = (double)m2[m];
        a.de_wet[m] = (double)(diam[m] * expf(1.5f * (lnsg[m] * lnsg[m])));
    }
}

// CRYSTALIZED( RH, .TRUE. ) (AEROSOL_CHEMISTRY.F:2047-2179)
HC_HD inline bool het_crystalized(const HetTables& T, const Aero& a, double rh)
{
    if (rh <= 0.01) return true;
    if (rh > 0.351) return false;
    const float nno3 = (a.conc[I_ANO3][0] + a.conc[I_ANO3][1]) / T.molwt[I_ANO3];
    const float nso4 = (a.conc[I_ASO4][0] + a.conc[I_ASO4][1]) / T.molwt[I_ASO4];
    const float nnh4 = (a.conc[I_ANH4][0] + a.conc[I_ANH4][1]) / T.molwt[I_ANH4];
    const float ncat = fmaxf(nnh4, 2.0f * nso4 + nno3);
    const float nani = nno3 + nso4;
    const float x = nnh4 / ncat, y = nso4 / nani;
    if (x < 0.50f || y < 0.22f) return false;
    const float x2 = x * x, xy = x * y, x2y = x2 * y, y2 = y * y, xy2 = x * y2;
    const float rden = 1.0f / (25.0f + (x - 0.7f) * (y - 0.5f));
    const float crh = 3143.44f + (63.07f * x) + (0.114f * x2) + (87.97f * y) - (125.73f * xy) + (0.586f * x2y)
                    + (0.95f * y2) - (1.384f * xy2) - (79692.5f * rden);
    return rh <= (double)crh;
}

// FREEZES (AEROSOL_CHEMISTRY.F:2182-2282)
HC_HD inline bool het_freezes(double temp, double rh)
{
    const double tst = 373.16, t0 = 273.16, logpst = 3.0057149, logp0 = 0.78583503;
    if (!(temp < t0)) return false;
    const double eirh = 1.61299 + temp * (4.4117437e-5 * temp - 1.4293888e-2);
    const double lirh = eirh - 0.005, uirh = eirh + 0.005;
    if (rh > uirh) return true;
    if (rh < lirh) return false;
    const double tsdt = tst / temp, tdts = temp / tst, t0dt = t0 / temp, tdt0 = temp / t0;
    const double logpw = -7.90298 * (tsdt - 1.0) + 5.02808 * log10(tsdt)
                       - 1.3816e-7 * (pow(10.0, 11.344 * (1.0 - tdts)) - 1.0)
                       + 8.1328e-3 * (pow(10.0, -3.49149 * (tsdt - 1.0)) - 1.0) + logpst;
    const double logpi = -9.09718 * (t0dt - 1.0) - 3.56654 * log10(t0dt) + .876793 * (1.0 - tdt0) + logp0;
    const double irh = pow(10.0, logpi - logpw);
    return rh > irh;
}

HC_HD inline float het_logitinv(float xx) { return 1.0f / (1.0f + expf(-xx)); }

// N2O5_GAMMA for GPARAM 0 (Davis et al., fine modes) and 5 (Bertram and Thornton, coarse)
// (AEROSOL_CHEMISTRY.F:1649-2044)
HC_HD inline double het_n2o5_gamma(const HetTables& T, const Aero& a, double temp, double rh, int gparam)
{
    if (gparam == 5) {
        const float a_bt = 3.2e-08f, beta_bt = 1.15e06f, delta = 1.3e-01f, k3ok2b = 6.0e-02f, k4ok2b = 29.0f;
        const float inv_vol = 1.0e-9f * F6PI / (float)a.wet_m3[2];
        const float ah2om = a.conc[I_AH2O][2] * inv_vol / T.molwt[I_AH2O];
        const float aclm = a.conc[I_ACL][2] * inv_vol / T.molwt[I_ACL];
        const float ano3m = a.conc[I_ANO3][2] * inv_vol / T.molwt[I_ANO3];
        const float k2fp = beta_bt - beta_bt * expf(-delta * ah2om);
        const float den1 = k3ok2b * (ah2om / ano3m), den2 = k4ok2b * (aclm / ano3m);
        const float den = den1 + 1.0f + den2;
        return (double)(a_bt * k2fp * (1.0f - 1.0f / den));
    }
    const bool crystal = het_crystalized(T, a, rh);
    if (het_freezes(temp, rh)) return 0.02;
    const float anh4 = a.conc[I_ANH4][0] + a.conc[I_ANH4][1];
    const float ano3 = a.conc[I_ANO3][0] + a.conc[I_ANO3][1];
    const float aso4 = a.conc[I_ASO4][0] + a.conc[I_ASO4][1];
    const float nno3 = ano3 / T.molwt[I_ANO3], nso4 = aso4 / T.molwt[I_ASO4], nnh4 = anh4 / T.molwt[I_ANH4];
    const float nani = nno3 + nso4;
    const float x3 = nno3 / nani;
    const float x2 = fmaxf(0.0f, fminf(1.0f - x3, nnh4 / nani - 1.0f));
    const float x1 = 1.0f - (x2 + x3);
    const float lam3 = -8.10774f + 4.902f * (float)rh;
    const float gam3 = fminf(het_logitinv(lam3), 0.0154f);
    if (crystal) {
        const float t293 = fmaxf(0.0f, (float)temp - 293.0f);
        const float lamd = -6.13376f + 3.592f * (float)rh - 0.19688f * t293;
        const float gamd = fminf(het_logitinv(lamd), 0.0124f);
        return (double)((x1 + x2) * gamd + x3 * fminf(gamd, gam3));
    }
    const float t291 = fmaxf(0.0f, (float)temp - 291.0f);
    const float rh46 = fminf(0.0f, (float)rh - 0.46f);
    const float lam2 = -3.64849f + 9.553f * rh46;
    const float lam1 = lam2 + 0.97579f - 0.20427f * t291;
    const float gam1 = fminf(het_logitinv(lam1), 0.08585f);
    const float gam2 = fminf(het_logitinv(lam2), 0.053f);
    return (double)((x1 * gam1) + (x2 * gam2) + (x3 * gam3));
}

// PNCOM_LOSS (AEROSOL_CHEMISTRY.F:1539-1646)
HC_HD inline double het_pncom_loss(float poc, float pncom)
{
    const double koheff = 2.5e-12;
    const float lower = 7.0f / 6.0f, upper = 11.0f / 3.0f;
    if ((double)poc <= 1.0e-30) return 0.0;
    const double ratio = (double)((poc + pncom) / poc);
    if (ratio > (double)lower && ratio < (double)upper)
        return 15.0 * koheff / (16.0 + ((double)upper - ratio) / (ratio - (double)lower));
    if (ratio >= (double)upper) return 15.0 / 16.0 * koheff;
    return 0.0;
}

// CALCISOPGAMMAS for IEPOX (NUMVOC = 1; AEROSOL_CHEMISTRY.F:2285-2555): the uptake
// coefficient, and the fractions of the uptake into non-sulfated (ftet) and sulfated (fos)
// products
HC_HD inline void het_isop_gammas(const HetTables& T, const Aero& a, double radius, double temperature,
                                  double& gamma, double& ftet, double& fos)
{
    const double inv_alpha = 1.0 / 0.02, diffusivity = 1.0e-9, rgas_latm = 0.08206;
    double acid[2];
    const double eqlbh = (double)(a.conc[I_AH3OP][1] / T.molwt[I_AH3OP]) * 1.0e-6;
    acid[0] = fmax(eqlbh, 0.0);
    double charge = 0.0;
    for (int s = 0; s < NSPC; ++s) {
        if (T.tracer[s] || missing(T, s, 1)) continue;
        charge = charge - (double)((float)T.charge[s] * a.conc[s][1] / T.molwt[s]);
    }
    acid[1] = fmax(charge * 1.0e-6 - acid[0], 0.0);
    double inv_volume = 0.0;
    for (int s = 0; s < NSPC; ++s) {
        if (T.tracer[s] || missing(T, s, 1)) continue;
        inv_volume = inv_volume + (double)(a.conc[s][1] / T.density[s]);
    }
    inv_volume = 1.0e6 / inv_volume;
    double kparticle = 0.0, kchemtet = 0.0, kchemos = 0.0;
    for (int i = 0; i < NNUC; ++i) {
        const int sp = T.nuc_spc[i];
        double nuc = (double)(a.conc[sp][1] / T.molwt[sp]) * 1.0e-6;
        const double ac = acid[T.nuc_acid[i] - 1];
        if (T.nuc_remove[i] >= 1) nuc = fmax(nuc - acid[T.nuc_remove[i] - 1], 0.0);
        const double kchem = T.nuc_kchem[i] * nuc * ac * (inv_volume * inv_volume);
        kparticle = kparticle + kchem;
        if (T.nuc_os[i]) kchemos = kchemos + kchem;
        else kchemtet = kchemtet + kchem;
    }
    const float temp = (float)temperature;   // HLCONST( 'IEPOX', temp, .False., 0.0 )
    const double heff = (double)(HL_IEPOX_A * expf(HL_IEPOX_E * ((298.0f - temp) / (298.0f * temp))));
    const double cfactor_iepox = sqrt(8.0e3 * (double)RGASUNIV / (MW_IEPOX * DPI));
    const double q = radius * sqrt(kparticle / diffusivity);
    if (q / tanh(q) > 1.0) {
        const double nu = cfactor_iepox * sqrt(temperature);
        const double denom = inv_alpha + nu * radius
                           / (4.0 * heff * rgas_latm * temperature * diffusivity * (q / tanh(q) - 1.0));
        gamma = 1.0 / denom;
        ftet = kchemtet / kparticle;
        fos = kchemos / kparticle;
    } else {
        gamma = ftet = fos = 0.0;
    }
}

// molecular-speed factor DSQRT( 8.0D3 * REAL( RGASUNIV, 8 ) / ( MW * DPI ) )
HC_HD inline double het_cfactor(double mw) { return sqrt(8.0e3 * (double)RGASUNIV / (mw * DPI)); }

// KHETERO of one cell: ae[r * n] row r of the CGRID aerosol block (ug/m3, #/m3, m2/m3),
// temp [K], press [Pa], wvapor [kg/kg], dens [kg/m3]; k[j] (j < NHET) in KHETERO's order
HC_HD inline void het_cell(const HetTables& T, const float* ae, long long n, float temp, float press, float wvapor,
                           float dens, double* k)
{
    Aero a;
    het_extract(T, ae, n, a);
    const double airtemp = (double)temp;
    const double h2ovp = (double)(press * wvapor / (EPSWATER + wvapor));
    const double inv_esatl = DL * exp(BL * (273.15 - airtemp) / (airtemp - 273.15 + CL));
    const double airrh = fmax(0.005, fmin(0.99, h2ovp * inv_esatl));
    const double cbar_coeff = (double)sqrtf(CFACTOR * temp);
    const double adjust_diff = (double)(powf(temp * INV_STDTEMP, 1.75f) * (STDATMPA / press));
    const double ppm_factor = 1.0e-3 * (double)(MWAIR / dens);
    const double rfactor = 60.0 * COEF1 * (double)(press / temp);
    const double cbar = cbar_coeff * INV_SQRT_MWN2O5;
    const double cbarno3 = het_cfactor(MW_NO3) * sqrt(airtemp);
    const double cbargly = het_cfactor(MW_GLY) * sqrt(airtemp);
    const double cbarmgly = het_cfactor(MW_MGLY) * sqrt(airtemp);
    const double cbarho2 = het_cfactor(MW_HO2) * sqrt(airtemp);
    const double cbar_clno3 = cbar_coeff * INV_SQRT_MWCLNO3;
    const double inv_diffusivity = 1.0 / (STD_DIFF_N2O5 * adjust_diff);
    const double inv_diff_clno3 = 1.0 / (STD_DIFF_CLNO3 * adjust_diff);
    const double inv_mwcl = (double)(1.0f / T.molwt[I_ACL]);
    const float mwclh2o = T.molwt[I_ACL] / T.molwt[I_AH2O];
    const float mwh2ocl = 1.0f / mwclh2o;
    double kn2o5[3], kno3[3], kgly[3], kmgly[3], kho2[3], cl_ppm[3], yield[3] = {0.0, 0.0, 0.0};
    double yieldij = 0.0;
    for (int m = 0; m < 3; ++m) {
        const double gamma = het_n2o5_gamma(T, a, airtemp, airrh, m <= 1 ? 0 : 5);
        const double xxf = a.wet_m2[m] / (4.0 + 0.5 * a.de_wet[m] * gamma * cbar * inv_diffusivity);
        kn2o5[m] = gamma * xxf;
        kno3[m] = GAMMA_NO3 * a.wet_m2[m] / (4.0 + 0.5 * a.de_wet[m] * GAMMA_NO3 * cbarno3 * inv_diffusivity)
                * cbarno3 * DPI;
        kgly[m] = GAMMA_GLY * a.wet_m2[m] / (4.0 + 0.5 * a.de_wet[m] * GAMMA_GLY * cbargly * inv_diffusivity)
                * cbargly * DPI;
        kmgly[m] = (double)0.09f * GAMMA_GLY * a.wet_m2[m]
                 / (4.0 + 0.5 * a.de_wet[m] * (double)0.09f * GAMMA_GLY * cbarmgly * inv_diffusivity) * cbarmgly * DPI;
        kho2[m] = GAMMA_HO2 * a.wet_m2[m] / (4.0 + 0.5 * a.de_wet[m] * GAMMA_HO2 * cbarho2 * inv_diffusivity)
                * cbarho2 * DPI;
        const float ah2o = a.conc[I_AH2O][m], acl = a.conc[I_ACL][m];
        cl_ppm[m] = ppm_factor * ((double)acl * inv_mwcl);
        if (ah2o > 5.0e-01f && acl > 1.0e-04f && mwh2ocl * acl > 1.0e-4f * ah2o)
            yield[m] = 1.0 / (1.0 + (1.0 / 483.0) * (double)(ah2o / acl) * (double)mwclh2o);
    }
    {
        const float ah2o = a.conc[I_AH2O][0] + a.conc[I_AH2O][1], acl = a.conc[I_ACL][0] + a.conc[I_ACL][1];
        if (ah2o > 5.0e-01f && acl > 1.0e-04f && mwh2ocl * acl > 1.0e-4f * ah2o)
            yieldij = 1.0 / (1.0 + (1.0 / 483.0) * (double)((ah2o / acl) * mwclh2o));
    }
    for (int m = 0; m < 3; ++m) kn2o5[m] = cbar * DPI * kn2o5[m];
    const double totsurfa = (a.wet_m2[0] + a.wet_m2[1]) * DPI;
    const double radius_i = 0.5 * a.de_wet[0], radius = 0.5 * a.de_wet[1];
    const double clno3_h2o_rxn_time = 4.0 * INV_GAMMA_CLNO3_H2O / cbar_clno3;
    const double cbariepox = het_cfactor(MW_IEPOX) * sqrt(airtemp);
    double gammaiepox, ftet, fos;
    het_isop_gammas(T, a, radius, airtemp, gammaiepox, ftet, fos);
    double kiepox = 0.0, aso4j_ppm = 0.0;
    if (gammaiepox > 1.0e-72) {
        kiepox = a.wet_m2[1] * DPI / (radius * inv_diffusivity + 4.0 / (cbariepox * gammaiepox));
        aso4j_ppm = ppm_factor * (double)a.conc[I_ASO4][1] * (double)(1.0f / T.molwt[I_ASO4]);
    }
    for (int j = 0; j < NHET; ++j) {
        double r = 0.0;
        switch (T.kind[j]) {
        case K_N2O5IJ: r = 60.0 * (kn2o5[0] + kn2o5[1]); break;
        case K_N2O5K: r = 60.0 * kn2o5[2]; break;
        case K_N2O5I: r = 60.0 * kn2o5[0]; break;
        case K_N2O5J: r = 60.0 * kn2o5[1]; break;
        case K_H2NO3PAIJ: r = 60.0 * AQUEOUS_FREQUENCY * fmax(1.0 - yieldij, 0.0); break;
        case K_H2NO3PBIJ: r = yieldij > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * yieldij / (cl_ppm[0] + cl_ppm[1]) : 0.0; break;
        case K_H2NO3PAK: r = 60.0 * AQUEOUS_FREQUENCY * fmax(1.0 - yield[2], 0.0); break;
        case K_H2NO3PBK: r = yield[2] > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * yield[2] / cl_ppm[2] : 0.0; break;
        case K_PNCOMLI: r = rfactor * het_pncom_loss(a.conc[I_APOC][0], a.conc[I_APNCOM][0]); break;
        case K_PNCOMLJ: r = rfactor * het_pncom_loss(a.conc[I_APOC][1], a.conc[I_APNCOM][1]); break;
        case K_NO2: r = 60.0 * fmax(0.0, 1.0e-04 * totsurfa); break;
        case K_IEPOX: r = 60.0 * kiepox; break;
        case K_TETROL: r = 60.0 * AQUEOUS_FREQUENCY * ftet; break;
        case K_IEPOXOS: r = aso4j_ppm > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * fos / aso4j_ppm : 0.0; break;
        case K_ISO3NOSJ: r = 60.0 * AQUEOUS_FREQUENCY * ftet; break;   // CRACMM's non-sulfated IEPOX SOA
        case K_ISO3OSJ: r = aso4j_ppm > 0.0 ? 60.0 * AQUEOUS_FREQUENCY * fos / aso4j_ppm : 0.0; break;
        case K_NO3: r = 60.0 * (kno3[0] + kno3[1]); break;
        case K_GLY: r = 60.0 * kgly[1]; break;
        case K_MGLY: r = 60.0 * kmgly[1]; break;
        case K_HO2: r = 60.0 * kho2[1]; break;
        case K_NTR2: {
            float con_toa = 0.0f;
            for (int s = 0; s < NSPC; ++s)
                if (T.om[s] && !T.tracer[s]) con_toa = con_toa + (a.conc[s][0] + a.conc[s][1]);
            float f_part = 0.0f;
            if (con_toa >= MIN_TOA)
                f_part = ON_ALPHA1 / (1.0f + ON_CSTAR1 / con_toa) + ON_ALPHA2 / (1.0f + ON_CSTAR2 / con_toa);
            if (airrh <= 0.2 || f_part <= 0.0f) r = 0.0;
            else if (airrh >= 0.4) r = (double)(f_part * KHON);
            else r = (double)(f_part * KHON) * (5.0 * airrh - 1.0);
            break;
        }
        case K_CLNO3_WAI: r = 60.0 * a.wet_m2[0] * DPI / (radius_i * inv_diff_clno3 + clno3_h2o_rxn_time); break;
        case K_CLNO3_WAJ: r = 60.0 * a.wet_m2[1] * DPI / (radius * inv_diff_clno3 + clno3_h2o_rxn_time); break;
        default: r = NAN;
        }
        k[j] = r;
    }
}

}  // namespace HET_NS
