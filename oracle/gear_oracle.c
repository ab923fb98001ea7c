/*
 * CPU oracle for CMAQ's SMVGEAR gas-chemistry solver.  TEST INFRASTRUCTURE ONLY: the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it; the product
 * path never does.  Included from ros3_oracle.c, whose block kernels it shares: the
 * symbolic set-up of SMVGEAR (JSPARSE, CCTM/src/gas/smvgear/grsprse.F) is the same
 * algorithm as ROS3's RBSPARSE, DECOMP and BACKSUB (grdecomp.F, grbacksub.F) perform the
 * same operations as RBDECOMP and RBSOLVE, and SUBFUN's derivative sums
 * (grsubfun.F:115-170) are RBFEVAL's.
 *
 * A plain-C restatement of the vectorised Gear solver, following its loops one for one:
 *   gear_coef          GRINIT and JSPARSE constants (grinit.F:163-171, grsprse.F:682-720,
 *                      PERTST of GRVARS.F:283-286)
 *   gear_optimal_atol  OPTIMAL_ATOL_PPM (GRVARS.F:597-708)
 *   gear_subfun        SUBFUN (grsubfun.F:97-176)
 *   gear_pderiv        PDERIV (grpderiv.F:118-230)
 *   oracle_smvgear     SMVGEAR (grsmvgear.F:230-1007) for one block of cells sharing the
 *                      step size and order; the reference's GO TO structure is kept as labels
 *   oracle_gear_chem   the Gear CHEM driver (grdriver.F:300-706: gather, stiffness
 *                      ordering pass, heap sort, write-back)
 *
 * Floating-point rule shared with the device code (as in ros3_oracle.c): every
 * "x +/- a*b" of the reference is one fused multiply-add, every other operation is
 * rounded on its own.  REAL(4) literals of the reference (0.1, 0.2, 1.1, 1.4, and the
 * single-precision ENQQ1-3 of JSPARSE) keep their REAL(4) values.
 *
 * Mixed-kind MAX( REAL(4), REAL(8) ) of the gather (grdriver.F:419-422) is evaluated in
 * REAL(8), as compilers that accept it promote the REAL(4) argument.
 */

#define G_MXORDER 7
#define G_MAXORD 5
#define G_MSTEP 3
#define G_MBETWEEN 50
#define G_MXLOWRED 20
#define G_NBINS 5
static const double G_HMAXDAY = 15.0, G_HMAXNIT = 5.0, G_HMIN = 1.0e-10, G_FRACDEC = 0.25;
static const double G_CONCMIN = 1.0e-30, G_ZBOUND = 1.0e-30;
static const double G_PT2 = 0.2, G_PT003 = 0.003, G_OMIC = 0.000001, G_OPT2MIC = 0.0000012,
                    G_OPT3MIC = 0.0000013, G_OPT4MIC = 0.0000014, G_HRMAX = 0.3;

/* Gear coefficients and tolerances; layout shared with the device (GearCoef in the CUDA
 * sources carries the same numbers). */
typedef struct {
    double aset[10][8];           /* ASET(10, 8): [nqq-1][j-1] */
    double pertst[G_MXORDER][3];  /* PERTST**2 */
    double enqq1[G_MXORDER], enqq2[G_MXORDER], enqq3[G_MXORDER], conpst[G_MXORDER], conp15[G_MXORDER];
    double errmax;                /* ERRMAX = REAL(GEAR_RTOL, 8) */
    double ylow;                  /* YLOW = REAL(GEAR_MIN_ATOL, 8) */
    double atol_level[G_NBINS + 1];
    double atol_floor;            /* REAL(GEAR_CONC_FLOOR, 8) */
    int max_iter;                 /* cap on SUBFUN calls per block and call (0: none) */
} GearCfg;

typedef struct {
    int nsteps, ncfail, nefail, npderiv, nsubfun, nnewt, maxord, status;
} GearStats;

/* GRINIT / JSPARSE constants and OPTIMAL_ATOL_PPM levels (first call). */
void oracle_gear_cfg(double rtol, float max_atol, float min_atol, float conc_floor, int max_iter, GearCfg* g)
{
    static const double pertst[3][G_MXORDER] = {
        {2.0, 4.5, 7.333, 10.42, 13.7, 17.15, 1.0},
        {3.0, 6.0, 9.167, 12.5, 15.98, 1.0, 1.0},
        {1.0, 1.0, 0.5, 0.1667, 0.04133, 0.008267, 1.0}};
    memset(g, 0, sizeof(*g));
    for (int q = 0; q < G_MXORDER; ++q) {
        const int nqq = q + 1;
        g->enqq1[q] = (double)(0.5f / (float)nqq);           /* REAL(4) expressions */
        g->enqq2[q] = (double)(0.5f / (float)(nqq + 1));
        g->enqq3[q] = (double)(0.5f / (float)(nqq + 2));
        g->conpst[q] = 1.0 / (pertst[0][q] * g->enqq3[q]);
        g->conp15[q] = 1.5 * g->conpst[q];
        for (int k = 0; k < 3; ++k) g->pertst[q][k] = pertst[k][q] * pertst[k][q];
    }
#define AS(i, j) g->aset[(i) - 1][(j) - 1]
    for (int i2 = 1; i2 <= 6; ++i2) { AS(i2, 2) = 1.0; AS(i2, 8) = 0.0; }
    AS(1, 1) = 1.0;
    AS(2, 1) = 2.0 / 3.0;        AS(2, 3) = 1.0 / 3.0;
    AS(3, 1) = 6.0 / 11.0;       AS(3, 3) = 6.0 / 11.0;       AS(3, 4) = 1.0 / 11.0;
    AS(4, 1) = 12.0 / 25.0;      AS(4, 3) = 0.70;             AS(4, 4) = 0.20;       AS(4, 5) = 0.02;
    AS(5, 1) = 60.0 / 137.0;     AS(5, 3) = 225.0 / 274.0;    AS(5, 4) = 85.0 / 274.0;
    AS(5, 5) = 15.0 / 274.0;     AS(5, 6) = 1.0 / 274.0;
    AS(6, 1) = 180.0 / 441.0;    AS(6, 3) = 406.0 / 441.0;    AS(6, 4) = 735.0 / 1764.0;
    AS(6, 5) = 175.0 / 1764.0;   AS(6, 6) = 21.0 / 1764.0;    AS(6, 7) = 1.0 / 1764.0;
#undef AS
    g->errmax = rtol;
    g->ylow = (double)min_atol;
    const double abhi = log10((double)max_atol), ablo = log10((double)min_atol);
    g->atol_level[0] = pow(10.0, abhi);
    g->atol_level[G_NBINS] = pow(10.0, ablo);
    for (int i = 2; i <= G_NBINS; ++i) {
        const double t = (abhi - ablo) * (double)(G_NBINS - i + 1) / (double)G_NBINS;
        g->atol_level[i - 1] = pow(10.0, ablo + t);
    }
    g->atol_floor = (double)conc_floor;
    g->max_iter = max_iter;
}

/* OPTIMAL_ATOL_PPM: per cell, the absolute tolerance of the bin where 40% of the species
 * above the floor are reached, counting from the highest level down. */
static void gear_optimal_atol(const double* cnew, int n, int ld, const GearCfg* g, double* ylowa)
{
    for (int c = 0; c < n; ++c) {
        int bins[G_NBINS + 1] = {0};
        for (int s = 0; s < MECH_NSPEC; ++s) {
            const double v = cnew[(size_t)s * ld + c];
            if (v >= g->atol_level[0]) bins[0]++;
            else if (v >= g->atol_level[1]) bins[1]++;
            else if (v >= g->atol_level[2]) bins[2]++;
            else if (v >= g->atol_level[3]) bins[3]++;
            else if (v >= g->atol_level[4]) bins[4]++;
            else if (v >= g->atol_floor) bins[5]++;
        }
        int cum[G_NBINS + 1];
        cum[0] = bins[0];
        for (int k = 1; k <= G_NBINS; ++k) cum[k] = bins[k] + cum[k - 1];
        const int cutoff = (int)(0.4f * (float)cum[G_NBINS]);
        int k = 0;
        while (k < G_NBINS && !(cum[k] > cutoff)) ++k;
        ylowa[c] = g->atol_level[k];
    }
}

typedef struct {
    Block b;             /* y = CNEW (new order), rki = RK, rxrat, cc2, vdiag, explic */
    double* conc;        /* CONC(ld, MXORDER*ISCHAN): Nordsieck history */
    double* gloss, *dtlos, *chold, *cest, *ceff;   /* (ld, ISCHAN) */
    double* blkconc;     /* initial CNEW, new order */
    double* dely, *ylowa, *yloweps, *yloweps1;     /* (ld) */
    double* cfini;       /* DDM-3D: state at the previous accepted step (ld, ISCHAN) */
    double* caveg;       /* DDM-3D: CAVEG (ld, ISCHAN) when not NULL (grsmvgear.F sens blocks) */
} GearBlock;

static void gear_alloc(GearBlock* g, int ld)
{
    block_alloc(&g->b, ld);
    const size_t ns = (size_t)MECH_NSPEC * ld;
    g->conc = calloc((size_t)G_MXORDER * ns, sizeof(double));
    g->gloss = calloc(ns, sizeof(double));
    g->dtlos = calloc(ns, sizeof(double));
    g->chold = calloc(ns, sizeof(double));
    g->cest = calloc(ns, sizeof(double));
    g->ceff = calloc(ns, sizeof(double));
    g->blkconc = calloc(ns, sizeof(double));
    g->dely = calloc((size_t)ld, sizeof(double));
    g->ylowa = calloc((size_t)ld, sizeof(double));
    g->yloweps = calloc((size_t)ld, sizeof(double));
    g->yloweps1 = calloc((size_t)ld, sizeof(double));
    g->cfini = calloc(ns, sizeof(double));
    g->caveg = NULL;
}

static void gear_free(GearBlock* g)
{
    block_free(&g->b);
    free(g->conc); free(g->gloss); free(g->dtlos); free(g->chold); free(g->cest); free(g->ceff);
    free(g->blkconc); free(g->dely); free(g->ylowa); free(g->yloweps); free(g->yloweps1); free(g->cfini);
}

/* SUBFUN: GLOSS = dc/dt at CNEW; a species at the floor does not lose mass further. */
static void gear_subfun(GearBlock* g, int ncsp, GearStats* st)
{
    const int n = g->b.ncells, ld = g->b.ld;
    st->nsubfun++;
    oracle_rbfeval(&g->b, ncsp, g->b.y, g->gloss);
    for (int i = 0; i < MECH_ISCHAN; ++i)
        for (int c = 0; c < n; ++c)
            if (g->b.y[(size_t)i * ld + c] <= G_ZBOUND && g->gloss[(size_t)i * ld + c] < 0.0)
                g->gloss[(size_t)i * ld + c] = 0.0;
}

/* PDERIV: the predictor matrix P = I - ASN1*DELT*J at CNEW (zeroed below ZBOUND),
 * R1DELT = -ASN1*DELT, into CC2 by the partial-derivative pointer lists. */
static void gear_pderiv(GearBlock* g, int ncsp, double r1delt, GearStats* st)
{
    Block* b = &g->b;
    const int n = b->ncells, ld = b->ld;
    st->npderiv++;
    const int iarry = mech_iarray[ncsp];
    const int nondiag = iarry - MECH_ISCHAN;
    for (int iar = 0; iar <= nondiag; ++iar)
        for (int c = 0; c < n; ++c) b->cc2[(size_t)iar * ld + c] = 0.0;
    for (int iar = nondiag + 1; iar <= iarry; ++iar)
        for (int c = 0; c < n; ++c) b->cc2[(size_t)iar * ld + c] = 1.0;
    for (int s = 0; s < MECH_ISCHAN; ++s)
        for (int c = 0; c < n; ++c) {
            const double v = b->y[(size_t)s * ld + c];
            g->ceff[(size_t)s * ld + c] = v <= G_ZBOUND ? 0.0 : v;
        }
    const double* ce = g->ceff;
    double* ex = b->explic;
    const int nu = mech_nuserat[ncsp];
    for (int nrx = 0; nrx < nu; ++nrx) {
        const int nrk = mech_nkuserat[ncsp * MECH_NRXNS + nrx];
        const int* irm = &mech_irm2[nrk * (3 + MECH_MXPRD)];
        const double* k = &b->rki[(size_t)nrk * ld];
        const int nre = mech_nreact[nrk];
        if (nre == 1) {
            for (int c = 0; c < n; ++c) ex[c] = k[c];
        } else if (nre == 2) {
            for (int c = 0; c < n; ++c) {
                ex[c] = k[c] * ce[(size_t)irm[1] * ld + c];
                ex[ld + c] = k[c] * ce[(size_t)irm[0] * ld + c];
            }
        } else if (nre == 3) {
            for (int c = 0; c < n; ++c) {
                const double cr2 = k[c] * ce[(size_t)irm[1] * ld + c];
                ex[c] = cr2 * ce[(size_t)irm[2] * ld + c];
                ex[ld + c] = k[c] * ce[(size_t)irm[0] * ld + c] * ce[(size_t)irm[2] * ld + c];
                ex[2 * ld + c] = cr2 * ce[(size_t)irm[0] * ld + c];
            }
        }
        for (int t = mech_loss_ptr[ncsp][nrk]; t < mech_loss_ptr[ncsp][nrk + 1]; ++t) {
            double* cc = &b->cc2[(size_t)mech_loss_iarp[ncsp][t] * ld];
            const double* e = &ex[(size_t)mech_loss_ial[ncsp][t] * ld];
            for (int c = 0; c < n; ++c) cc[c] = fma(-r1delt, e[c], cc[c]);
        }
        for (int t = mech_prod_ptr[ncsp][nrk]; t < mech_prod_ptr[ncsp][nrk + 1]; ++t) {
            double* cc = &b->cc2[(size_t)mech_prod_iarp[ncsp][t] * ld];
            const double* e = &ex[(size_t)mech_prod_ial[ncsp][t] * ld];
            const int ic = mech_prod_icoeff[ncsp][t];
            if (ic < 0) {
                for (int c = 0; c < n; ++c) cc[c] = fma(r1delt, e[c], cc[c]);
            } else {
                const double fracn = mech_sc[nrk * MECH_MXPRD + ic] * r1delt;
                for (int c = 0; c < n; ++c) cc[c] = fma(fracn, e[c], cc[c]);
            }
        }
    }
}

/* x**y of SMVGEAR's step-size estimates (grsmvgear.F:939, 955, 972): the portable
 * routine of portable_pow.h, which the device code (gear.cuh: gpow) repeats operation
 * for operation. */
#include "portable_pow.h"
static double gear_pow(double x, double y) { return portable_pow(x, y); }

static double g_min2(double a, double b) { return b < a ? b : a; }
static double g_max2(double a, double b) { return b > a ? b : a; }

/* largest DELY over the block's cells, from 0 (the reference's DER*MAX / RMSTOP loops) */
static double gear_maxdely(const GearBlock* g)
{
    double m = 0.0;
    for (int c = 0; c < g->b.ncells; ++c)
        if (g->dely[c] > m) m = g->dely[c];
    return m;
}

/* SMVGEAR on one block of cells sharing the step size and order.  CNEW (g->b.y) holds the
 * gathered concentrations on entry (and g->blkconc a copy) and the result on exit.
 * lsun selects H0FAC and HMAX, ncsp the day or night reaction list.  With ordering !=
 * NULL only the initial stiffness estimate is stored there (grsmvgear.F:346-351). */
static GearStats oracle_smvgear(GearBlock* g, int ncsp, int lsun, double chemstep, const GearCfg* cfg,
                                double* ordering)
{
    Block* b = &g->b;
    const int n = b->ncells, ld = b->ld, isc = MECH_ISCHAN;
    GearStats st;
    memset(&st, 0, sizeof(st));
    double* cnew = b->y;
    double* conc = g->conc;
#define CO(col, c) conc[(size_t)(col) * ld + (c)]
#define SP(arr, s, c) (arr)[(size_t)(s) * ld + (c)]
#define ASET(i, j) cfg->aset[(i) - 1][(j) - 1]
    if (g->caveg && !ordering) memset(g->caveg, 0, sizeof(double) * (size_t)isc * ld);   /* :273-274 */
    if (ordering) {
        for (int c = 0; c < n; ++c) g->ylowa[c] = cfg->ylow;
    } else {
        gear_optimal_atol(cnew, n, ld, cfg, g->ylowa);
    }
    const double eps = cfg->errmax, eps1 = 1.0 / eps;
    const double epslow = g_min2(eps, G_PT003);
    const double order = (double)isc;
    const double h0fac = lsun ? 0.0625 : 1.0;
    const double hmax = lsun ? G_HMAXDAY : G_HMAXNIT;
    const double abst2 = 1.0 / (chemstep * chemstep);
    int jfail = 0, nylowred = 0;
    int ifsuccess, idoub, nslp, jrestar, nqq = 1, nqqold = 0, kstep = 2, jeval = 1, l3 = 0, nqqisc = isc;
    int higher_order;
    double xelaps, told, rdelmax, hratio, asn1, timremain, delt = 0.0, rdelt = 1.0;
    double enqq = 0.0, eup = 0.0, edwn = 0.0, drate = 0.7, rmserr = 0.0, rmserrp, der2max = 0.0;
    double rdeltup = 0.0, rdeltsm, rdeltdn;

loop_begin:
    ifsuccess = 1;
    idoub = 2;
    xelaps = 0.0;
    told = xelaps;
    rdelmax = 10000.0;
    nslp = G_MBETWEEN;
    jrestar = 0;
    hratio = 0.0;
    asn1 = 1.0;
    for (int c = 0; c < n; ++c) g->yloweps1[c] = g->ylowa[c] * eps1;
    timremain = chemstep;

loop_initialize:
    gear_subfun(g, ncsp, &st);
    for (int c = 0; c < n; ++c) { g->yloweps[c] = g->ylowa[c] / epslow; g->dely[c] = 0.0; }
    for (int j = 0; j < isc; ++j)
        for (int c = 0; c < n; ++c) {
            const double e = SP(g->gloss, j, c) / (SP(cnew, j, c) + g->yloweps[c]);
            g->dely[c] = fma(e, e, g->dely[c]);
        }
    if (ordering) {
        for (int c = 0; c < n; ++c) ordering[c] = g->dely[c];
        return st;
    }
    {
        const double rmstop = gear_maxdely(g);
        delt = sqrt(epslow / (abst2 + rmstop / order)) * h0fac;
        delt = g_min2(delt, chemstep);
        delt = g_min2(delt, hmax);
        delt = g_max2(delt, G_HMIN);
    }
    nqq = 1;
    for (int j = 0; j < isc; ++j)
        for (int c = 0; c < n; ++c) {
            CO(j, c) = SP(cnew, j, c);
            CO(isc + j, c) = delt * SP(g->gloss, j, c);
        }
    nqqold = 0;
    rdelt = 1.0;
    jeval = 1;
    if (g->caveg)   /* CFINI = BLKCONC (grsmvgear.F:427-431) */
        for (int j = 0; j < isc; ++j)
            for (int c = 0; c < n; ++c) SP(g->cfini, j, c) = SP(g->blkconc, j, c);

loop_order:
    higher_order = 1;
    timremain = chemstep - xelaps;
    if (timremain <= G_OMIC) goto done;
    if (nqq != nqqold) {
        nqqold = nqq;
        kstep = nqq + 1;
        hratio = hratio * ASET(nqq, 1) / asn1;
        asn1 = ASET(nqq, 1);
        enqq = cfg->pertst[nqq - 1][0] * order;
        eup = cfg->pertst[nqq - 1][1] * order;
        edwn = cfg->pertst[nqq - 1][2] * order;
        nqqisc = nqq * isc;
    }
    rdelt = g_min2(g_min2(g_min2(rdelt, rdelmax), hmax / delt), timremain / delt);
    delt = delt * rdelt;
    hratio = hratio * rdelt;
    if (delt < G_HMIN) {
        for (int c = 0; c < n; ++c) g->ylowa[c] = g->ylowa[c] * (double)0.1f;
        nylowred++;
        if (nylowred < G_MXLOWRED) {
            memcpy(cnew, g->blkconc, sizeof(double) * (size_t)isc * ld);
            goto loop_begin;
        }
        st.status |= ST_DT_UNDERFLOW;
        goto failed;
    }
    if (rdelt != 1.0) {
        double rdelta = 1.0;
        int i1 = 0;
        for (int j = 2; j <= kstep; ++j) {
            rdelta = rdelta * rdelt;
            i1 += isc;
            for (int i = i1; i < i1 + isc; ++i)
                for (int c = 0; c < n; ++c) CO(i, c) = CO(i, c) * rdelta;
        }
    }
    if (ifsuccess == 1) {
        rdelmax = 10.0;
        if (st.nsteps % 3 == 2) gear_optimal_atol(cnew, n, ld, cfg, g->ylowa);
        for (int c = 0; c < n; ++c) g->yloweps1[c] = g->ylowa[c] * eps1;
        for (int j = 0; j < isc; ++j)
            for (int c = 0; c < n; ++c) SP(g->chold, j, c) = eps1 / (fabs(SP(cnew, j, c)) + g->yloweps1[c]);
    }
    if (fabs(hratio - 1.0) > G_HRMAX || st.nsteps >= nslp) jeval = 1;
    xelaps = xelaps + delt;
    {   /* prediction: multiply the history by the Pascal triangle matrix */
        int i1 = nqqisc;
        for (int jb = 1; jb <= nqq; ++jb) {
            i1 -= isc;
            for (int i = i1; i < nqqisc; ++i)
                for (int c = 0; c < n; ++c) CO(i, c) = CO(i, c) + CO(i + isc, c);
        }
    }

newton_start:
    l3 = 0;
    st.nnewt++;
    for (int i = 0; i < isc; ++i)
        for (int c = 0; c < n; ++c) { SP(cnew, i, c) = CO(i, c); SP(g->dtlos, i, c) = 0.0; }
    if (jeval == 1) {
        const double r1delt = -asn1 * delt;
        gear_pderiv(g, ncsp, r1delt, &st);
        oracle_rbdecomp(b, ncsp);
        jeval = -1;
        hratio = 1.0;
        nslp = st.nsteps + G_MBETWEEN;
        drate = 0.70;
    }

newton_iter:
    if (cfg->max_iter > 0 && st.nsubfun >= cfg->max_iter) {
        int i1 = nqqisc;   /* back to the last accepted history */
        for (int jb = 1; jb <= nqq; ++jb) {
            i1 -= isc;
            for (int i = i1; i < nqqisc; ++i)
                for (int c = 0; c < n; ++c) CO(i, c) = CO(i, c) - CO(i + isc, c);
        }
        st.status |= ST_MAXITER;
        goto failed;
    }
    gear_subfun(g, ncsp, &st);
    for (int i = 0; i < isc; ++i)
        for (int c = 0; c < n; ++c)
            SP(g->gloss, i, c) = fma(delt, SP(g->gloss, i, c), -(CO(isc + i, c) + SP(g->dtlos, i, c)));
    oracle_rbsolve(b, ncsp, g->gloss);
    for (int c = 0; c < n; ++c) g->dely[c] = 0.0;
    for (int i = 0; i < isc; ++i)
        for (int c = 0; c < n; ++c) {
            SP(g->dtlos, i, c) = SP(g->dtlos, i, c) + SP(g->gloss, i, c);
            SP(cnew, i, c) = fma(asn1, SP(g->dtlos, i, c), CO(i, c));
            const double e = SP(g->gloss, i, c) * SP(g->chold, i, c);
            g->dely[c] = fma(e, e, g->dely[c]);
        }
    rmserrp = rmserr;
    der2max = gear_maxdely(g);
    rmserr = sqrt(der2max / order);
    l3++;
    if (l3 > 1) {
        const double rmsrat = rmserr / rmserrp;
        drate = g_max2((double)0.2f * drate, rmsrat);
    }
    {
        const double dcon = rmserr * g_min2(cfg->conpst[nqq - 1], cfg->conp15[nqq - 1] * drate);
        if (dcon <= 1.0) goto converged;
    }
    if (l3 < G_MSTEP) goto newton_iter;
    /* convergence failure */
    st.ncfail++;
    if (jeval == 0) {
        jeval = 1;
        goto newton_start;
    }
    rdelmax = 2.0;
    xelaps = told;
    rdelt = G_FRACDEC;
    jeval = 1;
    ifsuccess = 0;
    {
        int i1 = nqqisc;
        for (int jb = 1; jb <= nqq; ++jb) {
            i1 -= isc;
            for (int i = i1; i < nqqisc; ++i)
                for (int c = 0; c < n; ++c) CO(i, c) = CO(i, c) - CO(i + isc, c);
        }
    }
    goto loop_order;

converged:
    jeval = 0;
    if (l3 > 1) {
        for (int c = 0; c < n; ++c) g->dely[c] = 0.0;
        for (int j = 0; j < isc; ++j)
            for (int c = 0; c < n; ++c) {
                const double e = SP(g->dtlos, j, c) * SP(g->chold, j, c);
                g->dely[c] = fma(e, e, g->dely[c]);
            }
        der2max = gear_maxdely(g);
    }
    if (der2max > enqq) {
        /* error test failure */
        st.nefail++;
        xelaps = told;
        jfail++;
        {
            int i1 = nqqisc;
            for (int jb = 1; jb <= nqq; ++jb) {
                i1 -= isc;
                for (int i = i1; i < nqqisc; ++i)
                    for (int c = 0; c < n; ++c) CO(i, c) = CO(i, c) - CO(i + isc, c);
            }
        }
        rdelmax = 2.0;
        if (jfail <= 6) {
            ifsuccess = 0;
            rdeltup = 0.0;
            higher_order = 0;
        } else if (jfail <= 20) {
            ifsuccess = 0;
            rdelt = G_FRACDEC;
            goto loop_order;
        } else {
            ifsuccess = 1;
            delt = delt * 0.1;
            rdelt = 1.0;
            jfail = 0;
            jrestar++;
            idoub = 5;
            for (int i = 0; i < isc; ++i)
                for (int c = 0; c < n; ++c) SP(cnew, i, c) = CO(i, c);
            if (jrestar == 100) {
                st.status |= ST_MAXITER;
                goto failed;
            }
            goto loop_initialize;
        }
    } else {
        /* error test passed */
        jfail = 0;
        ifsuccess = 1;
        told = xelaps;
        st.nsteps++;
        if (nqq > st.maxord) st.maxord = nqq;
        int i1 = -isc;
        for (int j = 1; j <= kstep; ++j) {
            i1 += isc;
            const double a = ASET(nqq, j);
            for (int i = i1; i < i1 + isc; ++i)
                for (int c = 0; c < n; ++c) CO(i, c) = fma(a, SP(g->dtlos, i - i1, c), CO(i, c));
        }
        for (int i = 0; i < isc; ++i)
            for (int c = 0; c < n; ++c)
                if (CO(i, c) <= G_CONCMIN) {
                    CO(i, c) = G_ZBOUND;
                    SP(cnew, i, c) = G_ZBOUND;
                    for (int k = 1; k <= 5; ++k) CO(i + k * isc, c) = 0.0;
                }
        if (g->caveg)   /* CAVEG += 0.5 (CFINI + CONC) DELT; CFINI = CONC (grsmvgear.F:841-849) */
            for (int i = 0; i < isc; ++i)
                for (int c = 0; c < n; ++c) {
                    const double cv = CO(i, c);
                    SP(g->caveg, i, c) = fma(0.5 * (SP(g->cfini, i, c) + cv), delt, SP(g->caveg, i, c));
                    SP(g->cfini, i, c) = cv;
                }
        if (idoub > 1) {
            idoub--;
            if (idoub == 1)
                for (int j = 0; j < isc; ++j)
                    for (int c = 0; c < n; ++c) SP(g->cest, j, c) = SP(g->dtlos, j, c);
            rdelt = 1.0;
            goto loop_order;
        }
    }

    /* step size and order for the next step */
    if (higher_order) {
        if (nqq < G_MAXORD) {
            for (int c = 0; c < n; ++c) g->dely[c] = 0.0;
            for (int j = 0; j < isc; ++j)
                for (int c = 0; c < n; ++c) {
                    const double e = (SP(g->dtlos, j, c) - SP(g->cest, j, c)) * SP(g->chold, j, c);
                    g->dely[c] = fma(e, e, g->dely[c]);
                }
            const double der3max = gear_maxdely(g);
            const double pr3 = (double)1.4f * gear_pow(der3max / eup, cfg->enqq3[nqq - 1]);
            rdeltup = 1.0 / (pr3 + G_OPT4MIC);
        } else {
            rdeltup = 0.0;
        }
    }
    higher_order = 1;
    {
        const double pr2 = 1.2 * gear_pow(der2max / enqq, cfg->enqq2[nqq - 1]);
        rdeltsm = 1.0 / (pr2 + G_OPT2MIC);
    }
    if (nqq > 1) {
        for (int c = 0; c < n; ++c) g->dely[c] = 0.0;
        const int col = (kstep - 1) * isc;
        for (int j = 0; j < isc; ++j)
            for (int c = 0; c < n; ++c) {
                const double e = CO(col + j, c) * SP(g->chold, j, c);
                g->dely[c] = fma(e, e, g->dely[c]);
            }
        const double der1max = gear_maxdely(g);
        const double pr1 = 1.3 * gear_pow(der1max / edwn, cfg->enqq1[nqq - 1]);
        rdeltdn = 1.0 / (pr1 + G_OPT3MIC);
    } else {
        rdeltdn = 0.0;
    }
    rdelt = g_max2(g_max2(rdeltsm, rdeltup), rdeltdn);
    if (rdelt < (double)1.1f && ifsuccess == 1) {
        idoub = 3;
        goto loop_order;
    }
    if (rdelt == rdeltdn) {
        nqq = nqq - 1;
        if (ifsuccess == 0) rdelt = g_min2(rdelt, 1.0);
    } else if (rdelt == rdeltup) {
        const double consmult = ASET(nqq, kstep) / (double)kstep;
        nqq = kstep;
        const int nqisc = nqq * isc;
        for (int j = 0; j < isc; ++j)
            for (int c = 0; c < n; ++c) CO(j + nqisc, c) = SP(g->dtlos, j, c) * consmult;
    }
    if (jfail >= 2) rdelt = g_min2(rdelt, G_PT2);
    idoub = nqq + 1;
    goto loop_order;

failed:
    /* the reference stops the run here; the cell keeps its last accepted state */
    for (int i = 0; i < isc; ++i)
        for (int c = 0; c < n; ++c) SP(cnew, i, c) = CO(i, c);
done:
    for (int i = 0; i < isc; ++i)
        for (int c = 0; c < n; ++c) {
            if (SP(cnew, i, c) <= G_ZBOUND) SP(cnew, i, c) = G_CONCMIN;
            if (!isfinite(SP(cnew, i, c))) st.status |= ST_NONFINITE;
        }
    if (g->caveg) {   /* CAVEG / CHEMSTEP floored at CONCMIN (grsmvgear.F:1007-1013) */
        const double rchem = 1.0 / chemstep;
        for (int i = 0; i < isc; ++i)
            for (int c = 0; c < n; ++c) SP(g->caveg, i, c) = g_max2(SP(g->caveg, i, c) * rchem, G_CONCMIN);
    }
#undef CO
#undef SP
#undef ASET
    return st;
}

/* Per-cell SMVGEAR (BLKSIZE = 1) of many cells: y[nspec*ncell] new order, updated in
 * place; rk[nrxns*ncell]; night[c] != 0: dark cell (night list, HMAXNIT, H0FAC 1).
 * stats[8*ncell] (may be NULL): per cell nsteps, ncfail, nefail, npderiv, nsubfun, nnewt,
 * maxord, status.  Returns the number of failed cells. */
int oracle_gear_cells(long ncell, double chemstep, const GearCfg* cfg, double* y, const double* rk,
                      const uint8_t* night, int* stats, int threads)
{
    int nbad = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : nbad)
#endif
    {
        GearBlock g;
        gear_alloc(&g, 1);
        g.b.ncells = 1;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (long c = 0; c < ncell; ++c) {
            for (int s = 0; s < MECH_NSPEC; ++s) g.b.y[s] = y[(size_t)s * ncell + c];
            memcpy(g.blkconc, g.b.y, sizeof(double) * MECH_NSPEC);
            for (int r = 0; r < MECH_NRXNS; ++r) g.b.rki[r] = rk[(size_t)r * ncell + c];
            const int dark = night[c] != 0;
            GearStats st = oracle_smvgear(&g, dark ? 1 : 0, !dark, chemstep, cfg, NULL);
            for (int s = 0; s < MECH_NSPEC; ++s) y[(size_t)s * ncell + c] = g.b.y[s];
            if (stats) {
                int* o = &stats[(size_t)8 * c];
                o[0] = st.nsteps; o[1] = st.ncfail; o[2] = st.nefail; o[3] = st.npderiv;
                o[4] = st.nsubfun; o[5] = st.nnewt; o[6] = st.maxord; o[7] = st.status;
            }
            nbad += st.status != 0;
        }
        gear_free(&g);
    }
    return nbad;
}

/* One Gear CHEM call (grdriver.F) on the whole grid with the given BLKSIZE; a->rtol is
 * GEAR_RTOL and the tolerances of cfg come from oracle_gear_cfg. */
int oracle_gear_chem(OracleChemArgs* a, const GearCfg* cfg)
{
    const long nxy = (long)a->ncols * a->nrows;
    const long noxyz = nxy * a->nlays;
    const long ncell = noxyz;
    const int blksize = a->blksize > 0 ? a->blksize : 50;
    int* ccol = malloc(sizeof(int) * noxyz);
    int* crow = malloc(sizeof(int) * noxyz);
    int* clev = malloc(sizeof(int) * noxyz);
    long nc = 0;
    for (int lev = 0; lev < a->nlays; ++lev)      /* grinit.F:176-187 */
        for (int col = 0; col < a->ncols; ++col)
            for (int row = 0; row < a->nrows; ++row) { ccol[nc] = col; crow[nc] = row; clev[nc] = lev; ++nc; }
    const long nblks = 1 + (noxyz - 1) / blksize;   /* grinit.F:189-215 */
    long iavg = 1 + (noxyz - 1) / nblks;
    if (iavg > blksize) iavg = blksize;
    long* blkcno = malloc(sizeof(long) * nblks);
    int* blklen = malloc(sizeof(int) * nblks);
    long off = 0;
    for (long k = 0; k < nblks - 1; ++k) { blkcno[k] = off; blklen[k] = (int)iavg; off += iavg; }
    blkcno[nblks - 1] = off;
    blklen[nblks - 1] = (int)(noxyz - (nblks - 1) * iavg);
    float fwd[MECH_NSPEC];
    double rev[MECH_NSPEC];
    for (int s = 0; s < MECH_NSPEC; ++s) {         /* GRVARS.F:548-551 */
        fwd[s] = 1.0e-3f * 28.9628f / (float)mech_molwt[s];
        rev[s] = (double)(1.0f / fwd[s]);
    }
    long* nordcell = malloc(sizeof(long) * noxyz);
    for (long c = 0; c < noxyz; ++c) nordcell[c] = c;
    double* errmx2 = calloc((size_t)noxyz, sizeof(double));
    const double chemstep = (double)a->tstep_sec / 60.0;
    const int lordering = (a->lreorder && nblks > 1 && blksize > 1) ? 1 : 0;
    long long tot_steps = 0, tot_fails = 0;
    int nfailed = 0;
#ifdef _OPENMP
    if (a->threads > 0) omp_set_num_threads(a->threads);
#endif
    for (int pass = 0; pass < 2; ++pass) {
        const int ordering_pass = (pass == 0 && lordering);
        if (pass == 0 && !lordering) continue;
#ifdef _OPENMP
#pragma omp parallel reduction(+ : tot_steps, tot_fails, nfailed)
#endif
        {
            GearBlock g;
            gear_alloc(&g, blksize);
            double* blktemp = malloc(sizeof(double) * blksize);
            double* blkpres = malloc(sizeof(double) * blksize);
            double* blkh2o = malloc(sizeof(double) * blksize);
            double* blkdens = malloc(sizeof(double) * blksize);
            float* blksvol = malloc(sizeof(float) * blksize);
            double* blksea = malloc(sizeof(double) * blksize);
            double* rjblk = malloc(sizeof(double) * blksize * MECH_NPHOTAB);
            double* blkhet = malloc(sizeof(double) * blksize * (MECH_NHETERO > 0 ? MECH_NHETERO : 1));
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 1)
#endif
            for (long blk = 0; blk < nblks; ++blk) {
                const int numcells = blklen[blk];
                const long offset = blkcno[blk];
                const int ncsp = gather_block(a, ccol, crow, clev, nordcell, offset, numcells, &g.b, blktemp,
                                              blkpres, blkh2o, blkdens, blksvol, blksea, rjblk, blkhet, fwd, 1);
                memcpy(g.blkconc, g.b.y, sizeof(double) * (size_t)MECH_NSPEC * blksize);
                const int lsun = ncsp == 0;
                if (ordering_pass) {
                    oracle_smvgear(&g, ncsp, lsun, chemstep, cfg, &errmx2[offset]);
                    continue;
                }
                GearStats st = oracle_smvgear(&g, ncsp, lsun, chemstep, cfg, NULL);
                tot_steps += st.nsteps;
                tot_fails += st.ncfail + st.nefail;
                nfailed += st.status != 0;
                for (int isp = 0; isp < MECH_ISCHAN; ++isp) {   /* grdriver.F:577-596 */
                    const int old = mech_inew2old[isp];
                    const int spc = a->cgrid_index[old];
                    for (int c = 0; c < numcells; ++c) {
                        const long cell = nordcell[offset + c];
                        const long gi = ccol[cell] + (long)a->ncols * (crow[cell] + (long)a->nrows * clev[cell]);
                        const double yv = g.b.y[(size_t)isp * g.b.ld + c];
                        a->conc[(size_t)spc * ncell + gi] =
                            a->convert[old] ? (float)(rev[old] * blkdens[c] * yv) : (float)yv;
                    }
                }
            }
            gear_free(&g);
            free(blktemp); free(blkpres); free(blkh2o); free(blkdens); free(blksvol); free(blksea);
            free(rjblk); free(blkhet);
        }
        if (ordering_pass) heap_sort_cells(errmx2, nordcell, noxyz);   /* grdriver.F:662-706 */
    }
    a->nsteps_total = tot_steps;
    a->nfails_total = tot_fails;
    a->nfailed_blocks = nfailed;
    free(ccol); free(crow); free(clev); free(blkcno); free(blklen); free(nordcell); free(errmx2);
    return nfailed;
}

size_t oracle_gear_cfg_size(void) { return sizeof(GearCfg); }

/* the step-size power, for the accuracy test */
double oracle_gear_pow(double x, double y) { return gear_pow(x, y); }
