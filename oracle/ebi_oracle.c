/*
 * CPU oracle for CMAQ's EBI gas-chemistry solver.  TEST INFRASTRUCTURE ONLY.
 *
 * Restates, per grid cell:
 *   oracle_chem_ebi   CCTM/src/gas/ebi_<mech>/hrdriver.F:290-460 (EBI step count, gather
 *                     with the driver's REAL(4)/REAL(8) conversions, CALC_RCONST, write-back)
 *   ebi_hrsolver      CCTM/src/gas/ebi_<mech>/hrsolver.F:212-440 (time steps, sub-steps,
 *                     Backward-Euler iterations, convergence test, step halving)
 * The mechanism-specific routines HRRATES, HRPRODLOSS, HRG1-HRG4 and the tables of
 * hrinit.F are translated from the reference into EBI_SOURCE.  Arithmetic is
 * uncontracted (-ffp-contract=off), as written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef MECH_SOURCE
#error "compile with -DMECH_SOURCE and -DEBI_SOURCE"
#endif
#include MECH_SOURCE
#include "oracle.h"

typedef struct {
    double yc[MECH_NSPEC], yc0[MECH_NSPEC], ycp[MECH_NSPEC], prod[MECH_NSPEC], loss[MECH_NSPEC],
        pneg[MECH_NSPEC];
    double rki[MECH_NRXNS], rxrat[MECH_NRXNS];
} EbiCell;

#define EBI_CELL_ARGS EbiCell* c
#define EBI_YC(i) c->yc[i]
#define EBI_YC0(i) c->yc0[i]
#define EBI_YCP(i) c->ycp[i]
#define EBI_RKI(r) c->rki[r]
#define EBI_RXRAT(r) c->rxrat[r]
#define EBI_PROD(i) c->prod[i]
#define EBI_LOSS(i) c->loss[i]
#define EBI_PNEG(i) c->pneg[i]
#include EBI_SOURCE

/* hrsolver.F:70-74 */
static const double EBI_DTMIN = 1.0e-08, EBI_EPSLON = 1.0e-30, EBI_MAXPRED = 1.0e+03, EBI_ZERO = 1.0e-40,
                    EBI_FLOOR = 1.0e-08;

/* HRSOLVER for one cell; returns 0, or ST_DT_UNDERFLOW when the sub-step fell to DTMIN
 * (the reference stops the run there).  n_it counts Backward-Euler iterations.  ycddm
 * (NULL: off): YCDDM += (0.5 DTC) (YC + YC0) at every converged sub-step (hrsolver.F:372-376). */
static int ebi_hrsolver(EbiCell* c, double ebi_tmstep, int n_ebi_steps, long* n_it, int max_iter, double* ycddm)
{
    int notmax[MECH_NSPEC];
    double dtc = ebi_tmstep;
    int nbkups = 0, n_inr_steps = 1, nebi = 1;
    int lebi_conv = 1;
    long iters = 0;
    for (int s = 0; s < MECH_NSPEC; ++s) notmax[s] = c->yc[s] <= EBI_MAXPRED;
    for (;;) {                                                   /* TSTEP_EBI */
        for (int ninr = 1; ninr <= n_inr_steps; ++ninr) {        /* SUBSTEP_EBI */
            if (lebi_conv) memcpy(c->yc0, c->yc, sizeof(c->yc));
            int converged = 0, mxfl = 0;
            for (int iter = 1; iter <= EBI_NEBITER; ++iter) {    /* ITER_SUBSTEP */
                if (max_iter > 0 && ++iters > max_iter) return ST_MAXITER;
                (*n_it)++;
                ebi_hrrates(c);
                ebi_hrg1(c, dtc);
                ebi_hrg2(c, dtc);
                ebi_hrg3(c, dtc);
                ebi_hrg4(c, dtc);
                ebi_hrprodloss(c);
                for (int e = 0; e < EBI_N_EBISP; ++e) {
                    const int s = ebi_ebisp[e];
                    c->ycp[s] = c->yc[s] * ((c->yc0[s] + c->prod[s] * dtc) / (c->yc[s] + c->loss[s] * dtc));
                }
                /* species with negative product stoichiometry (PAR in cb6r5; hrsolver.F:294-304) */
                for (int k = 0; k < EBI_NPNEG; ++k) {
                    const int p = ebi_pneg_species[k];
                    if (c->pneg[p] > 0.0) {
                        const double fxdloss = c->pneg[p] * dtc;
                        if (fxdloss >= c->yc0[p] + c->prod[p] * dtc) {
                            c->ycp[p] = 0.0;
                        } else {
                            const double varloss = fmax(c->loss[p] - c->pneg[p], EBI_ZERO);
                            c->ycp[p] = (c->yc0[p] + c->prod[p] * dtc - fxdloss) / (1.0 + varloss * dtc / c->yc[p]);
                        }
                    }
                }
                lebi_conv = 1;
                mxfl = 0;
                for (int s = 0; s < MECH_NSPEC; ++s) {
                    c->ycp[s] = fmax(EBI_ZERO, c->ycp[s]);
                    const double aerror = fmax(fabs(c->yc[s] - c->ycp[s]), EBI_EPSLON);
                    const double rerror = aerror / fmax(EBI_FLOOR, fabs(c->yc[s] + c->ycp[s]));
                    if (rerror > ebi_rtol[s] || aerror > 1.0e-5) lebi_conv = 0;
                    if (c->ycp[s] > EBI_MAXPRED && notmax[s]) {
                        mxfl = 1;
                        lebi_conv = 0;
                    }
                    c->yc[s] = c->ycp[s];
                }
                if (mxfl) break;
                if (lebi_conv) {
                    converged = 1;
                    if (ycddm)
                        for (int s = 0; s < MECH_NSPEC; ++s) ycddm[s] = fma(0.5 * dtc, c->yc[s] + c->yc0[s], ycddm[s]);
                    break;
                }
            }
            if (converged) continue;
            /* iterating for the sub-step failed: halve it, redo from YC0 */
            nbkups++;
            if (dtc > EBI_DTMIN) {
                memcpy(c->yc, c->yc0, sizeof(c->yc));
                dtc = 0.5 * dtc;
                n_inr_steps = 1 << nbkups;
                break;
            }
            return ST_DT_UNDERFLOW;
        }
        if (lebi_conv) {
            nebi++;
            if (nebi > n_ebi_steps) break;
            if (nbkups == 0) continue;
            nbkups = 0;
            n_inr_steps = 1;
            dtc = ebi_tmstep;
        }
    }
    return 0;
}

/* EBI step count and length (hrdriver.F:296-308) */
static void ebi_steps(int itmstep, int* n_ebi_steps, double* ebi_tmstep)
{
    const double chemstep = (double)itmstep / 60.0;
    const int delt_sec = (int)(EBI_DELTAT * 60.0 + 0.1);
    if (delt_sec >= itmstep) {
        *n_ebi_steps = 2;
        *ebi_tmstep = 0.5 * chemstep;
    } else {
        *n_ebi_steps = (itmstep % delt_sec == 0) ? itmstep / delt_sec : itmstep / delt_sec + 1;
        *ebi_tmstep = chemstep / (double)(*n_ebi_steps);
    }
}

int oracle_ebi_nebisp(void) { return EBI_N_EBISP; }

/* Solver level: n cells with given concentrations yc[nspec][n] (mechanism order, in place)
 * and rate constants rki[nrxns][n].  Returns the number of failed cells. */
int oracle_ebi_solve_cells(long n, int tstep_sec, double* yc, const double* rki, int* status, long* iters,
                           int threads)
{
    int n_ebi_steps;
    double ebi_tmstep;
    ebi_steps(tstep_sec, &n_ebi_steps, &ebi_tmstep);
    int nbad = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : nbad)
#endif
    for (long i = 0; i < n; ++i) {
        EbiCell c;
        memset(&c, 0, sizeof(c));
        for (int s = 0; s < MECH_NSPEC; ++s) c.yc[s] = yc[(size_t)s * n + i];
        for (int r = 0; r < MECH_NRXNS; ++r) c.rki[r] = rki[(size_t)r * n + i];
        long it = 0;
        const int st = ebi_hrsolver(&c, ebi_tmstep, n_ebi_steps, &it, 0, NULL);
        for (int s = 0; s < MECH_NSPEC; ++s) yc[(size_t)s * n + i] = c.yc[s];
        if (status) status[i] = st;
        if (iters) iters[i] = it;
        nbad += st != 0;
    }
    return nbad;
}

/* HRSOLVER for one cell (yc mechanism order, in place) with the DDM-3D average YCDDM of
 * the call: zeroed first (hrsolver.F:169-171), divided by CHEMSTEP and values below 1e-25
 * set to zero after (:443-447), also when the cell failed.  Returns the cell's status. */
int oracle_ebi_cell(double* yc, const double* rki, int tstep_sec, double* ycddm)
{
    int n_ebi_steps;
    double ebi_tmstep;
    ebi_steps(tstep_sec, &n_ebi_steps, &ebi_tmstep);
    EbiCell c;
    memset(&c, 0, sizeof(c));
    memcpy(c.yc, yc, sizeof(c.yc));
    memcpy(c.rki, rki, sizeof(c.rki));
    for (int s = 0; s < MECH_NSPEC; ++s) ycddm[s] = 0.0;
    long it = 0;
    const int st = ebi_hrsolver(&c, ebi_tmstep, n_ebi_steps, &it, 0, ycddm);
    const double chemstep = (double)tstep_sec / 60.0;
    for (int s = 0; s < MECH_NSPEC; ++s) {
        ycddm[s] = ycddm[s] / chemstep;
        if (ycddm[s] < 1.0e-25) ycddm[s] = 0.0;
    }
    memcpy(yc, c.yc, sizeof(c.yc));
    return st;
}

/* The EBI driver's gather of every cell (hrdriver.F:372-415): yc[nspec][ncell] mechanism
 * order, rki[nrxns][ncell] from CALC_RCONST, night[ncell] = no sunlight. */
void oracle_ebi_gather(const OracleChemArgs* a, double* yc, double* rki, uint8_t* night)
{
    const long nxy = (long)a->ncols * a->nrows;
    const long ncell = nxy * a->nlays;
    float fwd[MECH_NSPEC];
    for (int s = 0; s < MECH_NSPEC; ++s) fwd[s] = (float)((double)(1.0e-3f * 28.9628f) / mech_molwt[s]);
    const double pa2atm = (double)(1.0f / 101325.0f);
    const float maomv = 1.0e6f * 28.9628f / 18.0153f;
    for (long g = 0; g < ncell; ++g) {
        const long col2 = g % nxy;
        const float inv_dens = 1.0f / a->dens[g];
        for (int s = 0; s < MECH_NSPEC; ++s) {
            const float cv = a->conc[(size_t)a->cgrid_index[s] * ncell + g];
            yc[(size_t)s * ncell + g] =
                a->convert[s] ? (double)fmaxf(1.0e-30f, inv_dens * fwd[s] * cv) : (double)fmaxf(cv, 1.0e-30f);
        }
        const double temp = (double)a->ta[g];
        const double atmpres = pa2atm * (double)a->pres[g];
        const double h2o = (double)fmaxf(maomv * a->qv[g], 0.0f);
        const double seawater = fmax(0.0, (double)(a->ocean_szone[col2] - a->seaice[col2]));
        double rjin[MECH_NPHOTAB], het[MECH_NHETERO > 0 ? MECH_NHETERO : 1], rk[MECH_NRXNS];
        int lsun = 0;
        for (int k = 0; k < MECH_NPHOTAB; ++k) {
            rjin[k] = (double)a->rj[(size_t)k * ncell + g];
            if (rjin[k] > 0.0) lsun = 1;
        }
        for (int k = 0; k < MECH_NHETERO; ++k) het[k] = a->khetero[(size_t)g * MECH_NHETERO + k];
        mech_calc_rconst(1, 1, &temp, &atmpres, &h2o, rjin, het, lsun, &seawater, rk);
        for (int r = 0; r < MECH_NRXNS; ++r) rki[(size_t)r * ncell + g] = rk[r];
        night[g] = lsun ? 0 : 1;
    }
}

/* One EBI CHEM call (hrdriver.F) on the whole grid. */
int oracle_chem_ebi(OracleChemArgs* a)
{
    const long nxy = (long)a->ncols * a->nrows;
    const long ncell = nxy * a->nlays;
    int n_ebi_steps;
    double ebi_tmstep;
    ebi_steps(a->tstep_sec, &n_ebi_steps, &ebi_tmstep);
    /* hrinit.F:90-93: REAL(4) factors; the molecular weights are REAL(8) */
    float fwd[MECH_NSPEC], rev[MECH_NSPEC];
    for (int s = 0; s < MECH_NSPEC; ++s) {
        fwd[s] = (float)((double)(1.0e-3f * 28.9628f) / mech_molwt[s]);
        rev[s] = (float)((double)(1.0e+3f / 28.9628f) * mech_molwt[s]);
    }
    const double pa2atm = (double)(1.0f / 101325.0f);          /* hrdriver.F:224 */
    const float maomv = 1.0e6f * 28.9628f / 18.0153f;         /* hrdriver.F:106 */
    long long tot_it = 0;
    int nbad = 0;
#ifdef _OPENMP
    if (a->threads > 0) omp_set_num_threads(a->threads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : tot_it, nbad)
#endif
    for (long g = 0; g < ncell; ++g) {
        EbiCell c;
        memset(&c, 0, sizeof(c));
        const long col2 = g % nxy;
        const float inv_dens = 1.0f / a->dens[g];
        for (int s = 0; s < MECH_NSPEC; ++s) {
            const float cv = a->conc[(size_t)a->cgrid_index[s] * ncell + g];
            c.yc[s] = a->convert[s] ? (double)fmaxf(1.0e-30f, inv_dens * fwd[s] * cv) : (double)fmaxf(cv, 1.0e-30f);
        }
        const double temp = (double)a->ta[g];
        const double atmpres = pa2atm * (double)a->pres[g];
        const double h2o = (double)fmaxf(maomv * a->qv[g], 0.0f);
        const double seawater = fmax(0.0, (double)(a->ocean_szone[col2] - a->seaice[col2]));
        double rjin[MECH_NPHOTAB], het[MECH_NHETERO > 0 ? MECH_NHETERO : 1];
        int lsun = 0;
        for (int k = 0; k < MECH_NPHOTAB; ++k) {
            rjin[k] = (double)a->rj[(size_t)k * ncell + g];
            if (rjin[k] > 0.0) lsun = 1;
        }
        for (int k = 0; k < MECH_NHETERO; ++k) het[k] = a->khetero[(size_t)g * MECH_NHETERO + k];
        mech_calc_rconst(1, 1, &temp, &atmpres, &h2o, rjin, het, lsun, &seawater, c.rki);
        long it = 0;
        const int st = ebi_hrsolver(&c, ebi_tmstep, n_ebi_steps, &it, a->max_iter, NULL);
        tot_it += it;
        nbad += st != 0;
        const float dens = a->dens[g];
        for (int s = 0; s < MECH_NSPEC; ++s) {
            const double y = fmax(c.yc[s], 1.0e-30);
            a->conc[(size_t)a->cgrid_index[s] * ncell + g] =
                a->convert[s] ? (float)((double)(rev[s] * dens) * y) : (float)y;
        }
    }
    a->nsteps_total = tot_it;
    a->nfails_total = 0;
    a->nfailed_blocks = nbad;
    return nbad;
}
