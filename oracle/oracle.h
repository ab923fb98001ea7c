/* Shared declarations of the CPU oracle (test infrastructure only). */
#ifndef ORACLE_H
#define ORACLE_H

/* per-cell status bits (same meaning as the device code's) */
#define ST_DT_UNDERFLOW 1
#define ST_MAXITER 2
#define ST_NONFINITE 4

/* One CHEM call: arrays in CMAQ's Fortran layouts (see include/cmaqchem.h). */
typedef struct {
    int ncols, nrows, nlays, nspcsd;
    float* conc;                 /* CONC(ncols, nrows, nlays, nspcsd) Fortran order */
    const int* cgrid_index;      /* [nspec] 0-based */
    const int* convert;          /* [nspec] */
    const float* ta, *qv, *dens, *pres;      /* (ncols, nrows, nlays) */
    const float* seaice, *ocean_szone;       /* (ncols, nrows) */
    const float* rj;             /* (ncols, nrows, nlays, nphotab) */
    const double* khetero;       /* (nhet, ncols, nrows, nlays) */
    int tstep_sec;               /* TIME2SEC(TSTEP(2)) */
    double rtol, atol;           /* REAL(GLBL_RTOL, 8), REAL(GLBL_ATOL, 8) */
    int blksize;                 /* BLKSIZE (50 in the reference) */
    int lreorder;                /* LREORDER */
    int max_iter;
    int threads;
    /* outputs */
    long long nsteps_total, nfails_total;
    int nfailed_blocks;
} OracleChemArgs;

#endif
