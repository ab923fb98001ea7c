/*
 * cmaqchem.h -- C ABI of the GB300 gas-phase chemistry library (libcmaqchem.so).
 *
 * The library replaces the body of CMAQ's gas-chemistry operator
 *
 *     SUBROUTINE CHEM( CONC, JDATE, JTIME, TSTEP )
 *         CCTM/src/gas/ros3/rbdriver.F:20-785          (ROS3 solver)
 *         CCTM/src/gas/ebi_cb6r5_ae7_aq/hrdriver.F:20  (EBI solver)
 *         CCTM/src/gas/smvgear/grdriver.F:16           (SMVGEAR solver)
 *     called once per synchronisation step from CCTM/src/driver/sciproc.F:298
 *
 * The operator's implicit inputs, which the Fortran reads through modules, are
 * explicit arguments here: the met fields that CHEM interpolates to the step
 * midpoint (rbdriver.F:390-403), OCEAN + SZONE (rbdriver.F:253-259), the
 * photolysis rates RJ of PHOT_MOD and the heterogeneous rates KHETERO of
 * AEROSOL_CHEMISTRY (rbdriver.F:409, 499-511).
 *
 * Array layouts are the reference's Fortran layouts, so a Fortran caller passes
 * its arrays unchanged (the ISO_C_BINDING drop-in chem_gpu.F beside this header):
 *     conc    CONC(NCOLS, NROWS, NLAYS, NSPCSD)   REAL(4)
 *     ta, qv, dens, pres  (NCOLS, NROWS, NLAYS)   REAL(4)  K, kg/kg, kg/m3, Pa
 *     seaice, ocean_szone (NCOLS, NROWS)          REAL(4)  fractions
 *     rj      RJ(NCOLS, NROWS, NLAYS, NPHOTAB)    REAL(4)  1/min
 *     khetero KHETERO(NHETERO, NCOLS, NROWS, NLAYS) REAL(8)
 *
 * Errors: the reference stops the run (M3EXIT) on a step-size underflow
 * (rbsolver.F:532-585).  Here every call returns an int: 0 success, > 0 the
 * number of cells whose integration failed (their last accepted state is written
 * back and their status is available per cell), < 0 a fatal error whose text
 * cmaqchem_last_error() returns.  A handle is not re-entrant; use one handle per
 * thread.  No pointer passed in is retained after a call returns.
 */
#ifndef CMAQCHEM_H
#define CMAQCHEM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CMAQCHEM_SOLVER_ROS3 0
#define CMAQCHEM_SOLVER_EBI 1
#define CMAQCHEM_SOLVER_GEAR 2   /* SMVGEAR; cfg.rtol = REAL(GEAR_RTOL, 8), cfg.atol = REAL(GEAR_MIN_ATOL, 8) */

/* How cells are scheduled on the GPU; every mode integrates each cell with its own
 * step size (the reference with BLKSIZE = 1). */
#define CMAQCHEM_SCHED_STATIC 0   /* fixed cell -> thread assignment ("plain") */
#define CMAQCHEM_SCHED_QUEUE 1    /* persistent kernel, cells pulled from a work queue ("batched") */

/* per-cell status bits */
#define CMAQCHEM_CELL_DT_UNDERFLOW 1
#define CMAQCHEM_CELL_MAXITER 2
#define CMAQCHEM_CELL_NONFINITE 4

typedef struct cmaqchem_handle cmaqchem_handle;

typedef struct {
    const char* mechanism;     /* "cb6r5_ae7_aq" or "cracmm2" (MECHNAME of RXNS_DATA) */
    int solver;                /* CMAQCHEM_SOLVER_* */
    int schedule;              /* CMAQCHEM_SCHED_* */
    double rtol;               /* RTOL = REAL(GLBL_RTOL, 8) (rbinit.F:251; RUNTIME_VARS.F:178) */
    double atol;               /* ATOL = REAL(GLBL_ATOL, 8) [ppmV] (rbinit.F:250; RUNTIME_VARS.F:177) */
    int ncols, nrows, nlays;   /* local domain of this process (GRID_CONF) */
    int nspcsd;                /* number of CGRID species (CGRID_SPCS) */
    const int* cgrid_index;    /* [nspec] CGRID slot (1-based, as CGRID_INDEX) or NULL for the mechanism's table */
    int device;                /* CUDA device ordinal */
    int max_iter;              /* cap per cell and call on ROS3 step attempts or EBI iterations (<= 0: 100000) */
} cmaqchem_cfg;

/* With CMAQCHEM_SOLVER_EBI, accepted_steps counts Backward-Euler iterations and
 * rejected_steps / sunlit_attempts stay 0.  With CMAQCHEM_SOLVER_GEAR, rejected_steps
 * counts corrector convergence failures plus error-test failures. */
typedef struct {
    long long accepted_steps;  /* summed over cells */
    long long rejected_steps;
    long long failed_cells;    /* cells with a non-zero status */
    long long sunlit_cells;
    long long sunlit_attempts; /* step attempts (accepted + rejected) of sunlit cells */
    double device_ms;          /* device time of the call's kernels */
} cmaqchem_stats;

typedef struct {
    int nspec, nrxns, ischan, nphotab, nhetero;
    int iarray_day, iarray_night;       /* stored LU entries (day / night pattern) */
    double flops_step_day;              /* algorithmic FLOPs of one ROS3 step attempt of one cell */
    double flops_step_night;
} cmaqchem_mech_info;

/* Replaces the first-call set-up of CHEM: RBINIT, RBSPARSE, RESET_SPECIES_POINTERS
 * (rbdriver.F:226-371).  Allocates device tables and workspaces for the domain. */
int cmaqchem_init(const cmaqchem_cfg* cfg, cmaqchem_handle** out);

/* One CHEM call on host arrays (rbdriver.F:373-785): copies the inputs to the device,
 * integrates every cell over TSTEP(2) and copies CONC back.  tstep = TSTEP(3) HHMMSS.
 * Only the mechanism's CONC planes travel; with the work-queue schedule the grid moves
 * in chunks of consecutive cells whose copies overlap the integration of the previous
 * chunk.  Pinned host memory makes the copies asynchronous. */
int cmaqchem_step(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                  const float* dens, const float* pres, const float* seaice,
                  const float* ocean_szone, const float* rj, const double* khetero,
                  int jdate, int jtime, const int tstep[3], cmaqchem_stats* stats);

/* Same call on device-resident arrays (same layouts), enqueued on `stream` (a
 * cudaStream_t; NULL: the handle's own stream, which first waits for the work already on
 * the legacy default stream, so inputs written there are complete).  The entries below
 * that take a handle and a stream treat NULL the same way.  Returns after the stream is
 * idle. */
int cmaqchem_step_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                         const float* dens, const float* pres, const float* seaice,
                         const float* ocean_szone, const float* rj, const double* khetero,
                         int jdate, int jtime, const int tstep[3], void* stream,
                         cmaqchem_stats* stats);

/* nsteps consecutive CHEM calls on device arrays (same arguments as
 * cmaqchem_step_device), for hosts that run chemistry alone over several
 * synchronisation steps: the launches of one call are captured once as a CUDA graph
 * (re-captured when a pointer, TSTEP(2) or a tuning knob changes) and replayed nsteps
 * times with no host synchronisation in between; stats are summed over the calls.
 * The first call on a handle captures on the handle's own stream, so it must not be
 * made while another stream of the process is being captured. */
int cmaqchem_steps_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                          const float* dens, const float* pres, const float* seaice,
                          const float* ocean_szone, const float* rj, const double* khetero,
                          int jdate, int jtime, const int tstep[3], int nsteps, void* stream,
                          cmaqchem_stats* stats);

/* One CHEM call with first-order DDM-3D sensitivities (CCTM/src/ddm3d/DDM3D_CHEM.F:155,
 * SOLVE_DDM3D_CHEM, called per cell from rbdriver.F:619-651): after the concentrations,
 * every parameter's sensitivities in sengrid, the reference's SENGRID(NCOLS, NROWS, NLAYS,
 * NPMAX, NSPCSD) REAL(4) with nparam = NPMAX, advance over the step.  rate_mask
 * [nparam][nrxns] (device, may be NULL) marks the reactions of reaction-rate parameters
 * (IPT = 5: IRXN(NP, RXN) = 1); region [nparam][ncols*nrows*nlays] (device, may be NULL
 * for 1) weights their source as IREGION does.  Parameters with no reaction in the mask
 * (initial and boundary conditions, emissions) only propagate.  Any solver: the
 * time-averaged concentrations are ROS3's YAVE, SMVGEAR's CAVEG or EBI's YCDDM (the
 * sens blocks of rbsolver.F, grsmvgear.F and hrsolver.F). */
int cmaqchem_step_ddm_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                             const float* dens, const float* pres, const float* seaice,
                             const float* ocean_szone, const float* rj, const double* khetero,
                             int jdate, int jtime, const int tstep[3], float* sengrid, int nparam,
                             const unsigned char* rate_mask, const float* region, void* stream,
                             cmaqchem_stats* stats);

/* Per-cell status of the last step call (CMAQCHEM_CELL_* bits) and step attempts,
 * copied to host arrays of ncols*nrows*nlays ints (either may be NULL). */
int cmaqchem_cell_stats(cmaqchem_handle* h, int* status, int* attempts);

/* Solver-level entry replacing RBSOLVER (rbsolver.F:26) for cells with given rate
 * constants, device arrays:  y[ischan][ncell] in the solver's species order, updated in
 * place; rki[nrxns][ncell] (ppm, min units); night[ncell] = 1 for cells without
 * sunlight (night reaction list, rbsparse.F:275-279).  Per-cell outputs may be NULL. */
int cmaqchem_ros3_solve_device(cmaqchem_handle* h, long long ncell, double* y, const double* rki,
                               const unsigned char* night, double chemstep_min, int* status,
                               int* nsteps, int* nfails, void* stream);

/* Solver-level entry replacing HRSOLVER (CCTM/src/gas/ebi_<mech>/hrsolver.F:26) for cells
 * with given rate constants, device arrays: yc[nspec][ncell] in the mechanism's species
 * order (ppm), updated in place; rki[nrxns][ncell].  tstep_sec is the synchronisation
 * step in seconds, split into EBI steps as hrdriver.F:296-308 does.  Per-cell status
 * (CMAQCHEM_CELL_* bits) and Backward-Euler iteration counts may be NULL. */
int cmaqchem_ebi_solve_device(cmaqchem_handle* h, long long ncell, double* yc, const double* rki,
                              int tstep_sec, int* status, int* iterations, void* stream);

/* Solver-level entry replacing SMVGEAR (CCTM/src/gas/smvgear/grsmvgear.F:26) for cells with
 * given rate constants, one cell per block (BLKSIZE = 1), device arrays: y[nspec][ncell]
 * in the solver's species order (ppm), updated in place; rk[nrxns][ncell];
 * night[ncell] = 1 for cells without sunlight (night reaction list, HMAXNIT, H0FAC = 1).
 * The handle must have been made with CMAQCHEM_SOLVER_GEAR.  cell_stats (may be NULL)
 * receives per cell 8 ints: accepted steps, convergence failures, error-test failures,
 * Jacobian evaluations, right-hand-side evaluations, Newton starts, highest order used
 * and status (CMAQCHEM_CELL_* bits). */
int cmaqchem_gear_solve_device(cmaqchem_handle* h, long long ncell, double* y, const double* rk,
                               const unsigned char* night, double chemstep_min, int* cell_stats, void* stream);

/* SMVGEAR tolerances of a CMAQCHEM_SOLVER_GEAR handle, as the run-time settings
 * GEAR_MAX_ATOL, GEAR_MIN_ATOL and GEAR_CONC_FLOOR (ppmV, REAL(4); defaults 1e-7,
 * cfg.atol and 1e-12) from which OPTIMAL_ATOL_PPM picks each cell's absolute tolerance
 * (CCTM/src/gas/smvgear/GRVARS.F:597-708).  max_atol > min_atol > conc_floor. */
int cmaqchem_gear_tolerances(cmaqchem_handle* h, float max_atol, float min_atol, float conc_floor);

/* Discrete adjoint of RBSOLVER (no reference counterpart; the reference's gradient
 * tool is the forward DDM-3D of CCTM/src/ddm3d/DDM3D_CHEM.F).  Solver-level, device
 * arrays, species in the solver's order as for cmaqchem_ros3_solve_device.
 *
 * cmaqchem_adj_forward integrates nsync synchronisation steps of chemstep_min minutes
 * with rate constants rki[nrxns][ncell] (step k uses rki + k * rki_sync_stride; stride
 * 0 for constant rates) times kmult[nrxns] (NULL: 1) and the emission tendency
 * emis[ischan][ncell] ppm/min added to f (NULL: 0).  y[ischan][ncell] is advanced in
 * place; the state at the start of step k goes to checkpoints[k][ischan][ncell] and its
 * accepted steps per cell to nsteps[k][ncell].  Returns the number of failed cell-steps.
 *
 * tape (device, tape_bytes long, may be NULL) receives the state and step size of every
 * accepted step as the forward pass takes it, in linked blocks of 4 steps per cell and
 * synchronisation step: about (ischan + 1) * 8 bytes per accepted step plus 12 bytes
 * per cell and step.  Steps that do not fit are recorded as incomplete.
 *
 * cmaqchem_adj_backward takes lambda = dL/dy at the end of the window and returns in
 * it dL/dy at the start; it adds dL/d log kmult to grad_logk[nrxns] and dL/demis to
 * grad_emis[ischan][ncell] (may be NULL).  The other arguments must be those of the
 * forward call, whose checkpoints, step counts and tape it reads; the accepted step
 * sizes are held fixed (the discrete adjoint of the steps the forward pass took).  A
 * step whose tape is missing or incomplete is re-run from its checkpoint, which needs
 * device memory for that step's accepted steps: sum(nsteps[k]) * (ischan + 1) doubles
 * (bounded by the "adjoint_tape_mb" knob, cmaqchem_diag.h). */
int cmaqchem_adj_forward(cmaqchem_handle* h, long long ncell, double* y, const double* rki,
                         long long rki_sync_stride, const unsigned char* night, const double* kmult,
                         const double* emis, int nsync, double chemstep_min, double* checkpoints,
                         int* nsteps, void* tape, size_t tape_bytes, void* stream);
int cmaqchem_adj_backward(cmaqchem_handle* h, long long ncell, double* lambda, const double* rki,
                          long long rki_sync_stride, const unsigned char* night, const double* kmult,
                          const double* emis, int nsync, double chemstep_min, const double* checkpoints,
                          const int* nsteps, const void* tape, size_t tape_bytes, double* grad_logk,
                          double* grad_emis, void* stream);

/* Rate constants only (CALC_RCONST, RXNS_FUNC_MODULE.F90) for the handle's grid, device
 * arrays: rki[nrxns][ncell], sunlit[ncell]. */
int cmaqchem_rconst_device(cmaqchem_handle* h, const float* conc, const float* ta, const float* qv,
                           const float* dens, const float* pres, const float* seaice,
                           const float* ocean_szone, const float* rj, const double* khetero,
                           double* rki, unsigned char* sunlit, void* stream);

/* Mechanism sizes and species order (replaces RXNS_DATA / RBDATA module queries).
 * inew2old may be NULL, else it receives nspec ints (solver order -> mechanism order). */
int cmaqchem_mech_info_get(const char* mechanism, cmaqchem_mech_info* info, int* inew2old);

void cmaqchem_destroy(cmaqchem_handle* h);

/* Allocation-free variant of cmaqchem_ros3_solve_device.  It has no counterpart in the
 * reference.  It is for callers that cannot allocate device memory where they call the
 * chemistry: host models that own the whole device footprint through their own memory
 * pool, callers under a fixed device-memory budget, and loops that cannot accept the
 * device-wide synchronisation of cudaMalloc / cudaFree.  No handle is needed and the
 * call allocates nothing: the solver's workspace is a file-scope device array of
 * CMAQCHEM_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until exit;
 * the caller passes the device arrays y, rki, night and (optionally) status exactly as
 * for cmaqchem_ros3_solve_device.  The first call on a device, with that device current,
 * looks up the array's device address; make that first call before any stream capture.
 * The address is kept for the life of the process, so a cudaDeviceReset leaves it stale:
 * do not call this entry point again after resetting the device.  All calls share the
 * array: calls whose kernels overlap on the GPU race and must be serialised by the
 * caller.  ncell above CMAQCHEM_NOALLOC_MAX_CELLS is rejected, as is a mechanism whose
 * per-block workspace does not fit the array.  Runs on the current device and
 * synchronises `stream` before it returns 0, or -1 (text from cmaqchem_last_error). */
#define CMAQCHEM_NOALLOC_SCRATCH_BYTES (64ull << 20)
#define CMAQCHEM_NOALLOC_MAX_CELLS (1ll << 31)
int cmaqchem_ros3_solve_noalloc(const char* mechanism, long long ncell, double* y, const double* rki,
                                const unsigned char* night, double chemstep_min, double rtol,
                                double atol, int* status, void* stream);

/* KMT2 aqueous cloud chemistry (CCTM/src/cloud/acm_ae7_kmt2): the kinetic core of AQCHEM
 * (aqchem_kmt.F90:371-543: Henry's law constants, Initialize, Update_RCONST and the KPP
 * Rodas3 integration over TAUCLD) for ncell cloudy cells on the current device.  No
 * handle; the caller supplies a device workspace of cmaqchem_kmt2_workspace_doubles(nlanes)
 * doubles (nlanes >= 1): nlanes threads integrate the cells, each taking the next cell
 * of a queue (a counter at the end of the workspace, cleared on `stream` by the call)
 * when its cell ends, so one call's workspace serves any ncell.  Device arrays,
 * [element][cell]:
 *   params  [CMAQCHEM_KMT2_NPARAM][ncell]: TEMP2 (K), PRES_PA (Pa), TAUCLD (s), PRCRATE (mm/h),
 *           WCAVG, WTAVG (kg/m3), AIRM (mol/m2), ALFA0, ALFA3 (1/s), COSZEN, JH2O2 (1/s),
 *           GAS(LHO) (mol/mol), ISPC8, MTPYRAC, PHOTO (0/1); AQCHEM's REAL arguments are read
 *           as float, as the reference has them;
 *   var_mix [CMAQCHEM_KMT2_NVAR][ncell]: the KPP state as Initialize maps GAS and AEROSOL
 *           (aqchem_Initialize.F90:308-421, mol/molV; L_HPLUS and L_OHMIN are recomputed);
 *   var_out [CMAQCHEM_KMT2_NVAR][ncell]: the state at TAUCLD (molec/cm3, KPP's units);
 *           NaN for a cell whose set-up failed (IERR -101 or -102);
 *   fix_out [CMAQCHEM_KMT2_NFIX][ncell] or NULL: the fixed species (NaN as var_out);
 *   stats   [CMAQCHEM_KMT2_NSTAT][ncell] int: steps, accepted, rejected, f and J evaluations,
 *           factorisations, solves, singular factorisations, IERR (1 = success; < 0: the
 *           reference's ros_ErrorMsg codes, -101 / -102 for its MET DATA and initial pH
 *           errors, -100 after 16 integration passes), integration passes.
 * Synchronises the stream; returns 0, or -1 on bad arguments or a CUDA error. */
#define CMAQCHEM_KMT2_NVAR 161
#define CMAQCHEM_KMT2_NFIX 4
#define CMAQCHEM_KMT2_NPARAM 15
#define CMAQCHEM_KMT2_NSTAT 10
long long cmaqchem_kmt2_workspace_doubles(long long nlanes);
/* The lanes that fill `device` (its SMs times the resident lanes per SM the kernels are
 * built for), or -1 without such a device. */
long long cmaqchem_kmt2_default_lanes(int device);
/* The same integration on host arrays (same [element][cell] layouts; a Fortran caller
 * passes PARAMS(N, 15), VAR_MIX(N, 161), VAR_OUT(N, 161), FIX_OUT(N, 4) or NULL, STATS(N, 10))
 * on `device`: device buffers and the workspace are allocated for the call, the copies
 * are synchronous.  Returns 0 or -1. */
int cmaqchem_kmt2_solve(long long ncell, const double* params, const double* var_mix, double* var_out,
                        double* fix_out, int* stats, int device);
int cmaqchem_kmt2_solve_device(long long ncell, const double* params, const double* var_mix, double* var_out,
                               double* fix_out, int* stats, double* workspace, long long workspace_doubles,
                               void* stream);

/* The whole KMT2 AQCHEM (CCTM/src/cloud/acm_ae7_kmt2/aqchem_kmt.F90:21-978) for ncell cloudy
 * cells: the fractional weights and mass-balance start, Initialize's mapping of GAS and
 * AEROSOL into the KPP state (aqchem_Initialize.F90:290-421), the kinetic core of
 * cmaqchem_kmt2_solve_device, and the redistribution into GAS, AEROSOL, GASWDEP and AERWDEP
 * (aqchem_kmt.F90:546-976).  Device arrays, [element][cell]:
 *   params   [CMAQCHEM_KMT2_NPARAM][ncell] as for cmaqchem_kmt2_solve_device (the HO row is
 *            not read: GAS carries HO);
 *   gas      [CMAQCHEM_AQ_NGAS][ncell] in and out, AQ_DATA.F's order: SO2, HNO3, N2O5, CO2,
 *            NH3, H2O2, O3, FOA, MHP, PAA, H2SO4, HCL, GLY, MGLY, HO, IEPOX, IMAE, IHMML,
 *            HO2, NO2, HONO, HNO4, GCOL, CCOOH, HCHO, NO3RAD, CH3O2, HCHOP, PYRUV (mol/molV);
 *   aerosol  [naer * 3][ncell] in and out: AEROSOL(NAER, NMODES) flattened, surrogate i of
 *            mode m (0 Aitken, 1 accumulation, 2 coarse) at row i + naer * m;
 *   aer_index [CMAQCHEM_AQ_NSURROGATE] (host array): rows of AQCHEM's surrogates in the
 *            caller's aerosol list, in the order SO4, NH4, NO3, CL, NA, EC, POA, PRI, SOA,
 *            NUM, SOILC, SEASC, ANTHC, CAACC, MGACC, KACC, FEACC, MNACC, ORGC, TRACER_AKN,
 *            TRACER_ACC, TRACER_COR, PHG_AKN, PHG_ACC, PHG_COR, IETET, IEOS, DIMER, IMGA,
 *            IMOS, ISO3 (AQ_DATA.F's LSO4 ... LISO3, 0-based);
 *   factors  [CMAQCHEM_AQ_NFACTOR] (host array): the coarse crustal factors AQCHEM computes on
 *            its first call (aqchem_kmt.F90:329-365), SOIL_FE, CORS_FE, SOIL_MN, CORS_MN,
 *            SEAS_NA, SOIL_NA, CORS_NA, SEAS_MG, SOIL_MG, CORS_MG, SEAS_CA, SOIL_CA, CORS_CA,
 *            SEAS_K, SOIL_K, CORS_K;
 *   gas_wdep [CMAQCHEM_AQ_NGAS][ncell], aer_wdep [naer * 3][ncell] out (mm mol/L);
 *   out      [CMAQCHEM_AQ_NOUT][ncell] out: HPWDEP, BETASO4, FRACTR, FRACPOA, FRACPRI,
 *            FRACSOA, and the four mass-balance percentages AQCHEM checks (S, N without
 *            NH3, NH3/NH4, Cl), whose magnitude above 0.5 makes the reference warn;
 *   stats    [CMAQCHEM_KMT2_NSTAT][ncell] int as for cmaqchem_kmt2_solve_device.
 * A cell whose set-up fails gets NaN in every output.  The workspace is that of
 * cmaqchem_kmt2_solve_device (the mapped state lives in it between the mapping and the
 * set-up).  Synchronises the stream; returns 0 or -1. */
#define CMAQCHEM_AQ_NGAS 29
#define CMAQCHEM_AQ_NSURROGATE 31
#define CMAQCHEM_AQ_NFACTOR 16
#define CMAQCHEM_AQ_NOUT 10
int cmaqchem_aqchem_device(long long ncell, const double* params, double* gas, double* aerosol, int naer,
                           const int* aer_index, const double* factors, double* gas_wdep, double* aer_wdep,
                           double* out, int* stats, double* workspace, long long workspace_doubles, void* stream);

/* Heterogeneous rate constants KHETERO: HETCHEM_RATES (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:
 * 282-1535, with HETCHEM_EXTRACT_AERO, extract_aero, calcmoments, getpar, N2O5_GAMMA,
 * CALCISOPGAMMAS and PNCOM_LOSS) for ncell = NCOLS * NROWS * NLAYS grid cells, the step the
 * reference runs before CHEM (rbdriver.F:409).  Device arrays:
 *   ae       CONC(1, 1, 1, AE_STRT): the aerosol block of CGRID, nae rows of ncell REAL (ug/m3;
 *            NUM* #/m3; SRF* m2/m3), the AE namelist's species expanded by mode;
 *   ta, pres, qv, dens  (NCOLS, NROWS, NLAYS) REAL: K, Pa, kg/kg, kg/m3;
 *   khetero  KHETERO(NHETERO, NCOLS, NROWS, NLAYS) REAL(8) out, the mechanism's HETERO order,
 *            the array the CHEM entries take.
 * cmaqchem_hetchem_layout gives the block's rows, its first row in the mechanism's CGRID
 * (0-based) and NHETERO.  Built for cb6r5_ae7_aq and cracmm2 (CRACMM's IEPOX pair table,
 * the NO3 and HO2 uptake and the ISO3NOSJ / ISO3OSJ rates).  Synchronises the stream;
 * returns 0 or -1.  cmaqchem_hetchem_rates takes host arrays (device buffers for the call). */
#define CMAQCHEM_HET_CB6R5_NAE 84
#define CMAQCHEM_HET_CB6R5_AE_FIRST 131
#define CMAQCHEM_HET_CB6R5_NHETERO 17
#define CMAQCHEM_HET_CRACMM2_NAE 90
#define CMAQCHEM_HET_CRACMM2_AE_FIRST 184
#define CMAQCHEM_HET_CRACMM2_NHETERO 9
int cmaqchem_hetchem_layout(const char* mechanism, int* nae, int* ae_first, int* nhetero);
int cmaqchem_hetchem_rates_device(const char* mechanism, long long ncell, const float* ae, const float* ta,
                                  const float* pres, const float* qv, const float* dens, double* khetero,
                                  void* stream);
int cmaqchem_hetchem_rates(const char* mechanism, long long ncell, const float* ae, const float* ta,
                           const float* pres, const float* qv, const float* dens, double* khetero, int device);

/* Text of the last error of the calling thread; returns its length. */
int cmaqchem_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* CMAQCHEM_H */
