/* Discrete adjoint of the per-cell ROS3 integration -- CPU oracle restatement (test
 * infrastructure only; included at the end of ros3_oracle.c, whose tables and block
 * routines it uses).
 *
 * The reference has no adjoint: its gradient tool is the forward DDM-3D
 * (CCTM/src/ddm3d/DDM3D_CHEM.F).  This file restates, cell by cell and in the same
 * operation order, what the device kernels compute, so that their parity can be
 * checked to rounding level; the forward map it differentiates is the oracle's own
 * rbsolver loop (rbsolver.F:344-589) with a rate multiplier per reaction and an
 * emission tendency added to f.  With the accepted step sizes h fixed, one step is
 *
 *   A = J(Y) - I/(gamma h), K1 = A^-1(-f(Y)), YP = Y + K1, K2 = A^-1(-f(YP) - C21/h K1),
 *   K3 = A^-1(-f(YP) - C31/h K1 - C32/h K2), Y' = max(Y + B1 K1 + B2 K2 + B3 K3, CONMIN)
 *
 * and the reverse step follows by the chain rule (adj_step below).  oracle_adj_replay
 * re-runs that fixed-step map, whose finite differences check the adjoint itself.
 */

/* Storage slots of the L and U entries by row, from the solve's walk of CC2
 * (rbsolve.F), and their columns: built once per reaction list. */
typedef struct {
    int n_l, n_u;
    int* l_ptr;   /* [ISCHAN+1] transposed-L lists by column i: (slot, row k > i) */
    int* l_st;
    int* l_k;
    int* u_ptr;   /* [ISCHAN+1] transposed-U lists by column i: (slot, row k < i) */
    int* u_st;
    int* u_k;
} TransLists;

static TransLists g_trans[2];
static int g_trans_ready[2];

static void build_trans(int ncsp)
{
    TransLists* t = &g_trans[ncsp];
    const int n = MECH_ISCHAN;
    const int* kz = mech_kzero[ncsp];
    int nl = 0, nu = 0;
    for (int i = 0; i < n; ++i) { nl += mech_kzilch[ncsp][i]; nu += mech_mzilch[ncsp][i]; }
    int* lrow = malloc(sizeof(int) * (nl + 1));
    int* lcol = malloc(sizeof(int) * (nl + 1));
    int* lst = malloc(sizeof(int) * (nl + 1));
    int* urow = malloc(sizeof(int) * (nu + 1));
    int* ucol = malloc(sizeof(int) * (nu + 1));
    int* ust = malloc(sizeof(int) * (nu + 1));
    int ij = 1, a = 0, b = 0;
    for (int i = 0; i < n; ++i)
        for (int q = 0; q < mech_kzilch[ncsp][i]; ++q, ++ij) { lrow[a] = i; lcol[a] = kz[ij]; lst[a] = ij; ++a; }
    for (int i = n - 1; i >= 0; --i)
        for (int q = 0; q < mech_mzilch[ncsp][i]; ++q, ++ij) { urow[b] = i; ucol[b] = kz[ij]; ust[b] = ij; ++b; }
    t->n_l = nl; t->n_u = nu;
    t->l_ptr = calloc(n + 1, sizeof(int)); t->u_ptr = calloc(n + 1, sizeof(int));
    t->l_st = malloc(sizeof(int) * (nl + 1)); t->l_k = malloc(sizeof(int) * (nl + 1));
    t->u_st = malloc(sizeof(int) * (nu + 1)); t->u_k = malloc(sizeof(int) * (nu + 1));
    /* bucket by column, rows ascending within a column */
    for (int q = 0; q < nl; ++q) t->l_ptr[lcol[q] + 1]++;
    for (int q = 0; q < nu; ++q) t->u_ptr[ucol[q] + 1]++;
    for (int i = 0; i < n; ++i) { t->l_ptr[i + 1] += t->l_ptr[i]; t->u_ptr[i + 1] += t->u_ptr[i]; }
    int* fill = calloc(n, sizeof(int));
    for (int k = 0; k < n; ++k)             /* rows ascending */
        for (int q = 0; q < nl; ++q)
            if (lrow[q] == k) {
                const int c = lcol[q], pos = t->l_ptr[c] + fill[c]++;
                t->l_st[pos] = lst[q]; t->l_k[pos] = k;
            }
    memset(fill, 0, sizeof(int) * n);
    for (int k = 0; k < n; ++k)
        for (int q = 0; q < nu; ++q)
            if (urow[q] == k) {
                const int c = ucol[q], pos = t->u_ptr[c] + fill[c]++;
                t->u_st[pos] = ust[q]; t->u_k[pos] = k;
            }
    free(fill); free(lrow); free(lcol); free(lst); free(urow); free(ucol); free(ust);
}

static void ensure_trans(void)
{
#ifdef _OPENMP
#pragma omp critical(oracle_trans)
#endif
    {
        for (int d = 0; d < 2; ++d)
            if (!g_trans_ready[d]) { build_trans(d); g_trans_ready[d] = 1; }
    }
}

/* A^T x = b in place with the LU factors in b->cc2 / b->vdiag (ld = 1): U^T by ascending
 * rows, then L^T by descending rows, each row summing its column in ascending row order. */
static void solve_t(const Block* b, int ncsp, double* x)
{
    const TransLists* t = &g_trans[ncsp];
    for (int i = 0; i < MECH_ISCHAN; ++i) {
        double v = x[i];
        for (int q = t->u_ptr[i]; q < t->u_ptr[i + 1]; ++q) v = fma(-b->cc2[t->u_st[q]], x[t->u_k[q]], v);
        x[i] = v * b->vdiag[i];
    }
    for (int i = MECH_ISCHAN - 1; i >= 0; --i) {
        if (t->l_ptr[i] == t->l_ptr[i + 1]) continue;
        double v = x[i];
        for (int q = t->l_ptr[i]; q < t->l_ptr[i + 1]; ++q) v = fma(-b->cc2[t->l_st[q]], x[t->l_k[q]], v);
        x[i] = v;
    }
}

/* net stoichiometry of reaction r contracted with v: products (SC-weighted), then reactants */
static double stoich_sum(int r, const double* v)
{
    const int* irm = &mech_irm2[r * (3 + MECH_MXPRD)];
    double w = 0.0;
    int first = 1;
    for (int p = 0; p < mech_nprdct[r]; ++p) {
        const double sc = mech_sc[r * MECH_MXPRD + p];
        if (first) { w = sc * v[irm[3 + p]]; first = 0; }
        else w = fma(sc, v[irm[3 + p]], w);
    }
    for (int i = 0; i < mech_nreact[r]; ++i) {
        if (first) { w = -v[irm[i]]; first = 0; }
        else w = w - v[irm[i]];
    }
    return w;
}

/* out += J(y)^T phi; gk[r] += w_r(phi) R_r(y) */
static void adj_jtv(int ncsp, const double* rki, const double* y, const double* phi, double* out, double* gk)
{
    const int nu = mech_nuserat[ncsp];
    for (int q = 0; q < nu; ++q) {
        const int r = mech_nkuserat[ncsp * MECH_NRXNS + q];
        const int nre = mech_nreact[r];
        if (nre == 0 && mech_nprdct[r] == 0) continue;
        const int* a = &mech_irm2[r * (3 + MECH_MXPRD)];
        const double w = stoich_sum(r, phi);
        const double kw = rki[r] * w;
        if (nre == 0) {
            gk[r] = gk[r] + kw;
        } else if (nre == 1) {
            out[a[0]] = out[a[0]] + kw;
            gk[r] = fma(kw, y[a[0]], gk[r]);
        } else if (nre == 2) {
            out[a[0]] = fma(kw, y[a[1]], out[a[0]]);
            out[a[1]] = fma(kw, y[a[0]], out[a[1]]);
            gk[r] = fma(kw * y[a[0]], y[a[1]], gk[r]);
        } else {
            out[a[0]] = fma(kw * y[a[1]], y[a[2]], out[a[0]]);
            out[a[1]] = fma(kw * y[a[0]], y[a[2]], out[a[1]]);
            out[a[2]] = fma(kw * y[a[0]], y[a[1]], out[a[2]]);
            gk[r] = fma((kw * y[a[0]]) * y[a[1]], y[a[2]], gk[r]);
        }
    }
}

/* lam -= sum_i d/dy (nu_i . J(y) K_i); gk[r] -= sum_i d/dlog k_r (nu_i . J(y) K_i) */
static void adj_hess3(int ncsp, const double* rki, const double* y, const double* const nu[3],
                      const double* const kv[3], double* lam, double* gk)
{
    const int nrx = mech_nuserat[ncsp];
    for (int q = 0; q < nrx; ++q) {
        const int r = mech_nkuserat[ncsp * MECH_NRXNS + q];
        const int nre = mech_nreact[r];
        if (nre == 0) continue;
        const int* a = &mech_irm2[r * (3 + MECH_MXPRD)];
        const double w1 = stoich_sum(r, nu[0]), w2 = stoich_sum(r, nu[1]), w3 = stoich_sum(r, nu[2]);
        double wk[3];
        for (int j = 0; j < nre; ++j) {
            wk[j] = w1 * kv[0][a[j]];
            wk[j] = fma(w2, kv[1][a[j]], wk[j]);
            wk[j] = fma(w3, kv[2][a[j]], wk[j]);
        }
        const double kk = rki[r];
        if (nre == 1) {
            gk[r] = fma(-kk, wk[0], gk[r]);
        } else if (nre == 2) {
            gk[r] = fma(-kk, fma(y[a[1]], wk[0], y[a[0]] * wk[1]), gk[r]);
            lam[a[0]] = fma(-kk, wk[1], lam[a[0]]);
            lam[a[1]] = fma(-kk, wk[0], lam[a[1]]);
        } else {
            gk[r] = fma(-kk, fma(y[a[1]] * y[a[2]], wk[0], fma(y[a[0]] * y[a[2]], wk[1], (y[a[0]] * y[a[1]]) * wk[2])),
                        gk[r]);
            lam[a[0]] = fma(-kk, fma(y[a[2]], wk[1], y[a[1]] * wk[2]), lam[a[0]]);
            lam[a[1]] = fma(-kk, fma(y[a[2]], wk[0], y[a[0]] * wk[2]), lam[a[1]]);
            lam[a[2]] = fma(-kk, fma(y[a[1]], wk[0], y[a[0]] * wk[1]), lam[a[2]]);
        }
    }
}

/* One ROS3 step of the fixed-step map at b->y (ld = 1 block): K1..K3 and the LU of A
 * stay in the block; returns Y' (unclipped) in b->yp. */
static void fixed_step(Block* b, int ncsp, double h)
{
    const double dtinv = 1.0 / h, gdtinv = dtinv * RGAM;
    oracle_rbfeval(b, ncsp, b->y, b->ydot);
    oracle_rbjacob(b, ncsp, b->y);
    for (int j = 0; j < MECH_ISCHAN; ++j) b->cc2[mech_diag[ncsp][j]] = b->cc2[mech_diag[ncsp][j]] - gdtinv;
    oracle_rbdecomp(b, ncsp);
    for (int q = 0; q < MECH_ISCHAN; ++q) b->k1[q] = -b->ydot[q];
    oracle_rbsolve(b, ncsp, b->k1);
    for (int q = 0; q < MECH_ISCHAN; ++q) b->yp[q] = b->y[q] + b->k1[q];
    oracle_rbfeval(b, ncsp, b->yp, b->ydot);
    const double x21 = C21 * dtinv, x31 = C31 * dtinv, x32 = C32 * dtinv;
    for (int q = 0; q < MECH_ISCHAN; ++q) b->k2[q] = fma(-x21, b->k1[q], -b->ydot[q]);
    oracle_rbsolve(b, ncsp, b->k2);
    for (int q = 0; q < MECH_ISCHAN; ++q) b->k3[q] = fma(-x32, b->k2[q], fma(-x31, b->k1[q], -b->ydot[q]));
    oracle_rbsolve(b, ncsp, b->k3);
}

typedef struct {
    double lam[MECH_NSPEC], mu1[MECH_NSPEC], mu2[MECH_NSPEC], mu3[MECH_NSPEC];
    double phi[MECH_NSPEC], tmp[MECH_NSPEC], ypv[MECH_NSPEC], ge[MECH_NSPEC];
    double gk[MECH_NRXNS];
} AdjCell;

/* Adjoint of the accepted step that started at y with size h. */
static void adj_step(Block* b, int ncsp, const double* y, double h, AdjCell* a)
{
    memcpy(b->y, y, sizeof(double) * MECH_NSPEC);
    fixed_step(b, ncsp, h);
    const double dtinv = 1.0 / h;
    const double x21 = C21 * dtinv, x31 = C31 * dtinv, x32 = C32 * dtinv;
    const int n = MECH_ISCHAN;
    for (int q = 0; q < n; ++q) a->ypv[q] = b->yp[q];   /* YP = Y + K1 */
    for (int q = 0; q < n; ++q) {
        double yn = fma(B1, b->k1[q], b->y[q]);
        yn = fma(B2, b->k2[q], yn);
        yn = fma(B3, b->k3[q], yn);
        if (!(yn > CONMIN)) a->lam[q] = 0.0;
        a->mu3[q] = B3 * a->lam[q];
    }
    solve_t(b, ncsp, a->mu3);
    for (int q = 0; q < n; ++q) a->mu2[q] = fma(-x32, a->mu3[q], B2 * a->lam[q]);
    solve_t(b, ncsp, a->mu2);
    for (int q = 0; q < n; ++q) {
        const double phi = -a->mu3[q] - a->mu2[q];
        a->phi[q] = phi;
        a->ge[q] = a->ge[q] + phi;
        a->tmp[q] = 0.0;
    }
    adj_jtv(ncsp, b->rki, a->ypv, a->phi, a->tmp, a->gk);
    for (int q = 0; q < n; ++q) {
        const double lam = a->lam[q], t = a->tmp[q];
        const double mu = fma(-x21, a->mu2[q], fma(-x31, a->mu3[q], B1 * lam));
        a->mu1[q] = mu + t;
        a->lam[q] = lam + t;
    }
    solve_t(b, ncsp, a->mu1);
    for (int q = 0; q < n; ++q) {
        const double phi = -a->mu1[q];
        a->phi[q] = phi;
        a->ge[q] = a->ge[q] + phi;
    }
    adj_jtv(ncsp, b->rki, b->y, a->phi, a->lam, a->gk);
    const double* nu[3] = {a->mu1, a->mu2, a->mu3};
    const double* kv[3] = {b->k1, b->k2, b->k3};
    adj_hess3(ncsp, b->rki, b->y, nu, kv, a->lam, a->gk);
}

static void load_cell(Block* b, long n, long c, const double* rki, const double* kmult, const double* emis,
                      double* ebuf)
{
    for (int r = 0; r < MECH_NRXNS; ++r) {
        const double k = rki[(size_t)r * n + c];
        b->rki[r] = kmult ? k * kmult[r] : k;
    }
    for (int i = 0; i < MECH_ISCHAN; ++i) ebuf[i] = emis ? emis[(size_t)i * n + c] : 0.0;
    b->emis = ebuf;
}

/* Forward window: nsync steps of chemstep minutes; checkpoints ck[k][nspec][n], accepted
 * steps nsteps[k][n]; with hs != NULL (capacity hcap per cell and step) also the step
 * sizes hs[(k*n + c)*hcap + j].  Returns failed cell-steps. */
int oracle_adj_forward(long n, double* y, const double* rki, long rki_stride, const uint8_t* night,
                       const double* kmult, const double* emis, int nsync, double chemstep, double rtol,
                       double atol, double* ck, int* nsteps, double* hs, int hcap, int threads)
{
    int nbad = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : nbad)
#endif
    {
        Block b;
        block_alloc(&b, 1);
        b.ncells = 1;
        double* tape_y = malloc(sizeof(double) * MECH_NSPEC * (hcap > 0 ? hcap : 1));
        double ebuf[MECH_NSPEC];
        SolverCfg cfg = {rtol, atol, (double)(1.0f / (float)MECH_NSPEC), 100000};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (long c = 0; c < n; ++c) {
            for (int s = 0; s < MECH_NSPEC; ++s) b.y[s] = y[(size_t)s * n + c];
            for (int k = 0; k < nsync; ++k) {
                for (int s = 0; s < MECH_NSPEC; ++s) ck[((size_t)k * MECH_NSPEC + s) * n + c] = b.y[s];
                load_cell(&b, n, c, rki + (size_t)k * rki_stride, kmult, emis, ebuf);
                if (hs) {
                    b.tape_y = tape_y;
                    b.tape_h = hs + ((size_t)k * n + c) * hcap;
                    b.tape_cap = hcap;
                    b.tape_n = 0;
                }
                SolverStats st = oracle_rbsolver(&b, night[c] ? 1 : 0, chemstep, &cfg, NULL);
                nsteps[(size_t)k * n + c] = st.nsteps;
                nbad += st.status != 0 || (hs && b.tape_n > hcap);
            }
            for (int s = 0; s < MECH_NSPEC; ++s) y[(size_t)s * n + c] = b.y[s];
        }
        free(tape_y);
        block_free(&b);
    }
    return nbad;
}

/* Backward window: lam[nspec][n] in (dL/dy at the end) / out (at the start); gk[nrxns]
 * and ge[nspec][n] (may be NULL) accumulated.  Re-runs every step from its checkpoint
 * with a tape, then walks the tape backwards. */
int oracle_adj_backward(long n, double* lam, const double* rki, long rki_stride, const uint8_t* night,
                        const double* kmult, const double* emis, int nsync, double chemstep, double rtol,
                        double atol, const double* ck, const int* nsteps, double* gk, double* ge, int threads)
{
    ensure_trans();
    double* gk_cell = calloc((size_t)n * MECH_NRXNS, sizeof(double));
    int nbad = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : nbad)
#endif
    {
        Block b;
        block_alloc(&b, 1);
        b.ncells = 1;
        double ebuf[MECH_NSPEC];
        AdjCell* a = calloc(1, sizeof(AdjCell));
        SolverCfg cfg = {rtol, atol, (double)(1.0f / (float)MECH_NSPEC), 100000};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (long c = 0; c < n; ++c) {
            memset(a, 0, sizeof(*a));
            for (int s = 0; s < MECH_NSPEC; ++s) a->lam[s] = lam[(size_t)s * n + c];
            for (int k = nsync - 1; k >= 0; --k) {
                const int ns = nsteps[(size_t)k * n + c];
                const int ncsp = night[c] ? 1 : 0;
                load_cell(&b, n, c, rki + (size_t)k * rki_stride, kmult, emis, ebuf);
                double* ty = malloc(sizeof(double) * MECH_NSPEC * (ns > 0 ? ns : 1));
                double* th = malloc(sizeof(double) * (ns > 0 ? ns : 1));
                for (int s = 0; s < MECH_NSPEC; ++s) b.y[s] = ck[((size_t)k * MECH_NSPEC + s) * n + c];
                b.tape_y = ty; b.tape_h = th; b.tape_cap = ns; b.tape_n = 0;
                oracle_rbsolver(&b, ncsp, chemstep, &cfg, NULL);
                nbad += b.tape_n != ns;
                b.tape_y = NULL; b.tape_h = NULL;
                for (int j = (b.tape_n < ns ? b.tape_n : ns) - 1; j >= 0; --j)
                    adj_step(&b, ncsp, ty + (size_t)j * MECH_NSPEC, th[j], a);
                free(ty); free(th);
            }
            for (int s = 0; s < MECH_NSPEC; ++s) lam[(size_t)s * n + c] = a->lam[s];
            if (ge)
                for (int s = 0; s < MECH_NSPEC; ++s) ge[(size_t)s * n + c] += a->ge[s];
            memcpy(gk_cell + (size_t)c * MECH_NRXNS, a->gk, sizeof(double) * MECH_NRXNS);
        }
        free(a);
        block_free(&b);
    }
    for (long c = 0; c < n; ++c)
        for (int r = 0; r < MECH_NRXNS; ++r) gk[r] += gk_cell[(size_t)c * MECH_NRXNS + r];
    free(gk_cell);
    return nbad;
}

/* The fixed-step map: the same windows with the step sizes hs / counts nsteps of a
 * forward run, no error control.  y[nspec][n] advanced in place. */
void oracle_adj_replay(long n, double* y, const double* rki, long rki_stride, const uint8_t* night,
                       const double* kmult, const double* emis, int nsync, const int* nsteps, const double* hs,
                       int hcap, int threads)
{
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
#endif
    {
        Block b;
        block_alloc(&b, 1);
        b.ncells = 1;
        double ebuf[MECH_NSPEC];
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (long c = 0; c < n; ++c) {
            for (int s = 0; s < MECH_NSPEC; ++s) b.y[s] = y[(size_t)s * n + c];
            for (int k = 0; k < nsync; ++k) {
                load_cell(&b, n, c, rki + (size_t)k * rki_stride, kmult, emis, ebuf);
                const int ncsp = night[c] ? 1 : 0;
                const double* h = hs + ((size_t)k * n + c) * hcap;
                for (int j = 0; j < nsteps[(size_t)k * n + c] && j < hcap; ++j) {
                    fixed_step(&b, ncsp, h[j]);
                    for (int q = 0; q < MECH_ISCHAN; ++q) {
                        double yn = fma(B1, b.k1[q], b.y[q]);
                        yn = fma(B2, b.k2[q], yn);
                        yn = fma(B3, b.k3[q], yn);
                        b.y[q] = fmax(yn, CONMIN);
                    }
                }
            }
            for (int s = 0; s < MECH_NSPEC; ++s) y[(size_t)s * n + c] = b.y[s];
        }
        block_free(&b);
    }
}

/* ------------------------------------------------------------------ DDM-3D (reference gradient)
 *
 * First-order DDM-3D sensitivities of the chemistry as CMAQ computes them
 * (CCTM/src/ddm3d/DDM3D_CHEM.F:155-410, SOLVE_DDM3D_CHEM; driver hook rbdriver.F:619-651):
 * after each synchronisation step of length DT the sensitivity vector S of a parameter
 * is advanced by the Crank-Nicolson-type update
 *
 *     (I - DT/2 J(YAVE)) S_new = (I + DT/2 J(YAVE)) S_old + DT dF/dp(YAVE)
 *
 * with YAVE the step's time-averaged concentrations (rbsolver.F:468-475, 592-595) and J
 * the Jacobian of the mechanism (MECHANISM_FUNCTIONS.F:755, EVALUATE_F_JAC_MECH).  For a
 * reaction-rate parameter (IPT = 5) dF/dp is the rate of the reaction times its net
 * stoichiometry (DDM3D_CHEM.F:338-385); for an initial-condition parameter it is zero
 * and S starts at the unit vector.  The reference stores J in REAL(4) and factors with
 * LINPACK SGEFA/SGESL; here everything is REAL(8) with partial pivoting. */

static void dense_jac(const double* rki, const double* y, int ncsp, double* jac /* [n][n] row-major */)
{
    const int n = MECH_ISCHAN;
    memset(jac, 0, sizeof(double) * n * n);
    const int nu = mech_nuserat[ncsp];
    for (int q = 0; q < nu; ++q) {
        const int r = mech_nkuserat[ncsp * MECH_NRXNS + q];
        const int nre = mech_nreact[r];
        const int* a = &mech_irm2[r * (3 + MECH_MXPRD)];
        double ex[3] = {0, 0, 0};
        if (nre == 1) ex[0] = rki[r];
        else if (nre == 2) { ex[0] = rki[r] * y[a[1]]; ex[1] = rki[r] * y[a[0]]; }
        else if (nre == 3) {
            ex[0] = rki[r] * y[a[1]] * y[a[2]]; ex[1] = rki[r] * y[a[0]] * y[a[2]]; ex[2] = rki[r] * y[a[1]] * y[a[0]];
        }
        for (int j = 0; j < nre; ++j) {
            for (int i = 0; i < nre; ++i) jac[a[i] * n + a[j]] -= ex[j];
            for (int p = 0; p < mech_nprdct[r]; ++p) jac[a[3 + p] * n + a[j]] += mech_sc[r * MECH_MXPRD + p] * ex[j];
        }
    }
}

static void lu_factor(double* m, int* piv, int n)
{
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i) if (fabs(m[i * n + k]) > fabs(m[p * n + k])) p = i;
        piv[k] = p;
        if (p != k) for (int j = 0; j < n; ++j) { double t = m[k * n + j]; m[k * n + j] = m[p * n + j]; m[p * n + j] = t; }
        const double d = m[k * n + k];
        for (int i = k + 1; i < n; ++i) {
            const double l = m[i * n + k] / d;
            m[i * n + k] = l;
            if (l != 0.0) for (int j = k + 1; j < n; ++j) m[i * n + j] -= l * m[k * n + j];
        }
    }
}

static void lu_solve(const double* m, const int* piv, int n, double* b)
{
    for (int k = 0; k < n; ++k) { const int p = piv[k]; if (p != k) { double t = b[k]; b[k] = b[p]; b[p] = t; } }
    for (int i = 0; i < n; ++i) for (int j = 0; j < i; ++j) b[i] -= m[i * n + j] * b[j];
    for (int i = n - 1; i >= 0; --i) {
        for (int j = i + 1; j < n; ++j) b[i] -= m[i * n + j] * b[j];
        b[i] /= m[i * n + i];
    }
}

/* DDM-3D over a window.  Parameters: kind[p] = 0 initial condition of species idx[p]
 * (solver order), 1 log rate multiplier of reaction idx[p], 2 emission tendency of
 * species idx[p] (dF/dp = unit vector, the source DDM-3D adds for an emission
 * parameter; here the emission enters f, so DT times it is the step's source).  emis
 * [nspec][n] (or NULL) is the emission tendency of the forward.  Returns
 * s_end[p][nspec][n] and the end state in y (the forward is the oracle's rbsolver). */
int oracle_ebi_cell(double* yc, const double* rki, int tstep_sec, double* ycddm);   /* ebi_oracle.c */

int oracle_ddm3d_window(long n, double* y, const double* rki, long rki_stride, const uint8_t* night,
                        const double* kmult, const double* emis, int nsync, double chemstep, double rtol,
                        double atol, int nparam, const int* kind, const int* idx, double* s_end, int threads,
                        const void* gear_cfg, int ebi)
{
    /* gear_cfg != NULL: each step is SMVGEAR's (GearCfg of oracle_gear_cfg) and the averaged
     * concentrations are its CAVEG (grdriver.F hands CAVEG to SOLVE_DDM3D_CHEM); ebi != 0:
     * each step is HRSOLVER's and the averages its YCDDM (hrdriver.F:477-490) */
    const GearCfg* gcfg = (const GearCfg*)gear_cfg;
    int nbad = 0;
    const int ns = MECH_ISCHAN;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel reduction(+ : nbad)
#endif
    {
        Block b;
        block_alloc(&b, 1);
        b.ncells = 1;
        double* jac = malloc(sizeof(double) * ns * ns);
        double* am = malloc(sizeof(double) * ns * ns);
        int* piv = malloc(sizeof(int) * ns);
        double* sv = malloc(sizeof(double) * ns * (nparam > 0 ? nparam : 1));
        double yave[MECH_NSPEC], tmp[MECH_NSPEC], src[MECH_NSPEC], ebuf[MECH_NSPEC];
        SolverCfg cfg = {rtol, atol, (double)(1.0f / (float)MECH_NSPEC), 100000};
        GearBlock gb;
        if (gcfg) {
            gear_alloc(&gb, 1);
            gb.b.ncells = 1;
            gb.caveg = yave;
        }
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (long c = 0; c < n; ++c) {
            for (int s = 0; s < MECH_NSPEC; ++s) b.y[s] = y[(size_t)s * n + c];
            for (int p = 0; p < nparam; ++p)
                for (int s = 0; s < ns; ++s) sv[p * ns + s] = (kind[p] == 0 && idx[p] == s) ? 1.0 : 0.0;
            const int ncsp = night[c] ? 1 : 0;
            for (int k = 0; k < nsync; ++k) {
                load_cell(&b, n, c, rki + (size_t)k * rki_stride, kmult, emis, ebuf);
                memset(yave, 0, sizeof(yave));
                if (ebi) {
                    double ycm[MECH_NSPEC], ydd[MECH_NSPEC];
                    for (int s = 0; s < MECH_NSPEC; ++s) ycm[s] = b.y[mech_iold2new[s]];
                    nbad += oracle_ebi_cell(ycm, b.rki, (int)lround(chemstep * 60.0), ydd) != 0;
                    for (int s = 0; s < MECH_NSPEC; ++s) {
                        b.y[mech_iold2new[s]] = ycm[s];
                        yave[mech_iold2new[s]] = ydd[s];
                    }
                } else if (gcfg) {
                    memcpy(gb.b.y, b.y, sizeof(double) * MECH_NSPEC);
                    memcpy(gb.blkconc, b.y, sizeof(double) * MECH_NSPEC);
                    memcpy(gb.b.rki, b.rki, sizeof(double) * MECH_NRXNS);
                    GearStats gst = oracle_smvgear(&gb, ncsp, !night[c], chemstep, gcfg, NULL);
                    memcpy(b.y, gb.b.y, sizeof(double) * MECH_NSPEC);
                    nbad += gst.status != 0;
                } else {
                    b.yave = yave;
                    SolverStats st = oracle_rbsolver(&b, ncsp, chemstep, &cfg, NULL);
                    b.yave = NULL;
                    nbad += st.status != 0;
                    for (int s = 0; s < ns; ++s) yave[s] /= chemstep;
                }
                dense_jac(b.rki, yave, ncsp, jac);
                for (int i = 0; i < ns * ns; ++i) am[i] = -0.5 * chemstep * jac[i];
                for (int i = 0; i < ns; ++i) am[i * ns + i] += 1.0;
                lu_factor(am, piv, ns);
                for (int p = 0; p < nparam; ++p) {
                    double* sp = sv + p * ns;
                    memset(src, 0, sizeof(src));
                    if (kind[p] == 1) {   /* DT * stoichiometry * rate at YAVE */
                        const int r = idx[p];
                        const int* a = &mech_irm2[r * (3 + MECH_MXPRD)];
                        double rate = b.rki[r];
                        for (int i = 0; i < mech_nreact[r]; ++i) rate *= yave[a[i]];
                        for (int i = 0; i < mech_nreact[r]; ++i) src[a[i]] -= chemstep * rate;
                        for (int q = 0; q < mech_nprdct[r]; ++q) src[a[3 + q]] += chemstep * rate * mech_sc[r * MECH_MXPRD + q];
                    } else if (kind[p] == 2) {
                        src[idx[p]] = chemstep;
                    }
                    for (int i = 0; i < ns; ++i) {
                        double t = sp[i];
                        for (int j = 0; j < ns; ++j) t += 0.5 * chemstep * jac[i * ns + j] * sp[j];
                        tmp[i] = t + src[i];
                    }
                    lu_solve(am, piv, ns, tmp);
                    memcpy(sp, tmp, sizeof(double) * ns);
                }
            }
            for (int s = 0; s < MECH_NSPEC; ++s) y[(size_t)s * n + c] = b.y[s];
            for (int p = 0; p < nparam; ++p)
                for (int s = 0; s < ns; ++s) s_end[((size_t)p * ns + s) * n + c] = sv[p * ns + s];
        }
        free(jac); free(am); free(piv); free(sv);
        block_free(&b);
        if (gcfg) gear_free(&gb);
    }
    return nbad;
}
