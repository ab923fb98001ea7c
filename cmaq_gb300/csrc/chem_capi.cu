// C ABI of the chemistry library (include/cmaqchem.h).
//
// A handle holds what CMAQ's chemistry keeps in module SAVE state after its first call
// (rbdriver.F:226-371): mechanism tables (here: device tables and the generated code),
// the domain size and the solver's work arrays (here: per-warp device workspaces).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/cmaqchem.h"
#include "../../include/cmaqchem_diag.h"
#include "mech_ops.cuh"

extern const MechOps mech_ops_cb6r5_ae7_aq;
extern const MechOps mech_ops_cracmm2;

namespace {

thread_local std::string g_err;

int fail(const std::string& msg)
{
    g_err = msg;
    return -1;
}

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) return fail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
    } while (0)

const MechOps* find_mech(const char* name)
{
    if (!name) return nullptr;
    const MechOps* all[] = {&mech_ops_cb6r5_ae7_aq, &mech_ops_cracmm2};
    for (const MechOps* m : all)
        if (strcmp(m->name, name) == 0) return m;
    return nullptr;
}

// HHMMSS -> seconds (TIME2SEC of the I/O API)
int hhmmss_to_sec(int t)
{
    const int sign = t < 0 ? -1 : 1;
    t = t < 0 ? -t : t;
    return sign * ((t / 10000) * 3600 + ((t / 100) % 100) * 60 + t % 100);
}

}  // namespace

// error-text setter for the library's other translation units, not exported
__attribute__((visibility("hidden"))) void cmaqchem_set_error(const std::string& msg) { g_err = msg; }

struct cmaqchem_handle {
    const MechOps* ops = nullptr;
    cmaqchem_cfg cfg{};
    std::vector<int> cgrid_index;   // 0-based
    int device = 0, nsm = 0, bps = 1, nblocks = 0;
    long long ncell = 0;
    int ncolrow = 0;
    double rnspec = 0.0;
    int max_iter = 100000;
    int* d_cgrid_index = nullptr;
    int* d_convert = nullptr;
    float* d_fwd = nullptr;
    double* d_rev = nullptr;
    double* d_ws = nullptr;
    int* d_status = nullptr;
    int* d_steps = nullptr;
    unsigned long long* d_counters = nullptr;
    int* d_order = nullptr;
    unsigned int* d_hist = nullptr;
    unsigned long long* d_cursor = nullptr;
    unsigned long long* d_head = nullptr;
    bool have_history = false;
    // tuning knobs (cmaqchem_diag_set_tuning)
    int use_night = 1;
    int lockstep = 0;
    // device staging of the host-pointer entry point, allocated on first use
    float *s_conc = nullptr, *s_ta = nullptr, *s_qv = nullptr, *s_dens = nullptr, *s_pres = nullptr;
    float *s_seaice = nullptr, *s_osz = nullptr, *s_rj = nullptr;
    double* s_khet = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

void free_handle(cmaqchem_handle* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    void* ptrs[] = {h->d_cgrid_index, h->d_convert, h->d_fwd, h->d_rev, h->d_ws, h->d_status, h->d_steps,
                    h->d_counters, h->d_order, h->d_hist, h->d_cursor, h->d_head, h->s_conc, h->s_ta,
                    h->s_qv, h->s_dens, h->s_pres, h->s_seaice, h->s_osz, h->s_rj, h->s_khet};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

chem::GridArgs grid_args(cmaqchem_handle* h, float* conc, const float* ta, const float* qv, const float* dens,
                         const float* pres, const float* seaice, const float* osz, const float* rj,
                         const double* khet, double chemstep)
{
    chem::GridArgs a{};
    a.cgrid = conc;
    a.ncell = h->ncell;
    a.ncolrow = h->ncolrow;
    a.nspcsd = h->cfg.nspcsd;
    a.cgrid_index = h->d_cgrid_index;
    a.convert = h->d_convert;
    a.fwd_conv = h->d_fwd;
    a.rev_conv = h->d_rev;
    a.ta = ta;
    a.qv = qv;
    a.dens = dens;
    a.pres = pres;
    a.seaice = seaice;
    a.ocean_szone = osz;
    a.rj = rj;
    a.khet = khet;
    a.chemstep = chemstep;
    a.tol = ros3::Tol{h->cfg.rtol, h->cfg.atol, h->rnspec};
    a.ws = h->d_ws;
    a.max_iter = h->max_iter;
    a.cell_status = h->d_status;
    a.cell_steps = h->d_steps;
    a.counters = h->d_counters;
    a.use_night = h->use_night;
    return a;
}

int check_ptrs(const void* const* p, int n)
{
    for (int i = 0; i < n; ++i)
        if (!p[i]) return fail("null array argument");
    return 0;
}

}  // namespace

extern "C" int cmaqchem_last_error(char* buf, size_t len)
{
    if (buf && len) {
        strncpy(buf, g_err.c_str(), len - 1);
        buf[len - 1] = '\0';
    }
    return (int)g_err.size();
}

extern "C" int cmaqchem_mech_info_get(const char* mechanism, cmaqchem_mech_info* info, int* inew2old)
{
    const MechOps* m = find_mech(mechanism);
    if (!m) return fail(std::string("unknown mechanism ") + (mechanism ? mechanism : "(null)"));
    if (info) {
        info->nspec = m->nspec;
        info->nrxns = m->nrxns;
        info->ischan = m->ischan;
        info->nphotab = m->nphotab;
        info->nhetero = m->nhetero;
        info->iarray_day = m->iarray_day;
        info->iarray_night = m->iarray_night;
        info->flops_step_day = m->flops_step_day;
        info->flops_step_night = m->flops_step_night;
    }
    if (inew2old) memcpy(inew2old, m->inew2old, sizeof(int) * m->nspec);
    return 0;
}

extern "C" int cmaqchem_init(const cmaqchem_cfg* cfg, cmaqchem_handle** out)
{
    if (!cfg || !out) return fail("cmaqchem_init: null argument");
    *out = nullptr;
    const MechOps* m = find_mech(cfg->mechanism);
    if (!m) return fail(std::string("unknown mechanism ") + (cfg->mechanism ? cfg->mechanism : "(null)"));
    if (cfg->solver != CMAQCHEM_SOLVER_ROS3) return fail("only the ROS3 solver is available in this build");
    if (cfg->schedule != CMAQCHEM_SCHED_STATIC && cfg->schedule != CMAQCHEM_SCHED_QUEUE)
        return fail("unknown schedule");
    if (cfg->ncols <= 0 || cfg->nrows <= 0 || cfg->nlays <= 0) return fail("domain dimensions must be positive");
    if (!(cfg->rtol > 0.0) || !(cfg->atol > 0.0)) return fail("rtol and atol must be positive");
    auto* h = new cmaqchem_handle();
    h->ops = m;
    h->cfg = *cfg;
    h->cfg.cgrid_index = nullptr;
    h->device = cfg->device;
    h->ncolrow = cfg->ncols * cfg->nrows;
    h->ncell = (long long)h->ncolrow * cfg->nlays;
    h->max_iter = cfg->max_iter > 0 ? cfg->max_iter : 100000;
    h->rnspec = (double)(1.0f / (float)m->nspec);   // RNSPEC = 1.0 / FLOAT(N_SPEC), REAL(4)
    h->cgrid_index.resize(m->nspec);
    for (int s = 0; s < m->nspec; ++s) {
        const int ci = cfg->cgrid_index ? cfg->cgrid_index[s] - 1 : m->cgrid_index[s];
        if (ci < 0 || ci >= cfg->nspcsd) {
            delete h;
            return fail("cgrid_index out of range [1, nspcsd] for species " + std::to_string(s + 1));
        }
        h->cgrid_index[s] = ci;
    }
    std::vector<float> fwd(m->nspec);
    std::vector<double> rev(m->nspec);
    for (int s = 0; s < m->nspec; ++s) {   // rbinit.F:252-253, REAL(4)
        fwd[s] = 1.0e-3f * 28.9628f / (float)m->molwt[s];
        rev[s] = (double)(1.0f / fwd[s]);
    }
    int rc = 0;
    auto setup = [&]() -> int {
        CK(cudaSetDevice(h->device));
        CK(cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device));
        CK(m->occupancy(&h->bps));
        if (h->bps < 1) h->bps = 1;
        h->nblocks = h->nsm * h->bps;
        const size_t nwarps = (size_t)h->nblocks * chem::WARPS_PER_BLOCK;
        CK(cudaMalloc(&h->d_ws, nwarps * (size_t)m->ws_elems * 32 * sizeof(double)));
        CK(cudaMalloc(&h->d_cgrid_index, sizeof(int) * m->nspec));
        CK(cudaMalloc(&h->d_convert, sizeof(int) * m->nspec));
        CK(cudaMalloc(&h->d_fwd, sizeof(float) * m->nspec));
        CK(cudaMalloc(&h->d_rev, sizeof(double) * m->nspec));
        CK(cudaMemcpy(h->d_cgrid_index, h->cgrid_index.data(), sizeof(int) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_convert, m->convert, sizeof(int) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_fwd, fwd.data(), sizeof(float) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_rev, rev.data(), sizeof(double) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMalloc(&h->d_status, sizeof(int) * h->ncell));
        CK(cudaMalloc(&h->d_steps, sizeof(int) * h->ncell));
        CK(cudaMemset(h->d_status, 0, sizeof(int) * h->ncell));
        CK(cudaMemset(h->d_steps, 0, sizeof(int) * h->ncell));
        CK(cudaMalloc(&h->d_counters, sizeof(unsigned long long) * 5));
        CK(cudaMalloc(&h->d_order, sizeof(int) * h->ncell));
        CK(cudaMalloc(&h->d_hist, sizeof(unsigned int) * chem::QUEUE_BINS));
        CK(cudaMalloc(&h->d_cursor, sizeof(unsigned long long) * chem::QUEUE_BINS));
        CK(cudaMalloc(&h->d_head, sizeof(unsigned long long)));
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&h->ev0));
        CK(cudaEventCreate(&h->ev1));
        return 0;
    };
    rc = setup();
    if (rc != 0) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return 0;
}

extern "C" void cmaqchem_destroy(cmaqchem_handle* h) { free_handle(h); }

extern "C" int cmaqchem_diag_set_tuning(cmaqchem_handle* h, const char* key, int value)
{
    if (!h || !key) return fail("null argument");
    if (strcmp(key, "night_pattern") == 0) h->use_night = value != 0;
    else if (strcmp(key, "lockstep") == 0) h->lockstep = value != 0;
    else return fail(std::string("unknown tuning key ") + key);
    return 0;
}

static int step_device_impl(cmaqchem_handle* h, float* conc, const float* ta, const float* qv, const float* dens,
                            const float* pres, const float* seaice, const float* osz, const float* rj,
                            const double* khet, const int tstep[3], cudaStream_t s, cmaqchem_stats* stats)
{
    const void* ptrs[] = {conc, ta, qv, dens, pres, seaice, osz, rj, tstep, khet};
    if (check_ptrs(ptrs, h->ops->nhetero > 0 ? 10 : 9)) return -1;
    const int itmstep = hhmmss_to_sec(tstep[1]);
    if (itmstep <= 0) return fail("TSTEP(2) must be a positive HHMMSS interval");
    const double chemstep = (double)itmstep / 60.0;   // rbdriver.F:384-385
    CK(cudaSetDevice(h->device));
    chem::GridArgs a = grid_args(h, conc, ta, qv, dens, pres, seaice, osz, rj, khet, chemstep);
    CK(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 5, s));
    CK(cudaEventRecord(h->ev0, s));
    if (h->cfg.schedule == CMAQCHEM_SCHED_QUEUE) {
        chem::QueueArgs q{nullptr, h->d_head};
        if (h->have_history) {
            const int nb = 4 * h->nsm;
            CK(cudaMemsetAsync(h->d_hist, 0, sizeof(unsigned int) * chem::QUEUE_BINS, s));
            chem::k_queue_hist<<<nb, 256, 0, s>>>(h->d_steps, h->ncell, h->d_hist);
            CK(cudaGetLastError());
            chem::k_queue_scan<<<1, chem::QUEUE_BINS, 0, s>>>(h->d_hist, h->d_cursor);
            CK(cudaGetLastError());
            chem::k_queue_scatter<<<nb, 256, 0, s>>>(h->d_steps, h->ncell, h->d_cursor, h->d_order);
            CK(cudaGetLastError());
            q.order = h->d_order;
        }
        CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
        CK(h->ops->chem_queue(a, q, h->lockstep != 0, h->nblocks, s));
    } else {
        CK(h->ops->chem_static(a, h->nblocks, s));
    }
    CK(cudaEventRecord(h->ev1, s));
    unsigned long long cnt[5];
    CK(cudaMemcpyAsync(cnt, h->d_counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    h->have_history = true;
    float ms = 0.0f;
    CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    if (stats) {
        stats->accepted_steps = (long long)cnt[0];
        stats->rejected_steps = (long long)cnt[1];
        stats->failed_cells = (long long)cnt[2];
        stats->sunlit_cells = (long long)cnt[3];
        stats->sunlit_attempts = (long long)cnt[4];
        stats->device_ms = ms;
    }
    return (int)cnt[2];
}

extern "C" int cmaqchem_step_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                                    const float* dens, const float* pres, const float* seaice,
                                    const float* ocean_szone, const float* rj, const double* khetero, int jdate,
                                    int jtime, const int tstep[3], void* stream, cmaqchem_stats* stats)
{
    (void)jdate;
    (void)jtime;
    if (!h) return fail("null handle");
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    return step_device_impl(h, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero, tstep, s, stats);
}

extern "C" int cmaqchem_step(cmaqchem_handle* h, float* conc, const float* ta, const float* qv, const float* dens,
                             const float* pres, const float* seaice, const float* ocean_szone, const float* rj,
                             const double* khetero, int jdate, int jtime, const int tstep[3],
                             cmaqchem_stats* stats)
{
    (void)jdate;
    (void)jtime;
    if (!h) return fail("null handle");
    const void* ptrs[] = {conc, ta, qv, dens, pres, seaice, ocean_szone, rj, tstep, khetero};
    if (check_ptrs(ptrs, h->ops->nhetero > 0 ? 10 : 9)) return -1;
    CK(cudaSetDevice(h->device));
    const size_t nc = (size_t)h->ncell, ncr = (size_t)h->ncolrow;
    const size_t nconc = nc * h->cfg.nspcsd;
    if (!h->s_conc) {
        CK(cudaMalloc(&h->s_conc, sizeof(float) * nconc));
        CK(cudaMalloc(&h->s_ta, sizeof(float) * nc));
        CK(cudaMalloc(&h->s_qv, sizeof(float) * nc));
        CK(cudaMalloc(&h->s_dens, sizeof(float) * nc));
        CK(cudaMalloc(&h->s_pres, sizeof(float) * nc));
        CK(cudaMalloc(&h->s_seaice, sizeof(float) * ncr));
        CK(cudaMalloc(&h->s_osz, sizeof(float) * ncr));
        CK(cudaMalloc(&h->s_rj, sizeof(float) * nc * h->ops->nphotab));
        CK(cudaMalloc(&h->s_khet, sizeof(double) * nc * (h->ops->nhetero > 0 ? h->ops->nhetero : 1)));
    }
    cudaStream_t s = h->stream;
    CK(cudaMemcpyAsync(h->s_conc, conc, sizeof(float) * nconc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_ta, ta, sizeof(float) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_qv, qv, sizeof(float) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_dens, dens, sizeof(float) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_pres, pres, sizeof(float) * nc, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_seaice, seaice, sizeof(float) * ncr, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_osz, ocean_szone, sizeof(float) * ncr, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(h->s_rj, rj, sizeof(float) * nc * h->ops->nphotab, cudaMemcpyHostToDevice, s));
    if (h->ops->nhetero > 0)
        CK(cudaMemcpyAsync(h->s_khet, khetero, sizeof(double) * nc * h->ops->nhetero, cudaMemcpyHostToDevice, s));
    const int rc = step_device_impl(h, h->s_conc, h->s_ta, h->s_qv, h->s_dens, h->s_pres, h->s_seaice, h->s_osz,
                                    h->s_rj, h->s_khet, tstep, s, stats);
    if (rc < 0) return rc;
    CK(cudaMemcpyAsync(conc, h->s_conc, sizeof(float) * nconc, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return rc;
}

extern "C" int cmaqchem_cell_stats(cmaqchem_handle* h, int* status, int* attempts)
{
    if (!h) return fail("null handle");
    CK(cudaSetDevice(h->device));
    if (status) CK(cudaMemcpy(status, h->d_status, sizeof(int) * h->ncell, cudaMemcpyDeviceToHost));
    if (attempts) CK(cudaMemcpy(attempts, h->d_steps, sizeof(int) * h->ncell, cudaMemcpyDeviceToHost));
    return 0;
}

extern "C" int cmaqchem_ros3_solve_device(cmaqchem_handle* h, long long ncell, double* y, const double* rki,
                                          const unsigned char* night, double chemstep_min, int* status,
                                          int* nsteps, int* nfails, void* stream)
{
    if (!h) return fail("null handle");
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!y || !rki || !night) return fail("null array argument");
    if (!(chemstep_min > 0.0)) return fail("chemstep must be positive");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    chem::SolveArgs a{};
    a.y = y;
    a.rki = rki;
    a.night = night;
    a.ncell = ncell;
    a.chemstep = chemstep_min;
    a.tol = ros3::Tol{h->cfg.rtol, h->cfg.atol, h->rnspec};
    a.ws = h->d_ws;
    a.max_iter = h->max_iter;
    a.cell_status = status;
    a.cell_nsteps = nsteps;
    a.cell_nfails = nfails;
    CK(h->ops->solve(a, h->nblocks, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

extern "C" int cmaqchem_rconst_device(cmaqchem_handle* h, const float* conc, const float* ta, const float* qv,
                                      const float* dens, const float* pres, const float* seaice,
                                      const float* ocean_szone, const float* rj, const double* khetero,
                                      double* rki, unsigned char* sunlit, void* stream)
{
    if (!h) return fail("null handle");
    const void* ptrs[] = {conc, ta, qv, dens, pres, seaice, ocean_szone, rj, rki, khetero};
    if (check_ptrs(ptrs, h->ops->nhetero > 0 ? 10 : 9)) return -1;
    CK(cudaSetDevice(h->device));
    cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
    chem::GridArgs a = grid_args(h, const_cast<float*>(conc), ta, qv, dens, pres, seaice, ocean_szone, rj, khetero,
                                 1.0);
    CK(h->ops->rconst(a, rki, sunlit, h->nblocks, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}
