// C ABI of the chemistry library (include/cmaqchem.h).
//
// A handle holds what CMAQ's chemistry keeps in module SAVE state after its first call
// (rbdriver.F:226-371): mechanism tables (here: device tables and the generated code),
// the domain size and the solver's work arrays (here: per-warp device workspaces).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
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

constexpr int MAX_E2E_CHUNKS = 16;

// what a captured CHEM call depends on besides the handle's own buffers
struct GraphKey {
    const void* ptr[9];
    int itmstep;
};

struct cmaqchem_handle {
    const MechOps* ops = nullptr;
    cmaqchem_cfg cfg{};
    std::vector<int> cgrid_index;   // 0-based
    std::vector<int> conc_planes;   // distinct CGRID planes of the mechanism's species, ascending
    int device = 0, nsm = 0, bps = 1, nblocks = 0;
    long long ncell = 0;
    int ncolrow = 0;
    double rnspec = 0.0;
    int max_iter = 100000;
    int* d_cgrid_index = nullptr;
    int* d_convert = nullptr;
    float* d_fwd = nullptr;
    double* d_rev = nullptr;
    float* d_ebi_fwd = nullptr;     // EBI driver's FORWARD_CONV / REVERSE_CONV (hrinit.F:90-93)
    float* d_ebi_rev = nullptr;
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
    double dtmin = ros3::DTMIN;   // ROS3 minimum step (rbsolver.F:105), lowered only by a tuning knob
    // rate-constant pass of the work-queue ROS3 call: CALC_RCONST of every cell by whole warps
    // before the solver kernel, which then gathers the rates instead of evaluating them in
    // the few lanes it refills at a time (same numbers); allocated at set-up when it fits
    int rconst_pass = 1;
    double* d_rki_all = nullptr;
    uint8_t* d_sun_all = nullptr;
    int q_sync = 1;          // work-queue kernel: barriers between attempt phases
    int q_wpb = 8;           // work-queue kernel: warps per block
    int q_nblocks = 0;
    int q_bps_cap = 0;       // blocks per SM of the queue kernel, 0: as many as fit
    int ebi_warp = 1;        // EBI: 1 one cell per warp (shared memory), 0 one cell per lane
    int ebi_defer = 100;     // EBI: > 0 one cell per lane, cells past this many iterations per warp
                             // (100 measured best of 20-800 on CB6r5: +10 % over warps alone)
    int* d_ebi_def = nullptr;
    unsigned long long* d_ebi_ndef = nullptr;
    int ebiw_nblocks = 0;
    size_t ws_warps = 0;     // workspace capacity in warps
    int ws_elems = 0;        // workspace elements per lane (the solver's layout)
    // SMVGEAR
    gear::Coef gear_coef{};
    gear::Coef* d_gear_coef = nullptr;
    int gear_nblocks = 0;
    int gear_warp = 1;          // 1: one cell per warp in shared memory (k_gear_warp), 0: one per lane
    int gearw_nblocks = 0;
    float gear_max_atol = 1.0e-7f, gear_min_atol = 1.0e-9f, gear_floor = 1.0e-12f;
    // device staging of the host-pointer entry point, allocated on first use
    float *s_conc = nullptr, *s_ta = nullptr, *s_qv = nullptr, *s_dens = nullptr, *s_pres = nullptr;
    float *s_seaice = nullptr, *s_osz = nullptr, *s_rj = nullptr;
    double* s_khet = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_legacy = nullptr;   // orders the handle's stream after the legacy default stream
    // host-pointer path: copy stream and per-chunk events
    int e2e_chunks = 4;
    cudaStream_t copy_stream = nullptr, back_stream = nullptr;
    cudaEvent_t ev_in[MAX_E2E_CHUNKS] = {};
    cudaEvent_t ev_done[MAX_E2E_CHUNKS] = {};
    // discrete adjoint (allocated on first use, grown as needed)
    int adj_nblocks = 0;
    double* d_adj_ws = nullptr;
    double* d_tape_y = nullptr;
    double* d_tape_h = nullptr;
    size_t tape_cap = 0;               // entries
    long long* d_tape_off = nullptr;   // [nsync][ncell]
    size_t tape_off_cap = 0;
    long long* d_tiles = nullptr;      // [nsync][ntiles] scan tile bases
    long long* d_tape_tot = nullptr;   // [nsync]
    size_t tiles_cap = 0, tot_cap = 0;
    int* d_adj_order = nullptr;
    int* d_adj_status = nullptr;
    size_t adj_cell_cap = 0, adj_status_cap = 0;
    unsigned long long* d_adj_counters = nullptr;
    size_t adj_tape_budget = 0;        // bytes; 0: as large as the largest step needs and fits
    double* d_yave = nullptr;          // DDM-3D: time-averaged concentrations of the call
    // captured CHEM call of cmaqchem_steps_device
    cudaGraphExec_t graph_exec = nullptr;
    GraphKey graph_key{};
};

namespace {

void free_handle(cmaqchem_handle* h)
{
    if (!h) return;
    cudaSetDevice(h->device);
    void* ptrs[] = {h->d_cgrid_index, h->d_convert, h->d_fwd, h->d_rev, h->d_ebi_fwd, h->d_ebi_rev, h->d_ws, h->d_status, h->d_steps,
                    h->d_counters, h->d_order, h->d_hist, h->d_cursor, h->d_head, h->s_conc, h->s_ta,
                    h->s_qv, h->s_dens, h->s_pres, h->s_seaice, h->s_osz, h->s_rj, h->s_khet,
                    h->d_adj_ws, h->d_tape_y, h->d_tape_h, h->d_tape_off, h->d_tiles, h->d_tape_tot,
                    h->d_adj_order, h->d_adj_status, h->d_adj_counters, h->d_yave, h->d_gear_coef,
                    h->d_ebi_def, h->d_ebi_ndef, h->d_rki_all, h->d_sun_all};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    for (int i = 0; i < MAX_E2E_CHUNKS; ++i) {
        if (h->ev_in[i]) cudaEventDestroy(h->ev_in[i]);
        if (h->ev_done[i]) cudaEventDestroy(h->ev_done[i]);
    }
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->back_stream) cudaStreamDestroy(h->back_stream);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev_legacy) cudaEventDestroy(h->ev_legacy);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

// Grow the per-warp workspaces to `warps` (set-up calls only).
int ensure_ws(cmaqchem_handle* h, size_t warps)
{
    if (warps <= h->ws_warps) return 0;
    if (h->d_ws) CK(cudaFree(h->d_ws));
    h->d_ws = nullptr;
    CK(cudaMalloc(&h->d_ws, warps * (size_t)h->ws_elems * 32 * sizeof(double)));
    h->ws_warps = warps;
    return 0;
}

// The stream of a call: the caller's, or (stream null) the handle's own non-blocking
// stream, ordered after the work already on the legacy default stream, where a caller
// without a stream of its own (a PyTorch program on its default stream) wrote the inputs.
cudaStream_t call_stream(cmaqchem_handle* h, void* stream)
{
    if (stream) return (cudaStream_t)stream;
    if (cudaEventRecord(h->ev_legacy, cudaStreamLegacy) == cudaSuccess)
        cudaStreamWaitEvent(h->stream, h->ev_legacy, 0);
    return h->stream;
}

// Grid of the work-queue kernel for the handle's knobs: one persistent wave.
int configure_queue(cmaqchem_handle* h)
{
    int bps = 0;
    CK(h->ops->queue_occupancy(h->q_sync, h->q_wpb, &bps));
    if (bps < 1) bps = 1;
    if (h->q_bps_cap > 0 && bps > h->q_bps_cap) bps = h->q_bps_cap;
    h->q_nblocks = h->nsm * bps;
    return ensure_ws(h, (size_t)h->q_nblocks * h->q_wpb);
}

int upload_gear_coef(cmaqchem_handle* h)
{
    gear::coefficients(h->cfg.rtol, h->gear_max_atol, h->gear_min_atol, h->gear_floor, h->max_iter, &h->gear_coef);
    if (!h->d_gear_coef) CK(cudaMalloc(&h->d_gear_coef, sizeof(gear::Coef)));
    CK(cudaMemcpy(h->d_gear_coef, &h->gear_coef, sizeof(gear::Coef), cudaMemcpyHostToDevice));
    return 0;
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
    a.tol = ros3::Tol{h->cfg.rtol, h->cfg.atol, h->rnspec, h->dtmin};
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
    if (cfg->solver != CMAQCHEM_SOLVER_ROS3 && cfg->solver != CMAQCHEM_SOLVER_EBI &&
        cfg->solver != CMAQCHEM_SOLVER_GEAR)
        return fail("unknown solver");
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
    h->ws_elems = cfg->solver == CMAQCHEM_SOLVER_GEAR ? m->gear_ws_elems : m->ws_elems;
    if (cfg->solver == CMAQCHEM_SOLVER_GEAR) {
        h->gear_min_atol = (float)cfg->atol;   // cfg.atol = REAL(GEAR_MIN_ATOL, 8)
        if (!(h->gear_max_atol > h->gear_min_atol) || !(h->gear_min_atol > h->gear_floor)) {
            delete h;
            return fail("SMVGEAR needs GEAR_MAX_ATOL (1e-7) > atol > GEAR_CONC_FLOOR (1e-12)");
        }
    }
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
    h->conc_planes = h->cgrid_index;
    std::sort(h->conc_planes.begin(), h->conc_planes.end());
    h->conc_planes.erase(std::unique(h->conc_planes.begin(), h->conc_planes.end()), h->conc_planes.end());
    std::vector<float> fwd(m->nspec);
    std::vector<double> rev(m->nspec);
    for (int s = 0; s < m->nspec; ++s) {   // rbinit.F:252-253, REAL(4)
        fwd[s] = 1.0e-3f * 28.9628f / (float)m->molwt[s];
        rev[s] = (double)(1.0f / fwd[s]);
    }
    // hrinit.F:90-93: the EBI driver forms its factors in REAL(8) from REAL(4) constants
    // and the REAL(8) molecular weights, then stores them REAL(4)
    std::vector<float> ebi_fwd(m->nspec), ebi_rev(m->nspec);
    for (int s = 0; s < m->nspec; ++s) {
        ebi_fwd[s] = (float)((double)(1.0e-3f * 28.9628f) / m->molwt[s]);
        ebi_rev[s] = (float)((double)(1.0e+3f / 28.9628f) * m->molwt[s]);
    }
    int rc = 0;
    auto setup = [&]() -> int {
        CK(cudaSetDevice(h->device));
        CK(cudaDeviceGetAttribute(&h->nsm, cudaDevAttrMultiProcessorCount, h->device));
        CK(m->occupancy(&h->bps));
        if (h->bps < 1) h->bps = 1;
        h->nblocks = h->nsm * h->bps;
        if (ensure_ws(h, (size_t)h->nblocks * chem::WARPS_PER_BLOCK)) return -1;
        if (configure_queue(h)) return -1;
        if (cfg->solver == CMAQCHEM_SOLVER_GEAR) {
            int gb = 0;
            CK(m->gear_occupancy(&gb));
            h->gear_nblocks = h->nsm * (gb > 0 ? gb : 1);
            if (ensure_ws(h, (size_t)h->gear_nblocks * chem::GEAR_WPB)) return -1;
            int gw = 0;
            CK(m->gear_warp_occupancy(&gw));
            h->gearw_nblocks = h->nsm * (gw > 0 ? gw : 1);
            if (ensure_ws(h, (size_t)h->gearw_nblocks)) return -1;
            if (upload_gear_coef(h)) return -1;
        }
        if (cfg->solver == CMAQCHEM_SOLVER_EBI) {
            int bw = 0;
            CK(m->ebi_warp_occupancy(&bw));
            h->ebiw_nblocks = h->nsm * (bw > 0 ? bw : 1);
            if (ensure_ws(h, (size_t)h->ebiw_nblocks * chem::EBIW_WPB)) return -1;
            CK(cudaMalloc(&h->d_ebi_def, sizeof(int) * h->ncell));
            CK(cudaMalloc(&h->d_ebi_ndef, sizeof(unsigned long long)));
        }
        CK(cudaMalloc(&h->d_cgrid_index, sizeof(int) * m->nspec));
        CK(cudaMalloc(&h->d_convert, sizeof(int) * m->nspec));
        CK(cudaMalloc(&h->d_fwd, sizeof(float) * m->nspec));
        CK(cudaMalloc(&h->d_rev, sizeof(double) * m->nspec));
        CK(cudaMemcpy(h->d_cgrid_index, h->cgrid_index.data(), sizeof(int) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_convert, m->convert, sizeof(int) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_fwd, fwd.data(), sizeof(float) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_rev, rev.data(), sizeof(double) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMalloc(&h->d_ebi_fwd, sizeof(float) * m->nspec));
        CK(cudaMalloc(&h->d_ebi_rev, sizeof(float) * m->nspec));
        CK(cudaMemcpy(h->d_ebi_fwd, ebi_fwd.data(), sizeof(float) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMemcpy(h->d_ebi_rev, ebi_rev.data(), sizeof(float) * m->nspec, cudaMemcpyHostToDevice));
        CK(cudaMalloc(&h->d_status, sizeof(int) * h->ncell));
        CK(cudaMalloc(&h->d_steps, sizeof(int) * h->ncell));
        CK(cudaMemset(h->d_status, 0, sizeof(int) * h->ncell));
        CK(cudaMemset(h->d_steps, 0, sizeof(int) * h->ncell));
        CK(cudaMalloc(&h->d_counters, sizeof(unsigned long long) * 5));
        CK(cudaMalloc(&h->d_order, sizeof(int) * h->ncell));
        CK(cudaMalloc(&h->d_hist, sizeof(unsigned int) * chem::QUEUE_BINS));
        CK(cudaMalloc(&h->d_cursor, sizeof(unsigned long long) * chem::QUEUE_BINS));
        CK(cudaMalloc(&h->d_head, sizeof(unsigned long long)));
        if (cfg->solver == CMAQCHEM_SOLVER_ROS3 && cfg->schedule == CMAQCHEM_SCHED_QUEUE) {
            // the rate-constant pass's arrays, when they leave a quarter of the free memory
            const size_t bytes = sizeof(double) * (size_t)m->nrxns * h->ncell;
            size_t free_b = 0, total_b = 0;
            CK(cudaMemGetInfo(&free_b, &total_b));
            if (bytes + h->ncell < free_b - free_b / 4 && cudaMalloc(&h->d_rki_all, bytes) == cudaSuccess &&
                cudaMalloc(&h->d_sun_all, h->ncell) == cudaSuccess) {
                h->rconst_pass = 1;
            } else {
                cudaGetLastError();   // a failed allocation leaves the pass off, not an error
                if (h->d_rki_all) cudaFree(h->d_rki_all);
                h->d_rki_all = nullptr;
                h->d_sun_all = nullptr;
                h->rconst_pass = 0;
            }
        } else {
            h->rconst_pass = 0;
        }
        CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        CK(cudaEventCreate(&h->ev0));
        CK(cudaEventCreate(&h->ev1));
        CK(cudaEventCreateWithFlags(&h->ev_legacy, cudaEventDisableTiming));
        // the set-up memsets and copies above ran on the legacy default stream, which the
        // handle's non-blocking stream does not wait for
        CK(cudaDeviceSynchronize());
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
    CK(cudaSetDevice(h->device));
    if (strcmp(key, "night_pattern") == 0) {
        h->use_night = value != 0;
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        return 0;
    }
    if (strcmp(key, "lockstep") == 0) {
        if (value < 0 || value > 2) return fail("lockstep must be 0, 1 or 2");
        if (value == 0 && h->q_wpb != 8) return fail("lockstep 0 needs block_warps 8");
        h->q_sync = value;
    } else if (strcmp(key, "gear_warp") == 0) {
        h->gear_warp = value != 0;
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        return 0;
    } else if (strcmp(key, "ebi_defer") == 0) {
        if (value < 0) return fail("ebi_defer must be >= 0");
        h->ebi_defer = value;
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        return 0;
    } else if (strcmp(key, "ebi_warp") == 0) {
        h->ebi_warp = value != 0;
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        return 0;
    } else if (strcmp(key, "ros3_dtmin_exp") == 0) {
        // ROS3 minimum step 10^value min (the reference's DTMIN is 1e-8, value -8)
        if (value < -30 || value > -2) return fail("ros3_dtmin_exp must be in [-30, -2]");
        h->dtmin = pow(10.0, (double)value);
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        return 0;
    } else if (strcmp(key, "rconst_pass") == 0) {
        // 1: the work-queue ROS3 call evaluates CALC_RCONST in a pass of whole warps first
        // (when its arrays were allocated at set-up); 0: in the refilled lanes; same numbers
        h->rconst_pass = value != 0;
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        return 0;
    } else if (strcmp(key, "queue_history") == 0) {
        // 0: forget the previous call's step counts, so the next call starts with the work
        // queue of a fresh run's first call (cells in grid order)
        // (a set-up call: the device is idle before and after the clear, so no later call
        // on any stream can sort its queue by a half-cleared count array)
        if (value != 0) return fail("queue_history takes 0 (clear)");
        if (h->d_steps) {
            CK(cudaDeviceSynchronize());
            CK(cudaMemset(h->d_steps, 0, sizeof(int) * h->ncell));
            CK(cudaDeviceSynchronize());
        }
        h->have_history = false;
        return 0;
    } else if (strcmp(key, "host_chunks") == 0) {
        if (value < 1 || value > MAX_E2E_CHUNKS) return fail("host_chunks must be 1 .. 16");
        h->e2e_chunks = value;
        return 0;
    } else if (strcmp(key, "adjoint_tape_mb") == 0) {
        if (value < 0) return fail("adjoint_tape_mb must be >= 0");
        h->adj_tape_budget = (size_t)value << 20;
        return 0;
    } else if (strcmp(key, "blocks_per_sm") == 0) {
        if (value < 0 || value > 32) return fail("blocks_per_sm must be 0 (as many as fit) .. 32");
        h->q_bps_cap = value;
    } else if (strcmp(key, "block_warps") == 0) {
        if (value != 2 && value != 4 && value != 8) return fail("block_warps must be 2, 4 or 8");
        if (h->q_sync == 0 && value != 8) return fail("block_warps 2 or 4 needs lockstep 1 or 2");
        h->q_wpb = value;
    } else {
        return fail(std::string("unknown tuning key ") + key);
    }
    if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));   // launch shape changed
    h->graph_exec = nullptr;
    return configure_queue(h);
}

// Enqueue the launches of one CHEM call (no host synchronisation).  sort: order the work
// queue by the previous call's step attempts.
static int enqueue_step(cmaqchem_handle* h, const chem::GridArgs& a, int itmstep, cudaStream_t s, bool sort,
                        long long c0 = 0, long long c1 = -1)
{
    const bool ebi_solver = h->cfg.solver == CMAQCHEM_SOLVER_EBI;
    const bool gear_solver = h->cfg.solver == CMAQCHEM_SOLVER_GEAR;
    if (c1 < 0) c1 = h->ncell;
    const long long n = c1 - c0;
    if (h->cfg.schedule == CMAQCHEM_SCHED_QUEUE || ebi_solver || gear_solver) {
        chem::QueueArgs q{nullptr, h->d_head, n, c0};
        if (sort && (h->cfg.schedule == CMAQCHEM_SCHED_QUEUE || gear_solver)) {
            const int nb = 4 * h->nsm;
            CK(cudaMemsetAsync(h->d_hist, 0, sizeof(unsigned int) * chem::QUEUE_BINS, s));
            chem::k_queue_hist<<<nb, 256, 0, s>>>(h->d_steps + c0, n, h->d_hist);
            CK(cudaGetLastError());
            chem::k_queue_scan<<<1, chem::QUEUE_BINS, 0, s>>>(h->d_hist, h->d_cursor);
            CK(cudaGetLastError());
            chem::k_queue_scatter<<<nb, 256, 0, s>>>(h->d_steps + c0, n, h->d_cursor, h->d_order + c0);
            CK(cudaGetLastError());
            q.order = h->d_order + c0;
        }
        CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
        if (gear_solver) {
            chem::GearArgs g{};
            g.coef = h->d_gear_coef;
            if (h->gear_warp) CK(h->ops->gear_warp(a, q, g, true, h->gearw_nblocks, s));
            else CK(h->ops->gear(a, q, g, true, h->gear_nblocks, s));
        } else if (ebi_solver) {
            chem::EbiArgs e{};
            ebi::steps_for(itmstep, h->ops->ebi_deltat, &e.n_ebi_steps, &e.tmstep);
            e.fwd = h->d_ebi_fwd;
            e.rev = h->d_ebi_rev;
            if (h->ebi_defer > 0) {
                // one cell per lane for the cells that finish within ebi_defer iterations,
                // then one cell per warp for the others
                e.defer_after = h->ebi_defer;
                e.deferred = h->d_ebi_def;
                e.ndeferred = h->d_ebi_ndef;
                CK(cudaMemsetAsync(h->d_ebi_ndef, 0, sizeof(unsigned long long), s));
                CK(h->ops->chem_ebi(a, q, e, h->nblocks, s));
                chem::QueueArgs q2{h->d_ebi_def, h->d_head, 0, 0, h->d_ebi_ndef};
                chem::EbiArgs e2 = e;
                e2.defer_after = 0;
                CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
                CK(h->ops->chem_ebi_warp(a, q2, e2, h->ebiw_nblocks, s));
            } else if (h->ebi_warp) {
                CK(h->ops->chem_ebi_warp(a, q, e, h->ebiw_nblocks, s));
            } else {
                CK(h->ops->chem_ebi(a, q, e, h->nblocks, s));
            }
        } else if (h->rconst_pass && h->d_rki_all) {
            CK(h->ops->rconst_pass(a, c0, c1, h->d_rki_all, h->d_sun_all, h->nblocks, s));
            chem::GridArgs ap = a;
            ap.rki_all = h->d_rki_all;
            ap.sun_all = h->d_sun_all;
            CK(h->ops->chem_queue(ap, q, h->q_sync, h->q_wpb, h->q_nblocks, s));
        } else {
            CK(h->ops->chem_queue(a, q, h->q_sync, h->q_wpb, h->q_nblocks, s));
        }
    } else {
        CK(h->ops->chem_static(a, h->nblocks, s));
    }
    return 0;
}

static int finish_steps(cmaqchem_handle* h, cudaStream_t s, cmaqchem_stats* stats)
{
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
    if (enqueue_step(h, a, itmstep, s, h->have_history)) return -1;
    return finish_steps(h, s, stats);
}

extern "C" int cmaqchem_step_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                                    const float* dens, const float* pres, const float* seaice,
                                    const float* ocean_szone, const float* rj, const double* khetero, int jdate,
                                    int jtime, const int tstep[3], void* stream, cmaqchem_stats* stats)
{
    (void)jdate;
    (void)jtime;
    if (!h) return fail("null handle");
    cudaStream_t s = call_stream(h, stream);
    return step_device_impl(h, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero, tstep, s, stats);
}

extern "C" int cmaqchem_step_ddm_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                                        const float* dens, const float* pres, const float* seaice,
                                        const float* ocean_szone, const float* rj, const double* khetero,
                                        int jdate, int jtime, const int tstep[3], float* sengrid, int nparam,
                                        const unsigned char* rate_mask, const float* region, void* stream,
                                        cmaqchem_stats* stats)
{
    (void)jdate;
    (void)jtime;
    if (!h) return fail("null handle");
    if (nparam <= 0 || !sengrid) return fail("DDM-3D needs sengrid and nparam > 0");
    const void* ptrs[] = {conc, ta, qv, dens, pres, seaice, ocean_szone, rj, tstep, khetero};
    if (check_ptrs(ptrs, h->ops->nhetero > 0 ? 10 : 9)) return -1;
    const int itmstep = hhmmss_to_sec(tstep[1]);
    if (itmstep <= 0) return fail("TSTEP(2) must be a positive HHMMSS interval");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = call_stream(h, stream);
    if (!h->d_yave) CK(cudaMalloc(&h->d_yave, sizeof(double) * h->ops->ischan * h->ncell));
    chem::GridArgs a = grid_args(h, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero,
                                 (double)itmstep / 60.0);
    a.yave = h->d_yave;
    CK(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 5, s));
    CK(cudaEventRecord(h->ev0, s));
    if (enqueue_step(h, a, itmstep, s, h->have_history)) return -1;
    chem::DdmArgs d{sengrid, nparam, rate_mask, region, h->d_yave};
    a.counters = nullptr;
    a.cell_status = nullptr;
    a.cell_steps = nullptr;
    CK(h->ops->ddm_update(a, d, h->nblocks, s));
    return finish_steps(h, s, stats);
}

extern "C" int cmaqchem_steps_device(cmaqchem_handle* h, float* conc, const float* ta, const float* qv,
                                     const float* dens, const float* pres, const float* seaice,
                                     const float* ocean_szone, const float* rj, const double* khetero, int jdate,
                                     int jtime, const int tstep[3], int nsteps, void* stream, cmaqchem_stats* stats)
{
    (void)jdate;
    (void)jtime;
    if (!h) return fail("null handle");
    if (nsteps <= 0) return fail("nsteps must be positive");
    const void* ptrs[] = {conc, ta, qv, dens, pres, seaice, ocean_szone, rj, tstep, khetero};
    if (check_ptrs(ptrs, h->ops->nhetero > 0 ? 10 : 9)) return -1;
    const int itmstep = hhmmss_to_sec(tstep[1]);
    if (itmstep <= 0) return fail("TSTEP(2) must be a positive HHMMSS interval");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = call_stream(h, stream);
    GraphKey key{{conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero}, itmstep};
    if (!h->graph_exec || memcmp(&key, &h->graph_key, sizeof(key)) != 0) {
        if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
        h->graph_exec = nullptr;
        chem::GridArgs a = grid_args(h, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero,
                                     (double)itmstep / 60.0);
        // capture one call on the handle's own stream; the work queue is always ordered
        // (by zero counts before the first call, which is a plain permutation)
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_step(h, a, itmstep, h->stream, true);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return -1;
        }
        CK(ce);
        const cudaError_t ie = cudaGraphInstantiate(&h->graph_exec, g, 0);
        cudaGraphDestroy(g);
        CK(ie);
        h->graph_key = key;
    }
    CK(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 5, s));
    CK(cudaEventRecord(h->ev0, s));
    for (int i = 0; i < nsteps; ++i) CK(cudaGraphLaunch(h->graph_exec, s));
    return finish_steps(h, s, stats);
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
    const int itmstep = hhmmss_to_sec(tstep[1]);
    if (itmstep <= 0) return fail("TSTEP(2) must be a positive HHMMSS interval");
    cudaStream_t s = h->stream;
    cudaStream_t cs = h->copy_stream;       // host -> device
    if (!cs) {
        CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&h->back_stream, cudaStreamNonBlocking));
        cs = h->copy_stream;
        for (int i = 0; i < MAX_E2E_CHUNKS; ++i) {
            CK(cudaEventCreateWithFlags(&h->ev_in[i], cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&h->ev_done[i], cudaEventDisableTiming));
        }
    }
    // The grid is split into chunks of consecutive cells: the inputs of chunk i+1 travel
    // and the results of chunk i-1 come back while chunk i is integrated.  Only the
    // mechanism's CGRID planes are read and written by CHEM.
    const bool chunked = h->cfg.schedule == CMAQCHEM_SCHED_QUEUE || h->cfg.solver != CMAQCHEM_SOLVER_ROS3;
    const int nch = chunked ? std::max(1, std::min<int>(h->e2e_chunks, (int)std::min<long long>(MAX_E2E_CHUNKS, nc))) : 1;
    const int nhet = h->ops->nhetero;
    CK(cudaMemcpyAsync(h->s_seaice, seaice, sizeof(float) * ncr, cudaMemcpyHostToDevice, cs));
    CK(cudaMemcpyAsync(h->s_osz, ocean_szone, sizeof(float) * ncr, cudaMemcpyHostToDevice, cs));
    chem::GridArgs a = grid_args(h, h->s_conc, h->s_ta, h->s_qv, h->s_dens, h->s_pres, h->s_seaice, h->s_osz,
                                 h->s_rj, h->s_khet, (double)itmstep / 60.0);
    CK(cudaMemsetAsync(h->d_counters, 0, sizeof(unsigned long long) * 5, s));
    CK(cudaEventRecord(h->ev0, s));
    // uploads of every chunk in order on one stream, the integration of chunk i once its
    // inputs are in, its write-back on a third stream once it is integrated
    for (int i = 0; i < nch; ++i) {
        const size_t c0 = nc * i / nch, c1 = nc * (i + 1) / nch, n = c1 - c0;
        auto h2d = [&](void* dst, const void* src, size_t bytes) {
            return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, cs);
        };
        for (int p : h->conc_planes) CK(h2d(h->s_conc + p * nc + c0, conc + p * nc + c0, sizeof(float) * n));
        CK(h2d(h->s_ta + c0, ta + c0, sizeof(float) * n));
        CK(h2d(h->s_qv + c0, qv + c0, sizeof(float) * n));
        CK(h2d(h->s_dens + c0, dens + c0, sizeof(float) * n));
        CK(h2d(h->s_pres + c0, pres + c0, sizeof(float) * n));
        for (int k = 0; k < h->ops->nphotab; ++k) CK(h2d(h->s_rj + k * nc + c0, rj + k * nc + c0, sizeof(float) * n));
        if (nhet > 0) CK(h2d(h->s_khet + c0 * nhet, khetero + c0 * nhet, sizeof(double) * n * nhet));
        CK(cudaEventRecord(h->ev_in[i], cs));
    }
    for (int i = 0; i < nch; ++i) {
        const size_t c0 = nc * i / nch, c1 = nc * (i + 1) / nch, n = c1 - c0;
        CK(cudaStreamWaitEvent(s, h->ev_in[i], 0));
        if (nch == 1) {
            if (enqueue_step(h, a, itmstep, s, h->have_history)) return -1;
        } else {
            if (enqueue_step(h, a, itmstep, s, h->have_history, (long long)c0, (long long)c1)) return -1;
        }
        CK(cudaEventRecord(h->ev_done[i], s));
        CK(cudaStreamWaitEvent(h->back_stream, h->ev_done[i], 0));
        for (int p : h->conc_planes)
            CK(cudaMemcpyAsync(conc + p * nc + c0, h->s_conc + p * nc + c0, sizeof(float) * n,
                               cudaMemcpyDeviceToHost, h->back_stream));
    }
    const int rc = finish_steps(h, s, stats);
    CK(cudaStreamSynchronize(h->back_stream));
    return rc;
}

extern "C" int cmaqchem_cell_stats(cmaqchem_handle* h, int* status, int* attempts)
{
    if (!h) return fail("null handle");
    CK(cudaSetDevice(h->device));
    CK(cudaDeviceSynchronize());   // the counts of calls still running on the handle's stream
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
    cudaStream_t s = call_stream(h, stream);
    chem::SolveArgs a{};
    a.y = y;
    a.rki = rki;
    a.night = night;
    a.ncell = ncell;
    a.chemstep = chemstep_min;
    a.tol = ros3::Tol{h->cfg.rtol, h->cfg.atol, h->rnspec, h->dtmin};
    a.ws = h->d_ws;
    a.max_iter = h->max_iter;
    a.cell_status = status;
    a.cell_nsteps = nsteps;
    a.cell_nfails = nfails;
    CK(h->ops->solve(a, h->nblocks, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

extern "C" int cmaqchem_ebi_solve_device(cmaqchem_handle* h, long long ncell, double* yc, const double* rki,
                                         int tstep_sec, int* status, int* iterations, void* stream)
{
    if (!h) return fail("null handle");
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!yc || !rki) return fail("null array argument");
    if (tstep_sec <= 0) return fail("tstep_sec must be positive");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = call_stream(h, stream);
    chem::EbiSolveArgs a{};
    a.yc = yc;
    a.rki = rki;
    a.ncell = ncell;
    ebi::steps_for(tstep_sec, h->ops->ebi_deltat, &a.n_ebi_steps, &a.tmstep);
    a.ws = h->d_ws;
    a.max_iter = h->max_iter;
    a.cell_status = status;
    a.cell_iters = iterations;
    CK(h->ops->ebi_solve(a, h->nblocks, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

extern "C" int cmaqchem_gear_solve_device(cmaqchem_handle* h, long long ncell, double* y, const double* rk,
                                          const unsigned char* night, double chemstep_min, int* cell_stats,
                                          void* stream)
{
    if (!h) return fail("null handle");
    if (h->cfg.solver != CMAQCHEM_SOLVER_GEAR) return fail("the handle was not made for CMAQCHEM_SOLVER_GEAR");
    if (ncell < 0) return fail("ncell must be >= 0");
    if (ncell == 0) return 0;
    if (!y || !rk || !night) return fail("null array argument");
    if (!(chemstep_min > 0.0)) return fail("chemstep must be positive");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = call_stream(h, stream);
    chem::GridArgs a{};
    a.ncell = ncell;
    a.chemstep = chemstep_min;
    a.ws = h->d_ws;
    a.max_iter = h->max_iter;
    chem::QueueArgs q{nullptr, h->d_head, ncell, 0};
    chem::GearArgs g{};
    g.coef = h->d_gear_coef;
    g.y = y;
    g.rk = rk;
    g.night = night;
    g.cell_stats = cell_stats;
    CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
    if (h->gear_warp) CK(h->ops->gear_warp(a, q, g, false, h->gearw_nblocks, s));
    else CK(h->ops->gear(a, q, g, false, h->gear_nblocks, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

extern "C" int cmaqchem_gear_tolerances(cmaqchem_handle* h, float max_atol, float min_atol, float conc_floor)
{
    if (!h) return fail("null handle");
    if (h->cfg.solver != CMAQCHEM_SOLVER_GEAR) return fail("the handle was not made for CMAQCHEM_SOLVER_GEAR");
    if (!(max_atol > min_atol) || !(min_atol > conc_floor) || !(conc_floor > 0.0f))
        return fail("need max_atol > min_atol > conc_floor > 0");
    CK(cudaSetDevice(h->device));
    h->gear_max_atol = max_atol;
    h->gear_min_atol = min_atol;
    h->gear_floor = conc_floor;
    if (h->graph_exec) CK(cudaGraphExecDestroy(h->graph_exec));
    h->graph_exec = nullptr;
    return upload_gear_coef(h);
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
    cudaStream_t s = call_stream(h, stream);
    chem::GridArgs a = grid_args(h, const_cast<float*>(conc), ta, qv, dens, pres, seaice, ocean_szone, rj, khetero,
                                 1.0);
    CK(h->ops->rconst(a, rki, sunlit, h->nblocks, s));
    CK(cudaStreamSynchronize(s));
    return 0;
}

// ------------------------------------------------------------------ discrete adjoint

namespace {

template <class T>
int grow(T** p, size_t* cap, size_t need)
{
    if (need <= *cap) return 0;
    if (*p) CK(cudaFree(*p));
    *p = nullptr;
    *cap = 0;
    CK(cudaMalloc(p, need * sizeof(T)));
    *cap = need;
    return 0;
}

int adj_setup(cmaqchem_handle* h, long long ncell)
{
    if (!h->d_adj_ws) {
        int fb = 0, rb = 0;
        CK(h->ops->adj_occupancy(&fb, &rb));
        int bps = fb < rb ? fb : rb;
        if (bps < 1) bps = 1;
        h->adj_nblocks = h->nsm * bps;
        CK(cudaMalloc(&h->d_adj_ws, (size_t)h->adj_nblocks * adj::WPB * h->ops->adj_ws_elems * 32 * sizeof(double)));
        CK(cudaMalloc(&h->d_adj_counters, 3 * sizeof(unsigned long long)));
    }
    if (grow(&h->d_adj_order, &h->adj_cell_cap, (size_t)ncell)) return -1;
    if (grow(&h->d_adj_status, &h->adj_status_cap, (size_t)ncell)) return -1;
    return 0;
}

// queue order of the cells by step counts, most first
int adj_order(cmaqchem_handle* h, const int* steps, long long ncell, cudaStream_t s)
{
    const int nb = 4 * h->nsm;
    CK(cudaMemsetAsync(h->d_hist, 0, sizeof(unsigned int) * chem::QUEUE_BINS, s));
    chem::k_queue_hist<<<nb, 256, 0, s>>>(steps, ncell, h->d_hist);
    CK(cudaGetLastError());
    chem::k_queue_scan<<<1, chem::QUEUE_BINS, 0, s>>>(h->d_hist, h->d_cursor);
    CK(cudaGetLastError());
    chem::k_queue_scatter<<<nb, 256, 0, s>>>(steps, ncell, h->d_cursor, h->d_adj_order);
    CK(cudaGetLastError());
    return 0;
}

adj::Args adj_args(cmaqchem_handle* h, long long ncell, const double* rki, const unsigned char* night,
                   const double* kmult, const double* emis, double chemstep)
{
    adj::Args a{};
    a.ncell = ncell;
    a.chemstep = chemstep;
    a.tol = ros3::Tol{h->cfg.rtol, h->cfg.atol, h->rnspec, h->dtmin};
    a.max_iter = h->max_iter;
    a.ws = h->d_adj_ws;
    a.rki = rki;
    a.kmult = kmult;
    a.emis = emis;
    a.night = night;
    a.head = h->d_head;
    a.counters = h->d_adj_counters;
    return a;
}

// Carving of a caller's forward-tape buffer: head, per-step overflow counters, per-step
// last block and fill of every cell, then the block pool (previous-block links, step
// sizes, states).
struct TapePool {
    unsigned long long* head = nullptr;
    unsigned int* ovf = nullptr;
    long long* last_block = nullptr;
    int* last_fill = nullptr;
    long long* prev = nullptr;
    double* h = nullptr;
    double* y = nullptr;
    long long blocks = 0;
};

TapePool carve_pool(void* buf, size_t bytes, long long ncell, int nsync, int ischan)
{
    TapePool t;
    if (!buf) return t;
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    size_t off = 0;
    const size_t o_head = off; off = align(off + sizeof(unsigned long long));
    const size_t o_ovf = off; off = align(off + sizeof(unsigned int) * nsync);
    const size_t o_lb = off; off = align(off + sizeof(long long) * nsync * ncell);
    const size_t o_lf = off; off = align(off + sizeof(int) * nsync * ncell);
    if (bytes <= off) return t;
    const size_t per_block = sizeof(long long) + adj::TAPE_BLOCK * sizeof(double) * (1 + (size_t)ischan);
    const long long nb = (long long)((bytes - off - 3 * 256) / per_block);
    if (nb < 1) return t;
    char* b = (char*)buf;
    t.head = (unsigned long long*)(b + o_head);
    t.ovf = (unsigned int*)(b + o_ovf);
    t.last_block = (long long*)(b + o_lb);
    t.last_fill = (int*)(b + o_lf);
    t.prev = (long long*)(b + off); off = align(off + sizeof(long long) * nb);
    t.h = (double*)(b + off); off = align(off + sizeof(double) * nb * adj::TAPE_BLOCK);
    t.y = (double*)(b + off);
    t.blocks = nb;
    return t;
}

int adj_check(cmaqchem_handle* h, long long ncell, const void* y, const double* rki, const unsigned char* night,
              int nsync, double chemstep, const void* ck, const int* nsteps)
{
    if (!h) return fail("null handle");
    if (ncell <= 0) return fail("ncell must be positive");
    if (ncell > (long long)INT32_MAX) return fail("ncell must fit in 32 bits");
    if (!y || !rki || !night || !ck || !nsteps) return fail("null array argument");
    if (nsync <= 0) return fail("nsync must be positive");
    if (!(chemstep > 0.0)) return fail("chemstep must be positive");
    return 0;
}

}  // namespace

extern "C" int cmaqchem_adj_forward(cmaqchem_handle* h, long long ncell, double* y, const double* rki,
                                    long long rki_sync_stride, const unsigned char* night, const double* kmult,
                                    const double* emis, int nsync, double chemstep_min, double* checkpoints,
                                    int* nsteps, void* tape, size_t tape_bytes, void* stream)
{
    if (adj_check(h, ncell, y, rki, night, nsync, chemstep_min, checkpoints, nsteps)) return -1;
    CK(cudaSetDevice(h->device));
    cudaStream_t s = call_stream(h, stream);
    if (adj_setup(h, ncell)) return -1;
    CK(cudaMemsetAsync(h->d_adj_counters, 0, 3 * sizeof(unsigned long long), s));
    const TapePool pool = carve_pool(tape, tape_bytes, ncell, nsync, h->ops->ischan);
    if (pool.blocks > 0) {
        CK(cudaMemsetAsync(pool.head, 0, sizeof(unsigned long long), s));
        CK(cudaMemsetAsync(pool.ovf, 0, sizeof(unsigned int) * nsync, s));
    }
    const size_t plane = (size_t)h->ops->ischan * ncell;
    for (int k = 0; k < nsync; ++k) {
        double* ck = checkpoints + (size_t)k * plane;
        CK(cudaMemcpyAsync(ck, y, plane * sizeof(double), cudaMemcpyDeviceToDevice, s));
        adj::Args a = adj_args(h, ncell, rki + (size_t)k * rki_sync_stride, night, kmult, emis, chemstep_min);
        a.y_in = ck;
        a.y_out = y;
        a.nsteps = nsteps + (size_t)k * ncell;
        a.status = h->d_adj_status;
        if (pool.blocks > 0) {
            a.pool_y = pool.y;
            a.pool_h = pool.h;
            a.pool_prev = pool.prev;
            a.pool_blocks = pool.blocks;
            a.pool_head = pool.head;
            a.pool_ovf = pool.ovf + k;
            a.last_block = pool.last_block + (size_t)k * ncell;
            a.last_fill = pool.last_fill + (size_t)k * ncell;
        }
        if (k > 0) {
            if (adj_order(h, nsteps + (size_t)(k - 1) * ncell, ncell, s)) return -1;
            a.order = h->d_adj_order;
        }
        CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
        CK(h->ops->adj_forward(a, h->adj_nblocks, s));
    }
    unsigned long long cnt[3];
    CK(cudaMemcpyAsync(cnt, h->d_adj_counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return (int)cnt[2];
}

extern "C" int cmaqchem_adj_backward(cmaqchem_handle* h, long long ncell, double* lambda, const double* rki,
                                     long long rki_sync_stride, const unsigned char* night, const double* kmult,
                                     const double* emis, int nsync, double chemstep_min, const double* checkpoints,
                                     const int* nsteps, const void* tape, size_t tape_bytes, double* grad_logk,
                                     double* grad_emis, void* stream)
{
    if (adj_check(h, ncell, lambda, rki, night, nsync, chemstep_min, checkpoints, nsteps)) return -1;
    if (!grad_logk) return fail("null array argument");
    CK(cudaSetDevice(h->device));
    cudaStream_t s = call_stream(h, stream);
    if (adj_setup(h, ncell)) return -1;
    // steps whose tape the forward pass recorded completely skip the re-run
    const TapePool pool = carve_pool(const_cast<void*>(tape), tape_bytes, ncell, nsync, h->ops->ischan);
    std::vector<unsigned int> ovf(nsync, 1u);
    if (pool.blocks > 0) {
        CK(cudaMemcpyAsync(ovf.data(), pool.ovf, sizeof(unsigned int) * nsync, cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
    }
    bool need_rerun = false;
    for (unsigned int v : ovf) need_rerun = need_rerun || v != 0;
    if (!need_rerun) {
        CK(cudaMemsetAsync(h->d_adj_counters, 0, 3 * sizeof(unsigned long long), s));
        for (int k = nsync - 1; k >= 0; --k) {
            adj::Args a = adj_args(h, ncell, rki + (size_t)k * rki_sync_stride, night, kmult, emis, chemstep_min);
            a.nsteps = const_cast<int*>(nsteps) + (size_t)k * ncell;
            a.pool_y = pool.y;
            a.pool_h = pool.h;
            a.pool_prev = pool.prev;
            a.pool_blocks = pool.blocks;
            a.last_block = pool.last_block + (size_t)k * ncell;
            a.last_fill = pool.last_fill + (size_t)k * ncell;
            if (adj_order(h, a.nsteps, ncell, s)) return -1;
            a.order = h->d_adj_order;
            a.lam = lambda;
            a.grad_logk = grad_logk;
            a.grad_emis = grad_emis;
            CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
            CK(h->ops->adj_reverse(a, h->adj_nblocks, s));
        }
        unsigned long long cnt[3];
        CK(cudaMemcpyAsync(cnt, h->d_adj_counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (cnt[1] != (unsigned long long)ncell * nsync) return fail("reverse sweep did not visit every cell");
        return 0;
    }
    // tape offsets of every synchronisation step
    const int ntiles = (int)((ncell + adj::SCAN_TILE - 1) / adj::SCAN_TILE);
    if (grow(&h->d_tape_off, &h->tape_off_cap, (size_t)nsync * ncell)) return -1;
    if (grow(&h->d_tiles, &h->tiles_cap, (size_t)nsync * ntiles)) return -1;
    if (grow(&h->d_tape_tot, &h->tot_cap, (size_t)nsync)) return -1;
    for (int k = 0; k < nsync; ++k) {
        const int* v = nsteps + (size_t)k * ncell;
        long long* tiles = h->d_tiles + (size_t)k * ntiles;
        adj::k_scan_tiles<<<ntiles, 256, 0, s>>>(v, ncell, tiles);
        CK(cudaGetLastError());
        adj::k_scan_tile_sums<<<1, 32, 0, s>>>(tiles, ntiles, h->d_tape_tot + k);
        CK(cudaGetLastError());
        adj::k_scan_apply<<<ntiles, 256, 0, s>>>(v, ncell, tiles, h->d_tape_off + (size_t)k * ncell);
        CK(cudaGetLastError());
    }
    std::vector<long long> tot(nsync);
    CK(cudaMemcpyAsync(tot.data(), h->d_tape_tot, sizeof(long long) * nsync, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    long long tmax = 1;
    for (long long t : tot) {
        if (t < 0) return fail("negative step count");
        tmax = t > tmax ? t : tmax;
    }
    // tape capacity: the largest step's tape, or the budget (then steps run in cell batches)
    const size_t entry_bytes = (size_t)(h->ops->ischan + 1) * sizeof(double);
    size_t want = (size_t)tmax;
    if (h->adj_tape_budget > 0) want = std::min(want, std::max<size_t>(1, h->adj_tape_budget / entry_bytes));
    if (want > h->tape_cap || (h->adj_tape_budget > 0 && h->tape_cap * entry_bytes > h->adj_tape_budget)) {
        if (h->d_tape_y) CK(cudaFree(h->d_tape_y));
        if (h->d_tape_h) CK(cudaFree(h->d_tape_h));
        h->d_tape_y = nullptr;
        h->d_tape_h = nullptr;
        h->tape_cap = 0;
        for (;;) {   // without a budget, halve the request until it fits in free memory
            cudaError_t e = cudaMalloc(&h->d_tape_y, want * h->ops->ischan * sizeof(double));
            if (e == cudaSuccess) e = cudaMalloc(&h->d_tape_h, want * sizeof(double));
            if (e == cudaSuccess) break;
            cudaGetLastError();
            if (h->d_tape_y) cudaFree(h->d_tape_y);
            h->d_tape_y = nullptr;
            if (h->adj_tape_budget > 0 || want < 1024)
                return fail("adjoint tape of " + std::to_string((want * entry_bytes) >> 20) +
                            " MiB does not fit: " + cudaGetErrorString(e));
            want /= 2;
        }
        h->tape_cap = want;
    }
    CK(cudaMemsetAsync(h->d_adj_counters, 0, 3 * sizeof(unsigned long long), s));
    const size_t plane = (size_t)h->ops->ischan * ncell;
    std::vector<long long> off;
    std::vector<int> nst;
    for (int k = nsync - 1; k >= 0; --k) {
        if (pool.blocks > 0 && ovf[k] == 0) {   // this step's tape is complete in the pool
            adj::Args a = adj_args(h, ncell, rki + (size_t)k * rki_sync_stride, night, kmult, emis, chemstep_min);
            a.nsteps = const_cast<int*>(nsteps) + (size_t)k * ncell;
            a.pool_y = pool.y;
            a.pool_h = pool.h;
            a.pool_prev = pool.prev;
            a.pool_blocks = pool.blocks;
            a.last_block = pool.last_block + (size_t)k * ncell;
            a.last_fill = pool.last_fill + (size_t)k * ncell;
            if (adj_order(h, a.nsteps, ncell, s)) return -1;
            a.order = h->d_adj_order;
            a.lam = lambda;
            a.grad_logk = grad_logk;
            a.grad_emis = grad_emis;
            CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
            CK(h->ops->adj_reverse(a, h->adj_nblocks, s));
            continue;
        }
        adj::Args a = adj_args(h, ncell, rki + (size_t)k * rki_sync_stride, night, kmult, emis, chemstep_min);
        a.nsteps = const_cast<int*>(nsteps) + (size_t)k * ncell;
        a.tape_off = h->d_tape_off + (size_t)k * ncell;
        a.tape_y = h->d_tape_y;
        a.tape_h = h->d_tape_h;
        a.y_in = checkpoints + (size_t)k * plane;
        a.lam = nullptr;
        // batches of consecutive cells whose tapes fit the capacity (one batch if the step fits)
        std::vector<std::pair<long long, long long>> batches;
        if ((size_t)tot[k] <= h->tape_cap) {
            batches.push_back({0, ncell});
        } else {
            off.resize(ncell);
            nst.resize(ncell);
            CK(cudaMemcpyAsync(off.data(), a.tape_off, sizeof(long long) * ncell, cudaMemcpyDeviceToHost, s));
            CK(cudaMemcpyAsync(nst.data(), a.nsteps, sizeof(int) * ncell, cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            long long c0 = 0;
            while (c0 < ncell) {
                if ((size_t)nst[c0] > h->tape_cap) return fail("one cell's tape exceeds the adjoint tape budget");
                long long c1 = c0 + 1;
                while (c1 < ncell && (size_t)(off[c1] + nst[c1] - off[c0]) <= h->tape_cap) ++c1;
                batches.push_back({c0, c1});
                c0 = c1;
            }
        }
        for (const auto& bt : batches) {
            const bool whole = bt.first == 0 && bt.second == ncell;
            if (whole) {
                if (adj_order(h, a.nsteps, ncell, s)) return -1;
                a.order = h->d_adj_order;
                a.queue_len = 0;
                a.cell0 = 0;
                a.tape_base = 0;
            } else {
                a.order = nullptr;
                a.queue_len = bt.second - bt.first;
                a.cell0 = bt.first;
                a.tape_base = off[bt.first];
            }
            // re-run the step from its checkpoint, recording the tape
            a.lam = nullptr;
            a.grad_logk = nullptr;
            a.grad_emis = nullptr;
            CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
            CK(h->ops->adj_forward(a, h->adj_nblocks, s));
            // reverse sweep
            a.lam = lambda;
            a.grad_logk = grad_logk;
            a.grad_emis = grad_emis;
            CK(cudaMemsetAsync(h->d_head, 0, sizeof(unsigned long long), s));
            CK(h->ops->adj_reverse(a, h->adj_nblocks, s));
        }
    }
    unsigned long long cnt[3];
    CK(cudaMemcpyAsync(cnt, h->d_adj_counters, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (cnt[0] != 0) return fail("the re-run of a step took more accepted steps than the forward pass recorded");
    if (cnt[1] != (unsigned long long)ncell * nsync) return fail("reverse sweep did not visit every cell");
    return (int)cnt[2];
}
