// Discrete adjoint of the per-cell ROS3 integration (solver level), FP64.
//
// The forward map of one synchronisation step is the sequence of accepted ROS3 steps of
// rbsolver.F:344-589 for one cell, here with two extra inputs that the gradient needs:
// per-reaction rate multipliers (RKI = rki * kmult) and an emission tendency E added to
// f.  With the step sizes h_n of the accepted steps held fixed, step n maps
//
//   A = J(Y) - I/(gamma h),  K1 = A^-1 (-f(Y)),  YP = Y + K1,
//   K2 = A^-1 (-f(YP) - C21/h K1),  K3 = A^-1 (-f(YP) - C31/h K1 - C32/h K2),
//   Y' = max(Y + B1 K1 + B2 K2 + B3 K3, CONMIN)
//
// and its adjoint (lambda = dL/dY', nu_i = A^-T mu_i) is
//
//   lambda~ = lambda where Y' was not clipped, else 0
//   mu3 = B3 lambda~,                       nu3 = A^-T mu3
//   mu2 = B2 lambda~ - C32/h nu3,           nu2 = A^-T mu2
//   phi1 = -(nu3 + nu2),  t = J(YP)^T phi1
//   mu1 = B1 lambda~ - C31/h nu3 - C21/h nu2 + t,  nu1 = A^-T mu1
//   dL/dY = lambda~ + t + J(Y)^T (-nu1) - sum_i d/dY (nu_i . J(Y) K_i)
//   dL/dE += phi1 - nu1
//   dL/dlog k_r += w_r(phi1) R_r(YP) + w_r(-nu1) R_r(Y) - sum_i d/dlog k_r (nu_i . J(Y) K_i)
//
// The transposed solves reuse the LU factors that the step recomputes at Y.  The reverse
// sweep needs Y_n and h_n of every accepted step: a tape, recomputed per synchronisation
// step from the state checkpointed at its start, by the same kernel code as the forward,
// so the steps are identical.
//
// Kernels (one thread per cell, cells pulled from a work queue as in k_chem_ros3_queue):
//   k_adj_forward   one synchronisation step of every cell; records accepted steps per
//                   cell, or, given tape offsets, writes the tape
//   k_adj_reverse   reverse sweep of one synchronisation step over the tape
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "chem_kernels.cuh"

namespace adj {

constexpr int WPB = 8;
constexpr int THREADS = WPB * 32;
constexpr int TAPE_BLOCK = 4;

struct Args {
    long long ncell;
    double chemstep;               // minutes
    ros3::Tol tol;
    int max_iter;
    double* ws;                    // per-warp workspaces, ADJ_WS_ELEMS elements per lane
    const double* rki;             // [nrxns][ncell]
    const double* kmult;           // [nrxns] rate multipliers, or nullptr (1)
    const double* emis;            // [ischan][ncell] emission tendencies (ppm/min), or nullptr (0)
    const uint8_t* night;          // [ncell] 1: night reaction list
    const int* order;              // queue order, or nullptr for cell0, cell0 + 1, ...
    unsigned long long* head;      // queue head, zero before the launch
    long long queue_len;           // cells in the queue (0: ncell)
    long long cell0;               // first cell when order is nullptr
    long long tape_base;           // tape entry of tape_off == tape_base (a batch's first entry)
    // forward
    const double* y_in;            // [ischan][ncell] state at the start of the step
    double* y_out;                 // [ischan][ncell] state at its end, or nullptr
    int* nsteps;                   // [ncell] accepted steps: written by the recording forward,
                                   //         read by the tape forward (capacity) and the reverse
    int* status;                   // [ncell] forward status bits, or nullptr
    const long long* tape_off;     // [ncell] first tape entry of each cell (tape forward, reverse)
    double* tape_y;                // [entries][ischan] Y before each accepted step
    double* tape_h;                // [entries] its step size
    // tape recorded by the forward pass itself: linked blocks of TAPE_BLOCK accepted
    // steps per cell and synchronisation step, taken from a pool with one atomic each
    double* pool_y;                // [pool_blocks * TAPE_BLOCK][ischan]
    double* pool_h;                // [pool_blocks * TAPE_BLOCK]
    long long* pool_prev;          // [pool_blocks] previous block of the same cell and step, -1: none
    long long pool_blocks;
    unsigned long long* pool_head; // blocks taken so far
    unsigned int* pool_ovf;        // cells of this step whose tape did not fit (the step is re-run)
    long long* last_block;         // [ncell] last block of each cell in this step (-1: no accepted step)
    int* last_fill;                // [ncell] entries used in that block
    // reverse
    double* lam;                   // [ischan][ncell] dL/dY at the end of the step in, at its start out
    double* grad_logk;             // [nrxns] += dL/dlog kmult
    double* grad_emis;             // [ischan][ncell] += dL/dE, or nullptr
    unsigned long long* counters;  // [3] tape overruns, reversed cells, failed forward cells; or nullptr
};

template <class M>
__device__ __forceinline__ double* lane_ws(double* ws_all)
{
    const long long warp = (long long)blockIdx.x * WPB + (threadIdx.x >> 5);
    return ws_all + (size_t)warp * ((size_t)M::ADJ_WS_ELEMS * 32) + (threadIdx.x & 31);
}

// Rate constants and emission tendency of cell c into the workspace.
template <class M>
__device__ void load_cell_inputs(const Args& a, long long c, double* __restrict__ ws)
{
    for (int r = 0; r < M::NRXNS; ++r) {
        const double k = a.rki[(size_t)r * a.ncell + c];
        ws[(M::OFF_RKI + r) * 32] = a.kmult ? k * a.kmult[r] : k;
    }
    for (int i = 0; i < M::ISCHAN; ++i)
        ws[(M::ADJ_EMIS + i) * 32] = a.emis ? a.emis[(size_t)i * a.ncell + c] : 0.0;
}

// Next queue position for every idle lane (one atomic per warp); returns whether the
// queue is exhausted.  `cell` < 0 marks an idle lane.
__device__ __forceinline__ bool refill(const Args& a, long long& cell, bool& got)
{
    const int lane = threadIdx.x & 31;
    got = false;
    const unsigned long long qlen = (unsigned long long)(a.queue_len > 0 ? a.queue_len : a.ncell);
    const unsigned need = __ballot_sync(0xffffffffu, cell < 0);
    if (!need) return false;
    const int leader = __ffs(need) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(a.head, (unsigned long long)__popc(need));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (cell < 0) {
        const unsigned long long pos = base + __popc(need & ((1u << lane) - 1u));
        if (pos < qlen) {
            cell = a.order ? a.order[pos] : a.cell0 + (long long)pos;
            got = true;
        }
    }
    return __any_sync(0xffffffffu, base + __popc(need) >= qlen);
}

// One synchronisation step of every cell.  Without tape_off: records the accepted steps
// of each cell in nsteps.  With tape_off: stores Y and h of each accepted step at the
// cell's tape entries (at most nsteps[c] of them).
template <class M>
__global__ void __launch_bounds__(THREADS, 2) k_adj_forward(Args a)
{
    double* ws = lane_ws<M>(a.ws);
    const bool taping = a.tape_off != nullptr;
    const bool pooling = !taping && a.pool_y != nullptr;
    ros3::CellState s;
    long long cell = -1, base = 0, blk = -1;
    int cap = 0, written = -1, fill = TAPE_BLOCK;
    bool pool_ok = true;
    bool cnight = false, drained = false;
    unsigned long long overruns = 0, failed = 0;
    for (;;) {
        if (!drained) {
            bool got;
            drained = refill(a, cell, got);
            if (got) {
                for (int i = 0; i < M::ISCHAN; ++i) ws[(M::OFF_Y + i) * 32] = a.y_in[(size_t)i * a.ncell + cell];
                load_cell_inputs<M>(a, cell, ws);
                cnight = a.night[cell] != 0;
                ros3::start(s);
                if (taping) {
                    base = a.tape_off[cell] - a.tape_base;
                    cap = a.nsteps[cell];
                    written = -1;
                }
                if (pooling) {
                    blk = -1;
                    fill = TAPE_BLOCK;
                    written = -1;
                    pool_ok = true;
                }
            }
        }
        const bool busy = cell >= 0;
        // the block's warps run each step attempt together (barriers between its phases)
        if (!__syncthreads_or(busy)) break;
        const bool night = __syncthreads_and(!busy || cnight);
        double h = 0.0;
        const int nacc = s.st.nsteps;
        if (busy && taping) {
            // Y changes only when a step is accepted: copy it once per accepted step
            h = s.dt;
            if (s.tnow + h > a.chemstep) h = a.chemstep - s.tnow;
            if (written != nacc && nacc < cap) {
                double* t = a.tape_y + (size_t)(base + nacc) * M::ISCHAN;
                for (int i = 0; i < M::ISCHAN; ++i) t[i] = ws[(M::OFF_Y + i) * 32];
                written = nacc;
            }
        }
        if (busy && pooling && pool_ok) {
            h = s.dt;
            if (s.tnow + h > a.chemstep) h = a.chemstep - s.tnow;
            if (written != nacc) {   // a slot for this accepted-step candidate
                if (fill == TAPE_BLOCK) {
                    const unsigned long long nb = atomicAdd(a.pool_head, 1ull);
                    if ((long long)nb < a.pool_blocks) {
                        a.pool_prev[nb] = blk;
                        blk = (long long)nb;
                        fill = 0;
                    } else {
                        pool_ok = false;
                    }
                }
                if (pool_ok) {
                    double* t = a.pool_y + (size_t)(blk * TAPE_BLOCK + fill) * M::ISCHAN;
                    for (int i = 0; i < M::ISCHAN; ++i) t[i] = ws[(M::OFF_Y + i) * 32];
                    written = nacc;
                }
            }
        }
        ros3::attempt_phased<M, 1, true>(ws, s, a.chemstep, a.tol, night, a.max_iter, busy);
        if (busy) {
            if (taping && s.st.nsteps != nacc) {
                if (nacc < cap) a.tape_h[base + nacc] = h;
                else overruns++;
            }
            if (pooling && pool_ok && s.st.nsteps != nacc) {
                a.pool_h[blk * TAPE_BLOCK + fill] = h;
                fill++;
            }
            if (ros3::finished(s, a.chemstep)) {
                if (a.y_out)
                    for (int i = 0; i < M::ISCHAN; ++i) a.y_out[(size_t)i * a.ncell + cell] = ws[(M::OFF_Y + i) * 32];
                if (!taping) a.nsteps[cell] = s.st.nsteps;
                if (pooling) {
                    if (pool_ok) {
                        a.last_block[cell] = blk;
                        a.last_fill[cell] = fill;
                    } else {
                        atomicAdd(a.pool_ovf, 1u);
                    }
                }
                if (a.status) a.status[cell] = s.st.status;
                failed += s.st.status != ros3::ST_OK;
                cell = -1;
            }
        }
    }
    if (a.counters && overruns) atomicAdd(&a.counters[0], overruns);
    if (a.counters && failed) atomicAdd(&a.counters[2], failed);
}

// Adjoint of one accepted step at Y = ws[OFF_Y] with step size h; updates ADJ_LAM and
// accumulates ADJ_GE and ADJ_GK.  Every thread of the block calls it; lanes with go ==
// false do no work; the block passes a barrier between the phases so that its warps
// walk the (large) generated code together.
template <class M>
__device__ void reverse_step(double* __restrict__ ws, double h, bool night, bool go)
{
    using namespace ros3;
    const double dtinv = go ? 1.0 / h : 0.0;
    const double gdtinv = dtinv * RGAM;
    const double x21 = C21 * dtinv, x31 = C31 * dtinv, x32 = C32 * dtinv;
    // recompute the stages exactly as the forward step did
    if (go) {
        if (night) M::feval_1(ws, M::OFF_Y, M::OFF_F0); else M::feval_0(ws, M::OFF_Y, M::OFF_F0);
        add_emis<M>(ws, M::OFF_F0);
        if (night) M::explic_1(ws); else M::explic_0(ws);
    }
    __syncthreads();
    if (go) {
        if (night) M::jacdecomp_1(ws, gdtinv); else M::jacdecomp_0(ws, gdtinv);
        for (int n = 0; n < M::ISCHAN; ++n) ws[(M::OFF_K1 + n) * 32] = -ws[(M::OFF_F0 + n) * 32];
    }
    __syncthreads();
    solve_phase<M, 1>(ws, M::OFF_K1, night, go);
    if (go) {
        for (int n = 0; n < M::ISCHAN; ++n)
            ws[(M::OFF_YP + n) * 32] = ws[(M::OFF_Y + n) * 32] + ws[(M::OFF_K1 + n) * 32];
        if (night) M::feval_1(ws, M::OFF_YP, M::OFF_YDOT); else M::feval_0(ws, M::OFF_YP, M::OFF_YDOT);
        add_emis<M>(ws, M::OFF_YDOT);
        for (int n = 0; n < M::ISCHAN; ++n)
            ws[(M::OFF_K2 + n) * 32] = fma(-x21, ws[(M::OFF_K1 + n) * 32], -ws[(M::OFF_YDOT + n) * 32]);
    }
    __syncthreads();
    solve_phase<M, 1>(ws, M::OFF_K2, night, go);
    if (go) {
        for (int n = 0; n < M::ISCHAN; ++n) {
            const double t = fma(-x31, ws[(M::OFF_K1 + n) * 32], -ws[(M::OFF_YDOT + n) * 32]);
            ws[(M::OFF_K3 + n) * 32] = fma(-x32, ws[(M::OFF_K2 + n) * 32], t);
        }
    }
    solve_phase<M, 1>(ws, M::OFF_K3, night, go);
    if (go) {   // clipped components of Y' pass no gradient
        for (int n = 0; n < M::ISCHAN; ++n) {
            double yn = fma(B1, ws[(M::OFF_K1 + n) * 32], ws[(M::OFF_Y + n) * 32]);
            yn = fma(B2, ws[(M::OFF_K2 + n) * 32], yn);
            yn = fma(B3, ws[(M::OFF_K3 + n) * 32], yn);
            if (!(yn > CONMIN)) ws[(M::ADJ_LAM + n) * 32] = 0.0;
            ws[(M::ADJ_MU3 + n) * 32] = B3 * ws[(M::ADJ_LAM + n) * 32];
        }
        if (night) M::solve_t_1(ws, M::ADJ_MU3); else M::solve_t_0(ws, M::ADJ_MU3);
        for (int n = 0; n < M::ISCHAN; ++n)
            ws[(M::ADJ_MU2 + n) * 32] = fma(-x32, ws[(M::ADJ_MU3 + n) * 32], B2 * ws[(M::ADJ_LAM + n) * 32]);
    }
    __syncthreads();
    if (go) {
        if (night) M::solve_t_1(ws, M::ADJ_MU2); else M::solve_t_0(ws, M::ADJ_MU2);
        for (int n = 0; n < M::ISCHAN; ++n) {
            const double phi = -ws[(M::ADJ_MU3 + n) * 32] - ws[(M::ADJ_MU2 + n) * 32];
            ws[(M::ADJ_PHI + n) * 32] = phi;
            ws[(M::ADJ_GE + n) * 32] = ws[(M::ADJ_GE + n) * 32] + phi;
            ws[(M::ADJ_TMP + n) * 32] = 0.0;
        }
        if (night) M::adj_jtv_1(ws, M::OFF_YP, M::ADJ_PHI, M::ADJ_TMP);
        else M::adj_jtv_0(ws, M::OFF_YP, M::ADJ_PHI, M::ADJ_TMP);
        for (int n = 0; n < M::ISCHAN; ++n) {
            const double lam = ws[(M::ADJ_LAM + n) * 32];
            const double t = ws[(M::ADJ_TMP + n) * 32];
            const double mu = fma(-x21, ws[(M::ADJ_MU2 + n) * 32], fma(-x31, ws[(M::ADJ_MU3 + n) * 32], B1 * lam));
            ws[(M::ADJ_MU1 + n) * 32] = mu + t;
            ws[(M::ADJ_LAM + n) * 32] = lam + t;
        }
    }
    __syncthreads();
    if (go) {
        if (night) M::solve_t_1(ws, M::ADJ_MU1); else M::solve_t_0(ws, M::ADJ_MU1);
        for (int n = 0; n < M::ISCHAN; ++n) {
            const double phi = -ws[(M::ADJ_MU1 + n) * 32];
            ws[(M::ADJ_PHI + n) * 32] = phi;
            ws[(M::ADJ_GE + n) * 32] = ws[(M::ADJ_GE + n) * 32] + phi;
        }
        if (night) M::adj_jtv_1(ws, M::OFF_Y, M::ADJ_PHI, M::ADJ_LAM);
        else M::adj_jtv_0(ws, M::OFF_Y, M::ADJ_PHI, M::ADJ_LAM);
        if (night) M::adj_hess3_1(ws); else M::adj_hess3_0(ws);
    }
    __syncthreads();
}

// Reverse sweep of one synchronisation step: each cell walks its tape entries backwards.
// Cells are pulled from the queue (ordered by accepted steps, most first).
template <class M>
__global__ void __launch_bounds__(THREADS, 2) k_adj_reverse(Args a)
{
    double* ws = lane_ws<M>(a.ws);
    for (int r = 0; r < M::NRXNS; ++r) ws[(M::ADJ_GK + r) * 32] = 0.0;
    long long cell = -1, base = 0, blk = -1;
    int left = 0, fill = 0;
    const bool pooled = a.last_block != nullptr;
    bool cnight = false, drained = false;
    unsigned long long ncells = 0;
    for (;;) {
        if (!drained) {
            bool got;
            drained = refill(a, cell, got);
            if (got) {
                load_cell_inputs<M>(a, cell, ws);
                for (int i = 0; i < M::ISCHAN; ++i) {
                    ws[(M::ADJ_LAM + i) * 32] = a.lam[(size_t)i * a.ncell + cell];
                    ws[(M::ADJ_GE + i) * 32] = 0.0;
                }
                cnight = a.night[cell] != 0;
                left = a.nsteps[cell];
                if (pooled) {
                    blk = a.last_block[cell];
                    fill = a.last_fill[cell];
                } else {
                    base = a.tape_off[cell] - a.tape_base;
                }
            }
        }
        const bool busy = cell >= 0;
        if (!__syncthreads_or(busy)) break;
        const bool work = busy && left > 0;
        const bool night = __syncthreads_and(!work || cnight);
        double hstep = 0.0;
        if (work) {
            --left;
            size_t e;
            if (pooled) {
                if (fill == 0) {
                    blk = a.pool_prev[blk];
                    fill = TAPE_BLOCK;
                }
                --fill;
                e = (size_t)(blk * TAPE_BLOCK + fill);
            } else {
                e = (size_t)(base + left);
            }
            const double* t = (pooled ? a.pool_y : a.tape_y) + e * M::ISCHAN;
            for (int i = 0; i < M::ISCHAN; ++i) ws[(M::OFF_Y + i) * 32] = t[i];
            hstep = (pooled ? a.pool_h : a.tape_h)[e];
        }
        reverse_step<M>(ws, hstep, night, work);
        if (busy && left == 0) {
            for (int i = 0; i < M::ISCHAN; ++i) a.lam[(size_t)i * a.ncell + cell] = ws[(M::ADJ_LAM + i) * 32];
            if (a.grad_emis)
                for (int i = 0; i < M::ISCHAN; ++i) {
                    double* g = a.grad_emis + (size_t)i * a.ncell + cell;
                    *g = *g + ws[(M::ADJ_GE + i) * 32];
                }
            ncells++;
            cell = -1;
        }
    }
    // per-reaction gradients: warp sums, one atomic per warp and reaction
    for (int r = 0; r < M::NRXNS; ++r) {
        double v = ws[(M::ADJ_GK + r) * 32];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(&a.grad_logk[r], v);
    }
    if (a.counters && ncells) atomicAdd(&a.counters[1], ncells);
}

// Exclusive prefix sums of per-cell step counts into 64-bit tape offsets.
constexpr int SCAN_TILE = 2048;

static __global__ void k_scan_tiles(const int* __restrict__ v, long long n, long long* __restrict__ tile_sum)
{
    __shared__ long long part[256];
    const long long t0 = (long long)blockIdx.x * SCAN_TILE;
    long long s = 0;
    for (int i = threadIdx.x; i < SCAN_TILE; i += blockDim.x)
        if (t0 + i < n) s += v[t0 + i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) part[threadIdx.x] += part[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = part[0];
}

// one block: exclusive scan of the tile sums in place; total to *total
static __global__ void k_scan_tile_sums(long long* __restrict__ tile_sum, int ntiles, long long* __restrict__ total)
{
    if (threadIdx.x == 0) {
        long long acc = 0;
        for (int i = 0; i < ntiles; ++i) {
            const long long x = tile_sum[i];
            tile_sum[i] = acc;
            acc += x;
        }
        *total = acc;
    }
}

static __global__ void k_scan_apply(const int* __restrict__ v, long long n, const long long* __restrict__ tile_base,
                             long long* __restrict__ out)
{
    // 256 threads, each a contiguous run of SCAN_TILE / 256 elements
    constexpr int RUN = SCAN_TILE / 256;
    __shared__ long long part[256];
    const long long t0 = (long long)blockIdx.x * SCAN_TILE + (long long)threadIdx.x * RUN;
    long long s = 0;
    for (int i = 0; i < RUN; ++i)
        if (t0 + i < n) s += v[t0 + i];
    part[threadIdx.x] = s;
    __syncthreads();
    // inclusive Hillis-Steele scan of the 256 run sums
    for (int o = 1; o < 256; o <<= 1) {
        const long long x = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    long long acc = tile_base[blockIdx.x] + part[threadIdx.x] - s;
    for (int i = 0; i < RUN; ++i)
        if (t0 + i < n) {
            out[t0 + i] = acc;
            acc += v[t0 + i];
        }
}

}  // namespace adj
