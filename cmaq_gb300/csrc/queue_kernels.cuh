// Batched ("queue") scheduling of the per-cell ROS3 integration.
//
// The reference balances stiffness by a first pass that estimates each cell's
// stiffness, heap-sorts the cells and re-blocks them (rbdriver.F:430-434, 683-724;
// Jacobson 1994).  Here a persistent grid pulls cells from a device work queue: a lane
// that finishes its cell takes the next one at once, so a warp is no longer held by
// its slowest cell.  The queue is ordered by each cell's step attempts in the previous
// call, most first (a counting sort over step-count bins), so long cells start early
// and the tail is short.  Every cell is integrated exactly as in k_chem_ros3; the
// schedule changes no result bit.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "chem_kernels.cuh"

namespace chem {

constexpr int QUEUE_BINS = 256;

struct QueueArgs {
    const int* order;                 // queue order of cells relative to cell0, or nullptr for 0, 1, ...
    unsigned long long* head;         // next queue position (zeroed before the launch)
    long long qlen;                   // cells in the queue (0: the whole grid)
    long long cell0;                  // first cell of the range the queue covers
    const unsigned long long* qlen_dev;   // if set: the queue length, written by an earlier kernel
};

__device__ __forceinline__ unsigned long long queue_len(const QueueArgs& q, long long ncell)
{
    if (q.qlen_dev) return *q.qlen_dev;
    return (unsigned long long)(q.qlen > 0 ? q.qlen : ncell);
}

// SYNC > 0 ("lock-step"): the block's warps run each step attempt together, with
// barriers between its phases (SYNC = 1) or also between the generated chunks (SYNC = 2);
// the block leaves the loop only when none of its warps holds a cell.  WPB = warps per
// block.
// Launch bounds: CHEM_QUEUE_WARPS_PER_SM resident warps per SM (chem_kernels.cuh; the
// generated functions the kernel calls must be built for that register budget).
template <class M, int SYNC, int WPB>
__global__ void __launch_bounds__(WPB * 32, CHEM_QUEUE_WARPS_PER_SM / WPB > 0 ? CHEM_QUEUE_WARPS_PER_SM / WPB : 1)
    k_chem_ros3_queue(GridArgs a, QueueArgs q)
{
    constexpr bool LOCKSTEP = SYNC > 0;
    const int lane = threadIdx.x & 31;
    const long long warp = (long long)blockIdx.x * WPB + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    ros3::CellState s;
    s.tmark = clock64();
    long long cell = -1;
    bool sun = false;
    bool drained = false;
    unsigned long long acc_steps = 0, rej_steps = 0, failed = 0, sunlit = 0, sun_att = 0;
    for (;;) {
        // refill idle lanes with one atomic per warp
        if (!drained) {
            const unsigned need = __ballot_sync(0xffffffffu, cell < 0);
            if (need) {
                const int leader = __ffs(need) - 1;
                unsigned long long base = 0;
                if (lane == leader) base = atomicAdd(q.head, (unsigned long long)__popc(need));
                base = __shfl_sync(0xffffffffu, base, leader);
                if (cell < 0) {
                    const unsigned long long pos = base + __popc(need & ((1u << lane) - 1u));
                    if (pos < queue_len(q, a.ncell)) {
                        cell = q.cell0 + (q.order ? q.order[pos] : (long long)pos);
                        sun = gather_cell_pass<M>(a, cell, ws);
                        ros3::start(s);
                        if (a.yave) {
                            s.yave = true;
                            for (int i = 0; i < M::ISCHAN; ++i) ws[(M::OFF_YAVE + i) * 32] = 0.0;
                        }
                    }
                }
                drained = __any_sync(0xffffffffu, base + __popc(need) >= queue_len(q, a.ncell));
            }
        }
        const bool busy = cell >= 0;
        bool night;
        if (LOCKSTEP) {
            if (!__syncthreads_or(busy)) break;
            night = __syncthreads_and(!busy || !sun) && a.use_night;
            CHEM_PHASE_MARK(s, 6);
        } else {
            if (!__any_sync(0xffffffffu, busy)) break;
            night = __all_sync(0xffffffffu, !busy || !sun) && a.use_night;
        }
        ros3::attempt_phased<M, SYNC>(ws, s, a.chemstep, a.tol, night, a.max_iter, busy);
        if (busy) {
            if (ros3::finished(s, a.chemstep)) {
                scatter_cell<M>(a, cell, ws);
                if (a.yave) store_yave<M>(a, cell, ws);
                acc_steps += s.st.nsteps;
                rej_steps += s.st.nfails;
                failed += s.st.status != ros3::ST_OK;
                sunlit += sun;
                if (sun) sun_att += s.st.nsteps + s.st.nfails;
                if (a.cell_status) a.cell_status[cell] = s.st.status;
                if (a.cell_steps) a.cell_steps[cell] = s.st.nsteps + s.st.nfails;
                cell = -1;
            }
        }
    }
    if (a.counters) {
        for (int o = 16; o > 0; o >>= 1) {
            acc_steps += __shfl_down_sync(0xffffffffu, acc_steps, o);
            rej_steps += __shfl_down_sync(0xffffffffu, rej_steps, o);
            failed += __shfl_down_sync(0xffffffffu, failed, o);
            sunlit += __shfl_down_sync(0xffffffffu, sunlit, o);
            sun_att += __shfl_down_sync(0xffffffffu, sun_att, o);
        }
        if (lane == 0) {
            atomicAdd(&a.counters[0], acc_steps);
            atomicAdd(&a.counters[1], rej_steps);
            atomicAdd(&a.counters[2], failed);
            atomicAdd(&a.counters[3], sunlit);
            atomicAdd(&a.counters[4], sun_att);
        }
    }
}

// ---- queue ordering: counting sort of cells by previous step attempts, descending

__device__ __forceinline__ int queue_bin(int steps)
{
    const int b = steps < 0 ? 0 : (steps >= QUEUE_BINS ? QUEUE_BINS - 1 : steps);
    return QUEUE_BINS - 1 - b;   // bin 0 = most steps
}

static __global__ void k_queue_hist(const int* __restrict__ steps, long long ncell, unsigned int* __restrict__ hist)
{
    __shared__ unsigned int h[QUEUE_BINS];
    for (int i = threadIdx.x; i < QUEUE_BINS; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x)
        atomicAdd(&h[queue_bin(steps[c])], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < QUEUE_BINS; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// exclusive scan of the histogram into per-bin write cursors (one block of QUEUE_BINS threads)
static __global__ void k_queue_scan(const unsigned int* __restrict__ hist, unsigned long long* __restrict__ cursor)
{
    __shared__ unsigned long long v[QUEUE_BINS];
    const int t = threadIdx.x;
    v[t] = hist[t];
    __syncthreads();
    for (int o = 1; o < QUEUE_BINS; o <<= 1) {
        const unsigned long long x = t >= o ? v[t - o] : 0ull;
        __syncthreads();
        v[t] += x;
        __syncthreads();
    }
    cursor[t] = v[t] - hist[t];
}

static __global__ void k_queue_scatter(const int* __restrict__ steps, long long ncell,
                                unsigned long long* __restrict__ cursor, int* __restrict__ order)
{
    __shared__ unsigned int cnt[QUEUE_BINS];
    __shared__ unsigned long long base[QUEUE_BINS];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c0 = (long long)blockIdx.x * blockDim.x; c0 < ncell; c0 += stride) {
        for (int i = threadIdx.x; i < QUEUE_BINS; i += blockDim.x) cnt[i] = 0;
        __syncthreads();
        const long long c = c0 + threadIdx.x;
        int b = 0;
        unsigned int rank = 0;
        if (c < ncell) {
            b = queue_bin(steps[c]);
            rank = atomicAdd(&cnt[b], 1u);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < QUEUE_BINS; i += blockDim.x)
            base[i] = cnt[i] ? atomicAdd(&cursor[i], (unsigned long long)cnt[i]) : 0ull;
        __syncthreads();
        // base + rank < ncell when the counts are the ones k_queue_hist saw; the check keeps a
        // count array changed between the two kernels from writing past the order array
        if (c < ncell && base[b] + rank < (unsigned long long)ncell) order[base[b] + rank] = (int)c;
        __syncthreads();
    }
}

}  // namespace chem
