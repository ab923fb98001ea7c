// Grid-level kernels of the chemistry operator (one thread per grid cell).
//
// k_chem_ros3   restates one CHEM call of CCTM/src/gas/ros3/rbdriver.F for BLKSIZE = 1:
//               gather met, photolysis and heterogeneous rates and concentrations of a
//               cell with the reference's unit conversions and REAL(4) arithmetic
//               (rbdriver.F:460-511), rate constants (CALC_RCONST), ROS3 integration
//               (rbsolver.F) and write-back with the REAL(4) cast (rbdriver.F:577-595).
// k_ros3_solve  solver-level entry: Y (new species order) and RKI given, integrate.
// k_rconst      rate constants only (CALC_RCONST), for parity checks.
//
// CGRID layout is the reference's CONC(NCOLS, NROWS, NLAYS, NSPCSD) in Fortran order,
// i.e. species planes with the cell index col + ncols*(row + nrows*lay) fastest; all
// grid arrays are therefore already structure-of-arrays over cells.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "ros3.cuh"

namespace chem {

// Physical constants of CCTM/src/ICL/fixed/const/CONST.EXT evaluated in REAL(4), as the
// reference's PARAMETERs (rbdriver.F:110-114).
constexpr float STDATMPA = 101325.0f;
constexpr float MWAIR = 28.9628f;
constexpr float MWWAT = 18.0153f;
constexpr float PA2ATM = 1.0f / STDATMPA;
constexpr float MAOMV = MWAIR / MWWAT;
constexpr float CONCOFM = 1.0e+06f;
constexpr float QV_TO_PPM = CONCOFM * MAOMV;
constexpr float CONCMIN_F = 1.0e-30f;

constexpr int WARPS_PER_BLOCK = 8;
constexpr int THREADS_PER_BLOCK = WARPS_PER_BLOCK * 32;

struct GridArgs {
    float* cgrid;                  // [nspcsd][ncell]
    long long ncell;               // ncols * nrows * nlays
    int ncolrow;                   // ncols * nrows
    int nspcsd;
    const int* cgrid_index;        // [nspec] mechanism species (old order) -> CGRID slot, 0-based
    const int* convert;            // [nspec] 1 if the species is converted (aerosol units)
    const float* fwd_conv;         // [nspec] FORWARD_CONV (REAL(4))
    const double* rev_conv;        // [nspec] REVERSE_CONV
    const float* ta;               // [ncell] K
    const float* qv;               // [ncell] kg/kg
    const float* dens;             // [ncell] kg/m3
    const float* pres;             // [ncell] Pa
    const float* seaice;           // [ncolrow] fraction
    const float* ocean_szone;      // [ncolrow] OCEAN + SZONE fraction
    const float* rj;               // [nphotab][ncell] 1/min
    const double* khet;            // [ncell][nhet] KHETERO(NHET, C, R, L)
    double chemstep;               // minutes
    ros3::Tol tol;
    double* ws;                    // per-warp workspaces
    int max_iter;
    int* cell_status;              // [ncell] or nullptr
    int* cell_steps;               // [ncell] accepted + rejected step attempts, or nullptr
    unsigned long long* counters;  // [5]: accepted steps, rejected steps, failed cells, sunlit cells,
                                   //      step attempts of sunlit cells
    int use_night;                 // 1: all-dark warps use the night pattern; 0: day pattern always
    double* yave;                  // [ischan][ncell] time-averaged Y of the call (DDM-3D), or nullptr
    const double* rki_all;         // [nrxns][ncell] rate constants of the call's cells from k_rconst_pass, or
                                   // nullptr (gather_cell evaluates CALC_RCONST itself)
    const uint8_t* sun_all;        // [ncell] sunlight flags of the same pass
};

// DDM-3D: the cell's time-averaged concentrations (rbsolver.F:592-595) to a.yave
template <class M>
__device__ __forceinline__ void store_yave(const GridArgs& a, long long c, const double* __restrict__ ws)
{
    for (int i = 0; i < M::ISCHAN; ++i) a.yave[(size_t)i * a.ncell + c] = ws[(M::OFF_YAVE + i) * 32] / a.chemstep;
}

template <class M>
__device__ __forceinline__ double* warp_ws(double* ws_all, long long warp_global)
{
    return ws_all + (size_t)warp_global * ((size_t)M::WS_ELEMS * 32) + (threadIdx.x & 31);
}

// Gather one cell into ws (Y, RKI); returns the cell's sunlight flag.  floor64: the
// SMVGEAR driver's REAL(8) concentration floor (grdriver.F:419-422) instead of ROS3's
// REAL(4) one.
template <class M>
__device__ bool gather_cell(const GridArgs& a, long long c, double* __restrict__ ws, bool floor64 = false)
{
    const float taf = a.ta[c];
    const float densf = a.dens[c];
    const float svol = __fdiv_rn(1.0f, densf);
    const double temp = (double)taf;
    const double press = (double)__fmul_rn(PA2ATM, a.pres[c]);
    const double h2o = (double)fmaxf(__fmul_rn(QV_TO_PPM, a.qv[c]), 0.0f);
    const int col = (int)(c % a.ncolrow);
    const double seawater = (double)fmaxf(0.0f, __fsub_rn(a.ocean_szone[col], a.seaice[col]));
    for (int s = 0; s < M::ISCHAN; ++s) {
        const float conc = a.cgrid[(size_t)a.cgrid_index[s] * a.ncell + c];
        const float v = a.convert[s] ? __fmul_rn(__fmul_rn(a.fwd_conv[s], svol), conc) : conc;
        ws[(M::OFF_Y + M::iold2new(s)) * 32] = floor64 ? fmax((double)v, 1.0e-30) : (double)fmaxf(v, CONCMIN_F);
    }
    double rjv[M::NPHOTAB];
    bool sun = false;
#pragma unroll
    for (int k = 0; k < M::NPHOTAB; ++k) {
        rjv[k] = (double)a.rj[(size_t)k * a.ncell + c];
        sun = sun || (rjv[k] > 0.0);
    }
    double hetv[M::NHETERO];
#pragma unroll
    for (int k = 0; k < M::NHETERO; ++k) hetv[k] = a.khet[(size_t)c * M::NHETERO + k];
    M::rconst(ws, temp, press, h2o, seawater, sun ? 1 : 0, rjv, hetv);
    return sun;
}

// Gather one cell into ws: concentrations as gather_cell, and the rate constants from the
// call's rate-constant pass when there is one (the same numbers, computed by whole warps
// over consecutive cells instead of by the few lanes a work queue refills at a time).
template <class M>
__device__ bool gather_cell_pass(const GridArgs& a, long long c, double* __restrict__ ws)
{
    if (!a.rki_all) return gather_cell<M>(a, c, ws);
    const float densf = a.dens[c];
    const float svol = __fdiv_rn(1.0f, densf);
    for (int s = 0; s < M::ISCHAN; ++s) {
        const float conc = a.cgrid[(size_t)a.cgrid_index[s] * a.ncell + c];
        const float v = a.convert[s] ? __fmul_rn(__fmul_rn(a.fwd_conv[s], svol), conc) : conc;
        ws[(M::OFF_Y + M::iold2new(s)) * 32] = (double)fmaxf(v, CONCMIN_F);
    }
    for (int r = 0; r < M::NRXNS; ++r) ws[(M::OFF_RKI + r) * 32] = a.rki_all[(size_t)r * a.ncell + c];
    return a.sun_all[c] != 0;
}

template <class M>
__device__ void scatter_cell(const GridArgs& a, long long c, const double* __restrict__ ws)
{
    const double densd = (double)a.dens[c];
    for (int i = 0; i < M::ISCHAN; ++i) {
        const int old = M::inew2old(i);
        const double y = ws[(M::OFF_Y + i) * 32];
        float v;
        if (a.convert[old]) v = (float)((a.rev_conv[old] * densd) * y);
        else v = (float)y;
        a.cgrid[(size_t)a.cgrid_index[old] * a.ncell + c] = v;
    }
}

// One CHEM call, cells distributed statically: warp w takes cells [32w, 32w+32) then
// strides by the grid's warp count.  Each lane integrates its own cell.  Same occupancy
// target as the work-queue kernel (CHEM_QUEUE_WARPS_PER_SM), so that the two schedules
// differ only in how cells reach the lanes.
#ifndef CHEM_QUEUE_WARPS_PER_SM
#define CHEM_QUEUE_WARPS_PER_SM 12
#endif
template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK,
                                  CHEM_QUEUE_WARPS_PER_SM / WARPS_PER_BLOCK > 0 ? CHEM_QUEUE_WARPS_PER_SM / WARPS_PER_BLOCK : 1)
    k_chem_ros3(GridArgs a)
{
    const long long nwarps = (long long)gridDim.x * WARPS_PER_BLOCK;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    unsigned long long acc_steps = 0, rej_steps = 0, failed = 0, sunlit = 0, sun_att = 0;
    for (long long base = warp * 32; base < a.ncell; base += nwarps * 32) {
        const long long c = base + (threadIdx.x & 31);
        const bool active = c < a.ncell;
        bool sun = false;
        if (active) sun = gather_cell<M>(a, c, ws);
        const bool night = a.use_night && __all_sync(0xffffffffu, !sun);
        if (active) {
            ros3::CellStats st = ros3::integrate<M>(ws, a.chemstep, a.tol, night, a.max_iter, a.yave != nullptr);
            scatter_cell<M>(a, c, ws);
            if (a.yave) store_yave<M>(a, c, ws);
            acc_steps += st.nsteps;
            rej_steps += st.nfails;
            failed += st.status != ros3::ST_OK;
            sunlit += sun;
            if (sun) sun_att += st.nsteps + st.nfails;
            if (a.cell_status) a.cell_status[c] = st.status;
            if (a.cell_steps) a.cell_steps[c] = st.nsteps + st.nfails;
        }
    }
    if (a.counters) {
        // warp-reduce then one atomic per warp
        for (int o = 16; o > 0; o >>= 1) {
            acc_steps += __shfl_down_sync(0xffffffffu, acc_steps, o);
            rej_steps += __shfl_down_sync(0xffffffffu, rej_steps, o);
            failed += __shfl_down_sync(0xffffffffu, failed, o);
            sunlit += __shfl_down_sync(0xffffffffu, sunlit, o);
            sun_att += __shfl_down_sync(0xffffffffu, sun_att, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&a.counters[0], acc_steps);
            atomicAdd(&a.counters[1], rej_steps);
            atomicAdd(&a.counters[2], failed);
            atomicAdd(&a.counters[3], sunlit);
            atomicAdd(&a.counters[4], sun_att);
        }
    }
}

struct SolveArgs {
    double* y;                 // [ischan][ncell] new species order, updated in place
    const double* rki;         // [nrxns][ncell]
    const uint8_t* night;      // [ncell] 1 = use the night reaction list
    long long ncell;
    double chemstep;
    ros3::Tol tol;
    double* ws;
    int max_iter;
    int* cell_status;          // [ncell] or nullptr
    int* cell_nsteps;          // [ncell] accepted steps or nullptr
    int* cell_nfails;          // [ncell] rejected steps or nullptr
};

// Solver-level entry: the warp uses the night pattern only if all its cells are night cells
// (identical numbers either way).
template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK, 1) k_ros3_solve(SolveArgs a)
{
    const long long nwarps = (long long)gridDim.x * WARPS_PER_BLOCK;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    for (long long base = warp * 32; base < a.ncell; base += nwarps * 32) {
        const long long c = base + (threadIdx.x & 31);
        const bool active = c < a.ncell;
        bool nt = true;
        if (active) {
            for (int i = 0; i < M::ISCHAN; ++i) ws[(M::OFF_Y + i) * 32] = a.y[(size_t)i * a.ncell + c];
            for (int r = 0; r < M::NRXNS; ++r) ws[(M::OFF_RKI + r) * 32] = a.rki[(size_t)r * a.ncell + c];
            nt = a.night[c] != 0;
        }
        const bool night = __all_sync(0xffffffffu, nt);
        if (active) {
            ros3::CellStats st = ros3::integrate<M>(ws, a.chemstep, a.tol, night, a.max_iter);
            for (int i = 0; i < M::ISCHAN; ++i) a.y[(size_t)i * a.ncell + c] = ws[(M::OFF_Y + i) * 32];
            if (a.cell_status) a.cell_status[c] = st.status;
            if (a.cell_nsteps) a.cell_nsteps[c] = st.nsteps;
            if (a.cell_nfails) a.cell_nfails[c] = st.nfails;
        }
    }
}

// The rate-constant pass of a CHEM call: CALC_RCONST of cells [c0, c1) by whole warps in grid
// order into rki[nrxns][ncell] and sunlit[ncell], for gather_cell_pass.
template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK, 1) k_rconst_pass(GridArgs a, long long c0, long long c1,
                                                                      double* rki, uint8_t* sunlit)
{
    const long long nwarps = (long long)gridDim.x * WARPS_PER_BLOCK;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    for (long long base = c0 + warp * 32; base < c1; base += nwarps * 32) {
        const long long c = base + (threadIdx.x & 31);
        if (c < c1) {
            const bool sun = gather_cell<M>(a, c, ws);
            for (int r = 0; r < M::NRXNS; ++r) rki[(size_t)r * a.ncell + c] = ws[(M::OFF_RKI + r) * 32];
            sunlit[c] = sun ? 1 : 0;
        }
    }
}

// Rate constants of every cell into rki[nrxns][ncell] (gathered exactly as k_chem_ros3 does).
template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK, 1) k_rconst(GridArgs a, double* rki, uint8_t* sunlit)
{
    const long long nwarps = (long long)gridDim.x * WARPS_PER_BLOCK;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    for (long long base = warp * 32; base < a.ncell; base += nwarps * 32) {
        const long long c = base + (threadIdx.x & 31);
        if (c < a.ncell) {
            const bool sun = gather_cell<M>(a, c, ws);
            for (int r = 0; r < M::NRXNS; ++r) rki[(size_t)r * a.ncell + c] = ws[(M::OFF_RKI + r) * 32];
            if (sunlit) sunlit[c] = sun ? 1 : 0;
        }
    }
}

}  // namespace chem
