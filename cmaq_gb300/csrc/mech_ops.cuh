// Per-mechanism kernel table: each mechanism's translation unit instantiates the grid
// kernels for its generated device code and exports one MechOps object.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "chem_kernels.cuh"
#include "queue_kernels.cuh"

struct MechOps {
    const char* name;
    int nspec, nrxns, ischan, nphotab, nhetero, ws_elems, iarray_day, iarray_night;
    double flops_step_day, flops_step_night;
    const int* cgrid_index;   // [nspec] 0-based default CGRID slots
    const int* convert;       // [nspec]
    const double* molwt;      // [nspec]
    const int* inew2old;      // [nspec]
    const int* iold2new;      // [nspec]
    cudaError_t (*chem_static)(const chem::GridArgs&, int nblocks, cudaStream_t);
    cudaError_t (*chem_queue)(const chem::GridArgs&, const chem::QueueArgs&, bool lockstep, int nblocks,
                              cudaStream_t);
    cudaError_t (*solve)(const chem::SolveArgs&, int nblocks, cudaStream_t);
    cudaError_t (*rconst)(const chem::GridArgs&, double* rki, uint8_t* sunlit, int nblocks, cudaStream_t);
    cudaError_t (*occupancy)(int* blocks_per_sm);
};

#define DEFINE_MECH_OPS(NS, SYMBOL)                                                                 \
    namespace {                                                                                     \
    using T_ = NS::Traits;                                                                          \
    cudaError_t chem_static_(const chem::GridArgs& a, int nb, cudaStream_t s)                       \
    {                                                                                               \
        chem::k_chem_ros3<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a);                            \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t chem_queue_(const chem::GridArgs& a, const chem::QueueArgs& q, bool lockstep, int nb,   \
                            cudaStream_t s)                                                         \
    {                                                                                               \
        if (lockstep)                                                                               \
            chem::k_chem_ros3_queue<T_, true><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, q);         \
        else                                                                                        \
            chem::k_chem_ros3_queue<T_, false><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, q);        \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t solve_(const chem::SolveArgs& a, int nb, cudaStream_t s)                            \
    {                                                                                               \
        chem::k_ros3_solve<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a);                           \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t rconst_(const chem::GridArgs& a, double* rki, uint8_t* sun, int nb, cudaStream_t s) \
    {                                                                                               \
        chem::k_rconst<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, rki, sun);                     \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t occupancy_(int* bps)                                                                \
    {                                                                                               \
        int a = 0, b = 0;                                                                           \
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                              \
            &a, chem::k_chem_ros3<T_>, chem::THREADS_PER_BLOCK, 0);                                 \
        if (e != cudaSuccess) return e;                                                             \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                                          \
            &b, chem::k_chem_ros3_queue<T_, false>, chem::THREADS_PER_BLOCK, 0);                    \
        *bps = a < b ? a : b;                                                                       \
        return e;                                                                                   \
    }                                                                                               \
    }                                                                                               \
    extern const MechOps SYMBOL = {NS::NAME, T_::NSPEC, T_::NRXNS, T_::ISCHAN, T_::NPHOTAB,         \
                                   T_::NHETERO, T_::WS_ELEMS, T_::IARRAY_DAY, T_::IARRAY_NIGHT,     \
                                   NS::FLOPS_STEP_DAY, NS::FLOPS_STEP_NIGHT,                        \
                                   NS::h_cgrid_index, NS::h_convert, NS::h_molwt, NS::h_inew2old,   \
                                   NS::h_iold2new, chem_static_, chem_queue_, solve_, rconst_,      \
                                   occupancy_};
