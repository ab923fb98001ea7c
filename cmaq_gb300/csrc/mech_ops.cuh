// Per-mechanism kernel table: each mechanism's translation unit instantiates the grid
// kernels for its generated device code and exports one MechOps object.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "chem_kernels.cuh"
#include "queue_kernels.cuh"
#include "ebi.cuh"
#include "adjoint.cuh"
#include "ddm.cuh"
#include "gear.cuh"

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
    // sync: 0 free-running warps, 1 barriers between attempt phases, 2 also between chunks;
    // wpb: warps per block (2, 4 or 8)
    cudaError_t (*chem_queue)(const chem::GridArgs&, const chem::QueueArgs&, int sync, int wpb, int nblocks,
                              cudaStream_t);
    cudaError_t (*queue_occupancy)(int sync, int wpb, int* blocks_per_sm);
    cudaError_t (*solve)(const chem::SolveArgs&, int nblocks, cudaStream_t);
    cudaError_t (*chem_ebi)(const chem::GridArgs&, const chem::QueueArgs&, const chem::EbiArgs&, int nblocks,
                            cudaStream_t);
    cudaError_t (*ebi_solve)(const chem::EbiSolveArgs&, int nblocks, cudaStream_t);
    cudaError_t (*chem_ebi_warp)(const chem::GridArgs&, const chem::QueueArgs&, const chem::EbiArgs&, int nblocks,
                                 cudaStream_t);
    cudaError_t (*ebi_warp_occupancy)(int* blocks_per_sm);
    double ebi_deltat;
    int adj_ws_elems;
    cudaError_t (*adj_forward)(const adj::Args&, int nblocks, cudaStream_t);
    cudaError_t (*adj_reverse)(const adj::Args&, int nblocks, cudaStream_t);
    cudaError_t (*adj_occupancy)(int* forward_bps, int* reverse_bps);
    cudaError_t (*ddm_update)(const chem::GridArgs&, const chem::DdmArgs&, int nblocks, cudaStream_t);
    cudaError_t (*rconst)(const chem::GridArgs&, double* rki, uint8_t* sunlit, int nblocks, cudaStream_t);
    cudaError_t (*rconst_pass)(const chem::GridArgs&, long long c0, long long c1, double* rki, uint8_t* sunlit,
                               int nblocks, cudaStream_t);
    cudaError_t (*occupancy)(int* blocks_per_sm);
    int gear_ws_elems;
    // grid: one Gear CHEM call on GridArgs; otherwise the solver-level entry on GearArgs' arrays
    cudaError_t (*gear)(const chem::GridArgs&, const chem::QueueArgs&, const chem::GearArgs&, bool grid, int nblocks,
                        cudaStream_t);
    cudaError_t (*gear_occupancy)(int* blocks_per_sm);
    // one cell per warp with its workspace in shared memory (one-warp blocks)
    cudaError_t (*gear_warp)(const chem::GridArgs&, const chem::QueueArgs&, const chem::GearArgs&, bool grid,
                             int nblocks, cudaStream_t);
    cudaError_t (*gear_warp_occupancy)(int* blocks_per_sm);
};

#define DEFINE_MECH_OPS(NS, SYMBOL)                                                                 \
    namespace {                                                                                     \
    using T_ = NS::Traits;                                                                          \
    cudaError_t chem_static_(const chem::GridArgs& a, int nb, cudaStream_t s)                       \
    {                                                                                               \
        chem::k_chem_ros3<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a);                            \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    template <int SY, int W>                                                                        \
    cudaError_t launch_q_(const chem::GridArgs& a, const chem::QueueArgs& q, int nb, cudaStream_t s)  \
    {                                                                                               \
        chem::k_chem_ros3_queue<T_, SY, W><<<nb, W * 32, 0, s>>>(a, q);                             \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    template <int SY, int W>                                                                        \
    cudaError_t occ_q_(int* bps)                                                                    \
    {                                                                                               \
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, chem::k_chem_ros3_queue<T_, SY, W>, \
                                                             W * 32, 0);                            \
    }                                                                                               \
    cudaError_t chem_queue_(const chem::GridArgs& a, const chem::QueueArgs& q, int sync, int wpb, int nb, \
                            cudaStream_t s)                                                         \
    {                                                                                               \
        switch (sync * 16 + wpb) {                                                                  \
        case 0 * 16 + 8: return launch_q_<0, 8>(a, q, nb, s);                                       \
        case 1 * 16 + 8: return launch_q_<1, 8>(a, q, nb, s);                                       \
        case 2 * 16 + 8: return launch_q_<2, 8>(a, q, nb, s);                                       \
        case 1 * 16 + 4: return launch_q_<1, 4>(a, q, nb, s);                                       \
        case 2 * 16 + 4: return launch_q_<2, 4>(a, q, nb, s);                                       \
        case 1 * 16 + 2: return launch_q_<1, 2>(a, q, nb, s);                                       \
        case 2 * 16 + 2: return launch_q_<2, 2>(a, q, nb, s);                                       \
        default: return cudaErrorInvalidValue;                                                      \
        }                                                                                           \
    }                                                                                               \
    cudaError_t queue_occupancy_(int sync, int wpb, int* bps)                                       \
    {                                                                                               \
        switch (sync * 16 + wpb) {                                                                  \
        case 0 * 16 + 8: return occ_q_<0, 8>(bps);                                                  \
        case 1 * 16 + 8: return occ_q_<1, 8>(bps);                                                  \
        case 2 * 16 + 8: return occ_q_<2, 8>(bps);                                                  \
        case 1 * 16 + 4: return occ_q_<1, 4>(bps);                                                  \
        case 2 * 16 + 4: return occ_q_<2, 4>(bps);                                                  \
        case 1 * 16 + 2: return occ_q_<1, 2>(bps);                                                  \
        case 2 * 16 + 2: return occ_q_<2, 2>(bps);                                                  \
        default: return cudaErrorInvalidValue;                                                      \
        }                                                                                           \
    }                                                                                               \
    cudaError_t solve_(const chem::SolveArgs& a, int nb, cudaStream_t s)                            \
    {                                                                                               \
        chem::k_ros3_solve<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a);                           \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t chem_ebi_(const chem::GridArgs& a, const chem::QueueArgs& q, const chem::EbiArgs& e, int nb, \
                          cudaStream_t s)                                                           \
    {                                                                                               \
        chem::k_chem_ebi_queue<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, q, e);                 \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    size_t ebiw_smem_() { return (size_t)chem::EBIW_WPB * T_::EBIW_ELEMS * sizeof(double); }        \
    cudaError_t ebiw_attr_()                                                                        \
    {                                                                                               \
        cudaError_t r = cudaFuncSetAttribute(chem::k_chem_ebi_warp<T_>,                             \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ebiw_smem_()); \
        if (r != cudaSuccess) return r;                                                             \
        return cudaFuncSetAttribute(chem::k_chem_ebi_warp<T_>, cudaFuncAttributePreferredSharedMemoryCarveout, \
                                    (int)cudaSharedmemCarveoutMaxShared);                           \
    }                                                                                               \
    cudaError_t chem_ebi_warp_(const chem::GridArgs& a, const chem::QueueArgs& q, const chem::EbiArgs& e, \
                               int nb, cudaStream_t s)                                              \
    {                                                                                               \
        cudaError_t r = ebiw_attr_();                                                               \
        if (r != cudaSuccess) return r;                                                             \
        chem::k_chem_ebi_warp<T_><<<nb, chem::EBIW_WPB * 32, ebiw_smem_(), s>>>(a, q, e);           \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t ebi_warp_occupancy_(int* bps)                                                       \
    {                                                                                               \
        cudaError_t r = ebiw_attr_();                                                               \
        if (r != cudaSuccess) return r;                                                             \
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(bps, chem::k_chem_ebi_warp<T_>,        \
                                                             chem::EBIW_WPB * 32, ebiw_smem_());    \
    }                                                                                               \
    cudaError_t ebi_solve_(const chem::EbiSolveArgs& a, int nb, cudaStream_t s)                     \
    {                                                                                               \
        chem::k_ebi_solve<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a);                            \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t adj_forward_(const adj::Args& a, int nb, cudaStream_t s)                            \
    {                                                                                               \
        adj::k_adj_forward<T_><<<nb, adj::THREADS, 0, s>>>(a);                                      \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t adj_reverse_(const adj::Args& a, int nb, cudaStream_t s)                            \
    {                                                                                               \
        adj::k_adj_reverse<T_><<<nb, adj::THREADS, 0, s>>>(a);                                      \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t adj_occupancy_(int* f, int* r)                                                      \
    {                                                                                               \
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(f, adj::k_adj_forward<T_>, adj::THREADS, 0); \
        if (e != cudaSuccess) return e;                                                             \
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(r, adj::k_adj_reverse<T_>, adj::THREADS, 0); \
    }                                                                                               \
    cudaError_t ddm_update_(const chem::GridArgs& a, const chem::DdmArgs& d, int nb, cudaStream_t s) \
    {                                                                                               \
        chem::k_ddm_update<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, d);                        \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t rconst_(const chem::GridArgs& a, double* rki, uint8_t* sun, int nb, cudaStream_t s) \
    {                                                                                               \
        chem::k_rconst<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, rki, sun);                     \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t rconst_pass_(const chem::GridArgs& a, long long c0, long long c1, double* rki, uint8_t* sun, \
                             int nb, cudaStream_t s)                                                \
    {                                                                                               \
        chem::k_rconst_pass<T_><<<nb, chem::THREADS_PER_BLOCK, 0, s>>>(a, c0, c1, rki, sun);        \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t gear_(const chem::GridArgs& a, const chem::QueueArgs& q, const chem::GearArgs& g, bool grid, \
                      int nb, cudaStream_t s)                                                       \
    {                                                                                               \
        if (grid) chem::k_gear<T_, true><<<nb, chem::GEAR_WPB * 32, 0, s>>>(a, q, g);               \
        else chem::k_gear<T_, false><<<nb, chem::GEAR_WPB * 32, 0, s>>>(a, q, g);                   \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t gear_occupancy_(int* bps)                                                           \
    {                                                                                               \
        int a = 0, b = 0;                                                                           \
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, chem::k_gear<T_, true>,   \
                                                                      chem::GEAR_WPB * 32, 0);      \
        if (e != cudaSuccess) return e;                                                             \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, chem::k_gear<T_, false>, chem::GEAR_WPB * 32, 0); \
        *bps = a < b ? a : b;                                                                       \
        return e;                                                                                   \
    }                                                                                               \
    size_t gearw_smem_() { return (size_t)T_::GEAR_WS_ELEMS * sizeof(double); }                     \
    template <bool G>                                                                               \
    cudaError_t gearw_attr_()                                                                       \
    {                                                                                               \
        cudaError_t r = cudaFuncSetAttribute(chem::k_gear_warp<T_, G>,                              \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gearw_smem_()); \
        if (r != cudaSuccess) return r;                                                             \
        return cudaFuncSetAttribute(chem::k_gear_warp<T_, G>, cudaFuncAttributePreferredSharedMemoryCarveout, \
                                    (int)cudaSharedmemCarveoutMaxShared);                           \
    }                                                                                               \
    cudaError_t gear_warp_(const chem::GridArgs& a, const chem::QueueArgs& q, const chem::GearArgs& g, bool grid, \
                           int nb, cudaStream_t s)                                                  \
    {                                                                                               \
        cudaError_t r = grid ? gearw_attr_<true>() : gearw_attr_<false>();                          \
        if (r != cudaSuccess) return r;                                                             \
        if (grid) chem::k_gear_warp<T_, true><<<nb, 32, gearw_smem_(), s>>>(a, q, g);               \
        else chem::k_gear_warp<T_, false><<<nb, 32, gearw_smem_(), s>>>(a, q, g);                   \
        return cudaGetLastError();                                                                  \
    }                                                                                               \
    cudaError_t gear_warp_occupancy_(int* bps)                                                      \
    {                                                                                               \
        cudaError_t r = gearw_attr_<true>();                                                        \
        if (r == cudaSuccess) r = gearw_attr_<false>();                                             \
        if (r != cudaSuccess) return r;                                                             \
        int a = 0, b = 0;                                                                           \
        r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, chem::k_gear_warp<T_, true>, 32, gearw_smem_()); \
        if (r != cudaSuccess) return r;                                                             \
        r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, chem::k_gear_warp<T_, false>, 32, gearw_smem_()); \
        *bps = a < b ? a : b;                                                                       \
        return r;                                                                                   \
    }                                                                                               \
    cudaError_t occupancy_(int* bps)                                                                \
    {                                                                                               \
        int a = 0, b = 0;                                                                           \
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(                              \
            &a, chem::k_chem_ros3<T_>, chem::THREADS_PER_BLOCK, 0);                                 \
        if (e != cudaSuccess) return e;                                                             \
        e = occ_q_<1, 8>(&b);                                                                       \
        *bps = a < b ? a : b;                                                                       \
        return e;                                                                                   \
    }                                                                                               \
    }                                                                                               \
    extern const MechOps SYMBOL = {NS::NAME, T_::NSPEC, T_::NRXNS, T_::ISCHAN, T_::NPHOTAB,         \
                                   T_::NHETERO, T_::WS_ELEMS, T_::IARRAY_DAY, T_::IARRAY_NIGHT,     \
                                   NS::FLOPS_STEP_DAY, NS::FLOPS_STEP_NIGHT,                        \
                                   NS::h_cgrid_index, NS::h_convert, NS::h_molwt, NS::h_inew2old,   \
                                   NS::h_iold2new, chem_static_, chem_queue_, queue_occupancy_,     \
                                   solve_, chem_ebi_, ebi_solve_, chem_ebi_warp_, ebi_warp_occupancy_, \
                                   T_::EBI_DELTAT,                                                  \
                                   T_::ADJ_WS_ELEMS, adj_forward_, adj_reverse_, adj_occupancy_, ddm_update_,     \
                                   rconst_, rconst_pass_, occupancy_, T_::GEAR_WS_ELEMS, gear_, gear_occupancy_, \
                                   gear_warp_, gear_warp_occupancy_};
