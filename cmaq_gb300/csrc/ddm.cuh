// DDM-3D chemistry sensitivities on the GPU, first order.
//
// Restates SOLVE_DDM3D_CHEM (CCTM/src/ddm3d/DDM3D_CHEM.F:155-410) for every cell after a
// CHEM call: with YAVE the call's time-averaged concentrations (rbsolver.F:468-475,
// 592-595) and DT the synchronisation step, each parameter's sensitivity vector S is
// advanced by
//
//     (I - DT/2 J(YAVE)) S_new = (I + DT/2 J(YAVE)) S_old + DT dF/dp(YAVE)
//
// The reference forms J densely in REAL(4) (MECHANISM_FUNCTIONS.F:755) and factors with
// LINPACK SGEFA/SGESL; here the generated sparse LU of the ROS3 solver is reused in FP64:
// I - DT/2 J = -(DT/2) (J - (2/DT) I), so the LU of J - g I with g = 2/DT (what jacdecomp
// computes for a ROS3 step with gamma h = DT/2) solves it after scaling the right-hand
// side by -g.  Reaction-rate parameters (IPT = 5) add DT x IREGION x the rates of their
// reactions times the stoichiometry (DDM3D_CHEM.F:338-385); other first-order parameters
// (initial conditions, boundary, emissions handled outside chemistry) add nothing here.
// Sensitivities stay in the reference's SENGRID layout and precision: REAL(4)
// SENGRID(NCOLS,NROWS,NLAYS,NPMAX,NSPCSD), values below 1e-25 in magnitude set to 0.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "chem_kernels.cuh"

namespace chem {

struct DdmArgs {
    float* sengrid;                    // [nspcsd][nparam][ncell]
    int nparam;
    const unsigned char* rate_mask;    // [nparam][nrxns]: reaction r belongs to parameter p; or nullptr
    const float* region;               // [nparam][ncell] IREGION weights of rate parameters, or nullptr (1)
    const double* yave;                // [ischan][ncell] time-averaged concentrations of the call
};

template <class M>
__global__ void __launch_bounds__(THREADS_PER_BLOCK, 1) k_ddm_update(GridArgs a, DdmArgs d)
{
    const long long nwarps = (long long)gridDim.x * WARPS_PER_BLOCK;
    const long long warp = (long long)blockIdx.x * WARPS_PER_BLOCK + (threadIdx.x >> 5);
    double* ws = warp_ws<M>(a.ws, warp);
    const double dt = a.chemstep;
    const double g = 2.0 / dt;
    for (long long base = warp * 32; base < a.ncell; base += nwarps * 32) {
        const long long c = base + (threadIdx.x & 31);
        const bool active = c < a.ncell;
        bool sun = false;
        if (active) {
            sun = gather_cell<M>(a, c, ws);   // rate constants of the cell (CALC_RCONST)
            for (int i = 0; i < M::ISCHAN; ++i) ws[(M::OFF_Y + i) * 32] = d.yave[(size_t)i * a.ncell + c];
        }
        const bool night = a.use_night && __all_sync(0xffffffffu, !active || !sun);
        if (!active) continue;
        if (night) M::feval_1(ws, M::OFF_Y, M::OFF_F0); else M::feval_0(ws, M::OFF_Y, M::OFF_F0);  // RXRAT
        if (night) M::explic_1(ws); else M::explic_0(ws);
        if (night) M::jacdecomp_1(ws, g); else M::jacdecomp_0(ws, g);
        for (int p = 0; p < d.nparam; ++p) {
            for (int i = 0; i < M::ISCHAN; ++i) {
                const int plane = a.cgrid_index[M::inew2old(i)];
                double sv = (double)d.sengrid[((size_t)plane * d.nparam + p) * a.ncell + c];
                if (fabs(sv) < 1.0e-25) sv = 0.0;
                ws[(M::OFF_K1 + i) * 32] = sv;
                ws[(M::OFF_K2 + i) * 32] = 0.0;
            }
            if (night) M::ddm_jv_1(ws, M::OFF_Y, M::OFF_K1, M::OFF_K2);
            else M::ddm_jv_0(ws, M::OFF_Y, M::OFF_K1, M::OFF_K2);
            for (int i = 0; i < M::ISCHAN; ++i)
                ws[(M::OFF_K3 + i) * 32] = ws[(M::OFF_K1 + i) * 32] + 0.5 * dt * ws[(M::OFF_K2 + i) * 32];
            if (d.rate_mask) {
                const double w = d.region ? (double)d.region[(size_t)p * a.ncell + c] : 1.0;
                const unsigned char* mk = d.rate_mask + (size_t)p * M::NRXNS;
                if (night) M::ddm_src_1(ws, mk, dt * w, M::OFF_K3); else M::ddm_src_0(ws, mk, dt * w, M::OFF_K3);
            }
            for (int i = 0; i < M::ISCHAN; ++i) ws[(M::OFF_K3 + i) * 32] = -g * ws[(M::OFF_K3 + i) * 32];
            if (night) M::solve_1(ws, M::OFF_K3); else M::solve_0(ws, M::OFF_K3);
            for (int i = 0; i < M::ISCHAN; ++i) {
                const int plane = a.cgrid_index[M::inew2old(i)];
                const double x = ws[(M::OFF_K3 + i) * 32];
                d.sengrid[((size_t)plane * d.nparam + p) * a.ncell + c] = fabs(x) < 1.0e-25 ? 0.0f : (float)x;
            }
        }
    }
}

}  // namespace chem
