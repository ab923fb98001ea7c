// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#pragma once
#include <cuda_runtime.h>
#ifndef CHEM_HD
#define CHEM_HD __device__
#endif
// load of an LU factor or 1/U(i,i); a build may define it as a streaming load (__ldcs)
#ifndef CHEM_LDLU
#define CHEM_LDLU(p) (*(p))
#endif
// L2 prefetch of workspace entries a few rows ahead (build variant 'pf'); off by default
#ifdef CHEM_USE_PREFETCH
__device__ __forceinline__ void chem_prefetch_l2(const double* p)
{
    asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(p)));
}
#define CHEM_PREFETCH(p) chem_prefetch_l2(p)
#else
#define CHEM_PREFETCH(p) ((void)0)
#endif
// L1 prefetch of the entries the next row reads (build variant 'pfl1'); off by default
#ifdef CHEM_USE_PREFETCH_L1
__device__ __forceinline__ void chem_prefetch_l1(const double* p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(__cvta_generic_to_global(p)));
}
#define CHEM_PREFETCH_L1(p) chem_prefetch_l1(p)
#else
#define CHEM_PREFETCH_L1(p) ((void)0)
#endif
// 1/U(i,i): IEEE division by default; a build may use the correctly rounded
// reciprocal __drcp_rn, which gives the same bits
#ifndef CHEM_RCP
#define CHEM_RCP(x) (1.0 / (x))
#endif
namespace mech_cb6r5_ae7_aq {
constexpr const char* NAME = "cb6r5_ae7_aq";
constexpr int NSPEC = 149;
constexpr int NRXNS = 349;
constexpr int ISCHAN = 149;
constexpr int NPHOTAB = 32;
constexpr int NHETERO = 17;
constexpr int WS_ELEMS = 4265;
constexpr int OFF_Y = 0;
constexpr int OFF_YP = 149;
constexpr int OFF_YDOT = 298;
constexpr int OFF_F0 = 447;
constexpr int OFF_K1 = 596;
constexpr int OFF_K2 = 745;
constexpr int OFF_K3 = 894;
constexpr int OFF_RKI = 1043;
constexpr int OFF_RXRAT = 1392;
constexpr int OFF_LU = 2426;
constexpr int OFF_VDIAG = 4116;
constexpr int IARRAY_DAY = 1689;
constexpr int IARRAY_NIGHT = 1615;
constexpr int EBI_OFF_YC = 2426;
constexpr int EBI_OFF_YC0 = 2575;
constexpr int EBI_OFF_YCP = 2724;
constexpr int EBI_OFF_PROD = 2873;
constexpr int EBI_OFF_LOSS = 3022;
constexpr int EBI_OFF_PNEG = 3171;
constexpr int ADJ_WS_ELEMS = 5806;
constexpr int ADJ_LAM = 4265;
constexpr int ADJ_MU1 = 4414;
constexpr int ADJ_MU2 = 4563;
constexpr int ADJ_MU3 = 4712;
constexpr int ADJ_PHI = 4861;
constexpr int ADJ_TMP = 5010;
constexpr int ADJ_EMIS = 5159;
constexpr int ADJ_GE = 5308;
constexpr int ADJ_GK = 5457;
constexpr int OFF_YAVE = 2277;
constexpr int GEAR_WS_ELEMS = 5308;
constexpr int GEAR_CNEW = 0;
constexpr int GEAR_GLOSS = 298;
constexpr int GEAR_DTLOS = 596;
constexpr int GEAR_CHOLD = 745;
constexpr int GEAR_CEST = 894;
constexpr int GEAR_BLKCONC = 447;
constexpr int GEAR_CONC = 4265;
constexpr int GEAR_E = 149;
constexpr int GEAR_CAVEG = 2277;
constexpr int GEAR_CFINI = 5159;
constexpr int EBIW_YC = 0;
constexpr int EBIW_YC0 = 149;
constexpr int EBIW_YCP = 298;
constexpr int EBIW_PROD = 447;
constexpr int EBIW_LOSS = 596;
constexpr int EBIW_PNEG = 745;
constexpr int EBIW_NOTMAX = 894;
constexpr int EBIW_RKI = 1043;
constexpr int EBIW_RXRAT = 1392;
constexpr int EBIW_ELEMS = 1741;
constexpr double FLOPS_STEP_DAY = 36947.0;
constexpr double FLOPS_STEP_NIGHT = 34766.0;
extern __constant__ int c_inew2old[149];
extern __constant__ int c_iold2new[149];
static const int h_inew2old[149] = {112, 113, 114, 116, 117, 118, 120, 121, 14, 15, 43, 50, 68, 86, 101, 104, 105, 106, 108, 109, 110, 5, 122, 124, 126, 127, 41, 42, 46, 47, 49, 56, 60, 62, 73, 77, 80, 87, 94, 103, 9, 107, 19, 115, 119, 123, 125, 132, 143, 145, 148, 58, 59, 12, 36, 83, 85, 89, 99, 100, 102, 25, 48, 147, 64, 65, 67, 72, 84, 13, 98, 27, 131, 138, 139, 140, 142, 11, 79, 54, 81, 93, 96, 51, 20, 28, 128, 129, 130, 66, 29, 137, 75, 141, 144, 146, 97, 70, 53, 135, 136, 91, 95, 63, 82, 111, 45, 55, 8, 74, 90, 52, 78, 69, 32, 133, 134, 61, 34, 76, 38, 57, 21, 71, 92, 40, 33, 37, 22, 23, 2, 10, 44, 39, 31, 3, 30, 1, 17, 16, 35, 26, 88, 24, 0, 4, 18, 7, 6};
static const int h_iold2new[149] = {144, 137, 130, 135, 145, 21, 148, 147, 108, 40, 131, 77, 53, 69, 8, 9, 139, 138, 146, 42, 84, 122, 128, 129, 143, 61, 141, 71, 85, 90, 136, 134, 114, 126, 118, 140, 54, 127, 120, 133, 125, 26, 27, 10, 132, 106, 28, 29, 62, 30, 11, 83, 111, 98, 79, 107, 31, 121, 51, 52, 32, 117, 33, 103, 64, 65, 89, 66, 12, 113, 97, 123, 67, 34, 109, 92, 119, 35, 112, 78, 36, 80, 104, 55, 68, 56, 13, 37, 142, 57, 110, 101, 124, 81, 38, 102, 82, 96, 70, 58, 59, 14, 60, 39, 15, 16, 17, 41, 18, 19, 20, 105, 0, 1, 2, 43, 3, 4, 5, 44, 6, 7, 22, 45, 23, 46, 24, 25, 86, 87, 88, 72, 47, 115, 116, 99, 100, 91, 73, 74, 75, 93, 76, 48, 94, 49, 95, 63, 50};
static const int h_cgrid_index[149] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 34, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 33, 32, 49, 50, 51, 52, 53, 54, 55, 56, 57, 58, 59, 60, 61, 62, 64, 65, 69, 67, 66, 70, 71, 72, 73, 74, 75, 76, 77, 78, 79, 80, 81, 82, 83, 84, 85, 86, 87, 88, 89, 90, 91, 92, 93, 94, 95, 96, 124, 125, 126, 123, 97, 98, 99, 100, 101, 141, 142, 143, 63, 131, 176, 179, 68, 180, 181, 205, 177, 206, 207, 144, 178, 145, 146, 182, 184, 183, 185, 112, 113, 102, 103, 104, 105, 106, 107, 108, 110, 111, 109, 114, 115, 116, 117, 118, 119, 120, 121, 122, 127, 128};
static const int h_convert[149] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 1, 1, 1, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const double h_molwt[149] = {46.0, 30.0, 16.0, 48.0, 62.0, 16.0, 17.0, 33.0, 34.0, 108.0, 63.0, 47.0, 79.0, 64.0, 98.0, 98.0, 75.0, 47.0, 87.1, 121.0, 76.0, 60.0, 89.0, 44.0, 87.1, 135.0, 30.0, 48.0, 32.0, 90.1, 87.1, 87.1, 119.1, 135.1, 46.0, 28.0, 63.0, 58.1, 60.0, 58.0, 72.0, 30.1, 46.1, 72.1, 14.0, 58.1, 44.1, 89.1, 45.0, 29.0, 26.0, 28.0, 42.1, 56.1, 68.1, 117.1, 68.1, 70.1, 147.1, 118.1, 116.1, 115.0, 118.1, 149.1, 136.2, 136.2, 197.0, 136.2, 78.1, 108.1, 159.1, 84.0, 127.0, 92.1, 173.1, 141.0, 98.1, 106.2, 187.1, 155.0, 128.2, 187.2, 107.1, 124.1, 153.1, 161.0, 16.0, 71.0, 35.5, 52.5, 51.5, 64.5, 36.5, 81.5, 97.5, 179.0, 169.0, 158.0, 198.0, 204.0, 204.0, 112.0, 64.0, 64.0, 35.5, 35.5, 35.5, 118.1, 96.0, 168.2, 66.4, 231.0, 231.0, 168.0, 179.0, 206.0, 169.0, 158.0, 132.0, 248.0, 133.0, 273.0, 220.0, 220.0, 220.0, 220.0, 170.0, 170.0, 218.0, 230.0, 241.0, 253.0, 266.0, 136.0, 136.0, 135.0, 134.0, 135.0, 30.0, 44.0, 54.0, 56.1, 56.1, 92.0, 200.6, 200.6, 271.5, 62.0, 96.0};
__device__ void rconst(double* __restrict__ ws, double temp_in, double press, double h2o, double seawater, int lsunlight, const double* __restrict__ rjv, const double* __restrict__ hetv);
__device__ void feval_0(double* __restrict__ ws, int src, int dst);
__device__ void explic_0(double* __restrict__ ws);
__device__ void feval_1(double* __restrict__ ws, int src, int dst);
__device__ void explic_1(double* __restrict__ ws);
__device__ void gear_explic_0(double* __restrict__ ws);
__device__ void gear_pdecomp_0_0(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_1(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_2(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_3(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_4(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_5(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_6(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_7(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_8(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_9(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_10(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_11(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_12(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_13(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_14(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_15(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_16(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_17(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_18(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_19(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_20(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_21(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_22(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_23(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_24(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_25(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_26(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_27(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_28(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_29(double* __restrict__ ws, double r1delt);
__device__ void jacdecomp_0_0(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_1(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_2(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_3(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_4(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_5(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_6(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_7(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_8(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_9(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_10(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_11(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_12(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_13(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_14(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_15(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_16(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_17(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_18(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_19(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_20(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_21(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_22(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_23(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_24(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_25(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_26(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_27(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_28(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_29(double* __restrict__ ws, double gdtinv);
__device__ void solve_0_0(double* __restrict__ ws, int rhs);
__device__ void solve_0_1(double* __restrict__ ws, int rhs);
__device__ void solve_0_2(double* __restrict__ ws, int rhs);
__device__ void jacdecomp_1_0(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_1(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_2(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_3(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_4(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_5(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_6(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_7(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_8(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_9(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_10(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_11(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_12(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_13(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_14(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_15(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_16(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_17(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_18(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_19(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_20(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_21(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_22(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_23(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_24(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_25(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_26(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_27(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_28(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_29(double* __restrict__ ws, double gdtinv);
__device__ void solve_1_0(double* __restrict__ ws, int rhs);
__device__ void solve_1_1(double* __restrict__ ws, int rhs);
__device__ void solve_1_2(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_0(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_1(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_2(double* __restrict__ ws, int rhs);
__device__ void adj_jtv_0_0(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_1(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_2(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_3(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_4(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_5(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_6(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_7(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_hess3_0_0(double* __restrict__ ws);
__device__ void adj_hess3_0_1(double* __restrict__ ws);
__device__ void adj_hess3_0_2(double* __restrict__ ws);
__device__ void adj_hess3_0_3(double* __restrict__ ws);
__device__ void adj_hess3_0_4(double* __restrict__ ws);
__device__ void adj_hess3_0_5(double* __restrict__ ws);
__device__ void adj_hess3_0_6(double* __restrict__ ws);
__device__ void adj_hess3_0_7(double* __restrict__ ws);
__device__ void adj_hess3_0_8(double* __restrict__ ws);
__device__ void adj_hess3_0_9(double* __restrict__ ws);
__device__ void adj_hess3_0_10(double* __restrict__ ws);
__device__ void adj_hess3_0_11(double* __restrict__ ws);
__device__ void adj_hess3_0_12(double* __restrict__ ws);
__device__ void adj_hess3_0_13(double* __restrict__ ws);
__device__ void adj_hess3_0_14(double* __restrict__ ws);
__device__ void adj_hess3_0_15(double* __restrict__ ws);
__device__ void adj_hess3_0_16(double* __restrict__ ws);
__device__ void adj_hess3_0_17(double* __restrict__ ws);
__device__ void adj_hess3_0_18(double* __restrict__ ws);
__device__ void solve_t_1_0(double* __restrict__ ws, int rhs);
__device__ void solve_t_1_1(double* __restrict__ ws, int rhs);
__device__ void solve_t_1_2(double* __restrict__ ws, int rhs);
__device__ void adj_jtv_1_0(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_1(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_2(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_3(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_4(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_5(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_6(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_hess3_1_0(double* __restrict__ ws);
__device__ void adj_hess3_1_1(double* __restrict__ ws);
__device__ void adj_hess3_1_2(double* __restrict__ ws);
__device__ void adj_hess3_1_3(double* __restrict__ ws);
__device__ void adj_hess3_1_4(double* __restrict__ ws);
__device__ void adj_hess3_1_5(double* __restrict__ ws);
__device__ void adj_hess3_1_6(double* __restrict__ ws);
__device__ void adj_hess3_1_7(double* __restrict__ ws);
__device__ void adj_hess3_1_8(double* __restrict__ ws);
__device__ void adj_hess3_1_9(double* __restrict__ ws);
__device__ void adj_hess3_1_10(double* __restrict__ ws);
__device__ void adj_hess3_1_11(double* __restrict__ ws);
__device__ void adj_hess3_1_12(double* __restrict__ ws);
__device__ void adj_hess3_1_13(double* __restrict__ ws);
__device__ void adj_hess3_1_14(double* __restrict__ ws);
__device__ void adj_hess3_1_15(double* __restrict__ ws);
__device__ void adj_hess3_1_16(double* __restrict__ ws);
__device__ void ddm_jv_0_0(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_1(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_2(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_3(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_4(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_5(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_src_0_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_2(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_3(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_4(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_5(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_jv_1_0(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_1(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_2(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_3(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_4(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_5(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_src_1_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_2(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_3(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_4(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_5(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
extern __device__ const int c_gw_act_r[349];
extern __device__ const int c_gw_act_sp[1047];
extern __device__ const int c_gw_sum_ptr[150];
extern __device__ const int c_gw_sum_r[1738];
extern __device__ const int c_gw_sum_k[1738];
extern __device__ const int c_gw_lane_ptr[33];
extern __device__ const int c_gw_lane_sp[149];
extern __device__ const int c_gw_ex_r[268];
extern __device__ const int c_gw_ex_sp[804];
extern __device__ const int c_gw_ex_off[268];
extern __device__ const int c_gw_asm_ptr[1691];
extern __device__ const int c_gw_asm_src[3213];
extern __device__ const int c_gw_asm_kind[3213];
extern __device__ const int c_gw_piv_diag[149];
extern __device__ const int c_gw_lsc_ptr[150];
extern __device__ const int c_gw_lsc_st[883];
extern __device__ const int c_gw_up_ptr[150];
extern __device__ const int c_gw_up_ij[5247];
extern __device__ const int c_gw_up_ik[5247];
extern __device__ const int c_gw_up_kj[5247];
extern __device__ const int c_gw_fl_ptr[23];
extern __device__ const int c_gw_fl_row[149];
extern __device__ const int c_gw_bl_ptr[20];
extern __device__ const int c_gw_bl_row[149];
extern __device__ const int c_gw_fr_ptr[150];
extern __device__ const int c_gw_fr_st[883];
extern __device__ const int c_gw_fr_col[883];
extern __device__ const int c_gw_br_ptr[150];
extern __device__ const int c_gw_br_st[657];
extern __device__ const int c_gw_br_col[657];
extern __device__ const double c_gw_sum_c[1738];
extern __device__ const double c_gw_asm_c[3213];
constexpr int EBI_N_EBISP = 136;
constexpr double EBI_DELTAT = 2.5;
constexpr int EBI_NEBITER = 1000;
constexpr int EBI_NPNEG = 1;
extern __constant__ int c_ebi_ebisp[136];
extern __constant__ double c_ebi_rtol[149];
extern __constant__ int c_ebi_pneg[1];
__device__ void ebi_hrrates(double* __restrict__ ws);
__device__ void ebi_hrprodloss(double* __restrict__ ws);
__device__ void ebi_hrg1(double* __restrict__ ws, double dtc);
__device__ void ebi_hrg2(double* __restrict__ ws, double dtc);
__device__ void ebi_hrg3(double* __restrict__ ws, double dtc);
__device__ void ebi_hrg4(double* __restrict__ ws, double dtc);
constexpr int EBIW_NRATE = 328;
constexpr int EBIW_NPL = 273;
constexpr int EBIW_NTERM = 1109;
extern __device__ const int c_ebiw_rate_r[EBIW_NRATE];
extern __device__ const int c_ebiw_rate_nf[EBIW_NRATE];
extern __device__ const int c_ebiw_rate_sp[EBIW_NRATE * 3];
extern __device__ const int c_ebiw_pl_ptr[33];
extern __device__ const int c_ebiw_pl_kind[EBIW_NPL];
extern __device__ const int c_ebiw_pl_sp[EBIW_NPL];
extern __device__ const int c_ebiw_pl_t0[EBIW_NPL + 1];
extern __device__ const int c_ebiw_term_r[EBIW_NTERM > 0 ? EBIW_NTERM : 1];
extern __device__ const double c_ebiw_term_c[EBIW_NTERM > 0 ? EBIW_NTERM : 1];
namespace wsm {
__device__ void ebi_hrg1(double* __restrict__ sm, double dtc);
__device__ void ebi_hrg2(double* __restrict__ sm, double dtc);
__device__ void ebi_hrg3(double* __restrict__ sm, double dtc);
__device__ void ebi_hrg4(double* __restrict__ sm, double dtc);
}  // namespace wsm
__device__ __forceinline__ void gear_pdecomp_0(double* __restrict__ ws, double r1delt)
{
    gear_pdecomp_0_0(ws, r1delt);
    gear_pdecomp_0_1(ws, r1delt);
    gear_pdecomp_0_2(ws, r1delt);
    gear_pdecomp_0_3(ws, r1delt);
    gear_pdecomp_0_4(ws, r1delt);
    gear_pdecomp_0_5(ws, r1delt);
    gear_pdecomp_0_6(ws, r1delt);
    gear_pdecomp_0_7(ws, r1delt);
    gear_pdecomp_0_8(ws, r1delt);
    gear_pdecomp_0_9(ws, r1delt);
    gear_pdecomp_0_10(ws, r1delt);
    gear_pdecomp_0_11(ws, r1delt);
    gear_pdecomp_0_12(ws, r1delt);
    gear_pdecomp_0_13(ws, r1delt);
    gear_pdecomp_0_14(ws, r1delt);
    gear_pdecomp_0_15(ws, r1delt);
    gear_pdecomp_0_16(ws, r1delt);
    gear_pdecomp_0_17(ws, r1delt);
    gear_pdecomp_0_18(ws, r1delt);
    gear_pdecomp_0_19(ws, r1delt);
    gear_pdecomp_0_20(ws, r1delt);
    gear_pdecomp_0_21(ws, r1delt);
    gear_pdecomp_0_22(ws, r1delt);
    gear_pdecomp_0_23(ws, r1delt);
    gear_pdecomp_0_24(ws, r1delt);
    gear_pdecomp_0_25(ws, r1delt);
    gear_pdecomp_0_26(ws, r1delt);
    gear_pdecomp_0_27(ws, r1delt);
    gear_pdecomp_0_28(ws, r1delt);
    gear_pdecomp_0_29(ws, r1delt);
}
__device__ __forceinline__ void jacdecomp_0(double* __restrict__ ws, double gdtinv)
{
    jacdecomp_0_0(ws, gdtinv);
    jacdecomp_0_1(ws, gdtinv);
    jacdecomp_0_2(ws, gdtinv);
    jacdecomp_0_3(ws, gdtinv);
    jacdecomp_0_4(ws, gdtinv);
    jacdecomp_0_5(ws, gdtinv);
    jacdecomp_0_6(ws, gdtinv);
    jacdecomp_0_7(ws, gdtinv);
    jacdecomp_0_8(ws, gdtinv);
    jacdecomp_0_9(ws, gdtinv);
    jacdecomp_0_10(ws, gdtinv);
    jacdecomp_0_11(ws, gdtinv);
    jacdecomp_0_12(ws, gdtinv);
    jacdecomp_0_13(ws, gdtinv);
    jacdecomp_0_14(ws, gdtinv);
    jacdecomp_0_15(ws, gdtinv);
    jacdecomp_0_16(ws, gdtinv);
    jacdecomp_0_17(ws, gdtinv);
    jacdecomp_0_18(ws, gdtinv);
    jacdecomp_0_19(ws, gdtinv);
    jacdecomp_0_20(ws, gdtinv);
    jacdecomp_0_21(ws, gdtinv);
    jacdecomp_0_22(ws, gdtinv);
    jacdecomp_0_23(ws, gdtinv);
    jacdecomp_0_24(ws, gdtinv);
    jacdecomp_0_25(ws, gdtinv);
    jacdecomp_0_26(ws, gdtinv);
    jacdecomp_0_27(ws, gdtinv);
    jacdecomp_0_28(ws, gdtinv);
    jacdecomp_0_29(ws, gdtinv);
}
__device__ __forceinline__ void jacdecomp_0_sync(double* __restrict__ ws, double gdtinv, bool go)
{
    if (go) jacdecomp_0_0(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_1(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_2(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_3(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_4(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_5(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_6(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_7(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_8(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_9(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_10(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_11(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_12(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_13(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_14(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_15(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_16(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_17(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_18(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_19(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_20(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_21(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_22(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_23(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_24(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_25(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_26(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_27(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_28(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_29(ws, gdtinv);
    __syncthreads();
}
__device__ __forceinline__ void solve_0(double* __restrict__ ws, int rhs)
{
    solve_0_0(ws, rhs);
    solve_0_1(ws, rhs);
    solve_0_2(ws, rhs);
}
__device__ __forceinline__ void solve_0_sync(double* __restrict__ ws, int rhs, bool go)
{
    if (go) solve_0_0(ws, rhs);
    __syncthreads();
    if (go) solve_0_1(ws, rhs);
    __syncthreads();
    if (go) solve_0_2(ws, rhs);
    __syncthreads();
}
__device__ __forceinline__ void jacdecomp_1(double* __restrict__ ws, double gdtinv)
{
    jacdecomp_1_0(ws, gdtinv);
    jacdecomp_1_1(ws, gdtinv);
    jacdecomp_1_2(ws, gdtinv);
    jacdecomp_1_3(ws, gdtinv);
    jacdecomp_1_4(ws, gdtinv);
    jacdecomp_1_5(ws, gdtinv);
    jacdecomp_1_6(ws, gdtinv);
    jacdecomp_1_7(ws, gdtinv);
    jacdecomp_1_8(ws, gdtinv);
    jacdecomp_1_9(ws, gdtinv);
    jacdecomp_1_10(ws, gdtinv);
    jacdecomp_1_11(ws, gdtinv);
    jacdecomp_1_12(ws, gdtinv);
    jacdecomp_1_13(ws, gdtinv);
    jacdecomp_1_14(ws, gdtinv);
    jacdecomp_1_15(ws, gdtinv);
    jacdecomp_1_16(ws, gdtinv);
    jacdecomp_1_17(ws, gdtinv);
    jacdecomp_1_18(ws, gdtinv);
    jacdecomp_1_19(ws, gdtinv);
    jacdecomp_1_20(ws, gdtinv);
    jacdecomp_1_21(ws, gdtinv);
    jacdecomp_1_22(ws, gdtinv);
    jacdecomp_1_23(ws, gdtinv);
    jacdecomp_1_24(ws, gdtinv);
    jacdecomp_1_25(ws, gdtinv);
    jacdecomp_1_26(ws, gdtinv);
    jacdecomp_1_27(ws, gdtinv);
    jacdecomp_1_28(ws, gdtinv);
    jacdecomp_1_29(ws, gdtinv);
}
__device__ __forceinline__ void jacdecomp_1_sync(double* __restrict__ ws, double gdtinv, bool go)
{
    if (go) jacdecomp_1_0(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_1(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_2(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_3(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_4(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_5(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_6(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_7(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_8(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_9(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_10(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_11(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_12(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_13(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_14(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_15(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_16(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_17(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_18(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_19(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_20(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_21(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_22(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_23(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_24(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_25(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_26(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_27(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_28(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_29(ws, gdtinv);
    __syncthreads();
}
__device__ __forceinline__ void solve_1(double* __restrict__ ws, int rhs)
{
    solve_1_0(ws, rhs);
    solve_1_1(ws, rhs);
    solve_1_2(ws, rhs);
}
__device__ __forceinline__ void solve_1_sync(double* __restrict__ ws, int rhs, bool go)
{
    if (go) solve_1_0(ws, rhs);
    __syncthreads();
    if (go) solve_1_1(ws, rhs);
    __syncthreads();
    if (go) solve_1_2(ws, rhs);
    __syncthreads();
}
__device__ __forceinline__ void solve_t_0(double* __restrict__ ws, int rhs)
{
    solve_t_0_0(ws, rhs);
    solve_t_0_1(ws, rhs);
    solve_t_0_2(ws, rhs);
}
__device__ __forceinline__ void adj_jtv_0(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    adj_jtv_0_0(ws, yoff, phioff, outoff);
    adj_jtv_0_1(ws, yoff, phioff, outoff);
    adj_jtv_0_2(ws, yoff, phioff, outoff);
    adj_jtv_0_3(ws, yoff, phioff, outoff);
    adj_jtv_0_4(ws, yoff, phioff, outoff);
    adj_jtv_0_5(ws, yoff, phioff, outoff);
    adj_jtv_0_6(ws, yoff, phioff, outoff);
    adj_jtv_0_7(ws, yoff, phioff, outoff);
}
__device__ __forceinline__ void adj_hess3_0(double* __restrict__ ws)
{
    adj_hess3_0_0(ws);
    adj_hess3_0_1(ws);
    adj_hess3_0_2(ws);
    adj_hess3_0_3(ws);
    adj_hess3_0_4(ws);
    adj_hess3_0_5(ws);
    adj_hess3_0_6(ws);
    adj_hess3_0_7(ws);
    adj_hess3_0_8(ws);
    adj_hess3_0_9(ws);
    adj_hess3_0_10(ws);
    adj_hess3_0_11(ws);
    adj_hess3_0_12(ws);
    adj_hess3_0_13(ws);
    adj_hess3_0_14(ws);
    adj_hess3_0_15(ws);
    adj_hess3_0_16(ws);
    adj_hess3_0_17(ws);
    adj_hess3_0_18(ws);
}
__device__ __forceinline__ void solve_t_1(double* __restrict__ ws, int rhs)
{
    solve_t_1_0(ws, rhs);
    solve_t_1_1(ws, rhs);
    solve_t_1_2(ws, rhs);
}
__device__ __forceinline__ void adj_jtv_1(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    adj_jtv_1_0(ws, yoff, phioff, outoff);
    adj_jtv_1_1(ws, yoff, phioff, outoff);
    adj_jtv_1_2(ws, yoff, phioff, outoff);
    adj_jtv_1_3(ws, yoff, phioff, outoff);
    adj_jtv_1_4(ws, yoff, phioff, outoff);
    adj_jtv_1_5(ws, yoff, phioff, outoff);
    adj_jtv_1_6(ws, yoff, phioff, outoff);
}
__device__ __forceinline__ void adj_hess3_1(double* __restrict__ ws)
{
    adj_hess3_1_0(ws);
    adj_hess3_1_1(ws);
    adj_hess3_1_2(ws);
    adj_hess3_1_3(ws);
    adj_hess3_1_4(ws);
    adj_hess3_1_5(ws);
    adj_hess3_1_6(ws);
    adj_hess3_1_7(ws);
    adj_hess3_1_8(ws);
    adj_hess3_1_9(ws);
    adj_hess3_1_10(ws);
    adj_hess3_1_11(ws);
    adj_hess3_1_12(ws);
    adj_hess3_1_13(ws);
    adj_hess3_1_14(ws);
    adj_hess3_1_15(ws);
    adj_hess3_1_16(ws);
}
__device__ __forceinline__ void ddm_jv_0(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    ddm_jv_0_0(ws, yoff, voff, outoff);
    ddm_jv_0_1(ws, yoff, voff, outoff);
    ddm_jv_0_2(ws, yoff, voff, outoff);
    ddm_jv_0_3(ws, yoff, voff, outoff);
    ddm_jv_0_4(ws, yoff, voff, outoff);
    ddm_jv_0_5(ws, yoff, voff, outoff);
}
__device__ __forceinline__ void ddm_src_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    ddm_src_0_0(ws, mask, scale, outoff);
    ddm_src_0_1(ws, mask, scale, outoff);
    ddm_src_0_2(ws, mask, scale, outoff);
    ddm_src_0_3(ws, mask, scale, outoff);
    ddm_src_0_4(ws, mask, scale, outoff);
    ddm_src_0_5(ws, mask, scale, outoff);
}
__device__ __forceinline__ void ddm_jv_1(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    ddm_jv_1_0(ws, yoff, voff, outoff);
    ddm_jv_1_1(ws, yoff, voff, outoff);
    ddm_jv_1_2(ws, yoff, voff, outoff);
    ddm_jv_1_3(ws, yoff, voff, outoff);
    ddm_jv_1_4(ws, yoff, voff, outoff);
    ddm_jv_1_5(ws, yoff, voff, outoff);
}
__device__ __forceinline__ void ddm_src_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    ddm_src_1_0(ws, mask, scale, outoff);
    ddm_src_1_1(ws, mask, scale, outoff);
    ddm_src_1_2(ws, mask, scale, outoff);
    ddm_src_1_3(ws, mask, scale, outoff);
    ddm_src_1_4(ws, mask, scale, outoff);
    ddm_src_1_5(ws, mask, scale, outoff);
}
struct Traits {
    static constexpr int NSPEC = mech_cb6r5_ae7_aq::NSPEC;
    static constexpr int NRXNS = mech_cb6r5_ae7_aq::NRXNS;
    static constexpr int ISCHAN = mech_cb6r5_ae7_aq::ISCHAN;
    static constexpr int NPHOTAB = mech_cb6r5_ae7_aq::NPHOTAB;
    static constexpr int NHETERO = mech_cb6r5_ae7_aq::NHETERO;
    static constexpr int WS_ELEMS = mech_cb6r5_ae7_aq::WS_ELEMS;
    static constexpr int OFF_Y = mech_cb6r5_ae7_aq::OFF_Y;
    static constexpr int OFF_YP = mech_cb6r5_ae7_aq::OFF_YP;
    static constexpr int OFF_YDOT = mech_cb6r5_ae7_aq::OFF_YDOT;
    static constexpr int OFF_F0 = mech_cb6r5_ae7_aq::OFF_F0;
    static constexpr int OFF_K1 = mech_cb6r5_ae7_aq::OFF_K1;
    static constexpr int OFF_K2 = mech_cb6r5_ae7_aq::OFF_K2;
    static constexpr int OFF_K3 = mech_cb6r5_ae7_aq::OFF_K3;
    static constexpr int OFF_RKI = mech_cb6r5_ae7_aq::OFF_RKI;
    static constexpr int OFF_RXRAT = mech_cb6r5_ae7_aq::OFF_RXRAT;
    static constexpr int OFF_LU = mech_cb6r5_ae7_aq::OFF_LU;
    static constexpr int OFF_VDIAG = mech_cb6r5_ae7_aq::OFF_VDIAG;
    static constexpr int IARRAY_DAY = mech_cb6r5_ae7_aq::IARRAY_DAY;
    static constexpr int IARRAY_NIGHT = mech_cb6r5_ae7_aq::IARRAY_NIGHT;
    static constexpr int EBI_OFF_YC = mech_cb6r5_ae7_aq::EBI_OFF_YC;
    static constexpr int EBI_OFF_YC0 = mech_cb6r5_ae7_aq::EBI_OFF_YC0;
    static constexpr int EBI_OFF_YCP = mech_cb6r5_ae7_aq::EBI_OFF_YCP;
    static constexpr int EBI_OFF_PROD = mech_cb6r5_ae7_aq::EBI_OFF_PROD;
    static constexpr int EBI_OFF_LOSS = mech_cb6r5_ae7_aq::EBI_OFF_LOSS;
    static constexpr int EBI_OFF_PNEG = mech_cb6r5_ae7_aq::EBI_OFF_PNEG;
    static constexpr int ADJ_WS_ELEMS = mech_cb6r5_ae7_aq::ADJ_WS_ELEMS;
    static constexpr int ADJ_LAM = mech_cb6r5_ae7_aq::ADJ_LAM;
    static constexpr int ADJ_MU1 = mech_cb6r5_ae7_aq::ADJ_MU1;
    static constexpr int ADJ_MU2 = mech_cb6r5_ae7_aq::ADJ_MU2;
    static constexpr int ADJ_MU3 = mech_cb6r5_ae7_aq::ADJ_MU3;
    static constexpr int ADJ_PHI = mech_cb6r5_ae7_aq::ADJ_PHI;
    static constexpr int ADJ_TMP = mech_cb6r5_ae7_aq::ADJ_TMP;
    static constexpr int ADJ_EMIS = mech_cb6r5_ae7_aq::ADJ_EMIS;
    static constexpr int ADJ_GE = mech_cb6r5_ae7_aq::ADJ_GE;
    static constexpr int ADJ_GK = mech_cb6r5_ae7_aq::ADJ_GK;
    static constexpr int OFF_YAVE = mech_cb6r5_ae7_aq::OFF_YAVE;
    static constexpr int GEAR_WS_ELEMS = mech_cb6r5_ae7_aq::GEAR_WS_ELEMS;
    static constexpr int GEAR_CNEW = mech_cb6r5_ae7_aq::GEAR_CNEW;
    static constexpr int GEAR_GLOSS = mech_cb6r5_ae7_aq::GEAR_GLOSS;
    static constexpr int GEAR_DTLOS = mech_cb6r5_ae7_aq::GEAR_DTLOS;
    static constexpr int GEAR_CHOLD = mech_cb6r5_ae7_aq::GEAR_CHOLD;
    static constexpr int GEAR_CEST = mech_cb6r5_ae7_aq::GEAR_CEST;
    static constexpr int GEAR_BLKCONC = mech_cb6r5_ae7_aq::GEAR_BLKCONC;
    static constexpr int GEAR_CONC = mech_cb6r5_ae7_aq::GEAR_CONC;
    static constexpr int GEAR_E = mech_cb6r5_ae7_aq::GEAR_E;
    static constexpr int GEAR_CAVEG = mech_cb6r5_ae7_aq::GEAR_CAVEG;
    static constexpr int GEAR_CFINI = mech_cb6r5_ae7_aq::GEAR_CFINI;
    static constexpr int EBIW_YC = mech_cb6r5_ae7_aq::EBIW_YC;
    static constexpr int EBIW_YC0 = mech_cb6r5_ae7_aq::EBIW_YC0;
    static constexpr int EBIW_YCP = mech_cb6r5_ae7_aq::EBIW_YCP;
    static constexpr int EBIW_PROD = mech_cb6r5_ae7_aq::EBIW_PROD;
    static constexpr int EBIW_LOSS = mech_cb6r5_ae7_aq::EBIW_LOSS;
    static constexpr int EBIW_PNEG = mech_cb6r5_ae7_aq::EBIW_PNEG;
    static constexpr int EBIW_NOTMAX = mech_cb6r5_ae7_aq::EBIW_NOTMAX;
    static constexpr int EBIW_RKI = mech_cb6r5_ae7_aq::EBIW_RKI;
    static constexpr int EBIW_RXRAT = mech_cb6r5_ae7_aq::EBIW_RXRAT;
    static constexpr int EBIW_ELEMS = mech_cb6r5_ae7_aq::EBIW_ELEMS;
    static constexpr const char* name() { return mech_cb6r5_ae7_aq::NAME; }
    static __device__ __forceinline__ int iold2new(int s) { return mech_cb6r5_ae7_aq::c_iold2new[s]; }
    static __device__ __forceinline__ int inew2old(int i) { return mech_cb6r5_ae7_aq::c_inew2old[i]; }
    static __device__ __forceinline__ void feval_0(double* ws, int s, int t) { mech_cb6r5_ae7_aq::feval_0(ws, s, t); }
    static __device__ __forceinline__ void explic_0(double* ws) { mech_cb6r5_ae7_aq::explic_0(ws); }
    static __device__ __forceinline__ void gear_explic_0(double* ws) { mech_cb6r5_ae7_aq::gear_explic_0(ws); }
    static __device__ __forceinline__ void gear_pdecomp_0(double* ws, double r) { mech_cb6r5_ae7_aq::gear_pdecomp_0(ws, r); }
    static __device__ __forceinline__ void jacdecomp_0(double* ws, double g) { mech_cb6r5_ae7_aq::jacdecomp_0(ws, g); }
    static __device__ __forceinline__ void solve_0(double* ws, int r) { mech_cb6r5_ae7_aq::solve_0(ws, r); }
    static __device__ __forceinline__ void jacdecomp_0_sync(double* ws, double g, bool go) { mech_cb6r5_ae7_aq::jacdecomp_0_sync(ws, g, go); }
    static __device__ __forceinline__ void solve_0_sync(double* ws, int r, bool go) { mech_cb6r5_ae7_aq::solve_0_sync(ws, r, go); }
    static __device__ __forceinline__ void solve_t_0(double* ws, int r) { mech_cb6r5_ae7_aq::solve_t_0(ws, r); }
    static __device__ __forceinline__ void adj_jtv_0(double* ws, int y, int phi, int out) { mech_cb6r5_ae7_aq::adj_jtv_0(ws, y, phi, out); }
    static __device__ __forceinline__ void adj_hess3_0(double* ws) { mech_cb6r5_ae7_aq::adj_hess3_0(ws); }
    static __device__ __forceinline__ void ddm_jv_0(double* ws, int y, int v, int out) { mech_cb6r5_ae7_aq::ddm_jv_0(ws, y, v, out); }
    static __device__ __forceinline__ void ddm_src_0(double* ws, const unsigned char* mk, double sc, int out) { mech_cb6r5_ae7_aq::ddm_src_0(ws, mk, sc, out); }
    static __device__ __forceinline__ void feval_1(double* ws, int s, int t) { mech_cb6r5_ae7_aq::feval_1(ws, s, t); }
    static __device__ __forceinline__ void explic_1(double* ws) { mech_cb6r5_ae7_aq::explic_1(ws); }
    static __device__ __forceinline__ void jacdecomp_1(double* ws, double g) { mech_cb6r5_ae7_aq::jacdecomp_1(ws, g); }
    static __device__ __forceinline__ void solve_1(double* ws, int r) { mech_cb6r5_ae7_aq::solve_1(ws, r); }
    static __device__ __forceinline__ void jacdecomp_1_sync(double* ws, double g, bool go) { mech_cb6r5_ae7_aq::jacdecomp_1_sync(ws, g, go); }
    static __device__ __forceinline__ void solve_1_sync(double* ws, int r, bool go) { mech_cb6r5_ae7_aq::solve_1_sync(ws, r, go); }
    static __device__ __forceinline__ void solve_t_1(double* ws, int r) { mech_cb6r5_ae7_aq::solve_t_1(ws, r); }
    static __device__ __forceinline__ void adj_jtv_1(double* ws, int y, int phi, int out) { mech_cb6r5_ae7_aq::adj_jtv_1(ws, y, phi, out); }
    static __device__ __forceinline__ void adj_hess3_1(double* ws) { mech_cb6r5_ae7_aq::adj_hess3_1(ws); }
    static __device__ __forceinline__ void ddm_jv_1(double* ws, int y, int v, int out) { mech_cb6r5_ae7_aq::ddm_jv_1(ws, y, v, out); }
    static __device__ __forceinline__ void ddm_src_1(double* ws, const unsigned char* mk, double sc, int out) { mech_cb6r5_ae7_aq::ddm_src_1(ws, mk, sc, out); }
    static constexpr int EBI_N_EBISP = mech_cb6r5_ae7_aq::EBI_N_EBISP;
    static constexpr int EBI_NEBITER = mech_cb6r5_ae7_aq::EBI_NEBITER;
    static constexpr int EBI_NPNEG = mech_cb6r5_ae7_aq::EBI_NPNEG;
    static constexpr double EBI_DELTAT = mech_cb6r5_ae7_aq::EBI_DELTAT;
    static __device__ __forceinline__ int ebi_ebisp(int e) { return mech_cb6r5_ae7_aq::c_ebi_ebisp[e]; }
    static __device__ __forceinline__ double ebi_rtol(int i) { return mech_cb6r5_ae7_aq::c_ebi_rtol[i]; }
    static __device__ __forceinline__ int ebi_pneg(int k) { return mech_cb6r5_ae7_aq::c_ebi_pneg[k]; }
    static __device__ __forceinline__ void ebi_hrrates(double* ws) { mech_cb6r5_ae7_aq::ebi_hrrates(ws); }
    static __device__ __forceinline__ void ebi_hrprodloss(double* ws) { mech_cb6r5_ae7_aq::ebi_hrprodloss(ws); }
    static __device__ __forceinline__ void ebi_hrg1(double* ws, double dtc) { mech_cb6r5_ae7_aq::ebi_hrg1(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg1(double* sm, double dtc) { mech_cb6r5_ae7_aq::wsm::ebi_hrg1(sm, dtc); }
    static __device__ __forceinline__ void ebi_hrg2(double* ws, double dtc) { mech_cb6r5_ae7_aq::ebi_hrg2(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg2(double* sm, double dtc) { mech_cb6r5_ae7_aq::wsm::ebi_hrg2(sm, dtc); }
    static __device__ __forceinline__ void ebi_hrg3(double* ws, double dtc) { mech_cb6r5_ae7_aq::ebi_hrg3(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg3(double* sm, double dtc) { mech_cb6r5_ae7_aq::wsm::ebi_hrg3(sm, dtc); }
    static __device__ __forceinline__ void ebi_hrg4(double* ws, double dtc) { mech_cb6r5_ae7_aq::ebi_hrg4(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg4(double* sm, double dtc) { mech_cb6r5_ae7_aq::wsm::ebi_hrg4(sm, dtc); }
    static constexpr int EBIW_NRATE = mech_cb6r5_ae7_aq::EBIW_NRATE;
    static __device__ __forceinline__ const int* ebiw_rate_r() { return mech_cb6r5_ae7_aq::c_ebiw_rate_r; }
    static __device__ __forceinline__ const int* ebiw_rate_nf() { return mech_cb6r5_ae7_aq::c_ebiw_rate_nf; }
    static __device__ __forceinline__ const int* ebiw_rate_sp() { return mech_cb6r5_ae7_aq::c_ebiw_rate_sp; }
    static __device__ __forceinline__ const int* ebiw_pl_ptr() { return mech_cb6r5_ae7_aq::c_ebiw_pl_ptr; }
    static __device__ __forceinline__ const int* ebiw_pl_kind() { return mech_cb6r5_ae7_aq::c_ebiw_pl_kind; }
    static __device__ __forceinline__ const int* ebiw_pl_sp() { return mech_cb6r5_ae7_aq::c_ebiw_pl_sp; }
    static __device__ __forceinline__ const int* ebiw_pl_t0() { return mech_cb6r5_ae7_aq::c_ebiw_pl_t0; }
    static __device__ __forceinline__ const int* ebiw_term_r() { return mech_cb6r5_ae7_aq::c_ebiw_term_r; }
    static __device__ __forceinline__ const double* ebiw_term_c() { return mech_cb6r5_ae7_aq::c_ebiw_term_c; }
    static constexpr int GW_NACT = 349;
    static constexpr int GW_NEX = 268;
    static constexpr int GW_NFL = 22;
    static constexpr int GW_NBL = 19;
    static __device__ __forceinline__ const int* gw_act_r() { return mech_cb6r5_ae7_aq::c_gw_act_r; }
    static __device__ __forceinline__ const int* gw_act_sp() { return mech_cb6r5_ae7_aq::c_gw_act_sp; }
    static __device__ __forceinline__ const int* gw_sum_ptr() { return mech_cb6r5_ae7_aq::c_gw_sum_ptr; }
    static __device__ __forceinline__ const int* gw_sum_r() { return mech_cb6r5_ae7_aq::c_gw_sum_r; }
    static __device__ __forceinline__ const int* gw_sum_k() { return mech_cb6r5_ae7_aq::c_gw_sum_k; }
    static __device__ __forceinline__ const int* gw_lane_ptr() { return mech_cb6r5_ae7_aq::c_gw_lane_ptr; }
    static __device__ __forceinline__ const int* gw_lane_sp() { return mech_cb6r5_ae7_aq::c_gw_lane_sp; }
    static __device__ __forceinline__ const int* gw_ex_r() { return mech_cb6r5_ae7_aq::c_gw_ex_r; }
    static __device__ __forceinline__ const int* gw_ex_sp() { return mech_cb6r5_ae7_aq::c_gw_ex_sp; }
    static __device__ __forceinline__ const int* gw_ex_off() { return mech_cb6r5_ae7_aq::c_gw_ex_off; }
    static __device__ __forceinline__ const int* gw_asm_ptr() { return mech_cb6r5_ae7_aq::c_gw_asm_ptr; }
    static __device__ __forceinline__ const int* gw_asm_src() { return mech_cb6r5_ae7_aq::c_gw_asm_src; }
    static __device__ __forceinline__ const int* gw_asm_kind() { return mech_cb6r5_ae7_aq::c_gw_asm_kind; }
    static __device__ __forceinline__ const int* gw_piv_diag() { return mech_cb6r5_ae7_aq::c_gw_piv_diag; }
    static __device__ __forceinline__ const int* gw_lsc_ptr() { return mech_cb6r5_ae7_aq::c_gw_lsc_ptr; }
    static __device__ __forceinline__ const int* gw_lsc_st() { return mech_cb6r5_ae7_aq::c_gw_lsc_st; }
    static __device__ __forceinline__ const int* gw_up_ptr() { return mech_cb6r5_ae7_aq::c_gw_up_ptr; }
    static __device__ __forceinline__ const int* gw_up_ij() { return mech_cb6r5_ae7_aq::c_gw_up_ij; }
    static __device__ __forceinline__ const int* gw_up_ik() { return mech_cb6r5_ae7_aq::c_gw_up_ik; }
    static __device__ __forceinline__ const int* gw_up_kj() { return mech_cb6r5_ae7_aq::c_gw_up_kj; }
    static __device__ __forceinline__ const int* gw_fl_ptr() { return mech_cb6r5_ae7_aq::c_gw_fl_ptr; }
    static __device__ __forceinline__ const int* gw_fl_row() { return mech_cb6r5_ae7_aq::c_gw_fl_row; }
    static __device__ __forceinline__ const int* gw_bl_ptr() { return mech_cb6r5_ae7_aq::c_gw_bl_ptr; }
    static __device__ __forceinline__ const int* gw_bl_row() { return mech_cb6r5_ae7_aq::c_gw_bl_row; }
    static __device__ __forceinline__ const int* gw_fr_ptr() { return mech_cb6r5_ae7_aq::c_gw_fr_ptr; }
    static __device__ __forceinline__ const int* gw_fr_st() { return mech_cb6r5_ae7_aq::c_gw_fr_st; }
    static __device__ __forceinline__ const int* gw_fr_col() { return mech_cb6r5_ae7_aq::c_gw_fr_col; }
    static __device__ __forceinline__ const int* gw_br_ptr() { return mech_cb6r5_ae7_aq::c_gw_br_ptr; }
    static __device__ __forceinline__ const int* gw_br_st() { return mech_cb6r5_ae7_aq::c_gw_br_st; }
    static __device__ __forceinline__ const int* gw_br_col() { return mech_cb6r5_ae7_aq::c_gw_br_col; }
    static __device__ __forceinline__ const double* gw_sum_c() { return mech_cb6r5_ae7_aq::c_gw_sum_c; }
    static __device__ __forceinline__ const double* gw_asm_c() { return mech_cb6r5_ae7_aq::c_gw_asm_c; }
    static __device__ __forceinline__ void rconst(double* ws, double t, double p, double h, double sw, int sun,
                                                  const double* rj, const double* het) { mech_cb6r5_ae7_aq::rconst(ws, t, p, h, sw, sun, rj, het); }
};
}  // namespace mech_cb6r5_ae7_aq
