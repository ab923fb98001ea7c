// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
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
namespace mech_cracmm2 {
constexpr const char* NAME = "cracmm2";
constexpr int NSPEC = 189;
constexpr int NRXNS = 531;
constexpr int ISCHAN = 189;
constexpr int NPHOTAB = 32;
constexpr int NHETERO = 9;
constexpr int WS_ELEMS = 6958;
constexpr int OFF_Y = 0;
constexpr int OFF_YP = 189;
constexpr int OFF_YDOT = 378;
constexpr int OFF_F0 = 567;
constexpr int OFF_K1 = 756;
constexpr int OFF_K2 = 945;
constexpr int OFF_K3 = 1134;
constexpr int OFF_RKI = 1323;
constexpr int OFF_RXRAT = 1854;
constexpr int OFF_LU = 3484;
constexpr int OFF_VDIAG = 6769;
constexpr int IARRAY_DAY = 3284;
constexpr int IARRAY_NIGHT = 3199;
constexpr int EBI_OFF_YC = 3484;
constexpr int EBI_OFF_YC0 = 3673;
constexpr int EBI_OFF_YCP = 3862;
constexpr int EBI_OFF_PROD = 4051;
constexpr int EBI_OFF_LOSS = 4240;
constexpr int EBI_OFF_PNEG = 4429;
constexpr int ADJ_WS_ELEMS = 9001;
constexpr int ADJ_LAM = 6958;
constexpr int ADJ_MU1 = 7147;
constexpr int ADJ_MU2 = 7336;
constexpr int ADJ_MU3 = 7525;
constexpr int ADJ_PHI = 7714;
constexpr int ADJ_TMP = 7903;
constexpr int ADJ_EMIS = 8092;
constexpr int ADJ_GE = 8281;
constexpr int ADJ_GK = 8470;
constexpr int OFF_YAVE = 3295;
constexpr int GEAR_WS_ELEMS = 8281;
constexpr int GEAR_CNEW = 0;
constexpr int GEAR_GLOSS = 378;
constexpr int GEAR_DTLOS = 756;
constexpr int GEAR_CHOLD = 945;
constexpr int GEAR_CEST = 1134;
constexpr int GEAR_BLKCONC = 567;
constexpr int GEAR_CONC = 6958;
constexpr int GEAR_E = 189;
constexpr int GEAR_CAVEG = 3295;
constexpr int GEAR_CFINI = 8092;
constexpr int EBIW_YC = 0;
constexpr int EBIW_YC0 = 189;
constexpr int EBIW_YCP = 378;
constexpr int EBIW_PROD = 567;
constexpr int EBIW_LOSS = 756;
constexpr int EBIW_PNEG = 945;
constexpr int EBIW_NOTMAX = 1134;
constexpr int EBIW_RKI = 1323;
constexpr int EBIW_RXRAT = 1854;
constexpr int EBIW_ELEMS = 2385;
constexpr double FLOPS_STEP_DAY = 79988.0;
constexpr double FLOPS_STEP_NIGHT = 77148.0;
extern __constant__ int c_inew2old[189];
extern __constant__ int c_iold2new[189];
static const int h_inew2old[189] = {144, 147, 148, 184, 186, 47, 48, 49, 62, 67, 70, 72, 128, 129, 135, 142, 145, 146, 2, 149, 151, 153, 155, 157, 159, 161, 172, 176, 178, 183, 185, 187, 46, 143, 43, 54, 60, 8, 64, 66, 10, 74, 78, 79, 83, 86, 104, 105, 109, 131, 136, 76, 80, 45, 91, 101, 106, 110, 134, 50, 137, 162, 163, 164, 166, 168, 169, 171, 51, 81, 56, 125, 139, 1, 150, 152, 154, 156, 158, 160, 89, 99, 114, 116, 126, 127, 58, 75, 37, 92, 96, 97, 69, 108, 57, 111, 118, 71, 132, 133, 59, 36, 73, 68, 61, 65, 173, 177, 179, 188, 95, 130, 98, 53, 100, 41, 117, 85, 94, 102, 115, 20, 23, 88, 182, 3, 112, 113, 39, 27, 84, 87, 181, 119, 77, 34, 63, 44, 170, 35, 18, 122, 22, 24, 40, 175, 28, 167, 30, 180, 90, 138, 174, 121, 124, 140, 141, 9, 82, 165, 55, 93, 0, 29, 32, 25, 120, 26, 31, 52, 42, 33, 21, 123, 14, 103, 17, 13, 107, 38, 16, 19, 6, 12, 15, 5, 7, 11, 4};
static const int h_iold2new[189] = {162, 73, 18, 125, 188, 185, 182, 186, 37, 157, 40, 187, 183, 177, 174, 184, 180, 176, 140, 181, 121, 172, 142, 122, 143, 165, 167, 129, 146, 163, 148, 168, 164, 171, 135, 139, 101, 88, 179, 128, 144, 115, 170, 34, 137, 53, 32, 5, 6, 7, 59, 68, 169, 113, 35, 160, 70, 94, 86, 100, 36, 104, 8, 136, 38, 105, 39, 9, 103, 92, 10, 97, 11, 102, 41, 87, 51, 134, 42, 43, 52, 69, 158, 44, 130, 117, 45, 131, 123, 80, 150, 54, 89, 161, 118, 110, 90, 91, 112, 81, 114, 55, 119, 175, 46, 47, 56, 178, 93, 48, 57, 95, 126, 127, 82, 120, 83, 116, 96, 133, 166, 153, 141, 173, 154, 71, 84, 85, 12, 13, 111, 49, 98, 99, 58, 14, 50, 60, 151, 72, 155, 156, 15, 33, 0, 16, 17, 1, 2, 19, 74, 20, 75, 21, 76, 22, 77, 23, 78, 24, 79, 25, 61, 62, 63, 159, 64, 147, 65, 66, 138, 67, 26, 106, 152, 145, 27, 107, 28, 108, 149, 132, 124, 29, 3, 30, 4, 31, 109};
static const int h_cgrid_index[189] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 80, 51, 87, 22, 23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 119, 120, 41, 42, 43, 44, 45, 46, 47, 192, 48, 49, 53, 54, 55, 56, 57, 58, 59, 60, 61, 62, 63, 64, 69, 65, 66, 70, 67, 71, 73, 117, 116, 74, 107, 108, 118, 115, 105, 75, 76, 77, 82, 83, 84, 81, 91, 88, 92, 93, 94, 95, 96, 97, 98, 99, 100, 101, 102, 103, 104, 106, 110, 111, 112, 113, 114, 121, 122, 123, 78, 79, 85, 86, 124, 89, 178, 171, 133, 177, 173, 125, 126, 90, 134, 135, 127, 128, 129, 131, 132, 130, 136, 138, 166, 137, 172, 175, 193, 109, 267, 184, 268, 269, 270, 153, 159, 152, 158, 151, 157, 150, 156, 149, 155, 148, 154, 50, 165, 164, 163, 176, 162, 174, 161, 160, 169, 52, 142, 144, 167, 170, 141, 143, 139, 140, 168, 179, 180, 181, 271, 194, 272, 68, 72};
static const int h_convert[189] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0};
static const double h_molwt[189] = {48.0, 16.0, 16.0, 34.0, 17.0, 46.0, 30.0, 62.0, 47.0, 63.0, 79.0, 33.0, 30.0, 28.0, 44.0, 47.0, 58.0, 61.0, 58.0, 75.0, 84.1, 86.0, 168.0, 173.27, 168.0, 72.1, 74.0, 70.0, 101.0, 1.0, 70.1, 58.0, 72.0, 98.0, 112.1, 106.0, 139.0, 48.0, 62.0, 186.2, 176.2, 76.0, 119.0, 121.0, 215.0, 265.0, 108.0, 64.0, 98.0, 98.0, 30.1, 44.1, 75.0, 200.0, 72.1, 103.0, 28.1, 77.0, 42.0, 91.0, 70.1, 119.0, 26.0, 46.0, 78.11, 159.12, 110.1, 92.14, 173.14, 136.2, 106.2, 187.17, 106.2, 187.17, 68.1, 147.0, 162.1, 117.0, 118.0, 118.1, 150.1, 195.1, 60.0, 136.4, 185.0, 185.0, 136.3, 185.0, 185.0, 199.0, 89.0, 217.0, 89.0, 103.0, 117.0, 119.0, 119.0, 133.0, 84.0, 137.0, 125.0, 124.1, 123.0, 32.0, 46.1, 62.1, 102.0, 60.2, 91.0, 135.0, 147.1, 172.0, 136.0, 136.0, 230.0, 230.0, 230.0, 230.0, 155.0, 250.0, 158.2, 190.2, 100.1, 186.3, 202.3, 123.0, 109.0, 402.0, 247.0, 75.4, 56.1, 54.1, 103.0, 96.1, 145.1, 76.1, 204.4, 298.4, 282.4, 253.4, 242.4, 202.3, 66.4, 118.1, 136.2, 96.0, 216.2, 168.1, 150.1, 184.37, 215.36, 198.39, 229.38, 254.5, 285.49, 296.58, 327.57, 338.66, 369.65, 380.75, 411.74, 142.28, 231.36, 245.38, 301.49, 200.3, 343.57, 270.5, 385.65, 427.73, 312.5, 189.27, 176.3, 257.3, 232.3, 230.3, 190.33, 271.33, 128.17, 209.17, 194.2, 170.3, 142.2, 16.0, 215.0, 250.0, 265.0, 104.0, 153.0};
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
__device__ void gear_pdecomp_0_30(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_31(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_32(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_33(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_34(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_35(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_36(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_37(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_38(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_39(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_40(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_41(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_42(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_43(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_44(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_45(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_46(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_47(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_48(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_49(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_50(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_51(double* __restrict__ ws, double r1delt);
__device__ void gear_pdecomp_0_52(double* __restrict__ ws, double r1delt);
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
__device__ void jacdecomp_0_30(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_31(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_32(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_33(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_34(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_35(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_36(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_37(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_38(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_39(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_40(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_41(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_42(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_43(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_44(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_45(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_46(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_47(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_48(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_49(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_50(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_51(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_0_52(double* __restrict__ ws, double gdtinv);
__device__ void solve_0_0(double* __restrict__ ws, int rhs);
__device__ void solve_0_1(double* __restrict__ ws, int rhs);
__device__ void solve_0_2(double* __restrict__ ws, int rhs);
__device__ void solve_0_3(double* __restrict__ ws, int rhs);
__device__ void solve_0_4(double* __restrict__ ws, int rhs);
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
__device__ void jacdecomp_1_30(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_31(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_32(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_33(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_34(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_35(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_36(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_37(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_38(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_39(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_40(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_41(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_42(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_43(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_44(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_45(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_46(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_47(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_48(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_49(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_50(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_51(double* __restrict__ ws, double gdtinv);
__device__ void jacdecomp_1_52(double* __restrict__ ws, double gdtinv);
__device__ void solve_1_0(double* __restrict__ ws, int rhs);
__device__ void solve_1_1(double* __restrict__ ws, int rhs);
__device__ void solve_1_2(double* __restrict__ ws, int rhs);
__device__ void solve_1_3(double* __restrict__ ws, int rhs);
__device__ void solve_1_4(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_0(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_1(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_2(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_3(double* __restrict__ ws, int rhs);
__device__ void solve_t_0_4(double* __restrict__ ws, int rhs);
__device__ void adj_jtv_0_0(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_1(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_2(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_3(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_4(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_5(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_6(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_7(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_8(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_9(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_10(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_11(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_0_12(double* __restrict__ ws, int yoff, int phioff, int outoff);
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
__device__ void adj_hess3_0_19(double* __restrict__ ws);
__device__ void adj_hess3_0_20(double* __restrict__ ws);
__device__ void adj_hess3_0_21(double* __restrict__ ws);
__device__ void adj_hess3_0_22(double* __restrict__ ws);
__device__ void adj_hess3_0_23(double* __restrict__ ws);
__device__ void adj_hess3_0_24(double* __restrict__ ws);
__device__ void adj_hess3_0_25(double* __restrict__ ws);
__device__ void adj_hess3_0_26(double* __restrict__ ws);
__device__ void adj_hess3_0_27(double* __restrict__ ws);
__device__ void adj_hess3_0_28(double* __restrict__ ws);
__device__ void adj_hess3_0_29(double* __restrict__ ws);
__device__ void adj_hess3_0_30(double* __restrict__ ws);
__device__ void adj_hess3_0_31(double* __restrict__ ws);
__device__ void adj_hess3_0_32(double* __restrict__ ws);
__device__ void solve_t_1_0(double* __restrict__ ws, int rhs);
__device__ void solve_t_1_1(double* __restrict__ ws, int rhs);
__device__ void solve_t_1_2(double* __restrict__ ws, int rhs);
__device__ void solve_t_1_3(double* __restrict__ ws, int rhs);
__device__ void solve_t_1_4(double* __restrict__ ws, int rhs);
__device__ void adj_jtv_1_0(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_1(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_2(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_3(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_4(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_5(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_6(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_7(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_8(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_9(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_10(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_11(double* __restrict__ ws, int yoff, int phioff, int outoff);
__device__ void adj_jtv_1_12(double* __restrict__ ws, int yoff, int phioff, int outoff);
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
__device__ void adj_hess3_1_17(double* __restrict__ ws);
__device__ void adj_hess3_1_18(double* __restrict__ ws);
__device__ void adj_hess3_1_19(double* __restrict__ ws);
__device__ void adj_hess3_1_20(double* __restrict__ ws);
__device__ void adj_hess3_1_21(double* __restrict__ ws);
__device__ void adj_hess3_1_22(double* __restrict__ ws);
__device__ void adj_hess3_1_23(double* __restrict__ ws);
__device__ void adj_hess3_1_24(double* __restrict__ ws);
__device__ void adj_hess3_1_25(double* __restrict__ ws);
__device__ void adj_hess3_1_26(double* __restrict__ ws);
__device__ void adj_hess3_1_27(double* __restrict__ ws);
__device__ void adj_hess3_1_28(double* __restrict__ ws);
__device__ void adj_hess3_1_29(double* __restrict__ ws);
__device__ void adj_hess3_1_30(double* __restrict__ ws);
__device__ void ddm_jv_0_0(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_1(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_2(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_3(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_4(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_5(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_6(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_7(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_8(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_0_9(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_src_0_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_2(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_3(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_4(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_5(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_6(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_7(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_8(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_0_9(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_jv_1_0(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_1(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_2(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_3(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_4(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_5(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_6(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_7(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_8(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_jv_1_9(double* __restrict__ ws, int yoff, int voff, int outoff);
__device__ void ddm_src_1_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_2(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_3(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_4(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_5(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_6(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_7(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_8(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
__device__ void ddm_src_1_9(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff);
extern __device__ const int c_gw_act_r[531];
extern __device__ const int c_gw_act_sp[1593];
extern __device__ const int c_gw_sum_ptr[190];
extern __device__ const int c_gw_sum_r[3238];
extern __device__ const int c_gw_sum_k[3238];
extern __device__ const int c_gw_lane_ptr[33];
extern __device__ const int c_gw_lane_sp[189];
extern __device__ const int c_gw_ex_r[455];
extern __device__ const int c_gw_ex_sp[1365];
extern __device__ const int c_gw_ex_off[455];
extern __device__ const int c_gw_asm_ptr[3286];
extern __device__ const int c_gw_asm_src[6231];
extern __device__ const int c_gw_asm_kind[6231];
extern __device__ const int c_gw_piv_diag[189];
extern __device__ const int c_gw_lsc_ptr[190];
extern __device__ const int c_gw_lsc_st[1968];
extern __device__ const int c_gw_up_ptr[190];
extern __device__ const int c_gw_up_ij[15259];
extern __device__ const int c_gw_up_ik[15259];
extern __device__ const int c_gw_up_kj[15259];
extern __device__ const int c_gw_fl_ptr[30];
extern __device__ const int c_gw_fl_row[189];
extern __device__ const int c_gw_bl_ptr[26];
extern __device__ const int c_gw_bl_row[189];
extern __device__ const int c_gw_fr_ptr[190];
extern __device__ const int c_gw_fr_st[1968];
extern __device__ const int c_gw_fr_col[1968];
extern __device__ const int c_gw_br_ptr[190];
extern __device__ const int c_gw_br_st[1127];
extern __device__ const int c_gw_br_col[1127];
extern __device__ const double c_gw_sum_c[3238];
extern __device__ const double c_gw_asm_c[6231];
constexpr int EBI_N_EBISP = 176;
constexpr double EBI_DELTAT = 2.5;
constexpr int EBI_NEBITER = 1000;
constexpr int EBI_NPNEG = 0;
extern __constant__ int c_ebi_ebisp[176];
extern __constant__ double c_ebi_rtol[189];
extern __constant__ int c_ebi_pneg[1];
__device__ void ebi_hrrates(double* __restrict__ ws);
__device__ void ebi_hrprodloss(double* __restrict__ ws);
__device__ void ebi_hrg1(double* __restrict__ ws, double dtc);
__device__ void ebi_hrg2(double* __restrict__ ws, double dtc);
__device__ void ebi_hrg3(double* __restrict__ ws, double dtc);
__device__ void ebi_hrg4(double* __restrict__ ws, double dtc);
constexpr int EBIW_NRATE = 510;
constexpr int EBIW_NPL = 352;
constexpr int EBIW_NTERM = 2196;
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
    gear_pdecomp_0_30(ws, r1delt);
    gear_pdecomp_0_31(ws, r1delt);
    gear_pdecomp_0_32(ws, r1delt);
    gear_pdecomp_0_33(ws, r1delt);
    gear_pdecomp_0_34(ws, r1delt);
    gear_pdecomp_0_35(ws, r1delt);
    gear_pdecomp_0_36(ws, r1delt);
    gear_pdecomp_0_37(ws, r1delt);
    gear_pdecomp_0_38(ws, r1delt);
    gear_pdecomp_0_39(ws, r1delt);
    gear_pdecomp_0_40(ws, r1delt);
    gear_pdecomp_0_41(ws, r1delt);
    gear_pdecomp_0_42(ws, r1delt);
    gear_pdecomp_0_43(ws, r1delt);
    gear_pdecomp_0_44(ws, r1delt);
    gear_pdecomp_0_45(ws, r1delt);
    gear_pdecomp_0_46(ws, r1delt);
    gear_pdecomp_0_47(ws, r1delt);
    gear_pdecomp_0_48(ws, r1delt);
    gear_pdecomp_0_49(ws, r1delt);
    gear_pdecomp_0_50(ws, r1delt);
    gear_pdecomp_0_51(ws, r1delt);
    gear_pdecomp_0_52(ws, r1delt);
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
    jacdecomp_0_30(ws, gdtinv);
    jacdecomp_0_31(ws, gdtinv);
    jacdecomp_0_32(ws, gdtinv);
    jacdecomp_0_33(ws, gdtinv);
    jacdecomp_0_34(ws, gdtinv);
    jacdecomp_0_35(ws, gdtinv);
    jacdecomp_0_36(ws, gdtinv);
    jacdecomp_0_37(ws, gdtinv);
    jacdecomp_0_38(ws, gdtinv);
    jacdecomp_0_39(ws, gdtinv);
    jacdecomp_0_40(ws, gdtinv);
    jacdecomp_0_41(ws, gdtinv);
    jacdecomp_0_42(ws, gdtinv);
    jacdecomp_0_43(ws, gdtinv);
    jacdecomp_0_44(ws, gdtinv);
    jacdecomp_0_45(ws, gdtinv);
    jacdecomp_0_46(ws, gdtinv);
    jacdecomp_0_47(ws, gdtinv);
    jacdecomp_0_48(ws, gdtinv);
    jacdecomp_0_49(ws, gdtinv);
    jacdecomp_0_50(ws, gdtinv);
    jacdecomp_0_51(ws, gdtinv);
    jacdecomp_0_52(ws, gdtinv);
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
    if (go) jacdecomp_0_30(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_31(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_32(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_33(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_34(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_35(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_36(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_37(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_38(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_39(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_40(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_41(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_42(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_43(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_44(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_45(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_46(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_47(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_48(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_49(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_50(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_51(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_0_52(ws, gdtinv);
    __syncthreads();
}
__device__ __forceinline__ void solve_0(double* __restrict__ ws, int rhs)
{
    solve_0_0(ws, rhs);
    solve_0_1(ws, rhs);
    solve_0_2(ws, rhs);
    solve_0_3(ws, rhs);
    solve_0_4(ws, rhs);
}
__device__ __forceinline__ void solve_0_sync(double* __restrict__ ws, int rhs, bool go)
{
    if (go) solve_0_0(ws, rhs);
    __syncthreads();
    if (go) solve_0_1(ws, rhs);
    __syncthreads();
    if (go) solve_0_2(ws, rhs);
    __syncthreads();
    if (go) solve_0_3(ws, rhs);
    __syncthreads();
    if (go) solve_0_4(ws, rhs);
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
    jacdecomp_1_30(ws, gdtinv);
    jacdecomp_1_31(ws, gdtinv);
    jacdecomp_1_32(ws, gdtinv);
    jacdecomp_1_33(ws, gdtinv);
    jacdecomp_1_34(ws, gdtinv);
    jacdecomp_1_35(ws, gdtinv);
    jacdecomp_1_36(ws, gdtinv);
    jacdecomp_1_37(ws, gdtinv);
    jacdecomp_1_38(ws, gdtinv);
    jacdecomp_1_39(ws, gdtinv);
    jacdecomp_1_40(ws, gdtinv);
    jacdecomp_1_41(ws, gdtinv);
    jacdecomp_1_42(ws, gdtinv);
    jacdecomp_1_43(ws, gdtinv);
    jacdecomp_1_44(ws, gdtinv);
    jacdecomp_1_45(ws, gdtinv);
    jacdecomp_1_46(ws, gdtinv);
    jacdecomp_1_47(ws, gdtinv);
    jacdecomp_1_48(ws, gdtinv);
    jacdecomp_1_49(ws, gdtinv);
    jacdecomp_1_50(ws, gdtinv);
    jacdecomp_1_51(ws, gdtinv);
    jacdecomp_1_52(ws, gdtinv);
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
    if (go) jacdecomp_1_30(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_31(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_32(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_33(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_34(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_35(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_36(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_37(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_38(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_39(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_40(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_41(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_42(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_43(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_44(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_45(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_46(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_47(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_48(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_49(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_50(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_51(ws, gdtinv);
    __syncthreads();
    if (go) jacdecomp_1_52(ws, gdtinv);
    __syncthreads();
}
__device__ __forceinline__ void solve_1(double* __restrict__ ws, int rhs)
{
    solve_1_0(ws, rhs);
    solve_1_1(ws, rhs);
    solve_1_2(ws, rhs);
    solve_1_3(ws, rhs);
    solve_1_4(ws, rhs);
}
__device__ __forceinline__ void solve_1_sync(double* __restrict__ ws, int rhs, bool go)
{
    if (go) solve_1_0(ws, rhs);
    __syncthreads();
    if (go) solve_1_1(ws, rhs);
    __syncthreads();
    if (go) solve_1_2(ws, rhs);
    __syncthreads();
    if (go) solve_1_3(ws, rhs);
    __syncthreads();
    if (go) solve_1_4(ws, rhs);
    __syncthreads();
}
__device__ __forceinline__ void solve_t_0(double* __restrict__ ws, int rhs)
{
    solve_t_0_0(ws, rhs);
    solve_t_0_1(ws, rhs);
    solve_t_0_2(ws, rhs);
    solve_t_0_3(ws, rhs);
    solve_t_0_4(ws, rhs);
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
    adj_jtv_0_8(ws, yoff, phioff, outoff);
    adj_jtv_0_9(ws, yoff, phioff, outoff);
    adj_jtv_0_10(ws, yoff, phioff, outoff);
    adj_jtv_0_11(ws, yoff, phioff, outoff);
    adj_jtv_0_12(ws, yoff, phioff, outoff);
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
    adj_hess3_0_19(ws);
    adj_hess3_0_20(ws);
    adj_hess3_0_21(ws);
    adj_hess3_0_22(ws);
    adj_hess3_0_23(ws);
    adj_hess3_0_24(ws);
    adj_hess3_0_25(ws);
    adj_hess3_0_26(ws);
    adj_hess3_0_27(ws);
    adj_hess3_0_28(ws);
    adj_hess3_0_29(ws);
    adj_hess3_0_30(ws);
    adj_hess3_0_31(ws);
    adj_hess3_0_32(ws);
}
__device__ __forceinline__ void solve_t_1(double* __restrict__ ws, int rhs)
{
    solve_t_1_0(ws, rhs);
    solve_t_1_1(ws, rhs);
    solve_t_1_2(ws, rhs);
    solve_t_1_3(ws, rhs);
    solve_t_1_4(ws, rhs);
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
    adj_jtv_1_7(ws, yoff, phioff, outoff);
    adj_jtv_1_8(ws, yoff, phioff, outoff);
    adj_jtv_1_9(ws, yoff, phioff, outoff);
    adj_jtv_1_10(ws, yoff, phioff, outoff);
    adj_jtv_1_11(ws, yoff, phioff, outoff);
    adj_jtv_1_12(ws, yoff, phioff, outoff);
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
    adj_hess3_1_17(ws);
    adj_hess3_1_18(ws);
    adj_hess3_1_19(ws);
    adj_hess3_1_20(ws);
    adj_hess3_1_21(ws);
    adj_hess3_1_22(ws);
    adj_hess3_1_23(ws);
    adj_hess3_1_24(ws);
    adj_hess3_1_25(ws);
    adj_hess3_1_26(ws);
    adj_hess3_1_27(ws);
    adj_hess3_1_28(ws);
    adj_hess3_1_29(ws);
    adj_hess3_1_30(ws);
}
__device__ __forceinline__ void ddm_jv_0(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    ddm_jv_0_0(ws, yoff, voff, outoff);
    ddm_jv_0_1(ws, yoff, voff, outoff);
    ddm_jv_0_2(ws, yoff, voff, outoff);
    ddm_jv_0_3(ws, yoff, voff, outoff);
    ddm_jv_0_4(ws, yoff, voff, outoff);
    ddm_jv_0_5(ws, yoff, voff, outoff);
    ddm_jv_0_6(ws, yoff, voff, outoff);
    ddm_jv_0_7(ws, yoff, voff, outoff);
    ddm_jv_0_8(ws, yoff, voff, outoff);
    ddm_jv_0_9(ws, yoff, voff, outoff);
}
__device__ __forceinline__ void ddm_src_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    ddm_src_0_0(ws, mask, scale, outoff);
    ddm_src_0_1(ws, mask, scale, outoff);
    ddm_src_0_2(ws, mask, scale, outoff);
    ddm_src_0_3(ws, mask, scale, outoff);
    ddm_src_0_4(ws, mask, scale, outoff);
    ddm_src_0_5(ws, mask, scale, outoff);
    ddm_src_0_6(ws, mask, scale, outoff);
    ddm_src_0_7(ws, mask, scale, outoff);
    ddm_src_0_8(ws, mask, scale, outoff);
    ddm_src_0_9(ws, mask, scale, outoff);
}
__device__ __forceinline__ void ddm_jv_1(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    ddm_jv_1_0(ws, yoff, voff, outoff);
    ddm_jv_1_1(ws, yoff, voff, outoff);
    ddm_jv_1_2(ws, yoff, voff, outoff);
    ddm_jv_1_3(ws, yoff, voff, outoff);
    ddm_jv_1_4(ws, yoff, voff, outoff);
    ddm_jv_1_5(ws, yoff, voff, outoff);
    ddm_jv_1_6(ws, yoff, voff, outoff);
    ddm_jv_1_7(ws, yoff, voff, outoff);
    ddm_jv_1_8(ws, yoff, voff, outoff);
    ddm_jv_1_9(ws, yoff, voff, outoff);
}
__device__ __forceinline__ void ddm_src_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    ddm_src_1_0(ws, mask, scale, outoff);
    ddm_src_1_1(ws, mask, scale, outoff);
    ddm_src_1_2(ws, mask, scale, outoff);
    ddm_src_1_3(ws, mask, scale, outoff);
    ddm_src_1_4(ws, mask, scale, outoff);
    ddm_src_1_5(ws, mask, scale, outoff);
    ddm_src_1_6(ws, mask, scale, outoff);
    ddm_src_1_7(ws, mask, scale, outoff);
    ddm_src_1_8(ws, mask, scale, outoff);
    ddm_src_1_9(ws, mask, scale, outoff);
}
struct Traits {
    static constexpr int NSPEC = mech_cracmm2::NSPEC;
    static constexpr int NRXNS = mech_cracmm2::NRXNS;
    static constexpr int ISCHAN = mech_cracmm2::ISCHAN;
    static constexpr int NPHOTAB = mech_cracmm2::NPHOTAB;
    static constexpr int NHETERO = mech_cracmm2::NHETERO;
    static constexpr int WS_ELEMS = mech_cracmm2::WS_ELEMS;
    static constexpr int OFF_Y = mech_cracmm2::OFF_Y;
    static constexpr int OFF_YP = mech_cracmm2::OFF_YP;
    static constexpr int OFF_YDOT = mech_cracmm2::OFF_YDOT;
    static constexpr int OFF_F0 = mech_cracmm2::OFF_F0;
    static constexpr int OFF_K1 = mech_cracmm2::OFF_K1;
    static constexpr int OFF_K2 = mech_cracmm2::OFF_K2;
    static constexpr int OFF_K3 = mech_cracmm2::OFF_K3;
    static constexpr int OFF_RKI = mech_cracmm2::OFF_RKI;
    static constexpr int OFF_RXRAT = mech_cracmm2::OFF_RXRAT;
    static constexpr int OFF_LU = mech_cracmm2::OFF_LU;
    static constexpr int OFF_VDIAG = mech_cracmm2::OFF_VDIAG;
    static constexpr int IARRAY_DAY = mech_cracmm2::IARRAY_DAY;
    static constexpr int IARRAY_NIGHT = mech_cracmm2::IARRAY_NIGHT;
    static constexpr int EBI_OFF_YC = mech_cracmm2::EBI_OFF_YC;
    static constexpr int EBI_OFF_YC0 = mech_cracmm2::EBI_OFF_YC0;
    static constexpr int EBI_OFF_YCP = mech_cracmm2::EBI_OFF_YCP;
    static constexpr int EBI_OFF_PROD = mech_cracmm2::EBI_OFF_PROD;
    static constexpr int EBI_OFF_LOSS = mech_cracmm2::EBI_OFF_LOSS;
    static constexpr int EBI_OFF_PNEG = mech_cracmm2::EBI_OFF_PNEG;
    static constexpr int ADJ_WS_ELEMS = mech_cracmm2::ADJ_WS_ELEMS;
    static constexpr int ADJ_LAM = mech_cracmm2::ADJ_LAM;
    static constexpr int ADJ_MU1 = mech_cracmm2::ADJ_MU1;
    static constexpr int ADJ_MU2 = mech_cracmm2::ADJ_MU2;
    static constexpr int ADJ_MU3 = mech_cracmm2::ADJ_MU3;
    static constexpr int ADJ_PHI = mech_cracmm2::ADJ_PHI;
    static constexpr int ADJ_TMP = mech_cracmm2::ADJ_TMP;
    static constexpr int ADJ_EMIS = mech_cracmm2::ADJ_EMIS;
    static constexpr int ADJ_GE = mech_cracmm2::ADJ_GE;
    static constexpr int ADJ_GK = mech_cracmm2::ADJ_GK;
    static constexpr int OFF_YAVE = mech_cracmm2::OFF_YAVE;
    static constexpr int GEAR_WS_ELEMS = mech_cracmm2::GEAR_WS_ELEMS;
    static constexpr int GEAR_CNEW = mech_cracmm2::GEAR_CNEW;
    static constexpr int GEAR_GLOSS = mech_cracmm2::GEAR_GLOSS;
    static constexpr int GEAR_DTLOS = mech_cracmm2::GEAR_DTLOS;
    static constexpr int GEAR_CHOLD = mech_cracmm2::GEAR_CHOLD;
    static constexpr int GEAR_CEST = mech_cracmm2::GEAR_CEST;
    static constexpr int GEAR_BLKCONC = mech_cracmm2::GEAR_BLKCONC;
    static constexpr int GEAR_CONC = mech_cracmm2::GEAR_CONC;
    static constexpr int GEAR_E = mech_cracmm2::GEAR_E;
    static constexpr int GEAR_CAVEG = mech_cracmm2::GEAR_CAVEG;
    static constexpr int GEAR_CFINI = mech_cracmm2::GEAR_CFINI;
    static constexpr int EBIW_YC = mech_cracmm2::EBIW_YC;
    static constexpr int EBIW_YC0 = mech_cracmm2::EBIW_YC0;
    static constexpr int EBIW_YCP = mech_cracmm2::EBIW_YCP;
    static constexpr int EBIW_PROD = mech_cracmm2::EBIW_PROD;
    static constexpr int EBIW_LOSS = mech_cracmm2::EBIW_LOSS;
    static constexpr int EBIW_PNEG = mech_cracmm2::EBIW_PNEG;
    static constexpr int EBIW_NOTMAX = mech_cracmm2::EBIW_NOTMAX;
    static constexpr int EBIW_RKI = mech_cracmm2::EBIW_RKI;
    static constexpr int EBIW_RXRAT = mech_cracmm2::EBIW_RXRAT;
    static constexpr int EBIW_ELEMS = mech_cracmm2::EBIW_ELEMS;
    static constexpr const char* name() { return mech_cracmm2::NAME; }
    static __device__ __forceinline__ int iold2new(int s) { return mech_cracmm2::c_iold2new[s]; }
    static __device__ __forceinline__ int inew2old(int i) { return mech_cracmm2::c_inew2old[i]; }
    static __device__ __forceinline__ void feval_0(double* ws, int s, int t) { mech_cracmm2::feval_0(ws, s, t); }
    static __device__ __forceinline__ void explic_0(double* ws) { mech_cracmm2::explic_0(ws); }
    static __device__ __forceinline__ void gear_explic_0(double* ws) { mech_cracmm2::gear_explic_0(ws); }
    static __device__ __forceinline__ void gear_pdecomp_0(double* ws, double r) { mech_cracmm2::gear_pdecomp_0(ws, r); }
    static __device__ __forceinline__ void jacdecomp_0(double* ws, double g) { mech_cracmm2::jacdecomp_0(ws, g); }
    static __device__ __forceinline__ void solve_0(double* ws, int r) { mech_cracmm2::solve_0(ws, r); }
    static __device__ __forceinline__ void jacdecomp_0_sync(double* ws, double g, bool go) { mech_cracmm2::jacdecomp_0_sync(ws, g, go); }
    static __device__ __forceinline__ void solve_0_sync(double* ws, int r, bool go) { mech_cracmm2::solve_0_sync(ws, r, go); }
    static __device__ __forceinline__ void solve_t_0(double* ws, int r) { mech_cracmm2::solve_t_0(ws, r); }
    static __device__ __forceinline__ void adj_jtv_0(double* ws, int y, int phi, int out) { mech_cracmm2::adj_jtv_0(ws, y, phi, out); }
    static __device__ __forceinline__ void adj_hess3_0(double* ws) { mech_cracmm2::adj_hess3_0(ws); }
    static __device__ __forceinline__ void ddm_jv_0(double* ws, int y, int v, int out) { mech_cracmm2::ddm_jv_0(ws, y, v, out); }
    static __device__ __forceinline__ void ddm_src_0(double* ws, const unsigned char* mk, double sc, int out) { mech_cracmm2::ddm_src_0(ws, mk, sc, out); }
    static __device__ __forceinline__ void feval_1(double* ws, int s, int t) { mech_cracmm2::feval_1(ws, s, t); }
    static __device__ __forceinline__ void explic_1(double* ws) { mech_cracmm2::explic_1(ws); }
    static __device__ __forceinline__ void jacdecomp_1(double* ws, double g) { mech_cracmm2::jacdecomp_1(ws, g); }
    static __device__ __forceinline__ void solve_1(double* ws, int r) { mech_cracmm2::solve_1(ws, r); }
    static __device__ __forceinline__ void jacdecomp_1_sync(double* ws, double g, bool go) { mech_cracmm2::jacdecomp_1_sync(ws, g, go); }
    static __device__ __forceinline__ void solve_1_sync(double* ws, int r, bool go) { mech_cracmm2::solve_1_sync(ws, r, go); }
    static __device__ __forceinline__ void solve_t_1(double* ws, int r) { mech_cracmm2::solve_t_1(ws, r); }
    static __device__ __forceinline__ void adj_jtv_1(double* ws, int y, int phi, int out) { mech_cracmm2::adj_jtv_1(ws, y, phi, out); }
    static __device__ __forceinline__ void adj_hess3_1(double* ws) { mech_cracmm2::adj_hess3_1(ws); }
    static __device__ __forceinline__ void ddm_jv_1(double* ws, int y, int v, int out) { mech_cracmm2::ddm_jv_1(ws, y, v, out); }
    static __device__ __forceinline__ void ddm_src_1(double* ws, const unsigned char* mk, double sc, int out) { mech_cracmm2::ddm_src_1(ws, mk, sc, out); }
    static constexpr int EBI_N_EBISP = mech_cracmm2::EBI_N_EBISP;
    static constexpr int EBI_NEBITER = mech_cracmm2::EBI_NEBITER;
    static constexpr int EBI_NPNEG = mech_cracmm2::EBI_NPNEG;
    static constexpr double EBI_DELTAT = mech_cracmm2::EBI_DELTAT;
    static __device__ __forceinline__ int ebi_ebisp(int e) { return mech_cracmm2::c_ebi_ebisp[e]; }
    static __device__ __forceinline__ double ebi_rtol(int i) { return mech_cracmm2::c_ebi_rtol[i]; }
    static __device__ __forceinline__ int ebi_pneg(int k) { return mech_cracmm2::c_ebi_pneg[k]; }
    static __device__ __forceinline__ void ebi_hrrates(double* ws) { mech_cracmm2::ebi_hrrates(ws); }
    static __device__ __forceinline__ void ebi_hrprodloss(double* ws) { mech_cracmm2::ebi_hrprodloss(ws); }
    static __device__ __forceinline__ void ebi_hrg1(double* ws, double dtc) { mech_cracmm2::ebi_hrg1(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg1(double* sm, double dtc) { mech_cracmm2::wsm::ebi_hrg1(sm, dtc); }
    static __device__ __forceinline__ void ebi_hrg2(double* ws, double dtc) { mech_cracmm2::ebi_hrg2(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg2(double* sm, double dtc) { mech_cracmm2::wsm::ebi_hrg2(sm, dtc); }
    static __device__ __forceinline__ void ebi_hrg3(double* ws, double dtc) { mech_cracmm2::ebi_hrg3(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg3(double* sm, double dtc) { mech_cracmm2::wsm::ebi_hrg3(sm, dtc); }
    static __device__ __forceinline__ void ebi_hrg4(double* ws, double dtc) { mech_cracmm2::ebi_hrg4(ws, dtc); }
    static __device__ __forceinline__ void ebiw_hrg4(double* sm, double dtc) { mech_cracmm2::wsm::ebi_hrg4(sm, dtc); }
    static constexpr int EBIW_NRATE = mech_cracmm2::EBIW_NRATE;
    static __device__ __forceinline__ const int* ebiw_rate_r() { return mech_cracmm2::c_ebiw_rate_r; }
    static __device__ __forceinline__ const int* ebiw_rate_nf() { return mech_cracmm2::c_ebiw_rate_nf; }
    static __device__ __forceinline__ const int* ebiw_rate_sp() { return mech_cracmm2::c_ebiw_rate_sp; }
    static __device__ __forceinline__ const int* ebiw_pl_ptr() { return mech_cracmm2::c_ebiw_pl_ptr; }
    static __device__ __forceinline__ const int* ebiw_pl_kind() { return mech_cracmm2::c_ebiw_pl_kind; }
    static __device__ __forceinline__ const int* ebiw_pl_sp() { return mech_cracmm2::c_ebiw_pl_sp; }
    static __device__ __forceinline__ const int* ebiw_pl_t0() { return mech_cracmm2::c_ebiw_pl_t0; }
    static __device__ __forceinline__ const int* ebiw_term_r() { return mech_cracmm2::c_ebiw_term_r; }
    static __device__ __forceinline__ const double* ebiw_term_c() { return mech_cracmm2::c_ebiw_term_c; }
    static constexpr int GW_NACT = 531;
    static constexpr int GW_NEX = 455;
    static constexpr int GW_NFL = 29;
    static constexpr int GW_NBL = 25;
    static __device__ __forceinline__ const int* gw_act_r() { return mech_cracmm2::c_gw_act_r; }
    static __device__ __forceinline__ const int* gw_act_sp() { return mech_cracmm2::c_gw_act_sp; }
    static __device__ __forceinline__ const int* gw_sum_ptr() { return mech_cracmm2::c_gw_sum_ptr; }
    static __device__ __forceinline__ const int* gw_sum_r() { return mech_cracmm2::c_gw_sum_r; }
    static __device__ __forceinline__ const int* gw_sum_k() { return mech_cracmm2::c_gw_sum_k; }
    static __device__ __forceinline__ const int* gw_lane_ptr() { return mech_cracmm2::c_gw_lane_ptr; }
    static __device__ __forceinline__ const int* gw_lane_sp() { return mech_cracmm2::c_gw_lane_sp; }
    static __device__ __forceinline__ const int* gw_ex_r() { return mech_cracmm2::c_gw_ex_r; }
    static __device__ __forceinline__ const int* gw_ex_sp() { return mech_cracmm2::c_gw_ex_sp; }
    static __device__ __forceinline__ const int* gw_ex_off() { return mech_cracmm2::c_gw_ex_off; }
    static __device__ __forceinline__ const int* gw_asm_ptr() { return mech_cracmm2::c_gw_asm_ptr; }
    static __device__ __forceinline__ const int* gw_asm_src() { return mech_cracmm2::c_gw_asm_src; }
    static __device__ __forceinline__ const int* gw_asm_kind() { return mech_cracmm2::c_gw_asm_kind; }
    static __device__ __forceinline__ const int* gw_piv_diag() { return mech_cracmm2::c_gw_piv_diag; }
    static __device__ __forceinline__ const int* gw_lsc_ptr() { return mech_cracmm2::c_gw_lsc_ptr; }
    static __device__ __forceinline__ const int* gw_lsc_st() { return mech_cracmm2::c_gw_lsc_st; }
    static __device__ __forceinline__ const int* gw_up_ptr() { return mech_cracmm2::c_gw_up_ptr; }
    static __device__ __forceinline__ const int* gw_up_ij() { return mech_cracmm2::c_gw_up_ij; }
    static __device__ __forceinline__ const int* gw_up_ik() { return mech_cracmm2::c_gw_up_ik; }
    static __device__ __forceinline__ const int* gw_up_kj() { return mech_cracmm2::c_gw_up_kj; }
    static __device__ __forceinline__ const int* gw_fl_ptr() { return mech_cracmm2::c_gw_fl_ptr; }
    static __device__ __forceinline__ const int* gw_fl_row() { return mech_cracmm2::c_gw_fl_row; }
    static __device__ __forceinline__ const int* gw_bl_ptr() { return mech_cracmm2::c_gw_bl_ptr; }
    static __device__ __forceinline__ const int* gw_bl_row() { return mech_cracmm2::c_gw_bl_row; }
    static __device__ __forceinline__ const int* gw_fr_ptr() { return mech_cracmm2::c_gw_fr_ptr; }
    static __device__ __forceinline__ const int* gw_fr_st() { return mech_cracmm2::c_gw_fr_st; }
    static __device__ __forceinline__ const int* gw_fr_col() { return mech_cracmm2::c_gw_fr_col; }
    static __device__ __forceinline__ const int* gw_br_ptr() { return mech_cracmm2::c_gw_br_ptr; }
    static __device__ __forceinline__ const int* gw_br_st() { return mech_cracmm2::c_gw_br_st; }
    static __device__ __forceinline__ const int* gw_br_col() { return mech_cracmm2::c_gw_br_col; }
    static __device__ __forceinline__ const double* gw_sum_c() { return mech_cracmm2::c_gw_sum_c; }
    static __device__ __forceinline__ const double* gw_asm_c() { return mech_cracmm2::c_gw_asm_c; }
    static __device__ __forceinline__ void rconst(double* ws, double t, double p, double h, double sw, int sun,
                                                  const double* rj, const double* het) { mech_cracmm2::rconst(ws, t, p, h, sw, sun, rj, het); }
};
}  // namespace mech_cracmm2
