/* Generated by cmaq_gb300/mechgen/hetchem.py from CCTM/src/aero/aero6 and MECHS/cb6r5_ae7_aq:
 * the aerosol species of map_aero, the CGRID aerosol block, KHETERO's labels and the epoxide
 * acid / nucleophile pairs.  Test infrastructure (the oracle).  Do not edit. */
#pragma once

#define HO_NAE 84
#define HO_NSPC 54
#define HO_NHET 17
#define HO_NNUC 6

#define HO_ASO4 0
#define HO_ANO3 1
#define HO_ACL 2
#define HO_ANH4 3
#define HO_AH2O 17
#define HO_AH3OP 19
#define HO_APOC 8
#define HO_APNCOM 9

static const float ho_density[] = {1800.0f, 1800.0f, 2200.0f, 1800.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1000.0f, 1000.0f, 1000.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 2600.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f};
static const float ho_molwt[] = {96.0f, 62.0f, 35.5f, 18.0f, 23.0f, 24.3f, 39.1f, 40.1f, 220.0f, 220.0f, 12.0f, 55.8f, 200.0f, 27.0f, 28.1f, 47.9f, 54.9f, 18.0f, 18.0f, 19.0f, 132.0f, 133.0f, 168.2f, 273.0f, 206.0f, 248.0f, 177.0f, 100.0f, 100.0f, 23.75f, 231.0f, 168.0f, 300.0f, 200.0f, 186.0f, 184.0f, 170.0f, 168.0f, 66.4f, 218.0f, 230.0f, 241.0f, 253.0f, 266.0f, 136.0f, 136.0f, 135.0f, 135.0f, 134.0f, 170.0f, 198.0f, 179.0f, 169.0f, 158.0f};
static const float ho_min_conc[] = {1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f};
static const int ho_charge[] = {-2, -1, -1, 1, 1, 2, 1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int ho_tracer[] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int ho_no_m2wet[] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int ho_om[] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
static const int ho_row[] = {0, 1, 2, 6, 7, 8, 11, 12, 13, 3, 4, 5, 9, 10, -1, -1, 27, -1, -1, 28, -1, -1, 26, -1, 52, 53, -1, 54, 55, -1, 18, 19, -1, -1, 22, -1, 20, 21, -1, -1, 23, -1, -1, 24, -1, -1, 25, -1, -1, 29, -1, 39, 40, 41, -1, 38, -1, 42, 43, 44, -1, 14, -1, -1, 15, -1, -1, 46, -1, -1, 16, -1, -1, 47, -1, -1, 48, -1, -1, 17, -1, -1, -1, 31, -1, -1, 30, -1, -1, 45, -1, 50, -1, -1, 51, -1, -1, 78, -1, -1, 79, -1, -1, 80, -1, -1, 81, -1, -1, 82, -1, -1, 83, -1, -1, 49, -1, 57, 58, -1, 59, 60, -1, 61, 62, -1, -1, 63, -1, -1, 64, -1, 65, 66, -1, 67, 68, -1, 69, 70, -1, 71, 72, -1, -1, 73, -1, -1, 56, -1, -1, 74, -1, -1, 75, -1, -1, 76, -1, -1, 77, -1};   /* [spc][mode], -1: missing */
static const int ho_num_row[] = {32, 33, 34};
static const int ho_srf_row[] = {35, 36, 37};
static const int ho_nuc_spc[] = {17, 0, 1, 17, 0, 1};
static const int ho_nuc_acid[] = {1, 1, 1, 2, 2, 2};
static const int ho_nuc_remove[] = {0, 2, 0, 0, 2, 0};
static const int ho_nuc_os[] = {0, 1, 0, 0, 1, 0};
static const double ho_nuc_kchem[] = {0.0009, 0.00883, 0.0002, 1.31e-05, 2.92e-06, 2.92e-06};
static const char* const ho_hetero[] = {"HETERO_CLNO3_WAI", "HETERO_CLNO3_WAJ", "HETERO_NTR2", "HETERO_N2O5IJ", "HETERO_N2O5K", "HETERO_H2NO3PAIJ", "HETERO_H2NO3PAK", "HETERO_H2NO3PBIJ", "HETERO_H2NO3PBK", "HETERO_NO2", "HETERO_IEPOX", "HETERO_IEPOXOS", "HETERO_TETROL", "HETERO_GLY", "HETERO_MGLY", "HETERO_PNCOMLI", "HETERO_PNCOMLJ"};
static const double ho_mw_iepox = 118.1, ho_mw_gly = 58.0, ho_mw_mgly = 72.0, ho_mw_no3 = 62.0, ho_mw_ho2 = 33.0;
static const float ho_hl_iepox_a = 30000000.0f, ho_hl_iepox_e = 0.0f;
