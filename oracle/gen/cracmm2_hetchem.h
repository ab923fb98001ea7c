/* Generated by cmaq_gb300/mechgen/hetchem.py from CCTM/src/aero/aero6 and MECHS/cracmm2:
 * the aerosol species of map_aero, the CGRID aerosol block, KHETERO's labels and the epoxide
 * acid / nucleophile pairs.  Test infrastructure (the oracle).  Do not edit. */
#pragma once

#define HO_NAE 90
#define HO_NSPC 53
#define HO_NHET 9
#define HO_NNUC 6

#define HO_ASO4 0
#define HO_ANO3 1
#define HO_ACL 2
#define HO_ANH4 3
#define HO_AH2O 17
#define HO_AH3OP 19
#define HO_APOC 8
#define HO_APNCOM 9

static const float ho_density[] = {1800.0f, 1800.0f, 2200.0f, 1800.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1000.0f, 1000.0f, 1000.0f, 1400.0f, 1400.0f, 1400.0f, 2600.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f};
static const float ho_molwt[] = {96.0f, 62.0f, 35.5f, 18.0f, 23.0f, 24.3f, 39.1f, 40.1f, 220.0f, 220.0f, 12.0f, 55.8f, 200.0f, 27.0f, 28.1f, 47.9f, 54.9f, 18.0f, 18.0f, 19.0f, 250.0f, 402.0f, 177.0f, 100.0f, 100.0f, 23.75f, 136.2f, 216.2f, 66.4f, 176.2f, 422.83f, 408.8f, 394.77f, 380.75f, 338.66f, 296.58f, 282.4f, 232.3f, 194.2f, 312.5f, 230.3f, 190.2f, 242.4f, 202.3f, 270.5f, 202.3f, 200.3f, 186.3f, 200.0f, 168.1f, 150.1f, 215.0f, 265.0f};
static const float ho_min_conc[] = {1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f, 1e-23f};
static const int ho_charge[] = {-2, -1, -1, 1, 1, 2, 1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int ho_tracer[] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int ho_no_m2wet[] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
static const int ho_om[] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1};
static const int ho_row[] = {0, 1, 2, 6, 7, 8, 43, 44, 45, 3, 4, 5, 41, 42, -1, -1, 23, -1, -1, 24, -1, -1, 22, -1, 47, 48, -1, 49, 50, -1, 14, 15, -1, -1, 18, -1, 16, 17, -1, -1, 19, -1, -1, 20, -1, -1, 21, -1, -1, 25, -1, 35, 36, 37, -1, 34, -1, 38, 39, 40, -1, 11, -1, -1, 12, -1, -1, 13, -1, -1, -1, 27, -1, -1, 26, -1, -1, 46, -1, 84, -1, -1, 85, -1, -1, 10, -1, -1, 51, -1, 52, 53, -1, 54, 55, -1, 56, 57, -1, 58, 59, -1, -1, 60, -1, -1, 61, -1, 62, 63, -1, 64, 65, -1, 66, 67, -1, 68, 69, -1, 70, 71, -1, 72, 73, -1, 74, 75, -1, 76, 77, -1, 78, 79, -1, 80, 81, -1, -1, 82, -1, -1, 83, -1, -1, 9, -1, -1, 86, -1, -1, 87, -1, -1, 88, -1, -1, 89, -1};   /* [spc][mode], -1: missing */
static const int ho_num_row[] = {28, 29, 30};
static const int ho_srf_row[] = {31, 32, 33};
static const int ho_nuc_spc[] = {17, 0, 1, 17, 0, 1};
static const int ho_nuc_acid[] = {1, 1, 1, 2, 2, 2};
static const int ho_nuc_remove[] = {0, 2, 0, 0, 2, 0};
static const int ho_nuc_os[] = {0, 1, 0, 0, 1, 0};
static const double ho_nuc_kchem[] = {0.0009, 0.00883, 0.0002, 1.31e-05, 2.92e-06, 2.92e-06};
static const char* const ho_hetero[] = {"HETERO_GLY", "HETERO_MGLY", "HETERO_N2O5IJ", "HETERO_NO2", "HETERO_HO2", "HETERO_NO3", "HETERO_IEPOX", "HETERO_ISO3NOSJ", "HETERO_ISO3OSJ"};
static const double ho_mw_iepox = 118.1, ho_mw_gly = 58.0, ho_mw_mgly = 72.0, ho_mw_no3 = 62.0, ho_mw_ho2 = 33.0;
static const float ho_hl_iepox_a = 30000000.0f, ho_hl_iepox_e = 0.0f;
