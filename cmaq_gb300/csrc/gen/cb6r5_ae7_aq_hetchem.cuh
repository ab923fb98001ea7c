// Generated by cmaq_gb300/mechgen/hetchem.py from CCTM/src/aero/aero6 (AERO_DATA.F, AEROSOL_CHEMISTRY.F) and MECHS/cb6r5_ae7_aq.
// Included inside the mechanism's namespace by csrc/hetchem.cuh.  Do not edit.
#pragma once

constexpr int NAE = 84;      // CGRID rows of the aerosol block
constexpr int AE_FIRST = 131;  // its first row in the mechanism's CGRID (0-based)
constexpr int NSPC = 54;     // aerosol chemical species (map_aero order)
constexpr int NHET = 17;     // KHETERO rows
constexpr int NNUC = 6;      // epoxide acid / nucleophile pairs

constexpr int I_ASO4 = 0;
constexpr int I_ANO3 = 1;
constexpr int I_ACL = 2;
constexpr int I_ANH4 = 3;
constexpr int I_AH2O = 17;
constexpr int I_AH3OP = 19;
constexpr int I_APOC = 8;
constexpr int I_APNCOM = 9;

enum HetKind { K_N2O5IJ = 0, K_N2O5K = 1, K_H2NO3PAIJ = 2, K_H2NO3PBIJ = 3, K_H2NO3PAK = 4, K_H2NO3PBK = 5, K_NO2 = 6, K_IEPOX = 7, K_IEPOXOS = 8, K_TETROL = 9, K_GLY = 10, K_MGLY = 11, K_NTR2 = 12, K_CLNO3_WAI = 13, K_CLNO3_WAJ = 14, K_PNCOMLI = 15, K_PNCOMLJ = 16, K_NO3 = 17, K_HO2 = 18, K_N2O5I = 19, K_N2O5J = 20, K_ISO3NOSJ = 21, K_ISO3OSJ = 22 };

constexpr double MW_IEPOX = 118.1, MW_NO3 = 62.0, MW_GLY = 58.0, MW_MGLY = 72.0, MW_HO2 = 33.0;
constexpr float HL_IEPOX_A = 30000000.0f, HL_IEPOX_E = 0.0f;

struct HetTables {
    float density[NSPC];
    float molwt[NSPC];
    float min_conc[NSPC][3];
    double m3fac[NSPC];   // REAL( 1.0E-9 * f6pi / density, 8 ), the factor of the moment sums
    int charge[NSPC];
    unsigned char tracer[NSPC], no_m2wet[NSPC], om[NSPC];
    short row[NSPC][3];   // row in the aerosol block per mode, -1: missing
    short num_row[3], srf_row[3];
    int nuc_spc[NNUC], nuc_acid[NNUC], nuc_remove[NNUC], nuc_os[NNUC];
    double nuc_kchem[NNUC];
    int kind[NHET];   // HetKind of each KHETERO row
};

#define HET_TABLES_INIT \
    {{1800.0f, 1800.0f, 2200.0f, 1800.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1000.0f, 1000.0f, 1000.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 2600.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f}, \
     {96.0f, 62.0f, 35.5f, 18.0f, 23.0f, 24.3f, 39.1f, 40.1f, 220.0f, 220.0f, 12.0f, 55.8f, 200.0f, 27.0f, 28.1f, 47.9f, 54.9f, 18.0f, 18.0f, 19.0f, 132.0f, 133.0f, 168.2f, 273.0f, 206.0f, 248.0f, 177.0f, 100.0f, 100.0f, 23.75f, 231.0f, 168.0f, 300.0f, 200.0f, 186.0f, 184.0f, 170.0f, 168.0f, 66.4f, 218.0f, 230.0f, 241.0f, 253.0f, 266.0f, 136.0f, 136.0f, 135.0f, 135.0f, 134.0f, 170.0f, 198.0f, 179.0f, 169.0f, 158.0f}, \
     {{1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}}, \
     {1.0610328804797065e-12, 1.0610328804797065e-12, 8.681178063733863e-13, 1.0610328804797065e-12, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 1.3641851320453369e-12, 1.3641851320453369e-12, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 1.909859206547515e-12, 1.909859206547515e-12, 1.909859206547515e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 7.345612291174974e-13, 8.681178063733863e-13, 8.681178063733863e-13, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12}, \
     {-2, -1, -1, 1, 1, 2, 1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1}, \
     {{0, 1, 2}, {6, 7, 8}, {11, 12, 13}, {3, 4, 5}, {9, 10, -1}, {-1, 27, -1}, {-1, 28, -1}, {-1, 26, -1}, {52, 53, -1}, {54, 55, -1}, {18, 19, -1}, {-1, 22, -1}, {20, 21, -1}, {-1, 23, -1}, {-1, 24, -1}, {-1, 25, -1}, {-1, 29, -1}, {39, 40, 41}, {-1, 38, -1}, {42, 43, 44}, {-1, 14, -1}, {-1, 15, -1}, {-1, 46, -1}, {-1, 16, -1}, {-1, 47, -1}, {-1, 48, -1}, {-1, 17, -1}, {-1, -1, 31}, {-1, -1, 30}, {-1, -1, 45}, {-1, 50, -1}, {-1, 51, -1}, {-1, 78, -1}, {-1, 79, -1}, {-1, 80, -1}, {-1, 81, -1}, {-1, 82, -1}, {-1, 83, -1}, {-1, 49, -1}, {57, 58, -1}, {59, 60, -1}, {61, 62, -1}, {-1, 63, -1}, {-1, 64, -1}, {65, 66, -1}, {67, 68, -1}, {69, 70, -1}, {71, 72, -1}, {-1, 73, -1}, {-1, 56, -1}, {-1, 74, -1}, {-1, 75, -1}, {-1, 76, -1}, {-1, 77, -1}}, \
     {32, 33, 34}, {35, 36, 37}, \
     {17, 0, 1, 17, 0, 1}, {1, 1, 1, 2, 2, 2}, {0, 2, 0, 0, 2, 0}, {0, 1, 0, 0, 1, 0}, \
     {0.0009, 0.00883, 0.0002, 1.31e-05, 2.92e-06, 2.92e-06}, \
     {K_CLNO3_WAI, K_CLNO3_WAJ, K_NTR2, K_N2O5IJ, K_N2O5K, K_H2NO3PAIJ, K_H2NO3PAK, K_H2NO3PBIJ, K_H2NO3PBK, K_NO2, K_IEPOX, K_IEPOXOS, K_TETROL, K_GLY, K_MGLY, K_PNCOMLI, K_PNCOMLJ}}

// CGRID names of the aerosol block, for reference: ASO4I ASO4J ASO4K ANH4I ANH4J ANH4K ANO3I ANO3J ANO3K ANAI ANAJ ACLI ACLJ ACLK AISO1J AISO2J ASQTJ AORGCJ AECI AECJ AOTHRI AOTHRJ AFEJ AALJ ASIJ ATIJ ACAJ AMGJ AKJ AMNJ ACORS ASOIL NUMATKN NUMACC NUMCOR SRFATKN SRFACC SRFCOR AORGH2OJ AH2OI AH2OJ AH2OK AH3OPI AH3OPJ AH3OPK ASEACAT AISO3J AOLGAJ AOLGBJ AGLYJ AMTNO3J AMTHYDJ APOCI APOCJ APNCOMI APNCOMJ APCSOJ ALVPO1I ALVPO1J ASVPO1I ASVPO1J ASVPO2I ASVPO2J ASVPO3J AIVPO1J ALVOO1I ALVOO1J ALVOO2I ALVOO2J ASVOO1I ASVOO1J ASVOO2I ASVOO2J ASVOO3J AAVB1J AAVB2J AAVB3J AAVB4J AMT1J AMT2J AMT3J AMT4J AMT5J AMT6J
