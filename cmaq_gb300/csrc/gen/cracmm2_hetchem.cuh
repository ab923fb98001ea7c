// Generated by cmaq_gb300/mechgen/hetchem.py from CCTM/src/aero/aero6 (AERO_DATA.F, AEROSOL_CHEMISTRY.F) and MECHS/cracmm2.
// Included inside the mechanism's namespace by csrc/hetchem.cuh.  Do not edit.
#pragma once

constexpr int NAE = 90;      // CGRID rows of the aerosol block
constexpr int AE_FIRST = 184;  // its first row in the mechanism's CGRID (0-based)
constexpr int NSPC = 53;     // aerosol chemical species (map_aero order)
constexpr int NHET = 9;     // KHETERO rows
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
    {{1800.0f, 1800.0f, 2200.0f, 1800.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 2200.0f, 1000.0f, 1000.0f, 1000.0f, 1400.0f, 1400.0f, 1400.0f, 2600.0f, 2200.0f, 2200.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f, 1400.0f}, \
     {96.0f, 62.0f, 35.5f, 18.0f, 23.0f, 24.3f, 39.1f, 40.1f, 220.0f, 220.0f, 12.0f, 55.8f, 200.0f, 27.0f, 28.1f, 47.9f, 54.9f, 18.0f, 18.0f, 19.0f, 250.0f, 402.0f, 177.0f, 100.0f, 100.0f, 23.75f, 136.2f, 216.2f, 66.4f, 176.2f, 422.83f, 408.8f, 394.77f, 380.75f, 338.66f, 296.58f, 282.4f, 232.3f, 194.2f, 312.5f, 230.3f, 190.2f, 242.4f, 202.3f, 270.5f, 202.3f, 200.3f, 186.3f, 200.0f, 168.1f, 150.1f, 215.0f, 265.0f}, \
     {{1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}, {1e-23f, 1e-23f, 1e-23f}}, \
     {1.0610328804797065e-12, 1.0610328804797065e-12, 8.681178063733863e-13, 1.0610328804797065e-12, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 1.3641851320453369e-12, 1.3641851320453369e-12, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 8.681178063733863e-13, 1.909859206547515e-12, 1.909859206547515e-12, 1.909859206547515e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 7.345612291174974e-13, 8.681178063733863e-13, 8.681178063733863e-13, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12, 1.3641851320453369e-12}, \
     {-2, -1, -1, 1, 1, 2, 1, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0}, \
     {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1}, \
     {{0, 1, 2}, {6, 7, 8}, {43, 44, 45}, {3, 4, 5}, {41, 42, -1}, {-1, 23, -1}, {-1, 24, -1}, {-1, 22, -1}, {47, 48, -1}, {49, 50, -1}, {14, 15, -1}, {-1, 18, -1}, {16, 17, -1}, {-1, 19, -1}, {-1, 20, -1}, {-1, 21, -1}, {-1, 25, -1}, {35, 36, 37}, {-1, 34, -1}, {38, 39, 40}, {-1, 11, -1}, {-1, 12, -1}, {-1, 13, -1}, {-1, -1, 27}, {-1, -1, 26}, {-1, -1, 46}, {-1, 84, -1}, {-1, 85, -1}, {-1, 10, -1}, {-1, 51, -1}, {52, 53, -1}, {54, 55, -1}, {56, 57, -1}, {58, 59, -1}, {-1, 60, -1}, {-1, 61, -1}, {62, 63, -1}, {64, 65, -1}, {66, 67, -1}, {68, 69, -1}, {70, 71, -1}, {72, 73, -1}, {74, 75, -1}, {76, 77, -1}, {78, 79, -1}, {80, 81, -1}, {-1, 82, -1}, {-1, 83, -1}, {-1, 9, -1}, {-1, 86, -1}, {-1, 87, -1}, {-1, 88, -1}, {-1, 89, -1}}, \
     {28, 29, 30}, {31, 32, 33}, \
     {17, 0, 1, 17, 0, 1}, {1, 1, 1, 2, 2, 2}, {0, 2, 0, 0, 2, 0}, {0, 1, 0, 0, 1, 0}, \
     {0.0009, 0.00883, 0.0002, 1.31e-05, 2.92e-06, 2.92e-06}, \
     {K_GLY, K_MGLY, K_N2O5IJ, K_NO2, K_HO2, K_NO3, K_IEPOX, K_ISO3NOSJ, K_ISO3OSJ}}

// CGRID names of the aerosol block, for reference: ASO4I ASO4J ASO4K ANH4I ANH4J ANH4K ANO3I ANO3J ANO3K ASOATJ AGLYJ AHOMJ AELHOMJ AORGCJ AECI AECJ AOTHRI AOTHRJ AFEJ AALJ ASIJ ATIJ ACAJ AMGJ AKJ AMNJ ACORS ASOIL NUMATKN NUMACC NUMCOR SRFATKN SRFACC SRFCOR AORGH2OJ AH2OI AH2OJ AH2OK AH3OPI AH3OPJ AH3OPK ANAI ANAJ ACLI ACLJ ACLK ASEACAT APOCI APOCJ APNCOMI APNCOMJ AOP3J AROCN2ALKI AROCN2ALKJ AROCN1ALKI AROCN1ALKJ AROCP0ALKI AROCP0ALKJ AROCP1ALKI AROCP1ALKJ AROCP2ALKJ AROCP3ALKJ AROCN2OXY2I AROCN2OXY2J AROCN2OXY4I AROCN2OXY4J AROCN2OXY8I AROCN2OXY8J AROCN1OXY1I AROCN1OXY1J AROCN1OXY3I AROCN1OXY3J AROCN1OXY6I AROCN1OXY6J AROCP0OXY2I AROCP0OXY2J AROCP0OXY4I AROCP0OXY4J AROCP1OXY1I AROCP1OXY1J AROCP1OXY3I AROCP1OXY3J AROCP2OXY2J AROCP3OXY2J AISO3NOSJ AISO3OSJ AISO4J AISO5J ATRPNJ AHONITJ
