// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {

/* Rate-constant helpers, one per CMAQ rate form (RXNS_FUNC_MODULE.F90:15-160). */
CHEM_HD static inline double chem_power_t02(double tempot300, double a0, double b0)
{
    return a0 * pow(tempot300, b0);
}
CHEM_HD static inline double chem_arrhenius_t03(double inv_temp, double a0, double b0)
{
    return a0 * exp(b0 * inv_temp);
}
CHEM_HD static inline double chem_arrhenius_t04(double inv_temp, double tempot300, double a0, double b0, double c0)
{
    return a0 * exp(b0 * inv_temp) * pow(tempot300, c0);
}
CHEM_HD static inline double chem_falloff_t08(double inv_temp, double cair, double a0, double c0,
                                              double a2, double c2, double a3, double c3)
{
    double k0 = a0 * exp(c0 * inv_temp);
    double k2 = a2 * exp(c2 * inv_temp);
    double k3 = a3 * exp(c3 * inv_temp);
    k3 = k3 * cair;
    return k0 + k3 / (1.0 + k3 / k2);
}
CHEM_HD static inline double chem_falloff_t09(double inv_temp, double cair, double a1, double c1,
                                              double a2, double c2)
{
    double k1 = a1 * exp(c1 * inv_temp);
    double k2 = a2 * exp(c2 * inv_temp);
    return k1 + k2 * cair;
}
CHEM_HD static inline double chem_falloff_t10(double inv_temp, double tempot300, double cair,
                                              double a0, double b0, double c0, double a1, double b1,
                                              double c1, double ce, double cf)
{
    double k0 = a0 * cair * exp(b0 * inv_temp) * pow(tempot300, c0);
    double k1 = a1 * exp(b1 * inv_temp) * pow(tempot300, c1);
    double x = (1.0 / ce) * log10(k0 / k1);
    double kend = 1.0 + x * x;
    kend = 1.0 / kend;
    return (k0 / (1.0 + k0 / k1)) * pow(cf, kend);
}
CHEM_HD static inline double chem_falloff_t11(double inv_temp, double tempot300, double cair,
                                              double a1, double b1, double c1, double a2, double b2,
                                              double c2, double d1, double d2)
{
    double k1 = a1 * exp(c1 * inv_temp) * pow(tempot300, b1);
    double k2 = a2 * exp(c2 * inv_temp) * pow(tempot300, b2);
    double k3 = d1 * exp(d2 * inv_temp);
    return k1 + k2 * cair + k3;
}
CHEM_HD static inline double chem_halogen_falloff(double press, double a1, double b1, double a2,
                                                  double b2, double a3)
{
    double k = a1 * exp(b1 * press) + a2 * exp(b2 * press);
    return fmin(a3, k);
}

__constant__ int c_inew2old[149] = {112, 113, 114, 116, 117, 118, 120, 121, 14, 15, 43, 50, 68, 86, 101, 104, 105, 106, 108, 109, 110, 5, 122, 124, 126, 127, 41, 42, 46, 47, 49, 56, 60, 62, 73, 77, 80, 87, 94, 103, 9, 107, 19, 115, 119, 123, 125, 132, 143, 145, 148, 58, 59, 12, 36, 83, 85, 89, 99, 100, 102, 25, 48, 147, 64, 65, 67, 72, 84, 13, 98, 27, 131, 138, 139, 140, 142, 11, 79, 54, 81, 93, 96, 51, 20, 28, 128, 129, 130, 66, 29, 137, 75, 141, 144, 146, 97, 70, 53, 135, 136, 91, 95, 63, 82, 111, 45, 55, 8, 74, 90, 52, 78, 69, 32, 133, 134, 61, 34, 76, 38, 57, 21, 71, 92, 40, 33, 37, 22, 23, 2, 10, 44, 39, 31, 3, 30, 1, 17, 16, 35, 26, 88, 24, 0, 4, 18, 7, 6};
__constant__ int c_iold2new[149] = {144, 137, 130, 135, 145, 21, 148, 147, 108, 40, 131, 77, 53, 69, 8, 9, 139, 138, 146, 42, 84, 122, 128, 129, 143, 61, 141, 71, 85, 90, 136, 134, 114, 126, 118, 140, 54, 127, 120, 133, 125, 26, 27, 10, 132, 106, 28, 29, 62, 30, 11, 83, 111, 98, 79, 107, 31, 121, 51, 52, 32, 117, 33, 103, 64, 65, 89, 66, 12, 113, 97, 123, 67, 34, 109, 92, 119, 35, 112, 78, 36, 80, 104, 55, 68, 56, 13, 37, 142, 57, 110, 101, 124, 81, 38, 102, 82, 96, 70, 58, 59, 14, 60, 39, 15, 16, 17, 41, 18, 19, 20, 105, 0, 1, 2, 43, 3, 4, 5, 44, 6, 7, 22, 45, 23, 46, 24, 25, 86, 87, 88, 72, 47, 115, 116, 99, 100, 91, 73, 74, 75, 93, 76, 48, 94, 49, 95, 63, 50};
// Rate constants of one cell into ws[OFF_RKI + r] (CALC_RCONST, RXNS_FUNC_MODULE.F90).
__device__ __noinline__ void rconst(double* __restrict__ ws, double temp_in, double press, double h2o,
                                    double seawater, int lsunlight, const double* __restrict__ rjv,
                                    const double* __restrict__ hetv)
{
    /* RKI = 0 (RXNS_FUNC_MODULE.F90 CALC_RCONST) */
    ws[33376] = 0.0;
    ws[33408] = 0.0;
    ws[33440] = 0.0;
    ws[33472] = 0.0;
    ws[33504] = 0.0;
    ws[33536] = 0.0;
    ws[33568] = 0.0;
    ws[33600] = 0.0;
    ws[33632] = 0.0;
    ws[33664] = 0.0;
    ws[33696] = 0.0;
    ws[33728] = 0.0;
    ws[33760] = 0.0;
    ws[33792] = 0.0;
    ws[33824] = 0.0;
    ws[33856] = 0.0;
    ws[33888] = 0.0;
    ws[33920] = 0.0;
    ws[33952] = 0.0;
    ws[33984] = 0.0;
    ws[34016] = 0.0;
    ws[34048] = 0.0;
    ws[34080] = 0.0;
    ws[34112] = 0.0;
    ws[34144] = 0.0;
    ws[34176] = 0.0;
    ws[34208] = 0.0;
    ws[34240] = 0.0;
    ws[34272] = 0.0;
    ws[34304] = 0.0;
    ws[34336] = 0.0;
    ws[34368] = 0.0;
    ws[34400] = 0.0;
    ws[34432] = 0.0;
    ws[34464] = 0.0;
    ws[34496] = 0.0;
    ws[34528] = 0.0;
    ws[34560] = 0.0;
    ws[34592] = 0.0;
    ws[34624] = 0.0;
    ws[34656] = 0.0;
    ws[34688] = 0.0;
    ws[34720] = 0.0;
    ws[34752] = 0.0;
    ws[34784] = 0.0;
    ws[34816] = 0.0;
    ws[34848] = 0.0;
    ws[34880] = 0.0;
    ws[34912] = 0.0;
    ws[34944] = 0.0;
    ws[34976] = 0.0;
    ws[35008] = 0.0;
    ws[35040] = 0.0;
    ws[35072] = 0.0;
    ws[35104] = 0.0;
    ws[35136] = 0.0;
    ws[35168] = 0.0;
    ws[35200] = 0.0;
    ws[35232] = 0.0;
    ws[35264] = 0.0;
    ws[35296] = 0.0;
    ws[35328] = 0.0;
    ws[35360] = 0.0;
    ws[35392] = 0.0;
    ws[35424] = 0.0;
    ws[35456] = 0.0;
    ws[35488] = 0.0;
    ws[35520] = 0.0;
    ws[35552] = 0.0;
    ws[35584] = 0.0;
    ws[35616] = 0.0;
    ws[35648] = 0.0;
    ws[35680] = 0.0;
    ws[35712] = 0.0;
    ws[35744] = 0.0;
    ws[35776] = 0.0;
    ws[35808] = 0.0;
    ws[35840] = 0.0;
    ws[35872] = 0.0;
    ws[35904] = 0.0;
    ws[35936] = 0.0;
    ws[35968] = 0.0;
    ws[36000] = 0.0;
    ws[36032] = 0.0;
    ws[36064] = 0.0;
    ws[36096] = 0.0;
    ws[36128] = 0.0;
    ws[36160] = 0.0;
    ws[36192] = 0.0;
    ws[36224] = 0.0;
    ws[36256] = 0.0;
    ws[36288] = 0.0;
    ws[36320] = 0.0;
    ws[36352] = 0.0;
    ws[36384] = 0.0;
    ws[36416] = 0.0;
    ws[36448] = 0.0;
    ws[36480] = 0.0;
    ws[36512] = 0.0;
    ws[36544] = 0.0;
    ws[36576] = 0.0;
    ws[36608] = 0.0;
    ws[36640] = 0.0;
    ws[36672] = 0.0;
    ws[36704] = 0.0;
    ws[36736] = 0.0;
    ws[36768] = 0.0;
    ws[36800] = 0.0;
    ws[36832] = 0.0;
    ws[36864] = 0.0;
    ws[36896] = 0.0;
    ws[36928] = 0.0;
    ws[36960] = 0.0;
    ws[36992] = 0.0;
    ws[37024] = 0.0;
    ws[37056] = 0.0;
    ws[37088] = 0.0;
    ws[37120] = 0.0;
    ws[37152] = 0.0;
    ws[37184] = 0.0;
    ws[37216] = 0.0;
    ws[37248] = 0.0;
    ws[37280] = 0.0;
    ws[37312] = 0.0;
    ws[37344] = 0.0;
    ws[37376] = 0.0;
    ws[37408] = 0.0;
    ws[37440] = 0.0;
    ws[37472] = 0.0;
    ws[37504] = 0.0;
    ws[37536] = 0.0;
    ws[37568] = 0.0;
    ws[37600] = 0.0;
    ws[37632] = 0.0;
    ws[37664] = 0.0;
    ws[37696] = 0.0;
    ws[37728] = 0.0;
    ws[37760] = 0.0;
    ws[37792] = 0.0;
    ws[37824] = 0.0;
    ws[37856] = 0.0;
    ws[37888] = 0.0;
    ws[37920] = 0.0;
    ws[37952] = 0.0;
    ws[37984] = 0.0;
    ws[38016] = 0.0;
    ws[38048] = 0.0;
    ws[38080] = 0.0;
    ws[38112] = 0.0;
    ws[38144] = 0.0;
    ws[38176] = 0.0;
    ws[38208] = 0.0;
    ws[38240] = 0.0;
    ws[38272] = 0.0;
    ws[38304] = 0.0;
    ws[38336] = 0.0;
    ws[38368] = 0.0;
    ws[38400] = 0.0;
    ws[38432] = 0.0;
    ws[38464] = 0.0;
    ws[38496] = 0.0;
    ws[38528] = 0.0;
    ws[38560] = 0.0;
    ws[38592] = 0.0;
    ws[38624] = 0.0;
    ws[38656] = 0.0;
    ws[38688] = 0.0;
    ws[38720] = 0.0;
    ws[38752] = 0.0;
    ws[38784] = 0.0;
    ws[38816] = 0.0;
    ws[38848] = 0.0;
    ws[38880] = 0.0;
    ws[38912] = 0.0;
    ws[38944] = 0.0;
    ws[38976] = 0.0;
    ws[39008] = 0.0;
    ws[39040] = 0.0;
    ws[39072] = 0.0;
    ws[39104] = 0.0;
    ws[39136] = 0.0;
    ws[39168] = 0.0;
    ws[39200] = 0.0;
    ws[39232] = 0.0;
    ws[39264] = 0.0;
    ws[39296] = 0.0;
    ws[39328] = 0.0;
    ws[39360] = 0.0;
    ws[39392] = 0.0;
    ws[39424] = 0.0;
    ws[39456] = 0.0;
    ws[39488] = 0.0;
    ws[39520] = 0.0;
    ws[39552] = 0.0;
    ws[39584] = 0.0;
    ws[39616] = 0.0;
    ws[39648] = 0.0;
    ws[39680] = 0.0;
    ws[39712] = 0.0;
    ws[39744] = 0.0;
    ws[39776] = 0.0;
    ws[39808] = 0.0;
    ws[39840] = 0.0;
    ws[39872] = 0.0;
    ws[39904] = 0.0;
    ws[39936] = 0.0;
    ws[39968] = 0.0;
    ws[40000] = 0.0;
    ws[40032] = 0.0;
    ws[40064] = 0.0;
    ws[40096] = 0.0;
    ws[40128] = 0.0;
    ws[40160] = 0.0;
    ws[40192] = 0.0;
    ws[40224] = 0.0;
    ws[40256] = 0.0;
    ws[40288] = 0.0;
    ws[40320] = 0.0;
    ws[40352] = 0.0;
    ws[40384] = 0.0;
    ws[40416] = 0.0;
    ws[40448] = 0.0;
    ws[40480] = 0.0;
    ws[40512] = 0.0;
    ws[40544] = 0.0;
    ws[40576] = 0.0;
    ws[40608] = 0.0;
    ws[40640] = 0.0;
    ws[40672] = 0.0;
    ws[40704] = 0.0;
    ws[40736] = 0.0;
    ws[40768] = 0.0;
    ws[40800] = 0.0;
    ws[40832] = 0.0;
    ws[40864] = 0.0;
    ws[40896] = 0.0;
    ws[40928] = 0.0;
    ws[40960] = 0.0;
    ws[40992] = 0.0;
    ws[41024] = 0.0;
    ws[41056] = 0.0;
    ws[41088] = 0.0;
    ws[41120] = 0.0;
    ws[41152] = 0.0;
    ws[41184] = 0.0;
    ws[41216] = 0.0;
    ws[41248] = 0.0;
    ws[41280] = 0.0;
    ws[41312] = 0.0;
    ws[41344] = 0.0;
    ws[41376] = 0.0;
    ws[41408] = 0.0;
    ws[41440] = 0.0;
    ws[41472] = 0.0;
    ws[41504] = 0.0;
    ws[41536] = 0.0;
    ws[41568] = 0.0;
    ws[41600] = 0.0;
    ws[41632] = 0.0;
    ws[41664] = 0.0;
    ws[41696] = 0.0;
    ws[41728] = 0.0;
    ws[41760] = 0.0;
    ws[41792] = 0.0;
    ws[41824] = 0.0;
    ws[41856] = 0.0;
    ws[41888] = 0.0;
    ws[41920] = 0.0;
    ws[41952] = 0.0;
    ws[41984] = 0.0;
    ws[42016] = 0.0;
    ws[42048] = 0.0;
    ws[42080] = 0.0;
    ws[42112] = 0.0;
    ws[42144] = 0.0;
    ws[42176] = 0.0;
    ws[42208] = 0.0;
    ws[42240] = 0.0;
    ws[42272] = 0.0;
    ws[42304] = 0.0;
    ws[42336] = 0.0;
    ws[42368] = 0.0;
    ws[42400] = 0.0;
    ws[42432] = 0.0;
    ws[42464] = 0.0;
    ws[42496] = 0.0;
    ws[42528] = 0.0;
    ws[42560] = 0.0;
    ws[42592] = 0.0;
    ws[42624] = 0.0;
    ws[42656] = 0.0;
    ws[42688] = 0.0;
    ws[42720] = 0.0;
    ws[42752] = 0.0;
    ws[42784] = 0.0;
    ws[42816] = 0.0;
    ws[42848] = 0.0;
    ws[42880] = 0.0;
    ws[42912] = 0.0;
    ws[42944] = 0.0;
    ws[42976] = 0.0;
    ws[43008] = 0.0;
    ws[43040] = 0.0;
    ws[43072] = 0.0;
    ws[43104] = 0.0;
    ws[43136] = 0.0;
    ws[43168] = 0.0;
    ws[43200] = 0.0;
    ws[43232] = 0.0;
    ws[43264] = 0.0;
    ws[43296] = 0.0;
    ws[43328] = 0.0;
    ws[43360] = 0.0;
    ws[43392] = 0.0;
    ws[43424] = 0.0;
    ws[43456] = 0.0;
    ws[43488] = 0.0;
    ws[43520] = 0.0;
    ws[43552] = 0.0;
    ws[43584] = 0.0;
    ws[43616] = 0.0;
    ws[43648] = 0.0;
    ws[43680] = 0.0;
    ws[43712] = 0.0;
    ws[43744] = 0.0;
    ws[43776] = 0.0;
    ws[43808] = 0.0;
    ws[43840] = 0.0;
    ws[43872] = 0.0;
    ws[43904] = 0.0;
    ws[43936] = 0.0;
    ws[43968] = 0.0;
    ws[44000] = 0.0;
    ws[44032] = 0.0;
    ws[44064] = 0.0;
    ws[44096] = 0.0;
    ws[44128] = 0.0;
    ws[44160] = 0.0;
    ws[44192] = 0.0;
    ws[44224] = 0.0;
    ws[44256] = 0.0;
    ws[44288] = 0.0;
    ws[44320] = 0.0;
    ws[44352] = 0.0;
    ws[44384] = 0.0;
    ws[44416] = 0.0;
    ws[44448] = 0.0;
    ws[44480] = 0.0;
    ws[44512] = 0.0;
    if (lsunlight) {
        ws[33376] = rjv[0];
        ws[33600] = rjv[1];
        ws[33632] = rjv[2];
        ws[34016] = rjv[3];
        ws[34208] = rjv[4];
        ws[34240] = rjv[5];
        ws[34560] = rjv[6];
        ws[34720] = rjv[7];
        ws[34848] = rjv[8];
        ws[34944] = rjv[9];
        ws[35136] = rjv[10];
        ws[35392] = rjv[10];
        ws[36160] = rjv[11];
        ws[36224] = rjv[11];
        ws[36288] = rjv[12];
        ws[36448] = rjv[13];
        ws[36480] = rjv[14];
        ws[36800] = rjv[15];
        ws[36928] = rjv[16];
        ws[36992] = rjv[17];
        ws[37088] = rjv[18];
        ws[37152] = rjv[19];
        ws[37440] = rjv[20];
        ws[37472] = rjv[21];
        ws[38496] = rjv[22];
        ws[38560] = rjv[23];
        ws[39776] = rjv[12];
        ws[39808] = 0.05 * rjv[0];
        ws[39936] = 0.028 * rjv[0];
        ws[40576] = rjv[24];
        ws[40608] = rjv[25];
        ws[40832] = rjv[26];
        ws[41408] = rjv[27];
        ws[41472] = rjv[28];
        ws[41504] = rjv[29];
        ws[42656] = rjv[30];
        ws[43488] = rjv[13];
        ws[43520] = rjv[14];
        ws[43680] = rjv[15];
        ws[43968] = rjv[31];
        ws[44128] = rjv[31];
        if (seawater > 0.001) ws[42272] = (seawater * 60.0) * chem_halogen_falloff(press, 6.7006e-11, 10.743, 3.4153e-08, (-0.6713), 2e-06);
        else ws[42272] = 0.0;
    }
    {
        const double inv_temp = 1.0 / temp_in;
        const double cair = ((1000000.0 * 7339810000000000.0) * press) * inv_temp;
        const double cfact = 6e-05 * cair;
        const double cfact_squ = (6e-11 * cair) * cair;
        const double inv_cair = 1.0 / cair;
        const double inv_cfact = 60000000.0 * inv_cair;
        const double temp = temp_in;
        const double tempot300 = temp_in * 0.0033333333333333335;
        const double rfact = 1000000.0 * inv_cair;
        const double rfact_squ = (1000000000000.0 * inv_cair) * inv_cair;
        ws[33408] = cfact_squ * chem_power_t02(tempot300, 6e-34, (-2.6));
        ws[33440] = cfact * chem_arrhenius_t03(inv_temp, 2.07e-12, (-1400.0));
        ws[33472] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1e-31, 0.0, (-1.6), 5e-11, 0.0, 0.3, 0.84, 0.85);
        ws[33504] = cfact * chem_arrhenius_t03(inv_temp, 5.1e-12, 198.0);
        ws[33536] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.3e-31, 0.0, (-1.5), 2.3e-11, 0.0, 0.24, 1.03, 0.6);
        ws[33568] = cfact * chem_arrhenius_t03(inv_temp, 8e-12, (-2060.0));
        ws[33664] = cfact * chem_arrhenius_t03(inv_temp, 2.23e-11, 115.0);
        ws[33696] = 2.14e-10 * cfact;
        ws[33728] = cfact * chem_arrhenius_t03(inv_temp, 1.7e-12, (-940.0));
        ws[33760] = cfact * chem_arrhenius_t04(inv_temp, tempot300, 2.03e-16, 693.0, 4.57);
        ws[33792] = cfact * chem_arrhenius_t03(inv_temp, 2.4e-11, 110.0);
        ws[33824] = cfact * chem_arrhenius_t03(inv_temp, 3e-11, 200.0);
        ws[33856] = cfact * chem_arrhenius_t04(inv_temp, tempot300, 6.2e-14, 945.0, 2.6);
        ws[33888] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 9e-31, 0.0, (-3.2), 3.9e-11, 0.0, (-0.47), 1.23, 0.42);
        ws[33920] = cfact * chem_arrhenius_t03(inv_temp, 4.8e-11, 250.0);
        ws[33952] = cfact * chem_falloff_t09(inv_temp, cair, 2.2e-13, 600.0, 1.9e-33, 980.0);
        ws[33984] = cfact_squ * chem_falloff_t09(inv_temp, cair, 3.08e-34, 2800.0, 2.66e-54, 3180.0);
        ws[34048] = 1.8e-12 * cfact;
        ws[34080] = cfact * chem_arrhenius_t03(inv_temp, 1.4e-12, (-2000.0));
        ws[34112] = cfact_squ * chem_arrhenius_t03(inv_temp, 4.25e-39, 664.0);
        ws[34144] = cfact * chem_arrhenius_t03(inv_temp, 3.45e-12, 270.0);
        ws[34176] = cfact * chem_arrhenius_t03(inv_temp, 1.4e-13, (-2470.0));
        ws[34272] = cfact * chem_arrhenius_t03(inv_temp, 1.8e-11, 110.0);
        ws[34304] = cfact * chem_arrhenius_t03(inv_temp, 4.5e-14, (-1260.0));
        ws[34336] = 1.7e-11 * cfact;
        ws[34368] = 2e-11 * cfact;
        ws[34400] = 4e-12 * cfact;
        ws[34432] = 1e-17 * cfact;
        ws[34464] = cfact * chem_arrhenius_t03(inv_temp, 8.5e-13, (-2450.0));
        ws[34496] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 3.6e-30, 0.0, (-4.1), 1.9e-12, 0.0, 0.2, 1.33, 0.35);
        ws[34528] = 60.0 * chem_falloff_t10(inv_temp, tempot300, cair, 0.0013, (-11000.0), (-3.5), 970000000000000.0, (-11080.0), 0.1, 1.33, 0.35);
        ws[34592] = 1e-22 * cfact;
        ws[34624] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 7.4e-31, 0.0, (-2.4), 3.3e-11, 0.0, (-0.3), 0.87, 0.81);
        ws[34656] = 5e-40 * cfact_squ;
        ws[34688] = 1e-20 * cfact;
        ws[34752] = cfact * chem_arrhenius_t03(inv_temp, 2.5e-12, 260.0);
        ws[34784] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.8e-30, 0.0, (-3.0), 2.8e-11, 0.0, 0.0, 1.0, 0.6);
        ws[34816] = cfact * chem_falloff_t08(inv_temp, cair, 2.4e-14, 460.0, 2.7e-17, 2199.0, 6.5e-34, 1335.0);
        ws[34880] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.4e-31, 0.0, (-3.1), 4e-12, 0.0, 0.0, 1.26, 0.4);
        ws[34912] = 60.0 * chem_falloff_t10(inv_temp, tempot300, cair, 4.1e-05, (-10650.0), 0.0, 6000000000000000.0, (-11170.0), 0.0, 1.26, 0.4);
        ws[34976] = cfact * chem_arrhenius_t03(inv_temp, 3.2e-13, 690.0);
        ws[35008] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 2.8e-31, 0.0, (-2.6), 2e-12, 0.0, 0.0, 1.1, 0.53);
        ws[35040] = cfact * chem_arrhenius_t03(inv_temp, 7.5e-12, 290.0);
        ws[35072] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 3.61e-28, 0.0, (-6.87), 1.24e-11, 0.0, (-1.105), 1.41, 0.3);
        ws[35104] = 60.0 * chem_falloff_t10(inv_temp, tempot300, cair, 1.1e-05, (-10100.0), 0.0, 1.9e+17, (-14100.0), 0.0, 1.41, 0.3);
        ws[35168] = cfact * chem_arrhenius_t03(inv_temp, 3.14e-12, 580.0);
        ws[35200] = cfact * chem_arrhenius_t03(inv_temp, 4.4e-13, 1070.0);
        ws[35232] = cfact * chem_arrhenius_t03(inv_temp, 2.9e-12, 500.0);
        ws[35264] = ws[35232];
        ws[35296] = cfact * chem_arrhenius_t03(inv_temp, 6.7e-12, 340.0);
        ws[35328] = 0.84 * ws[35072];
        ws[35360] = 0.84 * ws[35104];
        ws[35424] = ws[35168];
        ws[35456] = ws[35200];
        ws[35488] = ws[35232];
        ws[35520] = cfact * chem_arrhenius_t03(inv_temp, 2.4e-12, 360.0);
        ws[35552] = cfact * chem_arrhenius_t03(inv_temp, 4.8e-13, 800.0);
        ws[35584] = cfact * chem_arrhenius_t03(inv_temp, 6.5e-14, 500.0);
        ws[35616] = cfact * chem_arrhenius_t03(inv_temp, 2.3e-12, 360.0);
        ws[35648] = cfact * chem_arrhenius_t03(inv_temp, 3.8e-13, 780.0);
        ws[35680] = cfact * chem_arrhenius_t03(inv_temp, 2e-12, 500.0);
        ws[35712] = ws[35584];
        ws[35744] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[35776] = cfact * chem_arrhenius_t03(inv_temp, 6.8e-13, 800.0);
        ws[35808] = ws[35200];
        ws[35840] = ws[35584];
        ws[35872] = ws[35744];
        ws[35904] = ws[35776];
        ws[35936] = ws[35200];
        ws[35968] = ws[35584];
        ws[36000] = ws[35744];
        ws[36032] = ws[35776];
        ws[36064] = ws[35200];
        ws[36096] = ws[35584];
        ws[36128] = cfact * chem_arrhenius_t03(inv_temp, 5.3e-12, 190.0);
        ws[36192] = cfact * chem_arrhenius_t03(inv_temp, 5.3e-12, 190.0);
        ws[36256] = 2e-12 * cfact;
        ws[36320] = 4.5e-13 * cfact;
        ws[36352] = cfact * chem_arrhenius_t03(inv_temp, 4e-14, 850.0);
        ws[36384] = cfact * chem_arrhenius_t03(inv_temp, 5.3e-12, 190.0);
        ws[36416] = cfact * chem_arrhenius_t03(inv_temp, 5.4e-12, 135.0);
        ws[36512] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-11, (-1600.0));
        ws[36544] = 5.5e-16 * cfact;
        ws[36576] = cfact * chem_arrhenius_t03(inv_temp, 9.7e-15, 625.0);
        ws[36608] = 60.0 * chem_arrhenius_t03(inv_temp, 2400000000000.0, (-7000.0));
        ws[36640] = 5.6e-12 * cfact;
        ws[36672] = cfact * chem_arrhenius_t03(inv_temp, 5.6e-15, 2300.0);
        ws[36704] = cfact * chem_arrhenius_t03(inv_temp, 1.8e-11, (-1100.0));
        ws[36736] = cfact * chem_arrhenius_t03(inv_temp, 4.7e-12, 345.0);
        ws[36768] = cfact * chem_arrhenius_t03(inv_temp, 1.4e-12, (-1860.0));
        ws[36832] = cfact * chem_arrhenius_t03(inv_temp, 1.3e-11, (-870.0));
        ws[36864] = cfact * chem_arrhenius_t03(inv_temp, 4.9e-12, 405.0);
        ws[36896] = 6.3e-15 * cfact;
        ws[36960] = 8e-12 * cfact;
        ws[37024] = ws[36768];
        ws[37056] = cfact * chem_arrhenius_t03(inv_temp, 3.1e-12, 340.0);
        ws[37120] = 4e-16 * cfact;
        ws[37184] = 5e-16 * cfact;
        ws[37216] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-12, 575.0);
        ws[37248] = cfact * chem_arrhenius_t03(inv_temp, 7.7e-12, (-2100.0));
        ws[37280] = cfact * chem_falloff_t09(inv_temp, cair, 1.44e-13, 0.0, 3.43e-33, 0.0);
        ws[37312] = cfact * chem_arrhenius_t03(inv_temp, 1.85e-12, (-1690.0));
        ws[37344] = cfact * chem_arrhenius_t03(inv_temp, 6.9e-12, (-1000.0));
        ws[37376] = cfact * chem_arrhenius_t03(inv_temp, 2.85e-12, (-345.0));
        ws[37408] = cfact * chem_arrhenius_t03(inv_temp, 3e-12, 20.0);
        ws[37504] = cfact * chem_arrhenius_t03(inv_temp, 1.41e-12, (-620.6));
        ws[37536] = cfact * chem_arrhenius_t03(inv_temp, 7.6e-12, (-585.0));
        ws[37568] = 8.1e-13 * cfact;
        ws[37600] = 60.0 * chem_arrhenius_t03(inv_temp, 5700000000000.0, (-5780.0));
        ws[37632] = cfact * chem_arrhenius_t03(inv_temp, 1.5e-14, (-200.0));
        ws[37664] = cfact * chem_arrhenius_t03(inv_temp, 8.6e-12, 400.0);
        ws[37696] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 5e-30, 0.0, (-1.5), 1e-12, 0.0, 0.0, 1.3, 0.37);
        ws[37728] = cfact * chem_arrhenius_t03(inv_temp, 1.04e-11, (-792.0));
        ws[37760] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 8.6e-29, 0.0, (-3.1), 9e-12, 0.0, (-0.85), 1.15, 0.48);
        ws[37792] = cfact * chem_arrhenius_t03(inv_temp, 6.82e-15, (-2500.0));
        ws[37824] = cfact * chem_arrhenius_t03(inv_temp, 3.3e-12, (-2880.0));
        ws[37856] = cfact * chem_arrhenius_t03(inv_temp, 1e-11, (-280.0));
        ws[37888] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 8e-27, 0.0, (-3.5), 3e-11, 0.0, (-1.0), 1.13, 0.5);
        ws[37920] = cfact * chem_arrhenius_t03(inv_temp, 5.5e-15, (-1880.0));
        ws[37952] = cfact * chem_arrhenius_t03(inv_temp, 4.6e-13, (-1155.0));
        ws[37984] = 2.3e-11 * cfact;
        ws[38016] = cfact * chem_arrhenius_t03(inv_temp, 1.05e-11, 519.0);
        ws[38048] = cfact * chem_arrhenius_t03(inv_temp, 4.7e-15, (-1013.0));
        ws[38080] = 3.7e-13 * cfact;
        ws[38112] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-11, 390.0);
        ws[38144] = 3e-11 * cfact;
        ws[38176] = cfact * chem_arrhenius_t03(inv_temp, 2.39e-12, 365.0);
        ws[38208] = cfact * chem_arrhenius_t03(inv_temp, 7.43e-13, 700.0);
        ws[38240] = ws[35200];
        ws[38272] = ws[35584];
        ws[38304] = 60.0 * chem_arrhenius_t03(inv_temp, 3300000000.0, (-8300.0));
        ws[38336] = cfact * chem_arrhenius_t03(inv_temp, 1.03e-14, (-1995.0));
        ws[38368] = cfact * chem_arrhenius_t03(inv_temp, 3.03e-12, (-448.0));
        ws[38400] = cfact * chem_arrhenius_t03(inv_temp, 5.58e-12, 511.0);
        ws[38432] = cfact * chem_arrhenius_t03(inv_temp, 3.88e-15, (-1770.0));
        ws[38464] = cfact * chem_arrhenius_t03(inv_temp, 4.1e-12, (-1860.0));
        ws[38528] = cfact * chem_arrhenius_t03(inv_temp, 2.23e-11, 372.0);
        ws[38592] = cfact * chem_arrhenius_t03(inv_temp, 6e-12, (-1860.0));
        ws[38624] = cfact * chem_arrhenius_t03(inv_temp, 5.78e-11, (-400.0));
        ws[38656] = cfact * chem_arrhenius_t03(inv_temp, 7.43e-13, 700.0);
        ws[38688] = cfact * chem_arrhenius_t03(inv_temp, 2.39e-12, 365.0);
        ws[38720] = ws[35200];
        ws[38752] = ws[35584];
        ws[38784] = 3.1e-11 * cfact;
        ws[38816] = 3.6e-11 * cfact;
        ws[38848] = cfact * chem_arrhenius_t03(inv_temp, 1.5e-11, 449.0);
        ws[38880] = cfact * chem_arrhenius_t03(inv_temp, 1.2e-15, (-821.0));
        ws[38912] = cfact * chem_arrhenius_t03(inv_temp, 3.7e-12, 175.0);
        ws[38944] = 3.6e-11 * cfact;
        ws[38976] = cfact * chem_arrhenius_t03(inv_temp, 1.5e-11, 449.0);
        ws[39008] = cfact * chem_arrhenius_t03(inv_temp, 1.2e-15, (-821.0));
        ws[39040] = cfact * chem_arrhenius_t03(inv_temp, 3.7e-12, 175.0);
        ws[39072] = cfact * chem_arrhenius_t03(inv_temp, 2.3e-12, (-190.0));
        ws[39104] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[39136] = ws[35200];
        ws[39168] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[39200] = ws[35584];
        ws[39232] = cfact * chem_arrhenius_t03(inv_temp, 1.8e-12, 340.0);
        ws[39264] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[39296] = ws[35200];
        ws[39328] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[39360] = ws[35584];
        ws[39392] = 1.85e-11 * cfact;
        ws[39424] = 1.85e-11 * cfact;
        ws[39456] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[39488] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[39520] = ws[35200];
        ws[39552] = ws[35584];
        ws[39584] = cfact * chem_arrhenius_t03(inv_temp, 1.7e-12, 950.0);
        ws[39616] = 1.4e-11 * cfact;
        ws[39648] = 2.1e-12 * cfact;
        ws[39680] = 5.5e-12 * cfact;
        ws[39712] = 1.53e-12 * cfact;
        ws[39744] = 3.8e-12 * cfact;
        ws[39840] = 9e-11 * cfact;
        ws[39872] = cfact * chem_arrhenius_t03(inv_temp, 1.08e-16, (-500.0));
        ws[39904] = 3e-12 * cfact;
        ws[39968] = 4.4e-11 * cfact;
        ws[40000] = cfact * chem_arrhenius_t03(inv_temp, 5.4e-17, (-500.0));
        ws[40032] = 3.8e-12 * cfact;
        ws[40064] = 5e-11 * cfact;
        ws[40096] = 1.7e-10 * cfact;
        ws[40128] = ws[35296];
        ws[40160] = ws[35328];
        ws[40192] = ws[35360];
        ws[40224] = ws[35168];
        ws[40256] = ws[35232];
        ws[40288] = ws[35200];
        ws[40320] = 3.6e-11 * cfact;
        ws[40352] = 3e-12 * cfact;
        ws[40384] = cfact * chem_arrhenius_t03(inv_temp, 1.85e-12, (-1690.0));
        ws[40416] = 60.0 * chem_falloff_t10(inv_temp, tempot300, cair, 2.37e-21, 0.0, 0.0, 0.407, 0.0, (-8.0), 1.0, 0.41);
        ws[40448] = 1.0 * 60.0;
        ws[40480] = 60.0 * chem_falloff_t10(inv_temp, tempot300, cair, 4.81e-20, 0.0, 0.0, 0.407, 0.0, (-8.0), 1.0, 0.41);
        ws[40512] = 1.0 * 60.0;
        ws[40544] = 1.1e-30 * cfact_squ;
        ws[40640] = cfact * chem_arrhenius_t03(inv_temp, 2.3e-11, (-200.0));
        ws[40672] = 1.63e-14 * cfact;
        ws[40704] = cfact * chem_arrhenius_t03(inv_temp, 6.4e-12, 290.0);
        ws[40736] = cfact * chem_arrhenius_t03(inv_temp, 2.2e-12, 340.0);
        ws[40768] = cfact * chem_arrhenius_t03(inv_temp, 3.2e-12, (-110.0));
        ws[40800] = 5e-13 * cfact;
        ws[40864] = cfact * chem_arrhenius_t03(inv_temp, 6.6e-12, (-1240.0));
        ws[40896] = 5e-11 * cfact;
        ws[40928] = 1.4e-10 * cfact;
        ws[40960] = cfact * chem_arrhenius_t03(inv_temp, 8.3e-11, (-100.0));
        ws[40992] = 1.07e-10 * cfact;
        ws[41024] = 2.5e-10 * cfact;
        ws[41056] = 3.5e-10 * cfact;
        ws[41088] = 4.3e-10 * cfact;
        ws[41120] = cfact * chem_arrhenius_t03(inv_temp, 8.2e-11, (-34.0));
        ws[41152] = 7.9e-11 * cfact;
        ws[41184] = 1.3e-10 * cfact;
        ws[41216] = 5.5e-11 * cfact;
        ws[41248] = cfact * chem_arrhenius_t03(inv_temp, 8.2e-11, 45.0);
        ws[41280] = cfact * chem_arrhenius_t04(inv_temp, tempot300, 6.58e-13, 58.0, 1.16);
        ws[41312] = 6.1e-11 * cfact;
        ws[41344] = 1.2e-10 * cfact;
        ws[41376] = 1.2e-10 * cfact;
        ws[41440] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.8e-31, 0.0, (-3.4), 1.5e-11, 0.0, (-1.9), 1.0, 0.6);
        ws[41536] = hetv[0];
        ws[41568] = hetv[1];
        ws[41600] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[41632] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[41664] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[41696] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[41728] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[41760] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[41792] = 1.16e-14 * cfact;
        ws[41824] = 1.97e-10 * cfact;
        ws[41856] = 1.9e-11 * cfact;
        ws[41888] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[41920] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[41952] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 374.0);
        ws[41984] = 1.4 * hetv[2];
        ws[42016] = hetv[3];
        ws[42048] = hetv[4];
        ws[42080] = hetv[5];
        ws[42112] = hetv[6];
        ws[42144] = hetv[7];
        ws[42176] = hetv[7];
        ws[42208] = hetv[8];
        ws[42240] = hetv[9];
        ws[42304] = hetv[10];
        ws[42336] = hetv[11];
        ws[42368] = hetv[12];
        ws[42400] = hetv[13];
        ws[42432] = hetv[14];
        ws[42464] = cfact * chem_arrhenius_t03(inv_temp, 2.6e-12, 380.0);
        ws[42496] = cfact * chem_arrhenius_t03(inv_temp, 2.65e-13, 1300.0);
        ws[42528] = 2.3e-12 * cfact;
        ws[42560] = 3.5e-14 * cfact;
        ws[42592] = 1.92e-10 * cfact;
        ws[42624] = 7.2e-12 * cfact;
        ws[42688] = 9.259e-05 * 60.0;
        ws[42720] = 9.4882e-06 * 60.0;
        ws[42752] = 9.4882e-06 * 60.0;
        ws[42784] = 9.4882e-06 * 60.0;
        ws[42816] = 9.4882e-06 * 60.0;
        ws[42848] = 9.4882e-06 * 60.0;
        ws[42880] = 9.4882e-06 * 60.0;
        ws[42912] = 2.5e-12 * cfact;
        ws[42944] = hetv[15];
        ws[42976] = 2.5e-12 * cfact;
        ws[43008] = hetv[16];
        ws[43040] = 1.25e-11 * cfact;
        ws[43072] = 4e-11 * cfact;
        ws[43104] = 4e-11 * cfact;
        ws[43136] = 4e-11 * cfact;
        ws[43168] = 4e-11 * cfact;
        ws[43200] = 4e-11 * cfact;
        ws[43232] = 4e-11 * cfact;
        ws[43264] = 4e-11 * cfact;
        ws[43296] = 4e-11 * cfact;
        ws[43328] = 4e-11 * cfact;
        ws[43360] = 4e-11 * cfact;
        ws[43392] = cfact * chem_arrhenius_t03(inv_temp, 5.4e-12, 135.0);
        ws[43424] = 5.5e-16 * cfact;
        ws[43456] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-11, (-1600.0));
        ws[43552] = cfact * chem_arrhenius_t03(inv_temp, 8.2e-11, (-34.0));
        ws[43584] = cfact * chem_arrhenius_t03(inv_temp, 4.7e-12, 345.0);
        ws[43616] = cfact * chem_arrhenius_t03(inv_temp, 1.4e-12, (-1860.0));
        ws[43648] = cfact * chem_arrhenius_t03(inv_temp, 1.8e-11, (-1100.0));
        ws[43712] = 7.9e-11 * cfact;
        ws[43744] = cfact * chem_arrhenius_t03(inv_temp, 1.48e-11, 448.0);
        ws[43776] = cfact * chem_arrhenius_t03(inv_temp, 1.34e-14, (-2283.0));
        ws[43808] = 1.79e-13 * cfact;
        ws[43840] = 2.51e-10 * cfact;
        ws[43872] = 2e-11 * cfact;
        ws[43904] = 2.61e-19 * cfact;
        ws[43936] = 1.15e-15 * cfact;
        ws[44000] = 2.37e-10 * cfact;
        ws[44032] = 2e-11 * cfact;
        ws[44064] = 2.61e-19 * cfact;
        ws[44096] = 1.15e-15 * cfact;
        ws[44160] = 2.37e-10 * cfact;
        ws[44192] = cfact * chem_arrhenius_t03(inv_temp, 1.8e-12, 340.0);
        ws[44224] = 6.1e-11 * cfact;
        ws[44256] = cfact * chem_arrhenius_t03(inv_temp, 2.11e-18, (-1256.5));
        ws[44288] = 2.6e-18 * cfact;
        ws[44320] = 8.5e-19 * cfact;
        ws[44352] = 7.7e-14 * cfact;
        ws[44384] = cfact_squ * chem_arrhenius_t03(inv_temp, 2.25e-33, 680.0);
        ws[44416] = cfact * chem_arrhenius_t03(inv_temp, 1.12e-11, (-250.0));
        ws[44448] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.99e-39, 5270.0, 0.0, 1.26e-10, (-340.0), 0.0, 1.0, 1.0);
        ws[44480] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 520.0);
        ws[44512] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-13, 2081.0);
        (void)cair; (void)cfact; (void)cfact_squ; (void)inv_cair; (void)inv_cfact; (void)inv_temp; (void)rfact; (void)rfact_squ; (void)temp; (void)tempot300;
    }
    ws[33408] = ws[33408] * 1000000.0;
    ws[33664] = ws[33664] * 1000000.0;
    ws[44384] = ws[44384] * 1000000.0;
    ws[33408] = ws[33408] * 209500.0;
    ws[34112] = ws[34112] * 209500.0;
    ws[37632] = ws[37632] * 209500.0;
    ws[33696] = ws[33696] * h2o;
    ws[33984] = ws[33984] * h2o;
    ws[34592] = ws[34592] * h2o;
    ws[34656] = ws[34656] * h2o;
    ws[40544] = ws[40544] * h2o;
    ws[37248] = ws[37248] * 0.56;
    ws[37312] = ws[37312] * 1.85;
    ws[40864] = ws[40864] * 1.85;
}
// f(y) for the day reaction list (rbfeval.F:80-151).
__device__ __noinline__ void feval_0(double* __restrict__ ws, int src, int dst)
{
    const double* __restrict__ yin = ws + src * 32;
    double* __restrict__ yout = ws + dst * 32;
    ws[44544] = (ws[33376]) * yin[4608];
    ws[44576] = (ws[33408]) * yin[4160];
    ws[44608] = ((ws[33440]) * yin[4320]) * yin[4384];
    ws[44640] = ((ws[33472]) * yin[4160]) * yin[4384];
    ws[44672] = ((ws[33504]) * yin[4160]) * yin[4608];
    ws[44704] = ((ws[33536]) * yin[4160]) * yin[4608];
    ws[44736] = ((ws[33568]) * yin[4160]) * yin[4320];
    ws[44768] = (ws[33600]) * yin[4320];
    ws[44800] = (ws[33632]) * yin[4320];
    ws[44832] = (ws[33664]) * yin[672];
    ws[44864] = (ws[33696]) * yin[672];
    ws[44896] = ((ws[33728]) * yin[4320]) * yin[4736];
    ws[44928] = ((ws[33760]) * yin[4320]) * yin[4704];
    ws[44960] = ((ws[33792]) * yin[4736]) * yin[4160];
    ws[44992] = ((ws[33824]) * yin[4704]) * yin[4160];
    ws[45024] = ((ws[33856]) * yin[4736]) * yin[4736];
    ws[45056] = ((ws[33888]) * yin[4736]) * yin[4736];
    ws[45088] = ((ws[33920]) * yin[4736]) * yin[4704];
    ws[45120] = ((ws[33952]) * yin[4704]) * yin[4704];
    ws[45152] = ((ws[33984]) * yin[4704]) * yin[4704];
    ws[45184] = (ws[34016]) * yin[3456];
    ws[45216] = ((ws[34048]) * yin[3456]) * yin[4736];
    ws[45248] = ((ws[34080]) * yin[3456]) * yin[4160];
    ws[45280] = ((ws[34112]) * yin[4384]) * yin[4384];
    ws[45312] = ((ws[34144]) * yin[4704]) * yin[4384];
    ws[45344] = ((ws[34176]) * yin[4608]) * yin[4320];
    ws[45376] = (ws[34208]) * yin[4640];
    ws[45408] = (ws[34240]) * yin[4640];
    ws[45440] = ((ws[34272]) * yin[4640]) * yin[4384];
    ws[45472] = ((ws[34304]) * yin[4640]) * yin[4608];
    ws[45504] = ((ws[34336]) * yin[4640]) * yin[4160];
    ws[45536] = ((ws[34368]) * yin[4640]) * yin[4736];
    ws[45568] = ((ws[34400]) * yin[4640]) * yin[4704];
    ws[45600] = ((ws[34432]) * yin[4640]) * yin[4320];
    ws[45632] = ((ws[34464]) * yin[4640]) * yin[4640];
    ws[45664] = ((ws[34496]) * yin[4640]) * yin[4608];
    ws[45696] = (ws[34528]) * yin[1280];
    ws[45728] = (ws[34560]) * yin[1280];
    ws[45760] = (ws[34592]) * yin[1280];
    ws[45792] = ((ws[34624]) * yin[4384]) * yin[4736];
    ws[45824] = ((ws[34656]) * yin[4384]) * yin[4608];
    ws[45856] = ((ws[34688]) * yin[2464]) * yin[2464];
    ws[45888] = (ws[34720]) * yin[2464];
    ws[45920] = ((ws[34752]) * yin[2464]) * yin[4736];
    ws[45952] = ((ws[34784]) * yin[4608]) * yin[4736];
    ws[45984] = ((ws[34816]) * yin[4192]) * yin[4736];
    ws[46016] = (ws[34848]) * yin[4192];
    ws[46048] = ((ws[34880]) * yin[4704]) * yin[4608];
    ws[46080] = (ws[34912]) * yin[1696];
    ws[46112] = (ws[34944]) * yin[1696];
    ws[46144] = ((ws[34976]) * yin[1696]) * yin[4736];
    ws[46176] = ((ws[35008]) * yin[2208]) * yin[4736];
    ws[46208] = ((ws[35040]) * yin[4448]) * yin[4384];
    ws[46240] = ((ws[35072]) * yin[4448]) * yin[4608];
    ws[46272] = (ws[35104]) * yin[1344];
    ws[46304] = (ws[35136]) * yin[1344];
    ws[46336] = ((ws[35168]) * yin[4448]) * yin[4704];
    ws[46368] = ((ws[35200]) * yin[4448]) * yin[4672];
    ws[46400] = ((ws[35232]) * yin[4448]) * yin[4448];
    ws[46432] = ((ws[35264]) * yin[4448]) * yin[4096];
    ws[46464] = ((ws[35296]) * yin[4096]) * yin[4384];
    ws[46496] = ((ws[35328]) * yin[4096]) * yin[4608];
    ws[46528] = (ws[35360]) * yin[1952];
    ws[46560] = (ws[35392]) * yin[1952];
    ws[46592] = ((ws[35424]) * yin[4096]) * yin[4704];
    ws[46624] = ((ws[35456]) * yin[4096]) * yin[4672];
    ws[46656] = ((ws[35488]) * yin[4096]) * yin[4096];
    ws[46688] = ((ws[35520]) * yin[4672]) * yin[4384];
    ws[46720] = ((ws[35552]) * yin[4672]) * yin[4704];
    ws[46752] = ((ws[35584]) * yin[4672]) * yin[4672];
    ws[46784] = ((ws[35616]) * yin[4416]) * yin[4384];
    ws[46816] = ((ws[35648]) * yin[4416]) * yin[4704];
    ws[46848] = ((ws[35680]) * yin[4416]) * yin[4448];
    ws[46880] = ((ws[35712]) * yin[4416]) * yin[4672];
    ws[46912] = ((ws[35744]) * yin[4576]) * yin[4384];
    ws[46944] = ((ws[35776]) * yin[4576]) * yin[4704];
    ws[46976] = ((ws[35808]) * yin[4576]) * yin[4448];
    ws[47008] = ((ws[35840]) * yin[4576]) * yin[4672];
    ws[47040] = ((ws[35872]) * yin[4352]) * yin[4384];
    ws[47072] = ((ws[35904]) * yin[4352]) * yin[4704];
    ws[47104] = ((ws[35936]) * yin[4352]) * yin[4448];
    ws[47136] = ((ws[35968]) * yin[4352]) * yin[4672];
    ws[47168] = ((ws[36000]) * yin[4288]) * yin[4384];
    ws[47200] = ((ws[36032]) * yin[4288]) * yin[4704];
    ws[47232] = ((ws[36064]) * yin[4288]) * yin[4448];
    ws[47264] = ((ws[36096]) * yin[4288]) * yin[4672];
    ws[47296] = ((ws[36128]) * yin[2272]) * yin[4736];
    ws[47328] = (ws[36160]) * yin[2272];
    ws[47360] = ((ws[36192]) * yin[2880]) * yin[4736];
    ws[47392] = (ws[36224]) * yin[2880];
    ws[47424] = ((ws[36256]) * yin[3648]) * yin[4736];
    ws[47456] = (ws[36288]) * yin[3648];
    ws[47488] = ((ws[36320]) * yin[3776]) * yin[4736];
    ws[47520] = ((ws[36352]) * yin[3904]) * yin[4736];
    ws[47552] = ((ws[36384]) * yin[2688]) * yin[4736];
    ws[47584] = ((ws[36416]) * yin[4512]) * yin[4736];
    ws[47616] = (ws[36448]) * yin[4512];
    ws[47648] = (ws[36480]) * yin[4512];
    ws[47680] = ((ws[36512]) * yin[4512]) * yin[4160];
    ws[47712] = ((ws[36544]) * yin[4512]) * yin[4640];
    ws[47744] = ((ws[36576]) * yin[4512]) * yin[4704];
    ws[47776] = (ws[36608]) * yin[1728];
    ws[47808] = ((ws[36640]) * yin[1728]) * yin[4384];
    ws[47840] = ((ws[36672]) * yin[1728]) * yin[4704];
    ws[47872] = ((ws[36704]) * yin[4128]) * yin[4160];
    ws[47904] = ((ws[36736]) * yin[4128]) * yin[4736];
    ws[47936] = ((ws[36768]) * yin[4128]) * yin[4640];
    ws[47968] = (ws[36800]) * yin[4128];
    ws[48000] = ((ws[36832]) * yin[4064]) * yin[4160];
    ws[48032] = ((ws[36864]) * yin[4064]) * yin[4736];
    ws[48064] = ((ws[36896]) * yin[4064]) * yin[4640];
    ws[48096] = (ws[36928]) * yin[4064];
    ws[48128] = ((ws[36960]) * yin[3840]) * yin[4736];
    ws[48160] = (ws[36992]) * yin[3840];
    ws[48192] = ((ws[37024]) * yin[3840]) * yin[4640];
    ws[48224] = ((ws[37056]) * yin[4256]) * yin[4736];
    ws[48256] = (ws[37088]) * yin[4256];
    ws[48288] = ((ws[37120]) * yin[4256]) * yin[4640];
    ws[48320] = (ws[37152]) * yin[4000];
    ws[48352] = ((ws[37184]) * yin[4000]) * yin[4640];
    ws[48384] = ((ws[37216]) * yin[4000]) * yin[4736];
    ws[48416] = (ws[37248]) * yin[4736];
    ws[48448] = ((ws[37280]) * yin[4480]) * yin[4736];
    ws[48480] = (ws[37312]) * yin[4736];
    ws[48512] = ((ws[37344]) * yin[832]) * yin[4736];
    ws[48544] = ((ws[37376]) * yin[2720]) * yin[4736];
    ws[48576] = ((ws[37408]) * yin[864]) * yin[4736];
    ws[48608] = (ws[37440]) * yin[320];
    ws[48640] = (ws[37472]) * yin[3392];
    ws[48672] = ((ws[37504]) * yin[3392]) * yin[4736];
    ws[48704] = ((ws[37536]) * yin[896]) * yin[4736];
    ws[48736] = ((ws[37568]) * yin[4224]) * yin[4736];
    ws[48768] = (ws[37600]) * yin[960];
    ws[48800] = (ws[37632]) * yin[960];
    ws[48832] = ((ws[37664]) * yin[960]) * yin[4608];
    ws[48864] = ((ws[37696]) * yin[352]) * yin[4736];
    ws[48896] = ((ws[37728]) * yin[2656]) * yin[4160];
    ws[48928] = ((ws[37760]) * yin[2656]) * yin[4736];
    ws[48960] = ((ws[37792]) * yin[2656]) * yin[4320];
    ws[48992] = ((ws[37824]) * yin[2656]) * yin[4640];
    ws[49024] = ((ws[37856]) * yin[3552]) * yin[4160];
    ws[49056] = ((ws[37888]) * yin[3552]) * yin[4736];
    ws[49088] = ((ws[37920]) * yin[3552]) * yin[4320];
    ws[49120] = ((ws[37952]) * yin[3552]) * yin[4640];
    ws[49152] = ((ws[37984]) * yin[3136]) * yin[4160];
    ws[49184] = ((ws[38016]) * yin[3136]) * yin[4736];
    ws[49216] = ((ws[38048]) * yin[3136]) * yin[4320];
    ws[49248] = ((ws[38080]) * yin[3136]) * yin[4640];
    ws[49280] = ((ws[38112]) * yin[2528]) * yin[4736];
    ws[49312] = ((ws[38144]) * yin[2528]) * yin[4160];
    ws[49344] = ((ws[38176]) * yin[3424]) * yin[4384];
    ws[49376] = ((ws[38208]) * yin[3424]) * yin[4704];
    ws[49408] = ((ws[38240]) * yin[3424]) * yin[4448];
    ws[49440] = ((ws[38272]) * yin[3424]) * yin[4672];
    ws[49472] = (ws[38304]) * yin[3424];
    ws[49504] = ((ws[38336]) * yin[2528]) * yin[4320];
    ws[49536] = ((ws[38368]) * yin[2528]) * yin[4640];
    ws[49568] = ((ws[38400]) * yin[3872]) * yin[4736];
    ws[49600] = ((ws[38432]) * yin[3872]) * yin[4320];
    ws[49632] = ((ws[38464]) * yin[3872]) * yin[4640];
    ws[49664] = (ws[38496]) * yin[3872];
    ws[49696] = ((ws[38528]) * yin[1664]) * yin[4736];
    ws[49728] = (ws[38560]) * yin[1024];
    ws[49760] = ((ws[38592]) * yin[1024]) * yin[4640];
    ws[49792] = ((ws[38624]) * yin[1056]) * yin[4736];
    ws[49824] = ((ws[38656]) * yin[3296]) * yin[4704];
    ws[49856] = ((ws[38688]) * yin[3296]) * yin[4384];
    ws[49888] = ((ws[38720]) * yin[3296]) * yin[4448];
    ws[49920] = ((ws[38752]) * yin[3296]) * yin[4672];
    ws[49952] = ((ws[38784]) * yin[1632]) * yin[4736];
    ws[49984] = ((ws[38816]) * yin[2048]) * yin[4160];
    ws[50016] = ((ws[38848]) * yin[2048]) * yin[4736];
    ws[50048] = ((ws[38880]) * yin[2048]) * yin[4320];
    ws[50080] = ((ws[38912]) * yin[2048]) * yin[4640];
    ws[50112] = ((ws[38944]) * yin[2112]) * yin[4160];
    ws[50144] = ((ws[38976]) * yin[2112]) * yin[4736];
    ws[50176] = ((ws[39008]) * yin[2112]) * yin[4320];
    ws[50208] = ((ws[39040]) * yin[2112]) * yin[4640];
    ws[50240] = ((ws[39072]) * yin[384]) * yin[4736];
    ws[50272] = ((ws[39104]) * yin[3104]) * yin[4384];
    ws[50304] = ((ws[39136]) * yin[3104]) * yin[4448];
    ws[50336] = ((ws[39168]) * yin[3104]) * yin[4704];
    ws[50368] = ((ws[39200]) * yin[3104]) * yin[4672];
    ws[50400] = ((ws[39232]) * yin[1088]) * yin[4736];
    ws[50432] = ((ws[39264]) * yin[3488]) * yin[4384];
    ws[50464] = ((ws[39296]) * yin[3488]) * yin[4448];
    ws[50496] = ((ws[39328]) * yin[3488]) * yin[4704];
    ws[50528] = ((ws[39360]) * yin[3488]) * yin[4672];
    ws[50560] = ((ws[39392]) * yin[1120]) * yin[4736];
    ws[50592] = ((ws[39424]) * yin[1152]) * yin[4736];
    ws[50624] = ((ws[39456]) * yin[3584]) * yin[4384];
    ws[50656] = ((ws[39488]) * yin[3584]) * yin[4704];
    ws[50688] = ((ws[39520]) * yin[3584]) * yin[4448];
    ws[50720] = ((ws[39552]) * yin[3584]) * yin[4672];
    ws[50752] = ((ws[39584]) * yin[3616]) * yin[4736];
    ws[50784] = ((ws[39616]) * yin[3616]) * yin[4640];
    ws[50816] = ((ws[39648]) * yin[3328]) * yin[4608];
    ws[50848] = ((ws[39680]) * yin[3328]) * yin[4704];
    ws[50880] = ((ws[39712]) * yin[2176]) * yin[4736];
    ws[50912] = ((ws[39744]) * yin[2176]) * yin[4640];
    ws[50944] = (ws[39776]) * yin[2176];
    ws[50976] = (ws[39808]) * yin[3808];
    ws[51008] = ((ws[39840]) * yin[3808]) * yin[4736];
    ws[51040] = ((ws[39872]) * yin[3808]) * yin[4320];
    ws[51072] = ((ws[39904]) * yin[3808]) * yin[4640];
    ws[51104] = (ws[39936]) * yin[3936];
    ws[51136] = ((ws[39968]) * yin[3936]) * yin[4736];
    ws[51168] = ((ws[40000]) * yin[3936]) * yin[4320];
    ws[51200] = ((ws[40032]) * yin[3936]) * yin[4640];
    ws[51232] = ((ws[40064]) * yin[1760]) * yin[4736];
    ws[51264] = ((ws[40096]) * yin[1760]) * yin[4640];
    ws[51296] = ((ws[40128]) * yin[3744]) * yin[4384];
    ws[51328] = ((ws[40160]) * yin[3744]) * yin[4608];
    ws[51360] = (ws[40192]) * yin[1792];
    ws[51392] = ((ws[40224]) * yin[3744]) * yin[4704];
    ws[51424] = ((ws[40256]) * yin[3744]) * yin[4448];
    ws[51456] = ((ws[40288]) * yin[3744]) * yin[4672];
    ws[51488] = ((ws[40320]) * yin[1792]) * yin[4736];
    ws[51520] = ((ws[40352]) * yin[1952]) * yin[4736];
    ws[51552] = ((ws[40384]) * yin[416]) * yin[4736];
    ws[51584] = (ws[40416]) * yin[928];
    ws[51616] = (ws[40448]) * yin[928];
    ws[51648] = (ws[40480]) * yin[1984];
    ws[51680] = (ws[40512]) * yin[1984];
    ws[51712] = ((ws[40544]) * yin[4608]) * yin[4736];
    ws[51744] = (ws[40576]) * yin[1184];
    ws[51776] = (ws[40608]) * yin[1824];
    ws[51808] = ((ws[40640]) * yin[4544]) * yin[4320];
    ws[51840] = ((ws[40672]) * yin[3520]) * yin[3520];
    ws[51872] = ((ws[40704]) * yin[3520]) * yin[4384];
    ws[51904] = ((ws[40736]) * yin[3520]) * yin[4704];
    ws[51936] = ((ws[40768]) * yin[3520]) * yin[4416];
    ws[51968] = ((ws[40800]) * yin[4736]) * yin[3232];
    ws[52000] = (ws[40832]) * yin[3232];
    ws[52032] = (ws[40864]) * yin[4544];
    ws[52064] = ((ws[40896]) * yin[4544]) * yin[4224];
    ws[52096] = ((ws[40928]) * yin[4544]) * yin[896];
    ws[52128] = ((ws[40960]) * yin[4544]) * yin[832];
    ws[52160] = ((ws[40992]) * yin[4544]) * yin[2656];
    ws[52192] = ((ws[41024]) * yin[4544]) * yin[3552];
    ws[52224] = ((ws[41056]) * yin[4544]) * yin[3136];
    ws[52256] = ((ws[41088]) * yin[4544]) * yin[2528];
    ws[52288] = ((ws[41120]) * yin[4544]) * yin[4512];
    ws[52320] = ((ws[41152]) * yin[4544]) * yin[4128];
    ws[52352] = ((ws[41184]) * yin[4544]) * yin[4064];
    ws[52384] = ((ws[41216]) * yin[4544]) * yin[2720];
    ws[52416] = ((ws[41248]) * yin[4544]) * yin[864];
    ws[52448] = ((ws[41280]) * yin[3968]) * yin[4736];
    ws[52480] = ((ws[41312]) * yin[4544]) * yin[1088];
    ws[52512] = ((ws[41344]) * yin[4544]) * yin[1120];
    ws[52544] = ((ws[41376]) * yin[4544]) * yin[1152];
    ws[52576] = (ws[41408]) * yin[2592];
    ws[52608] = ((ws[41440]) * yin[3520]) * yin[4608];
    ws[52640] = (ws[41472]) * yin[1216];
    ws[52672] = (ws[41504]) * yin[1216];
    ws[52704] = (ws[41536]) * yin[1216];
    ws[52736] = (ws[41568]) * yin[1216];
    ws[52768] = ((ws[41600]) * yin[2944]) * yin[4384];
    ws[52800] = ((ws[41632]) * yin[2944]) * yin[4704];
    ws[52832] = ((ws[41664]) * yin[2496]) * yin[4384];
    ws[52864] = ((ws[41696]) * yin[2496]) * yin[4704];
    ws[52896] = ((ws[41728]) * yin[2144]) * yin[4384];
    ws[52928] = ((ws[41760]) * yin[2144]) * yin[4704];
    ws[52960] = ((ws[41792]) * yin[1856]) * yin[4320];
    ws[52992] = ((ws[41824]) * yin[1856]) * yin[4736];
    ws[53024] = ((ws[41856]) * yin[1856]) * yin[4640];
    ws[53056] = ((ws[41888]) * yin[2560]) * yin[4384];
    ws[53088] = ((ws[41920]) * yin[2560]) * yin[4704];
    ws[53120] = ((ws[41952]) * yin[448]) * yin[4736];
    ws[53152] = (ws[41984]) * yin[4032];
    ws[53184] = (ws[42016]) * yin[1280];
    ws[53216] = (ws[42048]) * yin[1280];
    ws[53248] = (ws[42080]) * yin[1920];
    ws[53280] = (ws[42112]) * yin[1248];
    ws[53312] = ((ws[42144]) * yin[1920]) * yin[480];
    ws[53344] = ((ws[42176]) * yin[1920]) * yin[512];
    ws[53376] = ((ws[42208]) * yin[1248]) * yin[544];
    ws[53408] = (ws[42240]) * yin[4608];
    ws[53440] = (ws[42272]) * yin[4320];
    ws[53472] = (ws[42304]) * yin[1056];
    ws[53504] = ((ws[42336]) * yin[1312]) * yin[576];
    ws[53536] = (ws[42368]) * yin[1312];
    ws[53568] = (ws[42400]) * yin[4256];
    ws[53600] = (ws[42432]) * yin[4000];
    ws[53632] = ((ws[42464]) * yin[2848]) * yin[4384];
    ws[53664] = ((ws[42496]) * yin[2848]) * yin[4704];
    ws[53696] = ((ws[42528]) * yin[2848]) * yin[4640];
    ws[53728] = ((ws[42560]) * yin[2848]) * yin[4672];
    ws[53760] = ((ws[42592]) * yin[3360]) * yin[4544];
    ws[53792] = ((ws[42624]) * yin[3360]) * yin[4736];
    ws[53824] = (ws[42656]) * yin[3360];
    ws[53856] = (ws[42688]) * yin[0];
    ws[53888] = (ws[42720]) * yin[64];
    ws[53920] = (ws[42752]) * yin[96];
    ws[53952] = (ws[42784]) * yin[128];
    ws[53984] = (ws[42816]) * yin[160];
    ws[54016] = (ws[42848]) * yin[192];
    ws[54048] = (ws[42880]) * yin[224];
    ws[54080] = ((ws[42912]) * yin[704]) * yin[4736];
    ws[54112] = ((ws[42944]) * yin[1440]) * yin[4736];
    ws[54144] = ((ws[42976]) * yin[736]) * yin[4736];
    ws[54176] = ((ws[43008]) * yin[1472]) * yin[4736];
    ws[54208] = ((ws[43040]) * yin[768]) * yin[4736];
    ws[54240] = ((ws[43072]) * yin[2752]) * yin[4736];
    ws[54272] = ((ws[43104]) * yin[2784]) * yin[4736];
    ws[54304] = ((ws[43136]) * yin[2816]) * yin[4736];
    ws[54336] = ((ws[43168]) * yin[2304]) * yin[4736];
    ws[54368] = ((ws[43200]) * yin[1504]) * yin[4736];
    ws[54400] = ((ws[43232]) * yin[3680]) * yin[4736];
    ws[54432] = ((ws[43264]) * yin[3712]) * yin[4736];
    ws[54464] = ((ws[43296]) * yin[2912]) * yin[4736];
    ws[54496] = ((ws[43328]) * yin[3168]) * yin[4736];
    ws[54528] = ((ws[43360]) * yin[3200]) * yin[4736];
    ws[54560] = ((ws[43392]) * yin[2336]) * yin[4736];
    ws[54592] = ((ws[43424]) * yin[2336]) * yin[4640];
    ws[54624] = ((ws[43456]) * yin[2336]) * yin[4160];
    ws[54656] = (ws[43488]) * yin[2336];
    ws[54688] = (ws[43520]) * yin[2336];
    ws[54720] = ((ws[43552]) * yin[2336]) * yin[4544];
    ws[54752] = ((ws[43584]) * yin[2368]) * yin[4736];
    ws[54784] = ((ws[43616]) * yin[2368]) * yin[4640];
    ws[54816] = ((ws[43648]) * yin[2368]) * yin[4160];
    ws[54848] = (ws[43680]) * yin[2368];
    ws[54880] = ((ws[43712]) * yin[2368]) * yin[4544];
    ws[54912] = ((ws[43744]) * yin[2400]) * yin[4736];
    ws[54944] = ((ws[43776]) * yin[2400]) * yin[4320];
    ws[54976] = ((ws[43808]) * yin[2400]) * yin[4640];
    ws[55008] = ((ws[43840]) * yin[2400]) * yin[4544];
    ws[55040] = ((ws[43872]) * yin[2432]) * yin[4736];
    ws[55072] = ((ws[43904]) * yin[2432]) * yin[4320];
    ws[55104] = ((ws[43936]) * yin[2432]) * yin[4640];
    ws[55136] = (ws[43968]) * yin[2432];
    ws[55168] = ((ws[44000]) * yin[2432]) * yin[4544];
    ws[55200] = ((ws[44032]) * yin[2976]) * yin[4736];
    ws[55232] = ((ws[44064]) * yin[2976]) * yin[4320];
    ws[55264] = ((ws[44096]) * yin[2976]) * yin[4640];
    ws[55296] = (ws[44128]) * yin[2976];
    ws[55328] = ((ws[44160]) * yin[2976]) * yin[4544];
    ws[55360] = ((ws[44192]) * yin[1536]) * yin[4736];
    ws[55392] = ((ws[44224]) * yin[1536]) * yin[4544];
    ws[55424] = ((ws[44256]) * yin[3008]) * yin[4320];
    ws[55456] = ((ws[44288]) * yin[3008]) * yin[1184];
    ws[55488] = ((ws[44320]) * yin[3008]) * yin[3456];
    ws[55520] = ((ws[44352]) * yin[3008]) * yin[4736];
    ws[55552] = ((ws[44384]) * yin[3008]) * yin[4544];
    ws[55584] = ((ws[44416]) * yin[2016]) * yin[4736];
    ws[55616] = ((ws[44448]) * yin[2016]) * yin[4736];
    ws[55648] = ((ws[44480]) * yin[2016]) * yin[4640];
    ws[55680] = ((ws[44512]) * yin[2016]) * yin[4544];
    {
      double a = -ws[53856];
      yout[0] = a;
    }
    {
      double a = 1.0 * ws[53856];
      yout[32] = a;
    }
    {
      double a = -ws[53888];
      yout[64] = a;
    }
    {
      double a = -ws[53920];
      yout[96] = a;
    }
    {
      double a = -ws[53952];
      yout[128] = a;
    }
    {
      double a = -ws[53984];
      yout[160] = a;
    }
    {
      double a = -ws[54016];
      yout[192] = a;
    }
    {
      double a = -ws[54048];
      yout[224] = a;
    }
    {
      double a = 1.0 * ws[46176];
      yout[256] = a;
    }
    {
      double a = 1.0 * ws[46176];
      yout[288] = a;
    }
    {
      double a = -ws[48608];
      a = fma(0.2, ws[48768], a);
      a = fma(1.0, ws[48800], a);
      yout[320] = a;
    }
    {
      double a = -ws[48864];
      yout[352] = a;
    }
    {
      double a = -ws[50240];
      yout[384] = a;
    }
    {
      double a = -ws[51552];
      yout[416] = a;
    }
    {
      double a = -ws[53120];
      yout[448] = a;
    }
    {
      double a = -ws[53312];
      yout[480] = a;
    }
    {
      double a = -ws[53344];
      yout[512] = a;
    }
    {
      double a = -ws[53376];
      yout[544] = a;
    }
    {
      double a = -ws[53504];
      yout[576] = a;
    }
    {
      double a = 1.0 * ws[53504];
      a = fma(1.0, ws[53536], a);
      yout[608] = a;
    }
    {
      double a = 1.0 * ws[53568];
      a = fma(1.0, ws[53600], a);
      yout[640] = a;
    }
    {
      double a = 1.0 * ws[44800];
      a = a - ws[44832];
      a = a - ws[44864];
      yout[672] = a;
    }
    {
      double a = -ws[54080];
      a = fma(1.0, ws[54080], a);
      yout[704] = a;
    }
    {
      double a = -ws[54144];
      a = fma(1.0, ws[54144], a);
      yout[736] = a;
    }
    {
      double a = -ws[54208];
      yout[768] = a;
    }
    {
      double a = 1.0 * ws[54208];
      yout[800] = a;
    }
    {
      double a = -ws[48512];
      a = a - ws[52128];
      yout[832] = a;
    }
    {
      double a = -ws[48576];
      a = a - ws[52416];
      yout[864] = a;
    }
    {
      double a = -ws[48704];
      a = a - ws[52096];
      yout[896] = a;
    }
    {
      double a = 1.0 * ws[48704];
      a = a - ws[51584];
      a = a - ws[51616];
      yout[928] = a;
    }
    {
      double a = -ws[48768];
      a = fma(0.02, ws[48768], a);
      a = a - ws[48800];
      a = a - ws[48832];
      a = fma(0.874, ws[51680], a);
      yout[960] = a;
    }
    {
      double a = 1.0 * ws[49280];
      a = fma(1.0, ws[49536], a);
      yout[992] = a;
    }
    {
      double a = 1.0 * ws[49472];
      a = a - ws[49728];
      a = a - ws[49760];
      yout[1024] = a;
    }
    {
      double a = 0.904 * ws[49696];
      a = a - ws[49792];
      a = a - ws[53472];
      yout[1056] = a;
    }
    {
      double a = -ws[50400];
      a = a - ws[52480];
      yout[1088] = a;
    }
    {
      double a = -ws[50560];
      a = a - ws[52512];
      yout[1120] = a;
    }
    {
      double a = -ws[50592];
      a = a - ws[52544];
      yout[1152] = a;
    }
    {
      double a = -ws[51744];
      a = fma(0.3, ws[51840], a);
      a = a - ws[55456];
      a = fma(1.0, ws[55456], a);
      yout[1184] = a;
    }
    {
      double a = 1.0 * ws[52608];
      a = a - ws[52640];
      a = a - ws[52672];
      a = a - ws[52704];
      a = a - ws[52736];
      yout[1216] = a;
    }
    {
      double a = 1.0 * ws[53216];
      a = a - ws[53280];
      a = a - ws[53376];
      yout[1248] = a;
    }
    {
      double a = 1.0 * ws[45664];
      a = a - ws[45696];
      a = a - ws[45728];
      a = a - ws[45760];
      a = a - ws[53184];
      a = a - ws[53216];
      yout[1280] = a;
    }
    {
      double a = 1.0 * ws[53472];
      a = a - ws[53504];
      a = a - ws[53536];
      yout[1312] = a;
    }
    {
      double a = 1.0 * ws[46240];
      a = a - ws[46272];
      a = a - ws[46304];
      yout[1344] = a;
    }
    {
      double a = 0.907 * ws[53888];
      a = fma(0.925, ws[53920], a);
      a = fma(0.943, ws[53952], a);
      yout[1376] = a;
    }
    {
      double a = 0.5 * ws[53984];
      a = fma(0.5, ws[54016], a);
      a = fma(1.5, ws[54048], a);
      yout[1408] = a;
    }
    {
      double a = 1.25 * ws[54080];
      a = a - ws[54112];
      yout[1440] = a;
    }
    {
      double a = 1.25 * ws[54144];
      a = a - ws[54176];
      yout[1472] = a;
    }
    {
      double a = 0.0023 * ws[54240];
      a = a - ws[54368];
      yout[1504] = a;
    }
    {
      double a = -ws[55360];
      a = a - ws[55392];
      yout[1536] = a;
    }
    {
      double a = 0.5 * ws[55424];
      a = fma(0.5, ws[55520], a);
      yout[1568] = a;
    }
    {
      double a = 0.25 * ws[55616];
      a = fma(0.14, ws[55680], a);
      yout[1600] = a;
    }
    {
      double a = 0.1 * ws[49344];
      a = a - ws[49952];
      a = fma(0.104, ws[49952], a);
      yout[1632] = a;
    }
    {
      double a = 0.88 * ws[49376];
      a = a - ws[49696];
      yout[1664] = a;
    }
    {
      double a = 1.0 * ws[46048];
      a = a - ws[46080];
      a = a - ws[46112];
      a = a - ws[46144];
      yout[1696] = a;
    }
    {
      double a = 1.0 * ws[47744];
      a = a - ws[47776];
      a = a - ws[47808];
      a = a - ws[47840];
      yout[1728] = a;
    }
    {
      double a = 0.732 * ws[50752];
      a = a - ws[51232];
      a = a - ws[51264];
      yout[1760] = a;
    }
    {
      double a = 1.0 * ws[51328];
      a = a - ws[51360];
      a = a - ws[51488];
      yout[1792] = a;
    }
    {
      double a = -ws[51776];
      a = fma(1.0, ws[51904], a);
      a = fma(1.0, ws[52704], a);
      a = fma(1.0, ws[52736], a);
      yout[1824] = a;
    }
    {
      double a = -ws[52960];
      a = a - ws[52992];
      a = a - ws[53024];
      yout[1856] = a;
    }
    {
      double a = 1.0 * ws[52960];
      a = fma(1.0, ws[52992], a);
      a = fma(1.0, ws[53024], a);
      yout[1888] = a;
    }
    {
      double a = 1.0 * ws[53184];
      a = a - ws[53248];
      a = a - ws[53312];
      a = a - ws[53344];
      yout[1920] = a;
    }
    {
      double a = 1.0 * ws[46496];
      a = a - ws[46528];
      a = a - ws[46560];
      a = a - ws[51520];
      yout[1952] = a;
    }
    {
      double a = 1.0 * ws[48736];
      a = a - ws[51648];
      a = a - ws[51680];
      a = fma(1.0, ws[52064], a);
      yout[1984] = a;
    }
    {
      double a = -ws[55584];
      a = a - ws[55616];
      a = a - ws[55648];
      a = a - ws[55680];
      yout[2016] = a;
    }
    {
      double a = -ws[49984];
      a = a - ws[50016];
      a = a - ws[50048];
      a = a - ws[50080];
      yout[2048] = a;
    }
    {
      double a = 1.0 * ws[49984];
      a = fma(1.0, ws[50016], a);
      a = fma(1.0, ws[50048], a);
      a = fma(1.0, ws[50112], a);
      a = fma(1.0, ws[50144], a);
      a = fma(1.0, ws[50176], a);
      yout[2080] = a;
    }
    {
      double a = -ws[50112];
      a = a - ws[50144];
      a = a - ws[50176];
      a = a - ws[50208];
      yout[2112] = a;
    }
    {
      double a = 1.0 * ws[50240];
      a = a - ws[52896];
      a = a - ws[52928];
      yout[2144] = a;
    }
    {
      double a = 1.0 * ws[50816];
      a = a - ws[50880];
      a = a - ws[50912];
      a = a - ws[50944];
      yout[2176] = a;
    }
    {
      double a = -ws[46176];
      a = fma(1.0, ws[55584], a);
      a = fma(0.75, ws[55616], a);
      a = fma(1.0, ws[55648], a);
      a = fma(0.86, ws[55680], a);
      yout[2208] = a;
    }
    {
      double a = 0.14 * ws[52800];
      a = fma(0.193, ws[52864], a);
      a = fma(0.146, ws[52928], a);
      a = fma(0.473, ws[53088], a);
      yout[2240] = a;
    }
    {
      double a = 0.9 * ws[46816];
      a = a - ws[47296];
      a = a - ws[47328];
      a = fma(0.5, ws[47840], a);
      yout[2272] = a;
    }
    {
      double a = 0.0026 * ws[54240];
      a = fma(0.0035, ws[54272], a);
      a = fma(0.0005, ws[54304], a);
      a = a - ws[54336];
      a = fma(0.1043, ws[54336], a);
      yout[2304] = a;
    }
    {
      double a = -ws[54560];
      a = a - ws[54592];
      a = a - ws[54624];
      a = a - ws[54656];
      a = a - ws[54688];
      a = a - ws[54720];
      yout[2336] = a;
    }
    {
      double a = -ws[54752];
      a = a - ws[54784];
      a = a - ws[54816];
      a = a - ws[54848];
      a = a - ws[54880];
      yout[2368] = a;
    }
    {
      double a = -ws[54912];
      a = a - ws[54944];
      a = a - ws[54976];
      a = a - ws[55008];
      yout[2400] = a;
    }
    {
      double a = -ws[55040];
      a = a - ws[55072];
      a = a - ws[55104];
      a = a - ws[55136];
      a = a - ws[55168];
      yout[2432] = a;
    }
    {
      double a = 1.0 * ws[45792];
      a = fma(2.0, ws[45824], a);
      a = a - ws[45856];
      a = a - ws[45856];
      a = a - ws[45888];
      a = a - ws[45920];
      a = fma(1.0, ws[50944], a);
      a = fma(0.5, ws[53408], a);
      yout[2464] = a;
    }
    {
      double a = 1.0 * ws[50560];
      a = fma(1.0, ws[52512], a);
      a = a - ws[52832];
      a = a - ws[52864];
      yout[2496] = a;
    }
    {
      double a = -ws[49280];
      a = a - ws[49312];
      a = a - ws[49504];
      a = a - ws[49536];
      a = a - ws[52256];
      yout[2528] = a;
    }
    {
      double a = 1.0 * ws[50592];
      a = fma(1.0, ws[52544], a);
      a = a - ws[53056];
      a = a - ws[53088];
      yout[2560] = a;
    }
    {
      double a = -ws[52576];
      a = fma(1.0, ws[53312], a);
      a = fma(1.0, ws[53344], a);
      a = fma(1.0, ws[53376], a);
      yout[2592] = a;
    }
    {
      double a = 0.051 * ws[52768];
      a = fma(0.023, ws[52832], a);
      a = fma(0.225, ws[53056], a);
      a = fma(0.052, ws[53120], a);
      yout[2624] = a;
    }
    {
      double a = -ws[48896];
      a = a - ws[48928];
      a = a - ws[48960];
      a = a - ws[48992];
      a = a - ws[52160];
      yout[2656] = a;
    }
    {
      double a = 0.37 * ws[46336];
      a = fma(0.37, ws[46592], a);
      a = a - ws[47552];
      a = fma(0.37, ws[51392], a);
      yout[2688] = a;
    }
    {
      double a = 0.315 * ws[46880];
      a = fma(0.15, ws[48160], a);
      a = a - ws[48544];
      a = a - ws[52384];
      yout[2720] = a;
    }
    {
      double a = -ws[54240];
      a = fma(0.4857, ws[54240], a);
      a = fma(0.3003, ws[54272], a);
      a = fma(0.3856, ws[54304], a);
      a = fma(0.2181, ws[54336], a);
      a = fma(0.2412, ws[54368], a);
      yout[2752] = a;
    }
    {
      double a = 0.0062 * ws[54240];
      a = a - ws[54272];
      a = fma(0.2862, ws[54272], a);
      a = fma(0.095, ws[54304], a);
      a = fma(0.3063, ws[54336], a);
      a = fma(0.2089, ws[54368], a);
      yout[2784] = a;
    }
    {
      double a = 0.0025 * ws[54240];
      a = fma(0.0041, ws[54272], a);
      a = a - ws[54304];
      a = fma(0.1373, ws[54304], a);
      a = fma(0.0153, ws[54336], a);
      a = fma(0.3, ws[54368], a);
      yout[2816] = a;
    }
    {
      double a = 1.0 * ws[50080];
      a = a - ws[53632];
      a = a - ws[53664];
      a = a - ws[53696];
      a = a - ws[53728];
      yout[2848] = a;
    }
    {
      double a = 1.0 * ws[46944];
      a = fma(1.0, ws[47072], a);
      a = fma(1.0, ws[47200], a);
      a = a - ws[47360];
      a = a - ws[47392];
      yout[2880] = a;
    }
    {
      double a = 0.0123 * ws[54400];
      a = fma(0.0139, ws[54432], a);
      a = a - ws[54464];
      a = fma(0.2607, ws[54464], a);
      a = fma(0.0491, ws[54496], a);
      a = fma(0.064, ws[54528], a);
      yout[2912] = a;
    }
    {
      double a = 1.0 * ws[50400];
      a = fma(1.0, ws[52480], a);
      a = a - ws[52768];
      a = a - ws[52800];
      yout[2944] = a;
    }
    {
      double a = 0.58 * ws[54912];
      a = fma(0.52, ws[54944], a);
      a = fma(0.045, ws[54976], a);
      a = fma(0.58, ws[55008], a);
      a = a - ws[55200];
      a = a - ws[55232];
      a = a - ws[55264];
      a = a - ws[55296];
      a = a - ws[55328];
      yout[2976] = a;
    }
    {
      double a = -ws[55424];
      a = a - ws[55456];
      a = a - ws[55488];
      a = a - ws[55520];
      a = a - ws[55552];
      a = fma(0.5, ws[55552], a);
      yout[3008] = a;
    }
    {
      double a = 0.5 * ws[55424];
      a = fma(1.0, ws[55456], a);
      a = fma(1.0, ws[55488], a);
      a = fma(0.5, ws[55520], a);
      a = fma(0.5, ws[55552], a);
      yout[3040] = a;
    }
    {
      double a = 0.047 * ws[52768];
      a = fma(0.06, ws[52832], a);
      a = fma(0.392, ws[52896], a);
      a = fma(0.191, ws[53056], a);
      a = fma(0.081, ws[53120], a);
      yout[3072] = a;
    }
    {
      double a = 0.352 * ws[50240];
      a = a - ws[50272];
      a = a - ws[50304];
      a = a - ws[50336];
      a = a - ws[50368];
      yout[3104] = a;
    }
    {
      double a = -ws[49152];
      a = a - ws[49184];
      a = a - ws[49216];
      a = a - ws[49248];
      a = fma(0.029, ws[49696], a);
      a = a - ws[52224];
      yout[3136] = a;
    }
    {
      double a = 0.0019 * ws[54240];
      a = fma(0.1239, ws[54400], a);
      a = fma(0.1027, ws[54432], a);
      a = fma(0.0702, ws[54464], a);
      a = a - ws[54496];
      a = fma(0.2577, ws[54496], a);
      a = fma(0.0385, ws[54528], a);
      yout[3168] = a;
    }
    {
      double a = 0.0023 * ws[54240];
      a = fma(0.1831, ws[54400], a);
      a = fma(0.2045, ws[54432], a);
      a = fma(0.1116, ws[54464], a);
      a = fma(0.0739, ws[54496], a);
      a = a - ws[54528];
      a = fma(0.2667, ws[54528], a);
      yout[3200] = a;
    }
    {
      double a = -ws[51968];
      a = a - ws[52000];
      a = fma(1.0, ws[52160], a);
      a = fma(1.0, ws[52192], a);
      a = fma(0.7, ws[52224], a);
      a = fma(1.0, ws[52256], a);
      yout[3232] = a;
    }
    {
      double a = 0.016 * ws[52768];
      a = fma(0.015, ws[52832], a);
      a = fma(0.034, ws[52896], a);
      a = fma(0.028, ws[53056], a);
      a = fma(0.006, ws[53120], a);
      yout[3264] = a;
    }
    {
      double a = 1.0 * ws[49792];
      a = a - ws[49824];
      a = a - ws[49856];
      a = a - ws[49888];
      a = a - ws[49920];
      yout[3296] = a;
    }
    {
      double a = 0.2 * ws[50752];
      a = fma(0.3, ws[50784], a);
      a = a - ws[50816];
      a = a - ws[50848];
      a = fma(0.5, ws[50880], a);
      a = fma(0.5, ws[50912], a);
      a = fma(0.5, ws[51232], a);
      a = fma(1.0, ws[51264], a);
      yout[3328] = a;
    }
    {
      double a = 0.688 * ws[53632];
      a = fma(1.0, ws[53664], a);
      a = fma(0.422, ws[53696], a);
      a = fma(0.711, ws[53728], a);
      a = a - ws[53760];
      a = fma(0.37, ws[53760], a);
      a = a - ws[53792];
      a = fma(0.24, ws[53792], a);
      a = a - ws[53824];
      yout[3360] = a;
    }
    {
      double a = -ws[48640];
      a = a - ws[48672];
      a = fma(0.42, ws[48768], a);
      a = fma(0.137, ws[49568], a);
      a = fma(0.17, ws[49600], a);
      a = fma(0.17, ws[49664], a);
      a = fma(0.732, ws[51616], a);
      a = fma(1.0, ws[52096], a);
      yout[3392] = a;
    }
    {
      double a = 1.0 * ws[49280];
      a = a - ws[49344];
      a = a - ws[49376];
      a = a - ws[49408];
      a = a - ws[49440];
      a = a - ws[49472];
      a = fma(0.067, ws[49696], a);
      yout[3424] = a;
    }
    {
      double a = 1.0 * ws[45056];
      a = fma(1.0, ws[45120], a);
      a = fma(1.0, ws[45152], a);
      a = a - ws[45184];
      a = a - ws[45216];
      a = a - ws[45248];
      a = fma(0.04, ws[49088], a);
      a = fma(0.08, ws[49216], a);
      a = a - ws[55488];
      a = fma(1.0, ws[55488], a);
      yout[3456] = a;
    }
    {
      double a = 0.65 * ws[50400];
      a = a - ws[50432];
      a = a - ws[50464];
      a = a - ws[50496];
      a = a - ws[50528];
      a = fma(0.65, ws[52480], a);
      yout[3488] = a;
    }
    {
      double a = 1.0 * ws[51808];
      a = a - ws[51840];
      a = a - ws[51840];
      a = a - ws[51872];
      a = a - ws[51904];
      a = a - ws[51936];
      a = a - ws[52608];
      a = fma(1.0, ws[52640], a);
      a = fma(0.55, ws[55680], a);
      yout[3520] = a;
    }
    {
      double a = -ws[49024];
      a = a - ws[49056];
      a = a - ws[49088];
      a = a - ws[49120];
      a = fma(0.24, ws[49664], a);
      a = fma(0.098, ws[49952], a);
      a = a - ws[52192];
      a = fma(0.3, ws[52224], a);
      yout[3552] = a;
    }
    {
      double a = 0.544 * ws[50560];
      a = fma(0.544, ws[50592], a);
      a = a - ws[50624];
      a = a - ws[50656];
      a = a - ws[50688];
      a = a - ws[50720];
      a = fma(0.544, ws[52512], a);
      a = fma(0.544, ws[52544], a);
      yout[3584] = a;
    }
    {
      double a = 0.53 * ws[50240];
      a = fma(0.18, ws[50400], a);
      a = fma(0.155, ws[50560], a);
      a = fma(0.155, ws[50592], a);
      a = a - ws[50752];
      a = a - ws[50784];
      a = fma(1.0, ws[50848], a);
      a = fma(0.18, ws[52480], a);
      a = fma(0.155, ws[52512], a);
      a = fma(0.155, ws[52544], a);
      yout[3616] = a;
    }
    {
      double a = 0.5 * ws[47168];
      a = a - ws[47424];
      a = a - ws[47456];
      a = fma(1.0, ws[48832], a);
      a = fma(0.5, ws[48992], a);
      a = fma(0.5, ws[49120], a);
      a = fma(0.5, ws[49248], a);
      yout[3648] = a;
    }
    {
      double a = 0.2944 * ws[54240];
      a = fma(0.2239, ws[54272], a);
      a = fma(0.2051, ws[54304], a);
      a = fma(0.1893, ws[54336], a);
      a = fma(0.2028, ws[54368], a);
      a = a - ws[54400];
      a = fma(0.6664, ws[54400], a);
      a = fma(0.2858, ws[54432], a);
      a = fma(0.3303, ws[54464], a);
      a = fma(0.3444, ws[54496], a);
      a = fma(0.3886, ws[54528], a);
      yout[3680] = a;
    }
    {
      double a = 0.2021 * ws[54240];
      a = fma(0.182, ws[54272], a);
      a = fma(0.1764, ws[54304], a);
      a = fma(0.1668, ws[54336], a);
      a = fma(0.0471, ws[54368], a);
      a = fma(0.0143, ws[54400], a);
      a = a - ws[54432];
      a = fma(0.3931, ws[54432], a);
      a = fma(0.2272, ws[54464], a);
      a = fma(0.2749, ws[54496], a);
      a = fma(0.2421, ws[54528], a);
      yout[3712] = a;
    }
    {
      double a = 0.457 * ws[49568];
      a = fma(0.48, ws[50784], a);
      a = fma(1.0, ws[51104], a);
      a = fma(0.6, ws[51136], a);
      a = fma(1.0, ws[51200], a);
      a = a - ws[51296];
      a = a - ws[51328];
      a = fma(1.0, ws[51360], a);
      a = a - ws[51392];
      a = a - ws[51424];
      a = a - ws[51456];
      yout[3744] = a;
    }
    {
      double a = -ws[47488];
      a = fma(1.0, ws[47808], a);
      a = fma(0.5, ws[47840], a);
      a = fma(0.3, ws[48864], a);
      a = fma(0.42, ws[48960], a);
      a = fma(0.09, ws[49088], a);
      a = fma(0.15, ws[49600], a);
      a = fma(0.074, ws[49824], a);
      a = fma(0.185, ws[49952], a);
      yout[3776] = a;
    }
    {
      double a = 0.2 * ws[50432];
      a = fma(0.23, ws[50464], a);
      a = fma(0.23, ws[50528], a);
      a = fma(0.244, ws[50560], a);
      a = fma(0.244, ws[50592], a);
      a = fma(0.56, ws[50624], a);
      a = fma(0.65, ws[50688], a);
      a = fma(0.65, ws[50720], a);
      a = a - ws[50976];
      a = a - ws[51008];
      a = a - ws[51040];
      a = a - ws[51072];
      a = fma(0.244, ws[52512], a);
      a = fma(0.244, ws[52544], a);
      yout[3808] = a;
    }
    {
      double a = -ws[48128];
      a = a - ws[48160];
      a = a - ws[48192];
      a = fma(0.011, ws[48576], a);
      a = fma(0.22, ws[48928], a);
      a = fma(0.269, ws[49568], a);
      a = fma(0.113, ws[49632], a);
      a = fma(0.128, ws[49664], a);
      a = fma(0.275, ws[49824], a);
      a = fma(0.275, ws[49856], a);
      a = fma(0.22, ws[49888], a);
      a = fma(0.275, ws[49920], a);
      a = fma(0.331, ws[49952], a);
      yout[3840] = a;
    }
    {
      double a = 0.75 * ws[49312];
      a = fma(0.9, ws[49344], a);
      a = fma(0.12, ws[49376], a);
      a = fma(1.0, ws[49408], a);
      a = fma(1.0, ws[49440], a);
      a = fma(0.65, ws[49504], a);
      a = fma(0.35, ws[49536], a);
      a = a - ws[49568];
      a = a - ws[49600];
      a = a - ws[49632];
      a = a - ws[49664];
      a = fma(1.0, ws[49728], a);
      a = fma(1.0, ws[49760], a);
      a = fma(1.0, ws[52256], a);
      yout[3872] = a;
    }
    {
      double a = 0.13 * ws[46336];
      a = fma(0.13, ws[46592], a);
      a = fma(0.1, ws[46848], a);
      a = fma(0.2, ws[46976], a);
      a = fma(0.2, ws[47104], a);
      a = fma(0.2, ws[47232], a);
      a = a - ws[47520];
      a = fma(0.13, ws[49088], a);
      a = fma(0.08, ws[49216], a);
      a = fma(0.2, ws[49408], a);
      a = fma(0.2, ws[49888], a);
      a = fma(0.13, ws[51392], a);
      a = fma(0.2, ws[51456], a);
      yout[3904] = a;
    }
    {
      double a = 0.118 * ws[50240];
      a = fma(0.918, ws[50272], a);
      a = fma(1.0, ws[50304], a);
      a = fma(1.0, ws[50368], a);
      a = fma(0.1, ws[50400], a);
      a = fma(0.66, ws[50432], a);
      a = fma(0.77, ws[50464], a);
      a = fma(0.77, ws[50528], a);
      a = fma(0.3, ws[50624], a);
      a = fma(0.35, ws[50688], a);
      a = fma(0.35, ws[50720], a);
      a = fma(0.025, ws[50752], a);
      a = fma(1.0, ws[50944], a);
      a = fma(0.25, ws[51072], a);
      a = a - ws[51104];
      a = a - ws[51136];
      a = a - ws[51168];
      a = a - ws[51200];
      a = fma(0.1, ws[52480], a);
      yout[3936] = a;
    }
    {
      double a = 1.0 * ws[52032];
      a = fma(1.0, ws[52064], a);
      a = fma(1.0, ws[52096], a);
      a = fma(1.0, ws[52128], a);
      a = fma(0.3, ws[52224], a);
      a = fma(1.0, ws[52288], a);
      a = fma(1.0, ws[52320], a);
      a = fma(1.0, ws[52352], a);
      a = fma(1.0, ws[52384], a);
      a = fma(1.0, ws[52416], a);
      a = a - ws[52448];
      a = fma(1.0, ws[52480], a);
      a = fma(1.0, ws[52512], a);
      a = fma(1.0, ws[52544], a);
      a = fma(0.45, ws[55680], a);
      yout[3968] = a;
    }
    {
      double a = -ws[48320];
      a = a - ws[48352];
      a = a - ws[48384];
      a = fma(0.075, ws[49088], a);
      a = fma(0.06, ws[49216], a);
      a = fma(0.115, ws[49568], a);
      a = fma(0.531, ws[49600], a);
      a = fma(0.113, ws[49632], a);
      a = fma(0.275, ws[49824], a);
      a = fma(0.275, ws[49856], a);
      a = fma(0.22, ws[49888], a);
      a = fma(0.275, ws[49920], a);
      a = fma(0.443, ws[50432], a);
      a = fma(0.52, ws[50464], a);
      a = fma(0.52, ws[50528], a);
      a = fma(0.675, ws[50624], a);
      a = fma(0.77, ws[50688], a);
      a = fma(0.77, ws[50720], a);
      a = fma(0.24, ws[50784], a);
      a = fma(1.0, ws[51008], a);
      a = fma(1.2, ws[51040], a);
      a = fma(0.25, ws[51072], a);
      a = fma(0.24, ws[51168], a);
      a = a - ws[53600];
      yout[4000] = a;
    }
    {
      double a = 0.5 * ws[47168];
      a = fma(1.0, ws[47424], a);
      a = fma(0.65, ws[49536], a);
      a = fma(0.142, ws[49632], a);
      a = fma(0.266, ws[49952], a);
      a = fma(0.53, ws[50080], a);
      a = fma(0.53, ws[50208], a);
      a = fma(0.082, ws[50272], a);
      a = fma(0.14, ws[50432], a);
      a = fma(0.14, ws[50624], a);
      a = fma(1.0, ws[50880], a);
      a = fma(1.0, ws[50912], a);
      a = fma(0.5, ws[51072], a);
      a = fma(0.5, ws[51488], a);
      a = a - ws[53152];
      yout[4032] = a;
    }
    {
      double a = -ws[48000];
      a = a - ws[48032];
      a = a - ws[48064];
      a = a - ws[48096];
      a = fma(0.37, ws[48768], a);
      a = fma(0.3, ws[49024], a);
      a = fma(0.488, ws[49056], a);
      a = fma(0.27, ws[49088], a);
      a = fma(0.375, ws[49120], a);
      a = fma(0.66, ws[49152], a);
      a = fma(0.7, ws[49184], a);
      a = fma(0.442, ws[49216], a);
      a = fma(0.625, ws[49248], a);
      a = fma(0.15, ws[49504], a);
      a = fma(0.029, ws[49696], a);
      a = fma(0.078, ws[49952], a);
      a = fma(0.15, ws[49984], a);
      a = fma(0.47, ws[50016], a);
      a = fma(0.21, ws[50048], a);
      a = fma(0.47, ws[50080], a);
      a = fma(0.15, ws[50112], a);
      a = fma(0.47, ws[50144], a);
      a = fma(0.21, ws[50176], a);
      a = fma(0.47, ws[50208], a);
      a = fma(1.0, ws[51424], a);
      a = fma(0.8, ws[51456], a);
      a = fma(0.268, ws[51616], a);
      a = fma(0.126, ws[51680], a);
      a = fma(0.67, ws[52192], a);
      a = fma(0.55, ws[52224], a);
      a = a - ws[52352];
      yout[4064] = a;
    }
    {
      double a = -ws[46432];
      a = a - ws[46464];
      a = a - ws[46496];
      a = fma(1.0, ws[46528], a);
      a = fma(0.6, ws[46560], a);
      a = a - ws[46592];
      a = a - ws[46624];
      a = a - ws[46656];
      a = a - ws[46656];
      a = fma(1.0, ws[48000], a);
      a = fma(1.0, ws[48032], a);
      a = fma(1.0, ws[48064], a);
      a = fma(0.5, ws[48608], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.2, ws[49504], a);
      a = fma(0.717, ws[49632], a);
      a = fma(0.39, ws[50048], a);
      a = fma(0.39, ws[50176], a);
      a = fma(0.2, ws[51296], a);
      a = fma(1.0, ws[52352], a);
      yout[4096] = a;
    }
    {
      double a = 1.0 * ws[46432];
      a = fma(1.0, ws[46464], a);
      a = fma(0.4, ws[46560], a);
      a = a - ws[47872];
      a = a - ws[47904];
      a = a - ws[47936];
      a = a - ws[47968];
      a = fma(1.0, ws[48096], a);
      a = fma(0.991, ws[48512], a);
      a = fma(0.95, ws[48576], a);
      a = fma(0.5, ws[48608], a);
      a = fma(0.74, ws[48768], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.488, ws[49056], a);
      a = fma(0.295, ws[49088], a);
      a = fma(0.25, ws[49120], a);
      a = fma(1.24, ws[49152], a);
      a = fma(1.3, ws[49184], a);
      a = fma(0.732, ws[49216], a);
      a = fma(0.5, ws[49248], a);
      a = fma(0.04, ws[49600], a);
      a = fma(0.1, ws[51040], a);
      a = fma(0.02, ws[51168], a);
      a = fma(1.0, ws[51520], a);
      a = fma(0.991, ws[52128], a);
      a = fma(0.33, ws[52192], a);
      a = fma(0.45, ws[52224], a);
      a = a - ws[52320];
      a = fma(1.0, ws[52416], a);
      yout[4128] = a;
    }
    {
      double a = 1.0 * ws[44544];
      a = a - ws[44576];
      a = a - ws[44640];
      a = a - ws[44672];
      a = a - ws[44704];
      a = a - ws[44736];
      a = fma(1.0, ws[44768], a);
      a = fma(1.0, ws[44832], a);
      a = a - ws[44960];
      a = a - ws[44992];
      a = fma(1.0, ws[45024], a);
      a = a - ws[45248];
      a = fma(1.0, ws[45376], a);
      a = a - ws[45504];
      a = a - ws[47680];
      a = a - ws[47872];
      a = a - ws[48000];
      a = a - ws[48896];
      a = a - ws[49024];
      a = a - ws[49152];
      a = a - ws[49312];
      a = a - ws[49984];
      a = a - ws[50112];
      a = a - ws[54624];
      a = fma(1.0, ws[54624], a);
      a = a - ws[54816];
      a = fma(1.0, ws[54816], a);
      yout[4160] = a;
    }
    {
      double a = 2.0 * ws[45760];
      a = fma(1.0, ws[45952], a);
      a = a - ws[45984];
      a = a - ws[46016];
      a = fma(1.0, ws[47712], a);
      a = fma(1.0, ws[47936], a);
      a = fma(1.0, ws[48064], a);
      a = fma(1.0, ws[48192], a);
      a = fma(1.0, ws[48288], a);
      a = fma(1.0, ws[48352], a);
      a = fma(0.717, ws[49632], a);
      a = fma(1.0, ws[49760], a);
      a = fma(1.0, ws[50784], a);
      a = fma(1.0, ws[50912], a);
      a = fma(1.0, ws[51200], a);
      a = fma(1.0, ws[51264], a);
      a = fma(1.0, ws[51712], a);
      a = fma(1.0, ws[52704], a);
      a = fma(1.0, ws[52736], a);
      a = fma(1.0, ws[53152], a);
      a = fma(1.0, ws[53184], a);
      a = fma(1.0, ws[53216], a);
      a = fma(1.0, ws[53248], a);
      a = fma(1.0, ws[53280], a);
      a = fma(0.5, ws[53408], a);
      a = fma(1.0, ws[55648], a);
      yout[4192] = a;
    }
    {
      double a = -2.5 * ws[48608];
      a = a - ws[48736];
      a = fma(-2.7, ws[48768], a);
      a = fma(0.2, ws[49024], a);
      a = fma(-0.73, ws[49056], a);
      a = fma(-0.79, ws[49088], a);
      a = fma(-1.0, ws[49120], a);
      a = fma(0.1, ws[49152], a);
      a = fma(0.29, ws[49216], a);
      a = fma(1.0, ws[49248], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.35, ws[49504], a);
      a = fma(0.117, ws[49568], a);
      a = fma(0.717, ws[49632], a);
      a = fma(0.24, ws[49664], a);
      a = fma(2.175, ws[49824], a);
      a = fma(2.175, ws[49856], a);
      a = fma(1.74, ws[49888], a);
      a = fma(2.175, ws[49920], a);
      a = fma(2.7, ws[49952], a);
      a = fma(5.12, ws[49984], a);
      a = fma(1.66, ws[50016], a);
      a = fma(7.0, ws[50048], a);
      a = fma(5.12, ws[50112], a);
      a = fma(1.66, ws[50144], a);
      a = fma(7.0, ws[50176], a);
      a = fma(0.268, ws[51616], a);
      a = fma(-0.126, ws[51680], a);
      a = a - ws[52064];
      a = fma(-1.0, ws[52192], a);
      a = fma(0.3, ws[52224], a);
      yout[4224] = a;
    }
    {
      double a = 0.2 * ws[48128];
      a = fma(0.11, ws[48160], a);
      a = a - ws[48224];
      a = a - ws[48256];
      a = a - ws[48288];
      a = fma(0.7, ws[48864], a);
      a = fma(0.075, ws[49088], a);
      a = fma(0.24, ws[49216], a);
      a = fma(0.17, ws[49600], a);
      a = fma(0.275, ws[49824], a);
      a = fma(0.275, ws[49856], a);
      a = fma(0.22, ws[49888], a);
      a = fma(0.275, ws[49920], a);
      a = fma(0.918, ws[50272], a);
      a = fma(1.0, ws[50304], a);
      a = fma(1.0, ws[50368], a);
      a = fma(0.417, ws[50432], a);
      a = fma(0.48, ws[50464], a);
      a = fma(0.48, ws[50528], a);
      a = fma(0.221, ws[50624], a);
      a = fma(0.26, ws[50688], a);
      a = fma(0.26, ws[50720], a);
      a = fma(0.025, ws[50752], a);
      a = fma(0.24, ws[50784], a);
      a = fma(0.4, ws[50976], a);
      a = fma(0.4, ws[51008], a);
      a = fma(0.4, ws[51136], a);
      a = fma(1.4, ws[51168], a);
      a = fma(0.5, ws[51296], a);
      a = fma(0.5, ws[51488], a);
      a = a - ws[53568];
      yout[4256] = a;
    }
    {
      double a = -ws[47168];
      a = a - ws[47200];
      a = a - ws[47232];
      a = a - ws[47264];
      a = fma(0.06, ws[47360], a);
      a = fma(0.009, ws[48512], a);
      a = fma(0.04, ws[48768], a);
      a = fma(0.01, ws[49024], a);
      a = fma(0.024, ws[49056], a);
      a = fma(0.04, ws[49120], a);
      a = fma(0.04, ws[49248], a);
      a = fma(0.03, ws[49536], a);
      a = fma(0.022, ws[49568], a);
      a = fma(0.25, ws[50016], a);
      a = fma(0.18, ws[50048], a);
      a = fma(0.25, ws[50080], a);
      a = fma(0.25, ws[50144], a);
      a = fma(0.18, ws[50176], a);
      a = fma(0.25, ws[50208], a);
      a = fma(0.02, ws[50752], a);
      a = fma(0.1, ws[50784], a);
      a = fma(0.1, ws[51072], a);
      a = fma(1.0, ws[51584], a);
      a = fma(1.0, ws[51648], a);
      a = fma(0.03, ws[52096], a);
      a = fma(0.009, ws[52128], a);
      a = fma(0.04, ws[52256], a);
      yout[4288] = a;
    }
    {
      double a = 1.0 * ws[44576];
      a = a - ws[44608];
      a = a - ws[44736];
      a = a - ws[44768];
      a = a - ws[44800];
      a = a - ws[44896];
      a = a - ws[44928];
      a = a - ws[45344];
      a = a - ws[45600];
      a = fma(0.13, ws[46336], a);
      a = fma(0.13, ws[46592], a);
      a = a - ws[48960];
      a = a - ws[49088];
      a = a - ws[49216];
      a = a - ws[49504];
      a = a - ws[49600];
      a = a - ws[50048];
      a = a - ws[50176];
      a = a - ws[51040];
      a = a - ws[51168];
      a = fma(0.13, ws[51392], a);
      a = a - ws[51808];
      a = a - ws[52960];
      a = fma(1.0, ws[52960], a);
      a = a - ws[53440];
      a = a - ws[54944];
      a = fma(1.0, ws[54944], a);
      a = a - ws[55072];
      a = fma(1.0, ws[55072], a);
      a = a - ws[55232];
      a = fma(1.0, ws[55232], a);
      a = a - ws[55424];
      a = fma(1.0, ws[55424], a);
      yout[4320] = a;
    }
    {
      double a = -ws[47040];
      a = a - ws[47072];
      a = a - ws[47104];
      a = a - ws[47136];
      a = fma(0.2, ws[48224], a);
      a = fma(0.5, ws[48288], a);
      a = fma(1.0, ws[48352], a);
      a = fma(1.0, ws[48672], a);
      a = fma(0.5, ws[48992], a);
      a = fma(0.195, ws[49056], a);
      a = fma(0.48, ws[49120], a);
      a = fma(0.48, ws[49248], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.2, ws[49504], a);
      a = fma(0.33, ws[49536], a);
      a = fma(0.521, ws[49568], a);
      a = fma(0.142, ws[49632], a);
      a = fma(0.16, ws[49664], a);
      a = fma(0.63, ws[49952], a);
      a = fma(0.5, ws[50016], a);
      a = fma(0.69, ws[50048], a);
      a = fma(0.75, ws[50080], a);
      a = fma(0.5, ws[50144], a);
      a = fma(0.69, ws[50176], a);
      a = fma(0.75, ws[50208], a);
      a = fma(0.48, ws[50784], a);
      a = fma(0.45, ws[51072], a);
      a = fma(1.0, ws[51424], a);
      a = fma(0.874, ws[51680], a);
      a = fma(2.0, ws[52160], a);
      a = fma(2.0, ws[52192], a);
      a = fma(1.7, ws[52224], a);
      yout[4352] = a;
    }
    {
      double a = 1.0 * ws[44544];
      a = a - ws[44608];
      a = a - ws[44640];
      a = fma(1.0, ws[44672], a);
      a = a - ws[45280];
      a = a - ws[45280];
      a = a - ws[45312];
      a = fma(1.0, ws[45408], a);
      a = a - ws[45440];
      a = fma(1.0, ws[45472], a);
      a = a - ws[45792];
      a = a - ws[45824];
      a = fma(1.0, ws[45856], a);
      a = fma(1.0, ws[45888], a);
      a = a - ws[46208];
      a = a - ws[46464];
      a = a - ws[46688];
      a = fma(1.0, ws[46688], a);
      a = a - ws[46784];
      a = a - ws[46912];
      a = a - ws[47040];
      a = a - ws[47168];
      a = a - ws[47808];
      a = a - ws[49344];
      a = a - ws[49856];
      a = a - ws[50272];
      a = a - ws[50432];
      a = a - ws[50624];
      a = a - ws[51296];
      a = a - ws[51872];
      a = a - ws[52768];
      a = fma(1.0, ws[52768], a);
      a = a - ws[52832];
      a = fma(1.0, ws[52832], a);
      a = a - ws[52896];
      a = fma(1.0, ws[52896], a);
      a = a - ws[53056];
      a = fma(1.0, ws[53056], a);
      a = a - ws[53632];
      a = fma(1.0, ws[53632], a);
      yout[4384] = a;
    }
    {
      double a = 1.0 * ws[46208];
      a = fma(0.4, ws[46304], a);
      a = fma(0.5, ws[46336], a);
      a = fma(1.0, ws[46368], a);
      a = fma(2.0, ws[46400], a);
      a = fma(1.0, ws[46432], a);
      a = fma(0.5, ws[46592], a);
      a = fma(1.0, ws[46624], a);
      a = fma(2.0, ws[46656], a);
      a = a - ws[46784];
      a = a - ws[46816];
      a = a - ws[46848];
      a = fma(0.9, ws[46848], a);
      a = a - ws[46880];
      a = fma(0.8, ws[46976], a);
      a = fma(0.8, ws[47104], a);
      a = fma(0.8, ws[47232], a);
      a = fma(0.6, ws[47296], a);
      a = fma(1.0, ws[47328], a);
      a = fma(1.0, ws[47520], a);
      a = fma(1.0, ws[47968], a);
      a = fma(1.0, ws[48480], a);
      a = fma(0.5, ws[48608], a);
      a = fma(1.38, ws[48640], a);
      a = fma(0.8, ws[49408], a);
      a = fma(0.115, ws[49568], a);
      a = fma(0.34, ws[49664], a);
      a = fma(0.8, ws[49888], a);
      a = fma(1.0, ws[50304], a);
      a = fma(1.0, ws[50464], a);
      a = fma(1.0, ws[50688], a);
      a = fma(0.5, ws[51392], a);
      a = fma(1.0, ws[51424], a);
      a = fma(1.0, ws[51552], a);
      a = a - ws[51936];
      a = fma(1.0, ws[52032], a);
      a = fma(1.0, ws[55584], a);
      a = fma(1.0, ws[55616], a);
      a = fma(1.0, ws[55648], a);
      a = fma(1.0, ws[55680], a);
      yout[4416] = a;
    }
    {
      double a = -ws[46208];
      a = a - ws[46240];
      a = fma(1.0, ws[46272], a);
      a = fma(0.6, ws[46304], a);
      a = a - ws[46336];
      a = a - ws[46368];
      a = a - ws[46400];
      a = a - ws[46400];
      a = a - ws[46432];
      a = a - ws[46848];
      a = a - ws[46976];
      a = a - ws[47104];
      a = a - ws[47232];
      a = fma(1.0, ws[47552], a);
      a = fma(1.0, ws[47872], a);
      a = fma(1.0, ws[47904], a);
      a = fma(1.0, ws[47936], a);
      a = fma(0.8, ws[48128], a);
      a = fma(1.0, ws[48192], a);
      a = fma(1.0, ws[48320], a);
      a = fma(1.0, ws[48352], a);
      a = fma(1.0, ws[48384], a);
      a = fma(0.5, ws[48608], a);
      a = fma(0.62, ws[48640], a);
      a = fma(1.0, ws[48672], a);
      a = a - ws[49408];
      a = fma(0.269, ws[49568], a);
      a = fma(0.143, ws[49600], a);
      a = fma(0.208, ws[49664], a);
      a = a - ws[49888];
      a = a - ws[50304];
      a = a - ws[50464];
      a = a - ws[50688];
      a = fma(0.3, ws[50976], a);
      a = fma(0.6, ws[51040], a);
      a = fma(0.12, ws[51168], a);
      a = a - ws[51424];
      a = fma(1.0, ws[52320], a);
      yout[4448] = a;
    }
    {
      double a = 1.0 * ws[47584];
      a = fma(1.0, ws[47616], a);
      a = fma(1.0, ws[47648], a);
      a = fma(1.0, ws[47680], a);
      a = fma(1.0, ws[47712], a);
      a = fma(1.0, ws[47968], a);
      a = fma(1.0, ws[48096], a);
      a = fma(0.89, ws[48160], a);
      a = fma(1.8, ws[48224], a);
      a = fma(2.0, ws[48256], a);
      a = fma(1.5, ws[48288], a);
      a = fma(1.0, ws[48320], a);
      a = fma(1.0, ws[48384], a);
      a = a - ws[48448];
      a = fma(0.38, ws[48640], a);
      a = fma(0.3, ws[48864], a);
      a = fma(1.0, ws[48896], a);
      a = fma(0.35, ws[48960], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.378, ws[49088], a);
      a = fma(0.1, ws[49152], a);
      a = fma(0.245, ws[49216], a);
      a = fma(0.066, ws[49504], a);
      a = fma(0.137, ws[49568], a);
      a = fma(0.543, ws[49600], a);
      a = fma(0.251, ws[49824], a);
      a = fma(0.251, ws[49856], a);
      a = fma(0.2, ws[49888], a);
      a = fma(0.251, ws[49920], a);
      a = fma(0.001, ws[50048], a);
      a = fma(0.001, ws[50176], a);
      a = fma(0.7, ws[50976], a);
      a = fma(0.5, ws[51040], a);
      a = fma(1.0, ws[51104], a);
      a = fma(1.98, ws[51168], a);
      a = fma(0.5, ws[51296], a);
      a = fma(1.0, ws[51488], a);
      a = fma(1.0, ws[51968], a);
      a = fma(1.0, ws[52000], a);
      a = fma(1.0, ws[52288], a);
      yout[4480] = a;
    }
    {
      double a = 1.0 * ws[46784];
      a = fma(0.1, ws[46816], a);
      a = fma(1.0, ws[46848], a);
      a = fma(0.685, ws[46880], a);
      a = fma(0.4, ws[47296], a);
      a = a - ws[47584];
      a = a - ws[47616];
      a = a - ws[47648];
      a = a - ws[47680];
      a = a - ws[47712];
      a = a - ws[47744];
      a = fma(1.0, ws[47776], a);
      a = fma(0.74, ws[48160], a);
      a = fma(1.0, ws[48544], a);
      a = fma(0.078, ws[48576], a);
      a = fma(1.0, ws[48672], a);
      a = fma(1.0, ws[48896], a);
      a = fma(1.56, ws[48928], a);
      a = fma(1.0, ws[48960], a);
      a = fma(1.125, ws[48992], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.781, ws[49056], a);
      a = fma(0.555, ws[49088], a);
      a = fma(0.5, ws[49120], a);
      a = fma(0.128, ws[49216], a);
      a = fma(0.5, ws[49312], a);
      a = fma(0.673, ws[49344], a);
      a = fma(0.12, ws[49376], a);
      a = fma(0.598, ws[49408], a);
      a = fma(0.598, ws[49440], a);
      a = fma(0.6, ws[49504], a);
      a = fma(0.35, ws[49536], a);
      a = fma(0.231, ws[49600], a);
      a = fma(0.26, ws[49664], a);
      a = fma(0.375, ws[49824], a);
      a = fma(0.375, ws[49856], a);
      a = fma(0.3, ws[49888], a);
      a = fma(0.375, ws[49920], a);
      a = fma(0.592, ws[49952], a);
      a = fma(0.28, ws[50016], a);
      a = fma(0.24, ws[50048], a);
      a = fma(0.28, ws[50144], a);
      a = fma(0.24, ws[50176], a);
      a = fma(1.0, ws[50944], a);
      a = fma(0.08, ws[51168], a);
      a = fma(0.14, ws[51232], a);
      a = fma(1.0, ws[51936], a);
      a = fma(1.0, ws[52160], a);
      a = a - ws[52288];
      a = fma(1.0, ws[52384], a);
      a = fma(1.0, ws[55584], a);
      a = fma(1.0, ws[55648], a);
      a = fma(0.45, ws[55680], a);
      yout[4512] = a;
    }
    {
      double a = 2.0 * ws[51744];
      a = fma(1.0, ws[51776], a);
      a = a - ws[51808];
      a = fma(1.4, ws[51840], a);
      a = fma(1.0, ws[51872], a);
      a = fma(1.0, ws[51936], a);
      a = fma(1.0, ws[51968], a);
      a = fma(1.0, ws[52000], a);
      a = a - ws[52032];
      a = a - ws[52064];
      a = a - ws[52096];
      a = a - ws[52128];
      a = a - ws[52160];
      a = a - ws[52192];
      a = a - ws[52224];
      a = a - ws[52256];
      a = a - ws[52288];
      a = a - ws[52320];
      a = a - ws[52352];
      a = a - ws[52384];
      a = a - ws[52416];
      a = fma(1.0, ws[52448], a);
      a = a - ws[52480];
      a = a - ws[52512];
      a = a - ws[52544];
      a = fma(1.0, ws[52576], a);
      a = fma(1.0, ws[52672], a);
      a = a - ws[53760];
      a = fma(1.0, ws[53760], a);
      a = a - ws[54720];
      a = fma(1.0, ws[54720], a);
      a = a - ws[54880];
      a = fma(1.0, ws[54880], a);
      a = a - ws[55008];
      a = fma(1.0, ws[55008], a);
      a = a - ws[55168];
      a = fma(1.0, ws[55168], a);
      a = a - ws[55328];
      a = fma(1.0, ws[55328], a);
      a = a - ws[55392];
      a = fma(1.0, ws[55392], a);
      a = a - ws[55552];
      a = fma(1.0, ws[55552], a);
      a = a - ws[55680];
      yout[4544] = a;
    }
    {
      double a = 1.0 * ws[46432];
      a = fma(1.0, ws[46464], a);
      a = fma(0.4, ws[46560], a);
      a = a - ws[46912];
      a = a - ws[46944];
      a = a - ws[46976];
      a = a - ws[47008];
      a = fma(0.54, ws[47360], a);
      a = fma(1.0, ws[48096], a);
      a = fma(0.11, ws[48160], a);
      a = fma(0.991, ws[48512], a);
      a = fma(0.1, ws[48576], a);
      a = fma(0.5, ws[48608], a);
      a = fma(0.94, ws[48768], a);
      a = fma(0.7, ws[48896], a);
      a = fma(1.0, ws[48928], a);
      a = fma(0.5, ws[48992], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.976, ws[49056], a);
      a = fma(0.15, ws[49088], a);
      a = fma(0.48, ws[49120], a);
      a = fma(0.1, ws[49152], a);
      a = fma(1.0, ws[49184], a);
      a = fma(0.3, ws[49216], a);
      a = fma(0.48, ws[49248], a);
      a = fma(0.082, ws[49344], a);
      a = fma(0.072, ws[49408], a);
      a = fma(0.072, ws[49440], a);
      a = fma(0.64, ws[49536], a);
      a = fma(0.142, ws[49632], a);
      a = fma(0.34, ws[49664], a);
      a = fma(0.37, ws[49952], a);
      a = fma(0.75, ws[50016], a);
      a = fma(0.07, ws[50048], a);
      a = fma(0.28, ws[50080], a);
      a = fma(0.75, ws[50144], a);
      a = fma(0.07, ws[50176], a);
      a = fma(0.28, ws[50208], a);
      a = fma(0.07, ws[50400], a);
      a = fma(0.058, ws[50560], a);
      a = fma(0.058, ws[50592], a);
      a = fma(0.12, ws[50784], a);
      a = fma(1.0, ws[50976], a);
      a = fma(2.0, ws[51008], a);
      a = fma(0.3, ws[51040], a);
      a = fma(0.45, ws[51072], a);
      a = fma(0.4, ws[51136], a);
      a = fma(0.8, ws[51456], a);
      a = fma(1.0, ws[51616], a);
      a = fma(0.126, ws[51680], a);
      a = fma(0.97, ws[52096], a);
      a = fma(0.991, ws[52128], a);
      a = fma(0.96, ws[52256], a);
      a = fma(0.07, ws[52480], a);
      a = fma(0.058, ws[52512], a);
      a = fma(0.058, ws[52544], a);
      yout[4576] = a;
    }
    {
      double a = -ws[44544];
      a = fma(1.0, ws[44608], a);
      a = fma(1.0, ws[44640], a);
      a = a - ws[44672];
      a = a - ws[44704];
      a = fma(2.0, ws[45280], a);
      a = fma(1.0, ws[45312], a);
      a = a - ws[45344];
      a = fma(1.0, ws[45376], a);
      a = fma(2.0, ws[45440], a);
      a = a - ws[45472];
      a = fma(1.0, ws[45472], a);
      a = fma(1.0, ws[45504], a);
      a = fma(1.0, ws[45536], a);
      a = fma(1.0, ws[45568], a);
      a = fma(1.0, ws[45600], a);
      a = fma(2.0, ws[45632], a);
      a = a - ws[45664];
      a = fma(1.0, ws[45696], a);
      a = fma(1.0, ws[45728], a);
      a = a - ws[45824];
      a = fma(1.0, ws[45856], a);
      a = fma(1.0, ws[45920], a);
      a = a - ws[45952];
      a = fma(1.0, ws[46016], a);
      a = a - ws[46048];
      a = fma(1.0, ws[46080], a);
      a = fma(0.59, ws[46112], a);
      a = fma(1.0, ws[46144], a);
      a = fma(1.0, ws[46208], a);
      a = a - ws[46240];
      a = fma(1.0, ws[46272], a);
      a = fma(0.6, ws[46304], a);
      a = fma(1.0, ws[46464], a);
      a = a - ws[46496];
      a = fma(1.0, ws[46528], a);
      a = fma(0.6, ws[46560], a);
      a = fma(1.0, ws[46784], a);
      a = fma(1.0, ws[46912], a);
      a = fma(1.0, ws[47040], a);
      a = fma(1.0, ws[47456], a);
      a = fma(1.0, ws[47808], a);
      a = a - ws[48832];
      a = fma(0.5, ws[48992], a);
      a = fma(0.5, ws[49120], a);
      a = fma(0.5, ws[49248], a);
      a = fma(0.9, ws[49344], a);
      a = fma(0.35, ws[49536], a);
      a = fma(0.142, ws[49632], a);
      a = fma(1.0, ws[49856], a);
      a = fma(0.444, ws[49952], a);
      a = fma(0.47, ws[50080], a);
      a = fma(0.47, ws[50208], a);
      a = fma(0.918, ws[50272], a);
      a = fma(0.86, ws[50432], a);
      a = fma(0.86, ws[50624], a);
      a = a - ws[50816];
      a = fma(0.5, ws[51072], a);
      a = fma(1.0, ws[51296], a);
      a = a - ws[51328];
      a = fma(1.0, ws[51360], a);
      a = fma(0.5, ws[51488], a);
      a = fma(1.0, ws[51520], a);
      a = a - ws[51712];
      a = fma(1.0, ws[51872], a);
      a = fma(1.0, ws[52576], a);
      a = a - ws[52608];
      a = fma(1.0, ws[52640], a);
      a = a - ws[53408];
      yout[4608] = a;
    }
    {
      double a = 1.0 * ws[44704];
      a = fma(1.0, ws[45344], a);
      a = a - ws[45376];
      a = a - ws[45408];
      a = a - ws[45440];
      a = a - ws[45472];
      a = a - ws[45504];
      a = a - ws[45536];
      a = a - ws[45568];
      a = a - ws[45600];
      a = a - ws[45632];
      a = a - ws[45632];
      a = a - ws[45664];
      a = fma(1.0, ws[45696], a);
      a = fma(1.0, ws[45728], a);
      a = fma(1.0, ws[45984], a);
      a = fma(0.41, ws[46112], a);
      a = fma(0.4, ws[46304], a);
      a = fma(0.4, ws[46560], a);
      a = a - ws[47712];
      a = a - ws[47936];
      a = a - ws[48064];
      a = a - ws[48192];
      a = a - ws[48288];
      a = a - ws[48352];
      a = a - ws[48992];
      a = a - ws[49120];
      a = a - ws[49248];
      a = a - ws[49536];
      a = a - ws[49632];
      a = a - ws[49760];
      a = fma(0.185, ws[49952], a);
      a = a - ws[50080];
      a = a - ws[50208];
      a = a - ws[50784];
      a = a - ws[50912];
      a = a - ws[51072];
      a = a - ws[51200];
      a = a - ws[51264];
      a = fma(1.0, ws[52672], a);
      a = a - ws[53024];
      a = fma(1.0, ws[53024], a);
      a = a - ws[53696];
      a = fma(1.0, ws[53696], a);
      a = a - ws[54592];
      a = fma(1.0, ws[54592], a);
      a = a - ws[54784];
      a = fma(1.0, ws[54784], a);
      a = a - ws[54976];
      a = fma(1.0, ws[54976], a);
      a = a - ws[55104];
      a = fma(1.0, ws[55104], a);
      a = a - ws[55264];
      a = fma(1.0, ws[55264], a);
      a = a - ws[55648];
      yout[4640] = a;
    }
    {
      double a = 1.0 * ws[46208];
      a = fma(0.4, ws[46304], a);
      a = fma(0.5, ws[46336], a);
      a = a - ws[46368];
      a = fma(2.0, ws[46400], a);
      a = fma(2.0, ws[46432], a);
      a = fma(1.0, ws[46464], a);
      a = fma(0.4, ws[46560], a);
      a = fma(0.5, ws[46592], a);
      a = a - ws[46624];
      a = fma(2.0, ws[46656], a);
      a = a - ws[46688];
      a = a - ws[46720];
      a = a - ws[46752];
      a = a - ws[46752];
      a = fma(0.9, ws[46848], a);
      a = a - ws[46880];
      a = fma(1.0, ws[46880], a);
      a = fma(0.8, ws[46976], a);
      a = a - ws[47008];
      a = fma(1.0, ws[47008], a);
      a = fma(0.8, ws[47104], a);
      a = a - ws[47136];
      a = fma(1.0, ws[47136], a);
      a = fma(0.8, ws[47232], a);
      a = a - ws[47264];
      a = fma(1.0, ws[47264], a);
      a = fma(0.6, ws[47296], a);
      a = fma(1.0, ws[47328], a);
      a = fma(0.6, ws[47360], a);
      a = fma(1.0, ws[47520], a);
      a = fma(1.0, ws[47968], a);
      a = fma(1.0, ws[48096], a);
      a = fma(0.11, ws[48160], a);
      a = fma(0.2, ws[48224], a);
      a = fma(0.5, ws[48288], a);
      a = fma(1.0, ws[48352], a);
      a = fma(1.0, ws[48480], a);
      a = fma(1.0, ws[48512], a);
      a = fma(0.1, ws[48576], a);
      a = fma(1.0, ws[48608], a);
      a = fma(1.38, ws[48640], a);
      a = fma(1.0, ws[48672], a);
      a = fma(0.98, ws[48768], a);
      a = fma(0.7, ws[48896], a);
      a = fma(1.0, ws[48928], a);
      a = fma(1.0, ws[48992], a);
      a = fma(0.21, ws[49024], a);
      a = fma(1.195, ws[49056], a);
      a = fma(0.15, ws[49088], a);
      a = fma(1.0, ws[49120], a);
      a = fma(0.1, ws[49152], a);
      a = fma(1.0, ws[49184], a);
      a = fma(0.3, ws[49216], a);
      a = fma(1.0, ws[49248], a);
      a = fma(1.0, ws[49280], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.082, ws[49344], a);
      a = fma(0.872, ws[49408], a);
      a = a - ws[49440];
      a = fma(1.072, ws[49440], a);
      a = fma(0.2, ws[49504], a);
      a = fma(1.0, ws[49536], a);
      a = fma(0.658, ws[49568], a);
      a = fma(0.284, ws[49632], a);
      a = fma(0.84, ws[49664], a);
      a = fma(0.067, ws[49696], a);
      a = fma(1.0, ws[49792], a);
      a = fma(0.8, ws[49888], a);
      a = a - ws[49920];
      a = fma(1.0, ws[49920], a);
      a = fma(1.0, ws[49952], a);
      a = fma(1.5, ws[50016], a);
      a = fma(0.94, ws[50048], a);
      a = fma(1.28, ws[50080], a);
      a = fma(1.5, ws[50144], a);
      a = fma(0.94, ws[50176], a);
      a = fma(1.28, ws[50208], a);
      a = fma(0.352, ws[50240], a);
      a = fma(1.0, ws[50304], a);
      a = a - ws[50368];
      a = fma(1.0, ws[50368], a);
      a = fma(0.72, ws[50400], a);
      a = fma(1.0, ws[50464], a);
      a = a - ws[50528];
      a = fma(1.0, ws[50528], a);
      a = fma(0.602, ws[50560], a);
      a = fma(0.602, ws[50592], a);
      a = fma(1.0, ws[50688], a);
      a = a - ws[50720];
      a = fma(1.0, ws[50720], a);
      a = fma(0.02, ws[50752], a);
      a = fma(0.7, ws[50784], a);
      a = fma(2.0, ws[51008], a);
      a = fma(0.3, ws[51040], a);
      a = fma(1.0, ws[51072], a);
      a = fma(0.4, ws[51136], a);
      a = fma(0.5, ws[51392], a);
      a = fma(2.0, ws[51424], a);
      a = a - ws[51456];
      a = fma(1.8, ws[51456], a);
      a = fma(1.0, ws[51552], a);
      a = fma(1.0, ws[51584], a);
      a = fma(1.0, ws[51616], a);
      a = fma(1.0, ws[51648], a);
      a = fma(1.0, ws[51680], a);
      a = fma(1.0, ws[52032], a);
      a = fma(1.0, ws[52096], a);
      a = fma(1.0, ws[52128], a);
      a = fma(1.0, ws[52256], a);
      a = fma(0.72, ws[52480], a);
      a = fma(0.602, ws[52512], a);
      a = fma(0.602, ws[52544], a);
      a = a - ws[53728];
      a = fma(1.0, ws[53728], a);
      yout[4672] = a;
    }
    {
      double a = 1.0 * ws[44896];
      a = a - ws[44928];
      a = fma(1.0, ws[44960], a);
      a = a - ws[44992];
      a = a - ws[45088];
      a = a - ws[45120];
      a = a - ws[45120];
      a = a - ws[45152];
      a = a - ws[45152];
      a = fma(1.0, ws[45216], a);
      a = fma(1.0, ws[45248], a);
      a = a - ws[45312];
      a = fma(1.0, ws[45536], a);
      a = a - ws[45568];
      a = a - ws[46048];
      a = fma(1.0, ws[46080], a);
      a = fma(0.59, ws[46112], a);
      a = fma(1.0, ws[46176], a);
      a = a - ws[46336];
      a = a - ws[46592];
      a = a - ws[46720];
      a = fma(1.0, ws[46720], a);
      a = fma(1.0, ws[46784], a);
      a = a - ws[46816];
      a = fma(0.9, ws[46848], a);
      a = fma(0.37, ws[46880], a);
      a = fma(1.0, ws[46912], a);
      a = a - ws[46944];
      a = fma(0.8, ws[46976], a);
      a = fma(0.6, ws[47008], a);
      a = a - ws[47072];
      a = a - ws[47200];
      a = fma(0.8, ws[47232], a);
      a = fma(1.0, ws[47392], a);
      a = fma(1.0, ws[47488], a);
      a = fma(1.0, ws[47584], a);
      a = fma(2.0, ws[47616], a);
      a = fma(1.0, ws[47680], a);
      a = fma(1.0, ws[47712], a);
      a = a - ws[47744];
      a = fma(1.0, ws[47776], a);
      a = fma(1.0, ws[47808], a);
      a = a - ws[47840];
      a = fma(0.2, ws[47840], a);
      a = fma(1.0, ws[47968], a);
      a = fma(1.0, ws[48096], a);
      a = fma(0.2, ws[48128], a);
      a = fma(1.4, ws[48160], a);
      a = fma(1.0, ws[48224], a);
      a = fma(2.0, ws[48256], a);
      a = fma(1.0, ws[48288], a);
      a = fma(1.0, ws[48320], a);
      a = fma(1.0, ws[48416], a);
      a = fma(1.0, ws[48448], a);
      a = fma(1.0, ws[48544], a);
      a = fma(0.9, ws[48576], a);
      a = fma(1.0, ws[48800], a);
      a = fma(0.3, ws[48864], a);
      a = fma(1.0, ws[48896], a);
      a = fma(0.27, ws[48960], a);
      a = fma(0.1, ws[49024], a);
      a = fma(0.08, ws[49088], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.818, ws[49344], a);
      a = a - ws[49376];
      a = fma(0.12, ws[49376], a);
      a = fma(0.728, ws[49408], a);
      a = fma(0.728, ws[49440], a);
      a = fma(1.0, ws[49472], a);
      a = fma(0.066, ws[49504], a);
      a = fma(0.137, ws[49568], a);
      a = fma(0.398, ws[49600], a);
      a = fma(0.76, ws[49664], a);
      a = a - ws[49824];
      a = fma(0.825, ws[49824], a);
      a = fma(0.825, ws[49856], a);
      a = fma(0.66, ws[49888], a);
      a = fma(0.825, ws[49920], a);
      a = fma(0.53, ws[50240], a);
      a = fma(0.918, ws[50272], a);
      a = fma(1.0, ws[50304], a);
      a = a - ws[50336];
      a = fma(1.0, ws[50368], a);
      a = fma(0.18, ws[50400], a);
      a = fma(0.86, ws[50432], a);
      a = fma(1.0, ws[50464], a);
      a = a - ws[50496];
      a = fma(1.0, ws[50528], a);
      a = fma(0.155, ws[50560], a);
      a = fma(0.155, ws[50592], a);
      a = fma(0.86, ws[50624], a);
      a = a - ws[50656];
      a = fma(1.0, ws[50688], a);
      a = fma(1.0, ws[50720], a);
      a = fma(1.0, ws[50752], a);
      a = a - ws[50848];
      a = fma(1.0, ws[50944], a);
      a = fma(0.7, ws[50976], a);
      a = fma(1.0, ws[51104], a);
      a = fma(0.56, ws[51168], a);
      a = fma(0.2, ws[51232], a);
      a = fma(0.8, ws[51296], a);
      a = a - ws[51392];
      a = a - ws[51904];
      a = fma(1.0, ws[51936], a);
      a = fma(1.0, ws[52000], a);
      a = fma(1.0, ws[52160], a);
      a = fma(1.0, ws[52192], a);
      a = fma(1.0, ws[52224], a);
      a = fma(1.0, ws[52288], a);
      a = fma(1.0, ws[52384], a);
      a = fma(1.0, ws[52416], a);
      a = fma(0.18, ws[52480], a);
      a = fma(0.155, ws[52512], a);
      a = fma(0.155, ws[52544], a);
      a = a - ws[52800];
      a = fma(1.0, ws[52800], a);
      a = a - ws[52864];
      a = fma(1.0, ws[52864], a);
      a = a - ws[52928];
      a = fma(1.0, ws[52928], a);
      a = a - ws[53088];
      a = fma(1.0, ws[53088], a);
      a = a - ws[53664];
      a = fma(1.0, ws[53664], a);
      yout[4704] = a;
    }
    {
      double a = 2.0 * ws[44864];
      a = a - ws[44896];
      a = fma(1.0, ws[44928], a);
      a = a - ws[44960];
      a = fma(1.0, ws[44992], a);
      a = a - ws[45024];
      a = a - ws[45024];
      a = a - ws[45056];
      a = a - ws[45056];
      a = a - ws[45088];
      a = fma(2.0, ws[45184], a);
      a = a - ws[45216];
      a = fma(1.0, ws[45248], a);
      a = fma(1.0, ws[45312], a);
      a = a - ws[45536];
      a = fma(1.0, ws[45568], a);
      a = a - ws[45792];
      a = fma(1.0, ws[45888], a);
      a = a - ws[45920];
      a = a - ws[45952];
      a = a - ws[45984];
      a = fma(1.0, ws[46016], a);
      a = fma(0.41, ws[46112], a);
      a = a - ws[46144];
      a = a - ws[46176];
      a = fma(0.5, ws[46336], a);
      a = fma(0.5, ws[46592], a);
      a = a - ws[47296];
      a = fma(0.4, ws[47296], a);
      a = fma(1.0, ws[47328], a);
      a = a - ws[47360];
      a = fma(0.4, ws[47360], a);
      a = fma(1.0, ws[47392], a);
      a = a - ws[47424];
      a = a - ws[47488];
      a = a - ws[47520];
      a = a - ws[47552];
      a = a - ws[47584];
      a = fma(1.0, ws[47680], a);
      a = fma(0.2, ws[47840], a);
      a = fma(1.0, ws[47872], a);
      a = a - ws[47904];
      a = fma(1.0, ws[48000], a);
      a = a - ws[48032];
      a = a - ws[48128];
      a = fma(0.19, ws[48160], a);
      a = a - ws[48224];
      a = a - ws[48384];
      a = a - ws[48416];
      a = a - ws[48448];
      a = a - ws[48480];
      a = a - ws[48512];
      a = a - ws[48544];
      a = a - ws[48576];
      a = a - ws[48672];
      a = a - ws[48704];
      a = a - ws[48736];
      a = a - ws[48864];
      a = fma(0.7, ws[48864], a);
      a = fma(0.3, ws[48896], a);
      a = a - ws[48928];
      a = fma(0.17, ws[48960], a);
      a = fma(0.1, ws[49024], a);
      a = a - ws[49056];
      a = fma(0.334, ws[49088], a);
      a = a - ws[49184];
      a = fma(0.5, ws[49216], a);
      a = a - ws[49280];
      a = fma(0.12, ws[49376], a);
      a = fma(0.266, ws[49504], a);
      a = a - ws[49568];
      a = fma(0.461, ws[49600], a);
      a = a - ws[49696];
      a = fma(0.933, ws[49696], a);
      a = fma(1.0, ws[49728], a);
      a = a - ws[49792];
      a = fma(1.125, ws[49824], a);
      a = fma(0.125, ws[49856], a);
      a = fma(0.1, ws[49888], a);
      a = fma(0.125, ws[49920], a);
      a = a - ws[49952];
      a = a - ws[50016];
      a = fma(0.57, ws[50048], a);
      a = a - ws[50144];
      a = fma(0.57, ws[50176], a);
      a = a - ws[50240];
      a = fma(0.118, ws[50240], a);
      a = a - ws[50400];
      a = fma(0.1, ws[50400], a);
      a = a - ws[50560];
      a = fma(0.244, ws[50560], a);
      a = a - ws[50592];
      a = fma(0.244, ws[50592], a);
      a = a - ws[50752];
      a = a - ws[50880];
      a = a - ws[51008];
      a = fma(0.5, ws[51040], a);
      a = a - ws[51136];
      a = fma(0.5, ws[51168], a);
      a = a - ws[51232];
      a = fma(0.5, ws[51392], a);
      a = a - ws[51488];
      a = a - ws[51520];
      a = a - ws[51552];
      a = a - ws[51712];
      a = fma(1.0, ws[51776], a);
      a = a - ws[51968];
      a = a - ws[52448];
      a = fma(0.1, ws[52480], a);
      a = fma(0.244, ws[52512], a);
      a = fma(0.244, ws[52544], a);
      a = a - ws[52992];
      a = fma(1.0, ws[52992], a);
      a = a - ws[53120];
      a = fma(1.0, ws[53120], a);
      a = a - ws[53792];
      a = fma(1.0, ws[53792], a);
      a = a - ws[54080];
      a = fma(1.0, ws[54080], a);
      a = a - ws[54112];
      a = fma(1.0, ws[54112], a);
      a = a - ws[54144];
      a = fma(1.0, ws[54144], a);
      a = a - ws[54176];
      a = fma(1.0, ws[54176], a);
      a = a - ws[54208];
      a = fma(1.0, ws[54208], a);
      a = a - ws[54240];
      a = fma(1.0, ws[54240], a);
      a = a - ws[54272];
      a = fma(1.0, ws[54272], a);
      a = a - ws[54304];
      a = fma(1.0, ws[54304], a);
      a = a - ws[54336];
      a = fma(1.0, ws[54336], a);
      a = a - ws[54368];
      a = fma(1.0, ws[54368], a);
      a = a - ws[54400];
      a = fma(1.0, ws[54400], a);
      a = a - ws[54432];
      a = fma(1.0, ws[54432], a);
      a = a - ws[54464];
      a = fma(1.0, ws[54464], a);
      a = a - ws[54496];
      a = fma(1.0, ws[54496], a);
      a = a - ws[54528];
      a = fma(1.0, ws[54528], a);
      a = a - ws[54560];
      a = fma(1.0, ws[54560], a);
      a = a - ws[54752];
      a = fma(1.0, ws[54752], a);
      a = a - ws[54912];
      a = fma(1.0, ws[54912], a);
      a = a - ws[55040];
      a = fma(1.0, ws[55040], a);
      a = a - ws[55200];
      a = fma(1.0, ws[55200], a);
      a = a - ws[55360];
      a = fma(1.0, ws[55360], a);
      a = a - ws[55520];
      a = fma(1.0, ws[55520], a);
      a = a - ws[55584];
      a = a - ws[55616];
      yout[4736] = a;
    }
}
// Partial-derivative products of 2- and 3-reactant reactions (rbjacob.F:112-143).
__device__ __noinline__ void explic_0(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    { const double kk = ws[33440]; ws[55712] = kk * y[4384]; ws[55744] = kk * y[4320]; }
    { const double kk = ws[33472]; ws[55776] = kk * y[4384]; ws[55808] = kk * y[4160]; }
    { const double kk = ws[33504]; ws[55840] = kk * y[4608]; ws[55872] = kk * y[4160]; }
    { const double kk = ws[33536]; ws[55904] = kk * y[4608]; ws[55936] = kk * y[4160]; }
    { const double kk = ws[33568]; ws[55968] = kk * y[4320]; ws[56000] = kk * y[4160]; }
    { const double kk = ws[33728]; ws[56032] = kk * y[4736]; ws[56064] = kk * y[4320]; }
    { const double kk = ws[33760]; ws[56096] = kk * y[4704]; ws[56128] = kk * y[4320]; }
    { const double kk = ws[33792]; ws[56160] = kk * y[4160]; ws[56192] = kk * y[4736]; }
    { const double kk = ws[33824]; ws[56224] = kk * y[4160]; ws[56256] = kk * y[4704]; }
    { const double kk = ws[33856]; ws[56288] = kk * y[4736]; ws[56320] = kk * y[4736]; }
    { const double kk = ws[33888]; ws[56352] = kk * y[4736]; ws[56384] = kk * y[4736]; }
    { const double kk = ws[33920]; ws[56416] = kk * y[4704]; ws[56448] = kk * y[4736]; }
    { const double kk = ws[33952]; ws[56480] = kk * y[4704]; ws[56512] = kk * y[4704]; }
    { const double kk = ws[33984]; ws[56544] = kk * y[4704]; ws[56576] = kk * y[4704]; }
    { const double kk = ws[34048]; ws[56608] = kk * y[4736]; ws[56640] = kk * y[3456]; }
    { const double kk = ws[34080]; ws[56672] = kk * y[4160]; ws[56704] = kk * y[3456]; }
    { const double kk = ws[34112]; ws[56736] = kk * y[4384]; ws[56768] = kk * y[4384]; }
    { const double kk = ws[34144]; ws[56800] = kk * y[4384]; ws[56832] = kk * y[4704]; }
    { const double kk = ws[34176]; ws[56864] = kk * y[4320]; ws[56896] = kk * y[4608]; }
    { const double kk = ws[34272]; ws[56928] = kk * y[4384]; ws[56960] = kk * y[4640]; }
    { const double kk = ws[34304]; ws[56992] = kk * y[4608]; ws[57024] = kk * y[4640]; }
    { const double kk = ws[34336]; ws[57056] = kk * y[4160]; ws[57088] = kk * y[4640]; }
    { const double kk = ws[34368]; ws[57120] = kk * y[4736]; ws[57152] = kk * y[4640]; }
    { const double kk = ws[34400]; ws[57184] = kk * y[4704]; ws[57216] = kk * y[4640]; }
    { const double kk = ws[34432]; ws[57248] = kk * y[4320]; ws[57280] = kk * y[4640]; }
    { const double kk = ws[34464]; ws[57312] = kk * y[4640]; ws[57344] = kk * y[4640]; }
    { const double kk = ws[34496]; ws[57376] = kk * y[4608]; ws[57408] = kk * y[4640]; }
    { const double kk = ws[34624]; ws[57440] = kk * y[4736]; ws[57472] = kk * y[4384]; }
    { const double kk = ws[34656]; ws[57504] = kk * y[4608]; ws[57536] = kk * y[4384]; }
    { const double kk = ws[34688]; ws[57568] = kk * y[2464]; ws[57600] = kk * y[2464]; }
    { const double kk = ws[34752]; ws[57632] = kk * y[4736]; ws[57664] = kk * y[2464]; }
    { const double kk = ws[34784]; ws[57696] = kk * y[4736]; ws[57728] = kk * y[4608]; }
    { const double kk = ws[34816]; ws[57760] = kk * y[4736]; ws[57792] = kk * y[4192]; }
    { const double kk = ws[34880]; ws[57824] = kk * y[4608]; ws[57856] = kk * y[4704]; }
    { const double kk = ws[34976]; ws[57888] = kk * y[4736]; ws[57920] = kk * y[1696]; }
    { const double kk = ws[35008]; ws[57952] = kk * y[4736]; ws[57984] = kk * y[2208]; }
    { const double kk = ws[35040]; ws[58016] = kk * y[4384]; ws[58048] = kk * y[4448]; }
    { const double kk = ws[35072]; ws[58080] = kk * y[4608]; ws[58112] = kk * y[4448]; }
    { const double kk = ws[35168]; ws[58144] = kk * y[4704]; ws[58176] = kk * y[4448]; }
    { const double kk = ws[35200]; ws[58208] = kk * y[4672]; ws[58240] = kk * y[4448]; }
    { const double kk = ws[35232]; ws[58272] = kk * y[4448]; ws[58304] = kk * y[4448]; }
    { const double kk = ws[35264]; ws[58336] = kk * y[4096]; ws[58368] = kk * y[4448]; }
    { const double kk = ws[35296]; ws[58400] = kk * y[4384]; ws[58432] = kk * y[4096]; }
    { const double kk = ws[35328]; ws[58464] = kk * y[4608]; ws[58496] = kk * y[4096]; }
    { const double kk = ws[35424]; ws[58528] = kk * y[4704]; ws[58560] = kk * y[4096]; }
    { const double kk = ws[35456]; ws[58592] = kk * y[4672]; ws[58624] = kk * y[4096]; }
    { const double kk = ws[35488]; ws[58656] = kk * y[4096]; ws[58688] = kk * y[4096]; }
    { const double kk = ws[35520]; ws[58720] = kk * y[4384]; ws[58752] = kk * y[4672]; }
    { const double kk = ws[35552]; ws[58784] = kk * y[4704]; ws[58816] = kk * y[4672]; }
    { const double kk = ws[35584]; ws[58848] = kk * y[4672]; ws[58880] = kk * y[4672]; }
    { const double kk = ws[35616]; ws[58912] = kk * y[4384]; ws[58944] = kk * y[4416]; }
    { const double kk = ws[35648]; ws[58976] = kk * y[4704]; ws[59008] = kk * y[4416]; }
    { const double kk = ws[35680]; ws[59040] = kk * y[4448]; ws[59072] = kk * y[4416]; }
    { const double kk = ws[35712]; ws[59104] = kk * y[4672]; ws[59136] = kk * y[4416]; }
    { const double kk = ws[35744]; ws[59168] = kk * y[4384]; ws[59200] = kk * y[4576]; }
    { const double kk = ws[35776]; ws[59232] = kk * y[4704]; ws[59264] = kk * y[4576]; }
    { const double kk = ws[35808]; ws[59296] = kk * y[4448]; ws[59328] = kk * y[4576]; }
    { const double kk = ws[35840]; ws[59360] = kk * y[4672]; ws[59392] = kk * y[4576]; }
    { const double kk = ws[35872]; ws[59424] = kk * y[4384]; ws[59456] = kk * y[4352]; }
    { const double kk = ws[35904]; ws[59488] = kk * y[4704]; ws[59520] = kk * y[4352]; }
    { const double kk = ws[35936]; ws[59552] = kk * y[4448]; ws[59584] = kk * y[4352]; }
    { const double kk = ws[35968]; ws[59616] = kk * y[4672]; ws[59648] = kk * y[4352]; }
    { const double kk = ws[36000]; ws[59680] = kk * y[4384]; ws[59712] = kk * y[4288]; }
    { const double kk = ws[36032]; ws[59744] = kk * y[4704]; ws[59776] = kk * y[4288]; }
    { const double kk = ws[36064]; ws[59808] = kk * y[4448]; ws[59840] = kk * y[4288]; }
    { const double kk = ws[36096]; ws[59872] = kk * y[4672]; ws[59904] = kk * y[4288]; }
    { const double kk = ws[36128]; ws[59936] = kk * y[4736]; ws[59968] = kk * y[2272]; }
    { const double kk = ws[36192]; ws[60000] = kk * y[4736]; ws[60032] = kk * y[2880]; }
    { const double kk = ws[36256]; ws[60064] = kk * y[4736]; ws[60096] = kk * y[3648]; }
    { const double kk = ws[36320]; ws[60128] = kk * y[4736]; ws[60160] = kk * y[3776]; }
    { const double kk = ws[36352]; ws[60192] = kk * y[4736]; ws[60224] = kk * y[3904]; }
    { const double kk = ws[36384]; ws[60256] = kk * y[4736]; ws[60288] = kk * y[2688]; }
    { const double kk = ws[36416]; ws[60320] = kk * y[4736]; ws[60352] = kk * y[4512]; }
    { const double kk = ws[36512]; ws[60384] = kk * y[4160]; ws[60416] = kk * y[4512]; }
    { const double kk = ws[36544]; ws[60448] = kk * y[4640]; ws[60480] = kk * y[4512]; }
    { const double kk = ws[36576]; ws[60512] = kk * y[4704]; ws[60544] = kk * y[4512]; }
    { const double kk = ws[36640]; ws[60576] = kk * y[4384]; ws[60608] = kk * y[1728]; }
    { const double kk = ws[36672]; ws[60640] = kk * y[4704]; ws[60672] = kk * y[1728]; }
    { const double kk = ws[36704]; ws[60704] = kk * y[4160]; ws[60736] = kk * y[4128]; }
    { const double kk = ws[36736]; ws[60768] = kk * y[4736]; ws[60800] = kk * y[4128]; }
    { const double kk = ws[36768]; ws[60832] = kk * y[4640]; ws[60864] = kk * y[4128]; }
    { const double kk = ws[36832]; ws[60896] = kk * y[4160]; ws[60928] = kk * y[4064]; }
    { const double kk = ws[36864]; ws[60960] = kk * y[4736]; ws[60992] = kk * y[4064]; }
    { const double kk = ws[36896]; ws[61024] = kk * y[4640]; ws[61056] = kk * y[4064]; }
    { const double kk = ws[36960]; ws[61088] = kk * y[4736]; ws[61120] = kk * y[3840]; }
    { const double kk = ws[37024]; ws[61152] = kk * y[4640]; ws[61184] = kk * y[3840]; }
    { const double kk = ws[37056]; ws[61216] = kk * y[4736]; ws[61248] = kk * y[4256]; }
    { const double kk = ws[37120]; ws[61280] = kk * y[4640]; ws[61312] = kk * y[4256]; }
    { const double kk = ws[37184]; ws[61344] = kk * y[4640]; ws[61376] = kk * y[4000]; }
    { const double kk = ws[37216]; ws[61408] = kk * y[4736]; ws[61440] = kk * y[4000]; }
    { const double kk = ws[37280]; ws[61472] = kk * y[4736]; ws[61504] = kk * y[4480]; }
    { const double kk = ws[37344]; ws[61536] = kk * y[4736]; ws[61568] = kk * y[832]; }
    { const double kk = ws[37376]; ws[61600] = kk * y[4736]; ws[61632] = kk * y[2720]; }
    { const double kk = ws[37408]; ws[61664] = kk * y[4736]; ws[61696] = kk * y[864]; }
    { const double kk = ws[37504]; ws[61728] = kk * y[4736]; ws[61760] = kk * y[3392]; }
    { const double kk = ws[37536]; ws[61792] = kk * y[4736]; ws[61824] = kk * y[896]; }
    { const double kk = ws[37568]; ws[61856] = kk * y[4736]; ws[61888] = kk * y[4224]; }
    { const double kk = ws[37664]; ws[61920] = kk * y[4608]; ws[61952] = kk * y[960]; }
    { const double kk = ws[37696]; ws[61984] = kk * y[4736]; ws[62016] = kk * y[352]; }
    { const double kk = ws[37728]; ws[62048] = kk * y[4160]; ws[62080] = kk * y[2656]; }
    { const double kk = ws[37760]; ws[62112] = kk * y[4736]; ws[62144] = kk * y[2656]; }
    { const double kk = ws[37792]; ws[62176] = kk * y[4320]; ws[62208] = kk * y[2656]; }
    { const double kk = ws[37824]; ws[62240] = kk * y[4640]; ws[62272] = kk * y[2656]; }
    { const double kk = ws[37856]; ws[62304] = kk * y[4160]; ws[62336] = kk * y[3552]; }
    { const double kk = ws[37888]; ws[62368] = kk * y[4736]; ws[62400] = kk * y[3552]; }
    { const double kk = ws[37920]; ws[62432] = kk * y[4320]; ws[62464] = kk * y[3552]; }
    { const double kk = ws[37952]; ws[62496] = kk * y[4640]; ws[62528] = kk * y[3552]; }
    { const double kk = ws[37984]; ws[62560] = kk * y[4160]; ws[62592] = kk * y[3136]; }
    { const double kk = ws[38016]; ws[62624] = kk * y[4736]; ws[62656] = kk * y[3136]; }
    { const double kk = ws[38048]; ws[62688] = kk * y[4320]; ws[62720] = kk * y[3136]; }
    { const double kk = ws[38080]; ws[62752] = kk * y[4640]; ws[62784] = kk * y[3136]; }
    { const double kk = ws[38112]; ws[62816] = kk * y[4736]; ws[62848] = kk * y[2528]; }
    { const double kk = ws[38144]; ws[62880] = kk * y[4160]; ws[62912] = kk * y[2528]; }
    { const double kk = ws[38176]; ws[62944] = kk * y[4384]; ws[62976] = kk * y[3424]; }
    { const double kk = ws[38208]; ws[63008] = kk * y[4704]; ws[63040] = kk * y[3424]; }
    { const double kk = ws[38240]; ws[63072] = kk * y[4448]; ws[63104] = kk * y[3424]; }
    { const double kk = ws[38272]; ws[63136] = kk * y[4672]; ws[63168] = kk * y[3424]; }
    { const double kk = ws[38336]; ws[63200] = kk * y[4320]; ws[63232] = kk * y[2528]; }
    { const double kk = ws[38368]; ws[63264] = kk * y[4640]; ws[63296] = kk * y[2528]; }
    { const double kk = ws[38400]; ws[63328] = kk * y[4736]; ws[63360] = kk * y[3872]; }
    { const double kk = ws[38432]; ws[63392] = kk * y[4320]; ws[63424] = kk * y[3872]; }
    { const double kk = ws[38464]; ws[63456] = kk * y[4640]; ws[63488] = kk * y[3872]; }
    { const double kk = ws[38528]; ws[63520] = kk * y[4736]; ws[63552] = kk * y[1664]; }
    { const double kk = ws[38592]; ws[63584] = kk * y[4640]; ws[63616] = kk * y[1024]; }
    { const double kk = ws[38624]; ws[63648] = kk * y[4736]; ws[63680] = kk * y[1056]; }
    { const double kk = ws[38656]; ws[63712] = kk * y[4704]; ws[63744] = kk * y[3296]; }
    { const double kk = ws[38688]; ws[63776] = kk * y[4384]; ws[63808] = kk * y[3296]; }
    { const double kk = ws[38720]; ws[63840] = kk * y[4448]; ws[63872] = kk * y[3296]; }
    { const double kk = ws[38752]; ws[63904] = kk * y[4672]; ws[63936] = kk * y[3296]; }
    { const double kk = ws[38784]; ws[63968] = kk * y[4736]; ws[64000] = kk * y[1632]; }
    { const double kk = ws[38816]; ws[64032] = kk * y[4160]; ws[64064] = kk * y[2048]; }
    { const double kk = ws[38848]; ws[64096] = kk * y[4736]; ws[64128] = kk * y[2048]; }
    { const double kk = ws[38880]; ws[64160] = kk * y[4320]; ws[64192] = kk * y[2048]; }
    { const double kk = ws[38912]; ws[64224] = kk * y[4640]; ws[64256] = kk * y[2048]; }
    { const double kk = ws[38944]; ws[64288] = kk * y[4160]; ws[64320] = kk * y[2112]; }
    { const double kk = ws[38976]; ws[64352] = kk * y[4736]; ws[64384] = kk * y[2112]; }
    { const double kk = ws[39008]; ws[64416] = kk * y[4320]; ws[64448] = kk * y[2112]; }
    { const double kk = ws[39040]; ws[64480] = kk * y[4640]; ws[64512] = kk * y[2112]; }
    { const double kk = ws[39072]; ws[64544] = kk * y[4736]; ws[64576] = kk * y[384]; }
    { const double kk = ws[39104]; ws[64608] = kk * y[4384]; ws[64640] = kk * y[3104]; }
    { const double kk = ws[39136]; ws[64672] = kk * y[4448]; ws[64704] = kk * y[3104]; }
    { const double kk = ws[39168]; ws[64736] = kk * y[4704]; ws[64768] = kk * y[3104]; }
    { const double kk = ws[39200]; ws[64800] = kk * y[4672]; ws[64832] = kk * y[3104]; }
    { const double kk = ws[39232]; ws[64864] = kk * y[4736]; ws[64896] = kk * y[1088]; }
    { const double kk = ws[39264]; ws[64928] = kk * y[4384]; ws[64960] = kk * y[3488]; }
    { const double kk = ws[39296]; ws[64992] = kk * y[4448]; ws[65024] = kk * y[3488]; }
    { const double kk = ws[39328]; ws[65056] = kk * y[4704]; ws[65088] = kk * y[3488]; }
    { const double kk = ws[39360]; ws[65120] = kk * y[4672]; ws[65152] = kk * y[3488]; }
    { const double kk = ws[39392]; ws[65184] = kk * y[4736]; ws[65216] = kk * y[1120]; }
    { const double kk = ws[39424]; ws[65248] = kk * y[4736]; ws[65280] = kk * y[1152]; }
    { const double kk = ws[39456]; ws[65312] = kk * y[4384]; ws[65344] = kk * y[3584]; }
    { const double kk = ws[39488]; ws[65376] = kk * y[4704]; ws[65408] = kk * y[3584]; }
    { const double kk = ws[39520]; ws[65440] = kk * y[4448]; ws[65472] = kk * y[3584]; }
    { const double kk = ws[39552]; ws[65504] = kk * y[4672]; ws[65536] = kk * y[3584]; }
    { const double kk = ws[39584]; ws[65568] = kk * y[4736]; ws[65600] = kk * y[3616]; }
    { const double kk = ws[39616]; ws[65632] = kk * y[4640]; ws[65664] = kk * y[3616]; }
    { const double kk = ws[39648]; ws[65696] = kk * y[4608]; ws[65728] = kk * y[3328]; }
    { const double kk = ws[39680]; ws[65760] = kk * y[4704]; ws[65792] = kk * y[3328]; }
    { const double kk = ws[39712]; ws[65824] = kk * y[4736]; ws[65856] = kk * y[2176]; }
    { const double kk = ws[39744]; ws[65888] = kk * y[4640]; ws[65920] = kk * y[2176]; }
    { const double kk = ws[39840]; ws[65952] = kk * y[4736]; ws[65984] = kk * y[3808]; }
    { const double kk = ws[39872]; ws[66016] = kk * y[4320]; ws[66048] = kk * y[3808]; }
    { const double kk = ws[39904]; ws[66080] = kk * y[4640]; ws[66112] = kk * y[3808]; }
    { const double kk = ws[39968]; ws[66144] = kk * y[4736]; ws[66176] = kk * y[3936]; }
    { const double kk = ws[40000]; ws[66208] = kk * y[4320]; ws[66240] = kk * y[3936]; }
    { const double kk = ws[40032]; ws[66272] = kk * y[4640]; ws[66304] = kk * y[3936]; }
    { const double kk = ws[40064]; ws[66336] = kk * y[4736]; ws[66368] = kk * y[1760]; }
    { const double kk = ws[40096]; ws[66400] = kk * y[4640]; ws[66432] = kk * y[1760]; }
    { const double kk = ws[40128]; ws[66464] = kk * y[4384]; ws[66496] = kk * y[3744]; }
    { const double kk = ws[40160]; ws[66528] = kk * y[4608]; ws[66560] = kk * y[3744]; }
    { const double kk = ws[40224]; ws[66592] = kk * y[4704]; ws[66624] = kk * y[3744]; }
    { const double kk = ws[40256]; ws[66656] = kk * y[4448]; ws[66688] = kk * y[3744]; }
    { const double kk = ws[40288]; ws[66720] = kk * y[4672]; ws[66752] = kk * y[3744]; }
    { const double kk = ws[40320]; ws[66784] = kk * y[4736]; ws[66816] = kk * y[1792]; }
    { const double kk = ws[40352]; ws[66848] = kk * y[4736]; ws[66880] = kk * y[1952]; }
    { const double kk = ws[40384]; ws[66912] = kk * y[4736]; ws[66944] = kk * y[416]; }
    { const double kk = ws[40544]; ws[66976] = kk * y[4736]; ws[67008] = kk * y[4608]; }
    { const double kk = ws[40640]; ws[67040] = kk * y[4320]; ws[67072] = kk * y[4544]; }
    { const double kk = ws[40672]; ws[67104] = kk * y[3520]; ws[67136] = kk * y[3520]; }
    { const double kk = ws[40704]; ws[67168] = kk * y[4384]; ws[67200] = kk * y[3520]; }
    { const double kk = ws[40736]; ws[67232] = kk * y[4704]; ws[67264] = kk * y[3520]; }
    { const double kk = ws[40768]; ws[67296] = kk * y[4416]; ws[67328] = kk * y[3520]; }
    { const double kk = ws[40800]; ws[67360] = kk * y[3232]; ws[67392] = kk * y[4736]; }
    { const double kk = ws[40896]; ws[67424] = kk * y[4224]; ws[67456] = kk * y[4544]; }
    { const double kk = ws[40928]; ws[67488] = kk * y[896]; ws[67520] = kk * y[4544]; }
    { const double kk = ws[40960]; ws[67552] = kk * y[832]; ws[67584] = kk * y[4544]; }
    { const double kk = ws[40992]; ws[67616] = kk * y[2656]; ws[67648] = kk * y[4544]; }
    { const double kk = ws[41024]; ws[67680] = kk * y[3552]; ws[67712] = kk * y[4544]; }
    { const double kk = ws[41056]; ws[67744] = kk * y[3136]; ws[67776] = kk * y[4544]; }
    { const double kk = ws[41088]; ws[67808] = kk * y[2528]; ws[67840] = kk * y[4544]; }
    { const double kk = ws[41120]; ws[67872] = kk * y[4512]; ws[67904] = kk * y[4544]; }
    { const double kk = ws[41152]; ws[67936] = kk * y[4128]; ws[67968] = kk * y[4544]; }
    { const double kk = ws[41184]; ws[68000] = kk * y[4064]; ws[68032] = kk * y[4544]; }
    { const double kk = ws[41216]; ws[68064] = kk * y[2720]; ws[68096] = kk * y[4544]; }
    { const double kk = ws[41248]; ws[68128] = kk * y[864]; ws[68160] = kk * y[4544]; }
    { const double kk = ws[41280]; ws[68192] = kk * y[4736]; ws[68224] = kk * y[3968]; }
    { const double kk = ws[41312]; ws[68256] = kk * y[1088]; ws[68288] = kk * y[4544]; }
    { const double kk = ws[41344]; ws[68320] = kk * y[1120]; ws[68352] = kk * y[4544]; }
    { const double kk = ws[41376]; ws[68384] = kk * y[1152]; ws[68416] = kk * y[4544]; }
    { const double kk = ws[41440]; ws[68448] = kk * y[4608]; ws[68480] = kk * y[3520]; }
    { const double kk = ws[41600]; ws[68512] = kk * y[4384]; ws[68544] = kk * y[2944]; }
    { const double kk = ws[41632]; ws[68576] = kk * y[4704]; ws[68608] = kk * y[2944]; }
    { const double kk = ws[41664]; ws[68640] = kk * y[4384]; ws[68672] = kk * y[2496]; }
    { const double kk = ws[41696]; ws[68704] = kk * y[4704]; ws[68736] = kk * y[2496]; }
    { const double kk = ws[41728]; ws[68768] = kk * y[4384]; ws[68800] = kk * y[2144]; }
    { const double kk = ws[41760]; ws[68832] = kk * y[4704]; ws[68864] = kk * y[2144]; }
    { const double kk = ws[41792]; ws[68896] = kk * y[4320]; ws[68928] = kk * y[1856]; }
    { const double kk = ws[41824]; ws[68960] = kk * y[4736]; ws[68992] = kk * y[1856]; }
    { const double kk = ws[41856]; ws[69024] = kk * y[4640]; ws[69056] = kk * y[1856]; }
    { const double kk = ws[41888]; ws[69088] = kk * y[4384]; ws[69120] = kk * y[2560]; }
    { const double kk = ws[41920]; ws[69152] = kk * y[4704]; ws[69184] = kk * y[2560]; }
    { const double kk = ws[41952]; ws[69216] = kk * y[4736]; ws[69248] = kk * y[448]; }
    { const double kk = ws[42144]; ws[69280] = kk * y[480]; ws[69312] = kk * y[1920]; }
    { const double kk = ws[42176]; ws[69344] = kk * y[512]; ws[69376] = kk * y[1920]; }
    { const double kk = ws[42208]; ws[69408] = kk * y[544]; ws[69440] = kk * y[1248]; }
    { const double kk = ws[42336]; ws[69472] = kk * y[576]; ws[69504] = kk * y[1312]; }
    { const double kk = ws[42464]; ws[69536] = kk * y[4384]; ws[69568] = kk * y[2848]; }
    { const double kk = ws[42496]; ws[69600] = kk * y[4704]; ws[69632] = kk * y[2848]; }
    { const double kk = ws[42528]; ws[69664] = kk * y[4640]; ws[69696] = kk * y[2848]; }
    { const double kk = ws[42560]; ws[69728] = kk * y[4672]; ws[69760] = kk * y[2848]; }
    { const double kk = ws[42592]; ws[69792] = kk * y[4544]; ws[69824] = kk * y[3360]; }
    { const double kk = ws[42624]; ws[69856] = kk * y[4736]; ws[69888] = kk * y[3360]; }
    { const double kk = ws[42912]; ws[69920] = kk * y[4736]; ws[69952] = kk * y[704]; }
    { const double kk = ws[42944]; ws[69984] = kk * y[4736]; ws[70016] = kk * y[1440]; }
    { const double kk = ws[42976]; ws[70048] = kk * y[4736]; ws[70080] = kk * y[736]; }
    { const double kk = ws[43008]; ws[70112] = kk * y[4736]; ws[70144] = kk * y[1472]; }
    { const double kk = ws[43040]; ws[70176] = kk * y[4736]; ws[70208] = kk * y[768]; }
    { const double kk = ws[43072]; ws[70240] = kk * y[4736]; ws[70272] = kk * y[2752]; }
    { const double kk = ws[43104]; ws[70304] = kk * y[4736]; ws[70336] = kk * y[2784]; }
    { const double kk = ws[43136]; ws[70368] = kk * y[4736]; ws[70400] = kk * y[2816]; }
    { const double kk = ws[43168]; ws[70432] = kk * y[4736]; ws[70464] = kk * y[2304]; }
    { const double kk = ws[43200]; ws[70496] = kk * y[4736]; ws[70528] = kk * y[1504]; }
    { const double kk = ws[43232]; ws[70560] = kk * y[4736]; ws[70592] = kk * y[3680]; }
    { const double kk = ws[43264]; ws[70624] = kk * y[4736]; ws[70656] = kk * y[3712]; }
    { const double kk = ws[43296]; ws[70688] = kk * y[4736]; ws[70720] = kk * y[2912]; }
    { const double kk = ws[43328]; ws[70752] = kk * y[4736]; ws[70784] = kk * y[3168]; }
    { const double kk = ws[43360]; ws[70816] = kk * y[4736]; ws[70848] = kk * y[3200]; }
    { const double kk = ws[43392]; ws[70880] = kk * y[4736]; ws[70912] = kk * y[2336]; }
    { const double kk = ws[43424]; ws[70944] = kk * y[4640]; ws[70976] = kk * y[2336]; }
    { const double kk = ws[43456]; ws[71008] = kk * y[4160]; ws[71040] = kk * y[2336]; }
    { const double kk = ws[43552]; ws[71072] = kk * y[4544]; ws[71104] = kk * y[2336]; }
    { const double kk = ws[43584]; ws[71136] = kk * y[4736]; ws[71168] = kk * y[2368]; }
    { const double kk = ws[43616]; ws[71200] = kk * y[4640]; ws[71232] = kk * y[2368]; }
    { const double kk = ws[43648]; ws[71264] = kk * y[4160]; ws[71296] = kk * y[2368]; }
    { const double kk = ws[43712]; ws[71328] = kk * y[4544]; ws[71360] = kk * y[2368]; }
    { const double kk = ws[43744]; ws[71392] = kk * y[4736]; ws[71424] = kk * y[2400]; }
    { const double kk = ws[43776]; ws[71456] = kk * y[4320]; ws[71488] = kk * y[2400]; }
    { const double kk = ws[43808]; ws[71520] = kk * y[4640]; ws[71552] = kk * y[2400]; }
    { const double kk = ws[43840]; ws[71584] = kk * y[4544]; ws[71616] = kk * y[2400]; }
    { const double kk = ws[43872]; ws[71648] = kk * y[4736]; ws[71680] = kk * y[2432]; }
    { const double kk = ws[43904]; ws[71712] = kk * y[4320]; ws[71744] = kk * y[2432]; }
    { const double kk = ws[43936]; ws[71776] = kk * y[4640]; ws[71808] = kk * y[2432]; }
    { const double kk = ws[44000]; ws[71840] = kk * y[4544]; ws[71872] = kk * y[2432]; }
    { const double kk = ws[44032]; ws[71904] = kk * y[4736]; ws[71936] = kk * y[2976]; }
    { const double kk = ws[44064]; ws[71968] = kk * y[4320]; ws[72000] = kk * y[2976]; }
    { const double kk = ws[44096]; ws[72032] = kk * y[4640]; ws[72064] = kk * y[2976]; }
    { const double kk = ws[44160]; ws[72096] = kk * y[4544]; ws[72128] = kk * y[2976]; }
    { const double kk = ws[44192]; ws[72160] = kk * y[4736]; ws[72192] = kk * y[1536]; }
    { const double kk = ws[44224]; ws[72224] = kk * y[4544]; ws[72256] = kk * y[1536]; }
    { const double kk = ws[44256]; ws[72288] = kk * y[4320]; ws[72320] = kk * y[3008]; }
    { const double kk = ws[44288]; ws[72352] = kk * y[1184]; ws[72384] = kk * y[3008]; }
    { const double kk = ws[44320]; ws[72416] = kk * y[3456]; ws[72448] = kk * y[3008]; }
    { const double kk = ws[44352]; ws[72480] = kk * y[4736]; ws[72512] = kk * y[3008]; }
    { const double kk = ws[44384]; ws[72544] = kk * y[4544]; ws[72576] = kk * y[3008]; }
    { const double kk = ws[44416]; ws[72608] = kk * y[4736]; ws[72640] = kk * y[2016]; }
    { const double kk = ws[44448]; ws[72672] = kk * y[4736]; ws[72704] = kk * y[2016]; }
    { const double kk = ws[44480]; ws[72736] = kk * y[4640]; ws[72768] = kk * y[2016]; }
    { const double kk = ws[44512]; ws[72800] = kk * y[4544]; ws[72832] = kk * y[2016]; }
}
// f(y) for the night reaction list (rbfeval.F:80-151).
__device__ __noinline__ void feval_1(double* __restrict__ ws, int src, int dst)
{
    const double* __restrict__ yin = ws + src * 32;
    double* __restrict__ yout = ws + dst * 32;
    ws[44576] = (ws[33408]) * yin[4160];
    ws[44608] = ((ws[33440]) * yin[4320]) * yin[4384];
    ws[44640] = ((ws[33472]) * yin[4160]) * yin[4384];
    ws[44672] = ((ws[33504]) * yin[4160]) * yin[4608];
    ws[44704] = ((ws[33536]) * yin[4160]) * yin[4608];
    ws[44736] = ((ws[33568]) * yin[4160]) * yin[4320];
    ws[44832] = (ws[33664]) * yin[672];
    ws[44864] = (ws[33696]) * yin[672];
    ws[44896] = ((ws[33728]) * yin[4320]) * yin[4736];
    ws[44928] = ((ws[33760]) * yin[4320]) * yin[4704];
    ws[44960] = ((ws[33792]) * yin[4736]) * yin[4160];
    ws[44992] = ((ws[33824]) * yin[4704]) * yin[4160];
    ws[45024] = ((ws[33856]) * yin[4736]) * yin[4736];
    ws[45056] = ((ws[33888]) * yin[4736]) * yin[4736];
    ws[45088] = ((ws[33920]) * yin[4736]) * yin[4704];
    ws[45120] = ((ws[33952]) * yin[4704]) * yin[4704];
    ws[45152] = ((ws[33984]) * yin[4704]) * yin[4704];
    ws[45216] = ((ws[34048]) * yin[3456]) * yin[4736];
    ws[45248] = ((ws[34080]) * yin[3456]) * yin[4160];
    ws[45280] = ((ws[34112]) * yin[4384]) * yin[4384];
    ws[45312] = ((ws[34144]) * yin[4704]) * yin[4384];
    ws[45344] = ((ws[34176]) * yin[4608]) * yin[4320];
    ws[45440] = ((ws[34272]) * yin[4640]) * yin[4384];
    ws[45472] = ((ws[34304]) * yin[4640]) * yin[4608];
    ws[45504] = ((ws[34336]) * yin[4640]) * yin[4160];
    ws[45536] = ((ws[34368]) * yin[4640]) * yin[4736];
    ws[45568] = ((ws[34400]) * yin[4640]) * yin[4704];
    ws[45600] = ((ws[34432]) * yin[4640]) * yin[4320];
    ws[45632] = ((ws[34464]) * yin[4640]) * yin[4640];
    ws[45664] = ((ws[34496]) * yin[4640]) * yin[4608];
    ws[45696] = (ws[34528]) * yin[1280];
    ws[45760] = (ws[34592]) * yin[1280];
    ws[45792] = ((ws[34624]) * yin[4384]) * yin[4736];
    ws[45824] = ((ws[34656]) * yin[4384]) * yin[4608];
    ws[45856] = ((ws[34688]) * yin[2464]) * yin[2464];
    ws[45920] = ((ws[34752]) * yin[2464]) * yin[4736];
    ws[45952] = ((ws[34784]) * yin[4608]) * yin[4736];
    ws[45984] = ((ws[34816]) * yin[4192]) * yin[4736];
    ws[46048] = ((ws[34880]) * yin[4704]) * yin[4608];
    ws[46080] = (ws[34912]) * yin[1696];
    ws[46144] = ((ws[34976]) * yin[1696]) * yin[4736];
    ws[46176] = ((ws[35008]) * yin[2208]) * yin[4736];
    ws[46208] = ((ws[35040]) * yin[4448]) * yin[4384];
    ws[46240] = ((ws[35072]) * yin[4448]) * yin[4608];
    ws[46272] = (ws[35104]) * yin[1344];
    ws[46336] = ((ws[35168]) * yin[4448]) * yin[4704];
    ws[46368] = ((ws[35200]) * yin[4448]) * yin[4672];
    ws[46400] = ((ws[35232]) * yin[4448]) * yin[4448];
    ws[46432] = ((ws[35264]) * yin[4448]) * yin[4096];
    ws[46464] = ((ws[35296]) * yin[4096]) * yin[4384];
    ws[46496] = ((ws[35328]) * yin[4096]) * yin[4608];
    ws[46528] = (ws[35360]) * yin[1952];
    ws[46592] = ((ws[35424]) * yin[4096]) * yin[4704];
    ws[46624] = ((ws[35456]) * yin[4096]) * yin[4672];
    ws[46656] = ((ws[35488]) * yin[4096]) * yin[4096];
    ws[46688] = ((ws[35520]) * yin[4672]) * yin[4384];
    ws[46720] = ((ws[35552]) * yin[4672]) * yin[4704];
    ws[46752] = ((ws[35584]) * yin[4672]) * yin[4672];
    ws[46784] = ((ws[35616]) * yin[4416]) * yin[4384];
    ws[46816] = ((ws[35648]) * yin[4416]) * yin[4704];
    ws[46848] = ((ws[35680]) * yin[4416]) * yin[4448];
    ws[46880] = ((ws[35712]) * yin[4416]) * yin[4672];
    ws[46912] = ((ws[35744]) * yin[4576]) * yin[4384];
    ws[46944] = ((ws[35776]) * yin[4576]) * yin[4704];
    ws[46976] = ((ws[35808]) * yin[4576]) * yin[4448];
    ws[47008] = ((ws[35840]) * yin[4576]) * yin[4672];
    ws[47040] = ((ws[35872]) * yin[4352]) * yin[4384];
    ws[47072] = ((ws[35904]) * yin[4352]) * yin[4704];
    ws[47104] = ((ws[35936]) * yin[4352]) * yin[4448];
    ws[47136] = ((ws[35968]) * yin[4352]) * yin[4672];
    ws[47168] = ((ws[36000]) * yin[4288]) * yin[4384];
    ws[47200] = ((ws[36032]) * yin[4288]) * yin[4704];
    ws[47232] = ((ws[36064]) * yin[4288]) * yin[4448];
    ws[47264] = ((ws[36096]) * yin[4288]) * yin[4672];
    ws[47296] = ((ws[36128]) * yin[2272]) * yin[4736];
    ws[47360] = ((ws[36192]) * yin[2880]) * yin[4736];
    ws[47424] = ((ws[36256]) * yin[3648]) * yin[4736];
    ws[47488] = ((ws[36320]) * yin[3776]) * yin[4736];
    ws[47520] = ((ws[36352]) * yin[3904]) * yin[4736];
    ws[47552] = ((ws[36384]) * yin[2688]) * yin[4736];
    ws[47584] = ((ws[36416]) * yin[4512]) * yin[4736];
    ws[47680] = ((ws[36512]) * yin[4512]) * yin[4160];
    ws[47712] = ((ws[36544]) * yin[4512]) * yin[4640];
    ws[47744] = ((ws[36576]) * yin[4512]) * yin[4704];
    ws[47776] = (ws[36608]) * yin[1728];
    ws[47808] = ((ws[36640]) * yin[1728]) * yin[4384];
    ws[47840] = ((ws[36672]) * yin[1728]) * yin[4704];
    ws[47872] = ((ws[36704]) * yin[4128]) * yin[4160];
    ws[47904] = ((ws[36736]) * yin[4128]) * yin[4736];
    ws[47936] = ((ws[36768]) * yin[4128]) * yin[4640];
    ws[48000] = ((ws[36832]) * yin[4064]) * yin[4160];
    ws[48032] = ((ws[36864]) * yin[4064]) * yin[4736];
    ws[48064] = ((ws[36896]) * yin[4064]) * yin[4640];
    ws[48128] = ((ws[36960]) * yin[3840]) * yin[4736];
    ws[48192] = ((ws[37024]) * yin[3840]) * yin[4640];
    ws[48224] = ((ws[37056]) * yin[4256]) * yin[4736];
    ws[48288] = ((ws[37120]) * yin[4256]) * yin[4640];
    ws[48352] = ((ws[37184]) * yin[4000]) * yin[4640];
    ws[48384] = ((ws[37216]) * yin[4000]) * yin[4736];
    ws[48416] = (ws[37248]) * yin[4736];
    ws[48448] = ((ws[37280]) * yin[4480]) * yin[4736];
    ws[48480] = (ws[37312]) * yin[4736];
    ws[48512] = ((ws[37344]) * yin[832]) * yin[4736];
    ws[48544] = ((ws[37376]) * yin[2720]) * yin[4736];
    ws[48576] = ((ws[37408]) * yin[864]) * yin[4736];
    ws[48672] = ((ws[37504]) * yin[3392]) * yin[4736];
    ws[48704] = ((ws[37536]) * yin[896]) * yin[4736];
    ws[48736] = ((ws[37568]) * yin[4224]) * yin[4736];
    ws[48768] = (ws[37600]) * yin[960];
    ws[48800] = (ws[37632]) * yin[960];
    ws[48832] = ((ws[37664]) * yin[960]) * yin[4608];
    ws[48864] = ((ws[37696]) * yin[352]) * yin[4736];
    ws[48896] = ((ws[37728]) * yin[2656]) * yin[4160];
    ws[48928] = ((ws[37760]) * yin[2656]) * yin[4736];
    ws[48960] = ((ws[37792]) * yin[2656]) * yin[4320];
    ws[48992] = ((ws[37824]) * yin[2656]) * yin[4640];
    ws[49024] = ((ws[37856]) * yin[3552]) * yin[4160];
    ws[49056] = ((ws[37888]) * yin[3552]) * yin[4736];
    ws[49088] = ((ws[37920]) * yin[3552]) * yin[4320];
    ws[49120] = ((ws[37952]) * yin[3552]) * yin[4640];
    ws[49152] = ((ws[37984]) * yin[3136]) * yin[4160];
    ws[49184] = ((ws[38016]) * yin[3136]) * yin[4736];
    ws[49216] = ((ws[38048]) * yin[3136]) * yin[4320];
    ws[49248] = ((ws[38080]) * yin[3136]) * yin[4640];
    ws[49280] = ((ws[38112]) * yin[2528]) * yin[4736];
    ws[49312] = ((ws[38144]) * yin[2528]) * yin[4160];
    ws[49344] = ((ws[38176]) * yin[3424]) * yin[4384];
    ws[49376] = ((ws[38208]) * yin[3424]) * yin[4704];
    ws[49408] = ((ws[38240]) * yin[3424]) * yin[4448];
    ws[49440] = ((ws[38272]) * yin[3424]) * yin[4672];
    ws[49472] = (ws[38304]) * yin[3424];
    ws[49504] = ((ws[38336]) * yin[2528]) * yin[4320];
    ws[49536] = ((ws[38368]) * yin[2528]) * yin[4640];
    ws[49568] = ((ws[38400]) * yin[3872]) * yin[4736];
    ws[49600] = ((ws[38432]) * yin[3872]) * yin[4320];
    ws[49632] = ((ws[38464]) * yin[3872]) * yin[4640];
    ws[49696] = ((ws[38528]) * yin[1664]) * yin[4736];
    ws[49760] = ((ws[38592]) * yin[1024]) * yin[4640];
    ws[49792] = ((ws[38624]) * yin[1056]) * yin[4736];
    ws[49824] = ((ws[38656]) * yin[3296]) * yin[4704];
    ws[49856] = ((ws[38688]) * yin[3296]) * yin[4384];
    ws[49888] = ((ws[38720]) * yin[3296]) * yin[4448];
    ws[49920] = ((ws[38752]) * yin[3296]) * yin[4672];
    ws[49952] = ((ws[38784]) * yin[1632]) * yin[4736];
    ws[49984] = ((ws[38816]) * yin[2048]) * yin[4160];
    ws[50016] = ((ws[38848]) * yin[2048]) * yin[4736];
    ws[50048] = ((ws[38880]) * yin[2048]) * yin[4320];
    ws[50080] = ((ws[38912]) * yin[2048]) * yin[4640];
    ws[50112] = ((ws[38944]) * yin[2112]) * yin[4160];
    ws[50144] = ((ws[38976]) * yin[2112]) * yin[4736];
    ws[50176] = ((ws[39008]) * yin[2112]) * yin[4320];
    ws[50208] = ((ws[39040]) * yin[2112]) * yin[4640];
    ws[50240] = ((ws[39072]) * yin[384]) * yin[4736];
    ws[50272] = ((ws[39104]) * yin[3104]) * yin[4384];
    ws[50304] = ((ws[39136]) * yin[3104]) * yin[4448];
    ws[50336] = ((ws[39168]) * yin[3104]) * yin[4704];
    ws[50368] = ((ws[39200]) * yin[3104]) * yin[4672];
    ws[50400] = ((ws[39232]) * yin[1088]) * yin[4736];
    ws[50432] = ((ws[39264]) * yin[3488]) * yin[4384];
    ws[50464] = ((ws[39296]) * yin[3488]) * yin[4448];
    ws[50496] = ((ws[39328]) * yin[3488]) * yin[4704];
    ws[50528] = ((ws[39360]) * yin[3488]) * yin[4672];
    ws[50560] = ((ws[39392]) * yin[1120]) * yin[4736];
    ws[50592] = ((ws[39424]) * yin[1152]) * yin[4736];
    ws[50624] = ((ws[39456]) * yin[3584]) * yin[4384];
    ws[50656] = ((ws[39488]) * yin[3584]) * yin[4704];
    ws[50688] = ((ws[39520]) * yin[3584]) * yin[4448];
    ws[50720] = ((ws[39552]) * yin[3584]) * yin[4672];
    ws[50752] = ((ws[39584]) * yin[3616]) * yin[4736];
    ws[50784] = ((ws[39616]) * yin[3616]) * yin[4640];
    ws[50816] = ((ws[39648]) * yin[3328]) * yin[4608];
    ws[50848] = ((ws[39680]) * yin[3328]) * yin[4704];
    ws[50880] = ((ws[39712]) * yin[2176]) * yin[4736];
    ws[50912] = ((ws[39744]) * yin[2176]) * yin[4640];
    ws[51008] = ((ws[39840]) * yin[3808]) * yin[4736];
    ws[51040] = ((ws[39872]) * yin[3808]) * yin[4320];
    ws[51072] = ((ws[39904]) * yin[3808]) * yin[4640];
    ws[51136] = ((ws[39968]) * yin[3936]) * yin[4736];
    ws[51168] = ((ws[40000]) * yin[3936]) * yin[4320];
    ws[51200] = ((ws[40032]) * yin[3936]) * yin[4640];
    ws[51232] = ((ws[40064]) * yin[1760]) * yin[4736];
    ws[51264] = ((ws[40096]) * yin[1760]) * yin[4640];
    ws[51296] = ((ws[40128]) * yin[3744]) * yin[4384];
    ws[51328] = ((ws[40160]) * yin[3744]) * yin[4608];
    ws[51360] = (ws[40192]) * yin[1792];
    ws[51392] = ((ws[40224]) * yin[3744]) * yin[4704];
    ws[51424] = ((ws[40256]) * yin[3744]) * yin[4448];
    ws[51456] = ((ws[40288]) * yin[3744]) * yin[4672];
    ws[51488] = ((ws[40320]) * yin[1792]) * yin[4736];
    ws[51520] = ((ws[40352]) * yin[1952]) * yin[4736];
    ws[51552] = ((ws[40384]) * yin[416]) * yin[4736];
    ws[51584] = (ws[40416]) * yin[928];
    ws[51616] = (ws[40448]) * yin[928];
    ws[51648] = (ws[40480]) * yin[1984];
    ws[51680] = (ws[40512]) * yin[1984];
    ws[51712] = ((ws[40544]) * yin[4608]) * yin[4736];
    ws[51808] = ((ws[40640]) * yin[4544]) * yin[4320];
    ws[51840] = ((ws[40672]) * yin[3520]) * yin[3520];
    ws[51872] = ((ws[40704]) * yin[3520]) * yin[4384];
    ws[51904] = ((ws[40736]) * yin[3520]) * yin[4704];
    ws[51936] = ((ws[40768]) * yin[3520]) * yin[4416];
    ws[51968] = ((ws[40800]) * yin[4736]) * yin[3232];
    ws[52032] = (ws[40864]) * yin[4544];
    ws[52064] = ((ws[40896]) * yin[4544]) * yin[4224];
    ws[52096] = ((ws[40928]) * yin[4544]) * yin[896];
    ws[52128] = ((ws[40960]) * yin[4544]) * yin[832];
    ws[52160] = ((ws[40992]) * yin[4544]) * yin[2656];
    ws[52192] = ((ws[41024]) * yin[4544]) * yin[3552];
    ws[52224] = ((ws[41056]) * yin[4544]) * yin[3136];
    ws[52256] = ((ws[41088]) * yin[4544]) * yin[2528];
    ws[52288] = ((ws[41120]) * yin[4544]) * yin[4512];
    ws[52320] = ((ws[41152]) * yin[4544]) * yin[4128];
    ws[52352] = ((ws[41184]) * yin[4544]) * yin[4064];
    ws[52384] = ((ws[41216]) * yin[4544]) * yin[2720];
    ws[52416] = ((ws[41248]) * yin[4544]) * yin[864];
    ws[52448] = ((ws[41280]) * yin[3968]) * yin[4736];
    ws[52480] = ((ws[41312]) * yin[4544]) * yin[1088];
    ws[52512] = ((ws[41344]) * yin[4544]) * yin[1120];
    ws[52544] = ((ws[41376]) * yin[4544]) * yin[1152];
    ws[52608] = ((ws[41440]) * yin[3520]) * yin[4608];
    ws[52704] = (ws[41536]) * yin[1216];
    ws[52736] = (ws[41568]) * yin[1216];
    ws[52768] = ((ws[41600]) * yin[2944]) * yin[4384];
    ws[52800] = ((ws[41632]) * yin[2944]) * yin[4704];
    ws[52832] = ((ws[41664]) * yin[2496]) * yin[4384];
    ws[52864] = ((ws[41696]) * yin[2496]) * yin[4704];
    ws[52896] = ((ws[41728]) * yin[2144]) * yin[4384];
    ws[52928] = ((ws[41760]) * yin[2144]) * yin[4704];
    ws[52960] = ((ws[41792]) * yin[1856]) * yin[4320];
    ws[52992] = ((ws[41824]) * yin[1856]) * yin[4736];
    ws[53024] = ((ws[41856]) * yin[1856]) * yin[4640];
    ws[53056] = ((ws[41888]) * yin[2560]) * yin[4384];
    ws[53088] = ((ws[41920]) * yin[2560]) * yin[4704];
    ws[53120] = ((ws[41952]) * yin[448]) * yin[4736];
    ws[53152] = (ws[41984]) * yin[4032];
    ws[53184] = (ws[42016]) * yin[1280];
    ws[53216] = (ws[42048]) * yin[1280];
    ws[53248] = (ws[42080]) * yin[1920];
    ws[53280] = (ws[42112]) * yin[1248];
    ws[53312] = ((ws[42144]) * yin[1920]) * yin[480];
    ws[53344] = ((ws[42176]) * yin[1920]) * yin[512];
    ws[53376] = ((ws[42208]) * yin[1248]) * yin[544];
    ws[53408] = (ws[42240]) * yin[4608];
    ws[53472] = (ws[42304]) * yin[1056];
    ws[53504] = ((ws[42336]) * yin[1312]) * yin[576];
    ws[53536] = (ws[42368]) * yin[1312];
    ws[53568] = (ws[42400]) * yin[4256];
    ws[53600] = (ws[42432]) * yin[4000];
    ws[53632] = ((ws[42464]) * yin[2848]) * yin[4384];
    ws[53664] = ((ws[42496]) * yin[2848]) * yin[4704];
    ws[53696] = ((ws[42528]) * yin[2848]) * yin[4640];
    ws[53728] = ((ws[42560]) * yin[2848]) * yin[4672];
    ws[53760] = ((ws[42592]) * yin[3360]) * yin[4544];
    ws[53792] = ((ws[42624]) * yin[3360]) * yin[4736];
    ws[53856] = (ws[42688]) * yin[0];
    ws[53888] = (ws[42720]) * yin[64];
    ws[53920] = (ws[42752]) * yin[96];
    ws[53952] = (ws[42784]) * yin[128];
    ws[53984] = (ws[42816]) * yin[160];
    ws[54016] = (ws[42848]) * yin[192];
    ws[54048] = (ws[42880]) * yin[224];
    ws[54080] = ((ws[42912]) * yin[704]) * yin[4736];
    ws[54112] = ((ws[42944]) * yin[1440]) * yin[4736];
    ws[54144] = ((ws[42976]) * yin[736]) * yin[4736];
    ws[54176] = ((ws[43008]) * yin[1472]) * yin[4736];
    ws[54208] = ((ws[43040]) * yin[768]) * yin[4736];
    ws[54240] = ((ws[43072]) * yin[2752]) * yin[4736];
    ws[54272] = ((ws[43104]) * yin[2784]) * yin[4736];
    ws[54304] = ((ws[43136]) * yin[2816]) * yin[4736];
    ws[54336] = ((ws[43168]) * yin[2304]) * yin[4736];
    ws[54368] = ((ws[43200]) * yin[1504]) * yin[4736];
    ws[54400] = ((ws[43232]) * yin[3680]) * yin[4736];
    ws[54432] = ((ws[43264]) * yin[3712]) * yin[4736];
    ws[54464] = ((ws[43296]) * yin[2912]) * yin[4736];
    ws[54496] = ((ws[43328]) * yin[3168]) * yin[4736];
    ws[54528] = ((ws[43360]) * yin[3200]) * yin[4736];
    ws[54560] = ((ws[43392]) * yin[2336]) * yin[4736];
    ws[54592] = ((ws[43424]) * yin[2336]) * yin[4640];
    ws[54624] = ((ws[43456]) * yin[2336]) * yin[4160];
    ws[54720] = ((ws[43552]) * yin[2336]) * yin[4544];
    ws[54752] = ((ws[43584]) * yin[2368]) * yin[4736];
    ws[54784] = ((ws[43616]) * yin[2368]) * yin[4640];
    ws[54816] = ((ws[43648]) * yin[2368]) * yin[4160];
    ws[54880] = ((ws[43712]) * yin[2368]) * yin[4544];
    ws[54912] = ((ws[43744]) * yin[2400]) * yin[4736];
    ws[54944] = ((ws[43776]) * yin[2400]) * yin[4320];
    ws[54976] = ((ws[43808]) * yin[2400]) * yin[4640];
    ws[55008] = ((ws[43840]) * yin[2400]) * yin[4544];
    ws[55040] = ((ws[43872]) * yin[2432]) * yin[4736];
    ws[55072] = ((ws[43904]) * yin[2432]) * yin[4320];
    ws[55104] = ((ws[43936]) * yin[2432]) * yin[4640];
    ws[55168] = ((ws[44000]) * yin[2432]) * yin[4544];
    ws[55200] = ((ws[44032]) * yin[2976]) * yin[4736];
    ws[55232] = ((ws[44064]) * yin[2976]) * yin[4320];
    ws[55264] = ((ws[44096]) * yin[2976]) * yin[4640];
    ws[55328] = ((ws[44160]) * yin[2976]) * yin[4544];
    ws[55360] = ((ws[44192]) * yin[1536]) * yin[4736];
    ws[55392] = ((ws[44224]) * yin[1536]) * yin[4544];
    ws[55424] = ((ws[44256]) * yin[3008]) * yin[4320];
    ws[55456] = ((ws[44288]) * yin[3008]) * yin[1184];
    ws[55488] = ((ws[44320]) * yin[3008]) * yin[3456];
    ws[55520] = ((ws[44352]) * yin[3008]) * yin[4736];
    ws[55552] = ((ws[44384]) * yin[3008]) * yin[4544];
    ws[55584] = ((ws[44416]) * yin[2016]) * yin[4736];
    ws[55616] = ((ws[44448]) * yin[2016]) * yin[4736];
    ws[55648] = ((ws[44480]) * yin[2016]) * yin[4640];
    ws[55680] = ((ws[44512]) * yin[2016]) * yin[4544];
    {
      double a = -ws[53856];
      yout[0] = a;
    }
    {
      double a = 1.0 * ws[53856];
      yout[32] = a;
    }
    {
      double a = -ws[53888];
      yout[64] = a;
    }
    {
      double a = -ws[53920];
      yout[96] = a;
    }
    {
      double a = -ws[53952];
      yout[128] = a;
    }
    {
      double a = -ws[53984];
      yout[160] = a;
    }
    {
      double a = -ws[54016];
      yout[192] = a;
    }
    {
      double a = -ws[54048];
      yout[224] = a;
    }
    {
      double a = 1.0 * ws[46176];
      yout[256] = a;
    }
    {
      double a = 1.0 * ws[46176];
      yout[288] = a;
    }
    {
      double a = 0.2 * ws[48768];
      a = fma(1.0, ws[48800], a);
      yout[320] = a;
    }
    {
      double a = -ws[48864];
      yout[352] = a;
    }
    {
      double a = -ws[50240];
      yout[384] = a;
    }
    {
      double a = -ws[51552];
      yout[416] = a;
    }
    {
      double a = -ws[53120];
      yout[448] = a;
    }
    {
      double a = -ws[53312];
      yout[480] = a;
    }
    {
      double a = -ws[53344];
      yout[512] = a;
    }
    {
      double a = -ws[53376];
      yout[544] = a;
    }
    {
      double a = -ws[53504];
      yout[576] = a;
    }
    {
      double a = 1.0 * ws[53504];
      a = fma(1.0, ws[53536], a);
      yout[608] = a;
    }
    {
      double a = 1.0 * ws[53568];
      a = fma(1.0, ws[53600], a);
      yout[640] = a;
    }
    {
      double a = -ws[44832];
      a = a - ws[44864];
      yout[672] = a;
    }
    {
      double a = -ws[54080];
      a = fma(1.0, ws[54080], a);
      yout[704] = a;
    }
    {
      double a = -ws[54144];
      a = fma(1.0, ws[54144], a);
      yout[736] = a;
    }
    {
      double a = -ws[54208];
      yout[768] = a;
    }
    {
      double a = 1.0 * ws[54208];
      yout[800] = a;
    }
    {
      double a = -ws[48512];
      a = a - ws[52128];
      yout[832] = a;
    }
    {
      double a = -ws[48576];
      a = a - ws[52416];
      yout[864] = a;
    }
    {
      double a = -ws[48704];
      a = a - ws[52096];
      yout[896] = a;
    }
    {
      double a = 1.0 * ws[48704];
      a = a - ws[51584];
      a = a - ws[51616];
      yout[928] = a;
    }
    {
      double a = -ws[48768];
      a = fma(0.02, ws[48768], a);
      a = a - ws[48800];
      a = a - ws[48832];
      a = fma(0.874, ws[51680], a);
      yout[960] = a;
    }
    {
      double a = 1.0 * ws[49280];
      a = fma(1.0, ws[49536], a);
      yout[992] = a;
    }
    {
      double a = 1.0 * ws[49472];
      a = a - ws[49760];
      yout[1024] = a;
    }
    {
      double a = 0.904 * ws[49696];
      a = a - ws[49792];
      a = a - ws[53472];
      yout[1056] = a;
    }
    {
      double a = -ws[50400];
      a = a - ws[52480];
      yout[1088] = a;
    }
    {
      double a = -ws[50560];
      a = a - ws[52512];
      yout[1120] = a;
    }
    {
      double a = -ws[50592];
      a = a - ws[52544];
      yout[1152] = a;
    }
    {
      double a = 0.3 * ws[51840];
      a = a - ws[55456];
      a = fma(1.0, ws[55456], a);
      yout[1184] = a;
    }
    {
      double a = 1.0 * ws[52608];
      a = a - ws[52704];
      a = a - ws[52736];
      yout[1216] = a;
    }
    {
      double a = 1.0 * ws[53216];
      a = a - ws[53280];
      a = a - ws[53376];
      yout[1248] = a;
    }
    {
      double a = 1.0 * ws[45664];
      a = a - ws[45696];
      a = a - ws[45760];
      a = a - ws[53184];
      a = a - ws[53216];
      yout[1280] = a;
    }
    {
      double a = 1.0 * ws[53472];
      a = a - ws[53504];
      a = a - ws[53536];
      yout[1312] = a;
    }
    {
      double a = 1.0 * ws[46240];
      a = a - ws[46272];
      yout[1344] = a;
    }
    {
      double a = 0.907 * ws[53888];
      a = fma(0.925, ws[53920], a);
      a = fma(0.943, ws[53952], a);
      yout[1376] = a;
    }
    {
      double a = 0.5 * ws[53984];
      a = fma(0.5, ws[54016], a);
      a = fma(1.5, ws[54048], a);
      yout[1408] = a;
    }
    {
      double a = 1.25 * ws[54080];
      a = a - ws[54112];
      yout[1440] = a;
    }
    {
      double a = 1.25 * ws[54144];
      a = a - ws[54176];
      yout[1472] = a;
    }
    {
      double a = 0.0023 * ws[54240];
      a = a - ws[54368];
      yout[1504] = a;
    }
    {
      double a = -ws[55360];
      a = a - ws[55392];
      yout[1536] = a;
    }
    {
      double a = 0.5 * ws[55424];
      a = fma(0.5, ws[55520], a);
      yout[1568] = a;
    }
    {
      double a = 0.25 * ws[55616];
      a = fma(0.14, ws[55680], a);
      yout[1600] = a;
    }
    {
      double a = 0.1 * ws[49344];
      a = a - ws[49952];
      a = fma(0.104, ws[49952], a);
      yout[1632] = a;
    }
    {
      double a = 0.88 * ws[49376];
      a = a - ws[49696];
      yout[1664] = a;
    }
    {
      double a = 1.0 * ws[46048];
      a = a - ws[46080];
      a = a - ws[46144];
      yout[1696] = a;
    }
    {
      double a = 1.0 * ws[47744];
      a = a - ws[47776];
      a = a - ws[47808];
      a = a - ws[47840];
      yout[1728] = a;
    }
    {
      double a = 0.732 * ws[50752];
      a = a - ws[51232];
      a = a - ws[51264];
      yout[1760] = a;
    }
    {
      double a = 1.0 * ws[51328];
      a = a - ws[51360];
      a = a - ws[51488];
      yout[1792] = a;
    }
    {
      double a = 1.0 * ws[51904];
      a = fma(1.0, ws[52704], a);
      a = fma(1.0, ws[52736], a);
      yout[1824] = a;
    }
    {
      double a = -ws[52960];
      a = a - ws[52992];
      a = a - ws[53024];
      yout[1856] = a;
    }
    {
      double a = 1.0 * ws[52960];
      a = fma(1.0, ws[52992], a);
      a = fma(1.0, ws[53024], a);
      yout[1888] = a;
    }
    {
      double a = 1.0 * ws[53184];
      a = a - ws[53248];
      a = a - ws[53312];
      a = a - ws[53344];
      yout[1920] = a;
    }
    {
      double a = 1.0 * ws[46496];
      a = a - ws[46528];
      a = a - ws[51520];
      yout[1952] = a;
    }
    {
      double a = 1.0 * ws[48736];
      a = a - ws[51648];
      a = a - ws[51680];
      a = fma(1.0, ws[52064], a);
      yout[1984] = a;
    }
    {
      double a = -ws[55584];
      a = a - ws[55616];
      a = a - ws[55648];
      a = a - ws[55680];
      yout[2016] = a;
    }
    {
      double a = -ws[49984];
      a = a - ws[50016];
      a = a - ws[50048];
      a = a - ws[50080];
      yout[2048] = a;
    }
    {
      double a = 1.0 * ws[49984];
      a = fma(1.0, ws[50016], a);
      a = fma(1.0, ws[50048], a);
      a = fma(1.0, ws[50112], a);
      a = fma(1.0, ws[50144], a);
      a = fma(1.0, ws[50176], a);
      yout[2080] = a;
    }
    {
      double a = -ws[50112];
      a = a - ws[50144];
      a = a - ws[50176];
      a = a - ws[50208];
      yout[2112] = a;
    }
    {
      double a = 1.0 * ws[50240];
      a = a - ws[52896];
      a = a - ws[52928];
      yout[2144] = a;
    }
    {
      double a = 1.0 * ws[50816];
      a = a - ws[50880];
      a = a - ws[50912];
      yout[2176] = a;
    }
    {
      double a = -ws[46176];
      a = fma(1.0, ws[55584], a);
      a = fma(0.75, ws[55616], a);
      a = fma(1.0, ws[55648], a);
      a = fma(0.86, ws[55680], a);
      yout[2208] = a;
    }
    {
      double a = 0.14 * ws[52800];
      a = fma(0.193, ws[52864], a);
      a = fma(0.146, ws[52928], a);
      a = fma(0.473, ws[53088], a);
      yout[2240] = a;
    }
    {
      double a = 0.9 * ws[46816];
      a = a - ws[47296];
      a = fma(0.5, ws[47840], a);
      yout[2272] = a;
    }
    {
      double a = 0.0026 * ws[54240];
      a = fma(0.0035, ws[54272], a);
      a = fma(0.0005, ws[54304], a);
      a = a - ws[54336];
      a = fma(0.1043, ws[54336], a);
      yout[2304] = a;
    }
    {
      double a = -ws[54560];
      a = a - ws[54592];
      a = a - ws[54624];
      a = a - ws[54720];
      yout[2336] = a;
    }
    {
      double a = -ws[54752];
      a = a - ws[54784];
      a = a - ws[54816];
      a = a - ws[54880];
      yout[2368] = a;
    }
    {
      double a = -ws[54912];
      a = a - ws[54944];
      a = a - ws[54976];
      a = a - ws[55008];
      yout[2400] = a;
    }
    {
      double a = -ws[55040];
      a = a - ws[55072];
      a = a - ws[55104];
      a = a - ws[55168];
      yout[2432] = a;
    }
    {
      double a = 1.0 * ws[45792];
      a = fma(2.0, ws[45824], a);
      a = a - ws[45856];
      a = a - ws[45856];
      a = a - ws[45920];
      a = fma(0.5, ws[53408], a);
      yout[2464] = a;
    }
    {
      double a = 1.0 * ws[50560];
      a = fma(1.0, ws[52512], a);
      a = a - ws[52832];
      a = a - ws[52864];
      yout[2496] = a;
    }
    {
      double a = -ws[49280];
      a = a - ws[49312];
      a = a - ws[49504];
      a = a - ws[49536];
      a = a - ws[52256];
      yout[2528] = a;
    }
    {
      double a = 1.0 * ws[50592];
      a = fma(1.0, ws[52544], a);
      a = a - ws[53056];
      a = a - ws[53088];
      yout[2560] = a;
    }
    {
      double a = 1.0 * ws[53312];
      a = fma(1.0, ws[53344], a);
      a = fma(1.0, ws[53376], a);
      yout[2592] = a;
    }
    {
      double a = 0.051 * ws[52768];
      a = fma(0.023, ws[52832], a);
      a = fma(0.225, ws[53056], a);
      a = fma(0.052, ws[53120], a);
      yout[2624] = a;
    }
    {
      double a = -ws[48896];
      a = a - ws[48928];
      a = a - ws[48960];
      a = a - ws[48992];
      a = a - ws[52160];
      yout[2656] = a;
    }
    {
      double a = 0.37 * ws[46336];
      a = fma(0.37, ws[46592], a);
      a = a - ws[47552];
      a = fma(0.37, ws[51392], a);
      yout[2688] = a;
    }
    {
      double a = 0.315 * ws[46880];
      a = a - ws[48544];
      a = a - ws[52384];
      yout[2720] = a;
    }
    {
      double a = -ws[54240];
      a = fma(0.4857, ws[54240], a);
      a = fma(0.3003, ws[54272], a);
      a = fma(0.3856, ws[54304], a);
      a = fma(0.2181, ws[54336], a);
      a = fma(0.2412, ws[54368], a);
      yout[2752] = a;
    }
    {
      double a = 0.0062 * ws[54240];
      a = a - ws[54272];
      a = fma(0.2862, ws[54272], a);
      a = fma(0.095, ws[54304], a);
      a = fma(0.3063, ws[54336], a);
      a = fma(0.2089, ws[54368], a);
      yout[2784] = a;
    }
    {
      double a = 0.0025 * ws[54240];
      a = fma(0.0041, ws[54272], a);
      a = a - ws[54304];
      a = fma(0.1373, ws[54304], a);
      a = fma(0.0153, ws[54336], a);
      a = fma(0.3, ws[54368], a);
      yout[2816] = a;
    }
    {
      double a = 1.0 * ws[50080];
      a = a - ws[53632];
      a = a - ws[53664];
      a = a - ws[53696];
      a = a - ws[53728];
      yout[2848] = a;
    }
    {
      double a = 1.0 * ws[46944];
      a = fma(1.0, ws[47072], a);
      a = fma(1.0, ws[47200], a);
      a = a - ws[47360];
      yout[2880] = a;
    }
    {
      double a = 0.0123 * ws[54400];
      a = fma(0.0139, ws[54432], a);
      a = a - ws[54464];
      a = fma(0.2607, ws[54464], a);
      a = fma(0.0491, ws[54496], a);
      a = fma(0.064, ws[54528], a);
      yout[2912] = a;
    }
    {
      double a = 1.0 * ws[50400];
      a = fma(1.0, ws[52480], a);
      a = a - ws[52768];
      a = a - ws[52800];
      yout[2944] = a;
    }
    {
      double a = 0.58 * ws[54912];
      a = fma(0.52, ws[54944], a);
      a = fma(0.045, ws[54976], a);
      a = fma(0.58, ws[55008], a);
      a = a - ws[55200];
      a = a - ws[55232];
      a = a - ws[55264];
      a = a - ws[55328];
      yout[2976] = a;
    }
    {
      double a = -ws[55424];
      a = a - ws[55456];
      a = a - ws[55488];
      a = a - ws[55520];
      a = a - ws[55552];
      a = fma(0.5, ws[55552], a);
      yout[3008] = a;
    }
    {
      double a = 0.5 * ws[55424];
      a = fma(1.0, ws[55456], a);
      a = fma(1.0, ws[55488], a);
      a = fma(0.5, ws[55520], a);
      a = fma(0.5, ws[55552], a);
      yout[3040] = a;
    }
    {
      double a = 0.047 * ws[52768];
      a = fma(0.06, ws[52832], a);
      a = fma(0.392, ws[52896], a);
      a = fma(0.191, ws[53056], a);
      a = fma(0.081, ws[53120], a);
      yout[3072] = a;
    }
    {
      double a = 0.352 * ws[50240];
      a = a - ws[50272];
      a = a - ws[50304];
      a = a - ws[50336];
      a = a - ws[50368];
      yout[3104] = a;
    }
    {
      double a = -ws[49152];
      a = a - ws[49184];
      a = a - ws[49216];
      a = a - ws[49248];
      a = fma(0.029, ws[49696], a);
      a = a - ws[52224];
      yout[3136] = a;
    }
    {
      double a = 0.0019 * ws[54240];
      a = fma(0.1239, ws[54400], a);
      a = fma(0.1027, ws[54432], a);
      a = fma(0.0702, ws[54464], a);
      a = a - ws[54496];
      a = fma(0.2577, ws[54496], a);
      a = fma(0.0385, ws[54528], a);
      yout[3168] = a;
    }
    {
      double a = 0.0023 * ws[54240];
      a = fma(0.1831, ws[54400], a);
      a = fma(0.2045, ws[54432], a);
      a = fma(0.1116, ws[54464], a);
      a = fma(0.0739, ws[54496], a);
      a = a - ws[54528];
      a = fma(0.2667, ws[54528], a);
      yout[3200] = a;
    }
    {
      double a = -ws[51968];
      a = fma(1.0, ws[52160], a);
      a = fma(1.0, ws[52192], a);
      a = fma(0.7, ws[52224], a);
      a = fma(1.0, ws[52256], a);
      yout[3232] = a;
    }
    {
      double a = 0.016 * ws[52768];
      a = fma(0.015, ws[52832], a);
      a = fma(0.034, ws[52896], a);
      a = fma(0.028, ws[53056], a);
      a = fma(0.006, ws[53120], a);
      yout[3264] = a;
    }
    {
      double a = 1.0 * ws[49792];
      a = a - ws[49824];
      a = a - ws[49856];
      a = a - ws[49888];
      a = a - ws[49920];
      yout[3296] = a;
    }
    {
      double a = 0.2 * ws[50752];
      a = fma(0.3, ws[50784], a);
      a = a - ws[50816];
      a = a - ws[50848];
      a = fma(0.5, ws[50880], a);
      a = fma(0.5, ws[50912], a);
      a = fma(0.5, ws[51232], a);
      a = fma(1.0, ws[51264], a);
      yout[3328] = a;
    }
    {
      double a = 0.688 * ws[53632];
      a = fma(1.0, ws[53664], a);
      a = fma(0.422, ws[53696], a);
      a = fma(0.711, ws[53728], a);
      a = a - ws[53760];
      a = fma(0.37, ws[53760], a);
      a = a - ws[53792];
      a = fma(0.24, ws[53792], a);
      yout[3360] = a;
    }
    {
      double a = -ws[48672];
      a = fma(0.42, ws[48768], a);
      a = fma(0.137, ws[49568], a);
      a = fma(0.17, ws[49600], a);
      a = fma(0.732, ws[51616], a);
      a = fma(1.0, ws[52096], a);
      yout[3392] = a;
    }
    {
      double a = 1.0 * ws[49280];
      a = a - ws[49344];
      a = a - ws[49376];
      a = a - ws[49408];
      a = a - ws[49440];
      a = a - ws[49472];
      a = fma(0.067, ws[49696], a);
      yout[3424] = a;
    }
    {
      double a = 1.0 * ws[45056];
      a = fma(1.0, ws[45120], a);
      a = fma(1.0, ws[45152], a);
      a = a - ws[45216];
      a = a - ws[45248];
      a = fma(0.04, ws[49088], a);
      a = fma(0.08, ws[49216], a);
      a = a - ws[55488];
      a = fma(1.0, ws[55488], a);
      yout[3456] = a;
    }
    {
      double a = 0.65 * ws[50400];
      a = a - ws[50432];
      a = a - ws[50464];
      a = a - ws[50496];
      a = a - ws[50528];
      a = fma(0.65, ws[52480], a);
      yout[3488] = a;
    }
    {
      double a = 1.0 * ws[51808];
      a = a - ws[51840];
      a = a - ws[51840];
      a = a - ws[51872];
      a = a - ws[51904];
      a = a - ws[51936];
      a = a - ws[52608];
      a = fma(0.55, ws[55680], a);
      yout[3520] = a;
    }
    {
      double a = -ws[49024];
      a = a - ws[49056];
      a = a - ws[49088];
      a = a - ws[49120];
      a = fma(0.098, ws[49952], a);
      a = a - ws[52192];
      a = fma(0.3, ws[52224], a);
      yout[3552] = a;
    }
    {
      double a = 0.544 * ws[50560];
      a = fma(0.544, ws[50592], a);
      a = a - ws[50624];
      a = a - ws[50656];
      a = a - ws[50688];
      a = a - ws[50720];
      a = fma(0.544, ws[52512], a);
      a = fma(0.544, ws[52544], a);
      yout[3584] = a;
    }
    {
      double a = 0.53 * ws[50240];
      a = fma(0.18, ws[50400], a);
      a = fma(0.155, ws[50560], a);
      a = fma(0.155, ws[50592], a);
      a = a - ws[50752];
      a = a - ws[50784];
      a = fma(1.0, ws[50848], a);
      a = fma(0.18, ws[52480], a);
      a = fma(0.155, ws[52512], a);
      a = fma(0.155, ws[52544], a);
      yout[3616] = a;
    }
    {
      double a = 0.5 * ws[47168];
      a = a - ws[47424];
      a = fma(1.0, ws[48832], a);
      a = fma(0.5, ws[48992], a);
      a = fma(0.5, ws[49120], a);
      a = fma(0.5, ws[49248], a);
      yout[3648] = a;
    }
    {
      double a = 0.2944 * ws[54240];
      a = fma(0.2239, ws[54272], a);
      a = fma(0.2051, ws[54304], a);
      a = fma(0.1893, ws[54336], a);
      a = fma(0.2028, ws[54368], a);
      a = a - ws[54400];
      a = fma(0.6664, ws[54400], a);
      a = fma(0.2858, ws[54432], a);
      a = fma(0.3303, ws[54464], a);
      a = fma(0.3444, ws[54496], a);
      a = fma(0.3886, ws[54528], a);
      yout[3680] = a;
    }
    {
      double a = 0.2021 * ws[54240];
      a = fma(0.182, ws[54272], a);
      a = fma(0.1764, ws[54304], a);
      a = fma(0.1668, ws[54336], a);
      a = fma(0.0471, ws[54368], a);
      a = fma(0.0143, ws[54400], a);
      a = a - ws[54432];
      a = fma(0.3931, ws[54432], a);
      a = fma(0.2272, ws[54464], a);
      a = fma(0.2749, ws[54496], a);
      a = fma(0.2421, ws[54528], a);
      yout[3712] = a;
    }
    {
      double a = 0.457 * ws[49568];
      a = fma(0.48, ws[50784], a);
      a = fma(0.6, ws[51136], a);
      a = fma(1.0, ws[51200], a);
      a = a - ws[51296];
      a = a - ws[51328];
      a = fma(1.0, ws[51360], a);
      a = a - ws[51392];
      a = a - ws[51424];
      a = a - ws[51456];
      yout[3744] = a;
    }
    {
      double a = -ws[47488];
      a = fma(1.0, ws[47808], a);
      a = fma(0.5, ws[47840], a);
      a = fma(0.3, ws[48864], a);
      a = fma(0.42, ws[48960], a);
      a = fma(0.09, ws[49088], a);
      a = fma(0.15, ws[49600], a);
      a = fma(0.074, ws[49824], a);
      a = fma(0.185, ws[49952], a);
      yout[3776] = a;
    }
    {
      double a = 0.2 * ws[50432];
      a = fma(0.23, ws[50464], a);
      a = fma(0.23, ws[50528], a);
      a = fma(0.244, ws[50560], a);
      a = fma(0.244, ws[50592], a);
      a = fma(0.56, ws[50624], a);
      a = fma(0.65, ws[50688], a);
      a = fma(0.65, ws[50720], a);
      a = a - ws[51008];
      a = a - ws[51040];
      a = a - ws[51072];
      a = fma(0.244, ws[52512], a);
      a = fma(0.244, ws[52544], a);
      yout[3808] = a;
    }
    {
      double a = -ws[48128];
      a = a - ws[48192];
      a = fma(0.011, ws[48576], a);
      a = fma(0.22, ws[48928], a);
      a = fma(0.269, ws[49568], a);
      a = fma(0.113, ws[49632], a);
      a = fma(0.275, ws[49824], a);
      a = fma(0.275, ws[49856], a);
      a = fma(0.22, ws[49888], a);
      a = fma(0.275, ws[49920], a);
      a = fma(0.331, ws[49952], a);
      yout[3840] = a;
    }
    {
      double a = 0.75 * ws[49312];
      a = fma(0.9, ws[49344], a);
      a = fma(0.12, ws[49376], a);
      a = fma(1.0, ws[49408], a);
      a = fma(1.0, ws[49440], a);
      a = fma(0.65, ws[49504], a);
      a = fma(0.35, ws[49536], a);
      a = a - ws[49568];
      a = a - ws[49600];
      a = a - ws[49632];
      a = fma(1.0, ws[49760], a);
      a = fma(1.0, ws[52256], a);
      yout[3872] = a;
    }
    {
      double a = 0.13 * ws[46336];
      a = fma(0.13, ws[46592], a);
      a = fma(0.1, ws[46848], a);
      a = fma(0.2, ws[46976], a);
      a = fma(0.2, ws[47104], a);
      a = fma(0.2, ws[47232], a);
      a = a - ws[47520];
      a = fma(0.13, ws[49088], a);
      a = fma(0.08, ws[49216], a);
      a = fma(0.2, ws[49408], a);
      a = fma(0.2, ws[49888], a);
      a = fma(0.13, ws[51392], a);
      a = fma(0.2, ws[51456], a);
      yout[3904] = a;
    }
    {
      double a = 0.118 * ws[50240];
      a = fma(0.918, ws[50272], a);
      a = fma(1.0, ws[50304], a);
      a = fma(1.0, ws[50368], a);
      a = fma(0.1, ws[50400], a);
      a = fma(0.66, ws[50432], a);
      a = fma(0.77, ws[50464], a);
      a = fma(0.77, ws[50528], a);
      a = fma(0.3, ws[50624], a);
      a = fma(0.35, ws[50688], a);
      a = fma(0.35, ws[50720], a);
      a = fma(0.025, ws[50752], a);
      a = fma(0.25, ws[51072], a);
      a = a - ws[51136];
      a = a - ws[51168];
      a = a - ws[51200];
      a = fma(0.1, ws[52480], a);
      yout[3936] = a;
    }
    {
      double a = 1.0 * ws[52032];
      a = fma(1.0, ws[52064], a);
      a = fma(1.0, ws[52096], a);
      a = fma(1.0, ws[52128], a);
      a = fma(0.3, ws[52224], a);
      a = fma(1.0, ws[52288], a);
      a = fma(1.0, ws[52320], a);
      a = fma(1.0, ws[52352], a);
      a = fma(1.0, ws[52384], a);
      a = fma(1.0, ws[52416], a);
      a = a - ws[52448];
      a = fma(1.0, ws[52480], a);
      a = fma(1.0, ws[52512], a);
      a = fma(1.0, ws[52544], a);
      a = fma(0.45, ws[55680], a);
      yout[3968] = a;
    }
    {
      double a = -ws[48352];
      a = a - ws[48384];
      a = fma(0.075, ws[49088], a);
      a = fma(0.06, ws[49216], a);
      a = fma(0.115, ws[49568], a);
      a = fma(0.531, ws[49600], a);
      a = fma(0.113, ws[49632], a);
      a = fma(0.275, ws[49824], a);
      a = fma(0.275, ws[49856], a);
      a = fma(0.22, ws[49888], a);
      a = fma(0.275, ws[49920], a);
      a = fma(0.443, ws[50432], a);
      a = fma(0.52, ws[50464], a);
      a = fma(0.52, ws[50528], a);
      a = fma(0.675, ws[50624], a);
      a = fma(0.77, ws[50688], a);
      a = fma(0.77, ws[50720], a);
      a = fma(0.24, ws[50784], a);
      a = fma(1.0, ws[51008], a);
      a = fma(1.2, ws[51040], a);
      a = fma(0.25, ws[51072], a);
      a = fma(0.24, ws[51168], a);
      a = a - ws[53600];
      yout[4000] = a;
    }
    {
      double a = 0.5 * ws[47168];
      a = fma(1.0, ws[47424], a);
      a = fma(0.65, ws[49536], a);
      a = fma(0.142, ws[49632], a);
      a = fma(0.266, ws[49952], a);
      a = fma(0.53, ws[50080], a);
      a = fma(0.53, ws[50208], a);
      a = fma(0.082, ws[50272], a);
      a = fma(0.14, ws[50432], a);
      a = fma(0.14, ws[50624], a);
      a = fma(1.0, ws[50880], a);
      a = fma(1.0, ws[50912], a);
      a = fma(0.5, ws[51072], a);
      a = fma(0.5, ws[51488], a);
      a = a - ws[53152];
      yout[4032] = a;
    }
    {
      double a = -ws[48000];
      a = a - ws[48032];
      a = a - ws[48064];
      a = fma(0.37, ws[48768], a);
      a = fma(0.3, ws[49024], a);
      a = fma(0.488, ws[49056], a);
      a = fma(0.27, ws[49088], a);
      a = fma(0.375, ws[49120], a);
      a = fma(0.66, ws[49152], a);
      a = fma(0.7, ws[49184], a);
      a = fma(0.442, ws[49216], a);
      a = fma(0.625, ws[49248], a);
      a = fma(0.15, ws[49504], a);
      a = fma(0.029, ws[49696], a);
      a = fma(0.078, ws[49952], a);
      a = fma(0.15, ws[49984], a);
      a = fma(0.47, ws[50016], a);
      a = fma(0.21, ws[50048], a);
      a = fma(0.47, ws[50080], a);
      a = fma(0.15, ws[50112], a);
      a = fma(0.47, ws[50144], a);
      a = fma(0.21, ws[50176], a);
      a = fma(0.47, ws[50208], a);
      a = fma(1.0, ws[51424], a);
      a = fma(0.8, ws[51456], a);
      a = fma(0.268, ws[51616], a);
      a = fma(0.126, ws[51680], a);
      a = fma(0.67, ws[52192], a);
      a = fma(0.55, ws[52224], a);
      a = a - ws[52352];
      yout[4064] = a;
    }
    {
      double a = -ws[46432];
      a = a - ws[46464];
      a = a - ws[46496];
      a = fma(1.0, ws[46528], a);
      a = a - ws[46592];
      a = a - ws[46624];
      a = a - ws[46656];
      a = a - ws[46656];
      a = fma(1.0, ws[48000], a);
      a = fma(1.0, ws[48032], a);
      a = fma(1.0, ws[48064], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.2, ws[49504], a);
      a = fma(0.717, ws[49632], a);
      a = fma(0.39, ws[50048], a);
      a = fma(0.39, ws[50176], a);
      a = fma(0.2, ws[51296], a);
      a = fma(1.0, ws[52352], a);
      yout[4096] = a;
    }
    {
      double a = 1.0 * ws[46432];
      a = fma(1.0, ws[46464], a);
      a = a - ws[47872];
      a = a - ws[47904];
      a = a - ws[47936];
      a = fma(0.991, ws[48512], a);
      a = fma(0.95, ws[48576], a);
      a = fma(0.74, ws[48768], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.488, ws[49056], a);
      a = fma(0.295, ws[49088], a);
      a = fma(0.25, ws[49120], a);
      a = fma(1.24, ws[49152], a);
      a = fma(1.3, ws[49184], a);
      a = fma(0.732, ws[49216], a);
      a = fma(0.5, ws[49248], a);
      a = fma(0.04, ws[49600], a);
      a = fma(0.1, ws[51040], a);
      a = fma(0.02, ws[51168], a);
      a = fma(1.0, ws[51520], a);
      a = fma(0.991, ws[52128], a);
      a = fma(0.33, ws[52192], a);
      a = fma(0.45, ws[52224], a);
      a = a - ws[52320];
      a = fma(1.0, ws[52416], a);
      yout[4128] = a;
    }
    {
      double a = -ws[44576];
      a = a - ws[44640];
      a = a - ws[44672];
      a = a - ws[44704];
      a = a - ws[44736];
      a = fma(1.0, ws[44832], a);
      a = a - ws[44960];
      a = a - ws[44992];
      a = fma(1.0, ws[45024], a);
      a = a - ws[45248];
      a = a - ws[45504];
      a = a - ws[47680];
      a = a - ws[47872];
      a = a - ws[48000];
      a = a - ws[48896];
      a = a - ws[49024];
      a = a - ws[49152];
      a = a - ws[49312];
      a = a - ws[49984];
      a = a - ws[50112];
      a = a - ws[54624];
      a = fma(1.0, ws[54624], a);
      a = a - ws[54816];
      a = fma(1.0, ws[54816], a);
      yout[4160] = a;
    }
    {
      double a = 2.0 * ws[45760];
      a = fma(1.0, ws[45952], a);
      a = a - ws[45984];
      a = fma(1.0, ws[47712], a);
      a = fma(1.0, ws[47936], a);
      a = fma(1.0, ws[48064], a);
      a = fma(1.0, ws[48192], a);
      a = fma(1.0, ws[48288], a);
      a = fma(1.0, ws[48352], a);
      a = fma(0.717, ws[49632], a);
      a = fma(1.0, ws[49760], a);
      a = fma(1.0, ws[50784], a);
      a = fma(1.0, ws[50912], a);
      a = fma(1.0, ws[51200], a);
      a = fma(1.0, ws[51264], a);
      a = fma(1.0, ws[51712], a);
      a = fma(1.0, ws[52704], a);
      a = fma(1.0, ws[52736], a);
      a = fma(1.0, ws[53152], a);
      a = fma(1.0, ws[53184], a);
      a = fma(1.0, ws[53216], a);
      a = fma(1.0, ws[53248], a);
      a = fma(1.0, ws[53280], a);
      a = fma(0.5, ws[53408], a);
      a = fma(1.0, ws[55648], a);
      yout[4192] = a;
    }
    {
      double a = -ws[48736];
      a = fma(-2.7, ws[48768], a);
      a = fma(0.2, ws[49024], a);
      a = fma(-0.73, ws[49056], a);
      a = fma(-0.79, ws[49088], a);
      a = fma(-1.0, ws[49120], a);
      a = fma(0.1, ws[49152], a);
      a = fma(0.29, ws[49216], a);
      a = fma(1.0, ws[49248], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.35, ws[49504], a);
      a = fma(0.117, ws[49568], a);
      a = fma(0.717, ws[49632], a);
      a = fma(2.175, ws[49824], a);
      a = fma(2.175, ws[49856], a);
      a = fma(1.74, ws[49888], a);
      a = fma(2.175, ws[49920], a);
      a = fma(2.7, ws[49952], a);
      a = fma(5.12, ws[49984], a);
      a = fma(1.66, ws[50016], a);
      a = fma(7.0, ws[50048], a);
      a = fma(5.12, ws[50112], a);
      a = fma(1.66, ws[50144], a);
      a = fma(7.0, ws[50176], a);
      a = fma(0.268, ws[51616], a);
      a = fma(-0.126, ws[51680], a);
      a = a - ws[52064];
      a = fma(-1.0, ws[52192], a);
      a = fma(0.3, ws[52224], a);
      yout[4224] = a;
    }
    {
      double a = 0.2 * ws[48128];
      a = a - ws[48224];
      a = a - ws[48288];
      a = fma(0.7, ws[48864], a);
      a = fma(0.075, ws[49088], a);
      a = fma(0.24, ws[49216], a);
      a = fma(0.17, ws[49600], a);
      a = fma(0.275, ws[49824], a);
      a = fma(0.275, ws[49856], a);
      a = fma(0.22, ws[49888], a);
      a = fma(0.275, ws[49920], a);
      a = fma(0.918, ws[50272], a);
      a = fma(1.0, ws[50304], a);
      a = fma(1.0, ws[50368], a);
      a = fma(0.417, ws[50432], a);
      a = fma(0.48, ws[50464], a);
      a = fma(0.48, ws[50528], a);
      a = fma(0.221, ws[50624], a);
      a = fma(0.26, ws[50688], a);
      a = fma(0.26, ws[50720], a);
      a = fma(0.025, ws[50752], a);
      a = fma(0.24, ws[50784], a);
      a = fma(0.4, ws[51008], a);
      a = fma(0.4, ws[51136], a);
      a = fma(1.4, ws[51168], a);
      a = fma(0.5, ws[51296], a);
      a = fma(0.5, ws[51488], a);
      a = a - ws[53568];
      yout[4256] = a;
    }
    {
      double a = -ws[47168];
      a = a - ws[47200];
      a = a - ws[47232];
      a = a - ws[47264];
      a = fma(0.06, ws[47360], a);
      a = fma(0.009, ws[48512], a);
      a = fma(0.04, ws[48768], a);
      a = fma(0.01, ws[49024], a);
      a = fma(0.024, ws[49056], a);
      a = fma(0.04, ws[49120], a);
      a = fma(0.04, ws[49248], a);
      a = fma(0.03, ws[49536], a);
      a = fma(0.022, ws[49568], a);
      a = fma(0.25, ws[50016], a);
      a = fma(0.18, ws[50048], a);
      a = fma(0.25, ws[50080], a);
      a = fma(0.25, ws[50144], a);
      a = fma(0.18, ws[50176], a);
      a = fma(0.25, ws[50208], a);
      a = fma(0.02, ws[50752], a);
      a = fma(0.1, ws[50784], a);
      a = fma(0.1, ws[51072], a);
      a = fma(1.0, ws[51584], a);
      a = fma(1.0, ws[51648], a);
      a = fma(0.03, ws[52096], a);
      a = fma(0.009, ws[52128], a);
      a = fma(0.04, ws[52256], a);
      yout[4288] = a;
    }
    {
      double a = 1.0 * ws[44576];
      a = a - ws[44608];
      a = a - ws[44736];
      a = a - ws[44896];
      a = a - ws[44928];
      a = a - ws[45344];
      a = a - ws[45600];
      a = fma(0.13, ws[46336], a);
      a = fma(0.13, ws[46592], a);
      a = a - ws[48960];
      a = a - ws[49088];
      a = a - ws[49216];
      a = a - ws[49504];
      a = a - ws[49600];
      a = a - ws[50048];
      a = a - ws[50176];
      a = a - ws[51040];
      a = a - ws[51168];
      a = fma(0.13, ws[51392], a);
      a = a - ws[51808];
      a = a - ws[52960];
      a = fma(1.0, ws[52960], a);
      a = a - ws[54944];
      a = fma(1.0, ws[54944], a);
      a = a - ws[55072];
      a = fma(1.0, ws[55072], a);
      a = a - ws[55232];
      a = fma(1.0, ws[55232], a);
      a = a - ws[55424];
      a = fma(1.0, ws[55424], a);
      yout[4320] = a;
    }
    {
      double a = -ws[47040];
      a = a - ws[47072];
      a = a - ws[47104];
      a = a - ws[47136];
      a = fma(0.2, ws[48224], a);
      a = fma(0.5, ws[48288], a);
      a = fma(1.0, ws[48352], a);
      a = fma(1.0, ws[48672], a);
      a = fma(0.5, ws[48992], a);
      a = fma(0.195, ws[49056], a);
      a = fma(0.48, ws[49120], a);
      a = fma(0.48, ws[49248], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.2, ws[49504], a);
      a = fma(0.33, ws[49536], a);
      a = fma(0.521, ws[49568], a);
      a = fma(0.142, ws[49632], a);
      a = fma(0.63, ws[49952], a);
      a = fma(0.5, ws[50016], a);
      a = fma(0.69, ws[50048], a);
      a = fma(0.75, ws[50080], a);
      a = fma(0.5, ws[50144], a);
      a = fma(0.69, ws[50176], a);
      a = fma(0.75, ws[50208], a);
      a = fma(0.48, ws[50784], a);
      a = fma(0.45, ws[51072], a);
      a = fma(1.0, ws[51424], a);
      a = fma(0.874, ws[51680], a);
      a = fma(2.0, ws[52160], a);
      a = fma(2.0, ws[52192], a);
      a = fma(1.7, ws[52224], a);
      yout[4352] = a;
    }
    {
      double a = -ws[44608];
      a = a - ws[44640];
      a = fma(1.0, ws[44672], a);
      a = a - ws[45280];
      a = a - ws[45280];
      a = a - ws[45312];
      a = a - ws[45440];
      a = fma(1.0, ws[45472], a);
      a = a - ws[45792];
      a = a - ws[45824];
      a = fma(1.0, ws[45856], a);
      a = a - ws[46208];
      a = a - ws[46464];
      a = a - ws[46688];
      a = fma(1.0, ws[46688], a);
      a = a - ws[46784];
      a = a - ws[46912];
      a = a - ws[47040];
      a = a - ws[47168];
      a = a - ws[47808];
      a = a - ws[49344];
      a = a - ws[49856];
      a = a - ws[50272];
      a = a - ws[50432];
      a = a - ws[50624];
      a = a - ws[51296];
      a = a - ws[51872];
      a = a - ws[52768];
      a = fma(1.0, ws[52768], a);
      a = a - ws[52832];
      a = fma(1.0, ws[52832], a);
      a = a - ws[52896];
      a = fma(1.0, ws[52896], a);
      a = a - ws[53056];
      a = fma(1.0, ws[53056], a);
      a = a - ws[53632];
      a = fma(1.0, ws[53632], a);
      yout[4384] = a;
    }
    {
      double a = 1.0 * ws[46208];
      a = fma(0.5, ws[46336], a);
      a = fma(1.0, ws[46368], a);
      a = fma(2.0, ws[46400], a);
      a = fma(1.0, ws[46432], a);
      a = fma(0.5, ws[46592], a);
      a = fma(1.0, ws[46624], a);
      a = fma(2.0, ws[46656], a);
      a = a - ws[46784];
      a = a - ws[46816];
      a = a - ws[46848];
      a = fma(0.9, ws[46848], a);
      a = a - ws[46880];
      a = fma(0.8, ws[46976], a);
      a = fma(0.8, ws[47104], a);
      a = fma(0.8, ws[47232], a);
      a = fma(0.6, ws[47296], a);
      a = fma(1.0, ws[47520], a);
      a = fma(1.0, ws[48480], a);
      a = fma(0.8, ws[49408], a);
      a = fma(0.115, ws[49568], a);
      a = fma(0.8, ws[49888], a);
      a = fma(1.0, ws[50304], a);
      a = fma(1.0, ws[50464], a);
      a = fma(1.0, ws[50688], a);
      a = fma(0.5, ws[51392], a);
      a = fma(1.0, ws[51424], a);
      a = fma(1.0, ws[51552], a);
      a = a - ws[51936];
      a = fma(1.0, ws[52032], a);
      a = fma(1.0, ws[55584], a);
      a = fma(1.0, ws[55616], a);
      a = fma(1.0, ws[55648], a);
      a = fma(1.0, ws[55680], a);
      yout[4416] = a;
    }
    {
      double a = -ws[46208];
      a = a - ws[46240];
      a = fma(1.0, ws[46272], a);
      a = a - ws[46336];
      a = a - ws[46368];
      a = a - ws[46400];
      a = a - ws[46400];
      a = a - ws[46432];
      a = a - ws[46848];
      a = a - ws[46976];
      a = a - ws[47104];
      a = a - ws[47232];
      a = fma(1.0, ws[47552], a);
      a = fma(1.0, ws[47872], a);
      a = fma(1.0, ws[47904], a);
      a = fma(1.0, ws[47936], a);
      a = fma(0.8, ws[48128], a);
      a = fma(1.0, ws[48192], a);
      a = fma(1.0, ws[48352], a);
      a = fma(1.0, ws[48384], a);
      a = fma(1.0, ws[48672], a);
      a = a - ws[49408];
      a = fma(0.269, ws[49568], a);
      a = fma(0.143, ws[49600], a);
      a = a - ws[49888];
      a = a - ws[50304];
      a = a - ws[50464];
      a = a - ws[50688];
      a = fma(0.6, ws[51040], a);
      a = fma(0.12, ws[51168], a);
      a = a - ws[51424];
      a = fma(1.0, ws[52320], a);
      yout[4448] = a;
    }
    {
      double a = 1.0 * ws[47584];
      a = fma(1.0, ws[47680], a);
      a = fma(1.0, ws[47712], a);
      a = fma(1.8, ws[48224], a);
      a = fma(1.5, ws[48288], a);
      a = fma(1.0, ws[48384], a);
      a = a - ws[48448];
      a = fma(0.3, ws[48864], a);
      a = fma(1.0, ws[48896], a);
      a = fma(0.35, ws[48960], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.378, ws[49088], a);
      a = fma(0.1, ws[49152], a);
      a = fma(0.245, ws[49216], a);
      a = fma(0.066, ws[49504], a);
      a = fma(0.137, ws[49568], a);
      a = fma(0.543, ws[49600], a);
      a = fma(0.251, ws[49824], a);
      a = fma(0.251, ws[49856], a);
      a = fma(0.2, ws[49888], a);
      a = fma(0.251, ws[49920], a);
      a = fma(0.001, ws[50048], a);
      a = fma(0.001, ws[50176], a);
      a = fma(0.5, ws[51040], a);
      a = fma(1.98, ws[51168], a);
      a = fma(0.5, ws[51296], a);
      a = fma(1.0, ws[51488], a);
      a = fma(1.0, ws[51968], a);
      a = fma(1.0, ws[52288], a);
      yout[4480] = a;
    }
    {
      double a = 1.0 * ws[46784];
      a = fma(0.1, ws[46816], a);
      a = fma(1.0, ws[46848], a);
      a = fma(0.685, ws[46880], a);
      a = fma(0.4, ws[47296], a);
      a = a - ws[47584];
      a = a - ws[47680];
      a = a - ws[47712];
      a = a - ws[47744];
      a = fma(1.0, ws[47776], a);
      a = fma(1.0, ws[48544], a);
      a = fma(0.078, ws[48576], a);
      a = fma(1.0, ws[48672], a);
      a = fma(1.0, ws[48896], a);
      a = fma(1.56, ws[48928], a);
      a = fma(1.0, ws[48960], a);
      a = fma(1.125, ws[48992], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.781, ws[49056], a);
      a = fma(0.555, ws[49088], a);
      a = fma(0.5, ws[49120], a);
      a = fma(0.128, ws[49216], a);
      a = fma(0.5, ws[49312], a);
      a = fma(0.673, ws[49344], a);
      a = fma(0.12, ws[49376], a);
      a = fma(0.598, ws[49408], a);
      a = fma(0.598, ws[49440], a);
      a = fma(0.6, ws[49504], a);
      a = fma(0.35, ws[49536], a);
      a = fma(0.231, ws[49600], a);
      a = fma(0.375, ws[49824], a);
      a = fma(0.375, ws[49856], a);
      a = fma(0.3, ws[49888], a);
      a = fma(0.375, ws[49920], a);
      a = fma(0.592, ws[49952], a);
      a = fma(0.28, ws[50016], a);
      a = fma(0.24, ws[50048], a);
      a = fma(0.28, ws[50144], a);
      a = fma(0.24, ws[50176], a);
      a = fma(0.08, ws[51168], a);
      a = fma(0.14, ws[51232], a);
      a = fma(1.0, ws[51936], a);
      a = fma(1.0, ws[52160], a);
      a = a - ws[52288];
      a = fma(1.0, ws[52384], a);
      a = fma(1.0, ws[55584], a);
      a = fma(1.0, ws[55648], a);
      a = fma(0.45, ws[55680], a);
      yout[4512] = a;
    }
    {
      double a = -ws[51808];
      a = fma(1.4, ws[51840], a);
      a = fma(1.0, ws[51872], a);
      a = fma(1.0, ws[51936], a);
      a = fma(1.0, ws[51968], a);
      a = a - ws[52032];
      a = a - ws[52064];
      a = a - ws[52096];
      a = a - ws[52128];
      a = a - ws[52160];
      a = a - ws[52192];
      a = a - ws[52224];
      a = a - ws[52256];
      a = a - ws[52288];
      a = a - ws[52320];
      a = a - ws[52352];
      a = a - ws[52384];
      a = a - ws[52416];
      a = fma(1.0, ws[52448], a);
      a = a - ws[52480];
      a = a - ws[52512];
      a = a - ws[52544];
      a = a - ws[53760];
      a = fma(1.0, ws[53760], a);
      a = a - ws[54720];
      a = fma(1.0, ws[54720], a);
      a = a - ws[54880];
      a = fma(1.0, ws[54880], a);
      a = a - ws[55008];
      a = fma(1.0, ws[55008], a);
      a = a - ws[55168];
      a = fma(1.0, ws[55168], a);
      a = a - ws[55328];
      a = fma(1.0, ws[55328], a);
      a = a - ws[55392];
      a = fma(1.0, ws[55392], a);
      a = a - ws[55552];
      a = fma(1.0, ws[55552], a);
      a = a - ws[55680];
      yout[4544] = a;
    }
    {
      double a = 1.0 * ws[46432];
      a = fma(1.0, ws[46464], a);
      a = a - ws[46912];
      a = a - ws[46944];
      a = a - ws[46976];
      a = a - ws[47008];
      a = fma(0.54, ws[47360], a);
      a = fma(0.991, ws[48512], a);
      a = fma(0.1, ws[48576], a);
      a = fma(0.94, ws[48768], a);
      a = fma(0.7, ws[48896], a);
      a = fma(1.0, ws[48928], a);
      a = fma(0.5, ws[48992], a);
      a = fma(0.2, ws[49024], a);
      a = fma(0.976, ws[49056], a);
      a = fma(0.15, ws[49088], a);
      a = fma(0.48, ws[49120], a);
      a = fma(0.1, ws[49152], a);
      a = fma(1.0, ws[49184], a);
      a = fma(0.3, ws[49216], a);
      a = fma(0.48, ws[49248], a);
      a = fma(0.082, ws[49344], a);
      a = fma(0.072, ws[49408], a);
      a = fma(0.072, ws[49440], a);
      a = fma(0.64, ws[49536], a);
      a = fma(0.142, ws[49632], a);
      a = fma(0.37, ws[49952], a);
      a = fma(0.75, ws[50016], a);
      a = fma(0.07, ws[50048], a);
      a = fma(0.28, ws[50080], a);
      a = fma(0.75, ws[50144], a);
      a = fma(0.07, ws[50176], a);
      a = fma(0.28, ws[50208], a);
      a = fma(0.07, ws[50400], a);
      a = fma(0.058, ws[50560], a);
      a = fma(0.058, ws[50592], a);
      a = fma(0.12, ws[50784], a);
      a = fma(2.0, ws[51008], a);
      a = fma(0.3, ws[51040], a);
      a = fma(0.45, ws[51072], a);
      a = fma(0.4, ws[51136], a);
      a = fma(0.8, ws[51456], a);
      a = fma(1.0, ws[51616], a);
      a = fma(0.126, ws[51680], a);
      a = fma(0.97, ws[52096], a);
      a = fma(0.991, ws[52128], a);
      a = fma(0.96, ws[52256], a);
      a = fma(0.07, ws[52480], a);
      a = fma(0.058, ws[52512], a);
      a = fma(0.058, ws[52544], a);
      yout[4576] = a;
    }
    {
      double a = 1.0 * ws[44608];
      a = fma(1.0, ws[44640], a);
      a = a - ws[44672];
      a = a - ws[44704];
      a = fma(2.0, ws[45280], a);
      a = fma(1.0, ws[45312], a);
      a = a - ws[45344];
      a = fma(2.0, ws[45440], a);
      a = a - ws[45472];
      a = fma(1.0, ws[45472], a);
      a = fma(1.0, ws[45504], a);
      a = fma(1.0, ws[45536], a);
      a = fma(1.0, ws[45568], a);
      a = fma(1.0, ws[45600], a);
      a = fma(2.0, ws[45632], a);
      a = a - ws[45664];
      a = fma(1.0, ws[45696], a);
      a = a - ws[45824];
      a = fma(1.0, ws[45856], a);
      a = fma(1.0, ws[45920], a);
      a = a - ws[45952];
      a = a - ws[46048];
      a = fma(1.0, ws[46080], a);
      a = fma(1.0, ws[46144], a);
      a = fma(1.0, ws[46208], a);
      a = a - ws[46240];
      a = fma(1.0, ws[46272], a);
      a = fma(1.0, ws[46464], a);
      a = a - ws[46496];
      a = fma(1.0, ws[46528], a);
      a = fma(1.0, ws[46784], a);
      a = fma(1.0, ws[46912], a);
      a = fma(1.0, ws[47040], a);
      a = fma(1.0, ws[47808], a);
      a = a - ws[48832];
      a = fma(0.5, ws[48992], a);
      a = fma(0.5, ws[49120], a);
      a = fma(0.5, ws[49248], a);
      a = fma(0.9, ws[49344], a);
      a = fma(0.35, ws[49536], a);
      a = fma(0.142, ws[49632], a);
      a = fma(1.0, ws[49856], a);
      a = fma(0.444, ws[49952], a);
      a = fma(0.47, ws[50080], a);
      a = fma(0.47, ws[50208], a);
      a = fma(0.918, ws[50272], a);
      a = fma(0.86, ws[50432], a);
      a = fma(0.86, ws[50624], a);
      a = a - ws[50816];
      a = fma(0.5, ws[51072], a);
      a = fma(1.0, ws[51296], a);
      a = a - ws[51328];
      a = fma(1.0, ws[51360], a);
      a = fma(0.5, ws[51488], a);
      a = fma(1.0, ws[51520], a);
      a = a - ws[51712];
      a = fma(1.0, ws[51872], a);
      a = a - ws[52608];
      a = a - ws[53408];
      yout[4608] = a;
    }
    {
      double a = 1.0 * ws[44704];
      a = fma(1.0, ws[45344], a);
      a = a - ws[45440];
      a = a - ws[45472];
      a = a - ws[45504];
      a = a - ws[45536];
      a = a - ws[45568];
      a = a - ws[45600];
      a = a - ws[45632];
      a = a - ws[45632];
      a = a - ws[45664];
      a = fma(1.0, ws[45696], a);
      a = fma(1.0, ws[45984], a);
      a = a - ws[47712];
      a = a - ws[47936];
      a = a - ws[48064];
      a = a - ws[48192];
      a = a - ws[48288];
      a = a - ws[48352];
      a = a - ws[48992];
      a = a - ws[49120];
      a = a - ws[49248];
      a = a - ws[49536];
      a = a - ws[49632];
      a = a - ws[49760];
      a = fma(0.185, ws[49952], a);
      a = a - ws[50080];
      a = a - ws[50208];
      a = a - ws[50784];
      a = a - ws[50912];
      a = a - ws[51072];
      a = a - ws[51200];
      a = a - ws[51264];
      a = a - ws[53024];
      a = fma(1.0, ws[53024], a);
      a = a - ws[53696];
      a = fma(1.0, ws[53696], a);
      a = a - ws[54592];
      a = fma(1.0, ws[54592], a);
      a = a - ws[54784];
      a = fma(1.0, ws[54784], a);
      a = a - ws[54976];
      a = fma(1.0, ws[54976], a);
      a = a - ws[55104];
      a = fma(1.0, ws[55104], a);
      a = a - ws[55264];
      a = fma(1.0, ws[55264], a);
      a = a - ws[55648];
      yout[4640] = a;
    }
    {
      double a = 1.0 * ws[46208];
      a = fma(0.5, ws[46336], a);
      a = a - ws[46368];
      a = fma(2.0, ws[46400], a);
      a = fma(2.0, ws[46432], a);
      a = fma(1.0, ws[46464], a);
      a = fma(0.5, ws[46592], a);
      a = a - ws[46624];
      a = fma(2.0, ws[46656], a);
      a = a - ws[46688];
      a = a - ws[46720];
      a = a - ws[46752];
      a = a - ws[46752];
      a = fma(0.9, ws[46848], a);
      a = a - ws[46880];
      a = fma(1.0, ws[46880], a);
      a = fma(0.8, ws[46976], a);
      a = a - ws[47008];
      a = fma(1.0, ws[47008], a);
      a = fma(0.8, ws[47104], a);
      a = a - ws[47136];
      a = fma(1.0, ws[47136], a);
      a = fma(0.8, ws[47232], a);
      a = a - ws[47264];
      a = fma(1.0, ws[47264], a);
      a = fma(0.6, ws[47296], a);
      a = fma(0.6, ws[47360], a);
      a = fma(1.0, ws[47520], a);
      a = fma(0.2, ws[48224], a);
      a = fma(0.5, ws[48288], a);
      a = fma(1.0, ws[48352], a);
      a = fma(1.0, ws[48480], a);
      a = fma(1.0, ws[48512], a);
      a = fma(0.1, ws[48576], a);
      a = fma(1.0, ws[48672], a);
      a = fma(0.98, ws[48768], a);
      a = fma(0.7, ws[48896], a);
      a = fma(1.0, ws[48928], a);
      a = fma(1.0, ws[48992], a);
      a = fma(0.21, ws[49024], a);
      a = fma(1.195, ws[49056], a);
      a = fma(0.15, ws[49088], a);
      a = fma(1.0, ws[49120], a);
      a = fma(0.1, ws[49152], a);
      a = fma(1.0, ws[49184], a);
      a = fma(0.3, ws[49216], a);
      a = fma(1.0, ws[49248], a);
      a = fma(1.0, ws[49280], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.082, ws[49344], a);
      a = fma(0.872, ws[49408], a);
      a = a - ws[49440];
      a = fma(1.072, ws[49440], a);
      a = fma(0.2, ws[49504], a);
      a = fma(1.0, ws[49536], a);
      a = fma(0.658, ws[49568], a);
      a = fma(0.284, ws[49632], a);
      a = fma(0.067, ws[49696], a);
      a = fma(1.0, ws[49792], a);
      a = fma(0.8, ws[49888], a);
      a = a - ws[49920];
      a = fma(1.0, ws[49920], a);
      a = fma(1.0, ws[49952], a);
      a = fma(1.5, ws[50016], a);
      a = fma(0.94, ws[50048], a);
      a = fma(1.28, ws[50080], a);
      a = fma(1.5, ws[50144], a);
      a = fma(0.94, ws[50176], a);
      a = fma(1.28, ws[50208], a);
      a = fma(0.352, ws[50240], a);
      a = fma(1.0, ws[50304], a);
      a = a - ws[50368];
      a = fma(1.0, ws[50368], a);
      a = fma(0.72, ws[50400], a);
      a = fma(1.0, ws[50464], a);
      a = a - ws[50528];
      a = fma(1.0, ws[50528], a);
      a = fma(0.602, ws[50560], a);
      a = fma(0.602, ws[50592], a);
      a = fma(1.0, ws[50688], a);
      a = a - ws[50720];
      a = fma(1.0, ws[50720], a);
      a = fma(0.02, ws[50752], a);
      a = fma(0.7, ws[50784], a);
      a = fma(2.0, ws[51008], a);
      a = fma(0.3, ws[51040], a);
      a = fma(1.0, ws[51072], a);
      a = fma(0.4, ws[51136], a);
      a = fma(0.5, ws[51392], a);
      a = fma(2.0, ws[51424], a);
      a = a - ws[51456];
      a = fma(1.8, ws[51456], a);
      a = fma(1.0, ws[51552], a);
      a = fma(1.0, ws[51584], a);
      a = fma(1.0, ws[51616], a);
      a = fma(1.0, ws[51648], a);
      a = fma(1.0, ws[51680], a);
      a = fma(1.0, ws[52032], a);
      a = fma(1.0, ws[52096], a);
      a = fma(1.0, ws[52128], a);
      a = fma(1.0, ws[52256], a);
      a = fma(0.72, ws[52480], a);
      a = fma(0.602, ws[52512], a);
      a = fma(0.602, ws[52544], a);
      a = a - ws[53728];
      a = fma(1.0, ws[53728], a);
      yout[4672] = a;
    }
    {
      double a = 1.0 * ws[44896];
      a = a - ws[44928];
      a = fma(1.0, ws[44960], a);
      a = a - ws[44992];
      a = a - ws[45088];
      a = a - ws[45120];
      a = a - ws[45120];
      a = a - ws[45152];
      a = a - ws[45152];
      a = fma(1.0, ws[45216], a);
      a = fma(1.0, ws[45248], a);
      a = a - ws[45312];
      a = fma(1.0, ws[45536], a);
      a = a - ws[45568];
      a = a - ws[46048];
      a = fma(1.0, ws[46080], a);
      a = fma(1.0, ws[46176], a);
      a = a - ws[46336];
      a = a - ws[46592];
      a = a - ws[46720];
      a = fma(1.0, ws[46720], a);
      a = fma(1.0, ws[46784], a);
      a = a - ws[46816];
      a = fma(0.9, ws[46848], a);
      a = fma(0.37, ws[46880], a);
      a = fma(1.0, ws[46912], a);
      a = a - ws[46944];
      a = fma(0.8, ws[46976], a);
      a = fma(0.6, ws[47008], a);
      a = a - ws[47072];
      a = a - ws[47200];
      a = fma(0.8, ws[47232], a);
      a = fma(1.0, ws[47488], a);
      a = fma(1.0, ws[47584], a);
      a = fma(1.0, ws[47680], a);
      a = fma(1.0, ws[47712], a);
      a = a - ws[47744];
      a = fma(1.0, ws[47776], a);
      a = fma(1.0, ws[47808], a);
      a = a - ws[47840];
      a = fma(0.2, ws[47840], a);
      a = fma(0.2, ws[48128], a);
      a = fma(1.0, ws[48224], a);
      a = fma(1.0, ws[48288], a);
      a = fma(1.0, ws[48416], a);
      a = fma(1.0, ws[48448], a);
      a = fma(1.0, ws[48544], a);
      a = fma(0.9, ws[48576], a);
      a = fma(1.0, ws[48800], a);
      a = fma(0.3, ws[48864], a);
      a = fma(1.0, ws[48896], a);
      a = fma(0.27, ws[48960], a);
      a = fma(0.1, ws[49024], a);
      a = fma(0.08, ws[49088], a);
      a = fma(0.25, ws[49312], a);
      a = fma(0.818, ws[49344], a);
      a = a - ws[49376];
      a = fma(0.12, ws[49376], a);
      a = fma(0.728, ws[49408], a);
      a = fma(0.728, ws[49440], a);
      a = fma(1.0, ws[49472], a);
      a = fma(0.066, ws[49504], a);
      a = fma(0.137, ws[49568], a);
      a = fma(0.398, ws[49600], a);
      a = a - ws[49824];
      a = fma(0.825, ws[49824], a);
      a = fma(0.825, ws[49856], a);
      a = fma(0.66, ws[49888], a);
      a = fma(0.825, ws[49920], a);
      a = fma(0.53, ws[50240], a);
      a = fma(0.918, ws[50272], a);
      a = fma(1.0, ws[50304], a);
      a = a - ws[50336];
      a = fma(1.0, ws[50368], a);
      a = fma(0.18, ws[50400], a);
      a = fma(0.86, ws[50432], a);
      a = fma(1.0, ws[50464], a);
      a = a - ws[50496];
      a = fma(1.0, ws[50528], a);
      a = fma(0.155, ws[50560], a);
      a = fma(0.155, ws[50592], a);
      a = fma(0.86, ws[50624], a);
      a = a - ws[50656];
      a = fma(1.0, ws[50688], a);
      a = fma(1.0, ws[50720], a);
      a = fma(1.0, ws[50752], a);
      a = a - ws[50848];
      a = fma(0.56, ws[51168], a);
      a = fma(0.2, ws[51232], a);
      a = fma(0.8, ws[51296], a);
      a = a - ws[51392];
      a = a - ws[51904];
      a = fma(1.0, ws[51936], a);
      a = fma(1.0, ws[52160], a);
      a = fma(1.0, ws[52192], a);
      a = fma(1.0, ws[52224], a);
      a = fma(1.0, ws[52288], a);
      a = fma(1.0, ws[52384], a);
      a = fma(1.0, ws[52416], a);
      a = fma(0.18, ws[52480], a);
      a = fma(0.155, ws[52512], a);
      a = fma(0.155, ws[52544], a);
      a = a - ws[52800];
      a = fma(1.0, ws[52800], a);
      a = a - ws[52864];
      a = fma(1.0, ws[52864], a);
      a = a - ws[52928];
      a = fma(1.0, ws[52928], a);
      a = a - ws[53088];
      a = fma(1.0, ws[53088], a);
      a = a - ws[53664];
      a = fma(1.0, ws[53664], a);
      yout[4704] = a;
    }
    {
      double a = 2.0 * ws[44864];
      a = a - ws[44896];
      a = fma(1.0, ws[44928], a);
      a = a - ws[44960];
      a = fma(1.0, ws[44992], a);
      a = a - ws[45024];
      a = a - ws[45024];
      a = a - ws[45056];
      a = a - ws[45056];
      a = a - ws[45088];
      a = a - ws[45216];
      a = fma(1.0, ws[45248], a);
      a = fma(1.0, ws[45312], a);
      a = a - ws[45536];
      a = fma(1.0, ws[45568], a);
      a = a - ws[45792];
      a = a - ws[45920];
      a = a - ws[45952];
      a = a - ws[45984];
      a = a - ws[46144];
      a = a - ws[46176];
      a = fma(0.5, ws[46336], a);
      a = fma(0.5, ws[46592], a);
      a = a - ws[47296];
      a = fma(0.4, ws[47296], a);
      a = a - ws[47360];
      a = fma(0.4, ws[47360], a);
      a = a - ws[47424];
      a = a - ws[47488];
      a = a - ws[47520];
      a = a - ws[47552];
      a = a - ws[47584];
      a = fma(1.0, ws[47680], a);
      a = fma(0.2, ws[47840], a);
      a = fma(1.0, ws[47872], a);
      a = a - ws[47904];
      a = fma(1.0, ws[48000], a);
      a = a - ws[48032];
      a = a - ws[48128];
      a = a - ws[48224];
      a = a - ws[48384];
      a = a - ws[48416];
      a = a - ws[48448];
      a = a - ws[48480];
      a = a - ws[48512];
      a = a - ws[48544];
      a = a - ws[48576];
      a = a - ws[48672];
      a = a - ws[48704];
      a = a - ws[48736];
      a = a - ws[48864];
      a = fma(0.7, ws[48864], a);
      a = fma(0.3, ws[48896], a);
      a = a - ws[48928];
      a = fma(0.17, ws[48960], a);
      a = fma(0.1, ws[49024], a);
      a = a - ws[49056];
      a = fma(0.334, ws[49088], a);
      a = a - ws[49184];
      a = fma(0.5, ws[49216], a);
      a = a - ws[49280];
      a = fma(0.12, ws[49376], a);
      a = fma(0.266, ws[49504], a);
      a = a - ws[49568];
      a = fma(0.461, ws[49600], a);
      a = a - ws[49696];
      a = fma(0.933, ws[49696], a);
      a = a - ws[49792];
      a = fma(1.125, ws[49824], a);
      a = fma(0.125, ws[49856], a);
      a = fma(0.1, ws[49888], a);
      a = fma(0.125, ws[49920], a);
      a = a - ws[49952];
      a = a - ws[50016];
      a = fma(0.57, ws[50048], a);
      a = a - ws[50144];
      a = fma(0.57, ws[50176], a);
      a = a - ws[50240];
      a = fma(0.118, ws[50240], a);
      a = a - ws[50400];
      a = fma(0.1, ws[50400], a);
      a = a - ws[50560];
      a = fma(0.244, ws[50560], a);
      a = a - ws[50592];
      a = fma(0.244, ws[50592], a);
      a = a - ws[50752];
      a = a - ws[50880];
      a = a - ws[51008];
      a = fma(0.5, ws[51040], a);
      a = a - ws[51136];
      a = fma(0.5, ws[51168], a);
      a = a - ws[51232];
      a = fma(0.5, ws[51392], a);
      a = a - ws[51488];
      a = a - ws[51520];
      a = a - ws[51552];
      a = a - ws[51712];
      a = a - ws[51968];
      a = a - ws[52448];
      a = fma(0.1, ws[52480], a);
      a = fma(0.244, ws[52512], a);
      a = fma(0.244, ws[52544], a);
      a = a - ws[52992];
      a = fma(1.0, ws[52992], a);
      a = a - ws[53120];
      a = fma(1.0, ws[53120], a);
      a = a - ws[53792];
      a = fma(1.0, ws[53792], a);
      a = a - ws[54080];
      a = fma(1.0, ws[54080], a);
      a = a - ws[54112];
      a = fma(1.0, ws[54112], a);
      a = a - ws[54144];
      a = fma(1.0, ws[54144], a);
      a = a - ws[54176];
      a = fma(1.0, ws[54176], a);
      a = a - ws[54208];
      a = fma(1.0, ws[54208], a);
      a = a - ws[54240];
      a = fma(1.0, ws[54240], a);
      a = a - ws[54272];
      a = fma(1.0, ws[54272], a);
      a = a - ws[54304];
      a = fma(1.0, ws[54304], a);
      a = a - ws[54336];
      a = fma(1.0, ws[54336], a);
      a = a - ws[54368];
      a = fma(1.0, ws[54368], a);
      a = a - ws[54400];
      a = fma(1.0, ws[54400], a);
      a = a - ws[54432];
      a = fma(1.0, ws[54432], a);
      a = a - ws[54464];
      a = fma(1.0, ws[54464], a);
      a = a - ws[54496];
      a = fma(1.0, ws[54496], a);
      a = a - ws[54528];
      a = fma(1.0, ws[54528], a);
      a = a - ws[54560];
      a = fma(1.0, ws[54560], a);
      a = a - ws[54752];
      a = fma(1.0, ws[54752], a);
      a = a - ws[54912];
      a = fma(1.0, ws[54912], a);
      a = a - ws[55040];
      a = fma(1.0, ws[55040], a);
      a = a - ws[55200];
      a = fma(1.0, ws[55200], a);
      a = a - ws[55360];
      a = fma(1.0, ws[55360], a);
      a = a - ws[55520];
      a = fma(1.0, ws[55520], a);
      a = a - ws[55584];
      a = a - ws[55616];
      yout[4736] = a;
    }
}
// Partial-derivative products of 2- and 3-reactant reactions (rbjacob.F:112-143).
__device__ __noinline__ void explic_1(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    { const double kk = ws[33440]; ws[55712] = kk * y[4384]; ws[55744] = kk * y[4320]; }
    { const double kk = ws[33472]; ws[55776] = kk * y[4384]; ws[55808] = kk * y[4160]; }
    { const double kk = ws[33504]; ws[55840] = kk * y[4608]; ws[55872] = kk * y[4160]; }
    { const double kk = ws[33536]; ws[55904] = kk * y[4608]; ws[55936] = kk * y[4160]; }
    { const double kk = ws[33568]; ws[55968] = kk * y[4320]; ws[56000] = kk * y[4160]; }
    { const double kk = ws[33728]; ws[56032] = kk * y[4736]; ws[56064] = kk * y[4320]; }
    { const double kk = ws[33760]; ws[56096] = kk * y[4704]; ws[56128] = kk * y[4320]; }
    { const double kk = ws[33792]; ws[56160] = kk * y[4160]; ws[56192] = kk * y[4736]; }
    { const double kk = ws[33824]; ws[56224] = kk * y[4160]; ws[56256] = kk * y[4704]; }
    { const double kk = ws[33856]; ws[56288] = kk * y[4736]; ws[56320] = kk * y[4736]; }
    { const double kk = ws[33888]; ws[56352] = kk * y[4736]; ws[56384] = kk * y[4736]; }
    { const double kk = ws[33920]; ws[56416] = kk * y[4704]; ws[56448] = kk * y[4736]; }
    { const double kk = ws[33952]; ws[56480] = kk * y[4704]; ws[56512] = kk * y[4704]; }
    { const double kk = ws[33984]; ws[56544] = kk * y[4704]; ws[56576] = kk * y[4704]; }
    { const double kk = ws[34048]; ws[56608] = kk * y[4736]; ws[56640] = kk * y[3456]; }
    { const double kk = ws[34080]; ws[56672] = kk * y[4160]; ws[56704] = kk * y[3456]; }
    { const double kk = ws[34112]; ws[56736] = kk * y[4384]; ws[56768] = kk * y[4384]; }
    { const double kk = ws[34144]; ws[56800] = kk * y[4384]; ws[56832] = kk * y[4704]; }
    { const double kk = ws[34176]; ws[56864] = kk * y[4320]; ws[56896] = kk * y[4608]; }
    { const double kk = ws[34272]; ws[56928] = kk * y[4384]; ws[56960] = kk * y[4640]; }
    { const double kk = ws[34304]; ws[56992] = kk * y[4608]; ws[57024] = kk * y[4640]; }
    { const double kk = ws[34336]; ws[57056] = kk * y[4160]; ws[57088] = kk * y[4640]; }
    { const double kk = ws[34368]; ws[57120] = kk * y[4736]; ws[57152] = kk * y[4640]; }
    { const double kk = ws[34400]; ws[57184] = kk * y[4704]; ws[57216] = kk * y[4640]; }
    { const double kk = ws[34432]; ws[57248] = kk * y[4320]; ws[57280] = kk * y[4640]; }
    { const double kk = ws[34464]; ws[57312] = kk * y[4640]; ws[57344] = kk * y[4640]; }
    { const double kk = ws[34496]; ws[57376] = kk * y[4608]; ws[57408] = kk * y[4640]; }
    { const double kk = ws[34624]; ws[57440] = kk * y[4736]; ws[57472] = kk * y[4384]; }
    { const double kk = ws[34656]; ws[57504] = kk * y[4608]; ws[57536] = kk * y[4384]; }
    { const double kk = ws[34688]; ws[57568] = kk * y[2464]; ws[57600] = kk * y[2464]; }
    { const double kk = ws[34752]; ws[57632] = kk * y[4736]; ws[57664] = kk * y[2464]; }
    { const double kk = ws[34784]; ws[57696] = kk * y[4736]; ws[57728] = kk * y[4608]; }
    { const double kk = ws[34816]; ws[57760] = kk * y[4736]; ws[57792] = kk * y[4192]; }
    { const double kk = ws[34880]; ws[57824] = kk * y[4608]; ws[57856] = kk * y[4704]; }
    { const double kk = ws[34976]; ws[57888] = kk * y[4736]; ws[57920] = kk * y[1696]; }
    { const double kk = ws[35008]; ws[57952] = kk * y[4736]; ws[57984] = kk * y[2208]; }
    { const double kk = ws[35040]; ws[58016] = kk * y[4384]; ws[58048] = kk * y[4448]; }
    { const double kk = ws[35072]; ws[58080] = kk * y[4608]; ws[58112] = kk * y[4448]; }
    { const double kk = ws[35168]; ws[58144] = kk * y[4704]; ws[58176] = kk * y[4448]; }
    { const double kk = ws[35200]; ws[58208] = kk * y[4672]; ws[58240] = kk * y[4448]; }
    { const double kk = ws[35232]; ws[58272] = kk * y[4448]; ws[58304] = kk * y[4448]; }
    { const double kk = ws[35264]; ws[58336] = kk * y[4096]; ws[58368] = kk * y[4448]; }
    { const double kk = ws[35296]; ws[58400] = kk * y[4384]; ws[58432] = kk * y[4096]; }
    { const double kk = ws[35328]; ws[58464] = kk * y[4608]; ws[58496] = kk * y[4096]; }
    { const double kk = ws[35424]; ws[58528] = kk * y[4704]; ws[58560] = kk * y[4096]; }
    { const double kk = ws[35456]; ws[58592] = kk * y[4672]; ws[58624] = kk * y[4096]; }
    { const double kk = ws[35488]; ws[58656] = kk * y[4096]; ws[58688] = kk * y[4096]; }
    { const double kk = ws[35520]; ws[58720] = kk * y[4384]; ws[58752] = kk * y[4672]; }
    { const double kk = ws[35552]; ws[58784] = kk * y[4704]; ws[58816] = kk * y[4672]; }
    { const double kk = ws[35584]; ws[58848] = kk * y[4672]; ws[58880] = kk * y[4672]; }
    { const double kk = ws[35616]; ws[58912] = kk * y[4384]; ws[58944] = kk * y[4416]; }
    { const double kk = ws[35648]; ws[58976] = kk * y[4704]; ws[59008] = kk * y[4416]; }
    { const double kk = ws[35680]; ws[59040] = kk * y[4448]; ws[59072] = kk * y[4416]; }
    { const double kk = ws[35712]; ws[59104] = kk * y[4672]; ws[59136] = kk * y[4416]; }
    { const double kk = ws[35744]; ws[59168] = kk * y[4384]; ws[59200] = kk * y[4576]; }
    { const double kk = ws[35776]; ws[59232] = kk * y[4704]; ws[59264] = kk * y[4576]; }
    { const double kk = ws[35808]; ws[59296] = kk * y[4448]; ws[59328] = kk * y[4576]; }
    { const double kk = ws[35840]; ws[59360] = kk * y[4672]; ws[59392] = kk * y[4576]; }
    { const double kk = ws[35872]; ws[59424] = kk * y[4384]; ws[59456] = kk * y[4352]; }
    { const double kk = ws[35904]; ws[59488] = kk * y[4704]; ws[59520] = kk * y[4352]; }
    { const double kk = ws[35936]; ws[59552] = kk * y[4448]; ws[59584] = kk * y[4352]; }
    { const double kk = ws[35968]; ws[59616] = kk * y[4672]; ws[59648] = kk * y[4352]; }
    { const double kk = ws[36000]; ws[59680] = kk * y[4384]; ws[59712] = kk * y[4288]; }
    { const double kk = ws[36032]; ws[59744] = kk * y[4704]; ws[59776] = kk * y[4288]; }
    { const double kk = ws[36064]; ws[59808] = kk * y[4448]; ws[59840] = kk * y[4288]; }
    { const double kk = ws[36096]; ws[59872] = kk * y[4672]; ws[59904] = kk * y[4288]; }
    { const double kk = ws[36128]; ws[59936] = kk * y[4736]; ws[59968] = kk * y[2272]; }
    { const double kk = ws[36192]; ws[60000] = kk * y[4736]; ws[60032] = kk * y[2880]; }
    { const double kk = ws[36256]; ws[60064] = kk * y[4736]; ws[60096] = kk * y[3648]; }
    { const double kk = ws[36320]; ws[60128] = kk * y[4736]; ws[60160] = kk * y[3776]; }
    { const double kk = ws[36352]; ws[60192] = kk * y[4736]; ws[60224] = kk * y[3904]; }
    { const double kk = ws[36384]; ws[60256] = kk * y[4736]; ws[60288] = kk * y[2688]; }
    { const double kk = ws[36416]; ws[60320] = kk * y[4736]; ws[60352] = kk * y[4512]; }
    { const double kk = ws[36512]; ws[60384] = kk * y[4160]; ws[60416] = kk * y[4512]; }
    { const double kk = ws[36544]; ws[60448] = kk * y[4640]; ws[60480] = kk * y[4512]; }
    { const double kk = ws[36576]; ws[60512] = kk * y[4704]; ws[60544] = kk * y[4512]; }
    { const double kk = ws[36640]; ws[60576] = kk * y[4384]; ws[60608] = kk * y[1728]; }
    { const double kk = ws[36672]; ws[60640] = kk * y[4704]; ws[60672] = kk * y[1728]; }
    { const double kk = ws[36704]; ws[60704] = kk * y[4160]; ws[60736] = kk * y[4128]; }
    { const double kk = ws[36736]; ws[60768] = kk * y[4736]; ws[60800] = kk * y[4128]; }
    { const double kk = ws[36768]; ws[60832] = kk * y[4640]; ws[60864] = kk * y[4128]; }
    { const double kk = ws[36832]; ws[60896] = kk * y[4160]; ws[60928] = kk * y[4064]; }
    { const double kk = ws[36864]; ws[60960] = kk * y[4736]; ws[60992] = kk * y[4064]; }
    { const double kk = ws[36896]; ws[61024] = kk * y[4640]; ws[61056] = kk * y[4064]; }
    { const double kk = ws[36960]; ws[61088] = kk * y[4736]; ws[61120] = kk * y[3840]; }
    { const double kk = ws[37024]; ws[61152] = kk * y[4640]; ws[61184] = kk * y[3840]; }
    { const double kk = ws[37056]; ws[61216] = kk * y[4736]; ws[61248] = kk * y[4256]; }
    { const double kk = ws[37120]; ws[61280] = kk * y[4640]; ws[61312] = kk * y[4256]; }
    { const double kk = ws[37184]; ws[61344] = kk * y[4640]; ws[61376] = kk * y[4000]; }
    { const double kk = ws[37216]; ws[61408] = kk * y[4736]; ws[61440] = kk * y[4000]; }
    { const double kk = ws[37280]; ws[61472] = kk * y[4736]; ws[61504] = kk * y[4480]; }
    { const double kk = ws[37344]; ws[61536] = kk * y[4736]; ws[61568] = kk * y[832]; }
    { const double kk = ws[37376]; ws[61600] = kk * y[4736]; ws[61632] = kk * y[2720]; }
    { const double kk = ws[37408]; ws[61664] = kk * y[4736]; ws[61696] = kk * y[864]; }
    { const double kk = ws[37504]; ws[61728] = kk * y[4736]; ws[61760] = kk * y[3392]; }
    { const double kk = ws[37536]; ws[61792] = kk * y[4736]; ws[61824] = kk * y[896]; }
    { const double kk = ws[37568]; ws[61856] = kk * y[4736]; ws[61888] = kk * y[4224]; }
    { const double kk = ws[37664]; ws[61920] = kk * y[4608]; ws[61952] = kk * y[960]; }
    { const double kk = ws[37696]; ws[61984] = kk * y[4736]; ws[62016] = kk * y[352]; }
    { const double kk = ws[37728]; ws[62048] = kk * y[4160]; ws[62080] = kk * y[2656]; }
    { const double kk = ws[37760]; ws[62112] = kk * y[4736]; ws[62144] = kk * y[2656]; }
    { const double kk = ws[37792]; ws[62176] = kk * y[4320]; ws[62208] = kk * y[2656]; }
    { const double kk = ws[37824]; ws[62240] = kk * y[4640]; ws[62272] = kk * y[2656]; }
    { const double kk = ws[37856]; ws[62304] = kk * y[4160]; ws[62336] = kk * y[3552]; }
    { const double kk = ws[37888]; ws[62368] = kk * y[4736]; ws[62400] = kk * y[3552]; }
    { const double kk = ws[37920]; ws[62432] = kk * y[4320]; ws[62464] = kk * y[3552]; }
    { const double kk = ws[37952]; ws[62496] = kk * y[4640]; ws[62528] = kk * y[3552]; }
    { const double kk = ws[37984]; ws[62560] = kk * y[4160]; ws[62592] = kk * y[3136]; }
    { const double kk = ws[38016]; ws[62624] = kk * y[4736]; ws[62656] = kk * y[3136]; }
    { const double kk = ws[38048]; ws[62688] = kk * y[4320]; ws[62720] = kk * y[3136]; }
    { const double kk = ws[38080]; ws[62752] = kk * y[4640]; ws[62784] = kk * y[3136]; }
    { const double kk = ws[38112]; ws[62816] = kk * y[4736]; ws[62848] = kk * y[2528]; }
    { const double kk = ws[38144]; ws[62880] = kk * y[4160]; ws[62912] = kk * y[2528]; }
    { const double kk = ws[38176]; ws[62944] = kk * y[4384]; ws[62976] = kk * y[3424]; }
    { const double kk = ws[38208]; ws[63008] = kk * y[4704]; ws[63040] = kk * y[3424]; }
    { const double kk = ws[38240]; ws[63072] = kk * y[4448]; ws[63104] = kk * y[3424]; }
    { const double kk = ws[38272]; ws[63136] = kk * y[4672]; ws[63168] = kk * y[3424]; }
    { const double kk = ws[38336]; ws[63200] = kk * y[4320]; ws[63232] = kk * y[2528]; }
    { const double kk = ws[38368]; ws[63264] = kk * y[4640]; ws[63296] = kk * y[2528]; }
    { const double kk = ws[38400]; ws[63328] = kk * y[4736]; ws[63360] = kk * y[3872]; }
    { const double kk = ws[38432]; ws[63392] = kk * y[4320]; ws[63424] = kk * y[3872]; }
    { const double kk = ws[38464]; ws[63456] = kk * y[4640]; ws[63488] = kk * y[3872]; }
    { const double kk = ws[38528]; ws[63520] = kk * y[4736]; ws[63552] = kk * y[1664]; }
    { const double kk = ws[38592]; ws[63584] = kk * y[4640]; ws[63616] = kk * y[1024]; }
    { const double kk = ws[38624]; ws[63648] = kk * y[4736]; ws[63680] = kk * y[1056]; }
    { const double kk = ws[38656]; ws[63712] = kk * y[4704]; ws[63744] = kk * y[3296]; }
    { const double kk = ws[38688]; ws[63776] = kk * y[4384]; ws[63808] = kk * y[3296]; }
    { const double kk = ws[38720]; ws[63840] = kk * y[4448]; ws[63872] = kk * y[3296]; }
    { const double kk = ws[38752]; ws[63904] = kk * y[4672]; ws[63936] = kk * y[3296]; }
    { const double kk = ws[38784]; ws[63968] = kk * y[4736]; ws[64000] = kk * y[1632]; }
    { const double kk = ws[38816]; ws[64032] = kk * y[4160]; ws[64064] = kk * y[2048]; }
    { const double kk = ws[38848]; ws[64096] = kk * y[4736]; ws[64128] = kk * y[2048]; }
    { const double kk = ws[38880]; ws[64160] = kk * y[4320]; ws[64192] = kk * y[2048]; }
    { const double kk = ws[38912]; ws[64224] = kk * y[4640]; ws[64256] = kk * y[2048]; }
    { const double kk = ws[38944]; ws[64288] = kk * y[4160]; ws[64320] = kk * y[2112]; }
    { const double kk = ws[38976]; ws[64352] = kk * y[4736]; ws[64384] = kk * y[2112]; }
    { const double kk = ws[39008]; ws[64416] = kk * y[4320]; ws[64448] = kk * y[2112]; }
    { const double kk = ws[39040]; ws[64480] = kk * y[4640]; ws[64512] = kk * y[2112]; }
    { const double kk = ws[39072]; ws[64544] = kk * y[4736]; ws[64576] = kk * y[384]; }
    { const double kk = ws[39104]; ws[64608] = kk * y[4384]; ws[64640] = kk * y[3104]; }
    { const double kk = ws[39136]; ws[64672] = kk * y[4448]; ws[64704] = kk * y[3104]; }
    { const double kk = ws[39168]; ws[64736] = kk * y[4704]; ws[64768] = kk * y[3104]; }
    { const double kk = ws[39200]; ws[64800] = kk * y[4672]; ws[64832] = kk * y[3104]; }
    { const double kk = ws[39232]; ws[64864] = kk * y[4736]; ws[64896] = kk * y[1088]; }
    { const double kk = ws[39264]; ws[64928] = kk * y[4384]; ws[64960] = kk * y[3488]; }
    { const double kk = ws[39296]; ws[64992] = kk * y[4448]; ws[65024] = kk * y[3488]; }
    { const double kk = ws[39328]; ws[65056] = kk * y[4704]; ws[65088] = kk * y[3488]; }
    { const double kk = ws[39360]; ws[65120] = kk * y[4672]; ws[65152] = kk * y[3488]; }
    { const double kk = ws[39392]; ws[65184] = kk * y[4736]; ws[65216] = kk * y[1120]; }
    { const double kk = ws[39424]; ws[65248] = kk * y[4736]; ws[65280] = kk * y[1152]; }
    { const double kk = ws[39456]; ws[65312] = kk * y[4384]; ws[65344] = kk * y[3584]; }
    { const double kk = ws[39488]; ws[65376] = kk * y[4704]; ws[65408] = kk * y[3584]; }
    { const double kk = ws[39520]; ws[65440] = kk * y[4448]; ws[65472] = kk * y[3584]; }
    { const double kk = ws[39552]; ws[65504] = kk * y[4672]; ws[65536] = kk * y[3584]; }
    { const double kk = ws[39584]; ws[65568] = kk * y[4736]; ws[65600] = kk * y[3616]; }
    { const double kk = ws[39616]; ws[65632] = kk * y[4640]; ws[65664] = kk * y[3616]; }
    { const double kk = ws[39648]; ws[65696] = kk * y[4608]; ws[65728] = kk * y[3328]; }
    { const double kk = ws[39680]; ws[65760] = kk * y[4704]; ws[65792] = kk * y[3328]; }
    { const double kk = ws[39712]; ws[65824] = kk * y[4736]; ws[65856] = kk * y[2176]; }
    { const double kk = ws[39744]; ws[65888] = kk * y[4640]; ws[65920] = kk * y[2176]; }
    { const double kk = ws[39840]; ws[65952] = kk * y[4736]; ws[65984] = kk * y[3808]; }
    { const double kk = ws[39872]; ws[66016] = kk * y[4320]; ws[66048] = kk * y[3808]; }
    { const double kk = ws[39904]; ws[66080] = kk * y[4640]; ws[66112] = kk * y[3808]; }
    { const double kk = ws[39968]; ws[66144] = kk * y[4736]; ws[66176] = kk * y[3936]; }
    { const double kk = ws[40000]; ws[66208] = kk * y[4320]; ws[66240] = kk * y[3936]; }
    { const double kk = ws[40032]; ws[66272] = kk * y[4640]; ws[66304] = kk * y[3936]; }
    { const double kk = ws[40064]; ws[66336] = kk * y[4736]; ws[66368] = kk * y[1760]; }
    { const double kk = ws[40096]; ws[66400] = kk * y[4640]; ws[66432] = kk * y[1760]; }
    { const double kk = ws[40128]; ws[66464] = kk * y[4384]; ws[66496] = kk * y[3744]; }
    { const double kk = ws[40160]; ws[66528] = kk * y[4608]; ws[66560] = kk * y[3744]; }
    { const double kk = ws[40224]; ws[66592] = kk * y[4704]; ws[66624] = kk * y[3744]; }
    { const double kk = ws[40256]; ws[66656] = kk * y[4448]; ws[66688] = kk * y[3744]; }
    { const double kk = ws[40288]; ws[66720] = kk * y[4672]; ws[66752] = kk * y[3744]; }
    { const double kk = ws[40320]; ws[66784] = kk * y[4736]; ws[66816] = kk * y[1792]; }
    { const double kk = ws[40352]; ws[66848] = kk * y[4736]; ws[66880] = kk * y[1952]; }
    { const double kk = ws[40384]; ws[66912] = kk * y[4736]; ws[66944] = kk * y[416]; }
    { const double kk = ws[40544]; ws[66976] = kk * y[4736]; ws[67008] = kk * y[4608]; }
    { const double kk = ws[40640]; ws[67040] = kk * y[4320]; ws[67072] = kk * y[4544]; }
    { const double kk = ws[40672]; ws[67104] = kk * y[3520]; ws[67136] = kk * y[3520]; }
    { const double kk = ws[40704]; ws[67168] = kk * y[4384]; ws[67200] = kk * y[3520]; }
    { const double kk = ws[40736]; ws[67232] = kk * y[4704]; ws[67264] = kk * y[3520]; }
    { const double kk = ws[40768]; ws[67296] = kk * y[4416]; ws[67328] = kk * y[3520]; }
    { const double kk = ws[40800]; ws[67360] = kk * y[3232]; ws[67392] = kk * y[4736]; }
    { const double kk = ws[40896]; ws[67424] = kk * y[4224]; ws[67456] = kk * y[4544]; }
    { const double kk = ws[40928]; ws[67488] = kk * y[896]; ws[67520] = kk * y[4544]; }
    { const double kk = ws[40960]; ws[67552] = kk * y[832]; ws[67584] = kk * y[4544]; }
    { const double kk = ws[40992]; ws[67616] = kk * y[2656]; ws[67648] = kk * y[4544]; }
    { const double kk = ws[41024]; ws[67680] = kk * y[3552]; ws[67712] = kk * y[4544]; }
    { const double kk = ws[41056]; ws[67744] = kk * y[3136]; ws[67776] = kk * y[4544]; }
    { const double kk = ws[41088]; ws[67808] = kk * y[2528]; ws[67840] = kk * y[4544]; }
    { const double kk = ws[41120]; ws[67872] = kk * y[4512]; ws[67904] = kk * y[4544]; }
    { const double kk = ws[41152]; ws[67936] = kk * y[4128]; ws[67968] = kk * y[4544]; }
    { const double kk = ws[41184]; ws[68000] = kk * y[4064]; ws[68032] = kk * y[4544]; }
    { const double kk = ws[41216]; ws[68064] = kk * y[2720]; ws[68096] = kk * y[4544]; }
    { const double kk = ws[41248]; ws[68128] = kk * y[864]; ws[68160] = kk * y[4544]; }
    { const double kk = ws[41280]; ws[68192] = kk * y[4736]; ws[68224] = kk * y[3968]; }
    { const double kk = ws[41312]; ws[68256] = kk * y[1088]; ws[68288] = kk * y[4544]; }
    { const double kk = ws[41344]; ws[68320] = kk * y[1120]; ws[68352] = kk * y[4544]; }
    { const double kk = ws[41376]; ws[68384] = kk * y[1152]; ws[68416] = kk * y[4544]; }
    { const double kk = ws[41440]; ws[68448] = kk * y[4608]; ws[68480] = kk * y[3520]; }
    { const double kk = ws[41600]; ws[68512] = kk * y[4384]; ws[68544] = kk * y[2944]; }
    { const double kk = ws[41632]; ws[68576] = kk * y[4704]; ws[68608] = kk * y[2944]; }
    { const double kk = ws[41664]; ws[68640] = kk * y[4384]; ws[68672] = kk * y[2496]; }
    { const double kk = ws[41696]; ws[68704] = kk * y[4704]; ws[68736] = kk * y[2496]; }
    { const double kk = ws[41728]; ws[68768] = kk * y[4384]; ws[68800] = kk * y[2144]; }
    { const double kk = ws[41760]; ws[68832] = kk * y[4704]; ws[68864] = kk * y[2144]; }
    { const double kk = ws[41792]; ws[68896] = kk * y[4320]; ws[68928] = kk * y[1856]; }
    { const double kk = ws[41824]; ws[68960] = kk * y[4736]; ws[68992] = kk * y[1856]; }
    { const double kk = ws[41856]; ws[69024] = kk * y[4640]; ws[69056] = kk * y[1856]; }
    { const double kk = ws[41888]; ws[69088] = kk * y[4384]; ws[69120] = kk * y[2560]; }
    { const double kk = ws[41920]; ws[69152] = kk * y[4704]; ws[69184] = kk * y[2560]; }
    { const double kk = ws[41952]; ws[69216] = kk * y[4736]; ws[69248] = kk * y[448]; }
    { const double kk = ws[42144]; ws[69280] = kk * y[480]; ws[69312] = kk * y[1920]; }
    { const double kk = ws[42176]; ws[69344] = kk * y[512]; ws[69376] = kk * y[1920]; }
    { const double kk = ws[42208]; ws[69408] = kk * y[544]; ws[69440] = kk * y[1248]; }
    { const double kk = ws[42336]; ws[69472] = kk * y[576]; ws[69504] = kk * y[1312]; }
    { const double kk = ws[42464]; ws[69536] = kk * y[4384]; ws[69568] = kk * y[2848]; }
    { const double kk = ws[42496]; ws[69600] = kk * y[4704]; ws[69632] = kk * y[2848]; }
    { const double kk = ws[42528]; ws[69664] = kk * y[4640]; ws[69696] = kk * y[2848]; }
    { const double kk = ws[42560]; ws[69728] = kk * y[4672]; ws[69760] = kk * y[2848]; }
    { const double kk = ws[42592]; ws[69792] = kk * y[4544]; ws[69824] = kk * y[3360]; }
    { const double kk = ws[42624]; ws[69856] = kk * y[4736]; ws[69888] = kk * y[3360]; }
    { const double kk = ws[42912]; ws[69920] = kk * y[4736]; ws[69952] = kk * y[704]; }
    { const double kk = ws[42944]; ws[69984] = kk * y[4736]; ws[70016] = kk * y[1440]; }
    { const double kk = ws[42976]; ws[70048] = kk * y[4736]; ws[70080] = kk * y[736]; }
    { const double kk = ws[43008]; ws[70112] = kk * y[4736]; ws[70144] = kk * y[1472]; }
    { const double kk = ws[43040]; ws[70176] = kk * y[4736]; ws[70208] = kk * y[768]; }
    { const double kk = ws[43072]; ws[70240] = kk * y[4736]; ws[70272] = kk * y[2752]; }
    { const double kk = ws[43104]; ws[70304] = kk * y[4736]; ws[70336] = kk * y[2784]; }
    { const double kk = ws[43136]; ws[70368] = kk * y[4736]; ws[70400] = kk * y[2816]; }
    { const double kk = ws[43168]; ws[70432] = kk * y[4736]; ws[70464] = kk * y[2304]; }
    { const double kk = ws[43200]; ws[70496] = kk * y[4736]; ws[70528] = kk * y[1504]; }
    { const double kk = ws[43232]; ws[70560] = kk * y[4736]; ws[70592] = kk * y[3680]; }
    { const double kk = ws[43264]; ws[70624] = kk * y[4736]; ws[70656] = kk * y[3712]; }
    { const double kk = ws[43296]; ws[70688] = kk * y[4736]; ws[70720] = kk * y[2912]; }
    { const double kk = ws[43328]; ws[70752] = kk * y[4736]; ws[70784] = kk * y[3168]; }
    { const double kk = ws[43360]; ws[70816] = kk * y[4736]; ws[70848] = kk * y[3200]; }
    { const double kk = ws[43392]; ws[70880] = kk * y[4736]; ws[70912] = kk * y[2336]; }
    { const double kk = ws[43424]; ws[70944] = kk * y[4640]; ws[70976] = kk * y[2336]; }
    { const double kk = ws[43456]; ws[71008] = kk * y[4160]; ws[71040] = kk * y[2336]; }
    { const double kk = ws[43552]; ws[71072] = kk * y[4544]; ws[71104] = kk * y[2336]; }
    { const double kk = ws[43584]; ws[71136] = kk * y[4736]; ws[71168] = kk * y[2368]; }
    { const double kk = ws[43616]; ws[71200] = kk * y[4640]; ws[71232] = kk * y[2368]; }
    { const double kk = ws[43648]; ws[71264] = kk * y[4160]; ws[71296] = kk * y[2368]; }
    { const double kk = ws[43712]; ws[71328] = kk * y[4544]; ws[71360] = kk * y[2368]; }
    { const double kk = ws[43744]; ws[71392] = kk * y[4736]; ws[71424] = kk * y[2400]; }
    { const double kk = ws[43776]; ws[71456] = kk * y[4320]; ws[71488] = kk * y[2400]; }
    { const double kk = ws[43808]; ws[71520] = kk * y[4640]; ws[71552] = kk * y[2400]; }
    { const double kk = ws[43840]; ws[71584] = kk * y[4544]; ws[71616] = kk * y[2400]; }
    { const double kk = ws[43872]; ws[71648] = kk * y[4736]; ws[71680] = kk * y[2432]; }
    { const double kk = ws[43904]; ws[71712] = kk * y[4320]; ws[71744] = kk * y[2432]; }
    { const double kk = ws[43936]; ws[71776] = kk * y[4640]; ws[71808] = kk * y[2432]; }
    { const double kk = ws[44000]; ws[71840] = kk * y[4544]; ws[71872] = kk * y[2432]; }
    { const double kk = ws[44032]; ws[71904] = kk * y[4736]; ws[71936] = kk * y[2976]; }
    { const double kk = ws[44064]; ws[71968] = kk * y[4320]; ws[72000] = kk * y[2976]; }
    { const double kk = ws[44096]; ws[72032] = kk * y[4640]; ws[72064] = kk * y[2976]; }
    { const double kk = ws[44160]; ws[72096] = kk * y[4544]; ws[72128] = kk * y[2976]; }
    { const double kk = ws[44192]; ws[72160] = kk * y[4736]; ws[72192] = kk * y[1536]; }
    { const double kk = ws[44224]; ws[72224] = kk * y[4544]; ws[72256] = kk * y[1536]; }
    { const double kk = ws[44256]; ws[72288] = kk * y[4320]; ws[72320] = kk * y[3008]; }
    { const double kk = ws[44288]; ws[72352] = kk * y[1184]; ws[72384] = kk * y[3008]; }
    { const double kk = ws[44320]; ws[72416] = kk * y[3456]; ws[72448] = kk * y[3008]; }
    { const double kk = ws[44352]; ws[72480] = kk * y[4736]; ws[72512] = kk * y[3008]; }
    { const double kk = ws[44384]; ws[72544] = kk * y[4544]; ws[72576] = kk * y[3008]; }
    { const double kk = ws[44416]; ws[72608] = kk * y[4736]; ws[72640] = kk * y[2016]; }
    { const double kk = ws[44448]; ws[72672] = kk * y[4736]; ws[72704] = kk * y[2016]; }
    { const double kk = ws[44480]; ws[72736] = kk * y[4640]; ws[72768] = kk * y[2016]; }
    { const double kk = ws[44512]; ws[72800] = kk * y[4544]; ws[72832] = kk * y[2016]; }
}
// Partial-derivative products of 2- and 3-reactant reactions (grpderiv.F:163-189).
__device__ __noinline__ void gear_explic_0(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
#define CEFF_(v) ((v) <= 1.0e-30 ? 0.0 : (v))
    { const double kk = ws[33440]; ws[55712] = kk * CEFF_(y[4384]); ws[55744] = kk * CEFF_(y[4320]); }
    { const double kk = ws[33472]; ws[55776] = kk * CEFF_(y[4384]); ws[55808] = kk * CEFF_(y[4160]); }
    { const double kk = ws[33504]; ws[55840] = kk * CEFF_(y[4608]); ws[55872] = kk * CEFF_(y[4160]); }
    { const double kk = ws[33536]; ws[55904] = kk * CEFF_(y[4608]); ws[55936] = kk * CEFF_(y[4160]); }
    { const double kk = ws[33568]; ws[55968] = kk * CEFF_(y[4320]); ws[56000] = kk * CEFF_(y[4160]); }
    { const double kk = ws[33728]; ws[56032] = kk * CEFF_(y[4736]); ws[56064] = kk * CEFF_(y[4320]); }
    { const double kk = ws[33760]; ws[56096] = kk * CEFF_(y[4704]); ws[56128] = kk * CEFF_(y[4320]); }
    { const double kk = ws[33792]; ws[56160] = kk * CEFF_(y[4160]); ws[56192] = kk * CEFF_(y[4736]); }
    { const double kk = ws[33824]; ws[56224] = kk * CEFF_(y[4160]); ws[56256] = kk * CEFF_(y[4704]); }
    { const double kk = ws[33856]; ws[56288] = kk * CEFF_(y[4736]); ws[56320] = kk * CEFF_(y[4736]); }
    { const double kk = ws[33888]; ws[56352] = kk * CEFF_(y[4736]); ws[56384] = kk * CEFF_(y[4736]); }
    { const double kk = ws[33920]; ws[56416] = kk * CEFF_(y[4704]); ws[56448] = kk * CEFF_(y[4736]); }
    { const double kk = ws[33952]; ws[56480] = kk * CEFF_(y[4704]); ws[56512] = kk * CEFF_(y[4704]); }
    { const double kk = ws[33984]; ws[56544] = kk * CEFF_(y[4704]); ws[56576] = kk * CEFF_(y[4704]); }
    { const double kk = ws[34048]; ws[56608] = kk * CEFF_(y[4736]); ws[56640] = kk * CEFF_(y[3456]); }
    { const double kk = ws[34080]; ws[56672] = kk * CEFF_(y[4160]); ws[56704] = kk * CEFF_(y[3456]); }
    { const double kk = ws[34112]; ws[56736] = kk * CEFF_(y[4384]); ws[56768] = kk * CEFF_(y[4384]); }
    { const double kk = ws[34144]; ws[56800] = kk * CEFF_(y[4384]); ws[56832] = kk * CEFF_(y[4704]); }
    { const double kk = ws[34176]; ws[56864] = kk * CEFF_(y[4320]); ws[56896] = kk * CEFF_(y[4608]); }
    { const double kk = ws[34272]; ws[56928] = kk * CEFF_(y[4384]); ws[56960] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34304]; ws[56992] = kk * CEFF_(y[4608]); ws[57024] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34336]; ws[57056] = kk * CEFF_(y[4160]); ws[57088] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34368]; ws[57120] = kk * CEFF_(y[4736]); ws[57152] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34400]; ws[57184] = kk * CEFF_(y[4704]); ws[57216] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34432]; ws[57248] = kk * CEFF_(y[4320]); ws[57280] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34464]; ws[57312] = kk * CEFF_(y[4640]); ws[57344] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34496]; ws[57376] = kk * CEFF_(y[4608]); ws[57408] = kk * CEFF_(y[4640]); }
    { const double kk = ws[34624]; ws[57440] = kk * CEFF_(y[4736]); ws[57472] = kk * CEFF_(y[4384]); }
    { const double kk = ws[34656]; ws[57504] = kk * CEFF_(y[4608]); ws[57536] = kk * CEFF_(y[4384]); }
    { const double kk = ws[34688]; ws[57568] = kk * CEFF_(y[2464]); ws[57600] = kk * CEFF_(y[2464]); }
    { const double kk = ws[34752]; ws[57632] = kk * CEFF_(y[4736]); ws[57664] = kk * CEFF_(y[2464]); }
    { const double kk = ws[34784]; ws[57696] = kk * CEFF_(y[4736]); ws[57728] = kk * CEFF_(y[4608]); }
    { const double kk = ws[34816]; ws[57760] = kk * CEFF_(y[4736]); ws[57792] = kk * CEFF_(y[4192]); }
    { const double kk = ws[34880]; ws[57824] = kk * CEFF_(y[4608]); ws[57856] = kk * CEFF_(y[4704]); }
    { const double kk = ws[34976]; ws[57888] = kk * CEFF_(y[4736]); ws[57920] = kk * CEFF_(y[1696]); }
    { const double kk = ws[35008]; ws[57952] = kk * CEFF_(y[4736]); ws[57984] = kk * CEFF_(y[2208]); }
    { const double kk = ws[35040]; ws[58016] = kk * CEFF_(y[4384]); ws[58048] = kk * CEFF_(y[4448]); }
    { const double kk = ws[35072]; ws[58080] = kk * CEFF_(y[4608]); ws[58112] = kk * CEFF_(y[4448]); }
    { const double kk = ws[35168]; ws[58144] = kk * CEFF_(y[4704]); ws[58176] = kk * CEFF_(y[4448]); }
    { const double kk = ws[35200]; ws[58208] = kk * CEFF_(y[4672]); ws[58240] = kk * CEFF_(y[4448]); }
    { const double kk = ws[35232]; ws[58272] = kk * CEFF_(y[4448]); ws[58304] = kk * CEFF_(y[4448]); }
    { const double kk = ws[35264]; ws[58336] = kk * CEFF_(y[4096]); ws[58368] = kk * CEFF_(y[4448]); }
    { const double kk = ws[35296]; ws[58400] = kk * CEFF_(y[4384]); ws[58432] = kk * CEFF_(y[4096]); }
    { const double kk = ws[35328]; ws[58464] = kk * CEFF_(y[4608]); ws[58496] = kk * CEFF_(y[4096]); }
    { const double kk = ws[35424]; ws[58528] = kk * CEFF_(y[4704]); ws[58560] = kk * CEFF_(y[4096]); }
    { const double kk = ws[35456]; ws[58592] = kk * CEFF_(y[4672]); ws[58624] = kk * CEFF_(y[4096]); }
    { const double kk = ws[35488]; ws[58656] = kk * CEFF_(y[4096]); ws[58688] = kk * CEFF_(y[4096]); }
    { const double kk = ws[35520]; ws[58720] = kk * CEFF_(y[4384]); ws[58752] = kk * CEFF_(y[4672]); }
    { const double kk = ws[35552]; ws[58784] = kk * CEFF_(y[4704]); ws[58816] = kk * CEFF_(y[4672]); }
    { const double kk = ws[35584]; ws[58848] = kk * CEFF_(y[4672]); ws[58880] = kk * CEFF_(y[4672]); }
    { const double kk = ws[35616]; ws[58912] = kk * CEFF_(y[4384]); ws[58944] = kk * CEFF_(y[4416]); }
    { const double kk = ws[35648]; ws[58976] = kk * CEFF_(y[4704]); ws[59008] = kk * CEFF_(y[4416]); }
    { const double kk = ws[35680]; ws[59040] = kk * CEFF_(y[4448]); ws[59072] = kk * CEFF_(y[4416]); }
    { const double kk = ws[35712]; ws[59104] = kk * CEFF_(y[4672]); ws[59136] = kk * CEFF_(y[4416]); }
    { const double kk = ws[35744]; ws[59168] = kk * CEFF_(y[4384]); ws[59200] = kk * CEFF_(y[4576]); }
    { const double kk = ws[35776]; ws[59232] = kk * CEFF_(y[4704]); ws[59264] = kk * CEFF_(y[4576]); }
    { const double kk = ws[35808]; ws[59296] = kk * CEFF_(y[4448]); ws[59328] = kk * CEFF_(y[4576]); }
    { const double kk = ws[35840]; ws[59360] = kk * CEFF_(y[4672]); ws[59392] = kk * CEFF_(y[4576]); }
    { const double kk = ws[35872]; ws[59424] = kk * CEFF_(y[4384]); ws[59456] = kk * CEFF_(y[4352]); }
    { const double kk = ws[35904]; ws[59488] = kk * CEFF_(y[4704]); ws[59520] = kk * CEFF_(y[4352]); }
    { const double kk = ws[35936]; ws[59552] = kk * CEFF_(y[4448]); ws[59584] = kk * CEFF_(y[4352]); }
    { const double kk = ws[35968]; ws[59616] = kk * CEFF_(y[4672]); ws[59648] = kk * CEFF_(y[4352]); }
    { const double kk = ws[36000]; ws[59680] = kk * CEFF_(y[4384]); ws[59712] = kk * CEFF_(y[4288]); }
    { const double kk = ws[36032]; ws[59744] = kk * CEFF_(y[4704]); ws[59776] = kk * CEFF_(y[4288]); }
    { const double kk = ws[36064]; ws[59808] = kk * CEFF_(y[4448]); ws[59840] = kk * CEFF_(y[4288]); }
    { const double kk = ws[36096]; ws[59872] = kk * CEFF_(y[4672]); ws[59904] = kk * CEFF_(y[4288]); }
    { const double kk = ws[36128]; ws[59936] = kk * CEFF_(y[4736]); ws[59968] = kk * CEFF_(y[2272]); }
    { const double kk = ws[36192]; ws[60000] = kk * CEFF_(y[4736]); ws[60032] = kk * CEFF_(y[2880]); }
    { const double kk = ws[36256]; ws[60064] = kk * CEFF_(y[4736]); ws[60096] = kk * CEFF_(y[3648]); }
    { const double kk = ws[36320]; ws[60128] = kk * CEFF_(y[4736]); ws[60160] = kk * CEFF_(y[3776]); }
    { const double kk = ws[36352]; ws[60192] = kk * CEFF_(y[4736]); ws[60224] = kk * CEFF_(y[3904]); }
    { const double kk = ws[36384]; ws[60256] = kk * CEFF_(y[4736]); ws[60288] = kk * CEFF_(y[2688]); }
    { const double kk = ws[36416]; ws[60320] = kk * CEFF_(y[4736]); ws[60352] = kk * CEFF_(y[4512]); }
    { const double kk = ws[36512]; ws[60384] = kk * CEFF_(y[4160]); ws[60416] = kk * CEFF_(y[4512]); }
    { const double kk = ws[36544]; ws[60448] = kk * CEFF_(y[4640]); ws[60480] = kk * CEFF_(y[4512]); }
    { const double kk = ws[36576]; ws[60512] = kk * CEFF_(y[4704]); ws[60544] = kk * CEFF_(y[4512]); }
    { const double kk = ws[36640]; ws[60576] = kk * CEFF_(y[4384]); ws[60608] = kk * CEFF_(y[1728]); }
    { const double kk = ws[36672]; ws[60640] = kk * CEFF_(y[4704]); ws[60672] = kk * CEFF_(y[1728]); }
    { const double kk = ws[36704]; ws[60704] = kk * CEFF_(y[4160]); ws[60736] = kk * CEFF_(y[4128]); }
    { const double kk = ws[36736]; ws[60768] = kk * CEFF_(y[4736]); ws[60800] = kk * CEFF_(y[4128]); }
    { const double kk = ws[36768]; ws[60832] = kk * CEFF_(y[4640]); ws[60864] = kk * CEFF_(y[4128]); }
    { const double kk = ws[36832]; ws[60896] = kk * CEFF_(y[4160]); ws[60928] = kk * CEFF_(y[4064]); }
    { const double kk = ws[36864]; ws[60960] = kk * CEFF_(y[4736]); ws[60992] = kk * CEFF_(y[4064]); }
    { const double kk = ws[36896]; ws[61024] = kk * CEFF_(y[4640]); ws[61056] = kk * CEFF_(y[4064]); }
    { const double kk = ws[36960]; ws[61088] = kk * CEFF_(y[4736]); ws[61120] = kk * CEFF_(y[3840]); }
    { const double kk = ws[37024]; ws[61152] = kk * CEFF_(y[4640]); ws[61184] = kk * CEFF_(y[3840]); }
    { const double kk = ws[37056]; ws[61216] = kk * CEFF_(y[4736]); ws[61248] = kk * CEFF_(y[4256]); }
    { const double kk = ws[37120]; ws[61280] = kk * CEFF_(y[4640]); ws[61312] = kk * CEFF_(y[4256]); }
    { const double kk = ws[37184]; ws[61344] = kk * CEFF_(y[4640]); ws[61376] = kk * CEFF_(y[4000]); }
    { const double kk = ws[37216]; ws[61408] = kk * CEFF_(y[4736]); ws[61440] = kk * CEFF_(y[4000]); }
    { const double kk = ws[37280]; ws[61472] = kk * CEFF_(y[4736]); ws[61504] = kk * CEFF_(y[4480]); }
    { const double kk = ws[37344]; ws[61536] = kk * CEFF_(y[4736]); ws[61568] = kk * CEFF_(y[832]); }
    { const double kk = ws[37376]; ws[61600] = kk * CEFF_(y[4736]); ws[61632] = kk * CEFF_(y[2720]); }
    { const double kk = ws[37408]; ws[61664] = kk * CEFF_(y[4736]); ws[61696] = kk * CEFF_(y[864]); }
    { const double kk = ws[37504]; ws[61728] = kk * CEFF_(y[4736]); ws[61760] = kk * CEFF_(y[3392]); }
    { const double kk = ws[37536]; ws[61792] = kk * CEFF_(y[4736]); ws[61824] = kk * CEFF_(y[896]); }
    { const double kk = ws[37568]; ws[61856] = kk * CEFF_(y[4736]); ws[61888] = kk * CEFF_(y[4224]); }
    { const double kk = ws[37664]; ws[61920] = kk * CEFF_(y[4608]); ws[61952] = kk * CEFF_(y[960]); }
    { const double kk = ws[37696]; ws[61984] = kk * CEFF_(y[4736]); ws[62016] = kk * CEFF_(y[352]); }
    { const double kk = ws[37728]; ws[62048] = kk * CEFF_(y[4160]); ws[62080] = kk * CEFF_(y[2656]); }
    { const double kk = ws[37760]; ws[62112] = kk * CEFF_(y[4736]); ws[62144] = kk * CEFF_(y[2656]); }
    { const double kk = ws[37792]; ws[62176] = kk * CEFF_(y[4320]); ws[62208] = kk * CEFF_(y[2656]); }
    { const double kk = ws[37824]; ws[62240] = kk * CEFF_(y[4640]); ws[62272] = kk * CEFF_(y[2656]); }
    { const double kk = ws[37856]; ws[62304] = kk * CEFF_(y[4160]); ws[62336] = kk * CEFF_(y[3552]); }
    { const double kk = ws[37888]; ws[62368] = kk * CEFF_(y[4736]); ws[62400] = kk * CEFF_(y[3552]); }
    { const double kk = ws[37920]; ws[62432] = kk * CEFF_(y[4320]); ws[62464] = kk * CEFF_(y[3552]); }
    { const double kk = ws[37952]; ws[62496] = kk * CEFF_(y[4640]); ws[62528] = kk * CEFF_(y[3552]); }
    { const double kk = ws[37984]; ws[62560] = kk * CEFF_(y[4160]); ws[62592] = kk * CEFF_(y[3136]); }
    { const double kk = ws[38016]; ws[62624] = kk * CEFF_(y[4736]); ws[62656] = kk * CEFF_(y[3136]); }
    { const double kk = ws[38048]; ws[62688] = kk * CEFF_(y[4320]); ws[62720] = kk * CEFF_(y[3136]); }
    { const double kk = ws[38080]; ws[62752] = kk * CEFF_(y[4640]); ws[62784] = kk * CEFF_(y[3136]); }
    { const double kk = ws[38112]; ws[62816] = kk * CEFF_(y[4736]); ws[62848] = kk * CEFF_(y[2528]); }
    { const double kk = ws[38144]; ws[62880] = kk * CEFF_(y[4160]); ws[62912] = kk * CEFF_(y[2528]); }
    { const double kk = ws[38176]; ws[62944] = kk * CEFF_(y[4384]); ws[62976] = kk * CEFF_(y[3424]); }
    { const double kk = ws[38208]; ws[63008] = kk * CEFF_(y[4704]); ws[63040] = kk * CEFF_(y[3424]); }
    { const double kk = ws[38240]; ws[63072] = kk * CEFF_(y[4448]); ws[63104] = kk * CEFF_(y[3424]); }
    { const double kk = ws[38272]; ws[63136] = kk * CEFF_(y[4672]); ws[63168] = kk * CEFF_(y[3424]); }
    { const double kk = ws[38336]; ws[63200] = kk * CEFF_(y[4320]); ws[63232] = kk * CEFF_(y[2528]); }
    { const double kk = ws[38368]; ws[63264] = kk * CEFF_(y[4640]); ws[63296] = kk * CEFF_(y[2528]); }
    { const double kk = ws[38400]; ws[63328] = kk * CEFF_(y[4736]); ws[63360] = kk * CEFF_(y[3872]); }
    { const double kk = ws[38432]; ws[63392] = kk * CEFF_(y[4320]); ws[63424] = kk * CEFF_(y[3872]); }
    { const double kk = ws[38464]; ws[63456] = kk * CEFF_(y[4640]); ws[63488] = kk * CEFF_(y[3872]); }
    { const double kk = ws[38528]; ws[63520] = kk * CEFF_(y[4736]); ws[63552] = kk * CEFF_(y[1664]); }
    { const double kk = ws[38592]; ws[63584] = kk * CEFF_(y[4640]); ws[63616] = kk * CEFF_(y[1024]); }
    { const double kk = ws[38624]; ws[63648] = kk * CEFF_(y[4736]); ws[63680] = kk * CEFF_(y[1056]); }
    { const double kk = ws[38656]; ws[63712] = kk * CEFF_(y[4704]); ws[63744] = kk * CEFF_(y[3296]); }
    { const double kk = ws[38688]; ws[63776] = kk * CEFF_(y[4384]); ws[63808] = kk * CEFF_(y[3296]); }
    { const double kk = ws[38720]; ws[63840] = kk * CEFF_(y[4448]); ws[63872] = kk * CEFF_(y[3296]); }
    { const double kk = ws[38752]; ws[63904] = kk * CEFF_(y[4672]); ws[63936] = kk * CEFF_(y[3296]); }
    { const double kk = ws[38784]; ws[63968] = kk * CEFF_(y[4736]); ws[64000] = kk * CEFF_(y[1632]); }
    { const double kk = ws[38816]; ws[64032] = kk * CEFF_(y[4160]); ws[64064] = kk * CEFF_(y[2048]); }
    { const double kk = ws[38848]; ws[64096] = kk * CEFF_(y[4736]); ws[64128] = kk * CEFF_(y[2048]); }
    { const double kk = ws[38880]; ws[64160] = kk * CEFF_(y[4320]); ws[64192] = kk * CEFF_(y[2048]); }
    { const double kk = ws[38912]; ws[64224] = kk * CEFF_(y[4640]); ws[64256] = kk * CEFF_(y[2048]); }
    { const double kk = ws[38944]; ws[64288] = kk * CEFF_(y[4160]); ws[64320] = kk * CEFF_(y[2112]); }
    { const double kk = ws[38976]; ws[64352] = kk * CEFF_(y[4736]); ws[64384] = kk * CEFF_(y[2112]); }
    { const double kk = ws[39008]; ws[64416] = kk * CEFF_(y[4320]); ws[64448] = kk * CEFF_(y[2112]); }
    { const double kk = ws[39040]; ws[64480] = kk * CEFF_(y[4640]); ws[64512] = kk * CEFF_(y[2112]); }
    { const double kk = ws[39072]; ws[64544] = kk * CEFF_(y[4736]); ws[64576] = kk * CEFF_(y[384]); }
    { const double kk = ws[39104]; ws[64608] = kk * CEFF_(y[4384]); ws[64640] = kk * CEFF_(y[3104]); }
    { const double kk = ws[39136]; ws[64672] = kk * CEFF_(y[4448]); ws[64704] = kk * CEFF_(y[3104]); }
    { const double kk = ws[39168]; ws[64736] = kk * CEFF_(y[4704]); ws[64768] = kk * CEFF_(y[3104]); }
    { const double kk = ws[39200]; ws[64800] = kk * CEFF_(y[4672]); ws[64832] = kk * CEFF_(y[3104]); }
    { const double kk = ws[39232]; ws[64864] = kk * CEFF_(y[4736]); ws[64896] = kk * CEFF_(y[1088]); }
    { const double kk = ws[39264]; ws[64928] = kk * CEFF_(y[4384]); ws[64960] = kk * CEFF_(y[3488]); }
    { const double kk = ws[39296]; ws[64992] = kk * CEFF_(y[4448]); ws[65024] = kk * CEFF_(y[3488]); }
    { const double kk = ws[39328]; ws[65056] = kk * CEFF_(y[4704]); ws[65088] = kk * CEFF_(y[3488]); }
    { const double kk = ws[39360]; ws[65120] = kk * CEFF_(y[4672]); ws[65152] = kk * CEFF_(y[3488]); }
    { const double kk = ws[39392]; ws[65184] = kk * CEFF_(y[4736]); ws[65216] = kk * CEFF_(y[1120]); }
    { const double kk = ws[39424]; ws[65248] = kk * CEFF_(y[4736]); ws[65280] = kk * CEFF_(y[1152]); }
    { const double kk = ws[39456]; ws[65312] = kk * CEFF_(y[4384]); ws[65344] = kk * CEFF_(y[3584]); }
    { const double kk = ws[39488]; ws[65376] = kk * CEFF_(y[4704]); ws[65408] = kk * CEFF_(y[3584]); }
    { const double kk = ws[39520]; ws[65440] = kk * CEFF_(y[4448]); ws[65472] = kk * CEFF_(y[3584]); }
    { const double kk = ws[39552]; ws[65504] = kk * CEFF_(y[4672]); ws[65536] = kk * CEFF_(y[3584]); }
    { const double kk = ws[39584]; ws[65568] = kk * CEFF_(y[4736]); ws[65600] = kk * CEFF_(y[3616]); }
    { const double kk = ws[39616]; ws[65632] = kk * CEFF_(y[4640]); ws[65664] = kk * CEFF_(y[3616]); }
    { const double kk = ws[39648]; ws[65696] = kk * CEFF_(y[4608]); ws[65728] = kk * CEFF_(y[3328]); }
    { const double kk = ws[39680]; ws[65760] = kk * CEFF_(y[4704]); ws[65792] = kk * CEFF_(y[3328]); }
    { const double kk = ws[39712]; ws[65824] = kk * CEFF_(y[4736]); ws[65856] = kk * CEFF_(y[2176]); }
    { const double kk = ws[39744]; ws[65888] = kk * CEFF_(y[4640]); ws[65920] = kk * CEFF_(y[2176]); }
    { const double kk = ws[39840]; ws[65952] = kk * CEFF_(y[4736]); ws[65984] = kk * CEFF_(y[3808]); }
    { const double kk = ws[39872]; ws[66016] = kk * CEFF_(y[4320]); ws[66048] = kk * CEFF_(y[3808]); }
    { const double kk = ws[39904]; ws[66080] = kk * CEFF_(y[4640]); ws[66112] = kk * CEFF_(y[3808]); }
    { const double kk = ws[39968]; ws[66144] = kk * CEFF_(y[4736]); ws[66176] = kk * CEFF_(y[3936]); }
    { const double kk = ws[40000]; ws[66208] = kk * CEFF_(y[4320]); ws[66240] = kk * CEFF_(y[3936]); }
    { const double kk = ws[40032]; ws[66272] = kk * CEFF_(y[4640]); ws[66304] = kk * CEFF_(y[3936]); }
    { const double kk = ws[40064]; ws[66336] = kk * CEFF_(y[4736]); ws[66368] = kk * CEFF_(y[1760]); }
    { const double kk = ws[40096]; ws[66400] = kk * CEFF_(y[4640]); ws[66432] = kk * CEFF_(y[1760]); }
    { const double kk = ws[40128]; ws[66464] = kk * CEFF_(y[4384]); ws[66496] = kk * CEFF_(y[3744]); }
    { const double kk = ws[40160]; ws[66528] = kk * CEFF_(y[4608]); ws[66560] = kk * CEFF_(y[3744]); }
    { const double kk = ws[40224]; ws[66592] = kk * CEFF_(y[4704]); ws[66624] = kk * CEFF_(y[3744]); }
    { const double kk = ws[40256]; ws[66656] = kk * CEFF_(y[4448]); ws[66688] = kk * CEFF_(y[3744]); }
    { const double kk = ws[40288]; ws[66720] = kk * CEFF_(y[4672]); ws[66752] = kk * CEFF_(y[3744]); }
    { const double kk = ws[40320]; ws[66784] = kk * CEFF_(y[4736]); ws[66816] = kk * CEFF_(y[1792]); }
    { const double kk = ws[40352]; ws[66848] = kk * CEFF_(y[4736]); ws[66880] = kk * CEFF_(y[1952]); }
    { const double kk = ws[40384]; ws[66912] = kk * CEFF_(y[4736]); ws[66944] = kk * CEFF_(y[416]); }
    { const double kk = ws[40544]; ws[66976] = kk * CEFF_(y[4736]); ws[67008] = kk * CEFF_(y[4608]); }
    { const double kk = ws[40640]; ws[67040] = kk * CEFF_(y[4320]); ws[67072] = kk * CEFF_(y[4544]); }
    { const double kk = ws[40672]; ws[67104] = kk * CEFF_(y[3520]); ws[67136] = kk * CEFF_(y[3520]); }
    { const double kk = ws[40704]; ws[67168] = kk * CEFF_(y[4384]); ws[67200] = kk * CEFF_(y[3520]); }
    { const double kk = ws[40736]; ws[67232] = kk * CEFF_(y[4704]); ws[67264] = kk * CEFF_(y[3520]); }
    { const double kk = ws[40768]; ws[67296] = kk * CEFF_(y[4416]); ws[67328] = kk * CEFF_(y[3520]); }
    { const double kk = ws[40800]; ws[67360] = kk * CEFF_(y[3232]); ws[67392] = kk * CEFF_(y[4736]); }
    { const double kk = ws[40896]; ws[67424] = kk * CEFF_(y[4224]); ws[67456] = kk * CEFF_(y[4544]); }
    { const double kk = ws[40928]; ws[67488] = kk * CEFF_(y[896]); ws[67520] = kk * CEFF_(y[4544]); }
    { const double kk = ws[40960]; ws[67552] = kk * CEFF_(y[832]); ws[67584] = kk * CEFF_(y[4544]); }
    { const double kk = ws[40992]; ws[67616] = kk * CEFF_(y[2656]); ws[67648] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41024]; ws[67680] = kk * CEFF_(y[3552]); ws[67712] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41056]; ws[67744] = kk * CEFF_(y[3136]); ws[67776] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41088]; ws[67808] = kk * CEFF_(y[2528]); ws[67840] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41120]; ws[67872] = kk * CEFF_(y[4512]); ws[67904] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41152]; ws[67936] = kk * CEFF_(y[4128]); ws[67968] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41184]; ws[68000] = kk * CEFF_(y[4064]); ws[68032] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41216]; ws[68064] = kk * CEFF_(y[2720]); ws[68096] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41248]; ws[68128] = kk * CEFF_(y[864]); ws[68160] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41280]; ws[68192] = kk * CEFF_(y[4736]); ws[68224] = kk * CEFF_(y[3968]); }
    { const double kk = ws[41312]; ws[68256] = kk * CEFF_(y[1088]); ws[68288] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41344]; ws[68320] = kk * CEFF_(y[1120]); ws[68352] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41376]; ws[68384] = kk * CEFF_(y[1152]); ws[68416] = kk * CEFF_(y[4544]); }
    { const double kk = ws[41440]; ws[68448] = kk * CEFF_(y[4608]); ws[68480] = kk * CEFF_(y[3520]); }
    { const double kk = ws[41600]; ws[68512] = kk * CEFF_(y[4384]); ws[68544] = kk * CEFF_(y[2944]); }
    { const double kk = ws[41632]; ws[68576] = kk * CEFF_(y[4704]); ws[68608] = kk * CEFF_(y[2944]); }
    { const double kk = ws[41664]; ws[68640] = kk * CEFF_(y[4384]); ws[68672] = kk * CEFF_(y[2496]); }
    { const double kk = ws[41696]; ws[68704] = kk * CEFF_(y[4704]); ws[68736] = kk * CEFF_(y[2496]); }
    { const double kk = ws[41728]; ws[68768] = kk * CEFF_(y[4384]); ws[68800] = kk * CEFF_(y[2144]); }
    { const double kk = ws[41760]; ws[68832] = kk * CEFF_(y[4704]); ws[68864] = kk * CEFF_(y[2144]); }
    { const double kk = ws[41792]; ws[68896] = kk * CEFF_(y[4320]); ws[68928] = kk * CEFF_(y[1856]); }
    { const double kk = ws[41824]; ws[68960] = kk * CEFF_(y[4736]); ws[68992] = kk * CEFF_(y[1856]); }
    { const double kk = ws[41856]; ws[69024] = kk * CEFF_(y[4640]); ws[69056] = kk * CEFF_(y[1856]); }
    { const double kk = ws[41888]; ws[69088] = kk * CEFF_(y[4384]); ws[69120] = kk * CEFF_(y[2560]); }
    { const double kk = ws[41920]; ws[69152] = kk * CEFF_(y[4704]); ws[69184] = kk * CEFF_(y[2560]); }
    { const double kk = ws[41952]; ws[69216] = kk * CEFF_(y[4736]); ws[69248] = kk * CEFF_(y[448]); }
    { const double kk = ws[42144]; ws[69280] = kk * CEFF_(y[480]); ws[69312] = kk * CEFF_(y[1920]); }
    { const double kk = ws[42176]; ws[69344] = kk * CEFF_(y[512]); ws[69376] = kk * CEFF_(y[1920]); }
    { const double kk = ws[42208]; ws[69408] = kk * CEFF_(y[544]); ws[69440] = kk * CEFF_(y[1248]); }
    { const double kk = ws[42336]; ws[69472] = kk * CEFF_(y[576]); ws[69504] = kk * CEFF_(y[1312]); }
    { const double kk = ws[42464]; ws[69536] = kk * CEFF_(y[4384]); ws[69568] = kk * CEFF_(y[2848]); }
    { const double kk = ws[42496]; ws[69600] = kk * CEFF_(y[4704]); ws[69632] = kk * CEFF_(y[2848]); }
    { const double kk = ws[42528]; ws[69664] = kk * CEFF_(y[4640]); ws[69696] = kk * CEFF_(y[2848]); }
    { const double kk = ws[42560]; ws[69728] = kk * CEFF_(y[4672]); ws[69760] = kk * CEFF_(y[2848]); }
    { const double kk = ws[42592]; ws[69792] = kk * CEFF_(y[4544]); ws[69824] = kk * CEFF_(y[3360]); }
    { const double kk = ws[42624]; ws[69856] = kk * CEFF_(y[4736]); ws[69888] = kk * CEFF_(y[3360]); }
    { const double kk = ws[42912]; ws[69920] = kk * CEFF_(y[4736]); ws[69952] = kk * CEFF_(y[704]); }
    { const double kk = ws[42944]; ws[69984] = kk * CEFF_(y[4736]); ws[70016] = kk * CEFF_(y[1440]); }
    { const double kk = ws[42976]; ws[70048] = kk * CEFF_(y[4736]); ws[70080] = kk * CEFF_(y[736]); }
    { const double kk = ws[43008]; ws[70112] = kk * CEFF_(y[4736]); ws[70144] = kk * CEFF_(y[1472]); }
    { const double kk = ws[43040]; ws[70176] = kk * CEFF_(y[4736]); ws[70208] = kk * CEFF_(y[768]); }
    { const double kk = ws[43072]; ws[70240] = kk * CEFF_(y[4736]); ws[70272] = kk * CEFF_(y[2752]); }
    { const double kk = ws[43104]; ws[70304] = kk * CEFF_(y[4736]); ws[70336] = kk * CEFF_(y[2784]); }
    { const double kk = ws[43136]; ws[70368] = kk * CEFF_(y[4736]); ws[70400] = kk * CEFF_(y[2816]); }
    { const double kk = ws[43168]; ws[70432] = kk * CEFF_(y[4736]); ws[70464] = kk * CEFF_(y[2304]); }
    { const double kk = ws[43200]; ws[70496] = kk * CEFF_(y[4736]); ws[70528] = kk * CEFF_(y[1504]); }
    { const double kk = ws[43232]; ws[70560] = kk * CEFF_(y[4736]); ws[70592] = kk * CEFF_(y[3680]); }
    { const double kk = ws[43264]; ws[70624] = kk * CEFF_(y[4736]); ws[70656] = kk * CEFF_(y[3712]); }
    { const double kk = ws[43296]; ws[70688] = kk * CEFF_(y[4736]); ws[70720] = kk * CEFF_(y[2912]); }
    { const double kk = ws[43328]; ws[70752] = kk * CEFF_(y[4736]); ws[70784] = kk * CEFF_(y[3168]); }
    { const double kk = ws[43360]; ws[70816] = kk * CEFF_(y[4736]); ws[70848] = kk * CEFF_(y[3200]); }
    { const double kk = ws[43392]; ws[70880] = kk * CEFF_(y[4736]); ws[70912] = kk * CEFF_(y[2336]); }
    { const double kk = ws[43424]; ws[70944] = kk * CEFF_(y[4640]); ws[70976] = kk * CEFF_(y[2336]); }
    { const double kk = ws[43456]; ws[71008] = kk * CEFF_(y[4160]); ws[71040] = kk * CEFF_(y[2336]); }
    { const double kk = ws[43552]; ws[71072] = kk * CEFF_(y[4544]); ws[71104] = kk * CEFF_(y[2336]); }
    { const double kk = ws[43584]; ws[71136] = kk * CEFF_(y[4736]); ws[71168] = kk * CEFF_(y[2368]); }
    { const double kk = ws[43616]; ws[71200] = kk * CEFF_(y[4640]); ws[71232] = kk * CEFF_(y[2368]); }
    { const double kk = ws[43648]; ws[71264] = kk * CEFF_(y[4160]); ws[71296] = kk * CEFF_(y[2368]); }
    { const double kk = ws[43712]; ws[71328] = kk * CEFF_(y[4544]); ws[71360] = kk * CEFF_(y[2368]); }
    { const double kk = ws[43744]; ws[71392] = kk * CEFF_(y[4736]); ws[71424] = kk * CEFF_(y[2400]); }
    { const double kk = ws[43776]; ws[71456] = kk * CEFF_(y[4320]); ws[71488] = kk * CEFF_(y[2400]); }
    { const double kk = ws[43808]; ws[71520] = kk * CEFF_(y[4640]); ws[71552] = kk * CEFF_(y[2400]); }
    { const double kk = ws[43840]; ws[71584] = kk * CEFF_(y[4544]); ws[71616] = kk * CEFF_(y[2400]); }
    { const double kk = ws[43872]; ws[71648] = kk * CEFF_(y[4736]); ws[71680] = kk * CEFF_(y[2432]); }
    { const double kk = ws[43904]; ws[71712] = kk * CEFF_(y[4320]); ws[71744] = kk * CEFF_(y[2432]); }
    { const double kk = ws[43936]; ws[71776] = kk * CEFF_(y[4640]); ws[71808] = kk * CEFF_(y[2432]); }
    { const double kk = ws[44000]; ws[71840] = kk * CEFF_(y[4544]); ws[71872] = kk * CEFF_(y[2432]); }
    { const double kk = ws[44032]; ws[71904] = kk * CEFF_(y[4736]); ws[71936] = kk * CEFF_(y[2976]); }
    { const double kk = ws[44064]; ws[71968] = kk * CEFF_(y[4320]); ws[72000] = kk * CEFF_(y[2976]); }
    { const double kk = ws[44096]; ws[72032] = kk * CEFF_(y[4640]); ws[72064] = kk * CEFF_(y[2976]); }
    { const double kk = ws[44160]; ws[72096] = kk * CEFF_(y[4544]); ws[72128] = kk * CEFF_(y[2976]); }
    { const double kk = ws[44192]; ws[72160] = kk * CEFF_(y[4736]); ws[72192] = kk * CEFF_(y[1536]); }
    { const double kk = ws[44224]; ws[72224] = kk * CEFF_(y[4544]); ws[72256] = kk * CEFF_(y[1536]); }
    { const double kk = ws[44256]; ws[72288] = kk * CEFF_(y[4320]); ws[72320] = kk * CEFF_(y[3008]); }
    { const double kk = ws[44288]; ws[72352] = kk * CEFF_(y[1184]); ws[72384] = kk * CEFF_(y[3008]); }
    { const double kk = ws[44320]; ws[72416] = kk * CEFF_(y[3456]); ws[72448] = kk * CEFF_(y[3008]); }
    { const double kk = ws[44352]; ws[72480] = kk * CEFF_(y[4736]); ws[72512] = kk * CEFF_(y[3008]); }
    { const double kk = ws[44384]; ws[72544] = kk * CEFF_(y[4544]); ws[72576] = kk * CEFF_(y[3008]); }
    { const double kk = ws[44416]; ws[72608] = kk * CEFF_(y[4736]); ws[72640] = kk * CEFF_(y[2016]); }
    { const double kk = ws[44448]; ws[72672] = kk * CEFF_(y[4736]); ws[72704] = kk * CEFF_(y[2016]); }
    { const double kk = ws[44480]; ws[72736] = kk * CEFF_(y[4640]); ws[72768] = kk * CEFF_(y[2016]); }
    { const double kk = ws[44512]; ws[72800] = kk * CEFF_(y[4544]); ws[72832] = kk * CEFF_(y[2016]); }
#undef CEFF_
}
}  // namespace mech_cb6r5_ae7_aq
