// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {

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

__constant__ int c_inew2old[189] = {144, 147, 148, 184, 186, 47, 48, 49, 62, 67, 70, 72, 128, 129, 135, 142, 145, 146, 2, 149, 151, 153, 155, 157, 159, 161, 172, 176, 178, 183, 185, 187, 46, 143, 43, 54, 60, 8, 64, 66, 10, 74, 78, 79, 83, 86, 104, 105, 109, 131, 136, 76, 80, 45, 91, 101, 106, 110, 134, 50, 137, 162, 163, 164, 166, 168, 169, 171, 51, 81, 56, 125, 139, 1, 150, 152, 154, 156, 158, 160, 89, 99, 114, 116, 126, 127, 58, 75, 37, 92, 96, 97, 69, 108, 57, 111, 118, 71, 132, 133, 59, 36, 73, 68, 61, 65, 173, 177, 179, 188, 95, 130, 98, 53, 100, 41, 117, 85, 94, 102, 115, 20, 23, 88, 182, 3, 112, 113, 39, 27, 84, 87, 181, 119, 77, 34, 63, 44, 170, 35, 18, 122, 22, 24, 40, 175, 28, 167, 30, 180, 90, 138, 174, 121, 124, 140, 141, 9, 82, 165, 55, 93, 0, 29, 32, 25, 120, 26, 31, 52, 42, 33, 21, 123, 14, 103, 17, 13, 107, 38, 16, 19, 6, 12, 15, 5, 7, 11, 4};
__constant__ int c_iold2new[189] = {162, 73, 18, 125, 188, 185, 182, 186, 37, 157, 40, 187, 183, 177, 174, 184, 180, 176, 140, 181, 121, 172, 142, 122, 143, 165, 167, 129, 146, 163, 148, 168, 164, 171, 135, 139, 101, 88, 179, 128, 144, 115, 170, 34, 137, 53, 32, 5, 6, 7, 59, 68, 169, 113, 35, 160, 70, 94, 86, 100, 36, 104, 8, 136, 38, 105, 39, 9, 103, 92, 10, 97, 11, 102, 41, 87, 51, 134, 42, 43, 52, 69, 158, 44, 130, 117, 45, 131, 123, 80, 150, 54, 89, 161, 118, 110, 90, 91, 112, 81, 114, 55, 119, 175, 46, 47, 56, 178, 93, 48, 57, 95, 126, 127, 82, 120, 83, 116, 96, 133, 166, 153, 141, 173, 154, 71, 84, 85, 12, 13, 111, 49, 98, 99, 58, 14, 50, 60, 151, 72, 155, 156, 15, 33, 0, 16, 17, 1, 2, 19, 74, 20, 75, 21, 76, 22, 77, 23, 78, 24, 79, 25, 61, 62, 63, 159, 64, 147, 65, 66, 138, 67, 26, 106, 152, 145, 27, 107, 28, 108, 149, 132, 124, 29, 3, 30, 4, 31, 109};
// Rate constants of one cell into ws[OFF_RKI + r] (CALC_RCONST, RXNS_FUNC_MODULE.F90).
__device__ __noinline__ void rconst(double* __restrict__ ws, double temp_in, double press, double h2o,
                                    double seawater, int lsunlight, const double* __restrict__ rjv,
                                    const double* __restrict__ hetv)
{
    /* RKI = 0 (RXNS_FUNC_MODULE.F90 CALC_RCONST) */
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
    ws[44544] = 0.0;
    ws[44576] = 0.0;
    ws[44608] = 0.0;
    ws[44640] = 0.0;
    ws[44672] = 0.0;
    ws[44704] = 0.0;
    ws[44736] = 0.0;
    ws[44768] = 0.0;
    ws[44800] = 0.0;
    ws[44832] = 0.0;
    ws[44864] = 0.0;
    ws[44896] = 0.0;
    ws[44928] = 0.0;
    ws[44960] = 0.0;
    ws[44992] = 0.0;
    ws[45024] = 0.0;
    ws[45056] = 0.0;
    ws[45088] = 0.0;
    ws[45120] = 0.0;
    ws[45152] = 0.0;
    ws[45184] = 0.0;
    ws[45216] = 0.0;
    ws[45248] = 0.0;
    ws[45280] = 0.0;
    ws[45312] = 0.0;
    ws[45344] = 0.0;
    ws[45376] = 0.0;
    ws[45408] = 0.0;
    ws[45440] = 0.0;
    ws[45472] = 0.0;
    ws[45504] = 0.0;
    ws[45536] = 0.0;
    ws[45568] = 0.0;
    ws[45600] = 0.0;
    ws[45632] = 0.0;
    ws[45664] = 0.0;
    ws[45696] = 0.0;
    ws[45728] = 0.0;
    ws[45760] = 0.0;
    ws[45792] = 0.0;
    ws[45824] = 0.0;
    ws[45856] = 0.0;
    ws[45888] = 0.0;
    ws[45920] = 0.0;
    ws[45952] = 0.0;
    ws[45984] = 0.0;
    ws[46016] = 0.0;
    ws[46048] = 0.0;
    ws[46080] = 0.0;
    ws[46112] = 0.0;
    ws[46144] = 0.0;
    ws[46176] = 0.0;
    ws[46208] = 0.0;
    ws[46240] = 0.0;
    ws[46272] = 0.0;
    ws[46304] = 0.0;
    ws[46336] = 0.0;
    ws[46368] = 0.0;
    ws[46400] = 0.0;
    ws[46432] = 0.0;
    ws[46464] = 0.0;
    ws[46496] = 0.0;
    ws[46528] = 0.0;
    ws[46560] = 0.0;
    ws[46592] = 0.0;
    ws[46624] = 0.0;
    ws[46656] = 0.0;
    ws[46688] = 0.0;
    ws[46720] = 0.0;
    ws[46752] = 0.0;
    ws[46784] = 0.0;
    ws[46816] = 0.0;
    ws[46848] = 0.0;
    ws[46880] = 0.0;
    ws[46912] = 0.0;
    ws[46944] = 0.0;
    ws[46976] = 0.0;
    ws[47008] = 0.0;
    ws[47040] = 0.0;
    ws[47072] = 0.0;
    ws[47104] = 0.0;
    ws[47136] = 0.0;
    ws[47168] = 0.0;
    ws[47200] = 0.0;
    ws[47232] = 0.0;
    ws[47264] = 0.0;
    ws[47296] = 0.0;
    ws[47328] = 0.0;
    ws[47360] = 0.0;
    ws[47392] = 0.0;
    ws[47424] = 0.0;
    ws[47456] = 0.0;
    ws[47488] = 0.0;
    ws[47520] = 0.0;
    ws[47552] = 0.0;
    ws[47584] = 0.0;
    ws[47616] = 0.0;
    ws[47648] = 0.0;
    ws[47680] = 0.0;
    ws[47712] = 0.0;
    ws[47744] = 0.0;
    ws[47776] = 0.0;
    ws[47808] = 0.0;
    ws[47840] = 0.0;
    ws[47872] = 0.0;
    ws[47904] = 0.0;
    ws[47936] = 0.0;
    ws[47968] = 0.0;
    ws[48000] = 0.0;
    ws[48032] = 0.0;
    ws[48064] = 0.0;
    ws[48096] = 0.0;
    ws[48128] = 0.0;
    ws[48160] = 0.0;
    ws[48192] = 0.0;
    ws[48224] = 0.0;
    ws[48256] = 0.0;
    ws[48288] = 0.0;
    ws[48320] = 0.0;
    ws[48352] = 0.0;
    ws[48384] = 0.0;
    ws[48416] = 0.0;
    ws[48448] = 0.0;
    ws[48480] = 0.0;
    ws[48512] = 0.0;
    ws[48544] = 0.0;
    ws[48576] = 0.0;
    ws[48608] = 0.0;
    ws[48640] = 0.0;
    ws[48672] = 0.0;
    ws[48704] = 0.0;
    ws[48736] = 0.0;
    ws[48768] = 0.0;
    ws[48800] = 0.0;
    ws[48832] = 0.0;
    ws[48864] = 0.0;
    ws[48896] = 0.0;
    ws[48928] = 0.0;
    ws[48960] = 0.0;
    ws[48992] = 0.0;
    ws[49024] = 0.0;
    ws[49056] = 0.0;
    ws[49088] = 0.0;
    ws[49120] = 0.0;
    ws[49152] = 0.0;
    ws[49184] = 0.0;
    ws[49216] = 0.0;
    ws[49248] = 0.0;
    ws[49280] = 0.0;
    ws[49312] = 0.0;
    ws[49344] = 0.0;
    ws[49376] = 0.0;
    ws[49408] = 0.0;
    ws[49440] = 0.0;
    ws[49472] = 0.0;
    ws[49504] = 0.0;
    ws[49536] = 0.0;
    ws[49568] = 0.0;
    ws[49600] = 0.0;
    ws[49632] = 0.0;
    ws[49664] = 0.0;
    ws[49696] = 0.0;
    ws[49728] = 0.0;
    ws[49760] = 0.0;
    ws[49792] = 0.0;
    ws[49824] = 0.0;
    ws[49856] = 0.0;
    ws[49888] = 0.0;
    ws[49920] = 0.0;
    ws[49952] = 0.0;
    ws[49984] = 0.0;
    ws[50016] = 0.0;
    ws[50048] = 0.0;
    ws[50080] = 0.0;
    ws[50112] = 0.0;
    ws[50144] = 0.0;
    ws[50176] = 0.0;
    ws[50208] = 0.0;
    ws[50240] = 0.0;
    ws[50272] = 0.0;
    ws[50304] = 0.0;
    ws[50336] = 0.0;
    ws[50368] = 0.0;
    ws[50400] = 0.0;
    ws[50432] = 0.0;
    ws[50464] = 0.0;
    ws[50496] = 0.0;
    ws[50528] = 0.0;
    ws[50560] = 0.0;
    ws[50592] = 0.0;
    ws[50624] = 0.0;
    ws[50656] = 0.0;
    ws[50688] = 0.0;
    ws[50720] = 0.0;
    ws[50752] = 0.0;
    ws[50784] = 0.0;
    ws[50816] = 0.0;
    ws[50848] = 0.0;
    ws[50880] = 0.0;
    ws[50912] = 0.0;
    ws[50944] = 0.0;
    ws[50976] = 0.0;
    ws[51008] = 0.0;
    ws[51040] = 0.0;
    ws[51072] = 0.0;
    ws[51104] = 0.0;
    ws[51136] = 0.0;
    ws[51168] = 0.0;
    ws[51200] = 0.0;
    ws[51232] = 0.0;
    ws[51264] = 0.0;
    ws[51296] = 0.0;
    ws[51328] = 0.0;
    ws[51360] = 0.0;
    ws[51392] = 0.0;
    ws[51424] = 0.0;
    ws[51456] = 0.0;
    ws[51488] = 0.0;
    ws[51520] = 0.0;
    ws[51552] = 0.0;
    ws[51584] = 0.0;
    ws[51616] = 0.0;
    ws[51648] = 0.0;
    ws[51680] = 0.0;
    ws[51712] = 0.0;
    ws[51744] = 0.0;
    ws[51776] = 0.0;
    ws[51808] = 0.0;
    ws[51840] = 0.0;
    ws[51872] = 0.0;
    ws[51904] = 0.0;
    ws[51936] = 0.0;
    ws[51968] = 0.0;
    ws[52000] = 0.0;
    ws[52032] = 0.0;
    ws[52064] = 0.0;
    ws[52096] = 0.0;
    ws[52128] = 0.0;
    ws[52160] = 0.0;
    ws[52192] = 0.0;
    ws[52224] = 0.0;
    ws[52256] = 0.0;
    ws[52288] = 0.0;
    ws[52320] = 0.0;
    ws[52352] = 0.0;
    ws[52384] = 0.0;
    ws[52416] = 0.0;
    ws[52448] = 0.0;
    ws[52480] = 0.0;
    ws[52512] = 0.0;
    ws[52544] = 0.0;
    ws[52576] = 0.0;
    ws[52608] = 0.0;
    ws[52640] = 0.0;
    ws[52672] = 0.0;
    ws[52704] = 0.0;
    ws[52736] = 0.0;
    ws[52768] = 0.0;
    ws[52800] = 0.0;
    ws[52832] = 0.0;
    ws[52864] = 0.0;
    ws[52896] = 0.0;
    ws[52928] = 0.0;
    ws[52960] = 0.0;
    ws[52992] = 0.0;
    ws[53024] = 0.0;
    ws[53056] = 0.0;
    ws[53088] = 0.0;
    ws[53120] = 0.0;
    ws[53152] = 0.0;
    ws[53184] = 0.0;
    ws[53216] = 0.0;
    ws[53248] = 0.0;
    ws[53280] = 0.0;
    ws[53312] = 0.0;
    ws[53344] = 0.0;
    ws[53376] = 0.0;
    ws[53408] = 0.0;
    ws[53440] = 0.0;
    ws[53472] = 0.0;
    ws[53504] = 0.0;
    ws[53536] = 0.0;
    ws[53568] = 0.0;
    ws[53600] = 0.0;
    ws[53632] = 0.0;
    ws[53664] = 0.0;
    ws[53696] = 0.0;
    ws[53728] = 0.0;
    ws[53760] = 0.0;
    ws[53792] = 0.0;
    ws[53824] = 0.0;
    ws[53856] = 0.0;
    ws[53888] = 0.0;
    ws[53920] = 0.0;
    ws[53952] = 0.0;
    ws[53984] = 0.0;
    ws[54016] = 0.0;
    ws[54048] = 0.0;
    ws[54080] = 0.0;
    ws[54112] = 0.0;
    ws[54144] = 0.0;
    ws[54176] = 0.0;
    ws[54208] = 0.0;
    ws[54240] = 0.0;
    ws[54272] = 0.0;
    ws[54304] = 0.0;
    ws[54336] = 0.0;
    ws[54368] = 0.0;
    ws[54400] = 0.0;
    ws[54432] = 0.0;
    ws[54464] = 0.0;
    ws[54496] = 0.0;
    ws[54528] = 0.0;
    ws[54560] = 0.0;
    ws[54592] = 0.0;
    ws[54624] = 0.0;
    ws[54656] = 0.0;
    ws[54688] = 0.0;
    ws[54720] = 0.0;
    ws[54752] = 0.0;
    ws[54784] = 0.0;
    ws[54816] = 0.0;
    ws[54848] = 0.0;
    ws[54880] = 0.0;
    ws[54912] = 0.0;
    ws[54944] = 0.0;
    ws[54976] = 0.0;
    ws[55008] = 0.0;
    ws[55040] = 0.0;
    ws[55072] = 0.0;
    ws[55104] = 0.0;
    ws[55136] = 0.0;
    ws[55168] = 0.0;
    ws[55200] = 0.0;
    ws[55232] = 0.0;
    ws[55264] = 0.0;
    ws[55296] = 0.0;
    ws[55328] = 0.0;
    ws[55360] = 0.0;
    ws[55392] = 0.0;
    ws[55424] = 0.0;
    ws[55456] = 0.0;
    ws[55488] = 0.0;
    ws[55520] = 0.0;
    ws[55552] = 0.0;
    ws[55584] = 0.0;
    ws[55616] = 0.0;
    ws[55648] = 0.0;
    ws[55680] = 0.0;
    ws[55712] = 0.0;
    ws[55744] = 0.0;
    ws[55776] = 0.0;
    ws[55808] = 0.0;
    ws[55840] = 0.0;
    ws[55872] = 0.0;
    ws[55904] = 0.0;
    ws[55936] = 0.0;
    ws[55968] = 0.0;
    ws[56000] = 0.0;
    ws[56032] = 0.0;
    ws[56064] = 0.0;
    ws[56096] = 0.0;
    ws[56128] = 0.0;
    ws[56160] = 0.0;
    ws[56192] = 0.0;
    ws[56224] = 0.0;
    ws[56256] = 0.0;
    ws[56288] = 0.0;
    ws[56320] = 0.0;
    ws[56352] = 0.0;
    ws[56384] = 0.0;
    ws[56416] = 0.0;
    ws[56448] = 0.0;
    ws[56480] = 0.0;
    ws[56512] = 0.0;
    ws[56544] = 0.0;
    ws[56576] = 0.0;
    ws[56608] = 0.0;
    ws[56640] = 0.0;
    ws[56672] = 0.0;
    ws[56704] = 0.0;
    ws[56736] = 0.0;
    ws[56768] = 0.0;
    ws[56800] = 0.0;
    ws[56832] = 0.0;
    ws[56864] = 0.0;
    ws[56896] = 0.0;
    ws[56928] = 0.0;
    ws[56960] = 0.0;
    ws[56992] = 0.0;
    ws[57024] = 0.0;
    ws[57056] = 0.0;
    ws[57088] = 0.0;
    ws[57120] = 0.0;
    ws[57152] = 0.0;
    ws[57184] = 0.0;
    ws[57216] = 0.0;
    ws[57248] = 0.0;
    ws[57280] = 0.0;
    ws[57312] = 0.0;
    ws[57344] = 0.0;
    ws[57376] = 0.0;
    ws[57408] = 0.0;
    ws[57440] = 0.0;
    ws[57472] = 0.0;
    ws[57504] = 0.0;
    ws[57536] = 0.0;
    ws[57568] = 0.0;
    ws[57600] = 0.0;
    ws[57632] = 0.0;
    ws[57664] = 0.0;
    ws[57696] = 0.0;
    ws[57728] = 0.0;
    ws[57760] = 0.0;
    ws[57792] = 0.0;
    ws[57824] = 0.0;
    ws[57856] = 0.0;
    ws[57888] = 0.0;
    ws[57920] = 0.0;
    ws[57952] = 0.0;
    ws[57984] = 0.0;
    ws[58016] = 0.0;
    ws[58048] = 0.0;
    ws[58080] = 0.0;
    ws[58112] = 0.0;
    ws[58144] = 0.0;
    ws[58176] = 0.0;
    ws[58208] = 0.0;
    ws[58240] = 0.0;
    ws[58272] = 0.0;
    ws[58304] = 0.0;
    ws[58336] = 0.0;
    ws[58368] = 0.0;
    ws[58400] = 0.0;
    ws[58432] = 0.0;
    ws[58464] = 0.0;
    ws[58496] = 0.0;
    ws[58528] = 0.0;
    ws[58560] = 0.0;
    ws[58592] = 0.0;
    ws[58624] = 0.0;
    ws[58656] = 0.0;
    ws[58688] = 0.0;
    ws[58720] = 0.0;
    ws[58752] = 0.0;
    ws[58784] = 0.0;
    ws[58816] = 0.0;
    ws[58848] = 0.0;
    ws[58880] = 0.0;
    ws[58912] = 0.0;
    ws[58944] = 0.0;
    ws[58976] = 0.0;
    ws[59008] = 0.0;
    ws[59040] = 0.0;
    ws[59072] = 0.0;
    ws[59104] = 0.0;
    ws[59136] = 0.0;
    ws[59168] = 0.0;
    ws[59200] = 0.0;
    ws[59232] = 0.0;
    ws[59264] = 0.0;
    ws[59296] = 0.0;
    if (lsunlight) {
        ws[42336] = rjv[0];
        ws[42368] = rjv[1];
        ws[42400] = rjv[2];
        ws[42432] = rjv[3];
        ws[42464] = rjv[4];
        ws[42496] = rjv[5];
        ws[42528] = rjv[6];
        ws[42560] = rjv[7];
        ws[42592] = rjv[8];
        ws[42624] = rjv[9];
        ws[42656] = rjv[10];
        ws[42688] = rjv[11];
        ws[42720] = rjv[12];
        ws[42752] = rjv[13];
        ws[42784] = rjv[14];
        ws[42816] = rjv[15];
        ws[42848] = rjv[12];
        ws[42880] = rjv[12];
        ws[42912] = rjv[16];
        ws[42944] = rjv[17];
        ws[42976] = rjv[18];
        ws[43008] = rjv[19];
        ws[43040] = rjv[20];
        ws[43072] = rjv[21];
        ws[43104] = rjv[22];
        ws[43136] = rjv[23];
        ws[43168] = rjv[24];
        ws[43200] = rjv[24];
        ws[43232] = rjv[24];
        ws[43264] = rjv[25];
        ws[43296] = rjv[26];
        ws[43328] = rjv[26];
        ws[43360] = rjv[26];
        ws[43392] = rjv[26];
        ws[43424] = rjv[27];
        ws[43456] = rjv[28];
        ws[43488] = rjv[29];
        ws[43520] = rjv[30];
        ws[43552] = rjv[28];
        ws[43584] = rjv[28];
        ws[54976] = rjv[31];
        if (seawater > 0.001) ws[55968] = (seawater * 60.0) * chem_halogen_falloff(press, 6.7006e-11, 10.743, 3.4153e-08, (-0.6713), 2e-06);
        else ws[55968] = 0.0;
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
        ws[43616] = cfact * chem_arrhenius_t03(inv_temp, 1.7e-12, (-940.0));
        ws[43648] = cfact * chem_arrhenius_t03(inv_temp, 1e-14, (-490.0));
        ws[43680] = cfact * chem_arrhenius_t03(inv_temp, 3e-12, (-1500.0));
        ws[43712] = cfact * chem_arrhenius_t03(inv_temp, 1.2e-13, (-2450.0));
        ws[43744] = cfact_squ * chem_power_t02(tempot300, 6.1e-34, (-2.4));
        ws[43776] = cfact * chem_arrhenius_t03(inv_temp, 8e-12, (-2060.0));
        ws[43808] = cfact * chem_arrhenius_t03(inv_temp, 3.3e-11, 55.0);
        ws[43840] = cfact * chem_arrhenius_t03(inv_temp, 2.15e-11, 110.0);
        ws[43872] = cfact * chem_arrhenius_t03(inv_temp, 1.63e-10, 60.0);
        ws[43904] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-12, (-1800.0));
        ws[43936] = cfact * chem_arrhenius_t03(inv_temp, 4.8e-11, 250.0);
        ws[43968] = cfact * chem_falloff_t09(inv_temp, cair, 3e-13, 460.0, 2.1e-33, 920.0);
        ws[44000] = cfact_squ * chem_falloff_t09(inv_temp, cair, 4.2e-34, 2660.0, 2.94e-54, 3120.0);
        ws[44032] = cfact * chem_arrhenius_t03(inv_temp, 1.8e-12, 0.0);
        ws[44064] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 9.1e-32, 0.0, (-1.5), 3e-11, 0.0, 0.0, 1.0, 0.6);
        ws[44096] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 7.1e-31, 0.0, (-2.6), 3.6e-11, 0.0, (-0.1), 1.0, 0.6);
        ws[44128] = cfact * chem_arrhenius_t03(inv_temp, 3.44e-12, 260.0);
        ws[44160] = cfact * chem_falloff_t11(inv_temp, tempot300, cair, 6.095e-14, (-1.0), 270.0, 6.857e-34, 1.0, 270.0, (-5.968e-14), 270.0);
        ws[44192] = cfact_squ * chem_arrhenius_t03(inv_temp, 4.25e-39, 663.5);
        ws[44224] = cfact * chem_arrhenius_t03(inv_temp, 3e-12, 250.0);
        ws[44256] = cfact * chem_arrhenius_t03(inv_temp, 5.3e-12, 200.0);
        ws[44288] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 3.4e-31, 0.0, (-1.6), 2.3e-11, 0.0, (-0.2), 1.0, 0.6);
        ws[44320] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.8e-30, 0.0, (-3.0), 2.8e-11, 0.0, 0.0, 1.0, 0.6);
        ws[44352] = cfact * chem_falloff_t08(inv_temp, cair, 2.4e-14, 460.0, 2.7e-17, 2199.0, 6.5e-34, 1335.0);
        ws[44384] = 2e-11 * cfact;
        ws[44416] = 3.5e-12 * cfact;
        ws[44448] = cfact * chem_arrhenius_t03(inv_temp, 1.7e-11, 125.0);
        ws[44480] = cfact * chem_arrhenius_t03(inv_temp, 4.35e-14, (-1335.0));
        ws[44512] = cfact * chem_arrhenius_t03(inv_temp, 8.5e-13, (-2450.0));
        ws[44544] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 2.4e-30, 0.0, (-3.0), 1.6e-12, 0.0, 0.1, 1.0, 0.6);
        ws[44576] = (rfact * ws[44544]) * (1.7241e+26 * exp((-10840.0) * inv_temp));
        ws[44608] = 1e-22 * cfact;
        ws[44640] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1.9e-31, 0.0, (-3.4), 4e-12, 0.0, (-0.3), 1.0, 0.6);
        ws[44672] = (rfact * ws[44640]) * (4.7619e+26 * exp((-10900.0) * inv_temp));
        ws[44704] = cfact * chem_arrhenius_t03(inv_temp, 4.5e-13, 610.0);
        ws[44736] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 2.9e-31, 0.0, (-4.1), 1.7e-12, 0.0, 0.2, 1.0, 0.6);
        ws[44768] = cfact * chem_falloff_t09(inv_temp, cair, 1.44e-13, 0.0, 2.74e-33, 0.0);
        ws[44800] = cfact * chem_arrhenius_t03(inv_temp, 2.45e-12, (-1775.0));
        ws[44832] = cfact * chem_arrhenius_t03(inv_temp, 7.66e-12, (-1020.0));
        ws[44864] = cfact * chem_arrhenius_t03(inv_temp, 7.68e-12, (-370.0));
        ws[44896] = cfact * chem_arrhenius_t03(inv_temp, 1.01e-11, (-245.0));
        ws[44928] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 1e-28, 0.0, (-4.5), 8.8e-12, 0.0, (-0.85), 1.0, 0.6);
        ws[44960] = cfact * chem_arrhenius_t03(inv_temp, 5.72e-12, 500.0);
        ws[44992] = cfact * chem_arrhenius_t03(inv_temp, 1.33e-11, 500.0);
        ws[45024] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 5.5e-30, 0.0, 0.0, 8.3e-13, 0.0, 2.0, 1.0, 0.6);
        ws[45056] = cfact * chem_arrhenius_t03(inv_temp, 2.33e-12, (-193.0));
        ws[45088] = cfact * chem_arrhenius_t03(inv_temp, 1.81e-12, 354.0);
        ws[45120] = 2.33e-11 * cfact;
        ws[45152] = 7.16e-12 * cfact;
        ws[45184] = cfact * chem_arrhenius_t03(inv_temp, 1.58e-14, (-2000.0));
        ws[45216] = cfact * chem_arrhenius_t03(inv_temp, 2.95e-12, (-450.0));
        ws[45248] = cfact * chem_arrhenius_t03(inv_temp, 2.69e-11, 390.0);
        ws[45280] = cfact * chem_arrhenius_t03(inv_temp, 4.5e-13, 1300.0);
        ws[45312] = cfact * chem_arrhenius_t03(inv_temp, 6e-12, 350.0);
        ws[45344] = cfact * chem_arrhenius_t03(inv_temp, 4.6e-12, 200.0);
        ws[45376] = cfact * chem_arrhenius_t03(inv_temp, 2.97e-11, 390.0);
        ws[45408] = cfact * chem_arrhenius_t03(inv_temp, 3.14e-11, 580.0);
        ws[45440] = cfact * chem_arrhenius_t03(inv_temp, 9.42e-12, 580.0);
        ws[45472] = cfact * chem_arrhenius_t03(inv_temp, 2.4e-11, 390.0);
        ws[45504] = 1.5e-11 * cfact;
        ws[45536] = 4e-05 * 60.0;
        ws[45568] = 3e-12 * cfact;
        ws[45600] = cfact * chem_arrhenius_t03(inv_temp, 1.21e-11, 440.0);
        ws[45632] = cfact * chem_arrhenius_t03(inv_temp, 4.2e-11, 401.0);
        ws[45664] = cfact * chem_arrhenius_t03(inv_temp, 5.2e-12, 600.0);
        ws[45696] = 1.1e-10 * cfact;
        ws[45728] = cfact * chem_arrhenius_t03(inv_temp, 5.5e-12, 125.0);
        ws[45760] = cfact * chem_arrhenius_t03(inv_temp, 4.7e-12, 345.0);
        ws[45792] = cfact * chem_arrhenius_t03(inv_temp, 4.9e-12, 405.0);
        ws[45824] = cfact * chem_arrhenius_t04(inv_temp, tempot300, 4.56e-14, (-427.0), 3.65);
        ws[45856] = cfact * chem_arrhenius_t03(inv_temp, 1.5e-12, (-90.0));
        ws[45888] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-12, 10.0);
        ws[45920] = 3e-12 * cfact;
        ws[45952] = cfact * chem_arrhenius_t03(inv_temp, 8e-12, 380.0);
        ws[45984] = cfact * chem_arrhenius_t03(inv_temp, 2.6e-12, 610.0);
        ws[46016] = cfact * chem_arrhenius_t03(inv_temp, 5.77e-12, 533.0);
        ws[46048] = 1.1e-11 * cfact;
        ws[46080] = cfact * chem_arrhenius_t03(inv_temp, 9.26e-13, 830.0);
        ws[46112] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-11, 175.0);
        ws[46144] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-11, 175.0);
        ws[46176] = 1e-11 * cfact;
        ws[46208] = cfact * chem_arrhenius_t03(inv_temp, 5.32e-12, 243.0);
        ws[46240] = cfact * chem_arrhenius_t03(inv_temp, 6.75e-12, 405.0);
        ws[46272] = cfact * chem_arrhenius_t03(inv_temp, 4.65e-11, 0.0);
        ws[46304] = cfact * chem_arrhenius_t03(inv_temp, 2.05e-10, 0.0);
        ws[46336] = cfact * chem_arrhenius_t03(inv_temp, 2.85e-12, (-345.0));
        ws[46368] = cfact * chem_arrhenius_t03(inv_temp, 3e-12, 20.0);
        ws[46400] = cfact * chem_arrhenius_t03(inv_temp, 2.6e-12, 200.0);
        ws[46432] = 1.47e-11 * cfact;
        ws[46464] = cfact * chem_arrhenius_t03(inv_temp, 2.9e-12, 190.0);
        ws[46496] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-12, 190.0);
        ws[46528] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-12, 190.0);
        ws[46560] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-12, 190.0);
        ws[46592] = 3e-11 * cfact;
        ws[46624] = 4.5e-13 * cfact;
        ws[46656] = cfact * chem_arrhenius_t03(inv_temp, 4e-14, 850.0);
        ws[46688] = cfact * chem_arrhenius_t03(inv_temp, 2.93e-12, 190.0);
        ws[46720] = 4e-14 * cfact;
        ws[46752] = 4e-14 * cfact;
        ws[46784] = 3.2e-11 * cfact;
        ws[46816] = cfact * chem_arrhenius_t03(inv_temp, 5.31e-12, (-260.0));
        ws[46848] = 4.8e-12 * cfact;
        ws[46880] = cfact * chem_falloff_t08(inv_temp, cair, 2.4e-14, 460.0, 2.7e-17, 2199.0, 6.5e-34, 1335.0);
        ws[46912] = cfact * chem_arrhenius_t03(inv_temp, 9.14e-15, (-2580.0));
        ws[46944] = cfact * chem_arrhenius_t03(inv_temp, 4.33e-15, (-1800.0));
        ws[46976] = cfact * chem_arrhenius_t03(inv_temp, 4.4e-15, (-845.0));
        ws[47008] = cfact * chem_arrhenius_t03(inv_temp, 8.05e-16, (-640.0));
        ws[47040] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-15, (-770.0));
        ws[47072] = 8.3e-18 * cfact;
        ws[47104] = 1.67e-16 * cfact;
        ws[47136] = cfact * chem_arrhenius_t03(inv_temp, 1.36e-15, (-2112.0));
        ws[47168] = cfact * chem_arrhenius_t03(inv_temp, 8.5e-16, (-1520.0));
        ws[47200] = 1.66e-18 * cfact;
        ws[47232] = 2e-16 * cfact;
        ws[47264] = 2e-16 * cfact;
        ws[47296] = 9e-17 * cfact;
        ws[47328] = 2.86e-13 * cfact;
        ws[47360] = cfact * chem_arrhenius_t04(inv_temp, tempot300, 4.392e-13, (-2282.0), 2.0);
        ws[47392] = cfact * chem_arrhenius_t03(inv_temp, 1.79e-13, (-450.0));
        ws[47424] = cfact * chem_arrhenius_t03(inv_temp, 8.64e-13, 450.0);
        ws[47456] = cfact * chem_arrhenius_t03(inv_temp, 1.19e-12, 490.0);
        ws[47488] = 1.22e-11 * cfact;
        ws[47520] = cfact * chem_arrhenius_t03(inv_temp, 3.15e-13, (-448.0));
        ws[47552] = cfact * chem_arrhenius_t03(inv_temp, 2e-12, (-2440.0));
        ws[47584] = cfact * chem_arrhenius_t03(inv_temp, 1.4e-12, (-1900.0));
        ws[47616] = cfact * chem_arrhenius_t03(inv_temp, 3.76e-12, (-1900.0));
        ws[47648] = 3.4e-15 * cfact;
        ws[47680] = cfact * chem_arrhenius_t03(inv_temp, 5.02e-13, (-1076.0));
        ws[47712] = cfact * chem_arrhenius_t03(inv_temp, 2.9e-12, (-1900.0));
        ws[47744] = cfact * chem_arrhenius_t03(inv_temp, 3.76e-12, (-1900.0));
        ws[47776] = 3.78e-12 * cfact;
        ws[47808] = 1.06e-12 * cfact;
        ws[47840] = 2.01e-10 * cfact;
        ws[47872] = cfact * chem_arrhenius_t03(inv_temp, 2.2e-14, (-500.0));
        ws[47904] = 0.029 * 60.0;
        ws[47936] = 0.024 * 60.0;
        ws[47968] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 9.7e-29, 0.0, (-5.6), 9.3e-12, 0.0, (-1.5), 1.0, 0.6);
        ws[48000] = (rfact * ws[47968]) * (1.1111e+28 * exp((-14000.0) * inv_temp));
        ws[48032] = cfact * chem_falloff_t10(inv_temp, tempot300, cair, 9.7e-29, 0.0, (-5.6), 9.3e-12, 0.0, (-1.5), 1.0, 0.6);
        ws[48064] = (rfact * ws[48032]) * (1.1111e+28 * exp((-14000.0) * inv_temp));
        ws[48096] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-12, 181.0);
        ws[48128] = 60.0 * chem_arrhenius_t03(inv_temp, 1.6e+16, (-13486.0));
        ws[48160] = cfact * chem_arrhenius_t03(inv_temp, 2.8e-12, 300.0);
        ws[48192] = cfact * chem_arrhenius_t03(inv_temp, 2.6e-12, 365.0);
        ws[48224] = 4e-12 * cfact;
        ws[48256] = 4e-12 * cfact;
        ws[48288] = 9e-12 * cfact;
        ws[48320] = 4e-12 * cfact;
        ws[48352] = 4e-12 * cfact;
        ws[48384] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48416] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48448] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48480] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48512] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48544] = 4e-12 * cfact;
        ws[48576] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48608] = 4e-12 * cfact;
        ws[48640] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48672] = 4e-12 * cfact;
        ws[48704] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48736] = 4e-12 * cfact;
        ws[48768] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48800] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[48832] = cfact * chem_arrhenius_t03(inv_temp, 8.1e-12, 270.0);
        ws[48864] = cfact * chem_arrhenius_t03(inv_temp, 8.1e-12, 270.0);
        ws[48896] = cfact * chem_arrhenius_t03(inv_temp, 2.9e-12, 300.0);
        ws[48928] = 4e-12 * cfact;
        ws[48960] = 4e-12 * cfact;
        ws[48992] = cfact * chem_arrhenius_t03(inv_temp, 2.54e-12, 360.0);
        ws[49024] = cfact * chem_arrhenius_t03(inv_temp, 2.54e-12, 360.0);
        ws[49056] = cfact * chem_arrhenius_t03(inv_temp, 2.54e-12, 360.0);
        ws[49088] = cfact * chem_arrhenius_t03(inv_temp, 2.54e-12, 360.0);
        ws[49120] = 4e-12 * cfact;
        ws[49152] = 4e-12 * cfact;
        ws[49184] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[49216] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[49248] = 4e-12 * cfact;
        ws[49280] = 4e-12 * cfact;
        ws[49312] = 4e-12 * cfact;
        ws[49344] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[49376] = 4e-12 * cfact;
        ws[49408] = 2e-11 * cfact;
        ws[49440] = 2e-11 * cfact;
        ws[49472] = 2.08e-12 * cfact;
        ws[49504] = cfact * chem_arrhenius_t03(inv_temp, 4.1e-13, 750.0);
        ws[49536] = cfact * chem_arrhenius_t03(inv_temp, 7.5e-13, 700.0);
        ws[49568] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[49600] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[49632] = cfact * chem_arrhenius_t03(inv_temp, 1.9e-13, 1300.0);
        ws[49664] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[49696] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[49728] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[49760] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[49792] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[49824] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[49856] = cfact * chem_arrhenius_t03(inv_temp, 2.6e-13, 1300.0);
        ws[49888] = 1.5e-11 * cfact;
        ws[49920] = cfact * chem_arrhenius_t03(inv_temp, 2.71e-13, 1300.0);
        ws[49952] = 1.5e-11 * cfact;
        ws[49984] = cfact * chem_arrhenius_t03(inv_temp, 2.6e-13, 1300.0);
        ws[50016] = 1.5e-11 * cfact;
        ws[50048] = cfact * chem_arrhenius_t03(inv_temp, 2.71e-13, 1300.0);
        ws[50080] = 1.5e-11 * cfact;
        ws[50112] = cfact * chem_arrhenius_t03(inv_temp, 2.71e-13, 1300.0);
        ws[50144] = cfact * chem_arrhenius_t03(inv_temp, 2.73e-13, 1300.0);
        ws[50176] = cfact * chem_arrhenius_t03(inv_temp, 4.3e-13, 1040.0);
        ws[50208] = cfact * chem_arrhenius_t03(inv_temp, 4.3e-13, 1040.0);
        ws[50240] = cfact * chem_arrhenius_t03(inv_temp, 1.15e-13, 1300.0);
        ws[50272] = cfact * chem_arrhenius_t03(inv_temp, 1.15e-13, 1300.0);
        ws[50304] = cfact * chem_arrhenius_t03(inv_temp, 1.15e-13, 1300.0);
        ws[50336] = cfact * chem_arrhenius_t03(inv_temp, 1.82e-13, 1300.0);
        ws[50368] = cfact * chem_arrhenius_t03(inv_temp, 1.82e-13, 1300.0);
        ws[50400] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[50432] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[50464] = cfact * chem_arrhenius_t03(inv_temp, 3.75e-13, 980.0);
        ws[50496] = 1e-11 * cfact;
        ws[50528] = cfact * chem_arrhenius_t03(inv_temp, 3.75e-13, 980.0);
        ws[50560] = cfact * chem_arrhenius_t03(inv_temp, 1.15e-13, 1300.0);
        ws[50592] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[50624] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[50656] = cfact * chem_arrhenius_t03(inv_temp, 3.75e-13, 980.0);
        ws[50688] = cfact * chem_arrhenius_t03(inv_temp, 1.66e-13, 1300.0);
        ws[50720] = cfact * chem_arrhenius_t03(inv_temp, 9.5e-14, 390.0);
        ws[50752] = cfact * chem_arrhenius_t03(inv_temp, 1.18e-13, 158.0);
        ws[50784] = cfact * chem_arrhenius_t03(inv_temp, 9.46e-14, 431.0);
        ws[50816] = cfact * chem_arrhenius_t03(inv_temp, 1e-13, 467.0);
        ws[50848] = cfact * chem_arrhenius_t03(inv_temp, 1.71e-13, 708.0);
        ws[50880] = cfact * chem_arrhenius_t03(inv_temp, 1.46e-13, 708.0);
        ws[50912] = cfact * chem_arrhenius_t03(inv_temp, 9.18e-14, 708.0);
        ws[50944] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[50976] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51008] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51040] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51072] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-14, 221.0);
        ws[51104] = 2e-12 * cfact;
        ws[51136] = 1e-10 * cfact;
        ws[51168] = 2e-12 * cfact;
        ws[51200] = 1e-10 * cfact;
        ws[51232] = 2e-12 * cfact;
        ws[51264] = 1e-10 * cfact;
        ws[51296] = 2e-12 * cfact;
        ws[51328] = 1e-10 * cfact;
        ws[51360] = cfact * chem_arrhenius_t03(inv_temp, 2e-11, 500.0);
        ws[51392] = cfact * chem_arrhenius_t03(inv_temp, 2e-11, 500.0);
        ws[51424] = cfact * chem_arrhenius_t03(inv_temp, 7.5e-13, 500.0);
        ws[51456] = cfact * chem_arrhenius_t03(inv_temp, 6.91e-13, 508.0);
        ws[51488] = cfact * chem_arrhenius_t03(inv_temp, 6.91e-13, 508.0);
        ws[51520] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-14, 221.0);
        ws[51552] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-14, 221.0);
        ws[51584] = 8.37e-14 * cfact;
        ws[51616] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-14, 221.0);
        ws[51648] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51680] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51712] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51744] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[51776] = cfact * chem_arrhenius_t03(inv_temp, 7.5e-13, 500.0);
        ws[51808] = cfact * chem_arrhenius_t03(inv_temp, 1.6e-13, 708.0);
        ws[51840] = cfact * chem_arrhenius_t03(inv_temp, 9.68e-14, 708.0);
        ws[51872] = 3.56e-14 * cfact;
        ws[51904] = cfact * chem_arrhenius_t03(inv_temp, 5.99e-15, 1510.0);
        ws[51936] = cfact * chem_arrhenius_t03(inv_temp, 1.03e-12, 211.0);
        ws[51968] = cfact * chem_arrhenius_t03(inv_temp, 6.9e-13, 460.0);
        ws[52000] = cfact * chem_arrhenius_t03(inv_temp, 5.59e-13, 522.0);
        ws[52032] = cfact * chem_arrhenius_t03(inv_temp, 9.48e-13, 765.0);
        ws[52064] = cfact * chem_arrhenius_t03(inv_temp, 8.11e-13, 765.0);
        ws[52096] = cfact * chem_arrhenius_t03(inv_temp, 5.09e-13, 765.0);
        ws[52128] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[52160] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[52192] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[52224] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[52256] = cfact * chem_arrhenius_t03(inv_temp, 8.4e-14, 221.0);
        ws[52288] = cfact * chem_arrhenius_t03(inv_temp, 2e-12, 500.0);
        ws[52320] = 1e-10 * cfact;
        ws[52352] = cfact * chem_arrhenius_t03(inv_temp, 2e-12, 500.0);
        ws[52384] = 1e-10 * cfact;
        ws[52416] = cfact * chem_arrhenius_t03(inv_temp, 2e-12, 500.0);
        ws[52448] = 1e-10 * cfact;
        ws[52480] = cfact * chem_arrhenius_t03(inv_temp, 2e-12, 500.0);
        ws[52512] = 1e-10 * cfact;
        ws[52544] = cfact * chem_arrhenius_t03(inv_temp, 2.5e-12, 500.0);
        ws[52576] = cfact * chem_arrhenius_t03(inv_temp, 2.5e-12, 500.0);
        ws[52608] = cfact * chem_arrhenius_t03(inv_temp, 7.51e-13, 565.0);
        ws[52640] = cfact * chem_arrhenius_t03(inv_temp, 7.51e-13, 565.0);
        ws[52672] = cfact * chem_arrhenius_t03(inv_temp, 7.51e-13, 565.0);
        ws[52704] = cfact * chem_arrhenius_t03(inv_temp, 8.4e-14, 221.0);
        ws[52736] = cfact * chem_arrhenius_t03(inv_temp, 8.4e-14, 221.0);
        ws[52768] = cfact * chem_arrhenius_t03(inv_temp, 1.68e-12, 500.0);
        ws[52800] = cfact * chem_arrhenius_t03(inv_temp, 1.68e-12, 500.0);
        ws[52832] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[52864] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[52896] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 708.0);
        ws[52928] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 708.0);
        ws[52960] = cfact * chem_arrhenius_t03(inv_temp, 7.51e-13, 565.0);
        ws[52992] = cfact * chem_arrhenius_t03(inv_temp, 8.85e-13, 765.0);
        ws[53024] = cfact * chem_arrhenius_t03(inv_temp, 5.37e-13, 765.0);
        ws[53056] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 708.0);
        ws[53088] = cfact * chem_arrhenius_t03(inv_temp, 3.4e-14, 1560.0);
        ws[53120] = cfact * chem_arrhenius_t03(inv_temp, 2.5e-12, 500.0);
        ws[53152] = 1.2e-12 * cfact;
        ws[53184] = 1.2e-12 * cfact;
        ws[53216] = 1.2e-12 * cfact;
        ws[53248] = 1.2e-12 * cfact;
        ws[53280] = 1.2e-12 * cfact;
        ws[53312] = 1.2e-12 * cfact;
        ws[53344] = 1.2e-12 * cfact;
        ws[53376] = 2.3e-12 * cfact;
        ws[53408] = 2.3e-12 * cfact;
        ws[53440] = 2.3e-12 * cfact;
        ws[53472] = 2.3e-12 * cfact;
        ws[53504] = 1.2e-12 * cfact;
        ws[53536] = 2.3e-12 * cfact;
        ws[53568] = 2.3e-12 * cfact;
        ws[53600] = 2.3e-12 * cfact;
        ws[53632] = 2.3e-12 * cfact;
        ws[53664] = 4e-12 * cfact;
        ws[53696] = 4e-12 * cfact;
        ws[53728] = 1.2e-12 * cfact;
        ws[53760] = 1.2e-12 * cfact;
        ws[53792] = 1.2e-12 * cfact;
        ws[53824] = 1.2e-12 * cfact;
        ws[53856] = 1.2e-12 * cfact;
        ws[53888] = 2.5e-12 * cfact;
        ws[53920] = 2.5e-12 * cfact;
        ws[53952] = 2.5e-12 * cfact;
        ws[53984] = 2.5e-12 * cfact;
        ws[54016] = 1.2e-12 * cfact;
        ws[54048] = 1.2e-12 * cfact;
        ws[54080] = 1.2e-12 * cfact;
        ws[54112] = 1.2e-12 * cfact;
        ws[54144] = 1.2e-12 * cfact;
        ws[54176] = 1.2e-12 * cfact;
        ws[54208] = cfact * chem_arrhenius_t03(inv_temp, 7e-14, 1000.0);
        ws[54240] = cfact * chem_arrhenius_t03(inv_temp, 4.25e-14, 1000.0);
        ws[54272] = cfact * chem_arrhenius_t03(inv_temp, 2.96e-14, 1000.0);
        ws[54304] = 1.2e-12 * cfact;
        ws[54336] = cfact * chem_arrhenius_t03(inv_temp, 2.5e-12, 500.0);
        ws[54368] = cfact * chem_arrhenius_t03(inv_temp, 7.13e-17, 2950.0);
        ws[54400] = 1e-10 * cfact;
        ws[54432] = 1e-10 * cfact;
        ws[54464] = 1e-10 * cfact;
        ws[54496] = 1e-10 * cfact;
        ws[54528] = 1e-10 * cfact;
        ws[54560] = 1e-10 * cfact;
        ws[54592] = 1e-10 * cfact;
        ws[54624] = 1e-10 * cfact;
        ws[54656] = 1e-10 * cfact;
        ws[54688] = 1e-10 * cfact;
        ws[54720] = 1e-10 * cfact;
        ws[54752] = 1e-10 * cfact;
        ws[54784] = cfact * chem_arrhenius_t03(inv_temp, 5.78e-11, (-400.0));
        ws[54816] = 6.89e-12 * cfact;
        ws[54848] = 6.55e-14 * cfact;
        ws[54880] = cfact * chem_arrhenius_t03(inv_temp, 8e-12, 380.0);
        ws[54912] = 2.9e-19 * cfact;
        ws[54944] = 3.4e-15 * cfact;
        ws[55008] = cfact * chem_arrhenius_t03(inv_temp, 1.48e-11, 448.0);
        ws[55040] = 9.05e-12 * cfact;
        ws[55072] = 2.3e-12 * cfact;
        ws[55104] = 1.61e-11 * cfact;
        ws[55136] = 2.39e-12 * cfact;
        ws[55168] = 1.37e-11 * cfact;
        ws[55200] = cfact * chem_arrhenius_t03(inv_temp, 1.34e-14, (-2283.0));
        ws[55232] = 1e-13 * cfact;
        ws[55264] = 5.01e-11 * cfact;
        ws[55296] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[55328] = cfact * chem_arrhenius_t03(inv_temp, 3.75e-13, 980.0);
        ws[55360] = 4.4e-11 * cfact;
        ws[55392] = 3.43e-17 * cfact;
        ws[55424] = 8.99e-12 * cfact;
        ws[55456] = 1.2e-11 * cfact;
        ws[55488] = 1.9e-11 * cfact;
        ws[55520] = cfact * chem_arrhenius_t03(inv_temp, 2.84e-13, 1300.0);
        ws[55552] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[55584] = 2.3e-12 * cfact;
        ws[55616] = 1.2e-14 * cfact;
        ws[55648] = 1.97e-10 * cfact;
        ws[55680] = cfact * chem_arrhenius_t03(inv_temp, 2.84e-13, 1300.0);
        ws[55712] = 2.3e-12 * cfact;
        ws[55744] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[55776] = hetv[0];
        ws[55808] = hetv[1];
        ws[55840] = hetv[2];
        ws[55872] = hetv[3];
        ws[55904] = hetv[4];
        ws[55936] = hetv[5];
        ws[56000] = hetv[6];
        ws[56032] = hetv[7];
        ws[56064] = hetv[8];
        ws[56096] = 2.0 * hetv[6];
        ws[56128] = 0.5 * hetv[6];
        ws[56160] = 1.53e-11 * cfact;
        ws[56192] = 1.68e-11 * cfact;
        ws[56224] = 2.24e-11 * cfact;
        ws[56256] = 2.67e-11 * cfact;
        ws[56288] = 3.09e-11 * cfact;
        ws[56320] = 3.38e-11 * cfact;
        ws[56352] = 1.1e-11 * cfact;
        ws[56384] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56416] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56448] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56480] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56512] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56544] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56576] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[56608] = 2.3e-12 * cfact;
        ws[56640] = 2.3e-12 * cfact;
        ws[56672] = 2.3e-12 * cfact;
        ws[56704] = 2.3e-12 * cfact;
        ws[56736] = 2.3e-12 * cfact;
        ws[56768] = 2.3e-12 * cfact;
        ws[56800] = 2.3e-12 * cfact;
        ws[56832] = 2.17e-11 * cfact;
        ws[56864] = 2.2e-11 * cfact;
        ws[56896] = 2.25e-11 * cfact;
        ws[56928] = 2.26e-11 * cfact;
        ws[56960] = 2.27e-11 * cfact;
        ws[56992] = 2.27e-11 * cfact;
        ws[57024] = cfact * chem_arrhenius_t03(inv_temp, 2.66e-13, 1300.0);
        ws[57056] = 0.188 * 60.0;
        ws[57088] = 0.188 * 60.0;
        ws[57120] = 0.188 * 60.0;
        ws[57152] = 0.188 * 60.0;
        ws[57184] = 0.188 * 60.0;
        ws[57216] = 0.188 * 60.0;
        ws[57248] = 0.188 * 60.0;
        ws[57280] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57312] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57344] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57376] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57408] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57440] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57472] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[57504] = 2.3e-12 * cfact;
        ws[57536] = 2.3e-12 * cfact;
        ws[57568] = 2.3e-12 * cfact;
        ws[57600] = 2.3e-12 * cfact;
        ws[57632] = 2.3e-12 * cfact;
        ws[57664] = 2.3e-12 * cfact;
        ws[57696] = 2.3e-12 * cfact;
        ws[57728] = 2.17e-11 * cfact;
        ws[57760] = 2.2e-11 * cfact;
        ws[57792] = 2.25e-11 * cfact;
        ws[57824] = 2.26e-11 * cfact;
        ws[57856] = 2.27e-11 * cfact;
        ws[57888] = 2.27e-11 * cfact;
        ws[57920] = cfact * chem_arrhenius_t03(inv_temp, 2.66e-13, 1300.0);
        ws[57952] = 1.81e-11 * cfact;
        ws[57984] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[58016] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[58048] = 2.3e-12 * cfact;
        ws[58080] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[58112] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[58144] = 1.81e-11 * cfact;
        ws[58176] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[58208] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[58240] = 2.3e-12 * cfact;
        ws[58272] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[58304] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[58336] = 2.31e-11 * cfact;
        ws[58368] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-13, 1300.0);
        ws[58400] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[58432] = 2.3e-12 * cfact;
        ws[58464] = cfact * chem_arrhenius_t03(inv_temp, 3.56e-14, 708.0);
        ws[58496] = cfact * chem_arrhenius_t03(inv_temp, 7.4e-13, 765.0);
        ws[58528] = 5.9e-11 * cfact;
        ws[58560] = 6.07e-11 * cfact;
        ws[58592] = 5.54e-11 * cfact;
        ws[58624] = 5.63e-11 * cfact;
        ws[58656] = 5.46e-11 * cfact;
        ws[58688] = 4.5e-11 * cfact;
        ws[58720] = 5.17e-11 * cfact;
        ws[58752] = 4.73e-11 * cfact;
        ws[58784] = 4.6e-11 * cfact;
        ws[58816] = 3.8e-11 * cfact;
        ws[58848] = 3.93e-11 * cfact;
        ws[58880] = 3.52e-11 * cfact;
        ws[58912] = 3.12e-11 * cfact;
        ws[58944] = 2.4e-11 * cfact;
        ws[58976] = 2.05e-11 * cfact;
        ws[59008] = 4.69e-11 * cfact;
        ws[59040] = cfact * chem_arrhenius_t03(inv_temp, 2.45e-12, (-1775.0));
        ws[59072] = 9.26e-05 * 60.0;
        ws[59104] = 9.26e-05 * 60.0;
        ws[59136] = 5.8e-11 * cfact;
        ws[59168] = cfact * chem_arrhenius_t03(inv_temp, 2.91e-12, 1300.0);
        ws[59200] = cfact * chem_arrhenius_t03(inv_temp, 2.7e-12, 360.0);
        ws[59232] = 2.3e-12 * cfact;
        ws[59264] = 2.5e-13 * cfact;
        ws[59296] = 2.5e-13 * cfact;
        (void)cair; (void)cfact; (void)cfact_squ; (void)inv_cair; (void)inv_cfact; (void)inv_temp; (void)rfact; (void)rfact_squ; (void)temp; (void)tempot300;
    }
    ws[43744] = ws[43744] * 1000000.0;
    ws[43744] = ws[43744] * 209500.0;
    ws[43808] = ws[43808] * 209500.0;
    ws[44192] = ws[44192] * 209500.0;
    ws[43840] = ws[43840] * 780800.0;
    ws[43872] = ws[43872] * h2o;
    ws[44000] = ws[44000] * h2o;
    ws[44608] = ws[44608] * h2o;
    ws[43904] = ws[43904] * 0.56;
    ws[44800] = ws[44800] * 1.85;
}
// f(y) for the day reaction list (rbfeval.F:80-151).
__device__ __noinline__ void feval_0(double* __restrict__ ws, int src, int dst)
{
    const double* __restrict__ yin = ws + src * 32;
    double* __restrict__ yout = ws + dst * 32;
    ws[59328] = (ws[42336]) * yin[5184];
    ws[59360] = (ws[42368]) * yin[5184];
    ws[59392] = (ws[42400]) * yin[4000];
    ws[59424] = (ws[42432]) * yin[5920];
    ws[59456] = (ws[42464]) * yin[5952];
    ws[59488] = (ws[42496]) * yin[5952];
    ws[59520] = (ws[42528]) * yin[1184];
    ws[59552] = (ws[42560]) * yin[5024];
    ws[59584] = (ws[42592]) * yin[1280];
    ws[59616] = (ws[42624]) * yin[5856];
    ws[59648] = (ws[42656]) * yin[5856];
    ws[59680] = (ws[42688]) * yin[5568];
    ws[59712] = (ws[42720]) * yin[5760];
    ws[59744] = (ws[42752]) * yin[4480];
    ws[59776] = (ws[42784]) * yin[4480];
    ws[59808] = (ws[42816]) * yin[3872];
    ws[59840] = (ws[42848]) * yin[4544];
    ws[59872] = (ws[42880]) * yin[4576];
    ws[59904] = (ws[42912]) * yin[5280];
    ws[59936] = (ws[42944]) * yin[5504];
    ws[59968] = (ws[42976]) * yin[5344];
    ws[60000] = (ws[43008]) * yin[4128];
    ws[60032] = (ws[43040]) * yin[4736];
    ws[60064] = (ws[43072]) * yin[5376];
    ws[60096] = (ws[43104]) * yin[5376];
    ws[60128] = (ws[43136]) * yin[5376];
    ws[60160] = (ws[43168]) * yin[5248];
    ws[60192] = (ws[43200]) * yin[5472];
    ws[60224] = (ws[43232]) * yin[4320];
    ws[60256] = (ws[43264]) * yin[4448];
    ws[60288] = (ws[43296]) * yin[2816];
    ws[60320] = (ws[43328]) * yin[5728];
    ws[60352] = (ws[43360]) * yin[4096];
    ws[60384] = (ws[43392]) * yin[4608];
    ws[60416] = (ws[43424]) * yin[3680];
    ws[60448] = (ws[43456]) * yin[5440];
    ws[60480] = (ws[43488]) * yin[1088];
    ws[60512] = (ws[43520]) * yin[1088];
    ws[60544] = (ws[43552]) * yin[4384];
    ws[60576] = (ws[43584]) * yin[1696];
    ws[60608] = ((ws[43616]) * yin[5184]) * yin[6016];
    ws[60640] = ((ws[43648]) * yin[5184]) * yin[5984];
    ws[60672] = ((ws[43680]) * yin[5184]) * yin[5824];
    ws[60704] = ((ws[43712]) * yin[5184]) * yin[5920];
    ws[60736] = (ws[43744]) * yin[2336];
    ws[60768] = ((ws[43776]) * yin[2336]) * yin[5184];
    ws[60800] = (ws[43808]) * yin[576];
    ws[60832] = (ws[43840]) * yin[576];
    ws[60864] = (ws[43872]) * yin[576];
    ws[60896] = (ws[43904]) * yin[6016];
    ws[60928] = ((ws[43936]) * yin[6016]) * yin[5984];
    ws[60960] = ((ws[43968]) * yin[5984]) * yin[5984];
    ws[60992] = ((ws[44000]) * yin[5984]) * yin[5984];
    ws[61024] = ((ws[44032]) * yin[4000]) * yin[6016];
    ws[61056] = ((ws[44064]) * yin[5824]) * yin[2336];
    ws[61088] = ((ws[44096]) * yin[5824]) * yin[6016];
    ws[61120] = ((ws[44128]) * yin[5824]) * yin[5984];
    ws[61152] = ((ws[44160]) * yin[5824]) * yin[5984];
    ws[61184] = ((ws[44192]) * yin[5824]) * yin[5824];
    ws[61216] = ((ws[44224]) * yin[1184]) * yin[6016];
    ws[61248] = ((ws[44256]) * yin[5920]) * yin[2336];
    ws[61280] = ((ws[44288]) * yin[5920]) * yin[2336];
    ws[61312] = ((ws[44320]) * yin[5920]) * yin[6016];
    ws[61344] = ((ws[44352]) * yin[5024]) * yin[6016];
    ws[61376] = ((ws[44384]) * yin[5952]) * yin[6016];
    ws[61408] = ((ws[44416]) * yin[5952]) * yin[5984];
    ws[61440] = ((ws[44448]) * yin[5952]) * yin[5824];
    ws[61472] = ((ws[44480]) * yin[5952]) * yin[5920];
    ws[61504] = ((ws[44512]) * yin[5952]) * yin[5952];
    ws[61536] = ((ws[44544]) * yin[5952]) * yin[5920];
    ws[61568] = (ws[44576]) * yin[1024];
    ws[61600] = (ws[44608]) * yin[1024];
    ws[61632] = ((ws[44640]) * yin[5920]) * yin[5984];
    ws[61664] = (ws[44672]) * yin[1280];
    ws[61696] = ((ws[44704]) * yin[1280]) * yin[6016];
    ws[61728] = ((ws[44736]) * yin[160]) * yin[6016];
    ws[61760] = ((ws[44768]) * yin[5664]) * yin[6016];
    ws[61792] = (ws[44800]) * yin[6016];
    ws[61824] = ((ws[44832]) * yin[1888]) * yin[6016];
    ws[61856] = ((ws[44864]) * yin[2176]) * yin[6016];
    ws[61888] = ((ws[44896]) * yin[1120]) * yin[6016];
    ws[61920] = ((ws[44928]) * yin[2240]) * yin[6016];
    ws[61952] = ((ws[44960]) * yin[2752]) * yin[6016];
    ws[61984] = ((ws[44992]) * yin[1152]) * yin[6016];
    ws[62016] = ((ws[45024]) * yin[256]) * yin[6016];
    ws[62048] = ((ws[45056]) * yin[1216]) * yin[6016];
    ws[62080] = ((ws[45088]) * yin[288]) * yin[6016];
    ws[62112] = ((ws[45120]) * yin[320]) * yin[6016];
    ws[62144] = ((ws[45152]) * yin[352]) * yin[6016];
    ws[62176] = ((ws[45184]) * yin[1312]) * yin[5184];
    ws[62208] = ((ws[45216]) * yin[1312]) * yin[5952];
    ws[62240] = ((ws[45248]) * yin[1312]) * yin[6016];
    ws[62272] = ((ws[45280]) * yin[4288]) * yin[5984];
    ws[62304] = ((ws[45312]) * yin[4288]) * yin[5824];
    ws[62336] = ((ws[45344]) * yin[1344]) * yin[6016];
    ws[62368] = ((ws[45376]) * yin[1344]) * yin[6016];
    ws[62400] = ((ws[45408]) * yin[1632]) * yin[5984];
    ws[62432] = ((ws[45440]) * yin[1632]) * yin[5824];
    ws[62464] = ((ws[45472]) * yin[2784]) * yin[6016];
    ws[62496] = ((ws[45504]) * yin[6016]) * yin[2208];
    ws[62528] = (ws[45536]) * yin[2784];
    ws[62560] = ((ws[45568]) * yin[1664]) * yin[6016];
    ws[62592] = ((ws[45600]) * yin[1408]) * yin[6016];
    ws[62624] = ((ws[45632]) * yin[1440]) * yin[6016];
    ws[62656] = ((ws[45664]) * yin[4544]) * yin[6016];
    ws[62688] = ((ws[45696]) * yin[4576]) * yin[6016];
    ws[62720] = ((ws[45728]) * yin[5856]) * yin[6016];
    ws[62752] = ((ws[45760]) * yin[5568]) * yin[6016];
    ws[62784] = ((ws[45792]) * yin[5760]) * yin[6016];
    ws[62816] = ((ws[45824]) * yin[4480]) * yin[6016];
    ws[62848] = ((ws[45856]) * yin[5280]) * yin[6016];
    ws[62880] = ((ws[45888]) * yin[5504]) * yin[6016];
    ws[62912] = ((ws[45920]) * yin[5344]) * yin[6016];
    ws[62944] = ((ws[45952]) * yin[4128]) * yin[6016];
    ws[62976] = ((ws[45984]) * yin[4736]) * yin[6016];
    ws[63008] = ((ws[46016]) * yin[3872]) * yin[6016];
    ws[63040] = ((ws[46048]) * yin[5376]) * yin[6016];
    ws[63072] = ((ws[46080]) * yin[5248]) * yin[6016];
    ws[63104] = ((ws[46112]) * yin[5472]) * yin[6016];
    ws[63136] = ((ws[46144]) * yin[4320]) * yin[6016];
    ws[63168] = ((ws[46176]) * yin[3584]) * yin[6016];
    ws[63200] = ((ws[46208]) * yin[4448]) * yin[6016];
    ws[63232] = ((ws[46240]) * yin[1248]) * yin[6016];
    ws[63264] = ((ws[46272]) * yin[2944]) * yin[6016];
    ws[63296] = ((ws[46304]) * yin[1760]) * yin[6016];
    ws[63328] = ((ws[46336]) * yin[5600]) * yin[6016];
    ws[63360] = ((ws[46368]) * yin[1472]) * yin[6016];
    ws[63392] = ((ws[46400]) * yin[5056]) * yin[6016];
    ws[63424] = ((ws[46432]) * yin[1504]) * yin[6016];
    ws[63456] = ((ws[46464]) * yin[2816]) * yin[6016];
    ws[63488] = ((ws[46496]) * yin[5728]) * yin[6016];
    ws[63520] = ((ws[46528]) * yin[4096]) * yin[6016];
    ws[63552] = ((ws[46560]) * yin[4608]) * yin[6016];
    ws[63584] = ((ws[46592]) * yin[1792]) * yin[6016];
    ws[63616] = ((ws[46624]) * yin[4352]) * yin[6016];
    ws[63648] = ((ws[46656]) * yin[5696]) * yin[6016];
    ws[63680] = ((ws[46688]) * yin[3680]) * yin[6016];
    ws[63712] = ((ws[46720]) * yin[1088]) * yin[6016];
    ws[63744] = ((ws[46752]) * yin[1536]) * yin[6016];
    ws[63776] = ((ws[46784]) * yin[1824]) * yin[6016];
    ws[63808] = ((ws[46816]) * yin[5440]) * yin[6016];
    ws[63840] = ((ws[46848]) * yin[4384]) * yin[6016];
    ws[63872] = ((ws[46880]) * yin[1696]) * yin[6016];
    ws[63904] = ((ws[46912]) * yin[2240]) * yin[5184];
    ws[63936] = ((ws[46944]) * yin[2752]) * yin[5184];
    ws[63968] = ((ws[46976]) * yin[1152]) * yin[5184];
    ws[64000] = ((ws[47008]) * yin[1408]) * yin[5184];
    ws[64032] = ((ws[47040]) * yin[1440]) * yin[5184];
    ws[64064] = ((ws[47072]) * yin[4576]) * yin[5184];
    ws[64096] = ((ws[47104]) * yin[4384]) * yin[5184];
    ws[64128] = ((ws[47136]) * yin[4128]) * yin[5184];
    ws[64160] = ((ws[47168]) * yin[4736]) * yin[5184];
    ws[64192] = ((ws[47200]) * yin[3872]) * yin[5184];
    ws[64224] = ((ws[47232]) * yin[5472]) * yin[5184];
    ws[64256] = ((ws[47264]) * yin[4320]) * yin[5184];
    ws[64288] = ((ws[47296]) * yin[3584]) * yin[5184];
    ws[64320] = ((ws[47328]) * yin[3808]) * yin[5184];
    ws[64352] = ((ws[47360]) * yin[2240]) * yin[5952];
    ws[64384] = ((ws[47392]) * yin[2752]) * yin[5952];
    ws[64416] = ((ws[47424]) * yin[1152]) * yin[5952];
    ws[64448] = ((ws[47456]) * yin[1408]) * yin[5952];
    ws[64480] = ((ws[47488]) * yin[1440]) * yin[5952];
    ws[64512] = ((ws[47520]) * yin[4384]) * yin[5952];
    ws[64544] = ((ws[47552]) * yin[5856]) * yin[5952];
    ws[64576] = ((ws[47584]) * yin[5568]) * yin[5952];
    ws[64608] = ((ws[47616]) * yin[5760]) * yin[5952];
    ws[64640] = ((ws[47648]) * yin[4128]) * yin[5952];
    ws[64672] = ((ws[47680]) * yin[3872]) * yin[5952];
    ws[64704] = ((ws[47712]) * yin[5376]) * yin[5952];
    ws[64736] = ((ws[47744]) * yin[5248]) * yin[5952];
    ws[64768] = ((ws[47776]) * yin[1248]) * yin[5952];
    ws[64800] = ((ws[47808]) * yin[2944]) * yin[5952];
    ws[64832] = ((ws[47840]) * yin[1760]) * yin[5952];
    ws[64864] = ((ws[47872]) * yin[1824]) * yin[5952];
    ws[64896] = (ws[47904]) * yin[2560];
    ws[64928] = (ws[47936]) * yin[1728];
    ws[64960] = ((ws[47968]) * yin[5792]) * yin[5920];
    ws[64992] = (ws[48000]) * yin[1088];
    ws[65024] = ((ws[48032]) * yin[4800]) * yin[5920];
    ws[65056] = (ws[48064]) * yin[1536];
    ws[65088] = ((ws[48096]) * yin[4672]) * yin[5920];
    ws[65120] = (ws[48128]) * yin[1824];
    ws[65152] = ((ws[48160]) * yin[5888]) * yin[5824];
    ws[65184] = ((ws[48192]) * yin[5632]) * yin[5824];
    ws[65216] = ((ws[48224]) * yin[5408]) * yin[5824];
    ws[65248] = ((ws[48256]) * yin[5120]) * yin[5824];
    ws[65280] = ((ws[48288]) * yin[3008]) * yin[5824];
    ws[65312] = ((ws[48320]) * yin[3200]) * yin[5824];
    ws[65344] = ((ws[48352]) * yin[3328]) * yin[5824];
    ws[65376] = ((ws[48384]) * yin[3360]) * yin[5824];
    ws[65408] = ((ws[48416]) * yin[3296]) * yin[5824];
    ws[65440] = ((ws[48448]) * yin[3104]) * yin[5824];
    ws[65472] = ((ws[48480]) * yin[3264]) * yin[5824];
    ws[65504] = ((ws[48512]) * yin[4160]) * yin[5824];
    ws[65536] = ((ws[48544]) * yin[3744]) * yin[5824];
    ws[65568] = ((ws[48576]) * yin[2624]) * yin[5824];
    ws[65600] = ((ws[48608]) * yin[3840]) * yin[5824];
    ws[65632] = ((ws[48640]) * yin[4192]) * yin[5824];
    ws[65664] = ((ws[48672]) * yin[3936]) * yin[5824];
    ws[65696] = ((ws[48704]) * yin[2656]) * yin[5824];
    ws[65728] = ((ws[48736]) * yin[3712]) * yin[5824];
    ws[65760] = ((ws[48768]) * yin[2560]) * yin[5824];
    ws[65792] = ((ws[48800]) * yin[1728]) * yin[5824];
    ws[65824] = ((ws[48832]) * yin[5792]) * yin[5824];
    ws[65856] = ((ws[48864]) * yin[4800]) * yin[5824];
    ws[65888] = ((ws[48896]) * yin[2848]) * yin[5824];
    ws[65920] = ((ws[48928]) * yin[5152]) * yin[5824];
    ws[65952] = ((ws[48960]) * yin[3776]) * yin[5824];
    ws[65984] = ((ws[48992]) * yin[4672]) * yin[5824];
    ws[66016] = ((ws[49024]) * yin[3520]) * yin[5824];
    ws[66048] = ((ws[49056]) * yin[2880]) * yin[5824];
    ws[66080] = ((ws[49088]) * yin[2912]) * yin[5824];
    ws[66112] = ((ws[49120]) * yin[2592]) * yin[5824];
    ws[66144] = ((ws[49152]) * yin[2272]) * yin[5824];
    ws[66176] = ((ws[49184]) * yin[3648]) * yin[5824];
    ws[66208] = ((ws[49216]) * yin[3040]) * yin[5824];
    ws[66240] = ((ws[49248]) * yin[2976]) * yin[5824];
    ws[66272] = ((ws[49280]) * yin[4032]) * yin[5824];
    ws[66304] = ((ws[49312]) * yin[4064]) * yin[5824];
    ws[66336] = ((ws[49344]) * yin[3072]) * yin[5824];
    ws[66368] = ((ws[49376]) * yin[5216]) * yin[5824];
    ws[66400] = ((ws[49408]) * yin[2688]) * yin[5920];
    ws[66432] = ((ws[49440]) * yin[3232]) * yin[5920];
    ws[66464] = ((ws[49472]) * yin[3808]) * yin[5920];
    ws[66496] = ((ws[49504]) * yin[5888]) * yin[5984];
    ws[66528] = ((ws[49536]) * yin[5632]) * yin[5984];
    ws[66560] = ((ws[49568]) * yin[5408]) * yin[5984];
    ws[66592] = ((ws[49600]) * yin[5120]) * yin[5984];
    ws[66624] = ((ws[49632]) * yin[3008]) * yin[5984];
    ws[66656] = ((ws[49664]) * yin[3200]) * yin[5984];
    ws[66688] = ((ws[49696]) * yin[3328]) * yin[5984];
    ws[66720] = ((ws[49728]) * yin[3360]) * yin[5984];
    ws[66752] = ((ws[49760]) * yin[3296]) * yin[5984];
    ws[66784] = ((ws[49792]) * yin[3104]) * yin[5984];
    ws[66816] = ((ws[49824]) * yin[3264]) * yin[5984];
    ws[66848] = ((ws[49856]) * yin[4160]) * yin[5984];
    ws[66880] = ((ws[49888]) * yin[3744]) * yin[5984];
    ws[66912] = ((ws[49920]) * yin[2624]) * yin[5984];
    ws[66944] = ((ws[49952]) * yin[3840]) * yin[5984];
    ws[66976] = ((ws[49984]) * yin[4192]) * yin[5984];
    ws[67008] = ((ws[50016]) * yin[3936]) * yin[5984];
    ws[67040] = ((ws[50048]) * yin[2656]) * yin[5984];
    ws[67072] = ((ws[50080]) * yin[3712]) * yin[5984];
    ws[67104] = ((ws[50112]) * yin[2560]) * yin[5984];
    ws[67136] = ((ws[50144]) * yin[1728]) * yin[5984];
    ws[67168] = ((ws[50176]) * yin[5792]) * yin[5984];
    ws[67200] = ((ws[50208]) * yin[4800]) * yin[5984];
    ws[67232] = ((ws[50240]) * yin[2848]) * yin[5984];
    ws[67264] = ((ws[50272]) * yin[5152]) * yin[5984];
    ws[67296] = ((ws[50304]) * yin[3776]) * yin[5984];
    ws[67328] = ((ws[50336]) * yin[4672]) * yin[5984];
    ws[67360] = ((ws[50368]) * yin[3520]) * yin[5984];
    ws[67392] = ((ws[50400]) * yin[2880]) * yin[5984];
    ws[67424] = ((ws[50432]) * yin[2912]) * yin[5984];
    ws[67456] = ((ws[50464]) * yin[3648]) * yin[5984];
    ws[67488] = ((ws[50496]) * yin[3232]) * yin[5984];
    ws[67520] = ((ws[50528]) * yin[3040]) * yin[5984];
    ws[67552] = ((ws[50560]) * yin[2976]) * yin[5984];
    ws[67584] = ((ws[50592]) * yin[4032]) * yin[5984];
    ws[67616] = ((ws[50624]) * yin[4064]) * yin[5984];
    ws[67648] = ((ws[50656]) * yin[3072]) * yin[5984];
    ws[67680] = ((ws[50688]) * yin[5216]) * yin[5984];
    ws[67712] = ((ws[50720]) * yin[5888]) * yin[5888];
    ws[67744] = ((ws[50752]) * yin[5632]) * yin[5888];
    ws[67776] = ((ws[50784]) * yin[5408]) * yin[5888];
    ws[67808] = ((ws[50816]) * yin[5120]) * yin[5888];
    ws[67840] = ((ws[50848]) * yin[3008]) * yin[5888];
    ws[67872] = ((ws[50880]) * yin[3200]) * yin[5888];
    ws[67904] = ((ws[50912]) * yin[3328]) * yin[5888];
    ws[67936] = ((ws[50944]) * yin[3360]) * yin[5888];
    ws[67968] = ((ws[50976]) * yin[3296]) * yin[5888];
    ws[68000] = ((ws[51008]) * yin[3104]) * yin[5888];
    ws[68032] = ((ws[51040]) * yin[3264]) * yin[5888];
    ws[68064] = ((ws[51072]) * yin[4288]) * yin[5888];
    ws[68096] = ((ws[51104]) * yin[4160]) * yin[5888];
    ws[68128] = ((ws[51136]) * yin[3744]) * yin[5888];
    ws[68160] = ((ws[51168]) * yin[2624]) * yin[5888];
    ws[68192] = ((ws[51200]) * yin[3840]) * yin[5888];
    ws[68224] = ((ws[51232]) * yin[4192]) * yin[5888];
    ws[68256] = ((ws[51264]) * yin[3936]) * yin[5888];
    ws[68288] = ((ws[51296]) * yin[2656]) * yin[5888];
    ws[68320] = ((ws[51328]) * yin[3712]) * yin[5888];
    ws[68352] = ((ws[51360]) * yin[5792]) * yin[5888];
    ws[68384] = ((ws[51392]) * yin[4800]) * yin[5888];
    ws[68416] = ((ws[51424]) * yin[2848]) * yin[5888];
    ws[68448] = ((ws[51456]) * yin[5152]) * yin[5888];
    ws[68480] = ((ws[51488]) * yin[3776]) * yin[5888];
    ws[68512] = ((ws[51520]) * yin[4672]) * yin[5888];
    ws[68544] = ((ws[51552]) * yin[3520]) * yin[5888];
    ws[68576] = ((ws[51584]) * yin[2880]) * yin[5888];
    ws[68608] = ((ws[51616]) * yin[2912]) * yin[5888];
    ws[68640] = ((ws[51648]) * yin[2592]) * yin[5888];
    ws[68672] = ((ws[51680]) * yin[2272]) * yin[5888];
    ws[68704] = ((ws[51712]) * yin[3648]) * yin[5888];
    ws[68736] = ((ws[51744]) * yin[3040]) * yin[5888];
    ws[68768] = ((ws[51776]) * yin[2976]) * yin[5888];
    ws[68800] = ((ws[51808]) * yin[4032]) * yin[5888];
    ws[68832] = ((ws[51840]) * yin[4064]) * yin[5888];
    ws[68864] = ((ws[51872]) * yin[3072]) * yin[5888];
    ws[68896] = ((ws[51904]) * yin[5216]) * yin[5888];
    ws[68928] = ((ws[51936]) * yin[5632]) * yin[5792];
    ws[68960] = ((ws[51968]) * yin[5408]) * yin[5792];
    ws[68992] = ((ws[52000]) * yin[5120]) * yin[5792];
    ws[69024] = ((ws[52032]) * yin[3008]) * yin[5792];
    ws[69056] = ((ws[52064]) * yin[3200]) * yin[5792];
    ws[69088] = ((ws[52096]) * yin[3328]) * yin[5792];
    ws[69120] = ((ws[52128]) * yin[3360]) * yin[5792];
    ws[69152] = ((ws[52160]) * yin[3296]) * yin[5792];
    ws[69184] = ((ws[52192]) * yin[3104]) * yin[5792];
    ws[69216] = ((ws[52224]) * yin[3264]) * yin[5792];
    ws[69248] = ((ws[52256]) * yin[4288]) * yin[5792];
    ws[69280] = ((ws[52288]) * yin[4160]) * yin[5792];
    ws[69312] = ((ws[52320]) * yin[3744]) * yin[5792];
    ws[69344] = ((ws[52352]) * yin[2624]) * yin[5792];
    ws[69376] = ((ws[52384]) * yin[3840]) * yin[5792];
    ws[69408] = ((ws[52416]) * yin[4192]) * yin[5792];
    ws[69440] = ((ws[52448]) * yin[3936]) * yin[5792];
    ws[69472] = ((ws[52480]) * yin[2656]) * yin[5792];
    ws[69504] = ((ws[52512]) * yin[3712]) * yin[5792];
    ws[69536] = ((ws[52544]) * yin[5792]) * yin[5792];
    ws[69568] = ((ws[52576]) * yin[4800]) * yin[5792];
    ws[69600] = ((ws[52608]) * yin[2848]) * yin[5792];
    ws[69632] = ((ws[52640]) * yin[5152]) * yin[5792];
    ws[69664] = ((ws[52672]) * yin[3776]) * yin[5792];
    ws[69696] = ((ws[52704]) * yin[4672]) * yin[5792];
    ws[69728] = ((ws[52736]) * yin[3520]) * yin[5792];
    ws[69760] = ((ws[52768]) * yin[2880]) * yin[5792];
    ws[69792] = ((ws[52800]) * yin[2912]) * yin[5792];
    ws[69824] = ((ws[52832]) * yin[2592]) * yin[5792];
    ws[69856] = ((ws[52864]) * yin[2272]) * yin[5792];
    ws[69888] = ((ws[52896]) * yin[3648]) * yin[5792];
    ws[69920] = ((ws[52928]) * yin[3040]) * yin[5792];
    ws[69952] = ((ws[52960]) * yin[2976]) * yin[5792];
    ws[69984] = ((ws[52992]) * yin[4032]) * yin[5792];
    ws[70016] = ((ws[53024]) * yin[4064]) * yin[5792];
    ws[70048] = ((ws[53056]) * yin[3072]) * yin[5792];
    ws[70080] = ((ws[53088]) * yin[5216]) * yin[5792];
    ws[70112] = ((ws[53120]) * yin[4800]) * yin[4800];
    ws[70144] = ((ws[53152]) * yin[5888]) * yin[5952];
    ws[70176] = ((ws[53184]) * yin[5632]) * yin[5952];
    ws[70208] = ((ws[53216]) * yin[5408]) * yin[5952];
    ws[70240] = ((ws[53248]) * yin[5120]) * yin[5952];
    ws[70272] = ((ws[53280]) * yin[3008]) * yin[5952];
    ws[70304] = ((ws[53312]) * yin[3200]) * yin[5952];
    ws[70336] = ((ws[53344]) * yin[3328]) * yin[5952];
    ws[70368] = ((ws[53376]) * yin[3360]) * yin[5952];
    ws[70400] = ((ws[53408]) * yin[3296]) * yin[5952];
    ws[70432] = ((ws[53440]) * yin[3104]) * yin[5952];
    ws[70464] = ((ws[53472]) * yin[3264]) * yin[5952];
    ws[70496] = ((ws[53504]) * yin[4288]) * yin[5952];
    ws[70528] = ((ws[53536]) * yin[4160]) * yin[5952];
    ws[70560] = ((ws[53568]) * yin[4192]) * yin[5952];
    ws[70592] = ((ws[53600]) * yin[2624]) * yin[5952];
    ws[70624] = ((ws[53632]) * yin[2656]) * yin[5952];
    ws[70656] = ((ws[53664]) * yin[5792]) * yin[5952];
    ws[70688] = ((ws[53696]) * yin[4800]) * yin[5952];
    ws[70720] = ((ws[53728]) * yin[2848]) * yin[5952];
    ws[70752] = ((ws[53760]) * yin[5152]) * yin[5952];
    ws[70784] = ((ws[53792]) * yin[3776]) * yin[5952];
    ws[70816] = ((ws[53824]) * yin[4672]) * yin[5952];
    ws[70848] = ((ws[53856]) * yin[3520]) * yin[5952];
    ws[70880] = ((ws[53888]) * yin[2880]) * yin[5952];
    ws[70912] = ((ws[53920]) * yin[2912]) * yin[5952];
    ws[70944] = ((ws[53952]) * yin[2592]) * yin[5952];
    ws[70976] = ((ws[53984]) * yin[2272]) * yin[5952];
    ws[71008] = ((ws[54016]) * yin[3648]) * yin[5952];
    ws[71040] = ((ws[54048]) * yin[3040]) * yin[5952];
    ws[71072] = ((ws[54080]) * yin[2976]) * yin[5952];
    ws[71104] = ((ws[54112]) * yin[4032]) * yin[5952];
    ws[71136] = ((ws[54144]) * yin[4064]) * yin[5952];
    ws[71168] = ((ws[54176]) * yin[3072]) * yin[5952];
    ws[71200] = ((ws[54208]) * yin[4032]) * yin[4032];
    ws[71232] = ((ws[54240]) * yin[4032]) * yin[4064];
    ws[71264] = ((ws[54272]) * yin[4064]) * yin[4064];
    ws[71296] = ((ws[54304]) * yin[5216]) * yin[5952];
    ws[71328] = ((ws[54336]) * yin[5216]) * yin[4800];
    ws[71360] = ((ws[54368]) * yin[5216]) * yin[5216];
    ws[71392] = ((ws[54400]) * yin[3744]) * yin[4160];
    ws[71424] = ((ws[54432]) * yin[3744]) * yin[4192];
    ws[71456] = ((ws[54464]) * yin[3744]) * yin[4288];
    ws[71488] = ((ws[54496]) * yin[3936]) * yin[4160];
    ws[71520] = ((ws[54528]) * yin[3936]) * yin[4192];
    ws[71552] = ((ws[54560]) * yin[3936]) * yin[4288];
    ws[71584] = ((ws[54592]) * yin[3840]) * yin[4160];
    ws[71616] = ((ws[54624]) * yin[3840]) * yin[4192];
    ws[71648] = ((ws[54656]) * yin[3840]) * yin[4288];
    ws[71680] = ((ws[54688]) * yin[3712]) * yin[4160];
    ws[71712] = ((ws[54720]) * yin[3712]) * yin[4192];
    ws[71744] = ((ws[54752]) * yin[3712]) * yin[4288];
    ws[71776] = ((ws[54784]) * yin[1376]) * yin[6016];
    ws[71808] = ((ws[54816]) * yin[384]) * yin[6016];
    ws[71840] = ((ws[54848]) * yin[416]) * yin[6016];
    ws[71872] = ((ws[54880]) * yin[3552]) * yin[6016];
    ws[71904] = ((ws[54912]) * yin[3552]) * yin[5184];
    ws[71936] = ((ws[54944]) * yin[3552]) * yin[5952];
    ws[71968] = (ws[54976]) * yin[3552];
    ws[72000] = ((ws[55008]) * yin[1568]) * yin[6016];
    ws[72032] = ((ws[55040]) * yin[3136]) * yin[5824];
    ws[72064] = ((ws[55072]) * yin[3136]) * yin[5952];
    ws[72096] = ((ws[55104]) * yin[3136]) * yin[5984];
    ws[72128] = ((ws[55136]) * yin[3136]) * yin[5888];
    ws[72160] = ((ws[55168]) * yin[3136]) * yin[5792];
    ws[72192] = ((ws[55200]) * yin[1568]) * yin[5184];
    ws[72224] = ((ws[55232]) * yin[1568]) * yin[5952];
    ws[72256] = ((ws[55264]) * yin[3168]) * yin[6016];
    ws[72288] = ((ws[55296]) * yin[1856]) * yin[5824];
    ws[72320] = ((ws[55328]) * yin[1856]) * yin[5984];
    ws[72352] = ((ws[55360]) * yin[4512]) * yin[6016];
    ws[72384] = ((ws[55392]) * yin[3168]) * yin[5184];
    ws[72416] = ((ws[55424]) * yin[3168]) * yin[5952];
    ws[72448] = ((ws[55456]) * yin[448]) * yin[6016];
    ws[72480] = ((ws[55488]) * yin[1600]) * yin[5952];
    ws[72512] = ((ws[55520]) * yin[1920]) * yin[5984];
    ws[72544] = ((ws[55552]) * yin[1920]) * yin[5824];
    ws[72576] = ((ws[55584]) * yin[1920]) * yin[5952];
    ws[72608] = ((ws[55616]) * yin[1600]) * yin[5184];
    ws[72640] = ((ws[55648]) * yin[1600]) * yin[6016];
    ws[72672] = ((ws[55680]) * yin[2304]) * yin[5984];
    ws[72704] = ((ws[55712]) * yin[2304]) * yin[5952];
    ws[72736] = ((ws[55744]) * yin[2304]) * yin[5824];
    ws[72768] = (ws[55776]) * yin[5376];
    ws[72800] = (ws[55808]) * yin[5248];
    ws[72832] = (ws[55840]) * yin[1024];
    ws[72864] = (ws[55872]) * yin[5920];
    ws[72896] = (ws[55904]) * yin[5984];
    ws[72928] = (ws[55936]) * yin[5952];
    ws[72960] = (ws[55968]) * yin[5184];
    ws[72992] = (ws[56000]) * yin[1376];
    ws[73024] = (ws[56032]) * yin[1056];
    ws[73056] = ((ws[56064]) * yin[1056]) * yin[512];
    ws[73088] = (ws[56096]) * yin[1664];
    ws[73120] = (ws[56128]) * yin[2208];
    ws[73152] = ((ws[56160]) * yin[608]) * yin[6016];
    ws[73184] = ((ws[56192]) * yin[640]) * yin[6016];
    ws[73216] = ((ws[56224]) * yin[672]) * yin[6016];
    ws[73248] = ((ws[56256]) * yin[704]) * yin[6016];
    ws[73280] = ((ws[56288]) * yin[736]) * yin[6016];
    ws[73312] = ((ws[56320]) * yin[768]) * yin[6016];
    ws[73344] = ((ws[56352]) * yin[800]) * yin[6016];
    ws[73376] = ((ws[56384]) * yin[2368]) * yin[5824];
    ws[73408] = ((ws[56416]) * yin[2400]) * yin[5824];
    ws[73440] = ((ws[56448]) * yin[2432]) * yin[5824];
    ws[73472] = ((ws[56480]) * yin[2464]) * yin[5824];
    ws[73504] = ((ws[56512]) * yin[2496]) * yin[5824];
    ws[73536] = ((ws[56544]) * yin[2528]) * yin[5824];
    ws[73568] = ((ws[56576]) * yin[3904]) * yin[5824];
    ws[73600] = ((ws[56608]) * yin[2368]) * yin[5952];
    ws[73632] = ((ws[56640]) * yin[2400]) * yin[5952];
    ws[73664] = ((ws[56672]) * yin[2432]) * yin[5952];
    ws[73696] = ((ws[56704]) * yin[2464]) * yin[5952];
    ws[73728] = ((ws[56736]) * yin[2496]) * yin[5952];
    ws[73760] = ((ws[56768]) * yin[2528]) * yin[5952];
    ws[73792] = ((ws[56800]) * yin[3904]) * yin[5952];
    ws[73824] = ((ws[56832]) * yin[2368]) * yin[5984];
    ws[73856] = ((ws[56864]) * yin[2400]) * yin[5984];
    ws[73888] = ((ws[56896]) * yin[2432]) * yin[5984];
    ws[73920] = ((ws[56928]) * yin[2464]) * yin[5984];
    ws[73952] = ((ws[56960]) * yin[2496]) * yin[5984];
    ws[73984] = ((ws[56992]) * yin[2528]) * yin[5984];
    ws[74016] = ((ws[57024]) * yin[3904]) * yin[5984];
    ws[74048] = (ws[57056]) * yin[1952];
    ws[74080] = (ws[57088]) * yin[1984];
    ws[74112] = (ws[57120]) * yin[2016];
    ws[74144] = (ws[57152]) * yin[2048];
    ws[74176] = (ws[57184]) * yin[2080];
    ws[74208] = (ws[57216]) * yin[2112];
    ws[74240] = (ws[57248]) * yin[2144];
    ws[74272] = ((ws[57280]) * yin[1952]) * yin[5824];
    ws[74304] = ((ws[57312]) * yin[1984]) * yin[5824];
    ws[74336] = ((ws[57344]) * yin[2016]) * yin[5824];
    ws[74368] = ((ws[57376]) * yin[2048]) * yin[5824];
    ws[74400] = ((ws[57408]) * yin[2080]) * yin[5824];
    ws[74432] = ((ws[57440]) * yin[2112]) * yin[5824];
    ws[74464] = ((ws[57472]) * yin[2144]) * yin[5824];
    ws[74496] = ((ws[57504]) * yin[1952]) * yin[5952];
    ws[74528] = ((ws[57536]) * yin[1984]) * yin[5952];
    ws[74560] = ((ws[57568]) * yin[2016]) * yin[5952];
    ws[74592] = ((ws[57600]) * yin[2048]) * yin[5952];
    ws[74624] = ((ws[57632]) * yin[2080]) * yin[5952];
    ws[74656] = ((ws[57664]) * yin[2112]) * yin[5952];
    ws[74688] = ((ws[57696]) * yin[2144]) * yin[5952];
    ws[74720] = ((ws[57728]) * yin[1952]) * yin[5984];
    ws[74752] = ((ws[57760]) * yin[1984]) * yin[5984];
    ws[74784] = ((ws[57792]) * yin[2016]) * yin[5984];
    ws[74816] = ((ws[57824]) * yin[2048]) * yin[5984];
    ws[74848] = ((ws[57856]) * yin[2080]) * yin[5984];
    ws[74880] = ((ws[57888]) * yin[2112]) * yin[5984];
    ws[74912] = ((ws[57920]) * yin[2144]) * yin[5984];
    ws[74944] = ((ws[57952]) * yin[832]) * yin[6016];
    ws[74976] = ((ws[57984]) * yin[3392]) * yin[5984];
    ws[75008] = ((ws[58016]) * yin[3392]) * yin[5824];
    ws[75040] = ((ws[58048]) * yin[3392]) * yin[5952];
    ws[75072] = ((ws[58080]) * yin[3392]) * yin[5888];
    ws[75104] = ((ws[58112]) * yin[3392]) * yin[5792];
    ws[75136] = ((ws[58144]) * yin[864]) * yin[6016];
    ws[75168] = ((ws[58176]) * yin[3424]) * yin[5984];
    ws[75200] = ((ws[58208]) * yin[3424]) * yin[5824];
    ws[75232] = ((ws[58240]) * yin[3424]) * yin[5952];
    ws[75264] = ((ws[58272]) * yin[3424]) * yin[5888];
    ws[75296] = ((ws[58304]) * yin[3424]) * yin[5792];
    ws[75328] = ((ws[58336]) * yin[896]) * yin[6016];
    ws[75360] = ((ws[58368]) * yin[3456]) * yin[5984];
    ws[75392] = ((ws[58400]) * yin[3456]) * yin[5824];
    ws[75424] = ((ws[58432]) * yin[3456]) * yin[5952];
    ws[75456] = ((ws[58464]) * yin[3456]) * yin[5888];
    ws[75488] = ((ws[58496]) * yin[3456]) * yin[5792];
    ws[75520] = ((ws[58528]) * yin[4768]) * yin[6016];
    ws[75552] = ((ws[58560]) * yin[4864]) * yin[6016];
    ws[75584] = ((ws[58592]) * yin[4832]) * yin[6016];
    ws[75616] = ((ws[58624]) * yin[4896]) * yin[6016];
    ws[75648] = ((ws[58656]) * yin[4640]) * yin[6016];
    ws[75680] = ((ws[58688]) * yin[4416]) * yin[6016];
    ws[75712] = ((ws[58720]) * yin[4928]) * yin[6016];
    ws[75744] = ((ws[58752]) * yin[4960]) * yin[6016];
    ws[75776] = ((ws[58784]) * yin[4992]) * yin[6016];
    ws[75808] = ((ws[58816]) * yin[4704]) * yin[6016];
    ws[75840] = ((ws[58848]) * yin[5088]) * yin[6016];
    ws[75872] = ((ws[58880]) * yin[5536]) * yin[6016];
    ws[75904] = ((ws[58912]) * yin[5312]) * yin[6016];
    ws[75936] = ((ws[58944]) * yin[4224]) * yin[6016];
    ws[75968] = ((ws[58976]) * yin[3968]) * yin[6016];
    ws[76000] = ((ws[59008]) * yin[4608]) * yin[6016];
    ws[76032] = ((ws[59040]) * yin[928]) * yin[6016];
    ws[76064] = (ws[59072]) * yin[96];
    ws[76096] = (ws[59104]) * yin[128];
    ws[76128] = ((ws[59136]) * yin[992]) * yin[6016];
    ws[76160] = ((ws[59168]) * yin[3488]) * yin[5984];
    ws[76192] = ((ws[59200]) * yin[3488]) * yin[5824];
    ws[76224] = ((ws[59232]) * yin[3488]) * yin[5952];
    ws[76256] = ((ws[59264]) * yin[3488]) * yin[5888];
    ws[76288] = ((ws[59296]) * yin[3488]) * yin[5792];
    {
      double a = 1.0 * ws[73024];
      yout[0] = a;
    }
    {
      double a = 1.0 * ws[73088];
      yout[32] = a;
    }
    {
      double a = 1.0 * ws[73120];
      yout[64] = a;
    }
    {
      double a = -ws[76064];
      yout[96] = a;
    }
    {
      double a = -ws[76096];
      yout[128] = a;
    }
    {
      double a = -ws[61728];
      yout[160] = a;
    }
    {
      double a = 1.0 * ws[61728];
      yout[192] = a;
    }
    {
      double a = 1.0 * ws[61728];
      yout[224] = a;
    }
    {
      double a = -ws[62016];
      yout[256] = a;
    }
    {
      double a = -ws[62080];
      yout[288] = a;
    }
    {
      double a = -ws[62112];
      yout[320] = a;
    }
    {
      double a = -ws[62144];
      yout[352] = a;
    }
    {
      double a = -ws[71808];
      yout[384] = a;
    }
    {
      double a = -ws[71840];
      yout[416] = a;
    }
    {
      double a = -ws[72448];
      yout[448] = a;
    }
    {
      double a = 1.0 * ws[72768];
      a = fma(1.0, ws[72800], a);
      yout[480] = a;
    }
    {
      double a = -ws[73056];
      yout[512] = a;
    }
    {
      double a = 1.0 * ws[73056];
      yout[544] = a;
    }
    {
      double a = 1.0 * ws[59360];
      a = a - ws[60800];
      a = a - ws[60832];
      a = a - ws[60864];
      yout[576] = a;
    }
    {
      double a = -ws[73152];
      yout[608] = a;
    }
    {
      double a = -ws[73184];
      yout[640] = a;
    }
    {
      double a = -ws[73216];
      yout[672] = a;
    }
    {
      double a = -ws[73248];
      yout[704] = a;
    }
    {
      double a = -ws[73280];
      yout[736] = a;
    }
    {
      double a = -ws[73312];
      yout[768] = a;
    }
    {
      double a = -ws[73344];
      yout[800] = a;
    }
    {
      double a = -ws[74944];
      yout[832] = a;
    }
    {
      double a = -ws[75136];
      yout[864] = a;
    }
    {
      double a = -ws[75328];
      yout[896] = a;
    }
    {
      double a = -ws[76032];
      yout[928] = a;
    }
    {
      double a = 1.0 * ws[76064];
      a = fma(1.0, ws[76096], a);
      yout[960] = a;
    }
    {
      double a = -ws[76128];
      yout[992] = a;
    }
    {
      double a = 1.0 * ws[61536];
      a = a - ws[61568];
      a = a - ws[61600];
      a = a - ws[72832];
      yout[1024] = a;
    }
    {
      double a = 1.0 * ws[72992];
      a = a - ws[73024];
      a = a - ws[73056];
      yout[1056] = a;
    }
    {
      double a = -ws[60480];
      a = a - ws[60512];
      a = a - ws[63712];
      a = fma(1.0, ws[64960], a);
      a = a - ws[64992];
      yout[1088] = a;
    }
    {
      double a = -ws[61888];
      a = fma(0.006, ws[63936], a);
      yout[1120] = a;
    }
    {
      double a = -ws[61984];
      a = a - ws[63968];
      a = a - ws[64416];
      yout[1152] = a;
    }
    {
      double a = -ws[59520];
      a = fma(1.0, ws[61088], a);
      a = a - ws[61216];
      a = fma(0.5, ws[72864], a);
      yout[1184] = a;
    }
    {
      double a = -ws[62048];
      a = fma(0.032, ws[63936], a);
      yout[1216] = a;
    }
    {
      double a = 0.53 * ws[62048];
      a = a - ws[63232];
      a = a - ws[64768];
      yout[1248] = a;
    }
    {
      double a = -ws[59584];
      a = fma(1.0, ws[61632], a);
      a = a - ws[61664];
      a = a - ws[61696];
      yout[1280] = a;
    }
    {
      double a = -ws[62176];
      a = a - ws[62208];
      a = a - ws[62240];
      yout[1312] = a;
    }
    {
      double a = 1.0 * ws[62272];
      a = a - ws[62336];
      a = a - ws[62368];
      yout[1344] = a;
    }
    {
      double a = 0.44 * ws[62368];
      a = fma(0.17, ws[62464], a);
      a = a - ws[71776];
      a = a - ws[72992];
      yout[1376] = a;
    }
    {
      double a = -ws[62592];
      a = a - ws[64000];
      a = a - ws[64448];
      yout[1408] = a;
    }
    {
      double a = -ws[62624];
      a = a - ws[64032];
      a = a - ws[64480];
      yout[1440] = a;
    }
    {
      double a = -ws[63360];
      a = fma(0.25, ws[67744], a);
      yout[1472] = a;
    }
    {
      double a = -ws[63424];
      a = fma(0.25, ws[67840], a);
      yout[1504] = a;
    }
    {
      double a = -ws[63744];
      a = fma(1.0, ws[65024], a);
      a = a - ws[65056];
      yout[1536] = a;
    }
    {
      double a = -ws[72000];
      a = a - ws[72192];
      a = a - ws[72224];
      yout[1568] = a;
    }
    {
      double a = -ws[72480];
      a = a - ws[72608];
      a = a - ws[72640];
      yout[1600] = a;
    }
    {
      double a = 0.555 * ws[62208];
      a = a - ws[62400];
      a = a - ws[62432];
      yout[1632] = a;
    }
    {
      double a = 0.14 * ws[62368];
      a = fma(0.02, ws[62400], a);
      a = a - ws[62560];
      a = a - ws[73088];
      yout[1664] = a;
    }
    {
      double a = -ws[60576];
      a = fma(0.33, ws[63840], a);
      a = a - ws[63872];
      a = fma(0.33, ws[64096], a);
      a = fma(0.33, ws[64512], a);
      yout[1696] = a;
    }
    {
      double a = 0.83 * ws[62688];
      a = a - ws[64928];
      a = a - ws[65792];
      a = a - ws[67136];
      yout[1728] = a;
    }
    {
      double a = 0.619 * ws[63232];
      a = fma(0.584, ws[63264], a);
      a = a - ws[63296];
      a = a - ws[64832];
      yout[1760] = a;
    }
    {
      double a = -ws[63584];
      a = fma(1.0, ws[67328], a);
      a = fma(1.0, ws[67360], a);
      yout[1792] = a;
    }
    {
      double a = -ws[63776];
      a = a - ws[64864];
      a = fma(1.0, ws[65088], a);
      a = a - ws[65120];
      yout[1824] = a;
    }
    {
      double a = 0.51 * ws[72256];
      a = a - ws[72288];
      a = a - ws[72320];
      yout[1856] = a;
    }
    {
      double a = -ws[61824];
      a = fma(0.02, ws[63936], a);
      a = fma(0.01, ws[63968], a);
      yout[1888] = a;
    }
    {
      double a = 1.0 * ws[72480];
      a = a - ws[72512];
      a = a - ws[72544];
      a = a - ws[72576];
      yout[1920] = a;
    }
    {
      double a = 0.72 * ws[73376];
      a = fma(1.0, ws[73600], a);
      a = a - ws[74048];
      a = a - ws[74272];
      a = a - ws[74496];
      a = a - ws[74720];
      yout[1952] = a;
    }
    {
      double a = 0.72 * ws[73408];
      a = fma(1.0, ws[73632], a);
      a = a - ws[74080];
      a = a - ws[74304];
      a = a - ws[74528];
      a = a - ws[74752];
      yout[1984] = a;
    }
    {
      double a = 0.72 * ws[73440];
      a = fma(1.0, ws[73664], a);
      a = a - ws[74112];
      a = a - ws[74336];
      a = a - ws[74560];
      a = a - ws[74784];
      yout[2016] = a;
    }
    {
      double a = 0.72 * ws[73472];
      a = fma(1.0, ws[73696], a);
      a = a - ws[74144];
      a = a - ws[74368];
      a = a - ws[74592];
      a = a - ws[74816];
      yout[2048] = a;
    }
    {
      double a = 0.72 * ws[73504];
      a = fma(1.0, ws[73728], a);
      a = a - ws[74176];
      a = a - ws[74400];
      a = a - ws[74624];
      a = a - ws[74848];
      yout[2080] = a;
    }
    {
      double a = 0.72 * ws[73536];
      a = fma(1.0, ws[73760], a);
      a = a - ws[74208];
      a = a - ws[74432];
      a = a - ws[74656];
      a = a - ws[74880];
      yout[2112] = a;
    }
    {
      double a = 0.74 * ws[73568];
      a = fma(1.0, ws[73792], a);
      a = a - ws[74240];
      a = a - ws[74464];
      a = a - ws[74688];
      a = a - ws[74912];
      yout[2144] = a;
    }
    {
      double a = -ws[61856];
      a = fma(0.015, ws[63936], a);
      a = fma(0.01, ws[63968], a);
      a = fma(0.0665, ws[64000], a);
      yout[2176] = a;
    }
    {
      double a = 0.95 * ws[62400];
      a = fma(0.65, ws[62432], a);
      a = fma(0.35, ws[62464], a);
      a = a - ws[62496];
      a = a - ws[73120];
      yout[2208] = a;
    }
    {
      double a = -ws[61920];
      a = a - ws[63904];
      a = a - ws[64352];
      a = fma(0.25, ws[71968], a);
      a = fma(0.17, ws[72192], a);
      yout[2240] = a;
    }
    {
      double a = 1.0 * ws[66112];
      a = a - ws[66144];
      a = fma(1.0, ws[68640], a);
      a = a - ws[68672];
      a = fma(1.0, ws[69824], a);
      a = a - ws[69856];
      a = fma(1.0, ws[70944], a);
      a = a - ws[70976];
      yout[2272] = a;
    }
    {
      double a = 1.0 * ws[72640];
      a = a - ws[72672];
      a = a - ws[72704];
      a = a - ws[72736];
      yout[2304] = a;
    }
    {
      double a = 1.0 * ws[59328];
      a = fma(1.0, ws[59424], a);
      a = fma(1.0, ws[59488], a);
      a = a - ws[60736];
      a = a - ws[60768];
      a = fma(1.0, ws[60800], a);
      a = fma(1.0, ws[60832], a);
      a = a - ws[61056];
      a = a - ws[61248];
      a = a - ws[61280];
      yout[2336] = a;
    }
    {
      double a = 1.0 * ws[73152];
      a = a - ws[73376];
      a = a - ws[73600];
      a = a - ws[73824];
      yout[2368] = a;
    }
    {
      double a = 1.0 * ws[73184];
      a = a - ws[73408];
      a = a - ws[73632];
      a = a - ws[73856];
      yout[2400] = a;
    }
    {
      double a = 1.0 * ws[73216];
      a = a - ws[73440];
      a = a - ws[73664];
      a = a - ws[73888];
      yout[2432] = a;
    }
    {
      double a = 1.0 * ws[73248];
      a = a - ws[73472];
      a = a - ws[73696];
      a = a - ws[73920];
      yout[2464] = a;
    }
    {
      double a = 1.0 * ws[73280];
      a = a - ws[73504];
      a = a - ws[73728];
      a = a - ws[73952];
      yout[2496] = a;
    }
    {
      double a = 1.0 * ws[73312];
      a = a - ws[73536];
      a = a - ws[73760];
      a = a - ws[73984];
      yout[2528] = a;
    }
    {
      double a = 0.23 * ws[62656];
      a = fma(0.2145, ws[64000], a);
      a = a - ws[64896];
      a = a - ws[65760];
      a = a - ws[67104];
      yout[2560] = a;
    }
    {
      double a = 1.0 * ws[63200];
      a = a - ws[66112];
      a = a - ws[68640];
      a = a - ws[69824];
      a = a - ws[70944];
      yout[2592] = a;
    }
    {
      double a = 0.975 * ws[64448];
      a = a - ws[65568];
      a = a - ws[66912];
      a = a - ws[68160];
      a = a - ws[69344];
      a = a - ws[70592];
      yout[2624] = a;
    }
    {
      double a = 0.945 * ws[64480];
      a = a - ws[65696];
      a = a - ws[67040];
      a = a - ws[68288];
      a = a - ws[69472];
      a = a - ws[70624];
      yout[2656] = a;
    }
    {
      double a = 1.0 * ws[66144];
      a = a - ws[66400];
      a = fma(1.0, ws[68672], a);
      a = fma(1.0, ws[69856], a);
      a = fma(1.0, ws[70976], a);
      yout[2688] = a;
    }
    {
      double a = 0.04 * ws[71392];
      a = fma(0.04, ws[71424], a);
      a = fma(0.04, ws[71456], a);
      a = fma(0.04, ws[71488], a);
      a = fma(0.04, ws[71520], a);
      a = fma(0.04, ws[71552], a);
      a = fma(0.04, ws[71584], a);
      a = fma(0.04, ws[71616], a);
      a = fma(0.04, ws[71648], a);
      a = fma(0.04, ws[71680], a);
      a = fma(0.04, ws[71712], a);
      a = fma(0.04, ws[71744], a);
      yout[2720] = a;
    }
    {
      double a = -ws[61952];
      a = fma(0.153, ws[62176], a);
      a = a - ws[63936];
      a = a - ws[64384];
      a = fma(0.25, ws[72128], a);
      yout[2752] = a;
    }
    {
      double a = 0.045 * ws[62208];
      a = fma(0.13, ws[62304], a);
      a = fma(0.05, ws[62432], a);
      a = a - ws[62464];
      a = a - ws[62528];
      yout[2784] = a;
    }
    {
      double a = -ws[60288];
      a = a - ws[63456];
      a = fma(0.0385, ws[64000], a);
      a = fma(0.23, ws[64064], a);
      a = fma(1.0, ws[66496], a);
      yout[2816] = a;
    }
    {
      double a = 1.0 * ws[62816];
      a = a - ws[65888];
      a = a - ws[67232];
      a = a - ws[68416];
      a = a - ws[69600];
      a = a - ws[70720];
      yout[2848] = a;
    }
    {
      double a = 1.0 * ws[62976];
      a = a - ws[66048];
      a = a - ws[67392];
      a = a - ws[68576];
      a = a - ws[69760];
      a = a - ws[70880];
      yout[2880] = a;
    }
    {
      double a = 0.687 * ws[63008];
      a = a - ws[66080];
      a = a - ws[67424];
      a = a - ws[68608];
      a = a - ws[69792];
      a = a - ws[70912];
      yout[2912] = a;
    }
    {
      double a = 0.18 * ws[62080];
      a = fma(0.17, ws[62112], a);
      a = fma(0.18, ws[62144], a);
      a = a - ws[63264];
      a = a - ws[64800];
      a = fma(1.0, ws[67488], a);
      yout[2944] = a;
    }
    {
      double a = 0.36 * ws[63648];
      a = a - ws[66240];
      a = a - ws[67552];
      a = a - ws[68768];
      a = a - ws[69952];
      a = a - ws[71072];
      yout[2976] = a;
    }
    {
      double a = 1.0 * ws[61920];
      a = a - ws[65280];
      a = a - ws[66624];
      a = a - ws[67840];
      a = a - ws[69024];
      a = a - ws[70272];
      yout[3008] = a;
    }
    {
      double a = 1.0 * ws[64320];
      a = a - ws[66208];
      a = a - ws[67520];
      a = a - ws[68736];
      a = a - ws[69920];
      a = a - ws[71040];
      yout[3040] = a;
    }
    {
      double a = 0.424 * ws[64768];
      a = fma(0.4, ws[64800], a);
      a = a - ws[66336];
      a = a - ws[67648];
      a = a - ws[68864];
      a = a - ws[70048];
      a = a - ws[71168];
      yout[3072] = a;
    }
    {
      double a = 0.83 * ws[62112];
      a = a - ws[65440];
      a = a - ws[66784];
      a = a - ws[68000];
      a = a - ws[69184];
      a = a - ws[70432];
      yout[3104] = a;
    }
    {
      double a = 0.667 * ws[72000];
      a = a - ws[72032];
      a = a - ws[72064];
      a = a - ws[72096];
      a = a - ws[72128];
      a = a - ws[72160];
      yout[3136] = a;
    }
    {
      double a = 0.072 * ws[72032];
      a = fma(0.075, ws[72064], a);
      a = fma(0.037, ws[72128], a);
      a = fma(0.06, ws[72160], a);
      a = a - ws[72256];
      a = a - ws[72384];
      a = a - ws[72416];
      yout[3168] = a;
    }
    {
      double a = 1.0 * ws[61952];
      a = a - ws[65312];
      a = a - ws[66656];
      a = a - ws[67872];
      a = a - ws[69056];
      a = a - ws[70304];
      yout[3200] = a;
    }
    {
      double a = 1.0 * ws[60256];
      a = fma(0.059, ws[63232], a);
      a = fma(0.056, ws[63264], a);
      a = fma(0.339, ws[64768], a);
      a = fma(0.32, ws[64800], a);
      a = a - ws[66432];
      a = a - ws[67488];
      yout[3232] = a;
    }
    {
      double a = 0.82 * ws[62144];
      a = a - ws[65472];
      a = a - ws[66816];
      a = a - ws[68032];
      a = a - ws[69216];
      a = a - ws[70464];
      yout[3264] = a;
    }
    {
      double a = 0.82 * ws[62080];
      a = a - ws[65408];
      a = a - ws[66752];
      a = a - ws[67968];
      a = a - ws[69152];
      a = a - ws[70400];
      yout[3296] = a;
    }
    {
      double a = 1.0 * ws[61984];
      a = a - ws[65344];
      a = a - ws[66688];
      a = a - ws[67904];
      a = a - ws[69088];
      a = a - ws[70336];
      yout[3328] = a;
    }
    {
      double a = 0.47 * ws[62048];
      a = a - ws[65376];
      a = a - ws[66720];
      a = a - ws[67936];
      a = a - ws[69120];
      a = a - ws[70368];
      yout[3360] = a;
    }
    {
      double a = 0.84 * ws[74944];
      a = a - ws[74976];
      a = a - ws[75008];
      a = a - ws[75040];
      a = a - ws[75072];
      a = a - ws[75104];
      yout[3392] = a;
    }
    {
      double a = 0.84 * ws[75136];
      a = a - ws[75168];
      a = a - ws[75200];
      a = a - ws[75232];
      a = a - ws[75264];
      a = a - ws[75296];
      yout[3424] = a;
    }
    {
      double a = 0.84 * ws[75328];
      a = a - ws[75360];
      a = a - ws[75392];
      a = a - ws[75424];
      a = a - ws[75456];
      a = a - ws[75488];
      yout[3456] = a;
    }
    {
      double a = 1.0 * ws[76128];
      a = a - ws[76160];
      a = a - ws[76192];
      a = a - ws[76224];
      a = a - ws[76256];
      a = a - ws[76288];
      yout[3488] = a;
    }
    {
      double a = 0.43 * ws[62944];
      a = a - ws[66016];
      a = a - ws[67360];
      a = a - ws[68544];
      a = a - ws[69728];
      a = a - ws[70848];
      a = fma(0.43, ws[71872], a);
      yout[3520] = a;
    }
    {
      double a = -ws[71872];
      a = a - ws[71904];
      a = a - ws[71936];
      a = a - ws[71968];
      a = fma(0.895, ws[72032], a);
      a = fma(0.925, ws[72064], a);
      a = fma(0.463, ws[72128], a);
      a = fma(0.74, ws[72160], a);
      a = fma(0.62, ws[72192], a);
      a = fma(0.9, ws[72224], a);
      yout[3552] = a;
    }
    {
      double a = -ws[63168];
      a = a - ws[64288];
      a = fma(0.2495, ws[65376], a);
      a = fma(0.25, ws[67936], a);
      a = fma(0.25, ws[69120], a);
      a = fma(0.25, ws[70368], a);
      a = fma(0.2, ws[72416], a);
      yout[3584] = a;
    }
    {
      double a = 2.81e-05 * ws[61856];
      a = fma(0.00134, ws[61888], a);
      a = fma(0.152, ws[63232], a);
      a = fma(0.2, ws[63264], a);
      a = fma(0.152, ws[64768], a);
      a = fma(0.2, ws[64800], a);
      a = fma(0.149, ws[71808], a);
      a = fma(0.00101, ws[71840], a);
      a = fma(0.04, ws[72352], a);
      yout[3616] = a;
    }
    {
      double a = 0.17 * ws[63232];
      a = fma(0.16, ws[63264], a);
      a = fma(0.85, ws[64768], a);
      a = fma(0.08, ws[64800], a);
      a = a - ws[66176];
      a = a - ws[67456];
      a = a - ws[68704];
      a = a - ws[69888];
      a = a - ws[71008];
      yout[3648] = a;
    }
    {
      double a = -ws[60416];
      a = a - ws[63680];
      a = fma(0.11, ws[64288], a);
      a = fma(0.36, ws[65792], a);
      a = fma(0.1, ws[67136], a);
      a = fma(0.41, ws[67168], a);
      a = fma(0.41, ws[67200], a);
      yout[3680] = a;
    }
    {
      double a = 0.055 * ws[64480];
      a = a - ws[65728];
      a = a - ws[67072];
      a = a - ws[68320];
      a = a - ws[69504];
      a = a - ws[71680];
      a = a - ws[71712];
      a = a - ws[71744];
      yout[3712] = a;
    }
    {
      double a = 0.025 * ws[62592];
      a = a - ws[65536];
      a = a - ws[66880];
      a = a - ws[68128];
      a = a - ws[69312];
      a = a - ws[71392];
      a = a - ws[71424];
      a = a - ws[71456];
      yout[3744] = a;
    }
    {
      double a = 1.0 * ws[62880];
      a = a - ws[65952];
      a = a - ws[67296];
      a = a - ws[68480];
      a = a - ws[69664];
      a = a - ws[70784];
      a = fma(0.0794, ws[75552], a);
      a = fma(0.1068, ws[75712], a);
      yout[3776] = a;
    }
    {
      double a = 1.0 * ws[63296];
      a = a - ws[64320];
      a = fma(1.0, ws[64832], a);
      a = fma(1.0, ws[66208], a);
      a = a - ws[66464];
      a = fma(1.0, ws[68736], a);
      a = fma(1.0, ws[69920], a);
      a = fma(1.0, ws[71040], a);
      yout[3808] = a;
    }
    {
      double a = 0.025 * ws[64448];
      a = a - ws[65600];
      a = a - ws[66944];
      a = a - ws[68192];
      a = a - ws[69376];
      a = a - ws[71584];
      a = a - ws[71616];
      a = a - ws[71648];
      yout[3840] = a;
    }
    {
      double a = -ws[59808];
      a = fma(0.7, ws[60032], a);
      a = fma(0.33, ws[60544], a);
      a = a - ws[63008];
      a = a - ws[64192];
      a = a - ws[64672];
      a = fma(0.333, ws[72000], a);
      a = fma(0.019, ws[72128], a);
      a = fma(0.015, ws[72160], a);
      yout[3872] = a;
    }
    {
      double a = 1.0 * ws[59840];
      a = fma(1.0, ws[59872], a);
      a = fma(0.44, ws[63520], a);
      a = fma(0.44, ws[63552], a);
      a = fma(1.0, ws[73344], a);
      a = a - ws[73568];
      a = a - ws[73792];
      a = a - ws[74016];
      yout[3904] = a;
    }
    {
      double a = 0.055 * ws[62624];
      a = a - ws[65664];
      a = a - ws[67008];
      a = a - ws[68256];
      a = a - ws[69440];
      a = a - ws[71488];
      a = a - ws[71520];
      a = a - ws[71552];
      yout[3936] = a;
    }
    {
      double a = 0.0369 * ws[75584];
      a = fma(0.0748, ws[75680], a);
      a = fma(0.0421, ws[75744], a);
      a = fma(0.0911, ws[75808], a);
      a = fma(0.0595, ws[75840], a);
      a = fma(0.0661, ws[75872], a);
      a = fma(0.0745, ws[75904], a);
      a = fma(0.1398, ws[75936], a);
      a = a - ws[75968];
      a = fma(0.0957, ws[75968], a);
      yout[3968] = a;
    }
    {
      double a = -ws[59392];
      a = fma(1.0, ws[60960], a);
      a = fma(1.0, ws[60992], a);
      a = a - ws[61024];
      a = fma(0.09, ws[62176], a);
      a = fma(0.068, ws[63936], a);
      a = fma(0.026, ws[63968], a);
      a = fma(0.255, ws[64000], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.02, ws[64064], a);
      yout[4000] = a;
    }
    {
      double a = 0.8 * ws[64352];
      a = fma(0.43, ws[64384], a);
      a = fma(0.11, ws[64416], a);
      a = a - ws[66272];
      a = a - ws[67584];
      a = a - ws[68800];
      a = a - ws[69984];
      a = a - ws[71104];
      a = a - ws[71200];
      a = a - ws[71200];
      a = a - ws[71232];
      a = fma(0.9, ws[72224], a);
      yout[4032] = a;
    }
    {
      double a = 0.2 * ws[64352];
      a = fma(0.57, ws[64384], a);
      a = fma(0.89, ws[64416], a);
      a = a - ws[66304];
      a = a - ws[67616];
      a = a - ws[68832];
      a = a - ws[70016];
      a = a - ws[71136];
      a = a - ws[71232];
      a = a - ws[71264];
      a = a - ws[71264];
      a = fma(0.1, ws[72224], a);
      yout[4064] = a;
    }
    {
      double a = -ws[60352];
      a = a - ws[63520];
      a = fma(0.0715, ws[65504], a);
      a = fma(0.762, ws[66848], a);
      a = fma(0.9, ws[66976], a);
      a = fma(0.75, ws[67104], a);
      a = fma(0.9, ws[67136], a);
      a = fma(0.0845, ws[68096], a);
      a = fma(0.091, ws[69280], a);
      a = fma(0.091, ws[70528], a);
      yout[4096] = a;
    }
    {
      double a = -ws[60000];
      a = fma(0.3, ws[62176], a);
      a = fma(0.028, ws[62208], a);
      a = fma(0.03, ws[62240], a);
      a = fma(0.18, ws[62304], a);
      a = fma(0.03, ws[62368], a);
      a = fma(0.57, ws[62560], a);
      a = a - ws[62944];
      a = a - ws[64128];
      a = a - ws[64640];
      a = fma(0.159, ws[68064], a);
      a = fma(0.219, ws[69248], a);
      a = fma(0.318, ws[70496], a);
      yout[4128] = a;
    }
    {
      double a = 0.975 * ws[62592];
      a = a - ws[65504];
      a = a - ws[66848];
      a = a - ws[68096];
      a = a - ws[69280];
      a = a - ws[70528];
      a = a - ws[71392];
      a = a - ws[71488];
      a = a - ws[71584];
      a = a - ws[71680];
      yout[4160] = a;
    }
    {
      double a = 0.945 * ws[62624];
      a = a - ws[65632];
      a = a - ws[66976];
      a = a - ws[68224];
      a = a - ws[69408];
      a = a - ws[70560];
      a = a - ws[71424];
      a = a - ws[71520];
      a = a - ws[71616];
      a = a - ws[71712];
      yout[4192] = a;
    }
    {
      double a = 0.0325 * ws[75584];
      a = fma(0.0138, ws[75648], a);
      a = fma(0.0347, ws[75680], a);
      a = fma(0.0371, ws[75744], a);
      a = fma(0.0174, ws[75776], a);
      a = fma(0.0423, ws[75808], a);
      a = fma(0.0523, ws[75840], a);
      a = fma(0.0582, ws[75872], a);
      a = fma(0.0479, ws[75904], a);
      a = a - ws[75936];
      a = fma(0.0062, ws[75936], a);
      a = fma(0.0432, ws[75968], a);
      yout[4224] = a;
    }
    {
      double a = 1.0 * ws[64896];
      a = fma(1.0, ws[64928], a);
      a = fma(1.0, ws[65536], a);
      a = fma(1.0, ws[65600], a);
      a = fma(1.0, ws[65664], a);
      a = fma(1.0, ws[65728], a);
      a = fma(0.64, ws[65760], a);
      a = fma(1.0, ws[66880], a);
      a = fma(1.0, ws[66944], a);
      a = fma(1.0, ws[67008], a);
      a = fma(1.0, ws[67072], a);
      a = fma(0.25, ws[67104], a);
      a = fma(1.0, ws[68128], a);
      a = fma(1.0, ws[68192], a);
      a = fma(1.0, ws[68256], a);
      a = fma(1.0, ws[68320], a);
      a = fma(1.0, ws[69312], a);
      a = fma(1.0, ws[69376], a);
      a = fma(1.0, ws[69440], a);
      a = fma(1.0, ws[69504], a);
      a = fma(0.96, ws[71392], a);
      a = fma(0.96, ws[71424], a);
      a = fma(0.96, ws[71456], a);
      a = fma(0.96, ws[71488], a);
      a = fma(0.96, ws[71520], a);
      a = fma(0.96, ws[71552], a);
      a = fma(0.96, ws[71584], a);
      a = fma(0.96, ws[71616], a);
      a = fma(0.96, ws[71648], a);
      a = fma(0.96, ws[71680], a);
      a = fma(0.96, ws[71712], a);
      a = fma(0.96, ws[71744], a);
      yout[4256] = a;
    }
    {
      double a = 1.0 * ws[62240];
      a = a - ws[62272];
      a = a - ws[62304];
      a = fma(1.0, ws[62336], a);
      a = a - ws[68064];
      a = a - ws[69248];
      a = a - ws[70496];
      a = a - ws[71456];
      a = a - ws[71552];
      a = a - ws[71648];
      a = a - ws[71744];
      yout[4288] = a;
    }
    {
      double a = -ws[60224];
      a = a - ws[63136];
      a = a - ws[64256];
      a = fma(0.2495, ws[65376], a);
      a = fma(0.5984, ws[65440], a);
      a = fma(0.4564, ws[65472], a);
      a = fma(0.25, ws[67936], a);
      a = fma(0.5996, ws[68000], a);
      a = fma(0.4573, ws[68032], a);
      a = fma(0.25, ws[69120], a);
      a = fma(0.5996, ws[69184], a);
      a = fma(0.4573, ws[69216], a);
      a = fma(0.25, ws[70368], a);
      a = fma(0.5996, ws[70432], a);
      a = fma(0.4573, ws[70464], a);
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[4320] = a;
    }
    {
      double a = 0.35 * ws[62016];
      a = fma(0.28, ws[62176], a);
      a = a - ws[63616];
      a = fma(0.37, ws[63904], a);
      a = fma(0.03, ws[63936], a);
      a = fma(0.028, ws[64000], a);
      a = fma(0.15, ws[64064], a);
      a = fma(0.45, ws[64128], a);
      a = fma(0.07, ws[64160], a);
      a = fma(0.044, ws[64192], a);
      a = fma(0.25, ws[64288], a);
      yout[4352] = a;
    }
    {
      double a = -ws[60544];
      a = a - ws[63840];
      a = a - ws[64096];
      a = a - ws[64512];
      a = fma(0.237, ws[65504], a);
      a = fma(0.2345, ws[65568], a);
      a = fma(0.23, ws[65632], a);
      a = fma(0.57, ws[65696], a);
      a = fma(0.36, ws[65760], a);
      a = fma(0.64, ws[65792], a);
      a = fma(0.461, ws[66912], a);
      a = fma(0.77, ws[67040], a);
      a = fma(0.341, ws[68160], a);
      a = fma(0.69, ws[68288], a);
      a = fma(0.175, ws[69344], a);
      a = fma(0.54, ws[69472], a);
      a = fma(0.175, ws[70592], a);
      a = fma(0.54, ws[70624], a);
      yout[4384] = a;
    }
    {
      double a = 0.28 * ws[73536];
      a = fma(1.0, ws[73952], a);
      a = fma(1.0, ws[74176], a);
      a = fma(0.14, ws[74368], a);
      a = fma(0.86, ws[74400], a);
      a = fma(1.0, ws[74624], a);
      a = fma(1.0, ws[74784], a);
      a = fma(0.0096, ws[75584], a);
      a = a - ws[75680];
      a = fma(0.007, ws[75680], a);
      a = fma(0.0046, ws[75744], a);
      a = fma(0.0758, ws[75808], a);
      a = fma(0.0013, ws[75840], a);
      yout[4416] = a;
    }
    {
      double a = -ws[60256];
      a = a - ws[63200];
      a = fma(0.02, ws[63936], a);
      a = fma(0.0, ws[65376], a);
      a = fma(0.0852, ws[65408], a);
      a = fma(0.0481, ws[65440], a);
      a = fma(0.0852, ws[65472], a);
      a = fma(0.0, ws[67936], a);
      a = fma(0.0854, ws[67968], a);
      a = fma(0.0482, ws[68000], a);
      a = fma(0.0854, ws[68032], a);
      a = fma(0.0, ws[69120], a);
      a = fma(0.0854, ws[69152], a);
      a = fma(0.0482, ws[69184], a);
      a = fma(0.0854, ws[69216], a);
      a = fma(0.0, ws[70368], a);
      a = fma(0.0854, ws[70400], a);
      a = fma(0.0482, ws[70432], a);
      a = fma(0.0854, ws[70464], a);
      a = fma(0.0594, ws[75008], a);
      a = fma(0.0595, ws[75040], a);
      a = fma(0.0595, ws[75072], a);
      a = fma(0.0595, ws[75104], a);
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      a = fma(1.0, ws[76256], a);
      a = fma(1.0, ws[76288], a);
      yout[4448] = a;
    }
    {
      double a = -ws[59744];
      a = a - ws[59776];
      a = a - ws[62816];
      a = fma(0.03, ws[63936], a);
      a = fma(0.11, ws[63968], a);
      a = fma(0.165, ws[65216], a);
      a = fma(0.217, ws[65248], a);
      a = fma(0.06, ws[65312], a);
      a = fma(0.2, ws[65344], a);
      a = fma(0.0865, ws[65504], a);
      a = fma(0.039, ws[66848], a);
      a = fma(0.067, ws[68096], a);
      a = fma(0.1165, ws[69280], a);
      a = fma(0.095, ws[70208], a);
      a = fma(0.247, ws[70240], a);
      a = fma(0.09, ws[70304], a);
      a = fma(0.2, ws[70336], a);
      a = fma(0.1165, ws[70528], a);
      yout[4480] = a;
    }
    {
      double a = 0.499 * ws[65376];
      a = fma(0.3651, ws[65408], a);
      a = fma(0.3515, ws[65440], a);
      a = fma(0.4564, ws[65472], a);
      a = fma(0.5, ws[67936], a);
      a = fma(0.3659, ws[67968], a);
      a = fma(0.3522, ws[68000], a);
      a = fma(0.4573, ws[68032], a);
      a = fma(0.5, ws[69120], a);
      a = fma(0.3659, ws[69152], a);
      a = fma(0.3522, ws[69184], a);
      a = fma(0.4573, ws[69216], a);
      a = fma(0.5, ws[70368], a);
      a = fma(0.3659, ws[70400], a);
      a = fma(0.3522, ws[70432], a);
      a = fma(0.4573, ws[70464], a);
      a = fma(0.92, ws[72288], a);
      a = fma(0.4, ws[72320], a);
      a = a - ws[72352];
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[4512] = a;
    }
    {
      double a = -ws[59840];
      a = a - ws[62656];
      a = fma(0.27, ws[63840], a);
      a = fma(0.2535, ws[64000], a);
      a = fma(0.27, ws[64096], a);
      a = fma(0.27, ws[64512], a);
      a = fma(0.195, ws[65504], a);
      a = fma(0.6045, ws[65568], a);
      a = fma(0.1885, ws[66848], a);
      a = fma(0.455, ws[66912], a);
      a = fma(0.273, ws[68096], a);
      a = fma(0.533, ws[68160], a);
      a = fma(0.2535, ws[69280], a);
      a = fma(0.65, ws[69344], a);
      a = fma(0.2535, ws[70528], a);
      a = fma(0.65, ws[70592], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71680], a);
      yout[4544] = a;
    }
    {
      double a = -ws[59872];
      a = a - ws[62688];
      a = fma(0.66, ws[64032], a);
      a = a - ws[64064];
      a = fma(0.1285, ws[65504], a);
      a = fma(0.77, ws[65632], a);
      a = fma(0.43, ws[65696], a);
      a = fma(0.039, ws[66848], a);
      a = fma(0.1, ws[66976], a);
      a = fma(0.23, ws[67040], a);
      a = fma(0.2205, ws[68096], a);
      a = fma(1.0, ws[68224], a);
      a = fma(0.31, ws[68288], a);
      a = fma(0.1725, ws[69280], a);
      a = fma(1.0, ws[69408], a);
      a = fma(0.46, ws[69472], a);
      a = fma(0.1725, ws[70528], a);
      a = fma(1.0, ws[70560], a);
      a = fma(0.46, ws[70624], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71712], a);
      yout[4576] = a;
    }
    {
      double a = -ws[60384];
      a = a - ws[63552];
      a = fma(0.6747, ws[66784], a);
      a = fma(0.6341, ws[66816], a);
      a = fma(0.0308, ws[75552], a);
      a = fma(0.0026, ws[75584], a);
      a = fma(0.0163, ws[75680], a);
      a = fma(0.0105, ws[75744], a);
      a = fma(0.0154, ws[75776], a);
      a = fma(0.0066, ws[75808], a);
      a = fma(0.0041, ws[75840], a);
      a = fma(0.0506, ws[75872], a);
      a = fma(0.0607, ws[75904], a);
      a = fma(0.0216, ws[75936], a);
      a = fma(0.0316, ws[75968], a);
      a = a - ws[76000];
      yout[4608] = a;
    }
    {
      double a = 0.0001 * ws[75008];
      a = fma(0.0152, ws[75552], a);
      a = fma(0.0298, ws[75584], a);
      a = a - ws[75648];
      a = fma(0.0076, ws[75648], a);
      a = fma(0.0305, ws[75680], a);
      a = fma(0.0183, ws[75712], a);
      a = fma(0.0657, ws[75744], a);
      a = fma(0.0452, ws[75776], a);
      a = fma(0.1193, ws[75808], a);
      a = fma(0.1118, ws[75840], a);
      a = fma(0.0489, ws[75872], a);
      a = fma(0.0246, ws[75904], a);
      a = fma(0.0146, ws[75936], a);
      a = fma(0.0049, ws[75968], a);
      yout[4640] = a;
    }
    {
      double a = 0.33 * ws[60000];
      a = fma(0.3, ws[60032], a);
      a = fma(0.1, ws[62176], a);
      a = fma(0.57, ws[62944], a);
      a = fma(0.21, ws[63168], a);
      a = fma(1.0, ws[63584], a);
      a = fma(0.32, ws[64640], a);
      a = fma(1.0, ws[64864], a);
      a = a - ws[65088];
      a = fma(1.0, ws[65120], a);
      a = a - ws[65984];
      a = a - ws[67328];
      a = a - ws[68512];
      a = a - ws[69696];
      a = a - ws[70816];
      a = fma(0.57, ws[71872], a);
      a = fma(0.32, ws[71936], a);
      yout[4672] = a;
    }
    {
      double a = 0.28 * ws[73472];
      a = fma(1.0, ws[73888], a);
      a = fma(1.0, ws[74112], a);
      a = fma(0.86, ws[74336], a);
      a = fma(1.0, ws[74560], a);
      a = fma(0.0199, ws[75584], a);
      a = fma(0.0075, ws[75648], a);
      a = fma(0.0352, ws[75680], a);
      a = fma(0.0215, ws[75744], a);
      a = a - ws[75808];
      a = fma(0.0118, ws[75808], a);
      a = fma(0.0068, ws[75840], a);
      a = fma(0.0013, ws[75872], a);
      a = fma(0.0073, ws[75904], a);
      a = fma(0.0031, ws[75936], a);
      a = fma(0.0022, ws[75968], a);
      yout[4704] = a;
    }
    {
      double a = -ws[60032];
      a = fma(0.14, ws[62176], a);
      a = fma(0.26, ws[62208], a);
      a = fma(0.51, ws[62304], a);
      a = fma(0.13, ws[62368], a);
      a = fma(0.15, ws[62432], a);
      a = fma(0.43, ws[62560], a);
      a = a - ws[62976];
      a = a - ws[64160];
      a = fma(0.25, ws[68064], a);
      a = fma(0.305, ws[69248], a);
      a = fma(0.5, ws[70496], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.231, ws[72128], a);
      a = fma(0.185, ws[72160], a);
      yout[4736] = a;
    }
    {
      double a = 0.0357 * ws[75360];
      a = fma(0.0001, ws[75392], a);
      a = a - ws[75520];
      a = fma(0.0854, ws[75520], a);
      a = fma(0.464, ws[75552], a);
      a = fma(0.1041, ws[75584], a);
      a = fma(0.2036, ws[75616], a);
      a = fma(0.2792, ws[75648], a);
      a = fma(0.0074, ws[75680], a);
      a = fma(0.2822, ws[75712], a);
      a = fma(0.0659, ws[75744], a);
      a = fma(0.1778, ws[75776], a);
      a = fma(0.0023, ws[75808], a);
      a = fma(0.0445, ws[75840], a);
      a = fma(0.0317, ws[75872], a);
      a = fma(0.0117, ws[75904], a);
      a = fma(0.1188, ws[76000], a);
      yout[4768] = a;
    }
    {
      double a = 0.77 * ws[62656];
      a = fma(0.17, ws[62688], a);
      a = fma(1.0, ws[62784], a);
      a = fma(0.2805, ws[64000], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.6, ws[64224], a);
      a = fma(0.6, ws[64256], a);
      a = fma(1.0, ws[64608], a);
      a = a - ws[65024];
      a = fma(1.0, ws[65056], a);
      a = a - ws[65856];
      a = a - ws[67200];
      a = a - ws[68384];
      a = a - ws[69568];
      a = a - ws[70112];
      a = a - ws[70112];
      a = a - ws[70688];
      a = a - ws[71328];
      yout[4800] = a;
    }
    {
      double a = 0.018 * ws[72608];
      a = fma(1.0, ws[73984], a);
      a = fma(1.0, ws[74208], a);
      a = fma(0.14, ws[74400], a);
      a = fma(1.0, ws[74432], a);
      a = fma(1.0, ws[74656], a);
      a = fma(1.0, ws[74816], a);
      a = fma(1.0, ws[74848], a);
      a = fma(1.0, ws[74880], a);
      a = a - ws[75584];
      a = fma(0.2141, ws[75584], a);
      a = fma(0.0088, ws[75648], a);
      a = fma(0.7261, ws[75680], a);
      a = fma(0.1156, ws[75744], a);
      a = fma(0.0004, ws[75776], a);
      a = fma(0.3349, ws[75808], a);
      a = fma(0.0104, ws[75840], a);
      a = fma(0.0009, ws[75872], a);
      a = fma(0.0006, ws[75936], a);
      yout[4832] = a;
    }
    {
      double a = 0.0357 * ws[74976];
      a = fma(0.0357, ws[75168], a);
      a = fma(0.0001, ws[75200], a);
      a = a - ws[75552];
      a = fma(0.1977, ws[75552], a);
      a = fma(0.5638, ws[75584], a);
      a = fma(0.0071, ws[75616], a);
      a = fma(0.4025, ws[75648], a);
      a = fma(0.119, ws[75680], a);
      a = fma(0.1165, ws[75712], a);
      a = fma(0.4579, ws[75744], a);
      a = fma(0.1924, ws[75776], a);
      a = fma(0.134, ws[75808], a);
      a = fma(0.1726, ws[75840], a);
      a = fma(0.0765, ws[75872], a);
      a = fma(0.0167, ws[75904], a);
      a = fma(0.0103, ws[75936], a);
      a = fma(0.0008, ws[76000], a);
      yout[4864] = a;
    }
    {
      double a = 0.0008 * ws[65376];
      a = fma(0.0006, ws[65408], a);
      a = fma(0.3979, ws[66720], a);
      a = fma(0.2805, ws[66752], a);
      a = fma(0.0121, ws[75552], a);
      a = fma(0.0153, ws[75584], a);
      a = a - ws[75616];
      a = fma(0.0319, ws[75648], a);
      a = fma(0.0122, ws[75680], a);
      a = fma(0.032, ws[75712], a);
      a = fma(0.0325, ws[75744], a);
      a = fma(0.074, ws[75776], a);
      a = fma(0.008, ws[75808], a);
      a = fma(0.0513, ws[75840], a);
      a = fma(0.0526, ws[75872], a);
      a = fma(0.048, ws[75904], a);
      a = fma(0.009, ws[75936], a);
      a = fma(0.0061, ws[75968], a);
      a = fma(0.039, ws[76000], a);
      yout[4896] = a;
    }
    {
      double a = 0.0006 * ws[65440];
      a = fma(0.0006, ws[65472], a);
      a = fma(0.2771, ws[66784], a);
      a = fma(0.2805, ws[66816], a);
      a = fma(1.0, ws[72512], a);
      a = fma(0.0624, ws[75552], a);
      a = fma(0.0189, ws[75584], a);
      a = fma(0.0194, ws[75648], a);
      a = fma(0.0291, ws[75680], a);
      a = a - ws[75712];
      a = fma(0.0011, ws[75712], a);
      a = fma(0.0307, ws[75744], a);
      a = fma(0.0631, ws[75776], a);
      a = fma(0.0292, ws[75808], a);
      a = fma(0.1337, ws[75840], a);
      a = fma(0.155, ws[75872], a);
      a = fma(0.0881, ws[75904], a);
      a = fma(0.0702, ws[75936], a);
      a = fma(0.0224, ws[75968], a);
      a = fma(0.0114, ws[76000], a);
      yout[4928] = a;
    }
    {
      double a = 1.0 * ws[72672];
      a = fma(0.28, ws[73504], a);
      a = fma(1.0, ws[73920], a);
      a = fma(1.0, ws[74144], a);
      a = fma(0.14, ws[74336], a);
      a = fma(0.86, ws[74368], a);
      a = fma(1.0, ws[74592], a);
      a = fma(1.0, ws[74752], a);
      a = fma(0.9048, ws[75168], a);
      a = fma(0.0456, ws[75584], a);
      a = fma(0.0104, ws[75648], a);
      a = fma(0.0454, ws[75680], a);
      a = a - ws[75744];
      a = fma(0.0024, ws[75744], a);
      a = fma(0.0007, ws[75776], a);
      a = fma(0.0766, ws[75808], a);
      a = fma(0.0403, ws[75840], a);
      a = fma(0.0155, ws[75872], a);
      a = fma(0.0153, ws[75936], a);
      yout[4960] = a;
    }
    {
      double a = 0.247 * ws[72736];
      a = fma(0.14, ws[74304], a);
      a = fma(1.0, ws[74720], a);
      a = fma(0.9048, ws[74976], a);
      a = fma(0.0018, ws[75200], a);
      a = fma(0.9048, ws[75360], a);
      a = fma(0.0388, ws[75552], a);
      a = fma(0.0314, ws[75584], a);
      a = fma(0.051, ws[75648], a);
      a = fma(0.0234, ws[75680], a);
      a = fma(0.0395, ws[75744], a);
      a = a - ws[75776];
      a = fma(0.0006, ws[75776], a);
      a = fma(0.0277, ws[75808], a);
      a = fma(0.0511, ws[75840], a);
      a = fma(0.1051, ws[75872], a);
      a = fma(0.0916, ws[75904], a);
      a = fma(0.1038, ws[75936], a);
      a = fma(0.0503, ws[75968], a);
      yout[4992] = a;
    }
    {
      double a = -ws[59552];
      a = fma(1.0, ws[61152], a);
      a = fma(1.0, ws[61312], a);
      a = a - ws[61344];
      a = fma(0.3, ws[61408], a);
      a = fma(2.0, ws[61600], a);
      a = fma(1.0, ws[62528], a);
      a = fma(1.0, ws[64544], a);
      a = fma(1.0, ws[64576], a);
      a = fma(1.0, ws[64608], a);
      a = fma(0.32, ws[64640], a);
      a = fma(1.0, ws[64704], a);
      a = fma(1.0, ws[64736], a);
      a = fma(0.424, ws[64768], a);
      a = fma(0.4, ws[64800], a);
      a = fma(1.0, ws[64832], a);
      a = fma(0.32, ws[71936], a);
      a = fma(2.0, ws[72832], a);
      a = fma(0.5, ws[72864], a);
      a = fma(1.0, ws[72928], a);
      a = fma(1.0, ws[73120], a);
      a = fma(1.0, ws[76064], a);
      a = fma(1.0, ws[76096], a);
      yout[5024] = a;
    }
    {
      double a = 1.0 * ws[62528];
      a = a - ws[63392];
      a = fma(0.25, ws[67776], a);
      a = fma(0.25, ws[67808], a);
      a = fma(0.25, ws[67872], a);
      a = fma(0.25, ws[67904], a);
      a = fma(0.25, ws[68064], a);
      a = fma(0.25, ws[68416], a);
      a = fma(0.25, ws[68448], a);
      a = fma(0.25, ws[68480], a);
      a = fma(0.25, ws[68512], a);
      a = fma(0.25, ws[68544], a);
      a = fma(0.25, ws[68576], a);
      a = fma(0.25, ws[68608], a);
      a = fma(0.25, ws[68832], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71680], a);
      a = fma(0.48, ws[71712], a);
      a = fma(0.48, ws[71744], a);
      yout[5056] = a;
    }
    {
      double a = 0.28 * ws[73440];
      a = fma(1.0, ws[73856], a);
      a = fma(1.0, ws[74080], a);
      a = fma(0.14, ws[74272], a);
      a = fma(0.86, ws[74304], a);
      a = fma(1.0, ws[74528], a);
      a = fma(1.0, ws[74912], a);
      a = fma(0.0018, ws[75008], a);
      a = fma(0.0018, ws[75392], a);
      a = fma(0.0491, ws[75552], a);
      a = fma(0.0459, ws[75584], a);
      a = fma(0.0512, ws[75648], a);
      a = fma(0.0624, ws[75680], a);
      a = fma(0.066, ws[75712], a);
      a = fma(0.0539, ws[75744], a);
      a = fma(0.0227, ws[75776], a);
      a = fma(0.0651, ws[75808], a);
      a = a - ws[75840];
      a = fma(0.0236, ws[75840], a);
      a = fma(0.0535, ws[75872], a);
      a = fma(0.0972, ws[75904], a);
      a = fma(0.165, ws[75936], a);
      a = fma(0.0879, ws[75968], a);
      yout[5088] = a;
    }
    {
      double a = 1.0 * ws[61888];
      a = fma(0.02, ws[63936], a);
      a = a - ws[65248];
      a = a - ws[66592];
      a = a - ws[67808];
      a = a - ws[68992];
      a = a - ws[70240];
      a = fma(0.0794, ws[75552], a);
      a = fma(0.0925, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.1753, ws[75648], a);
      a = fma(0.0537, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.1055, ws[75744], a);
      a = fma(0.222, ws[75776], a);
      a = fma(0.0654, ws[75808], a);
      a = fma(0.1489, ws[75840], a);
      a = fma(0.1656, ws[75872], a);
      a = fma(0.173, ws[75904], a);
      a = fma(0.128, ws[75936], a);
      a = fma(0.1544, ws[75968], a);
      yout[5120] = a;
    }
    {
      double a = 1.0 * ws[62848];
      a = a - ws[65920];
      a = a - ws[67264];
      a = a - ws[68448];
      a = a - ws[69632];
      a = a - ws[70752];
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5152] = a;
    }
    {
      double a = -ws[59328];
      a = a - ws[59360];
      a = a - ws[60608];
      a = a - ws[60640];
      a = a - ws[60672];
      a = a - ws[60704];
      a = fma(1.0, ws[60736], a);
      a = a - ws[60768];
      a = a - ws[62176];
      a = a - ws[63904];
      a = a - ws[63936];
      a = a - ws[63968];
      a = a - ws[64000];
      a = a - ws[64032];
      a = a - ws[64064];
      a = a - ws[64096];
      a = a - ws[64128];
      a = a - ws[64160];
      a = a - ws[64192];
      a = a - ws[64224];
      a = a - ws[64256];
      a = a - ws[64288];
      a = a - ws[64320];
      a = a - ws[71904];
      a = a - ws[72192];
      a = a - ws[72384];
      a = a - ws[72608];
      a = a - ws[72960];
      yout[5184] = a;
    }
    {
      double a = 0.34 * ws[60000];
      a = fma(0.2, ws[60192], a);
      a = fma(0.2, ws[60224], a);
      a = fma(0.07, ws[63488], a);
      a = fma(0.07, ws[63520], a);
      a = fma(0.07, ws[63552], a);
      a = fma(0.35, ws[63680], a);
      a = fma(1.0, ws[63712], a);
      a = fma(1.0, ws[63744], a);
      a = fma(0.01, ws[64160], a);
      a = fma(0.1, ws[64192], a);
      a = fma(0.6, ws[64224], a);
      a = fma(0.6, ws[64256], a);
      a = fma(0.68, ws[64640], a);
      a = fma(1.0, ws[64672], a);
      a = fma(0.089, ws[65216], a);
      a = fma(0.235, ws[65248], a);
      a = fma(0.16, ws[65952], a);
      a = fma(0.7, ws[66048], a);
      a = a - ws[66368];
      a = a - ws[67680];
      a = fma(0.026, ws[67776], a);
      a = fma(0.191, ws[67808], a);
      a = fma(1.16, ws[68576], a);
      a = a - ws[68896];
      a = fma(0.026, ws[68960], a);
      a = fma(0.191, ws[68992], a);
      a = fma(1.16, ws[69760], a);
      a = a - ws[70080];
      a = fma(0.092, ws[70208], a);
      a = fma(0.485, ws[70240], a);
      a = fma(0.7, ws[70880], a);
      a = a - ws[71296];
      a = a - ws[71328];
      a = a - ws[71360];
      a = a - ws[71360];
      a = fma(0.68, ws[71936], a);
      yout[5216] = a;
    }
    {
      double a = -ws[60160];
      a = fma(0.5, ws[60192], a);
      a = fma(0.5, ws[60224], a);
      a = fma(0.05, ws[62240], a);
      a = fma(0.04, ws[62368], a);
      a = fma(1.0, ws[62912], a);
      a = a - ws[63072];
      a = fma(0.01, ws[63104], a);
      a = fma(0.01, ws[63136], a);
      a = fma(0.01, ws[63168], a);
      a = fma(0.5, ws[64128], a);
      a = fma(0.54, ws[64160], a);
      a = fma(0.003, ws[64192], a);
      a = fma(0.08, ws[64224], a);
      a = fma(0.08, ws[64256], a);
      a = fma(0.68, ws[64640], a);
      a = a - ws[64736];
      a = fma(0.3651, ws[65408], a);
      a = fma(0.247, ws[65440], a);
      a = fma(0.3651, ws[65472], a);
      a = fma(0.54, ws[65952], a);
      a = fma(0.3, ws[66048], a);
      a = fma(0.21, ws[66080], a);
      a = fma(0.3659, ws[67968], a);
      a = fma(0.2475, ws[68000], a);
      a = fma(0.3659, ws[68032], a);
      a = fma(0.5, ws[68576], a);
      a = fma(0.105, ws[68608], a);
      a = fma(0.3659, ws[69152], a);
      a = fma(0.2475, ws[69184], a);
      a = fma(0.3659, ws[69216], a);
      a = fma(0.5, ws[69760], a);
      a = fma(0.105, ws[69792], a);
      a = fma(0.3659, ws[70400], a);
      a = fma(0.2475, ws[70432], a);
      a = fma(0.3659, ws[70464], a);
      a = fma(0.3, ws[70880], a);
      a = fma(0.21, ws[70912], a);
      a = fma(0.68, ws[71936], a);
      a = a - ws[72800];
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[5248] = a;
    }
    {
      double a = -ws[59904];
      a = a - ws[62848];
      a = fma(0.13, ws[63136], a);
      a = fma(0.06, ws[63936], a);
      a = fma(0.042, ws[65216], a);
      a = fma(0.033, ws[65248], a);
      a = fma(0.13, ws[65312], a);
      a = fma(0.075, ws[70208], a);
      a = fma(0.063, ws[70240], a);
      a = fma(0.18, ws[70304], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5280] = a;
    }
    {
      double a = 0.0012 * ws[65376];
      a = fma(0.0013, ws[65408], a);
      a = fma(0.28, ws[73376], a);
      a = fma(1.0, ws[74240], a);
      a = fma(0.16, ws[74944], a);
      a = fma(0.0595, ws[74976], a);
      a = fma(0.0001, ws[75008], a);
      a = fma(0.0594, ws[75200], a);
      a = fma(0.0595, ws[75232], a);
      a = fma(0.0595, ws[75264], a);
      a = fma(0.0595, ws[75296], a);
      a = fma(0.0595, ws[75392], a);
      a = fma(0.0595, ws[75424], a);
      a = fma(0.0595, ws[75456], a);
      a = fma(0.0595, ws[75488], a);
      a = fma(0.0183, ws[75552], a);
      a = fma(0.0455, ws[75584], a);
      a = fma(0.0512, ws[75648], a);
      a = fma(0.0509, ws[75680], a);
      a = fma(0.0246, ws[75712], a);
      a = fma(0.0519, ws[75744], a);
      a = fma(0.0649, ws[75776], a);
      a = fma(0.0668, ws[75808], a);
      a = fma(0.0733, ws[75840], a);
      a = fma(0.0426, ws[75872], a);
      a = a - ws[75904];
      a = fma(0.0024, ws[75904], a);
      a = fma(0.0724, ws[75936], a);
      a = fma(0.1463, ws[75968], a);
      yout[5312] = a;
    }
    {
      double a = -ws[59968];
      a = fma(1.0, ws[60576], a);
      a = a - ws[62912];
      a = fma(1.0, ws[63776], a);
      a = fma(1.0, ws[63872], a);
      a = fma(0.01, ws[63936], a);
      a = fma(0.044, ws[63968], a);
      a = fma(0.272, ws[65248], a);
      a = fma(0.02, ws[65344], a);
      a = fma(1.0, ws[66016], a);
      a = fma(0.32, ws[66176], a);
      a = fma(0.016, ws[68064], a);
      a = fma(0.5, ws[68544], a);
      a = fma(0.32, ws[68704], a);
      a = fma(0.5, ws[69728], a);
      a = fma(0.32, ws[69888], a);
      a = fma(0.275, ws[70240], a);
      a = fma(0.04, ws[70336], a);
      a = fma(0.033, ws[70496], a);
      a = fma(1.0, ws[70848], a);
      a = fma(0.32, ws[71008], a);
      a = fma(0.613, ws[72448], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      yout[5344] = a;
    }
    {
      double a = -ws[60064];
      a = a - ws[60096];
      a = a - ws[60128];
      a = fma(0.5, ws[60192], a);
      a = fma(0.5, ws[60224], a);
      a = fma(0.65, ws[62016], a);
      a = fma(0.02, ws[62368], a);
      a = a - ws[63040];
      a = fma(0.1, ws[63104], a);
      a = fma(0.1, ws[63136], a);
      a = fma(0.27, ws[63168], a);
      a = fma(0.491, ws[64192], a);
      a = fma(0.05, ws[64224], a);
      a = fma(0.05, ws[64256], a);
      a = fma(0.48, ws[64288], a);
      a = a - ws[64704];
      a = fma(0.998, ws[65376], a);
      a = fma(0.5477, ws[65408], a);
      a = fma(0.7029, ws[65440], a);
      a = fma(0.5477, ws[65472], a);
      a = fma(0.18, ws[66080], a);
      a = fma(0.68, ws[66176], a);
      a = fma(1.0, ws[66240], a);
      a = fma(1.0, ws[66336], a);
      a = fma(0.05, ws[67776], a);
      a = fma(1.0, ws[67936], a);
      a = fma(0.5488, ws[67968], a);
      a = fma(0.7043, ws[68000], a);
      a = fma(0.5488, ws[68032], a);
      a = fma(0.018, ws[68064], a);
      a = fma(0.135, ws[68608], a);
      a = fma(0.68, ws[68704], a);
      a = fma(1.0, ws[68768], a);
      a = fma(0.7, ws[68864], a);
      a = fma(0.067, ws[68960], a);
      a = fma(1.0, ws[69120], a);
      a = fma(0.5488, ws[69152], a);
      a = fma(0.7043, ws[69184], a);
      a = fma(0.5488, ws[69216], a);
      a = fma(0.18, ws[69792], a);
      a = fma(0.68, ws[69888], a);
      a = fma(1.0, ws[69952], a);
      a = fma(0.7, ws[70048], a);
      a = fma(1.0, ws[70368], a);
      a = fma(0.5488, ws[70400], a);
      a = fma(0.7043, ws[70432], a);
      a = fma(0.5488, ws[70464], a);
      a = fma(0.024, ws[70496], a);
      a = fma(0.18, ws[70912], a);
      a = fma(0.68, ws[71008], a);
      a = fma(1.0, ws[71072], a);
      a = fma(1.0, ws[71168], a);
      a = fma(0.62, ws[71904], a);
      a = fma(0.31, ws[72352], a);
      a = a - ws[72768];
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[5376] = a;
    }
    {
      double a = 1.0 * ws[61856];
      a = fma(0.44, ws[63488], a);
      a = fma(1.0, ws[63808], a);
      a = fma(0.04, ws[63936], a);
      a = fma(0.04, ws[63968], a);
      a = a - ws[65216];
      a = a - ws[66560];
      a = a - ws[67776];
      a = a - ws[68960];
      a = a - ws[70208];
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5408] = a;
    }
    {
      double a = -ws[60448];
      a = a - ws[63808];
      a = fma(1.0, ws[64672], a);
      a = fma(0.065, ws[65216], a);
      a = fma(0.136, ws[65248], a);
      a = fma(0.03, ws[65312], a);
      a = fma(0.05, ws[65344], a);
      a = fma(0.0, ws[65376], a);
      a = fma(0.0002, ws[65408], a);
      a = fma(0.0001, ws[65440], a);
      a = fma(0.0002, ws[65472], a);
      a = fma(0.07, ws[65568], a);
      a = fma(0.07, ws[65696], a);
      a = fma(1.0, ws[66272], a);
      a = fma(1.0, ws[66400], a);
      a = fma(1.0, ws[66432], a);
      a = fma(1.0, ws[66464], a);
      a = fma(1.0, ws[67584], a);
      a = fma(1.0, ws[67616], a);
      a = fma(1.0, ws[68800], a);
      a = fma(0.5, ws[68832], a);
      a = fma(0.3, ws[68864], a);
      a = fma(1.0, ws[69984], a);
      a = fma(0.3, ws[70048], a);
      a = fma(1.0, ws[71104], a);
      a = fma(2.0, ws[71200], a);
      a = fma(1.5, ws[71232], a);
      a = fma(1.0, ws[71264], a);
      a = fma(0.032, ws[72032], a);
      a = fma(0.08, ws[72288], a);
      a = fma(0.26, ws[73568], a);
      a = fma(0.12, ws[74464], a);
      yout[5440] = a;
    }
    {
      double a = -ws[60192];
      a = a - ws[63104];
      a = a - ws[64224];
      a = fma(0.7, ws[64256], a);
      a = fma(0.7, ws[64288], a);
      a = fma(0.5477, ws[65408], a);
      a = fma(0.67, ws[65920], a);
      a = fma(0.5488, ws[67968], a);
      a = fma(0.334, ws[68448], a);
      a = fma(0.5, ws[68480], a);
      a = fma(0.5488, ws[69152], a);
      a = fma(0.334, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.5488, ws[70400], a);
      a = fma(0.67, ws[70752], a);
      a = fma(1.0, ws[70784], a);
      a = fma(0.49, ws[72256], a);
      a = fma(0.8, ws[72416], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5472] = a;
    }
    {
      double a = 0.216 * ws[59808];
      a = a - ws[59936];
      a = fma(0.8, ws[60448], a);
      a = fma(0.67, ws[60544], a);
      a = a - ws[62880];
      a = fma(0.78, ws[63104], a);
      a = fma(0.41, ws[63488], a);
      a = fma(0.41, ws[63520], a);
      a = fma(0.41, ws[63552], a);
      a = fma(0.38, ws[63840], a);
      a = fma(0.017, ws[63968], a);
      a = fma(0.1785, ws[64000], a);
      a = fma(0.38, ws[64096], a);
      a = fma(0.028, ws[64192], a);
      a = fma(0.38, ws[64512], a);
      a = fma(0.033, ws[65248], a);
      a = fma(0.09, ws[65344], a);
      a = fma(0.084, ws[65504], a);
      a = fma(0.007, ws[65568], a);
      a = fma(0.7, ws[66080], a);
      a = fma(0.464, ws[66304], a);
      a = fma(0.0105, ws[66848], a);
      a = fma(0.007, ws[66912], a);
      a = fma(0.497, ws[67776], a);
      a = fma(0.618, ws[67808], a);
      a = fma(0.045, ws[67872], a);
      a = fma(0.218, ws[67904], a);
      a = fma(0.1835, ws[68096], a);
      a = fma(0.007, ws[68160], a);
      a = fma(0.525, ws[68608], a);
      a = fma(0.348, ws[68832], a);
      a = fma(0.662, ws[68960], a);
      a = fma(0.824, ws[68992], a);
      a = fma(0.06, ws[69056], a);
      a = fma(0.29, ws[69088], a);
      a = fma(0.112, ws[69280], a);
      a = fma(0.007, ws[69344], a);
      a = fma(0.7, ws[69792], a);
      a = fma(0.464, ws[70016], a);
      a = fma(0.06, ws[70240], a);
      a = fma(0.11, ws[70336], a);
      a = fma(0.112, ws[70528], a);
      a = fma(0.007, ws[70592], a);
      a = fma(0.7, ws[70912], a);
      a = fma(0.464, ws[71136], a);
      a = fma(0.149, ws[71232], a);
      a = fma(0.285, ws[71264], a);
      a = fma(0.65, ws[72352], a);
      a = fma(0.88, ws[74464], a);
      a = fma(1.0, ws[74688], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.1068, ws[75712], a);
      yout[5504] = a;
    }
    {
      double a = 0.0013 * ws[65440];
      a = fma(0.0013, ws[65472], a);
      a = fma(1.0, ws[72544], a);
      a = fma(1.0, ws[72576], a);
      a = fma(0.982, ws[72608], a);
      a = fma(1.0, ws[72704], a);
      a = fma(0.753, ws[72736], a);
      a = fma(0.28, ws[73408], a);
      a = fma(1.0, ws[73824], a);
      a = fma(1.0, ws[74048], a);
      a = fma(0.86, ws[74272], a);
      a = fma(1.0, ws[74496], a);
      a = fma(0.16, ws[75136], a);
      a = fma(0.0595, ws[75168], a);
      a = fma(0.0001, ws[75200], a);
      a = fma(0.16, ws[75328], a);
      a = fma(0.0595, ws[75360], a);
      a = fma(0.0398, ws[75552], a);
      a = fma(0.0452, ws[75584], a);
      a = fma(0.0462, ws[75648], a);
      a = fma(0.0518, ws[75680], a);
      a = fma(0.0535, ws[75712], a);
      a = fma(0.0516, ws[75744], a);
      a = fma(0.0585, ws[75776], a);
      a = fma(0.0709, ws[75808], a);
      a = fma(0.0293, ws[75840], a);
      a = a - ws[75872];
      a = fma(0.0086, ws[75872], a);
      a = fma(0.0456, ws[75904], a);
      a = fma(0.1566, ws[75936], a);
      a = fma(0.1384, ws[75968], a);
      a = fma(1.0, ws[76160], a);
      yout[5536] = a;
    }
    {
      double a = -ws[59680];
      a = a - ws[62752];
      a = fma(1.0, ws[63360], a);
      a = fma(0.184, ws[63392], a);
      a = fma(0.01, ws[63936], a);
      a = fma(0.457, ws[63968], a);
      a = fma(0.42, ws[64192], a);
      a = a - ws[64576];
      a = fma(1.0, ws[65184], a);
      a = fma(0.504, ws[65216], a);
      a = fma(0.045, ws[65248], a);
      a = fma(0.012, ws[65312], a);
      a = fma(0.81, ws[65344], a);
      a = fma(0.75, ws[67744], a);
      a = fma(1.0, ws[68928], a);
      a = fma(1.0, ws[70176], a);
      a = fma(0.519, ws[70208], a);
      a = fma(0.048, ws[70240], a);
      a = fma(0.02, ws[70304], a);
      a = fma(0.85, ws[70336], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5568] = a;
    }
    {
      double a = -ws[63328];
      a = fma(0.63, ws[67712], a);
      a = fma(0.25, ws[67744], a);
      a = fma(0.25, ws[67776], a);
      a = fma(0.25, ws[67808], a);
      a = fma(0.25, ws[67840], a);
      a = fma(0.25, ws[67872], a);
      a = fma(0.25, ws[67904], a);
      a = fma(0.32, ws[67936], a);
      a = fma(0.32, ws[67968], a);
      a = fma(0.32, ws[68000], a);
      a = fma(0.32, ws[68032], a);
      a = fma(0.25, ws[68064], a);
      a = fma(0.1105, ws[68096], a);
      a = fma(0.25, ws[68128], a);
      a = fma(0.043, ws[68160], a);
      a = fma(0.25, ws[68192], a);
      a = fma(0.25, ws[68224], a);
      a = fma(0.25, ws[68256], a);
      a = fma(0.09, ws[68288], a);
      a = fma(0.25, ws[68320], a);
      a = fma(0.25, ws[68416], a);
      a = fma(0.25, ws[68448], a);
      a = fma(0.25, ws[68480], a);
      a = fma(0.25, ws[68512], a);
      a = fma(0.25, ws[68544], a);
      a = fma(0.25, ws[68576], a);
      a = fma(0.25, ws[68608], a);
      a = fma(0.25, ws[68832], a);
      a = fma(0.32, ws[72128], a);
      a = fma(0.32, ws[75072], a);
      a = fma(0.32, ws[75264], a);
      a = fma(0.32, ws[75456], a);
      a = fma(0.32, ws[76256], a);
      yout[5600] = a;
    }
    {
      double a = 1.0 * ws[59712];
      a = fma(1.0, ws[59904], a);
      a = fma(1.5, ws[59936], a);
      a = fma(1.0, ws[61824], a);
      a = fma(0.06, ws[63936], a);
      a = fma(0.07, ws[63968], a);
      a = a - ws[65184];
      a = fma(0.048, ws[65216], a);
      a = fma(0.231, ws[65248], a);
      a = fma(1.0, ws[65856], a);
      a = a - ws[66528];
      a = fma(0.44, ws[67200], a);
      a = a - ws[67744];
      a = fma(0.026, ws[67776], a);
      a = fma(0.14, ws[67808], a);
      a = a - ws[68928];
      a = fma(0.026, ws[68960], a);
      a = fma(0.14, ws[68992], a);
      a = fma(1.0, ws[69568], a);
      a = fma(2.0, ws[70112], a);
      a = a - ws[70176];
      a = fma(0.503, ws[70208], a);
      a = fma(0.28, ws[70240], a);
      a = fma(1.0, ws[70688], a);
      a = fma(1.0, ws[71328], a);
      a = fma(0.852, ws[71808], a);
      a = fma(1.0, ws[71840], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5632] = a;
    }
    {
      double a = 1.0 * ws[59616];
      a = fma(1.0, ws[59648], a);
      a = fma(1.0, ws[59680], a);
      a = fma(1.0, ws[59712], a);
      a = fma(1.0, ws[59776], a);
      a = fma(1.22, ws[59808], a);
      a = fma(1.0, ws[59840], a);
      a = fma(1.0, ws[59872], a);
      a = fma(0.1, ws[59904], a);
      a = fma(0.5, ws[59936], a);
      a = fma(0.67, ws[60000], a);
      a = fma(0.7, ws[60032], a);
      a = fma(2.0, ws[60064], a);
      a = fma(1.0, ws[60096], a);
      a = fma(2.0, ws[60128], a);
      a = fma(1.0, ws[60160], a);
      a = fma(1.0, ws[60192], a);
      a = fma(1.0, ws[60224], a);
      a = fma(1.0, ws[60256], a);
      a = a - ws[61760];
      a = fma(0.35, ws[62016], a);
      a = fma(0.22, ws[62176], a);
      a = fma(1.0, ws[62368], a);
      a = fma(1.0, ws[62496], a);
      a = fma(1.0, ws[62720], a);
      a = fma(2.0, ws[63040], a);
      a = fma(1.0, ws[63072], a);
      a = fma(0.33, ws[63104], a);
      a = fma(0.33, ws[63136], a);
      a = fma(0.11, ws[63168], a);
      a = fma(0.43, ws[63904], a);
      a = fma(0.43, ws[63936], a);
      a = fma(0.37, ws[63968], a);
      a = fma(0.1105, ws[64000], a);
      a = fma(0.22, ws[64128], a);
      a = fma(0.56, ws[64160], a);
      a = fma(0.243, ws[64192], a);
      a = fma(1.5, ws[64224], a);
      a = fma(1.5, ws[64256], a);
      a = fma(1.5, ws[64288], a);
      a = fma(1.0, ws[64544], a);
      a = fma(0.668, ws[64672], a);
      a = fma(2.0, ws[64704], a);
      a = fma(1.0, ws[64736], a);
      a = fma(0.65, ws[65984], a);
      a = fma(0.61, ws[66080], a);
      a = fma(0.5, ws[68512], a);
      a = fma(0.305, ws[68608], a);
      a = fma(0.5, ws[69696], a);
      a = fma(0.5, ws[69792], a);
      a = fma(1.0, ws[70816], a);
      a = fma(0.61, ws[70912], a);
      a = fma(0.84, ws[71904], a);
      a = fma(1.0, ws[71968], a);
      a = fma(0.63, ws[72192], a);
      a = fma(0.43, ws[72352], a);
      yout[5664] = a;
    }
    {
      double a = -ws[63648];
      a = fma(0.06, ws[63936], a);
      a = fma(0.017, ws[63968], a);
      a = fma(0.0065, ws[64000], a);
      a = fma(0.01, ws[64032], a);
      a = fma(0.07, ws[64160], a);
      a = fma(0.25, ws[64288], a);
      a = fma(0.15, ws[67168], a);
      a = fma(0.15, ws[67200], a);
      a = fma(0.1, ws[68352], a);
      a = fma(0.1, ws[68384], a);
      a = fma(0.125, ws[68416], a);
      a = fma(0.067, ws[68512], a);
      a = fma(0.292, ws[68576], a);
      a = fma(0.5, ws[68928], a);
      a = fma(0.5, ws[68960], a);
      a = fma(0.5, ws[68992], a);
      a = fma(0.5, ws[69024], a);
      a = fma(0.5, ws[69056], a);
      a = fma(0.5, ws[69088], a);
      a = fma(0.3, ws[69120], a);
      a = fma(0.3, ws[69152], a);
      a = fma(0.3, ws[69184], a);
      a = fma(0.3, ws[69216], a);
      a = fma(0.5, ws[69248], a);
      a = fma(0.5, ws[69312], a);
      a = fma(0.5, ws[69376], a);
      a = fma(0.5, ws[69440], a);
      a = fma(0.5, ws[69504], a);
      a = fma(0.75, ws[69600], a);
      a = fma(0.5, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.635, ws[69696], a);
      a = fma(0.5, ws[69728], a);
      a = fma(1.083, ws[69760], a);
      a = fma(0.5, ws[69792], a);
      a = fma(0.5, ws[70016], a);
      a = fma(0.3, ws[72160], a);
      a = fma(0.3, ws[75104], a);
      a = fma(0.3, ws[75296], a);
      a = fma(0.3, ws[75488], a);
      a = fma(0.3, ws[76288], a);
      yout[5696] = a;
    }
    {
      double a = -ws[60320];
      a = fma(0.78, ws[63136], a);
      a = fma(0.79, ws[63168], a);
      a = a - ws[63488];
      a = fma(0.65, ws[64224], a);
      a = fma(0.65, ws[64256], a);
      a = fma(0.68, ws[66176], a);
      a = fma(1.0, ws[66336], a);
      a = fma(1.0, ws[66528], a);
      a = fma(1.0, ws[66560], a);
      a = fma(1.0, ws[66592], a);
      a = fma(1.0, ws[66624], a);
      a = fma(1.0, ws[66656], a);
      a = fma(1.0, ws[66688], a);
      a = fma(0.6021, ws[66720], a);
      a = fma(0.7195, ws[66752], a);
      a = fma(0.0482, ws[66784], a);
      a = fma(0.0854, ws[66816], a);
      a = fma(0.85, ws[67232], a);
      a = fma(1.0, ws[67264], a);
      a = fma(1.0, ws[67296], a);
      a = fma(1.0, ws[67392], a);
      a = fma(1.0, ws[67424], a);
      a = fma(1.0, ws[67456], a);
      a = fma(1.0, ws[67520], a);
      a = fma(1.0, ws[67552], a);
      a = fma(1.0, ws[67648], a);
      a = fma(1.0, ws[67680], a);
      a = fma(0.68, ws[68704], a);
      a = fma(0.7, ws[68864], a);
      a = fma(0.68, ws[69888], a);
      a = fma(0.7, ws[70048], a);
      a = fma(0.68, ws[71008], a);
      a = fma(1.0, ws[71168], a);
      a = fma(1.0, ws[72096], a);
      a = fma(0.6, ws[72320], a);
      a = fma(1.0, ws[74016], a);
      a = fma(0.004, ws[75552], a);
      a = fma(0.0135, ws[75648], a);
      a = fma(0.0062, ws[75680], a);
      a = fma(0.0054, ws[75712], a);
      a = fma(0.017, ws[75776], a);
      a = fma(0.0025, ws[75808], a);
      a = fma(0.0023, ws[75840], a);
      a = fma(0.0114, ws[75872], a);
      a = fma(0.0155, ws[75904], a);
      a = fma(0.0384, ws[75936], a);
      a = fma(0.0585, ws[75968], a);
      yout[5728] = a;
    }
    {
      double a = -ws[59712];
      a = fma(0.434, ws[59808], a);
      a = fma(1.0, ws[60320], a);
      a = fma(1.0, ws[60352], a);
      a = fma(1.0, ws[60384], a);
      a = fma(0.2, ws[60448], a);
      a = a - ws[62784];
      a = fma(0.4, ws[63104], a);
      a = fma(0.719, ws[63392], a);
      a = fma(1.0, ws[63424], a);
      a = fma(0.08, ws[63488], a);
      a = fma(0.08, ws[63520], a);
      a = fma(0.08, ws[63552], a);
      a = fma(0.02, ws[63840], a);
      a = fma(0.44, ws[63936], a);
      a = fma(0.73, ws[63968], a);
      a = fma(1.0, ws[64064], a);
      a = fma(0.02, ws[64096], a);
      a = fma(0.1, ws[64160], a);
      a = fma(0.02, ws[64512], a);
      a = a - ws[64608];
      a = fma(0.332, ws[64672], a);
      a = fma(0.132, ws[65216], a);
      a = fma(0.203, ws[65248], a);
      a = fma(0.2, ws[65280], a);
      a = fma(0.44, ws[65312], a);
      a = fma(0.68, ws[65344], a);
      a = fma(0.284, ws[65504], a);
      a = fma(0.154, ws[65568], a);
      a = fma(0.46, ws[65952], a);
      a = fma(0.7, ws[66048], a);
      a = fma(0.27, ws[66080], a);
      a = fma(1.24, ws[66304], a);
      a = fma(0.077, ws[66912], a);
      a = fma(0.198, ws[67776], a);
      a = fma(0.251, ws[67808], a);
      a = fma(0.15, ws[67840], a);
      a = fma(0.705, ws[67872], a);
      a = fma(1.28, ws[67904], a);
      a = fma(0.023, ws[68064], a);
      a = fma(0.2385, ws[68096], a);
      a = fma(0.119, ws[68160], a);
      a = fma(1.75, ws[68576], a);
      a = fma(0.203, ws[68608], a);
      a = fma(0.93, ws[68832], a);
      a = fma(0.273, ws[68960], a);
      a = fma(0.381, ws[68992], a);
      a = fma(0.2, ws[69024], a);
      a = fma(0.94, ws[69056], a);
      a = fma(1.71, ws[69088], a);
      a = fma(0.371, ws[69280], a);
      a = fma(0.168, ws[69344], a);
      a = fma(2.3, ws[69760], a);
      a = fma(0.27, ws[69792], a);
      a = fma(1.24, ws[70016], a);
      a = fma(0.147, ws[70208], a);
      a = fma(0.241, ws[70240], a);
      a = fma(0.2, ws[70272], a);
      a = fma(0.47, ws[70304], a);
      a = fma(0.72, ws[70336], a);
      a = fma(0.031, ws[70496], a);
      a = fma(0.371, ws[70528], a);
      a = fma(0.168, ws[70592], a);
      a = fma(0.7, ws[70880], a);
      a = fma(0.27, ws[70912], a);
      a = fma(1.24, ws[71136], a);
      a = fma(0.64, ws[71232], a);
      a = fma(1.21, ws[71264], a);
      a = fma(1.0, ws[72384], a);
      a = fma(0.387, ws[72448], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5760] = a;
    }
    {
      double a = 1.0 * ws[59744];
      a = fma(0.784, ws[59808], a);
      a = fma(0.9, ws[59904], a);
      a = fma(0.5, ws[59936], a);
      a = fma(1.0, ws[59968], a);
      a = fma(0.67, ws[60000], a);
      a = fma(1.0, ws[60160], a);
      a = fma(0.25, ws[60192], a);
      a = fma(0.25, ws[60224], a);
      a = fma(1.0, ws[60480], a);
      a = fma(0.018, ws[62176], a);
      a = fma(0.11, ws[62368], a);
      a = fma(1.0, ws[62752], a);
      a = fma(0.313, ws[63008], a);
      a = fma(1.0, ws[63072], a);
      a = fma(0.65, ws[63680], a);
      a = fma(0.09, ws[63968], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.1, ws[64128], a);
      a = fma(0.28, ws[64160], a);
      a = fma(0.002, ws[64192], a);
      a = fma(1.0, ws[64576], a);
      a = fma(1.0, ws[64736], a);
      a = a - ws[64960];
      a = fma(1.0, ws[64992], a);
      a = a - ws[65824];
      a = fma(1.0, ws[65888], a);
      a = fma(0.23, ws[65952], a);
      a = fma(0.35, ws[65984], a);
      a = fma(0.7, ws[66048], a);
      a = a - ws[67168];
      a = fma(0.15, ws[67232], a);
      a = a - ws[68352];
      a = fma(0.5, ws[68416], a);
      a = fma(0.269, ws[68512], a);
      a = fma(1.16, ws[68576], a);
      a = a - ws[68928];
      a = a - ws[68960];
      a = a - ws[68992];
      a = a - ws[69024];
      a = a - ws[69056];
      a = a - ws[69088];
      a = a - ws[69120];
      a = a - ws[69152];
      a = a - ws[69184];
      a = a - ws[69216];
      a = a - ws[69248];
      a = a - ws[69280];
      a = a - ws[69312];
      a = a - ws[69344];
      a = a - ws[69376];
      a = a - ws[69408];
      a = a - ws[69440];
      a = a - ws[69472];
      a = a - ws[69504];
      a = a - ws[69536];
      a = a - ws[69536];
      a = a - ws[69568];
      a = a - ws[69600];
      a = fma(0.5, ws[69600], a);
      a = a - ws[69632];
      a = a - ws[69664];
      a = a - ws[69696];
      a = fma(0.269, ws[69696], a);
      a = a - ws[69728];
      a = a - ws[69760];
      a = fma(1.16, ws[69760], a);
      a = a - ws[69792];
      a = a - ws[69824];
      a = a - ws[69856];
      a = a - ws[69888];
      a = a - ws[69920];
      a = a - ws[69952];
      a = a - ws[69984];
      a = a - ws[70016];
      a = a - ws[70048];
      a = a - ws[70080];
      a = a - ws[70656];
      a = fma(1.0, ws[70720], a);
      a = fma(0.538, ws[70816], a);
      a = fma(0.7, ws[70880], a);
      a = fma(0.354, ws[71968], a);
      a = a - ws[72160];
      a = a - ws[75104];
      a = a - ws[75296];
      a = a - ws[75488];
      a = a - ws[76288];
      yout[5792] = a;
    }
    {
      double a = 1.0 * ws[59424];
      a = fma(1.0, ws[59456], a);
      a = fma(1.0, ws[59520], a);
      a = a - ws[60672];
      a = a - ws[61056];
      a = a - ws[61088];
      a = a - ws[61120];
      a = a - ws[61152];
      a = a - ws[61184];
      a = a - ws[61184];
      a = fma(1.0, ws[61248], a);
      a = a - ws[61440];
      a = fma(1.0, ws[61472], a);
      a = a - ws[62304];
      a = a - ws[62432];
      a = a - ws[65152];
      a = a - ws[65184];
      a = a - ws[65216];
      a = a - ws[65248];
      a = a - ws[65280];
      a = a - ws[65312];
      a = a - ws[65344];
      a = a - ws[65376];
      a = a - ws[65408];
      a = a - ws[65440];
      a = a - ws[65472];
      a = a - ws[65504];
      a = a - ws[65536];
      a = a - ws[65568];
      a = a - ws[65600];
      a = a - ws[65632];
      a = a - ws[65664];
      a = a - ws[65696];
      a = a - ws[65728];
      a = a - ws[65760];
      a = a - ws[65792];
      a = a - ws[65824];
      a = a - ws[65856];
      a = a - ws[65888];
      a = a - ws[65920];
      a = a - ws[65952];
      a = a - ws[65984];
      a = a - ws[66016];
      a = a - ws[66048];
      a = a - ws[66080];
      a = a - ws[66112];
      a = a - ws[66144];
      a = a - ws[66176];
      a = a - ws[66208];
      a = a - ws[66240];
      a = a - ws[66272];
      a = a - ws[66304];
      a = a - ws[66336];
      a = a - ws[66368];
      a = a - ws[72032];
      a = a - ws[72288];
      a = a - ws[72544];
      a = a - ws[72736];
      a = a - ws[73376];
      a = a - ws[73408];
      a = a - ws[73440];
      a = a - ws[73472];
      a = a - ws[73504];
      a = a - ws[73536];
      a = a - ws[73568];
      a = a - ws[74272];
      a = a - ws[74304];
      a = a - ws[74336];
      a = a - ws[74368];
      a = a - ws[74400];
      a = a - ws[74432];
      a = a - ws[74464];
      a = a - ws[75008];
      a = a - ws[75200];
      a = a - ws[75392];
      a = a - ws[76192];
      yout[5824] = a;
    }
    {
      double a = -ws[59616];
      a = a - ws[59648];
      a = fma(0.35, ws[59808], a);
      a = fma(1.0, ws[59968], a);
      a = fma(0.67, ws[60000], a);
      a = fma(1.0, ws[60096], a);
      a = fma(1.0, ws[60288], a);
      a = fma(1.0, ws[62176], a);
      a = fma(0.35, ws[62208], a);
      a = fma(0.25, ws[62240], a);
      a = fma(0.4, ws[62304], a);
      a = fma(0.2, ws[62432], a);
      a = fma(1.0, ws[62496], a);
      a = a - ws[62720];
      a = fma(1.0, ws[63328], a);
      a = fma(0.35, ws[63456], a);
      a = fma(0.35, ws[63680], a);
      a = fma(1.0, ws[63712], a);
      a = fma(1.0, ws[63744], a);
      a = fma(0.21, ws[63840], a);
      a = fma(1.0, ws[63904], a);
      a = fma(0.56, ws[63936], a);
      a = fma(0.09, ws[63968], a);
      a = fma(0.459, ws[64000], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.62, ws[64064], a);
      a = fma(0.21, ws[64096], a);
      a = fma(0.1, ws[64160], a);
      a = fma(0.08, ws[64192], a);
      a = fma(0.05, ws[64224], a);
      a = fma(0.05, ws[64256], a);
      a = fma(0.21, ws[64512], a);
      a = a - ws[64544];
      a = fma(0.68, ws[64640], a);
      a = fma(0.332, ws[64672], a);
      a = fma(1.0, ws[65152], a);
      a = fma(0.018, ws[65248], a);
      a = fma(1.6, ws[65280], a);
      a = fma(0.78, ws[65312], a);
      a = fma(0.308, ws[65504], a);
      a = fma(0.007, ws[65568], a);
      a = fma(0.43, ws[65632], a);
      a = fma(0.36, ws[65792], a);
      a = fma(1.0, ws[65888], a);
      a = fma(0.33, ws[65920], a);
      a = fma(0.65, ws[65984], a);
      a = fma(0.5, ws[66016], a);
      a = fma(0.3, ws[66048], a);
      a = fma(0.03, ws[66080], a);
      a = fma(0.287, ws[66304], a);
      a = fma(0.0625, ws[66848], a);
      a = fma(0.007, ws[66912], a);
      a = fma(0.06, ws[66976], a);
      a = fma(0.1, ws[67136], a);
      a = fma(0.15, ws[67232], a);
      a = fma(1.37, ws[67712], a);
      a = fma(0.75, ws[67744], a);
      a = fma(0.827, ws[67776], a);
      a = fma(0.777, ws[67808], a);
      a = fma(1.95, ws[67840], a);
      a = fma(1.5, ws[67872], a);
      a = fma(0.75, ws[67904], a);
      a = fma(0.68, ws[67936], a);
      a = fma(0.68, ws[67968], a);
      a = fma(0.68, ws[68000], a);
      a = fma(0.68, ws[68032], a);
      a = fma(1.31, ws[68064], a);
      a = fma(1.0295, ws[68096], a);
      a = fma(0.75, ws[68128], a);
      a = fma(0.964, ws[68160], a);
      a = fma(0.75, ws[68192], a);
      a = fma(1.03, ws[68224], a);
      a = fma(0.75, ws[68256], a);
      a = fma(0.91, ws[68288], a);
      a = fma(0.75, ws[68320], a);
      a = fma(1.0, ws[68352], a);
      a = fma(1.0, ws[68384], a);
      a = fma(1.5, ws[68416], a);
      a = fma(1.0, ws[68448], a);
      a = fma(0.75, ws[68480], a);
      a = fma(1.66, ws[68512], a);
      a = fma(1.5, ws[68544], a);
      a = fma(1.5, ws[68576], a);
      a = fma(0.773, ws[68608], a);
      a = fma(1.0, ws[68640], a);
      a = fma(1.0, ws[68672], a);
      a = fma(1.0, ws[68704], a);
      a = fma(1.0, ws[68736], a);
      a = fma(1.0, ws[68768], a);
      a = fma(1.0, ws[68800], a);
      a = fma(0.965, ws[68832], a);
      a = fma(1.0, ws[68864], a);
      a = fma(1.0, ws[68896], a);
      a = fma(0.13, ws[68960], a);
      a = fma(0.042, ws[68992], a);
      a = fma(1.6, ws[69024], a);
      a = fma(1.0, ws[69056], a);
      a = fma(1.048, ws[69248], a);
      a = fma(0.403, ws[69280], a);
      a = fma(0.007, ws[69344], a);
      a = fma(0.56, ws[69408], a);
      a = fma(1.0, ws[69600], a);
      a = fma(0.33, ws[69632], a);
      a = fma(1.0, ws[69696], a);
      a = fma(1.0, ws[69728], a);
      a = fma(1.0, ws[69760], a);
      a = fma(0.03, ws[69792], a);
      a = fma(0.287, ws[70016], a);
      a = fma(1.0, ws[70144], a);
      a = fma(0.024, ws[70240], a);
      a = fma(1.6, ws[70272], a);
      a = fma(0.79, ws[70304], a);
      a = fma(0.75, ws[70496], a);
      a = fma(0.403, ws[70528], a);
      a = fma(0.56, ws[70560], a);
      a = fma(0.007, ws[70592], a);
      a = fma(1.0, ws[70720], a);
      a = fma(0.33, ws[70752], a);
      a = fma(1.0, ws[70816], a);
      a = fma(1.0, ws[70848], a);
      a = fma(0.3, ws[70880], a);
      a = fma(0.03, ws[70912], a);
      a = fma(0.287, ws[71136], a);
      a = fma(0.202, ws[71232], a);
      a = fma(0.504, ws[71264], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.72, ws[71904], a);
      a = fma(0.68, ws[71936], a);
      a = fma(0.15, ws[71968], a);
      a = fma(0.895, ws[72032], a);
      a = fma(0.925, ws[72064], a);
      a = fma(1.143, ws[72128], a);
      a = fma(0.74, ws[72160], a);
      a = fma(0.83, ws[72192], a);
      a = fma(0.68, ws[75072], a);
      a = fma(0.68, ws[75264], a);
      a = fma(0.68, ws[75456], a);
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      a = fma(1.68, ws[76256], a);
      a = fma(1.0, ws[76288], a);
      yout[5856] = a;
    }
    {
      double a = 1.0 * ws[59680];
      a = fma(1.0, ws[59744], a);
      a = fma(2.0, ws[59776], a);
      a = fma(0.1, ws[59904], a);
      a = fma(0.3, ws[60032], a);
      a = fma(1.0, ws[60416], a);
      a = fma(1.0, ws[60512], a);
      a = fma(1.0, ws[61792], a);
      a = fma(0.4, ws[62176], a);
      a = fma(0.65, ws[63456], a);
      a = fma(0.64, ws[63648], a);
      a = fma(0.08, ws[63936], a);
      a = fma(0.32, ws[63968], a);
      a = fma(0.008, ws[64192], a);
      a = a - ws[65152];
      a = fma(0.131, ws[65216], a);
      a = fma(0.051, ws[65248], a);
      a = fma(1.0, ws[65824], a);
      a = fma(0.65, ws[65984], a);
      a = a - ws[66496];
      a = fma(0.44, ws[67168], a);
      a = a - ws[67712];
      a = a - ws[67712];
      a = a - ws[67744];
      a = a - ws[67776];
      a = fma(0.08, ws[67776], a);
      a = a - ws[67808];
      a = fma(0.018, ws[67808], a);
      a = a - ws[67840];
      a = a - ws[67872];
      a = a - ws[67904];
      a = a - ws[67936];
      a = a - ws[67968];
      a = a - ws[68000];
      a = a - ws[68032];
      a = a - ws[68064];
      a = a - ws[68096];
      a = a - ws[68128];
      a = a - ws[68160];
      a = a - ws[68192];
      a = a - ws[68224];
      a = a - ws[68256];
      a = a - ws[68288];
      a = a - ws[68320];
      a = a - ws[68352];
      a = fma(0.9, ws[68352], a);
      a = a - ws[68384];
      a = fma(0.9, ws[68384], a);
      a = a - ws[68416];
      a = a - ws[68448];
      a = a - ws[68480];
      a = a - ws[68512];
      a = fma(0.25, ws[68512], a);
      a = a - ws[68544];
      a = a - ws[68576];
      a = a - ws[68608];
      a = a - ws[68640];
      a = a - ws[68672];
      a = a - ws[68704];
      a = a - ws[68736];
      a = a - ws[68768];
      a = a - ws[68800];
      a = a - ws[68832];
      a = a - ws[68864];
      a = a - ws[68896];
      a = fma(0.5, ws[68928], a);
      a = fma(0.58, ws[68960], a);
      a = fma(0.518, ws[68992], a);
      a = fma(0.5, ws[69024], a);
      a = fma(0.5, ws[69056], a);
      a = fma(0.5, ws[69088], a);
      a = fma(0.7, ws[69120], a);
      a = fma(0.7, ws[69152], a);
      a = fma(0.7, ws[69184], a);
      a = fma(0.7, ws[69216], a);
      a = fma(0.5, ws[69248], a);
      a = fma(1.0, ws[69280], a);
      a = fma(0.5, ws[69312], a);
      a = fma(1.0, ws[69344], a);
      a = fma(0.5, ws[69376], a);
      a = fma(1.0, ws[69408], a);
      a = fma(0.5, ws[69440], a);
      a = fma(1.0, ws[69472], a);
      a = fma(0.5, ws[69504], a);
      a = fma(2.0, ws[69536], a);
      a = fma(1.0, ws[69568], a);
      a = fma(0.5, ws[69600], a);
      a = fma(0.5, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.5, ws[69696], a);
      a = fma(0.5, ws[69728], a);
      a = fma(0.5, ws[69760], a);
      a = fma(0.5, ws[69792], a);
      a = fma(1.0, ws[69824], a);
      a = fma(1.0, ws[69856], a);
      a = fma(1.0, ws[69888], a);
      a = fma(1.0, ws[69920], a);
      a = fma(1.0, ws[69952], a);
      a = fma(1.0, ws[69984], a);
      a = fma(0.5, ws[70016], a);
      a = fma(1.0, ws[70048], a);
      a = fma(1.0, ws[70080], a);
      a = a - ws[70144];
      a = fma(0.14, ws[70208], a);
      a = fma(0.055, ws[70240], a);
      a = fma(1.0, ws[70656], a);
      a = fma(0.027, ws[71968], a);
      a = a - ws[72128];
      a = fma(0.7, ws[72160], a);
      a = fma(0.17, ws[72288], a);
      a = fma(0.08, ws[72320], a);
      a = fma(0.34, ws[72352], a);
      a = a - ws[75072];
      a = fma(0.7, ws[75104], a);
      a = a - ws[75264];
      a = fma(0.7, ws[75296], a);
      a = a - ws[75456];
      a = fma(0.7, ws[75488], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      a = fma(1.0, ws[76032], a);
      a = a - ws[76256];
      a = fma(0.7, ws[76288], a);
      yout[5888] = a;
    }
    {
      double a = -ws[59424];
      a = fma(1.0, ws[59488], a);
      a = fma(1.0, ws[59552], a);
      a = fma(0.8, ws[59584], a);
      a = fma(1.0, ws[60448], a);
      a = fma(1.0, ws[60480], a);
      a = fma(1.0, ws[60544], a);
      a = fma(1.0, ws[60576], a);
      a = fma(1.0, ws[60672], a);
      a = a - ws[60704];
      a = fma(1.0, ws[61056], a);
      a = fma(1.0, ws[61120], a);
      a = fma(2.0, ws[61184], a);
      a = fma(1.0, ws[61216], a);
      a = a - ws[61248];
      a = a - ws[61280];
      a = a - ws[61312];
      a = fma(1.0, ws[61376], a);
      a = fma(0.7, ws[61408], a);
      a = fma(2.0, ws[61440], a);
      a = a - ws[61472];
      a = fma(1.0, ws[61472], a);
      a = fma(2.0, ws[61504], a);
      a = a - ws[61536];
      a = fma(1.0, ws[61568], a);
      a = a - ws[61632];
      a = fma(1.0, ws[61664], a);
      a = fma(1.0, ws[61696], a);
      a = fma(0.4, ws[62208], a);
      a = fma(0.87, ws[62304], a);
      a = fma(1.3, ws[62432], a);
      a = fma(0.65, ws[62464], a);
      a = fma(1.0, ws[62496], a);
      a = fma(1.0, ws[63776], a);
      a = fma(1.0, ws[63808], a);
      a = fma(0.67, ws[63840], a);
      a = fma(0.67, ws[64096], a);
      a = fma(0.67, ws[64512], a);
      a = fma(0.68, ws[64640], a);
      a = fma(1.0, ws[64864], a);
      a = a - ws[64960];
      a = fma(1.0, ws[64992], a);
      a = a - ws[65024];
      a = fma(1.0, ws[65056], a);
      a = a - ws[65088];
      a = fma(1.0, ws[65120], a);
      a = fma(1.0, ws[65152], a);
      a = fma(1.0, ws[65184], a);
      a = fma(0.935, ws[65216], a);
      a = fma(0.864, ws[65248], a);
      a = fma(1.0, ws[65280], a);
      a = fma(0.97, ws[65312], a);
      a = fma(0.95, ws[65344], a);
      a = fma(0.998, ws[65376], a);
      a = fma(0.998, ws[65408], a);
      a = fma(0.998, ws[65440], a);
      a = fma(0.998, ws[65472], a);
      a = fma(0.763, ws[65504], a);
      a = fma(0.82, ws[65536], a);
      a = fma(1.6955, ws[65568], a);
      a = fma(0.82, ws[65600], a);
      a = fma(0.77, ws[65632], a);
      a = fma(0.77, ws[65664], a);
      a = fma(1.36, ws[65696], a);
      a = fma(0.77, ws[65728], a);
      a = fma(0.64, ws[65760], a);
      a = fma(0.36, ws[65792], a);
      a = fma(1.0, ws[65824], a);
      a = fma(1.0, ws[65856], a);
      a = fma(1.0, ws[65888], a);
      a = fma(1.0, ws[65920], a);
      a = fma(1.0, ws[65952], a);
      a = fma(1.0, ws[65984], a);
      a = fma(1.0, ws[66016], a);
      a = fma(1.0, ws[66048], a);
      a = fma(1.0, ws[66080], a);
      a = fma(1.0, ws[66112], a);
      a = fma(1.0, ws[66144], a);
      a = fma(1.0, ws[66176], a);
      a = fma(1.0, ws[66208], a);
      a = fma(1.0, ws[66240], a);
      a = fma(1.0, ws[66272], a);
      a = fma(2.0, ws[66304], a);
      a = fma(2.0, ws[66336], a);
      a = fma(1.0, ws[66368], a);
      a = a - ws[66400];
      a = a - ws[66432];
      a = a - ws[66464];
      a = fma(0.539, ws[66912], a);
      a = fma(0.23, ws[67040], a);
      a = fma(0.659, ws[68160], a);
      a = fma(0.75, ws[68192], a);
      a = fma(0.31, ws[68288], a);
      a = fma(0.75, ws[68320], a);
      a = fma(1.0, ws[68544], a);
      a = fma(0.5, ws[68832], a);
      a = fma(0.7, ws[68864], a);
      a = fma(0.825, ws[69344], a);
      a = fma(0.5, ws[69376], a);
      a = fma(0.46, ws[69472], a);
      a = fma(0.5, ws[69504], a);
      a = fma(1.0, ws[69728], a);
      a = fma(1.0, ws[70016], a);
      a = fma(0.7, ws[70048], a);
      a = fma(1.0, ws[70144], a);
      a = fma(1.0, ws[70176], a);
      a = fma(1.0, ws[70208], a);
      a = fma(1.0, ws[70240], a);
      a = fma(1.0, ws[70272], a);
      a = fma(1.0, ws[70304], a);
      a = fma(1.0, ws[70336], a);
      a = fma(1.0, ws[70368], a);
      a = fma(1.0, ws[70400], a);
      a = fma(1.0, ws[70432], a);
      a = fma(1.0, ws[70464], a);
      a = fma(1.0, ws[70496], a);
      a = fma(1.0, ws[70528], a);
      a = fma(1.0, ws[70560], a);
      a = fma(1.825, ws[70592], a);
      a = fma(1.46, ws[70624], a);
      a = fma(1.0, ws[70656], a);
      a = fma(1.0, ws[70688], a);
      a = fma(1.0, ws[70720], a);
      a = fma(1.0, ws[70752], a);
      a = fma(1.0, ws[70784], a);
      a = fma(1.0, ws[70816], a);
      a = fma(1.0, ws[70848], a);
      a = fma(1.0, ws[70880], a);
      a = fma(1.0, ws[70912], a);
      a = fma(1.0, ws[70944], a);
      a = fma(1.0, ws[70976], a);
      a = fma(1.0, ws[71008], a);
      a = fma(1.0, ws[71040], a);
      a = fma(1.0, ws[71072], a);
      a = fma(1.0, ws[71104], a);
      a = fma(2.0, ws[71136], a);
      a = fma(2.0, ws[71168], a);
      a = fma(0.5, ws[71232], a);
      a = fma(1.0, ws[71264], a);
      a = fma(1.0, ws[71296], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71680], a);
      a = fma(0.48, ws[71712], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.68, ws[71936], a);
      a = fma(0.968, ws[72032], a);
      a = fma(1.0, ws[72064], a);
      a = fma(0.92, ws[72288], a);
      a = fma(1.0, ws[72416], a);
      a = fma(2.0, ws[72544], a);
      a = fma(2.0, ws[72576], a);
      a = fma(0.753, ws[72736], a);
      a = a - ws[72864];
      a = fma(0.72, ws[73376], a);
      a = fma(0.72, ws[73408], a);
      a = fma(0.72, ws[73440], a);
      a = fma(0.72, ws[73472], a);
      a = fma(0.72, ws[73504], a);
      a = fma(0.72, ws[73536], a);
      a = fma(0.74, ws[73568], a);
      a = fma(1.0, ws[73600], a);
      a = fma(1.0, ws[73632], a);
      a = fma(1.0, ws[73664], a);
      a = fma(1.0, ws[73696], a);
      a = fma(1.0, ws[73728], a);
      a = fma(1.0, ws[73760], a);
      a = fma(1.0, ws[73792], a);
      a = fma(0.86, ws[74272], a);
      a = fma(0.86, ws[74304], a);
      a = fma(0.86, ws[74336], a);
      a = fma(0.86, ws[74368], a);
      a = fma(0.86, ws[74400], a);
      a = fma(0.86, ws[74432], a);
      a = fma(0.88, ws[74464], a);
      a = fma(1.0, ws[74496], a);
      a = fma(1.0, ws[74528], a);
      a = fma(1.0, ws[74560], a);
      a = fma(1.0, ws[74592], a);
      a = fma(1.0, ws[74624], a);
      a = fma(1.0, ws[74656], a);
      a = fma(1.0, ws[74688], a);
      a = fma(0.998, ws[75008], a);
      a = fma(1.0, ws[75040], a);
      a = fma(0.998, ws[75200], a);
      a = fma(1.0, ws[75232], a);
      a = fma(0.998, ws[75392], a);
      a = fma(1.0, ws[75424], a);
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      yout[5920] = a;
    }
    {
      double a = -ws[59456];
      a = a - ws[59488];
      a = fma(0.2, ws[59584], a);
      a = fma(1.0, ws[60512], a);
      a = fma(1.0, ws[60704], a);
      a = fma(1.0, ws[61280], a);
      a = fma(1.0, ws[61344], a);
      a = a - ws[61376];
      a = a - ws[61408];
      a = a - ws[61440];
      a = a - ws[61472];
      a = a - ws[61504];
      a = a - ws[61504];
      a = a - ws[61536];
      a = fma(1.0, ws[61568], a);
      a = a - ws[62208];
      a = fma(1.0, ws[63712], a);
      a = fma(1.0, ws[63744], a);
      a = fma(1.0, ws[63872], a);
      a = a - ws[64352];
      a = a - ws[64384];
      a = a - ws[64416];
      a = a - ws[64448];
      a = a - ws[64480];
      a = a - ws[64512];
      a = a - ws[64544];
      a = a - ws[64576];
      a = a - ws[64608];
      a = a - ws[64640];
      a = a - ws[64672];
      a = a - ws[64704];
      a = a - ws[64736];
      a = a - ws[64768];
      a = a - ws[64800];
      a = a - ws[64832];
      a = a - ws[64864];
      a = a - ws[70144];
      a = a - ws[70176];
      a = a - ws[70208];
      a = a - ws[70240];
      a = a - ws[70272];
      a = a - ws[70304];
      a = a - ws[70336];
      a = a - ws[70368];
      a = a - ws[70400];
      a = a - ws[70432];
      a = a - ws[70464];
      a = a - ws[70496];
      a = a - ws[70528];
      a = a - ws[70560];
      a = a - ws[70592];
      a = a - ws[70624];
      a = a - ws[70656];
      a = a - ws[70688];
      a = a - ws[70720];
      a = a - ws[70752];
      a = a - ws[70784];
      a = a - ws[70816];
      a = a - ws[70848];
      a = a - ws[70880];
      a = a - ws[70912];
      a = a - ws[70944];
      a = a - ws[70976];
      a = a - ws[71008];
      a = a - ws[71040];
      a = a - ws[71072];
      a = a - ws[71104];
      a = a - ws[71136];
      a = a - ws[71168];
      a = a - ws[71296];
      a = a - ws[71936];
      a = a - ws[72064];
      a = a - ws[72224];
      a = a - ws[72416];
      a = a - ws[72480];
      a = a - ws[72576];
      a = a - ws[72704];
      a = a - ws[72928];
      a = a - ws[73600];
      a = a - ws[73632];
      a = a - ws[73664];
      a = a - ws[73696];
      a = a - ws[73728];
      a = a - ws[73760];
      a = a - ws[73792];
      a = a - ws[74496];
      a = a - ws[74528];
      a = a - ws[74560];
      a = a - ws[74592];
      a = a - ws[74624];
      a = a - ws[74656];
      a = a - ws[74688];
      a = a - ws[75040];
      a = a - ws[75232];
      a = a - ws[75424];
      a = a - ws[76224];
      yout[5952] = a;
    }
    {
      double a = 0.8 * ws[59584];
      a = fma(2.0, ws[59648], a);
      a = fma(1.0, ws[59680], a);
      a = fma(1.0, ws[59712], a);
      a = fma(1.22, ws[59808], a);
      a = fma(1.0, ws[59840], a);
      a = fma(1.0, ws[59872], a);
      a = fma(1.0, ws[59968], a);
      a = fma(0.66, ws[60000], a);
      a = fma(2.0, ws[60128], a);
      a = fma(1.0, ws[60160], a);
      a = fma(1.5, ws[60192], a);
      a = fma(1.5, ws[60224], a);
      a = fma(1.0, ws[60256], a);
      a = fma(1.0, ws[60288], a);
      a = fma(1.0, ws[60320], a);
      a = fma(1.0, ws[60352], a);
      a = fma(1.0, ws[60384], a);
      a = fma(1.0, ws[60448], a);
      a = fma(1.0, ws[60608], a);
      a = a - ws[60640];
      a = fma(1.0, ws[60896], a);
      a = a - ws[60928];
      a = a - ws[60960];
      a = a - ws[60960];
      a = a - ws[60992];
      a = a - ws[60992];
      a = fma(1.0, ws[61024], a);
      a = a - ws[61120];
      a = a - ws[61152];
      a = fma(1.0, ws[61376], a);
      a = a - ws[61408];
      a = a - ws[61632];
      a = fma(1.0, ws[61664], a);
      a = fma(1.0, ws[61728], a);
      a = fma(1.0, ws[61760], a);
      a = fma(0.35, ws[62016], a);
      a = fma(0.53, ws[62048], a);
      a = fma(0.18, ws[62080], a);
      a = fma(0.17, ws[62112], a);
      a = fma(0.18, ws[62144], a);
      a = fma(0.25, ws[62176], a);
      a = a - ws[62272];
      a = fma(0.07, ws[62272], a);
      a = fma(0.88, ws[62304], a);
      a = fma(0.34, ws[62368], a);
      a = a - ws[62400];
      a = fma(0.3, ws[62496], a);
      a = fma(1.0, ws[62720], a);
      a = fma(1.0, ws[62912], a);
      a = fma(1.0, ws[63040], a);
      a = fma(0.52, ws[63104], a);
      a = fma(0.52, ws[63136], a);
      a = fma(0.56, ws[63168], a);
      a = fma(0.619, ws[63232], a);
      a = fma(0.584, ws[63264], a);
      a = fma(1.0, ws[63328], a);
      a = fma(1.0, ws[63360], a);
      a = fma(1.0, ws[63392], a);
      a = fma(1.0, ws[63424], a);
      a = fma(1.0, ws[63616], a);
      a = fma(0.15, ws[63904], a);
      a = fma(0.32, ws[63936], a);
      a = fma(0.07, ws[63968], a);
      a = fma(0.1105, ws[64000], a);
      a = fma(0.14, ws[64128], a);
      a = fma(0.11, ws[64160], a);
      a = fma(0.072, ws[64192], a);
      a = fma(1.0, ws[64224], a);
      a = fma(1.0, ws[64256], a);
      a = fma(1.0, ws[64288], a);
      a = fma(1.0, ws[64544], a);
      a = fma(1.0, ws[64672], a);
      a = fma(1.0, ws[64704], a);
      a = fma(1.0, ws[65152], a);
      a = fma(1.0, ws[65184], a);
      a = fma(0.66, ws[65216], a);
      a = fma(0.2, ws[65248], a);
      a = fma(1.0, ws[65280], a);
      a = fma(0.78, ws[65312], a);
      a = fma(0.83, ws[65344], a);
      a = fma(0.998, ws[65376], a);
      a = fma(0.998, ws[65408], a);
      a = fma(0.998, ws[65440], a);
      a = fma(0.998, ws[65472], a);
      a = fma(0.763, ws[65504], a);
      a = fma(0.1645, ws[65568], a);
      a = fma(0.77, ws[65632], a);
      a = fma(0.5, ws[65696], a);
      a = fma(0.36, ws[65792], a);
      a = fma(0.67, ws[65920], a);
      a = fma(0.77, ws[65952], a);
      a = fma(0.5, ws[66016], a);
      a = fma(0.3, ws[66048], a);
      a = fma(1.0, ws[66080], a);
      a = fma(1.0, ws[66176], a);
      a = fma(1.0, ws[66240], a);
      a = fma(1.0, ws[66272], a);
      a = a - ws[66496];
      a = a - ws[66528];
      a = a - ws[66560];
      a = a - ws[66592];
      a = a - ws[66624];
      a = a - ws[66656];
      a = a - ws[66688];
      a = a - ws[66720];
      a = a - ws[66752];
      a = a - ws[66784];
      a = a - ws[66816];
      a = a - ws[66848];
      a = fma(0.3225, ws[66848], a);
      a = a - ws[66880];
      a = a - ws[66912];
      a = a - ws[66944];
      a = a - ws[66976];
      a = fma(0.1, ws[66976], a);
      a = a - ws[67008];
      a = a - ws[67040];
      a = fma(0.27, ws[67040], a);
      a = a - ws[67072];
      a = a - ws[67104];
      a = a - ws[67136];
      a = fma(0.1, ws[67136], a);
      a = a - ws[67168];
      a = a - ws[67200];
      a = a - ws[67232];
      a = a - ws[67264];
      a = a - ws[67296];
      a = a - ws[67328];
      a = a - ws[67360];
      a = a - ws[67392];
      a = a - ws[67424];
      a = a - ws[67456];
      a = a - ws[67488];
      a = a - ws[67520];
      a = a - ws[67552];
      a = a - ws[67584];
      a = a - ws[67616];
      a = a - ws[67648];
      a = a - ws[67680];
      a = fma(0.74, ws[67712], a);
      a = fma(1.0, ws[67744], a);
      a = fma(0.894, ws[67776], a);
      a = fma(0.842, ws[67808], a);
      a = fma(1.0, ws[67840], a);
      a = fma(1.0, ws[67872], a);
      a = fma(1.0, ws[67904], a);
      a = fma(1.37, ws[67936], a);
      a = fma(1.2846, ws[67968], a);
      a = fma(1.3218, ws[68000], a);
      a = fma(1.2846, ws[68032], a);
      a = fma(1.0, ws[68064], a);
      a = fma(1.279, ws[68096], a);
      a = fma(1.0, ws[68128], a);
      a = fma(0.918, ws[68160], a);
      a = fma(0.75, ws[68192], a);
      a = fma(1.0, ws[68224], a);
      a = fma(1.0, ws[68256], a);
      a = fma(1.01, ws[68288], a);
      a = fma(0.75, ws[68320], a);
      a = fma(0.9, ws[68352], a);
      a = fma(0.9, ws[68384], a);
      a = fma(0.5, ws[68416], a);
      a = fma(0.834, ws[68448], a);
      a = fma(1.0, ws[68480], a);
      a = fma(0.5, ws[68512], a);
      a = fma(1.0, ws[68544], a);
      a = fma(1.0, ws[68576], a);
      a = fma(1.0, ws[68608], a);
      a = fma(1.0, ws[68640], a);
      a = fma(1.0, ws[68672], a);
      a = fma(2.0, ws[68704], a);
      a = fma(1.0, ws[68736], a);
      a = fma(1.0, ws[68768], a);
      a = fma(2.0, ws[68800], a);
      a = fma(0.5, ws[68832], a);
      a = fma(1.0, ws[68864], a);
      a = fma(1.0, ws[68896], a);
      a = fma(0.5, ws[68928], a);
      a = fma(0.394, ws[68960], a);
      a = fma(0.342, ws[68992], a);
      a = fma(0.5, ws[69024], a);
      a = fma(0.5, ws[69056], a);
      a = fma(0.5, ws[69088], a);
      a = fma(1.0, ws[69120], a);
      a = fma(0.9146, ws[69152], a);
      a = fma(0.9518, ws[69184], a);
      a = fma(0.9146, ws[69216], a);
      a = fma(0.5, ws[69248], a);
      a = fma(1.0, ws[69280], a);
      a = fma(0.175, ws[69344], a);
      a = fma(1.0, ws[69408], a);
      a = fma(0.54, ws[69472], a);
      a = fma(0.33, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.5, ws[69728], a);
      a = fma(0.5, ws[69760], a);
      a = fma(0.5, ws[69792], a);
      a = fma(2.0, ws[69888], a);
      a = fma(1.0, ws[69920], a);
      a = fma(1.0, ws[69984], a);
      a = fma(1.0, ws[70048], a);
      a = fma(1.0, ws[70144], a);
      a = fma(1.0, ws[70176], a);
      a = fma(0.254, ws[70208], a);
      a = fma(0.488, ws[70240], a);
      a = fma(1.0, ws[70272], a);
      a = fma(0.79, ws[70304], a);
      a = fma(0.86, ws[70336], a);
      a = fma(1.0, ws[70368], a);
      a = fma(0.9146, ws[70400], a);
      a = fma(0.9518, ws[70432], a);
      a = fma(0.9146, ws[70464], a);
      a = fma(1.0, ws[70496], a);
      a = fma(1.0, ws[70528], a);
      a = fma(1.0, ws[70560], a);
      a = fma(0.175, ws[70592], a);
      a = fma(0.54, ws[70624], a);
      a = fma(0.67, ws[70752], a);
      a = fma(1.0, ws[70784], a);
      a = fma(1.0, ws[70848], a);
      a = fma(0.3, ws[70880], a);
      a = fma(1.0, ws[70912], a);
      a = fma(1.0, ws[71008], a);
      a = fma(1.0, ws[71072], a);
      a = fma(1.0, ws[71104], a);
      a = fma(1.0, ws[71200], a);
      a = fma(0.5, ws[71232], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71680], a);
      a = fma(0.48, ws[71712], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.56, ws[71904], a);
      a = fma(0.477, ws[71968], a);
      a = fma(0.333, ws[72000], a);
      a = fma(0.968, ws[72032], a);
      a = fma(1.0, ws[72064], a);
      a = a - ws[72096];
      a = fma(0.87, ws[72128], a);
      a = fma(0.8, ws[72160], a);
      a = fma(0.42, ws[72192], a);
      a = fma(0.49, ws[72256], a);
      a = fma(0.75, ws[72288], a);
      a = a - ws[72320];
      a = fma(0.32, ws[72320], a);
      a = fma(0.66, ws[72352], a);
      a = fma(1.0, ws[72448], a);
      a = a - ws[72512];
      a = a - ws[72672];
      a = a - ws[72896];
      a = a - ws[73824];
      a = a - ws[73856];
      a = a - ws[73888];
      a = a - ws[73920];
      a = a - ws[73952];
      a = a - ws[73984];
      a = a - ws[74016];
      a = fma(1.0, ws[74048], a);
      a = fma(1.0, ws[74080], a);
      a = fma(1.0, ws[74112], a);
      a = fma(1.0, ws[74144], a);
      a = fma(1.0, ws[74176], a);
      a = fma(1.0, ws[74208], a);
      a = fma(1.0, ws[74240], a);
      a = fma(0.86, ws[74272], a);
      a = fma(0.86, ws[74304], a);
      a = fma(0.86, ws[74336], a);
      a = fma(0.86, ws[74368], a);
      a = fma(0.86, ws[74400], a);
      a = fma(0.86, ws[74432], a);
      a = fma(0.88, ws[74464], a);
      a = fma(1.0, ws[74496], a);
      a = fma(1.0, ws[74528], a);
      a = fma(1.0, ws[74560], a);
      a = fma(1.0, ws[74592], a);
      a = fma(1.0, ws[74624], a);
      a = fma(1.0, ws[74656], a);
      a = fma(1.0, ws[74688], a);
      a = a - ws[74720];
      a = a - ws[74752];
      a = a - ws[74784];
      a = a - ws[74816];
      a = a - ws[74848];
      a = a - ws[74880];
      a = a - ws[74912];
      a = fma(0.16, ws[74944], a);
      a = a - ws[74976];
      a = fma(0.998, ws[75008], a);
      a = fma(0.9405, ws[75040], a);
      a = fma(1.3105, ws[75072], a);
      a = fma(0.9405, ws[75104], a);
      a = fma(0.16, ws[75136], a);
      a = a - ws[75168];
      a = fma(0.998, ws[75200], a);
      a = fma(0.9405, ws[75232], a);
      a = fma(1.3105, ws[75264], a);
      a = fma(0.9405, ws[75296], a);
      a = fma(0.16, ws[75328], a);
      a = a - ws[75360];
      a = fma(0.998, ws[75392], a);
      a = fma(0.9405, ws[75424], a);
      a = fma(1.3105, ws[75456], a);
      a = fma(0.9405, ws[75488], a);
      a = a - ws[76160];
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      a = fma(1.37, ws[76256], a);
      a = fma(1.0, ws[76288], a);
      yout[5984] = a;
    }
    {
      double a = 2.0 * ws[59392];
      a = fma(1.0, ws[59520], a);
      a = fma(1.0, ws[59552], a);
      a = fma(0.2, ws[59584], a);
      a = fma(0.34, ws[60000], a);
      a = fma(1.0, ws[60288], a);
      a = fma(1.0, ws[60320], a);
      a = fma(1.0, ws[60352], a);
      a = fma(1.0, ws[60384], a);
      a = fma(1.0, ws[60416], a);
      a = a - ws[60608];
      a = fma(1.0, ws[60640], a);
      a = fma(2.0, ws[60864], a);
      a = a - ws[60896];
      a = a - ws[60928];
      a = a - ws[61024];
      a = a - ws[61088];
      a = fma(1.0, ws[61120], a);
      a = a - ws[61216];
      a = a - ws[61312];
      a = a - ws[61344];
      a = a - ws[61376];
      a = fma(0.7, ws[61408], a);
      a = a - ws[61696];
      a = a - ws[61728];
      a = a - ws[61760];
      a = a - ws[61792];
      a = a - ws[61824];
      a = a - ws[61856];
      a = a - ws[61888];
      a = a - ws[61920];
      a = a - ws[61952];
      a = a - ws[61984];
      a = a - ws[62016];
      a = fma(0.65, ws[62016], a);
      a = a - ws[62048];
      a = a - ws[62080];
      a = a - ws[62112];
      a = a - ws[62144];
      a = fma(0.25, ws[62176], a);
      a = a - ws[62240];
      a = fma(0.5, ws[62272], a);
      a = a - ws[62336];
      a = a - ws[62368];
      a = fma(2.0, ws[62368], a);
      a = fma(0.45, ws[62400], a);
      a = a - ws[62464];
      a = fma(1.0, ws[62464], a);
      a = a - ws[62496];
      a = a - ws[62560];
      a = a - ws[62592];
      a = a - ws[62624];
      a = a - ws[62656];
      a = a - ws[62688];
      a = a - ws[62720];
      a = a - ws[62752];
      a = a - ws[62784];
      a = a - ws[62816];
      a = a - ws[62848];
      a = a - ws[62880];
      a = a - ws[62912];
      a = a - ws[62944];
      a = a - ws[62976];
      a = a - ws[63008];
      a = a - ws[63040];
      a = a - ws[63072];
      a = a - ws[63104];
      a = a - ws[63136];
      a = a - ws[63168];
      a = a - ws[63200];
      a = a - ws[63232];
      a = a - ws[63264];
      a = a - ws[63296];
      a = a - ws[63328];
      a = a - ws[63360];
      a = a - ws[63392];
      a = a - ws[63424];
      a = a - ws[63456];
      a = fma(0.35, ws[63456], a);
      a = a - ws[63488];
      a = fma(0.01, ws[63488], a);
      a = a - ws[63520];
      a = fma(0.01, ws[63520], a);
      a = a - ws[63552];
      a = fma(0.01, ws[63552], a);
      a = a - ws[63584];
      a = a - ws[63616];
      a = a - ws[63648];
      a = a - ws[63680];
      a = fma(0.35, ws[63680], a);
      a = a - ws[63712];
      a = a - ws[63744];
      a = a - ws[63776];
      a = a - ws[63808];
      a = a - ws[63840];
      a = a - ws[63872];
      a = fma(0.08, ws[63904], a);
      a = fma(0.22, ws[63936], a);
      a = fma(0.46, ws[63968], a);
      a = fma(0.6055, ws[64000], a);
      a = fma(0.66, ws[64032], a);
      a = fma(0.09, ws[64064], a);
      a = fma(0.19, ws[64128], a);
      a = fma(0.16, ws[64160], a);
      a = fma(0.1, ws[64192], a);
      a = fma(0.05, ws[64224], a);
      a = fma(0.05, ws[64256], a);
      a = fma(0.05, ws[64288], a);
      a = fma(0.82, ws[65536], a);
      a = fma(0.82, ws[65600], a);
      a = fma(0.77, ws[65664], a);
      a = fma(0.77, ws[65728], a);
      a = fma(0.238, ws[66848], a);
      a = fma(0.6195, ws[66912], a);
      a = fma(0.1, ws[66976], a);
      a = fma(0.5, ws[67040], a);
      a = fma(0.25, ws[67104], a);
      a = fma(0.1, ws[67136], a);
      a = fma(0.44, ws[67168], a);
      a = fma(0.44, ws[67200], a);
      a = fma(0.15, ws[67232], a);
      a = fma(0.5, ws[69312], a);
      a = fma(0.5, ws[69440], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71552], a);
      a = a - ws[71776];
      a = fma(1.0, ws[71776], a);
      a = a - ws[71808];
      a = a - ws[71840];
      a = a - ws[71872];
      a = fma(0.28, ws[71904], a);
      a = fma(0.204, ws[71968], a);
      a = a - ws[72000];
      a = fma(0.08, ws[72192], a);
      a = a - ws[72256];
      a = fma(0.4, ws[72320], a);
      a = a - ws[72352];
      a = fma(0.02, ws[72384], a);
      a = a - ws[72448];
      a = a - ws[72640];
      a = a - ws[73152];
      a = a - ws[73184];
      a = a - ws[73216];
      a = a - ws[73248];
      a = a - ws[73280];
      a = a - ws[73312];
      a = a - ws[73344];
      a = a - ws[74944];
      a = a - ws[75136];
      a = a - ws[75328];
      a = a - ws[75520];
      a = fma(1.0, ws[75520], a);
      a = a - ws[75552];
      a = fma(1.0, ws[75552], a);
      a = a - ws[75584];
      a = fma(1.0, ws[75584], a);
      a = a - ws[75616];
      a = fma(1.0, ws[75616], a);
      a = a - ws[75648];
      a = fma(1.0, ws[75648], a);
      a = a - ws[75680];
      a = fma(1.0, ws[75680], a);
      a = a - ws[75712];
      a = fma(1.0, ws[75712], a);
      a = a - ws[75744];
      a = fma(1.0, ws[75744], a);
      a = a - ws[75776];
      a = fma(1.0, ws[75776], a);
      a = a - ws[75808];
      a = fma(1.0, ws[75808], a);
      a = a - ws[75840];
      a = fma(1.0, ws[75840], a);
      a = a - ws[75872];
      a = fma(1.0, ws[75872], a);
      a = a - ws[75904];
      a = fma(1.0, ws[75904], a);
      a = a - ws[75936];
      a = fma(1.0, ws[75936], a);
      a = a - ws[75968];
      a = fma(1.0, ws[75968], a);
      a = a - ws[76000];
      a = fma(1.0, ws[76000], a);
      a = a - ws[76032];
      a = a - ws[76128];
      yout[6016] = a;
    }
}
// Partial-derivative products of 2- and 3-reactant reactions (rbjacob.F:112-143).
__device__ __noinline__ void explic_0(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    { const double kk = ws[43616]; ws[76320] = kk * y[6016]; ws[76352] = kk * y[5184]; }
    { const double kk = ws[43648]; ws[76384] = kk * y[5984]; ws[76416] = kk * y[5184]; }
    { const double kk = ws[43680]; ws[76448] = kk * y[5824]; ws[76480] = kk * y[5184]; }
    { const double kk = ws[43712]; ws[76512] = kk * y[5920]; ws[76544] = kk * y[5184]; }
    { const double kk = ws[43776]; ws[76576] = kk * y[5184]; ws[76608] = kk * y[2336]; }
    { const double kk = ws[43936]; ws[76640] = kk * y[5984]; ws[76672] = kk * y[6016]; }
    { const double kk = ws[43968]; ws[76704] = kk * y[5984]; ws[76736] = kk * y[5984]; }
    { const double kk = ws[44000]; ws[76768] = kk * y[5984]; ws[76800] = kk * y[5984]; }
    { const double kk = ws[44032]; ws[76832] = kk * y[6016]; ws[76864] = kk * y[4000]; }
    { const double kk = ws[44064]; ws[76896] = kk * y[2336]; ws[76928] = kk * y[5824]; }
    { const double kk = ws[44096]; ws[76960] = kk * y[6016]; ws[76992] = kk * y[5824]; }
    { const double kk = ws[44128]; ws[77024] = kk * y[5984]; ws[77056] = kk * y[5824]; }
    { const double kk = ws[44160]; ws[77088] = kk * y[5984]; ws[77120] = kk * y[5824]; }
    { const double kk = ws[44192]; ws[77152] = kk * y[5824]; ws[77184] = kk * y[5824]; }
    { const double kk = ws[44224]; ws[77216] = kk * y[6016]; ws[77248] = kk * y[1184]; }
    { const double kk = ws[44256]; ws[77280] = kk * y[2336]; ws[77312] = kk * y[5920]; }
    { const double kk = ws[44288]; ws[77344] = kk * y[2336]; ws[77376] = kk * y[5920]; }
    { const double kk = ws[44320]; ws[77408] = kk * y[6016]; ws[77440] = kk * y[5920]; }
    { const double kk = ws[44352]; ws[77472] = kk * y[6016]; ws[77504] = kk * y[5024]; }
    { const double kk = ws[44384]; ws[77536] = kk * y[6016]; ws[77568] = kk * y[5952]; }
    { const double kk = ws[44416]; ws[77600] = kk * y[5984]; ws[77632] = kk * y[5952]; }
    { const double kk = ws[44448]; ws[77664] = kk * y[5824]; ws[77696] = kk * y[5952]; }
    { const double kk = ws[44480]; ws[77728] = kk * y[5920]; ws[77760] = kk * y[5952]; }
    { const double kk = ws[44512]; ws[77792] = kk * y[5952]; ws[77824] = kk * y[5952]; }
    { const double kk = ws[44544]; ws[77856] = kk * y[5920]; ws[77888] = kk * y[5952]; }
    { const double kk = ws[44640]; ws[77920] = kk * y[5984]; ws[77952] = kk * y[5920]; }
    { const double kk = ws[44704]; ws[77984] = kk * y[6016]; ws[78016] = kk * y[1280]; }
    { const double kk = ws[44736]; ws[78048] = kk * y[6016]; ws[78080] = kk * y[160]; }
    { const double kk = ws[44768]; ws[78112] = kk * y[6016]; ws[78144] = kk * y[5664]; }
    { const double kk = ws[44832]; ws[78176] = kk * y[6016]; ws[78208] = kk * y[1888]; }
    { const double kk = ws[44864]; ws[78240] = kk * y[6016]; ws[78272] = kk * y[2176]; }
    { const double kk = ws[44896]; ws[78304] = kk * y[6016]; ws[78336] = kk * y[1120]; }
    { const double kk = ws[44928]; ws[78368] = kk * y[6016]; ws[78400] = kk * y[2240]; }
    { const double kk = ws[44960]; ws[78432] = kk * y[6016]; ws[78464] = kk * y[2752]; }
    { const double kk = ws[44992]; ws[78496] = kk * y[6016]; ws[78528] = kk * y[1152]; }
    { const double kk = ws[45024]; ws[78560] = kk * y[6016]; ws[78592] = kk * y[256]; }
    { const double kk = ws[45056]; ws[78624] = kk * y[6016]; ws[78656] = kk * y[1216]; }
    { const double kk = ws[45088]; ws[78688] = kk * y[6016]; ws[78720] = kk * y[288]; }
    { const double kk = ws[45120]; ws[78752] = kk * y[6016]; ws[78784] = kk * y[320]; }
    { const double kk = ws[45152]; ws[78816] = kk * y[6016]; ws[78848] = kk * y[352]; }
    { const double kk = ws[45184]; ws[78880] = kk * y[5184]; ws[78912] = kk * y[1312]; }
    { const double kk = ws[45216]; ws[78944] = kk * y[5952]; ws[78976] = kk * y[1312]; }
    { const double kk = ws[45248]; ws[79008] = kk * y[6016]; ws[79040] = kk * y[1312]; }
    { const double kk = ws[45280]; ws[79072] = kk * y[5984]; ws[79104] = kk * y[4288]; }
    { const double kk = ws[45312]; ws[79136] = kk * y[5824]; ws[79168] = kk * y[4288]; }
    { const double kk = ws[45344]; ws[79200] = kk * y[6016]; ws[79232] = kk * y[1344]; }
    { const double kk = ws[45376]; ws[79264] = kk * y[6016]; ws[79296] = kk * y[1344]; }
    { const double kk = ws[45408]; ws[79328] = kk * y[5984]; ws[79360] = kk * y[1632]; }
    { const double kk = ws[45440]; ws[79392] = kk * y[5824]; ws[79424] = kk * y[1632]; }
    { const double kk = ws[45472]; ws[79456] = kk * y[6016]; ws[79488] = kk * y[2784]; }
    { const double kk = ws[45504]; ws[79520] = kk * y[2208]; ws[79552] = kk * y[6016]; }
    { const double kk = ws[45568]; ws[79584] = kk * y[6016]; ws[79616] = kk * y[1664]; }
    { const double kk = ws[45600]; ws[79648] = kk * y[6016]; ws[79680] = kk * y[1408]; }
    { const double kk = ws[45632]; ws[79712] = kk * y[6016]; ws[79744] = kk * y[1440]; }
    { const double kk = ws[45664]; ws[79776] = kk * y[6016]; ws[79808] = kk * y[4544]; }
    { const double kk = ws[45696]; ws[79840] = kk * y[6016]; ws[79872] = kk * y[4576]; }
    { const double kk = ws[45728]; ws[79904] = kk * y[6016]; ws[79936] = kk * y[5856]; }
    { const double kk = ws[45760]; ws[79968] = kk * y[6016]; ws[80000] = kk * y[5568]; }
    { const double kk = ws[45792]; ws[80032] = kk * y[6016]; ws[80064] = kk * y[5760]; }
    { const double kk = ws[45824]; ws[80096] = kk * y[6016]; ws[80128] = kk * y[4480]; }
    { const double kk = ws[45856]; ws[80160] = kk * y[6016]; ws[80192] = kk * y[5280]; }
    { const double kk = ws[45888]; ws[80224] = kk * y[6016]; ws[80256] = kk * y[5504]; }
    { const double kk = ws[45920]; ws[80288] = kk * y[6016]; ws[80320] = kk * y[5344]; }
    { const double kk = ws[45952]; ws[80352] = kk * y[6016]; ws[80384] = kk * y[4128]; }
    { const double kk = ws[45984]; ws[80416] = kk * y[6016]; ws[80448] = kk * y[4736]; }
    { const double kk = ws[46016]; ws[80480] = kk * y[6016]; ws[80512] = kk * y[3872]; }
    { const double kk = ws[46048]; ws[80544] = kk * y[6016]; ws[80576] = kk * y[5376]; }
    { const double kk = ws[46080]; ws[80608] = kk * y[6016]; ws[80640] = kk * y[5248]; }
    { const double kk = ws[46112]; ws[80672] = kk * y[6016]; ws[80704] = kk * y[5472]; }
    { const double kk = ws[46144]; ws[80736] = kk * y[6016]; ws[80768] = kk * y[4320]; }
    { const double kk = ws[46176]; ws[80800] = kk * y[6016]; ws[80832] = kk * y[3584]; }
    { const double kk = ws[46208]; ws[80864] = kk * y[6016]; ws[80896] = kk * y[4448]; }
    { const double kk = ws[46240]; ws[80928] = kk * y[6016]; ws[80960] = kk * y[1248]; }
    { const double kk = ws[46272]; ws[80992] = kk * y[6016]; ws[81024] = kk * y[2944]; }
    { const double kk = ws[46304]; ws[81056] = kk * y[6016]; ws[81088] = kk * y[1760]; }
    { const double kk = ws[46336]; ws[81120] = kk * y[6016]; ws[81152] = kk * y[5600]; }
    { const double kk = ws[46368]; ws[81184] = kk * y[6016]; ws[81216] = kk * y[1472]; }
    { const double kk = ws[46400]; ws[81248] = kk * y[6016]; ws[81280] = kk * y[5056]; }
    { const double kk = ws[46432]; ws[81312] = kk * y[6016]; ws[81344] = kk * y[1504]; }
    { const double kk = ws[46464]; ws[81376] = kk * y[6016]; ws[81408] = kk * y[2816]; }
    { const double kk = ws[46496]; ws[81440] = kk * y[6016]; ws[81472] = kk * y[5728]; }
    { const double kk = ws[46528]; ws[81504] = kk * y[6016]; ws[81536] = kk * y[4096]; }
    { const double kk = ws[46560]; ws[81568] = kk * y[6016]; ws[81600] = kk * y[4608]; }
    { const double kk = ws[46592]; ws[81632] = kk * y[6016]; ws[81664] = kk * y[1792]; }
    { const double kk = ws[46624]; ws[81696] = kk * y[6016]; ws[81728] = kk * y[4352]; }
    { const double kk = ws[46656]; ws[81760] = kk * y[6016]; ws[81792] = kk * y[5696]; }
    { const double kk = ws[46688]; ws[81824] = kk * y[6016]; ws[81856] = kk * y[3680]; }
    { const double kk = ws[46720]; ws[81888] = kk * y[6016]; ws[81920] = kk * y[1088]; }
    { const double kk = ws[46752]; ws[81952] = kk * y[6016]; ws[81984] = kk * y[1536]; }
    { const double kk = ws[46784]; ws[82016] = kk * y[6016]; ws[82048] = kk * y[1824]; }
    { const double kk = ws[46816]; ws[82080] = kk * y[6016]; ws[82112] = kk * y[5440]; }
    { const double kk = ws[46848]; ws[82144] = kk * y[6016]; ws[82176] = kk * y[4384]; }
    { const double kk = ws[46880]; ws[82208] = kk * y[6016]; ws[82240] = kk * y[1696]; }
    { const double kk = ws[46912]; ws[82272] = kk * y[5184]; ws[82304] = kk * y[2240]; }
    { const double kk = ws[46944]; ws[82336] = kk * y[5184]; ws[82368] = kk * y[2752]; }
    { const double kk = ws[46976]; ws[82400] = kk * y[5184]; ws[82432] = kk * y[1152]; }
    { const double kk = ws[47008]; ws[82464] = kk * y[5184]; ws[82496] = kk * y[1408]; }
    { const double kk = ws[47040]; ws[82528] = kk * y[5184]; ws[82560] = kk * y[1440]; }
    { const double kk = ws[47072]; ws[82592] = kk * y[5184]; ws[82624] = kk * y[4576]; }
    { const double kk = ws[47104]; ws[82656] = kk * y[5184]; ws[82688] = kk * y[4384]; }
    { const double kk = ws[47136]; ws[82720] = kk * y[5184]; ws[82752] = kk * y[4128]; }
    { const double kk = ws[47168]; ws[82784] = kk * y[5184]; ws[82816] = kk * y[4736]; }
    { const double kk = ws[47200]; ws[82848] = kk * y[5184]; ws[82880] = kk * y[3872]; }
    { const double kk = ws[47232]; ws[82912] = kk * y[5184]; ws[82944] = kk * y[5472]; }
    { const double kk = ws[47264]; ws[82976] = kk * y[5184]; ws[83008] = kk * y[4320]; }
    { const double kk = ws[47296]; ws[83040] = kk * y[5184]; ws[83072] = kk * y[3584]; }
    { const double kk = ws[47328]; ws[83104] = kk * y[5184]; ws[83136] = kk * y[3808]; }
    { const double kk = ws[47360]; ws[83168] = kk * y[5952]; ws[83200] = kk * y[2240]; }
    { const double kk = ws[47392]; ws[83232] = kk * y[5952]; ws[83264] = kk * y[2752]; }
    { const double kk = ws[47424]; ws[83296] = kk * y[5952]; ws[83328] = kk * y[1152]; }
    { const double kk = ws[47456]; ws[83360] = kk * y[5952]; ws[83392] = kk * y[1408]; }
    { const double kk = ws[47488]; ws[83424] = kk * y[5952]; ws[83456] = kk * y[1440]; }
    { const double kk = ws[47520]; ws[83488] = kk * y[5952]; ws[83520] = kk * y[4384]; }
    { const double kk = ws[47552]; ws[83552] = kk * y[5952]; ws[83584] = kk * y[5856]; }
    { const double kk = ws[47584]; ws[83616] = kk * y[5952]; ws[83648] = kk * y[5568]; }
    { const double kk = ws[47616]; ws[83680] = kk * y[5952]; ws[83712] = kk * y[5760]; }
    { const double kk = ws[47648]; ws[83744] = kk * y[5952]; ws[83776] = kk * y[4128]; }
    { const double kk = ws[47680]; ws[83808] = kk * y[5952]; ws[83840] = kk * y[3872]; }
    { const double kk = ws[47712]; ws[83872] = kk * y[5952]; ws[83904] = kk * y[5376]; }
    { const double kk = ws[47744]; ws[83936] = kk * y[5952]; ws[83968] = kk * y[5248]; }
    { const double kk = ws[47776]; ws[84000] = kk * y[5952]; ws[84032] = kk * y[1248]; }
    { const double kk = ws[47808]; ws[84064] = kk * y[5952]; ws[84096] = kk * y[2944]; }
    { const double kk = ws[47840]; ws[84128] = kk * y[5952]; ws[84160] = kk * y[1760]; }
    { const double kk = ws[47872]; ws[84192] = kk * y[5952]; ws[84224] = kk * y[1824]; }
    { const double kk = ws[47968]; ws[84256] = kk * y[5920]; ws[84288] = kk * y[5792]; }
    { const double kk = ws[48032]; ws[84320] = kk * y[5920]; ws[84352] = kk * y[4800]; }
    { const double kk = ws[48096]; ws[84384] = kk * y[5920]; ws[84416] = kk * y[4672]; }
    { const double kk = ws[48160]; ws[84448] = kk * y[5824]; ws[84480] = kk * y[5888]; }
    { const double kk = ws[48192]; ws[84512] = kk * y[5824]; ws[84544] = kk * y[5632]; }
    { const double kk = ws[48224]; ws[84576] = kk * y[5824]; ws[84608] = kk * y[5408]; }
    { const double kk = ws[48256]; ws[84640] = kk * y[5824]; ws[84672] = kk * y[5120]; }
    { const double kk = ws[48288]; ws[84704] = kk * y[5824]; ws[84736] = kk * y[3008]; }
    { const double kk = ws[48320]; ws[84768] = kk * y[5824]; ws[84800] = kk * y[3200]; }
    { const double kk = ws[48352]; ws[84832] = kk * y[5824]; ws[84864] = kk * y[3328]; }
    { const double kk = ws[48384]; ws[84896] = kk * y[5824]; ws[84928] = kk * y[3360]; }
    { const double kk = ws[48416]; ws[84960] = kk * y[5824]; ws[84992] = kk * y[3296]; }
    { const double kk = ws[48448]; ws[85024] = kk * y[5824]; ws[85056] = kk * y[3104]; }
    { const double kk = ws[48480]; ws[85088] = kk * y[5824]; ws[85120] = kk * y[3264]; }
    { const double kk = ws[48512]; ws[85152] = kk * y[5824]; ws[85184] = kk * y[4160]; }
    { const double kk = ws[48544]; ws[85216] = kk * y[5824]; ws[85248] = kk * y[3744]; }
    { const double kk = ws[48576]; ws[85280] = kk * y[5824]; ws[85312] = kk * y[2624]; }
    { const double kk = ws[48608]; ws[85344] = kk * y[5824]; ws[85376] = kk * y[3840]; }
    { const double kk = ws[48640]; ws[85408] = kk * y[5824]; ws[85440] = kk * y[4192]; }
    { const double kk = ws[48672]; ws[85472] = kk * y[5824]; ws[85504] = kk * y[3936]; }
    { const double kk = ws[48704]; ws[85536] = kk * y[5824]; ws[85568] = kk * y[2656]; }
    { const double kk = ws[48736]; ws[85600] = kk * y[5824]; ws[85632] = kk * y[3712]; }
    { const double kk = ws[48768]; ws[85664] = kk * y[5824]; ws[85696] = kk * y[2560]; }
    { const double kk = ws[48800]; ws[85728] = kk * y[5824]; ws[85760] = kk * y[1728]; }
    { const double kk = ws[48832]; ws[85792] = kk * y[5824]; ws[85824] = kk * y[5792]; }
    { const double kk = ws[48864]; ws[85856] = kk * y[5824]; ws[85888] = kk * y[4800]; }
    { const double kk = ws[48896]; ws[85920] = kk * y[5824]; ws[85952] = kk * y[2848]; }
    { const double kk = ws[48928]; ws[85984] = kk * y[5824]; ws[86016] = kk * y[5152]; }
    { const double kk = ws[48960]; ws[86048] = kk * y[5824]; ws[86080] = kk * y[3776]; }
    { const double kk = ws[48992]; ws[86112] = kk * y[5824]; ws[86144] = kk * y[4672]; }
    { const double kk = ws[49024]; ws[86176] = kk * y[5824]; ws[86208] = kk * y[3520]; }
    { const double kk = ws[49056]; ws[86240] = kk * y[5824]; ws[86272] = kk * y[2880]; }
    { const double kk = ws[49088]; ws[86304] = kk * y[5824]; ws[86336] = kk * y[2912]; }
    { const double kk = ws[49120]; ws[86368] = kk * y[5824]; ws[86400] = kk * y[2592]; }
    { const double kk = ws[49152]; ws[86432] = kk * y[5824]; ws[86464] = kk * y[2272]; }
    { const double kk = ws[49184]; ws[86496] = kk * y[5824]; ws[86528] = kk * y[3648]; }
    { const double kk = ws[49216]; ws[86560] = kk * y[5824]; ws[86592] = kk * y[3040]; }
    { const double kk = ws[49248]; ws[86624] = kk * y[5824]; ws[86656] = kk * y[2976]; }
    { const double kk = ws[49280]; ws[86688] = kk * y[5824]; ws[86720] = kk * y[4032]; }
    { const double kk = ws[49312]; ws[86752] = kk * y[5824]; ws[86784] = kk * y[4064]; }
    { const double kk = ws[49344]; ws[86816] = kk * y[5824]; ws[86848] = kk * y[3072]; }
    { const double kk = ws[49376]; ws[86880] = kk * y[5824]; ws[86912] = kk * y[5216]; }
    { const double kk = ws[49408]; ws[86944] = kk * y[5920]; ws[86976] = kk * y[2688]; }
    { const double kk = ws[49440]; ws[87008] = kk * y[5920]; ws[87040] = kk * y[3232]; }
    { const double kk = ws[49472]; ws[87072] = kk * y[5920]; ws[87104] = kk * y[3808]; }
    { const double kk = ws[49504]; ws[87136] = kk * y[5984]; ws[87168] = kk * y[5888]; }
    { const double kk = ws[49536]; ws[87200] = kk * y[5984]; ws[87232] = kk * y[5632]; }
    { const double kk = ws[49568]; ws[87264] = kk * y[5984]; ws[87296] = kk * y[5408]; }
    { const double kk = ws[49600]; ws[87328] = kk * y[5984]; ws[87360] = kk * y[5120]; }
    { const double kk = ws[49632]; ws[87392] = kk * y[5984]; ws[87424] = kk * y[3008]; }
    { const double kk = ws[49664]; ws[87456] = kk * y[5984]; ws[87488] = kk * y[3200]; }
    { const double kk = ws[49696]; ws[87520] = kk * y[5984]; ws[87552] = kk * y[3328]; }
    { const double kk = ws[49728]; ws[87584] = kk * y[5984]; ws[87616] = kk * y[3360]; }
    { const double kk = ws[49760]; ws[87648] = kk * y[5984]; ws[87680] = kk * y[3296]; }
    { const double kk = ws[49792]; ws[87712] = kk * y[5984]; ws[87744] = kk * y[3104]; }
    { const double kk = ws[49824]; ws[87776] = kk * y[5984]; ws[87808] = kk * y[3264]; }
    { const double kk = ws[49856]; ws[87840] = kk * y[5984]; ws[87872] = kk * y[4160]; }
    { const double kk = ws[49888]; ws[87904] = kk * y[5984]; ws[87936] = kk * y[3744]; }
    { const double kk = ws[49920]; ws[87968] = kk * y[5984]; ws[88000] = kk * y[2624]; }
    { const double kk = ws[49952]; ws[88032] = kk * y[5984]; ws[88064] = kk * y[3840]; }
    { const double kk = ws[49984]; ws[88096] = kk * y[5984]; ws[88128] = kk * y[4192]; }
    { const double kk = ws[50016]; ws[88160] = kk * y[5984]; ws[88192] = kk * y[3936]; }
    { const double kk = ws[50048]; ws[88224] = kk * y[5984]; ws[88256] = kk * y[2656]; }
    { const double kk = ws[50080]; ws[88288] = kk * y[5984]; ws[88320] = kk * y[3712]; }
    { const double kk = ws[50112]; ws[88352] = kk * y[5984]; ws[88384] = kk * y[2560]; }
    { const double kk = ws[50144]; ws[88416] = kk * y[5984]; ws[88448] = kk * y[1728]; }
    { const double kk = ws[50176]; ws[88480] = kk * y[5984]; ws[88512] = kk * y[5792]; }
    { const double kk = ws[50208]; ws[88544] = kk * y[5984]; ws[88576] = kk * y[4800]; }
    { const double kk = ws[50240]; ws[88608] = kk * y[5984]; ws[88640] = kk * y[2848]; }
    { const double kk = ws[50272]; ws[88672] = kk * y[5984]; ws[88704] = kk * y[5152]; }
    { const double kk = ws[50304]; ws[88736] = kk * y[5984]; ws[88768] = kk * y[3776]; }
    { const double kk = ws[50336]; ws[88800] = kk * y[5984]; ws[88832] = kk * y[4672]; }
    { const double kk = ws[50368]; ws[88864] = kk * y[5984]; ws[88896] = kk * y[3520]; }
    { const double kk = ws[50400]; ws[88928] = kk * y[5984]; ws[88960] = kk * y[2880]; }
    { const double kk = ws[50432]; ws[88992] = kk * y[5984]; ws[89024] = kk * y[2912]; }
    { const double kk = ws[50464]; ws[89056] = kk * y[5984]; ws[89088] = kk * y[3648]; }
    { const double kk = ws[50496]; ws[89120] = kk * y[5984]; ws[89152] = kk * y[3232]; }
    { const double kk = ws[50528]; ws[89184] = kk * y[5984]; ws[89216] = kk * y[3040]; }
    { const double kk = ws[50560]; ws[89248] = kk * y[5984]; ws[89280] = kk * y[2976]; }
    { const double kk = ws[50592]; ws[89312] = kk * y[5984]; ws[89344] = kk * y[4032]; }
    { const double kk = ws[50624]; ws[89376] = kk * y[5984]; ws[89408] = kk * y[4064]; }
    { const double kk = ws[50656]; ws[89440] = kk * y[5984]; ws[89472] = kk * y[3072]; }
    { const double kk = ws[50688]; ws[89504] = kk * y[5984]; ws[89536] = kk * y[5216]; }
    { const double kk = ws[50720]; ws[89568] = kk * y[5888]; ws[89600] = kk * y[5888]; }
    { const double kk = ws[50752]; ws[89632] = kk * y[5888]; ws[89664] = kk * y[5632]; }
    { const double kk = ws[50784]; ws[89696] = kk * y[5888]; ws[89728] = kk * y[5408]; }
    { const double kk = ws[50816]; ws[89760] = kk * y[5888]; ws[89792] = kk * y[5120]; }
    { const double kk = ws[50848]; ws[89824] = kk * y[5888]; ws[89856] = kk * y[3008]; }
    { const double kk = ws[50880]; ws[89888] = kk * y[5888]; ws[89920] = kk * y[3200]; }
    { const double kk = ws[50912]; ws[89952] = kk * y[5888]; ws[89984] = kk * y[3328]; }
    { const double kk = ws[50944]; ws[90016] = kk * y[5888]; ws[90048] = kk * y[3360]; }
    { const double kk = ws[50976]; ws[90080] = kk * y[5888]; ws[90112] = kk * y[3296]; }
    { const double kk = ws[51008]; ws[90144] = kk * y[5888]; ws[90176] = kk * y[3104]; }
    { const double kk = ws[51040]; ws[90208] = kk * y[5888]; ws[90240] = kk * y[3264]; }
    { const double kk = ws[51072]; ws[90272] = kk * y[5888]; ws[90304] = kk * y[4288]; }
    { const double kk = ws[51104]; ws[90336] = kk * y[5888]; ws[90368] = kk * y[4160]; }
    { const double kk = ws[51136]; ws[90400] = kk * y[5888]; ws[90432] = kk * y[3744]; }
    { const double kk = ws[51168]; ws[90464] = kk * y[5888]; ws[90496] = kk * y[2624]; }
    { const double kk = ws[51200]; ws[90528] = kk * y[5888]; ws[90560] = kk * y[3840]; }
    { const double kk = ws[51232]; ws[90592] = kk * y[5888]; ws[90624] = kk * y[4192]; }
    { const double kk = ws[51264]; ws[90656] = kk * y[5888]; ws[90688] = kk * y[3936]; }
    { const double kk = ws[51296]; ws[90720] = kk * y[5888]; ws[90752] = kk * y[2656]; }
    { const double kk = ws[51328]; ws[90784] = kk * y[5888]; ws[90816] = kk * y[3712]; }
    { const double kk = ws[51360]; ws[90848] = kk * y[5888]; ws[90880] = kk * y[5792]; }
    { const double kk = ws[51392]; ws[90912] = kk * y[5888]; ws[90944] = kk * y[4800]; }
    { const double kk = ws[51424]; ws[90976] = kk * y[5888]; ws[91008] = kk * y[2848]; }
    { const double kk = ws[51456]; ws[91040] = kk * y[5888]; ws[91072] = kk * y[5152]; }
    { const double kk = ws[51488]; ws[91104] = kk * y[5888]; ws[91136] = kk * y[3776]; }
    { const double kk = ws[51520]; ws[91168] = kk * y[5888]; ws[91200] = kk * y[4672]; }
    { const double kk = ws[51552]; ws[91232] = kk * y[5888]; ws[91264] = kk * y[3520]; }
    { const double kk = ws[51584]; ws[91296] = kk * y[5888]; ws[91328] = kk * y[2880]; }
    { const double kk = ws[51616]; ws[91360] = kk * y[5888]; ws[91392] = kk * y[2912]; }
    { const double kk = ws[51648]; ws[91424] = kk * y[5888]; ws[91456] = kk * y[2592]; }
    { const double kk = ws[51680]; ws[91488] = kk * y[5888]; ws[91520] = kk * y[2272]; }
    { const double kk = ws[51712]; ws[91552] = kk * y[5888]; ws[91584] = kk * y[3648]; }
    { const double kk = ws[51744]; ws[91616] = kk * y[5888]; ws[91648] = kk * y[3040]; }
    { const double kk = ws[51776]; ws[91680] = kk * y[5888]; ws[91712] = kk * y[2976]; }
    { const double kk = ws[51808]; ws[91744] = kk * y[5888]; ws[91776] = kk * y[4032]; }
    { const double kk = ws[51840]; ws[91808] = kk * y[5888]; ws[91840] = kk * y[4064]; }
    { const double kk = ws[51872]; ws[91872] = kk * y[5888]; ws[91904] = kk * y[3072]; }
    { const double kk = ws[51904]; ws[91936] = kk * y[5888]; ws[91968] = kk * y[5216]; }
    { const double kk = ws[51936]; ws[92000] = kk * y[5792]; ws[92032] = kk * y[5632]; }
    { const double kk = ws[51968]; ws[92064] = kk * y[5792]; ws[92096] = kk * y[5408]; }
    { const double kk = ws[52000]; ws[92128] = kk * y[5792]; ws[92160] = kk * y[5120]; }
    { const double kk = ws[52032]; ws[92192] = kk * y[5792]; ws[92224] = kk * y[3008]; }
    { const double kk = ws[52064]; ws[92256] = kk * y[5792]; ws[92288] = kk * y[3200]; }
    { const double kk = ws[52096]; ws[92320] = kk * y[5792]; ws[92352] = kk * y[3328]; }
    { const double kk = ws[52128]; ws[92384] = kk * y[5792]; ws[92416] = kk * y[3360]; }
    { const double kk = ws[52160]; ws[92448] = kk * y[5792]; ws[92480] = kk * y[3296]; }
    { const double kk = ws[52192]; ws[92512] = kk * y[5792]; ws[92544] = kk * y[3104]; }
    { const double kk = ws[52224]; ws[92576] = kk * y[5792]; ws[92608] = kk * y[3264]; }
    { const double kk = ws[52256]; ws[92640] = kk * y[5792]; ws[92672] = kk * y[4288]; }
    { const double kk = ws[52288]; ws[92704] = kk * y[5792]; ws[92736] = kk * y[4160]; }
    { const double kk = ws[52320]; ws[92768] = kk * y[5792]; ws[92800] = kk * y[3744]; }
    { const double kk = ws[52352]; ws[92832] = kk * y[5792]; ws[92864] = kk * y[2624]; }
    { const double kk = ws[52384]; ws[92896] = kk * y[5792]; ws[92928] = kk * y[3840]; }
    { const double kk = ws[52416]; ws[92960] = kk * y[5792]; ws[92992] = kk * y[4192]; }
    { const double kk = ws[52448]; ws[93024] = kk * y[5792]; ws[93056] = kk * y[3936]; }
    { const double kk = ws[52480]; ws[93088] = kk * y[5792]; ws[93120] = kk * y[2656]; }
    { const double kk = ws[52512]; ws[93152] = kk * y[5792]; ws[93184] = kk * y[3712]; }
    { const double kk = ws[52544]; ws[93216] = kk * y[5792]; ws[93248] = kk * y[5792]; }
    { const double kk = ws[52576]; ws[93280] = kk * y[5792]; ws[93312] = kk * y[4800]; }
    { const double kk = ws[52608]; ws[93344] = kk * y[5792]; ws[93376] = kk * y[2848]; }
    { const double kk = ws[52640]; ws[93408] = kk * y[5792]; ws[93440] = kk * y[5152]; }
    { const double kk = ws[52672]; ws[93472] = kk * y[5792]; ws[93504] = kk * y[3776]; }
    { const double kk = ws[52704]; ws[93536] = kk * y[5792]; ws[93568] = kk * y[4672]; }
    { const double kk = ws[52736]; ws[93600] = kk * y[5792]; ws[93632] = kk * y[3520]; }
    { const double kk = ws[52768]; ws[93664] = kk * y[5792]; ws[93696] = kk * y[2880]; }
    { const double kk = ws[52800]; ws[93728] = kk * y[5792]; ws[93760] = kk * y[2912]; }
    { const double kk = ws[52832]; ws[93792] = kk * y[5792]; ws[93824] = kk * y[2592]; }
    { const double kk = ws[52864]; ws[93856] = kk * y[5792]; ws[93888] = kk * y[2272]; }
    { const double kk = ws[52896]; ws[93920] = kk * y[5792]; ws[93952] = kk * y[3648]; }
    { const double kk = ws[52928]; ws[93984] = kk * y[5792]; ws[94016] = kk * y[3040]; }
    { const double kk = ws[52960]; ws[94048] = kk * y[5792]; ws[94080] = kk * y[2976]; }
    { const double kk = ws[52992]; ws[94112] = kk * y[5792]; ws[94144] = kk * y[4032]; }
    { const double kk = ws[53024]; ws[94176] = kk * y[5792]; ws[94208] = kk * y[4064]; }
    { const double kk = ws[53056]; ws[94240] = kk * y[5792]; ws[94272] = kk * y[3072]; }
    { const double kk = ws[53088]; ws[94304] = kk * y[5792]; ws[94336] = kk * y[5216]; }
    { const double kk = ws[53120]; ws[94368] = kk * y[4800]; ws[94400] = kk * y[4800]; }
    { const double kk = ws[53152]; ws[94432] = kk * y[5952]; ws[94464] = kk * y[5888]; }
    { const double kk = ws[53184]; ws[94496] = kk * y[5952]; ws[94528] = kk * y[5632]; }
    { const double kk = ws[53216]; ws[94560] = kk * y[5952]; ws[94592] = kk * y[5408]; }
    { const double kk = ws[53248]; ws[94624] = kk * y[5952]; ws[94656] = kk * y[5120]; }
    { const double kk = ws[53280]; ws[94688] = kk * y[5952]; ws[94720] = kk * y[3008]; }
    { const double kk = ws[53312]; ws[94752] = kk * y[5952]; ws[94784] = kk * y[3200]; }
    { const double kk = ws[53344]; ws[94816] = kk * y[5952]; ws[94848] = kk * y[3328]; }
    { const double kk = ws[53376]; ws[94880] = kk * y[5952]; ws[94912] = kk * y[3360]; }
    { const double kk = ws[53408]; ws[94944] = kk * y[5952]; ws[94976] = kk * y[3296]; }
    { const double kk = ws[53440]; ws[95008] = kk * y[5952]; ws[95040] = kk * y[3104]; }
    { const double kk = ws[53472]; ws[95072] = kk * y[5952]; ws[95104] = kk * y[3264]; }
    { const double kk = ws[53504]; ws[95136] = kk * y[5952]; ws[95168] = kk * y[4288]; }
    { const double kk = ws[53536]; ws[95200] = kk * y[5952]; ws[95232] = kk * y[4160]; }
    { const double kk = ws[53568]; ws[95264] = kk * y[5952]; ws[95296] = kk * y[4192]; }
    { const double kk = ws[53600]; ws[95328] = kk * y[5952]; ws[95360] = kk * y[2624]; }
    { const double kk = ws[53632]; ws[95392] = kk * y[5952]; ws[95424] = kk * y[2656]; }
    { const double kk = ws[53664]; ws[95456] = kk * y[5952]; ws[95488] = kk * y[5792]; }
    { const double kk = ws[53696]; ws[95520] = kk * y[5952]; ws[95552] = kk * y[4800]; }
    { const double kk = ws[53728]; ws[95584] = kk * y[5952]; ws[95616] = kk * y[2848]; }
    { const double kk = ws[53760]; ws[95648] = kk * y[5952]; ws[95680] = kk * y[5152]; }
    { const double kk = ws[53792]; ws[95712] = kk * y[5952]; ws[95744] = kk * y[3776]; }
    { const double kk = ws[53824]; ws[95776] = kk * y[5952]; ws[95808] = kk * y[4672]; }
    { const double kk = ws[53856]; ws[95840] = kk * y[5952]; ws[95872] = kk * y[3520]; }
    { const double kk = ws[53888]; ws[95904] = kk * y[5952]; ws[95936] = kk * y[2880]; }
    { const double kk = ws[53920]; ws[95968] = kk * y[5952]; ws[96000] = kk * y[2912]; }
    { const double kk = ws[53952]; ws[96032] = kk * y[5952]; ws[96064] = kk * y[2592]; }
    { const double kk = ws[53984]; ws[96096] = kk * y[5952]; ws[96128] = kk * y[2272]; }
    { const double kk = ws[54016]; ws[96160] = kk * y[5952]; ws[96192] = kk * y[3648]; }
    { const double kk = ws[54048]; ws[96224] = kk * y[5952]; ws[96256] = kk * y[3040]; }
    { const double kk = ws[54080]; ws[96288] = kk * y[5952]; ws[96320] = kk * y[2976]; }
    { const double kk = ws[54112]; ws[96352] = kk * y[5952]; ws[96384] = kk * y[4032]; }
    { const double kk = ws[54144]; ws[96416] = kk * y[5952]; ws[96448] = kk * y[4064]; }
    { const double kk = ws[54176]; ws[96480] = kk * y[5952]; ws[96512] = kk * y[3072]; }
    { const double kk = ws[54208]; ws[96544] = kk * y[4032]; ws[96576] = kk * y[4032]; }
    { const double kk = ws[54240]; ws[96608] = kk * y[4064]; ws[96640] = kk * y[4032]; }
    { const double kk = ws[54272]; ws[96672] = kk * y[4064]; ws[96704] = kk * y[4064]; }
    { const double kk = ws[54304]; ws[96736] = kk * y[5952]; ws[96768] = kk * y[5216]; }
    { const double kk = ws[54336]; ws[96800] = kk * y[4800]; ws[96832] = kk * y[5216]; }
    { const double kk = ws[54368]; ws[96864] = kk * y[5216]; ws[96896] = kk * y[5216]; }
    { const double kk = ws[54400]; ws[96928] = kk * y[4160]; ws[96960] = kk * y[3744]; }
    { const double kk = ws[54432]; ws[96992] = kk * y[4192]; ws[97024] = kk * y[3744]; }
    { const double kk = ws[54464]; ws[97056] = kk * y[4288]; ws[97088] = kk * y[3744]; }
    { const double kk = ws[54496]; ws[97120] = kk * y[4160]; ws[97152] = kk * y[3936]; }
    { const double kk = ws[54528]; ws[97184] = kk * y[4192]; ws[97216] = kk * y[3936]; }
    { const double kk = ws[54560]; ws[97248] = kk * y[4288]; ws[97280] = kk * y[3936]; }
    { const double kk = ws[54592]; ws[97312] = kk * y[4160]; ws[97344] = kk * y[3840]; }
    { const double kk = ws[54624]; ws[97376] = kk * y[4192]; ws[97408] = kk * y[3840]; }
    { const double kk = ws[54656]; ws[97440] = kk * y[4288]; ws[97472] = kk * y[3840]; }
    { const double kk = ws[54688]; ws[97504] = kk * y[4160]; ws[97536] = kk * y[3712]; }
    { const double kk = ws[54720]; ws[97568] = kk * y[4192]; ws[97600] = kk * y[3712]; }
    { const double kk = ws[54752]; ws[97632] = kk * y[4288]; ws[97664] = kk * y[3712]; }
    { const double kk = ws[54784]; ws[97696] = kk * y[6016]; ws[97728] = kk * y[1376]; }
    { const double kk = ws[54816]; ws[97760] = kk * y[6016]; ws[97792] = kk * y[384]; }
    { const double kk = ws[54848]; ws[97824] = kk * y[6016]; ws[97856] = kk * y[416]; }
    { const double kk = ws[54880]; ws[97888] = kk * y[6016]; ws[97920] = kk * y[3552]; }
    { const double kk = ws[54912]; ws[97952] = kk * y[5184]; ws[97984] = kk * y[3552]; }
    { const double kk = ws[54944]; ws[98016] = kk * y[5952]; ws[98048] = kk * y[3552]; }
    { const double kk = ws[55008]; ws[98080] = kk * y[6016]; ws[98112] = kk * y[1568]; }
    { const double kk = ws[55040]; ws[98144] = kk * y[5824]; ws[98176] = kk * y[3136]; }
    { const double kk = ws[55072]; ws[98208] = kk * y[5952]; ws[98240] = kk * y[3136]; }
    { const double kk = ws[55104]; ws[98272] = kk * y[5984]; ws[98304] = kk * y[3136]; }
    { const double kk = ws[55136]; ws[98336] = kk * y[5888]; ws[98368] = kk * y[3136]; }
    { const double kk = ws[55168]; ws[98400] = kk * y[5792]; ws[98432] = kk * y[3136]; }
    { const double kk = ws[55200]; ws[98464] = kk * y[5184]; ws[98496] = kk * y[1568]; }
    { const double kk = ws[55232]; ws[98528] = kk * y[5952]; ws[98560] = kk * y[1568]; }
    { const double kk = ws[55264]; ws[98592] = kk * y[6016]; ws[98624] = kk * y[3168]; }
    { const double kk = ws[55296]; ws[98656] = kk * y[5824]; ws[98688] = kk * y[1856]; }
    { const double kk = ws[55328]; ws[98720] = kk * y[5984]; ws[98752] = kk * y[1856]; }
    { const double kk = ws[55360]; ws[98784] = kk * y[6016]; ws[98816] = kk * y[4512]; }
    { const double kk = ws[55392]; ws[98848] = kk * y[5184]; ws[98880] = kk * y[3168]; }
    { const double kk = ws[55424]; ws[98912] = kk * y[5952]; ws[98944] = kk * y[3168]; }
    { const double kk = ws[55456]; ws[98976] = kk * y[6016]; ws[99008] = kk * y[448]; }
    { const double kk = ws[55488]; ws[99040] = kk * y[5952]; ws[99072] = kk * y[1600]; }
    { const double kk = ws[55520]; ws[99104] = kk * y[5984]; ws[99136] = kk * y[1920]; }
    { const double kk = ws[55552]; ws[99168] = kk * y[5824]; ws[99200] = kk * y[1920]; }
    { const double kk = ws[55584]; ws[99232] = kk * y[5952]; ws[99264] = kk * y[1920]; }
    { const double kk = ws[55616]; ws[99296] = kk * y[5184]; ws[99328] = kk * y[1600]; }
    { const double kk = ws[55648]; ws[99360] = kk * y[6016]; ws[99392] = kk * y[1600]; }
    { const double kk = ws[55680]; ws[99424] = kk * y[5984]; ws[99456] = kk * y[2304]; }
    { const double kk = ws[55712]; ws[99488] = kk * y[5952]; ws[99520] = kk * y[2304]; }
    { const double kk = ws[55744]; ws[99552] = kk * y[5824]; ws[99584] = kk * y[2304]; }
    { const double kk = ws[56064]; ws[99616] = kk * y[512]; ws[99648] = kk * y[1056]; }
    { const double kk = ws[56160]; ws[99680] = kk * y[6016]; ws[99712] = kk * y[608]; }
    { const double kk = ws[56192]; ws[99744] = kk * y[6016]; ws[99776] = kk * y[640]; }
    { const double kk = ws[56224]; ws[99808] = kk * y[6016]; ws[99840] = kk * y[672]; }
    { const double kk = ws[56256]; ws[99872] = kk * y[6016]; ws[99904] = kk * y[704]; }
    { const double kk = ws[56288]; ws[99936] = kk * y[6016]; ws[99968] = kk * y[736]; }
    { const double kk = ws[56320]; ws[100000] = kk * y[6016]; ws[100032] = kk * y[768]; }
    { const double kk = ws[56352]; ws[100064] = kk * y[6016]; ws[100096] = kk * y[800]; }
    { const double kk = ws[56384]; ws[100128] = kk * y[5824]; ws[100160] = kk * y[2368]; }
    { const double kk = ws[56416]; ws[100192] = kk * y[5824]; ws[100224] = kk * y[2400]; }
    { const double kk = ws[56448]; ws[100256] = kk * y[5824]; ws[100288] = kk * y[2432]; }
    { const double kk = ws[56480]; ws[100320] = kk * y[5824]; ws[100352] = kk * y[2464]; }
    { const double kk = ws[56512]; ws[100384] = kk * y[5824]; ws[100416] = kk * y[2496]; }
    { const double kk = ws[56544]; ws[100448] = kk * y[5824]; ws[100480] = kk * y[2528]; }
    { const double kk = ws[56576]; ws[100512] = kk * y[5824]; ws[100544] = kk * y[3904]; }
    { const double kk = ws[56608]; ws[100576] = kk * y[5952]; ws[100608] = kk * y[2368]; }
    { const double kk = ws[56640]; ws[100640] = kk * y[5952]; ws[100672] = kk * y[2400]; }
    { const double kk = ws[56672]; ws[100704] = kk * y[5952]; ws[100736] = kk * y[2432]; }
    { const double kk = ws[56704]; ws[100768] = kk * y[5952]; ws[100800] = kk * y[2464]; }
    { const double kk = ws[56736]; ws[100832] = kk * y[5952]; ws[100864] = kk * y[2496]; }
    { const double kk = ws[56768]; ws[100896] = kk * y[5952]; ws[100928] = kk * y[2528]; }
    { const double kk = ws[56800]; ws[100960] = kk * y[5952]; ws[100992] = kk * y[3904]; }
    { const double kk = ws[56832]; ws[101024] = kk * y[5984]; ws[101056] = kk * y[2368]; }
    { const double kk = ws[56864]; ws[101088] = kk * y[5984]; ws[101120] = kk * y[2400]; }
    { const double kk = ws[56896]; ws[101152] = kk * y[5984]; ws[101184] = kk * y[2432]; }
    { const double kk = ws[56928]; ws[101216] = kk * y[5984]; ws[101248] = kk * y[2464]; }
    { const double kk = ws[56960]; ws[101280] = kk * y[5984]; ws[101312] = kk * y[2496]; }
    { const double kk = ws[56992]; ws[101344] = kk * y[5984]; ws[101376] = kk * y[2528]; }
    { const double kk = ws[57024]; ws[101408] = kk * y[5984]; ws[101440] = kk * y[3904]; }
    { const double kk = ws[57280]; ws[101472] = kk * y[5824]; ws[101504] = kk * y[1952]; }
    { const double kk = ws[57312]; ws[101536] = kk * y[5824]; ws[101568] = kk * y[1984]; }
    { const double kk = ws[57344]; ws[101600] = kk * y[5824]; ws[101632] = kk * y[2016]; }
    { const double kk = ws[57376]; ws[101664] = kk * y[5824]; ws[101696] = kk * y[2048]; }
    { const double kk = ws[57408]; ws[101728] = kk * y[5824]; ws[101760] = kk * y[2080]; }
    { const double kk = ws[57440]; ws[101792] = kk * y[5824]; ws[101824] = kk * y[2112]; }
    { const double kk = ws[57472]; ws[101856] = kk * y[5824]; ws[101888] = kk * y[2144]; }
    { const double kk = ws[57504]; ws[101920] = kk * y[5952]; ws[101952] = kk * y[1952]; }
    { const double kk = ws[57536]; ws[101984] = kk * y[5952]; ws[102016] = kk * y[1984]; }
    { const double kk = ws[57568]; ws[102048] = kk * y[5952]; ws[102080] = kk * y[2016]; }
    { const double kk = ws[57600]; ws[102112] = kk * y[5952]; ws[102144] = kk * y[2048]; }
    { const double kk = ws[57632]; ws[102176] = kk * y[5952]; ws[102208] = kk * y[2080]; }
    { const double kk = ws[57664]; ws[102240] = kk * y[5952]; ws[102272] = kk * y[2112]; }
    { const double kk = ws[57696]; ws[102304] = kk * y[5952]; ws[102336] = kk * y[2144]; }
    { const double kk = ws[57728]; ws[102368] = kk * y[5984]; ws[102400] = kk * y[1952]; }
    { const double kk = ws[57760]; ws[102432] = kk * y[5984]; ws[102464] = kk * y[1984]; }
    { const double kk = ws[57792]; ws[102496] = kk * y[5984]; ws[102528] = kk * y[2016]; }
    { const double kk = ws[57824]; ws[102560] = kk * y[5984]; ws[102592] = kk * y[2048]; }
    { const double kk = ws[57856]; ws[102624] = kk * y[5984]; ws[102656] = kk * y[2080]; }
    { const double kk = ws[57888]; ws[102688] = kk * y[5984]; ws[102720] = kk * y[2112]; }
    { const double kk = ws[57920]; ws[102752] = kk * y[5984]; ws[102784] = kk * y[2144]; }
    { const double kk = ws[57952]; ws[102816] = kk * y[6016]; ws[102848] = kk * y[832]; }
    { const double kk = ws[57984]; ws[102880] = kk * y[5984]; ws[102912] = kk * y[3392]; }
    { const double kk = ws[58016]; ws[102944] = kk * y[5824]; ws[102976] = kk * y[3392]; }
    { const double kk = ws[58048]; ws[103008] = kk * y[5952]; ws[103040] = kk * y[3392]; }
    { const double kk = ws[58080]; ws[103072] = kk * y[5888]; ws[103104] = kk * y[3392]; }
    { const double kk = ws[58112]; ws[103136] = kk * y[5792]; ws[103168] = kk * y[3392]; }
    { const double kk = ws[58144]; ws[103200] = kk * y[6016]; ws[103232] = kk * y[864]; }
    { const double kk = ws[58176]; ws[103264] = kk * y[5984]; ws[103296] = kk * y[3424]; }
    { const double kk = ws[58208]; ws[103328] = kk * y[5824]; ws[103360] = kk * y[3424]; }
    { const double kk = ws[58240]; ws[103392] = kk * y[5952]; ws[103424] = kk * y[3424]; }
    { const double kk = ws[58272]; ws[103456] = kk * y[5888]; ws[103488] = kk * y[3424]; }
    { const double kk = ws[58304]; ws[103520] = kk * y[5792]; ws[103552] = kk * y[3424]; }
    { const double kk = ws[58336]; ws[103584] = kk * y[6016]; ws[103616] = kk * y[896]; }
    { const double kk = ws[58368]; ws[103648] = kk * y[5984]; ws[103680] = kk * y[3456]; }
    { const double kk = ws[58400]; ws[103712] = kk * y[5824]; ws[103744] = kk * y[3456]; }
    { const double kk = ws[58432]; ws[103776] = kk * y[5952]; ws[103808] = kk * y[3456]; }
    { const double kk = ws[58464]; ws[103840] = kk * y[5888]; ws[103872] = kk * y[3456]; }
    { const double kk = ws[58496]; ws[103904] = kk * y[5792]; ws[103936] = kk * y[3456]; }
    { const double kk = ws[58528]; ws[103968] = kk * y[6016]; ws[104000] = kk * y[4768]; }
    { const double kk = ws[58560]; ws[104032] = kk * y[6016]; ws[104064] = kk * y[4864]; }
    { const double kk = ws[58592]; ws[104096] = kk * y[6016]; ws[104128] = kk * y[4832]; }
    { const double kk = ws[58624]; ws[104160] = kk * y[6016]; ws[104192] = kk * y[4896]; }
    { const double kk = ws[58656]; ws[104224] = kk * y[6016]; ws[104256] = kk * y[4640]; }
    { const double kk = ws[58688]; ws[104288] = kk * y[6016]; ws[104320] = kk * y[4416]; }
    { const double kk = ws[58720]; ws[104352] = kk * y[6016]; ws[104384] = kk * y[4928]; }
    { const double kk = ws[58752]; ws[104416] = kk * y[6016]; ws[104448] = kk * y[4960]; }
    { const double kk = ws[58784]; ws[104480] = kk * y[6016]; ws[104512] = kk * y[4992]; }
    { const double kk = ws[58816]; ws[104544] = kk * y[6016]; ws[104576] = kk * y[4704]; }
    { const double kk = ws[58848]; ws[104608] = kk * y[6016]; ws[104640] = kk * y[5088]; }
    { const double kk = ws[58880]; ws[104672] = kk * y[6016]; ws[104704] = kk * y[5536]; }
    { const double kk = ws[58912]; ws[104736] = kk * y[6016]; ws[104768] = kk * y[5312]; }
    { const double kk = ws[58944]; ws[104800] = kk * y[6016]; ws[104832] = kk * y[4224]; }
    { const double kk = ws[58976]; ws[104864] = kk * y[6016]; ws[104896] = kk * y[3968]; }
    { const double kk = ws[59008]; ws[104928] = kk * y[6016]; ws[104960] = kk * y[4608]; }
    { const double kk = ws[59040]; ws[104992] = kk * y[6016]; ws[105024] = kk * y[928]; }
    { const double kk = ws[59136]; ws[105056] = kk * y[6016]; ws[105088] = kk * y[992]; }
    { const double kk = ws[59168]; ws[105120] = kk * y[5984]; ws[105152] = kk * y[3488]; }
    { const double kk = ws[59200]; ws[105184] = kk * y[5824]; ws[105216] = kk * y[3488]; }
    { const double kk = ws[59232]; ws[105248] = kk * y[5952]; ws[105280] = kk * y[3488]; }
    { const double kk = ws[59264]; ws[105312] = kk * y[5888]; ws[105344] = kk * y[3488]; }
    { const double kk = ws[59296]; ws[105376] = kk * y[5792]; ws[105408] = kk * y[3488]; }
}
// f(y) for the night reaction list (rbfeval.F:80-151).
__device__ __noinline__ void feval_1(double* __restrict__ ws, int src, int dst)
{
    const double* __restrict__ yin = ws + src * 32;
    double* __restrict__ yout = ws + dst * 32;
    ws[60608] = ((ws[43616]) * yin[5184]) * yin[6016];
    ws[60640] = ((ws[43648]) * yin[5184]) * yin[5984];
    ws[60672] = ((ws[43680]) * yin[5184]) * yin[5824];
    ws[60704] = ((ws[43712]) * yin[5184]) * yin[5920];
    ws[60736] = (ws[43744]) * yin[2336];
    ws[60768] = ((ws[43776]) * yin[2336]) * yin[5184];
    ws[60800] = (ws[43808]) * yin[576];
    ws[60832] = (ws[43840]) * yin[576];
    ws[60864] = (ws[43872]) * yin[576];
    ws[60896] = (ws[43904]) * yin[6016];
    ws[60928] = ((ws[43936]) * yin[6016]) * yin[5984];
    ws[60960] = ((ws[43968]) * yin[5984]) * yin[5984];
    ws[60992] = ((ws[44000]) * yin[5984]) * yin[5984];
    ws[61024] = ((ws[44032]) * yin[4000]) * yin[6016];
    ws[61056] = ((ws[44064]) * yin[5824]) * yin[2336];
    ws[61088] = ((ws[44096]) * yin[5824]) * yin[6016];
    ws[61120] = ((ws[44128]) * yin[5824]) * yin[5984];
    ws[61152] = ((ws[44160]) * yin[5824]) * yin[5984];
    ws[61184] = ((ws[44192]) * yin[5824]) * yin[5824];
    ws[61216] = ((ws[44224]) * yin[1184]) * yin[6016];
    ws[61248] = ((ws[44256]) * yin[5920]) * yin[2336];
    ws[61280] = ((ws[44288]) * yin[5920]) * yin[2336];
    ws[61312] = ((ws[44320]) * yin[5920]) * yin[6016];
    ws[61344] = ((ws[44352]) * yin[5024]) * yin[6016];
    ws[61376] = ((ws[44384]) * yin[5952]) * yin[6016];
    ws[61408] = ((ws[44416]) * yin[5952]) * yin[5984];
    ws[61440] = ((ws[44448]) * yin[5952]) * yin[5824];
    ws[61472] = ((ws[44480]) * yin[5952]) * yin[5920];
    ws[61504] = ((ws[44512]) * yin[5952]) * yin[5952];
    ws[61536] = ((ws[44544]) * yin[5952]) * yin[5920];
    ws[61568] = (ws[44576]) * yin[1024];
    ws[61600] = (ws[44608]) * yin[1024];
    ws[61632] = ((ws[44640]) * yin[5920]) * yin[5984];
    ws[61664] = (ws[44672]) * yin[1280];
    ws[61696] = ((ws[44704]) * yin[1280]) * yin[6016];
    ws[61728] = ((ws[44736]) * yin[160]) * yin[6016];
    ws[61760] = ((ws[44768]) * yin[5664]) * yin[6016];
    ws[61792] = (ws[44800]) * yin[6016];
    ws[61824] = ((ws[44832]) * yin[1888]) * yin[6016];
    ws[61856] = ((ws[44864]) * yin[2176]) * yin[6016];
    ws[61888] = ((ws[44896]) * yin[1120]) * yin[6016];
    ws[61920] = ((ws[44928]) * yin[2240]) * yin[6016];
    ws[61952] = ((ws[44960]) * yin[2752]) * yin[6016];
    ws[61984] = ((ws[44992]) * yin[1152]) * yin[6016];
    ws[62016] = ((ws[45024]) * yin[256]) * yin[6016];
    ws[62048] = ((ws[45056]) * yin[1216]) * yin[6016];
    ws[62080] = ((ws[45088]) * yin[288]) * yin[6016];
    ws[62112] = ((ws[45120]) * yin[320]) * yin[6016];
    ws[62144] = ((ws[45152]) * yin[352]) * yin[6016];
    ws[62176] = ((ws[45184]) * yin[1312]) * yin[5184];
    ws[62208] = ((ws[45216]) * yin[1312]) * yin[5952];
    ws[62240] = ((ws[45248]) * yin[1312]) * yin[6016];
    ws[62272] = ((ws[45280]) * yin[4288]) * yin[5984];
    ws[62304] = ((ws[45312]) * yin[4288]) * yin[5824];
    ws[62336] = ((ws[45344]) * yin[1344]) * yin[6016];
    ws[62368] = ((ws[45376]) * yin[1344]) * yin[6016];
    ws[62400] = ((ws[45408]) * yin[1632]) * yin[5984];
    ws[62432] = ((ws[45440]) * yin[1632]) * yin[5824];
    ws[62464] = ((ws[45472]) * yin[2784]) * yin[6016];
    ws[62496] = ((ws[45504]) * yin[6016]) * yin[2208];
    ws[62528] = (ws[45536]) * yin[2784];
    ws[62560] = ((ws[45568]) * yin[1664]) * yin[6016];
    ws[62592] = ((ws[45600]) * yin[1408]) * yin[6016];
    ws[62624] = ((ws[45632]) * yin[1440]) * yin[6016];
    ws[62656] = ((ws[45664]) * yin[4544]) * yin[6016];
    ws[62688] = ((ws[45696]) * yin[4576]) * yin[6016];
    ws[62720] = ((ws[45728]) * yin[5856]) * yin[6016];
    ws[62752] = ((ws[45760]) * yin[5568]) * yin[6016];
    ws[62784] = ((ws[45792]) * yin[5760]) * yin[6016];
    ws[62816] = ((ws[45824]) * yin[4480]) * yin[6016];
    ws[62848] = ((ws[45856]) * yin[5280]) * yin[6016];
    ws[62880] = ((ws[45888]) * yin[5504]) * yin[6016];
    ws[62912] = ((ws[45920]) * yin[5344]) * yin[6016];
    ws[62944] = ((ws[45952]) * yin[4128]) * yin[6016];
    ws[62976] = ((ws[45984]) * yin[4736]) * yin[6016];
    ws[63008] = ((ws[46016]) * yin[3872]) * yin[6016];
    ws[63040] = ((ws[46048]) * yin[5376]) * yin[6016];
    ws[63072] = ((ws[46080]) * yin[5248]) * yin[6016];
    ws[63104] = ((ws[46112]) * yin[5472]) * yin[6016];
    ws[63136] = ((ws[46144]) * yin[4320]) * yin[6016];
    ws[63168] = ((ws[46176]) * yin[3584]) * yin[6016];
    ws[63200] = ((ws[46208]) * yin[4448]) * yin[6016];
    ws[63232] = ((ws[46240]) * yin[1248]) * yin[6016];
    ws[63264] = ((ws[46272]) * yin[2944]) * yin[6016];
    ws[63296] = ((ws[46304]) * yin[1760]) * yin[6016];
    ws[63328] = ((ws[46336]) * yin[5600]) * yin[6016];
    ws[63360] = ((ws[46368]) * yin[1472]) * yin[6016];
    ws[63392] = ((ws[46400]) * yin[5056]) * yin[6016];
    ws[63424] = ((ws[46432]) * yin[1504]) * yin[6016];
    ws[63456] = ((ws[46464]) * yin[2816]) * yin[6016];
    ws[63488] = ((ws[46496]) * yin[5728]) * yin[6016];
    ws[63520] = ((ws[46528]) * yin[4096]) * yin[6016];
    ws[63552] = ((ws[46560]) * yin[4608]) * yin[6016];
    ws[63584] = ((ws[46592]) * yin[1792]) * yin[6016];
    ws[63616] = ((ws[46624]) * yin[4352]) * yin[6016];
    ws[63648] = ((ws[46656]) * yin[5696]) * yin[6016];
    ws[63680] = ((ws[46688]) * yin[3680]) * yin[6016];
    ws[63712] = ((ws[46720]) * yin[1088]) * yin[6016];
    ws[63744] = ((ws[46752]) * yin[1536]) * yin[6016];
    ws[63776] = ((ws[46784]) * yin[1824]) * yin[6016];
    ws[63808] = ((ws[46816]) * yin[5440]) * yin[6016];
    ws[63840] = ((ws[46848]) * yin[4384]) * yin[6016];
    ws[63872] = ((ws[46880]) * yin[1696]) * yin[6016];
    ws[63904] = ((ws[46912]) * yin[2240]) * yin[5184];
    ws[63936] = ((ws[46944]) * yin[2752]) * yin[5184];
    ws[63968] = ((ws[46976]) * yin[1152]) * yin[5184];
    ws[64000] = ((ws[47008]) * yin[1408]) * yin[5184];
    ws[64032] = ((ws[47040]) * yin[1440]) * yin[5184];
    ws[64064] = ((ws[47072]) * yin[4576]) * yin[5184];
    ws[64096] = ((ws[47104]) * yin[4384]) * yin[5184];
    ws[64128] = ((ws[47136]) * yin[4128]) * yin[5184];
    ws[64160] = ((ws[47168]) * yin[4736]) * yin[5184];
    ws[64192] = ((ws[47200]) * yin[3872]) * yin[5184];
    ws[64224] = ((ws[47232]) * yin[5472]) * yin[5184];
    ws[64256] = ((ws[47264]) * yin[4320]) * yin[5184];
    ws[64288] = ((ws[47296]) * yin[3584]) * yin[5184];
    ws[64320] = ((ws[47328]) * yin[3808]) * yin[5184];
    ws[64352] = ((ws[47360]) * yin[2240]) * yin[5952];
    ws[64384] = ((ws[47392]) * yin[2752]) * yin[5952];
    ws[64416] = ((ws[47424]) * yin[1152]) * yin[5952];
    ws[64448] = ((ws[47456]) * yin[1408]) * yin[5952];
    ws[64480] = ((ws[47488]) * yin[1440]) * yin[5952];
    ws[64512] = ((ws[47520]) * yin[4384]) * yin[5952];
    ws[64544] = ((ws[47552]) * yin[5856]) * yin[5952];
    ws[64576] = ((ws[47584]) * yin[5568]) * yin[5952];
    ws[64608] = ((ws[47616]) * yin[5760]) * yin[5952];
    ws[64640] = ((ws[47648]) * yin[4128]) * yin[5952];
    ws[64672] = ((ws[47680]) * yin[3872]) * yin[5952];
    ws[64704] = ((ws[47712]) * yin[5376]) * yin[5952];
    ws[64736] = ((ws[47744]) * yin[5248]) * yin[5952];
    ws[64768] = ((ws[47776]) * yin[1248]) * yin[5952];
    ws[64800] = ((ws[47808]) * yin[2944]) * yin[5952];
    ws[64832] = ((ws[47840]) * yin[1760]) * yin[5952];
    ws[64864] = ((ws[47872]) * yin[1824]) * yin[5952];
    ws[64896] = (ws[47904]) * yin[2560];
    ws[64928] = (ws[47936]) * yin[1728];
    ws[64960] = ((ws[47968]) * yin[5792]) * yin[5920];
    ws[64992] = (ws[48000]) * yin[1088];
    ws[65024] = ((ws[48032]) * yin[4800]) * yin[5920];
    ws[65056] = (ws[48064]) * yin[1536];
    ws[65088] = ((ws[48096]) * yin[4672]) * yin[5920];
    ws[65120] = (ws[48128]) * yin[1824];
    ws[65152] = ((ws[48160]) * yin[5888]) * yin[5824];
    ws[65184] = ((ws[48192]) * yin[5632]) * yin[5824];
    ws[65216] = ((ws[48224]) * yin[5408]) * yin[5824];
    ws[65248] = ((ws[48256]) * yin[5120]) * yin[5824];
    ws[65280] = ((ws[48288]) * yin[3008]) * yin[5824];
    ws[65312] = ((ws[48320]) * yin[3200]) * yin[5824];
    ws[65344] = ((ws[48352]) * yin[3328]) * yin[5824];
    ws[65376] = ((ws[48384]) * yin[3360]) * yin[5824];
    ws[65408] = ((ws[48416]) * yin[3296]) * yin[5824];
    ws[65440] = ((ws[48448]) * yin[3104]) * yin[5824];
    ws[65472] = ((ws[48480]) * yin[3264]) * yin[5824];
    ws[65504] = ((ws[48512]) * yin[4160]) * yin[5824];
    ws[65536] = ((ws[48544]) * yin[3744]) * yin[5824];
    ws[65568] = ((ws[48576]) * yin[2624]) * yin[5824];
    ws[65600] = ((ws[48608]) * yin[3840]) * yin[5824];
    ws[65632] = ((ws[48640]) * yin[4192]) * yin[5824];
    ws[65664] = ((ws[48672]) * yin[3936]) * yin[5824];
    ws[65696] = ((ws[48704]) * yin[2656]) * yin[5824];
    ws[65728] = ((ws[48736]) * yin[3712]) * yin[5824];
    ws[65760] = ((ws[48768]) * yin[2560]) * yin[5824];
    ws[65792] = ((ws[48800]) * yin[1728]) * yin[5824];
    ws[65824] = ((ws[48832]) * yin[5792]) * yin[5824];
    ws[65856] = ((ws[48864]) * yin[4800]) * yin[5824];
    ws[65888] = ((ws[48896]) * yin[2848]) * yin[5824];
    ws[65920] = ((ws[48928]) * yin[5152]) * yin[5824];
    ws[65952] = ((ws[48960]) * yin[3776]) * yin[5824];
    ws[65984] = ((ws[48992]) * yin[4672]) * yin[5824];
    ws[66016] = ((ws[49024]) * yin[3520]) * yin[5824];
    ws[66048] = ((ws[49056]) * yin[2880]) * yin[5824];
    ws[66080] = ((ws[49088]) * yin[2912]) * yin[5824];
    ws[66112] = ((ws[49120]) * yin[2592]) * yin[5824];
    ws[66144] = ((ws[49152]) * yin[2272]) * yin[5824];
    ws[66176] = ((ws[49184]) * yin[3648]) * yin[5824];
    ws[66208] = ((ws[49216]) * yin[3040]) * yin[5824];
    ws[66240] = ((ws[49248]) * yin[2976]) * yin[5824];
    ws[66272] = ((ws[49280]) * yin[4032]) * yin[5824];
    ws[66304] = ((ws[49312]) * yin[4064]) * yin[5824];
    ws[66336] = ((ws[49344]) * yin[3072]) * yin[5824];
    ws[66368] = ((ws[49376]) * yin[5216]) * yin[5824];
    ws[66400] = ((ws[49408]) * yin[2688]) * yin[5920];
    ws[66432] = ((ws[49440]) * yin[3232]) * yin[5920];
    ws[66464] = ((ws[49472]) * yin[3808]) * yin[5920];
    ws[66496] = ((ws[49504]) * yin[5888]) * yin[5984];
    ws[66528] = ((ws[49536]) * yin[5632]) * yin[5984];
    ws[66560] = ((ws[49568]) * yin[5408]) * yin[5984];
    ws[66592] = ((ws[49600]) * yin[5120]) * yin[5984];
    ws[66624] = ((ws[49632]) * yin[3008]) * yin[5984];
    ws[66656] = ((ws[49664]) * yin[3200]) * yin[5984];
    ws[66688] = ((ws[49696]) * yin[3328]) * yin[5984];
    ws[66720] = ((ws[49728]) * yin[3360]) * yin[5984];
    ws[66752] = ((ws[49760]) * yin[3296]) * yin[5984];
    ws[66784] = ((ws[49792]) * yin[3104]) * yin[5984];
    ws[66816] = ((ws[49824]) * yin[3264]) * yin[5984];
    ws[66848] = ((ws[49856]) * yin[4160]) * yin[5984];
    ws[66880] = ((ws[49888]) * yin[3744]) * yin[5984];
    ws[66912] = ((ws[49920]) * yin[2624]) * yin[5984];
    ws[66944] = ((ws[49952]) * yin[3840]) * yin[5984];
    ws[66976] = ((ws[49984]) * yin[4192]) * yin[5984];
    ws[67008] = ((ws[50016]) * yin[3936]) * yin[5984];
    ws[67040] = ((ws[50048]) * yin[2656]) * yin[5984];
    ws[67072] = ((ws[50080]) * yin[3712]) * yin[5984];
    ws[67104] = ((ws[50112]) * yin[2560]) * yin[5984];
    ws[67136] = ((ws[50144]) * yin[1728]) * yin[5984];
    ws[67168] = ((ws[50176]) * yin[5792]) * yin[5984];
    ws[67200] = ((ws[50208]) * yin[4800]) * yin[5984];
    ws[67232] = ((ws[50240]) * yin[2848]) * yin[5984];
    ws[67264] = ((ws[50272]) * yin[5152]) * yin[5984];
    ws[67296] = ((ws[50304]) * yin[3776]) * yin[5984];
    ws[67328] = ((ws[50336]) * yin[4672]) * yin[5984];
    ws[67360] = ((ws[50368]) * yin[3520]) * yin[5984];
    ws[67392] = ((ws[50400]) * yin[2880]) * yin[5984];
    ws[67424] = ((ws[50432]) * yin[2912]) * yin[5984];
    ws[67456] = ((ws[50464]) * yin[3648]) * yin[5984];
    ws[67488] = ((ws[50496]) * yin[3232]) * yin[5984];
    ws[67520] = ((ws[50528]) * yin[3040]) * yin[5984];
    ws[67552] = ((ws[50560]) * yin[2976]) * yin[5984];
    ws[67584] = ((ws[50592]) * yin[4032]) * yin[5984];
    ws[67616] = ((ws[50624]) * yin[4064]) * yin[5984];
    ws[67648] = ((ws[50656]) * yin[3072]) * yin[5984];
    ws[67680] = ((ws[50688]) * yin[5216]) * yin[5984];
    ws[67712] = ((ws[50720]) * yin[5888]) * yin[5888];
    ws[67744] = ((ws[50752]) * yin[5632]) * yin[5888];
    ws[67776] = ((ws[50784]) * yin[5408]) * yin[5888];
    ws[67808] = ((ws[50816]) * yin[5120]) * yin[5888];
    ws[67840] = ((ws[50848]) * yin[3008]) * yin[5888];
    ws[67872] = ((ws[50880]) * yin[3200]) * yin[5888];
    ws[67904] = ((ws[50912]) * yin[3328]) * yin[5888];
    ws[67936] = ((ws[50944]) * yin[3360]) * yin[5888];
    ws[67968] = ((ws[50976]) * yin[3296]) * yin[5888];
    ws[68000] = ((ws[51008]) * yin[3104]) * yin[5888];
    ws[68032] = ((ws[51040]) * yin[3264]) * yin[5888];
    ws[68064] = ((ws[51072]) * yin[4288]) * yin[5888];
    ws[68096] = ((ws[51104]) * yin[4160]) * yin[5888];
    ws[68128] = ((ws[51136]) * yin[3744]) * yin[5888];
    ws[68160] = ((ws[51168]) * yin[2624]) * yin[5888];
    ws[68192] = ((ws[51200]) * yin[3840]) * yin[5888];
    ws[68224] = ((ws[51232]) * yin[4192]) * yin[5888];
    ws[68256] = ((ws[51264]) * yin[3936]) * yin[5888];
    ws[68288] = ((ws[51296]) * yin[2656]) * yin[5888];
    ws[68320] = ((ws[51328]) * yin[3712]) * yin[5888];
    ws[68352] = ((ws[51360]) * yin[5792]) * yin[5888];
    ws[68384] = ((ws[51392]) * yin[4800]) * yin[5888];
    ws[68416] = ((ws[51424]) * yin[2848]) * yin[5888];
    ws[68448] = ((ws[51456]) * yin[5152]) * yin[5888];
    ws[68480] = ((ws[51488]) * yin[3776]) * yin[5888];
    ws[68512] = ((ws[51520]) * yin[4672]) * yin[5888];
    ws[68544] = ((ws[51552]) * yin[3520]) * yin[5888];
    ws[68576] = ((ws[51584]) * yin[2880]) * yin[5888];
    ws[68608] = ((ws[51616]) * yin[2912]) * yin[5888];
    ws[68640] = ((ws[51648]) * yin[2592]) * yin[5888];
    ws[68672] = ((ws[51680]) * yin[2272]) * yin[5888];
    ws[68704] = ((ws[51712]) * yin[3648]) * yin[5888];
    ws[68736] = ((ws[51744]) * yin[3040]) * yin[5888];
    ws[68768] = ((ws[51776]) * yin[2976]) * yin[5888];
    ws[68800] = ((ws[51808]) * yin[4032]) * yin[5888];
    ws[68832] = ((ws[51840]) * yin[4064]) * yin[5888];
    ws[68864] = ((ws[51872]) * yin[3072]) * yin[5888];
    ws[68896] = ((ws[51904]) * yin[5216]) * yin[5888];
    ws[68928] = ((ws[51936]) * yin[5632]) * yin[5792];
    ws[68960] = ((ws[51968]) * yin[5408]) * yin[5792];
    ws[68992] = ((ws[52000]) * yin[5120]) * yin[5792];
    ws[69024] = ((ws[52032]) * yin[3008]) * yin[5792];
    ws[69056] = ((ws[52064]) * yin[3200]) * yin[5792];
    ws[69088] = ((ws[52096]) * yin[3328]) * yin[5792];
    ws[69120] = ((ws[52128]) * yin[3360]) * yin[5792];
    ws[69152] = ((ws[52160]) * yin[3296]) * yin[5792];
    ws[69184] = ((ws[52192]) * yin[3104]) * yin[5792];
    ws[69216] = ((ws[52224]) * yin[3264]) * yin[5792];
    ws[69248] = ((ws[52256]) * yin[4288]) * yin[5792];
    ws[69280] = ((ws[52288]) * yin[4160]) * yin[5792];
    ws[69312] = ((ws[52320]) * yin[3744]) * yin[5792];
    ws[69344] = ((ws[52352]) * yin[2624]) * yin[5792];
    ws[69376] = ((ws[52384]) * yin[3840]) * yin[5792];
    ws[69408] = ((ws[52416]) * yin[4192]) * yin[5792];
    ws[69440] = ((ws[52448]) * yin[3936]) * yin[5792];
    ws[69472] = ((ws[52480]) * yin[2656]) * yin[5792];
    ws[69504] = ((ws[52512]) * yin[3712]) * yin[5792];
    ws[69536] = ((ws[52544]) * yin[5792]) * yin[5792];
    ws[69568] = ((ws[52576]) * yin[4800]) * yin[5792];
    ws[69600] = ((ws[52608]) * yin[2848]) * yin[5792];
    ws[69632] = ((ws[52640]) * yin[5152]) * yin[5792];
    ws[69664] = ((ws[52672]) * yin[3776]) * yin[5792];
    ws[69696] = ((ws[52704]) * yin[4672]) * yin[5792];
    ws[69728] = ((ws[52736]) * yin[3520]) * yin[5792];
    ws[69760] = ((ws[52768]) * yin[2880]) * yin[5792];
    ws[69792] = ((ws[52800]) * yin[2912]) * yin[5792];
    ws[69824] = ((ws[52832]) * yin[2592]) * yin[5792];
    ws[69856] = ((ws[52864]) * yin[2272]) * yin[5792];
    ws[69888] = ((ws[52896]) * yin[3648]) * yin[5792];
    ws[69920] = ((ws[52928]) * yin[3040]) * yin[5792];
    ws[69952] = ((ws[52960]) * yin[2976]) * yin[5792];
    ws[69984] = ((ws[52992]) * yin[4032]) * yin[5792];
    ws[70016] = ((ws[53024]) * yin[4064]) * yin[5792];
    ws[70048] = ((ws[53056]) * yin[3072]) * yin[5792];
    ws[70080] = ((ws[53088]) * yin[5216]) * yin[5792];
    ws[70112] = ((ws[53120]) * yin[4800]) * yin[4800];
    ws[70144] = ((ws[53152]) * yin[5888]) * yin[5952];
    ws[70176] = ((ws[53184]) * yin[5632]) * yin[5952];
    ws[70208] = ((ws[53216]) * yin[5408]) * yin[5952];
    ws[70240] = ((ws[53248]) * yin[5120]) * yin[5952];
    ws[70272] = ((ws[53280]) * yin[3008]) * yin[5952];
    ws[70304] = ((ws[53312]) * yin[3200]) * yin[5952];
    ws[70336] = ((ws[53344]) * yin[3328]) * yin[5952];
    ws[70368] = ((ws[53376]) * yin[3360]) * yin[5952];
    ws[70400] = ((ws[53408]) * yin[3296]) * yin[5952];
    ws[70432] = ((ws[53440]) * yin[3104]) * yin[5952];
    ws[70464] = ((ws[53472]) * yin[3264]) * yin[5952];
    ws[70496] = ((ws[53504]) * yin[4288]) * yin[5952];
    ws[70528] = ((ws[53536]) * yin[4160]) * yin[5952];
    ws[70560] = ((ws[53568]) * yin[4192]) * yin[5952];
    ws[70592] = ((ws[53600]) * yin[2624]) * yin[5952];
    ws[70624] = ((ws[53632]) * yin[2656]) * yin[5952];
    ws[70656] = ((ws[53664]) * yin[5792]) * yin[5952];
    ws[70688] = ((ws[53696]) * yin[4800]) * yin[5952];
    ws[70720] = ((ws[53728]) * yin[2848]) * yin[5952];
    ws[70752] = ((ws[53760]) * yin[5152]) * yin[5952];
    ws[70784] = ((ws[53792]) * yin[3776]) * yin[5952];
    ws[70816] = ((ws[53824]) * yin[4672]) * yin[5952];
    ws[70848] = ((ws[53856]) * yin[3520]) * yin[5952];
    ws[70880] = ((ws[53888]) * yin[2880]) * yin[5952];
    ws[70912] = ((ws[53920]) * yin[2912]) * yin[5952];
    ws[70944] = ((ws[53952]) * yin[2592]) * yin[5952];
    ws[70976] = ((ws[53984]) * yin[2272]) * yin[5952];
    ws[71008] = ((ws[54016]) * yin[3648]) * yin[5952];
    ws[71040] = ((ws[54048]) * yin[3040]) * yin[5952];
    ws[71072] = ((ws[54080]) * yin[2976]) * yin[5952];
    ws[71104] = ((ws[54112]) * yin[4032]) * yin[5952];
    ws[71136] = ((ws[54144]) * yin[4064]) * yin[5952];
    ws[71168] = ((ws[54176]) * yin[3072]) * yin[5952];
    ws[71200] = ((ws[54208]) * yin[4032]) * yin[4032];
    ws[71232] = ((ws[54240]) * yin[4032]) * yin[4064];
    ws[71264] = ((ws[54272]) * yin[4064]) * yin[4064];
    ws[71296] = ((ws[54304]) * yin[5216]) * yin[5952];
    ws[71328] = ((ws[54336]) * yin[5216]) * yin[4800];
    ws[71360] = ((ws[54368]) * yin[5216]) * yin[5216];
    ws[71392] = ((ws[54400]) * yin[3744]) * yin[4160];
    ws[71424] = ((ws[54432]) * yin[3744]) * yin[4192];
    ws[71456] = ((ws[54464]) * yin[3744]) * yin[4288];
    ws[71488] = ((ws[54496]) * yin[3936]) * yin[4160];
    ws[71520] = ((ws[54528]) * yin[3936]) * yin[4192];
    ws[71552] = ((ws[54560]) * yin[3936]) * yin[4288];
    ws[71584] = ((ws[54592]) * yin[3840]) * yin[4160];
    ws[71616] = ((ws[54624]) * yin[3840]) * yin[4192];
    ws[71648] = ((ws[54656]) * yin[3840]) * yin[4288];
    ws[71680] = ((ws[54688]) * yin[3712]) * yin[4160];
    ws[71712] = ((ws[54720]) * yin[3712]) * yin[4192];
    ws[71744] = ((ws[54752]) * yin[3712]) * yin[4288];
    ws[71776] = ((ws[54784]) * yin[1376]) * yin[6016];
    ws[71808] = ((ws[54816]) * yin[384]) * yin[6016];
    ws[71840] = ((ws[54848]) * yin[416]) * yin[6016];
    ws[71872] = ((ws[54880]) * yin[3552]) * yin[6016];
    ws[71904] = ((ws[54912]) * yin[3552]) * yin[5184];
    ws[71936] = ((ws[54944]) * yin[3552]) * yin[5952];
    ws[72000] = ((ws[55008]) * yin[1568]) * yin[6016];
    ws[72032] = ((ws[55040]) * yin[3136]) * yin[5824];
    ws[72064] = ((ws[55072]) * yin[3136]) * yin[5952];
    ws[72096] = ((ws[55104]) * yin[3136]) * yin[5984];
    ws[72128] = ((ws[55136]) * yin[3136]) * yin[5888];
    ws[72160] = ((ws[55168]) * yin[3136]) * yin[5792];
    ws[72192] = ((ws[55200]) * yin[1568]) * yin[5184];
    ws[72224] = ((ws[55232]) * yin[1568]) * yin[5952];
    ws[72256] = ((ws[55264]) * yin[3168]) * yin[6016];
    ws[72288] = ((ws[55296]) * yin[1856]) * yin[5824];
    ws[72320] = ((ws[55328]) * yin[1856]) * yin[5984];
    ws[72352] = ((ws[55360]) * yin[4512]) * yin[6016];
    ws[72384] = ((ws[55392]) * yin[3168]) * yin[5184];
    ws[72416] = ((ws[55424]) * yin[3168]) * yin[5952];
    ws[72448] = ((ws[55456]) * yin[448]) * yin[6016];
    ws[72480] = ((ws[55488]) * yin[1600]) * yin[5952];
    ws[72512] = ((ws[55520]) * yin[1920]) * yin[5984];
    ws[72544] = ((ws[55552]) * yin[1920]) * yin[5824];
    ws[72576] = ((ws[55584]) * yin[1920]) * yin[5952];
    ws[72608] = ((ws[55616]) * yin[1600]) * yin[5184];
    ws[72640] = ((ws[55648]) * yin[1600]) * yin[6016];
    ws[72672] = ((ws[55680]) * yin[2304]) * yin[5984];
    ws[72704] = ((ws[55712]) * yin[2304]) * yin[5952];
    ws[72736] = ((ws[55744]) * yin[2304]) * yin[5824];
    ws[72768] = (ws[55776]) * yin[5376];
    ws[72800] = (ws[55808]) * yin[5248];
    ws[72832] = (ws[55840]) * yin[1024];
    ws[72864] = (ws[55872]) * yin[5920];
    ws[72896] = (ws[55904]) * yin[5984];
    ws[72928] = (ws[55936]) * yin[5952];
    ws[72992] = (ws[56000]) * yin[1376];
    ws[73024] = (ws[56032]) * yin[1056];
    ws[73056] = ((ws[56064]) * yin[1056]) * yin[512];
    ws[73088] = (ws[56096]) * yin[1664];
    ws[73120] = (ws[56128]) * yin[2208];
    ws[73152] = ((ws[56160]) * yin[608]) * yin[6016];
    ws[73184] = ((ws[56192]) * yin[640]) * yin[6016];
    ws[73216] = ((ws[56224]) * yin[672]) * yin[6016];
    ws[73248] = ((ws[56256]) * yin[704]) * yin[6016];
    ws[73280] = ((ws[56288]) * yin[736]) * yin[6016];
    ws[73312] = ((ws[56320]) * yin[768]) * yin[6016];
    ws[73344] = ((ws[56352]) * yin[800]) * yin[6016];
    ws[73376] = ((ws[56384]) * yin[2368]) * yin[5824];
    ws[73408] = ((ws[56416]) * yin[2400]) * yin[5824];
    ws[73440] = ((ws[56448]) * yin[2432]) * yin[5824];
    ws[73472] = ((ws[56480]) * yin[2464]) * yin[5824];
    ws[73504] = ((ws[56512]) * yin[2496]) * yin[5824];
    ws[73536] = ((ws[56544]) * yin[2528]) * yin[5824];
    ws[73568] = ((ws[56576]) * yin[3904]) * yin[5824];
    ws[73600] = ((ws[56608]) * yin[2368]) * yin[5952];
    ws[73632] = ((ws[56640]) * yin[2400]) * yin[5952];
    ws[73664] = ((ws[56672]) * yin[2432]) * yin[5952];
    ws[73696] = ((ws[56704]) * yin[2464]) * yin[5952];
    ws[73728] = ((ws[56736]) * yin[2496]) * yin[5952];
    ws[73760] = ((ws[56768]) * yin[2528]) * yin[5952];
    ws[73792] = ((ws[56800]) * yin[3904]) * yin[5952];
    ws[73824] = ((ws[56832]) * yin[2368]) * yin[5984];
    ws[73856] = ((ws[56864]) * yin[2400]) * yin[5984];
    ws[73888] = ((ws[56896]) * yin[2432]) * yin[5984];
    ws[73920] = ((ws[56928]) * yin[2464]) * yin[5984];
    ws[73952] = ((ws[56960]) * yin[2496]) * yin[5984];
    ws[73984] = ((ws[56992]) * yin[2528]) * yin[5984];
    ws[74016] = ((ws[57024]) * yin[3904]) * yin[5984];
    ws[74048] = (ws[57056]) * yin[1952];
    ws[74080] = (ws[57088]) * yin[1984];
    ws[74112] = (ws[57120]) * yin[2016];
    ws[74144] = (ws[57152]) * yin[2048];
    ws[74176] = (ws[57184]) * yin[2080];
    ws[74208] = (ws[57216]) * yin[2112];
    ws[74240] = (ws[57248]) * yin[2144];
    ws[74272] = ((ws[57280]) * yin[1952]) * yin[5824];
    ws[74304] = ((ws[57312]) * yin[1984]) * yin[5824];
    ws[74336] = ((ws[57344]) * yin[2016]) * yin[5824];
    ws[74368] = ((ws[57376]) * yin[2048]) * yin[5824];
    ws[74400] = ((ws[57408]) * yin[2080]) * yin[5824];
    ws[74432] = ((ws[57440]) * yin[2112]) * yin[5824];
    ws[74464] = ((ws[57472]) * yin[2144]) * yin[5824];
    ws[74496] = ((ws[57504]) * yin[1952]) * yin[5952];
    ws[74528] = ((ws[57536]) * yin[1984]) * yin[5952];
    ws[74560] = ((ws[57568]) * yin[2016]) * yin[5952];
    ws[74592] = ((ws[57600]) * yin[2048]) * yin[5952];
    ws[74624] = ((ws[57632]) * yin[2080]) * yin[5952];
    ws[74656] = ((ws[57664]) * yin[2112]) * yin[5952];
    ws[74688] = ((ws[57696]) * yin[2144]) * yin[5952];
    ws[74720] = ((ws[57728]) * yin[1952]) * yin[5984];
    ws[74752] = ((ws[57760]) * yin[1984]) * yin[5984];
    ws[74784] = ((ws[57792]) * yin[2016]) * yin[5984];
    ws[74816] = ((ws[57824]) * yin[2048]) * yin[5984];
    ws[74848] = ((ws[57856]) * yin[2080]) * yin[5984];
    ws[74880] = ((ws[57888]) * yin[2112]) * yin[5984];
    ws[74912] = ((ws[57920]) * yin[2144]) * yin[5984];
    ws[74944] = ((ws[57952]) * yin[832]) * yin[6016];
    ws[74976] = ((ws[57984]) * yin[3392]) * yin[5984];
    ws[75008] = ((ws[58016]) * yin[3392]) * yin[5824];
    ws[75040] = ((ws[58048]) * yin[3392]) * yin[5952];
    ws[75072] = ((ws[58080]) * yin[3392]) * yin[5888];
    ws[75104] = ((ws[58112]) * yin[3392]) * yin[5792];
    ws[75136] = ((ws[58144]) * yin[864]) * yin[6016];
    ws[75168] = ((ws[58176]) * yin[3424]) * yin[5984];
    ws[75200] = ((ws[58208]) * yin[3424]) * yin[5824];
    ws[75232] = ((ws[58240]) * yin[3424]) * yin[5952];
    ws[75264] = ((ws[58272]) * yin[3424]) * yin[5888];
    ws[75296] = ((ws[58304]) * yin[3424]) * yin[5792];
    ws[75328] = ((ws[58336]) * yin[896]) * yin[6016];
    ws[75360] = ((ws[58368]) * yin[3456]) * yin[5984];
    ws[75392] = ((ws[58400]) * yin[3456]) * yin[5824];
    ws[75424] = ((ws[58432]) * yin[3456]) * yin[5952];
    ws[75456] = ((ws[58464]) * yin[3456]) * yin[5888];
    ws[75488] = ((ws[58496]) * yin[3456]) * yin[5792];
    ws[75520] = ((ws[58528]) * yin[4768]) * yin[6016];
    ws[75552] = ((ws[58560]) * yin[4864]) * yin[6016];
    ws[75584] = ((ws[58592]) * yin[4832]) * yin[6016];
    ws[75616] = ((ws[58624]) * yin[4896]) * yin[6016];
    ws[75648] = ((ws[58656]) * yin[4640]) * yin[6016];
    ws[75680] = ((ws[58688]) * yin[4416]) * yin[6016];
    ws[75712] = ((ws[58720]) * yin[4928]) * yin[6016];
    ws[75744] = ((ws[58752]) * yin[4960]) * yin[6016];
    ws[75776] = ((ws[58784]) * yin[4992]) * yin[6016];
    ws[75808] = ((ws[58816]) * yin[4704]) * yin[6016];
    ws[75840] = ((ws[58848]) * yin[5088]) * yin[6016];
    ws[75872] = ((ws[58880]) * yin[5536]) * yin[6016];
    ws[75904] = ((ws[58912]) * yin[5312]) * yin[6016];
    ws[75936] = ((ws[58944]) * yin[4224]) * yin[6016];
    ws[75968] = ((ws[58976]) * yin[3968]) * yin[6016];
    ws[76000] = ((ws[59008]) * yin[4608]) * yin[6016];
    ws[76032] = ((ws[59040]) * yin[928]) * yin[6016];
    ws[76064] = (ws[59072]) * yin[96];
    ws[76096] = (ws[59104]) * yin[128];
    ws[76128] = ((ws[59136]) * yin[992]) * yin[6016];
    ws[76160] = ((ws[59168]) * yin[3488]) * yin[5984];
    ws[76192] = ((ws[59200]) * yin[3488]) * yin[5824];
    ws[76224] = ((ws[59232]) * yin[3488]) * yin[5952];
    ws[76256] = ((ws[59264]) * yin[3488]) * yin[5888];
    ws[76288] = ((ws[59296]) * yin[3488]) * yin[5792];
    {
      double a = 1.0 * ws[73024];
      yout[0] = a;
    }
    {
      double a = 1.0 * ws[73088];
      yout[32] = a;
    }
    {
      double a = 1.0 * ws[73120];
      yout[64] = a;
    }
    {
      double a = -ws[76064];
      yout[96] = a;
    }
    {
      double a = -ws[76096];
      yout[128] = a;
    }
    {
      double a = -ws[61728];
      yout[160] = a;
    }
    {
      double a = 1.0 * ws[61728];
      yout[192] = a;
    }
    {
      double a = 1.0 * ws[61728];
      yout[224] = a;
    }
    {
      double a = -ws[62016];
      yout[256] = a;
    }
    {
      double a = -ws[62080];
      yout[288] = a;
    }
    {
      double a = -ws[62112];
      yout[320] = a;
    }
    {
      double a = -ws[62144];
      yout[352] = a;
    }
    {
      double a = -ws[71808];
      yout[384] = a;
    }
    {
      double a = -ws[71840];
      yout[416] = a;
    }
    {
      double a = -ws[72448];
      yout[448] = a;
    }
    {
      double a = 1.0 * ws[72768];
      a = fma(1.0, ws[72800], a);
      yout[480] = a;
    }
    {
      double a = -ws[73056];
      yout[512] = a;
    }
    {
      double a = 1.0 * ws[73056];
      yout[544] = a;
    }
    {
      double a = -ws[60800];
      a = a - ws[60832];
      a = a - ws[60864];
      yout[576] = a;
    }
    {
      double a = -ws[73152];
      yout[608] = a;
    }
    {
      double a = -ws[73184];
      yout[640] = a;
    }
    {
      double a = -ws[73216];
      yout[672] = a;
    }
    {
      double a = -ws[73248];
      yout[704] = a;
    }
    {
      double a = -ws[73280];
      yout[736] = a;
    }
    {
      double a = -ws[73312];
      yout[768] = a;
    }
    {
      double a = -ws[73344];
      yout[800] = a;
    }
    {
      double a = -ws[74944];
      yout[832] = a;
    }
    {
      double a = -ws[75136];
      yout[864] = a;
    }
    {
      double a = -ws[75328];
      yout[896] = a;
    }
    {
      double a = -ws[76032];
      yout[928] = a;
    }
    {
      double a = 1.0 * ws[76064];
      a = fma(1.0, ws[76096], a);
      yout[960] = a;
    }
    {
      double a = -ws[76128];
      yout[992] = a;
    }
    {
      double a = 1.0 * ws[61536];
      a = a - ws[61568];
      a = a - ws[61600];
      a = a - ws[72832];
      yout[1024] = a;
    }
    {
      double a = 1.0 * ws[72992];
      a = a - ws[73024];
      a = a - ws[73056];
      yout[1056] = a;
    }
    {
      double a = -ws[63712];
      a = fma(1.0, ws[64960], a);
      a = a - ws[64992];
      yout[1088] = a;
    }
    {
      double a = -ws[61888];
      a = fma(0.006, ws[63936], a);
      yout[1120] = a;
    }
    {
      double a = -ws[61984];
      a = a - ws[63968];
      a = a - ws[64416];
      yout[1152] = a;
    }
    {
      double a = 1.0 * ws[61088];
      a = a - ws[61216];
      a = fma(0.5, ws[72864], a);
      yout[1184] = a;
    }
    {
      double a = -ws[62048];
      a = fma(0.032, ws[63936], a);
      yout[1216] = a;
    }
    {
      double a = 0.53 * ws[62048];
      a = a - ws[63232];
      a = a - ws[64768];
      yout[1248] = a;
    }
    {
      double a = 1.0 * ws[61632];
      a = a - ws[61664];
      a = a - ws[61696];
      yout[1280] = a;
    }
    {
      double a = -ws[62176];
      a = a - ws[62208];
      a = a - ws[62240];
      yout[1312] = a;
    }
    {
      double a = 1.0 * ws[62272];
      a = a - ws[62336];
      a = a - ws[62368];
      yout[1344] = a;
    }
    {
      double a = 0.44 * ws[62368];
      a = fma(0.17, ws[62464], a);
      a = a - ws[71776];
      a = a - ws[72992];
      yout[1376] = a;
    }
    {
      double a = -ws[62592];
      a = a - ws[64000];
      a = a - ws[64448];
      yout[1408] = a;
    }
    {
      double a = -ws[62624];
      a = a - ws[64032];
      a = a - ws[64480];
      yout[1440] = a;
    }
    {
      double a = -ws[63360];
      a = fma(0.25, ws[67744], a);
      yout[1472] = a;
    }
    {
      double a = -ws[63424];
      a = fma(0.25, ws[67840], a);
      yout[1504] = a;
    }
    {
      double a = -ws[63744];
      a = fma(1.0, ws[65024], a);
      a = a - ws[65056];
      yout[1536] = a;
    }
    {
      double a = -ws[72000];
      a = a - ws[72192];
      a = a - ws[72224];
      yout[1568] = a;
    }
    {
      double a = -ws[72480];
      a = a - ws[72608];
      a = a - ws[72640];
      yout[1600] = a;
    }
    {
      double a = 0.555 * ws[62208];
      a = a - ws[62400];
      a = a - ws[62432];
      yout[1632] = a;
    }
    {
      double a = 0.14 * ws[62368];
      a = fma(0.02, ws[62400], a);
      a = a - ws[62560];
      a = a - ws[73088];
      yout[1664] = a;
    }
    {
      double a = 0.33 * ws[63840];
      a = a - ws[63872];
      a = fma(0.33, ws[64096], a);
      a = fma(0.33, ws[64512], a);
      yout[1696] = a;
    }
    {
      double a = 0.83 * ws[62688];
      a = a - ws[64928];
      a = a - ws[65792];
      a = a - ws[67136];
      yout[1728] = a;
    }
    {
      double a = 0.619 * ws[63232];
      a = fma(0.584, ws[63264], a);
      a = a - ws[63296];
      a = a - ws[64832];
      yout[1760] = a;
    }
    {
      double a = -ws[63584];
      a = fma(1.0, ws[67328], a);
      a = fma(1.0, ws[67360], a);
      yout[1792] = a;
    }
    {
      double a = -ws[63776];
      a = a - ws[64864];
      a = fma(1.0, ws[65088], a);
      a = a - ws[65120];
      yout[1824] = a;
    }
    {
      double a = 0.51 * ws[72256];
      a = a - ws[72288];
      a = a - ws[72320];
      yout[1856] = a;
    }
    {
      double a = -ws[61824];
      a = fma(0.02, ws[63936], a);
      a = fma(0.01, ws[63968], a);
      yout[1888] = a;
    }
    {
      double a = 1.0 * ws[72480];
      a = a - ws[72512];
      a = a - ws[72544];
      a = a - ws[72576];
      yout[1920] = a;
    }
    {
      double a = 0.72 * ws[73376];
      a = fma(1.0, ws[73600], a);
      a = a - ws[74048];
      a = a - ws[74272];
      a = a - ws[74496];
      a = a - ws[74720];
      yout[1952] = a;
    }
    {
      double a = 0.72 * ws[73408];
      a = fma(1.0, ws[73632], a);
      a = a - ws[74080];
      a = a - ws[74304];
      a = a - ws[74528];
      a = a - ws[74752];
      yout[1984] = a;
    }
    {
      double a = 0.72 * ws[73440];
      a = fma(1.0, ws[73664], a);
      a = a - ws[74112];
      a = a - ws[74336];
      a = a - ws[74560];
      a = a - ws[74784];
      yout[2016] = a;
    }
    {
      double a = 0.72 * ws[73472];
      a = fma(1.0, ws[73696], a);
      a = a - ws[74144];
      a = a - ws[74368];
      a = a - ws[74592];
      a = a - ws[74816];
      yout[2048] = a;
    }
    {
      double a = 0.72 * ws[73504];
      a = fma(1.0, ws[73728], a);
      a = a - ws[74176];
      a = a - ws[74400];
      a = a - ws[74624];
      a = a - ws[74848];
      yout[2080] = a;
    }
    {
      double a = 0.72 * ws[73536];
      a = fma(1.0, ws[73760], a);
      a = a - ws[74208];
      a = a - ws[74432];
      a = a - ws[74656];
      a = a - ws[74880];
      yout[2112] = a;
    }
    {
      double a = 0.74 * ws[73568];
      a = fma(1.0, ws[73792], a);
      a = a - ws[74240];
      a = a - ws[74464];
      a = a - ws[74688];
      a = a - ws[74912];
      yout[2144] = a;
    }
    {
      double a = -ws[61856];
      a = fma(0.015, ws[63936], a);
      a = fma(0.01, ws[63968], a);
      a = fma(0.0665, ws[64000], a);
      yout[2176] = a;
    }
    {
      double a = 0.95 * ws[62400];
      a = fma(0.65, ws[62432], a);
      a = fma(0.35, ws[62464], a);
      a = a - ws[62496];
      a = a - ws[73120];
      yout[2208] = a;
    }
    {
      double a = -ws[61920];
      a = a - ws[63904];
      a = a - ws[64352];
      a = fma(0.17, ws[72192], a);
      yout[2240] = a;
    }
    {
      double a = 1.0 * ws[66112];
      a = a - ws[66144];
      a = fma(1.0, ws[68640], a);
      a = a - ws[68672];
      a = fma(1.0, ws[69824], a);
      a = a - ws[69856];
      a = fma(1.0, ws[70944], a);
      a = a - ws[70976];
      yout[2272] = a;
    }
    {
      double a = 1.0 * ws[72640];
      a = a - ws[72672];
      a = a - ws[72704];
      a = a - ws[72736];
      yout[2304] = a;
    }
    {
      double a = -ws[60736];
      a = a - ws[60768];
      a = fma(1.0, ws[60800], a);
      a = fma(1.0, ws[60832], a);
      a = a - ws[61056];
      a = a - ws[61248];
      a = a - ws[61280];
      yout[2336] = a;
    }
    {
      double a = 1.0 * ws[73152];
      a = a - ws[73376];
      a = a - ws[73600];
      a = a - ws[73824];
      yout[2368] = a;
    }
    {
      double a = 1.0 * ws[73184];
      a = a - ws[73408];
      a = a - ws[73632];
      a = a - ws[73856];
      yout[2400] = a;
    }
    {
      double a = 1.0 * ws[73216];
      a = a - ws[73440];
      a = a - ws[73664];
      a = a - ws[73888];
      yout[2432] = a;
    }
    {
      double a = 1.0 * ws[73248];
      a = a - ws[73472];
      a = a - ws[73696];
      a = a - ws[73920];
      yout[2464] = a;
    }
    {
      double a = 1.0 * ws[73280];
      a = a - ws[73504];
      a = a - ws[73728];
      a = a - ws[73952];
      yout[2496] = a;
    }
    {
      double a = 1.0 * ws[73312];
      a = a - ws[73536];
      a = a - ws[73760];
      a = a - ws[73984];
      yout[2528] = a;
    }
    {
      double a = 0.23 * ws[62656];
      a = fma(0.2145, ws[64000], a);
      a = a - ws[64896];
      a = a - ws[65760];
      a = a - ws[67104];
      yout[2560] = a;
    }
    {
      double a = 1.0 * ws[63200];
      a = a - ws[66112];
      a = a - ws[68640];
      a = a - ws[69824];
      a = a - ws[70944];
      yout[2592] = a;
    }
    {
      double a = 0.975 * ws[64448];
      a = a - ws[65568];
      a = a - ws[66912];
      a = a - ws[68160];
      a = a - ws[69344];
      a = a - ws[70592];
      yout[2624] = a;
    }
    {
      double a = 0.945 * ws[64480];
      a = a - ws[65696];
      a = a - ws[67040];
      a = a - ws[68288];
      a = a - ws[69472];
      a = a - ws[70624];
      yout[2656] = a;
    }
    {
      double a = 1.0 * ws[66144];
      a = a - ws[66400];
      a = fma(1.0, ws[68672], a);
      a = fma(1.0, ws[69856], a);
      a = fma(1.0, ws[70976], a);
      yout[2688] = a;
    }
    {
      double a = 0.04 * ws[71392];
      a = fma(0.04, ws[71424], a);
      a = fma(0.04, ws[71456], a);
      a = fma(0.04, ws[71488], a);
      a = fma(0.04, ws[71520], a);
      a = fma(0.04, ws[71552], a);
      a = fma(0.04, ws[71584], a);
      a = fma(0.04, ws[71616], a);
      a = fma(0.04, ws[71648], a);
      a = fma(0.04, ws[71680], a);
      a = fma(0.04, ws[71712], a);
      a = fma(0.04, ws[71744], a);
      yout[2720] = a;
    }
    {
      double a = -ws[61952];
      a = fma(0.153, ws[62176], a);
      a = a - ws[63936];
      a = a - ws[64384];
      a = fma(0.25, ws[72128], a);
      yout[2752] = a;
    }
    {
      double a = 0.045 * ws[62208];
      a = fma(0.13, ws[62304], a);
      a = fma(0.05, ws[62432], a);
      a = a - ws[62464];
      a = a - ws[62528];
      yout[2784] = a;
    }
    {
      double a = -ws[63456];
      a = fma(0.0385, ws[64000], a);
      a = fma(0.23, ws[64064], a);
      a = fma(1.0, ws[66496], a);
      yout[2816] = a;
    }
    {
      double a = 1.0 * ws[62816];
      a = a - ws[65888];
      a = a - ws[67232];
      a = a - ws[68416];
      a = a - ws[69600];
      a = a - ws[70720];
      yout[2848] = a;
    }
    {
      double a = 1.0 * ws[62976];
      a = a - ws[66048];
      a = a - ws[67392];
      a = a - ws[68576];
      a = a - ws[69760];
      a = a - ws[70880];
      yout[2880] = a;
    }
    {
      double a = 0.687 * ws[63008];
      a = a - ws[66080];
      a = a - ws[67424];
      a = a - ws[68608];
      a = a - ws[69792];
      a = a - ws[70912];
      yout[2912] = a;
    }
    {
      double a = 0.18 * ws[62080];
      a = fma(0.17, ws[62112], a);
      a = fma(0.18, ws[62144], a);
      a = a - ws[63264];
      a = a - ws[64800];
      a = fma(1.0, ws[67488], a);
      yout[2944] = a;
    }
    {
      double a = 0.36 * ws[63648];
      a = a - ws[66240];
      a = a - ws[67552];
      a = a - ws[68768];
      a = a - ws[69952];
      a = a - ws[71072];
      yout[2976] = a;
    }
    {
      double a = 1.0 * ws[61920];
      a = a - ws[65280];
      a = a - ws[66624];
      a = a - ws[67840];
      a = a - ws[69024];
      a = a - ws[70272];
      yout[3008] = a;
    }
    {
      double a = 1.0 * ws[64320];
      a = a - ws[66208];
      a = a - ws[67520];
      a = a - ws[68736];
      a = a - ws[69920];
      a = a - ws[71040];
      yout[3040] = a;
    }
    {
      double a = 0.424 * ws[64768];
      a = fma(0.4, ws[64800], a);
      a = a - ws[66336];
      a = a - ws[67648];
      a = a - ws[68864];
      a = a - ws[70048];
      a = a - ws[71168];
      yout[3072] = a;
    }
    {
      double a = 0.83 * ws[62112];
      a = a - ws[65440];
      a = a - ws[66784];
      a = a - ws[68000];
      a = a - ws[69184];
      a = a - ws[70432];
      yout[3104] = a;
    }
    {
      double a = 0.667 * ws[72000];
      a = a - ws[72032];
      a = a - ws[72064];
      a = a - ws[72096];
      a = a - ws[72128];
      a = a - ws[72160];
      yout[3136] = a;
    }
    {
      double a = 0.072 * ws[72032];
      a = fma(0.075, ws[72064], a);
      a = fma(0.037, ws[72128], a);
      a = fma(0.06, ws[72160], a);
      a = a - ws[72256];
      a = a - ws[72384];
      a = a - ws[72416];
      yout[3168] = a;
    }
    {
      double a = 1.0 * ws[61952];
      a = a - ws[65312];
      a = a - ws[66656];
      a = a - ws[67872];
      a = a - ws[69056];
      a = a - ws[70304];
      yout[3200] = a;
    }
    {
      double a = 0.059 * ws[63232];
      a = fma(0.056, ws[63264], a);
      a = fma(0.339, ws[64768], a);
      a = fma(0.32, ws[64800], a);
      a = a - ws[66432];
      a = a - ws[67488];
      yout[3232] = a;
    }
    {
      double a = 0.82 * ws[62144];
      a = a - ws[65472];
      a = a - ws[66816];
      a = a - ws[68032];
      a = a - ws[69216];
      a = a - ws[70464];
      yout[3264] = a;
    }
    {
      double a = 0.82 * ws[62080];
      a = a - ws[65408];
      a = a - ws[66752];
      a = a - ws[67968];
      a = a - ws[69152];
      a = a - ws[70400];
      yout[3296] = a;
    }
    {
      double a = 1.0 * ws[61984];
      a = a - ws[65344];
      a = a - ws[66688];
      a = a - ws[67904];
      a = a - ws[69088];
      a = a - ws[70336];
      yout[3328] = a;
    }
    {
      double a = 0.47 * ws[62048];
      a = a - ws[65376];
      a = a - ws[66720];
      a = a - ws[67936];
      a = a - ws[69120];
      a = a - ws[70368];
      yout[3360] = a;
    }
    {
      double a = 0.84 * ws[74944];
      a = a - ws[74976];
      a = a - ws[75008];
      a = a - ws[75040];
      a = a - ws[75072];
      a = a - ws[75104];
      yout[3392] = a;
    }
    {
      double a = 0.84 * ws[75136];
      a = a - ws[75168];
      a = a - ws[75200];
      a = a - ws[75232];
      a = a - ws[75264];
      a = a - ws[75296];
      yout[3424] = a;
    }
    {
      double a = 0.84 * ws[75328];
      a = a - ws[75360];
      a = a - ws[75392];
      a = a - ws[75424];
      a = a - ws[75456];
      a = a - ws[75488];
      yout[3456] = a;
    }
    {
      double a = 1.0 * ws[76128];
      a = a - ws[76160];
      a = a - ws[76192];
      a = a - ws[76224];
      a = a - ws[76256];
      a = a - ws[76288];
      yout[3488] = a;
    }
    {
      double a = 0.43 * ws[62944];
      a = a - ws[66016];
      a = a - ws[67360];
      a = a - ws[68544];
      a = a - ws[69728];
      a = a - ws[70848];
      a = fma(0.43, ws[71872], a);
      yout[3520] = a;
    }
    {
      double a = -ws[71872];
      a = a - ws[71904];
      a = a - ws[71936];
      a = fma(0.895, ws[72032], a);
      a = fma(0.925, ws[72064], a);
      a = fma(0.463, ws[72128], a);
      a = fma(0.74, ws[72160], a);
      a = fma(0.62, ws[72192], a);
      a = fma(0.9, ws[72224], a);
      yout[3552] = a;
    }
    {
      double a = -ws[63168];
      a = a - ws[64288];
      a = fma(0.2495, ws[65376], a);
      a = fma(0.25, ws[67936], a);
      a = fma(0.25, ws[69120], a);
      a = fma(0.25, ws[70368], a);
      a = fma(0.2, ws[72416], a);
      yout[3584] = a;
    }
    {
      double a = 2.81e-05 * ws[61856];
      a = fma(0.00134, ws[61888], a);
      a = fma(0.152, ws[63232], a);
      a = fma(0.2, ws[63264], a);
      a = fma(0.152, ws[64768], a);
      a = fma(0.2, ws[64800], a);
      a = fma(0.149, ws[71808], a);
      a = fma(0.00101, ws[71840], a);
      a = fma(0.04, ws[72352], a);
      yout[3616] = a;
    }
    {
      double a = 0.17 * ws[63232];
      a = fma(0.16, ws[63264], a);
      a = fma(0.85, ws[64768], a);
      a = fma(0.08, ws[64800], a);
      a = a - ws[66176];
      a = a - ws[67456];
      a = a - ws[68704];
      a = a - ws[69888];
      a = a - ws[71008];
      yout[3648] = a;
    }
    {
      double a = -ws[63680];
      a = fma(0.11, ws[64288], a);
      a = fma(0.36, ws[65792], a);
      a = fma(0.1, ws[67136], a);
      a = fma(0.41, ws[67168], a);
      a = fma(0.41, ws[67200], a);
      yout[3680] = a;
    }
    {
      double a = 0.055 * ws[64480];
      a = a - ws[65728];
      a = a - ws[67072];
      a = a - ws[68320];
      a = a - ws[69504];
      a = a - ws[71680];
      a = a - ws[71712];
      a = a - ws[71744];
      yout[3712] = a;
    }
    {
      double a = 0.025 * ws[62592];
      a = a - ws[65536];
      a = a - ws[66880];
      a = a - ws[68128];
      a = a - ws[69312];
      a = a - ws[71392];
      a = a - ws[71424];
      a = a - ws[71456];
      yout[3744] = a;
    }
    {
      double a = 1.0 * ws[62880];
      a = a - ws[65952];
      a = a - ws[67296];
      a = a - ws[68480];
      a = a - ws[69664];
      a = a - ws[70784];
      a = fma(0.0794, ws[75552], a);
      a = fma(0.1068, ws[75712], a);
      yout[3776] = a;
    }
    {
      double a = 1.0 * ws[63296];
      a = a - ws[64320];
      a = fma(1.0, ws[64832], a);
      a = fma(1.0, ws[66208], a);
      a = a - ws[66464];
      a = fma(1.0, ws[68736], a);
      a = fma(1.0, ws[69920], a);
      a = fma(1.0, ws[71040], a);
      yout[3808] = a;
    }
    {
      double a = 0.025 * ws[64448];
      a = a - ws[65600];
      a = a - ws[66944];
      a = a - ws[68192];
      a = a - ws[69376];
      a = a - ws[71584];
      a = a - ws[71616];
      a = a - ws[71648];
      yout[3840] = a;
    }
    {
      double a = -ws[63008];
      a = a - ws[64192];
      a = a - ws[64672];
      a = fma(0.333, ws[72000], a);
      a = fma(0.019, ws[72128], a);
      a = fma(0.015, ws[72160], a);
      yout[3872] = a;
    }
    {
      double a = 0.44 * ws[63520];
      a = fma(0.44, ws[63552], a);
      a = fma(1.0, ws[73344], a);
      a = a - ws[73568];
      a = a - ws[73792];
      a = a - ws[74016];
      yout[3904] = a;
    }
    {
      double a = 0.055 * ws[62624];
      a = a - ws[65664];
      a = a - ws[67008];
      a = a - ws[68256];
      a = a - ws[69440];
      a = a - ws[71488];
      a = a - ws[71520];
      a = a - ws[71552];
      yout[3936] = a;
    }
    {
      double a = 0.0369 * ws[75584];
      a = fma(0.0748, ws[75680], a);
      a = fma(0.0421, ws[75744], a);
      a = fma(0.0911, ws[75808], a);
      a = fma(0.0595, ws[75840], a);
      a = fma(0.0661, ws[75872], a);
      a = fma(0.0745, ws[75904], a);
      a = fma(0.1398, ws[75936], a);
      a = a - ws[75968];
      a = fma(0.0957, ws[75968], a);
      yout[3968] = a;
    }
    {
      double a = 1.0 * ws[60960];
      a = fma(1.0, ws[60992], a);
      a = a - ws[61024];
      a = fma(0.09, ws[62176], a);
      a = fma(0.068, ws[63936], a);
      a = fma(0.026, ws[63968], a);
      a = fma(0.255, ws[64000], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.02, ws[64064], a);
      yout[4000] = a;
    }
    {
      double a = 0.8 * ws[64352];
      a = fma(0.43, ws[64384], a);
      a = fma(0.11, ws[64416], a);
      a = a - ws[66272];
      a = a - ws[67584];
      a = a - ws[68800];
      a = a - ws[69984];
      a = a - ws[71104];
      a = a - ws[71200];
      a = a - ws[71200];
      a = a - ws[71232];
      a = fma(0.9, ws[72224], a);
      yout[4032] = a;
    }
    {
      double a = 0.2 * ws[64352];
      a = fma(0.57, ws[64384], a);
      a = fma(0.89, ws[64416], a);
      a = a - ws[66304];
      a = a - ws[67616];
      a = a - ws[68832];
      a = a - ws[70016];
      a = a - ws[71136];
      a = a - ws[71232];
      a = a - ws[71264];
      a = a - ws[71264];
      a = fma(0.1, ws[72224], a);
      yout[4064] = a;
    }
    {
      double a = -ws[63520];
      a = fma(0.0715, ws[65504], a);
      a = fma(0.762, ws[66848], a);
      a = fma(0.9, ws[66976], a);
      a = fma(0.75, ws[67104], a);
      a = fma(0.9, ws[67136], a);
      a = fma(0.0845, ws[68096], a);
      a = fma(0.091, ws[69280], a);
      a = fma(0.091, ws[70528], a);
      yout[4096] = a;
    }
    {
      double a = 0.3 * ws[62176];
      a = fma(0.028, ws[62208], a);
      a = fma(0.03, ws[62240], a);
      a = fma(0.18, ws[62304], a);
      a = fma(0.03, ws[62368], a);
      a = fma(0.57, ws[62560], a);
      a = a - ws[62944];
      a = a - ws[64128];
      a = a - ws[64640];
      a = fma(0.159, ws[68064], a);
      a = fma(0.219, ws[69248], a);
      a = fma(0.318, ws[70496], a);
      yout[4128] = a;
    }
    {
      double a = 0.975 * ws[62592];
      a = a - ws[65504];
      a = a - ws[66848];
      a = a - ws[68096];
      a = a - ws[69280];
      a = a - ws[70528];
      a = a - ws[71392];
      a = a - ws[71488];
      a = a - ws[71584];
      a = a - ws[71680];
      yout[4160] = a;
    }
    {
      double a = 0.945 * ws[62624];
      a = a - ws[65632];
      a = a - ws[66976];
      a = a - ws[68224];
      a = a - ws[69408];
      a = a - ws[70560];
      a = a - ws[71424];
      a = a - ws[71520];
      a = a - ws[71616];
      a = a - ws[71712];
      yout[4192] = a;
    }
    {
      double a = 0.0325 * ws[75584];
      a = fma(0.0138, ws[75648], a);
      a = fma(0.0347, ws[75680], a);
      a = fma(0.0371, ws[75744], a);
      a = fma(0.0174, ws[75776], a);
      a = fma(0.0423, ws[75808], a);
      a = fma(0.0523, ws[75840], a);
      a = fma(0.0582, ws[75872], a);
      a = fma(0.0479, ws[75904], a);
      a = a - ws[75936];
      a = fma(0.0062, ws[75936], a);
      a = fma(0.0432, ws[75968], a);
      yout[4224] = a;
    }
    {
      double a = 1.0 * ws[64896];
      a = fma(1.0, ws[64928], a);
      a = fma(1.0, ws[65536], a);
      a = fma(1.0, ws[65600], a);
      a = fma(1.0, ws[65664], a);
      a = fma(1.0, ws[65728], a);
      a = fma(0.64, ws[65760], a);
      a = fma(1.0, ws[66880], a);
      a = fma(1.0, ws[66944], a);
      a = fma(1.0, ws[67008], a);
      a = fma(1.0, ws[67072], a);
      a = fma(0.25, ws[67104], a);
      a = fma(1.0, ws[68128], a);
      a = fma(1.0, ws[68192], a);
      a = fma(1.0, ws[68256], a);
      a = fma(1.0, ws[68320], a);
      a = fma(1.0, ws[69312], a);
      a = fma(1.0, ws[69376], a);
      a = fma(1.0, ws[69440], a);
      a = fma(1.0, ws[69504], a);
      a = fma(0.96, ws[71392], a);
      a = fma(0.96, ws[71424], a);
      a = fma(0.96, ws[71456], a);
      a = fma(0.96, ws[71488], a);
      a = fma(0.96, ws[71520], a);
      a = fma(0.96, ws[71552], a);
      a = fma(0.96, ws[71584], a);
      a = fma(0.96, ws[71616], a);
      a = fma(0.96, ws[71648], a);
      a = fma(0.96, ws[71680], a);
      a = fma(0.96, ws[71712], a);
      a = fma(0.96, ws[71744], a);
      yout[4256] = a;
    }
    {
      double a = 1.0 * ws[62240];
      a = a - ws[62272];
      a = a - ws[62304];
      a = fma(1.0, ws[62336], a);
      a = a - ws[68064];
      a = a - ws[69248];
      a = a - ws[70496];
      a = a - ws[71456];
      a = a - ws[71552];
      a = a - ws[71648];
      a = a - ws[71744];
      yout[4288] = a;
    }
    {
      double a = -ws[63136];
      a = a - ws[64256];
      a = fma(0.2495, ws[65376], a);
      a = fma(0.5984, ws[65440], a);
      a = fma(0.4564, ws[65472], a);
      a = fma(0.25, ws[67936], a);
      a = fma(0.5996, ws[68000], a);
      a = fma(0.4573, ws[68032], a);
      a = fma(0.25, ws[69120], a);
      a = fma(0.5996, ws[69184], a);
      a = fma(0.4573, ws[69216], a);
      a = fma(0.25, ws[70368], a);
      a = fma(0.5996, ws[70432], a);
      a = fma(0.4573, ws[70464], a);
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[4320] = a;
    }
    {
      double a = 0.35 * ws[62016];
      a = fma(0.28, ws[62176], a);
      a = a - ws[63616];
      a = fma(0.37, ws[63904], a);
      a = fma(0.03, ws[63936], a);
      a = fma(0.028, ws[64000], a);
      a = fma(0.15, ws[64064], a);
      a = fma(0.45, ws[64128], a);
      a = fma(0.07, ws[64160], a);
      a = fma(0.044, ws[64192], a);
      a = fma(0.25, ws[64288], a);
      yout[4352] = a;
    }
    {
      double a = -ws[63840];
      a = a - ws[64096];
      a = a - ws[64512];
      a = fma(0.237, ws[65504], a);
      a = fma(0.2345, ws[65568], a);
      a = fma(0.23, ws[65632], a);
      a = fma(0.57, ws[65696], a);
      a = fma(0.36, ws[65760], a);
      a = fma(0.64, ws[65792], a);
      a = fma(0.461, ws[66912], a);
      a = fma(0.77, ws[67040], a);
      a = fma(0.341, ws[68160], a);
      a = fma(0.69, ws[68288], a);
      a = fma(0.175, ws[69344], a);
      a = fma(0.54, ws[69472], a);
      a = fma(0.175, ws[70592], a);
      a = fma(0.54, ws[70624], a);
      yout[4384] = a;
    }
    {
      double a = 0.28 * ws[73536];
      a = fma(1.0, ws[73952], a);
      a = fma(1.0, ws[74176], a);
      a = fma(0.14, ws[74368], a);
      a = fma(0.86, ws[74400], a);
      a = fma(1.0, ws[74624], a);
      a = fma(1.0, ws[74784], a);
      a = fma(0.0096, ws[75584], a);
      a = a - ws[75680];
      a = fma(0.007, ws[75680], a);
      a = fma(0.0046, ws[75744], a);
      a = fma(0.0758, ws[75808], a);
      a = fma(0.0013, ws[75840], a);
      yout[4416] = a;
    }
    {
      double a = -ws[63200];
      a = fma(0.02, ws[63936], a);
      a = fma(0.0, ws[65376], a);
      a = fma(0.0852, ws[65408], a);
      a = fma(0.0481, ws[65440], a);
      a = fma(0.0852, ws[65472], a);
      a = fma(0.0, ws[67936], a);
      a = fma(0.0854, ws[67968], a);
      a = fma(0.0482, ws[68000], a);
      a = fma(0.0854, ws[68032], a);
      a = fma(0.0, ws[69120], a);
      a = fma(0.0854, ws[69152], a);
      a = fma(0.0482, ws[69184], a);
      a = fma(0.0854, ws[69216], a);
      a = fma(0.0, ws[70368], a);
      a = fma(0.0854, ws[70400], a);
      a = fma(0.0482, ws[70432], a);
      a = fma(0.0854, ws[70464], a);
      a = fma(0.0594, ws[75008], a);
      a = fma(0.0595, ws[75040], a);
      a = fma(0.0595, ws[75072], a);
      a = fma(0.0595, ws[75104], a);
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      a = fma(1.0, ws[76256], a);
      a = fma(1.0, ws[76288], a);
      yout[4448] = a;
    }
    {
      double a = -ws[62816];
      a = fma(0.03, ws[63936], a);
      a = fma(0.11, ws[63968], a);
      a = fma(0.165, ws[65216], a);
      a = fma(0.217, ws[65248], a);
      a = fma(0.06, ws[65312], a);
      a = fma(0.2, ws[65344], a);
      a = fma(0.0865, ws[65504], a);
      a = fma(0.039, ws[66848], a);
      a = fma(0.067, ws[68096], a);
      a = fma(0.1165, ws[69280], a);
      a = fma(0.095, ws[70208], a);
      a = fma(0.247, ws[70240], a);
      a = fma(0.09, ws[70304], a);
      a = fma(0.2, ws[70336], a);
      a = fma(0.1165, ws[70528], a);
      yout[4480] = a;
    }
    {
      double a = 0.499 * ws[65376];
      a = fma(0.3651, ws[65408], a);
      a = fma(0.3515, ws[65440], a);
      a = fma(0.4564, ws[65472], a);
      a = fma(0.5, ws[67936], a);
      a = fma(0.3659, ws[67968], a);
      a = fma(0.3522, ws[68000], a);
      a = fma(0.4573, ws[68032], a);
      a = fma(0.5, ws[69120], a);
      a = fma(0.3659, ws[69152], a);
      a = fma(0.3522, ws[69184], a);
      a = fma(0.4573, ws[69216], a);
      a = fma(0.5, ws[70368], a);
      a = fma(0.3659, ws[70400], a);
      a = fma(0.3522, ws[70432], a);
      a = fma(0.4573, ws[70464], a);
      a = fma(0.92, ws[72288], a);
      a = fma(0.4, ws[72320], a);
      a = a - ws[72352];
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[4512] = a;
    }
    {
      double a = -ws[62656];
      a = fma(0.27, ws[63840], a);
      a = fma(0.2535, ws[64000], a);
      a = fma(0.27, ws[64096], a);
      a = fma(0.27, ws[64512], a);
      a = fma(0.195, ws[65504], a);
      a = fma(0.6045, ws[65568], a);
      a = fma(0.1885, ws[66848], a);
      a = fma(0.455, ws[66912], a);
      a = fma(0.273, ws[68096], a);
      a = fma(0.533, ws[68160], a);
      a = fma(0.2535, ws[69280], a);
      a = fma(0.65, ws[69344], a);
      a = fma(0.2535, ws[70528], a);
      a = fma(0.65, ws[70592], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71680], a);
      yout[4544] = a;
    }
    {
      double a = -ws[62688];
      a = fma(0.66, ws[64032], a);
      a = a - ws[64064];
      a = fma(0.1285, ws[65504], a);
      a = fma(0.77, ws[65632], a);
      a = fma(0.43, ws[65696], a);
      a = fma(0.039, ws[66848], a);
      a = fma(0.1, ws[66976], a);
      a = fma(0.23, ws[67040], a);
      a = fma(0.2205, ws[68096], a);
      a = fma(1.0, ws[68224], a);
      a = fma(0.31, ws[68288], a);
      a = fma(0.1725, ws[69280], a);
      a = fma(1.0, ws[69408], a);
      a = fma(0.46, ws[69472], a);
      a = fma(0.1725, ws[70528], a);
      a = fma(1.0, ws[70560], a);
      a = fma(0.46, ws[70624], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71712], a);
      yout[4576] = a;
    }
    {
      double a = -ws[63552];
      a = fma(0.6747, ws[66784], a);
      a = fma(0.6341, ws[66816], a);
      a = fma(0.0308, ws[75552], a);
      a = fma(0.0026, ws[75584], a);
      a = fma(0.0163, ws[75680], a);
      a = fma(0.0105, ws[75744], a);
      a = fma(0.0154, ws[75776], a);
      a = fma(0.0066, ws[75808], a);
      a = fma(0.0041, ws[75840], a);
      a = fma(0.0506, ws[75872], a);
      a = fma(0.0607, ws[75904], a);
      a = fma(0.0216, ws[75936], a);
      a = fma(0.0316, ws[75968], a);
      a = a - ws[76000];
      yout[4608] = a;
    }
    {
      double a = 0.0001 * ws[75008];
      a = fma(0.0152, ws[75552], a);
      a = fma(0.0298, ws[75584], a);
      a = a - ws[75648];
      a = fma(0.0076, ws[75648], a);
      a = fma(0.0305, ws[75680], a);
      a = fma(0.0183, ws[75712], a);
      a = fma(0.0657, ws[75744], a);
      a = fma(0.0452, ws[75776], a);
      a = fma(0.1193, ws[75808], a);
      a = fma(0.1118, ws[75840], a);
      a = fma(0.0489, ws[75872], a);
      a = fma(0.0246, ws[75904], a);
      a = fma(0.0146, ws[75936], a);
      a = fma(0.0049, ws[75968], a);
      yout[4640] = a;
    }
    {
      double a = 0.1 * ws[62176];
      a = fma(0.57, ws[62944], a);
      a = fma(0.21, ws[63168], a);
      a = fma(1.0, ws[63584], a);
      a = fma(0.32, ws[64640], a);
      a = fma(1.0, ws[64864], a);
      a = a - ws[65088];
      a = fma(1.0, ws[65120], a);
      a = a - ws[65984];
      a = a - ws[67328];
      a = a - ws[68512];
      a = a - ws[69696];
      a = a - ws[70816];
      a = fma(0.57, ws[71872], a);
      a = fma(0.32, ws[71936], a);
      yout[4672] = a;
    }
    {
      double a = 0.28 * ws[73472];
      a = fma(1.0, ws[73888], a);
      a = fma(1.0, ws[74112], a);
      a = fma(0.86, ws[74336], a);
      a = fma(1.0, ws[74560], a);
      a = fma(0.0199, ws[75584], a);
      a = fma(0.0075, ws[75648], a);
      a = fma(0.0352, ws[75680], a);
      a = fma(0.0215, ws[75744], a);
      a = a - ws[75808];
      a = fma(0.0118, ws[75808], a);
      a = fma(0.0068, ws[75840], a);
      a = fma(0.0013, ws[75872], a);
      a = fma(0.0073, ws[75904], a);
      a = fma(0.0031, ws[75936], a);
      a = fma(0.0022, ws[75968], a);
      yout[4704] = a;
    }
    {
      double a = 0.14 * ws[62176];
      a = fma(0.26, ws[62208], a);
      a = fma(0.51, ws[62304], a);
      a = fma(0.13, ws[62368], a);
      a = fma(0.15, ws[62432], a);
      a = fma(0.43, ws[62560], a);
      a = a - ws[62976];
      a = a - ws[64160];
      a = fma(0.25, ws[68064], a);
      a = fma(0.305, ws[69248], a);
      a = fma(0.5, ws[70496], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.231, ws[72128], a);
      a = fma(0.185, ws[72160], a);
      yout[4736] = a;
    }
    {
      double a = 0.0357 * ws[75360];
      a = fma(0.0001, ws[75392], a);
      a = a - ws[75520];
      a = fma(0.0854, ws[75520], a);
      a = fma(0.464, ws[75552], a);
      a = fma(0.1041, ws[75584], a);
      a = fma(0.2036, ws[75616], a);
      a = fma(0.2792, ws[75648], a);
      a = fma(0.0074, ws[75680], a);
      a = fma(0.2822, ws[75712], a);
      a = fma(0.0659, ws[75744], a);
      a = fma(0.1778, ws[75776], a);
      a = fma(0.0023, ws[75808], a);
      a = fma(0.0445, ws[75840], a);
      a = fma(0.0317, ws[75872], a);
      a = fma(0.0117, ws[75904], a);
      a = fma(0.1188, ws[76000], a);
      yout[4768] = a;
    }
    {
      double a = 0.77 * ws[62656];
      a = fma(0.17, ws[62688], a);
      a = fma(1.0, ws[62784], a);
      a = fma(0.2805, ws[64000], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.6, ws[64224], a);
      a = fma(0.6, ws[64256], a);
      a = fma(1.0, ws[64608], a);
      a = a - ws[65024];
      a = fma(1.0, ws[65056], a);
      a = a - ws[65856];
      a = a - ws[67200];
      a = a - ws[68384];
      a = a - ws[69568];
      a = a - ws[70112];
      a = a - ws[70112];
      a = a - ws[70688];
      a = a - ws[71328];
      yout[4800] = a;
    }
    {
      double a = 0.018 * ws[72608];
      a = fma(1.0, ws[73984], a);
      a = fma(1.0, ws[74208], a);
      a = fma(0.14, ws[74400], a);
      a = fma(1.0, ws[74432], a);
      a = fma(1.0, ws[74656], a);
      a = fma(1.0, ws[74816], a);
      a = fma(1.0, ws[74848], a);
      a = fma(1.0, ws[74880], a);
      a = a - ws[75584];
      a = fma(0.2141, ws[75584], a);
      a = fma(0.0088, ws[75648], a);
      a = fma(0.7261, ws[75680], a);
      a = fma(0.1156, ws[75744], a);
      a = fma(0.0004, ws[75776], a);
      a = fma(0.3349, ws[75808], a);
      a = fma(0.0104, ws[75840], a);
      a = fma(0.0009, ws[75872], a);
      a = fma(0.0006, ws[75936], a);
      yout[4832] = a;
    }
    {
      double a = 0.0357 * ws[74976];
      a = fma(0.0357, ws[75168], a);
      a = fma(0.0001, ws[75200], a);
      a = a - ws[75552];
      a = fma(0.1977, ws[75552], a);
      a = fma(0.5638, ws[75584], a);
      a = fma(0.0071, ws[75616], a);
      a = fma(0.4025, ws[75648], a);
      a = fma(0.119, ws[75680], a);
      a = fma(0.1165, ws[75712], a);
      a = fma(0.4579, ws[75744], a);
      a = fma(0.1924, ws[75776], a);
      a = fma(0.134, ws[75808], a);
      a = fma(0.1726, ws[75840], a);
      a = fma(0.0765, ws[75872], a);
      a = fma(0.0167, ws[75904], a);
      a = fma(0.0103, ws[75936], a);
      a = fma(0.0008, ws[76000], a);
      yout[4864] = a;
    }
    {
      double a = 0.0008 * ws[65376];
      a = fma(0.0006, ws[65408], a);
      a = fma(0.3979, ws[66720], a);
      a = fma(0.2805, ws[66752], a);
      a = fma(0.0121, ws[75552], a);
      a = fma(0.0153, ws[75584], a);
      a = a - ws[75616];
      a = fma(0.0319, ws[75648], a);
      a = fma(0.0122, ws[75680], a);
      a = fma(0.032, ws[75712], a);
      a = fma(0.0325, ws[75744], a);
      a = fma(0.074, ws[75776], a);
      a = fma(0.008, ws[75808], a);
      a = fma(0.0513, ws[75840], a);
      a = fma(0.0526, ws[75872], a);
      a = fma(0.048, ws[75904], a);
      a = fma(0.009, ws[75936], a);
      a = fma(0.0061, ws[75968], a);
      a = fma(0.039, ws[76000], a);
      yout[4896] = a;
    }
    {
      double a = 0.0006 * ws[65440];
      a = fma(0.0006, ws[65472], a);
      a = fma(0.2771, ws[66784], a);
      a = fma(0.2805, ws[66816], a);
      a = fma(1.0, ws[72512], a);
      a = fma(0.0624, ws[75552], a);
      a = fma(0.0189, ws[75584], a);
      a = fma(0.0194, ws[75648], a);
      a = fma(0.0291, ws[75680], a);
      a = a - ws[75712];
      a = fma(0.0011, ws[75712], a);
      a = fma(0.0307, ws[75744], a);
      a = fma(0.0631, ws[75776], a);
      a = fma(0.0292, ws[75808], a);
      a = fma(0.1337, ws[75840], a);
      a = fma(0.155, ws[75872], a);
      a = fma(0.0881, ws[75904], a);
      a = fma(0.0702, ws[75936], a);
      a = fma(0.0224, ws[75968], a);
      a = fma(0.0114, ws[76000], a);
      yout[4928] = a;
    }
    {
      double a = 1.0 * ws[72672];
      a = fma(0.28, ws[73504], a);
      a = fma(1.0, ws[73920], a);
      a = fma(1.0, ws[74144], a);
      a = fma(0.14, ws[74336], a);
      a = fma(0.86, ws[74368], a);
      a = fma(1.0, ws[74592], a);
      a = fma(1.0, ws[74752], a);
      a = fma(0.9048, ws[75168], a);
      a = fma(0.0456, ws[75584], a);
      a = fma(0.0104, ws[75648], a);
      a = fma(0.0454, ws[75680], a);
      a = a - ws[75744];
      a = fma(0.0024, ws[75744], a);
      a = fma(0.0007, ws[75776], a);
      a = fma(0.0766, ws[75808], a);
      a = fma(0.0403, ws[75840], a);
      a = fma(0.0155, ws[75872], a);
      a = fma(0.0153, ws[75936], a);
      yout[4960] = a;
    }
    {
      double a = 0.247 * ws[72736];
      a = fma(0.14, ws[74304], a);
      a = fma(1.0, ws[74720], a);
      a = fma(0.9048, ws[74976], a);
      a = fma(0.0018, ws[75200], a);
      a = fma(0.9048, ws[75360], a);
      a = fma(0.0388, ws[75552], a);
      a = fma(0.0314, ws[75584], a);
      a = fma(0.051, ws[75648], a);
      a = fma(0.0234, ws[75680], a);
      a = fma(0.0395, ws[75744], a);
      a = a - ws[75776];
      a = fma(0.0006, ws[75776], a);
      a = fma(0.0277, ws[75808], a);
      a = fma(0.0511, ws[75840], a);
      a = fma(0.1051, ws[75872], a);
      a = fma(0.0916, ws[75904], a);
      a = fma(0.1038, ws[75936], a);
      a = fma(0.0503, ws[75968], a);
      yout[4992] = a;
    }
    {
      double a = 1.0 * ws[61152];
      a = fma(1.0, ws[61312], a);
      a = a - ws[61344];
      a = fma(0.3, ws[61408], a);
      a = fma(2.0, ws[61600], a);
      a = fma(1.0, ws[62528], a);
      a = fma(1.0, ws[64544], a);
      a = fma(1.0, ws[64576], a);
      a = fma(1.0, ws[64608], a);
      a = fma(0.32, ws[64640], a);
      a = fma(1.0, ws[64704], a);
      a = fma(1.0, ws[64736], a);
      a = fma(0.424, ws[64768], a);
      a = fma(0.4, ws[64800], a);
      a = fma(1.0, ws[64832], a);
      a = fma(0.32, ws[71936], a);
      a = fma(2.0, ws[72832], a);
      a = fma(0.5, ws[72864], a);
      a = fma(1.0, ws[72928], a);
      a = fma(1.0, ws[73120], a);
      a = fma(1.0, ws[76064], a);
      a = fma(1.0, ws[76096], a);
      yout[5024] = a;
    }
    {
      double a = 1.0 * ws[62528];
      a = a - ws[63392];
      a = fma(0.25, ws[67776], a);
      a = fma(0.25, ws[67808], a);
      a = fma(0.25, ws[67872], a);
      a = fma(0.25, ws[67904], a);
      a = fma(0.25, ws[68064], a);
      a = fma(0.25, ws[68416], a);
      a = fma(0.25, ws[68448], a);
      a = fma(0.25, ws[68480], a);
      a = fma(0.25, ws[68512], a);
      a = fma(0.25, ws[68544], a);
      a = fma(0.25, ws[68576], a);
      a = fma(0.25, ws[68608], a);
      a = fma(0.25, ws[68832], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71680], a);
      a = fma(0.48, ws[71712], a);
      a = fma(0.48, ws[71744], a);
      yout[5056] = a;
    }
    {
      double a = 0.28 * ws[73440];
      a = fma(1.0, ws[73856], a);
      a = fma(1.0, ws[74080], a);
      a = fma(0.14, ws[74272], a);
      a = fma(0.86, ws[74304], a);
      a = fma(1.0, ws[74528], a);
      a = fma(1.0, ws[74912], a);
      a = fma(0.0018, ws[75008], a);
      a = fma(0.0018, ws[75392], a);
      a = fma(0.0491, ws[75552], a);
      a = fma(0.0459, ws[75584], a);
      a = fma(0.0512, ws[75648], a);
      a = fma(0.0624, ws[75680], a);
      a = fma(0.066, ws[75712], a);
      a = fma(0.0539, ws[75744], a);
      a = fma(0.0227, ws[75776], a);
      a = fma(0.0651, ws[75808], a);
      a = a - ws[75840];
      a = fma(0.0236, ws[75840], a);
      a = fma(0.0535, ws[75872], a);
      a = fma(0.0972, ws[75904], a);
      a = fma(0.165, ws[75936], a);
      a = fma(0.0879, ws[75968], a);
      yout[5088] = a;
    }
    {
      double a = 1.0 * ws[61888];
      a = fma(0.02, ws[63936], a);
      a = a - ws[65248];
      a = a - ws[66592];
      a = a - ws[67808];
      a = a - ws[68992];
      a = a - ws[70240];
      a = fma(0.0794, ws[75552], a);
      a = fma(0.0925, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.1753, ws[75648], a);
      a = fma(0.0537, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.1055, ws[75744], a);
      a = fma(0.222, ws[75776], a);
      a = fma(0.0654, ws[75808], a);
      a = fma(0.1489, ws[75840], a);
      a = fma(0.1656, ws[75872], a);
      a = fma(0.173, ws[75904], a);
      a = fma(0.128, ws[75936], a);
      a = fma(0.1544, ws[75968], a);
      yout[5120] = a;
    }
    {
      double a = 1.0 * ws[62848];
      a = a - ws[65920];
      a = a - ws[67264];
      a = a - ws[68448];
      a = a - ws[69632];
      a = a - ws[70752];
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5152] = a;
    }
    {
      double a = -ws[60608];
      a = a - ws[60640];
      a = a - ws[60672];
      a = a - ws[60704];
      a = fma(1.0, ws[60736], a);
      a = a - ws[60768];
      a = a - ws[62176];
      a = a - ws[63904];
      a = a - ws[63936];
      a = a - ws[63968];
      a = a - ws[64000];
      a = a - ws[64032];
      a = a - ws[64064];
      a = a - ws[64096];
      a = a - ws[64128];
      a = a - ws[64160];
      a = a - ws[64192];
      a = a - ws[64224];
      a = a - ws[64256];
      a = a - ws[64288];
      a = a - ws[64320];
      a = a - ws[71904];
      a = a - ws[72192];
      a = a - ws[72384];
      a = a - ws[72608];
      yout[5184] = a;
    }
    {
      double a = 0.07 * ws[63488];
      a = fma(0.07, ws[63520], a);
      a = fma(0.07, ws[63552], a);
      a = fma(0.35, ws[63680], a);
      a = fma(1.0, ws[63712], a);
      a = fma(1.0, ws[63744], a);
      a = fma(0.01, ws[64160], a);
      a = fma(0.1, ws[64192], a);
      a = fma(0.6, ws[64224], a);
      a = fma(0.6, ws[64256], a);
      a = fma(0.68, ws[64640], a);
      a = fma(1.0, ws[64672], a);
      a = fma(0.089, ws[65216], a);
      a = fma(0.235, ws[65248], a);
      a = fma(0.16, ws[65952], a);
      a = fma(0.7, ws[66048], a);
      a = a - ws[66368];
      a = a - ws[67680];
      a = fma(0.026, ws[67776], a);
      a = fma(0.191, ws[67808], a);
      a = fma(1.16, ws[68576], a);
      a = a - ws[68896];
      a = fma(0.026, ws[68960], a);
      a = fma(0.191, ws[68992], a);
      a = fma(1.16, ws[69760], a);
      a = a - ws[70080];
      a = fma(0.092, ws[70208], a);
      a = fma(0.485, ws[70240], a);
      a = fma(0.7, ws[70880], a);
      a = a - ws[71296];
      a = a - ws[71328];
      a = a - ws[71360];
      a = a - ws[71360];
      a = fma(0.68, ws[71936], a);
      yout[5216] = a;
    }
    {
      double a = 0.05 * ws[62240];
      a = fma(0.04, ws[62368], a);
      a = fma(1.0, ws[62912], a);
      a = a - ws[63072];
      a = fma(0.01, ws[63104], a);
      a = fma(0.01, ws[63136], a);
      a = fma(0.01, ws[63168], a);
      a = fma(0.5, ws[64128], a);
      a = fma(0.54, ws[64160], a);
      a = fma(0.003, ws[64192], a);
      a = fma(0.08, ws[64224], a);
      a = fma(0.08, ws[64256], a);
      a = fma(0.68, ws[64640], a);
      a = a - ws[64736];
      a = fma(0.3651, ws[65408], a);
      a = fma(0.247, ws[65440], a);
      a = fma(0.3651, ws[65472], a);
      a = fma(0.54, ws[65952], a);
      a = fma(0.3, ws[66048], a);
      a = fma(0.21, ws[66080], a);
      a = fma(0.3659, ws[67968], a);
      a = fma(0.2475, ws[68000], a);
      a = fma(0.3659, ws[68032], a);
      a = fma(0.5, ws[68576], a);
      a = fma(0.105, ws[68608], a);
      a = fma(0.3659, ws[69152], a);
      a = fma(0.2475, ws[69184], a);
      a = fma(0.3659, ws[69216], a);
      a = fma(0.5, ws[69760], a);
      a = fma(0.105, ws[69792], a);
      a = fma(0.3659, ws[70400], a);
      a = fma(0.2475, ws[70432], a);
      a = fma(0.3659, ws[70464], a);
      a = fma(0.3, ws[70880], a);
      a = fma(0.21, ws[70912], a);
      a = fma(0.68, ws[71936], a);
      a = a - ws[72800];
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[5248] = a;
    }
    {
      double a = -ws[62848];
      a = fma(0.13, ws[63136], a);
      a = fma(0.06, ws[63936], a);
      a = fma(0.042, ws[65216], a);
      a = fma(0.033, ws[65248], a);
      a = fma(0.13, ws[65312], a);
      a = fma(0.075, ws[70208], a);
      a = fma(0.063, ws[70240], a);
      a = fma(0.18, ws[70304], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5280] = a;
    }
    {
      double a = 0.0012 * ws[65376];
      a = fma(0.0013, ws[65408], a);
      a = fma(0.28, ws[73376], a);
      a = fma(1.0, ws[74240], a);
      a = fma(0.16, ws[74944], a);
      a = fma(0.0595, ws[74976], a);
      a = fma(0.0001, ws[75008], a);
      a = fma(0.0594, ws[75200], a);
      a = fma(0.0595, ws[75232], a);
      a = fma(0.0595, ws[75264], a);
      a = fma(0.0595, ws[75296], a);
      a = fma(0.0595, ws[75392], a);
      a = fma(0.0595, ws[75424], a);
      a = fma(0.0595, ws[75456], a);
      a = fma(0.0595, ws[75488], a);
      a = fma(0.0183, ws[75552], a);
      a = fma(0.0455, ws[75584], a);
      a = fma(0.0512, ws[75648], a);
      a = fma(0.0509, ws[75680], a);
      a = fma(0.0246, ws[75712], a);
      a = fma(0.0519, ws[75744], a);
      a = fma(0.0649, ws[75776], a);
      a = fma(0.0668, ws[75808], a);
      a = fma(0.0733, ws[75840], a);
      a = fma(0.0426, ws[75872], a);
      a = a - ws[75904];
      a = fma(0.0024, ws[75904], a);
      a = fma(0.0724, ws[75936], a);
      a = fma(0.1463, ws[75968], a);
      yout[5312] = a;
    }
    {
      double a = -ws[62912];
      a = fma(1.0, ws[63776], a);
      a = fma(1.0, ws[63872], a);
      a = fma(0.01, ws[63936], a);
      a = fma(0.044, ws[63968], a);
      a = fma(0.272, ws[65248], a);
      a = fma(0.02, ws[65344], a);
      a = fma(1.0, ws[66016], a);
      a = fma(0.32, ws[66176], a);
      a = fma(0.016, ws[68064], a);
      a = fma(0.5, ws[68544], a);
      a = fma(0.32, ws[68704], a);
      a = fma(0.5, ws[69728], a);
      a = fma(0.32, ws[69888], a);
      a = fma(0.275, ws[70240], a);
      a = fma(0.04, ws[70336], a);
      a = fma(0.033, ws[70496], a);
      a = fma(1.0, ws[70848], a);
      a = fma(0.32, ws[71008], a);
      a = fma(0.613, ws[72448], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      yout[5344] = a;
    }
    {
      double a = 0.65 * ws[62016];
      a = fma(0.02, ws[62368], a);
      a = a - ws[63040];
      a = fma(0.1, ws[63104], a);
      a = fma(0.1, ws[63136], a);
      a = fma(0.27, ws[63168], a);
      a = fma(0.491, ws[64192], a);
      a = fma(0.05, ws[64224], a);
      a = fma(0.05, ws[64256], a);
      a = fma(0.48, ws[64288], a);
      a = a - ws[64704];
      a = fma(0.998, ws[65376], a);
      a = fma(0.5477, ws[65408], a);
      a = fma(0.7029, ws[65440], a);
      a = fma(0.5477, ws[65472], a);
      a = fma(0.18, ws[66080], a);
      a = fma(0.68, ws[66176], a);
      a = fma(1.0, ws[66240], a);
      a = fma(1.0, ws[66336], a);
      a = fma(0.05, ws[67776], a);
      a = fma(1.0, ws[67936], a);
      a = fma(0.5488, ws[67968], a);
      a = fma(0.7043, ws[68000], a);
      a = fma(0.5488, ws[68032], a);
      a = fma(0.018, ws[68064], a);
      a = fma(0.135, ws[68608], a);
      a = fma(0.68, ws[68704], a);
      a = fma(1.0, ws[68768], a);
      a = fma(0.7, ws[68864], a);
      a = fma(0.067, ws[68960], a);
      a = fma(1.0, ws[69120], a);
      a = fma(0.5488, ws[69152], a);
      a = fma(0.7043, ws[69184], a);
      a = fma(0.5488, ws[69216], a);
      a = fma(0.18, ws[69792], a);
      a = fma(0.68, ws[69888], a);
      a = fma(1.0, ws[69952], a);
      a = fma(0.7, ws[70048], a);
      a = fma(1.0, ws[70368], a);
      a = fma(0.5488, ws[70400], a);
      a = fma(0.7043, ws[70432], a);
      a = fma(0.5488, ws[70464], a);
      a = fma(0.024, ws[70496], a);
      a = fma(0.18, ws[70912], a);
      a = fma(0.68, ws[71008], a);
      a = fma(1.0, ws[71072], a);
      a = fma(1.0, ws[71168], a);
      a = fma(0.62, ws[71904], a);
      a = fma(0.31, ws[72352], a);
      a = a - ws[72768];
      a = fma(0.4693, ws[75008], a);
      a = fma(0.4702, ws[75040], a);
      a = fma(0.4702, ws[75072], a);
      a = fma(0.4702, ws[75104], a);
      a = fma(0.4693, ws[75200], a);
      a = fma(0.4702, ws[75232], a);
      a = fma(0.4702, ws[75264], a);
      a = fma(0.4702, ws[75296], a);
      a = fma(0.4693, ws[75392], a);
      a = fma(0.4702, ws[75424], a);
      a = fma(0.4702, ws[75456], a);
      a = fma(0.4702, ws[75488], a);
      yout[5376] = a;
    }
    {
      double a = 1.0 * ws[61856];
      a = fma(0.44, ws[63488], a);
      a = fma(1.0, ws[63808], a);
      a = fma(0.04, ws[63936], a);
      a = fma(0.04, ws[63968], a);
      a = a - ws[65216];
      a = a - ws[66560];
      a = a - ws[67776];
      a = a - ws[68960];
      a = a - ws[70208];
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5408] = a;
    }
    {
      double a = -ws[63808];
      a = fma(1.0, ws[64672], a);
      a = fma(0.065, ws[65216], a);
      a = fma(0.136, ws[65248], a);
      a = fma(0.03, ws[65312], a);
      a = fma(0.05, ws[65344], a);
      a = fma(0.0, ws[65376], a);
      a = fma(0.0002, ws[65408], a);
      a = fma(0.0001, ws[65440], a);
      a = fma(0.0002, ws[65472], a);
      a = fma(0.07, ws[65568], a);
      a = fma(0.07, ws[65696], a);
      a = fma(1.0, ws[66272], a);
      a = fma(1.0, ws[66400], a);
      a = fma(1.0, ws[66432], a);
      a = fma(1.0, ws[66464], a);
      a = fma(1.0, ws[67584], a);
      a = fma(1.0, ws[67616], a);
      a = fma(1.0, ws[68800], a);
      a = fma(0.5, ws[68832], a);
      a = fma(0.3, ws[68864], a);
      a = fma(1.0, ws[69984], a);
      a = fma(0.3, ws[70048], a);
      a = fma(1.0, ws[71104], a);
      a = fma(2.0, ws[71200], a);
      a = fma(1.5, ws[71232], a);
      a = fma(1.0, ws[71264], a);
      a = fma(0.032, ws[72032], a);
      a = fma(0.08, ws[72288], a);
      a = fma(0.26, ws[73568], a);
      a = fma(0.12, ws[74464], a);
      yout[5440] = a;
    }
    {
      double a = -ws[63104];
      a = a - ws[64224];
      a = fma(0.7, ws[64256], a);
      a = fma(0.7, ws[64288], a);
      a = fma(0.5477, ws[65408], a);
      a = fma(0.67, ws[65920], a);
      a = fma(0.5488, ws[67968], a);
      a = fma(0.334, ws[68448], a);
      a = fma(0.5, ws[68480], a);
      a = fma(0.5488, ws[69152], a);
      a = fma(0.334, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.5488, ws[70400], a);
      a = fma(0.67, ws[70752], a);
      a = fma(1.0, ws[70784], a);
      a = fma(0.49, ws[72256], a);
      a = fma(0.8, ws[72416], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5472] = a;
    }
    {
      double a = -ws[62880];
      a = fma(0.78, ws[63104], a);
      a = fma(0.41, ws[63488], a);
      a = fma(0.41, ws[63520], a);
      a = fma(0.41, ws[63552], a);
      a = fma(0.38, ws[63840], a);
      a = fma(0.017, ws[63968], a);
      a = fma(0.1785, ws[64000], a);
      a = fma(0.38, ws[64096], a);
      a = fma(0.028, ws[64192], a);
      a = fma(0.38, ws[64512], a);
      a = fma(0.033, ws[65248], a);
      a = fma(0.09, ws[65344], a);
      a = fma(0.084, ws[65504], a);
      a = fma(0.007, ws[65568], a);
      a = fma(0.7, ws[66080], a);
      a = fma(0.464, ws[66304], a);
      a = fma(0.0105, ws[66848], a);
      a = fma(0.007, ws[66912], a);
      a = fma(0.497, ws[67776], a);
      a = fma(0.618, ws[67808], a);
      a = fma(0.045, ws[67872], a);
      a = fma(0.218, ws[67904], a);
      a = fma(0.1835, ws[68096], a);
      a = fma(0.007, ws[68160], a);
      a = fma(0.525, ws[68608], a);
      a = fma(0.348, ws[68832], a);
      a = fma(0.662, ws[68960], a);
      a = fma(0.824, ws[68992], a);
      a = fma(0.06, ws[69056], a);
      a = fma(0.29, ws[69088], a);
      a = fma(0.112, ws[69280], a);
      a = fma(0.007, ws[69344], a);
      a = fma(0.7, ws[69792], a);
      a = fma(0.464, ws[70016], a);
      a = fma(0.06, ws[70240], a);
      a = fma(0.11, ws[70336], a);
      a = fma(0.112, ws[70528], a);
      a = fma(0.007, ws[70592], a);
      a = fma(0.7, ws[70912], a);
      a = fma(0.464, ws[71136], a);
      a = fma(0.149, ws[71232], a);
      a = fma(0.285, ws[71264], a);
      a = fma(0.65, ws[72352], a);
      a = fma(0.88, ws[74464], a);
      a = fma(1.0, ws[74688], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.1068, ws[75712], a);
      yout[5504] = a;
    }
    {
      double a = 0.0013 * ws[65440];
      a = fma(0.0013, ws[65472], a);
      a = fma(1.0, ws[72544], a);
      a = fma(1.0, ws[72576], a);
      a = fma(0.982, ws[72608], a);
      a = fma(1.0, ws[72704], a);
      a = fma(0.753, ws[72736], a);
      a = fma(0.28, ws[73408], a);
      a = fma(1.0, ws[73824], a);
      a = fma(1.0, ws[74048], a);
      a = fma(0.86, ws[74272], a);
      a = fma(1.0, ws[74496], a);
      a = fma(0.16, ws[75136], a);
      a = fma(0.0595, ws[75168], a);
      a = fma(0.0001, ws[75200], a);
      a = fma(0.16, ws[75328], a);
      a = fma(0.0595, ws[75360], a);
      a = fma(0.0398, ws[75552], a);
      a = fma(0.0452, ws[75584], a);
      a = fma(0.0462, ws[75648], a);
      a = fma(0.0518, ws[75680], a);
      a = fma(0.0535, ws[75712], a);
      a = fma(0.0516, ws[75744], a);
      a = fma(0.0585, ws[75776], a);
      a = fma(0.0709, ws[75808], a);
      a = fma(0.0293, ws[75840], a);
      a = a - ws[75872];
      a = fma(0.0086, ws[75872], a);
      a = fma(0.0456, ws[75904], a);
      a = fma(0.1566, ws[75936], a);
      a = fma(0.1384, ws[75968], a);
      a = fma(1.0, ws[76160], a);
      yout[5536] = a;
    }
    {
      double a = -ws[62752];
      a = fma(1.0, ws[63360], a);
      a = fma(0.184, ws[63392], a);
      a = fma(0.01, ws[63936], a);
      a = fma(0.457, ws[63968], a);
      a = fma(0.42, ws[64192], a);
      a = a - ws[64576];
      a = fma(1.0, ws[65184], a);
      a = fma(0.504, ws[65216], a);
      a = fma(0.045, ws[65248], a);
      a = fma(0.012, ws[65312], a);
      a = fma(0.81, ws[65344], a);
      a = fma(0.75, ws[67744], a);
      a = fma(1.0, ws[68928], a);
      a = fma(1.0, ws[70176], a);
      a = fma(0.519, ws[70208], a);
      a = fma(0.048, ws[70240], a);
      a = fma(0.02, ws[70304], a);
      a = fma(0.85, ws[70336], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5568] = a;
    }
    {
      double a = -ws[63328];
      a = fma(0.63, ws[67712], a);
      a = fma(0.25, ws[67744], a);
      a = fma(0.25, ws[67776], a);
      a = fma(0.25, ws[67808], a);
      a = fma(0.25, ws[67840], a);
      a = fma(0.25, ws[67872], a);
      a = fma(0.25, ws[67904], a);
      a = fma(0.32, ws[67936], a);
      a = fma(0.32, ws[67968], a);
      a = fma(0.32, ws[68000], a);
      a = fma(0.32, ws[68032], a);
      a = fma(0.25, ws[68064], a);
      a = fma(0.1105, ws[68096], a);
      a = fma(0.25, ws[68128], a);
      a = fma(0.043, ws[68160], a);
      a = fma(0.25, ws[68192], a);
      a = fma(0.25, ws[68224], a);
      a = fma(0.25, ws[68256], a);
      a = fma(0.09, ws[68288], a);
      a = fma(0.25, ws[68320], a);
      a = fma(0.25, ws[68416], a);
      a = fma(0.25, ws[68448], a);
      a = fma(0.25, ws[68480], a);
      a = fma(0.25, ws[68512], a);
      a = fma(0.25, ws[68544], a);
      a = fma(0.25, ws[68576], a);
      a = fma(0.25, ws[68608], a);
      a = fma(0.25, ws[68832], a);
      a = fma(0.32, ws[72128], a);
      a = fma(0.32, ws[75072], a);
      a = fma(0.32, ws[75264], a);
      a = fma(0.32, ws[75456], a);
      a = fma(0.32, ws[76256], a);
      yout[5600] = a;
    }
    {
      double a = 1.0 * ws[61824];
      a = fma(0.06, ws[63936], a);
      a = fma(0.07, ws[63968], a);
      a = a - ws[65184];
      a = fma(0.048, ws[65216], a);
      a = fma(0.231, ws[65248], a);
      a = fma(1.0, ws[65856], a);
      a = a - ws[66528];
      a = fma(0.44, ws[67200], a);
      a = a - ws[67744];
      a = fma(0.026, ws[67776], a);
      a = fma(0.14, ws[67808], a);
      a = a - ws[68928];
      a = fma(0.026, ws[68960], a);
      a = fma(0.14, ws[68992], a);
      a = fma(1.0, ws[69568], a);
      a = fma(2.0, ws[70112], a);
      a = a - ws[70176];
      a = fma(0.503, ws[70208], a);
      a = fma(0.28, ws[70240], a);
      a = fma(1.0, ws[70688], a);
      a = fma(1.0, ws[71328], a);
      a = fma(0.852, ws[71808], a);
      a = fma(1.0, ws[71840], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5632] = a;
    }
    {
      double a = -ws[61760];
      a = fma(0.35, ws[62016], a);
      a = fma(0.22, ws[62176], a);
      a = fma(1.0, ws[62368], a);
      a = fma(1.0, ws[62496], a);
      a = fma(1.0, ws[62720], a);
      a = fma(2.0, ws[63040], a);
      a = fma(1.0, ws[63072], a);
      a = fma(0.33, ws[63104], a);
      a = fma(0.33, ws[63136], a);
      a = fma(0.11, ws[63168], a);
      a = fma(0.43, ws[63904], a);
      a = fma(0.43, ws[63936], a);
      a = fma(0.37, ws[63968], a);
      a = fma(0.1105, ws[64000], a);
      a = fma(0.22, ws[64128], a);
      a = fma(0.56, ws[64160], a);
      a = fma(0.243, ws[64192], a);
      a = fma(1.5, ws[64224], a);
      a = fma(1.5, ws[64256], a);
      a = fma(1.5, ws[64288], a);
      a = fma(1.0, ws[64544], a);
      a = fma(0.668, ws[64672], a);
      a = fma(2.0, ws[64704], a);
      a = fma(1.0, ws[64736], a);
      a = fma(0.65, ws[65984], a);
      a = fma(0.61, ws[66080], a);
      a = fma(0.5, ws[68512], a);
      a = fma(0.305, ws[68608], a);
      a = fma(0.5, ws[69696], a);
      a = fma(0.5, ws[69792], a);
      a = fma(1.0, ws[70816], a);
      a = fma(0.61, ws[70912], a);
      a = fma(0.84, ws[71904], a);
      a = fma(0.63, ws[72192], a);
      a = fma(0.43, ws[72352], a);
      yout[5664] = a;
    }
    {
      double a = -ws[63648];
      a = fma(0.06, ws[63936], a);
      a = fma(0.017, ws[63968], a);
      a = fma(0.0065, ws[64000], a);
      a = fma(0.01, ws[64032], a);
      a = fma(0.07, ws[64160], a);
      a = fma(0.25, ws[64288], a);
      a = fma(0.15, ws[67168], a);
      a = fma(0.15, ws[67200], a);
      a = fma(0.1, ws[68352], a);
      a = fma(0.1, ws[68384], a);
      a = fma(0.125, ws[68416], a);
      a = fma(0.067, ws[68512], a);
      a = fma(0.292, ws[68576], a);
      a = fma(0.5, ws[68928], a);
      a = fma(0.5, ws[68960], a);
      a = fma(0.5, ws[68992], a);
      a = fma(0.5, ws[69024], a);
      a = fma(0.5, ws[69056], a);
      a = fma(0.5, ws[69088], a);
      a = fma(0.3, ws[69120], a);
      a = fma(0.3, ws[69152], a);
      a = fma(0.3, ws[69184], a);
      a = fma(0.3, ws[69216], a);
      a = fma(0.5, ws[69248], a);
      a = fma(0.5, ws[69312], a);
      a = fma(0.5, ws[69376], a);
      a = fma(0.5, ws[69440], a);
      a = fma(0.5, ws[69504], a);
      a = fma(0.75, ws[69600], a);
      a = fma(0.5, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.635, ws[69696], a);
      a = fma(0.5, ws[69728], a);
      a = fma(1.083, ws[69760], a);
      a = fma(0.5, ws[69792], a);
      a = fma(0.5, ws[70016], a);
      a = fma(0.3, ws[72160], a);
      a = fma(0.3, ws[75104], a);
      a = fma(0.3, ws[75296], a);
      a = fma(0.3, ws[75488], a);
      a = fma(0.3, ws[76288], a);
      yout[5696] = a;
    }
    {
      double a = 0.78 * ws[63136];
      a = fma(0.79, ws[63168], a);
      a = a - ws[63488];
      a = fma(0.65, ws[64224], a);
      a = fma(0.65, ws[64256], a);
      a = fma(0.68, ws[66176], a);
      a = fma(1.0, ws[66336], a);
      a = fma(1.0, ws[66528], a);
      a = fma(1.0, ws[66560], a);
      a = fma(1.0, ws[66592], a);
      a = fma(1.0, ws[66624], a);
      a = fma(1.0, ws[66656], a);
      a = fma(1.0, ws[66688], a);
      a = fma(0.6021, ws[66720], a);
      a = fma(0.7195, ws[66752], a);
      a = fma(0.0482, ws[66784], a);
      a = fma(0.0854, ws[66816], a);
      a = fma(0.85, ws[67232], a);
      a = fma(1.0, ws[67264], a);
      a = fma(1.0, ws[67296], a);
      a = fma(1.0, ws[67392], a);
      a = fma(1.0, ws[67424], a);
      a = fma(1.0, ws[67456], a);
      a = fma(1.0, ws[67520], a);
      a = fma(1.0, ws[67552], a);
      a = fma(1.0, ws[67648], a);
      a = fma(1.0, ws[67680], a);
      a = fma(0.68, ws[68704], a);
      a = fma(0.7, ws[68864], a);
      a = fma(0.68, ws[69888], a);
      a = fma(0.7, ws[70048], a);
      a = fma(0.68, ws[71008], a);
      a = fma(1.0, ws[71168], a);
      a = fma(1.0, ws[72096], a);
      a = fma(0.6, ws[72320], a);
      a = fma(1.0, ws[74016], a);
      a = fma(0.004, ws[75552], a);
      a = fma(0.0135, ws[75648], a);
      a = fma(0.0062, ws[75680], a);
      a = fma(0.0054, ws[75712], a);
      a = fma(0.017, ws[75776], a);
      a = fma(0.0025, ws[75808], a);
      a = fma(0.0023, ws[75840], a);
      a = fma(0.0114, ws[75872], a);
      a = fma(0.0155, ws[75904], a);
      a = fma(0.0384, ws[75936], a);
      a = fma(0.0585, ws[75968], a);
      yout[5728] = a;
    }
    {
      double a = -ws[62784];
      a = fma(0.4, ws[63104], a);
      a = fma(0.719, ws[63392], a);
      a = fma(1.0, ws[63424], a);
      a = fma(0.08, ws[63488], a);
      a = fma(0.08, ws[63520], a);
      a = fma(0.08, ws[63552], a);
      a = fma(0.02, ws[63840], a);
      a = fma(0.44, ws[63936], a);
      a = fma(0.73, ws[63968], a);
      a = fma(1.0, ws[64064], a);
      a = fma(0.02, ws[64096], a);
      a = fma(0.1, ws[64160], a);
      a = fma(0.02, ws[64512], a);
      a = a - ws[64608];
      a = fma(0.332, ws[64672], a);
      a = fma(0.132, ws[65216], a);
      a = fma(0.203, ws[65248], a);
      a = fma(0.2, ws[65280], a);
      a = fma(0.44, ws[65312], a);
      a = fma(0.68, ws[65344], a);
      a = fma(0.284, ws[65504], a);
      a = fma(0.154, ws[65568], a);
      a = fma(0.46, ws[65952], a);
      a = fma(0.7, ws[66048], a);
      a = fma(0.27, ws[66080], a);
      a = fma(1.24, ws[66304], a);
      a = fma(0.077, ws[66912], a);
      a = fma(0.198, ws[67776], a);
      a = fma(0.251, ws[67808], a);
      a = fma(0.15, ws[67840], a);
      a = fma(0.705, ws[67872], a);
      a = fma(1.28, ws[67904], a);
      a = fma(0.023, ws[68064], a);
      a = fma(0.2385, ws[68096], a);
      a = fma(0.119, ws[68160], a);
      a = fma(1.75, ws[68576], a);
      a = fma(0.203, ws[68608], a);
      a = fma(0.93, ws[68832], a);
      a = fma(0.273, ws[68960], a);
      a = fma(0.381, ws[68992], a);
      a = fma(0.2, ws[69024], a);
      a = fma(0.94, ws[69056], a);
      a = fma(1.71, ws[69088], a);
      a = fma(0.371, ws[69280], a);
      a = fma(0.168, ws[69344], a);
      a = fma(2.3, ws[69760], a);
      a = fma(0.27, ws[69792], a);
      a = fma(1.24, ws[70016], a);
      a = fma(0.147, ws[70208], a);
      a = fma(0.241, ws[70240], a);
      a = fma(0.2, ws[70272], a);
      a = fma(0.47, ws[70304], a);
      a = fma(0.72, ws[70336], a);
      a = fma(0.031, ws[70496], a);
      a = fma(0.371, ws[70528], a);
      a = fma(0.168, ws[70592], a);
      a = fma(0.7, ws[70880], a);
      a = fma(0.27, ws[70912], a);
      a = fma(1.24, ws[71136], a);
      a = fma(0.64, ws[71232], a);
      a = fma(1.21, ws[71264], a);
      a = fma(1.0, ws[72384], a);
      a = fma(0.387, ws[72448], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      yout[5760] = a;
    }
    {
      double a = 0.018 * ws[62176];
      a = fma(0.11, ws[62368], a);
      a = fma(1.0, ws[62752], a);
      a = fma(0.313, ws[63008], a);
      a = fma(1.0, ws[63072], a);
      a = fma(0.65, ws[63680], a);
      a = fma(0.09, ws[63968], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.1, ws[64128], a);
      a = fma(0.28, ws[64160], a);
      a = fma(0.002, ws[64192], a);
      a = fma(1.0, ws[64576], a);
      a = fma(1.0, ws[64736], a);
      a = a - ws[64960];
      a = fma(1.0, ws[64992], a);
      a = a - ws[65824];
      a = fma(1.0, ws[65888], a);
      a = fma(0.23, ws[65952], a);
      a = fma(0.35, ws[65984], a);
      a = fma(0.7, ws[66048], a);
      a = a - ws[67168];
      a = fma(0.15, ws[67232], a);
      a = a - ws[68352];
      a = fma(0.5, ws[68416], a);
      a = fma(0.269, ws[68512], a);
      a = fma(1.16, ws[68576], a);
      a = a - ws[68928];
      a = a - ws[68960];
      a = a - ws[68992];
      a = a - ws[69024];
      a = a - ws[69056];
      a = a - ws[69088];
      a = a - ws[69120];
      a = a - ws[69152];
      a = a - ws[69184];
      a = a - ws[69216];
      a = a - ws[69248];
      a = a - ws[69280];
      a = a - ws[69312];
      a = a - ws[69344];
      a = a - ws[69376];
      a = a - ws[69408];
      a = a - ws[69440];
      a = a - ws[69472];
      a = a - ws[69504];
      a = a - ws[69536];
      a = a - ws[69536];
      a = a - ws[69568];
      a = a - ws[69600];
      a = fma(0.5, ws[69600], a);
      a = a - ws[69632];
      a = a - ws[69664];
      a = a - ws[69696];
      a = fma(0.269, ws[69696], a);
      a = a - ws[69728];
      a = a - ws[69760];
      a = fma(1.16, ws[69760], a);
      a = a - ws[69792];
      a = a - ws[69824];
      a = a - ws[69856];
      a = a - ws[69888];
      a = a - ws[69920];
      a = a - ws[69952];
      a = a - ws[69984];
      a = a - ws[70016];
      a = a - ws[70048];
      a = a - ws[70080];
      a = a - ws[70656];
      a = fma(1.0, ws[70720], a);
      a = fma(0.538, ws[70816], a);
      a = fma(0.7, ws[70880], a);
      a = a - ws[72160];
      a = a - ws[75104];
      a = a - ws[75296];
      a = a - ws[75488];
      a = a - ws[76288];
      yout[5792] = a;
    }
    {
      double a = -ws[60672];
      a = a - ws[61056];
      a = a - ws[61088];
      a = a - ws[61120];
      a = a - ws[61152];
      a = a - ws[61184];
      a = a - ws[61184];
      a = fma(1.0, ws[61248], a);
      a = a - ws[61440];
      a = fma(1.0, ws[61472], a);
      a = a - ws[62304];
      a = a - ws[62432];
      a = a - ws[65152];
      a = a - ws[65184];
      a = a - ws[65216];
      a = a - ws[65248];
      a = a - ws[65280];
      a = a - ws[65312];
      a = a - ws[65344];
      a = a - ws[65376];
      a = a - ws[65408];
      a = a - ws[65440];
      a = a - ws[65472];
      a = a - ws[65504];
      a = a - ws[65536];
      a = a - ws[65568];
      a = a - ws[65600];
      a = a - ws[65632];
      a = a - ws[65664];
      a = a - ws[65696];
      a = a - ws[65728];
      a = a - ws[65760];
      a = a - ws[65792];
      a = a - ws[65824];
      a = a - ws[65856];
      a = a - ws[65888];
      a = a - ws[65920];
      a = a - ws[65952];
      a = a - ws[65984];
      a = a - ws[66016];
      a = a - ws[66048];
      a = a - ws[66080];
      a = a - ws[66112];
      a = a - ws[66144];
      a = a - ws[66176];
      a = a - ws[66208];
      a = a - ws[66240];
      a = a - ws[66272];
      a = a - ws[66304];
      a = a - ws[66336];
      a = a - ws[66368];
      a = a - ws[72032];
      a = a - ws[72288];
      a = a - ws[72544];
      a = a - ws[72736];
      a = a - ws[73376];
      a = a - ws[73408];
      a = a - ws[73440];
      a = a - ws[73472];
      a = a - ws[73504];
      a = a - ws[73536];
      a = a - ws[73568];
      a = a - ws[74272];
      a = a - ws[74304];
      a = a - ws[74336];
      a = a - ws[74368];
      a = a - ws[74400];
      a = a - ws[74432];
      a = a - ws[74464];
      a = a - ws[75008];
      a = a - ws[75200];
      a = a - ws[75392];
      a = a - ws[76192];
      yout[5824] = a;
    }
    {
      double a = 1.0 * ws[62176];
      a = fma(0.35, ws[62208], a);
      a = fma(0.25, ws[62240], a);
      a = fma(0.4, ws[62304], a);
      a = fma(0.2, ws[62432], a);
      a = fma(1.0, ws[62496], a);
      a = a - ws[62720];
      a = fma(1.0, ws[63328], a);
      a = fma(0.35, ws[63456], a);
      a = fma(0.35, ws[63680], a);
      a = fma(1.0, ws[63712], a);
      a = fma(1.0, ws[63744], a);
      a = fma(0.21, ws[63840], a);
      a = fma(1.0, ws[63904], a);
      a = fma(0.56, ws[63936], a);
      a = fma(0.09, ws[63968], a);
      a = fma(0.459, ws[64000], a);
      a = fma(0.33, ws[64032], a);
      a = fma(0.62, ws[64064], a);
      a = fma(0.21, ws[64096], a);
      a = fma(0.1, ws[64160], a);
      a = fma(0.08, ws[64192], a);
      a = fma(0.05, ws[64224], a);
      a = fma(0.05, ws[64256], a);
      a = fma(0.21, ws[64512], a);
      a = a - ws[64544];
      a = fma(0.68, ws[64640], a);
      a = fma(0.332, ws[64672], a);
      a = fma(1.0, ws[65152], a);
      a = fma(0.018, ws[65248], a);
      a = fma(1.6, ws[65280], a);
      a = fma(0.78, ws[65312], a);
      a = fma(0.308, ws[65504], a);
      a = fma(0.007, ws[65568], a);
      a = fma(0.43, ws[65632], a);
      a = fma(0.36, ws[65792], a);
      a = fma(1.0, ws[65888], a);
      a = fma(0.33, ws[65920], a);
      a = fma(0.65, ws[65984], a);
      a = fma(0.5, ws[66016], a);
      a = fma(0.3, ws[66048], a);
      a = fma(0.03, ws[66080], a);
      a = fma(0.287, ws[66304], a);
      a = fma(0.0625, ws[66848], a);
      a = fma(0.007, ws[66912], a);
      a = fma(0.06, ws[66976], a);
      a = fma(0.1, ws[67136], a);
      a = fma(0.15, ws[67232], a);
      a = fma(1.37, ws[67712], a);
      a = fma(0.75, ws[67744], a);
      a = fma(0.827, ws[67776], a);
      a = fma(0.777, ws[67808], a);
      a = fma(1.95, ws[67840], a);
      a = fma(1.5, ws[67872], a);
      a = fma(0.75, ws[67904], a);
      a = fma(0.68, ws[67936], a);
      a = fma(0.68, ws[67968], a);
      a = fma(0.68, ws[68000], a);
      a = fma(0.68, ws[68032], a);
      a = fma(1.31, ws[68064], a);
      a = fma(1.0295, ws[68096], a);
      a = fma(0.75, ws[68128], a);
      a = fma(0.964, ws[68160], a);
      a = fma(0.75, ws[68192], a);
      a = fma(1.03, ws[68224], a);
      a = fma(0.75, ws[68256], a);
      a = fma(0.91, ws[68288], a);
      a = fma(0.75, ws[68320], a);
      a = fma(1.0, ws[68352], a);
      a = fma(1.0, ws[68384], a);
      a = fma(1.5, ws[68416], a);
      a = fma(1.0, ws[68448], a);
      a = fma(0.75, ws[68480], a);
      a = fma(1.66, ws[68512], a);
      a = fma(1.5, ws[68544], a);
      a = fma(1.5, ws[68576], a);
      a = fma(0.773, ws[68608], a);
      a = fma(1.0, ws[68640], a);
      a = fma(1.0, ws[68672], a);
      a = fma(1.0, ws[68704], a);
      a = fma(1.0, ws[68736], a);
      a = fma(1.0, ws[68768], a);
      a = fma(1.0, ws[68800], a);
      a = fma(0.965, ws[68832], a);
      a = fma(1.0, ws[68864], a);
      a = fma(1.0, ws[68896], a);
      a = fma(0.13, ws[68960], a);
      a = fma(0.042, ws[68992], a);
      a = fma(1.6, ws[69024], a);
      a = fma(1.0, ws[69056], a);
      a = fma(1.048, ws[69248], a);
      a = fma(0.403, ws[69280], a);
      a = fma(0.007, ws[69344], a);
      a = fma(0.56, ws[69408], a);
      a = fma(1.0, ws[69600], a);
      a = fma(0.33, ws[69632], a);
      a = fma(1.0, ws[69696], a);
      a = fma(1.0, ws[69728], a);
      a = fma(1.0, ws[69760], a);
      a = fma(0.03, ws[69792], a);
      a = fma(0.287, ws[70016], a);
      a = fma(1.0, ws[70144], a);
      a = fma(0.024, ws[70240], a);
      a = fma(1.6, ws[70272], a);
      a = fma(0.79, ws[70304], a);
      a = fma(0.75, ws[70496], a);
      a = fma(0.403, ws[70528], a);
      a = fma(0.56, ws[70560], a);
      a = fma(0.007, ws[70592], a);
      a = fma(1.0, ws[70720], a);
      a = fma(0.33, ws[70752], a);
      a = fma(1.0, ws[70816], a);
      a = fma(1.0, ws[70848], a);
      a = fma(0.3, ws[70880], a);
      a = fma(0.03, ws[70912], a);
      a = fma(0.287, ws[71136], a);
      a = fma(0.202, ws[71232], a);
      a = fma(0.504, ws[71264], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.72, ws[71904], a);
      a = fma(0.68, ws[71936], a);
      a = fma(0.895, ws[72032], a);
      a = fma(0.925, ws[72064], a);
      a = fma(1.143, ws[72128], a);
      a = fma(0.74, ws[72160], a);
      a = fma(0.83, ws[72192], a);
      a = fma(0.68, ws[75072], a);
      a = fma(0.68, ws[75264], a);
      a = fma(0.68, ws[75456], a);
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      a = fma(1.68, ws[76256], a);
      a = fma(1.0, ws[76288], a);
      yout[5856] = a;
    }
    {
      double a = 1.0 * ws[61792];
      a = fma(0.4, ws[62176], a);
      a = fma(0.65, ws[63456], a);
      a = fma(0.64, ws[63648], a);
      a = fma(0.08, ws[63936], a);
      a = fma(0.32, ws[63968], a);
      a = fma(0.008, ws[64192], a);
      a = a - ws[65152];
      a = fma(0.131, ws[65216], a);
      a = fma(0.051, ws[65248], a);
      a = fma(1.0, ws[65824], a);
      a = fma(0.65, ws[65984], a);
      a = a - ws[66496];
      a = fma(0.44, ws[67168], a);
      a = a - ws[67712];
      a = a - ws[67712];
      a = a - ws[67744];
      a = a - ws[67776];
      a = fma(0.08, ws[67776], a);
      a = a - ws[67808];
      a = fma(0.018, ws[67808], a);
      a = a - ws[67840];
      a = a - ws[67872];
      a = a - ws[67904];
      a = a - ws[67936];
      a = a - ws[67968];
      a = a - ws[68000];
      a = a - ws[68032];
      a = a - ws[68064];
      a = a - ws[68096];
      a = a - ws[68128];
      a = a - ws[68160];
      a = a - ws[68192];
      a = a - ws[68224];
      a = a - ws[68256];
      a = a - ws[68288];
      a = a - ws[68320];
      a = a - ws[68352];
      a = fma(0.9, ws[68352], a);
      a = a - ws[68384];
      a = fma(0.9, ws[68384], a);
      a = a - ws[68416];
      a = a - ws[68448];
      a = a - ws[68480];
      a = a - ws[68512];
      a = fma(0.25, ws[68512], a);
      a = a - ws[68544];
      a = a - ws[68576];
      a = a - ws[68608];
      a = a - ws[68640];
      a = a - ws[68672];
      a = a - ws[68704];
      a = a - ws[68736];
      a = a - ws[68768];
      a = a - ws[68800];
      a = a - ws[68832];
      a = a - ws[68864];
      a = a - ws[68896];
      a = fma(0.5, ws[68928], a);
      a = fma(0.58, ws[68960], a);
      a = fma(0.518, ws[68992], a);
      a = fma(0.5, ws[69024], a);
      a = fma(0.5, ws[69056], a);
      a = fma(0.5, ws[69088], a);
      a = fma(0.7, ws[69120], a);
      a = fma(0.7, ws[69152], a);
      a = fma(0.7, ws[69184], a);
      a = fma(0.7, ws[69216], a);
      a = fma(0.5, ws[69248], a);
      a = fma(1.0, ws[69280], a);
      a = fma(0.5, ws[69312], a);
      a = fma(1.0, ws[69344], a);
      a = fma(0.5, ws[69376], a);
      a = fma(1.0, ws[69408], a);
      a = fma(0.5, ws[69440], a);
      a = fma(1.0, ws[69472], a);
      a = fma(0.5, ws[69504], a);
      a = fma(2.0, ws[69536], a);
      a = fma(1.0, ws[69568], a);
      a = fma(0.5, ws[69600], a);
      a = fma(0.5, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.5, ws[69696], a);
      a = fma(0.5, ws[69728], a);
      a = fma(0.5, ws[69760], a);
      a = fma(0.5, ws[69792], a);
      a = fma(1.0, ws[69824], a);
      a = fma(1.0, ws[69856], a);
      a = fma(1.0, ws[69888], a);
      a = fma(1.0, ws[69920], a);
      a = fma(1.0, ws[69952], a);
      a = fma(1.0, ws[69984], a);
      a = fma(0.5, ws[70016], a);
      a = fma(1.0, ws[70048], a);
      a = fma(1.0, ws[70080], a);
      a = a - ws[70144];
      a = fma(0.14, ws[70208], a);
      a = fma(0.055, ws[70240], a);
      a = fma(1.0, ws[70656], a);
      a = a - ws[72128];
      a = fma(0.7, ws[72160], a);
      a = fma(0.17, ws[72288], a);
      a = fma(0.08, ws[72320], a);
      a = fma(0.34, ws[72352], a);
      a = a - ws[75072];
      a = fma(0.7, ws[75104], a);
      a = a - ws[75264];
      a = fma(0.7, ws[75296], a);
      a = a - ws[75456];
      a = fma(0.7, ws[75488], a);
      a = fma(0.2581, ws[75520], a);
      a = fma(0.0794, ws[75552], a);
      a = fma(0.039, ws[75584], a);
      a = fma(0.184, ws[75616], a);
      a = fma(0.0646, ws[75648], a);
      a = fma(0.0244, ws[75680], a);
      a = fma(0.1068, ws[75712], a);
      a = fma(0.0445, ws[75744], a);
      a = fma(0.0818, ws[75776], a);
      a = fma(0.0297, ws[75808], a);
      a = fma(0.0628, ws[75840], a);
      a = fma(0.0698, ws[75872], a);
      a = fma(0.0786, ws[75904], a);
      a = fma(0.0526, ws[75936], a);
      a = fma(0.0571, ws[75968], a);
      a = fma(0.2266, ws[76000], a);
      a = fma(1.0, ws[76032], a);
      a = a - ws[76256];
      a = fma(0.7, ws[76288], a);
      yout[5888] = a;
    }
    {
      double a = 1.0 * ws[60672];
      a = a - ws[60704];
      a = fma(1.0, ws[61056], a);
      a = fma(1.0, ws[61120], a);
      a = fma(2.0, ws[61184], a);
      a = fma(1.0, ws[61216], a);
      a = a - ws[61248];
      a = a - ws[61280];
      a = a - ws[61312];
      a = fma(1.0, ws[61376], a);
      a = fma(0.7, ws[61408], a);
      a = fma(2.0, ws[61440], a);
      a = a - ws[61472];
      a = fma(1.0, ws[61472], a);
      a = fma(2.0, ws[61504], a);
      a = a - ws[61536];
      a = fma(1.0, ws[61568], a);
      a = a - ws[61632];
      a = fma(1.0, ws[61664], a);
      a = fma(1.0, ws[61696], a);
      a = fma(0.4, ws[62208], a);
      a = fma(0.87, ws[62304], a);
      a = fma(1.3, ws[62432], a);
      a = fma(0.65, ws[62464], a);
      a = fma(1.0, ws[62496], a);
      a = fma(1.0, ws[63776], a);
      a = fma(1.0, ws[63808], a);
      a = fma(0.67, ws[63840], a);
      a = fma(0.67, ws[64096], a);
      a = fma(0.67, ws[64512], a);
      a = fma(0.68, ws[64640], a);
      a = fma(1.0, ws[64864], a);
      a = a - ws[64960];
      a = fma(1.0, ws[64992], a);
      a = a - ws[65024];
      a = fma(1.0, ws[65056], a);
      a = a - ws[65088];
      a = fma(1.0, ws[65120], a);
      a = fma(1.0, ws[65152], a);
      a = fma(1.0, ws[65184], a);
      a = fma(0.935, ws[65216], a);
      a = fma(0.864, ws[65248], a);
      a = fma(1.0, ws[65280], a);
      a = fma(0.97, ws[65312], a);
      a = fma(0.95, ws[65344], a);
      a = fma(0.998, ws[65376], a);
      a = fma(0.998, ws[65408], a);
      a = fma(0.998, ws[65440], a);
      a = fma(0.998, ws[65472], a);
      a = fma(0.763, ws[65504], a);
      a = fma(0.82, ws[65536], a);
      a = fma(1.6955, ws[65568], a);
      a = fma(0.82, ws[65600], a);
      a = fma(0.77, ws[65632], a);
      a = fma(0.77, ws[65664], a);
      a = fma(1.36, ws[65696], a);
      a = fma(0.77, ws[65728], a);
      a = fma(0.64, ws[65760], a);
      a = fma(0.36, ws[65792], a);
      a = fma(1.0, ws[65824], a);
      a = fma(1.0, ws[65856], a);
      a = fma(1.0, ws[65888], a);
      a = fma(1.0, ws[65920], a);
      a = fma(1.0, ws[65952], a);
      a = fma(1.0, ws[65984], a);
      a = fma(1.0, ws[66016], a);
      a = fma(1.0, ws[66048], a);
      a = fma(1.0, ws[66080], a);
      a = fma(1.0, ws[66112], a);
      a = fma(1.0, ws[66144], a);
      a = fma(1.0, ws[66176], a);
      a = fma(1.0, ws[66208], a);
      a = fma(1.0, ws[66240], a);
      a = fma(1.0, ws[66272], a);
      a = fma(2.0, ws[66304], a);
      a = fma(2.0, ws[66336], a);
      a = fma(1.0, ws[66368], a);
      a = a - ws[66400];
      a = a - ws[66432];
      a = a - ws[66464];
      a = fma(0.539, ws[66912], a);
      a = fma(0.23, ws[67040], a);
      a = fma(0.659, ws[68160], a);
      a = fma(0.75, ws[68192], a);
      a = fma(0.31, ws[68288], a);
      a = fma(0.75, ws[68320], a);
      a = fma(1.0, ws[68544], a);
      a = fma(0.5, ws[68832], a);
      a = fma(0.7, ws[68864], a);
      a = fma(0.825, ws[69344], a);
      a = fma(0.5, ws[69376], a);
      a = fma(0.46, ws[69472], a);
      a = fma(0.5, ws[69504], a);
      a = fma(1.0, ws[69728], a);
      a = fma(1.0, ws[70016], a);
      a = fma(0.7, ws[70048], a);
      a = fma(1.0, ws[70144], a);
      a = fma(1.0, ws[70176], a);
      a = fma(1.0, ws[70208], a);
      a = fma(1.0, ws[70240], a);
      a = fma(1.0, ws[70272], a);
      a = fma(1.0, ws[70304], a);
      a = fma(1.0, ws[70336], a);
      a = fma(1.0, ws[70368], a);
      a = fma(1.0, ws[70400], a);
      a = fma(1.0, ws[70432], a);
      a = fma(1.0, ws[70464], a);
      a = fma(1.0, ws[70496], a);
      a = fma(1.0, ws[70528], a);
      a = fma(1.0, ws[70560], a);
      a = fma(1.825, ws[70592], a);
      a = fma(1.46, ws[70624], a);
      a = fma(1.0, ws[70656], a);
      a = fma(1.0, ws[70688], a);
      a = fma(1.0, ws[70720], a);
      a = fma(1.0, ws[70752], a);
      a = fma(1.0, ws[70784], a);
      a = fma(1.0, ws[70816], a);
      a = fma(1.0, ws[70848], a);
      a = fma(1.0, ws[70880], a);
      a = fma(1.0, ws[70912], a);
      a = fma(1.0, ws[70944], a);
      a = fma(1.0, ws[70976], a);
      a = fma(1.0, ws[71008], a);
      a = fma(1.0, ws[71040], a);
      a = fma(1.0, ws[71072], a);
      a = fma(1.0, ws[71104], a);
      a = fma(2.0, ws[71136], a);
      a = fma(2.0, ws[71168], a);
      a = fma(0.5, ws[71232], a);
      a = fma(1.0, ws[71264], a);
      a = fma(1.0, ws[71296], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71680], a);
      a = fma(0.48, ws[71712], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.68, ws[71936], a);
      a = fma(0.968, ws[72032], a);
      a = fma(1.0, ws[72064], a);
      a = fma(0.92, ws[72288], a);
      a = fma(1.0, ws[72416], a);
      a = fma(2.0, ws[72544], a);
      a = fma(2.0, ws[72576], a);
      a = fma(0.753, ws[72736], a);
      a = a - ws[72864];
      a = fma(0.72, ws[73376], a);
      a = fma(0.72, ws[73408], a);
      a = fma(0.72, ws[73440], a);
      a = fma(0.72, ws[73472], a);
      a = fma(0.72, ws[73504], a);
      a = fma(0.72, ws[73536], a);
      a = fma(0.74, ws[73568], a);
      a = fma(1.0, ws[73600], a);
      a = fma(1.0, ws[73632], a);
      a = fma(1.0, ws[73664], a);
      a = fma(1.0, ws[73696], a);
      a = fma(1.0, ws[73728], a);
      a = fma(1.0, ws[73760], a);
      a = fma(1.0, ws[73792], a);
      a = fma(0.86, ws[74272], a);
      a = fma(0.86, ws[74304], a);
      a = fma(0.86, ws[74336], a);
      a = fma(0.86, ws[74368], a);
      a = fma(0.86, ws[74400], a);
      a = fma(0.86, ws[74432], a);
      a = fma(0.88, ws[74464], a);
      a = fma(1.0, ws[74496], a);
      a = fma(1.0, ws[74528], a);
      a = fma(1.0, ws[74560], a);
      a = fma(1.0, ws[74592], a);
      a = fma(1.0, ws[74624], a);
      a = fma(1.0, ws[74656], a);
      a = fma(1.0, ws[74688], a);
      a = fma(0.998, ws[75008], a);
      a = fma(1.0, ws[75040], a);
      a = fma(0.998, ws[75200], a);
      a = fma(1.0, ws[75232], a);
      a = fma(0.998, ws[75392], a);
      a = fma(1.0, ws[75424], a);
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      yout[5920] = a;
    }
    {
      double a = 1.0 * ws[60704];
      a = fma(1.0, ws[61280], a);
      a = fma(1.0, ws[61344], a);
      a = a - ws[61376];
      a = a - ws[61408];
      a = a - ws[61440];
      a = a - ws[61472];
      a = a - ws[61504];
      a = a - ws[61504];
      a = a - ws[61536];
      a = fma(1.0, ws[61568], a);
      a = a - ws[62208];
      a = fma(1.0, ws[63712], a);
      a = fma(1.0, ws[63744], a);
      a = fma(1.0, ws[63872], a);
      a = a - ws[64352];
      a = a - ws[64384];
      a = a - ws[64416];
      a = a - ws[64448];
      a = a - ws[64480];
      a = a - ws[64512];
      a = a - ws[64544];
      a = a - ws[64576];
      a = a - ws[64608];
      a = a - ws[64640];
      a = a - ws[64672];
      a = a - ws[64704];
      a = a - ws[64736];
      a = a - ws[64768];
      a = a - ws[64800];
      a = a - ws[64832];
      a = a - ws[64864];
      a = a - ws[70144];
      a = a - ws[70176];
      a = a - ws[70208];
      a = a - ws[70240];
      a = a - ws[70272];
      a = a - ws[70304];
      a = a - ws[70336];
      a = a - ws[70368];
      a = a - ws[70400];
      a = a - ws[70432];
      a = a - ws[70464];
      a = a - ws[70496];
      a = a - ws[70528];
      a = a - ws[70560];
      a = a - ws[70592];
      a = a - ws[70624];
      a = a - ws[70656];
      a = a - ws[70688];
      a = a - ws[70720];
      a = a - ws[70752];
      a = a - ws[70784];
      a = a - ws[70816];
      a = a - ws[70848];
      a = a - ws[70880];
      a = a - ws[70912];
      a = a - ws[70944];
      a = a - ws[70976];
      a = a - ws[71008];
      a = a - ws[71040];
      a = a - ws[71072];
      a = a - ws[71104];
      a = a - ws[71136];
      a = a - ws[71168];
      a = a - ws[71296];
      a = a - ws[71936];
      a = a - ws[72064];
      a = a - ws[72224];
      a = a - ws[72416];
      a = a - ws[72480];
      a = a - ws[72576];
      a = a - ws[72704];
      a = a - ws[72928];
      a = a - ws[73600];
      a = a - ws[73632];
      a = a - ws[73664];
      a = a - ws[73696];
      a = a - ws[73728];
      a = a - ws[73760];
      a = a - ws[73792];
      a = a - ws[74496];
      a = a - ws[74528];
      a = a - ws[74560];
      a = a - ws[74592];
      a = a - ws[74624];
      a = a - ws[74656];
      a = a - ws[74688];
      a = a - ws[75040];
      a = a - ws[75232];
      a = a - ws[75424];
      a = a - ws[76224];
      yout[5952] = a;
    }
    {
      double a = 1.0 * ws[60608];
      a = a - ws[60640];
      a = fma(1.0, ws[60896], a);
      a = a - ws[60928];
      a = a - ws[60960];
      a = a - ws[60960];
      a = a - ws[60992];
      a = a - ws[60992];
      a = fma(1.0, ws[61024], a);
      a = a - ws[61120];
      a = a - ws[61152];
      a = fma(1.0, ws[61376], a);
      a = a - ws[61408];
      a = a - ws[61632];
      a = fma(1.0, ws[61664], a);
      a = fma(1.0, ws[61728], a);
      a = fma(1.0, ws[61760], a);
      a = fma(0.35, ws[62016], a);
      a = fma(0.53, ws[62048], a);
      a = fma(0.18, ws[62080], a);
      a = fma(0.17, ws[62112], a);
      a = fma(0.18, ws[62144], a);
      a = fma(0.25, ws[62176], a);
      a = a - ws[62272];
      a = fma(0.07, ws[62272], a);
      a = fma(0.88, ws[62304], a);
      a = fma(0.34, ws[62368], a);
      a = a - ws[62400];
      a = fma(0.3, ws[62496], a);
      a = fma(1.0, ws[62720], a);
      a = fma(1.0, ws[62912], a);
      a = fma(1.0, ws[63040], a);
      a = fma(0.52, ws[63104], a);
      a = fma(0.52, ws[63136], a);
      a = fma(0.56, ws[63168], a);
      a = fma(0.619, ws[63232], a);
      a = fma(0.584, ws[63264], a);
      a = fma(1.0, ws[63328], a);
      a = fma(1.0, ws[63360], a);
      a = fma(1.0, ws[63392], a);
      a = fma(1.0, ws[63424], a);
      a = fma(1.0, ws[63616], a);
      a = fma(0.15, ws[63904], a);
      a = fma(0.32, ws[63936], a);
      a = fma(0.07, ws[63968], a);
      a = fma(0.1105, ws[64000], a);
      a = fma(0.14, ws[64128], a);
      a = fma(0.11, ws[64160], a);
      a = fma(0.072, ws[64192], a);
      a = fma(1.0, ws[64224], a);
      a = fma(1.0, ws[64256], a);
      a = fma(1.0, ws[64288], a);
      a = fma(1.0, ws[64544], a);
      a = fma(1.0, ws[64672], a);
      a = fma(1.0, ws[64704], a);
      a = fma(1.0, ws[65152], a);
      a = fma(1.0, ws[65184], a);
      a = fma(0.66, ws[65216], a);
      a = fma(0.2, ws[65248], a);
      a = fma(1.0, ws[65280], a);
      a = fma(0.78, ws[65312], a);
      a = fma(0.83, ws[65344], a);
      a = fma(0.998, ws[65376], a);
      a = fma(0.998, ws[65408], a);
      a = fma(0.998, ws[65440], a);
      a = fma(0.998, ws[65472], a);
      a = fma(0.763, ws[65504], a);
      a = fma(0.1645, ws[65568], a);
      a = fma(0.77, ws[65632], a);
      a = fma(0.5, ws[65696], a);
      a = fma(0.36, ws[65792], a);
      a = fma(0.67, ws[65920], a);
      a = fma(0.77, ws[65952], a);
      a = fma(0.5, ws[66016], a);
      a = fma(0.3, ws[66048], a);
      a = fma(1.0, ws[66080], a);
      a = fma(1.0, ws[66176], a);
      a = fma(1.0, ws[66240], a);
      a = fma(1.0, ws[66272], a);
      a = a - ws[66496];
      a = a - ws[66528];
      a = a - ws[66560];
      a = a - ws[66592];
      a = a - ws[66624];
      a = a - ws[66656];
      a = a - ws[66688];
      a = a - ws[66720];
      a = a - ws[66752];
      a = a - ws[66784];
      a = a - ws[66816];
      a = a - ws[66848];
      a = fma(0.3225, ws[66848], a);
      a = a - ws[66880];
      a = a - ws[66912];
      a = a - ws[66944];
      a = a - ws[66976];
      a = fma(0.1, ws[66976], a);
      a = a - ws[67008];
      a = a - ws[67040];
      a = fma(0.27, ws[67040], a);
      a = a - ws[67072];
      a = a - ws[67104];
      a = a - ws[67136];
      a = fma(0.1, ws[67136], a);
      a = a - ws[67168];
      a = a - ws[67200];
      a = a - ws[67232];
      a = a - ws[67264];
      a = a - ws[67296];
      a = a - ws[67328];
      a = a - ws[67360];
      a = a - ws[67392];
      a = a - ws[67424];
      a = a - ws[67456];
      a = a - ws[67488];
      a = a - ws[67520];
      a = a - ws[67552];
      a = a - ws[67584];
      a = a - ws[67616];
      a = a - ws[67648];
      a = a - ws[67680];
      a = fma(0.74, ws[67712], a);
      a = fma(1.0, ws[67744], a);
      a = fma(0.894, ws[67776], a);
      a = fma(0.842, ws[67808], a);
      a = fma(1.0, ws[67840], a);
      a = fma(1.0, ws[67872], a);
      a = fma(1.0, ws[67904], a);
      a = fma(1.37, ws[67936], a);
      a = fma(1.2846, ws[67968], a);
      a = fma(1.3218, ws[68000], a);
      a = fma(1.2846, ws[68032], a);
      a = fma(1.0, ws[68064], a);
      a = fma(1.279, ws[68096], a);
      a = fma(1.0, ws[68128], a);
      a = fma(0.918, ws[68160], a);
      a = fma(0.75, ws[68192], a);
      a = fma(1.0, ws[68224], a);
      a = fma(1.0, ws[68256], a);
      a = fma(1.01, ws[68288], a);
      a = fma(0.75, ws[68320], a);
      a = fma(0.9, ws[68352], a);
      a = fma(0.9, ws[68384], a);
      a = fma(0.5, ws[68416], a);
      a = fma(0.834, ws[68448], a);
      a = fma(1.0, ws[68480], a);
      a = fma(0.5, ws[68512], a);
      a = fma(1.0, ws[68544], a);
      a = fma(1.0, ws[68576], a);
      a = fma(1.0, ws[68608], a);
      a = fma(1.0, ws[68640], a);
      a = fma(1.0, ws[68672], a);
      a = fma(2.0, ws[68704], a);
      a = fma(1.0, ws[68736], a);
      a = fma(1.0, ws[68768], a);
      a = fma(2.0, ws[68800], a);
      a = fma(0.5, ws[68832], a);
      a = fma(1.0, ws[68864], a);
      a = fma(1.0, ws[68896], a);
      a = fma(0.5, ws[68928], a);
      a = fma(0.394, ws[68960], a);
      a = fma(0.342, ws[68992], a);
      a = fma(0.5, ws[69024], a);
      a = fma(0.5, ws[69056], a);
      a = fma(0.5, ws[69088], a);
      a = fma(1.0, ws[69120], a);
      a = fma(0.9146, ws[69152], a);
      a = fma(0.9518, ws[69184], a);
      a = fma(0.9146, ws[69216], a);
      a = fma(0.5, ws[69248], a);
      a = fma(1.0, ws[69280], a);
      a = fma(0.175, ws[69344], a);
      a = fma(1.0, ws[69408], a);
      a = fma(0.54, ws[69472], a);
      a = fma(0.33, ws[69632], a);
      a = fma(0.5, ws[69664], a);
      a = fma(0.5, ws[69728], a);
      a = fma(0.5, ws[69760], a);
      a = fma(0.5, ws[69792], a);
      a = fma(2.0, ws[69888], a);
      a = fma(1.0, ws[69920], a);
      a = fma(1.0, ws[69984], a);
      a = fma(1.0, ws[70048], a);
      a = fma(1.0, ws[70144], a);
      a = fma(1.0, ws[70176], a);
      a = fma(0.254, ws[70208], a);
      a = fma(0.488, ws[70240], a);
      a = fma(1.0, ws[70272], a);
      a = fma(0.79, ws[70304], a);
      a = fma(0.86, ws[70336], a);
      a = fma(1.0, ws[70368], a);
      a = fma(0.9146, ws[70400], a);
      a = fma(0.9518, ws[70432], a);
      a = fma(0.9146, ws[70464], a);
      a = fma(1.0, ws[70496], a);
      a = fma(1.0, ws[70528], a);
      a = fma(1.0, ws[70560], a);
      a = fma(0.175, ws[70592], a);
      a = fma(0.54, ws[70624], a);
      a = fma(0.67, ws[70752], a);
      a = fma(1.0, ws[70784], a);
      a = fma(1.0, ws[70848], a);
      a = fma(0.3, ws[70880], a);
      a = fma(1.0, ws[70912], a);
      a = fma(1.0, ws[71008], a);
      a = fma(1.0, ws[71072], a);
      a = fma(1.0, ws[71104], a);
      a = fma(1.0, ws[71200], a);
      a = fma(0.5, ws[71232], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71552], a);
      a = fma(0.48, ws[71584], a);
      a = fma(0.48, ws[71616], a);
      a = fma(0.48, ws[71648], a);
      a = fma(0.48, ws[71680], a);
      a = fma(0.48, ws[71712], a);
      a = fma(0.48, ws[71744], a);
      a = fma(0.56, ws[71904], a);
      a = fma(0.333, ws[72000], a);
      a = fma(0.968, ws[72032], a);
      a = fma(1.0, ws[72064], a);
      a = a - ws[72096];
      a = fma(0.87, ws[72128], a);
      a = fma(0.8, ws[72160], a);
      a = fma(0.42, ws[72192], a);
      a = fma(0.49, ws[72256], a);
      a = fma(0.75, ws[72288], a);
      a = a - ws[72320];
      a = fma(0.32, ws[72320], a);
      a = fma(0.66, ws[72352], a);
      a = fma(1.0, ws[72448], a);
      a = a - ws[72512];
      a = a - ws[72672];
      a = a - ws[72896];
      a = a - ws[73824];
      a = a - ws[73856];
      a = a - ws[73888];
      a = a - ws[73920];
      a = a - ws[73952];
      a = a - ws[73984];
      a = a - ws[74016];
      a = fma(1.0, ws[74048], a);
      a = fma(1.0, ws[74080], a);
      a = fma(1.0, ws[74112], a);
      a = fma(1.0, ws[74144], a);
      a = fma(1.0, ws[74176], a);
      a = fma(1.0, ws[74208], a);
      a = fma(1.0, ws[74240], a);
      a = fma(0.86, ws[74272], a);
      a = fma(0.86, ws[74304], a);
      a = fma(0.86, ws[74336], a);
      a = fma(0.86, ws[74368], a);
      a = fma(0.86, ws[74400], a);
      a = fma(0.86, ws[74432], a);
      a = fma(0.88, ws[74464], a);
      a = fma(1.0, ws[74496], a);
      a = fma(1.0, ws[74528], a);
      a = fma(1.0, ws[74560], a);
      a = fma(1.0, ws[74592], a);
      a = fma(1.0, ws[74624], a);
      a = fma(1.0, ws[74656], a);
      a = fma(1.0, ws[74688], a);
      a = a - ws[74720];
      a = a - ws[74752];
      a = a - ws[74784];
      a = a - ws[74816];
      a = a - ws[74848];
      a = a - ws[74880];
      a = a - ws[74912];
      a = fma(0.16, ws[74944], a);
      a = a - ws[74976];
      a = fma(0.998, ws[75008], a);
      a = fma(0.9405, ws[75040], a);
      a = fma(1.3105, ws[75072], a);
      a = fma(0.9405, ws[75104], a);
      a = fma(0.16, ws[75136], a);
      a = a - ws[75168];
      a = fma(0.998, ws[75200], a);
      a = fma(0.9405, ws[75232], a);
      a = fma(1.3105, ws[75264], a);
      a = fma(0.9405, ws[75296], a);
      a = fma(0.16, ws[75328], a);
      a = a - ws[75360];
      a = fma(0.998, ws[75392], a);
      a = fma(0.9405, ws[75424], a);
      a = fma(1.3105, ws[75456], a);
      a = fma(0.9405, ws[75488], a);
      a = a - ws[76160];
      a = fma(1.0, ws[76192], a);
      a = fma(1.0, ws[76224], a);
      a = fma(1.37, ws[76256], a);
      a = fma(1.0, ws[76288], a);
      yout[5984] = a;
    }
    {
      double a = -ws[60608];
      a = fma(1.0, ws[60640], a);
      a = fma(2.0, ws[60864], a);
      a = a - ws[60896];
      a = a - ws[60928];
      a = a - ws[61024];
      a = a - ws[61088];
      a = fma(1.0, ws[61120], a);
      a = a - ws[61216];
      a = a - ws[61312];
      a = a - ws[61344];
      a = a - ws[61376];
      a = fma(0.7, ws[61408], a);
      a = a - ws[61696];
      a = a - ws[61728];
      a = a - ws[61760];
      a = a - ws[61792];
      a = a - ws[61824];
      a = a - ws[61856];
      a = a - ws[61888];
      a = a - ws[61920];
      a = a - ws[61952];
      a = a - ws[61984];
      a = a - ws[62016];
      a = fma(0.65, ws[62016], a);
      a = a - ws[62048];
      a = a - ws[62080];
      a = a - ws[62112];
      a = a - ws[62144];
      a = fma(0.25, ws[62176], a);
      a = a - ws[62240];
      a = fma(0.5, ws[62272], a);
      a = a - ws[62336];
      a = a - ws[62368];
      a = fma(2.0, ws[62368], a);
      a = fma(0.45, ws[62400], a);
      a = a - ws[62464];
      a = fma(1.0, ws[62464], a);
      a = a - ws[62496];
      a = a - ws[62560];
      a = a - ws[62592];
      a = a - ws[62624];
      a = a - ws[62656];
      a = a - ws[62688];
      a = a - ws[62720];
      a = a - ws[62752];
      a = a - ws[62784];
      a = a - ws[62816];
      a = a - ws[62848];
      a = a - ws[62880];
      a = a - ws[62912];
      a = a - ws[62944];
      a = a - ws[62976];
      a = a - ws[63008];
      a = a - ws[63040];
      a = a - ws[63072];
      a = a - ws[63104];
      a = a - ws[63136];
      a = a - ws[63168];
      a = a - ws[63200];
      a = a - ws[63232];
      a = a - ws[63264];
      a = a - ws[63296];
      a = a - ws[63328];
      a = a - ws[63360];
      a = a - ws[63392];
      a = a - ws[63424];
      a = a - ws[63456];
      a = fma(0.35, ws[63456], a);
      a = a - ws[63488];
      a = fma(0.01, ws[63488], a);
      a = a - ws[63520];
      a = fma(0.01, ws[63520], a);
      a = a - ws[63552];
      a = fma(0.01, ws[63552], a);
      a = a - ws[63584];
      a = a - ws[63616];
      a = a - ws[63648];
      a = a - ws[63680];
      a = fma(0.35, ws[63680], a);
      a = a - ws[63712];
      a = a - ws[63744];
      a = a - ws[63776];
      a = a - ws[63808];
      a = a - ws[63840];
      a = a - ws[63872];
      a = fma(0.08, ws[63904], a);
      a = fma(0.22, ws[63936], a);
      a = fma(0.46, ws[63968], a);
      a = fma(0.6055, ws[64000], a);
      a = fma(0.66, ws[64032], a);
      a = fma(0.09, ws[64064], a);
      a = fma(0.19, ws[64128], a);
      a = fma(0.16, ws[64160], a);
      a = fma(0.1, ws[64192], a);
      a = fma(0.05, ws[64224], a);
      a = fma(0.05, ws[64256], a);
      a = fma(0.05, ws[64288], a);
      a = fma(0.82, ws[65536], a);
      a = fma(0.82, ws[65600], a);
      a = fma(0.77, ws[65664], a);
      a = fma(0.77, ws[65728], a);
      a = fma(0.238, ws[66848], a);
      a = fma(0.6195, ws[66912], a);
      a = fma(0.1, ws[66976], a);
      a = fma(0.5, ws[67040], a);
      a = fma(0.25, ws[67104], a);
      a = fma(0.1, ws[67136], a);
      a = fma(0.44, ws[67168], a);
      a = fma(0.44, ws[67200], a);
      a = fma(0.15, ws[67232], a);
      a = fma(0.5, ws[69312], a);
      a = fma(0.5, ws[69440], a);
      a = fma(0.48, ws[71392], a);
      a = fma(0.48, ws[71424], a);
      a = fma(0.48, ws[71456], a);
      a = fma(0.48, ws[71488], a);
      a = fma(0.48, ws[71520], a);
      a = fma(0.48, ws[71552], a);
      a = a - ws[71776];
      a = fma(1.0, ws[71776], a);
      a = a - ws[71808];
      a = a - ws[71840];
      a = a - ws[71872];
      a = fma(0.28, ws[71904], a);
      a = a - ws[72000];
      a = fma(0.08, ws[72192], a);
      a = a - ws[72256];
      a = fma(0.4, ws[72320], a);
      a = a - ws[72352];
      a = fma(0.02, ws[72384], a);
      a = a - ws[72448];
      a = a - ws[72640];
      a = a - ws[73152];
      a = a - ws[73184];
      a = a - ws[73216];
      a = a - ws[73248];
      a = a - ws[73280];
      a = a - ws[73312];
      a = a - ws[73344];
      a = a - ws[74944];
      a = a - ws[75136];
      a = a - ws[75328];
      a = a - ws[75520];
      a = fma(1.0, ws[75520], a);
      a = a - ws[75552];
      a = fma(1.0, ws[75552], a);
      a = a - ws[75584];
      a = fma(1.0, ws[75584], a);
      a = a - ws[75616];
      a = fma(1.0, ws[75616], a);
      a = a - ws[75648];
      a = fma(1.0, ws[75648], a);
      a = a - ws[75680];
      a = fma(1.0, ws[75680], a);
      a = a - ws[75712];
      a = fma(1.0, ws[75712], a);
      a = a - ws[75744];
      a = fma(1.0, ws[75744], a);
      a = a - ws[75776];
      a = fma(1.0, ws[75776], a);
      a = a - ws[75808];
      a = fma(1.0, ws[75808], a);
      a = a - ws[75840];
      a = fma(1.0, ws[75840], a);
      a = a - ws[75872];
      a = fma(1.0, ws[75872], a);
      a = a - ws[75904];
      a = fma(1.0, ws[75904], a);
      a = a - ws[75936];
      a = fma(1.0, ws[75936], a);
      a = a - ws[75968];
      a = fma(1.0, ws[75968], a);
      a = a - ws[76000];
      a = fma(1.0, ws[76000], a);
      a = a - ws[76032];
      a = a - ws[76128];
      yout[6016] = a;
    }
}
// Partial-derivative products of 2- and 3-reactant reactions (rbjacob.F:112-143).
__device__ __noinline__ void explic_1(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    { const double kk = ws[43616]; ws[76320] = kk * y[6016]; ws[76352] = kk * y[5184]; }
    { const double kk = ws[43648]; ws[76384] = kk * y[5984]; ws[76416] = kk * y[5184]; }
    { const double kk = ws[43680]; ws[76448] = kk * y[5824]; ws[76480] = kk * y[5184]; }
    { const double kk = ws[43712]; ws[76512] = kk * y[5920]; ws[76544] = kk * y[5184]; }
    { const double kk = ws[43776]; ws[76576] = kk * y[5184]; ws[76608] = kk * y[2336]; }
    { const double kk = ws[43936]; ws[76640] = kk * y[5984]; ws[76672] = kk * y[6016]; }
    { const double kk = ws[43968]; ws[76704] = kk * y[5984]; ws[76736] = kk * y[5984]; }
    { const double kk = ws[44000]; ws[76768] = kk * y[5984]; ws[76800] = kk * y[5984]; }
    { const double kk = ws[44032]; ws[76832] = kk * y[6016]; ws[76864] = kk * y[4000]; }
    { const double kk = ws[44064]; ws[76896] = kk * y[2336]; ws[76928] = kk * y[5824]; }
    { const double kk = ws[44096]; ws[76960] = kk * y[6016]; ws[76992] = kk * y[5824]; }
    { const double kk = ws[44128]; ws[77024] = kk * y[5984]; ws[77056] = kk * y[5824]; }
    { const double kk = ws[44160]; ws[77088] = kk * y[5984]; ws[77120] = kk * y[5824]; }
    { const double kk = ws[44192]; ws[77152] = kk * y[5824]; ws[77184] = kk * y[5824]; }
    { const double kk = ws[44224]; ws[77216] = kk * y[6016]; ws[77248] = kk * y[1184]; }
    { const double kk = ws[44256]; ws[77280] = kk * y[2336]; ws[77312] = kk * y[5920]; }
    { const double kk = ws[44288]; ws[77344] = kk * y[2336]; ws[77376] = kk * y[5920]; }
    { const double kk = ws[44320]; ws[77408] = kk * y[6016]; ws[77440] = kk * y[5920]; }
    { const double kk = ws[44352]; ws[77472] = kk * y[6016]; ws[77504] = kk * y[5024]; }
    { const double kk = ws[44384]; ws[77536] = kk * y[6016]; ws[77568] = kk * y[5952]; }
    { const double kk = ws[44416]; ws[77600] = kk * y[5984]; ws[77632] = kk * y[5952]; }
    { const double kk = ws[44448]; ws[77664] = kk * y[5824]; ws[77696] = kk * y[5952]; }
    { const double kk = ws[44480]; ws[77728] = kk * y[5920]; ws[77760] = kk * y[5952]; }
    { const double kk = ws[44512]; ws[77792] = kk * y[5952]; ws[77824] = kk * y[5952]; }
    { const double kk = ws[44544]; ws[77856] = kk * y[5920]; ws[77888] = kk * y[5952]; }
    { const double kk = ws[44640]; ws[77920] = kk * y[5984]; ws[77952] = kk * y[5920]; }
    { const double kk = ws[44704]; ws[77984] = kk * y[6016]; ws[78016] = kk * y[1280]; }
    { const double kk = ws[44736]; ws[78048] = kk * y[6016]; ws[78080] = kk * y[160]; }
    { const double kk = ws[44768]; ws[78112] = kk * y[6016]; ws[78144] = kk * y[5664]; }
    { const double kk = ws[44832]; ws[78176] = kk * y[6016]; ws[78208] = kk * y[1888]; }
    { const double kk = ws[44864]; ws[78240] = kk * y[6016]; ws[78272] = kk * y[2176]; }
    { const double kk = ws[44896]; ws[78304] = kk * y[6016]; ws[78336] = kk * y[1120]; }
    { const double kk = ws[44928]; ws[78368] = kk * y[6016]; ws[78400] = kk * y[2240]; }
    { const double kk = ws[44960]; ws[78432] = kk * y[6016]; ws[78464] = kk * y[2752]; }
    { const double kk = ws[44992]; ws[78496] = kk * y[6016]; ws[78528] = kk * y[1152]; }
    { const double kk = ws[45024]; ws[78560] = kk * y[6016]; ws[78592] = kk * y[256]; }
    { const double kk = ws[45056]; ws[78624] = kk * y[6016]; ws[78656] = kk * y[1216]; }
    { const double kk = ws[45088]; ws[78688] = kk * y[6016]; ws[78720] = kk * y[288]; }
    { const double kk = ws[45120]; ws[78752] = kk * y[6016]; ws[78784] = kk * y[320]; }
    { const double kk = ws[45152]; ws[78816] = kk * y[6016]; ws[78848] = kk * y[352]; }
    { const double kk = ws[45184]; ws[78880] = kk * y[5184]; ws[78912] = kk * y[1312]; }
    { const double kk = ws[45216]; ws[78944] = kk * y[5952]; ws[78976] = kk * y[1312]; }
    { const double kk = ws[45248]; ws[79008] = kk * y[6016]; ws[79040] = kk * y[1312]; }
    { const double kk = ws[45280]; ws[79072] = kk * y[5984]; ws[79104] = kk * y[4288]; }
    { const double kk = ws[45312]; ws[79136] = kk * y[5824]; ws[79168] = kk * y[4288]; }
    { const double kk = ws[45344]; ws[79200] = kk * y[6016]; ws[79232] = kk * y[1344]; }
    { const double kk = ws[45376]; ws[79264] = kk * y[6016]; ws[79296] = kk * y[1344]; }
    { const double kk = ws[45408]; ws[79328] = kk * y[5984]; ws[79360] = kk * y[1632]; }
    { const double kk = ws[45440]; ws[79392] = kk * y[5824]; ws[79424] = kk * y[1632]; }
    { const double kk = ws[45472]; ws[79456] = kk * y[6016]; ws[79488] = kk * y[2784]; }
    { const double kk = ws[45504]; ws[79520] = kk * y[2208]; ws[79552] = kk * y[6016]; }
    { const double kk = ws[45568]; ws[79584] = kk * y[6016]; ws[79616] = kk * y[1664]; }
    { const double kk = ws[45600]; ws[79648] = kk * y[6016]; ws[79680] = kk * y[1408]; }
    { const double kk = ws[45632]; ws[79712] = kk * y[6016]; ws[79744] = kk * y[1440]; }
    { const double kk = ws[45664]; ws[79776] = kk * y[6016]; ws[79808] = kk * y[4544]; }
    { const double kk = ws[45696]; ws[79840] = kk * y[6016]; ws[79872] = kk * y[4576]; }
    { const double kk = ws[45728]; ws[79904] = kk * y[6016]; ws[79936] = kk * y[5856]; }
    { const double kk = ws[45760]; ws[79968] = kk * y[6016]; ws[80000] = kk * y[5568]; }
    { const double kk = ws[45792]; ws[80032] = kk * y[6016]; ws[80064] = kk * y[5760]; }
    { const double kk = ws[45824]; ws[80096] = kk * y[6016]; ws[80128] = kk * y[4480]; }
    { const double kk = ws[45856]; ws[80160] = kk * y[6016]; ws[80192] = kk * y[5280]; }
    { const double kk = ws[45888]; ws[80224] = kk * y[6016]; ws[80256] = kk * y[5504]; }
    { const double kk = ws[45920]; ws[80288] = kk * y[6016]; ws[80320] = kk * y[5344]; }
    { const double kk = ws[45952]; ws[80352] = kk * y[6016]; ws[80384] = kk * y[4128]; }
    { const double kk = ws[45984]; ws[80416] = kk * y[6016]; ws[80448] = kk * y[4736]; }
    { const double kk = ws[46016]; ws[80480] = kk * y[6016]; ws[80512] = kk * y[3872]; }
    { const double kk = ws[46048]; ws[80544] = kk * y[6016]; ws[80576] = kk * y[5376]; }
    { const double kk = ws[46080]; ws[80608] = kk * y[6016]; ws[80640] = kk * y[5248]; }
    { const double kk = ws[46112]; ws[80672] = kk * y[6016]; ws[80704] = kk * y[5472]; }
    { const double kk = ws[46144]; ws[80736] = kk * y[6016]; ws[80768] = kk * y[4320]; }
    { const double kk = ws[46176]; ws[80800] = kk * y[6016]; ws[80832] = kk * y[3584]; }
    { const double kk = ws[46208]; ws[80864] = kk * y[6016]; ws[80896] = kk * y[4448]; }
    { const double kk = ws[46240]; ws[80928] = kk * y[6016]; ws[80960] = kk * y[1248]; }
    { const double kk = ws[46272]; ws[80992] = kk * y[6016]; ws[81024] = kk * y[2944]; }
    { const double kk = ws[46304]; ws[81056] = kk * y[6016]; ws[81088] = kk * y[1760]; }
    { const double kk = ws[46336]; ws[81120] = kk * y[6016]; ws[81152] = kk * y[5600]; }
    { const double kk = ws[46368]; ws[81184] = kk * y[6016]; ws[81216] = kk * y[1472]; }
    { const double kk = ws[46400]; ws[81248] = kk * y[6016]; ws[81280] = kk * y[5056]; }
    { const double kk = ws[46432]; ws[81312] = kk * y[6016]; ws[81344] = kk * y[1504]; }
    { const double kk = ws[46464]; ws[81376] = kk * y[6016]; ws[81408] = kk * y[2816]; }
    { const double kk = ws[46496]; ws[81440] = kk * y[6016]; ws[81472] = kk * y[5728]; }
    { const double kk = ws[46528]; ws[81504] = kk * y[6016]; ws[81536] = kk * y[4096]; }
    { const double kk = ws[46560]; ws[81568] = kk * y[6016]; ws[81600] = kk * y[4608]; }
    { const double kk = ws[46592]; ws[81632] = kk * y[6016]; ws[81664] = kk * y[1792]; }
    { const double kk = ws[46624]; ws[81696] = kk * y[6016]; ws[81728] = kk * y[4352]; }
    { const double kk = ws[46656]; ws[81760] = kk * y[6016]; ws[81792] = kk * y[5696]; }
    { const double kk = ws[46688]; ws[81824] = kk * y[6016]; ws[81856] = kk * y[3680]; }
    { const double kk = ws[46720]; ws[81888] = kk * y[6016]; ws[81920] = kk * y[1088]; }
    { const double kk = ws[46752]; ws[81952] = kk * y[6016]; ws[81984] = kk * y[1536]; }
    { const double kk = ws[46784]; ws[82016] = kk * y[6016]; ws[82048] = kk * y[1824]; }
    { const double kk = ws[46816]; ws[82080] = kk * y[6016]; ws[82112] = kk * y[5440]; }
    { const double kk = ws[46848]; ws[82144] = kk * y[6016]; ws[82176] = kk * y[4384]; }
    { const double kk = ws[46880]; ws[82208] = kk * y[6016]; ws[82240] = kk * y[1696]; }
    { const double kk = ws[46912]; ws[82272] = kk * y[5184]; ws[82304] = kk * y[2240]; }
    { const double kk = ws[46944]; ws[82336] = kk * y[5184]; ws[82368] = kk * y[2752]; }
    { const double kk = ws[46976]; ws[82400] = kk * y[5184]; ws[82432] = kk * y[1152]; }
    { const double kk = ws[47008]; ws[82464] = kk * y[5184]; ws[82496] = kk * y[1408]; }
    { const double kk = ws[47040]; ws[82528] = kk * y[5184]; ws[82560] = kk * y[1440]; }
    { const double kk = ws[47072]; ws[82592] = kk * y[5184]; ws[82624] = kk * y[4576]; }
    { const double kk = ws[47104]; ws[82656] = kk * y[5184]; ws[82688] = kk * y[4384]; }
    { const double kk = ws[47136]; ws[82720] = kk * y[5184]; ws[82752] = kk * y[4128]; }
    { const double kk = ws[47168]; ws[82784] = kk * y[5184]; ws[82816] = kk * y[4736]; }
    { const double kk = ws[47200]; ws[82848] = kk * y[5184]; ws[82880] = kk * y[3872]; }
    { const double kk = ws[47232]; ws[82912] = kk * y[5184]; ws[82944] = kk * y[5472]; }
    { const double kk = ws[47264]; ws[82976] = kk * y[5184]; ws[83008] = kk * y[4320]; }
    { const double kk = ws[47296]; ws[83040] = kk * y[5184]; ws[83072] = kk * y[3584]; }
    { const double kk = ws[47328]; ws[83104] = kk * y[5184]; ws[83136] = kk * y[3808]; }
    { const double kk = ws[47360]; ws[83168] = kk * y[5952]; ws[83200] = kk * y[2240]; }
    { const double kk = ws[47392]; ws[83232] = kk * y[5952]; ws[83264] = kk * y[2752]; }
    { const double kk = ws[47424]; ws[83296] = kk * y[5952]; ws[83328] = kk * y[1152]; }
    { const double kk = ws[47456]; ws[83360] = kk * y[5952]; ws[83392] = kk * y[1408]; }
    { const double kk = ws[47488]; ws[83424] = kk * y[5952]; ws[83456] = kk * y[1440]; }
    { const double kk = ws[47520]; ws[83488] = kk * y[5952]; ws[83520] = kk * y[4384]; }
    { const double kk = ws[47552]; ws[83552] = kk * y[5952]; ws[83584] = kk * y[5856]; }
    { const double kk = ws[47584]; ws[83616] = kk * y[5952]; ws[83648] = kk * y[5568]; }
    { const double kk = ws[47616]; ws[83680] = kk * y[5952]; ws[83712] = kk * y[5760]; }
    { const double kk = ws[47648]; ws[83744] = kk * y[5952]; ws[83776] = kk * y[4128]; }
    { const double kk = ws[47680]; ws[83808] = kk * y[5952]; ws[83840] = kk * y[3872]; }
    { const double kk = ws[47712]; ws[83872] = kk * y[5952]; ws[83904] = kk * y[5376]; }
    { const double kk = ws[47744]; ws[83936] = kk * y[5952]; ws[83968] = kk * y[5248]; }
    { const double kk = ws[47776]; ws[84000] = kk * y[5952]; ws[84032] = kk * y[1248]; }
    { const double kk = ws[47808]; ws[84064] = kk * y[5952]; ws[84096] = kk * y[2944]; }
    { const double kk = ws[47840]; ws[84128] = kk * y[5952]; ws[84160] = kk * y[1760]; }
    { const double kk = ws[47872]; ws[84192] = kk * y[5952]; ws[84224] = kk * y[1824]; }
    { const double kk = ws[47968]; ws[84256] = kk * y[5920]; ws[84288] = kk * y[5792]; }
    { const double kk = ws[48032]; ws[84320] = kk * y[5920]; ws[84352] = kk * y[4800]; }
    { const double kk = ws[48096]; ws[84384] = kk * y[5920]; ws[84416] = kk * y[4672]; }
    { const double kk = ws[48160]; ws[84448] = kk * y[5824]; ws[84480] = kk * y[5888]; }
    { const double kk = ws[48192]; ws[84512] = kk * y[5824]; ws[84544] = kk * y[5632]; }
    { const double kk = ws[48224]; ws[84576] = kk * y[5824]; ws[84608] = kk * y[5408]; }
    { const double kk = ws[48256]; ws[84640] = kk * y[5824]; ws[84672] = kk * y[5120]; }
    { const double kk = ws[48288]; ws[84704] = kk * y[5824]; ws[84736] = kk * y[3008]; }
    { const double kk = ws[48320]; ws[84768] = kk * y[5824]; ws[84800] = kk * y[3200]; }
    { const double kk = ws[48352]; ws[84832] = kk * y[5824]; ws[84864] = kk * y[3328]; }
    { const double kk = ws[48384]; ws[84896] = kk * y[5824]; ws[84928] = kk * y[3360]; }
    { const double kk = ws[48416]; ws[84960] = kk * y[5824]; ws[84992] = kk * y[3296]; }
    { const double kk = ws[48448]; ws[85024] = kk * y[5824]; ws[85056] = kk * y[3104]; }
    { const double kk = ws[48480]; ws[85088] = kk * y[5824]; ws[85120] = kk * y[3264]; }
    { const double kk = ws[48512]; ws[85152] = kk * y[5824]; ws[85184] = kk * y[4160]; }
    { const double kk = ws[48544]; ws[85216] = kk * y[5824]; ws[85248] = kk * y[3744]; }
    { const double kk = ws[48576]; ws[85280] = kk * y[5824]; ws[85312] = kk * y[2624]; }
    { const double kk = ws[48608]; ws[85344] = kk * y[5824]; ws[85376] = kk * y[3840]; }
    { const double kk = ws[48640]; ws[85408] = kk * y[5824]; ws[85440] = kk * y[4192]; }
    { const double kk = ws[48672]; ws[85472] = kk * y[5824]; ws[85504] = kk * y[3936]; }
    { const double kk = ws[48704]; ws[85536] = kk * y[5824]; ws[85568] = kk * y[2656]; }
    { const double kk = ws[48736]; ws[85600] = kk * y[5824]; ws[85632] = kk * y[3712]; }
    { const double kk = ws[48768]; ws[85664] = kk * y[5824]; ws[85696] = kk * y[2560]; }
    { const double kk = ws[48800]; ws[85728] = kk * y[5824]; ws[85760] = kk * y[1728]; }
    { const double kk = ws[48832]; ws[85792] = kk * y[5824]; ws[85824] = kk * y[5792]; }
    { const double kk = ws[48864]; ws[85856] = kk * y[5824]; ws[85888] = kk * y[4800]; }
    { const double kk = ws[48896]; ws[85920] = kk * y[5824]; ws[85952] = kk * y[2848]; }
    { const double kk = ws[48928]; ws[85984] = kk * y[5824]; ws[86016] = kk * y[5152]; }
    { const double kk = ws[48960]; ws[86048] = kk * y[5824]; ws[86080] = kk * y[3776]; }
    { const double kk = ws[48992]; ws[86112] = kk * y[5824]; ws[86144] = kk * y[4672]; }
    { const double kk = ws[49024]; ws[86176] = kk * y[5824]; ws[86208] = kk * y[3520]; }
    { const double kk = ws[49056]; ws[86240] = kk * y[5824]; ws[86272] = kk * y[2880]; }
    { const double kk = ws[49088]; ws[86304] = kk * y[5824]; ws[86336] = kk * y[2912]; }
    { const double kk = ws[49120]; ws[86368] = kk * y[5824]; ws[86400] = kk * y[2592]; }
    { const double kk = ws[49152]; ws[86432] = kk * y[5824]; ws[86464] = kk * y[2272]; }
    { const double kk = ws[49184]; ws[86496] = kk * y[5824]; ws[86528] = kk * y[3648]; }
    { const double kk = ws[49216]; ws[86560] = kk * y[5824]; ws[86592] = kk * y[3040]; }
    { const double kk = ws[49248]; ws[86624] = kk * y[5824]; ws[86656] = kk * y[2976]; }
    { const double kk = ws[49280]; ws[86688] = kk * y[5824]; ws[86720] = kk * y[4032]; }
    { const double kk = ws[49312]; ws[86752] = kk * y[5824]; ws[86784] = kk * y[4064]; }
    { const double kk = ws[49344]; ws[86816] = kk * y[5824]; ws[86848] = kk * y[3072]; }
    { const double kk = ws[49376]; ws[86880] = kk * y[5824]; ws[86912] = kk * y[5216]; }
    { const double kk = ws[49408]; ws[86944] = kk * y[5920]; ws[86976] = kk * y[2688]; }
    { const double kk = ws[49440]; ws[87008] = kk * y[5920]; ws[87040] = kk * y[3232]; }
    { const double kk = ws[49472]; ws[87072] = kk * y[5920]; ws[87104] = kk * y[3808]; }
    { const double kk = ws[49504]; ws[87136] = kk * y[5984]; ws[87168] = kk * y[5888]; }
    { const double kk = ws[49536]; ws[87200] = kk * y[5984]; ws[87232] = kk * y[5632]; }
    { const double kk = ws[49568]; ws[87264] = kk * y[5984]; ws[87296] = kk * y[5408]; }
    { const double kk = ws[49600]; ws[87328] = kk * y[5984]; ws[87360] = kk * y[5120]; }
    { const double kk = ws[49632]; ws[87392] = kk * y[5984]; ws[87424] = kk * y[3008]; }
    { const double kk = ws[49664]; ws[87456] = kk * y[5984]; ws[87488] = kk * y[3200]; }
    { const double kk = ws[49696]; ws[87520] = kk * y[5984]; ws[87552] = kk * y[3328]; }
    { const double kk = ws[49728]; ws[87584] = kk * y[5984]; ws[87616] = kk * y[3360]; }
    { const double kk = ws[49760]; ws[87648] = kk * y[5984]; ws[87680] = kk * y[3296]; }
    { const double kk = ws[49792]; ws[87712] = kk * y[5984]; ws[87744] = kk * y[3104]; }
    { const double kk = ws[49824]; ws[87776] = kk * y[5984]; ws[87808] = kk * y[3264]; }
    { const double kk = ws[49856]; ws[87840] = kk * y[5984]; ws[87872] = kk * y[4160]; }
    { const double kk = ws[49888]; ws[87904] = kk * y[5984]; ws[87936] = kk * y[3744]; }
    { const double kk = ws[49920]; ws[87968] = kk * y[5984]; ws[88000] = kk * y[2624]; }
    { const double kk = ws[49952]; ws[88032] = kk * y[5984]; ws[88064] = kk * y[3840]; }
    { const double kk = ws[49984]; ws[88096] = kk * y[5984]; ws[88128] = kk * y[4192]; }
    { const double kk = ws[50016]; ws[88160] = kk * y[5984]; ws[88192] = kk * y[3936]; }
    { const double kk = ws[50048]; ws[88224] = kk * y[5984]; ws[88256] = kk * y[2656]; }
    { const double kk = ws[50080]; ws[88288] = kk * y[5984]; ws[88320] = kk * y[3712]; }
    { const double kk = ws[50112]; ws[88352] = kk * y[5984]; ws[88384] = kk * y[2560]; }
    { const double kk = ws[50144]; ws[88416] = kk * y[5984]; ws[88448] = kk * y[1728]; }
    { const double kk = ws[50176]; ws[88480] = kk * y[5984]; ws[88512] = kk * y[5792]; }
    { const double kk = ws[50208]; ws[88544] = kk * y[5984]; ws[88576] = kk * y[4800]; }
    { const double kk = ws[50240]; ws[88608] = kk * y[5984]; ws[88640] = kk * y[2848]; }
    { const double kk = ws[50272]; ws[88672] = kk * y[5984]; ws[88704] = kk * y[5152]; }
    { const double kk = ws[50304]; ws[88736] = kk * y[5984]; ws[88768] = kk * y[3776]; }
    { const double kk = ws[50336]; ws[88800] = kk * y[5984]; ws[88832] = kk * y[4672]; }
    { const double kk = ws[50368]; ws[88864] = kk * y[5984]; ws[88896] = kk * y[3520]; }
    { const double kk = ws[50400]; ws[88928] = kk * y[5984]; ws[88960] = kk * y[2880]; }
    { const double kk = ws[50432]; ws[88992] = kk * y[5984]; ws[89024] = kk * y[2912]; }
    { const double kk = ws[50464]; ws[89056] = kk * y[5984]; ws[89088] = kk * y[3648]; }
    { const double kk = ws[50496]; ws[89120] = kk * y[5984]; ws[89152] = kk * y[3232]; }
    { const double kk = ws[50528]; ws[89184] = kk * y[5984]; ws[89216] = kk * y[3040]; }
    { const double kk = ws[50560]; ws[89248] = kk * y[5984]; ws[89280] = kk * y[2976]; }
    { const double kk = ws[50592]; ws[89312] = kk * y[5984]; ws[89344] = kk * y[4032]; }
    { const double kk = ws[50624]; ws[89376] = kk * y[5984]; ws[89408] = kk * y[4064]; }
    { const double kk = ws[50656]; ws[89440] = kk * y[5984]; ws[89472] = kk * y[3072]; }
    { const double kk = ws[50688]; ws[89504] = kk * y[5984]; ws[89536] = kk * y[5216]; }
    { const double kk = ws[50720]; ws[89568] = kk * y[5888]; ws[89600] = kk * y[5888]; }
    { const double kk = ws[50752]; ws[89632] = kk * y[5888]; ws[89664] = kk * y[5632]; }
    { const double kk = ws[50784]; ws[89696] = kk * y[5888]; ws[89728] = kk * y[5408]; }
    { const double kk = ws[50816]; ws[89760] = kk * y[5888]; ws[89792] = kk * y[5120]; }
    { const double kk = ws[50848]; ws[89824] = kk * y[5888]; ws[89856] = kk * y[3008]; }
    { const double kk = ws[50880]; ws[89888] = kk * y[5888]; ws[89920] = kk * y[3200]; }
    { const double kk = ws[50912]; ws[89952] = kk * y[5888]; ws[89984] = kk * y[3328]; }
    { const double kk = ws[50944]; ws[90016] = kk * y[5888]; ws[90048] = kk * y[3360]; }
    { const double kk = ws[50976]; ws[90080] = kk * y[5888]; ws[90112] = kk * y[3296]; }
    { const double kk = ws[51008]; ws[90144] = kk * y[5888]; ws[90176] = kk * y[3104]; }
    { const double kk = ws[51040]; ws[90208] = kk * y[5888]; ws[90240] = kk * y[3264]; }
    { const double kk = ws[51072]; ws[90272] = kk * y[5888]; ws[90304] = kk * y[4288]; }
    { const double kk = ws[51104]; ws[90336] = kk * y[5888]; ws[90368] = kk * y[4160]; }
    { const double kk = ws[51136]; ws[90400] = kk * y[5888]; ws[90432] = kk * y[3744]; }
    { const double kk = ws[51168]; ws[90464] = kk * y[5888]; ws[90496] = kk * y[2624]; }
    { const double kk = ws[51200]; ws[90528] = kk * y[5888]; ws[90560] = kk * y[3840]; }
    { const double kk = ws[51232]; ws[90592] = kk * y[5888]; ws[90624] = kk * y[4192]; }
    { const double kk = ws[51264]; ws[90656] = kk * y[5888]; ws[90688] = kk * y[3936]; }
    { const double kk = ws[51296]; ws[90720] = kk * y[5888]; ws[90752] = kk * y[2656]; }
    { const double kk = ws[51328]; ws[90784] = kk * y[5888]; ws[90816] = kk * y[3712]; }
    { const double kk = ws[51360]; ws[90848] = kk * y[5888]; ws[90880] = kk * y[5792]; }
    { const double kk = ws[51392]; ws[90912] = kk * y[5888]; ws[90944] = kk * y[4800]; }
    { const double kk = ws[51424]; ws[90976] = kk * y[5888]; ws[91008] = kk * y[2848]; }
    { const double kk = ws[51456]; ws[91040] = kk * y[5888]; ws[91072] = kk * y[5152]; }
    { const double kk = ws[51488]; ws[91104] = kk * y[5888]; ws[91136] = kk * y[3776]; }
    { const double kk = ws[51520]; ws[91168] = kk * y[5888]; ws[91200] = kk * y[4672]; }
    { const double kk = ws[51552]; ws[91232] = kk * y[5888]; ws[91264] = kk * y[3520]; }
    { const double kk = ws[51584]; ws[91296] = kk * y[5888]; ws[91328] = kk * y[2880]; }
    { const double kk = ws[51616]; ws[91360] = kk * y[5888]; ws[91392] = kk * y[2912]; }
    { const double kk = ws[51648]; ws[91424] = kk * y[5888]; ws[91456] = kk * y[2592]; }
    { const double kk = ws[51680]; ws[91488] = kk * y[5888]; ws[91520] = kk * y[2272]; }
    { const double kk = ws[51712]; ws[91552] = kk * y[5888]; ws[91584] = kk * y[3648]; }
    { const double kk = ws[51744]; ws[91616] = kk * y[5888]; ws[91648] = kk * y[3040]; }
    { const double kk = ws[51776]; ws[91680] = kk * y[5888]; ws[91712] = kk * y[2976]; }
    { const double kk = ws[51808]; ws[91744] = kk * y[5888]; ws[91776] = kk * y[4032]; }
    { const double kk = ws[51840]; ws[91808] = kk * y[5888]; ws[91840] = kk * y[4064]; }
    { const double kk = ws[51872]; ws[91872] = kk * y[5888]; ws[91904] = kk * y[3072]; }
    { const double kk = ws[51904]; ws[91936] = kk * y[5888]; ws[91968] = kk * y[5216]; }
    { const double kk = ws[51936]; ws[92000] = kk * y[5792]; ws[92032] = kk * y[5632]; }
    { const double kk = ws[51968]; ws[92064] = kk * y[5792]; ws[92096] = kk * y[5408]; }
    { const double kk = ws[52000]; ws[92128] = kk * y[5792]; ws[92160] = kk * y[5120]; }
    { const double kk = ws[52032]; ws[92192] = kk * y[5792]; ws[92224] = kk * y[3008]; }
    { const double kk = ws[52064]; ws[92256] = kk * y[5792]; ws[92288] = kk * y[3200]; }
    { const double kk = ws[52096]; ws[92320] = kk * y[5792]; ws[92352] = kk * y[3328]; }
    { const double kk = ws[52128]; ws[92384] = kk * y[5792]; ws[92416] = kk * y[3360]; }
    { const double kk = ws[52160]; ws[92448] = kk * y[5792]; ws[92480] = kk * y[3296]; }
    { const double kk = ws[52192]; ws[92512] = kk * y[5792]; ws[92544] = kk * y[3104]; }
    { const double kk = ws[52224]; ws[92576] = kk * y[5792]; ws[92608] = kk * y[3264]; }
    { const double kk = ws[52256]; ws[92640] = kk * y[5792]; ws[92672] = kk * y[4288]; }
    { const double kk = ws[52288]; ws[92704] = kk * y[5792]; ws[92736] = kk * y[4160]; }
    { const double kk = ws[52320]; ws[92768] = kk * y[5792]; ws[92800] = kk * y[3744]; }
    { const double kk = ws[52352]; ws[92832] = kk * y[5792]; ws[92864] = kk * y[2624]; }
    { const double kk = ws[52384]; ws[92896] = kk * y[5792]; ws[92928] = kk * y[3840]; }
    { const double kk = ws[52416]; ws[92960] = kk * y[5792]; ws[92992] = kk * y[4192]; }
    { const double kk = ws[52448]; ws[93024] = kk * y[5792]; ws[93056] = kk * y[3936]; }
    { const double kk = ws[52480]; ws[93088] = kk * y[5792]; ws[93120] = kk * y[2656]; }
    { const double kk = ws[52512]; ws[93152] = kk * y[5792]; ws[93184] = kk * y[3712]; }
    { const double kk = ws[52544]; ws[93216] = kk * y[5792]; ws[93248] = kk * y[5792]; }
    { const double kk = ws[52576]; ws[93280] = kk * y[5792]; ws[93312] = kk * y[4800]; }
    { const double kk = ws[52608]; ws[93344] = kk * y[5792]; ws[93376] = kk * y[2848]; }
    { const double kk = ws[52640]; ws[93408] = kk * y[5792]; ws[93440] = kk * y[5152]; }
    { const double kk = ws[52672]; ws[93472] = kk * y[5792]; ws[93504] = kk * y[3776]; }
    { const double kk = ws[52704]; ws[93536] = kk * y[5792]; ws[93568] = kk * y[4672]; }
    { const double kk = ws[52736]; ws[93600] = kk * y[5792]; ws[93632] = kk * y[3520]; }
    { const double kk = ws[52768]; ws[93664] = kk * y[5792]; ws[93696] = kk * y[2880]; }
    { const double kk = ws[52800]; ws[93728] = kk * y[5792]; ws[93760] = kk * y[2912]; }
    { const double kk = ws[52832]; ws[93792] = kk * y[5792]; ws[93824] = kk * y[2592]; }
    { const double kk = ws[52864]; ws[93856] = kk * y[5792]; ws[93888] = kk * y[2272]; }
    { const double kk = ws[52896]; ws[93920] = kk * y[5792]; ws[93952] = kk * y[3648]; }
    { const double kk = ws[52928]; ws[93984] = kk * y[5792]; ws[94016] = kk * y[3040]; }
    { const double kk = ws[52960]; ws[94048] = kk * y[5792]; ws[94080] = kk * y[2976]; }
    { const double kk = ws[52992]; ws[94112] = kk * y[5792]; ws[94144] = kk * y[4032]; }
    { const double kk = ws[53024]; ws[94176] = kk * y[5792]; ws[94208] = kk * y[4064]; }
    { const double kk = ws[53056]; ws[94240] = kk * y[5792]; ws[94272] = kk * y[3072]; }
    { const double kk = ws[53088]; ws[94304] = kk * y[5792]; ws[94336] = kk * y[5216]; }
    { const double kk = ws[53120]; ws[94368] = kk * y[4800]; ws[94400] = kk * y[4800]; }
    { const double kk = ws[53152]; ws[94432] = kk * y[5952]; ws[94464] = kk * y[5888]; }
    { const double kk = ws[53184]; ws[94496] = kk * y[5952]; ws[94528] = kk * y[5632]; }
    { const double kk = ws[53216]; ws[94560] = kk * y[5952]; ws[94592] = kk * y[5408]; }
    { const double kk = ws[53248]; ws[94624] = kk * y[5952]; ws[94656] = kk * y[5120]; }
    { const double kk = ws[53280]; ws[94688] = kk * y[5952]; ws[94720] = kk * y[3008]; }
    { const double kk = ws[53312]; ws[94752] = kk * y[5952]; ws[94784] = kk * y[3200]; }
    { const double kk = ws[53344]; ws[94816] = kk * y[5952]; ws[94848] = kk * y[3328]; }
    { const double kk = ws[53376]; ws[94880] = kk * y[5952]; ws[94912] = kk * y[3360]; }
    { const double kk = ws[53408]; ws[94944] = kk * y[5952]; ws[94976] = kk * y[3296]; }
    { const double kk = ws[53440]; ws[95008] = kk * y[5952]; ws[95040] = kk * y[3104]; }
    { const double kk = ws[53472]; ws[95072] = kk * y[5952]; ws[95104] = kk * y[3264]; }
    { const double kk = ws[53504]; ws[95136] = kk * y[5952]; ws[95168] = kk * y[4288]; }
    { const double kk = ws[53536]; ws[95200] = kk * y[5952]; ws[95232] = kk * y[4160]; }
    { const double kk = ws[53568]; ws[95264] = kk * y[5952]; ws[95296] = kk * y[4192]; }
    { const double kk = ws[53600]; ws[95328] = kk * y[5952]; ws[95360] = kk * y[2624]; }
    { const double kk = ws[53632]; ws[95392] = kk * y[5952]; ws[95424] = kk * y[2656]; }
    { const double kk = ws[53664]; ws[95456] = kk * y[5952]; ws[95488] = kk * y[5792]; }
    { const double kk = ws[53696]; ws[95520] = kk * y[5952]; ws[95552] = kk * y[4800]; }
    { const double kk = ws[53728]; ws[95584] = kk * y[5952]; ws[95616] = kk * y[2848]; }
    { const double kk = ws[53760]; ws[95648] = kk * y[5952]; ws[95680] = kk * y[5152]; }
    { const double kk = ws[53792]; ws[95712] = kk * y[5952]; ws[95744] = kk * y[3776]; }
    { const double kk = ws[53824]; ws[95776] = kk * y[5952]; ws[95808] = kk * y[4672]; }
    { const double kk = ws[53856]; ws[95840] = kk * y[5952]; ws[95872] = kk * y[3520]; }
    { const double kk = ws[53888]; ws[95904] = kk * y[5952]; ws[95936] = kk * y[2880]; }
    { const double kk = ws[53920]; ws[95968] = kk * y[5952]; ws[96000] = kk * y[2912]; }
    { const double kk = ws[53952]; ws[96032] = kk * y[5952]; ws[96064] = kk * y[2592]; }
    { const double kk = ws[53984]; ws[96096] = kk * y[5952]; ws[96128] = kk * y[2272]; }
    { const double kk = ws[54016]; ws[96160] = kk * y[5952]; ws[96192] = kk * y[3648]; }
    { const double kk = ws[54048]; ws[96224] = kk * y[5952]; ws[96256] = kk * y[3040]; }
    { const double kk = ws[54080]; ws[96288] = kk * y[5952]; ws[96320] = kk * y[2976]; }
    { const double kk = ws[54112]; ws[96352] = kk * y[5952]; ws[96384] = kk * y[4032]; }
    { const double kk = ws[54144]; ws[96416] = kk * y[5952]; ws[96448] = kk * y[4064]; }
    { const double kk = ws[54176]; ws[96480] = kk * y[5952]; ws[96512] = kk * y[3072]; }
    { const double kk = ws[54208]; ws[96544] = kk * y[4032]; ws[96576] = kk * y[4032]; }
    { const double kk = ws[54240]; ws[96608] = kk * y[4064]; ws[96640] = kk * y[4032]; }
    { const double kk = ws[54272]; ws[96672] = kk * y[4064]; ws[96704] = kk * y[4064]; }
    { const double kk = ws[54304]; ws[96736] = kk * y[5952]; ws[96768] = kk * y[5216]; }
    { const double kk = ws[54336]; ws[96800] = kk * y[4800]; ws[96832] = kk * y[5216]; }
    { const double kk = ws[54368]; ws[96864] = kk * y[5216]; ws[96896] = kk * y[5216]; }
    { const double kk = ws[54400]; ws[96928] = kk * y[4160]; ws[96960] = kk * y[3744]; }
    { const double kk = ws[54432]; ws[96992] = kk * y[4192]; ws[97024] = kk * y[3744]; }
    { const double kk = ws[54464]; ws[97056] = kk * y[4288]; ws[97088] = kk * y[3744]; }
    { const double kk = ws[54496]; ws[97120] = kk * y[4160]; ws[97152] = kk * y[3936]; }
    { const double kk = ws[54528]; ws[97184] = kk * y[4192]; ws[97216] = kk * y[3936]; }
    { const double kk = ws[54560]; ws[97248] = kk * y[4288]; ws[97280] = kk * y[3936]; }
    { const double kk = ws[54592]; ws[97312] = kk * y[4160]; ws[97344] = kk * y[3840]; }
    { const double kk = ws[54624]; ws[97376] = kk * y[4192]; ws[97408] = kk * y[3840]; }
    { const double kk = ws[54656]; ws[97440] = kk * y[4288]; ws[97472] = kk * y[3840]; }
    { const double kk = ws[54688]; ws[97504] = kk * y[4160]; ws[97536] = kk * y[3712]; }
    { const double kk = ws[54720]; ws[97568] = kk * y[4192]; ws[97600] = kk * y[3712]; }
    { const double kk = ws[54752]; ws[97632] = kk * y[4288]; ws[97664] = kk * y[3712]; }
    { const double kk = ws[54784]; ws[97696] = kk * y[6016]; ws[97728] = kk * y[1376]; }
    { const double kk = ws[54816]; ws[97760] = kk * y[6016]; ws[97792] = kk * y[384]; }
    { const double kk = ws[54848]; ws[97824] = kk * y[6016]; ws[97856] = kk * y[416]; }
    { const double kk = ws[54880]; ws[97888] = kk * y[6016]; ws[97920] = kk * y[3552]; }
    { const double kk = ws[54912]; ws[97952] = kk * y[5184]; ws[97984] = kk * y[3552]; }
    { const double kk = ws[54944]; ws[98016] = kk * y[5952]; ws[98048] = kk * y[3552]; }
    { const double kk = ws[55008]; ws[98080] = kk * y[6016]; ws[98112] = kk * y[1568]; }
    { const double kk = ws[55040]; ws[98144] = kk * y[5824]; ws[98176] = kk * y[3136]; }
    { const double kk = ws[55072]; ws[98208] = kk * y[5952]; ws[98240] = kk * y[3136]; }
    { const double kk = ws[55104]; ws[98272] = kk * y[5984]; ws[98304] = kk * y[3136]; }
    { const double kk = ws[55136]; ws[98336] = kk * y[5888]; ws[98368] = kk * y[3136]; }
    { const double kk = ws[55168]; ws[98400] = kk * y[5792]; ws[98432] = kk * y[3136]; }
    { const double kk = ws[55200]; ws[98464] = kk * y[5184]; ws[98496] = kk * y[1568]; }
    { const double kk = ws[55232]; ws[98528] = kk * y[5952]; ws[98560] = kk * y[1568]; }
    { const double kk = ws[55264]; ws[98592] = kk * y[6016]; ws[98624] = kk * y[3168]; }
    { const double kk = ws[55296]; ws[98656] = kk * y[5824]; ws[98688] = kk * y[1856]; }
    { const double kk = ws[55328]; ws[98720] = kk * y[5984]; ws[98752] = kk * y[1856]; }
    { const double kk = ws[55360]; ws[98784] = kk * y[6016]; ws[98816] = kk * y[4512]; }
    { const double kk = ws[55392]; ws[98848] = kk * y[5184]; ws[98880] = kk * y[3168]; }
    { const double kk = ws[55424]; ws[98912] = kk * y[5952]; ws[98944] = kk * y[3168]; }
    { const double kk = ws[55456]; ws[98976] = kk * y[6016]; ws[99008] = kk * y[448]; }
    { const double kk = ws[55488]; ws[99040] = kk * y[5952]; ws[99072] = kk * y[1600]; }
    { const double kk = ws[55520]; ws[99104] = kk * y[5984]; ws[99136] = kk * y[1920]; }
    { const double kk = ws[55552]; ws[99168] = kk * y[5824]; ws[99200] = kk * y[1920]; }
    { const double kk = ws[55584]; ws[99232] = kk * y[5952]; ws[99264] = kk * y[1920]; }
    { const double kk = ws[55616]; ws[99296] = kk * y[5184]; ws[99328] = kk * y[1600]; }
    { const double kk = ws[55648]; ws[99360] = kk * y[6016]; ws[99392] = kk * y[1600]; }
    { const double kk = ws[55680]; ws[99424] = kk * y[5984]; ws[99456] = kk * y[2304]; }
    { const double kk = ws[55712]; ws[99488] = kk * y[5952]; ws[99520] = kk * y[2304]; }
    { const double kk = ws[55744]; ws[99552] = kk * y[5824]; ws[99584] = kk * y[2304]; }
    { const double kk = ws[56064]; ws[99616] = kk * y[512]; ws[99648] = kk * y[1056]; }
    { const double kk = ws[56160]; ws[99680] = kk * y[6016]; ws[99712] = kk * y[608]; }
    { const double kk = ws[56192]; ws[99744] = kk * y[6016]; ws[99776] = kk * y[640]; }
    { const double kk = ws[56224]; ws[99808] = kk * y[6016]; ws[99840] = kk * y[672]; }
    { const double kk = ws[56256]; ws[99872] = kk * y[6016]; ws[99904] = kk * y[704]; }
    { const double kk = ws[56288]; ws[99936] = kk * y[6016]; ws[99968] = kk * y[736]; }
    { const double kk = ws[56320]; ws[100000] = kk * y[6016]; ws[100032] = kk * y[768]; }
    { const double kk = ws[56352]; ws[100064] = kk * y[6016]; ws[100096] = kk * y[800]; }
    { const double kk = ws[56384]; ws[100128] = kk * y[5824]; ws[100160] = kk * y[2368]; }
    { const double kk = ws[56416]; ws[100192] = kk * y[5824]; ws[100224] = kk * y[2400]; }
    { const double kk = ws[56448]; ws[100256] = kk * y[5824]; ws[100288] = kk * y[2432]; }
    { const double kk = ws[56480]; ws[100320] = kk * y[5824]; ws[100352] = kk * y[2464]; }
    { const double kk = ws[56512]; ws[100384] = kk * y[5824]; ws[100416] = kk * y[2496]; }
    { const double kk = ws[56544]; ws[100448] = kk * y[5824]; ws[100480] = kk * y[2528]; }
    { const double kk = ws[56576]; ws[100512] = kk * y[5824]; ws[100544] = kk * y[3904]; }
    { const double kk = ws[56608]; ws[100576] = kk * y[5952]; ws[100608] = kk * y[2368]; }
    { const double kk = ws[56640]; ws[100640] = kk * y[5952]; ws[100672] = kk * y[2400]; }
    { const double kk = ws[56672]; ws[100704] = kk * y[5952]; ws[100736] = kk * y[2432]; }
    { const double kk = ws[56704]; ws[100768] = kk * y[5952]; ws[100800] = kk * y[2464]; }
    { const double kk = ws[56736]; ws[100832] = kk * y[5952]; ws[100864] = kk * y[2496]; }
    { const double kk = ws[56768]; ws[100896] = kk * y[5952]; ws[100928] = kk * y[2528]; }
    { const double kk = ws[56800]; ws[100960] = kk * y[5952]; ws[100992] = kk * y[3904]; }
    { const double kk = ws[56832]; ws[101024] = kk * y[5984]; ws[101056] = kk * y[2368]; }
    { const double kk = ws[56864]; ws[101088] = kk * y[5984]; ws[101120] = kk * y[2400]; }
    { const double kk = ws[56896]; ws[101152] = kk * y[5984]; ws[101184] = kk * y[2432]; }
    { const double kk = ws[56928]; ws[101216] = kk * y[5984]; ws[101248] = kk * y[2464]; }
    { const double kk = ws[56960]; ws[101280] = kk * y[5984]; ws[101312] = kk * y[2496]; }
    { const double kk = ws[56992]; ws[101344] = kk * y[5984]; ws[101376] = kk * y[2528]; }
    { const double kk = ws[57024]; ws[101408] = kk * y[5984]; ws[101440] = kk * y[3904]; }
    { const double kk = ws[57280]; ws[101472] = kk * y[5824]; ws[101504] = kk * y[1952]; }
    { const double kk = ws[57312]; ws[101536] = kk * y[5824]; ws[101568] = kk * y[1984]; }
    { const double kk = ws[57344]; ws[101600] = kk * y[5824]; ws[101632] = kk * y[2016]; }
    { const double kk = ws[57376]; ws[101664] = kk * y[5824]; ws[101696] = kk * y[2048]; }
    { const double kk = ws[57408]; ws[101728] = kk * y[5824]; ws[101760] = kk * y[2080]; }
    { const double kk = ws[57440]; ws[101792] = kk * y[5824]; ws[101824] = kk * y[2112]; }
    { const double kk = ws[57472]; ws[101856] = kk * y[5824]; ws[101888] = kk * y[2144]; }
    { const double kk = ws[57504]; ws[101920] = kk * y[5952]; ws[101952] = kk * y[1952]; }
    { const double kk = ws[57536]; ws[101984] = kk * y[5952]; ws[102016] = kk * y[1984]; }
    { const double kk = ws[57568]; ws[102048] = kk * y[5952]; ws[102080] = kk * y[2016]; }
    { const double kk = ws[57600]; ws[102112] = kk * y[5952]; ws[102144] = kk * y[2048]; }
    { const double kk = ws[57632]; ws[102176] = kk * y[5952]; ws[102208] = kk * y[2080]; }
    { const double kk = ws[57664]; ws[102240] = kk * y[5952]; ws[102272] = kk * y[2112]; }
    { const double kk = ws[57696]; ws[102304] = kk * y[5952]; ws[102336] = kk * y[2144]; }
    { const double kk = ws[57728]; ws[102368] = kk * y[5984]; ws[102400] = kk * y[1952]; }
    { const double kk = ws[57760]; ws[102432] = kk * y[5984]; ws[102464] = kk * y[1984]; }
    { const double kk = ws[57792]; ws[102496] = kk * y[5984]; ws[102528] = kk * y[2016]; }
    { const double kk = ws[57824]; ws[102560] = kk * y[5984]; ws[102592] = kk * y[2048]; }
    { const double kk = ws[57856]; ws[102624] = kk * y[5984]; ws[102656] = kk * y[2080]; }
    { const double kk = ws[57888]; ws[102688] = kk * y[5984]; ws[102720] = kk * y[2112]; }
    { const double kk = ws[57920]; ws[102752] = kk * y[5984]; ws[102784] = kk * y[2144]; }
    { const double kk = ws[57952]; ws[102816] = kk * y[6016]; ws[102848] = kk * y[832]; }
    { const double kk = ws[57984]; ws[102880] = kk * y[5984]; ws[102912] = kk * y[3392]; }
    { const double kk = ws[58016]; ws[102944] = kk * y[5824]; ws[102976] = kk * y[3392]; }
    { const double kk = ws[58048]; ws[103008] = kk * y[5952]; ws[103040] = kk * y[3392]; }
    { const double kk = ws[58080]; ws[103072] = kk * y[5888]; ws[103104] = kk * y[3392]; }
    { const double kk = ws[58112]; ws[103136] = kk * y[5792]; ws[103168] = kk * y[3392]; }
    { const double kk = ws[58144]; ws[103200] = kk * y[6016]; ws[103232] = kk * y[864]; }
    { const double kk = ws[58176]; ws[103264] = kk * y[5984]; ws[103296] = kk * y[3424]; }
    { const double kk = ws[58208]; ws[103328] = kk * y[5824]; ws[103360] = kk * y[3424]; }
    { const double kk = ws[58240]; ws[103392] = kk * y[5952]; ws[103424] = kk * y[3424]; }
    { const double kk = ws[58272]; ws[103456] = kk * y[5888]; ws[103488] = kk * y[3424]; }
    { const double kk = ws[58304]; ws[103520] = kk * y[5792]; ws[103552] = kk * y[3424]; }
    { const double kk = ws[58336]; ws[103584] = kk * y[6016]; ws[103616] = kk * y[896]; }
    { const double kk = ws[58368]; ws[103648] = kk * y[5984]; ws[103680] = kk * y[3456]; }
    { const double kk = ws[58400]; ws[103712] = kk * y[5824]; ws[103744] = kk * y[3456]; }
    { const double kk = ws[58432]; ws[103776] = kk * y[5952]; ws[103808] = kk * y[3456]; }
    { const double kk = ws[58464]; ws[103840] = kk * y[5888]; ws[103872] = kk * y[3456]; }
    { const double kk = ws[58496]; ws[103904] = kk * y[5792]; ws[103936] = kk * y[3456]; }
    { const double kk = ws[58528]; ws[103968] = kk * y[6016]; ws[104000] = kk * y[4768]; }
    { const double kk = ws[58560]; ws[104032] = kk * y[6016]; ws[104064] = kk * y[4864]; }
    { const double kk = ws[58592]; ws[104096] = kk * y[6016]; ws[104128] = kk * y[4832]; }
    { const double kk = ws[58624]; ws[104160] = kk * y[6016]; ws[104192] = kk * y[4896]; }
    { const double kk = ws[58656]; ws[104224] = kk * y[6016]; ws[104256] = kk * y[4640]; }
    { const double kk = ws[58688]; ws[104288] = kk * y[6016]; ws[104320] = kk * y[4416]; }
    { const double kk = ws[58720]; ws[104352] = kk * y[6016]; ws[104384] = kk * y[4928]; }
    { const double kk = ws[58752]; ws[104416] = kk * y[6016]; ws[104448] = kk * y[4960]; }
    { const double kk = ws[58784]; ws[104480] = kk * y[6016]; ws[104512] = kk * y[4992]; }
    { const double kk = ws[58816]; ws[104544] = kk * y[6016]; ws[104576] = kk * y[4704]; }
    { const double kk = ws[58848]; ws[104608] = kk * y[6016]; ws[104640] = kk * y[5088]; }
    { const double kk = ws[58880]; ws[104672] = kk * y[6016]; ws[104704] = kk * y[5536]; }
    { const double kk = ws[58912]; ws[104736] = kk * y[6016]; ws[104768] = kk * y[5312]; }
    { const double kk = ws[58944]; ws[104800] = kk * y[6016]; ws[104832] = kk * y[4224]; }
    { const double kk = ws[58976]; ws[104864] = kk * y[6016]; ws[104896] = kk * y[3968]; }
    { const double kk = ws[59008]; ws[104928] = kk * y[6016]; ws[104960] = kk * y[4608]; }
    { const double kk = ws[59040]; ws[104992] = kk * y[6016]; ws[105024] = kk * y[928]; }
    { const double kk = ws[59136]; ws[105056] = kk * y[6016]; ws[105088] = kk * y[992]; }
    { const double kk = ws[59168]; ws[105120] = kk * y[5984]; ws[105152] = kk * y[3488]; }
    { const double kk = ws[59200]; ws[105184] = kk * y[5824]; ws[105216] = kk * y[3488]; }
    { const double kk = ws[59232]; ws[105248] = kk * y[5952]; ws[105280] = kk * y[3488]; }
    { const double kk = ws[59264]; ws[105312] = kk * y[5888]; ws[105344] = kk * y[3488]; }
    { const double kk = ws[59296]; ws[105376] = kk * y[5792]; ws[105408] = kk * y[3488]; }
}
// Partial-derivative products of 2- and 3-reactant reactions (grpderiv.F:163-189).
__device__ __noinline__ void gear_explic_0(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
#define CEFF_(v) ((v) <= 1.0e-30 ? 0.0 : (v))
    { const double kk = ws[43616]; ws[76320] = kk * CEFF_(y[6016]); ws[76352] = kk * CEFF_(y[5184]); }
    { const double kk = ws[43648]; ws[76384] = kk * CEFF_(y[5984]); ws[76416] = kk * CEFF_(y[5184]); }
    { const double kk = ws[43680]; ws[76448] = kk * CEFF_(y[5824]); ws[76480] = kk * CEFF_(y[5184]); }
    { const double kk = ws[43712]; ws[76512] = kk * CEFF_(y[5920]); ws[76544] = kk * CEFF_(y[5184]); }
    { const double kk = ws[43776]; ws[76576] = kk * CEFF_(y[5184]); ws[76608] = kk * CEFF_(y[2336]); }
    { const double kk = ws[43936]; ws[76640] = kk * CEFF_(y[5984]); ws[76672] = kk * CEFF_(y[6016]); }
    { const double kk = ws[43968]; ws[76704] = kk * CEFF_(y[5984]); ws[76736] = kk * CEFF_(y[5984]); }
    { const double kk = ws[44000]; ws[76768] = kk * CEFF_(y[5984]); ws[76800] = kk * CEFF_(y[5984]); }
    { const double kk = ws[44032]; ws[76832] = kk * CEFF_(y[6016]); ws[76864] = kk * CEFF_(y[4000]); }
    { const double kk = ws[44064]; ws[76896] = kk * CEFF_(y[2336]); ws[76928] = kk * CEFF_(y[5824]); }
    { const double kk = ws[44096]; ws[76960] = kk * CEFF_(y[6016]); ws[76992] = kk * CEFF_(y[5824]); }
    { const double kk = ws[44128]; ws[77024] = kk * CEFF_(y[5984]); ws[77056] = kk * CEFF_(y[5824]); }
    { const double kk = ws[44160]; ws[77088] = kk * CEFF_(y[5984]); ws[77120] = kk * CEFF_(y[5824]); }
    { const double kk = ws[44192]; ws[77152] = kk * CEFF_(y[5824]); ws[77184] = kk * CEFF_(y[5824]); }
    { const double kk = ws[44224]; ws[77216] = kk * CEFF_(y[6016]); ws[77248] = kk * CEFF_(y[1184]); }
    { const double kk = ws[44256]; ws[77280] = kk * CEFF_(y[2336]); ws[77312] = kk * CEFF_(y[5920]); }
    { const double kk = ws[44288]; ws[77344] = kk * CEFF_(y[2336]); ws[77376] = kk * CEFF_(y[5920]); }
    { const double kk = ws[44320]; ws[77408] = kk * CEFF_(y[6016]); ws[77440] = kk * CEFF_(y[5920]); }
    { const double kk = ws[44352]; ws[77472] = kk * CEFF_(y[6016]); ws[77504] = kk * CEFF_(y[5024]); }
    { const double kk = ws[44384]; ws[77536] = kk * CEFF_(y[6016]); ws[77568] = kk * CEFF_(y[5952]); }
    { const double kk = ws[44416]; ws[77600] = kk * CEFF_(y[5984]); ws[77632] = kk * CEFF_(y[5952]); }
    { const double kk = ws[44448]; ws[77664] = kk * CEFF_(y[5824]); ws[77696] = kk * CEFF_(y[5952]); }
    { const double kk = ws[44480]; ws[77728] = kk * CEFF_(y[5920]); ws[77760] = kk * CEFF_(y[5952]); }
    { const double kk = ws[44512]; ws[77792] = kk * CEFF_(y[5952]); ws[77824] = kk * CEFF_(y[5952]); }
    { const double kk = ws[44544]; ws[77856] = kk * CEFF_(y[5920]); ws[77888] = kk * CEFF_(y[5952]); }
    { const double kk = ws[44640]; ws[77920] = kk * CEFF_(y[5984]); ws[77952] = kk * CEFF_(y[5920]); }
    { const double kk = ws[44704]; ws[77984] = kk * CEFF_(y[6016]); ws[78016] = kk * CEFF_(y[1280]); }
    { const double kk = ws[44736]; ws[78048] = kk * CEFF_(y[6016]); ws[78080] = kk * CEFF_(y[160]); }
    { const double kk = ws[44768]; ws[78112] = kk * CEFF_(y[6016]); ws[78144] = kk * CEFF_(y[5664]); }
    { const double kk = ws[44832]; ws[78176] = kk * CEFF_(y[6016]); ws[78208] = kk * CEFF_(y[1888]); }
    { const double kk = ws[44864]; ws[78240] = kk * CEFF_(y[6016]); ws[78272] = kk * CEFF_(y[2176]); }
    { const double kk = ws[44896]; ws[78304] = kk * CEFF_(y[6016]); ws[78336] = kk * CEFF_(y[1120]); }
    { const double kk = ws[44928]; ws[78368] = kk * CEFF_(y[6016]); ws[78400] = kk * CEFF_(y[2240]); }
    { const double kk = ws[44960]; ws[78432] = kk * CEFF_(y[6016]); ws[78464] = kk * CEFF_(y[2752]); }
    { const double kk = ws[44992]; ws[78496] = kk * CEFF_(y[6016]); ws[78528] = kk * CEFF_(y[1152]); }
    { const double kk = ws[45024]; ws[78560] = kk * CEFF_(y[6016]); ws[78592] = kk * CEFF_(y[256]); }
    { const double kk = ws[45056]; ws[78624] = kk * CEFF_(y[6016]); ws[78656] = kk * CEFF_(y[1216]); }
    { const double kk = ws[45088]; ws[78688] = kk * CEFF_(y[6016]); ws[78720] = kk * CEFF_(y[288]); }
    { const double kk = ws[45120]; ws[78752] = kk * CEFF_(y[6016]); ws[78784] = kk * CEFF_(y[320]); }
    { const double kk = ws[45152]; ws[78816] = kk * CEFF_(y[6016]); ws[78848] = kk * CEFF_(y[352]); }
    { const double kk = ws[45184]; ws[78880] = kk * CEFF_(y[5184]); ws[78912] = kk * CEFF_(y[1312]); }
    { const double kk = ws[45216]; ws[78944] = kk * CEFF_(y[5952]); ws[78976] = kk * CEFF_(y[1312]); }
    { const double kk = ws[45248]; ws[79008] = kk * CEFF_(y[6016]); ws[79040] = kk * CEFF_(y[1312]); }
    { const double kk = ws[45280]; ws[79072] = kk * CEFF_(y[5984]); ws[79104] = kk * CEFF_(y[4288]); }
    { const double kk = ws[45312]; ws[79136] = kk * CEFF_(y[5824]); ws[79168] = kk * CEFF_(y[4288]); }
    { const double kk = ws[45344]; ws[79200] = kk * CEFF_(y[6016]); ws[79232] = kk * CEFF_(y[1344]); }
    { const double kk = ws[45376]; ws[79264] = kk * CEFF_(y[6016]); ws[79296] = kk * CEFF_(y[1344]); }
    { const double kk = ws[45408]; ws[79328] = kk * CEFF_(y[5984]); ws[79360] = kk * CEFF_(y[1632]); }
    { const double kk = ws[45440]; ws[79392] = kk * CEFF_(y[5824]); ws[79424] = kk * CEFF_(y[1632]); }
    { const double kk = ws[45472]; ws[79456] = kk * CEFF_(y[6016]); ws[79488] = kk * CEFF_(y[2784]); }
    { const double kk = ws[45504]; ws[79520] = kk * CEFF_(y[2208]); ws[79552] = kk * CEFF_(y[6016]); }
    { const double kk = ws[45568]; ws[79584] = kk * CEFF_(y[6016]); ws[79616] = kk * CEFF_(y[1664]); }
    { const double kk = ws[45600]; ws[79648] = kk * CEFF_(y[6016]); ws[79680] = kk * CEFF_(y[1408]); }
    { const double kk = ws[45632]; ws[79712] = kk * CEFF_(y[6016]); ws[79744] = kk * CEFF_(y[1440]); }
    { const double kk = ws[45664]; ws[79776] = kk * CEFF_(y[6016]); ws[79808] = kk * CEFF_(y[4544]); }
    { const double kk = ws[45696]; ws[79840] = kk * CEFF_(y[6016]); ws[79872] = kk * CEFF_(y[4576]); }
    { const double kk = ws[45728]; ws[79904] = kk * CEFF_(y[6016]); ws[79936] = kk * CEFF_(y[5856]); }
    { const double kk = ws[45760]; ws[79968] = kk * CEFF_(y[6016]); ws[80000] = kk * CEFF_(y[5568]); }
    { const double kk = ws[45792]; ws[80032] = kk * CEFF_(y[6016]); ws[80064] = kk * CEFF_(y[5760]); }
    { const double kk = ws[45824]; ws[80096] = kk * CEFF_(y[6016]); ws[80128] = kk * CEFF_(y[4480]); }
    { const double kk = ws[45856]; ws[80160] = kk * CEFF_(y[6016]); ws[80192] = kk * CEFF_(y[5280]); }
    { const double kk = ws[45888]; ws[80224] = kk * CEFF_(y[6016]); ws[80256] = kk * CEFF_(y[5504]); }
    { const double kk = ws[45920]; ws[80288] = kk * CEFF_(y[6016]); ws[80320] = kk * CEFF_(y[5344]); }
    { const double kk = ws[45952]; ws[80352] = kk * CEFF_(y[6016]); ws[80384] = kk * CEFF_(y[4128]); }
    { const double kk = ws[45984]; ws[80416] = kk * CEFF_(y[6016]); ws[80448] = kk * CEFF_(y[4736]); }
    { const double kk = ws[46016]; ws[80480] = kk * CEFF_(y[6016]); ws[80512] = kk * CEFF_(y[3872]); }
    { const double kk = ws[46048]; ws[80544] = kk * CEFF_(y[6016]); ws[80576] = kk * CEFF_(y[5376]); }
    { const double kk = ws[46080]; ws[80608] = kk * CEFF_(y[6016]); ws[80640] = kk * CEFF_(y[5248]); }
    { const double kk = ws[46112]; ws[80672] = kk * CEFF_(y[6016]); ws[80704] = kk * CEFF_(y[5472]); }
    { const double kk = ws[46144]; ws[80736] = kk * CEFF_(y[6016]); ws[80768] = kk * CEFF_(y[4320]); }
    { const double kk = ws[46176]; ws[80800] = kk * CEFF_(y[6016]); ws[80832] = kk * CEFF_(y[3584]); }
    { const double kk = ws[46208]; ws[80864] = kk * CEFF_(y[6016]); ws[80896] = kk * CEFF_(y[4448]); }
    { const double kk = ws[46240]; ws[80928] = kk * CEFF_(y[6016]); ws[80960] = kk * CEFF_(y[1248]); }
    { const double kk = ws[46272]; ws[80992] = kk * CEFF_(y[6016]); ws[81024] = kk * CEFF_(y[2944]); }
    { const double kk = ws[46304]; ws[81056] = kk * CEFF_(y[6016]); ws[81088] = kk * CEFF_(y[1760]); }
    { const double kk = ws[46336]; ws[81120] = kk * CEFF_(y[6016]); ws[81152] = kk * CEFF_(y[5600]); }
    { const double kk = ws[46368]; ws[81184] = kk * CEFF_(y[6016]); ws[81216] = kk * CEFF_(y[1472]); }
    { const double kk = ws[46400]; ws[81248] = kk * CEFF_(y[6016]); ws[81280] = kk * CEFF_(y[5056]); }
    { const double kk = ws[46432]; ws[81312] = kk * CEFF_(y[6016]); ws[81344] = kk * CEFF_(y[1504]); }
    { const double kk = ws[46464]; ws[81376] = kk * CEFF_(y[6016]); ws[81408] = kk * CEFF_(y[2816]); }
    { const double kk = ws[46496]; ws[81440] = kk * CEFF_(y[6016]); ws[81472] = kk * CEFF_(y[5728]); }
    { const double kk = ws[46528]; ws[81504] = kk * CEFF_(y[6016]); ws[81536] = kk * CEFF_(y[4096]); }
    { const double kk = ws[46560]; ws[81568] = kk * CEFF_(y[6016]); ws[81600] = kk * CEFF_(y[4608]); }
    { const double kk = ws[46592]; ws[81632] = kk * CEFF_(y[6016]); ws[81664] = kk * CEFF_(y[1792]); }
    { const double kk = ws[46624]; ws[81696] = kk * CEFF_(y[6016]); ws[81728] = kk * CEFF_(y[4352]); }
    { const double kk = ws[46656]; ws[81760] = kk * CEFF_(y[6016]); ws[81792] = kk * CEFF_(y[5696]); }
    { const double kk = ws[46688]; ws[81824] = kk * CEFF_(y[6016]); ws[81856] = kk * CEFF_(y[3680]); }
    { const double kk = ws[46720]; ws[81888] = kk * CEFF_(y[6016]); ws[81920] = kk * CEFF_(y[1088]); }
    { const double kk = ws[46752]; ws[81952] = kk * CEFF_(y[6016]); ws[81984] = kk * CEFF_(y[1536]); }
    { const double kk = ws[46784]; ws[82016] = kk * CEFF_(y[6016]); ws[82048] = kk * CEFF_(y[1824]); }
    { const double kk = ws[46816]; ws[82080] = kk * CEFF_(y[6016]); ws[82112] = kk * CEFF_(y[5440]); }
    { const double kk = ws[46848]; ws[82144] = kk * CEFF_(y[6016]); ws[82176] = kk * CEFF_(y[4384]); }
    { const double kk = ws[46880]; ws[82208] = kk * CEFF_(y[6016]); ws[82240] = kk * CEFF_(y[1696]); }
    { const double kk = ws[46912]; ws[82272] = kk * CEFF_(y[5184]); ws[82304] = kk * CEFF_(y[2240]); }
    { const double kk = ws[46944]; ws[82336] = kk * CEFF_(y[5184]); ws[82368] = kk * CEFF_(y[2752]); }
    { const double kk = ws[46976]; ws[82400] = kk * CEFF_(y[5184]); ws[82432] = kk * CEFF_(y[1152]); }
    { const double kk = ws[47008]; ws[82464] = kk * CEFF_(y[5184]); ws[82496] = kk * CEFF_(y[1408]); }
    { const double kk = ws[47040]; ws[82528] = kk * CEFF_(y[5184]); ws[82560] = kk * CEFF_(y[1440]); }
    { const double kk = ws[47072]; ws[82592] = kk * CEFF_(y[5184]); ws[82624] = kk * CEFF_(y[4576]); }
    { const double kk = ws[47104]; ws[82656] = kk * CEFF_(y[5184]); ws[82688] = kk * CEFF_(y[4384]); }
    { const double kk = ws[47136]; ws[82720] = kk * CEFF_(y[5184]); ws[82752] = kk * CEFF_(y[4128]); }
    { const double kk = ws[47168]; ws[82784] = kk * CEFF_(y[5184]); ws[82816] = kk * CEFF_(y[4736]); }
    { const double kk = ws[47200]; ws[82848] = kk * CEFF_(y[5184]); ws[82880] = kk * CEFF_(y[3872]); }
    { const double kk = ws[47232]; ws[82912] = kk * CEFF_(y[5184]); ws[82944] = kk * CEFF_(y[5472]); }
    { const double kk = ws[47264]; ws[82976] = kk * CEFF_(y[5184]); ws[83008] = kk * CEFF_(y[4320]); }
    { const double kk = ws[47296]; ws[83040] = kk * CEFF_(y[5184]); ws[83072] = kk * CEFF_(y[3584]); }
    { const double kk = ws[47328]; ws[83104] = kk * CEFF_(y[5184]); ws[83136] = kk * CEFF_(y[3808]); }
    { const double kk = ws[47360]; ws[83168] = kk * CEFF_(y[5952]); ws[83200] = kk * CEFF_(y[2240]); }
    { const double kk = ws[47392]; ws[83232] = kk * CEFF_(y[5952]); ws[83264] = kk * CEFF_(y[2752]); }
    { const double kk = ws[47424]; ws[83296] = kk * CEFF_(y[5952]); ws[83328] = kk * CEFF_(y[1152]); }
    { const double kk = ws[47456]; ws[83360] = kk * CEFF_(y[5952]); ws[83392] = kk * CEFF_(y[1408]); }
    { const double kk = ws[47488]; ws[83424] = kk * CEFF_(y[5952]); ws[83456] = kk * CEFF_(y[1440]); }
    { const double kk = ws[47520]; ws[83488] = kk * CEFF_(y[5952]); ws[83520] = kk * CEFF_(y[4384]); }
    { const double kk = ws[47552]; ws[83552] = kk * CEFF_(y[5952]); ws[83584] = kk * CEFF_(y[5856]); }
    { const double kk = ws[47584]; ws[83616] = kk * CEFF_(y[5952]); ws[83648] = kk * CEFF_(y[5568]); }
    { const double kk = ws[47616]; ws[83680] = kk * CEFF_(y[5952]); ws[83712] = kk * CEFF_(y[5760]); }
    { const double kk = ws[47648]; ws[83744] = kk * CEFF_(y[5952]); ws[83776] = kk * CEFF_(y[4128]); }
    { const double kk = ws[47680]; ws[83808] = kk * CEFF_(y[5952]); ws[83840] = kk * CEFF_(y[3872]); }
    { const double kk = ws[47712]; ws[83872] = kk * CEFF_(y[5952]); ws[83904] = kk * CEFF_(y[5376]); }
    { const double kk = ws[47744]; ws[83936] = kk * CEFF_(y[5952]); ws[83968] = kk * CEFF_(y[5248]); }
    { const double kk = ws[47776]; ws[84000] = kk * CEFF_(y[5952]); ws[84032] = kk * CEFF_(y[1248]); }
    { const double kk = ws[47808]; ws[84064] = kk * CEFF_(y[5952]); ws[84096] = kk * CEFF_(y[2944]); }
    { const double kk = ws[47840]; ws[84128] = kk * CEFF_(y[5952]); ws[84160] = kk * CEFF_(y[1760]); }
    { const double kk = ws[47872]; ws[84192] = kk * CEFF_(y[5952]); ws[84224] = kk * CEFF_(y[1824]); }
    { const double kk = ws[47968]; ws[84256] = kk * CEFF_(y[5920]); ws[84288] = kk * CEFF_(y[5792]); }
    { const double kk = ws[48032]; ws[84320] = kk * CEFF_(y[5920]); ws[84352] = kk * CEFF_(y[4800]); }
    { const double kk = ws[48096]; ws[84384] = kk * CEFF_(y[5920]); ws[84416] = kk * CEFF_(y[4672]); }
    { const double kk = ws[48160]; ws[84448] = kk * CEFF_(y[5824]); ws[84480] = kk * CEFF_(y[5888]); }
    { const double kk = ws[48192]; ws[84512] = kk * CEFF_(y[5824]); ws[84544] = kk * CEFF_(y[5632]); }
    { const double kk = ws[48224]; ws[84576] = kk * CEFF_(y[5824]); ws[84608] = kk * CEFF_(y[5408]); }
    { const double kk = ws[48256]; ws[84640] = kk * CEFF_(y[5824]); ws[84672] = kk * CEFF_(y[5120]); }
    { const double kk = ws[48288]; ws[84704] = kk * CEFF_(y[5824]); ws[84736] = kk * CEFF_(y[3008]); }
    { const double kk = ws[48320]; ws[84768] = kk * CEFF_(y[5824]); ws[84800] = kk * CEFF_(y[3200]); }
    { const double kk = ws[48352]; ws[84832] = kk * CEFF_(y[5824]); ws[84864] = kk * CEFF_(y[3328]); }
    { const double kk = ws[48384]; ws[84896] = kk * CEFF_(y[5824]); ws[84928] = kk * CEFF_(y[3360]); }
    { const double kk = ws[48416]; ws[84960] = kk * CEFF_(y[5824]); ws[84992] = kk * CEFF_(y[3296]); }
    { const double kk = ws[48448]; ws[85024] = kk * CEFF_(y[5824]); ws[85056] = kk * CEFF_(y[3104]); }
    { const double kk = ws[48480]; ws[85088] = kk * CEFF_(y[5824]); ws[85120] = kk * CEFF_(y[3264]); }
    { const double kk = ws[48512]; ws[85152] = kk * CEFF_(y[5824]); ws[85184] = kk * CEFF_(y[4160]); }
    { const double kk = ws[48544]; ws[85216] = kk * CEFF_(y[5824]); ws[85248] = kk * CEFF_(y[3744]); }
    { const double kk = ws[48576]; ws[85280] = kk * CEFF_(y[5824]); ws[85312] = kk * CEFF_(y[2624]); }
    { const double kk = ws[48608]; ws[85344] = kk * CEFF_(y[5824]); ws[85376] = kk * CEFF_(y[3840]); }
    { const double kk = ws[48640]; ws[85408] = kk * CEFF_(y[5824]); ws[85440] = kk * CEFF_(y[4192]); }
    { const double kk = ws[48672]; ws[85472] = kk * CEFF_(y[5824]); ws[85504] = kk * CEFF_(y[3936]); }
    { const double kk = ws[48704]; ws[85536] = kk * CEFF_(y[5824]); ws[85568] = kk * CEFF_(y[2656]); }
    { const double kk = ws[48736]; ws[85600] = kk * CEFF_(y[5824]); ws[85632] = kk * CEFF_(y[3712]); }
    { const double kk = ws[48768]; ws[85664] = kk * CEFF_(y[5824]); ws[85696] = kk * CEFF_(y[2560]); }
    { const double kk = ws[48800]; ws[85728] = kk * CEFF_(y[5824]); ws[85760] = kk * CEFF_(y[1728]); }
    { const double kk = ws[48832]; ws[85792] = kk * CEFF_(y[5824]); ws[85824] = kk * CEFF_(y[5792]); }
    { const double kk = ws[48864]; ws[85856] = kk * CEFF_(y[5824]); ws[85888] = kk * CEFF_(y[4800]); }
    { const double kk = ws[48896]; ws[85920] = kk * CEFF_(y[5824]); ws[85952] = kk * CEFF_(y[2848]); }
    { const double kk = ws[48928]; ws[85984] = kk * CEFF_(y[5824]); ws[86016] = kk * CEFF_(y[5152]); }
    { const double kk = ws[48960]; ws[86048] = kk * CEFF_(y[5824]); ws[86080] = kk * CEFF_(y[3776]); }
    { const double kk = ws[48992]; ws[86112] = kk * CEFF_(y[5824]); ws[86144] = kk * CEFF_(y[4672]); }
    { const double kk = ws[49024]; ws[86176] = kk * CEFF_(y[5824]); ws[86208] = kk * CEFF_(y[3520]); }
    { const double kk = ws[49056]; ws[86240] = kk * CEFF_(y[5824]); ws[86272] = kk * CEFF_(y[2880]); }
    { const double kk = ws[49088]; ws[86304] = kk * CEFF_(y[5824]); ws[86336] = kk * CEFF_(y[2912]); }
    { const double kk = ws[49120]; ws[86368] = kk * CEFF_(y[5824]); ws[86400] = kk * CEFF_(y[2592]); }
    { const double kk = ws[49152]; ws[86432] = kk * CEFF_(y[5824]); ws[86464] = kk * CEFF_(y[2272]); }
    { const double kk = ws[49184]; ws[86496] = kk * CEFF_(y[5824]); ws[86528] = kk * CEFF_(y[3648]); }
    { const double kk = ws[49216]; ws[86560] = kk * CEFF_(y[5824]); ws[86592] = kk * CEFF_(y[3040]); }
    { const double kk = ws[49248]; ws[86624] = kk * CEFF_(y[5824]); ws[86656] = kk * CEFF_(y[2976]); }
    { const double kk = ws[49280]; ws[86688] = kk * CEFF_(y[5824]); ws[86720] = kk * CEFF_(y[4032]); }
    { const double kk = ws[49312]; ws[86752] = kk * CEFF_(y[5824]); ws[86784] = kk * CEFF_(y[4064]); }
    { const double kk = ws[49344]; ws[86816] = kk * CEFF_(y[5824]); ws[86848] = kk * CEFF_(y[3072]); }
    { const double kk = ws[49376]; ws[86880] = kk * CEFF_(y[5824]); ws[86912] = kk * CEFF_(y[5216]); }
    { const double kk = ws[49408]; ws[86944] = kk * CEFF_(y[5920]); ws[86976] = kk * CEFF_(y[2688]); }
    { const double kk = ws[49440]; ws[87008] = kk * CEFF_(y[5920]); ws[87040] = kk * CEFF_(y[3232]); }
    { const double kk = ws[49472]; ws[87072] = kk * CEFF_(y[5920]); ws[87104] = kk * CEFF_(y[3808]); }
    { const double kk = ws[49504]; ws[87136] = kk * CEFF_(y[5984]); ws[87168] = kk * CEFF_(y[5888]); }
    { const double kk = ws[49536]; ws[87200] = kk * CEFF_(y[5984]); ws[87232] = kk * CEFF_(y[5632]); }
    { const double kk = ws[49568]; ws[87264] = kk * CEFF_(y[5984]); ws[87296] = kk * CEFF_(y[5408]); }
    { const double kk = ws[49600]; ws[87328] = kk * CEFF_(y[5984]); ws[87360] = kk * CEFF_(y[5120]); }
    { const double kk = ws[49632]; ws[87392] = kk * CEFF_(y[5984]); ws[87424] = kk * CEFF_(y[3008]); }
    { const double kk = ws[49664]; ws[87456] = kk * CEFF_(y[5984]); ws[87488] = kk * CEFF_(y[3200]); }
    { const double kk = ws[49696]; ws[87520] = kk * CEFF_(y[5984]); ws[87552] = kk * CEFF_(y[3328]); }
    { const double kk = ws[49728]; ws[87584] = kk * CEFF_(y[5984]); ws[87616] = kk * CEFF_(y[3360]); }
    { const double kk = ws[49760]; ws[87648] = kk * CEFF_(y[5984]); ws[87680] = kk * CEFF_(y[3296]); }
    { const double kk = ws[49792]; ws[87712] = kk * CEFF_(y[5984]); ws[87744] = kk * CEFF_(y[3104]); }
    { const double kk = ws[49824]; ws[87776] = kk * CEFF_(y[5984]); ws[87808] = kk * CEFF_(y[3264]); }
    { const double kk = ws[49856]; ws[87840] = kk * CEFF_(y[5984]); ws[87872] = kk * CEFF_(y[4160]); }
    { const double kk = ws[49888]; ws[87904] = kk * CEFF_(y[5984]); ws[87936] = kk * CEFF_(y[3744]); }
    { const double kk = ws[49920]; ws[87968] = kk * CEFF_(y[5984]); ws[88000] = kk * CEFF_(y[2624]); }
    { const double kk = ws[49952]; ws[88032] = kk * CEFF_(y[5984]); ws[88064] = kk * CEFF_(y[3840]); }
    { const double kk = ws[49984]; ws[88096] = kk * CEFF_(y[5984]); ws[88128] = kk * CEFF_(y[4192]); }
    { const double kk = ws[50016]; ws[88160] = kk * CEFF_(y[5984]); ws[88192] = kk * CEFF_(y[3936]); }
    { const double kk = ws[50048]; ws[88224] = kk * CEFF_(y[5984]); ws[88256] = kk * CEFF_(y[2656]); }
    { const double kk = ws[50080]; ws[88288] = kk * CEFF_(y[5984]); ws[88320] = kk * CEFF_(y[3712]); }
    { const double kk = ws[50112]; ws[88352] = kk * CEFF_(y[5984]); ws[88384] = kk * CEFF_(y[2560]); }
    { const double kk = ws[50144]; ws[88416] = kk * CEFF_(y[5984]); ws[88448] = kk * CEFF_(y[1728]); }
    { const double kk = ws[50176]; ws[88480] = kk * CEFF_(y[5984]); ws[88512] = kk * CEFF_(y[5792]); }
    { const double kk = ws[50208]; ws[88544] = kk * CEFF_(y[5984]); ws[88576] = kk * CEFF_(y[4800]); }
    { const double kk = ws[50240]; ws[88608] = kk * CEFF_(y[5984]); ws[88640] = kk * CEFF_(y[2848]); }
    { const double kk = ws[50272]; ws[88672] = kk * CEFF_(y[5984]); ws[88704] = kk * CEFF_(y[5152]); }
    { const double kk = ws[50304]; ws[88736] = kk * CEFF_(y[5984]); ws[88768] = kk * CEFF_(y[3776]); }
    { const double kk = ws[50336]; ws[88800] = kk * CEFF_(y[5984]); ws[88832] = kk * CEFF_(y[4672]); }
    { const double kk = ws[50368]; ws[88864] = kk * CEFF_(y[5984]); ws[88896] = kk * CEFF_(y[3520]); }
    { const double kk = ws[50400]; ws[88928] = kk * CEFF_(y[5984]); ws[88960] = kk * CEFF_(y[2880]); }
    { const double kk = ws[50432]; ws[88992] = kk * CEFF_(y[5984]); ws[89024] = kk * CEFF_(y[2912]); }
    { const double kk = ws[50464]; ws[89056] = kk * CEFF_(y[5984]); ws[89088] = kk * CEFF_(y[3648]); }
    { const double kk = ws[50496]; ws[89120] = kk * CEFF_(y[5984]); ws[89152] = kk * CEFF_(y[3232]); }
    { const double kk = ws[50528]; ws[89184] = kk * CEFF_(y[5984]); ws[89216] = kk * CEFF_(y[3040]); }
    { const double kk = ws[50560]; ws[89248] = kk * CEFF_(y[5984]); ws[89280] = kk * CEFF_(y[2976]); }
    { const double kk = ws[50592]; ws[89312] = kk * CEFF_(y[5984]); ws[89344] = kk * CEFF_(y[4032]); }
    { const double kk = ws[50624]; ws[89376] = kk * CEFF_(y[5984]); ws[89408] = kk * CEFF_(y[4064]); }
    { const double kk = ws[50656]; ws[89440] = kk * CEFF_(y[5984]); ws[89472] = kk * CEFF_(y[3072]); }
    { const double kk = ws[50688]; ws[89504] = kk * CEFF_(y[5984]); ws[89536] = kk * CEFF_(y[5216]); }
    { const double kk = ws[50720]; ws[89568] = kk * CEFF_(y[5888]); ws[89600] = kk * CEFF_(y[5888]); }
    { const double kk = ws[50752]; ws[89632] = kk * CEFF_(y[5888]); ws[89664] = kk * CEFF_(y[5632]); }
    { const double kk = ws[50784]; ws[89696] = kk * CEFF_(y[5888]); ws[89728] = kk * CEFF_(y[5408]); }
    { const double kk = ws[50816]; ws[89760] = kk * CEFF_(y[5888]); ws[89792] = kk * CEFF_(y[5120]); }
    { const double kk = ws[50848]; ws[89824] = kk * CEFF_(y[5888]); ws[89856] = kk * CEFF_(y[3008]); }
    { const double kk = ws[50880]; ws[89888] = kk * CEFF_(y[5888]); ws[89920] = kk * CEFF_(y[3200]); }
    { const double kk = ws[50912]; ws[89952] = kk * CEFF_(y[5888]); ws[89984] = kk * CEFF_(y[3328]); }
    { const double kk = ws[50944]; ws[90016] = kk * CEFF_(y[5888]); ws[90048] = kk * CEFF_(y[3360]); }
    { const double kk = ws[50976]; ws[90080] = kk * CEFF_(y[5888]); ws[90112] = kk * CEFF_(y[3296]); }
    { const double kk = ws[51008]; ws[90144] = kk * CEFF_(y[5888]); ws[90176] = kk * CEFF_(y[3104]); }
    { const double kk = ws[51040]; ws[90208] = kk * CEFF_(y[5888]); ws[90240] = kk * CEFF_(y[3264]); }
    { const double kk = ws[51072]; ws[90272] = kk * CEFF_(y[5888]); ws[90304] = kk * CEFF_(y[4288]); }
    { const double kk = ws[51104]; ws[90336] = kk * CEFF_(y[5888]); ws[90368] = kk * CEFF_(y[4160]); }
    { const double kk = ws[51136]; ws[90400] = kk * CEFF_(y[5888]); ws[90432] = kk * CEFF_(y[3744]); }
    { const double kk = ws[51168]; ws[90464] = kk * CEFF_(y[5888]); ws[90496] = kk * CEFF_(y[2624]); }
    { const double kk = ws[51200]; ws[90528] = kk * CEFF_(y[5888]); ws[90560] = kk * CEFF_(y[3840]); }
    { const double kk = ws[51232]; ws[90592] = kk * CEFF_(y[5888]); ws[90624] = kk * CEFF_(y[4192]); }
    { const double kk = ws[51264]; ws[90656] = kk * CEFF_(y[5888]); ws[90688] = kk * CEFF_(y[3936]); }
    { const double kk = ws[51296]; ws[90720] = kk * CEFF_(y[5888]); ws[90752] = kk * CEFF_(y[2656]); }
    { const double kk = ws[51328]; ws[90784] = kk * CEFF_(y[5888]); ws[90816] = kk * CEFF_(y[3712]); }
    { const double kk = ws[51360]; ws[90848] = kk * CEFF_(y[5888]); ws[90880] = kk * CEFF_(y[5792]); }
    { const double kk = ws[51392]; ws[90912] = kk * CEFF_(y[5888]); ws[90944] = kk * CEFF_(y[4800]); }
    { const double kk = ws[51424]; ws[90976] = kk * CEFF_(y[5888]); ws[91008] = kk * CEFF_(y[2848]); }
    { const double kk = ws[51456]; ws[91040] = kk * CEFF_(y[5888]); ws[91072] = kk * CEFF_(y[5152]); }
    { const double kk = ws[51488]; ws[91104] = kk * CEFF_(y[5888]); ws[91136] = kk * CEFF_(y[3776]); }
    { const double kk = ws[51520]; ws[91168] = kk * CEFF_(y[5888]); ws[91200] = kk * CEFF_(y[4672]); }
    { const double kk = ws[51552]; ws[91232] = kk * CEFF_(y[5888]); ws[91264] = kk * CEFF_(y[3520]); }
    { const double kk = ws[51584]; ws[91296] = kk * CEFF_(y[5888]); ws[91328] = kk * CEFF_(y[2880]); }
    { const double kk = ws[51616]; ws[91360] = kk * CEFF_(y[5888]); ws[91392] = kk * CEFF_(y[2912]); }
    { const double kk = ws[51648]; ws[91424] = kk * CEFF_(y[5888]); ws[91456] = kk * CEFF_(y[2592]); }
    { const double kk = ws[51680]; ws[91488] = kk * CEFF_(y[5888]); ws[91520] = kk * CEFF_(y[2272]); }
    { const double kk = ws[51712]; ws[91552] = kk * CEFF_(y[5888]); ws[91584] = kk * CEFF_(y[3648]); }
    { const double kk = ws[51744]; ws[91616] = kk * CEFF_(y[5888]); ws[91648] = kk * CEFF_(y[3040]); }
    { const double kk = ws[51776]; ws[91680] = kk * CEFF_(y[5888]); ws[91712] = kk * CEFF_(y[2976]); }
    { const double kk = ws[51808]; ws[91744] = kk * CEFF_(y[5888]); ws[91776] = kk * CEFF_(y[4032]); }
    { const double kk = ws[51840]; ws[91808] = kk * CEFF_(y[5888]); ws[91840] = kk * CEFF_(y[4064]); }
    { const double kk = ws[51872]; ws[91872] = kk * CEFF_(y[5888]); ws[91904] = kk * CEFF_(y[3072]); }
    { const double kk = ws[51904]; ws[91936] = kk * CEFF_(y[5888]); ws[91968] = kk * CEFF_(y[5216]); }
    { const double kk = ws[51936]; ws[92000] = kk * CEFF_(y[5792]); ws[92032] = kk * CEFF_(y[5632]); }
    { const double kk = ws[51968]; ws[92064] = kk * CEFF_(y[5792]); ws[92096] = kk * CEFF_(y[5408]); }
    { const double kk = ws[52000]; ws[92128] = kk * CEFF_(y[5792]); ws[92160] = kk * CEFF_(y[5120]); }
    { const double kk = ws[52032]; ws[92192] = kk * CEFF_(y[5792]); ws[92224] = kk * CEFF_(y[3008]); }
    { const double kk = ws[52064]; ws[92256] = kk * CEFF_(y[5792]); ws[92288] = kk * CEFF_(y[3200]); }
    { const double kk = ws[52096]; ws[92320] = kk * CEFF_(y[5792]); ws[92352] = kk * CEFF_(y[3328]); }
    { const double kk = ws[52128]; ws[92384] = kk * CEFF_(y[5792]); ws[92416] = kk * CEFF_(y[3360]); }
    { const double kk = ws[52160]; ws[92448] = kk * CEFF_(y[5792]); ws[92480] = kk * CEFF_(y[3296]); }
    { const double kk = ws[52192]; ws[92512] = kk * CEFF_(y[5792]); ws[92544] = kk * CEFF_(y[3104]); }
    { const double kk = ws[52224]; ws[92576] = kk * CEFF_(y[5792]); ws[92608] = kk * CEFF_(y[3264]); }
    { const double kk = ws[52256]; ws[92640] = kk * CEFF_(y[5792]); ws[92672] = kk * CEFF_(y[4288]); }
    { const double kk = ws[52288]; ws[92704] = kk * CEFF_(y[5792]); ws[92736] = kk * CEFF_(y[4160]); }
    { const double kk = ws[52320]; ws[92768] = kk * CEFF_(y[5792]); ws[92800] = kk * CEFF_(y[3744]); }
    { const double kk = ws[52352]; ws[92832] = kk * CEFF_(y[5792]); ws[92864] = kk * CEFF_(y[2624]); }
    { const double kk = ws[52384]; ws[92896] = kk * CEFF_(y[5792]); ws[92928] = kk * CEFF_(y[3840]); }
    { const double kk = ws[52416]; ws[92960] = kk * CEFF_(y[5792]); ws[92992] = kk * CEFF_(y[4192]); }
    { const double kk = ws[52448]; ws[93024] = kk * CEFF_(y[5792]); ws[93056] = kk * CEFF_(y[3936]); }
    { const double kk = ws[52480]; ws[93088] = kk * CEFF_(y[5792]); ws[93120] = kk * CEFF_(y[2656]); }
    { const double kk = ws[52512]; ws[93152] = kk * CEFF_(y[5792]); ws[93184] = kk * CEFF_(y[3712]); }
    { const double kk = ws[52544]; ws[93216] = kk * CEFF_(y[5792]); ws[93248] = kk * CEFF_(y[5792]); }
    { const double kk = ws[52576]; ws[93280] = kk * CEFF_(y[5792]); ws[93312] = kk * CEFF_(y[4800]); }
    { const double kk = ws[52608]; ws[93344] = kk * CEFF_(y[5792]); ws[93376] = kk * CEFF_(y[2848]); }
    { const double kk = ws[52640]; ws[93408] = kk * CEFF_(y[5792]); ws[93440] = kk * CEFF_(y[5152]); }
    { const double kk = ws[52672]; ws[93472] = kk * CEFF_(y[5792]); ws[93504] = kk * CEFF_(y[3776]); }
    { const double kk = ws[52704]; ws[93536] = kk * CEFF_(y[5792]); ws[93568] = kk * CEFF_(y[4672]); }
    { const double kk = ws[52736]; ws[93600] = kk * CEFF_(y[5792]); ws[93632] = kk * CEFF_(y[3520]); }
    { const double kk = ws[52768]; ws[93664] = kk * CEFF_(y[5792]); ws[93696] = kk * CEFF_(y[2880]); }
    { const double kk = ws[52800]; ws[93728] = kk * CEFF_(y[5792]); ws[93760] = kk * CEFF_(y[2912]); }
    { const double kk = ws[52832]; ws[93792] = kk * CEFF_(y[5792]); ws[93824] = kk * CEFF_(y[2592]); }
    { const double kk = ws[52864]; ws[93856] = kk * CEFF_(y[5792]); ws[93888] = kk * CEFF_(y[2272]); }
    { const double kk = ws[52896]; ws[93920] = kk * CEFF_(y[5792]); ws[93952] = kk * CEFF_(y[3648]); }
    { const double kk = ws[52928]; ws[93984] = kk * CEFF_(y[5792]); ws[94016] = kk * CEFF_(y[3040]); }
    { const double kk = ws[52960]; ws[94048] = kk * CEFF_(y[5792]); ws[94080] = kk * CEFF_(y[2976]); }
    { const double kk = ws[52992]; ws[94112] = kk * CEFF_(y[5792]); ws[94144] = kk * CEFF_(y[4032]); }
    { const double kk = ws[53024]; ws[94176] = kk * CEFF_(y[5792]); ws[94208] = kk * CEFF_(y[4064]); }
    { const double kk = ws[53056]; ws[94240] = kk * CEFF_(y[5792]); ws[94272] = kk * CEFF_(y[3072]); }
    { const double kk = ws[53088]; ws[94304] = kk * CEFF_(y[5792]); ws[94336] = kk * CEFF_(y[5216]); }
    { const double kk = ws[53120]; ws[94368] = kk * CEFF_(y[4800]); ws[94400] = kk * CEFF_(y[4800]); }
    { const double kk = ws[53152]; ws[94432] = kk * CEFF_(y[5952]); ws[94464] = kk * CEFF_(y[5888]); }
    { const double kk = ws[53184]; ws[94496] = kk * CEFF_(y[5952]); ws[94528] = kk * CEFF_(y[5632]); }
    { const double kk = ws[53216]; ws[94560] = kk * CEFF_(y[5952]); ws[94592] = kk * CEFF_(y[5408]); }
    { const double kk = ws[53248]; ws[94624] = kk * CEFF_(y[5952]); ws[94656] = kk * CEFF_(y[5120]); }
    { const double kk = ws[53280]; ws[94688] = kk * CEFF_(y[5952]); ws[94720] = kk * CEFF_(y[3008]); }
    { const double kk = ws[53312]; ws[94752] = kk * CEFF_(y[5952]); ws[94784] = kk * CEFF_(y[3200]); }
    { const double kk = ws[53344]; ws[94816] = kk * CEFF_(y[5952]); ws[94848] = kk * CEFF_(y[3328]); }
    { const double kk = ws[53376]; ws[94880] = kk * CEFF_(y[5952]); ws[94912] = kk * CEFF_(y[3360]); }
    { const double kk = ws[53408]; ws[94944] = kk * CEFF_(y[5952]); ws[94976] = kk * CEFF_(y[3296]); }
    { const double kk = ws[53440]; ws[95008] = kk * CEFF_(y[5952]); ws[95040] = kk * CEFF_(y[3104]); }
    { const double kk = ws[53472]; ws[95072] = kk * CEFF_(y[5952]); ws[95104] = kk * CEFF_(y[3264]); }
    { const double kk = ws[53504]; ws[95136] = kk * CEFF_(y[5952]); ws[95168] = kk * CEFF_(y[4288]); }
    { const double kk = ws[53536]; ws[95200] = kk * CEFF_(y[5952]); ws[95232] = kk * CEFF_(y[4160]); }
    { const double kk = ws[53568]; ws[95264] = kk * CEFF_(y[5952]); ws[95296] = kk * CEFF_(y[4192]); }
    { const double kk = ws[53600]; ws[95328] = kk * CEFF_(y[5952]); ws[95360] = kk * CEFF_(y[2624]); }
    { const double kk = ws[53632]; ws[95392] = kk * CEFF_(y[5952]); ws[95424] = kk * CEFF_(y[2656]); }
    { const double kk = ws[53664]; ws[95456] = kk * CEFF_(y[5952]); ws[95488] = kk * CEFF_(y[5792]); }
    { const double kk = ws[53696]; ws[95520] = kk * CEFF_(y[5952]); ws[95552] = kk * CEFF_(y[4800]); }
    { const double kk = ws[53728]; ws[95584] = kk * CEFF_(y[5952]); ws[95616] = kk * CEFF_(y[2848]); }
    { const double kk = ws[53760]; ws[95648] = kk * CEFF_(y[5952]); ws[95680] = kk * CEFF_(y[5152]); }
    { const double kk = ws[53792]; ws[95712] = kk * CEFF_(y[5952]); ws[95744] = kk * CEFF_(y[3776]); }
    { const double kk = ws[53824]; ws[95776] = kk * CEFF_(y[5952]); ws[95808] = kk * CEFF_(y[4672]); }
    { const double kk = ws[53856]; ws[95840] = kk * CEFF_(y[5952]); ws[95872] = kk * CEFF_(y[3520]); }
    { const double kk = ws[53888]; ws[95904] = kk * CEFF_(y[5952]); ws[95936] = kk * CEFF_(y[2880]); }
    { const double kk = ws[53920]; ws[95968] = kk * CEFF_(y[5952]); ws[96000] = kk * CEFF_(y[2912]); }
    { const double kk = ws[53952]; ws[96032] = kk * CEFF_(y[5952]); ws[96064] = kk * CEFF_(y[2592]); }
    { const double kk = ws[53984]; ws[96096] = kk * CEFF_(y[5952]); ws[96128] = kk * CEFF_(y[2272]); }
    { const double kk = ws[54016]; ws[96160] = kk * CEFF_(y[5952]); ws[96192] = kk * CEFF_(y[3648]); }
    { const double kk = ws[54048]; ws[96224] = kk * CEFF_(y[5952]); ws[96256] = kk * CEFF_(y[3040]); }
    { const double kk = ws[54080]; ws[96288] = kk * CEFF_(y[5952]); ws[96320] = kk * CEFF_(y[2976]); }
    { const double kk = ws[54112]; ws[96352] = kk * CEFF_(y[5952]); ws[96384] = kk * CEFF_(y[4032]); }
    { const double kk = ws[54144]; ws[96416] = kk * CEFF_(y[5952]); ws[96448] = kk * CEFF_(y[4064]); }
    { const double kk = ws[54176]; ws[96480] = kk * CEFF_(y[5952]); ws[96512] = kk * CEFF_(y[3072]); }
    { const double kk = ws[54208]; ws[96544] = kk * CEFF_(y[4032]); ws[96576] = kk * CEFF_(y[4032]); }
    { const double kk = ws[54240]; ws[96608] = kk * CEFF_(y[4064]); ws[96640] = kk * CEFF_(y[4032]); }
    { const double kk = ws[54272]; ws[96672] = kk * CEFF_(y[4064]); ws[96704] = kk * CEFF_(y[4064]); }
    { const double kk = ws[54304]; ws[96736] = kk * CEFF_(y[5952]); ws[96768] = kk * CEFF_(y[5216]); }
    { const double kk = ws[54336]; ws[96800] = kk * CEFF_(y[4800]); ws[96832] = kk * CEFF_(y[5216]); }
    { const double kk = ws[54368]; ws[96864] = kk * CEFF_(y[5216]); ws[96896] = kk * CEFF_(y[5216]); }
    { const double kk = ws[54400]; ws[96928] = kk * CEFF_(y[4160]); ws[96960] = kk * CEFF_(y[3744]); }
    { const double kk = ws[54432]; ws[96992] = kk * CEFF_(y[4192]); ws[97024] = kk * CEFF_(y[3744]); }
    { const double kk = ws[54464]; ws[97056] = kk * CEFF_(y[4288]); ws[97088] = kk * CEFF_(y[3744]); }
    { const double kk = ws[54496]; ws[97120] = kk * CEFF_(y[4160]); ws[97152] = kk * CEFF_(y[3936]); }
    { const double kk = ws[54528]; ws[97184] = kk * CEFF_(y[4192]); ws[97216] = kk * CEFF_(y[3936]); }
    { const double kk = ws[54560]; ws[97248] = kk * CEFF_(y[4288]); ws[97280] = kk * CEFF_(y[3936]); }
    { const double kk = ws[54592]; ws[97312] = kk * CEFF_(y[4160]); ws[97344] = kk * CEFF_(y[3840]); }
    { const double kk = ws[54624]; ws[97376] = kk * CEFF_(y[4192]); ws[97408] = kk * CEFF_(y[3840]); }
    { const double kk = ws[54656]; ws[97440] = kk * CEFF_(y[4288]); ws[97472] = kk * CEFF_(y[3840]); }
    { const double kk = ws[54688]; ws[97504] = kk * CEFF_(y[4160]); ws[97536] = kk * CEFF_(y[3712]); }
    { const double kk = ws[54720]; ws[97568] = kk * CEFF_(y[4192]); ws[97600] = kk * CEFF_(y[3712]); }
    { const double kk = ws[54752]; ws[97632] = kk * CEFF_(y[4288]); ws[97664] = kk * CEFF_(y[3712]); }
    { const double kk = ws[54784]; ws[97696] = kk * CEFF_(y[6016]); ws[97728] = kk * CEFF_(y[1376]); }
    { const double kk = ws[54816]; ws[97760] = kk * CEFF_(y[6016]); ws[97792] = kk * CEFF_(y[384]); }
    { const double kk = ws[54848]; ws[97824] = kk * CEFF_(y[6016]); ws[97856] = kk * CEFF_(y[416]); }
    { const double kk = ws[54880]; ws[97888] = kk * CEFF_(y[6016]); ws[97920] = kk * CEFF_(y[3552]); }
    { const double kk = ws[54912]; ws[97952] = kk * CEFF_(y[5184]); ws[97984] = kk * CEFF_(y[3552]); }
    { const double kk = ws[54944]; ws[98016] = kk * CEFF_(y[5952]); ws[98048] = kk * CEFF_(y[3552]); }
    { const double kk = ws[55008]; ws[98080] = kk * CEFF_(y[6016]); ws[98112] = kk * CEFF_(y[1568]); }
    { const double kk = ws[55040]; ws[98144] = kk * CEFF_(y[5824]); ws[98176] = kk * CEFF_(y[3136]); }
    { const double kk = ws[55072]; ws[98208] = kk * CEFF_(y[5952]); ws[98240] = kk * CEFF_(y[3136]); }
    { const double kk = ws[55104]; ws[98272] = kk * CEFF_(y[5984]); ws[98304] = kk * CEFF_(y[3136]); }
    { const double kk = ws[55136]; ws[98336] = kk * CEFF_(y[5888]); ws[98368] = kk * CEFF_(y[3136]); }
    { const double kk = ws[55168]; ws[98400] = kk * CEFF_(y[5792]); ws[98432] = kk * CEFF_(y[3136]); }
    { const double kk = ws[55200]; ws[98464] = kk * CEFF_(y[5184]); ws[98496] = kk * CEFF_(y[1568]); }
    { const double kk = ws[55232]; ws[98528] = kk * CEFF_(y[5952]); ws[98560] = kk * CEFF_(y[1568]); }
    { const double kk = ws[55264]; ws[98592] = kk * CEFF_(y[6016]); ws[98624] = kk * CEFF_(y[3168]); }
    { const double kk = ws[55296]; ws[98656] = kk * CEFF_(y[5824]); ws[98688] = kk * CEFF_(y[1856]); }
    { const double kk = ws[55328]; ws[98720] = kk * CEFF_(y[5984]); ws[98752] = kk * CEFF_(y[1856]); }
    { const double kk = ws[55360]; ws[98784] = kk * CEFF_(y[6016]); ws[98816] = kk * CEFF_(y[4512]); }
    { const double kk = ws[55392]; ws[98848] = kk * CEFF_(y[5184]); ws[98880] = kk * CEFF_(y[3168]); }
    { const double kk = ws[55424]; ws[98912] = kk * CEFF_(y[5952]); ws[98944] = kk * CEFF_(y[3168]); }
    { const double kk = ws[55456]; ws[98976] = kk * CEFF_(y[6016]); ws[99008] = kk * CEFF_(y[448]); }
    { const double kk = ws[55488]; ws[99040] = kk * CEFF_(y[5952]); ws[99072] = kk * CEFF_(y[1600]); }
    { const double kk = ws[55520]; ws[99104] = kk * CEFF_(y[5984]); ws[99136] = kk * CEFF_(y[1920]); }
    { const double kk = ws[55552]; ws[99168] = kk * CEFF_(y[5824]); ws[99200] = kk * CEFF_(y[1920]); }
    { const double kk = ws[55584]; ws[99232] = kk * CEFF_(y[5952]); ws[99264] = kk * CEFF_(y[1920]); }
    { const double kk = ws[55616]; ws[99296] = kk * CEFF_(y[5184]); ws[99328] = kk * CEFF_(y[1600]); }
    { const double kk = ws[55648]; ws[99360] = kk * CEFF_(y[6016]); ws[99392] = kk * CEFF_(y[1600]); }
    { const double kk = ws[55680]; ws[99424] = kk * CEFF_(y[5984]); ws[99456] = kk * CEFF_(y[2304]); }
    { const double kk = ws[55712]; ws[99488] = kk * CEFF_(y[5952]); ws[99520] = kk * CEFF_(y[2304]); }
    { const double kk = ws[55744]; ws[99552] = kk * CEFF_(y[5824]); ws[99584] = kk * CEFF_(y[2304]); }
    { const double kk = ws[56064]; ws[99616] = kk * CEFF_(y[512]); ws[99648] = kk * CEFF_(y[1056]); }
    { const double kk = ws[56160]; ws[99680] = kk * CEFF_(y[6016]); ws[99712] = kk * CEFF_(y[608]); }
    { const double kk = ws[56192]; ws[99744] = kk * CEFF_(y[6016]); ws[99776] = kk * CEFF_(y[640]); }
    { const double kk = ws[56224]; ws[99808] = kk * CEFF_(y[6016]); ws[99840] = kk * CEFF_(y[672]); }
    { const double kk = ws[56256]; ws[99872] = kk * CEFF_(y[6016]); ws[99904] = kk * CEFF_(y[704]); }
    { const double kk = ws[56288]; ws[99936] = kk * CEFF_(y[6016]); ws[99968] = kk * CEFF_(y[736]); }
    { const double kk = ws[56320]; ws[100000] = kk * CEFF_(y[6016]); ws[100032] = kk * CEFF_(y[768]); }
    { const double kk = ws[56352]; ws[100064] = kk * CEFF_(y[6016]); ws[100096] = kk * CEFF_(y[800]); }
    { const double kk = ws[56384]; ws[100128] = kk * CEFF_(y[5824]); ws[100160] = kk * CEFF_(y[2368]); }
    { const double kk = ws[56416]; ws[100192] = kk * CEFF_(y[5824]); ws[100224] = kk * CEFF_(y[2400]); }
    { const double kk = ws[56448]; ws[100256] = kk * CEFF_(y[5824]); ws[100288] = kk * CEFF_(y[2432]); }
    { const double kk = ws[56480]; ws[100320] = kk * CEFF_(y[5824]); ws[100352] = kk * CEFF_(y[2464]); }
    { const double kk = ws[56512]; ws[100384] = kk * CEFF_(y[5824]); ws[100416] = kk * CEFF_(y[2496]); }
    { const double kk = ws[56544]; ws[100448] = kk * CEFF_(y[5824]); ws[100480] = kk * CEFF_(y[2528]); }
    { const double kk = ws[56576]; ws[100512] = kk * CEFF_(y[5824]); ws[100544] = kk * CEFF_(y[3904]); }
    { const double kk = ws[56608]; ws[100576] = kk * CEFF_(y[5952]); ws[100608] = kk * CEFF_(y[2368]); }
    { const double kk = ws[56640]; ws[100640] = kk * CEFF_(y[5952]); ws[100672] = kk * CEFF_(y[2400]); }
    { const double kk = ws[56672]; ws[100704] = kk * CEFF_(y[5952]); ws[100736] = kk * CEFF_(y[2432]); }
    { const double kk = ws[56704]; ws[100768] = kk * CEFF_(y[5952]); ws[100800] = kk * CEFF_(y[2464]); }
    { const double kk = ws[56736]; ws[100832] = kk * CEFF_(y[5952]); ws[100864] = kk * CEFF_(y[2496]); }
    { const double kk = ws[56768]; ws[100896] = kk * CEFF_(y[5952]); ws[100928] = kk * CEFF_(y[2528]); }
    { const double kk = ws[56800]; ws[100960] = kk * CEFF_(y[5952]); ws[100992] = kk * CEFF_(y[3904]); }
    { const double kk = ws[56832]; ws[101024] = kk * CEFF_(y[5984]); ws[101056] = kk * CEFF_(y[2368]); }
    { const double kk = ws[56864]; ws[101088] = kk * CEFF_(y[5984]); ws[101120] = kk * CEFF_(y[2400]); }
    { const double kk = ws[56896]; ws[101152] = kk * CEFF_(y[5984]); ws[101184] = kk * CEFF_(y[2432]); }
    { const double kk = ws[56928]; ws[101216] = kk * CEFF_(y[5984]); ws[101248] = kk * CEFF_(y[2464]); }
    { const double kk = ws[56960]; ws[101280] = kk * CEFF_(y[5984]); ws[101312] = kk * CEFF_(y[2496]); }
    { const double kk = ws[56992]; ws[101344] = kk * CEFF_(y[5984]); ws[101376] = kk * CEFF_(y[2528]); }
    { const double kk = ws[57024]; ws[101408] = kk * CEFF_(y[5984]); ws[101440] = kk * CEFF_(y[3904]); }
    { const double kk = ws[57280]; ws[101472] = kk * CEFF_(y[5824]); ws[101504] = kk * CEFF_(y[1952]); }
    { const double kk = ws[57312]; ws[101536] = kk * CEFF_(y[5824]); ws[101568] = kk * CEFF_(y[1984]); }
    { const double kk = ws[57344]; ws[101600] = kk * CEFF_(y[5824]); ws[101632] = kk * CEFF_(y[2016]); }
    { const double kk = ws[57376]; ws[101664] = kk * CEFF_(y[5824]); ws[101696] = kk * CEFF_(y[2048]); }
    { const double kk = ws[57408]; ws[101728] = kk * CEFF_(y[5824]); ws[101760] = kk * CEFF_(y[2080]); }
    { const double kk = ws[57440]; ws[101792] = kk * CEFF_(y[5824]); ws[101824] = kk * CEFF_(y[2112]); }
    { const double kk = ws[57472]; ws[101856] = kk * CEFF_(y[5824]); ws[101888] = kk * CEFF_(y[2144]); }
    { const double kk = ws[57504]; ws[101920] = kk * CEFF_(y[5952]); ws[101952] = kk * CEFF_(y[1952]); }
    { const double kk = ws[57536]; ws[101984] = kk * CEFF_(y[5952]); ws[102016] = kk * CEFF_(y[1984]); }
    { const double kk = ws[57568]; ws[102048] = kk * CEFF_(y[5952]); ws[102080] = kk * CEFF_(y[2016]); }
    { const double kk = ws[57600]; ws[102112] = kk * CEFF_(y[5952]); ws[102144] = kk * CEFF_(y[2048]); }
    { const double kk = ws[57632]; ws[102176] = kk * CEFF_(y[5952]); ws[102208] = kk * CEFF_(y[2080]); }
    { const double kk = ws[57664]; ws[102240] = kk * CEFF_(y[5952]); ws[102272] = kk * CEFF_(y[2112]); }
    { const double kk = ws[57696]; ws[102304] = kk * CEFF_(y[5952]); ws[102336] = kk * CEFF_(y[2144]); }
    { const double kk = ws[57728]; ws[102368] = kk * CEFF_(y[5984]); ws[102400] = kk * CEFF_(y[1952]); }
    { const double kk = ws[57760]; ws[102432] = kk * CEFF_(y[5984]); ws[102464] = kk * CEFF_(y[1984]); }
    { const double kk = ws[57792]; ws[102496] = kk * CEFF_(y[5984]); ws[102528] = kk * CEFF_(y[2016]); }
    { const double kk = ws[57824]; ws[102560] = kk * CEFF_(y[5984]); ws[102592] = kk * CEFF_(y[2048]); }
    { const double kk = ws[57856]; ws[102624] = kk * CEFF_(y[5984]); ws[102656] = kk * CEFF_(y[2080]); }
    { const double kk = ws[57888]; ws[102688] = kk * CEFF_(y[5984]); ws[102720] = kk * CEFF_(y[2112]); }
    { const double kk = ws[57920]; ws[102752] = kk * CEFF_(y[5984]); ws[102784] = kk * CEFF_(y[2144]); }
    { const double kk = ws[57952]; ws[102816] = kk * CEFF_(y[6016]); ws[102848] = kk * CEFF_(y[832]); }
    { const double kk = ws[57984]; ws[102880] = kk * CEFF_(y[5984]); ws[102912] = kk * CEFF_(y[3392]); }
    { const double kk = ws[58016]; ws[102944] = kk * CEFF_(y[5824]); ws[102976] = kk * CEFF_(y[3392]); }
    { const double kk = ws[58048]; ws[103008] = kk * CEFF_(y[5952]); ws[103040] = kk * CEFF_(y[3392]); }
    { const double kk = ws[58080]; ws[103072] = kk * CEFF_(y[5888]); ws[103104] = kk * CEFF_(y[3392]); }
    { const double kk = ws[58112]; ws[103136] = kk * CEFF_(y[5792]); ws[103168] = kk * CEFF_(y[3392]); }
    { const double kk = ws[58144]; ws[103200] = kk * CEFF_(y[6016]); ws[103232] = kk * CEFF_(y[864]); }
    { const double kk = ws[58176]; ws[103264] = kk * CEFF_(y[5984]); ws[103296] = kk * CEFF_(y[3424]); }
    { const double kk = ws[58208]; ws[103328] = kk * CEFF_(y[5824]); ws[103360] = kk * CEFF_(y[3424]); }
    { const double kk = ws[58240]; ws[103392] = kk * CEFF_(y[5952]); ws[103424] = kk * CEFF_(y[3424]); }
    { const double kk = ws[58272]; ws[103456] = kk * CEFF_(y[5888]); ws[103488] = kk * CEFF_(y[3424]); }
    { const double kk = ws[58304]; ws[103520] = kk * CEFF_(y[5792]); ws[103552] = kk * CEFF_(y[3424]); }
    { const double kk = ws[58336]; ws[103584] = kk * CEFF_(y[6016]); ws[103616] = kk * CEFF_(y[896]); }
    { const double kk = ws[58368]; ws[103648] = kk * CEFF_(y[5984]); ws[103680] = kk * CEFF_(y[3456]); }
    { const double kk = ws[58400]; ws[103712] = kk * CEFF_(y[5824]); ws[103744] = kk * CEFF_(y[3456]); }
    { const double kk = ws[58432]; ws[103776] = kk * CEFF_(y[5952]); ws[103808] = kk * CEFF_(y[3456]); }
    { const double kk = ws[58464]; ws[103840] = kk * CEFF_(y[5888]); ws[103872] = kk * CEFF_(y[3456]); }
    { const double kk = ws[58496]; ws[103904] = kk * CEFF_(y[5792]); ws[103936] = kk * CEFF_(y[3456]); }
    { const double kk = ws[58528]; ws[103968] = kk * CEFF_(y[6016]); ws[104000] = kk * CEFF_(y[4768]); }
    { const double kk = ws[58560]; ws[104032] = kk * CEFF_(y[6016]); ws[104064] = kk * CEFF_(y[4864]); }
    { const double kk = ws[58592]; ws[104096] = kk * CEFF_(y[6016]); ws[104128] = kk * CEFF_(y[4832]); }
    { const double kk = ws[58624]; ws[104160] = kk * CEFF_(y[6016]); ws[104192] = kk * CEFF_(y[4896]); }
    { const double kk = ws[58656]; ws[104224] = kk * CEFF_(y[6016]); ws[104256] = kk * CEFF_(y[4640]); }
    { const double kk = ws[58688]; ws[104288] = kk * CEFF_(y[6016]); ws[104320] = kk * CEFF_(y[4416]); }
    { const double kk = ws[58720]; ws[104352] = kk * CEFF_(y[6016]); ws[104384] = kk * CEFF_(y[4928]); }
    { const double kk = ws[58752]; ws[104416] = kk * CEFF_(y[6016]); ws[104448] = kk * CEFF_(y[4960]); }
    { const double kk = ws[58784]; ws[104480] = kk * CEFF_(y[6016]); ws[104512] = kk * CEFF_(y[4992]); }
    { const double kk = ws[58816]; ws[104544] = kk * CEFF_(y[6016]); ws[104576] = kk * CEFF_(y[4704]); }
    { const double kk = ws[58848]; ws[104608] = kk * CEFF_(y[6016]); ws[104640] = kk * CEFF_(y[5088]); }
    { const double kk = ws[58880]; ws[104672] = kk * CEFF_(y[6016]); ws[104704] = kk * CEFF_(y[5536]); }
    { const double kk = ws[58912]; ws[104736] = kk * CEFF_(y[6016]); ws[104768] = kk * CEFF_(y[5312]); }
    { const double kk = ws[58944]; ws[104800] = kk * CEFF_(y[6016]); ws[104832] = kk * CEFF_(y[4224]); }
    { const double kk = ws[58976]; ws[104864] = kk * CEFF_(y[6016]); ws[104896] = kk * CEFF_(y[3968]); }
    { const double kk = ws[59008]; ws[104928] = kk * CEFF_(y[6016]); ws[104960] = kk * CEFF_(y[4608]); }
    { const double kk = ws[59040]; ws[104992] = kk * CEFF_(y[6016]); ws[105024] = kk * CEFF_(y[928]); }
    { const double kk = ws[59136]; ws[105056] = kk * CEFF_(y[6016]); ws[105088] = kk * CEFF_(y[992]); }
    { const double kk = ws[59168]; ws[105120] = kk * CEFF_(y[5984]); ws[105152] = kk * CEFF_(y[3488]); }
    { const double kk = ws[59200]; ws[105184] = kk * CEFF_(y[5824]); ws[105216] = kk * CEFF_(y[3488]); }
    { const double kk = ws[59232]; ws[105248] = kk * CEFF_(y[5952]); ws[105280] = kk * CEFF_(y[3488]); }
    { const double kk = ws[59264]; ws[105312] = kk * CEFF_(y[5888]); ws[105344] = kk * CEFF_(y[3488]); }
    { const double kk = ws[59296]; ws[105376] = kk * CEFF_(y[5792]); ws[105408] = kk * CEFF_(y[3488]); }
#undef CEFF_
}
}  // namespace mech_cracmm2
