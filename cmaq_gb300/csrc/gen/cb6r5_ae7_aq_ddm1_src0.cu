// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void ddm_src_1_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[1]) {
      const double q = scale * ws[44576];
      out[4160] = out[4160] - q;
      out[4320] = fma(1.0, q, out[4320]);
    }
    if (mask[2]) {
      const double q = scale * ws[44608];
      out[4320] = out[4320] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[3]) {
      const double q = scale * ws[44640];
      out[4160] = out[4160] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[4]) {
      const double q = scale * ws[44672];
      out[4160] = out[4160] - q;
      out[4608] = out[4608] - q;
      out[4384] = fma(1.0, q, out[4384]);
    }
    if (mask[5]) {
      const double q = scale * ws[44704];
      out[4160] = out[4160] - q;
      out[4608] = out[4608] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[6]) {
      const double q = scale * ws[44736];
      out[4160] = out[4160] - q;
      out[4320] = out[4320] - q;
    }
    if (mask[9]) {
      const double q = scale * ws[44832];
      out[672] = out[672] - q;
      out[4160] = fma(1.0, q, out[4160]);
    }
    if (mask[10]) {
      const double q = scale * ws[44864];
      out[672] = out[672] - q;
      out[4736] = fma(2.0, q, out[4736]);
    }
    if (mask[11]) {
      const double q = scale * ws[44896];
      out[4320] = out[4320] - q;
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[12]) {
      const double q = scale * ws[44928];
      out[4320] = out[4320] - q;
      out[4704] = out[4704] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[13]) {
      const double q = scale * ws[44960];
      out[4736] = out[4736] - q;
      out[4160] = out[4160] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[14]) {
      const double q = scale * ws[44992];
      out[4704] = out[4704] - q;
      out[4160] = out[4160] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[15]) {
      const double q = scale * ws[45024];
      out[4736] = out[4736] - q;
      out[4736] = out[4736] - q;
      out[4160] = fma(1.0, q, out[4160]);
    }
    if (mask[16]) {
      const double q = scale * ws[45056];
      out[4736] = out[4736] - q;
      out[4736] = out[4736] - q;
      out[3456] = fma(1.0, q, out[3456]);
    }
    if (mask[17]) {
      const double q = scale * ws[45088];
      out[4736] = out[4736] - q;
      out[4704] = out[4704] - q;
    }
    if (mask[18]) {
      const double q = scale * ws[45120];
      out[4704] = out[4704] - q;
      out[4704] = out[4704] - q;
      out[3456] = fma(1.0, q, out[3456]);
    }
    if (mask[19]) {
      const double q = scale * ws[45152];
      out[4704] = out[4704] - q;
      out[4704] = out[4704] - q;
      out[3456] = fma(1.0, q, out[3456]);
    }
    if (mask[21]) {
      const double q = scale * ws[45216];
      out[3456] = out[3456] - q;
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[22]) {
      const double q = scale * ws[45248];
      out[3456] = out[3456] - q;
      out[4160] = out[4160] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[23]) {
      const double q = scale * ws[45280];
      out[4384] = out[4384] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(2.0, q, out[4608]);
    }
    if (mask[24]) {
      const double q = scale * ws[45312];
      out[4704] = out[4704] - q;
      out[4384] = out[4384] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[25]) {
      const double q = scale * ws[45344];
      out[4608] = out[4608] - q;
      out[4320] = out[4320] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[28]) {
      const double q = scale * ws[45440];
      out[4640] = out[4640] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(2.0, q, out[4608]);
    }
    if (mask[29]) {
      const double q = scale * ws[45472];
      out[4640] = out[4640] - q;
      out[4608] = out[4608] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[30]) {
      const double q = scale * ws[45504];
      out[4640] = out[4640] - q;
      out[4160] = out[4160] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[31]) {
      const double q = scale * ws[45536];
      out[4640] = out[4640] - q;
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[32]) {
      const double q = scale * ws[45568];
      out[4640] = out[4640] - q;
      out[4704] = out[4704] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[33]) {
      const double q = scale * ws[45600];
      out[4640] = out[4640] - q;
      out[4320] = out[4320] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[34]) {
      const double q = scale * ws[45632];
      out[4640] = out[4640] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(2.0, q, out[4608]);
    }
    if (mask[35]) {
      const double q = scale * ws[45664];
      out[4640] = out[4640] - q;
      out[4608] = out[4608] - q;
      out[1280] = fma(1.0, q, out[1280]);
    }
    if (mask[36]) {
      const double q = scale * ws[45696];
      out[1280] = out[1280] - q;
      out[4640] = fma(1.0, q, out[4640]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[38]) {
      const double q = scale * ws[45760];
      out[1280] = out[1280] - q;
      out[4192] = fma(2.0, q, out[4192]);
    }
    if (mask[39]) {
      const double q = scale * ws[45792];
      out[4384] = out[4384] - q;
      out[4736] = out[4736] - q;
      out[2464] = fma(1.0, q, out[2464]);
    }
    if (mask[40]) {
      const double q = scale * ws[45824];
      out[4384] = out[4384] - q;
      out[4608] = out[4608] - q;
      out[2464] = fma(2.0, q, out[2464]);
    }
    if (mask[41]) {
      const double q = scale * ws[45856];
      out[2464] = out[2464] - q;
      out[2464] = out[2464] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[43]) {
      const double q = scale * ws[45920];
      out[2464] = out[2464] - q;
      out[4736] = out[4736] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[44]) {
      const double q = scale * ws[45952];
      out[4608] = out[4608] - q;
      out[4736] = out[4736] - q;
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[45]) {
      const double q = scale * ws[45984];
      out[4192] = out[4192] - q;
      out[4736] = out[4736] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[47]) {
      const double q = scale * ws[46048];
      out[4704] = out[4704] - q;
      out[4608] = out[4608] - q;
      out[1696] = fma(1.0, q, out[1696]);
    }
    if (mask[48]) {
      const double q = scale * ws[46080];
      out[1696] = out[1696] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[50]) {
      const double q = scale * ws[46144];
      out[1696] = out[1696] - q;
      out[4736] = out[4736] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[51]) {
      const double q = scale * ws[46176];
      out[2208] = out[2208] - q;
      out[4736] = out[4736] - q;
      out[256] = fma(1.0, q, out[256]);
      out[4704] = fma(1.0, q, out[4704]);
      out[288] = fma(1.0, q, out[288]);
    }
    if (mask[52]) {
      const double q = scale * ws[46208];
      out[4448] = out[4448] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[53]) {
      const double q = scale * ws[46240];
      out[4448] = out[4448] - q;
      out[4608] = out[4608] - q;
      out[1344] = fma(1.0, q, out[1344]);
    }
    if (mask[54]) {
      const double q = scale * ws[46272];
      out[1344] = out[1344] - q;
      out[4608] = fma(1.0, q, out[4608]);
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[56]) {
      const double q = scale * ws[46336];
      out[4448] = out[4448] - q;
      out[4704] = out[4704] - q;
      out[2688] = fma(0.37, q, out[2688]);
      out[3904] = fma(0.13, q, out[3904]);
      out[4320] = fma(0.13, q, out[4320]);
      out[4416] = fma(0.5, q, out[4416]);
      out[4672] = fma(0.5, q, out[4672]);
      out[4736] = fma(0.5, q, out[4736]);
    }
    if (mask[57]) {
      const double q = scale * ws[46368];
      out[4448] = out[4448] - q;
      out[4672] = out[4672] - q;
      out[4416] = fma(1.0, q, out[4416]);
    }
    if (mask[58]) {
      const double q = scale * ws[46400];
      out[4448] = out[4448] - q;
      out[4448] = out[4448] - q;
      out[4416] = fma(2.0, q, out[4416]);
      out[4672] = fma(2.0, q, out[4672]);
    }
    if (mask[59]) {
      const double q = scale * ws[46432];
      out[4448] = out[4448] - q;
      out[4096] = out[4096] - q;
      out[4416] = fma(1.0, q, out[4416]);
      out[4128] = fma(1.0, q, out[4128]);
      out[4576] = fma(1.0, q, out[4576]);
      out[4672] = fma(2.0, q, out[4672]);
    }
    if (mask[60]) {
      const double q = scale * ws[46464];
      out[4096] = out[4096] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
      out[4128] = fma(1.0, q, out[4128]);
      out[4576] = fma(1.0, q, out[4576]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[61]) {
      const double q = scale * ws[46496];
      out[4096] = out[4096] - q;
      out[4608] = out[4608] - q;
      out[1952] = fma(1.0, q, out[1952]);
    }
    if (mask[62]) {
      const double q = scale * ws[46528];
      out[1952] = out[1952] - q;
      out[4608] = fma(1.0, q, out[4608]);
      out[4096] = fma(1.0, q, out[4096]);
    }
    if (mask[64]) {
      const double q = scale * ws[46592];
      out[4096] = out[4096] - q;
      out[4704] = out[4704] - q;
      out[2688] = fma(0.37, q, out[2688]);
      out[3904] = fma(0.13, q, out[3904]);
      out[4320] = fma(0.13, q, out[4320]);
      out[4736] = fma(0.5, q, out[4736]);
      out[4416] = fma(0.5, q, out[4416]);
      out[4672] = fma(0.5, q, out[4672]);
    }
    if (mask[65]) {
      const double q = scale * ws[46624];
      out[4096] = out[4096] - q;
      out[4672] = out[4672] - q;
      out[4416] = fma(1.0, q, out[4416]);
    }
    if (mask[66]) {
      const double q = scale * ws[46656];
      out[4096] = out[4096] - q;
      out[4096] = out[4096] - q;
      out[4416] = fma(2.0, q, out[4416]);
      out[4672] = fma(2.0, q, out[4672]);
    }
    if (mask[67]) {
      const double q = scale * ws[46688];
      out[4672] = out[4672] - q;
      out[4384] = out[4384] - q;
      out[4384] = fma(1.0, q, out[4384]);
    }
    if (mask[68]) {
      const double q = scale * ws[46720];
      out[4672] = out[4672] - q;
      out[4704] = out[4704] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[69]) {
      const double q = scale * ws[46752];
      out[4672] = out[4672] - q;
      out[4672] = out[4672] - q;
    }
    if (mask[70]) {
      const double q = scale * ws[46784];
      out[4416] = out[4416] - q;
      out[4384] = out[4384] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[71]) {
      const double q = scale * ws[46816];
      out[4416] = out[4416] - q;
      out[4704] = out[4704] - q;
      out[2272] = fma(0.9, q, out[2272]);
      out[4512] = fma(0.1, q, out[4512]);
    }
    if (mask[72]) {
      const double q = scale * ws[46848];
      out[4416] = out[4416] - q;
      out[4448] = out[4448] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4704] = fma(0.9, q, out[4704]);
      out[4416] = fma(0.9, q, out[4416]);
      out[3904] = fma(0.1, q, out[3904]);
      out[4672] = fma(0.9, q, out[4672]);
    }
    if (mask[73]) {
      const double q = scale * ws[46880];
      out[4416] = out[4416] - q;
      out[4672] = out[4672] - q;
      out[4512] = fma(0.685, q, out[4512]);
      out[2720] = fma(0.315, q, out[2720]);
      out[4704] = fma(0.37, q, out[4704]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[74]) {
      const double q = scale * ws[46912];
      out[4576] = out[4576] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[75]) {
      const double q = scale * ws[46944];
      out[4576] = out[4576] - q;
      out[4704] = out[4704] - q;
      out[2880] = fma(1.0, q, out[2880]);
    }
    if (mask[76]) {
      const double q = scale * ws[46976];
      out[4576] = out[4576] - q;
      out[4448] = out[4448] - q;
      out[4704] = fma(0.8, q, out[4704]);
      out[4416] = fma(0.8, q, out[4416]);
      out[3904] = fma(0.2, q, out[3904]);
      out[4672] = fma(0.8, q, out[4672]);
    }
    if (mask[77]) {
      const double q = scale * ws[47008];
      out[4576] = out[4576] - q;
      out[4672] = out[4672] - q;
      out[4704] = fma(0.6, q, out[4704]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[78]) {
      const double q = scale * ws[47040];
      out[4352] = out[4352] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[79]) {
      const double q = scale * ws[47072];
      out[4352] = out[4352] - q;
      out[4704] = out[4704] - q;
      out[2880] = fma(1.0, q, out[2880]);
    }
    if (mask[80]) {
      const double q = scale * ws[47104];
      out[4352] = out[4352] - q;
      out[4448] = out[4448] - q;
      out[4416] = fma(0.8, q, out[4416]);
      out[3904] = fma(0.2, q, out[3904]);
      out[4672] = fma(0.8, q, out[4672]);
    }
    if (mask[81]) {
      const double q = scale * ws[47136];
      out[4352] = out[4352] - q;
      out[4672] = out[4672] - q;
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[82]) {
      const double q = scale * ws[47168];
      out[4288] = out[4288] - q;
      out[4384] = out[4384] - q;
      out[3648] = fma(0.5, q, out[3648]);
      out[4032] = fma(0.5, q, out[4032]);
    }
    if (mask[83]) {
      const double q = scale * ws[47200];
      out[4288] = out[4288] - q;
      out[4704] = out[4704] - q;
      out[2880] = fma(1.0, q, out[2880]);
    }
    if (mask[84]) {
      const double q = scale * ws[47232];
      out[4288] = out[4288] - q;
      out[4448] = out[4448] - q;
      out[4704] = fma(0.8, q, out[4704]);
      out[4416] = fma(0.8, q, out[4416]);
      out[3904] = fma(0.2, q, out[3904]);
      out[4672] = fma(0.8, q, out[4672]);
    }
    if (mask[85]) {
      const double q = scale * ws[47264];
      out[4288] = out[4288] - q;
      out[4672] = out[4672] - q;
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[86]) {
      const double q = scale * ws[47296];
      out[2272] = out[2272] - q;
      out[4736] = out[4736] - q;
      out[4416] = fma(0.6, q, out[4416]);
      out[4672] = fma(0.6, q, out[4672]);
      out[4512] = fma(0.4, q, out[4512]);
      out[4736] = fma(0.4, q, out[4736]);
    }
}
__device__ __noinline__ void ddm_src_1_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[88]) {
      const double q = scale * ws[47360];
      out[2880] = out[2880] - q;
      out[4736] = out[4736] - q;
      out[4576] = fma(0.54, q, out[4576]);
      out[4288] = fma(0.06, q, out[4288]);
      out[4672] = fma(0.6, q, out[4672]);
      out[4736] = fma(0.4, q, out[4736]);
    }
    if (mask[90]) {
      const double q = scale * ws[47424];
      out[3648] = out[3648] - q;
      out[4736] = out[4736] - q;
      out[4032] = fma(1.0, q, out[4032]);
    }
    if (mask[92]) {
      const double q = scale * ws[47488];
      out[3776] = out[3776] - q;
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[93]) {
      const double q = scale * ws[47520];
      out[3904] = out[3904] - q;
      out[4736] = out[4736] - q;
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[94]) {
      const double q = scale * ws[47552];
      out[2688] = out[2688] - q;
      out[4736] = out[4736] - q;
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[95]) {
      const double q = scale * ws[47584];
      out[4512] = out[4512] - q;
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[4480] = fma(1.0, q, out[4480]);
    }
    if (mask[98]) {
      const double q = scale * ws[47680];
      out[4512] = out[4512] - q;
      out[4160] = out[4160] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4480] = fma(1.0, q, out[4480]);
    }
    if (mask[99]) {
      const double q = scale * ws[47712];
      out[4512] = out[4512] - q;
      out[4640] = out[4640] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4480] = fma(1.0, q, out[4480]);
    }
    if (mask[100]) {
      const double q = scale * ws[47744];
      out[4512] = out[4512] - q;
      out[4704] = out[4704] - q;
      out[1728] = fma(1.0, q, out[1728]);
    }
    if (mask[101]) {
      const double q = scale * ws[47776];
      out[1728] = out[1728] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[102]) {
      const double q = scale * ws[47808];
      out[1728] = out[1728] - q;
      out[4384] = out[4384] - q;
      out[3776] = fma(1.0, q, out[3776]);
      out[4608] = fma(1.0, q, out[4608]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[103]) {
      const double q = scale * ws[47840];
      out[1728] = out[1728] - q;
      out[4704] = out[4704] - q;
      out[2272] = fma(0.5, q, out[2272]);
      out[3776] = fma(0.5, q, out[3776]);
      out[4736] = fma(0.2, q, out[4736]);
      out[4704] = fma(0.2, q, out[4704]);
    }
    if (mask[104]) {
      const double q = scale * ws[47872];
      out[4128] = out[4128] - q;
      out[4160] = out[4160] - q;
      out[4448] = fma(1.0, q, out[4448]);
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[105]) {
      const double q = scale * ws[47904];
      out[4128] = out[4128] - q;
      out[4736] = out[4736] - q;
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[106]) {
      const double q = scale * ws[47936];
      out[4128] = out[4128] - q;
      out[4640] = out[4640] - q;
      out[4448] = fma(1.0, q, out[4448]);
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[108]) {
      const double q = scale * ws[48000];
      out[4064] = out[4064] - q;
      out[4160] = out[4160] - q;
      out[4096] = fma(1.0, q, out[4096]);
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[109]) {
      const double q = scale * ws[48032];
      out[4064] = out[4064] - q;
      out[4736] = out[4736] - q;
      out[4096] = fma(1.0, q, out[4096]);
    }
    if (mask[110]) {
      const double q = scale * ws[48064];
      out[4064] = out[4064] - q;
      out[4640] = out[4640] - q;
      out[4096] = fma(1.0, q, out[4096]);
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[112]) {
      const double q = scale * ws[48128];
      out[3840] = out[3840] - q;
      out[4736] = out[4736] - q;
      out[4256] = fma(0.2, q, out[4256]);
      out[4704] = fma(0.2, q, out[4704]);
      out[4448] = fma(0.8, q, out[4448]);
    }
    if (mask[114]) {
      const double q = scale * ws[48192];
      out[3840] = out[3840] - q;
      out[4640] = out[4640] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[115]) {
      const double q = scale * ws[48224];
      out[4256] = out[4256] - q;
      out[4736] = out[4736] - q;
      out[4480] = fma(1.8, q, out[4480]);
      out[4352] = fma(0.2, q, out[4352]);
      out[4672] = fma(0.2, q, out[4672]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[117]) {
      const double q = scale * ws[48288];
      out[4256] = out[4256] - q;
      out[4640] = out[4640] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[4480] = fma(1.5, q, out[4480]);
      out[4352] = fma(0.5, q, out[4352]);
      out[4672] = fma(0.5, q, out[4672]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[119]) {
      const double q = scale * ws[48352];
      out[4000] = out[4000] - q;
      out[4640] = out[4640] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[4448] = fma(1.0, q, out[4448]);
      out[4352] = fma(1.0, q, out[4352]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[120]) {
      const double q = scale * ws[48384];
      out[4000] = out[4000] - q;
      out[4736] = out[4736] - q;
      out[4448] = fma(1.0, q, out[4448]);
      out[4480] = fma(1.0, q, out[4480]);
    }
    if (mask[121]) {
      const double q = scale * ws[48416];
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[122]) {
      const double q = scale * ws[48448];
      out[4480] = out[4480] - q;
      out[4736] = out[4736] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[123]) {
      const double q = scale * ws[48480];
      out[4736] = out[4736] - q;
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[124]) {
      const double q = scale * ws[48512];
      out[832] = out[832] - q;
      out[4736] = out[4736] - q;
      out[4128] = fma(0.991, q, out[4128]);
      out[4576] = fma(0.991, q, out[4576]);
      out[4288] = fma(0.009, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[125]) {
      const double q = scale * ws[48544];
      out[2720] = out[2720] - q;
      out[4736] = out[4736] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[126]) {
      const double q = scale * ws[48576];
      out[864] = out[864] - q;
      out[4736] = out[4736] - q;
      out[4128] = fma(0.95, q, out[4128]);
      out[4704] = fma(0.9, q, out[4704]);
      out[4576] = fma(0.1, q, out[4576]);
      out[4672] = fma(0.1, q, out[4672]);
      out[4512] = fma(0.078, q, out[4512]);
      out[3840] = fma(0.011, q, out[3840]);
    }
    if (mask[129]) {
      const double q = scale * ws[48672];
      out[3392] = out[3392] - q;
      out[4736] = out[4736] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4448] = fma(1.0, q, out[4448]);
      out[4352] = fma(1.0, q, out[4352]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[130]) {
      const double q = scale * ws[48704];
      out[896] = out[896] - q;
      out[4736] = out[4736] - q;
      out[928] = fma(1.0, q, out[928]);
    }
    if (mask[131]) {
      const double q = scale * ws[48736];
      out[4224] = out[4224] - q;
      out[4736] = out[4736] - q;
      out[1984] = fma(1.0, q, out[1984]);
    }
    if (mask[132]) {
      const double q = scale * ws[48768];
      out[960] = out[960] - q;
      out[320] = fma(0.2, q, out[320]);
      out[3392] = fma(0.42, q, out[3392]);
      out[4128] = fma(0.74, q, out[4128]);
      out[4064] = fma(0.37, q, out[4064]);
      out[4288] = fma(0.04, q, out[4288]);
      out[4576] = fma(0.94, q, out[4576]);
      out[4672] = fma(0.98, q, out[4672]);
      out[960] = fma(0.02, q, out[960]);
      out[4224] = fma(-2.7, q, out[4224]);
    }
    if (mask[133]) {
      const double q = scale * ws[48800];
      out[960] = out[960] - q;
      out[320] = fma(1.0, q, out[320]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[134]) {
      const double q = scale * ws[48832];
      out[960] = out[960] - q;
      out[4608] = out[4608] - q;
      out[3648] = fma(1.0, q, out[3648]);
    }
    if (mask[135]) {
      const double q = scale * ws[48864];
      out[352] = out[352] - q;
      out[4736] = out[4736] - q;
      out[4256] = fma(0.7, q, out[4256]);
      out[4736] = fma(0.7, q, out[4736]);
      out[3776] = fma(0.3, q, out[3776]);
      out[4480] = fma(0.3, q, out[4480]);
      out[4704] = fma(0.3, q, out[4704]);
    }
    if (mask[136]) {
      const double q = scale * ws[48896];
      out[2656] = out[2656] - q;
      out[4160] = out[4160] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4480] = fma(1.0, q, out[4480]);
      out[4576] = fma(0.7, q, out[4576]);
      out[4672] = fma(0.7, q, out[4672]);
      out[4736] = fma(0.3, q, out[4736]);
    }
    if (mask[137]) {
      const double q = scale * ws[48928];
      out[2656] = out[2656] - q;
      out[4736] = out[4736] - q;
      out[4576] = fma(1.0, q, out[4576]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4512] = fma(1.56, q, out[4512]);
      out[3840] = fma(0.22, q, out[3840]);
    }
    if (mask[138]) {
      const double q = scale * ws[48960];
      out[2656] = out[2656] - q;
      out[4320] = out[4320] - q;
      out[4512] = fma(1.0, q, out[4512]);
      out[4480] = fma(0.35, q, out[4480]);
      out[4704] = fma(0.27, q, out[4704]);
      out[4736] = fma(0.17, q, out[4736]);
      out[3776] = fma(0.42, q, out[3776]);
    }
    if (mask[139]) {
      const double q = scale * ws[48992];
      out[2656] = out[2656] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.5, q, out[4608]);
      out[3648] = fma(0.5, q, out[3648]);
      out[4576] = fma(0.5, q, out[4576]);
      out[4352] = fma(0.5, q, out[4352]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4512] = fma(1.125, q, out[4512]);
    }
    if (mask[140]) {
      const double q = scale * ws[49024];
      out[3552] = out[3552] - q;
      out[4160] = out[4160] - q;
      out[4128] = fma(0.2, q, out[4128]);
      out[4064] = fma(0.3, q, out[4064]);
      out[4704] = fma(0.1, q, out[4704]);
      out[4576] = fma(0.2, q, out[4576]);
      out[4480] = fma(0.2, q, out[4480]);
      out[4512] = fma(0.2, q, out[4512]);
      out[4288] = fma(0.01, q, out[4288]);
      out[4672] = fma(0.21, q, out[4672]);
      out[4224] = fma(0.2, q, out[4224]);
      out[4736] = fma(0.1, q, out[4736]);
    }
    if (mask[141]) {
      const double q = scale * ws[49056];
      out[3552] = out[3552] - q;
      out[4736] = out[4736] - q;
      out[4512] = fma(0.781, q, out[4512]);
      out[4128] = fma(0.488, q, out[4128]);
      out[4064] = fma(0.488, q, out[4064]);
      out[4576] = fma(0.976, q, out[4576]);
      out[4352] = fma(0.195, q, out[4352]);
      out[4288] = fma(0.024, q, out[4288]);
      out[4672] = fma(1.195, q, out[4672]);
      out[4224] = fma(-0.73, q, out[4224]);
    }
    if (mask[142]) {
      const double q = scale * ws[49088];
      out[3552] = out[3552] - q;
      out[4320] = out[4320] - q;
      out[4128] = fma(0.295, q, out[4128]);
      out[4512] = fma(0.555, q, out[4512]);
      out[4064] = fma(0.27, q, out[4064]);
      out[4576] = fma(0.15, q, out[4576]);
      out[4672] = fma(0.15, q, out[4672]);
      out[4736] = fma(0.334, q, out[4736]);
      out[4704] = fma(0.08, q, out[4704]);
      out[4480] = fma(0.378, q, out[4480]);
      out[4256] = fma(0.075, q, out[4256]);
      out[4000] = fma(0.075, q, out[4000]);
      out[3776] = fma(0.09, q, out[3776]);
      out[3904] = fma(0.13, q, out[3904]);
      out[3456] = fma(0.04, q, out[3456]);
      out[4224] = fma(-0.79, q, out[4224]);
    }
    if (mask[143]) {
      const double q = scale * ws[49120];
      out[3552] = out[3552] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.5, q, out[4608]);
      out[3648] = fma(0.5, q, out[3648]);
      out[4352] = fma(0.48, q, out[4352]);
      out[4576] = fma(0.48, q, out[4576]);
      out[4288] = fma(0.04, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4512] = fma(0.5, q, out[4512]);
      out[4128] = fma(0.25, q, out[4128]);
      out[4064] = fma(0.375, q, out[4064]);
      out[4224] = fma(-1.0, q, out[4224]);
    }
    if (mask[144]) {
      const double q = scale * ws[49152];
      out[3136] = out[3136] - q;
      out[4160] = out[4160] - q;
      out[4128] = fma(1.24, q, out[4128]);
      out[4064] = fma(0.66, q, out[4064]);
      out[4576] = fma(0.1, q, out[4576]);
      out[4672] = fma(0.1, q, out[4672]);
      out[4480] = fma(0.1, q, out[4480]);
      out[4224] = fma(0.1, q, out[4224]);
    }
    if (mask[145]) {
      const double q = scale * ws[49184];
      out[3136] = out[3136] - q;
      out[4736] = out[4736] - q;
      out[4128] = fma(1.3, q, out[4128]);
      out[4064] = fma(0.7, q, out[4064]);
      out[4576] = fma(1.0, q, out[4576]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[146]) {
      const double q = scale * ws[49216];
      out[3136] = out[3136] - q;
      out[4320] = out[4320] - q;
      out[4128] = fma(0.732, q, out[4128]);
      out[4064] = fma(0.442, q, out[4064]);
      out[4512] = fma(0.128, q, out[4512]);
      out[4480] = fma(0.245, q, out[4480]);
      out[4736] = fma(0.5, q, out[4736]);
      out[4576] = fma(0.3, q, out[4576]);
      out[4672] = fma(0.3, q, out[4672]);
      out[4256] = fma(0.24, q, out[4256]);
      out[4000] = fma(0.06, q, out[4000]);
      out[4224] = fma(0.29, q, out[4224]);
      out[3904] = fma(0.08, q, out[3904]);
      out[3456] = fma(0.08, q, out[3456]);
    }
    if (mask[147]) {
      const double q = scale * ws[49248];
      out[3136] = out[3136] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.5, q, out[4608]);
      out[3648] = fma(0.5, q, out[3648]);
      out[4352] = fma(0.48, q, out[4352]);
      out[4576] = fma(0.48, q, out[4576]);
      out[4288] = fma(0.04, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4128] = fma(0.5, q, out[4128]);
      out[4064] = fma(0.625, q, out[4064]);
      out[4224] = fma(1.0, q, out[4224]);
    }
    if (mask[148]) {
      const double q = scale * ws[49280];
      out[2528] = out[2528] - q;
      out[4736] = out[4736] - q;
      out[3424] = fma(1.0, q, out[3424]);
      out[4672] = fma(1.0, q, out[4672]);
      out[992] = fma(1.0, q, out[992]);
    }
    if (mask[149]) {
      const double q = scale * ws[49312];
      out[2528] = out[2528] - q;
      out[4160] = out[4160] - q;
      out[3872] = fma(0.75, q, out[3872]);
      out[4512] = fma(0.5, q, out[4512]);
      out[4352] = fma(0.25, q, out[4352]);
      out[4672] = fma(0.25, q, out[4672]);
      out[4704] = fma(0.25, q, out[4704]);
      out[4096] = fma(0.25, q, out[4096]);
      out[4224] = fma(0.25, q, out[4224]);
    }
    if (mask[150]) {
      const double q = scale * ws[49344];
      out[3424] = out[3424] - q;
      out[4384] = out[4384] - q;
      out[1632] = fma(0.1, q, out[1632]);
      out[4608] = fma(0.9, q, out[4608]);
      out[4512] = fma(0.673, q, out[4512]);
      out[3872] = fma(0.9, q, out[3872]);
      out[4704] = fma(0.818, q, out[4704]);
      out[4576] = fma(0.082, q, out[4576]);
      out[4672] = fma(0.082, q, out[4672]);
    }
    if (mask[151]) {
      const double q = scale * ws[49376];
      out[3424] = out[3424] - q;
      out[4704] = out[4704] - q;
      out[1664] = fma(0.88, q, out[1664]);
      out[4736] = fma(0.12, q, out[4736]);
      out[4704] = fma(0.12, q, out[4704]);
      out[4512] = fma(0.12, q, out[4512]);
      out[3872] = fma(0.12, q, out[3872]);
    }
    if (mask[152]) {
      const double q = scale * ws[49408];
      out[3424] = out[3424] - q;
      out[4448] = out[4448] - q;
      out[4512] = fma(0.598, q, out[4512]);
      out[3872] = fma(1.0, q, out[3872]);
      out[4704] = fma(0.728, q, out[4704]);
      out[4576] = fma(0.072, q, out[4576]);
      out[4416] = fma(0.8, q, out[4416]);
      out[3904] = fma(0.2, q, out[3904]);
      out[4672] = fma(0.872, q, out[4672]);
    }
    if (mask[153]) {
      const double q = scale * ws[49440];
      out[3424] = out[3424] - q;
      out[4672] = out[4672] - q;
      out[4512] = fma(0.598, q, out[4512]);
      out[3872] = fma(1.0, q, out[3872]);
      out[4704] = fma(0.728, q, out[4704]);
      out[4576] = fma(0.072, q, out[4576]);
      out[4672] = fma(1.072, q, out[4672]);
    }
    if (mask[154]) {
      const double q = scale * ws[49472];
      out[3424] = out[3424] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[1024] = fma(1.0, q, out[1024]);
    }
}
__device__ __noinline__ void ddm_src_1_2(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[155]) {
      const double q = scale * ws[49504];
      out[2528] = out[2528] - q;
      out[4320] = out[4320] - q;
      out[4512] = fma(0.6, q, out[4512]);
      out[3872] = fma(0.65, q, out[3872]);
      out[4064] = fma(0.15, q, out[4064]);
      out[4096] = fma(0.2, q, out[4096]);
      out[4224] = fma(0.35, q, out[4224]);
      out[4736] = fma(0.266, q, out[4736]);
      out[4352] = fma(0.2, q, out[4352]);
      out[4672] = fma(0.2, q, out[4672]);
      out[4704] = fma(0.066, q, out[4704]);
      out[4480] = fma(0.066, q, out[4480]);
    }
    if (mask[156]) {
      const double q = scale * ws[49536];
      out[2528] = out[2528] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.35, q, out[4608]);
      out[4032] = fma(0.65, q, out[4032]);
      out[4576] = fma(0.64, q, out[4576]);
      out[4352] = fma(0.33, q, out[4352]);
      out[4288] = fma(0.03, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4512] = fma(0.35, q, out[4512]);
      out[3872] = fma(0.35, q, out[3872]);
      out[992] = fma(1.0, q, out[992]);
    }
    if (mask[157]) {
      const double q = scale * ws[49568];
      out[3872] = out[3872] - q;
      out[4736] = out[4736] - q;
      out[4288] = fma(0.022, q, out[4288]);
      out[4352] = fma(0.521, q, out[4352]);
      out[4000] = fma(0.115, q, out[4000]);
      out[4416] = fma(0.115, q, out[4416]);
      out[3840] = fma(0.269, q, out[3840]);
      out[4448] = fma(0.269, q, out[4448]);
      out[3744] = fma(0.457, q, out[3744]);
      out[4224] = fma(0.117, q, out[4224]);
      out[3392] = fma(0.137, q, out[3392]);
      out[4480] = fma(0.137, q, out[4480]);
      out[4704] = fma(0.137, q, out[4704]);
      out[4672] = fma(0.658, q, out[4672]);
    }
    if (mask[158]) {
      const double q = scale * ws[49600];
      out[3872] = out[3872] - q;
      out[4320] = out[4320] - q;
      out[4128] = fma(0.04, q, out[4128]);
      out[4512] = fma(0.231, q, out[4512]);
      out[4000] = fma(0.531, q, out[4000]);
      out[4256] = fma(0.17, q, out[4256]);
      out[3392] = fma(0.17, q, out[3392]);
      out[4480] = fma(0.543, q, out[4480]);
      out[4736] = fma(0.461, q, out[4736]);
      out[3776] = fma(0.15, q, out[3776]);
      out[4704] = fma(0.398, q, out[4704]);
      out[4448] = fma(0.143, q, out[4448]);
    }
    if (mask[159]) {
      const double q = scale * ws[49632];
      out[3872] = out[3872] - q;
      out[4640] = out[4640] - q;
      out[4192] = fma(0.717, q, out[4192]);
      out[4032] = fma(0.142, q, out[4032]);
      out[4608] = fma(0.142, q, out[4608]);
      out[4352] = fma(0.142, q, out[4352]);
      out[4576] = fma(0.142, q, out[4576]);
      out[3840] = fma(0.113, q, out[3840]);
      out[4000] = fma(0.113, q, out[4000]);
      out[4224] = fma(0.717, q, out[4224]);
      out[4096] = fma(0.717, q, out[4096]);
      out[4672] = fma(0.284, q, out[4672]);
    }
    if (mask[161]) {
      const double q = scale * ws[49696];
      out[1664] = out[1664] - q;
      out[4736] = out[4736] - q;
      out[1056] = fma(0.904, q, out[1056]);
      out[4736] = fma(0.933, q, out[4736]);
      out[3424] = fma(0.067, q, out[3424]);
      out[4672] = fma(0.067, q, out[4672]);
      out[3136] = fma(0.029, q, out[3136]);
      out[4064] = fma(0.029, q, out[4064]);
    }
    if (mask[163]) {
      const double q = scale * ws[49760];
      out[1024] = out[1024] - q;
      out[4640] = out[4640] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[3872] = fma(1.0, q, out[3872]);
    }
    if (mask[164]) {
      const double q = scale * ws[49792];
      out[1056] = out[1056] - q;
      out[4736] = out[4736] - q;
      out[3296] = fma(1.0, q, out[3296]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[165]) {
      const double q = scale * ws[49824];
      out[3296] = out[3296] - q;
      out[4704] = out[4704] - q;
      out[3840] = fma(0.275, q, out[3840]);
      out[4256] = fma(0.275, q, out[4256]);
      out[4000] = fma(0.275, q, out[4000]);
      out[4736] = fma(1.125, q, out[4736]);
      out[4704] = fma(0.825, q, out[4704]);
      out[4512] = fma(0.375, q, out[4512]);
      out[3776] = fma(0.074, q, out[3776]);
      out[4480] = fma(0.251, q, out[4480]);
      out[4224] = fma(2.175, q, out[4224]);
    }
    if (mask[166]) {
      const double q = scale * ws[49856];
      out[3296] = out[3296] - q;
      out[4384] = out[4384] - q;
      out[3840] = fma(0.275, q, out[3840]);
      out[4256] = fma(0.275, q, out[4256]);
      out[4000] = fma(0.275, q, out[4000]);
      out[4736] = fma(0.125, q, out[4736]);
      out[4704] = fma(0.825, q, out[4704]);
      out[4512] = fma(0.375, q, out[4512]);
      out[4608] = fma(1.0, q, out[4608]);
      out[4480] = fma(0.251, q, out[4480]);
      out[4224] = fma(2.175, q, out[4224]);
    }
    if (mask[167]) {
      const double q = scale * ws[49888];
      out[3296] = out[3296] - q;
      out[4448] = out[4448] - q;
      out[3840] = fma(0.22, q, out[3840]);
      out[4256] = fma(0.22, q, out[4256]);
      out[4000] = fma(0.22, q, out[4000]);
      out[4736] = fma(0.1, q, out[4736]);
      out[4704] = fma(0.66, q, out[4704]);
      out[4512] = fma(0.3, q, out[4512]);
      out[4480] = fma(0.2, q, out[4480]);
      out[4224] = fma(1.74, q, out[4224]);
      out[4416] = fma(0.8, q, out[4416]);
      out[3904] = fma(0.2, q, out[3904]);
      out[4672] = fma(0.8, q, out[4672]);
    }
    if (mask[168]) {
      const double q = scale * ws[49920];
      out[3296] = out[3296] - q;
      out[4672] = out[4672] - q;
      out[3840] = fma(0.275, q, out[3840]);
      out[4256] = fma(0.275, q, out[4256]);
      out[4000] = fma(0.275, q, out[4000]);
      out[4736] = fma(0.125, q, out[4736]);
      out[4704] = fma(0.825, q, out[4704]);
      out[4512] = fma(0.375, q, out[4512]);
      out[4480] = fma(0.251, q, out[4480]);
      out[4224] = fma(2.175, q, out[4224]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[169]) {
      const double q = scale * ws[49952];
      out[1632] = out[1632] - q;
      out[4736] = out[4736] - q;
      out[4352] = fma(0.63, q, out[4352]);
      out[4576] = fma(0.37, q, out[4576]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4608] = fma(0.444, q, out[4608]);
      out[4640] = fma(0.185, q, out[4640]);
      out[1632] = fma(0.104, q, out[1632]);
      out[4512] = fma(0.592, q, out[4512]);
      out[3840] = fma(0.331, q, out[3840]);
      out[3776] = fma(0.185, q, out[3776]);
      out[4224] = fma(2.7, q, out[4224]);
      out[3552] = fma(0.098, q, out[3552]);
      out[4064] = fma(0.078, q, out[4064]);
      out[4032] = fma(0.266, q, out[4032]);
    }
    if (mask[170]) {
      const double q = scale * ws[49984];
      out[2048] = out[2048] - q;
      out[4160] = out[4160] - q;
      out[4064] = fma(0.15, q, out[4064]);
      out[4224] = fma(5.12, q, out[4224]);
      out[2080] = fma(1.0, q, out[2080]);
    }
    if (mask[171]) {
      const double q = scale * ws[50016];
      out[2048] = out[2048] - q;
      out[4736] = out[4736] - q;
      out[4576] = fma(0.75, q, out[4576]);
      out[4352] = fma(0.5, q, out[4352]);
      out[4288] = fma(0.25, q, out[4288]);
      out[4672] = fma(1.5, q, out[4672]);
      out[4512] = fma(0.28, q, out[4512]);
      out[4224] = fma(1.66, q, out[4224]);
      out[4064] = fma(0.47, q, out[4064]);
      out[2080] = fma(1.0, q, out[2080]);
    }
    if (mask[172]) {
      const double q = scale * ws[50048];
      out[2048] = out[2048] - q;
      out[4320] = out[4320] - q;
      out[4736] = fma(0.57, q, out[4736]);
      out[4576] = fma(0.07, q, out[4576]);
      out[4352] = fma(0.69, q, out[4352]);
      out[4288] = fma(0.18, q, out[4288]);
      out[4672] = fma(0.94, q, out[4672]);
      out[4512] = fma(0.24, q, out[4512]);
      out[4480] = fma(0.001, q, out[4480]);
      out[4224] = fma(7.0, q, out[4224]);
      out[4064] = fma(0.21, q, out[4064]);
      out[4096] = fma(0.39, q, out[4096]);
      out[2080] = fma(1.0, q, out[2080]);
    }
    if (mask[173]) {
      const double q = scale * ws[50080];
      out[2048] = out[2048] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.47, q, out[4608]);
      out[4576] = fma(0.28, q, out[4576]);
      out[4352] = fma(0.75, q, out[4352]);
      out[4288] = fma(0.25, q, out[4288]);
      out[4672] = fma(1.28, q, out[4672]);
      out[4064] = fma(0.47, q, out[4064]);
      out[4032] = fma(0.53, q, out[4032]);
      out[2848] = fma(1.0, q, out[2848]);
    }
    if (mask[174]) {
      const double q = scale * ws[50112];
      out[2112] = out[2112] - q;
      out[4160] = out[4160] - q;
      out[4064] = fma(0.15, q, out[4064]);
      out[4224] = fma(5.12, q, out[4224]);
      out[2080] = fma(1.0, q, out[2080]);
    }
    if (mask[175]) {
      const double q = scale * ws[50144];
      out[2112] = out[2112] - q;
      out[4736] = out[4736] - q;
      out[4576] = fma(0.75, q, out[4576]);
      out[4352] = fma(0.5, q, out[4352]);
      out[4288] = fma(0.25, q, out[4288]);
      out[4672] = fma(1.5, q, out[4672]);
      out[4512] = fma(0.28, q, out[4512]);
      out[4224] = fma(1.66, q, out[4224]);
      out[4064] = fma(0.47, q, out[4064]);
      out[2080] = fma(1.0, q, out[2080]);
    }
    if (mask[176]) {
      const double q = scale * ws[50176];
      out[2112] = out[2112] - q;
      out[4320] = out[4320] - q;
      out[4736] = fma(0.57, q, out[4736]);
      out[4576] = fma(0.07, q, out[4576]);
      out[4352] = fma(0.69, q, out[4352]);
      out[4288] = fma(0.18, q, out[4288]);
      out[4672] = fma(0.94, q, out[4672]);
      out[4512] = fma(0.24, q, out[4512]);
      out[4480] = fma(0.001, q, out[4480]);
      out[4224] = fma(7.0, q, out[4224]);
      out[4064] = fma(0.21, q, out[4064]);
      out[4096] = fma(0.39, q, out[4096]);
      out[2080] = fma(1.0, q, out[2080]);
    }
    if (mask[177]) {
      const double q = scale * ws[50208];
      out[2112] = out[2112] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.47, q, out[4608]);
      out[4576] = fma(0.28, q, out[4576]);
      out[4352] = fma(0.75, q, out[4352]);
      out[4288] = fma(0.25, q, out[4288]);
      out[4672] = fma(1.28, q, out[4672]);
      out[4064] = fma(0.47, q, out[4064]);
      out[4032] = fma(0.53, q, out[4032]);
    }
    if (mask[178]) {
      const double q = scale * ws[50240];
      out[384] = out[384] - q;
      out[4736] = out[4736] - q;
      out[3616] = fma(0.53, q, out[3616]);
      out[3104] = fma(0.352, q, out[3104]);
      out[4672] = fma(0.352, q, out[4672]);
      out[3936] = fma(0.118, q, out[3936]);
      out[4736] = fma(0.118, q, out[4736]);
      out[4704] = fma(0.53, q, out[4704]);
      out[2144] = fma(1.0, q, out[2144]);
    }
    if (mask[179]) {
      const double q = scale * ws[50272];
      out[3104] = out[3104] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(0.918, q, out[4608]);
      out[4032] = fma(0.082, q, out[4032]);
      out[4256] = fma(0.918, q, out[4256]);
      out[3936] = fma(0.918, q, out[3936]);
      out[4704] = fma(0.918, q, out[4704]);
    }
    if (mask[180]) {
      const double q = scale * ws[50304];
      out[3104] = out[3104] - q;
      out[4448] = out[4448] - q;
      out[4256] = fma(1.0, q, out[4256]);
      out[3936] = fma(1.0, q, out[3936]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[181]) {
      const double q = scale * ws[50336];
      out[3104] = out[3104] - q;
      out[4704] = out[4704] - q;
    }
    if (mask[182]) {
      const double q = scale * ws[50368];
      out[3104] = out[3104] - q;
      out[4672] = out[4672] - q;
      out[4256] = fma(1.0, q, out[4256]);
      out[3936] = fma(1.0, q, out[3936]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[183]) {
      const double q = scale * ws[50400];
      out[1088] = out[1088] - q;
      out[4736] = out[4736] - q;
      out[3616] = fma(0.18, q, out[3616]);
      out[3488] = fma(0.65, q, out[3488]);
      out[4672] = fma(0.72, q, out[4672]);
      out[3936] = fma(0.1, q, out[3936]);
      out[4736] = fma(0.1, q, out[4736]);
      out[4576] = fma(0.07, q, out[4576]);
      out[4704] = fma(0.18, q, out[4704]);
      out[2944] = fma(1.0, q, out[2944]);
    }
    if (mask[184]) {
      const double q = scale * ws[50432];
      out[3488] = out[3488] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(0.86, q, out[4608]);
      out[4032] = fma(0.14, q, out[4032]);
      out[4256] = fma(0.417, q, out[4256]);
      out[4000] = fma(0.443, q, out[4000]);
      out[3936] = fma(0.66, q, out[3936]);
      out[3808] = fma(0.2, q, out[3808]);
      out[4704] = fma(0.86, q, out[4704]);
    }
    if (mask[185]) {
      const double q = scale * ws[50464];
      out[3488] = out[3488] - q;
      out[4448] = out[4448] - q;
      out[4256] = fma(0.48, q, out[4256]);
      out[4000] = fma(0.52, q, out[4000]);
      out[3936] = fma(0.77, q, out[3936]);
      out[3808] = fma(0.23, q, out[3808]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[186]) {
      const double q = scale * ws[50496];
      out[3488] = out[3488] - q;
      out[4704] = out[4704] - q;
    }
    if (mask[187]) {
      const double q = scale * ws[50528];
      out[3488] = out[3488] - q;
      out[4672] = out[4672] - q;
      out[4256] = fma(0.48, q, out[4256]);
      out[4000] = fma(0.52, q, out[4000]);
      out[3936] = fma(0.77, q, out[3936]);
      out[3808] = fma(0.23, q, out[3808]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[188]) {
      const double q = scale * ws[50560];
      out[1120] = out[1120] - q;
      out[4736] = out[4736] - q;
      out[3616] = fma(0.155, q, out[3616]);
      out[3584] = fma(0.544, q, out[3584]);
      out[4672] = fma(0.602, q, out[4672]);
      out[3808] = fma(0.244, q, out[3808]);
      out[4736] = fma(0.244, q, out[4736]);
      out[4576] = fma(0.058, q, out[4576]);
      out[4704] = fma(0.155, q, out[4704]);
      out[2496] = fma(1.0, q, out[2496]);
    }
    if (mask[189]) {
      const double q = scale * ws[50592];
      out[1152] = out[1152] - q;
      out[4736] = out[4736] - q;
      out[3616] = fma(0.155, q, out[3616]);
      out[3584] = fma(0.544, q, out[3584]);
      out[4672] = fma(0.602, q, out[4672]);
      out[3808] = fma(0.244, q, out[3808]);
      out[4736] = fma(0.244, q, out[4736]);
      out[4576] = fma(0.058, q, out[4576]);
      out[4704] = fma(0.155, q, out[4704]);
      out[2560] = fma(1.0, q, out[2560]);
    }
    if (mask[190]) {
      const double q = scale * ws[50624];
      out[3584] = out[3584] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(0.86, q, out[4608]);
      out[4032] = fma(0.14, q, out[4032]);
      out[4256] = fma(0.221, q, out[4256]);
      out[4000] = fma(0.675, q, out[4000]);
      out[3936] = fma(0.3, q, out[3936]);
      out[3808] = fma(0.56, q, out[3808]);
      out[4704] = fma(0.86, q, out[4704]);
    }
    if (mask[191]) {
      const double q = scale * ws[50656];
      out[3584] = out[3584] - q;
      out[4704] = out[4704] - q;
    }
    if (mask[192]) {
      const double q = scale * ws[50688];
      out[3584] = out[3584] - q;
      out[4448] = out[4448] - q;
      out[4256] = fma(0.26, q, out[4256]);
      out[4000] = fma(0.77, q, out[4000]);
      out[3936] = fma(0.35, q, out[3936]);
      out[3808] = fma(0.65, q, out[3808]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[193]) {
      const double q = scale * ws[50720];
      out[3584] = out[3584] - q;
      out[4672] = out[4672] - q;
      out[4256] = fma(0.26, q, out[4256]);
      out[4000] = fma(0.77, q, out[4000]);
      out[3936] = fma(0.35, q, out[3936]);
      out[3808] = fma(0.65, q, out[3808]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[194]) {
      const double q = scale * ws[50752];
      out[3616] = out[3616] - q;
      out[4736] = out[4736] - q;
      out[4256] = fma(0.025, q, out[4256]);
      out[3936] = fma(0.025, q, out[3936]);
      out[4704] = fma(1.0, q, out[4704]);
      out[3328] = fma(0.2, q, out[3328]);
      out[1760] = fma(0.732, q, out[1760]);
      out[4288] = fma(0.02, q, out[4288]);
      out[4672] = fma(0.02, q, out[4672]);
    }
    if (mask[195]) {
      const double q = scale * ws[50784];
      out[3616] = out[3616] - q;
      out[4640] = out[4640] - q;
      out[3328] = fma(0.3, q, out[3328]);
      out[4192] = fma(1.0, q, out[4192]);
      out[4352] = fma(0.48, q, out[4352]);
      out[4576] = fma(0.12, q, out[4576]);
      out[4256] = fma(0.24, q, out[4256]);
      out[4000] = fma(0.24, q, out[4000]);
      out[3744] = fma(0.48, q, out[3744]);
      out[4288] = fma(0.1, q, out[4288]);
      out[4672] = fma(0.7, q, out[4672]);
    }
    if (mask[196]) {
      const double q = scale * ws[50816];
      out[3328] = out[3328] - q;
      out[4608] = out[4608] - q;
      out[2176] = fma(1.0, q, out[2176]);
    }
    if (mask[197]) {
      const double q = scale * ws[50848];
      out[3328] = out[3328] - q;
      out[4704] = out[4704] - q;
      out[3616] = fma(1.0, q, out[3616]);
    }
    if (mask[198]) {
      const double q = scale * ws[50880];
      out[2176] = out[2176] - q;
      out[4736] = out[4736] - q;
      out[4032] = fma(1.0, q, out[4032]);
      out[3328] = fma(0.5, q, out[3328]);
    }
    if (mask[199]) {
      const double q = scale * ws[50912];
      out[2176] = out[2176] - q;
      out[4640] = out[4640] - q;
      out[4032] = fma(1.0, q, out[4032]);
      out[3328] = fma(0.5, q, out[3328]);
      out[4192] = fma(1.0, q, out[4192]);
    }
}
__device__ __noinline__ void ddm_src_1_3(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[202]) {
      const double q = scale * ws[51008];
      out[3808] = out[3808] - q;
      out[4736] = out[4736] - q;
      out[4000] = fma(1.0, q, out[4000]);
      out[4256] = fma(0.4, q, out[4256]);
      out[4576] = fma(2.0, q, out[4576]);
      out[4672] = fma(2.0, q, out[4672]);
    }
    if (mask[203]) {
      const double q = scale * ws[51040];
      out[3808] = out[3808] - q;
      out[4320] = out[4320] - q;
      out[4000] = fma(1.2, q, out[4000]);
      out[4736] = fma(0.5, q, out[4736]);
      out[4448] = fma(0.6, q, out[4448]);
      out[4128] = fma(0.1, q, out[4128]);
      out[4480] = fma(0.5, q, out[4480]);
      out[4576] = fma(0.3, q, out[4576]);
      out[4672] = fma(0.3, q, out[4672]);
    }
    if (mask[204]) {
      const double q = scale * ws[51072];
      out[3808] = out[3808] - q;
      out[4640] = out[4640] - q;
      out[4608] = fma(0.5, q, out[4608]);
      out[4032] = fma(0.5, q, out[4032]);
      out[4576] = fma(0.45, q, out[4576]);
      out[4352] = fma(0.45, q, out[4352]);
      out[4288] = fma(0.1, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
      out[3936] = fma(0.25, q, out[3936]);
      out[4000] = fma(0.25, q, out[4000]);
    }
    if (mask[206]) {
      const double q = scale * ws[51136];
      out[3936] = out[3936] - q;
      out[4736] = out[4736] - q;
      out[3744] = fma(0.6, q, out[3744]);
      out[4576] = fma(0.4, q, out[4576]);
      out[4672] = fma(0.4, q, out[4672]);
      out[4256] = fma(0.4, q, out[4256]);
    }
    if (mask[207]) {
      const double q = scale * ws[51168];
      out[3936] = out[3936] - q;
      out[4320] = out[4320] - q;
      out[4256] = fma(1.4, q, out[4256]);
      out[4000] = fma(0.24, q, out[4000]);
      out[4736] = fma(0.5, q, out[4736]);
      out[4448] = fma(0.12, q, out[4448]);
      out[4512] = fma(0.08, q, out[4512]);
      out[4128] = fma(0.02, q, out[4128]);
      out[4480] = fma(1.98, q, out[4480]);
      out[4704] = fma(0.56, q, out[4704]);
    }
    if (mask[208]) {
      const double q = scale * ws[51200];
      out[3936] = out[3936] - q;
      out[4640] = out[4640] - q;
      out[3744] = fma(1.0, q, out[3744]);
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[209]) {
      const double q = scale * ws[51232];
      out[1760] = out[1760] - q;
      out[4736] = out[4736] - q;
      out[4512] = fma(0.14, q, out[4512]);
      out[4704] = fma(0.2, q, out[4704]);
      out[3328] = fma(0.5, q, out[3328]);
    }
    if (mask[210]) {
      const double q = scale * ws[51264];
      out[1760] = out[1760] - q;
      out[4640] = out[4640] - q;
      out[3328] = fma(1.0, q, out[3328]);
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[211]) {
      const double q = scale * ws[51296];
      out[3744] = out[3744] - q;
      out[4384] = out[4384] - q;
      out[4608] = fma(1.0, q, out[4608]);
      out[4256] = fma(0.5, q, out[4256]);
      out[4480] = fma(0.5, q, out[4480]);
      out[4704] = fma(0.8, q, out[4704]);
      out[4096] = fma(0.2, q, out[4096]);
    }
    if (mask[212]) {
      const double q = scale * ws[51328];
      out[3744] = out[3744] - q;
      out[4608] = out[4608] - q;
      out[1792] = fma(1.0, q, out[1792]);
    }
    if (mask[213]) {
      const double q = scale * ws[51360];
      out[1792] = out[1792] - q;
      out[3744] = fma(1.0, q, out[3744]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[214]) {
      const double q = scale * ws[51392];
      out[3744] = out[3744] - q;
      out[4704] = out[4704] - q;
      out[2688] = fma(0.37, q, out[2688]);
      out[3904] = fma(0.13, q, out[3904]);
      out[4320] = fma(0.13, q, out[4320]);
      out[4736] = fma(0.5, q, out[4736]);
      out[4416] = fma(0.5, q, out[4416]);
      out[4672] = fma(0.5, q, out[4672]);
    }
    if (mask[215]) {
      const double q = scale * ws[51424];
      out[3744] = out[3744] - q;
      out[4448] = out[4448] - q;
      out[4416] = fma(1.0, q, out[4416]);
      out[4352] = fma(1.0, q, out[4352]);
      out[4064] = fma(1.0, q, out[4064]);
      out[4672] = fma(2.0, q, out[4672]);
    }
    if (mask[216]) {
      const double q = scale * ws[51456];
      out[3744] = out[3744] - q;
      out[4672] = out[4672] - q;
      out[4576] = fma(0.8, q, out[4576]);
      out[4064] = fma(0.8, q, out[4064]);
      out[4672] = fma(1.8, q, out[4672]);
      out[3904] = fma(0.2, q, out[3904]);
    }
    if (mask[217]) {
      const double q = scale * ws[51488];
      out[1792] = out[1792] - q;
      out[4736] = out[4736] - q;
      out[4608] = fma(0.5, q, out[4608]);
      out[4256] = fma(0.5, q, out[4256]);
      out[4480] = fma(1.0, q, out[4480]);
      out[4032] = fma(0.5, q, out[4032]);
    }
    if (mask[218]) {
      const double q = scale * ws[51520];
      out[1952] = out[1952] - q;
      out[4736] = out[4736] - q;
      out[4128] = fma(1.0, q, out[4128]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[219]) {
      const double q = scale * ws[51552];
      out[416] = out[416] - q;
      out[4736] = out[4736] - q;
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[220]) {
      const double q = scale * ws[51584];
      out[928] = out[928] - q;
      out[4288] = fma(1.0, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[221]) {
      const double q = scale * ws[51616];
      out[928] = out[928] - q;
      out[3392] = fma(0.732, q, out[3392]);
      out[4064] = fma(0.268, q, out[4064]);
      out[4224] = fma(0.268, q, out[4224]);
      out[4576] = fma(1.0, q, out[4576]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[222]) {
      const double q = scale * ws[51648];
      out[1984] = out[1984] - q;
      out[4288] = fma(1.0, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[223]) {
      const double q = scale * ws[51680];
      out[1984] = out[1984] - q;
      out[4064] = fma(0.126, q, out[4064]);
      out[960] = fma(0.874, q, out[960]);
      out[4576] = fma(0.126, q, out[4576]);
      out[4352] = fma(0.874, q, out[4352]);
      out[4672] = fma(1.0, q, out[4672]);
      out[4224] = fma(-0.126, q, out[4224]);
    }
    if (mask[224]) {
      const double q = scale * ws[51712];
      out[4608] = out[4608] - q;
      out[4736] = out[4736] - q;
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[227]) {
      const double q = scale * ws[51808];
      out[4544] = out[4544] - q;
      out[4320] = out[4320] - q;
      out[3520] = fma(1.0, q, out[3520]);
    }
    if (mask[228]) {
      const double q = scale * ws[51840];
      out[3520] = out[3520] - q;
      out[3520] = out[3520] - q;
      out[1184] = fma(0.3, q, out[1184]);
      out[4544] = fma(1.4, q, out[4544]);
    }
    if (mask[229]) {
      const double q = scale * ws[51872];
      out[3520] = out[3520] - q;
      out[4384] = out[4384] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[230]) {
      const double q = scale * ws[51904];
      out[3520] = out[3520] - q;
      out[4704] = out[4704] - q;
      out[1824] = fma(1.0, q, out[1824]);
    }
    if (mask[231]) {
      const double q = scale * ws[51936];
      out[3520] = out[3520] - q;
      out[4416] = out[4416] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[4512] = fma(1.0, q, out[4512]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[232]) {
      const double q = scale * ws[51968];
      out[4736] = out[4736] - q;
      out[3232] = out[3232] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[4480] = fma(1.0, q, out[4480]);
    }
    if (mask[234]) {
      const double q = scale * ws[52032];
      out[4544] = out[4544] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[235]) {
      const double q = scale * ws[52064];
      out[4544] = out[4544] - q;
      out[4224] = out[4224] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[1984] = fma(1.0, q, out[1984]);
    }
    if (mask[236]) {
      const double q = scale * ws[52096];
      out[4544] = out[4544] - q;
      out[896] = out[896] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[3392] = fma(1.0, q, out[3392]);
      out[4576] = fma(0.97, q, out[4576]);
      out[4288] = fma(0.03, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[237]) {
      const double q = scale * ws[52128];
      out[4544] = out[4544] - q;
      out[832] = out[832] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4128] = fma(0.991, q, out[4128]);
      out[4576] = fma(0.991, q, out[4576]);
      out[4288] = fma(0.009, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[238]) {
      const double q = scale * ws[52160];
      out[4544] = out[4544] - q;
      out[2656] = out[2656] - q;
      out[3232] = fma(1.0, q, out[3232]);
      out[4352] = fma(2.0, q, out[4352]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4512] = fma(1.0, q, out[4512]);
    }
    if (mask[239]) {
      const double q = scale * ws[52192];
      out[4544] = out[4544] - q;
      out[3552] = out[3552] - q;
      out[3232] = fma(1.0, q, out[3232]);
      out[4128] = fma(0.33, q, out[4128]);
      out[4064] = fma(0.67, q, out[4064]);
      out[4352] = fma(2.0, q, out[4352]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4224] = fma(-1.0, q, out[4224]);
    }
    if (mask[240]) {
      const double q = scale * ws[52224];
      out[4544] = out[4544] - q;
      out[3136] = out[3136] - q;
      out[3968] = fma(0.3, q, out[3968]);
      out[3232] = fma(0.7, q, out[3232]);
      out[4128] = fma(0.45, q, out[4128]);
      out[4064] = fma(0.55, q, out[4064]);
      out[3552] = fma(0.3, q, out[3552]);
      out[4224] = fma(0.3, q, out[4224]);
      out[4352] = fma(1.7, q, out[4352]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[241]) {
      const double q = scale * ws[52256];
      out[4544] = out[4544] - q;
      out[2528] = out[2528] - q;
      out[3232] = fma(1.0, q, out[3232]);
      out[3872] = fma(1.0, q, out[3872]);
      out[4576] = fma(0.96, q, out[4576]);
      out[4288] = fma(0.04, q, out[4288]);
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[242]) {
      const double q = scale * ws[52288];
      out[4544] = out[4544] - q;
      out[4512] = out[4512] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4480] = fma(1.0, q, out[4480]);
    }
    if (mask[243]) {
      const double q = scale * ws[52320];
      out[4544] = out[4544] - q;
      out[4128] = out[4128] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[244]) {
      const double q = scale * ws[52352];
      out[4544] = out[4544] - q;
      out[4064] = out[4064] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4096] = fma(1.0, q, out[4096]);
    }
    if (mask[245]) {
      const double q = scale * ws[52384];
      out[4544] = out[4544] - q;
      out[2720] = out[2720] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4512] = fma(1.0, q, out[4512]);
    }
    if (mask[246]) {
      const double q = scale * ws[52416];
      out[4544] = out[4544] - q;
      out[864] = out[864] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[4704] = fma(1.0, q, out[4704]);
      out[4128] = fma(1.0, q, out[4128]);
    }
    if (mask[247]) {
      const double q = scale * ws[52448];
      out[3968] = out[3968] - q;
      out[4736] = out[4736] - q;
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[248]) {
      const double q = scale * ws[52480];
      out[4544] = out[4544] - q;
      out[1088] = out[1088] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[3616] = fma(0.18, q, out[3616]);
      out[3488] = fma(0.65, q, out[3488]);
      out[4672] = fma(0.72, q, out[4672]);
      out[3936] = fma(0.1, q, out[3936]);
      out[4736] = fma(0.1, q, out[4736]);
      out[4576] = fma(0.07, q, out[4576]);
      out[4704] = fma(0.18, q, out[4704]);
      out[2944] = fma(1.0, q, out[2944]);
    }
    if (mask[249]) {
      const double q = scale * ws[52512];
      out[4544] = out[4544] - q;
      out[1120] = out[1120] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[3616] = fma(0.155, q, out[3616]);
      out[3584] = fma(0.544, q, out[3584]);
      out[4672] = fma(0.602, q, out[4672]);
      out[3808] = fma(0.244, q, out[3808]);
      out[4736] = fma(0.244, q, out[4736]);
      out[4576] = fma(0.058, q, out[4576]);
      out[4704] = fma(0.155, q, out[4704]);
      out[2496] = fma(1.0, q, out[2496]);
    }
    if (mask[250]) {
      const double q = scale * ws[52544];
      out[4544] = out[4544] - q;
      out[1152] = out[1152] - q;
      out[3968] = fma(1.0, q, out[3968]);
      out[3616] = fma(0.155, q, out[3616]);
      out[3584] = fma(0.544, q, out[3584]);
      out[4672] = fma(0.602, q, out[4672]);
      out[3808] = fma(0.244, q, out[3808]);
      out[4736] = fma(0.244, q, out[4736]);
      out[4576] = fma(0.058, q, out[4576]);
      out[4704] = fma(0.155, q, out[4704]);
      out[2560] = fma(1.0, q, out[2560]);
    }
    if (mask[252]) {
      const double q = scale * ws[52608];
      out[3520] = out[3520] - q;
      out[4608] = out[4608] - q;
      out[1216] = fma(1.0, q, out[1216]);
    }
    if (mask[255]) {
      const double q = scale * ws[52704];
      out[1216] = out[1216] - q;
      out[1824] = fma(1.0, q, out[1824]);
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[256]) {
      const double q = scale * ws[52736];
      out[1216] = out[1216] - q;
      out[1824] = fma(1.0, q, out[1824]);
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[257]) {
      const double q = scale * ws[52768];
      out[2944] = out[2944] - q;
      out[4384] = out[4384] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[3264] = fma(0.016, q, out[3264]);
      out[2624] = fma(0.051, q, out[2624]);
      out[3072] = fma(0.047, q, out[3072]);
    }
    if (mask[258]) {
      const double q = scale * ws[52800];
      out[2944] = out[2944] - q;
      out[4704] = out[4704] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[2240] = fma(0.14, q, out[2240]);
    }
    if (mask[259]) {
      const double q = scale * ws[52832];
      out[2496] = out[2496] - q;
      out[4384] = out[4384] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[3264] = fma(0.015, q, out[3264]);
      out[2624] = fma(0.023, q, out[2624]);
      out[3072] = fma(0.06, q, out[3072]);
    }
    if (mask[260]) {
      const double q = scale * ws[52864];
      out[2496] = out[2496] - q;
      out[4704] = out[4704] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[2240] = fma(0.193, q, out[2240]);
    }
    if (mask[261]) {
      const double q = scale * ws[52896];
      out[2144] = out[2144] - q;
      out[4384] = out[4384] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[3264] = fma(0.034, q, out[3264]);
      out[3072] = fma(0.392, q, out[3072]);
    }
    if (mask[262]) {
      const double q = scale * ws[52928];
      out[2144] = out[2144] - q;
      out[4704] = out[4704] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[2240] = fma(0.146, q, out[2240]);
    }
    if (mask[263]) {
      const double q = scale * ws[52960];
      out[1856] = out[1856] - q;
      out[4320] = out[4320] - q;
      out[4320] = fma(1.0, q, out[4320]);
      out[1888] = fma(1.0, q, out[1888]);
    }
    if (mask[264]) {
      const double q = scale * ws[52992];
      out[1856] = out[1856] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[1888] = fma(1.0, q, out[1888]);
    }
    if (mask[265]) {
      const double q = scale * ws[53024];
      out[1856] = out[1856] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
      out[1888] = fma(1.0, q, out[1888]);
    }
    if (mask[266]) {
      const double q = scale * ws[53056];
      out[2560] = out[2560] - q;
      out[4384] = out[4384] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[3264] = fma(0.028, q, out[3264]);
      out[2624] = fma(0.225, q, out[2624]);
      out[3072] = fma(0.191, q, out[3072]);
    }
    if (mask[267]) {
      const double q = scale * ws[53088];
      out[2560] = out[2560] - q;
      out[4704] = out[4704] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[2240] = fma(0.473, q, out[2240]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
