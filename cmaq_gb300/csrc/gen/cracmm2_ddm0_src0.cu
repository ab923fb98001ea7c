// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void ddm_src_0_0(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[0]) {
      const double q = scale * ws[59328];
      out[5184] = out[5184] - q;
      out[2336] = fma(1.0, q, out[2336]);
    }
    if (mask[1]) {
      const double q = scale * ws[59360];
      out[5184] = out[5184] - q;
      out[576] = fma(1.0, q, out[576]);
    }
    if (mask[2]) {
      const double q = scale * ws[59392];
      out[4000] = out[4000] - q;
      out[6016] = fma(2.0, q, out[6016]);
    }
    if (mask[3]) {
      const double q = scale * ws[59424];
      out[5920] = out[5920] - q;
      out[2336] = fma(1.0, q, out[2336]);
      out[5824] = fma(1.0, q, out[5824]);
    }
    if (mask[4]) {
      const double q = scale * ws[59456];
      out[5952] = out[5952] - q;
      out[5824] = fma(1.0, q, out[5824]);
    }
    if (mask[5]) {
      const double q = scale * ws[59488];
      out[5952] = out[5952] - q;
      out[2336] = fma(1.0, q, out[2336]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[6]) {
      const double q = scale * ws[59520];
      out[1184] = out[1184] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5824] = fma(1.0, q, out[5824]);
    }
    if (mask[7]) {
      const double q = scale * ws[59552];
      out[5024] = out[5024] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[8]) {
      const double q = scale * ws[59584];
      out[1280] = out[1280] - q;
      out[6016] = fma(0.2, q, out[6016]);
      out[5984] = fma(0.8, q, out[5984]);
      out[5920] = fma(0.8, q, out[5920]);
      out[5952] = fma(0.2, q, out[5952]);
    }
    if (mask[9]) {
      const double q = scale * ws[59616];
      out[5856] = out[5856] - q;
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[10]) {
      const double q = scale * ws[59648];
      out[5856] = out[5856] - q;
      out[5984] = fma(2.0, q, out[5984]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[11]) {
      const double q = scale * ws[59680];
      out[5568] = out[5568] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[12]) {
      const double q = scale * ws[59712];
      out[5760] = out[5760] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5632] = fma(1.0, q, out[5632]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[13]) {
      const double q = scale * ws[59744];
      out[4480] = out[4480] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5792] = fma(1.0, q, out[5792]);
    }
    if (mask[14]) {
      const double q = scale * ws[59776];
      out[4480] = out[4480] - q;
      out[5888] = fma(2.0, q, out[5888]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[15]) {
      const double q = scale * ws[59808];
      out[3872] = out[3872] - q;
      out[5984] = fma(1.22, q, out[5984]);
      out[5792] = fma(0.784, q, out[5792]);
      out[5664] = fma(1.22, q, out[5664]);
      out[5856] = fma(0.35, q, out[5856]);
      out[5760] = fma(0.434, q, out[5760]);
      out[5504] = fma(0.216, q, out[5504]);
    }
    if (mask[16]) {
      const double q = scale * ws[59840];
      out[4544] = out[4544] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[3904] = fma(1.0, q, out[3904]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[17]) {
      const double q = scale * ws[59872];
      out[4576] = out[4576] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[3904] = fma(1.0, q, out[3904]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[18]) {
      const double q = scale * ws[59904];
      out[5280] = out[5280] - q;
      out[5888] = fma(0.1, q, out[5888]);
      out[5632] = fma(1.0, q, out[5632]);
      out[5792] = fma(0.9, q, out[5792]);
      out[5664] = fma(0.1, q, out[5664]);
    }
    if (mask[19]) {
      const double q = scale * ws[59936];
      out[5504] = out[5504] - q;
      out[5632] = fma(1.5, q, out[5632]);
      out[5792] = fma(0.5, q, out[5792]);
      out[5664] = fma(0.5, q, out[5664]);
    }
    if (mask[20]) {
      const double q = scale * ws[59968];
      out[5344] = out[5344] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5792] = fma(1.0, q, out[5792]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[21]) {
      const double q = scale * ws[60000];
      out[4128] = out[4128] - q;
      out[6016] = fma(0.34, q, out[6016]);
      out[5984] = fma(0.66, q, out[5984]);
      out[5792] = fma(0.67, q, out[5792]);
      out[4672] = fma(0.33, q, out[4672]);
      out[5216] = fma(0.34, q, out[5216]);
      out[5664] = fma(0.67, q, out[5664]);
      out[5856] = fma(0.67, q, out[5856]);
    }
    if (mask[22]) {
      const double q = scale * ws[60032];
      out[4736] = out[4736] - q;
      out[5888] = fma(0.3, q, out[5888]);
      out[4672] = fma(0.3, q, out[4672]);
      out[5664] = fma(0.7, q, out[5664]);
      out[3872] = fma(0.7, q, out[3872]);
    }
    if (mask[23]) {
      const double q = scale * ws[60064];
      out[5376] = out[5376] - q;
      out[5664] = fma(2.0, q, out[5664]);
    }
    if (mask[24]) {
      const double q = scale * ws[60096];
      out[5376] = out[5376] - q;
      out[5856] = fma(1.0, q, out[5856]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[25]) {
      const double q = scale * ws[60128];
      out[5376] = out[5376] - q;
      out[5984] = fma(2.0, q, out[5984]);
      out[5664] = fma(2.0, q, out[5664]);
    }
    if (mask[26]) {
      const double q = scale * ws[60160];
      out[5248] = out[5248] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5792] = fma(1.0, q, out[5792]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[27]) {
      const double q = scale * ws[60192];
      out[5472] = out[5472] - q;
      out[5984] = fma(1.5, q, out[5984]);
      out[5792] = fma(0.25, q, out[5792]);
      out[5216] = fma(0.2, q, out[5216]);
      out[5664] = fma(1.0, q, out[5664]);
      out[5376] = fma(0.5, q, out[5376]);
      out[5248] = fma(0.5, q, out[5248]);
    }
    if (mask[28]) {
      const double q = scale * ws[60224];
      out[4320] = out[4320] - q;
      out[5984] = fma(1.5, q, out[5984]);
      out[5792] = fma(0.25, q, out[5792]);
      out[5216] = fma(0.2, q, out[5216]);
      out[5664] = fma(1.0, q, out[5664]);
      out[5376] = fma(0.5, q, out[5376]);
      out[5248] = fma(0.5, q, out[5248]);
    }
    if (mask[29]) {
      const double q = scale * ws[60256];
      out[4448] = out[4448] - q;
      out[3232] = fma(1.0, q, out[3232]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[30]) {
      const double q = scale * ws[60288];
      out[2816] = out[2816] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[31]) {
      const double q = scale * ws[60320];
      out[5728] = out[5728] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5760] = fma(1.0, q, out[5760]);
    }
    if (mask[32]) {
      const double q = scale * ws[60352];
      out[4096] = out[4096] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5760] = fma(1.0, q, out[5760]);
    }
    if (mask[33]) {
      const double q = scale * ws[60384];
      out[4608] = out[4608] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5760] = fma(1.0, q, out[5760]);
    }
    if (mask[34]) {
      const double q = scale * ws[60416];
      out[3680] = out[3680] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[5888] = fma(1.0, q, out[5888]);
    }
    if (mask[35]) {
      const double q = scale * ws[60448];
      out[5440] = out[5440] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5760] = fma(0.2, q, out[5760]);
      out[5504] = fma(0.8, q, out[5504]);
    }
    if (mask[36]) {
      const double q = scale * ws[60480];
      out[1088] = out[1088] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[37]) {
      const double q = scale * ws[60512];
      out[1088] = out[1088] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5952] = fma(1.0, q, out[5952]);
    }
    if (mask[38]) {
      const double q = scale * ws[60544];
      out[4384] = out[4384] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5504] = fma(0.67, q, out[5504]);
      out[3872] = fma(0.33, q, out[3872]);
    }
    if (mask[39]) {
      const double q = scale * ws[60576];
      out[1696] = out[1696] - q;
      out[5344] = fma(1.0, q, out[5344]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[40]) {
      const double q = scale * ws[60608];
      out[5184] = out[5184] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[41]) {
      const double q = scale * ws[60640];
      out[5184] = out[5184] - q;
      out[5984] = out[5984] - q;
      out[6016] = fma(1.0, q, out[6016]);
    }
    if (mask[42]) {
      const double q = scale * ws[60672];
      out[5184] = out[5184] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[43]) {
      const double q = scale * ws[60704];
      out[5184] = out[5184] - q;
      out[5920] = out[5920] - q;
      out[5952] = fma(1.0, q, out[5952]);
    }
    if (mask[44]) {
      const double q = scale * ws[60736];
      out[2336] = out[2336] - q;
      out[5184] = fma(1.0, q, out[5184]);
    }
    if (mask[45]) {
      const double q = scale * ws[60768];
      out[2336] = out[2336] - q;
      out[5184] = out[5184] - q;
    }
    if (mask[46]) {
      const double q = scale * ws[60800];
      out[576] = out[576] - q;
      out[2336] = fma(1.0, q, out[2336]);
    }
    if (mask[47]) {
      const double q = scale * ws[60832];
      out[576] = out[576] - q;
      out[2336] = fma(1.0, q, out[2336]);
    }
    if (mask[48]) {
      const double q = scale * ws[60864];
      out[576] = out[576] - q;
      out[6016] = fma(2.0, q, out[6016]);
    }
    if (mask[49]) {
      const double q = scale * ws[60896];
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[50]) {
      const double q = scale * ws[60928];
      out[6016] = out[6016] - q;
      out[5984] = out[5984] - q;
    }
    if (mask[51]) {
      const double q = scale * ws[60960];
      out[5984] = out[5984] - q;
      out[5984] = out[5984] - q;
      out[4000] = fma(1.0, q, out[4000]);
    }
    if (mask[52]) {
      const double q = scale * ws[60992];
      out[5984] = out[5984] - q;
      out[5984] = out[5984] - q;
      out[4000] = fma(1.0, q, out[4000]);
    }
    if (mask[53]) {
      const double q = scale * ws[61024];
      out[4000] = out[4000] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[54]) {
      const double q = scale * ws[61056];
      out[5824] = out[5824] - q;
      out[2336] = out[2336] - q;
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[55]) {
      const double q = scale * ws[61088];
      out[5824] = out[5824] - q;
      out[6016] = out[6016] - q;
      out[1184] = fma(1.0, q, out[1184]);
    }
    if (mask[56]) {
      const double q = scale * ws[61120];
      out[5824] = out[5824] - q;
      out[5984] = out[5984] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[6016] = fma(1.0, q, out[6016]);
    }
    if (mask[57]) {
      const double q = scale * ws[61152];
      out[5824] = out[5824] - q;
      out[5984] = out[5984] - q;
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[58]) {
      const double q = scale * ws[61184];
      out[5824] = out[5824] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(2.0, q, out[5920]);
    }
    if (mask[59]) {
      const double q = scale * ws[61216];
      out[1184] = out[1184] - q;
      out[6016] = out[6016] - q;
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[60]) {
      const double q = scale * ws[61248];
      out[5920] = out[5920] - q;
      out[2336] = out[2336] - q;
      out[5824] = fma(1.0, q, out[5824]);
    }
    if (mask[61]) {
      const double q = scale * ws[61280];
      out[5920] = out[5920] - q;
      out[2336] = out[2336] - q;
      out[5952] = fma(1.0, q, out[5952]);
    }
    if (mask[62]) {
      const double q = scale * ws[61312];
      out[5920] = out[5920] - q;
      out[6016] = out[6016] - q;
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[63]) {
      const double q = scale * ws[61344];
      out[5024] = out[5024] - q;
      out[6016] = out[6016] - q;
      out[5952] = fma(1.0, q, out[5952]);
    }
    if (mask[64]) {
      const double q = scale * ws[61376];
      out[5952] = out[5952] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[65]) {
      const double q = scale * ws[61408];
      out[5952] = out[5952] - q;
      out[5984] = out[5984] - q;
      out[6016] = fma(0.7, q, out[6016]);
      out[5920] = fma(0.7, q, out[5920]);
      out[5024] = fma(0.3, q, out[5024]);
    }
    if (mask[66]) {
      const double q = scale * ws[61440];
      out[5952] = out[5952] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(2.0, q, out[5920]);
    }
    if (mask[67]) {
      const double q = scale * ws[61472];
      out[5952] = out[5952] - q;
      out[5920] = out[5920] - q;
      out[5824] = fma(1.0, q, out[5824]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[68]) {
      const double q = scale * ws[61504];
      out[5952] = out[5952] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(2.0, q, out[5920]);
    }
    if (mask[69]) {
      const double q = scale * ws[61536];
      out[5952] = out[5952] - q;
      out[5920] = out[5920] - q;
      out[1024] = fma(1.0, q, out[1024]);
    }
    if (mask[70]) {
      const double q = scale * ws[61568];
      out[1024] = out[1024] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5952] = fma(1.0, q, out[5952]);
    }
    if (mask[71]) {
      const double q = scale * ws[61600];
      out[1024] = out[1024] - q;
      out[5024] = fma(2.0, q, out[5024]);
    }
    if (mask[72]) {
      const double q = scale * ws[61632];
      out[5920] = out[5920] - q;
      out[5984] = out[5984] - q;
      out[1280] = fma(1.0, q, out[1280]);
    }
    if (mask[73]) {
      const double q = scale * ws[61664];
      out[1280] = out[1280] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[74]) {
      const double q = scale * ws[61696];
      out[1280] = out[1280] - q;
      out[6016] = out[6016] - q;
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[75]) {
      const double q = scale * ws[61728];
      out[160] = out[160] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[192] = fma(1.0, q, out[192]);
      out[224] = fma(1.0, q, out[224]);
    }
    if (mask[76]) {
      const double q = scale * ws[61760];
      out[5664] = out[5664] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[77]) {
      const double q = scale * ws[61792];
      out[6016] = out[6016] - q;
      out[5888] = fma(1.0, q, out[5888]);
    }
}
__device__ __noinline__ void ddm_src_0_1(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[78]) {
      const double q = scale * ws[61824];
      out[1888] = out[1888] - q;
      out[6016] = out[6016] - q;
      out[5632] = fma(1.0, q, out[5632]);
    }
    if (mask[79]) {
      const double q = scale * ws[61856];
      out[2176] = out[2176] - q;
      out[6016] = out[6016] - q;
      out[5408] = fma(1.0, q, out[5408]);
      out[3616] = fma(2.81e-05, q, out[3616]);
    }
    if (mask[80]) {
      const double q = scale * ws[61888];
      out[1120] = out[1120] - q;
      out[6016] = out[6016] - q;
      out[5120] = fma(1.0, q, out[5120]);
      out[3616] = fma(0.00134, q, out[3616]);
    }
    if (mask[81]) {
      const double q = scale * ws[61920];
      out[2240] = out[2240] - q;
      out[6016] = out[6016] - q;
      out[3008] = fma(1.0, q, out[3008]);
    }
    if (mask[82]) {
      const double q = scale * ws[61952];
      out[2752] = out[2752] - q;
      out[6016] = out[6016] - q;
      out[3200] = fma(1.0, q, out[3200]);
    }
    if (mask[83]) {
      const double q = scale * ws[61984];
      out[1152] = out[1152] - q;
      out[6016] = out[6016] - q;
      out[3328] = fma(1.0, q, out[3328]);
    }
    if (mask[84]) {
      const double q = scale * ws[62016];
      out[256] = out[256] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(0.65, q, out[6016]);
      out[5984] = fma(0.35, q, out[5984]);
      out[5664] = fma(0.35, q, out[5664]);
      out[5376] = fma(0.65, q, out[5376]);
      out[4352] = fma(0.35, q, out[4352]);
    }
    if (mask[85]) {
      const double q = scale * ws[62048];
      out[1216] = out[1216] - q;
      out[6016] = out[6016] - q;
      out[3360] = fma(0.47, q, out[3360]);
      out[1248] = fma(0.53, q, out[1248]);
      out[5984] = fma(0.53, q, out[5984]);
    }
    if (mask[86]) {
      const double q = scale * ws[62080];
      out[288] = out[288] - q;
      out[6016] = out[6016] - q;
      out[3296] = fma(0.82, q, out[3296]);
      out[2944] = fma(0.18, q, out[2944]);
      out[5984] = fma(0.18, q, out[5984]);
    }
    if (mask[87]) {
      const double q = scale * ws[62112];
      out[320] = out[320] - q;
      out[6016] = out[6016] - q;
      out[3104] = fma(0.83, q, out[3104]);
      out[2944] = fma(0.17, q, out[2944]);
      out[5984] = fma(0.17, q, out[5984]);
    }
    if (mask[88]) {
      const double q = scale * ws[62144];
      out[352] = out[352] - q;
      out[6016] = out[6016] - q;
      out[3264] = fma(0.82, q, out[3264]);
      out[2944] = fma(0.18, q, out[2944]);
      out[5984] = fma(0.18, q, out[5984]);
    }
    if (mask[89]) {
      const double q = scale * ws[62176];
      out[1312] = out[1312] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.25, q, out[6016]);
      out[5984] = fma(0.25, q, out[5984]);
      out[5888] = fma(0.4, q, out[5888]);
      out[5792] = fma(0.018, q, out[5792]);
      out[4672] = fma(0.1, q, out[4672]);
      out[4000] = fma(0.09, q, out[4000]);
      out[5664] = fma(0.22, q, out[5664]);
      out[5856] = fma(1.0, q, out[5856]);
      out[4128] = fma(0.3, q, out[4128]);
      out[4736] = fma(0.14, q, out[4736]);
      out[4352] = fma(0.28, q, out[4352]);
      out[2752] = fma(0.153, q, out[2752]);
    }
    if (mask[90]) {
      const double q = scale * ws[62208];
      out[1312] = out[1312] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(0.4, q, out[5920]);
      out[2784] = fma(0.045, q, out[2784]);
      out[5856] = fma(0.35, q, out[5856]);
      out[1632] = fma(0.555, q, out[1632]);
      out[4736] = fma(0.26, q, out[4736]);
      out[4128] = fma(0.028, q, out[4128]);
    }
    if (mask[91]) {
      const double q = scale * ws[62240];
      out[1312] = out[1312] - q;
      out[6016] = out[6016] - q;
      out[4288] = fma(1.0, q, out[4288]);
      out[5856] = fma(0.25, q, out[5856]);
      out[4128] = fma(0.03, q, out[4128]);
      out[5248] = fma(0.05, q, out[5248]);
    }
    if (mask[92]) {
      const double q = scale * ws[62272];
      out[4288] = out[4288] - q;
      out[5984] = out[5984] - q;
      out[1344] = fma(1.0, q, out[1344]);
      out[5984] = fma(0.07, q, out[5984]);
      out[6016] = fma(0.5, q, out[6016]);
    }
    if (mask[93]) {
      const double q = scale * ws[62304];
      out[4288] = out[4288] - q;
      out[5824] = out[5824] - q;
      out[2784] = fma(0.13, q, out[2784]);
      out[5856] = fma(0.4, q, out[5856]);
      out[5984] = fma(0.88, q, out[5984]);
      out[5920] = fma(0.87, q, out[5920]);
      out[4128] = fma(0.18, q, out[4128]);
      out[4736] = fma(0.51, q, out[4736]);
    }
    if (mask[94]) {
      const double q = scale * ws[62336];
      out[1344] = out[1344] - q;
      out[6016] = out[6016] - q;
      out[4288] = fma(1.0, q, out[4288]);
    }
    if (mask[95]) {
      const double q = scale * ws[62368];
      out[1344] = out[1344] - q;
      out[6016] = out[6016] - q;
      out[5248] = fma(0.04, q, out[5248]);
      out[5376] = fma(0.02, q, out[5376]);
      out[4736] = fma(0.13, q, out[4736]);
      out[1376] = fma(0.44, q, out[1376]);
      out[5792] = fma(0.11, q, out[5792]);
      out[4128] = fma(0.03, q, out[4128]);
      out[6016] = fma(2.0, q, out[6016]);
      out[5984] = fma(0.34, q, out[5984]);
      out[1664] = fma(0.14, q, out[1664]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[96]) {
      const double q = scale * ws[62400];
      out[1632] = out[1632] - q;
      out[5984] = out[5984] - q;
      out[6016] = fma(0.45, q, out[6016]);
      out[2208] = fma(0.95, q, out[2208]);
      out[1664] = fma(0.02, q, out[1664]);
    }
    if (mask[97]) {
      const double q = scale * ws[62432];
      out[1632] = out[1632] - q;
      out[5824] = out[5824] - q;
      out[4736] = fma(0.15, q, out[4736]);
      out[2208] = fma(0.65, q, out[2208]);
      out[2784] = fma(0.05, q, out[2784]);
      out[5856] = fma(0.2, q, out[5856]);
      out[5920] = fma(1.3, q, out[5920]);
    }
    if (mask[98]) {
      const double q = scale * ws[62464];
      out[2784] = out[2784] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[2208] = fma(0.35, q, out[2208]);
      out[1376] = fma(0.17, q, out[1376]);
      out[5920] = fma(0.65, q, out[5920]);
    }
    if (mask[99]) {
      const double q = scale * ws[62496];
      out[6016] = out[6016] - q;
      out[2208] = out[2208] - q;
      out[5664] = fma(1.0, q, out[5664]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.3, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[100]) {
      const double q = scale * ws[62528];
      out[2784] = out[2784] - q;
      out[5024] = fma(1.0, q, out[5024]);
      out[5056] = fma(1.0, q, out[5056]);
    }
    if (mask[101]) {
      const double q = scale * ws[62560];
      out[1664] = out[1664] - q;
      out[6016] = out[6016] - q;
      out[4128] = fma(0.57, q, out[4128]);
      out[4736] = fma(0.43, q, out[4736]);
    }
    if (mask[102]) {
      const double q = scale * ws[62592];
      out[1408] = out[1408] - q;
      out[6016] = out[6016] - q;
      out[4160] = fma(0.975, q, out[4160]);
      out[3744] = fma(0.025, q, out[3744]);
    }
    if (mask[103]) {
      const double q = scale * ws[62624];
      out[1440] = out[1440] - q;
      out[6016] = out[6016] - q;
      out[4192] = fma(0.945, q, out[4192]);
      out[3936] = fma(0.055, q, out[3936]);
    }
    if (mask[104]) {
      const double q = scale * ws[62656];
      out[4544] = out[4544] - q;
      out[6016] = out[6016] - q;
      out[2560] = fma(0.23, q, out[2560]);
      out[4800] = fma(0.77, q, out[4800]);
    }
    if (mask[105]) {
      const double q = scale * ws[62688];
      out[4576] = out[4576] - q;
      out[6016] = out[6016] - q;
      out[1728] = fma(0.83, q, out[1728]);
      out[4800] = fma(0.17, q, out[4800]);
    }
    if (mask[106]) {
      const double q = scale * ws[62720];
      out[5856] = out[5856] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[107]) {
      const double q = scale * ws[62752];
      out[5568] = out[5568] - q;
      out[6016] = out[6016] - q;
      out[5792] = fma(1.0, q, out[5792]);
    }
    if (mask[108]) {
      const double q = scale * ws[62784];
      out[5760] = out[5760] - q;
      out[6016] = out[6016] - q;
      out[4800] = fma(1.0, q, out[4800]);
    }
    if (mask[109]) {
      const double q = scale * ws[62816];
      out[4480] = out[4480] - q;
      out[6016] = out[6016] - q;
      out[2848] = fma(1.0, q, out[2848]);
    }
    if (mask[110]) {
      const double q = scale * ws[62848];
      out[5280] = out[5280] - q;
      out[6016] = out[6016] - q;
      out[5152] = fma(1.0, q, out[5152]);
    }
    if (mask[111]) {
      const double q = scale * ws[62880];
      out[5504] = out[5504] - q;
      out[6016] = out[6016] - q;
      out[3776] = fma(1.0, q, out[3776]);
    }
    if (mask[112]) {
      const double q = scale * ws[62912];
      out[5344] = out[5344] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5248] = fma(1.0, q, out[5248]);
    }
    if (mask[113]) {
      const double q = scale * ws[62944];
      out[4128] = out[4128] - q;
      out[6016] = out[6016] - q;
      out[4672] = fma(0.57, q, out[4672]);
      out[3520] = fma(0.43, q, out[3520]);
    }
    if (mask[114]) {
      const double q = scale * ws[62976];
      out[4736] = out[4736] - q;
      out[6016] = out[6016] - q;
      out[2880] = fma(1.0, q, out[2880]);
    }
    if (mask[115]) {
      const double q = scale * ws[63008];
      out[3872] = out[3872] - q;
      out[6016] = out[6016] - q;
      out[5792] = fma(0.313, q, out[5792]);
      out[2912] = fma(0.687, q, out[2912]);
    }
    if (mask[116]) {
      const double q = scale * ws[63040];
      out[5376] = out[5376] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(2.0, q, out[5664]);
    }
    if (mask[117]) {
      const double q = scale * ws[63072];
      out[5248] = out[5248] - q;
      out[6016] = out[6016] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5664] = fma(1.0, q, out[5664]);
    }
    if (mask[118]) {
      const double q = scale * ws[63104];
      out[5472] = out[5472] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(0.52, q, out[5984]);
      out[5664] = fma(0.33, q, out[5664]);
      out[5760] = fma(0.4, q, out[5760]);
      out[5504] = fma(0.78, q, out[5504]);
      out[5376] = fma(0.1, q, out[5376]);
      out[5248] = fma(0.01, q, out[5248]);
    }
    if (mask[119]) {
      const double q = scale * ws[63136];
      out[4320] = out[4320] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(0.52, q, out[5984]);
      out[5664] = fma(0.33, q, out[5664]);
      out[5280] = fma(0.13, q, out[5280]);
      out[5376] = fma(0.1, q, out[5376]);
      out[5248] = fma(0.01, q, out[5248]);
      out[5728] = fma(0.78, q, out[5728]);
    }
    if (mask[120]) {
      const double q = scale * ws[63168];
      out[3584] = out[3584] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(0.56, q, out[5984]);
      out[4672] = fma(0.21, q, out[4672]);
      out[5664] = fma(0.11, q, out[5664]);
      out[5376] = fma(0.27, q, out[5376]);
      out[5248] = fma(0.01, q, out[5248]);
      out[5728] = fma(0.79, q, out[5728]);
    }
    if (mask[121]) {
      const double q = scale * ws[63200];
      out[4448] = out[4448] - q;
      out[6016] = out[6016] - q;
      out[2592] = fma(1.0, q, out[2592]);
    }
    if (mask[122]) {
      const double q = scale * ws[63232];
      out[1248] = out[1248] - q;
      out[6016] = out[6016] - q;
      out[3616] = fma(0.152, q, out[3616]);
      out[5984] = fma(0.619, q, out[5984]);
      out[3648] = fma(0.17, q, out[3648]);
      out[3232] = fma(0.059, q, out[3232]);
      out[1760] = fma(0.619, q, out[1760]);
    }
    if (mask[123]) {
      const double q = scale * ws[63264];
      out[2944] = out[2944] - q;
      out[6016] = out[6016] - q;
      out[3616] = fma(0.2, q, out[3616]);
      out[5984] = fma(0.584, q, out[5984]);
      out[3648] = fma(0.16, q, out[3648]);
      out[3232] = fma(0.056, q, out[3232]);
      out[1760] = fma(0.584, q, out[1760]);
    }
    if (mask[124]) {
      const double q = scale * ws[63296];
      out[1760] = out[1760] - q;
      out[6016] = out[6016] - q;
      out[3808] = fma(1.0, q, out[3808]);
    }
    if (mask[125]) {
      const double q = scale * ws[63328];
      out[5600] = out[5600] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[126]) {
      const double q = scale * ws[63360];
      out[1472] = out[1472] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5568] = fma(1.0, q, out[5568]);
    }
    if (mask[127]) {
      const double q = scale * ws[63392];
      out[5056] = out[5056] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5760] = fma(0.719, q, out[5760]);
      out[5568] = fma(0.184, q, out[5568]);
    }
    if (mask[128]) {
      const double q = scale * ws[63424];
      out[1504] = out[1504] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5760] = fma(1.0, q, out[5760]);
    }
    if (mask[129]) {
      const double q = scale * ws[63456];
      out[2816] = out[2816] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(0.35, q, out[6016]);
      out[5888] = fma(0.65, q, out[5888]);
      out[5856] = fma(0.35, q, out[5856]);
    }
    if (mask[130]) {
      const double q = scale * ws[63488];
      out[5728] = out[5728] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(0.01, q, out[6016]);
      out[5408] = fma(0.44, q, out[5408]);
      out[5216] = fma(0.07, q, out[5216]);
      out[5760] = fma(0.08, q, out[5760]);
      out[5504] = fma(0.41, q, out[5504]);
    }
    if (mask[131]) {
      const double q = scale * ws[63520];
      out[4096] = out[4096] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(0.01, q, out[6016]);
      out[3904] = fma(0.44, q, out[3904]);
      out[5216] = fma(0.07, q, out[5216]);
      out[5760] = fma(0.08, q, out[5760]);
      out[5504] = fma(0.41, q, out[5504]);
    }
    if (mask[132]) {
      const double q = scale * ws[63552];
      out[4608] = out[4608] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(0.01, q, out[6016]);
      out[3904] = fma(0.44, q, out[3904]);
      out[5216] = fma(0.07, q, out[5216]);
      out[5760] = fma(0.08, q, out[5760]);
      out[5504] = fma(0.41, q, out[5504]);
    }
    if (mask[133]) {
      const double q = scale * ws[63584];
      out[1792] = out[1792] - q;
      out[6016] = out[6016] - q;
      out[4672] = fma(1.0, q, out[4672]);
    }
    if (mask[134]) {
      const double q = scale * ws[63616];
      out[4352] = out[4352] - q;
      out[6016] = out[6016] - q;
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[135]) {
      const double q = scale * ws[63648];
      out[5696] = out[5696] - q;
      out[6016] = out[6016] - q;
      out[5888] = fma(0.64, q, out[5888]);
      out[2976] = fma(0.36, q, out[2976]);
    }
    if (mask[136]) {
      const double q = scale * ws[63680];
      out[3680] = out[3680] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(0.35, q, out[6016]);
      out[5792] = fma(0.65, q, out[5792]);
      out[5216] = fma(0.35, q, out[5216]);
      out[5856] = fma(0.35, q, out[5856]);
    }
    if (mask[137]) {
      const double q = scale * ws[63712];
      out[1088] = out[1088] - q;
      out[6016] = out[6016] - q;
      out[5216] = fma(1.0, q, out[5216]);
      out[5952] = fma(1.0, q, out[5952]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[138]) {
      const double q = scale * ws[63744];
      out[1536] = out[1536] - q;
      out[6016] = out[6016] - q;
      out[5216] = fma(1.0, q, out[5216]);
      out[5952] = fma(1.0, q, out[5952]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[139]) {
      const double q = scale * ws[63776];
      out[1824] = out[1824] - q;
      out[6016] = out[6016] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5344] = fma(1.0, q, out[5344]);
    }
}
__device__ __noinline__ void ddm_src_0_2(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[140]) {
      const double q = scale * ws[63808];
      out[5440] = out[5440] - q;
      out[6016] = out[6016] - q;
      out[5408] = fma(1.0, q, out[5408]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[141]) {
      const double q = scale * ws[63840];
      out[4384] = out[4384] - q;
      out[6016] = out[6016] - q;
      out[1696] = fma(0.33, q, out[1696]);
      out[5920] = fma(0.67, q, out[5920]);
      out[4544] = fma(0.27, q, out[4544]);
      out[5504] = fma(0.38, q, out[5504]);
      out[5856] = fma(0.21, q, out[5856]);
      out[5760] = fma(0.02, q, out[5760]);
    }
    if (mask[142]) {
      const double q = scale * ws[63872];
      out[1696] = out[1696] - q;
      out[6016] = out[6016] - q;
      out[5344] = fma(1.0, q, out[5344]);
      out[5952] = fma(1.0, q, out[5952]);
    }
    if (mask[143]) {
      const double q = scale * ws[63904];
      out[2240] = out[2240] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.08, q, out[6016]);
      out[5984] = fma(0.15, q, out[5984]);
      out[5664] = fma(0.43, q, out[5664]);
      out[5856] = fma(1.0, q, out[5856]);
      out[4352] = fma(0.37, q, out[4352]);
    }
    if (mask[144]) {
      const double q = scale * ws[63936];
      out[2752] = out[2752] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.22, q, out[6016]);
      out[5984] = fma(0.32, q, out[5984]);
      out[5888] = fma(0.08, q, out[5888]);
      out[5632] = fma(0.06, q, out[5632]);
      out[5408] = fma(0.04, q, out[5408]);
      out[5120] = fma(0.02, q, out[5120]);
      out[4000] = fma(0.068, q, out[4000]);
      out[5664] = fma(0.43, q, out[5664]);
      out[1888] = fma(0.02, q, out[1888]);
      out[2176] = fma(0.015, q, out[2176]);
      out[1120] = fma(0.006, q, out[1120]);
      out[1216] = fma(0.032, q, out[1216]);
      out[5856] = fma(0.56, q, out[5856]);
      out[5568] = fma(0.01, q, out[5568]);
      out[5760] = fma(0.44, q, out[5760]);
      out[4480] = fma(0.03, q, out[4480]);
      out[4448] = fma(0.02, q, out[4448]);
      out[5280] = fma(0.06, q, out[5280]);
      out[5344] = fma(0.01, q, out[5344]);
      out[4352] = fma(0.03, q, out[4352]);
      out[5696] = fma(0.06, q, out[5696]);
    }
    if (mask[145]) {
      const double q = scale * ws[63968];
      out[1152] = out[1152] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.46, q, out[6016]);
      out[5984] = fma(0.07, q, out[5984]);
      out[5888] = fma(0.32, q, out[5888]);
      out[5632] = fma(0.07, q, out[5632]);
      out[5408] = fma(0.04, q, out[5408]);
      out[5792] = fma(0.09, q, out[5792]);
      out[5664] = fma(0.37, q, out[5664]);
      out[4000] = fma(0.026, q, out[4000]);
      out[1888] = fma(0.01, q, out[1888]);
      out[2176] = fma(0.01, q, out[2176]);
      out[5856] = fma(0.09, q, out[5856]);
      out[5568] = fma(0.457, q, out[5568]);
      out[5760] = fma(0.73, q, out[5760]);
      out[4480] = fma(0.11, q, out[4480]);
      out[5504] = fma(0.017, q, out[5504]);
      out[5344] = fma(0.044, q, out[5344]);
      out[5696] = fma(0.017, q, out[5696]);
    }
    if (mask[146]) {
      const double q = scale * ws[64000];
      out[1408] = out[1408] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.6055, q, out[6016]);
      out[2560] = fma(0.2145, q, out[2560]);
      out[4000] = fma(0.255, q, out[4000]);
      out[4544] = fma(0.2535, q, out[4544]);
      out[5696] = fma(0.0065, q, out[5696]);
      out[5984] = fma(0.1105, q, out[5984]);
      out[5664] = fma(0.1105, q, out[5664]);
      out[5856] = fma(0.459, q, out[5856]);
      out[4800] = fma(0.2805, q, out[4800]);
      out[5504] = fma(0.1785, q, out[5504]);
      out[2176] = fma(0.0665, q, out[2176]);
      out[2816] = fma(0.0385, q, out[2816]);
      out[4352] = fma(0.028, q, out[4352]);
    }
    if (mask[147]) {
      const double q = scale * ws[64032];
      out[1440] = out[1440] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.66, q, out[6016]);
      out[4576] = fma(0.66, q, out[4576]);
      out[5792] = fma(0.33, q, out[5792]);
      out[5856] = fma(0.33, q, out[5856]);
      out[4800] = fma(0.33, q, out[4800]);
      out[4000] = fma(0.33, q, out[4000]);
      out[5696] = fma(0.01, q, out[5696]);
    }
    if (mask[148]) {
      const double q = scale * ws[64064];
      out[4576] = out[4576] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.09, q, out[6016]);
      out[5760] = fma(1.0, q, out[5760]);
      out[5856] = fma(0.62, q, out[5856]);
      out[2816] = fma(0.23, q, out[2816]);
      out[4000] = fma(0.02, q, out[4000]);
      out[4352] = fma(0.15, q, out[4352]);
    }
    if (mask[149]) {
      const double q = scale * ws[64096];
      out[4384] = out[4384] - q;
      out[5184] = out[5184] - q;
      out[1696] = fma(0.33, q, out[1696]);
      out[5920] = fma(0.67, q, out[5920]);
      out[4544] = fma(0.27, q, out[4544]);
      out[5504] = fma(0.38, q, out[5504]);
      out[5856] = fma(0.21, q, out[5856]);
      out[5760] = fma(0.02, q, out[5760]);
    }
    if (mask[150]) {
      const double q = scale * ws[64128];
      out[4128] = out[4128] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.19, q, out[6016]);
      out[5984] = fma(0.14, q, out[5984]);
      out[5792] = fma(0.1, q, out[5792]);
      out[5664] = fma(0.22, q, out[5664]);
      out[5248] = fma(0.5, q, out[5248]);
      out[4352] = fma(0.45, q, out[4352]);
    }
    if (mask[151]) {
      const double q = scale * ws[64160];
      out[4736] = out[4736] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.16, q, out[6016]);
      out[5984] = fma(0.11, q, out[5984]);
      out[5792] = fma(0.28, q, out[5792]);
      out[5216] = fma(0.01, q, out[5216]);
      out[5664] = fma(0.56, q, out[5664]);
      out[5856] = fma(0.1, q, out[5856]);
      out[5248] = fma(0.54, q, out[5248]);
      out[4352] = fma(0.07, q, out[4352]);
      out[5696] = fma(0.07, q, out[5696]);
      out[5760] = fma(0.1, q, out[5760]);
    }
    if (mask[152]) {
      const double q = scale * ws[64192];
      out[3872] = out[3872] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.1, q, out[6016]);
      out[5984] = fma(0.072, q, out[5984]);
      out[5888] = fma(0.008, q, out[5888]);
      out[5792] = fma(0.002, q, out[5792]);
      out[5216] = fma(0.1, q, out[5216]);
      out[5664] = fma(0.243, q, out[5664]);
      out[5856] = fma(0.08, q, out[5856]);
      out[5568] = fma(0.42, q, out[5568]);
      out[5504] = fma(0.028, q, out[5504]);
      out[5376] = fma(0.491, q, out[5376]);
      out[5248] = fma(0.003, q, out[5248]);
      out[4352] = fma(0.044, q, out[4352]);
    }
    if (mask[153]) {
      const double q = scale * ws[64224];
      out[5472] = out[5472] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.05, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[4800] = fma(0.6, q, out[4800]);
      out[5216] = fma(0.6, q, out[5216]);
      out[5664] = fma(1.5, q, out[5664]);
      out[5856] = fma(0.05, q, out[5856]);
      out[5376] = fma(0.05, q, out[5376]);
      out[5248] = fma(0.08, q, out[5248]);
      out[5728] = fma(0.65, q, out[5728]);
    }
    if (mask[154]) {
      const double q = scale * ws[64256];
      out[4320] = out[4320] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.05, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[4800] = fma(0.6, q, out[4800]);
      out[5216] = fma(0.6, q, out[5216]);
      out[5664] = fma(1.5, q, out[5664]);
      out[5856] = fma(0.05, q, out[5856]);
      out[5376] = fma(0.05, q, out[5376]);
      out[5248] = fma(0.08, q, out[5248]);
      out[5472] = fma(0.7, q, out[5472]);
      out[5728] = fma(0.65, q, out[5728]);
    }
    if (mask[155]) {
      const double q = scale * ws[64288];
      out[3584] = out[3584] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.05, q, out[6016]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(1.5, q, out[5664]);
      out[5376] = fma(0.48, q, out[5376]);
      out[5472] = fma(0.7, q, out[5472]);
      out[4352] = fma(0.25, q, out[4352]);
      out[5696] = fma(0.25, q, out[5696]);
      out[3680] = fma(0.11, q, out[3680]);
    }
    if (mask[156]) {
      const double q = scale * ws[64320];
      out[3808] = out[3808] - q;
      out[5184] = out[5184] - q;
      out[3040] = fma(1.0, q, out[3040]);
    }
    if (mask[157]) {
      const double q = scale * ws[64352];
      out[2240] = out[2240] - q;
      out[5952] = out[5952] - q;
      out[4032] = fma(0.8, q, out[4032]);
      out[4064] = fma(0.2, q, out[4064]);
    }
    if (mask[158]) {
      const double q = scale * ws[64384];
      out[2752] = out[2752] - q;
      out[5952] = out[5952] - q;
      out[4032] = fma(0.43, q, out[4032]);
      out[4064] = fma(0.57, q, out[4064]);
    }
    if (mask[159]) {
      const double q = scale * ws[64416];
      out[1152] = out[1152] - q;
      out[5952] = out[5952] - q;
      out[4032] = fma(0.11, q, out[4032]);
      out[4064] = fma(0.89, q, out[4064]);
    }
    if (mask[160]) {
      const double q = scale * ws[64448];
      out[1408] = out[1408] - q;
      out[5952] = out[5952] - q;
      out[2624] = fma(0.975, q, out[2624]);
      out[3840] = fma(0.025, q, out[3840]);
    }
    if (mask[161]) {
      const double q = scale * ws[64480];
      out[1440] = out[1440] - q;
      out[5952] = out[5952] - q;
      out[2656] = fma(0.945, q, out[2656]);
      out[3712] = fma(0.055, q, out[3712]);
    }
    if (mask[162]) {
      const double q = scale * ws[64512];
      out[4384] = out[4384] - q;
      out[5952] = out[5952] - q;
      out[1696] = fma(0.33, q, out[1696]);
      out[5920] = fma(0.67, q, out[5920]);
      out[4544] = fma(0.27, q, out[4544]);
      out[5504] = fma(0.38, q, out[5504]);
      out[5856] = fma(0.21, q, out[5856]);
      out[5760] = fma(0.02, q, out[5760]);
    }
    if (mask[163]) {
      const double q = scale * ws[64544];
      out[5856] = out[5856] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(1.0, q, out[5664]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[164]) {
      const double q = scale * ws[64576];
      out[5568] = out[5568] - q;
      out[5952] = out[5952] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[165]) {
      const double q = scale * ws[64608];
      out[5760] = out[5760] - q;
      out[5952] = out[5952] - q;
      out[4800] = fma(1.0, q, out[4800]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[166]) {
      const double q = scale * ws[64640];
      out[4128] = out[4128] - q;
      out[5952] = out[5952] - q;
      out[5856] = fma(0.68, q, out[5856]);
      out[4672] = fma(0.32, q, out[4672]);
      out[5216] = fma(0.68, q, out[5216]);
      out[5248] = fma(0.68, q, out[5248]);
      out[5024] = fma(0.32, q, out[5024]);
      out[5920] = fma(0.68, q, out[5920]);
    }
    if (mask[167]) {
      const double q = scale * ws[64672];
      out[3872] = out[3872] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5216] = fma(1.0, q, out[5216]);
      out[5664] = fma(0.668, q, out[5664]);
      out[5856] = fma(0.332, q, out[5856]);
      out[5760] = fma(0.332, q, out[5760]);
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[168]) {
      const double q = scale * ws[64704];
      out[5376] = out[5376] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(2.0, q, out[5664]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[169]) {
      const double q = scale * ws[64736];
      out[5248] = out[5248] - q;
      out[5952] = out[5952] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5664] = fma(1.0, q, out[5664]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[170]) {
      const double q = scale * ws[64768];
      out[1248] = out[1248] - q;
      out[5952] = out[5952] - q;
      out[3616] = fma(0.152, q, out[3616]);
      out[3232] = fma(0.339, q, out[3232]);
      out[3648] = fma(0.85, q, out[3648]);
      out[3072] = fma(0.424, q, out[3072]);
      out[5024] = fma(0.424, q, out[5024]);
    }
    if (mask[171]) {
      const double q = scale * ws[64800];
      out[2944] = out[2944] - q;
      out[5952] = out[5952] - q;
      out[3616] = fma(0.2, q, out[3616]);
      out[3232] = fma(0.32, q, out[3232]);
      out[3648] = fma(0.08, q, out[3648]);
      out[3072] = fma(0.4, q, out[3072]);
      out[5024] = fma(0.4, q, out[5024]);
    }
    if (mask[172]) {
      const double q = scale * ws[64832];
      out[1760] = out[1760] - q;
      out[5952] = out[5952] - q;
      out[3808] = fma(1.0, q, out[3808]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[173]) {
      const double q = scale * ws[64864];
      out[1824] = out[1824] - q;
      out[5952] = out[5952] - q;
      out[4672] = fma(1.0, q, out[4672]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[174]) {
      const double q = scale * ws[64896];
      out[2560] = out[2560] - q;
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[175]) {
      const double q = scale * ws[64928];
      out[1728] = out[1728] - q;
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[176]) {
      const double q = scale * ws[64960];
      out[5792] = out[5792] - q;
      out[5920] = out[5920] - q;
      out[1088] = fma(1.0, q, out[1088]);
    }
    if (mask[177]) {
      const double q = scale * ws[64992];
      out[1088] = out[1088] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[178]) {
      const double q = scale * ws[65024];
      out[4800] = out[4800] - q;
      out[5920] = out[5920] - q;
      out[1536] = fma(1.0, q, out[1536]);
    }
    if (mask[179]) {
      const double q = scale * ws[65056];
      out[1536] = out[1536] - q;
      out[4800] = fma(1.0, q, out[4800]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[180]) {
      const double q = scale * ws[65088];
      out[4672] = out[4672] - q;
      out[5920] = out[5920] - q;
      out[1824] = fma(1.0, q, out[1824]);
    }
    if (mask[181]) {
      const double q = scale * ws[65120];
      out[1824] = out[1824] - q;
      out[4672] = fma(1.0, q, out[4672]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[182]) {
      const double q = scale * ws[65152];
      out[5888] = out[5888] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[183]) {
      const double q = scale * ws[65184];
      out[5632] = out[5632] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5568] = fma(1.0, q, out[5568]);
    }
    if (mask[184]) {
      const double q = scale * ws[65216];
      out[5408] = out[5408] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.66, q, out[5984]);
      out[5888] = fma(0.131, q, out[5888]);
      out[5632] = fma(0.048, q, out[5632]);
      out[5216] = fma(0.089, q, out[5216]);
      out[5920] = fma(0.935, q, out[5920]);
      out[5568] = fma(0.504, q, out[5568]);
      out[5760] = fma(0.132, q, out[5760]);
      out[4480] = fma(0.165, q, out[4480]);
      out[5280] = fma(0.042, q, out[5280]);
      out[5440] = fma(0.065, q, out[5440]);
    }
    if (mask[185]) {
      const double q = scale * ws[65248];
      out[5120] = out[5120] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.2, q, out[5984]);
      out[5888] = fma(0.051, q, out[5888]);
      out[5632] = fma(0.231, q, out[5632]);
      out[5216] = fma(0.235, q, out[5216]);
      out[5920] = fma(0.864, q, out[5920]);
      out[5856] = fma(0.018, q, out[5856]);
      out[5568] = fma(0.045, q, out[5568]);
      out[5760] = fma(0.203, q, out[5760]);
      out[5280] = fma(0.033, q, out[5280]);
      out[4480] = fma(0.217, q, out[4480]);
      out[5504] = fma(0.033, q, out[5504]);
      out[5344] = fma(0.272, q, out[5344]);
      out[5440] = fma(0.136, q, out[5440]);
    }
    if (mask[186]) {
      const double q = scale * ws[65280];
      out[3008] = out[3008] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(1.6, q, out[5856]);
      out[5760] = fma(0.2, q, out[5760]);
    }
    if (mask[187]) {
      const double q = scale * ws[65312];
      out[3200] = out[3200] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.78, q, out[5984]);
      out[5920] = fma(0.97, q, out[5920]);
      out[5856] = fma(0.78, q, out[5856]);
      out[5568] = fma(0.012, q, out[5568]);
      out[5760] = fma(0.44, q, out[5760]);
      out[4480] = fma(0.06, q, out[4480]);
      out[5280] = fma(0.13, q, out[5280]);
      out[5440] = fma(0.03, q, out[5440]);
    }
    if (mask[188]) {
      const double q = scale * ws[65344];
      out[3328] = out[3328] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.83, q, out[5984]);
      out[5920] = fma(0.95, q, out[5920]);
      out[5568] = fma(0.81, q, out[5568]);
      out[5760] = fma(0.68, q, out[5760]);
      out[4480] = fma(0.2, q, out[4480]);
      out[5504] = fma(0.09, q, out[5504]);
      out[5344] = fma(0.02, q, out[5344]);
      out[5440] = fma(0.05, q, out[5440]);
    }
}
__device__ __noinline__ void ddm_src_0_3(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[189]) {
      const double q = scale * ws[65376];
      out[3360] = out[3360] - q;
      out[5824] = out[5824] - q;
      out[5440] = fma(0.0, q, out[5440]);
      out[5312] = fma(0.0012, q, out[5312]);
      out[4896] = fma(0.0008, q, out[4896]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[4448] = fma(0.0, q, out[4448]);
      out[5376] = fma(0.998, q, out[5376]);
      out[4512] = fma(0.499, q, out[4512]);
      out[4320] = fma(0.2495, q, out[4320]);
      out[3584] = fma(0.2495, q, out[3584]);
    }
    if (mask[190]) {
      const double q = scale * ws[65408];
      out[3296] = out[3296] - q;
      out[5824] = out[5824] - q;
      out[5440] = fma(0.0002, q, out[5440]);
      out[5312] = fma(0.0013, q, out[5312]);
      out[4896] = fma(0.0006, q, out[4896]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[4448] = fma(0.0852, q, out[4448]);
      out[5376] = fma(0.5477, q, out[5376]);
      out[5248] = fma(0.3651, q, out[5248]);
      out[4512] = fma(0.3651, q, out[4512]);
      out[5472] = fma(0.5477, q, out[5472]);
    }
    if (mask[191]) {
      const double q = scale * ws[65440];
      out[3104] = out[3104] - q;
      out[5824] = out[5824] - q;
      out[5440] = fma(0.0001, q, out[5440]);
      out[5536] = fma(0.0013, q, out[5536]);
      out[4928] = fma(0.0006, q, out[4928]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[4448] = fma(0.0481, q, out[4448]);
      out[5376] = fma(0.7029, q, out[5376]);
      out[5248] = fma(0.247, q, out[5248]);
      out[4512] = fma(0.3515, q, out[4512]);
      out[4320] = fma(0.5984, q, out[4320]);
    }
    if (mask[192]) {
      const double q = scale * ws[65472];
      out[3264] = out[3264] - q;
      out[5824] = out[5824] - q;
      out[5440] = fma(0.0002, q, out[5440]);
      out[5536] = fma(0.0013, q, out[5536]);
      out[4928] = fma(0.0006, q, out[4928]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[4448] = fma(0.0852, q, out[4448]);
      out[5376] = fma(0.5477, q, out[5376]);
      out[5248] = fma(0.3651, q, out[5248]);
      out[4512] = fma(0.4564, q, out[4512]);
      out[4320] = fma(0.4564, q, out[4320]);
    }
    if (mask[193]) {
      const double q = scale * ws[65504];
      out[4160] = out[4160] - q;
      out[5824] = out[5824] - q;
      out[4384] = fma(0.237, q, out[4384]);
      out[5984] = fma(0.763, q, out[5984]);
      out[5920] = fma(0.763, q, out[5920]);
      out[4544] = fma(0.195, q, out[4544]);
      out[5760] = fma(0.284, q, out[5760]);
      out[4480] = fma(0.0865, q, out[4480]);
      out[4576] = fma(0.1285, q, out[4576]);
      out[5856] = fma(0.308, q, out[5856]);
      out[4096] = fma(0.0715, q, out[4096]);
      out[5504] = fma(0.084, q, out[5504]);
    }
    if (mask[194]) {
      const double q = scale * ws[65536];
      out[3744] = out[3744] - q;
      out[5824] = out[5824] - q;
      out[6016] = fma(0.82, q, out[6016]);
      out[5920] = fma(0.82, q, out[5920]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[195]) {
      const double q = scale * ws[65568];
      out[2624] = out[2624] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.6955, q, out[5920]);
      out[4384] = fma(0.2345, q, out[4384]);
      out[5440] = fma(0.07, q, out[5440]);
      out[4544] = fma(0.6045, q, out[4544]);
      out[5760] = fma(0.154, q, out[5760]);
      out[5504] = fma(0.007, q, out[5504]);
      out[5856] = fma(0.007, q, out[5856]);
      out[5984] = fma(0.1645, q, out[5984]);
    }
    if (mask[196]) {
      const double q = scale * ws[65600];
      out[3840] = out[3840] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(0.82, q, out[5920]);
      out[6016] = fma(0.82, q, out[6016]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[197]) {
      const double q = scale * ws[65632];
      out[4192] = out[4192] - q;
      out[5824] = out[5824] - q;
      out[4384] = fma(0.23, q, out[4384]);
      out[5920] = fma(0.77, q, out[5920]);
      out[4576] = fma(0.77, q, out[4576]);
      out[5984] = fma(0.77, q, out[5984]);
      out[5856] = fma(0.43, q, out[5856]);
    }
    if (mask[198]) {
      const double q = scale * ws[65664];
      out[3936] = out[3936] - q;
      out[5824] = out[5824] - q;
      out[6016] = fma(0.77, q, out[6016]);
      out[5920] = fma(0.77, q, out[5920]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[199]) {
      const double q = scale * ws[65696];
      out[2656] = out[2656] - q;
      out[5824] = out[5824] - q;
      out[4384] = fma(0.57, q, out[4384]);
      out[5440] = fma(0.07, q, out[5440]);
      out[5920] = fma(1.36, q, out[5920]);
      out[4576] = fma(0.43, q, out[4576]);
      out[5984] = fma(0.5, q, out[5984]);
    }
    if (mask[200]) {
      const double q = scale * ws[65728];
      out[3712] = out[3712] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(0.77, q, out[5920]);
      out[6016] = fma(0.77, q, out[6016]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[201]) {
      const double q = scale * ws[65760];
      out[2560] = out[2560] - q;
      out[5824] = out[5824] - q;
      out[4384] = fma(0.36, q, out[4384]);
      out[4256] = fma(0.64, q, out[4256]);
      out[5920] = fma(0.64, q, out[5920]);
    }
    if (mask[202]) {
      const double q = scale * ws[65792];
      out[1728] = out[1728] - q;
      out[5824] = out[5824] - q;
      out[4384] = fma(0.64, q, out[4384]);
      out[5920] = fma(0.36, q, out[5920]);
      out[5984] = fma(0.36, q, out[5984]);
      out[5856] = fma(0.36, q, out[5856]);
      out[3680] = fma(0.36, q, out[3680]);
    }
    if (mask[203]) {
      const double q = scale * ws[65824];
      out[5792] = out[5792] - q;
      out[5824] = out[5824] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[204]) {
      const double q = scale * ws[65856];
      out[4800] = out[4800] - q;
      out[5824] = out[5824] - q;
      out[5632] = fma(1.0, q, out[5632]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[205]) {
      const double q = scale * ws[65888];
      out[2848] = out[2848] - q;
      out[5824] = out[5824] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[206]) {
      const double q = scale * ws[65920];
      out[5152] = out[5152] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.67, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.33, q, out[5856]);
      out[5472] = fma(0.67, q, out[5472]);
    }
    if (mask[207]) {
      const double q = scale * ws[65952];
      out[3776] = out[3776] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.77, q, out[5984]);
      out[5792] = fma(0.23, q, out[5792]);
      out[5216] = fma(0.16, q, out[5216]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5760] = fma(0.46, q, out[5760]);
      out[5248] = fma(0.54, q, out[5248]);
    }
    if (mask[208]) {
      const double q = scale * ws[65984];
      out[4672] = out[4672] - q;
      out[5824] = out[5824] - q;
      out[5888] = fma(0.65, q, out[5888]);
      out[5792] = fma(0.35, q, out[5792]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5664] = fma(0.65, q, out[5664]);
      out[5856] = fma(0.65, q, out[5856]);
    }
    if (mask[209]) {
      const double q = scale * ws[66016];
      out[3520] = out[3520] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.5, q, out[5984]);
      out[5856] = fma(0.5, q, out[5856]);
      out[5344] = fma(1.0, q, out[5344]);
    }
    if (mask[210]) {
      const double q = scale * ws[66048];
      out[2880] = out[2880] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.3, q, out[5984]);
      out[5792] = fma(0.7, q, out[5792]);
      out[5216] = fma(0.7, q, out[5216]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.3, q, out[5856]);
      out[5760] = fma(0.7, q, out[5760]);
      out[5248] = fma(0.3, q, out[5248]);
    }
    if (mask[211]) {
      const double q = scale * ws[66080];
      out[2912] = out[2912] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5664] = fma(0.61, q, out[5664]);
      out[5856] = fma(0.03, q, out[5856]);
      out[5760] = fma(0.27, q, out[5760]);
      out[5376] = fma(0.18, q, out[5376]);
      out[5504] = fma(0.7, q, out[5504]);
      out[5248] = fma(0.21, q, out[5248]);
    }
    if (mask[212]) {
      const double q = scale * ws[66112];
      out[2592] = out[2592] - q;
      out[5824] = out[5824] - q;
      out[2272] = fma(1.0, q, out[2272]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[213]) {
      const double q = scale * ws[66144];
      out[2272] = out[2272] - q;
      out[5824] = out[5824] - q;
      out[2688] = fma(1.0, q, out[2688]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[214]) {
      const double q = scale * ws[66176];
      out[3648] = out[3648] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5344] = fma(0.32, q, out[5344]);
      out[5376] = fma(0.68, q, out[5376]);
      out[5728] = fma(0.68, q, out[5728]);
    }
    if (mask[215]) {
      const double q = scale * ws[66208];
      out[3040] = out[3040] - q;
      out[5824] = out[5824] - q;
      out[3808] = fma(1.0, q, out[3808]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[216]) {
      const double q = scale * ws[66240];
      out[2976] = out[2976] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5376] = fma(1.0, q, out[5376]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[217]) {
      const double q = scale * ws[66272];
      out[4032] = out[4032] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[218]) {
      const double q = scale * ws[66304];
      out[4064] = out[4064] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(2.0, q, out[5920]);
      out[5856] = fma(0.287, q, out[5856]);
      out[5760] = fma(1.24, q, out[5760]);
      out[5504] = fma(0.464, q, out[5504]);
    }
    if (mask[219]) {
      const double q = scale * ws[66336];
      out[3072] = out[3072] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(2.0, q, out[5920]);
      out[5376] = fma(1.0, q, out[5376]);
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[220]) {
      const double q = scale * ws[66368];
      out[5216] = out[5216] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[221]) {
      const double q = scale * ws[66400];
      out[2688] = out[2688] - q;
      out[5920] = out[5920] - q;
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[222]) {
      const double q = scale * ws[66432];
      out[3232] = out[3232] - q;
      out[5920] = out[5920] - q;
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[223]) {
      const double q = scale * ws[66464];
      out[3808] = out[3808] - q;
      out[5920] = out[5920] - q;
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[224]) {
      const double q = scale * ws[66496];
      out[5888] = out[5888] - q;
      out[5984] = out[5984] - q;
      out[2816] = fma(1.0, q, out[2816]);
    }
    if (mask[225]) {
      const double q = scale * ws[66528];
      out[5632] = out[5632] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[226]) {
      const double q = scale * ws[66560];
      out[5408] = out[5408] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[227]) {
      const double q = scale * ws[66592];
      out[5120] = out[5120] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[228]) {
      const double q = scale * ws[66624];
      out[3008] = out[3008] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[229]) {
      const double q = scale * ws[66656];
      out[3200] = out[3200] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[230]) {
      const double q = scale * ws[66688];
      out[3328] = out[3328] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[231]) {
      const double q = scale * ws[66720];
      out[3360] = out[3360] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(0.6021, q, out[5728]);
      out[4896] = fma(0.3979, q, out[4896]);
    }
    if (mask[232]) {
      const double q = scale * ws[66752];
      out[3296] = out[3296] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(0.7195, q, out[5728]);
      out[4896] = fma(0.2805, q, out[4896]);
    }
    if (mask[233]) {
      const double q = scale * ws[66784];
      out[3104] = out[3104] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(0.0482, q, out[5728]);
      out[4608] = fma(0.6747, q, out[4608]);
      out[4928] = fma(0.2771, q, out[4928]);
    }
    if (mask[234]) {
      const double q = scale * ws[66816];
      out[3264] = out[3264] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(0.0854, q, out[5728]);
      out[4608] = fma(0.6341, q, out[4608]);
      out[4928] = fma(0.2805, q, out[4928]);
    }
    if (mask[235]) {
      const double q = scale * ws[66848];
      out[4160] = out[4160] - q;
      out[5984] = out[5984] - q;
      out[4480] = fma(0.039, q, out[4480]);
      out[4576] = fma(0.039, q, out[4576]);
      out[5856] = fma(0.0625, q, out[5856]);
      out[4096] = fma(0.762, q, out[4096]);
      out[5984] = fma(0.3225, q, out[5984]);
      out[4544] = fma(0.1885, q, out[4544]);
      out[6016] = fma(0.238, q, out[6016]);
      out[5504] = fma(0.0105, q, out[5504]);
    }
    if (mask[236]) {
      const double q = scale * ws[66880];
      out[3744] = out[3744] - q;
      out[5984] = out[5984] - q;
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[237]) {
      const double q = scale * ws[66912];
      out[2624] = out[2624] - q;
      out[5984] = out[5984] - q;
      out[4384] = fma(0.461, q, out[4384]);
      out[4544] = fma(0.455, q, out[4544]);
      out[5920] = fma(0.539, q, out[5920]);
      out[6016] = fma(0.6195, q, out[6016]);
      out[5760] = fma(0.077, q, out[5760]);
      out[5504] = fma(0.007, q, out[5504]);
      out[5856] = fma(0.007, q, out[5856]);
    }
    if (mask[238]) {
      const double q = scale * ws[66944];
      out[3840] = out[3840] - q;
      out[5984] = out[5984] - q;
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[239]) {
      const double q = scale * ws[66976];
      out[4192] = out[4192] - q;
      out[5984] = out[5984] - q;
      out[4096] = fma(0.9, q, out[4096]);
      out[4576] = fma(0.1, q, out[4576]);
      out[6016] = fma(0.1, q, out[6016]);
      out[5984] = fma(0.1, q, out[5984]);
      out[5856] = fma(0.06, q, out[5856]);
    }
    if (mask[240]) {
      const double q = scale * ws[67008];
      out[3936] = out[3936] - q;
      out[5984] = out[5984] - q;
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[241]) {
      const double q = scale * ws[67040];
      out[2656] = out[2656] - q;
      out[5984] = out[5984] - q;
      out[4384] = fma(0.77, q, out[4384]);
      out[6016] = fma(0.5, q, out[6016]);
      out[4576] = fma(0.23, q, out[4576]);
      out[5920] = fma(0.23, q, out[5920]);
      out[5984] = fma(0.27, q, out[5984]);
    }
    if (mask[242]) {
      const double q = scale * ws[67072];
      out[3712] = out[3712] - q;
      out[5984] = out[5984] - q;
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[243]) {
      const double q = scale * ws[67104];
      out[2560] = out[2560] - q;
      out[5984] = out[5984] - q;
      out[4096] = fma(0.75, q, out[4096]);
      out[6016] = fma(0.25, q, out[6016]);
      out[4256] = fma(0.25, q, out[4256]);
    }
    if (mask[244]) {
      const double q = scale * ws[67136];
      out[1728] = out[1728] - q;
      out[5984] = out[5984] - q;
      out[4096] = fma(0.9, q, out[4096]);
      out[6016] = fma(0.1, q, out[6016]);
      out[5984] = fma(0.1, q, out[5984]);
      out[5856] = fma(0.1, q, out[5856]);
      out[3680] = fma(0.1, q, out[3680]);
    }
    if (mask[245]) {
      const double q = scale * ws[67168];
      out[5792] = out[5792] - q;
      out[5984] = out[5984] - q;
      out[6016] = fma(0.44, q, out[6016]);
      out[5888] = fma(0.44, q, out[5888]);
      out[5696] = fma(0.15, q, out[5696]);
      out[3680] = fma(0.41, q, out[3680]);
    }
}
}  // namespace mech_cracmm2
