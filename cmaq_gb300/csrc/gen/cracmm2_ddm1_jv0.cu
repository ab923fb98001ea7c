// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void ddm_jv_1_0(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[43616] * fma(y[6016], v[5184], y[5184] * v[6016]);
      out[5184] = out[5184] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[43648] * fma(y[5984], v[5184], y[5184] * v[5984]);
      out[5184] = out[5184] - dr;
      out[5984] = out[5984] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
    }
    {
      const double dr = ws[43680] * fma(y[5824], v[5184], y[5184] * v[5824]);
      out[5184] = out[5184] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[43712] * fma(y[5920], v[5184], y[5184] * v[5920]);
      out[5184] = out[5184] - dr;
      out[5920] = out[5920] - dr;
      out[5952] = fma(1.0, dr, out[5952]);
    }
    {
      const double dr = ws[43744] * v[2336];
      out[2336] = out[2336] - dr;
      out[5184] = fma(1.0, dr, out[5184]);
    }
    {
      const double dr = ws[43776] * fma(y[5184], v[2336], y[2336] * v[5184]);
      out[2336] = out[2336] - dr;
      out[5184] = out[5184] - dr;
    }
    {
      const double dr = ws[43808] * v[576];
      out[576] = out[576] - dr;
      out[2336] = fma(1.0, dr, out[2336]);
    }
    {
      const double dr = ws[43840] * v[576];
      out[576] = out[576] - dr;
      out[2336] = fma(1.0, dr, out[2336]);
    }
    {
      const double dr = ws[43872] * v[576];
      out[576] = out[576] - dr;
      out[6016] = fma(2.0, dr, out[6016]);
    }
    {
      const double dr = ws[43904] * v[6016];
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[43936] * fma(y[5984], v[6016], y[6016] * v[5984]);
      out[6016] = out[6016] - dr;
      out[5984] = out[5984] - dr;
    }
    {
      const double dr = ws[43968] * fma(y[5984], v[5984], y[5984] * v[5984]);
      out[5984] = out[5984] - dr;
      out[5984] = out[5984] - dr;
      out[4000] = fma(1.0, dr, out[4000]);
    }
    {
      const double dr = ws[44000] * fma(y[5984], v[5984], y[5984] * v[5984]);
      out[5984] = out[5984] - dr;
      out[5984] = out[5984] - dr;
      out[4000] = fma(1.0, dr, out[4000]);
    }
    {
      const double dr = ws[44032] * fma(y[6016], v[4000], y[4000] * v[6016]);
      out[4000] = out[4000] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[44064] * fma(y[2336], v[5824], y[5824] * v[2336]);
      out[5824] = out[5824] - dr;
      out[2336] = out[2336] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[44096] * fma(y[6016], v[5824], y[5824] * v[6016]);
      out[5824] = out[5824] - dr;
      out[6016] = out[6016] - dr;
      out[1184] = fma(1.0, dr, out[1184]);
    }
    {
      const double dr = ws[44128] * fma(y[5984], v[5824], y[5824] * v[5984]);
      out[5824] = out[5824] - dr;
      out[5984] = out[5984] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[6016] = fma(1.0, dr, out[6016]);
    }
    {
      const double dr = ws[44160] * fma(y[5984], v[5824], y[5824] * v[5984]);
      out[5824] = out[5824] - dr;
      out[5984] = out[5984] - dr;
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[44192] * fma(y[5824], v[5824], y[5824] * v[5824]);
      out[5824] = out[5824] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
    }
    {
      const double dr = ws[44224] * fma(y[6016], v[1184], y[1184] * v[6016]);
      out[1184] = out[1184] - dr;
      out[6016] = out[6016] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[44256] * fma(y[2336], v[5920], y[5920] * v[2336]);
      out[5920] = out[5920] - dr;
      out[2336] = out[2336] - dr;
      out[5824] = fma(1.0, dr, out[5824]);
    }
    {
      const double dr = ws[44288] * fma(y[2336], v[5920], y[5920] * v[2336]);
      out[5920] = out[5920] - dr;
      out[2336] = out[2336] - dr;
      out[5952] = fma(1.0, dr, out[5952]);
    }
    {
      const double dr = ws[44320] * fma(y[6016], v[5920], y[5920] * v[6016]);
      out[5920] = out[5920] - dr;
      out[6016] = out[6016] - dr;
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[44352] * fma(y[6016], v[5024], y[5024] * v[6016]);
      out[5024] = out[5024] - dr;
      out[6016] = out[6016] - dr;
      out[5952] = fma(1.0, dr, out[5952]);
    }
    {
      const double dr = ws[44384] * fma(y[6016], v[5952], y[5952] * v[6016]);
      out[5952] = out[5952] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[44416] * fma(y[5984], v[5952], y[5952] * v[5984]);
      out[5952] = out[5952] - dr;
      out[5984] = out[5984] - dr;
      out[6016] = fma(0.7, dr, out[6016]);
      out[5920] = fma(0.7, dr, out[5920]);
      out[5024] = fma(0.3, dr, out[5024]);
    }
    {
      const double dr = ws[44448] * fma(y[5824], v[5952], y[5952] * v[5824]);
      out[5952] = out[5952] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
    }
    {
      const double dr = ws[44480] * fma(y[5920], v[5952], y[5952] * v[5920]);
      out[5952] = out[5952] - dr;
      out[5920] = out[5920] - dr;
      out[5824] = fma(1.0, dr, out[5824]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[44512] * fma(y[5952], v[5952], y[5952] * v[5952]);
      out[5952] = out[5952] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
    }
    {
      const double dr = ws[44544] * fma(y[5920], v[5952], y[5952] * v[5920]);
      out[5952] = out[5952] - dr;
      out[5920] = out[5920] - dr;
      out[1024] = fma(1.0, dr, out[1024]);
    }
    {
      const double dr = ws[44576] * v[1024];
      out[1024] = out[1024] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5952] = fma(1.0, dr, out[5952]);
    }
    {
      const double dr = ws[44608] * v[1024];
      out[1024] = out[1024] - dr;
      out[5024] = fma(2.0, dr, out[5024]);
    }
    {
      const double dr = ws[44640] * fma(y[5984], v[5920], y[5920] * v[5984]);
      out[5920] = out[5920] - dr;
      out[5984] = out[5984] - dr;
      out[1280] = fma(1.0, dr, out[1280]);
    }
    {
      const double dr = ws[44672] * v[1280];
      out[1280] = out[1280] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[44704] * fma(y[6016], v[1280], y[1280] * v[6016]);
      out[1280] = out[1280] - dr;
      out[6016] = out[6016] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[44736] * fma(y[6016], v[160], y[160] * v[6016]);
      out[160] = out[160] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[192] = fma(1.0, dr, out[192]);
      out[224] = fma(1.0, dr, out[224]);
    }
    {
      const double dr = ws[44768] * fma(y[6016], v[5664], y[5664] * v[6016]);
      out[5664] = out[5664] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[44800] * v[6016];
      out[6016] = out[6016] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
    }
    {
      const double dr = ws[44832] * fma(y[6016], v[1888], y[1888] * v[6016]);
      out[1888] = out[1888] - dr;
      out[6016] = out[6016] - dr;
      out[5632] = fma(1.0, dr, out[5632]);
    }
    {
      const double dr = ws[44864] * fma(y[6016], v[2176], y[2176] * v[6016]);
      out[2176] = out[2176] - dr;
      out[6016] = out[6016] - dr;
      out[5408] = fma(1.0, dr, out[5408]);
      out[3616] = fma(2.81e-05, dr, out[3616]);
    }
    {
      const double dr = ws[44896] * fma(y[6016], v[1120], y[1120] * v[6016]);
      out[1120] = out[1120] - dr;
      out[6016] = out[6016] - dr;
      out[5120] = fma(1.0, dr, out[5120]);
      out[3616] = fma(0.00134, dr, out[3616]);
    }
    {
      const double dr = ws[44928] * fma(y[6016], v[2240], y[2240] * v[6016]);
      out[2240] = out[2240] - dr;
      out[6016] = out[6016] - dr;
      out[3008] = fma(1.0, dr, out[3008]);
    }
    {
      const double dr = ws[44960] * fma(y[6016], v[2752], y[2752] * v[6016]);
      out[2752] = out[2752] - dr;
      out[6016] = out[6016] - dr;
      out[3200] = fma(1.0, dr, out[3200]);
    }
    {
      const double dr = ws[44992] * fma(y[6016], v[1152], y[1152] * v[6016]);
      out[1152] = out[1152] - dr;
      out[6016] = out[6016] - dr;
      out[3328] = fma(1.0, dr, out[3328]);
    }
    {
      const double dr = ws[45024] * fma(y[6016], v[256], y[256] * v[6016]);
      out[256] = out[256] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(0.65, dr, out[6016]);
      out[5984] = fma(0.35, dr, out[5984]);
      out[5664] = fma(0.35, dr, out[5664]);
      out[5376] = fma(0.65, dr, out[5376]);
      out[4352] = fma(0.35, dr, out[4352]);
    }
    {
      const double dr = ws[45056] * fma(y[6016], v[1216], y[1216] * v[6016]);
      out[1216] = out[1216] - dr;
      out[6016] = out[6016] - dr;
      out[3360] = fma(0.47, dr, out[3360]);
      out[1248] = fma(0.53, dr, out[1248]);
      out[5984] = fma(0.53, dr, out[5984]);
    }
    {
      const double dr = ws[45088] * fma(y[6016], v[288], y[288] * v[6016]);
      out[288] = out[288] - dr;
      out[6016] = out[6016] - dr;
      out[3296] = fma(0.82, dr, out[3296]);
      out[2944] = fma(0.18, dr, out[2944]);
      out[5984] = fma(0.18, dr, out[5984]);
    }
    {
      const double dr = ws[45120] * fma(y[6016], v[320], y[320] * v[6016]);
      out[320] = out[320] - dr;
      out[6016] = out[6016] - dr;
      out[3104] = fma(0.83, dr, out[3104]);
      out[2944] = fma(0.17, dr, out[2944]);
      out[5984] = fma(0.17, dr, out[5984]);
    }
    {
      const double dr = ws[45152] * fma(y[6016], v[352], y[352] * v[6016]);
      out[352] = out[352] - dr;
      out[6016] = out[6016] - dr;
      out[3264] = fma(0.82, dr, out[3264]);
      out[2944] = fma(0.18, dr, out[2944]);
      out[5984] = fma(0.18, dr, out[5984]);
    }
    {
      const double dr = ws[45184] * fma(y[5184], v[1312], y[1312] * v[5184]);
      out[1312] = out[1312] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.25, dr, out[6016]);
      out[5984] = fma(0.25, dr, out[5984]);
      out[5888] = fma(0.4, dr, out[5888]);
      out[5792] = fma(0.018, dr, out[5792]);
      out[4672] = fma(0.1, dr, out[4672]);
      out[4000] = fma(0.09, dr, out[4000]);
      out[5664] = fma(0.22, dr, out[5664]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[4128] = fma(0.3, dr, out[4128]);
      out[4736] = fma(0.14, dr, out[4736]);
      out[4352] = fma(0.28, dr, out[4352]);
      out[2752] = fma(0.153, dr, out[2752]);
    }
    {
      const double dr = ws[45216] * fma(y[5952], v[1312], y[1312] * v[5952]);
      out[1312] = out[1312] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(0.4, dr, out[5920]);
      out[2784] = fma(0.045, dr, out[2784]);
      out[5856] = fma(0.35, dr, out[5856]);
      out[1632] = fma(0.555, dr, out[1632]);
      out[4736] = fma(0.26, dr, out[4736]);
      out[4128] = fma(0.028, dr, out[4128]);
    }
    {
      const double dr = ws[45248] * fma(y[6016], v[1312], y[1312] * v[6016]);
      out[1312] = out[1312] - dr;
      out[6016] = out[6016] - dr;
      out[4288] = fma(1.0, dr, out[4288]);
      out[5856] = fma(0.25, dr, out[5856]);
      out[4128] = fma(0.03, dr, out[4128]);
      out[5248] = fma(0.05, dr, out[5248]);
    }
    {
      const double dr = ws[45280] * fma(y[5984], v[4288], y[4288] * v[5984]);
      out[4288] = out[4288] - dr;
      out[5984] = out[5984] - dr;
      out[1344] = fma(1.0, dr, out[1344]);
      out[5984] = fma(0.07, dr, out[5984]);
      out[6016] = fma(0.5, dr, out[6016]);
    }
    {
      const double dr = ws[45312] * fma(y[5824], v[4288], y[4288] * v[5824]);
      out[4288] = out[4288] - dr;
      out[5824] = out[5824] - dr;
      out[2784] = fma(0.13, dr, out[2784]);
      out[5856] = fma(0.4, dr, out[5856]);
      out[5984] = fma(0.88, dr, out[5984]);
      out[5920] = fma(0.87, dr, out[5920]);
      out[4128] = fma(0.18, dr, out[4128]);
      out[4736] = fma(0.51, dr, out[4736]);
    }
    {
      const double dr = ws[45344] * fma(y[6016], v[1344], y[1344] * v[6016]);
      out[1344] = out[1344] - dr;
      out[6016] = out[6016] - dr;
      out[4288] = fma(1.0, dr, out[4288]);
    }
    {
      const double dr = ws[45376] * fma(y[6016], v[1344], y[1344] * v[6016]);
      out[1344] = out[1344] - dr;
      out[6016] = out[6016] - dr;
      out[5248] = fma(0.04, dr, out[5248]);
      out[5376] = fma(0.02, dr, out[5376]);
      out[4736] = fma(0.13, dr, out[4736]);
      out[1376] = fma(0.44, dr, out[1376]);
      out[5792] = fma(0.11, dr, out[5792]);
      out[4128] = fma(0.03, dr, out[4128]);
      out[6016] = fma(2.0, dr, out[6016]);
      out[5984] = fma(0.34, dr, out[5984]);
      out[1664] = fma(0.14, dr, out[1664]);
      out[5664] = fma(1.0, dr, out[5664]);
    }
    {
      const double dr = ws[45408] * fma(y[5984], v[1632], y[1632] * v[5984]);
      out[1632] = out[1632] - dr;
      out[5984] = out[5984] - dr;
      out[6016] = fma(0.45, dr, out[6016]);
      out[2208] = fma(0.95, dr, out[2208]);
      out[1664] = fma(0.02, dr, out[1664]);
    }
    {
      const double dr = ws[45440] * fma(y[5824], v[1632], y[1632] * v[5824]);
      out[1632] = out[1632] - dr;
      out[5824] = out[5824] - dr;
      out[4736] = fma(0.15, dr, out[4736]);
      out[2208] = fma(0.65, dr, out[2208]);
      out[2784] = fma(0.05, dr, out[2784]);
      out[5856] = fma(0.2, dr, out[5856]);
      out[5920] = fma(1.3, dr, out[5920]);
    }
    {
      const double dr = ws[45472] * fma(y[6016], v[2784], y[2784] * v[6016]);
      out[2784] = out[2784] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[2208] = fma(0.35, dr, out[2208]);
      out[1376] = fma(0.17, dr, out[1376]);
      out[5920] = fma(0.65, dr, out[5920]);
    }
    {
      const double dr = ws[45504] * fma(y[2208], v[6016], y[6016] * v[2208]);
      out[6016] = out[6016] - dr;
      out[2208] = out[2208] - dr;
      out[5664] = fma(1.0, dr, out[5664]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.3, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[45536] * v[2784];
      out[2784] = out[2784] - dr;
      out[5024] = fma(1.0, dr, out[5024]);
      out[5056] = fma(1.0, dr, out[5056]);
    }
    {
      const double dr = ws[45568] * fma(y[6016], v[1664], y[1664] * v[6016]);
      out[1664] = out[1664] - dr;
      out[6016] = out[6016] - dr;
      out[4128] = fma(0.57, dr, out[4128]);
      out[4736] = fma(0.43, dr, out[4736]);
    }
    {
      const double dr = ws[45600] * fma(y[6016], v[1408], y[1408] * v[6016]);
      out[1408] = out[1408] - dr;
      out[6016] = out[6016] - dr;
      out[4160] = fma(0.975, dr, out[4160]);
      out[3744] = fma(0.025, dr, out[3744]);
    }
    {
      const double dr = ws[45632] * fma(y[6016], v[1440], y[1440] * v[6016]);
      out[1440] = out[1440] - dr;
      out[6016] = out[6016] - dr;
      out[4192] = fma(0.945, dr, out[4192]);
      out[3936] = fma(0.055, dr, out[3936]);
    }
    {
      const double dr = ws[45664] * fma(y[6016], v[4544], y[4544] * v[6016]);
      out[4544] = out[4544] - dr;
      out[6016] = out[6016] - dr;
      out[2560] = fma(0.23, dr, out[2560]);
      out[4800] = fma(0.77, dr, out[4800]);
    }
    {
      const double dr = ws[45696] * fma(y[6016], v[4576], y[4576] * v[6016]);
      out[4576] = out[4576] - dr;
      out[6016] = out[6016] - dr;
      out[1728] = fma(0.83, dr, out[1728]);
      out[4800] = fma(0.17, dr, out[4800]);
    }
    {
      const double dr = ws[45728] * fma(y[6016], v[5856], y[5856] * v[6016]);
      out[5856] = out[5856] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5664] = fma(1.0, dr, out[5664]);
    }
    {
      const double dr = ws[45760] * fma(y[6016], v[5568], y[5568] * v[6016]);
      out[5568] = out[5568] - dr;
      out[6016] = out[6016] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
    }
    {
      const double dr = ws[45792] * fma(y[6016], v[5760], y[5760] * v[6016]);
      out[5760] = out[5760] - dr;
      out[6016] = out[6016] - dr;
      out[4800] = fma(1.0, dr, out[4800]);
    }
    {
      const double dr = ws[45824] * fma(y[6016], v[4480], y[4480] * v[6016]);
      out[4480] = out[4480] - dr;
      out[6016] = out[6016] - dr;
      out[2848] = fma(1.0, dr, out[2848]);
    }
    {
      const double dr = ws[45856] * fma(y[6016], v[5280], y[5280] * v[6016]);
      out[5280] = out[5280] - dr;
      out[6016] = out[6016] - dr;
      out[5152] = fma(1.0, dr, out[5152]);
    }
    {
      const double dr = ws[45888] * fma(y[6016], v[5504], y[5504] * v[6016]);
      out[5504] = out[5504] - dr;
      out[6016] = out[6016] - dr;
      out[3776] = fma(1.0, dr, out[3776]);
    }
}
__device__ __noinline__ void ddm_jv_1_1(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[45920] * fma(y[6016], v[5344], y[5344] * v[6016]);
      out[5344] = out[5344] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5248] = fma(1.0, dr, out[5248]);
    }
    {
      const double dr = ws[45952] * fma(y[6016], v[4128], y[4128] * v[6016]);
      out[4128] = out[4128] - dr;
      out[6016] = out[6016] - dr;
      out[4672] = fma(0.57, dr, out[4672]);
      out[3520] = fma(0.43, dr, out[3520]);
    }
    {
      const double dr = ws[45984] * fma(y[6016], v[4736], y[4736] * v[6016]);
      out[4736] = out[4736] - dr;
      out[6016] = out[6016] - dr;
      out[2880] = fma(1.0, dr, out[2880]);
    }
    {
      const double dr = ws[46016] * fma(y[6016], v[3872], y[3872] * v[6016]);
      out[3872] = out[3872] - dr;
      out[6016] = out[6016] - dr;
      out[5792] = fma(0.313, dr, out[5792]);
      out[2912] = fma(0.687, dr, out[2912]);
    }
    {
      const double dr = ws[46048] * fma(y[6016], v[5376], y[5376] * v[6016]);
      out[5376] = out[5376] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5664] = fma(2.0, dr, out[5664]);
    }
    {
      const double dr = ws[46080] * fma(y[6016], v[5248], y[5248] * v[6016]);
      out[5248] = out[5248] - dr;
      out[6016] = out[6016] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
      out[5664] = fma(1.0, dr, out[5664]);
    }
    {
      const double dr = ws[46112] * fma(y[6016], v[5472], y[5472] * v[6016]);
      out[5472] = out[5472] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(0.52, dr, out[5984]);
      out[5664] = fma(0.33, dr, out[5664]);
      out[5760] = fma(0.4, dr, out[5760]);
      out[5504] = fma(0.78, dr, out[5504]);
      out[5376] = fma(0.1, dr, out[5376]);
      out[5248] = fma(0.01, dr, out[5248]);
    }
    {
      const double dr = ws[46144] * fma(y[6016], v[4320], y[4320] * v[6016]);
      out[4320] = out[4320] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(0.52, dr, out[5984]);
      out[5664] = fma(0.33, dr, out[5664]);
      out[5280] = fma(0.13, dr, out[5280]);
      out[5376] = fma(0.1, dr, out[5376]);
      out[5248] = fma(0.01, dr, out[5248]);
      out[5728] = fma(0.78, dr, out[5728]);
    }
    {
      const double dr = ws[46176] * fma(y[6016], v[3584], y[3584] * v[6016]);
      out[3584] = out[3584] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(0.56, dr, out[5984]);
      out[4672] = fma(0.21, dr, out[4672]);
      out[5664] = fma(0.11, dr, out[5664]);
      out[5376] = fma(0.27, dr, out[5376]);
      out[5248] = fma(0.01, dr, out[5248]);
      out[5728] = fma(0.79, dr, out[5728]);
    }
    {
      const double dr = ws[46208] * fma(y[6016], v[4448], y[4448] * v[6016]);
      out[4448] = out[4448] - dr;
      out[6016] = out[6016] - dr;
      out[2592] = fma(1.0, dr, out[2592]);
    }
    {
      const double dr = ws[46240] * fma(y[6016], v[1248], y[1248] * v[6016]);
      out[1248] = out[1248] - dr;
      out[6016] = out[6016] - dr;
      out[3616] = fma(0.152, dr, out[3616]);
      out[5984] = fma(0.619, dr, out[5984]);
      out[3648] = fma(0.17, dr, out[3648]);
      out[3232] = fma(0.059, dr, out[3232]);
      out[1760] = fma(0.619, dr, out[1760]);
    }
    {
      const double dr = ws[46272] * fma(y[6016], v[2944], y[2944] * v[6016]);
      out[2944] = out[2944] - dr;
      out[6016] = out[6016] - dr;
      out[3616] = fma(0.2, dr, out[3616]);
      out[5984] = fma(0.584, dr, out[5984]);
      out[3648] = fma(0.16, dr, out[3648]);
      out[3232] = fma(0.056, dr, out[3232]);
      out[1760] = fma(0.584, dr, out[1760]);
    }
    {
      const double dr = ws[46304] * fma(y[6016], v[1760], y[1760] * v[6016]);
      out[1760] = out[1760] - dr;
      out[6016] = out[6016] - dr;
      out[3808] = fma(1.0, dr, out[3808]);
    }
    {
      const double dr = ws[46336] * fma(y[6016], v[5600], y[5600] * v[6016]);
      out[5600] = out[5600] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[46368] * fma(y[6016], v[1472], y[1472] * v[6016]);
      out[1472] = out[1472] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5568] = fma(1.0, dr, out[5568]);
    }
    {
      const double dr = ws[46400] * fma(y[6016], v[5056], y[5056] * v[6016]);
      out[5056] = out[5056] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5760] = fma(0.719, dr, out[5760]);
      out[5568] = fma(0.184, dr, out[5568]);
    }
    {
      const double dr = ws[46432] * fma(y[6016], v[1504], y[1504] * v[6016]);
      out[1504] = out[1504] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5760] = fma(1.0, dr, out[5760]);
    }
    {
      const double dr = ws[46464] * fma(y[6016], v[2816], y[2816] * v[6016]);
      out[2816] = out[2816] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(0.35, dr, out[6016]);
      out[5888] = fma(0.65, dr, out[5888]);
      out[5856] = fma(0.35, dr, out[5856]);
    }
    {
      const double dr = ws[46496] * fma(y[6016], v[5728], y[5728] * v[6016]);
      out[5728] = out[5728] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(0.01, dr, out[6016]);
      out[5408] = fma(0.44, dr, out[5408]);
      out[5216] = fma(0.07, dr, out[5216]);
      out[5760] = fma(0.08, dr, out[5760]);
      out[5504] = fma(0.41, dr, out[5504]);
    }
    {
      const double dr = ws[46528] * fma(y[6016], v[4096], y[4096] * v[6016]);
      out[4096] = out[4096] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(0.01, dr, out[6016]);
      out[3904] = fma(0.44, dr, out[3904]);
      out[5216] = fma(0.07, dr, out[5216]);
      out[5760] = fma(0.08, dr, out[5760]);
      out[5504] = fma(0.41, dr, out[5504]);
    }
    {
      const double dr = ws[46560] * fma(y[6016], v[4608], y[4608] * v[6016]);
      out[4608] = out[4608] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(0.01, dr, out[6016]);
      out[3904] = fma(0.44, dr, out[3904]);
      out[5216] = fma(0.07, dr, out[5216]);
      out[5760] = fma(0.08, dr, out[5760]);
      out[5504] = fma(0.41, dr, out[5504]);
    }
    {
      const double dr = ws[46592] * fma(y[6016], v[1792], y[1792] * v[6016]);
      out[1792] = out[1792] - dr;
      out[6016] = out[6016] - dr;
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[46624] * fma(y[6016], v[4352], y[4352] * v[6016]);
      out[4352] = out[4352] - dr;
      out[6016] = out[6016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[46656] * fma(y[6016], v[5696], y[5696] * v[6016]);
      out[5696] = out[5696] - dr;
      out[6016] = out[6016] - dr;
      out[5888] = fma(0.64, dr, out[5888]);
      out[2976] = fma(0.36, dr, out[2976]);
    }
    {
      const double dr = ws[46688] * fma(y[6016], v[3680], y[3680] * v[6016]);
      out[3680] = out[3680] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(0.35, dr, out[6016]);
      out[5792] = fma(0.65, dr, out[5792]);
      out[5216] = fma(0.35, dr, out[5216]);
      out[5856] = fma(0.35, dr, out[5856]);
    }
    {
      const double dr = ws[46720] * fma(y[6016], v[1088], y[1088] * v[6016]);
      out[1088] = out[1088] - dr;
      out[6016] = out[6016] - dr;
      out[5216] = fma(1.0, dr, out[5216]);
      out[5952] = fma(1.0, dr, out[5952]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[46752] * fma(y[6016], v[1536], y[1536] * v[6016]);
      out[1536] = out[1536] - dr;
      out[6016] = out[6016] - dr;
      out[5216] = fma(1.0, dr, out[5216]);
      out[5952] = fma(1.0, dr, out[5952]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[46784] * fma(y[6016], v[1824], y[1824] * v[6016]);
      out[1824] = out[1824] - dr;
      out[6016] = out[6016] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5344] = fma(1.0, dr, out[5344]);
    }
    {
      const double dr = ws[46816] * fma(y[6016], v[5440], y[5440] * v[6016]);
      out[5440] = out[5440] - dr;
      out[6016] = out[6016] - dr;
      out[5408] = fma(1.0, dr, out[5408]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[46848] * fma(y[6016], v[4384], y[4384] * v[6016]);
      out[4384] = out[4384] - dr;
      out[6016] = out[6016] - dr;
      out[1696] = fma(0.33, dr, out[1696]);
      out[5920] = fma(0.67, dr, out[5920]);
      out[4544] = fma(0.27, dr, out[4544]);
      out[5504] = fma(0.38, dr, out[5504]);
      out[5856] = fma(0.21, dr, out[5856]);
      out[5760] = fma(0.02, dr, out[5760]);
    }
    {
      const double dr = ws[46880] * fma(y[6016], v[1696], y[1696] * v[6016]);
      out[1696] = out[1696] - dr;
      out[6016] = out[6016] - dr;
      out[5344] = fma(1.0, dr, out[5344]);
      out[5952] = fma(1.0, dr, out[5952]);
    }
    {
      const double dr = ws[46912] * fma(y[5184], v[2240], y[2240] * v[5184]);
      out[2240] = out[2240] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.08, dr, out[6016]);
      out[5984] = fma(0.15, dr, out[5984]);
      out[5664] = fma(0.43, dr, out[5664]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[4352] = fma(0.37, dr, out[4352]);
    }
    {
      const double dr = ws[46944] * fma(y[5184], v[2752], y[2752] * v[5184]);
      out[2752] = out[2752] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.22, dr, out[6016]);
      out[5984] = fma(0.32, dr, out[5984]);
      out[5888] = fma(0.08, dr, out[5888]);
      out[5632] = fma(0.06, dr, out[5632]);
      out[5408] = fma(0.04, dr, out[5408]);
      out[5120] = fma(0.02, dr, out[5120]);
      out[4000] = fma(0.068, dr, out[4000]);
      out[5664] = fma(0.43, dr, out[5664]);
      out[1888] = fma(0.02, dr, out[1888]);
      out[2176] = fma(0.015, dr, out[2176]);
      out[1120] = fma(0.006, dr, out[1120]);
      out[1216] = fma(0.032, dr, out[1216]);
      out[5856] = fma(0.56, dr, out[5856]);
      out[5568] = fma(0.01, dr, out[5568]);
      out[5760] = fma(0.44, dr, out[5760]);
      out[4480] = fma(0.03, dr, out[4480]);
      out[4448] = fma(0.02, dr, out[4448]);
      out[5280] = fma(0.06, dr, out[5280]);
      out[5344] = fma(0.01, dr, out[5344]);
      out[4352] = fma(0.03, dr, out[4352]);
      out[5696] = fma(0.06, dr, out[5696]);
    }
    {
      const double dr = ws[46976] * fma(y[5184], v[1152], y[1152] * v[5184]);
      out[1152] = out[1152] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.46, dr, out[6016]);
      out[5984] = fma(0.07, dr, out[5984]);
      out[5888] = fma(0.32, dr, out[5888]);
      out[5632] = fma(0.07, dr, out[5632]);
      out[5408] = fma(0.04, dr, out[5408]);
      out[5792] = fma(0.09, dr, out[5792]);
      out[5664] = fma(0.37, dr, out[5664]);
      out[4000] = fma(0.026, dr, out[4000]);
      out[1888] = fma(0.01, dr, out[1888]);
      out[2176] = fma(0.01, dr, out[2176]);
      out[5856] = fma(0.09, dr, out[5856]);
      out[5568] = fma(0.457, dr, out[5568]);
      out[5760] = fma(0.73, dr, out[5760]);
      out[4480] = fma(0.11, dr, out[4480]);
      out[5504] = fma(0.017, dr, out[5504]);
      out[5344] = fma(0.044, dr, out[5344]);
      out[5696] = fma(0.017, dr, out[5696]);
    }
    {
      const double dr = ws[47008] * fma(y[5184], v[1408], y[1408] * v[5184]);
      out[1408] = out[1408] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.6055, dr, out[6016]);
      out[2560] = fma(0.2145, dr, out[2560]);
      out[4000] = fma(0.255, dr, out[4000]);
      out[4544] = fma(0.2535, dr, out[4544]);
      out[5696] = fma(0.0065, dr, out[5696]);
      out[5984] = fma(0.1105, dr, out[5984]);
      out[5664] = fma(0.1105, dr, out[5664]);
      out[5856] = fma(0.459, dr, out[5856]);
      out[4800] = fma(0.2805, dr, out[4800]);
      out[5504] = fma(0.1785, dr, out[5504]);
      out[2176] = fma(0.0665, dr, out[2176]);
      out[2816] = fma(0.0385, dr, out[2816]);
      out[4352] = fma(0.028, dr, out[4352]);
    }
    {
      const double dr = ws[47040] * fma(y[5184], v[1440], y[1440] * v[5184]);
      out[1440] = out[1440] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.66, dr, out[6016]);
      out[4576] = fma(0.66, dr, out[4576]);
      out[5792] = fma(0.33, dr, out[5792]);
      out[5856] = fma(0.33, dr, out[5856]);
      out[4800] = fma(0.33, dr, out[4800]);
      out[4000] = fma(0.33, dr, out[4000]);
      out[5696] = fma(0.01, dr, out[5696]);
    }
    {
      const double dr = ws[47072] * fma(y[5184], v[4576], y[4576] * v[5184]);
      out[4576] = out[4576] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.09, dr, out[6016]);
      out[5760] = fma(1.0, dr, out[5760]);
      out[5856] = fma(0.62, dr, out[5856]);
      out[2816] = fma(0.23, dr, out[2816]);
      out[4000] = fma(0.02, dr, out[4000]);
      out[4352] = fma(0.15, dr, out[4352]);
    }
    {
      const double dr = ws[47104] * fma(y[5184], v[4384], y[4384] * v[5184]);
      out[4384] = out[4384] - dr;
      out[5184] = out[5184] - dr;
      out[1696] = fma(0.33, dr, out[1696]);
      out[5920] = fma(0.67, dr, out[5920]);
      out[4544] = fma(0.27, dr, out[4544]);
      out[5504] = fma(0.38, dr, out[5504]);
      out[5856] = fma(0.21, dr, out[5856]);
      out[5760] = fma(0.02, dr, out[5760]);
    }
    {
      const double dr = ws[47136] * fma(y[5184], v[4128], y[4128] * v[5184]);
      out[4128] = out[4128] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.19, dr, out[6016]);
      out[5984] = fma(0.14, dr, out[5984]);
      out[5792] = fma(0.1, dr, out[5792]);
      out[5664] = fma(0.22, dr, out[5664]);
      out[5248] = fma(0.5, dr, out[5248]);
      out[4352] = fma(0.45, dr, out[4352]);
    }
    {
      const double dr = ws[47168] * fma(y[5184], v[4736], y[4736] * v[5184]);
      out[4736] = out[4736] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.16, dr, out[6016]);
      out[5984] = fma(0.11, dr, out[5984]);
      out[5792] = fma(0.28, dr, out[5792]);
      out[5216] = fma(0.01, dr, out[5216]);
      out[5664] = fma(0.56, dr, out[5664]);
      out[5856] = fma(0.1, dr, out[5856]);
      out[5248] = fma(0.54, dr, out[5248]);
      out[4352] = fma(0.07, dr, out[4352]);
      out[5696] = fma(0.07, dr, out[5696]);
      out[5760] = fma(0.1, dr, out[5760]);
    }
    {
      const double dr = ws[47200] * fma(y[5184], v[3872], y[3872] * v[5184]);
      out[3872] = out[3872] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.1, dr, out[6016]);
      out[5984] = fma(0.072, dr, out[5984]);
      out[5888] = fma(0.008, dr, out[5888]);
      out[5792] = fma(0.002, dr, out[5792]);
      out[5216] = fma(0.1, dr, out[5216]);
      out[5664] = fma(0.243, dr, out[5664]);
      out[5856] = fma(0.08, dr, out[5856]);
      out[5568] = fma(0.42, dr, out[5568]);
      out[5504] = fma(0.028, dr, out[5504]);
      out[5376] = fma(0.491, dr, out[5376]);
      out[5248] = fma(0.003, dr, out[5248]);
      out[4352] = fma(0.044, dr, out[4352]);
    }
    {
      const double dr = ws[47232] * fma(y[5184], v[5472], y[5472] * v[5184]);
      out[5472] = out[5472] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.05, dr, out[6016]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[4800] = fma(0.6, dr, out[4800]);
      out[5216] = fma(0.6, dr, out[5216]);
      out[5664] = fma(1.5, dr, out[5664]);
      out[5856] = fma(0.05, dr, out[5856]);
      out[5376] = fma(0.05, dr, out[5376]);
      out[5248] = fma(0.08, dr, out[5248]);
      out[5728] = fma(0.65, dr, out[5728]);
    }
    {
      const double dr = ws[47264] * fma(y[5184], v[4320], y[4320] * v[5184]);
      out[4320] = out[4320] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.05, dr, out[6016]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[4800] = fma(0.6, dr, out[4800]);
      out[5216] = fma(0.6, dr, out[5216]);
      out[5664] = fma(1.5, dr, out[5664]);
      out[5856] = fma(0.05, dr, out[5856]);
      out[5376] = fma(0.05, dr, out[5376]);
      out[5248] = fma(0.08, dr, out[5248]);
      out[5472] = fma(0.7, dr, out[5472]);
      out[5728] = fma(0.65, dr, out[5728]);
    }
    {
      const double dr = ws[47296] * fma(y[5184], v[3584], y[3584] * v[5184]);
      out[3584] = out[3584] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.05, dr, out[6016]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5664] = fma(1.5, dr, out[5664]);
      out[5376] = fma(0.48, dr, out[5376]);
      out[5472] = fma(0.7, dr, out[5472]);
      out[4352] = fma(0.25, dr, out[4352]);
      out[5696] = fma(0.25, dr, out[5696]);
      out[3680] = fma(0.11, dr, out[3680]);
    }
    {
      const double dr = ws[47328] * fma(y[5184], v[3808], y[3808] * v[5184]);
      out[3808] = out[3808] - dr;
      out[5184] = out[5184] - dr;
      out[3040] = fma(1.0, dr, out[3040]);
    }
    {
      const double dr = ws[47360] * fma(y[5952], v[2240], y[2240] * v[5952]);
      out[2240] = out[2240] - dr;
      out[5952] = out[5952] - dr;
      out[4032] = fma(0.8, dr, out[4032]);
      out[4064] = fma(0.2, dr, out[4064]);
    }
    {
      const double dr = ws[47392] * fma(y[5952], v[2752], y[2752] * v[5952]);
      out[2752] = out[2752] - dr;
      out[5952] = out[5952] - dr;
      out[4032] = fma(0.43, dr, out[4032]);
      out[4064] = fma(0.57, dr, out[4064]);
    }
    {
      const double dr = ws[47424] * fma(y[5952], v[1152], y[1152] * v[5952]);
      out[1152] = out[1152] - dr;
      out[5952] = out[5952] - dr;
      out[4032] = fma(0.11, dr, out[4032]);
      out[4064] = fma(0.89, dr, out[4064]);
    }
    {
      const double dr = ws[47456] * fma(y[5952], v[1408], y[1408] * v[5952]);
      out[1408] = out[1408] - dr;
      out[5952] = out[5952] - dr;
      out[2624] = fma(0.975, dr, out[2624]);
      out[3840] = fma(0.025, dr, out[3840]);
    }
    {
      const double dr = ws[47488] * fma(y[5952], v[1440], y[1440] * v[5952]);
      out[1440] = out[1440] - dr;
      out[5952] = out[5952] - dr;
      out[2656] = fma(0.945, dr, out[2656]);
      out[3712] = fma(0.055, dr, out[3712]);
    }
    {
      const double dr = ws[47520] * fma(y[5952], v[4384], y[4384] * v[5952]);
      out[4384] = out[4384] - dr;
      out[5952] = out[5952] - dr;
      out[1696] = fma(0.33, dr, out[1696]);
      out[5920] = fma(0.67, dr, out[5920]);
      out[4544] = fma(0.27, dr, out[4544]);
      out[5504] = fma(0.38, dr, out[5504]);
      out[5856] = fma(0.21, dr, out[5856]);
      out[5760] = fma(0.02, dr, out[5760]);
    }
}
__device__ __noinline__ void ddm_jv_1_2(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[47552] * fma(y[5952], v[5856], y[5856] * v[5952]);
      out[5856] = out[5856] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5664] = fma(1.0, dr, out[5664]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[47584] * fma(y[5952], v[5568], y[5568] * v[5952]);
      out[5568] = out[5568] - dr;
      out[5952] = out[5952] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[47616] * fma(y[5952], v[5760], y[5760] * v[5952]);
      out[5760] = out[5760] - dr;
      out[5952] = out[5952] - dr;
      out[4800] = fma(1.0, dr, out[4800]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[47648] * fma(y[5952], v[4128], y[4128] * v[5952]);
      out[4128] = out[4128] - dr;
      out[5952] = out[5952] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[4672] = fma(0.32, dr, out[4672]);
      out[5216] = fma(0.68, dr, out[5216]);
      out[5248] = fma(0.68, dr, out[5248]);
      out[5024] = fma(0.32, dr, out[5024]);
      out[5920] = fma(0.68, dr, out[5920]);
    }
    {
      const double dr = ws[47680] * fma(y[5952], v[3872], y[3872] * v[5952]);
      out[3872] = out[3872] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5216] = fma(1.0, dr, out[5216]);
      out[5664] = fma(0.668, dr, out[5664]);
      out[5856] = fma(0.332, dr, out[5856]);
      out[5760] = fma(0.332, dr, out[5760]);
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[47712] * fma(y[5952], v[5376], y[5376] * v[5952]);
      out[5376] = out[5376] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5664] = fma(2.0, dr, out[5664]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[47744] * fma(y[5952], v[5248], y[5248] * v[5952]);
      out[5248] = out[5248] - dr;
      out[5952] = out[5952] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
      out[5664] = fma(1.0, dr, out[5664]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[47776] * fma(y[5952], v[1248], y[1248] * v[5952]);
      out[1248] = out[1248] - dr;
      out[5952] = out[5952] - dr;
      out[3616] = fma(0.152, dr, out[3616]);
      out[3232] = fma(0.339, dr, out[3232]);
      out[3648] = fma(0.85, dr, out[3648]);
      out[3072] = fma(0.424, dr, out[3072]);
      out[5024] = fma(0.424, dr, out[5024]);
    }
    {
      const double dr = ws[47808] * fma(y[5952], v[2944], y[2944] * v[5952]);
      out[2944] = out[2944] - dr;
      out[5952] = out[5952] - dr;
      out[3616] = fma(0.2, dr, out[3616]);
      out[3232] = fma(0.32, dr, out[3232]);
      out[3648] = fma(0.08, dr, out[3648]);
      out[3072] = fma(0.4, dr, out[3072]);
      out[5024] = fma(0.4, dr, out[5024]);
    }
    {
      const double dr = ws[47840] * fma(y[5952], v[1760], y[1760] * v[5952]);
      out[1760] = out[1760] - dr;
      out[5952] = out[5952] - dr;
      out[3808] = fma(1.0, dr, out[3808]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[47872] * fma(y[5952], v[1824], y[1824] * v[5952]);
      out[1824] = out[1824] - dr;
      out[5952] = out[5952] - dr;
      out[4672] = fma(1.0, dr, out[4672]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[47904] * v[2560];
      out[2560] = out[2560] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[47936] * v[1728];
      out[1728] = out[1728] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[47968] * fma(y[5920], v[5792], y[5792] * v[5920]);
      out[5792] = out[5792] - dr;
      out[5920] = out[5920] - dr;
      out[1088] = fma(1.0, dr, out[1088]);
    }
    {
      const double dr = ws[48000] * v[1088];
      out[1088] = out[1088] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[48032] * fma(y[5920], v[4800], y[4800] * v[5920]);
      out[4800] = out[4800] - dr;
      out[5920] = out[5920] - dr;
      out[1536] = fma(1.0, dr, out[1536]);
    }
    {
      const double dr = ws[48064] * v[1536];
      out[1536] = out[1536] - dr;
      out[4800] = fma(1.0, dr, out[4800]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[48096] * fma(y[5920], v[4672], y[4672] * v[5920]);
      out[4672] = out[4672] - dr;
      out[5920] = out[5920] - dr;
      out[1824] = fma(1.0, dr, out[1824]);
    }
    {
      const double dr = ws[48128] * v[1824];
      out[1824] = out[1824] - dr;
      out[4672] = fma(1.0, dr, out[4672]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[48160] * fma(y[5824], v[5888], y[5888] * v[5824]);
      out[5888] = out[5888] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[48192] * fma(y[5824], v[5632], y[5632] * v[5824]);
      out[5632] = out[5632] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5568] = fma(1.0, dr, out[5568]);
    }
    {
      const double dr = ws[48224] * fma(y[5824], v[5408], y[5408] * v[5824]);
      out[5408] = out[5408] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.66, dr, out[5984]);
      out[5888] = fma(0.131, dr, out[5888]);
      out[5632] = fma(0.048, dr, out[5632]);
      out[5216] = fma(0.089, dr, out[5216]);
      out[5920] = fma(0.935, dr, out[5920]);
      out[5568] = fma(0.504, dr, out[5568]);
      out[5760] = fma(0.132, dr, out[5760]);
      out[4480] = fma(0.165, dr, out[4480]);
      out[5280] = fma(0.042, dr, out[5280]);
      out[5440] = fma(0.065, dr, out[5440]);
    }
    {
      const double dr = ws[48256] * fma(y[5824], v[5120], y[5120] * v[5824]);
      out[5120] = out[5120] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.2, dr, out[5984]);
      out[5888] = fma(0.051, dr, out[5888]);
      out[5632] = fma(0.231, dr, out[5632]);
      out[5216] = fma(0.235, dr, out[5216]);
      out[5920] = fma(0.864, dr, out[5920]);
      out[5856] = fma(0.018, dr, out[5856]);
      out[5568] = fma(0.045, dr, out[5568]);
      out[5760] = fma(0.203, dr, out[5760]);
      out[5280] = fma(0.033, dr, out[5280]);
      out[4480] = fma(0.217, dr, out[4480]);
      out[5504] = fma(0.033, dr, out[5504]);
      out[5344] = fma(0.272, dr, out[5344]);
      out[5440] = fma(0.136, dr, out[5440]);
    }
    {
      const double dr = ws[48288] * fma(y[5824], v[3008], y[3008] * v[5824]);
      out[3008] = out[3008] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(1.6, dr, out[5856]);
      out[5760] = fma(0.2, dr, out[5760]);
    }
    {
      const double dr = ws[48320] * fma(y[5824], v[3200], y[3200] * v[5824]);
      out[3200] = out[3200] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.78, dr, out[5984]);
      out[5920] = fma(0.97, dr, out[5920]);
      out[5856] = fma(0.78, dr, out[5856]);
      out[5568] = fma(0.012, dr, out[5568]);
      out[5760] = fma(0.44, dr, out[5760]);
      out[4480] = fma(0.06, dr, out[4480]);
      out[5280] = fma(0.13, dr, out[5280]);
      out[5440] = fma(0.03, dr, out[5440]);
    }
    {
      const double dr = ws[48352] * fma(y[5824], v[3328], y[3328] * v[5824]);
      out[3328] = out[3328] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.83, dr, out[5984]);
      out[5920] = fma(0.95, dr, out[5920]);
      out[5568] = fma(0.81, dr, out[5568]);
      out[5760] = fma(0.68, dr, out[5760]);
      out[4480] = fma(0.2, dr, out[4480]);
      out[5504] = fma(0.09, dr, out[5504]);
      out[5344] = fma(0.02, dr, out[5344]);
      out[5440] = fma(0.05, dr, out[5440]);
    }
    {
      const double dr = ws[48384] * fma(y[5824], v[3360], y[3360] * v[5824]);
      out[3360] = out[3360] - dr;
      out[5824] = out[5824] - dr;
      out[5440] = fma(0.0, dr, out[5440]);
      out[5312] = fma(0.0012, dr, out[5312]);
      out[4896] = fma(0.0008, dr, out[4896]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[4448] = fma(0.0, dr, out[4448]);
      out[5376] = fma(0.998, dr, out[5376]);
      out[4512] = fma(0.499, dr, out[4512]);
      out[4320] = fma(0.2495, dr, out[4320]);
      out[3584] = fma(0.2495, dr, out[3584]);
    }
    {
      const double dr = ws[48416] * fma(y[5824], v[3296], y[3296] * v[5824]);
      out[3296] = out[3296] - dr;
      out[5824] = out[5824] - dr;
      out[5440] = fma(0.0002, dr, out[5440]);
      out[5312] = fma(0.0013, dr, out[5312]);
      out[4896] = fma(0.0006, dr, out[4896]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[4448] = fma(0.0852, dr, out[4448]);
      out[5376] = fma(0.5477, dr, out[5376]);
      out[5248] = fma(0.3651, dr, out[5248]);
      out[4512] = fma(0.3651, dr, out[4512]);
      out[5472] = fma(0.5477, dr, out[5472]);
    }
    {
      const double dr = ws[48448] * fma(y[5824], v[3104], y[3104] * v[5824]);
      out[3104] = out[3104] - dr;
      out[5824] = out[5824] - dr;
      out[5440] = fma(0.0001, dr, out[5440]);
      out[5536] = fma(0.0013, dr, out[5536]);
      out[4928] = fma(0.0006, dr, out[4928]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[4448] = fma(0.0481, dr, out[4448]);
      out[5376] = fma(0.7029, dr, out[5376]);
      out[5248] = fma(0.247, dr, out[5248]);
      out[4512] = fma(0.3515, dr, out[4512]);
      out[4320] = fma(0.5984, dr, out[4320]);
    }
    {
      const double dr = ws[48480] * fma(y[5824], v[3264], y[3264] * v[5824]);
      out[3264] = out[3264] - dr;
      out[5824] = out[5824] - dr;
      out[5440] = fma(0.0002, dr, out[5440]);
      out[5536] = fma(0.0013, dr, out[5536]);
      out[4928] = fma(0.0006, dr, out[4928]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[4448] = fma(0.0852, dr, out[4448]);
      out[5376] = fma(0.5477, dr, out[5376]);
      out[5248] = fma(0.3651, dr, out[5248]);
      out[4512] = fma(0.4564, dr, out[4512]);
      out[4320] = fma(0.4564, dr, out[4320]);
    }
    {
      const double dr = ws[48512] * fma(y[5824], v[4160], y[4160] * v[5824]);
      out[4160] = out[4160] - dr;
      out[5824] = out[5824] - dr;
      out[4384] = fma(0.237, dr, out[4384]);
      out[5984] = fma(0.763, dr, out[5984]);
      out[5920] = fma(0.763, dr, out[5920]);
      out[4544] = fma(0.195, dr, out[4544]);
      out[5760] = fma(0.284, dr, out[5760]);
      out[4480] = fma(0.0865, dr, out[4480]);
      out[4576] = fma(0.1285, dr, out[4576]);
      out[5856] = fma(0.308, dr, out[5856]);
      out[4096] = fma(0.0715, dr, out[4096]);
      out[5504] = fma(0.084, dr, out[5504]);
    }
    {
      const double dr = ws[48544] * fma(y[5824], v[3744], y[3744] * v[5824]);
      out[3744] = out[3744] - dr;
      out[5824] = out[5824] - dr;
      out[6016] = fma(0.82, dr, out[6016]);
      out[5920] = fma(0.82, dr, out[5920]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[48576] * fma(y[5824], v[2624], y[2624] * v[5824]);
      out[2624] = out[2624] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.6955, dr, out[5920]);
      out[4384] = fma(0.2345, dr, out[4384]);
      out[5440] = fma(0.07, dr, out[5440]);
      out[4544] = fma(0.6045, dr, out[4544]);
      out[5760] = fma(0.154, dr, out[5760]);
      out[5504] = fma(0.007, dr, out[5504]);
      out[5856] = fma(0.007, dr, out[5856]);
      out[5984] = fma(0.1645, dr, out[5984]);
    }
    {
      const double dr = ws[48608] * fma(y[5824], v[3840], y[3840] * v[5824]);
      out[3840] = out[3840] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(0.82, dr, out[5920]);
      out[6016] = fma(0.82, dr, out[6016]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[48640] * fma(y[5824], v[4192], y[4192] * v[5824]);
      out[4192] = out[4192] - dr;
      out[5824] = out[5824] - dr;
      out[4384] = fma(0.23, dr, out[4384]);
      out[5920] = fma(0.77, dr, out[5920]);
      out[4576] = fma(0.77, dr, out[4576]);
      out[5984] = fma(0.77, dr, out[5984]);
      out[5856] = fma(0.43, dr, out[5856]);
    }
    {
      const double dr = ws[48672] * fma(y[5824], v[3936], y[3936] * v[5824]);
      out[3936] = out[3936] - dr;
      out[5824] = out[5824] - dr;
      out[6016] = fma(0.77, dr, out[6016]);
      out[5920] = fma(0.77, dr, out[5920]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[48704] * fma(y[5824], v[2656], y[2656] * v[5824]);
      out[2656] = out[2656] - dr;
      out[5824] = out[5824] - dr;
      out[4384] = fma(0.57, dr, out[4384]);
      out[5440] = fma(0.07, dr, out[5440]);
      out[5920] = fma(1.36, dr, out[5920]);
      out[4576] = fma(0.43, dr, out[4576]);
      out[5984] = fma(0.5, dr, out[5984]);
    }
    {
      const double dr = ws[48736] * fma(y[5824], v[3712], y[3712] * v[5824]);
      out[3712] = out[3712] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(0.77, dr, out[5920]);
      out[6016] = fma(0.77, dr, out[6016]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[48768] * fma(y[5824], v[2560], y[2560] * v[5824]);
      out[2560] = out[2560] - dr;
      out[5824] = out[5824] - dr;
      out[4384] = fma(0.36, dr, out[4384]);
      out[4256] = fma(0.64, dr, out[4256]);
      out[5920] = fma(0.64, dr, out[5920]);
    }
    {
      const double dr = ws[48800] * fma(y[5824], v[1728], y[1728] * v[5824]);
      out[1728] = out[1728] - dr;
      out[5824] = out[5824] - dr;
      out[4384] = fma(0.64, dr, out[4384]);
      out[5920] = fma(0.36, dr, out[5920]);
      out[5984] = fma(0.36, dr, out[5984]);
      out[5856] = fma(0.36, dr, out[5856]);
      out[3680] = fma(0.36, dr, out[3680]);
    }
    {
      const double dr = ws[48832] * fma(y[5824], v[5792], y[5792] * v[5824]);
      out[5792] = out[5792] - dr;
      out[5824] = out[5824] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[48864] * fma(y[5824], v[4800], y[4800] * v[5824]);
      out[4800] = out[4800] - dr;
      out[5824] = out[5824] - dr;
      out[5632] = fma(1.0, dr, out[5632]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[48896] * fma(y[5824], v[2848], y[2848] * v[5824]);
      out[2848] = out[2848] - dr;
      out[5824] = out[5824] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[48928] * fma(y[5824], v[5152], y[5152] * v[5824]);
      out[5152] = out[5152] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.67, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.33, dr, out[5856]);
      out[5472] = fma(0.67, dr, out[5472]);
    }
    {
      const double dr = ws[48960] * fma(y[5824], v[3776], y[3776] * v[5824]);
      out[3776] = out[3776] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.77, dr, out[5984]);
      out[5792] = fma(0.23, dr, out[5792]);
      out[5216] = fma(0.16, dr, out[5216]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5760] = fma(0.46, dr, out[5760]);
      out[5248] = fma(0.54, dr, out[5248]);
    }
    {
      const double dr = ws[48992] * fma(y[5824], v[4672], y[4672] * v[5824]);
      out[4672] = out[4672] - dr;
      out[5824] = out[5824] - dr;
      out[5888] = fma(0.65, dr, out[5888]);
      out[5792] = fma(0.35, dr, out[5792]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5664] = fma(0.65, dr, out[5664]);
      out[5856] = fma(0.65, dr, out[5856]);
    }
    {
      const double dr = ws[49024] * fma(y[5824], v[3520], y[3520] * v[5824]);
      out[3520] = out[3520] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.5, dr, out[5984]);
      out[5856] = fma(0.5, dr, out[5856]);
      out[5344] = fma(1.0, dr, out[5344]);
    }
    {
      const double dr = ws[49056] * fma(y[5824], v[2880], y[2880] * v[5824]);
      out[2880] = out[2880] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.3, dr, out[5984]);
      out[5792] = fma(0.7, dr, out[5792]);
      out[5216] = fma(0.7, dr, out[5216]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.3, dr, out[5856]);
      out[5760] = fma(0.7, dr, out[5760]);
      out[5248] = fma(0.3, dr, out[5248]);
    }
    {
      const double dr = ws[49088] * fma(y[5824], v[2912], y[2912] * v[5824]);
      out[2912] = out[2912] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5664] = fma(0.61, dr, out[5664]);
      out[5856] = fma(0.03, dr, out[5856]);
      out[5760] = fma(0.27, dr, out[5760]);
      out[5376] = fma(0.18, dr, out[5376]);
      out[5504] = fma(0.7, dr, out[5504]);
      out[5248] = fma(0.21, dr, out[5248]);
    }
    {
      const double dr = ws[49120] * fma(y[5824], v[2592], y[2592] * v[5824]);
      out[2592] = out[2592] - dr;
      out[5824] = out[5824] - dr;
      out[2272] = fma(1.0, dr, out[2272]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[49152] * fma(y[5824], v[2272], y[2272] * v[5824]);
      out[2272] = out[2272] - dr;
      out[5824] = out[5824] - dr;
      out[2688] = fma(1.0, dr, out[2688]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[49184] * fma(y[5824], v[3648], y[3648] * v[5824]);
      out[3648] = out[3648] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5344] = fma(0.32, dr, out[5344]);
      out[5376] = fma(0.68, dr, out[5376]);
      out[5728] = fma(0.68, dr, out[5728]);
    }
    {
      const double dr = ws[49216] * fma(y[5824], v[3040], y[3040] * v[5824]);
      out[3040] = out[3040] - dr;
      out[5824] = out[5824] - dr;
      out[3808] = fma(1.0, dr, out[3808]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
}
__device__ __noinline__ void ddm_jv_1_3(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[49248] * fma(y[5824], v[2976], y[2976] * v[5824]);
      out[2976] = out[2976] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[49280] * fma(y[5824], v[4032], y[4032] * v[5824]);
      out[4032] = out[4032] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[49312] * fma(y[5824], v[4064], y[4064] * v[5824]);
      out[4064] = out[4064] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
      out[5856] = fma(0.287, dr, out[5856]);
      out[5760] = fma(1.24, dr, out[5760]);
      out[5504] = fma(0.464, dr, out[5504]);
    }
    {
      const double dr = ws[49344] * fma(y[5824], v[3072], y[3072] * v[5824]);
      out[3072] = out[3072] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49376] * fma(y[5824], v[5216], y[5216] * v[5824]);
      out[5216] = out[5216] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[49408] * fma(y[5920], v[2688], y[2688] * v[5920]);
      out[2688] = out[2688] - dr;
      out[5920] = out[5920] - dr;
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[49440] * fma(y[5920], v[3232], y[3232] * v[5920]);
      out[3232] = out[3232] - dr;
      out[5920] = out[5920] - dr;
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[49472] * fma(y[5920], v[3808], y[3808] * v[5920]);
      out[3808] = out[3808] - dr;
      out[5920] = out[5920] - dr;
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[49504] * fma(y[5984], v[5888], y[5888] * v[5984]);
      out[5888] = out[5888] - dr;
      out[5984] = out[5984] - dr;
      out[2816] = fma(1.0, dr, out[2816]);
    }
    {
      const double dr = ws[49536] * fma(y[5984], v[5632], y[5632] * v[5984]);
      out[5632] = out[5632] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49568] * fma(y[5984], v[5408], y[5408] * v[5984]);
      out[5408] = out[5408] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49600] * fma(y[5984], v[5120], y[5120] * v[5984]);
      out[5120] = out[5120] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49632] * fma(y[5984], v[3008], y[3008] * v[5984]);
      out[3008] = out[3008] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49664] * fma(y[5984], v[3200], y[3200] * v[5984]);
      out[3200] = out[3200] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49696] * fma(y[5984], v[3328], y[3328] * v[5984]);
      out[3328] = out[3328] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[49728] * fma(y[5984], v[3360], y[3360] * v[5984]);
      out[3360] = out[3360] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(0.6021, dr, out[5728]);
      out[4896] = fma(0.3979, dr, out[4896]);
    }
    {
      const double dr = ws[49760] * fma(y[5984], v[3296], y[3296] * v[5984]);
      out[3296] = out[3296] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(0.7195, dr, out[5728]);
      out[4896] = fma(0.2805, dr, out[4896]);
    }
    {
      const double dr = ws[49792] * fma(y[5984], v[3104], y[3104] * v[5984]);
      out[3104] = out[3104] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(0.0482, dr, out[5728]);
      out[4608] = fma(0.6747, dr, out[4608]);
      out[4928] = fma(0.2771, dr, out[4928]);
    }
    {
      const double dr = ws[49824] * fma(y[5984], v[3264], y[3264] * v[5984]);
      out[3264] = out[3264] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(0.0854, dr, out[5728]);
      out[4608] = fma(0.6341, dr, out[4608]);
      out[4928] = fma(0.2805, dr, out[4928]);
    }
    {
      const double dr = ws[49856] * fma(y[5984], v[4160], y[4160] * v[5984]);
      out[4160] = out[4160] - dr;
      out[5984] = out[5984] - dr;
      out[4480] = fma(0.039, dr, out[4480]);
      out[4576] = fma(0.039, dr, out[4576]);
      out[5856] = fma(0.0625, dr, out[5856]);
      out[4096] = fma(0.762, dr, out[4096]);
      out[5984] = fma(0.3225, dr, out[5984]);
      out[4544] = fma(0.1885, dr, out[4544]);
      out[6016] = fma(0.238, dr, out[6016]);
      out[5504] = fma(0.0105, dr, out[5504]);
    }
    {
      const double dr = ws[49888] * fma(y[5984], v[3744], y[3744] * v[5984]);
      out[3744] = out[3744] - dr;
      out[5984] = out[5984] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[49920] * fma(y[5984], v[2624], y[2624] * v[5984]);
      out[2624] = out[2624] - dr;
      out[5984] = out[5984] - dr;
      out[4384] = fma(0.461, dr, out[4384]);
      out[4544] = fma(0.455, dr, out[4544]);
      out[5920] = fma(0.539, dr, out[5920]);
      out[6016] = fma(0.6195, dr, out[6016]);
      out[5760] = fma(0.077, dr, out[5760]);
      out[5504] = fma(0.007, dr, out[5504]);
      out[5856] = fma(0.007, dr, out[5856]);
    }
    {
      const double dr = ws[49952] * fma(y[5984], v[3840], y[3840] * v[5984]);
      out[3840] = out[3840] - dr;
      out[5984] = out[5984] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[49984] * fma(y[5984], v[4192], y[4192] * v[5984]);
      out[4192] = out[4192] - dr;
      out[5984] = out[5984] - dr;
      out[4096] = fma(0.9, dr, out[4096]);
      out[4576] = fma(0.1, dr, out[4576]);
      out[6016] = fma(0.1, dr, out[6016]);
      out[5984] = fma(0.1, dr, out[5984]);
      out[5856] = fma(0.06, dr, out[5856]);
    }
    {
      const double dr = ws[50016] * fma(y[5984], v[3936], y[3936] * v[5984]);
      out[3936] = out[3936] - dr;
      out[5984] = out[5984] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[50048] * fma(y[5984], v[2656], y[2656] * v[5984]);
      out[2656] = out[2656] - dr;
      out[5984] = out[5984] - dr;
      out[4384] = fma(0.77, dr, out[4384]);
      out[6016] = fma(0.5, dr, out[6016]);
      out[4576] = fma(0.23, dr, out[4576]);
      out[5920] = fma(0.23, dr, out[5920]);
      out[5984] = fma(0.27, dr, out[5984]);
    }
    {
      const double dr = ws[50080] * fma(y[5984], v[3712], y[3712] * v[5984]);
      out[3712] = out[3712] - dr;
      out[5984] = out[5984] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[50112] * fma(y[5984], v[2560], y[2560] * v[5984]);
      out[2560] = out[2560] - dr;
      out[5984] = out[5984] - dr;
      out[4096] = fma(0.75, dr, out[4096]);
      out[6016] = fma(0.25, dr, out[6016]);
      out[4256] = fma(0.25, dr, out[4256]);
    }
    {
      const double dr = ws[50144] * fma(y[5984], v[1728], y[1728] * v[5984]);
      out[1728] = out[1728] - dr;
      out[5984] = out[5984] - dr;
      out[4096] = fma(0.9, dr, out[4096]);
      out[6016] = fma(0.1, dr, out[6016]);
      out[5984] = fma(0.1, dr, out[5984]);
      out[5856] = fma(0.1, dr, out[5856]);
      out[3680] = fma(0.1, dr, out[3680]);
    }
    {
      const double dr = ws[50176] * fma(y[5984], v[5792], y[5792] * v[5984]);
      out[5792] = out[5792] - dr;
      out[5984] = out[5984] - dr;
      out[6016] = fma(0.44, dr, out[6016]);
      out[5888] = fma(0.44, dr, out[5888]);
      out[5696] = fma(0.15, dr, out[5696]);
      out[3680] = fma(0.41, dr, out[3680]);
    }
    {
      const double dr = ws[50208] * fma(y[5984], v[4800], y[4800] * v[5984]);
      out[4800] = out[4800] - dr;
      out[5984] = out[5984] - dr;
      out[6016] = fma(0.44, dr, out[6016]);
      out[5632] = fma(0.44, dr, out[5632]);
      out[5696] = fma(0.15, dr, out[5696]);
      out[3680] = fma(0.41, dr, out[3680]);
    }
    {
      const double dr = ws[50240] * fma(y[5984], v[2848], y[2848] * v[5984]);
      out[2848] = out[2848] - dr;
      out[5984] = out[5984] - dr;
      out[6016] = fma(0.15, dr, out[6016]);
      out[5792] = fma(0.15, dr, out[5792]);
      out[5856] = fma(0.15, dr, out[5856]);
      out[5728] = fma(0.85, dr, out[5728]);
    }
    {
      const double dr = ws[50272] * fma(y[5984], v[5152], y[5152] * v[5984]);
      out[5152] = out[5152] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50304] * fma(y[5984], v[3776], y[3776] * v[5984]);
      out[3776] = out[3776] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50336] * fma(y[5984], v[4672], y[4672] * v[5984]);
      out[4672] = out[4672] - dr;
      out[5984] = out[5984] - dr;
      out[1792] = fma(1.0, dr, out[1792]);
    }
    {
      const double dr = ws[50368] * fma(y[5984], v[3520], y[3520] * v[5984]);
      out[3520] = out[3520] - dr;
      out[5984] = out[5984] - dr;
      out[1792] = fma(1.0, dr, out[1792]);
    }
    {
      const double dr = ws[50400] * fma(y[5984], v[2880], y[2880] * v[5984]);
      out[2880] = out[2880] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50432] * fma(y[5984], v[2912], y[2912] * v[5984]);
      out[2912] = out[2912] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50464] * fma(y[5984], v[3648], y[3648] * v[5984]);
      out[3648] = out[3648] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50496] * fma(y[5984], v[3232], y[3232] * v[5984]);
      out[3232] = out[3232] - dr;
      out[5984] = out[5984] - dr;
      out[2944] = fma(1.0, dr, out[2944]);
    }
    {
      const double dr = ws[50528] * fma(y[5984], v[3040], y[3040] * v[5984]);
      out[3040] = out[3040] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50560] * fma(y[5984], v[2976], y[2976] * v[5984]);
      out[2976] = out[2976] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50592] * fma(y[5984], v[4032], y[4032] * v[5984]);
      out[4032] = out[4032] - dr;
      out[5984] = out[5984] - dr;
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[50624] * fma(y[5984], v[4064], y[4064] * v[5984]);
      out[4064] = out[4064] - dr;
      out[5984] = out[5984] - dr;
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[50656] * fma(y[5984], v[3072], y[3072] * v[5984]);
      out[3072] = out[3072] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50688] * fma(y[5984], v[5216], y[5216] * v[5984]);
      out[5216] = out[5216] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[50720] * fma(y[5888], v[5888], y[5888] * v[5888]);
      out[5888] = out[5888] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.74, dr, out[5984]);
      out[5856] = fma(1.37, dr, out[5856]);
      out[5600] = fma(0.63, dr, out[5600]);
    }
    {
      const double dr = ws[50752] * fma(y[5888], v[5632], y[5632] * v[5888]);
      out[5632] = out[5632] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[5568] = fma(0.75, dr, out[5568]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[1472] = fma(0.25, dr, out[1472]);
    }
    {
      const double dr = ws[50784] * fma(y[5888], v[5408], y[5408] * v[5888]);
      out[5408] = out[5408] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.894, dr, out[5984]);
      out[5888] = fma(0.08, dr, out[5888]);
      out[5632] = fma(0.026, dr, out[5632]);
      out[5216] = fma(0.026, dr, out[5216]);
      out[5856] = fma(0.827, dr, out[5856]);
      out[5760] = fma(0.198, dr, out[5760]);
      out[5504] = fma(0.497, dr, out[5504]);
      out[5376] = fma(0.05, dr, out[5376]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[50816] * fma(y[5888], v[5120], y[5120] * v[5888]);
      out[5120] = out[5120] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.842, dr, out[5984]);
      out[5888] = fma(0.018, dr, out[5888]);
      out[5632] = fma(0.14, dr, out[5632]);
      out[5216] = fma(0.191, dr, out[5216]);
      out[5856] = fma(0.777, dr, out[5856]);
      out[5760] = fma(0.251, dr, out[5760]);
      out[5504] = fma(0.618, dr, out[5504]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[50848] * fma(y[5888], v[3008], y[3008] * v[5888]);
      out[3008] = out[3008] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.95, dr, out[5856]);
      out[5760] = fma(0.15, dr, out[5760]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[1504] = fma(0.25, dr, out[1504]);
    }
    {
      const double dr = ws[50880] * fma(y[5888], v[3200], y[3200] * v[5888]);
      out[3200] = out[3200] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.5, dr, out[5856]);
      out[5760] = fma(0.705, dr, out[5760]);
      out[5504] = fma(0.045, dr, out[5504]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[50912] * fma(y[5888], v[3328], y[3328] * v[5888]);
      out[3328] = out[3328] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[5760] = fma(1.28, dr, out[5760]);
      out[5504] = fma(0.218, dr, out[5504]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[50944] * fma(y[5888], v[3360], y[3360] * v[5888]);
      out[3360] = out[3360] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[5984] = fma(1.37, dr, out[5984]);
      out[5600] = fma(0.32, dr, out[5600]);
      out[4448] = fma(0.0, dr, out[4448]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[4512] = fma(0.5, dr, out[4512]);
      out[4320] = fma(0.25, dr, out[4320]);
      out[3584] = fma(0.25, dr, out[3584]);
    }
    {
      const double dr = ws[50976] * fma(y[5888], v[3296], y[3296] * v[5888]);
      out[3296] = out[3296] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[5984] = fma(1.2846, dr, out[5984]);
      out[5600] = fma(0.32, dr, out[5600]);
      out[4448] = fma(0.0854, dr, out[4448]);
      out[5376] = fma(0.5488, dr, out[5376]);
      out[5248] = fma(0.3659, dr, out[5248]);
      out[4512] = fma(0.3659, dr, out[4512]);
      out[5472] = fma(0.5488, dr, out[5472]);
    }
    {
      const double dr = ws[51008] * fma(y[5888], v[3104], y[3104] * v[5888]);
      out[3104] = out[3104] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[5984] = fma(1.3218, dr, out[5984]);
      out[5600] = fma(0.32, dr, out[5600]);
      out[4448] = fma(0.0482, dr, out[4448]);
      out[5376] = fma(0.7043, dr, out[5376]);
      out[5248] = fma(0.2475, dr, out[5248]);
      out[4512] = fma(0.3522, dr, out[4512]);
      out[4320] = fma(0.5996, dr, out[4320]);
    }
    {
      const double dr = ws[51040] * fma(y[5888], v[3264], y[3264] * v[5888]);
      out[3264] = out[3264] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[5984] = fma(1.2846, dr, out[5984]);
      out[5600] = fma(0.32, dr, out[5600]);
      out[4448] = fma(0.0854, dr, out[4448]);
      out[5376] = fma(0.5488, dr, out[5376]);
      out[5248] = fma(0.3659, dr, out[5248]);
      out[4512] = fma(0.4573, dr, out[4512]);
      out[4320] = fma(0.4573, dr, out[4320]);
    }
    {
      const double dr = ws[51072] * fma(y[5888], v[4288], y[4288] * v[5888]);
      out[4288] = out[4288] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.31, dr, out[5856]);
      out[4128] = fma(0.159, dr, out[4128]);
      out[4736] = fma(0.25, dr, out[4736]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
      out[5760] = fma(0.023, dr, out[5760]);
      out[5376] = fma(0.018, dr, out[5376]);
      out[5344] = fma(0.016, dr, out[5344]);
    }
    {
      const double dr = ws[51104] * fma(y[5888], v[4160], y[4160] * v[5888]);
      out[4160] = out[4160] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(1.0295, dr, out[5856]);
      out[4576] = fma(0.2205, dr, out[4576]);
      out[4544] = fma(0.273, dr, out[4544]);
      out[5760] = fma(0.2385, dr, out[5760]);
      out[4096] = fma(0.0845, dr, out[4096]);
      out[5600] = fma(0.1105, dr, out[5600]);
      out[5504] = fma(0.1835, dr, out[5504]);
      out[4480] = fma(0.067, dr, out[4480]);
      out[5984] = fma(1.279, dr, out[5984]);
    }
    {
      const double dr = ws[51136] * fma(y[5888], v[3744], y[3744] * v[5888]);
      out[3744] = out[3744] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
}
}  // namespace mech_cracmm2
