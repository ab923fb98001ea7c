// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void solve_0_0(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 105440;
    const double* __restrict__ vd = ws + 210560;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[0];
      b[0] = x;
    }
    {
      double x = b[32];
      b[32] = x;
    }
    {
      double x = b[64];
      b[64] = x;
    }
    {
      double x = b[96];
      b[96] = x;
    }
    {
      double x = b[128];
      b[128] = x;
    }
    {
      double x = b[160];
      b[160] = x;
    }
    {
      double x = b[192];
      x = fma(-lu[32], b[160], x);
      b[192] = x;
    }
    {
      double x = b[224];
      x = fma(-lu[64], b[160], x);
      b[224] = x;
    }
    {
      double x = b[256];
      b[256] = x;
    }
    {
      double x = b[288];
      b[288] = x;
    }
    {
      double x = b[320];
      b[320] = x;
    }
    {
      double x = b[352];
      b[352] = x;
    }
    {
      double x = b[384];
      b[384] = x;
    }
    {
      double x = b[416];
      b[416] = x;
    }
    {
      double x = b[448];
      b[448] = x;
    }
    {
      double x = b[480];
      b[480] = x;
    }
    {
      double x = b[512];
      b[512] = x;
    }
    {
      double x = b[544];
      x = fma(-lu[96], b[512], x);
      b[544] = x;
    }
    {
      double x = b[576];
      b[576] = x;
    }
    {
      double x = b[608];
      b[608] = x;
    }
    {
      double x = b[640];
      b[640] = x;
    }
    {
      double x = b[672];
      b[672] = x;
    }
    {
      double x = b[704];
      b[704] = x;
    }
    {
      double x = b[736];
      b[736] = x;
    }
    {
      double x = b[768];
      b[768] = x;
    }
    {
      double x = b[800];
      b[800] = x;
    }
    {
      double x = b[832];
      b[832] = x;
    }
    {
      double x = b[864];
      b[864] = x;
    }
    {
      double x = b[896];
      b[896] = x;
    }
    {
      double x = b[928];
      b[928] = x;
    }
    {
      double x = b[960];
      x = fma(-lu[128], b[96], x);
      x = fma(-lu[160], b[128], x);
      b[960] = x;
    }
    {
      double x = b[992];
      b[992] = x;
    }
    {
      double x = b[1024];
      b[1024] = x;
    }
    {
      double x = b[1056];
      x = fma(-lu[192], b[512], x);
      b[1056] = x;
    }
    {
      double x = b[1088];
      b[1088] = x;
    }
    {
      double x = b[1120];
      b[1120] = x;
    }
    {
      double x = b[1152];
      b[1152] = x;
    }
    {
      double x = b[1184];
      b[1184] = x;
    }
    {
      double x = b[1216];
      b[1216] = x;
    }
    {
      double x = b[1248];
      x = fma(-lu[224], b[1216], x);
      b[1248] = x;
    }
    {
      double x = b[1280];
      b[1280] = x;
    }
    {
      double x = b[1312];
      b[1312] = x;
    }
    {
      double x = b[1344];
      b[1344] = x;
    }
    {
      double x = b[1376];
      x = fma(-lu[256], b[1344], x);
      b[1376] = x;
    }
    {
      double x = b[1408];
      b[1408] = x;
    }
    {
      double x = b[1440];
      b[1440] = x;
    }
    {
      double x = b[1472];
      b[1472] = x;
    }
    {
      double x = b[1504];
      b[1504] = x;
    }
    {
      double x = b[1536];
      b[1536] = x;
    }
    {
      double x = b[1568];
      b[1568] = x;
    }
    {
      double x = b[1600];
      b[1600] = x;
    }
    {
      double x = b[1632];
      x = fma(-lu[288], b[1312], x);
      b[1632] = x;
    }
    {
      double x = b[1664];
      x = fma(-lu[320], b[1344], x);
      x = fma(-lu[352], b[1632], x);
      b[1664] = x;
    }
    {
      double x = b[1696];
      b[1696] = x;
    }
    {
      double x = b[1728];
      b[1728] = x;
    }
    {
      double x = b[1760];
      x = fma(-lu[384], b[1248], x);
      b[1760] = x;
    }
    {
      double x = b[1792];
      b[1792] = x;
    }
    {
      double x = b[1824];
      b[1824] = x;
    }
    {
      double x = b[1856];
      b[1856] = x;
    }
    {
      double x = b[1888];
      x = fma(-lu[416], b[1152], x);
      b[1888] = x;
    }
    {
      double x = b[1920];
      x = fma(-lu[448], b[1600], x);
      b[1920] = x;
    }
    {
      double x = b[1952];
      b[1952] = x;
    }
    {
      double x = b[1984];
      b[1984] = x;
    }
    {
      double x = b[2016];
      b[2016] = x;
    }
    {
      double x = b[2048];
      b[2048] = x;
    }
    {
      double x = b[2080];
      b[2080] = x;
    }
    {
      double x = b[2112];
      b[2112] = x;
    }
    {
      double x = b[2144];
      b[2144] = x;
    }
    {
      double x = b[2176];
      x = fma(-lu[480], b[1152], x);
      x = fma(-lu[512], b[1408], x);
      b[2176] = x;
    }
    {
      double x = b[2208];
      x = fma(-lu[544], b[1632], x);
      b[2208] = x;
    }
    {
      double x = b[2240];
      x = fma(-lu[576], b[1568], x);
      b[2240] = x;
    }
    {
      double x = b[2272];
      b[2272] = x;
    }
    {
      double x = b[2304];
      x = fma(-lu[608], b[1600], x);
      b[2304] = x;
    }
    {
      double x = b[2336];
      x = fma(-lu[640], b[576], x);
      b[2336] = x;
    }
    {
      double x = b[2368];
      x = fma(-lu[672], b[608], x);
      b[2368] = x;
    }
    {
      double x = b[2400];
      x = fma(-lu[704], b[640], x);
      b[2400] = x;
    }
    {
      double x = b[2432];
      x = fma(-lu[736], b[672], x);
      b[2432] = x;
    }
    {
      double x = b[2464];
      x = fma(-lu[768], b[704], x);
      b[2464] = x;
    }
    {
      double x = b[2496];
      x = fma(-lu[800], b[736], x);
      b[2496] = x;
    }
    {
      double x = b[2528];
      x = fma(-lu[832], b[768], x);
      b[2528] = x;
    }
    {
      double x = b[2560];
      x = fma(-lu[864], b[1408], x);
      b[2560] = x;
    }
    {
      double x = b[2592];
      b[2592] = x;
    }
    {
      double x = b[2624];
      x = fma(-lu[896], b[1408], x);
      b[2624] = x;
    }
    {
      double x = b[2656];
      x = fma(-lu[928], b[1440], x);
      b[2656] = x;
    }
    {
      double x = b[2688];
      x = fma(-lu[960], b[2272], x);
      x = fma(-lu[992], b[2592], x);
      b[2688] = x;
    }
    {
      double x = b[2720];
      b[2720] = x;
    }
    {
      double x = b[2752];
      x = fma(-lu[1024], b[1312], x);
      b[2752] = x;
    }
    {
      double x = b[2784];
      x = fma(-lu[1056], b[1312], x);
      x = fma(-lu[1088], b[1632], x);
      b[2784] = x;
    }
    {
      double x = b[2816];
      x = fma(-lu[1120], b[1408], x);
      b[2816] = x;
    }
    {
      double x = b[2848];
      b[2848] = x;
    }
    {
      double x = b[2880];
      b[2880] = x;
    }
    {
      double x = b[2912];
      b[2912] = x;
    }
    {
      double x = b[2944];
      x = fma(-lu[1152], b[288], x);
      x = fma(-lu[1184], b[320], x);
      x = fma(-lu[1216], b[352], x);
      b[2944] = x;
    }
    {
      double x = b[2976];
      b[2976] = x;
    }
    {
      double x = b[3008];
      x = fma(-lu[1248], b[2240], x);
      b[3008] = x;
    }
    {
      double x = b[3040];
      b[3040] = x;
    }
    {
      double x = b[3072];
      x = fma(-lu[1280], b[1248], x);
      x = fma(-lu[1312], b[2752], x);
      x = fma(-lu[1344], b[2944], x);
      b[3072] = x;
    }
    {
      double x = b[3104];
      x = fma(-lu[1376], b[320], x);
      b[3104] = x;
    }
    {
      double x = b[3136];
      x = fma(-lu[1408], b[1568], x);
      b[3136] = x;
    }
    {
      double x = b[3168];
      x = fma(-lu[1440], b[3136], x);
      b[3168] = x;
    }
    {
      double x = b[3200];
      x = fma(-lu[1472], b[2752], x);
      x = fma(-lu[1504], b[3136], x);
      b[3200] = x;
    }
    {
      double x = b[3232];
      x = fma(-lu[1536], b[1248], x);
      x = fma(-lu[1568], b[2752], x);
      x = fma(-lu[1600], b[2944], x);
      x = fma(-lu[1632], b[3136], x);
      b[3232] = x;
    }
    {
      double x = b[3264];
      x = fma(-lu[1664], b[352], x);
      b[3264] = x;
    }
    {
      double x = b[3296];
      x = fma(-lu[1696], b[288], x);
      b[3296] = x;
    }
    {
      double x = b[3328];
      x = fma(-lu[1728], b[1152], x);
      b[3328] = x;
    }
    {
      double x = b[3360];
      x = fma(-lu[1760], b[1216], x);
      x = fma(-lu[1792], b[2752], x);
      x = fma(-lu[1824], b[3136], x);
      b[3360] = x;
    }
    {
      double x = b[3392];
      x = fma(-lu[1856], b[832], x);
      b[3392] = x;
    }
    {
      double x = b[3424];
      x = fma(-lu[1888], b[864], x);
      b[3424] = x;
    }
    {
      double x = b[3456];
      x = fma(-lu[1920], b[896], x);
      b[3456] = x;
    }
    {
      double x = b[3488];
      x = fma(-lu[1952], b[992], x);
      b[3488] = x;
    }
    {
      double x = b[3520];
      b[3520] = x;
    }
    {
      double x = b[3552];
      x = fma(-lu[1984], b[1568], x);
      x = fma(-lu[2016], b[3136], x);
      b[3552] = x;
    }
    {
      double x = b[3584];
      x = fma(-lu[2048], b[3168], x);
      x = fma(-lu[2080], b[3360], x);
      b[3584] = x;
    }
    {
      double x = b[3616];
      x = fma(-lu[2112], b[384], x);
      x = fma(-lu[2144], b[416], x);
      x = fma(-lu[2176], b[1120], x);
      x = fma(-lu[2208], b[1248], x);
      x = fma(-lu[2240], b[2176], x);
      x = fma(-lu[2272], b[2752], x);
      x = fma(-lu[2304], b[2944], x);
      x = fma(-lu[2336], b[3136], x);
      x = fma(-lu[2368], b[3232], x);
      b[3616] = x;
    }
    {
      double x = b[3648];
      x = fma(-lu[2400], b[1248], x);
      x = fma(-lu[2432], b[2752], x);
      x = fma(-lu[2464], b[2944], x);
      x = fma(-lu[2496], b[3136], x);
      x = fma(-lu[2528], b[3232], x);
      b[3648] = x;
    }
    {
      double x = b[3680];
      x = fma(-lu[2560], b[1728], x);
      x = fma(-lu[2592], b[3584], x);
      b[3680] = x;
    }
    {
      double x = b[3712];
      x = fma(-lu[2624], b[1440], x);
      b[3712] = x;
    }
    {
      double x = b[3744];
      x = fma(-lu[2656], b[1408], x);
      b[3744] = x;
    }
    {
      double x = b[3776];
      b[3776] = x;
    }
    {
      double x = b[3808];
      x = fma(-lu[2688], b[1760], x);
      x = fma(-lu[2720], b[2752], x);
      x = fma(-lu[2752], b[2944], x);
      x = fma(-lu[2784], b[3040], x);
      x = fma(-lu[2816], b[3136], x);
      x = fma(-lu[2848], b[3232], x);
      b[3808] = x;
    }
    {
      double x = b[3840];
      x = fma(-lu[2880], b[1408], x);
      b[3840] = x;
    }
    {
      double x = b[3872];
      x = fma(-lu[2912], b[1568], x);
      x = fma(-lu[2944], b[3136], x);
      b[3872] = x;
    }
    {
      double x = b[3904];
      x = fma(-lu[2976], b[800], x);
      b[3904] = x;
    }
    {
      double x = b[3936];
      x = fma(-lu[3008], b[1440], x);
      b[3936] = x;
    }
    {
      double x = b[3968];
      b[3968] = x;
    }
    {
      double x = b[4000];
      x = fma(-lu[3040], b[1152], x);
      x = fma(-lu[3072], b[1312], x);
      x = fma(-lu[3104], b[1408], x);
      x = fma(-lu[3136], b[1440], x);
      x = fma(-lu[3168], b[2752], x);
      x = fma(-lu[3200], b[3136], x);
      b[4000] = x;
    }
    {
      double x = b[4032];
      x = fma(-lu[3232], b[1152], x);
      x = fma(-lu[3264], b[1568], x);
      x = fma(-lu[3296], b[2240], x);
      x = fma(-lu[3328], b[2752], x);
      x = fma(-lu[3360], b[3136], x);
      x = fma(-lu[3392], b[3552], x);
      b[4032] = x;
    }
    {
      double x = b[4064];
      x = fma(-lu[3424], b[1152], x);
      x = fma(-lu[3456], b[1568], x);
      x = fma(-lu[3488], b[2240], x);
      x = fma(-lu[3520], b[2752], x);
      x = fma(-lu[3552], b[3136], x);
      x = fma(-lu[3584], b[3552], x);
      x = fma(-lu[3616], b[4032], x);
      b[4064] = x;
    }
    {
      double x = b[4096];
      x = fma(-lu[3648], b[1728], x);
      x = fma(-lu[3680], b[2560], x);
      b[4096] = x;
    }
    {
      double x = b[4128];
      x = fma(-lu[3712], b[1312], x);
      x = fma(-lu[3744], b[1344], x);
      x = fma(-lu[3776], b[1664], x);
      b[4128] = x;
    }
    {
      double x = b[4160];
      x = fma(-lu[3808], b[1408], x);
      x = fma(-lu[3840], b[3712], x);
      x = fma(-lu[3872], b[3744], x);
      x = fma(-lu[3904], b[3840], x);
      x = fma(-lu[3936], b[3936], x);
      b[4160] = x;
    }
    {
      double x = b[4192];
      x = fma(-lu[3968], b[1440], x);
      x = fma(-lu[4000], b[3712], x);
      x = fma(-lu[4032], b[3744], x);
      x = fma(-lu[4064], b[3840], x);
      x = fma(-lu[4096], b[3936], x);
      x = fma(-lu[4128], b[4160], x);
      b[4192] = x;
    }
    {
      double x = b[4224];
      x = fma(-lu[4160], b[3968], x);
      b[4224] = x;
    }
    {
      double x = b[4256];
      x = fma(-lu[4192], b[1728], x);
      x = fma(-lu[4224], b[2560], x);
      x = fma(-lu[4256], b[3712], x);
      x = fma(-lu[4288], b[3744], x);
      x = fma(-lu[4320], b[3840], x);
      x = fma(-lu[4352], b[3936], x);
      x = fma(-lu[4384], b[4160], x);
      x = fma(-lu[4416], b[4192], x);
      b[4256] = x;
    }
    {
      double x = b[4288];
      x = fma(-lu[4448], b[1312], x);
      x = fma(-lu[4480], b[1344], x);
      x = fma(-lu[4512], b[3712], x);
      x = fma(-lu[4544], b[3744], x);
      x = fma(-lu[4576], b[3840], x);
      x = fma(-lu[4608], b[3936], x);
      x = fma(-lu[4640], b[4160], x);
      x = fma(-lu[4672], b[4192], x);
      b[4288] = x;
    }
    {
      double x = b[4320];
      x = fma(-lu[4704], b[3104], x);
      x = fma(-lu[4736], b[3264], x);
      x = fma(-lu[4768], b[3360], x);
      x = fma(-lu[4800], b[3392], x);
      x = fma(-lu[4832], b[3424], x);
      x = fma(-lu[4864], b[3456], x);
      b[4320] = x;
    }
    {
      double x = b[4352];
      x = fma(-lu[4896], b[256], x);
      x = fma(-lu[4928], b[1312], x);
      x = fma(-lu[4960], b[1408], x);
      x = fma(-lu[4992], b[2240], x);
      x = fma(-lu[5024], b[2752], x);
      x = fma(-lu[5056], b[3136], x);
      x = fma(-lu[5088], b[3552], x);
      x = fma(-lu[5120], b[3584], x);
      x = fma(-lu[5152], b[3872], x);
      x = fma(-lu[5184], b[4128], x);
      x = fma(-lu[5216], b[4288], x);
      b[4352] = x;
    }
    {
      double x = b[4384];
      x = fma(-lu[5248], b[1728], x);
      x = fma(-lu[5280], b[2560], x);
      x = fma(-lu[5312], b[2624], x);
      x = fma(-lu[5344], b[2656], x);
      x = fma(-lu[5376], b[4160], x);
      x = fma(-lu[5408], b[4192], x);
      x = fma(-lu[5440], b[4288], x);
      b[4384] = x;
    }
    {
      double x = b[4416];
      x = fma(-lu[5472], b[2016], x);
      x = fma(-lu[5504], b[2048], x);
      x = fma(-lu[5536], b[2080], x);
      x = fma(-lu[5568], b[2432], x);
      x = fma(-lu[5600], b[2464], x);
      x = fma(-lu[5632], b[2496], x);
      x = fma(-lu[5664], b[2528], x);
      b[4416] = x;
    }
    {
      double x = b[4448];
      x = fma(-lu[5696], b[2752], x);
      x = fma(-lu[5728], b[3104], x);
      x = fma(-lu[5760], b[3136], x);
      x = fma(-lu[5792], b[3264], x);
      x = fma(-lu[5824], b[3296], x);
      x = fma(-lu[5856], b[3360], x);
      x = fma(-lu[5888], b[3392], x);
      x = fma(-lu[5920], b[3488], x);
      b[4448] = x;
    }
    {
      double x = b[4480];
      x = fma(-lu[5952], b[1152], x);
      x = fma(-lu[5984], b[2752], x);
      x = fma(-lu[6016], b[3136], x);
      x = fma(-lu[6048], b[3200], x);
      x = fma(-lu[6080], b[3328], x);
      x = fma(-lu[6112], b[4160], x);
      x = fma(-lu[6144], b[4192], x);
      x = fma(-lu[6176], b[4288], x);
      b[4480] = x;
    }
    {
      double x = b[4512];
      x = fma(-lu[6208], b[1856], x);
      x = fma(-lu[6240], b[3104], x);
      x = fma(-lu[6272], b[3168], x);
      x = fma(-lu[6304], b[3264], x);
      x = fma(-lu[6336], b[3296], x);
      x = fma(-lu[6368], b[3360], x);
      x = fma(-lu[6400], b[3392], x);
      x = fma(-lu[6432], b[3424], x);
      x = fma(-lu[6464], b[3456], x);
      b[4512] = x;
    }
    {
      double x = b[4544];
      x = fma(-lu[6496], b[1408], x);
      x = fma(-lu[6528], b[2624], x);
      x = fma(-lu[6560], b[3712], x);
      x = fma(-lu[6592], b[3744], x);
      x = fma(-lu[6624], b[3840], x);
      x = fma(-lu[6656], b[3936], x);
      x = fma(-lu[6688], b[4160], x);
      x = fma(-lu[6720], b[4192], x);
      x = fma(-lu[6752], b[4288], x);
      x = fma(-lu[6784], b[4384], x);
      b[4544] = x;
    }
    {
      double x = b[4576];
      x = fma(-lu[6816], b[1440], x);
      x = fma(-lu[6848], b[2656], x);
      x = fma(-lu[6880], b[3712], x);
      x = fma(-lu[6912], b[3744], x);
      x = fma(-lu[6944], b[3840], x);
      x = fma(-lu[6976], b[3936], x);
      x = fma(-lu[7008], b[4160], x);
      x = fma(-lu[7040], b[4192], x);
      x = fma(-lu[7072], b[4288], x);
      b[4576] = x;
    }
    {
      double x = b[4608];
      x = fma(-lu[7104], b[3104], x);
      x = fma(-lu[7136], b[3264], x);
      x = fma(-lu[7168], b[3968], x);
      x = fma(-lu[7200], b[4224], x);
      x = fma(-lu[7232], b[4416], x);
      b[4608] = x;
    }
    {
      double x = b[4640];
      x = fma(-lu[7264], b[3392], x);
      x = fma(-lu[7296], b[3968], x);
      x = fma(-lu[7328], b[4224], x);
      x = fma(-lu[7360], b[4416], x);
      b[4640] = x;
    }
    {
      double x = b[4672];
      x = fma(-lu[7392], b[1312], x);
      x = fma(-lu[7424], b[1792], x);
      x = fma(-lu[7456], b[1824], x);
      x = fma(-lu[7488], b[3520], x);
      x = fma(-lu[7520], b[3552], x);
      x = fma(-lu[7552], b[3584], x);
      x = fma(-lu[7584], b[4128], x);
      x = fma(-lu[7616], b[4288], x);
      b[4672] = x;
    }
    {
      double x = b[4704];
      x = fma(-lu[7648], b[2016], x);
      x = fma(-lu[7680], b[2432], x);
      x = fma(-lu[7712], b[2464], x);
      x = fma(-lu[7744], b[3968], x);
      x = fma(-lu[7776], b[4224], x);
      x = fma(-lu[7808], b[4416], x);
      x = fma(-lu[7840], b[4640], x);
      b[4704] = x;
    }
    {
      double x = b[4736];
      x = fma(-lu[7872], b[1312], x);
      x = fma(-lu[7904], b[1344], x);
      x = fma(-lu[7936], b[1632], x);
      x = fma(-lu[7968], b[1664], x);
      x = fma(-lu[8000], b[3136], x);
      x = fma(-lu[8032], b[3712], x);
      x = fma(-lu[8064], b[3744], x);
      x = fma(-lu[8096], b[3840], x);
      x = fma(-lu[8128], b[3936], x);
      x = fma(-lu[8160], b[4160], x);
      x = fma(-lu[8192], b[4192], x);
      x = fma(-lu[8224], b[4288], x);
      b[4736] = x;
    }
    {
      double x = b[4768];
      x = fma(-lu[8256], b[3456], x);
      x = fma(-lu[8288], b[4416], x);
      x = fma(-lu[8320], b[4608], x);
      x = fma(-lu[8352], b[4640], x);
      x = fma(-lu[8384], b[4704], x);
      b[4768] = x;
    }
    {
      double x = b[4800];
      x = fma(-lu[8416], b[1408], x);
      x = fma(-lu[8448], b[1440], x);
      x = fma(-lu[8480], b[1536], x);
      x = fma(-lu[8512], b[4320], x);
      x = fma(-lu[8544], b[4544], x);
      x = fma(-lu[8576], b[4576], x);
      b[4800] = x;
    }
    {
      double x = b[4832];
      x = fma(-lu[8608], b[1600], x);
      x = fma(-lu[8640], b[2048], x);
      x = fma(-lu[8672], b[2080], x);
      x = fma(-lu[8704], b[2112], x);
      x = fma(-lu[8736], b[2464], x);
      x = fma(-lu[8768], b[2496], x);
      x = fma(-lu[8800], b[2528], x);
      x = fma(-lu[8832], b[4224], x);
      x = fma(-lu[8864], b[4416], x);
      x = fma(-lu[8896], b[4640], x);
      x = fma(-lu[8928], b[4704], x);
      b[4832] = x;
    }
    {
      double x = b[4864];
      x = fma(-lu[8960], b[3392], x);
      x = fma(-lu[8992], b[3424], x);
      x = fma(-lu[9024], b[4224], x);
      x = fma(-lu[9056], b[4416], x);
      x = fma(-lu[9088], b[4608], x);
      x = fma(-lu[9120], b[4640], x);
      x = fma(-lu[9152], b[4704], x);
      x = fma(-lu[9184], b[4832], x);
      b[4864] = x;
    }
    {
      double x = b[4896];
      x = fma(-lu[9216], b[3296], x);
      x = fma(-lu[9248], b[3360], x);
      x = fma(-lu[9280], b[3968], x);
      x = fma(-lu[9312], b[4224], x);
      x = fma(-lu[9344], b[4416], x);
      x = fma(-lu[9376], b[4608], x);
      x = fma(-lu[9408], b[4640], x);
      x = fma(-lu[9440], b[4704], x);
      x = fma(-lu[9472], b[4832], x);
      x = fma(-lu[9504], b[4864], x);
      b[4896] = x;
    }
    {
      double x = b[4928];
      x = fma(-lu[9536], b[1920], x);
      x = fma(-lu[9568], b[3104], x);
      x = fma(-lu[9600], b[3264], x);
      x = fma(-lu[9632], b[3968], x);
      x = fma(-lu[9664], b[4224], x);
      x = fma(-lu[9696], b[4416], x);
      x = fma(-lu[9728], b[4608], x);
      x = fma(-lu[9760], b[4640], x);
      x = fma(-lu[9792], b[4704], x);
      x = fma(-lu[9824], b[4832], x);
      x = fma(-lu[9856], b[4864], x);
      x = fma(-lu[9888], b[4896], x);
      b[4928] = x;
    }
    {
      double x = b[4960];
      x = fma(-lu[9920], b[1984], x);
      x = fma(-lu[9952], b[2016], x);
      x = fma(-lu[9984], b[2048], x);
      x = fma(-lu[10016], b[2304], x);
      x = fma(-lu[10048], b[2400], x);
      x = fma(-lu[10080], b[2432], x);
      x = fma(-lu[10112], b[2464], x);
      x = fma(-lu[10144], b[2496], x);
      x = fma(-lu[10176], b[3424], x);
      x = fma(-lu[10208], b[4224], x);
      x = fma(-lu[10240], b[4416], x);
      x = fma(-lu[10272], b[4640], x);
      x = fma(-lu[10304], b[4704], x);
      x = fma(-lu[10336], b[4832], x);
      x = fma(-lu[10368], b[4864], x);
      x = fma(-lu[10400], b[4896], x);
      x = fma(-lu[10432], b[4928], x);
      b[4960] = x;
    }
    {
      double x = b[4992];
      x = fma(-lu[10464], b[1952], x);
      x = fma(-lu[10496], b[1984], x);
      x = fma(-lu[10528], b[2304], x);
      x = fma(-lu[10560], b[2368], x);
      x = fma(-lu[10592], b[2400], x);
      x = fma(-lu[10624], b[3392], x);
      x = fma(-lu[10656], b[3424], x);
      x = fma(-lu[10688], b[3456], x);
      x = fma(-lu[10720], b[3968], x);
      x = fma(-lu[10752], b[4224], x);
      x = fma(-lu[10784], b[4416], x);
      x = fma(-lu[10816], b[4640], x);
      x = fma(-lu[10848], b[4704], x);
      x = fma(-lu[10880], b[4832], x);
      x = fma(-lu[10912], b[4864], x);
      x = fma(-lu[10944], b[4896], x);
      x = fma(-lu[10976], b[4928], x);
      x = fma(-lu[11008], b[4960], x);
      b[4992] = x;
    }
    {
      double x = b[5024];
      x = fma(-lu[11040], b[96], x);
      x = fma(-lu[11072], b[128], x);
      x = fma(-lu[11104], b[1024], x);
      x = fma(-lu[11136], b[1248], x);
      x = fma(-lu[11168], b[1760], x);
      x = fma(-lu[11200], b[2208], x);
      x = fma(-lu[11232], b[2752], x);
      x = fma(-lu[11264], b[2784], x);
      x = fma(-lu[11296], b[2944], x);
      x = fma(-lu[11328], b[3136], x);
      x = fma(-lu[11360], b[3232], x);
      x = fma(-lu[11392], b[3552], x);
      x = fma(-lu[11424], b[4128], x);
      x = fma(-lu[11456], b[4288], x);
      x = fma(-lu[11488], b[4448], x);
      b[5024] = x;
    }
    {
      double x = b[5056];
      x = fma(-lu[11520], b[2784], x);
      x = fma(-lu[11552], b[2848], x);
      x = fma(-lu[11584], b[2880], x);
      x = fma(-lu[11616], b[2912], x);
      x = fma(-lu[11648], b[3200], x);
      x = fma(-lu[11680], b[3328], x);
      x = fma(-lu[11712], b[3520], x);
      x = fma(-lu[11744], b[3552], x);
      x = fma(-lu[11776], b[3712], x);
      x = fma(-lu[11808], b[3744], x);
      x = fma(-lu[11840], b[3776], x);
      x = fma(-lu[11872], b[3840], x);
      x = fma(-lu[11904], b[3872], x);
      x = fma(-lu[11936], b[3936], x);
      x = fma(-lu[11968], b[4064], x);
      x = fma(-lu[12000], b[4128], x);
      x = fma(-lu[12032], b[4160], x);
      x = fma(-lu[12064], b[4192], x);
      x = fma(-lu[12096], b[4288], x);
      x = fma(-lu[12128], b[4384], x);
      x = fma(-lu[12160], b[4480], x);
      x = fma(-lu[12192], b[4544], x);
      x = fma(-lu[12224], b[4576], x);
      x = fma(-lu[12256], b[4672], x);
      x = fma(-lu[12288], b[4736], x);
      x = fma(-lu[12320], b[4864], x);
      x = fma(-lu[12352], b[4896], x);
      x = fma(-lu[12384], b[4928], x);
      x = fma(-lu[12416], b[4960], x);
      x = fma(-lu[12448], b[4992], x);
      b[5056] = x;
    }
    {
      double x = b[5088];
      x = fma(-lu[12480], b[1952], x);
      x = fma(-lu[12512], b[1984], x);
      x = fma(-lu[12544], b[2144], x);
      x = fma(-lu[12576], b[2368], x);
      x = fma(-lu[12608], b[2400], x);
      x = fma(-lu[12640], b[2432], x);
      x = fma(-lu[12672], b[3392], x);
      x = fma(-lu[12704], b[3456], x);
      x = fma(-lu[12736], b[3904], x);
      x = fma(-lu[12768], b[3968], x);
      x = fma(-lu[12800], b[4096], x);
      x = fma(-lu[12832], b[4160], x);
      x = fma(-lu[12864], b[4192], x);
      x = fma(-lu[12896], b[4224], x);
      x = fma(-lu[12928], b[4288], x);
      x = fma(-lu[12960], b[4416], x);
      x = fma(-lu[12992], b[4544], x);
      x = fma(-lu[13024], b[4576], x);
      x = fma(-lu[13056], b[4608], x);
      x = fma(-lu[13088], b[4640], x);
      x = fma(-lu[13120], b[4704], x);
      x = fma(-lu[13152], b[4832], x);
      x = fma(-lu[13184], b[4864], x);
      x = fma(-lu[13216], b[4896], x);
      x = fma(-lu[13248], b[4928], x);
      x = fma(-lu[13280], b[4960], x);
      x = fma(-lu[13312], b[4992], x);
      b[5088] = x;
    }
    {
      double x = b[5120];
      x = fma(-lu[13344], b[1120], x);
      x = fma(-lu[13376], b[2752], x);
      x = fma(-lu[13408], b[3136], x);
      x = fma(-lu[13440], b[3968], x);
      x = fma(-lu[13472], b[4224], x);
      x = fma(-lu[13504], b[4416], x);
      x = fma(-lu[13536], b[4640], x);
      x = fma(-lu[13568], b[4704], x);
      x = fma(-lu[13600], b[4832], x);
      x = fma(-lu[13632], b[4864], x);
      x = fma(-lu[13664], b[4896], x);
      x = fma(-lu[13696], b[4928], x);
      x = fma(-lu[13728], b[4960], x);
      x = fma(-lu[13760], b[4992], x);
      x = fma(-lu[13792], b[5088], x);
      b[5120] = x;
    }
    {
      double x = b[5152];
      x = fma(-lu[13824], b[3968], x);
      x = fma(-lu[13856], b[4224], x);
      x = fma(-lu[13888], b[4416], x);
      x = fma(-lu[13920], b[4608], x);
      x = fma(-lu[13952], b[4640], x);
      x = fma(-lu[13984], b[4704], x);
      x = fma(-lu[14016], b[4768], x);
      x = fma(-lu[14048], b[4832], x);
      x = fma(-lu[14080], b[4864], x);
      x = fma(-lu[14112], b[4896], x);
      x = fma(-lu[14144], b[4928], x);
      x = fma(-lu[14176], b[4960], x);
      x = fma(-lu[14208], b[4992], x);
      x = fma(-lu[14240], b[5088], x);
      b[5152] = x;
    }
    {
      double x = b[5184];
      x = fma(-lu[14272], b[1152], x);
      x = fma(-lu[14304], b[1312], x);
      x = fma(-lu[14336], b[1408], x);
      x = fma(-lu[14368], b[1440], x);
      x = fma(-lu[14400], b[1568], x);
      x = fma(-lu[14432], b[1600], x);
      x = fma(-lu[14464], b[2240], x);
      x = fma(-lu[14496], b[2336], x);
      x = fma(-lu[14528], b[2752], x);
      x = fma(-lu[14560], b[3136], x);
      x = fma(-lu[14592], b[3168], x);
      x = fma(-lu[14624], b[3552], x);
      x = fma(-lu[14656], b[3584], x);
      x = fma(-lu[14688], b[3808], x);
      x = fma(-lu[14720], b[3872], x);
      x = fma(-lu[14752], b[4128], x);
      x = fma(-lu[14784], b[4288], x);
      x = fma(-lu[14816], b[4320], x);
      x = fma(-lu[14848], b[4384], x);
      x = fma(-lu[14880], b[4448], x);
      x = fma(-lu[14912], b[4544], x);
      x = fma(-lu[14944], b[4576], x);
      x = fma(-lu[14976], b[4736], x);
      b[5184] = x;
    }
    {
      double x = b[5216];
      x = fma(-lu[15008], b[1088], x);
      x = fma(-lu[15040], b[1536], x);
      x = fma(-lu[15072], b[2880], x);
      x = fma(-lu[15104], b[3552], x);
      x = fma(-lu[15136], b[3680], x);
      x = fma(-lu[15168], b[3776], x);
      x = fma(-lu[15200], b[3872], x);
      x = fma(-lu[15232], b[4096], x);
      x = fma(-lu[15264], b[4128], x);
      x = fma(-lu[15296], b[4160], x);
      x = fma(-lu[15328], b[4192], x);
      x = fma(-lu[15360], b[4288], x);
      x = fma(-lu[15392], b[4320], x);
      x = fma(-lu[15424], b[4384], x);
      x = fma(-lu[15456], b[4544], x);
      x = fma(-lu[15488], b[4576], x);
      x = fma(-lu[15520], b[4608], x);
      x = fma(-lu[15552], b[4640], x);
      x = fma(-lu[15584], b[4704], x);
      x = fma(-lu[15616], b[4736], x);
      x = fma(-lu[15648], b[4800], x);
      x = fma(-lu[15680], b[4832], x);
      x = fma(-lu[15712], b[4864], x);
      x = fma(-lu[15744], b[4896], x);
      x = fma(-lu[15776], b[4928], x);
      x = fma(-lu[15808], b[4960], x);
      x = fma(-lu[15840], b[4992], x);
      x = fma(-lu[15872], b[5088], x);
      x = fma(-lu[15904], b[5120], x);
      x = fma(-lu[15936], b[5184], x);
      b[5216] = x;
    }
    {
      double x = b[5248];
      x = fma(-lu[15968], b[1312], x);
      x = fma(-lu[16000], b[1344], x);
      x = fma(-lu[16032], b[2880], x);
      x = fma(-lu[16064], b[2912], x);
      x = fma(-lu[16096], b[3104], x);
      x = fma(-lu[16128], b[3264], x);
      x = fma(-lu[16160], b[3296], x);
      x = fma(-lu[16192], b[3392], x);
      x = fma(-lu[16224], b[3424], x);
      x = fma(-lu[16256], b[3456], x);
      x = fma(-lu[16288], b[3552], x);
      x = fma(-lu[16320], b[3584], x);
      x = fma(-lu[16352], b[3776], x);
      x = fma(-lu[16384], b[3872], x);
      x = fma(-lu[16416], b[4128], x);
      x = fma(-lu[16448], b[4288], x);
      x = fma(-lu[16480], b[4320], x);
      x = fma(-lu[16512], b[4384], x);
      x = fma(-lu[16544], b[4544], x);
      x = fma(-lu[16576], b[4576], x);
      x = fma(-lu[16608], b[4736], x);
      x = fma(-lu[16640], b[4864], x);
      x = fma(-lu[16672], b[4896], x);
      x = fma(-lu[16704], b[4928], x);
      x = fma(-lu[16736], b[4960], x);
      x = fma(-lu[16768], b[4992], x);
      x = fma(-lu[16800], b[5088], x);
      x = fma(-lu[16832], b[5184], x);
      b[5248] = x;
    }
    {
      double x = b[5280];
      x = fma(-lu[16864], b[2752], x);
      x = fma(-lu[16896], b[3136], x);
      x = fma(-lu[16928], b[3200], x);
      x = fma(-lu[16960], b[3968], x);
      x = fma(-lu[16992], b[4224], x);
      x = fma(-lu[17024], b[4320], x);
      x = fma(-lu[17056], b[4416], x);
      x = fma(-lu[17088], b[4608], x);
      x = fma(-lu[17120], b[4640], x);
      x = fma(-lu[17152], b[4704], x);
      x = fma(-lu[17184], b[4768], x);
      x = fma(-lu[17216], b[4832], x);
      x = fma(-lu[17248], b[4864], x);
      x = fma(-lu[17280], b[4896], x);
      x = fma(-lu[17312], b[4928], x);
      x = fma(-lu[17344], b[4960], x);
      x = fma(-lu[17376], b[4992], x);
      x = fma(-lu[17408], b[5088], x);
      x = fma(-lu[17440], b[5120], x);
      x = fma(-lu[17472], b[5184], x);
      b[5280] = x;
    }
    {
      double x = b[5312];
      x = fma(-lu[17504], b[832], x);
      x = fma(-lu[17536], b[2144], x);
      x = fma(-lu[17568], b[2368], x);
      x = fma(-lu[17600], b[3296], x);
      x = fma(-lu[17632], b[3360], x);
      x = fma(-lu[17664], b[3392], x);
      x = fma(-lu[17696], b[3424], x);
      x = fma(-lu[17728], b[3456], x);
      x = fma(-lu[17760], b[3904], x);
      x = fma(-lu[17792], b[3968], x);
      x = fma(-lu[17824], b[4096], x);
      x = fma(-lu[17856], b[4160], x);
      x = fma(-lu[17888], b[4192], x);
      x = fma(-lu[17920], b[4224], x);
      x = fma(-lu[17952], b[4288], x);
      x = fma(-lu[17984], b[4416], x);
      x = fma(-lu[18016], b[4544], x);
      x = fma(-lu[18048], b[4576], x);
      x = fma(-lu[18080], b[4608], x);
      x = fma(-lu[18112], b[4640], x);
      x = fma(-lu[18144], b[4704], x);
      x = fma(-lu[18176], b[4832], x);
      x = fma(-lu[18208], b[4864], x);
      x = fma(-lu[18240], b[4896], x);
      x = fma(-lu[18272], b[4928], x);
      x = fma(-lu[18304], b[4960], x);
      x = fma(-lu[18336], b[4992], x);
      x = fma(-lu[18368], b[5088], x);
      x = fma(-lu[18400], b[5184], x);
      b[5312] = x;
    }
    {
      double x = b[5344];
      x = fma(-lu[18432], b[448], x);
      x = fma(-lu[18464], b[1152], x);
      x = fma(-lu[18496], b[1696], x);
      x = fma(-lu[18528], b[1824], x);
      x = fma(-lu[18560], b[2752], x);
      x = fma(-lu[18592], b[3136], x);
      x = fma(-lu[18624], b[3328], x);
      x = fma(-lu[18656], b[3520], x);
      x = fma(-lu[18688], b[3552], x);
      x = fma(-lu[18720], b[3648], x);
      x = fma(-lu[18752], b[3968], x);
      x = fma(-lu[18784], b[4128], x);
      x = fma(-lu[18816], b[4224], x);
      x = fma(-lu[18848], b[4288], x);
      x = fma(-lu[18880], b[4384], x);
      x = fma(-lu[18912], b[4416], x);
      x = fma(-lu[18944], b[4448], x);
      x = fma(-lu[18976], b[4544], x);
      x = fma(-lu[19008], b[4576], x);
      x = fma(-lu[19040], b[4640], x);
      x = fma(-lu[19072], b[4672], x);
      x = fma(-lu[19104], b[4704], x);
      x = fma(-lu[19136], b[4736], x);
      x = fma(-lu[19168], b[4832], x);
      x = fma(-lu[19200], b[4864], x);
      x = fma(-lu[19232], b[4896], x);
      x = fma(-lu[19264], b[4928], x);
      x = fma(-lu[19296], b[4960], x);
      x = fma(-lu[19328], b[4992], x);
      x = fma(-lu[19360], b[5088], x);
      x = fma(-lu[19392], b[5120], x);
      x = fma(-lu[19424], b[5184], x);
      x = fma(-lu[19456], b[5312], x);
      b[5344] = x;
    }
}
__device__ __noinline__ void solve_0_1(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 105440;
    const double* __restrict__ vd = ws + 210560;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[5376];
      x = fma(-lu[19488], b[256], x);
      x = fma(-lu[19520], b[1344], x);
      x = fma(-lu[19552], b[2912], x);
      x = fma(-lu[19584], b[2976], x);
      x = fma(-lu[19616], b[3072], x);
      x = fma(-lu[19648], b[3104], x);
      x = fma(-lu[19680], b[3136], x);
      x = fma(-lu[19712], b[3232], x);
      x = fma(-lu[19744], b[3264], x);
      x = fma(-lu[19776], b[3296], x);
      x = fma(-lu[19808], b[3360], x);
      x = fma(-lu[19840], b[3392], x);
      x = fma(-lu[19872], b[3424], x);
      x = fma(-lu[19904], b[3456], x);
      x = fma(-lu[19936], b[3552], x);
      x = fma(-lu[19968], b[3584], x);
      x = fma(-lu[20000], b[3648], x);
      x = fma(-lu[20032], b[3872], x);
      x = fma(-lu[20064], b[4288], x);
      x = fma(-lu[20096], b[4320], x);
      x = fma(-lu[20128], b[4384], x);
      x = fma(-lu[20160], b[4448], x);
      x = fma(-lu[20192], b[4512], x);
      x = fma(-lu[20224], b[4544], x);
      x = fma(-lu[20256], b[4576], x);
      x = fma(-lu[20288], b[4736], x);
      x = fma(-lu[20320], b[5184], x);
      b[5376] = x;
    }
    {
      double x = b[5408];
      x = fma(-lu[20352], b[1152], x);
      x = fma(-lu[20384], b[2176], x);
      x = fma(-lu[20416], b[2752], x);
      x = fma(-lu[20448], b[3136], x);
      x = fma(-lu[20480], b[3968], x);
      x = fma(-lu[20512], b[4224], x);
      x = fma(-lu[20544], b[4416], x);
      x = fma(-lu[20576], b[4608], x);
      x = fma(-lu[20608], b[4640], x);
      x = fma(-lu[20640], b[4704], x);
      x = fma(-lu[20672], b[4768], x);
      x = fma(-lu[20704], b[4832], x);
      x = fma(-lu[20736], b[4864], x);
      x = fma(-lu[20768], b[4896], x);
      x = fma(-lu[20800], b[4928], x);
      x = fma(-lu[20832], b[4960], x);
      x = fma(-lu[20864], b[4992], x);
      x = fma(-lu[20896], b[5088], x);
      x = fma(-lu[20928], b[5184], x);
      x = fma(-lu[20960], b[5312], x);
      b[5408] = x;
    }
    {
      double x = b[5440];
      x = fma(-lu[20992], b[1856], x);
      x = fma(-lu[21024], b[2144], x);
      x = fma(-lu[21056], b[2624], x);
      x = fma(-lu[21088], b[2656], x);
      x = fma(-lu[21120], b[2688], x);
      x = fma(-lu[21152], b[3072], x);
      x = fma(-lu[21184], b[3104], x);
      x = fma(-lu[21216], b[3136], x);
      x = fma(-lu[21248], b[3168], x);
      x = fma(-lu[21280], b[3200], x);
      x = fma(-lu[21312], b[3232], x);
      x = fma(-lu[21344], b[3264], x);
      x = fma(-lu[21376], b[3296], x);
      x = fma(-lu[21408], b[3328], x);
      x = fma(-lu[21440], b[3360], x);
      x = fma(-lu[21472], b[3808], x);
      x = fma(-lu[21504], b[3872], x);
      x = fma(-lu[21536], b[3904], x);
      x = fma(-lu[21568], b[4032], x);
      x = fma(-lu[21600], b[4064], x);
      x = fma(-lu[21632], b[4096], x);
      x = fma(-lu[21664], b[4160], x);
      x = fma(-lu[21696], b[4192], x);
      x = fma(-lu[21728], b[4288], x);
      x = fma(-lu[21760], b[4384], x);
      x = fma(-lu[21792], b[4448], x);
      x = fma(-lu[21824], b[4544], x);
      x = fma(-lu[21856], b[4576], x);
      x = fma(-lu[21888], b[4608], x);
      x = fma(-lu[21920], b[4640], x);
      x = fma(-lu[21952], b[4704], x);
      x = fma(-lu[21984], b[4736], x);
      x = fma(-lu[22016], b[4832], x);
      x = fma(-lu[22048], b[4864], x);
      x = fma(-lu[22080], b[4896], x);
      x = fma(-lu[22112], b[4928], x);
      x = fma(-lu[22144], b[4960], x);
      x = fma(-lu[22176], b[4992], x);
      x = fma(-lu[22208], b[5088], x);
      x = fma(-lu[22240], b[5120], x);
      x = fma(-lu[22272], b[5184], x);
      x = fma(-lu[22304], b[5312], x);
      x = fma(-lu[22336], b[5408], x);
      b[5440] = x;
    }
    {
      double x = b[5472];
      x = fma(-lu[22368], b[3168], x);
      x = fma(-lu[22400], b[3296], x);
      x = fma(-lu[22432], b[3584], x);
      x = fma(-lu[22464], b[3776], x);
      x = fma(-lu[22496], b[3968], x);
      x = fma(-lu[22528], b[4224], x);
      x = fma(-lu[22560], b[4320], x);
      x = fma(-lu[22592], b[4416], x);
      x = fma(-lu[22624], b[4608], x);
      x = fma(-lu[22656], b[4640], x);
      x = fma(-lu[22688], b[4704], x);
      x = fma(-lu[22720], b[4768], x);
      x = fma(-lu[22752], b[4832], x);
      x = fma(-lu[22784], b[4864], x);
      x = fma(-lu[22816], b[4896], x);
      x = fma(-lu[22848], b[4928], x);
      x = fma(-lu[22880], b[4960], x);
      x = fma(-lu[22912], b[4992], x);
      x = fma(-lu[22944], b[5088], x);
      x = fma(-lu[22976], b[5152], x);
      x = fma(-lu[23008], b[5184], x);
      x = fma(-lu[23040], b[5280], x);
      x = fma(-lu[23072], b[5312], x);
      x = fma(-lu[23104], b[5408], x);
      x = fma(-lu[23136], b[5440], x);
      b[5472] = x;
    }
    {
      double x = b[5504];
      x = fma(-lu[23168], b[1152], x);
      x = fma(-lu[23200], b[1408], x);
      x = fma(-lu[23232], b[2144], x);
      x = fma(-lu[23264], b[2624], x);
      x = fma(-lu[23296], b[2912], x);
      x = fma(-lu[23328], b[3200], x);
      x = fma(-lu[23360], b[3328], x);
      x = fma(-lu[23392], b[3872], x);
      x = fma(-lu[23424], b[3904], x);
      x = fma(-lu[23456], b[4032], x);
      x = fma(-lu[23488], b[4064], x);
      x = fma(-lu[23520], b[4096], x);
      x = fma(-lu[23552], b[4160], x);
      x = fma(-lu[23584], b[4192], x);
      x = fma(-lu[23616], b[4288], x);
      x = fma(-lu[23648], b[4384], x);
      x = fma(-lu[23680], b[4512], x);
      x = fma(-lu[23712], b[4544], x);
      x = fma(-lu[23744], b[4576], x);
      x = fma(-lu[23776], b[4608], x);
      x = fma(-lu[23808], b[4640], x);
      x = fma(-lu[23840], b[4704], x);
      x = fma(-lu[23872], b[4736], x);
      x = fma(-lu[23904], b[4832], x);
      x = fma(-lu[23936], b[4864], x);
      x = fma(-lu[23968], b[4896], x);
      x = fma(-lu[24000], b[4928], x);
      x = fma(-lu[24032], b[4960], x);
      x = fma(-lu[24064], b[4992], x);
      x = fma(-lu[24096], b[5088], x);
      x = fma(-lu[24128], b[5120], x);
      x = fma(-lu[24160], b[5184], x);
      x = fma(-lu[24192], b[5312], x);
      x = fma(-lu[24224], b[5408], x);
      x = fma(-lu[24256], b[5440], x);
      x = fma(-lu[24288], b[5472], x);
      b[5504] = x;
    }
    {
      double x = b[5536];
      x = fma(-lu[24320], b[864], x);
      x = fma(-lu[24352], b[896], x);
      x = fma(-lu[24384], b[1600], x);
      x = fma(-lu[24416], b[1920], x);
      x = fma(-lu[24448], b[1952], x);
      x = fma(-lu[24480], b[2304], x);
      x = fma(-lu[24512], b[2368], x);
      x = fma(-lu[24544], b[2400], x);
      x = fma(-lu[24576], b[3104], x);
      x = fma(-lu[24608], b[3264], x);
      x = fma(-lu[24640], b[3424], x);
      x = fma(-lu[24672], b[3456], x);
      x = fma(-lu[24704], b[3488], x);
      x = fma(-lu[24736], b[3968], x);
      x = fma(-lu[24768], b[4224], x);
      x = fma(-lu[24800], b[4416], x);
      x = fma(-lu[24832], b[4640], x);
      x = fma(-lu[24864], b[4704], x);
      x = fma(-lu[24896], b[4832], x);
      x = fma(-lu[24928], b[4864], x);
      x = fma(-lu[24960], b[4896], x);
      x = fma(-lu[24992], b[4928], x);
      x = fma(-lu[25024], b[4960], x);
      x = fma(-lu[25056], b[4992], x);
      x = fma(-lu[25088], b[5088], x);
      x = fma(-lu[25120], b[5184], x);
      x = fma(-lu[25152], b[5312], x);
      x = fma(-lu[25184], b[5472], x);
      x = fma(-lu[25216], b[5504], x);
      b[5536] = x;
    }
    {
      double x = b[5568];
      x = fma(-lu[25248], b[1152], x);
      x = fma(-lu[25280], b[1472], x);
      x = fma(-lu[25312], b[2752], x);
      x = fma(-lu[25344], b[3136], x);
      x = fma(-lu[25376], b[3200], x);
      x = fma(-lu[25408], b[3328], x);
      x = fma(-lu[25440], b[3872], x);
      x = fma(-lu[25472], b[3968], x);
      x = fma(-lu[25504], b[4224], x);
      x = fma(-lu[25536], b[4384], x);
      x = fma(-lu[25568], b[4416], x);
      x = fma(-lu[25600], b[4544], x);
      x = fma(-lu[25632], b[4576], x);
      x = fma(-lu[25664], b[4608], x);
      x = fma(-lu[25696], b[4640], x);
      x = fma(-lu[25728], b[4704], x);
      x = fma(-lu[25760], b[4736], x);
      x = fma(-lu[25792], b[4768], x);
      x = fma(-lu[25824], b[4832], x);
      x = fma(-lu[25856], b[4864], x);
      x = fma(-lu[25888], b[4896], x);
      x = fma(-lu[25920], b[4928], x);
      x = fma(-lu[25952], b[4960], x);
      x = fma(-lu[25984], b[4992], x);
      x = fma(-lu[26016], b[5056], x);
      x = fma(-lu[26048], b[5088], x);
      x = fma(-lu[26080], b[5120], x);
      x = fma(-lu[26112], b[5152], x);
      x = fma(-lu[26144], b[5184], x);
      x = fma(-lu[26176], b[5280], x);
      x = fma(-lu[26208], b[5312], x);
      x = fma(-lu[26240], b[5408], x);
      x = fma(-lu[26272], b[5440], x);
      x = fma(-lu[26304], b[5472], x);
      x = fma(-lu[26336], b[5504], x);
      x = fma(-lu[26368], b[5536], x);
      b[5568] = x;
    }
    {
      double x = b[5600];
      x = fma(-lu[26400], b[2624], x);
      x = fma(-lu[26432], b[2656], x);
      x = fma(-lu[26464], b[2848], x);
      x = fma(-lu[26496], b[2880], x);
      x = fma(-lu[26528], b[2912], x);
      x = fma(-lu[26560], b[3008], x);
      x = fma(-lu[26592], b[3104], x);
      x = fma(-lu[26624], b[3136], x);
      x = fma(-lu[26656], b[3200], x);
      x = fma(-lu[26688], b[3264], x);
      x = fma(-lu[26720], b[3296], x);
      x = fma(-lu[26752], b[3328], x);
      x = fma(-lu[26784], b[3360], x);
      x = fma(-lu[26816], b[3392], x);
      x = fma(-lu[26848], b[3424], x);
      x = fma(-lu[26880], b[3456], x);
      x = fma(-lu[26912], b[3488], x);
      x = fma(-lu[26944], b[3520], x);
      x = fma(-lu[26976], b[3552], x);
      x = fma(-lu[27008], b[3712], x);
      x = fma(-lu[27040], b[3744], x);
      x = fma(-lu[27072], b[3776], x);
      x = fma(-lu[27104], b[3840], x);
      x = fma(-lu[27136], b[3872], x);
      x = fma(-lu[27168], b[3936], x);
      x = fma(-lu[27200], b[4064], x);
      x = fma(-lu[27232], b[4128], x);
      x = fma(-lu[27264], b[4160], x);
      x = fma(-lu[27296], b[4192], x);
      x = fma(-lu[27328], b[4288], x);
      x = fma(-lu[27360], b[4384], x);
      x = fma(-lu[27392], b[4480], x);
      x = fma(-lu[27424], b[4544], x);
      x = fma(-lu[27456], b[4576], x);
      x = fma(-lu[27488], b[4672], x);
      x = fma(-lu[27520], b[4736], x);
      x = fma(-lu[27552], b[4864], x);
      x = fma(-lu[27584], b[4896], x);
      x = fma(-lu[27616], b[4928], x);
      x = fma(-lu[27648], b[4960], x);
      x = fma(-lu[27680], b[4992], x);
      x = fma(-lu[27712], b[5088], x);
      x = fma(-lu[27744], b[5120], x);
      x = fma(-lu[27776], b[5152], x);
      x = fma(-lu[27808], b[5184], x);
      x = fma(-lu[27840], b[5280], x);
      x = fma(-lu[27872], b[5312], x);
      x = fma(-lu[27904], b[5408], x);
      x = fma(-lu[27936], b[5440], x);
      x = fma(-lu[27968], b[5472], x);
      x = fma(-lu[28000], b[5504], x);
      x = fma(-lu[28032], b[5536], x);
      b[5600] = x;
    }
    {
      double x = b[5632];
      x = fma(-lu[28064], b[384], x);
      x = fma(-lu[28096], b[416], x);
      x = fma(-lu[28128], b[1152], x);
      x = fma(-lu[28160], b[1888], x);
      x = fma(-lu[28192], b[2752], x);
      x = fma(-lu[28224], b[3136], x);
      x = fma(-lu[28256], b[3968], x);
      x = fma(-lu[28288], b[4224], x);
      x = fma(-lu[28320], b[4416], x);
      x = fma(-lu[28352], b[4608], x);
      x = fma(-lu[28384], b[4640], x);
      x = fma(-lu[28416], b[4704], x);
      x = fma(-lu[28448], b[4768], x);
      x = fma(-lu[28480], b[4800], x);
      x = fma(-lu[28512], b[4832], x);
      x = fma(-lu[28544], b[4864], x);
      x = fma(-lu[28576], b[4896], x);
      x = fma(-lu[28608], b[4928], x);
      x = fma(-lu[28640], b[4960], x);
      x = fma(-lu[28672], b[4992], x);
      x = fma(-lu[28704], b[5088], x);
      x = fma(-lu[28736], b[5120], x);
      x = fma(-lu[28768], b[5184], x);
      x = fma(-lu[28800], b[5216], x);
      x = fma(-lu[28832], b[5280], x);
      x = fma(-lu[28864], b[5312], x);
      x = fma(-lu[28896], b[5408], x);
      x = fma(-lu[28928], b[5440], x);
      x = fma(-lu[28960], b[5472], x);
      x = fma(-lu[28992], b[5504], x);
      x = fma(-lu[29024], b[5536], x);
      b[5632] = x;
    }
    {
      double x = b[5664];
      x = fma(-lu[29056], b[256], x);
      x = fma(-lu[29088], b[1152], x);
      x = fma(-lu[29120], b[1312], x);
      x = fma(-lu[29152], b[1344], x);
      x = fma(-lu[29184], b[1408], x);
      x = fma(-lu[29216], b[1568], x);
      x = fma(-lu[29248], b[2208], x);
      x = fma(-lu[29280], b[2240], x);
      x = fma(-lu[29312], b[2752], x);
      x = fma(-lu[29344], b[2784], x);
      x = fma(-lu[29376], b[2912], x);
      x = fma(-lu[29408], b[3136], x);
      x = fma(-lu[29440], b[3552], x);
      x = fma(-lu[29472], b[3584], x);
      x = fma(-lu[29504], b[3872], x);
      x = fma(-lu[29536], b[4128], x);
      x = fma(-lu[29568], b[4288], x);
      x = fma(-lu[29600], b[4320], x);
      x = fma(-lu[29632], b[4384], x);
      x = fma(-lu[29664], b[4448], x);
      x = fma(-lu[29696], b[4480], x);
      x = fma(-lu[29728], b[4512], x);
      x = fma(-lu[29760], b[4544], x);
      x = fma(-lu[29792], b[4576], x);
      x = fma(-lu[29824], b[4672], x);
      x = fma(-lu[29856], b[4736], x);
      x = fma(-lu[29888], b[5120], x);
      x = fma(-lu[29920], b[5184], x);
      x = fma(-lu[29952], b[5248], x);
      x = fma(-lu[29984], b[5280], x);
      x = fma(-lu[30016], b[5312], x);
      x = fma(-lu[30048], b[5344], x);
      x = fma(-lu[30080], b[5376], x);
      x = fma(-lu[30112], b[5408], x);
      x = fma(-lu[30144], b[5440], x);
      x = fma(-lu[30176], b[5472], x);
      x = fma(-lu[30208], b[5504], x);
      x = fma(-lu[30240], b[5536], x);
      x = fma(-lu[30272], b[5568], x);
      x = fma(-lu[30304], b[5632], x);
      b[5664] = x;
    }
    {
      double x = b[5696];
      x = fma(-lu[30336], b[1152], x);
      x = fma(-lu[30368], b[1408], x);
      x = fma(-lu[30400], b[1440], x);
      x = fma(-lu[30432], b[2752], x);
      x = fma(-lu[30464], b[2848], x);
      x = fma(-lu[30496], b[2880], x);
      x = fma(-lu[30528], b[2912], x);
      x = fma(-lu[30560], b[3008], x);
      x = fma(-lu[30592], b[3104], x);
      x = fma(-lu[30624], b[3136], x);
      x = fma(-lu[30656], b[3200], x);
      x = fma(-lu[30688], b[3264], x);
      x = fma(-lu[30720], b[3296], x);
      x = fma(-lu[30752], b[3328], x);
      x = fma(-lu[30784], b[3360], x);
      x = fma(-lu[30816], b[3392], x);
      x = fma(-lu[30848], b[3424], x);
      x = fma(-lu[30880], b[3456], x);
      x = fma(-lu[30912], b[3488], x);
      x = fma(-lu[30944], b[3520], x);
      x = fma(-lu[30976], b[3552], x);
      x = fma(-lu[31008], b[3584], x);
      x = fma(-lu[31040], b[3712], x);
      x = fma(-lu[31072], b[3744], x);
      x = fma(-lu[31104], b[3776], x);
      x = fma(-lu[31136], b[3840], x);
      x = fma(-lu[31168], b[3872], x);
      x = fma(-lu[31200], b[3936], x);
      x = fma(-lu[31232], b[4064], x);
      x = fma(-lu[31264], b[4128], x);
      x = fma(-lu[31296], b[4160], x);
      x = fma(-lu[31328], b[4192], x);
      x = fma(-lu[31360], b[4288], x);
      x = fma(-lu[31392], b[4384], x);
      x = fma(-lu[31424], b[4480], x);
      x = fma(-lu[31456], b[4544], x);
      x = fma(-lu[31488], b[4576], x);
      x = fma(-lu[31520], b[4672], x);
      x = fma(-lu[31552], b[4736], x);
      x = fma(-lu[31584], b[4800], x);
      x = fma(-lu[31616], b[4864], x);
      x = fma(-lu[31648], b[4896], x);
      x = fma(-lu[31680], b[4928], x);
      x = fma(-lu[31712], b[4960], x);
      x = fma(-lu[31744], b[4992], x);
      x = fma(-lu[31776], b[5088], x);
      x = fma(-lu[31808], b[5120], x);
      x = fma(-lu[31840], b[5152], x);
      x = fma(-lu[31872], b[5184], x);
      x = fma(-lu[31904], b[5216], x);
      x = fma(-lu[31936], b[5280], x);
      x = fma(-lu[31968], b[5312], x);
      x = fma(-lu[32000], b[5408], x);
      x = fma(-lu[32032], b[5440], x);
      x = fma(-lu[32064], b[5472], x);
      x = fma(-lu[32096], b[5504], x);
      x = fma(-lu[32128], b[5536], x);
      x = fma(-lu[32160], b[5632], x);
      b[5696] = x;
    }
    {
      double x = b[5728];
      x = fma(-lu[32192], b[1856], x);
      x = fma(-lu[32224], b[2848], x);
      x = fma(-lu[32256], b[2880], x);
      x = fma(-lu[32288], b[2912], x);
      x = fma(-lu[32320], b[2976], x);
      x = fma(-lu[32352], b[3008], x);
      x = fma(-lu[32384], b[3040], x);
      x = fma(-lu[32416], b[3072], x);
      x = fma(-lu[32448], b[3104], x);
      x = fma(-lu[32480], b[3136], x);
      x = fma(-lu[32512], b[3168], x);
      x = fma(-lu[32544], b[3200], x);
      x = fma(-lu[32576], b[3232], x);
      x = fma(-lu[32608], b[3264], x);
      x = fma(-lu[32640], b[3296], x);
      x = fma(-lu[32672], b[3328], x);
      x = fma(-lu[32704], b[3360], x);
      x = fma(-lu[32736], b[3552], x);
      x = fma(-lu[32768], b[3584], x);
      x = fma(-lu[32800], b[3648], x);
      x = fma(-lu[32832], b[3776], x);
      x = fma(-lu[32864], b[3808], x);
      x = fma(-lu[32896], b[3872], x);
      x = fma(-lu[32928], b[3904], x);
      x = fma(-lu[32960], b[3968], x);
      x = fma(-lu[32992], b[4096], x);
      x = fma(-lu[33024], b[4160], x);
      x = fma(-lu[33056], b[4192], x);
      x = fma(-lu[33088], b[4224], x);
      x = fma(-lu[33120], b[4288], x);
      x = fma(-lu[33152], b[4320], x);
      x = fma(-lu[33184], b[4384], x);
      x = fma(-lu[33216], b[4416], x);
      x = fma(-lu[33248], b[4448], x);
      x = fma(-lu[33280], b[4480], x);
      x = fma(-lu[33312], b[4544], x);
      x = fma(-lu[33344], b[4576], x);
      x = fma(-lu[33376], b[4608], x);
      x = fma(-lu[33408], b[4640], x);
      x = fma(-lu[33440], b[4704], x);
      x = fma(-lu[33472], b[4736], x);
      x = fma(-lu[33504], b[4832], x);
      x = fma(-lu[33536], b[4864], x);
      x = fma(-lu[33568], b[4896], x);
      x = fma(-lu[33600], b[4928], x);
      x = fma(-lu[33632], b[4960], x);
      x = fma(-lu[33664], b[4992], x);
      x = fma(-lu[33696], b[5088], x);
      x = fma(-lu[33728], b[5120], x);
      x = fma(-lu[33760], b[5152], x);
      x = fma(-lu[33792], b[5184], x);
      x = fma(-lu[33824], b[5216], x);
      x = fma(-lu[33856], b[5280], x);
      x = fma(-lu[33888], b[5312], x);
      x = fma(-lu[33920], b[5408], x);
      x = fma(-lu[33952], b[5440], x);
      x = fma(-lu[33984], b[5472], x);
      x = fma(-lu[34016], b[5504], x);
      x = fma(-lu[34048], b[5536], x);
      x = fma(-lu[34080], b[5632], x);
      x = fma(-lu[34112], b[5696], x);
      b[5728] = x;
    }
    {
      double x = b[5760];
      x = fma(-lu[34144], b[448], x);
      x = fma(-lu[34176], b[1152], x);
      x = fma(-lu[34208], b[1504], x);
      x = fma(-lu[34240], b[2624], x);
      x = fma(-lu[34272], b[2752], x);
      x = fma(-lu[34304], b[2880], x);
      x = fma(-lu[34336], b[2912], x);
      x = fma(-lu[34368], b[3008], x);
      x = fma(-lu[34400], b[3136], x);
      x = fma(-lu[34432], b[3168], x);
      x = fma(-lu[34464], b[3200], x);
      x = fma(-lu[34496], b[3328], x);
      x = fma(-lu[34528], b[3552], x);
      x = fma(-lu[34560], b[3776], x);
      x = fma(-lu[34592], b[3872], x);
      x = fma(-lu[34624], b[3968], x);
      x = fma(-lu[34656], b[4032], x);
      x = fma(-lu[34688], b[4064], x);
      x = fma(-lu[34720], b[4096], x);
      x = fma(-lu[34752], b[4160], x);
      x = fma(-lu[34784], b[4192], x);
      x = fma(-lu[34816], b[4224], x);
      x = fma(-lu[34848], b[4288], x);
      x = fma(-lu[34880], b[4384], x);
      x = fma(-lu[34912], b[4416], x);
      x = fma(-lu[34944], b[4544], x);
      x = fma(-lu[34976], b[4576], x);
      x = fma(-lu[35008], b[4608], x);
      x = fma(-lu[35040], b[4640], x);
      x = fma(-lu[35072], b[4704], x);
      x = fma(-lu[35104], b[4736], x);
      x = fma(-lu[35136], b[4768], x);
      x = fma(-lu[35168], b[4832], x);
      x = fma(-lu[35200], b[4864], x);
      x = fma(-lu[35232], b[4896], x);
      x = fma(-lu[35264], b[4928], x);
      x = fma(-lu[35296], b[4960], x);
      x = fma(-lu[35328], b[4992], x);
      x = fma(-lu[35360], b[5056], x);
      x = fma(-lu[35392], b[5088], x);
      x = fma(-lu[35424], b[5120], x);
      x = fma(-lu[35456], b[5152], x);
      x = fma(-lu[35488], b[5184], x);
      x = fma(-lu[35520], b[5280], x);
      x = fma(-lu[35552], b[5312], x);
      x = fma(-lu[35584], b[5408], x);
      x = fma(-lu[35616], b[5440], x);
      x = fma(-lu[35648], b[5472], x);
      x = fma(-lu[35680], b[5504], x);
      x = fma(-lu[35712], b[5536], x);
      x = fma(-lu[35744], b[5728], x);
      b[5760] = x;
    }
    {
      double x = b[5792];
      x = fma(-lu[35776], b[1088], x);
      x = fma(-lu[35808], b[1152], x);
      x = fma(-lu[35840], b[1312], x);
      x = fma(-lu[35872], b[1344], x);
      x = fma(-lu[35904], b[1440], x);
      x = fma(-lu[35936], b[2272], x);
      x = fma(-lu[35968], b[2592], x);
      x = fma(-lu[36000], b[2624], x);
      x = fma(-lu[36032], b[2656], x);
      x = fma(-lu[36064], b[2848], x);
      x = fma(-lu[36096], b[2880], x);
      x = fma(-lu[36128], b[2912], x);
      x = fma(-lu[36160], b[2976], x);
      x = fma(-lu[36192], b[3008], x);
      x = fma(-lu[36224], b[3040], x);
      x = fma(-lu[36256], b[3072], x);
      x = fma(-lu[36288], b[3104], x);
      x = fma(-lu[36320], b[3136], x);
      x = fma(-lu[36352], b[3200], x);
      x = fma(-lu[36384], b[3232], x);
      x = fma(-lu[36416], b[3264], x);
      x = fma(-lu[36448], b[3296], x);
      x = fma(-lu[36480], b[3328], x);
      x = fma(-lu[36512], b[3360], x);
      x = fma(-lu[36544], b[3392], x);
      x = fma(-lu[36576], b[3424], x);
      x = fma(-lu[36608], b[3456], x);
      x = fma(-lu[36640], b[3488], x);
      x = fma(-lu[36672], b[3520], x);
      x = fma(-lu[36704], b[3552], x);
      x = fma(-lu[36736], b[3648], x);
      x = fma(-lu[36768], b[3680], x);
      x = fma(-lu[36800], b[3712], x);
      x = fma(-lu[36832], b[3744], x);
      x = fma(-lu[36864], b[3776], x);
      x = fma(-lu[36896], b[3808], x);
      x = fma(-lu[36928], b[3840], x);
      x = fma(-lu[36960], b[3872], x);
      x = fma(-lu[36992], b[3936], x);
      x = fma(-lu[37024], b[4032], x);
      x = fma(-lu[37056], b[4064], x);
      x = fma(-lu[37088], b[4128], x);
      x = fma(-lu[37120], b[4160], x);
      x = fma(-lu[37152], b[4192], x);
      x = fma(-lu[37184], b[4288], x);
      x = fma(-lu[37216], b[4320], x);
      x = fma(-lu[37248], b[4384], x);
      x = fma(-lu[37280], b[4448], x);
      x = fma(-lu[37312], b[4480], x);
      x = fma(-lu[37344], b[4544], x);
      x = fma(-lu[37376], b[4576], x);
      x = fma(-lu[37408], b[4672], x);
      x = fma(-lu[37440], b[4736], x);
      x = fma(-lu[37472], b[4800], x);
      x = fma(-lu[37504], b[4864], x);
      x = fma(-lu[37536], b[4896], x);
      x = fma(-lu[37568], b[4928], x);
      x = fma(-lu[37600], b[4960], x);
      x = fma(-lu[37632], b[4992], x);
      x = fma(-lu[37664], b[5088], x);
      x = fma(-lu[37696], b[5120], x);
      x = fma(-lu[37728], b[5152], x);
      x = fma(-lu[37760], b[5184], x);
      x = fma(-lu[37792], b[5216], x);
      x = fma(-lu[37824], b[5248], x);
      x = fma(-lu[37856], b[5280], x);
      x = fma(-lu[37888], b[5312], x);
      x = fma(-lu[37920], b[5344], x);
      x = fma(-lu[37952], b[5408], x);
      x = fma(-lu[37984], b[5440], x);
      x = fma(-lu[38016], b[5472], x);
      x = fma(-lu[38048], b[5504], x);
      x = fma(-lu[38080], b[5536], x);
      x = fma(-lu[38112], b[5568], x);
      x = fma(-lu[38144], b[5632], x);
      x = fma(-lu[38176], b[5696], x);
      x = fma(-lu[38208], b[5728], x);
      x = fma(-lu[38240], b[5760], x);
      b[5792] = x;
    }
    {
      double x = b[5824];
      x = fma(-lu[38272], b[1184], x);
      x = fma(-lu[38304], b[1632], x);
      x = fma(-lu[38336], b[1728], x);
      x = fma(-lu[38368], b[1856], x);
      x = fma(-lu[38400], b[1920], x);
      x = fma(-lu[38432], b[1952], x);
      x = fma(-lu[38464], b[1984], x);
      x = fma(-lu[38496], b[2016], x);
      x = fma(-lu[38528], b[2048], x);
      x = fma(-lu[38560], b[2080], x);
      x = fma(-lu[38592], b[2112], x);
      x = fma(-lu[38624], b[2144], x);
      x = fma(-lu[38656], b[2272], x);
      x = fma(-lu[38688], b[2304], x);
      x = fma(-lu[38720], b[2336], x);
      x = fma(-lu[38752], b[2368], x);
      x = fma(-lu[38784], b[2400], x);
      x = fma(-lu[38816], b[2432], x);
      x = fma(-lu[38848], b[2464], x);
      x = fma(-lu[38880], b[2496], x);
      x = fma(-lu[38912], b[2528], x);
      x = fma(-lu[38944], b[2560], x);
      x = fma(-lu[38976], b[2592], x);
      x = fma(-lu[39008], b[2624], x);
      x = fma(-lu[39040], b[2656], x);
      x = fma(-lu[39072], b[2848], x);
      x = fma(-lu[39104], b[2880], x);
      x = fma(-lu[39136], b[2912], x);
      x = fma(-lu[39168], b[2976], x);
      x = fma(-lu[39200], b[3008], x);
      x = fma(-lu[39232], b[3040], x);
      x = fma(-lu[39264], b[3072], x);
      x = fma(-lu[39296], b[3104], x);
      x = fma(-lu[39328], b[3136], x);
      x = fma(-lu[39360], b[3168], x);
      x = fma(-lu[39392], b[3200], x);
      x = fma(-lu[39424], b[3232], x);
      x = fma(-lu[39456], b[3264], x);
      x = fma(-lu[39488], b[3296], x);
      x = fma(-lu[39520], b[3328], x);
      x = fma(-lu[39552], b[3360], x);
      x = fma(-lu[39584], b[3392], x);
      x = fma(-lu[39616], b[3424], x);
      x = fma(-lu[39648], b[3456], x);
      x = fma(-lu[39680], b[3488], x);
      x = fma(-lu[39712], b[3520], x);
      x = fma(-lu[39744], b[3552], x);
      x = fma(-lu[39776], b[3648], x);
      x = fma(-lu[39808], b[3712], x);
      x = fma(-lu[39840], b[3744], x);
      x = fma(-lu[39872], b[3776], x);
      x = fma(-lu[39904], b[3808], x);
      x = fma(-lu[39936], b[3840], x);
      x = fma(-lu[39968], b[3872], x);
      x = fma(-lu[40000], b[3904], x);
      x = fma(-lu[40032], b[3936], x);
      x = fma(-lu[40064], b[4032], x);
      x = fma(-lu[40096], b[4064], x);
      x = fma(-lu[40128], b[4096], x);
      x = fma(-lu[40160], b[4128], x);
      x = fma(-lu[40192], b[4160], x);
      x = fma(-lu[40224], b[4192], x);
      x = fma(-lu[40256], b[4288], x);
      x = fma(-lu[40288], b[4384], x);
      x = fma(-lu[40320], b[4448], x);
      x = fma(-lu[40352], b[4480], x);
      x = fma(-lu[40384], b[4544], x);
      x = fma(-lu[40416], b[4576], x);
      x = fma(-lu[40448], b[4608], x);
      x = fma(-lu[40480], b[4640], x);
      x = fma(-lu[40512], b[4672], x);
      x = fma(-lu[40544], b[4704], x);
      x = fma(-lu[40576], b[4736], x);
      x = fma(-lu[40608], b[4800], x);
      x = fma(-lu[40640], b[4832], x);
      x = fma(-lu[40672], b[4864], x);
      x = fma(-lu[40704], b[4896], x);
      x = fma(-lu[40736], b[4928], x);
      x = fma(-lu[40768], b[4960], x);
      x = fma(-lu[40800], b[4992], x);
      x = fma(-lu[40832], b[5088], x);
      x = fma(-lu[40864], b[5120], x);
      x = fma(-lu[40896], b[5152], x);
      x = fma(-lu[40928], b[5184], x);
      x = fma(-lu[40960], b[5216], x);
      x = fma(-lu[40992], b[5280], x);
      x = fma(-lu[41024], b[5312], x);
      x = fma(-lu[41056], b[5408], x);
      x = fma(-lu[41088], b[5440], x);
      x = fma(-lu[41120], b[5472], x);
      x = fma(-lu[41152], b[5504], x);
      x = fma(-lu[41184], b[5536], x);
      x = fma(-lu[41216], b[5632], x);
      x = fma(-lu[41248], b[5696], x);
      x = fma(-lu[41280], b[5728], x);
      x = fma(-lu[41312], b[5760], x);
      x = fma(-lu[41344], b[5792], x);
      b[5824] = x;
    }
    {
      double x = b[5856];
      x = fma(-lu[41376], b[1088], x);
      x = fma(-lu[41408], b[1152], x);
      x = fma(-lu[41440], b[1312], x);
      x = fma(-lu[41472], b[1408], x);
      x = fma(-lu[41504], b[1440], x);
      x = fma(-lu[41536], b[1536], x);
      x = fma(-lu[41568], b[1568], x);
      x = fma(-lu[41600], b[1632], x);
      x = fma(-lu[41632], b[1728], x);
      x = fma(-lu[41664], b[2208], x);
      x = fma(-lu[41696], b[2240], x);
      x = fma(-lu[41728], b[2272], x);
      x = fma(-lu[41760], b[2592], x);
      x = fma(-lu[41792], b[2624], x);
      x = fma(-lu[41824], b[2656], x);
      x = fma(-lu[41856], b[2752], x);
      x = fma(-lu[41888], b[2784], x);
      x = fma(-lu[41920], b[2816], x);
      x = fma(-lu[41952], b[2848], x);
      x = fma(-lu[41984], b[2880], x);
      x = fma(-lu[42016], b[2912], x);
      x = fma(-lu[42048], b[2976], x);
      x = fma(-lu[42080], b[3008], x);
      x = fma(-lu[42112], b[3040], x);
      x = fma(-lu[42144], b[3072], x);
      x = fma(-lu[42176], b[3104], x);
      x = fma(-lu[42208], b[3136], x);
      x = fma(-lu[42240], b[3200], x);
      x = fma(-lu[42272], b[3232], x);
      x = fma(-lu[42304], b[3264], x);
      x = fma(-lu[42336], b[3296], x);
      x = fma(-lu[42368], b[3328], x);
      x = fma(-lu[42400], b[3360], x);
      x = fma(-lu[42432], b[3392], x);
      x = fma(-lu[42464], b[3424], x);
      x = fma(-lu[42496], b[3456], x);
      x = fma(-lu[42528], b[3488], x);
      x = fma(-lu[42560], b[3520], x);
      x = fma(-lu[42592], b[3552], x);
      x = fma(-lu[42624], b[3648], x);
      x = fma(-lu[42656], b[3680], x);
      x = fma(-lu[42688], b[3712], x);
      x = fma(-lu[42720], b[3744], x);
      x = fma(-lu[42752], b[3776], x);
      x = fma(-lu[42784], b[3808], x);
      x = fma(-lu[42816], b[3840], x);
      x = fma(-lu[42848], b[3872], x);
      x = fma(-lu[42880], b[3936], x);
      x = fma(-lu[42912], b[4032], x);
      x = fma(-lu[42944], b[4064], x);
      x = fma(-lu[42976], b[4128], x);
      x = fma(-lu[43008], b[4160], x);
      x = fma(-lu[43040], b[4192], x);
      x = fma(-lu[43072], b[4288], x);
      x = fma(-lu[43104], b[4320], x);
      x = fma(-lu[43136], b[4384], x);
      x = fma(-lu[43168], b[4448], x);
      x = fma(-lu[43200], b[4480], x);
      x = fma(-lu[43232], b[4544], x);
      x = fma(-lu[43264], b[4576], x);
      x = fma(-lu[43296], b[4672], x);
      x = fma(-lu[43328], b[4736], x);
      x = fma(-lu[43360], b[4800], x);
      x = fma(-lu[43392], b[4864], x);
      x = fma(-lu[43424], b[4896], x);
      x = fma(-lu[43456], b[4928], x);
      x = fma(-lu[43488], b[4960], x);
      x = fma(-lu[43520], b[4992], x);
      x = fma(-lu[43552], b[5088], x);
      x = fma(-lu[43584], b[5120], x);
      x = fma(-lu[43616], b[5152], x);
      x = fma(-lu[43648], b[5184], x);
      x = fma(-lu[43680], b[5216], x);
      x = fma(-lu[43712], b[5280], x);
      x = fma(-lu[43744], b[5312], x);
      x = fma(-lu[43776], b[5344], x);
      x = fma(-lu[43808], b[5376], x);
      x = fma(-lu[43840], b[5408], x);
      x = fma(-lu[43872], b[5440], x);
      x = fma(-lu[43904], b[5472], x);
      x = fma(-lu[43936], b[5504], x);
      x = fma(-lu[43968], b[5536], x);
      x = fma(-lu[44000], b[5600], x);
      x = fma(-lu[44032], b[5632], x);
      x = fma(-lu[44064], b[5696], x);
      x = fma(-lu[44096], b[5728], x);
      x = fma(-lu[44128], b[5760], x);
      x = fma(-lu[44160], b[5792], x);
      x = fma(-lu[44192], b[5824], x);
      b[5856] = x;
    }
}
__device__ __noinline__ void solve_0_2(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 105440;
    const double* __restrict__ vd = ws + 210560;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[5888];
      x = fma(-lu[44224], b[928], x);
      x = fma(-lu[44256], b[1088], x);
      x = fma(-lu[44288], b[1152], x);
      x = fma(-lu[44320], b[1312], x);
      x = fma(-lu[44352], b[1856], x);
      x = fma(-lu[44384], b[2272], x);
      x = fma(-lu[44416], b[2592], x);
      x = fma(-lu[44448], b[2624], x);
      x = fma(-lu[44480], b[2656], x);
      x = fma(-lu[44512], b[2752], x);
      x = fma(-lu[44544], b[2816], x);
      x = fma(-lu[44576], b[2848], x);
      x = fma(-lu[44608], b[2880], x);
      x = fma(-lu[44640], b[2912], x);
      x = fma(-lu[44672], b[2976], x);
      x = fma(-lu[44704], b[3008], x);
      x = fma(-lu[44736], b[3040], x);
      x = fma(-lu[44768], b[3072], x);
      x = fma(-lu[44800], b[3104], x);
      x = fma(-lu[44832], b[3136], x);
      x = fma(-lu[44864], b[3168], x);
      x = fma(-lu[44896], b[3200], x);
      x = fma(-lu[44928], b[3232], x);
      x = fma(-lu[44960], b[3264], x);
      x = fma(-lu[44992], b[3296], x);
      x = fma(-lu[45024], b[3328], x);
      x = fma(-lu[45056], b[3360], x);
      x = fma(-lu[45088], b[3392], x);
      x = fma(-lu[45120], b[3424], x);
      x = fma(-lu[45152], b[3456], x);
      x = fma(-lu[45184], b[3488], x);
      x = fma(-lu[45216], b[3520], x);
      x = fma(-lu[45248], b[3552], x);
      x = fma(-lu[45280], b[3648], x);
      x = fma(-lu[45312], b[3680], x);
      x = fma(-lu[45344], b[3712], x);
      x = fma(-lu[45376], b[3744], x);
      x = fma(-lu[45408], b[3776], x);
      x = fma(-lu[45440], b[3808], x);
      x = fma(-lu[45472], b[3840], x);
      x = fma(-lu[45504], b[3872], x);
      x = fma(-lu[45536], b[3936], x);
      x = fma(-lu[45568], b[3968], x);
      x = fma(-lu[45600], b[4032], x);
      x = fma(-lu[45632], b[4064], x);
      x = fma(-lu[45664], b[4128], x);
      x = fma(-lu[45696], b[4160], x);
      x = fma(-lu[45728], b[4192], x);
      x = fma(-lu[45760], b[4224], x);
      x = fma(-lu[45792], b[4288], x);
      x = fma(-lu[45824], b[4384], x);
      x = fma(-lu[45856], b[4416], x);
      x = fma(-lu[45888], b[4448], x);
      x = fma(-lu[45920], b[4480], x);
      x = fma(-lu[45952], b[4512], x);
      x = fma(-lu[45984], b[4544], x);
      x = fma(-lu[46016], b[4576], x);
      x = fma(-lu[46048], b[4608], x);
      x = fma(-lu[46080], b[4640], x);
      x = fma(-lu[46112], b[4672], x);
      x = fma(-lu[46144], b[4704], x);
      x = fma(-lu[46176], b[4736], x);
      x = fma(-lu[46208], b[4768], x);
      x = fma(-lu[46240], b[4800], x);
      x = fma(-lu[46272], b[4832], x);
      x = fma(-lu[46304], b[4864], x);
      x = fma(-lu[46336], b[4896], x);
      x = fma(-lu[46368], b[4928], x);
      x = fma(-lu[46400], b[4960], x);
      x = fma(-lu[46432], b[4992], x);
      x = fma(-lu[46464], b[5088], x);
      x = fma(-lu[46496], b[5120], x);
      x = fma(-lu[46528], b[5152], x);
      x = fma(-lu[46560], b[5184], x);
      x = fma(-lu[46592], b[5216], x);
      x = fma(-lu[46624], b[5280], x);
      x = fma(-lu[46656], b[5312], x);
      x = fma(-lu[46688], b[5408], x);
      x = fma(-lu[46720], b[5440], x);
      x = fma(-lu[46752], b[5472], x);
      x = fma(-lu[46784], b[5504], x);
      x = fma(-lu[46816], b[5536], x);
      x = fma(-lu[46848], b[5568], x);
      x = fma(-lu[46880], b[5632], x);
      x = fma(-lu[46912], b[5696], x);
      x = fma(-lu[46944], b[5728], x);
      x = fma(-lu[46976], b[5760], x);
      x = fma(-lu[47008], b[5792], x);
      x = fma(-lu[47040], b[5824], x);
      b[5888] = x;
    }
    {
      double x = b[5920];
      x = fma(-lu[47072], b[1024], x);
      x = fma(-lu[47104], b[1088], x);
      x = fma(-lu[47136], b[1184], x);
      x = fma(-lu[47168], b[1280], x);
      x = fma(-lu[47200], b[1312], x);
      x = fma(-lu[47232], b[1536], x);
      x = fma(-lu[47264], b[1632], x);
      x = fma(-lu[47296], b[1696], x);
      x = fma(-lu[47328], b[1728], x);
      x = fma(-lu[47360], b[1824], x);
      x = fma(-lu[47392], b[1856], x);
      x = fma(-lu[47424], b[1920], x);
      x = fma(-lu[47456], b[1952], x);
      x = fma(-lu[47488], b[1984], x);
      x = fma(-lu[47520], b[2016], x);
      x = fma(-lu[47552], b[2048], x);
      x = fma(-lu[47584], b[2080], x);
      x = fma(-lu[47616], b[2112], x);
      x = fma(-lu[47648], b[2144], x);
      x = fma(-lu[47680], b[2208], x);
      x = fma(-lu[47712], b[2272], x);
      x = fma(-lu[47744], b[2304], x);
      x = fma(-lu[47776], b[2336], x);
      x = fma(-lu[47808], b[2368], x);
      x = fma(-lu[47840], b[2400], x);
      x = fma(-lu[47872], b[2432], x);
      x = fma(-lu[47904], b[2464], x);
      x = fma(-lu[47936], b[2496], x);
      x = fma(-lu[47968], b[2528], x);
      x = fma(-lu[48000], b[2560], x);
      x = fma(-lu[48032], b[2592], x);
      x = fma(-lu[48064], b[2624], x);
      x = fma(-lu[48096], b[2656], x);
      x = fma(-lu[48128], b[2688], x);
      x = fma(-lu[48160], b[2784], x);
      x = fma(-lu[48192], b[2848], x);
      x = fma(-lu[48224], b[2880], x);
      x = fma(-lu[48256], b[2912], x);
      x = fma(-lu[48288], b[2976], x);
      x = fma(-lu[48320], b[3008], x);
      x = fma(-lu[48352], b[3040], x);
      x = fma(-lu[48384], b[3072], x);
      x = fma(-lu[48416], b[3104], x);
      x = fma(-lu[48448], b[3136], x);
      x = fma(-lu[48480], b[3168], x);
      x = fma(-lu[48512], b[3200], x);
      x = fma(-lu[48544], b[3232], x);
      x = fma(-lu[48576], b[3264], x);
      x = fma(-lu[48608], b[3296], x);
      x = fma(-lu[48640], b[3328], x);
      x = fma(-lu[48672], b[3360], x);
      x = fma(-lu[48704], b[3392], x);
      x = fma(-lu[48736], b[3424], x);
      x = fma(-lu[48768], b[3456], x);
      x = fma(-lu[48800], b[3488], x);
      x = fma(-lu[48832], b[3520], x);
      x = fma(-lu[48864], b[3552], x);
      x = fma(-lu[48896], b[3648], x);
      x = fma(-lu[48928], b[3712], x);
      x = fma(-lu[48960], b[3744], x);
      x = fma(-lu[48992], b[3776], x);
      x = fma(-lu[49024], b[3808], x);
      x = fma(-lu[49056], b[3840], x);
      x = fma(-lu[49088], b[3872], x);
      x = fma(-lu[49120], b[3904], x);
      x = fma(-lu[49152], b[3936], x);
      x = fma(-lu[49184], b[4032], x);
      x = fma(-lu[49216], b[4064], x);
      x = fma(-lu[49248], b[4096], x);
      x = fma(-lu[49280], b[4128], x);
      x = fma(-lu[49312], b[4160], x);
      x = fma(-lu[49344], b[4192], x);
      x = fma(-lu[49376], b[4288], x);
      x = fma(-lu[49408], b[4384], x);
      x = fma(-lu[49440], b[4448], x);
      x = fma(-lu[49472], b[4480], x);
      x = fma(-lu[49504], b[4544], x);
      x = fma(-lu[49536], b[4576], x);
      x = fma(-lu[49568], b[4608], x);
      x = fma(-lu[49600], b[4640], x);
      x = fma(-lu[49632], b[4672], x);
      x = fma(-lu[49664], b[4704], x);
      x = fma(-lu[49696], b[4736], x);
      x = fma(-lu[49728], b[4800], x);
      x = fma(-lu[49760], b[4832], x);
      x = fma(-lu[49792], b[4864], x);
      x = fma(-lu[49824], b[4896], x);
      x = fma(-lu[49856], b[4928], x);
      x = fma(-lu[49888], b[4960], x);
      x = fma(-lu[49920], b[4992], x);
      x = fma(-lu[49952], b[5024], x);
      x = fma(-lu[49984], b[5088], x);
      x = fma(-lu[50016], b[5120], x);
      x = fma(-lu[50048], b[5152], x);
      x = fma(-lu[50080], b[5184], x);
      x = fma(-lu[50112], b[5216], x);
      x = fma(-lu[50144], b[5248], x);
      x = fma(-lu[50176], b[5280], x);
      x = fma(-lu[50208], b[5312], x);
      x = fma(-lu[50240], b[5344], x);
      x = fma(-lu[50272], b[5376], x);
      x = fma(-lu[50304], b[5408], x);
      x = fma(-lu[50336], b[5440], x);
      x = fma(-lu[50368], b[5472], x);
      x = fma(-lu[50400], b[5504], x);
      x = fma(-lu[50432], b[5536], x);
      x = fma(-lu[50464], b[5568], x);
      x = fma(-lu[50496], b[5632], x);
      x = fma(-lu[50528], b[5696], x);
      x = fma(-lu[50560], b[5728], x);
      x = fma(-lu[50592], b[5760], x);
      x = fma(-lu[50624], b[5792], x);
      x = fma(-lu[50656], b[5824], x);
      x = fma(-lu[50688], b[5856], x);
      x = fma(-lu[50720], b[5888], x);
      b[5920] = x;
    }
    {
      double x = b[5952];
      x = fma(-lu[50752], b[1024], x);
      x = fma(-lu[50784], b[1088], x);
      x = fma(-lu[50816], b[1152], x);
      x = fma(-lu[50848], b[1248], x);
      x = fma(-lu[50880], b[1280], x);
      x = fma(-lu[50912], b[1312], x);
      x = fma(-lu[50944], b[1408], x);
      x = fma(-lu[50976], b[1440], x);
      x = fma(-lu[51008], b[1536], x);
      x = fma(-lu[51040], b[1568], x);
      x = fma(-lu[51072], b[1600], x);
      x = fma(-lu[51104], b[1696], x);
      x = fma(-lu[51136], b[1760], x);
      x = fma(-lu[51168], b[1824], x);
      x = fma(-lu[51200], b[1920], x);
      x = fma(-lu[51232], b[1952], x);
      x = fma(-lu[51264], b[1984], x);
      x = fma(-lu[51296], b[2016], x);
      x = fma(-lu[51328], b[2048], x);
      x = fma(-lu[51360], b[2080], x);
      x = fma(-lu[51392], b[2112], x);
      x = fma(-lu[51424], b[2144], x);
      x = fma(-lu[51456], b[2240], x);
      x = fma(-lu[51488], b[2272], x);
      x = fma(-lu[51520], b[2304], x);
      x = fma(-lu[51552], b[2336], x);
      x = fma(-lu[51584], b[2368], x);
      x = fma(-lu[51616], b[2400], x);
      x = fma(-lu[51648], b[2432], x);
      x = fma(-lu[51680], b[2464], x);
      x = fma(-lu[51712], b[2496], x);
      x = fma(-lu[51744], b[2528], x);
      x = fma(-lu[51776], b[2592], x);
      x = fma(-lu[51808], b[2624], x);
      x = fma(-lu[51840], b[2656], x);
      x = fma(-lu[51872], b[2752], x);
      x = fma(-lu[51904], b[2848], x);
      x = fma(-lu[51936], b[2880], x);
      x = fma(-lu[51968], b[2912], x);
      x = fma(-lu[52000], b[2944], x);
      x = fma(-lu[52032], b[2976], x);
      x = fma(-lu[52064], b[3008], x);
      x = fma(-lu[52096], b[3040], x);
      x = fma(-lu[52128], b[3072], x);
      x = fma(-lu[52160], b[3104], x);
      x = fma(-lu[52192], b[3136], x);
      x = fma(-lu[52224], b[3168], x);
      x = fma(-lu[52256], b[3200], x);
      x = fma(-lu[52288], b[3232], x);
      x = fma(-lu[52320], b[3264], x);
      x = fma(-lu[52352], b[3296], x);
      x = fma(-lu[52384], b[3328], x);
      x = fma(-lu[52416], b[3360], x);
      x = fma(-lu[52448], b[3392], x);
      x = fma(-lu[52480], b[3424], x);
      x = fma(-lu[52512], b[3456], x);
      x = fma(-lu[52544], b[3488], x);
      x = fma(-lu[52576], b[3520], x);
      x = fma(-lu[52608], b[3552], x);
      x = fma(-lu[52640], b[3648], x);
      x = fma(-lu[52672], b[3776], x);
      x = fma(-lu[52704], b[3808], x);
      x = fma(-lu[52736], b[3872], x);
      x = fma(-lu[52768], b[3904], x);
      x = fma(-lu[52800], b[4032], x);
      x = fma(-lu[52832], b[4064], x);
      x = fma(-lu[52864], b[4096], x);
      x = fma(-lu[52896], b[4128], x);
      x = fma(-lu[52928], b[4160], x);
      x = fma(-lu[52960], b[4192], x);
      x = fma(-lu[52992], b[4288], x);
      x = fma(-lu[53024], b[4384], x);
      x = fma(-lu[53056], b[4448], x);
      x = fma(-lu[53088], b[4480], x);
      x = fma(-lu[53120], b[4544], x);
      x = fma(-lu[53152], b[4576], x);
      x = fma(-lu[53184], b[4608], x);
      x = fma(-lu[53216], b[4640], x);
      x = fma(-lu[53248], b[4672], x);
      x = fma(-lu[53280], b[4704], x);
      x = fma(-lu[53312], b[4736], x);
      x = fma(-lu[53344], b[4800], x);
      x = fma(-lu[53376], b[4832], x);
      x = fma(-lu[53408], b[4864], x);
      x = fma(-lu[53440], b[4896], x);
      x = fma(-lu[53472], b[4928], x);
      x = fma(-lu[53504], b[4960], x);
      x = fma(-lu[53536], b[4992], x);
      x = fma(-lu[53568], b[5024], x);
      x = fma(-lu[53600], b[5088], x);
      x = fma(-lu[53632], b[5120], x);
      x = fma(-lu[53664], b[5152], x);
      x = fma(-lu[53696], b[5184], x);
      x = fma(-lu[53728], b[5216], x);
      x = fma(-lu[53760], b[5248], x);
      x = fma(-lu[53792], b[5280], x);
      x = fma(-lu[53824], b[5312], x);
      x = fma(-lu[53856], b[5344], x);
      x = fma(-lu[53888], b[5376], x);
      x = fma(-lu[53920], b[5408], x);
      x = fma(-lu[53952], b[5440], x);
      x = fma(-lu[53984], b[5472], x);
      x = fma(-lu[54016], b[5504], x);
      x = fma(-lu[54048], b[5536], x);
      x = fma(-lu[54080], b[5568], x);
      x = fma(-lu[54112], b[5632], x);
      x = fma(-lu[54144], b[5696], x);
      x = fma(-lu[54176], b[5728], x);
      x = fma(-lu[54208], b[5760], x);
      x = fma(-lu[54240], b[5792], x);
      x = fma(-lu[54272], b[5824], x);
      x = fma(-lu[54304], b[5856], x);
      x = fma(-lu[54336], b[5888], x);
      x = fma(-lu[54368], b[5920], x);
      b[5952] = x;
    }
    {
      double x = b[5984];
      x = fma(-lu[54400], b[160], x);
      x = fma(-lu[54432], b[256], x);
      x = fma(-lu[54464], b[288], x);
      x = fma(-lu[54496], b[320], x);
      x = fma(-lu[54528], b[352], x);
      x = fma(-lu[54560], b[448], x);
      x = fma(-lu[54592], b[832], x);
      x = fma(-lu[54624], b[864], x);
      x = fma(-lu[54656], b[896], x);
      x = fma(-lu[54688], b[1152], x);
      x = fma(-lu[54720], b[1216], x);
      x = fma(-lu[54752], b[1248], x);
      x = fma(-lu[54784], b[1280], x);
      x = fma(-lu[54816], b[1312], x);
      x = fma(-lu[54848], b[1344], x);
      x = fma(-lu[54880], b[1408], x);
      x = fma(-lu[54912], b[1472], x);
      x = fma(-lu[54944], b[1504], x);
      x = fma(-lu[54976], b[1568], x);
      x = fma(-lu[55008], b[1632], x);
      x = fma(-lu[55040], b[1728], x);
      x = fma(-lu[55072], b[1856], x);
      x = fma(-lu[55104], b[1920], x);
      x = fma(-lu[55136], b[1952], x);
      x = fma(-lu[55168], b[1984], x);
      x = fma(-lu[55200], b[2016], x);
      x = fma(-lu[55232], b[2048], x);
      x = fma(-lu[55264], b[2080], x);
      x = fma(-lu[55296], b[2112], x);
      x = fma(-lu[55328], b[2144], x);
      x = fma(-lu[55360], b[2208], x);
      x = fma(-lu[55392], b[2240], x);
      x = fma(-lu[55424], b[2272], x);
      x = fma(-lu[55456], b[2304], x);
      x = fma(-lu[55488], b[2368], x);
      x = fma(-lu[55520], b[2400], x);
      x = fma(-lu[55552], b[2432], x);
      x = fma(-lu[55584], b[2464], x);
      x = fma(-lu[55616], b[2496], x);
      x = fma(-lu[55648], b[2528], x);
      x = fma(-lu[55680], b[2560], x);
      x = fma(-lu[55712], b[2592], x);
      x = fma(-lu[55744], b[2624], x);
      x = fma(-lu[55776], b[2656], x);
      x = fma(-lu[55808], b[2752], x);
      x = fma(-lu[55840], b[2784], x);
      x = fma(-lu[55872], b[2816], x);
      x = fma(-lu[55904], b[2848], x);
      x = fma(-lu[55936], b[2880], x);
      x = fma(-lu[55968], b[2912], x);
      x = fma(-lu[56000], b[2944], x);
      x = fma(-lu[56032], b[2976], x);
      x = fma(-lu[56064], b[3008], x);
      x = fma(-lu[56096], b[3040], x);
      x = fma(-lu[56128], b[3072], x);
      x = fma(-lu[56160], b[3104], x);
      x = fma(-lu[56192], b[3136], x);
      x = fma(-lu[56224], b[3168], x);
      x = fma(-lu[56256], b[3200], x);
      x = fma(-lu[56288], b[3232], x);
      x = fma(-lu[56320], b[3264], x);
      x = fma(-lu[56352], b[3296], x);
      x = fma(-lu[56384], b[3328], x);
      x = fma(-lu[56416], b[3360], x);
      x = fma(-lu[56448], b[3392], x);
      x = fma(-lu[56480], b[3424], x);
      x = fma(-lu[56512], b[3456], x);
      x = fma(-lu[56544], b[3488], x);
      x = fma(-lu[56576], b[3520], x);
      x = fma(-lu[56608], b[3552], x);
      x = fma(-lu[56640], b[3584], x);
      x = fma(-lu[56672], b[3648], x);
      x = fma(-lu[56704], b[3712], x);
      x = fma(-lu[56736], b[3744], x);
      x = fma(-lu[56768], b[3776], x);
      x = fma(-lu[56800], b[3808], x);
      x = fma(-lu[56832], b[3840], x);
      x = fma(-lu[56864], b[3872], x);
      x = fma(-lu[56896], b[3904], x);
      x = fma(-lu[56928], b[3936], x);
      x = fma(-lu[56960], b[4000], x);
      x = fma(-lu[56992], b[4032], x);
      x = fma(-lu[57024], b[4064], x);
      x = fma(-lu[57056], b[4096], x);
      x = fma(-lu[57088], b[4128], x);
      x = fma(-lu[57120], b[4160], x);
      x = fma(-lu[57152], b[4192], x);
      x = fma(-lu[57184], b[4288], x);
      x = fma(-lu[57216], b[4320], x);
      x = fma(-lu[57248], b[4352], x);
      x = fma(-lu[57280], b[4384], x);
      x = fma(-lu[57312], b[4448], x);
      x = fma(-lu[57344], b[4480], x);
      x = fma(-lu[57376], b[4512], x);
      x = fma(-lu[57408], b[4544], x);
      x = fma(-lu[57440], b[4576], x);
      x = fma(-lu[57472], b[4608], x);
      x = fma(-lu[57504], b[4640], x);
      x = fma(-lu[57536], b[4672], x);
      x = fma(-lu[57568], b[4704], x);
      x = fma(-lu[57600], b[4736], x);
      x = fma(-lu[57632], b[4800], x);
      x = fma(-lu[57664], b[4832], x);
      x = fma(-lu[57696], b[4864], x);
      x = fma(-lu[57728], b[4896], x);
      x = fma(-lu[57760], b[4928], x);
      x = fma(-lu[57792], b[4960], x);
      x = fma(-lu[57824], b[4992], x);
      x = fma(-lu[57856], b[5056], x);
      x = fma(-lu[57888], b[5088], x);
      x = fma(-lu[57920], b[5120], x);
      x = fma(-lu[57952], b[5152], x);
      x = fma(-lu[57984], b[5184], x);
      x = fma(-lu[58016], b[5216], x);
      x = fma(-lu[58048], b[5248], x);
      x = fma(-lu[58080], b[5280], x);
      x = fma(-lu[58112], b[5312], x);
      x = fma(-lu[58144], b[5344], x);
      x = fma(-lu[58176], b[5376], x);
      x = fma(-lu[58208], b[5408], x);
      x = fma(-lu[58240], b[5440], x);
      x = fma(-lu[58272], b[5472], x);
      x = fma(-lu[58304], b[5504], x);
      x = fma(-lu[58336], b[5536], x);
      x = fma(-lu[58368], b[5568], x);
      x = fma(-lu[58400], b[5600], x);
      x = fma(-lu[58432], b[5632], x);
      x = fma(-lu[58464], b[5664], x);
      x = fma(-lu[58496], b[5696], x);
      x = fma(-lu[58528], b[5728], x);
      x = fma(-lu[58560], b[5760], x);
      x = fma(-lu[58592], b[5792], x);
      x = fma(-lu[58624], b[5824], x);
      x = fma(-lu[58656], b[5856], x);
      x = fma(-lu[58688], b[5888], x);
      x = fma(-lu[58720], b[5920], x);
      x = fma(-lu[58752], b[5952], x);
      b[5984] = x;
    }
    {
      double x = b[6016];
      x = fma(-lu[58784], b[160], x);
      x = fma(-lu[58816], b[256], x);
      x = fma(-lu[58848], b[288], x);
      x = fma(-lu[58880], b[320], x);
      x = fma(-lu[58912], b[352], x);
      x = fma(-lu[58944], b[384], x);
      x = fma(-lu[58976], b[416], x);
      x = fma(-lu[59008], b[448], x);
      x = fma(-lu[59040], b[576], x);
      x = fma(-lu[59072], b[608], x);
      x = fma(-lu[59104], b[640], x);
      x = fma(-lu[59136], b[672], x);
      x = fma(-lu[59168], b[704], x);
      x = fma(-lu[59200], b[736], x);
      x = fma(-lu[59232], b[768], x);
      x = fma(-lu[59264], b[800], x);
      x = fma(-lu[59296], b[832], x);
      x = fma(-lu[59328], b[864], x);
      x = fma(-lu[59360], b[896], x);
      x = fma(-lu[59392], b[928], x);
      x = fma(-lu[59424], b[992], x);
      x = fma(-lu[59456], b[1088], x);
      x = fma(-lu[59488], b[1120], x);
      x = fma(-lu[59520], b[1152], x);
      x = fma(-lu[59552], b[1184], x);
      x = fma(-lu[59584], b[1216], x);
      x = fma(-lu[59616], b[1248], x);
      x = fma(-lu[59648], b[1280], x);
      x = fma(-lu[59680], b[1312], x);
      x = fma(-lu[59712], b[1344], x);
      x = fma(-lu[59744], b[1376], x);
      x = fma(-lu[59776], b[1408], x);
      x = fma(-lu[59808], b[1440], x);
      x = fma(-lu[59840], b[1472], x);
      x = fma(-lu[59872], b[1504], x);
      x = fma(-lu[59904], b[1536], x);
      x = fma(-lu[59936], b[1568], x);
      x = fma(-lu[59968], b[1600], x);
      x = fma(-lu[60000], b[1632], x);
      x = fma(-lu[60032], b[1664], x);
      x = fma(-lu[60064], b[1696], x);
      x = fma(-lu[60096], b[1728], x);
      x = fma(-lu[60128], b[1760], x);
      x = fma(-lu[60160], b[1792], x);
      x = fma(-lu[60192], b[1824], x);
      x = fma(-lu[60224], b[1856], x);
      x = fma(-lu[60256], b[1888], x);
      x = fma(-lu[60288], b[2176], x);
      x = fma(-lu[60320], b[2208], x);
      x = fma(-lu[60352], b[2240], x);
      x = fma(-lu[60384], b[2560], x);
      x = fma(-lu[60416], b[2624], x);
      x = fma(-lu[60448], b[2656], x);
      x = fma(-lu[60480], b[2752], x);
      x = fma(-lu[60512], b[2784], x);
      x = fma(-lu[60544], b[2816], x);
      x = fma(-lu[60576], b[2848], x);
      x = fma(-lu[60608], b[2944], x);
      x = fma(-lu[60640], b[3008], x);
      x = fma(-lu[60672], b[3136], x);
      x = fma(-lu[60704], b[3168], x);
      x = fma(-lu[60736], b[3232], x);
      x = fma(-lu[60768], b[3520], x);
      x = fma(-lu[60800], b[3552], x);
      x = fma(-lu[60832], b[3584], x);
      x = fma(-lu[60864], b[3680], x);
      x = fma(-lu[60896], b[3712], x);
      x = fma(-lu[60928], b[3744], x);
      x = fma(-lu[60960], b[3840], x);
      x = fma(-lu[60992], b[3872], x);
      x = fma(-lu[61024], b[3936], x);
      x = fma(-lu[61056], b[3968], x);
      x = fma(-lu[61088], b[4000], x);
      x = fma(-lu[61120], b[4096], x);
      x = fma(-lu[61152], b[4128], x);
      x = fma(-lu[61184], b[4160], x);
      x = fma(-lu[61216], b[4192], x);
      x = fma(-lu[61248], b[4224], x);
      x = fma(-lu[61280], b[4288], x);
      x = fma(-lu[61312], b[4320], x);
      x = fma(-lu[61344], b[4352], x);
      x = fma(-lu[61376], b[4384], x);
      x = fma(-lu[61408], b[4416], x);
      x = fma(-lu[61440], b[4448], x);
      x = fma(-lu[61472], b[4480], x);
      x = fma(-lu[61504], b[4512], x);
      x = fma(-lu[61536], b[4544], x);
      x = fma(-lu[61568], b[4576], x);
      x = fma(-lu[61600], b[4608], x);
      x = fma(-lu[61632], b[4640], x);
      x = fma(-lu[61664], b[4672], x);
      x = fma(-lu[61696], b[4704], x);
      x = fma(-lu[61728], b[4736], x);
      x = fma(-lu[61760], b[4768], x);
      x = fma(-lu[61792], b[4800], x);
      x = fma(-lu[61824], b[4832], x);
      x = fma(-lu[61856], b[4864], x);
      x = fma(-lu[61888], b[4896], x);
      x = fma(-lu[61920], b[4928], x);
      x = fma(-lu[61952], b[4960], x);
      x = fma(-lu[61984], b[4992], x);
      x = fma(-lu[62016], b[5024], x);
      x = fma(-lu[62048], b[5056], x);
      x = fma(-lu[62080], b[5088], x);
      x = fma(-lu[62112], b[5120], x);
      x = fma(-lu[62144], b[5152], x);
      x = fma(-lu[62176], b[5184], x);
      x = fma(-lu[62208], b[5216], x);
      x = fma(-lu[62240], b[5248], x);
      x = fma(-lu[62272], b[5280], x);
      x = fma(-lu[62304], b[5312], x);
      x = fma(-lu[62336], b[5344], x);
      x = fma(-lu[62368], b[5376], x);
      x = fma(-lu[62400], b[5408], x);
      x = fma(-lu[62432], b[5440], x);
      x = fma(-lu[62464], b[5472], x);
      x = fma(-lu[62496], b[5504], x);
      x = fma(-lu[62528], b[5536], x);
      x = fma(-lu[62560], b[5568], x);
      x = fma(-lu[62592], b[5600], x);
      x = fma(-lu[62624], b[5632], x);
      x = fma(-lu[62656], b[5664], x);
      x = fma(-lu[62688], b[5696], x);
      x = fma(-lu[62720], b[5728], x);
      x = fma(-lu[62752], b[5760], x);
      x = fma(-lu[62784], b[5792], x);
      x = fma(-lu[62816], b[5824], x);
      x = fma(-lu[62848], b[5856], x);
      x = fma(-lu[62880], b[5888], x);
      x = fma(-lu[62912], b[5920], x);
      x = fma(-lu[62944], b[5952], x);
      x = fma(-lu[62976], b[5984], x);
      b[6016] = x;
    }
    {
      double x = b[6016];
      b[6016] = x * vd[6016];
    }
    {
      double x = b[5984];
      x = fma(-lu[63008], b[6016], x);
      b[5984] = x * vd[5984];
    }
    {
      double x = b[5952];
      x = fma(-lu[63040], b[5984], x);
      x = fma(-lu[63072], b[6016], x);
      b[5952] = x * vd[5952];
    }
    {
      double x = b[5920];
      x = fma(-lu[63104], b[5952], x);
      x = fma(-lu[63136], b[5984], x);
      x = fma(-lu[63168], b[6016], x);
      b[5920] = x * vd[5920];
    }
    {
      double x = b[5888];
      x = fma(-lu[63200], b[5920], x);
      x = fma(-lu[63232], b[5952], x);
      x = fma(-lu[63264], b[5984], x);
      x = fma(-lu[63296], b[6016], x);
      b[5888] = x * vd[5888];
    }
    {
      double x = b[5856];
      x = fma(-lu[63328], b[5888], x);
      x = fma(-lu[63360], b[5920], x);
      x = fma(-lu[63392], b[5952], x);
      x = fma(-lu[63424], b[5984], x);
      x = fma(-lu[63456], b[6016], x);
      b[5856] = x * vd[5856];
    }
    {
      double x = b[5824];
      x = fma(-lu[63488], b[5888], x);
      x = fma(-lu[63520], b[5920], x);
      x = fma(-lu[63552], b[5952], x);
      x = fma(-lu[63584], b[5984], x);
      x = fma(-lu[63616], b[6016], x);
      b[5824] = x * vd[5824];
    }
    {
      double x = b[5792];
      x = fma(-lu[63648], b[5824], x);
      x = fma(-lu[63680], b[5888], x);
      x = fma(-lu[63712], b[5920], x);
      x = fma(-lu[63744], b[5952], x);
      x = fma(-lu[63776], b[5984], x);
      x = fma(-lu[63808], b[6016], x);
      b[5792] = x * vd[5792];
    }
    {
      double x = b[5760];
      x = fma(-lu[63840], b[5792], x);
      x = fma(-lu[63872], b[5824], x);
      x = fma(-lu[63904], b[5888], x);
      x = fma(-lu[63936], b[5920], x);
      x = fma(-lu[63968], b[5952], x);
      x = fma(-lu[64000], b[5984], x);
      x = fma(-lu[64032], b[6016], x);
      b[5760] = x * vd[5760];
    }
    {
      double x = b[5728];
      x = fma(-lu[64064], b[5760], x);
      x = fma(-lu[64096], b[5792], x);
      x = fma(-lu[64128], b[5824], x);
      x = fma(-lu[64160], b[5888], x);
      x = fma(-lu[64192], b[5920], x);
      x = fma(-lu[64224], b[5952], x);
      x = fma(-lu[64256], b[5984], x);
      x = fma(-lu[64288], b[6016], x);
      b[5728] = x * vd[5728];
    }
    {
      double x = b[5696];
      x = fma(-lu[64320], b[5728], x);
      x = fma(-lu[64352], b[5760], x);
      x = fma(-lu[64384], b[5792], x);
      x = fma(-lu[64416], b[5824], x);
      x = fma(-lu[64448], b[5888], x);
      x = fma(-lu[64480], b[5920], x);
      x = fma(-lu[64512], b[5952], x);
      x = fma(-lu[64544], b[5984], x);
      x = fma(-lu[64576], b[6016], x);
      b[5696] = x * vd[5696];
    }
    {
      double x = b[5664];
      x = fma(-lu[64608], b[5696], x);
      x = fma(-lu[64640], b[5728], x);
      x = fma(-lu[64672], b[5760], x);
      x = fma(-lu[64704], b[5792], x);
      x = fma(-lu[64736], b[5824], x);
      x = fma(-lu[64768], b[5856], x);
      x = fma(-lu[64800], b[5888], x);
      x = fma(-lu[64832], b[5920], x);
      x = fma(-lu[64864], b[5952], x);
      x = fma(-lu[64896], b[5984], x);
      x = fma(-lu[64928], b[6016], x);
      b[5664] = x * vd[5664];
    }
    {
      double x = b[5632];
      x = fma(-lu[64960], b[5728], x);
      x = fma(-lu[64992], b[5760], x);
      x = fma(-lu[65024], b[5792], x);
      x = fma(-lu[65056], b[5824], x);
      x = fma(-lu[65088], b[5888], x);
      x = fma(-lu[65120], b[5920], x);
      x = fma(-lu[65152], b[5952], x);
      x = fma(-lu[65184], b[5984], x);
      x = fma(-lu[65216], b[6016], x);
      b[5632] = x * vd[5632];
    }
    {
      double x = b[5600];
      x = fma(-lu[65248], b[5632], x);
      x = fma(-lu[65280], b[5728], x);
      x = fma(-lu[65312], b[5792], x);
      x = fma(-lu[65344], b[5824], x);
      x = fma(-lu[65376], b[5888], x);
      x = fma(-lu[65408], b[5920], x);
      x = fma(-lu[65440], b[5952], x);
      x = fma(-lu[65472], b[5984], x);
      x = fma(-lu[65504], b[6016], x);
      b[5600] = x * vd[5600];
    }
    {
      double x = b[5568];
      x = fma(-lu[65536], b[5632], x);
      x = fma(-lu[65568], b[5728], x);
      x = fma(-lu[65600], b[5792], x);
      x = fma(-lu[65632], b[5824], x);
      x = fma(-lu[65664], b[5888], x);
      x = fma(-lu[65696], b[5920], x);
      x = fma(-lu[65728], b[5952], x);
      x = fma(-lu[65760], b[5984], x);
      x = fma(-lu[65792], b[6016], x);
      b[5568] = x * vd[5568];
    }
    {
      double x = b[5536];
      x = fma(-lu[65824], b[5728], x);
      x = fma(-lu[65856], b[5792], x);
      x = fma(-lu[65888], b[5824], x);
      x = fma(-lu[65920], b[5888], x);
      x = fma(-lu[65952], b[5920], x);
      x = fma(-lu[65984], b[5952], x);
      x = fma(-lu[66016], b[5984], x);
      x = fma(-lu[66048], b[6016], x);
      b[5536] = x * vd[5536];
    }
    {
      double x = b[5504];
      x = fma(-lu[66080], b[5536], x);
      x = fma(-lu[66112], b[5728], x);
      x = fma(-lu[66144], b[5792], x);
      x = fma(-lu[66176], b[5824], x);
      x = fma(-lu[66208], b[5888], x);
      x = fma(-lu[66240], b[5920], x);
      x = fma(-lu[66272], b[5952], x);
      x = fma(-lu[66304], b[5984], x);
      x = fma(-lu[66336], b[6016], x);
      b[5504] = x * vd[5504];
    }
    {
      double x = b[5472];
      x = fma(-lu[66368], b[5504], x);
      x = fma(-lu[66400], b[5536], x);
      x = fma(-lu[66432], b[5728], x);
      x = fma(-lu[66464], b[5792], x);
      x = fma(-lu[66496], b[5824], x);
      x = fma(-lu[66528], b[5888], x);
      x = fma(-lu[66560], b[5920], x);
      x = fma(-lu[66592], b[5952], x);
      x = fma(-lu[66624], b[5984], x);
      x = fma(-lu[66656], b[6016], x);
      b[5472] = x * vd[5472];
    }
    {
      double x = b[5440];
      x = fma(-lu[66688], b[5472], x);
      x = fma(-lu[66720], b[5536], x);
      x = fma(-lu[66752], b[5728], x);
      x = fma(-lu[66784], b[5792], x);
      x = fma(-lu[66816], b[5824], x);
      x = fma(-lu[66848], b[5888], x);
      x = fma(-lu[66880], b[5920], x);
      x = fma(-lu[66912], b[5952], x);
      x = fma(-lu[66944], b[5984], x);
      x = fma(-lu[66976], b[6016], x);
      b[5440] = x * vd[5440];
    }
    {
      double x = b[5408];
      x = fma(-lu[67008], b[5440], x);
      x = fma(-lu[67040], b[5472], x);
      x = fma(-lu[67072], b[5536], x);
      x = fma(-lu[67104], b[5728], x);
      x = fma(-lu[67136], b[5792], x);
      x = fma(-lu[67168], b[5824], x);
      x = fma(-lu[67200], b[5888], x);
      x = fma(-lu[67232], b[5920], x);
      x = fma(-lu[67264], b[5952], x);
      x = fma(-lu[67296], b[5984], x);
      x = fma(-lu[67328], b[6016], x);
      b[5408] = x * vd[5408];
    }
    {
      double x = b[5376];
      x = fma(-lu[67360], b[5408], x);
      x = fma(-lu[67392], b[5472], x);
      x = fma(-lu[67424], b[5696], x);
      x = fma(-lu[67456], b[5792], x);
      x = fma(-lu[67488], b[5824], x);
      x = fma(-lu[67520], b[5888], x);
      x = fma(-lu[67552], b[5920], x);
      x = fma(-lu[67584], b[5952], x);
      x = fma(-lu[67616], b[5984], x);
      x = fma(-lu[67648], b[6016], x);
      b[5376] = x * vd[5376];
    }
    {
      double x = b[5344];
      x = fma(-lu[67680], b[5472], x);
      x = fma(-lu[67712], b[5536], x);
      x = fma(-lu[67744], b[5792], x);
      x = fma(-lu[67776], b[5824], x);
      x = fma(-lu[67808], b[5888], x);
      x = fma(-lu[67840], b[5920], x);
      x = fma(-lu[67872], b[5952], x);
      x = fma(-lu[67904], b[5984], x);
      x = fma(-lu[67936], b[6016], x);
      b[5344] = x * vd[5344];
    }
    {
      double x = b[5312];
      x = fma(-lu[67968], b[5472], x);
      x = fma(-lu[68000], b[5536], x);
      x = fma(-lu[68032], b[5792], x);
      x = fma(-lu[68064], b[5824], x);
      x = fma(-lu[68096], b[5888], x);
      x = fma(-lu[68128], b[5920], x);
      x = fma(-lu[68160], b[5952], x);
      x = fma(-lu[68192], b[5984], x);
      x = fma(-lu[68224], b[6016], x);
      b[5312] = x * vd[5312];
    }
    {
      double x = b[5280];
      x = fma(-lu[68256], b[5312], x);
      x = fma(-lu[68288], b[5408], x);
      x = fma(-lu[68320], b[5472], x);
      x = fma(-lu[68352], b[5536], x);
      x = fma(-lu[68384], b[5792], x);
      x = fma(-lu[68416], b[5824], x);
      x = fma(-lu[68448], b[5888], x);
      x = fma(-lu[68480], b[5920], x);
      x = fma(-lu[68512], b[5952], x);
      x = fma(-lu[68544], b[5984], x);
      x = fma(-lu[68576], b[6016], x);
      b[5280] = x * vd[5280];
    }
}
__device__ __noinline__ void solve_0_3(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 105440;
    const double* __restrict__ vd = ws + 210560;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[5248];
      x = fma(-lu[68608], b[5312], x);
      x = fma(-lu[68640], b[5344], x);
      x = fma(-lu[68672], b[5472], x);
      x = fma(-lu[68704], b[5504], x);
      x = fma(-lu[68736], b[5536], x);
      x = fma(-lu[68768], b[5792], x);
      x = fma(-lu[68800], b[5824], x);
      x = fma(-lu[68832], b[5888], x);
      x = fma(-lu[68864], b[5920], x);
      x = fma(-lu[68896], b[5952], x);
      x = fma(-lu[68928], b[5984], x);
      x = fma(-lu[68960], b[6016], x);
      b[5248] = x * vd[5248];
    }
    {
      double x = b[5216];
      x = fma(-lu[68992], b[5312], x);
      x = fma(-lu[69024], b[5408], x);
      x = fma(-lu[69056], b[5472], x);
      x = fma(-lu[69088], b[5504], x);
      x = fma(-lu[69120], b[5536], x);
      x = fma(-lu[69152], b[5728], x);
      x = fma(-lu[69184], b[5760], x);
      x = fma(-lu[69216], b[5792], x);
      x = fma(-lu[69248], b[5824], x);
      x = fma(-lu[69280], b[5888], x);
      x = fma(-lu[69312], b[5920], x);
      x = fma(-lu[69344], b[5952], x);
      x = fma(-lu[69376], b[5984], x);
      x = fma(-lu[69408], b[6016], x);
      b[5216] = x * vd[5216];
    }
    {
      double x = b[5184];
      x = fma(-lu[69440], b[5472], x);
      x = fma(-lu[69472], b[5792], x);
      x = fma(-lu[69504], b[5824], x);
      x = fma(-lu[69536], b[5888], x);
      x = fma(-lu[69568], b[5920], x);
      x = fma(-lu[69600], b[5952], x);
      x = fma(-lu[69632], b[5984], x);
      x = fma(-lu[69664], b[6016], x);
      b[5184] = x * vd[5184];
    }
    {
      double x = b[5152];
      x = fma(-lu[69696], b[5184], x);
      x = fma(-lu[69728], b[5280], x);
      x = fma(-lu[69760], b[5312], x);
      x = fma(-lu[69792], b[5536], x);
      x = fma(-lu[69824], b[5792], x);
      x = fma(-lu[69856], b[5824], x);
      x = fma(-lu[69888], b[5888], x);
      x = fma(-lu[69920], b[5952], x);
      x = fma(-lu[69952], b[5984], x);
      x = fma(-lu[69984], b[6016], x);
      b[5152] = x * vd[5152];
    }
    {
      double x = b[5120];
      x = fma(-lu[70016], b[5184], x);
      x = fma(-lu[70048], b[5312], x);
      x = fma(-lu[70080], b[5536], x);
      x = fma(-lu[70112], b[5792], x);
      x = fma(-lu[70144], b[5824], x);
      x = fma(-lu[70176], b[5888], x);
      x = fma(-lu[70208], b[5952], x);
      x = fma(-lu[70240], b[5984], x);
      x = fma(-lu[70272], b[6016], x);
      b[5120] = x * vd[5120];
    }
    {
      double x = b[5088];
      x = fma(-lu[70304], b[5184], x);
      x = fma(-lu[70336], b[5312], x);
      x = fma(-lu[70368], b[5536], x);
      x = fma(-lu[70400], b[5792], x);
      x = fma(-lu[70432], b[5824], x);
      x = fma(-lu[70464], b[5888], x);
      x = fma(-lu[70496], b[5952], x);
      x = fma(-lu[70528], b[5984], x);
      x = fma(-lu[70560], b[6016], x);
      b[5088] = x * vd[5088];
    }
    {
      double x = b[5056];
      x = fma(-lu[70592], b[5088], x);
      x = fma(-lu[70624], b[5120], x);
      x = fma(-lu[70656], b[5152], x);
      x = fma(-lu[70688], b[5184], x);
      x = fma(-lu[70720], b[5312], x);
      x = fma(-lu[70752], b[5408], x);
      x = fma(-lu[70784], b[5504], x);
      x = fma(-lu[70816], b[5536], x);
      x = fma(-lu[70848], b[5792], x);
      x = fma(-lu[70880], b[5824], x);
      x = fma(-lu[70912], b[5888], x);
      x = fma(-lu[70944], b[5920], x);
      x = fma(-lu[70976], b[5952], x);
      x = fma(-lu[71008], b[5984], x);
      x = fma(-lu[71040], b[6016], x);
      b[5056] = x * vd[5056];
    }
    {
      double x = b[5024];
      x = fma(-lu[71072], b[5184], x);
      x = fma(-lu[71104], b[5248], x);
      x = fma(-lu[71136], b[5376], x);
      x = fma(-lu[71168], b[5568], x);
      x = fma(-lu[71200], b[5760], x);
      x = fma(-lu[71232], b[5792], x);
      x = fma(-lu[71264], b[5824], x);
      x = fma(-lu[71296], b[5856], x);
      x = fma(-lu[71328], b[5888], x);
      x = fma(-lu[71360], b[5920], x);
      x = fma(-lu[71392], b[5952], x);
      x = fma(-lu[71424], b[5984], x);
      x = fma(-lu[71456], b[6016], x);
      b[5024] = x * vd[5024];
    }
    {
      double x = b[4992];
      x = fma(-lu[71488], b[5088], x);
      x = fma(-lu[71520], b[5184], x);
      x = fma(-lu[71552], b[5312], x);
      x = fma(-lu[71584], b[5536], x);
      x = fma(-lu[71616], b[5792], x);
      x = fma(-lu[71648], b[5824], x);
      x = fma(-lu[71680], b[5888], x);
      x = fma(-lu[71712], b[5952], x);
      x = fma(-lu[71744], b[5984], x);
      x = fma(-lu[71776], b[6016], x);
      b[4992] = x * vd[4992];
    }
    {
      double x = b[4960];
      x = fma(-lu[71808], b[4992], x);
      x = fma(-lu[71840], b[5088], x);
      x = fma(-lu[71872], b[5184], x);
      x = fma(-lu[71904], b[5312], x);
      x = fma(-lu[71936], b[5536], x);
      x = fma(-lu[71968], b[5792], x);
      x = fma(-lu[72000], b[5824], x);
      x = fma(-lu[72032], b[5888], x);
      x = fma(-lu[72064], b[5952], x);
      x = fma(-lu[72096], b[5984], x);
      x = fma(-lu[72128], b[6016], x);
      b[4960] = x * vd[4960];
    }
    {
      double x = b[4928];
      x = fma(-lu[72160], b[4960], x);
      x = fma(-lu[72192], b[4992], x);
      x = fma(-lu[72224], b[5088], x);
      x = fma(-lu[72256], b[5184], x);
      x = fma(-lu[72288], b[5312], x);
      x = fma(-lu[72320], b[5536], x);
      x = fma(-lu[72352], b[5792], x);
      x = fma(-lu[72384], b[5824], x);
      x = fma(-lu[72416], b[5888], x);
      x = fma(-lu[72448], b[5952], x);
      x = fma(-lu[72480], b[5984], x);
      x = fma(-lu[72512], b[6016], x);
      b[4928] = x * vd[4928];
    }
    {
      double x = b[4896];
      x = fma(-lu[72544], b[4928], x);
      x = fma(-lu[72576], b[4960], x);
      x = fma(-lu[72608], b[4992], x);
      x = fma(-lu[72640], b[5088], x);
      x = fma(-lu[72672], b[5184], x);
      x = fma(-lu[72704], b[5312], x);
      x = fma(-lu[72736], b[5536], x);
      x = fma(-lu[72768], b[5792], x);
      x = fma(-lu[72800], b[5824], x);
      x = fma(-lu[72832], b[5888], x);
      x = fma(-lu[72864], b[5952], x);
      x = fma(-lu[72896], b[5984], x);
      x = fma(-lu[72928], b[6016], x);
      b[4896] = x * vd[4896];
    }
    {
      double x = b[4864];
      x = fma(-lu[72960], b[4896], x);
      x = fma(-lu[72992], b[4928], x);
      x = fma(-lu[73024], b[4960], x);
      x = fma(-lu[73056], b[4992], x);
      x = fma(-lu[73088], b[5088], x);
      x = fma(-lu[73120], b[5184], x);
      x = fma(-lu[73152], b[5312], x);
      x = fma(-lu[73184], b[5536], x);
      x = fma(-lu[73216], b[5792], x);
      x = fma(-lu[73248], b[5824], x);
      x = fma(-lu[73280], b[5888], x);
      x = fma(-lu[73312], b[5952], x);
      x = fma(-lu[73344], b[5984], x);
      x = fma(-lu[73376], b[6016], x);
      b[4864] = x * vd[4864];
    }
    {
      double x = b[4832];
      x = fma(-lu[73408], b[4864], x);
      x = fma(-lu[73440], b[4928], x);
      x = fma(-lu[73472], b[4960], x);
      x = fma(-lu[73504], b[4992], x);
      x = fma(-lu[73536], b[5088], x);
      x = fma(-lu[73568], b[5184], x);
      x = fma(-lu[73600], b[5312], x);
      x = fma(-lu[73632], b[5536], x);
      x = fma(-lu[73664], b[5792], x);
      x = fma(-lu[73696], b[5824], x);
      x = fma(-lu[73728], b[5888], x);
      x = fma(-lu[73760], b[5952], x);
      x = fma(-lu[73792], b[5984], x);
      x = fma(-lu[73824], b[6016], x);
      b[4832] = x * vd[4832];
    }
    {
      double x = b[4800];
      x = fma(-lu[73856], b[5184], x);
      x = fma(-lu[73888], b[5216], x);
      x = fma(-lu[73920], b[5472], x);
      x = fma(-lu[73952], b[5760], x);
      x = fma(-lu[73984], b[5792], x);
      x = fma(-lu[74016], b[5824], x);
      x = fma(-lu[74048], b[5888], x);
      x = fma(-lu[74080], b[5920], x);
      x = fma(-lu[74112], b[5952], x);
      x = fma(-lu[74144], b[5984], x);
      x = fma(-lu[74176], b[6016], x);
      b[4800] = x * vd[4800];
    }
    {
      double x = b[4768];
      x = fma(-lu[74208], b[4832], x);
      x = fma(-lu[74240], b[4864], x);
      x = fma(-lu[74272], b[4896], x);
      x = fma(-lu[74304], b[4928], x);
      x = fma(-lu[74336], b[4960], x);
      x = fma(-lu[74368], b[4992], x);
      x = fma(-lu[74400], b[5088], x);
      x = fma(-lu[74432], b[5312], x);
      x = fma(-lu[74464], b[5536], x);
      x = fma(-lu[74496], b[5792], x);
      x = fma(-lu[74528], b[5824], x);
      x = fma(-lu[74560], b[5888], x);
      x = fma(-lu[74592], b[5952], x);
      x = fma(-lu[74624], b[5984], x);
      x = fma(-lu[74656], b[6016], x);
      b[4768] = x * vd[4768];
    }
    {
      double x = b[4736];
      x = fma(-lu[74688], b[5184], x);
      x = fma(-lu[74720], b[5792], x);
      x = fma(-lu[74752], b[5824], x);
      x = fma(-lu[74784], b[5888], x);
      x = fma(-lu[74816], b[5952], x);
      x = fma(-lu[74848], b[5984], x);
      x = fma(-lu[74880], b[6016], x);
      b[4736] = x * vd[4736];
    }
    {
      double x = b[4704];
      x = fma(-lu[74912], b[4832], x);
      x = fma(-lu[74944], b[4864], x);
      x = fma(-lu[74976], b[4928], x);
      x = fma(-lu[75008], b[4960], x);
      x = fma(-lu[75040], b[4992], x);
      x = fma(-lu[75072], b[5088], x);
      x = fma(-lu[75104], b[5312], x);
      x = fma(-lu[75136], b[5536], x);
      x = fma(-lu[75168], b[5792], x);
      x = fma(-lu[75200], b[5824], x);
      x = fma(-lu[75232], b[5888], x);
      x = fma(-lu[75264], b[5952], x);
      x = fma(-lu[75296], b[5984], x);
      x = fma(-lu[75328], b[6016], x);
      b[4704] = x * vd[4704];
    }
    {
      double x = b[4672];
      x = fma(-lu[75360], b[4736], x);
      x = fma(-lu[75392], b[5184], x);
      x = fma(-lu[75424], b[5792], x);
      x = fma(-lu[75456], b[5824], x);
      x = fma(-lu[75488], b[5888], x);
      x = fma(-lu[75520], b[5920], x);
      x = fma(-lu[75552], b[5952], x);
      x = fma(-lu[75584], b[5984], x);
      x = fma(-lu[75616], b[6016], x);
      b[4672] = x * vd[4672];
    }
    {
      double x = b[4640];
      x = fma(-lu[75648], b[4704], x);
      x = fma(-lu[75680], b[4832], x);
      x = fma(-lu[75712], b[4864], x);
      x = fma(-lu[75744], b[4928], x);
      x = fma(-lu[75776], b[4960], x);
      x = fma(-lu[75808], b[4992], x);
      x = fma(-lu[75840], b[5088], x);
      x = fma(-lu[75872], b[5312], x);
      x = fma(-lu[75904], b[5536], x);
      x = fma(-lu[75936], b[5792], x);
      x = fma(-lu[75968], b[5824], x);
      x = fma(-lu[76000], b[5888], x);
      x = fma(-lu[76032], b[5952], x);
      x = fma(-lu[76064], b[5984], x);
      x = fma(-lu[76096], b[6016], x);
      b[4640] = x * vd[4640];
    }
    {
      double x = b[4608];
      x = fma(-lu[76128], b[4640], x);
      x = fma(-lu[76160], b[4704], x);
      x = fma(-lu[76192], b[4832], x);
      x = fma(-lu[76224], b[4864], x);
      x = fma(-lu[76256], b[4960], x);
      x = fma(-lu[76288], b[4992], x);
      x = fma(-lu[76320], b[5088], x);
      x = fma(-lu[76352], b[5312], x);
      x = fma(-lu[76384], b[5536], x);
      x = fma(-lu[76416], b[5792], x);
      x = fma(-lu[76448], b[5824], x);
      x = fma(-lu[76480], b[5888], x);
      x = fma(-lu[76512], b[5952], x);
      x = fma(-lu[76544], b[5984], x);
      x = fma(-lu[76576], b[6016], x);
      b[4608] = x * vd[4608];
    }
    {
      double x = b[4576];
      x = fma(-lu[76608], b[5184], x);
      x = fma(-lu[76640], b[5792], x);
      x = fma(-lu[76672], b[5824], x);
      x = fma(-lu[76704], b[5888], x);
      x = fma(-lu[76736], b[5952], x);
      x = fma(-lu[76768], b[5984], x);
      x = fma(-lu[76800], b[6016], x);
      b[4576] = x * vd[4576];
    }
    {
      double x = b[4544];
      x = fma(-lu[76832], b[4576], x);
      x = fma(-lu[76864], b[5184], x);
      x = fma(-lu[76896], b[5792], x);
      x = fma(-lu[76928], b[5824], x);
      x = fma(-lu[76960], b[5888], x);
      x = fma(-lu[76992], b[5952], x);
      x = fma(-lu[77024], b[5984], x);
      x = fma(-lu[77056], b[6016], x);
      b[4544] = x * vd[4544];
    }
    {
      double x = b[4512];
      x = fma(-lu[77088], b[5184], x);
      x = fma(-lu[77120], b[5792], x);
      x = fma(-lu[77152], b[5824], x);
      x = fma(-lu[77184], b[5888], x);
      x = fma(-lu[77216], b[5952], x);
      x = fma(-lu[77248], b[5984], x);
      x = fma(-lu[77280], b[6016], x);
      b[4512] = x * vd[4512];
    }
    {
      double x = b[4480];
      x = fma(-lu[77312], b[5120], x);
      x = fma(-lu[77344], b[5184], x);
      x = fma(-lu[77376], b[5408], x);
      x = fma(-lu[77408], b[5792], x);
      x = fma(-lu[77440], b[5824], x);
      x = fma(-lu[77472], b[5888], x);
      x = fma(-lu[77504], b[5952], x);
      x = fma(-lu[77536], b[5984], x);
      x = fma(-lu[77568], b[6016], x);
      b[4480] = x * vd[4480];
    }
    {
      double x = b[4448];
      x = fma(-lu[77600], b[5184], x);
      x = fma(-lu[77632], b[5792], x);
      x = fma(-lu[77664], b[5824], x);
      x = fma(-lu[77696], b[5888], x);
      x = fma(-lu[77728], b[5952], x);
      x = fma(-lu[77760], b[5984], x);
      x = fma(-lu[77792], b[6016], x);
      b[4448] = x * vd[4448];
    }
    {
      double x = b[4416];
      x = fma(-lu[77824], b[4704], x);
      x = fma(-lu[77856], b[4832], x);
      x = fma(-lu[77888], b[4960], x);
      x = fma(-lu[77920], b[5088], x);
      x = fma(-lu[77952], b[5824], x);
      x = fma(-lu[77984], b[5952], x);
      x = fma(-lu[78016], b[5984], x);
      x = fma(-lu[78048], b[6016], x);
      b[4416] = x * vd[4416];
    }
    {
      double x = b[4384];
      x = fma(-lu[78080], b[4544], x);
      x = fma(-lu[78112], b[4576], x);
      x = fma(-lu[78144], b[5184], x);
      x = fma(-lu[78176], b[5792], x);
      x = fma(-lu[78208], b[5824], x);
      x = fma(-lu[78240], b[5888], x);
      x = fma(-lu[78272], b[5952], x);
      x = fma(-lu[78304], b[5984], x);
      x = fma(-lu[78336], b[6016], x);
      b[4384] = x * vd[4384];
    }
    {
      double x = b[4352];
      x = fma(-lu[78368], b[4384], x);
      x = fma(-lu[78400], b[4576], x);
      x = fma(-lu[78432], b[4736], x);
      x = fma(-lu[78464], b[5184], x);
      x = fma(-lu[78496], b[5792], x);
      x = fma(-lu[78528], b[5824], x);
      x = fma(-lu[78560], b[5888], x);
      x = fma(-lu[78592], b[5952], x);
      x = fma(-lu[78624], b[5984], x);
      x = fma(-lu[78656], b[6016], x);
      b[4352] = x * vd[4352];
    }
    {
      double x = b[4320];
      x = fma(-lu[78688], b[5184], x);
      x = fma(-lu[78720], b[5792], x);
      x = fma(-lu[78752], b[5824], x);
      x = fma(-lu[78784], b[5888], x);
      x = fma(-lu[78816], b[5952], x);
      x = fma(-lu[78848], b[5984], x);
      x = fma(-lu[78880], b[6016], x);
      b[4320] = x * vd[4320];
    }
    {
      double x = b[4288];
      x = fma(-lu[78912], b[5184], x);
      x = fma(-lu[78944], b[5792], x);
      x = fma(-lu[78976], b[5824], x);
      x = fma(-lu[79008], b[5888], x);
      x = fma(-lu[79040], b[5952], x);
      x = fma(-lu[79072], b[5984], x);
      x = fma(-lu[79104], b[6016], x);
      b[4288] = x * vd[4288];
    }
    {
      double x = b[4256];
      x = fma(-lu[79136], b[4288], x);
      x = fma(-lu[79168], b[4544], x);
      x = fma(-lu[79200], b[4576], x);
      x = fma(-lu[79232], b[5184], x);
      x = fma(-lu[79264], b[5792], x);
      x = fma(-lu[79296], b[5824], x);
      x = fma(-lu[79328], b[5888], x);
      x = fma(-lu[79360], b[5952], x);
      x = fma(-lu[79392], b[5984], x);
      x = fma(-lu[79424], b[6016], x);
      b[4256] = x * vd[4256];
    }
    {
      double x = b[4224];
      x = fma(-lu[79456], b[4416], x);
      x = fma(-lu[79488], b[4640], x);
      x = fma(-lu[79520], b[4704], x);
      x = fma(-lu[79552], b[4832], x);
      x = fma(-lu[79584], b[4960], x);
      x = fma(-lu[79616], b[4992], x);
      x = fma(-lu[79648], b[5088], x);
      x = fma(-lu[79680], b[5312], x);
      x = fma(-lu[79712], b[5536], x);
      x = fma(-lu[79744], b[6016], x);
      b[4224] = x * vd[4224];
    }
    {
      double x = b[4192];
      x = fma(-lu[79776], b[4288], x);
      x = fma(-lu[79808], b[5184], x);
      x = fma(-lu[79840], b[5792], x);
      x = fma(-lu[79872], b[5824], x);
      x = fma(-lu[79904], b[5888], x);
      x = fma(-lu[79936], b[5952], x);
      x = fma(-lu[79968], b[5984], x);
      x = fma(-lu[80000], b[6016], x);
      b[4192] = x * vd[4192];
    }
    {
      double x = b[4160];
      x = fma(-lu[80032], b[4192], x);
      x = fma(-lu[80064], b[4288], x);
      x = fma(-lu[80096], b[5184], x);
      x = fma(-lu[80128], b[5792], x);
      x = fma(-lu[80160], b[5824], x);
      x = fma(-lu[80192], b[5888], x);
      x = fma(-lu[80224], b[5952], x);
      x = fma(-lu[80256], b[5984], x);
      x = fma(-lu[80288], b[6016], x);
      b[4160] = x * vd[4160];
    }
    {
      double x = b[4128];
      x = fma(-lu[80320], b[4288], x);
      x = fma(-lu[80352], b[5184], x);
      x = fma(-lu[80384], b[5792], x);
      x = fma(-lu[80416], b[5824], x);
      x = fma(-lu[80448], b[5888], x);
      x = fma(-lu[80480], b[5952], x);
      x = fma(-lu[80512], b[5984], x);
      x = fma(-lu[80544], b[6016], x);
      b[4128] = x * vd[4128];
    }
    {
      double x = b[4096];
      x = fma(-lu[80576], b[4160], x);
      x = fma(-lu[80608], b[4192], x);
      x = fma(-lu[80640], b[4544], x);
      x = fma(-lu[80672], b[4576], x);
      x = fma(-lu[80704], b[5184], x);
      x = fma(-lu[80736], b[5792], x);
      x = fma(-lu[80768], b[5824], x);
      x = fma(-lu[80800], b[5888], x);
      x = fma(-lu[80832], b[5952], x);
      x = fma(-lu[80864], b[5984], x);
      x = fma(-lu[80896], b[6016], x);
      b[4096] = x * vd[4096];
    }
    {
      double x = b[4064];
      x = fma(-lu[80928], b[5184], x);
      x = fma(-lu[80960], b[5792], x);
      x = fma(-lu[80992], b[5824], x);
      x = fma(-lu[81024], b[5888], x);
      x = fma(-lu[81056], b[5952], x);
      x = fma(-lu[81088], b[5984], x);
      x = fma(-lu[81120], b[6016], x);
      b[4064] = x * vd[4064];
    }
    {
      double x = b[4032];
      x = fma(-lu[81152], b[4064], x);
      x = fma(-lu[81184], b[5184], x);
      x = fma(-lu[81216], b[5792], x);
      x = fma(-lu[81248], b[5824], x);
      x = fma(-lu[81280], b[5888], x);
      x = fma(-lu[81312], b[5952], x);
      x = fma(-lu[81344], b[5984], x);
      x = fma(-lu[81376], b[6016], x);
      b[4032] = x * vd[4032];
    }
    {
      double x = b[4000];
      x = fma(-lu[81408], b[4576], x);
      x = fma(-lu[81440], b[5184], x);
      x = fma(-lu[81472], b[5792], x);
      x = fma(-lu[81504], b[5824], x);
      x = fma(-lu[81536], b[5888], x);
      x = fma(-lu[81568], b[5952], x);
      x = fma(-lu[81600], b[5984], x);
      x = fma(-lu[81632], b[6016], x);
      b[4000] = x * vd[4000];
    }
    {
      double x = b[3968];
      x = fma(-lu[81664], b[4224], x);
      x = fma(-lu[81696], b[4416], x);
      x = fma(-lu[81728], b[4704], x);
      x = fma(-lu[81760], b[4832], x);
      x = fma(-lu[81792], b[4960], x);
      x = fma(-lu[81824], b[5088], x);
      x = fma(-lu[81856], b[5312], x);
      x = fma(-lu[81888], b[5536], x);
      x = fma(-lu[81920], b[6016], x);
      b[3968] = x * vd[3968];
    }
    {
      double x = b[3936];
      x = fma(-lu[81952], b[4160], x);
      x = fma(-lu[81984], b[4192], x);
      x = fma(-lu[82016], b[4288], x);
      x = fma(-lu[82048], b[5184], x);
      x = fma(-lu[82080], b[5792], x);
      x = fma(-lu[82112], b[5824], x);
      x = fma(-lu[82144], b[5888], x);
      x = fma(-lu[82176], b[5952], x);
      x = fma(-lu[82208], b[5984], x);
      x = fma(-lu[82240], b[6016], x);
      b[3936] = x * vd[3936];
    }
    {
      double x = b[3904];
      x = fma(-lu[82272], b[4096], x);
      x = fma(-lu[82304], b[4544], x);
      x = fma(-lu[82336], b[4576], x);
      x = fma(-lu[82368], b[4608], x);
      x = fma(-lu[82400], b[5824], x);
      x = fma(-lu[82432], b[5952], x);
      x = fma(-lu[82464], b[5984], x);
      x = fma(-lu[82496], b[6016], x);
      b[3904] = x * vd[3904];
    }
    {
      double x = b[3872];
      x = fma(-lu[82528], b[4384], x);
      x = fma(-lu[82560], b[4736], x);
      x = fma(-lu[82592], b[5184], x);
      x = fma(-lu[82624], b[5792], x);
      x = fma(-lu[82656], b[5824], x);
      x = fma(-lu[82688], b[5888], x);
      x = fma(-lu[82720], b[5952], x);
      x = fma(-lu[82752], b[5984], x);
      x = fma(-lu[82784], b[6016], x);
      b[3872] = x * vd[3872];
    }
    {
      double x = b[3840];
      x = fma(-lu[82816], b[4160], x);
      x = fma(-lu[82848], b[4192], x);
      x = fma(-lu[82880], b[4288], x);
      x = fma(-lu[82912], b[5184], x);
      x = fma(-lu[82944], b[5792], x);
      x = fma(-lu[82976], b[5824], x);
      x = fma(-lu[83008], b[5888], x);
      x = fma(-lu[83040], b[5952], x);
      x = fma(-lu[83072], b[5984], x);
      x = fma(-lu[83104], b[6016], x);
      b[3840] = x * vd[3840];
    }
    {
      double x = b[3808];
      x = fma(-lu[83136], b[4448], x);
      x = fma(-lu[83168], b[5184], x);
      x = fma(-lu[83200], b[5792], x);
      x = fma(-lu[83232], b[5824], x);
      x = fma(-lu[83264], b[5888], x);
      x = fma(-lu[83296], b[5920], x);
      x = fma(-lu[83328], b[5952], x);
      x = fma(-lu[83360], b[5984], x);
      x = fma(-lu[83392], b[6016], x);
      b[3808] = x * vd[3808];
    }
    {
      double x = b[3776];
      x = fma(-lu[83424], b[4864], x);
      x = fma(-lu[83456], b[4928], x);
      x = fma(-lu[83488], b[5504], x);
      x = fma(-lu[83520], b[5792], x);
      x = fma(-lu[83552], b[5824], x);
      x = fma(-lu[83584], b[5888], x);
      x = fma(-lu[83616], b[5952], x);
      x = fma(-lu[83648], b[5984], x);
      x = fma(-lu[83680], b[6016], x);
      b[3776] = x * vd[3776];
    }
    {
      double x = b[3744];
      x = fma(-lu[83712], b[4160], x);
      x = fma(-lu[83744], b[4192], x);
      x = fma(-lu[83776], b[4288], x);
      x = fma(-lu[83808], b[5184], x);
      x = fma(-lu[83840], b[5792], x);
      x = fma(-lu[83872], b[5824], x);
      x = fma(-lu[83904], b[5888], x);
      x = fma(-lu[83936], b[5952], x);
      x = fma(-lu[83968], b[5984], x);
      x = fma(-lu[84000], b[6016], x);
      b[3744] = x * vd[3744];
    }
    {
      double x = b[3712];
      x = fma(-lu[84032], b[4160], x);
      x = fma(-lu[84064], b[4192], x);
      x = fma(-lu[84096], b[4288], x);
      x = fma(-lu[84128], b[5184], x);
      x = fma(-lu[84160], b[5792], x);
      x = fma(-lu[84192], b[5824], x);
      x = fma(-lu[84224], b[5888], x);
      x = fma(-lu[84256], b[5952], x);
      x = fma(-lu[84288], b[5984], x);
      x = fma(-lu[84320], b[6016], x);
      b[3712] = x * vd[3712];
    }
    {
      double x = b[3680];
      x = fma(-lu[84352], b[4576], x);
      x = fma(-lu[84384], b[4800], x);
      x = fma(-lu[84416], b[5184], x);
      x = fma(-lu[84448], b[5792], x);
      x = fma(-lu[84480], b[5824], x);
      x = fma(-lu[84512], b[5888], x);
      x = fma(-lu[84544], b[5952], x);
      x = fma(-lu[84576], b[5984], x);
      x = fma(-lu[84608], b[6016], x);
      b[3680] = x * vd[3680];
    }
    {
      double x = b[3648];
      x = fma(-lu[84640], b[4448], x);
      x = fma(-lu[84672], b[5184], x);
      x = fma(-lu[84704], b[5792], x);
      x = fma(-lu[84736], b[5824], x);
      x = fma(-lu[84768], b[5888], x);
      x = fma(-lu[84800], b[5920], x);
      x = fma(-lu[84832], b[5952], x);
      x = fma(-lu[84864], b[5984], x);
      x = fma(-lu[84896], b[6016], x);
      b[3648] = x * vd[3648];
    }
    {
      double x = b[3616];
      x = fma(-lu[84928], b[4448], x);
      x = fma(-lu[84960], b[4512], x);
      x = fma(-lu[84992], b[5184], x);
      x = fma(-lu[85024], b[5792], x);
      x = fma(-lu[85056], b[5824], x);
      x = fma(-lu[85088], b[5888], x);
      x = fma(-lu[85120], b[5920], x);
      x = fma(-lu[85152], b[5952], x);
      x = fma(-lu[85184], b[5984], x);
      x = fma(-lu[85216], b[6016], x);
      b[3616] = x * vd[3616];
    }
    {
      double x = b[3584];
      x = fma(-lu[85248], b[5184], x);
      x = fma(-lu[85280], b[5792], x);
      x = fma(-lu[85312], b[5824], x);
      x = fma(-lu[85344], b[5888], x);
      x = fma(-lu[85376], b[5952], x);
      x = fma(-lu[85408], b[5984], x);
      x = fma(-lu[85440], b[6016], x);
      b[3584] = x * vd[3584];
    }
    {
      double x = b[3552];
      x = fma(-lu[85472], b[5184], x);
      x = fma(-lu[85504], b[5792], x);
      x = fma(-lu[85536], b[5824], x);
      x = fma(-lu[85568], b[5888], x);
      x = fma(-lu[85600], b[5952], x);
      x = fma(-lu[85632], b[5984], x);
      x = fma(-lu[85664], b[6016], x);
      b[3552] = x * vd[3552];
    }
    {
      double x = b[3520];
      x = fma(-lu[85696], b[3552], x);
      x = fma(-lu[85728], b[4128], x);
      x = fma(-lu[85760], b[5792], x);
      x = fma(-lu[85792], b[5824], x);
      x = fma(-lu[85824], b[5888], x);
      x = fma(-lu[85856], b[5952], x);
      x = fma(-lu[85888], b[5984], x);
      x = fma(-lu[85920], b[6016], x);
      b[3520] = x * vd[3520];
    }
    {
      double x = b[3488];
      x = fma(-lu[85952], b[5792], x);
      x = fma(-lu[85984], b[5824], x);
      x = fma(-lu[86016], b[5888], x);
      x = fma(-lu[86048], b[5952], x);
      x = fma(-lu[86080], b[5984], x);
      x = fma(-lu[86112], b[6016], x);
      b[3488] = x * vd[3488];
    }
    {
      double x = b[3456];
      x = fma(-lu[86144], b[5792], x);
      x = fma(-lu[86176], b[5824], x);
      x = fma(-lu[86208], b[5888], x);
      x = fma(-lu[86240], b[5952], x);
      x = fma(-lu[86272], b[5984], x);
      x = fma(-lu[86304], b[6016], x);
      b[3456] = x * vd[3456];
    }
    {
      double x = b[3424];
      x = fma(-lu[86336], b[5792], x);
      x = fma(-lu[86368], b[5824], x);
      x = fma(-lu[86400], b[5888], x);
      x = fma(-lu[86432], b[5952], x);
      x = fma(-lu[86464], b[5984], x);
      x = fma(-lu[86496], b[6016], x);
      b[3424] = x * vd[3424];
    }
    {
      double x = b[3392];
      x = fma(-lu[86528], b[5792], x);
      x = fma(-lu[86560], b[5824], x);
      x = fma(-lu[86592], b[5888], x);
      x = fma(-lu[86624], b[5952], x);
      x = fma(-lu[86656], b[5984], x);
      x = fma(-lu[86688], b[6016], x);
      b[3392] = x * vd[3392];
    }
    {
      double x = b[3360];
      x = fma(-lu[86720], b[5184], x);
      x = fma(-lu[86752], b[5792], x);
      x = fma(-lu[86784], b[5824], x);
      x = fma(-lu[86816], b[5888], x);
      x = fma(-lu[86848], b[5952], x);
      x = fma(-lu[86880], b[5984], x);
      x = fma(-lu[86912], b[6016], x);
      b[3360] = x * vd[3360];
    }
    {
      double x = b[3328];
      x = fma(-lu[86944], b[5184], x);
      x = fma(-lu[86976], b[5792], x);
      x = fma(-lu[87008], b[5824], x);
      x = fma(-lu[87040], b[5888], x);
      x = fma(-lu[87072], b[5952], x);
      x = fma(-lu[87104], b[5984], x);
      x = fma(-lu[87136], b[6016], x);
      b[3328] = x * vd[3328];
    }
    {
      double x = b[3296];
      x = fma(-lu[87168], b[5792], x);
      x = fma(-lu[87200], b[5824], x);
      x = fma(-lu[87232], b[5888], x);
      x = fma(-lu[87264], b[5952], x);
      x = fma(-lu[87296], b[5984], x);
      x = fma(-lu[87328], b[6016], x);
      b[3296] = x * vd[3296];
    }
    {
      double x = b[3264];
      x = fma(-lu[87360], b[5792], x);
      x = fma(-lu[87392], b[5824], x);
      x = fma(-lu[87424], b[5888], x);
      x = fma(-lu[87456], b[5952], x);
      x = fma(-lu[87488], b[5984], x);
      x = fma(-lu[87520], b[6016], x);
      b[3264] = x * vd[3264];
    }
    {
      double x = b[3232];
      x = fma(-lu[87552], b[4448], x);
      x = fma(-lu[87584], b[5184], x);
      x = fma(-lu[87616], b[5792], x);
      x = fma(-lu[87648], b[5824], x);
      x = fma(-lu[87680], b[5888], x);
      x = fma(-lu[87712], b[5920], x);
      x = fma(-lu[87744], b[5952], x);
      x = fma(-lu[87776], b[5984], x);
      x = fma(-lu[87808], b[6016], x);
      b[3232] = x * vd[3232];
    }
    {
      double x = b[3200];
      x = fma(-lu[87840], b[5184], x);
      x = fma(-lu[87872], b[5792], x);
      x = fma(-lu[87904], b[5824], x);
      x = fma(-lu[87936], b[5888], x);
      x = fma(-lu[87968], b[5952], x);
      x = fma(-lu[88000], b[5984], x);
      x = fma(-lu[88032], b[6016], x);
      b[3200] = x * vd[3200];
    }
    {
      double x = b[3168];
      x = fma(-lu[88064], b[5184], x);
      x = fma(-lu[88096], b[5792], x);
      x = fma(-lu[88128], b[5824], x);
      x = fma(-lu[88160], b[5888], x);
      x = fma(-lu[88192], b[5952], x);
      x = fma(-lu[88224], b[5984], x);
      x = fma(-lu[88256], b[6016], x);
      b[3168] = x * vd[3168];
    }
    {
      double x = b[3136];
      x = fma(-lu[88288], b[5184], x);
      x = fma(-lu[88320], b[5792], x);
      x = fma(-lu[88352], b[5824], x);
      x = fma(-lu[88384], b[5888], x);
      x = fma(-lu[88416], b[5952], x);
      x = fma(-lu[88448], b[5984], x);
      x = fma(-lu[88480], b[6016], x);
      b[3136] = x * vd[3136];
    }
    {
      double x = b[3104];
      x = fma(-lu[88512], b[5792], x);
      x = fma(-lu[88544], b[5824], x);
      x = fma(-lu[88576], b[5888], x);
      x = fma(-lu[88608], b[5952], x);
      x = fma(-lu[88640], b[5984], x);
      x = fma(-lu[88672], b[6016], x);
      b[3104] = x * vd[3104];
    }
    {
      double x = b[3072];
      x = fma(-lu[88704], b[3136], x);
      x = fma(-lu[88736], b[3232], x);
      x = fma(-lu[88768], b[5184], x);
      x = fma(-lu[88800], b[5792], x);
      x = fma(-lu[88832], b[5824], x);
      x = fma(-lu[88864], b[5888], x);
      x = fma(-lu[88896], b[5952], x);
      x = fma(-lu[88928], b[5984], x);
      x = fma(-lu[88960], b[6016], x);
      b[3072] = x * vd[3072];
    }
    {
      double x = b[3040];
      x = fma(-lu[88992], b[3808], x);
      x = fma(-lu[89024], b[5184], x);
      x = fma(-lu[89056], b[5792], x);
      x = fma(-lu[89088], b[5824], x);
      x = fma(-lu[89120], b[5888], x);
      x = fma(-lu[89152], b[5952], x);
      x = fma(-lu[89184], b[5984], x);
      b[3040] = x * vd[3040];
    }
    {
      double x = b[3008];
      x = fma(-lu[89216], b[3552], x);
      x = fma(-lu[89248], b[5184], x);
      x = fma(-lu[89280], b[5792], x);
      x = fma(-lu[89312], b[5824], x);
      x = fma(-lu[89344], b[5888], x);
      x = fma(-lu[89376], b[5952], x);
      x = fma(-lu[89408], b[5984], x);
      x = fma(-lu[89440], b[6016], x);
      b[3008] = x * vd[3008];
    }
    {
      double x = b[2976];
      x = fma(-lu[89472], b[5696], x);
      x = fma(-lu[89504], b[5792], x);
      x = fma(-lu[89536], b[5824], x);
      x = fma(-lu[89568], b[5888], x);
      x = fma(-lu[89600], b[5952], x);
      x = fma(-lu[89632], b[5984], x);
      x = fma(-lu[89664], b[6016], x);
      b[2976] = x * vd[2976];
    }
    {
      double x = b[2944];
      x = fma(-lu[89696], b[3232], x);
      x = fma(-lu[89728], b[5952], x);
      x = fma(-lu[89760], b[5984], x);
      x = fma(-lu[89792], b[6016], x);
      b[2944] = x * vd[2944];
    }
    {
      double x = b[2912];
      x = fma(-lu[89824], b[3872], x);
      x = fma(-lu[89856], b[5792], x);
      x = fma(-lu[89888], b[5824], x);
      x = fma(-lu[89920], b[5888], x);
      x = fma(-lu[89952], b[5952], x);
      x = fma(-lu[89984], b[5984], x);
      x = fma(-lu[90016], b[6016], x);
      b[2912] = x * vd[2912];
    }
    {
      double x = b[2880];
      x = fma(-lu[90048], b[4736], x);
      x = fma(-lu[90080], b[5792], x);
      x = fma(-lu[90112], b[5824], x);
      x = fma(-lu[90144], b[5888], x);
      x = fma(-lu[90176], b[5952], x);
      x = fma(-lu[90208], b[5984], x);
      x = fma(-lu[90240], b[6016], x);
      b[2880] = x * vd[2880];
    }
    {
      double x = b[2848];
      x = fma(-lu[90272], b[4480], x);
      x = fma(-lu[90304], b[5792], x);
      x = fma(-lu[90336], b[5824], x);
      x = fma(-lu[90368], b[5888], x);
      x = fma(-lu[90400], b[5952], x);
      x = fma(-lu[90432], b[5984], x);
      x = fma(-lu[90464], b[6016], x);
      b[2848] = x * vd[2848];
    }
    {
      double x = b[2816];
      x = fma(-lu[90496], b[4576], x);
      x = fma(-lu[90528], b[5184], x);
      x = fma(-lu[90560], b[5888], x);
      x = fma(-lu[90592], b[5952], x);
      x = fma(-lu[90624], b[5984], x);
      x = fma(-lu[90656], b[6016], x);
      b[2816] = x * vd[2816];
    }
    {
      double x = b[2784];
      x = fma(-lu[90688], b[4288], x);
      x = fma(-lu[90720], b[5184], x);
      x = fma(-lu[90752], b[5824], x);
      x = fma(-lu[90784], b[5952], x);
      x = fma(-lu[90816], b[5984], x);
      x = fma(-lu[90848], b[6016], x);
      b[2784] = x * vd[2784];
    }
    {
      double x = b[2752];
      x = fma(-lu[90880], b[3136], x);
      x = fma(-lu[90912], b[5184], x);
      x = fma(-lu[90944], b[5888], x);
      x = fma(-lu[90976], b[5952], x);
      x = fma(-lu[91008], b[6016], x);
      b[2752] = x * vd[2752];
    }
    {
      double x = b[2720];
      x = fma(-lu[91040], b[3712], x);
      x = fma(-lu[91072], b[3744], x);
      x = fma(-lu[91104], b[3840], x);
      x = fma(-lu[91136], b[3936], x);
      x = fma(-lu[91168], b[4160], x);
      x = fma(-lu[91200], b[4192], x);
      x = fma(-lu[91232], b[4288], x);
      b[2720] = x * vd[2720];
    }
    {
      double x = b[2688];
      x = fma(-lu[91264], b[4448], x);
      x = fma(-lu[91296], b[5792], x);
      x = fma(-lu[91328], b[5824], x);
      x = fma(-lu[91360], b[5888], x);
      x = fma(-lu[91392], b[5920], x);
      x = fma(-lu[91424], b[5952], x);
      x = fma(-lu[91456], b[6016], x);
      b[2688] = x * vd[2688];
    }
}
__device__ __noinline__ void solve_0_4(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 105440;
    const double* __restrict__ vd = ws + 210560;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[2656];
      x = fma(-lu[91488], b[5184], x);
      x = fma(-lu[91520], b[5792], x);
      x = fma(-lu[91552], b[5824], x);
      x = fma(-lu[91584], b[5888], x);
      x = fma(-lu[91616], b[5952], x);
      x = fma(-lu[91648], b[5984], x);
      x = fma(-lu[91680], b[6016], x);
      b[2656] = x * vd[2656];
    }
    {
      double x = b[2624];
      x = fma(-lu[91712], b[5184], x);
      x = fma(-lu[91744], b[5792], x);
      x = fma(-lu[91776], b[5824], x);
      x = fma(-lu[91808], b[5888], x);
      x = fma(-lu[91840], b[5952], x);
      x = fma(-lu[91872], b[5984], x);
      x = fma(-lu[91904], b[6016], x);
      b[2624] = x * vd[2624];
    }
    {
      double x = b[2592];
      x = fma(-lu[91936], b[4448], x);
      x = fma(-lu[91968], b[5792], x);
      x = fma(-lu[92000], b[5824], x);
      x = fma(-lu[92032], b[5888], x);
      x = fma(-lu[92064], b[5952], x);
      x = fma(-lu[92096], b[6016], x);
      b[2592] = x * vd[2592];
    }
    {
      double x = b[2560];
      x = fma(-lu[92128], b[4544], x);
      x = fma(-lu[92160], b[5184], x);
      x = fma(-lu[92192], b[5824], x);
      x = fma(-lu[92224], b[5952], x);
      x = fma(-lu[92256], b[5984], x);
      x = fma(-lu[92288], b[6016], x);
      b[2560] = x * vd[2560];
    }
    {
      double x = b[2528];
      x = fma(-lu[92320], b[5824], x);
      x = fma(-lu[92352], b[5952], x);
      x = fma(-lu[92384], b[5984], x);
      x = fma(-lu[92416], b[6016], x);
      b[2528] = x * vd[2528];
    }
    {
      double x = b[2496];
      x = fma(-lu[92448], b[5824], x);
      x = fma(-lu[92480], b[5952], x);
      x = fma(-lu[92512], b[5984], x);
      x = fma(-lu[92544], b[6016], x);
      b[2496] = x * vd[2496];
    }
    {
      double x = b[2464];
      x = fma(-lu[92576], b[5824], x);
      x = fma(-lu[92608], b[5952], x);
      x = fma(-lu[92640], b[5984], x);
      x = fma(-lu[92672], b[6016], x);
      b[2464] = x * vd[2464];
    }
    {
      double x = b[2432];
      x = fma(-lu[92704], b[5824], x);
      x = fma(-lu[92736], b[5952], x);
      x = fma(-lu[92768], b[5984], x);
      x = fma(-lu[92800], b[6016], x);
      b[2432] = x * vd[2432];
    }
    {
      double x = b[2400];
      x = fma(-lu[92832], b[5824], x);
      x = fma(-lu[92864], b[5952], x);
      x = fma(-lu[92896], b[5984], x);
      x = fma(-lu[92928], b[6016], x);
      b[2400] = x * vd[2400];
    }
    {
      double x = b[2368];
      x = fma(-lu[92960], b[5824], x);
      x = fma(-lu[92992], b[5952], x);
      x = fma(-lu[93024], b[5984], x);
      x = fma(-lu[93056], b[6016], x);
      b[2368] = x * vd[2368];
    }
    {
      double x = b[2336];
      x = fma(-lu[93088], b[5184], x);
      x = fma(-lu[93120], b[5824], x);
      x = fma(-lu[93152], b[5920], x);
      x = fma(-lu[93184], b[5952], x);
      b[2336] = x * vd[2336];
    }
    {
      double x = b[2304];
      x = fma(-lu[93216], b[5184], x);
      x = fma(-lu[93248], b[5824], x);
      x = fma(-lu[93280], b[5952], x);
      x = fma(-lu[93312], b[5984], x);
      x = fma(-lu[93344], b[6016], x);
      b[2304] = x * vd[2304];
    }
    {
      double x = b[2272];
      x = fma(-lu[93376], b[2592], x);
      x = fma(-lu[93408], b[5792], x);
      x = fma(-lu[93440], b[5824], x);
      x = fma(-lu[93472], b[5888], x);
      x = fma(-lu[93504], b[5952], x);
      b[2272] = x * vd[2272];
    }
    {
      double x = b[2240];
      x = fma(-lu[93536], b[3552], x);
      x = fma(-lu[93568], b[5184], x);
      x = fma(-lu[93600], b[5952], x);
      x = fma(-lu[93632], b[6016], x);
      b[2240] = x * vd[2240];
    }
    {
      double x = b[2208];
      x = fma(-lu[93664], b[2784], x);
      x = fma(-lu[93696], b[5184], x);
      x = fma(-lu[93728], b[5824], x);
      x = fma(-lu[93760], b[5952], x);
      x = fma(-lu[93792], b[5984], x);
      x = fma(-lu[93824], b[6016], x);
      b[2208] = x * vd[2208];
    }
    {
      double x = b[2176];
      x = fma(-lu[93856], b[2752], x);
      x = fma(-lu[93888], b[5184], x);
      x = fma(-lu[93920], b[5952], x);
      x = fma(-lu[93952], b[6016], x);
      b[2176] = x * vd[2176];
    }
    {
      double x = b[2144];
      x = fma(-lu[93984], b[3904], x);
      x = fma(-lu[94016], b[5824], x);
      x = fma(-lu[94048], b[5952], x);
      x = fma(-lu[94080], b[5984], x);
      b[2144] = x * vd[2144];
    }
    {
      double x = b[2112];
      x = fma(-lu[94112], b[2528], x);
      x = fma(-lu[94144], b[5824], x);
      x = fma(-lu[94176], b[5952], x);
      x = fma(-lu[94208], b[5984], x);
      b[2112] = x * vd[2112];
    }
    {
      double x = b[2080];
      x = fma(-lu[94240], b[2496], x);
      x = fma(-lu[94272], b[5824], x);
      x = fma(-lu[94304], b[5952], x);
      x = fma(-lu[94336], b[5984], x);
      b[2080] = x * vd[2080];
    }
    {
      double x = b[2048];
      x = fma(-lu[94368], b[2464], x);
      x = fma(-lu[94400], b[5824], x);
      x = fma(-lu[94432], b[5952], x);
      x = fma(-lu[94464], b[5984], x);
      b[2048] = x * vd[2048];
    }
    {
      double x = b[2016];
      x = fma(-lu[94496], b[2432], x);
      x = fma(-lu[94528], b[5824], x);
      x = fma(-lu[94560], b[5952], x);
      x = fma(-lu[94592], b[5984], x);
      b[2016] = x * vd[2016];
    }
    {
      double x = b[1984];
      x = fma(-lu[94624], b[2400], x);
      x = fma(-lu[94656], b[5824], x);
      x = fma(-lu[94688], b[5952], x);
      x = fma(-lu[94720], b[5984], x);
      b[1984] = x * vd[1984];
    }
    {
      double x = b[1952];
      x = fma(-lu[94752], b[2368], x);
      x = fma(-lu[94784], b[5824], x);
      x = fma(-lu[94816], b[5952], x);
      x = fma(-lu[94848], b[5984], x);
      b[1952] = x * vd[1952];
    }
    {
      double x = b[1920];
      x = fma(-lu[94880], b[5184], x);
      x = fma(-lu[94912], b[5824], x);
      x = fma(-lu[94944], b[5952], x);
      x = fma(-lu[94976], b[5984], x);
      x = fma(-lu[95008], b[6016], x);
      b[1920] = x * vd[1920];
    }
    {
      double x = b[1888];
      x = fma(-lu[95040], b[2752], x);
      x = fma(-lu[95072], b[5184], x);
      x = fma(-lu[95104], b[5952], x);
      x = fma(-lu[95136], b[6016], x);
      b[1888] = x * vd[1888];
    }
    {
      double x = b[1856];
      x = fma(-lu[95168], b[3168], x);
      x = fma(-lu[95200], b[5824], x);
      x = fma(-lu[95232], b[5984], x);
      x = fma(-lu[95264], b[6016], x);
      b[1856] = x * vd[1856];
    }
    {
      double x = b[1824];
      x = fma(-lu[95296], b[4672], x);
      x = fma(-lu[95328], b[5920], x);
      x = fma(-lu[95360], b[5952], x);
      x = fma(-lu[95392], b[6016], x);
      b[1824] = x * vd[1824];
    }
    {
      double x = b[1792];
      x = fma(-lu[95424], b[3520], x);
      x = fma(-lu[95456], b[4672], x);
      x = fma(-lu[95488], b[5984], x);
      x = fma(-lu[95520], b[6016], x);
      b[1792] = x * vd[1792];
    }
    {
      double x = b[1760];
      x = fma(-lu[95552], b[2752], x);
      x = fma(-lu[95584], b[2944], x);
      x = fma(-lu[95616], b[5184], x);
      x = fma(-lu[95648], b[5952], x);
      x = fma(-lu[95680], b[6016], x);
      b[1760] = x * vd[1760];
    }
    {
      double x = b[1728];
      x = fma(-lu[95712], b[4576], x);
      x = fma(-lu[95744], b[5824], x);
      x = fma(-lu[95776], b[5984], x);
      x = fma(-lu[95808], b[6016], x);
      b[1728] = x * vd[1728];
    }
    {
      double x = b[1696];
      x = fma(-lu[95840], b[4384], x);
      x = fma(-lu[95872], b[5184], x);
      x = fma(-lu[95904], b[5952], x);
      x = fma(-lu[95936], b[6016], x);
      b[1696] = x * vd[1696];
    }
    {
      double x = b[1664];
      x = fma(-lu[95968], b[4288], x);
      x = fma(-lu[96000], b[5184], x);
      x = fma(-lu[96032], b[5824], x);
      x = fma(-lu[96064], b[5952], x);
      x = fma(-lu[96096], b[5984], x);
      x = fma(-lu[96128], b[6016], x);
      b[1664] = x * vd[1664];
    }
    {
      double x = b[1632];
      x = fma(-lu[96160], b[5184], x);
      x = fma(-lu[96192], b[5824], x);
      x = fma(-lu[96224], b[5952], x);
      x = fma(-lu[96256], b[5984], x);
      x = fma(-lu[96288], b[6016], x);
      b[1632] = x * vd[1632];
    }
    {
      double x = b[1600];
      x = fma(-lu[96320], b[5184], x);
      x = fma(-lu[96352], b[5952], x);
      x = fma(-lu[96384], b[6016], x);
      b[1600] = x * vd[1600];
    }
    {
      double x = b[1568];
      x = fma(-lu[96416], b[5184], x);
      x = fma(-lu[96448], b[5952], x);
      x = fma(-lu[96480], b[6016], x);
      b[1568] = x * vd[1568];
    }
    {
      double x = b[1536];
      x = fma(-lu[96512], b[4800], x);
      x = fma(-lu[96544], b[5920], x);
      x = fma(-lu[96576], b[6016], x);
      b[1536] = x * vd[1536];
    }
    {
      double x = b[1504];
      x = fma(-lu[96608], b[3008], x);
      x = fma(-lu[96640], b[5888], x);
      x = fma(-lu[96672], b[6016], x);
      b[1504] = x * vd[1504];
    }
    {
      double x = b[1472];
      x = fma(-lu[96704], b[5632], x);
      x = fma(-lu[96736], b[5888], x);
      x = fma(-lu[96768], b[6016], x);
      b[1472] = x * vd[1472];
    }
    {
      double x = b[1440];
      x = fma(-lu[96800], b[5184], x);
      x = fma(-lu[96832], b[5952], x);
      x = fma(-lu[96864], b[6016], x);
      b[1440] = x * vd[1440];
    }
    {
      double x = b[1408];
      x = fma(-lu[96896], b[5184], x);
      x = fma(-lu[96928], b[5952], x);
      x = fma(-lu[96960], b[6016], x);
      b[1408] = x * vd[1408];
    }
    {
      double x = b[1376];
      x = fma(-lu[96992], b[2784], x);
      x = fma(-lu[97024], b[4288], x);
      x = fma(-lu[97056], b[5984], x);
      x = fma(-lu[97088], b[6016], x);
      b[1376] = x * vd[1376];
    }
    {
      double x = b[1344];
      x = fma(-lu[97120], b[4288], x);
      x = fma(-lu[97152], b[5984], x);
      x = fma(-lu[97184], b[6016], x);
      b[1344] = x * vd[1344];
    }
    {
      double x = b[1312];
      x = fma(-lu[97216], b[5184], x);
      x = fma(-lu[97248], b[5952], x);
      x = fma(-lu[97280], b[6016], x);
      b[1312] = x * vd[1312];
    }
    {
      double x = b[1280];
      x = fma(-lu[97312], b[5920], x);
      x = fma(-lu[97344], b[5984], x);
      x = fma(-lu[97376], b[6016], x);
      b[1280] = x * vd[1280];
    }
    {
      double x = b[1248];
      x = fma(-lu[97408], b[2752], x);
      x = fma(-lu[97440], b[5184], x);
      x = fma(-lu[97472], b[5952], x);
      x = fma(-lu[97504], b[6016], x);
      b[1248] = x * vd[1248];
    }
    {
      double x = b[1216];
      x = fma(-lu[97536], b[2752], x);
      x = fma(-lu[97568], b[5184], x);
      x = fma(-lu[97600], b[6016], x);
      b[1216] = x * vd[1216];
    }
    {
      double x = b[1184];
      x = fma(-lu[97632], b[5824], x);
      x = fma(-lu[97664], b[5920], x);
      x = fma(-lu[97696], b[6016], x);
      b[1184] = x * vd[1184];
    }
    {
      double x = b[1152];
      x = fma(-lu[97728], b[5184], x);
      x = fma(-lu[97760], b[5952], x);
      x = fma(-lu[97792], b[6016], x);
      b[1152] = x * vd[1152];
    }
    {
      double x = b[1120];
      x = fma(-lu[97824], b[2752], x);
      x = fma(-lu[97856], b[5184], x);
      x = fma(-lu[97888], b[6016], x);
      b[1120] = x * vd[1120];
    }
    {
      double x = b[1088];
      x = fma(-lu[97920], b[5792], x);
      x = fma(-lu[97952], b[5920], x);
      x = fma(-lu[97984], b[6016], x);
      b[1088] = x * vd[1088];
    }
    {
      double x = b[1056];
      x = fma(-lu[98016], b[1376], x);
      b[1056] = x * vd[1056];
    }
    {
      double x = b[1024];
      x = fma(-lu[98048], b[5920], x);
      x = fma(-lu[98080], b[5952], x);
      b[1024] = x * vd[1024];
    }
    {
      double x = b[992];
      x = fma(-lu[98112], b[6016], x);
      b[992] = x * vd[992];
    }
    {
      double x = b[960];
      b[960] = x * vd[960];
    }
    {
      double x = b[928];
      x = fma(-lu[98144], b[6016], x);
      b[928] = x * vd[928];
    }
    {
      double x = b[896];
      x = fma(-lu[98176], b[6016], x);
      b[896] = x * vd[896];
    }
    {
      double x = b[864];
      x = fma(-lu[98208], b[6016], x);
      b[864] = x * vd[864];
    }
    {
      double x = b[832];
      x = fma(-lu[98240], b[6016], x);
      b[832] = x * vd[832];
    }
    {
      double x = b[800];
      x = fma(-lu[98272], b[6016], x);
      b[800] = x * vd[800];
    }
    {
      double x = b[768];
      x = fma(-lu[98304], b[6016], x);
      b[768] = x * vd[768];
    }
    {
      double x = b[736];
      x = fma(-lu[98336], b[6016], x);
      b[736] = x * vd[736];
    }
    {
      double x = b[704];
      x = fma(-lu[98368], b[6016], x);
      b[704] = x * vd[704];
    }
    {
      double x = b[672];
      x = fma(-lu[98400], b[6016], x);
      b[672] = x * vd[672];
    }
    {
      double x = b[640];
      x = fma(-lu[98432], b[6016], x);
      b[640] = x * vd[640];
    }
    {
      double x = b[608];
      x = fma(-lu[98464], b[6016], x);
      b[608] = x * vd[608];
    }
    {
      double x = b[576];
      x = fma(-lu[98496], b[5184], x);
      b[576] = x * vd[576];
    }
    {
      double x = b[544];
      x = fma(-lu[98528], b[1056], x);
      b[544] = x * vd[544];
    }
    {
      double x = b[512];
      x = fma(-lu[98560], b[1056], x);
      b[512] = x * vd[512];
    }
    {
      double x = b[480];
      x = fma(-lu[98592], b[5248], x);
      x = fma(-lu[98624], b[5376], x);
      b[480] = x * vd[480];
    }
    {
      double x = b[448];
      x = fma(-lu[98656], b[6016], x);
      b[448] = x * vd[448];
    }
    {
      double x = b[416];
      x = fma(-lu[98688], b[6016], x);
      b[416] = x * vd[416];
    }
    {
      double x = b[384];
      x = fma(-lu[98720], b[6016], x);
      b[384] = x * vd[384];
    }
    {
      double x = b[352];
      x = fma(-lu[98752], b[6016], x);
      b[352] = x * vd[352];
    }
    {
      double x = b[320];
      x = fma(-lu[98784], b[6016], x);
      b[320] = x * vd[320];
    }
    {
      double x = b[288];
      x = fma(-lu[98816], b[6016], x);
      b[288] = x * vd[288];
    }
    {
      double x = b[256];
      x = fma(-lu[98848], b[6016], x);
      b[256] = x * vd[256];
    }
    {
      double x = b[224];
      x = fma(-lu[98880], b[6016], x);
      b[224] = x * vd[224];
    }
    {
      double x = b[192];
      x = fma(-lu[98912], b[6016], x);
      b[192] = x * vd[192];
    }
    {
      double x = b[160];
      x = fma(-lu[98944], b[6016], x);
      b[160] = x * vd[160];
    }
    {
      double x = b[128];
      b[128] = x * vd[128];
    }
    {
      double x = b[96];
      b[96] = x * vd[96];
    }
    {
      double x = b[64];
      x = fma(-lu[98976], b[2208], x);
      b[64] = x * vd[64];
    }
    {
      double x = b[32];
      x = fma(-lu[99008], b[1664], x);
      b[32] = x * vd[32];
    }
    {
      double x = b[0];
      x = fma(-lu[99040], b[1056], x);
      b[0] = x * vd[0];
    }
}
}  // namespace mech_cracmm2
