// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void solve_1_0(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
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
      CHEM_PREFETCH(ws + 111520);
      double x = b[128];
      b[128] = x;
    }
    {
      CHEM_PREFETCH(ws + 111552);
      double x = b[160];
      b[160] = x;
    }
    {
      double x = b[192];
      x = fma(-CHEM_LDLU(lu + 32), b[160], x);
      b[192] = x;
    }
    {
      double x = b[224];
      x = fma(-CHEM_LDLU(lu + 64), b[160], x);
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
      CHEM_PREFETCH(ws + 111584);
      double x = b[480];
      b[480] = x;
    }
    {
      double x = b[512];
      b[512] = x;
    }
    {
      double x = b[544];
      x = fma(-CHEM_LDLU(lu + 96), b[512], x);
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
      CHEM_PREFETCH(ws + 111616);
      CHEM_PREFETCH(ws + 111648);
      double x = b[896];
      b[896] = x;
    }
    {
      double x = b[928];
      b[928] = x;
    }
    {
      double x = b[960];
      x = fma(-CHEM_LDLU(lu + 128), b[96], x);
      x = fma(-CHEM_LDLU(lu + 160), b[128], x);
      b[960] = x;
    }
    {
      CHEM_PREFETCH(ws + 111680);
      double x = b[992];
      b[992] = x;
    }
    {
      double x = b[1024];
      b[1024] = x;
    }
    {
      double x = b[1056];
      x = fma(-CHEM_LDLU(lu + 192), b[512], x);
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
      CHEM_PREFETCH(ws + 111712);
      double x = b[1184];
      b[1184] = x;
    }
    {
      double x = b[1216];
      b[1216] = x;
    }
    {
      double x = b[1248];
      x = fma(-CHEM_LDLU(lu + 224), b[1216], x);
      b[1248] = x;
    }
    {
      double x = b[1280];
      b[1280] = x;
    }
    {
      CHEM_PREFETCH(ws + 111744);
      double x = b[1312];
      b[1312] = x;
    }
    {
      double x = b[1344];
      b[1344] = x;
    }
    {
      double x = b[1376];
      x = fma(-CHEM_LDLU(lu + 256), b[1344], x);
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
      CHEM_PREFETCH(ws + 111776);
      double x = b[1568];
      b[1568] = x;
    }
    {
      CHEM_PREFETCH(ws + 111808);
      CHEM_PREFETCH(ws + 111840);
      double x = b[1600];
      b[1600] = x;
    }
    {
      double x = b[1632];
      x = fma(-CHEM_LDLU(lu + 288), b[1312], x);
      b[1632] = x;
    }
    {
      double x = b[1664];
      x = fma(-CHEM_LDLU(lu + 320), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 352), b[1632], x);
      b[1664] = x;
    }
    {
      CHEM_PREFETCH(ws + 111872);
      double x = b[1696];
      b[1696] = x;
    }
    {
      double x = b[1728];
      b[1728] = x;
    }
    {
      double x = b[1760];
      x = fma(-CHEM_LDLU(lu + 384), b[1248], x);
      b[1760] = x;
    }
    {
      double x = b[1792];
      b[1792] = x;
    }
    {
      CHEM_PREFETCH(ws + 111904);
      double x = b[1824];
      b[1824] = x;
    }
    {
      CHEM_PREFETCH(ws + 111936);
      double x = b[1856];
      b[1856] = x;
    }
    {
      double x = b[1888];
      x = fma(-CHEM_LDLU(lu + 416), b[1152], x);
      b[1888] = x;
    }
    {
      double x = b[1920];
      x = fma(-CHEM_LDLU(lu + 448), b[1600], x);
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
      CHEM_PREFETCH(ws + 111968);
      CHEM_PREFETCH(ws + 112000);
      double x = b[2112];
      b[2112] = x;
    }
    {
      CHEM_PREFETCH(ws + 112032);
      double x = b[2144];
      b[2144] = x;
    }
    {
      CHEM_PREFETCH(ws + 112064);
      double x = b[2176];
      x = fma(-CHEM_LDLU(lu + 480), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 512), b[1408], x);
      b[2176] = x;
    }
    {
      double x = b[2208];
      x = fma(-CHEM_LDLU(lu + 544), b[1632], x);
      b[2208] = x;
    }
    {
      CHEM_PREFETCH(ws + 112096);
      double x = b[2240];
      x = fma(-CHEM_LDLU(lu + 576), b[1568], x);
      b[2240] = x;
    }
    {
      CHEM_PREFETCH(ws + 112128);
      double x = b[2272];
      b[2272] = x;
    }
    {
      CHEM_PREFETCH(ws + 112160);
      double x = b[2304];
      x = fma(-CHEM_LDLU(lu + 608), b[1600], x);
      b[2304] = x;
    }
    {
      CHEM_PREFETCH(ws + 112192);
      double x = b[2336];
      x = fma(-CHEM_LDLU(lu + 640), b[576], x);
      b[2336] = x;
    }
    {
      CHEM_PREFETCH(ws + 112224);
      double x = b[2368];
      x = fma(-CHEM_LDLU(lu + 672), b[608], x);
      b[2368] = x;
    }
    {
      CHEM_PREFETCH(ws + 112256);
      double x = b[2400];
      x = fma(-CHEM_LDLU(lu + 704), b[640], x);
      b[2400] = x;
    }
    {
      CHEM_PREFETCH(ws + 112288);
      double x = b[2432];
      x = fma(-CHEM_LDLU(lu + 736), b[672], x);
      b[2432] = x;
    }
    {
      CHEM_PREFETCH(ws + 112320);
      double x = b[2464];
      x = fma(-CHEM_LDLU(lu + 768), b[704], x);
      b[2464] = x;
    }
    {
      CHEM_PREFETCH(ws + 112352);
      double x = b[2496];
      x = fma(-CHEM_LDLU(lu + 800), b[736], x);
      b[2496] = x;
    }
    {
      double x = b[2528];
      x = fma(-CHEM_LDLU(lu + 832), b[768], x);
      b[2528] = x;
    }
    {
      CHEM_PREFETCH(ws + 112384);
      double x = b[2560];
      x = fma(-CHEM_LDLU(lu + 864), b[1408], x);
      b[2560] = x;
    }
    {
      CHEM_PREFETCH(ws + 112416);
      double x = b[2592];
      b[2592] = x;
    }
    {
      CHEM_PREFETCH(ws + 112448);
      CHEM_PREFETCH(ws + 112480);
      double x = b[2624];
      x = fma(-CHEM_LDLU(lu + 896), b[1408], x);
      b[2624] = x;
    }
    {
      double x = b[2656];
      x = fma(-CHEM_LDLU(lu + 928), b[1440], x);
      b[2656] = x;
    }
    {
      CHEM_PREFETCH(ws + 112512);
      double x = b[2688];
      x = fma(-CHEM_LDLU(lu + 960), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 992), b[2592], x);
      b[2688] = x;
    }
    {
      CHEM_PREFETCH(ws + 112544);
      CHEM_PREFETCH(ws + 112576);
      double x = b[2720];
      b[2720] = x;
    }
    {
      CHEM_PREFETCH(ws + 112608);
      double x = b[2752];
      x = fma(-CHEM_LDLU(lu + 1024), b[1312], x);
      b[2752] = x;
    }
    {
      double x = b[2784];
      x = fma(-CHEM_LDLU(lu + 1056), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 1088), b[1632], x);
      b[2784] = x;
    }
    {
      double x = b[2816];
      x = fma(-CHEM_LDLU(lu + 1120), b[1408], x);
      b[2816] = x;
    }
    {
      double x = b[2848];
      b[2848] = x;
    }
    {
      CHEM_PREFETCH(ws + 112640);
      CHEM_PREFETCH(ws + 112672);
      CHEM_PREFETCH(ws + 112704);
      double x = b[2880];
      b[2880] = x;
    }
    {
      double x = b[2912];
      b[2912] = x;
    }
    {
      CHEM_PREFETCH(ws + 112736);
      double x = b[2944];
      x = fma(-CHEM_LDLU(lu + 1152), b[288], x);
      x = fma(-CHEM_LDLU(lu + 1184), b[320], x);
      x = fma(-CHEM_LDLU(lu + 1216), b[352], x);
      b[2944] = x;
    }
    {
      double x = b[2976];
      b[2976] = x;
    }
    {
      CHEM_PREFETCH(ws + 112768);
      CHEM_PREFETCH(ws + 112800);
      CHEM_PREFETCH(ws + 112832);
      double x = b[3008];
      x = fma(-CHEM_LDLU(lu + 1248), b[2240], x);
      b[3008] = x;
    }
    {
      CHEM_PREFETCH(ws + 112864);
      double x = b[3040];
      b[3040] = x;
    }
    {
      CHEM_PREFETCH(ws + 112896);
      double x = b[3072];
      x = fma(-CHEM_LDLU(lu + 1280), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 1312), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1344), b[2944], x);
      b[3072] = x;
    }
    {
      CHEM_PREFETCH(ws + 112928);
      double x = b[3104];
      x = fma(-CHEM_LDLU(lu + 1376), b[320], x);
      b[3104] = x;
    }
    {
      CHEM_PREFETCH(ws + 112960);
      CHEM_PREFETCH(ws + 112992);
      double x = b[3136];
      x = fma(-CHEM_LDLU(lu + 1408), b[1568], x);
      b[3136] = x;
    }
    {
      CHEM_PREFETCH(ws + 113024);
      CHEM_PREFETCH(ws + 113056);
      CHEM_PREFETCH(ws + 113088);
      CHEM_PREFETCH(ws + 113120);
      double x = b[3168];
      x = fma(-CHEM_LDLU(lu + 1440), b[3136], x);
      b[3168] = x;
    }
    {
      CHEM_PREFETCH(ws + 113152);
      double x = b[3200];
      x = fma(-CHEM_LDLU(lu + 1472), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1504), b[3136], x);
      b[3200] = x;
    }
    {
      CHEM_PREFETCH(ws + 113184);
      double x = b[3232];
      x = fma(-CHEM_LDLU(lu + 1536), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 1568), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1600), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 1632), b[3136], x);
      b[3232] = x;
    }
    {
      CHEM_PREFETCH(ws + 113216);
      double x = b[3264];
      x = fma(-CHEM_LDLU(lu + 1664), b[352], x);
      b[3264] = x;
    }
    {
      CHEM_PREFETCH(ws + 113248);
      CHEM_PREFETCH(ws + 113280);
      CHEM_PREFETCH(ws + 113312);
      double x = b[3296];
      x = fma(-CHEM_LDLU(lu + 1696), b[288], x);
      b[3296] = x;
    }
    {
      CHEM_PREFETCH(ws + 113344);
      double x = b[3328];
      x = fma(-CHEM_LDLU(lu + 1728), b[1152], x);
      b[3328] = x;
    }
    {
      CHEM_PREFETCH(ws + 113376);
      double x = b[3360];
      x = fma(-CHEM_LDLU(lu + 1760), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 1792), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1824), b[3136], x);
      b[3360] = x;
    }
    {
      CHEM_PREFETCH(ws + 113408);
      double x = b[3392];
      x = fma(-CHEM_LDLU(lu + 1856), b[832], x);
      b[3392] = x;
    }
    {
      CHEM_PREFETCH(ws + 113440);
      double x = b[3424];
      x = fma(-CHEM_LDLU(lu + 1888), b[864], x);
      b[3424] = x;
    }
    {
      double x = b[3456];
      x = fma(-CHEM_LDLU(lu + 1920), b[896], x);
      b[3456] = x;
    }
    {
      CHEM_PREFETCH(ws + 113472);
      CHEM_PREFETCH(ws + 113504);
      double x = b[3488];
      x = fma(-CHEM_LDLU(lu + 1952), b[992], x);
      b[3488] = x;
    }
    {
      CHEM_PREFETCH(ws + 113536);
      CHEM_PREFETCH(ws + 113568);
      double x = b[3520];
      b[3520] = x;
    }
    {
      CHEM_PREFETCH(ws + 113600);
      CHEM_PREFETCH(ws + 113632);
      CHEM_PREFETCH(ws + 113664);
      CHEM_PREFETCH(ws + 113696);
      CHEM_PREFETCH(ws + 113728);
      CHEM_PREFETCH(ws + 113760);
      CHEM_PREFETCH(ws + 113792);
      CHEM_PREFETCH(ws + 113824);
      CHEM_PREFETCH(ws + 113856);
      double x = b[3552];
      x = fma(-CHEM_LDLU(lu + 1984), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 2016), b[3136], x);
      b[3552] = x;
    }
    {
      CHEM_PREFETCH(ws + 113888);
      CHEM_PREFETCH(ws + 113920);
      CHEM_PREFETCH(ws + 113952);
      CHEM_PREFETCH(ws + 113984);
      CHEM_PREFETCH(ws + 114016);
      double x = b[3584];
      x = fma(-CHEM_LDLU(lu + 2048), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 2080), b[3360], x);
      b[3584] = x;
    }
    {
      CHEM_PREFETCH(ws + 114048);
      CHEM_PREFETCH(ws + 114080);
      double x = b[3616];
      x = fma(-CHEM_LDLU(lu + 2112), b[384], x);
      x = fma(-CHEM_LDLU(lu + 2144), b[416], x);
      x = fma(-CHEM_LDLU(lu + 2176), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 2208), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 2240), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 2272), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 2304), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 2336), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 2368), b[3232], x);
      b[3616] = x;
    }
    {
      CHEM_PREFETCH(ws + 114112);
      double x = b[3648];
      x = fma(-CHEM_LDLU(lu + 2400), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 2432), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 2464), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 2496), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 2528), b[3232], x);
      b[3648] = x;
    }
    {
      CHEM_PREFETCH(ws + 114144);
      double x = b[3680];
      x = fma(-CHEM_LDLU(lu + 2560), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 2592), b[3584], x);
      b[3680] = x;
    }
    {
      double x = b[3712];
      x = fma(-CHEM_LDLU(lu + 2624), b[1440], x);
      b[3712] = x;
    }
    {
      CHEM_PREFETCH(ws + 114176);
      CHEM_PREFETCH(ws + 114208);
      CHEM_PREFETCH(ws + 114240);
      CHEM_PREFETCH(ws + 114272);
      CHEM_PREFETCH(ws + 114304);
      CHEM_PREFETCH(ws + 114336);
      double x = b[3744];
      x = fma(-CHEM_LDLU(lu + 2656), b[1408], x);
      b[3744] = x;
    }
    {
      CHEM_PREFETCH(ws + 114368);
      double x = b[3776];
      b[3776] = x;
    }
    {
      CHEM_PREFETCH(ws + 114400);
      CHEM_PREFETCH(ws + 114432);
      double x = b[3808];
      x = fma(-CHEM_LDLU(lu + 2688), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 2720), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 2752), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 2784), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 2816), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 2848), b[3232], x);
      b[3808] = x;
    }
    {
      CHEM_PREFETCH(ws + 114464);
      double x = b[3840];
      x = fma(-CHEM_LDLU(lu + 2880), b[1408], x);
      b[3840] = x;
    }
    {
      CHEM_PREFETCH(ws + 114496);
      double x = b[3872];
      x = fma(-CHEM_LDLU(lu + 2912), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 2944), b[3136], x);
      b[3872] = x;
    }
    {
      double x = b[3904];
      x = fma(-CHEM_LDLU(lu + 2976), b[800], x);
      b[3904] = x;
    }
    {
      CHEM_PREFETCH(ws + 114528);
      CHEM_PREFETCH(ws + 114560);
      CHEM_PREFETCH(ws + 114592);
      CHEM_PREFETCH(ws + 114624);
      CHEM_PREFETCH(ws + 114656);
      CHEM_PREFETCH(ws + 114688);
      double x = b[3936];
      x = fma(-CHEM_LDLU(lu + 3008), b[1440], x);
      b[3936] = x;
    }
    {
      CHEM_PREFETCH(ws + 114720);
      CHEM_PREFETCH(ws + 114752);
      CHEM_PREFETCH(ws + 114784);
      CHEM_PREFETCH(ws + 114816);
      CHEM_PREFETCH(ws + 114848);
      double x = b[3968];
      b[3968] = x;
    }
    {
      CHEM_PREFETCH(ws + 114880);
      CHEM_PREFETCH(ws + 114912);
      CHEM_PREFETCH(ws + 114944);
      CHEM_PREFETCH(ws + 114976);
      CHEM_PREFETCH(ws + 115008);
      CHEM_PREFETCH(ws + 115040);
      double x = b[4000];
      x = fma(-CHEM_LDLU(lu + 3040), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 3072), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 3104), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 3136), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 3168), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 3200), b[3136], x);
      b[4000] = x;
    }
    {
      CHEM_PREFETCH(ws + 115072);
      CHEM_PREFETCH(ws + 115104);
      double x = b[4032];
      x = fma(-CHEM_LDLU(lu + 3232), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 3264), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 3296), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 3328), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 3360), b[3136], x);
      b[4032] = x;
    }
    {
      CHEM_PREFETCH(ws + 115136);
      CHEM_PREFETCH(ws + 115168);
      CHEM_PREFETCH(ws + 115200);
      double x = b[4064];
      x = fma(-CHEM_LDLU(lu + 3392), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 3424), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 3456), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 3488), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 3520), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 3552), b[4032], x);
      b[4064] = x;
    }
    {
      CHEM_PREFETCH(ws + 115232);
      CHEM_PREFETCH(ws + 115264);
      CHEM_PREFETCH(ws + 115296);
      CHEM_PREFETCH(ws + 115328);
      CHEM_PREFETCH(ws + 115360);
      double x = b[4096];
      x = fma(-CHEM_LDLU(lu + 3584), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 3616), b[2560], x);
      b[4096] = x;
    }
    {
      CHEM_PREFETCH(ws + 115392);
      CHEM_PREFETCH(ws + 115424);
      CHEM_PREFETCH(ws + 115456);
      CHEM_PREFETCH(ws + 115488);
      CHEM_PREFETCH(ws + 115520);
      CHEM_PREFETCH(ws + 115552);
      double x = b[4128];
      x = fma(-CHEM_LDLU(lu + 3648), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 3680), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 3712), b[1664], x);
      b[4128] = x;
    }
    {
      CHEM_PREFETCH(ws + 115584);
      double x = b[4160];
      x = fma(-CHEM_LDLU(lu + 3744), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 3776), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 3808), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 3840), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 3872), b[3936], x);
      b[4160] = x;
    }
    {
      CHEM_PREFETCH(ws + 115616);
      CHEM_PREFETCH(ws + 115648);
      CHEM_PREFETCH(ws + 115680);
      CHEM_PREFETCH(ws + 115712);
      CHEM_PREFETCH(ws + 115744);
      CHEM_PREFETCH(ws + 115776);
      CHEM_PREFETCH(ws + 115808);
      CHEM_PREFETCH(ws + 115840);
      double x = b[4192];
      x = fma(-CHEM_LDLU(lu + 3904), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 3936), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 3968), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 4000), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 4032), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 4064), b[4160], x);
      b[4192] = x;
    }
    {
      CHEM_PREFETCH(ws + 115872);
      CHEM_PREFETCH(ws + 115904);
      CHEM_PREFETCH(ws + 115936);
      CHEM_PREFETCH(ws + 115968);
      CHEM_PREFETCH(ws + 116000);
      CHEM_PREFETCH(ws + 116032);
      CHEM_PREFETCH(ws + 116064);
      CHEM_PREFETCH(ws + 116096);
      double x = b[4224];
      x = fma(-CHEM_LDLU(lu + 4096), b[3968], x);
      b[4224] = x;
    }
    {
      CHEM_PREFETCH(ws + 116128);
      CHEM_PREFETCH(ws + 116160);
      CHEM_PREFETCH(ws + 116192);
      CHEM_PREFETCH(ws + 116224);
      CHEM_PREFETCH(ws + 116256);
      CHEM_PREFETCH(ws + 116288);
      double x = b[4256];
      x = fma(-CHEM_LDLU(lu + 4128), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 4160), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 4192), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 4224), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 4256), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 4288), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 4320), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 4352), b[4192], x);
      b[4256] = x;
    }
    {
      CHEM_PREFETCH(ws + 116320);
      CHEM_PREFETCH(ws + 116352);
      CHEM_PREFETCH(ws + 116384);
      CHEM_PREFETCH(ws + 116416);
      CHEM_PREFETCH(ws + 116448);
      CHEM_PREFETCH(ws + 116480);
      CHEM_PREFETCH(ws + 116512);
      CHEM_PREFETCH(ws + 116544);
      CHEM_PREFETCH(ws + 116576);
      CHEM_PREFETCH(ws + 116608);
      double x = b[4288];
      x = fma(-CHEM_LDLU(lu + 4384), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 4416), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 4448), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 4480), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 4512), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 4544), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 4576), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 4608), b[4192], x);
      b[4288] = x;
    }
    {
      CHEM_PREFETCH(ws + 116640);
      CHEM_PREFETCH(ws + 116672);
      CHEM_PREFETCH(ws + 116704);
      CHEM_PREFETCH(ws + 116736);
      CHEM_PREFETCH(ws + 116768);
      CHEM_PREFETCH(ws + 116800);
      CHEM_PREFETCH(ws + 116832);
      double x = b[4320];
      x = fma(-CHEM_LDLU(lu + 4640), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 4672), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 4704), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 4736), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 4768), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 4800), b[3456], x);
      b[4320] = x;
    }
    {
      CHEM_PREFETCH(ws + 116864);
      CHEM_PREFETCH(ws + 116896);
      CHEM_PREFETCH(ws + 116928);
      CHEM_PREFETCH(ws + 116960);
      CHEM_PREFETCH(ws + 116992);
      CHEM_PREFETCH(ws + 117024);
      CHEM_PREFETCH(ws + 117056);
      double x = b[4352];
      x = fma(-CHEM_LDLU(lu + 4832), b[256], x);
      x = fma(-CHEM_LDLU(lu + 4864), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 4896), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 4928), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 4960), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 4992), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 5024), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 5056), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 5088), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 5120), b[4288], x);
      b[4352] = x;
    }
    {
      CHEM_PREFETCH(ws + 117088);
      CHEM_PREFETCH(ws + 117120);
      CHEM_PREFETCH(ws + 117152);
      CHEM_PREFETCH(ws + 117184);
      CHEM_PREFETCH(ws + 117216);
      CHEM_PREFETCH(ws + 117248);
      CHEM_PREFETCH(ws + 117280);
      CHEM_PREFETCH(ws + 117312);
      double x = b[4384];
      x = fma(-CHEM_LDLU(lu + 5152), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 5184), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 5216), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 5248), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 5280), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 5312), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 5344), b[4288], x);
      b[4384] = x;
    }
    {
      CHEM_PREFETCH(ws + 117344);
      CHEM_PREFETCH(ws + 117376);
      CHEM_PREFETCH(ws + 117408);
      CHEM_PREFETCH(ws + 117440);
      CHEM_PREFETCH(ws + 117472);
      CHEM_PREFETCH(ws + 117504);
      CHEM_PREFETCH(ws + 117536);
      CHEM_PREFETCH(ws + 117568);
      double x = b[4416];
      x = fma(-CHEM_LDLU(lu + 5376), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 5408), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 5440), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 5472), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 5504), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 5536), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 5568), b[2528], x);
      b[4416] = x;
    }
    {
      CHEM_PREFETCH(ws + 117600);
      CHEM_PREFETCH(ws + 117632);
      CHEM_PREFETCH(ws + 117664);
      CHEM_PREFETCH(ws + 117696);
      CHEM_PREFETCH(ws + 117728);
      CHEM_PREFETCH(ws + 117760);
      CHEM_PREFETCH(ws + 117792);
      CHEM_PREFETCH(ws + 117824);
      CHEM_PREFETCH(ws + 117856);
      double x = b[4448];
      x = fma(-CHEM_LDLU(lu + 5600), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 5632), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 5664), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 5696), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 5728), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 5760), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 5792), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 5824), b[3488], x);
      b[4448] = x;
    }
    {
      CHEM_PREFETCH(ws + 117888);
      CHEM_PREFETCH(ws + 117920);
      CHEM_PREFETCH(ws + 117952);
      CHEM_PREFETCH(ws + 117984);
      CHEM_PREFETCH(ws + 118016);
      CHEM_PREFETCH(ws + 118048);
      CHEM_PREFETCH(ws + 118080);
      CHEM_PREFETCH(ws + 118112);
      CHEM_PREFETCH(ws + 118144);
      CHEM_PREFETCH(ws + 118176);
      double x = b[4480];
      x = fma(-CHEM_LDLU(lu + 5856), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 5888), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 5920), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 5952), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 5984), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 6016), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 6048), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 6080), b[4288], x);
      b[4480] = x;
    }
    {
      CHEM_PREFETCH(ws + 118208);
      CHEM_PREFETCH(ws + 118240);
      CHEM_PREFETCH(ws + 118272);
      CHEM_PREFETCH(ws + 118304);
      CHEM_PREFETCH(ws + 118336);
      CHEM_PREFETCH(ws + 118368);
      CHEM_PREFETCH(ws + 118400);
      CHEM_PREFETCH(ws + 118432);
      CHEM_PREFETCH(ws + 118464);
      double x = b[4512];
      x = fma(-CHEM_LDLU(lu + 6112), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 6144), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 6176), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 6208), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 6240), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 6272), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 6304), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 6336), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 6368), b[3456], x);
      b[4512] = x;
    }
    {
      CHEM_PREFETCH(ws + 118496);
      CHEM_PREFETCH(ws + 118528);
      CHEM_PREFETCH(ws + 118560);
      CHEM_PREFETCH(ws + 118592);
      CHEM_PREFETCH(ws + 118624);
      double x = b[4544];
      x = fma(-CHEM_LDLU(lu + 6400), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 6432), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 6464), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 6496), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 6528), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 6560), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 6592), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 6624), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 6656), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 6688), b[4384], x);
      b[4544] = x;
    }
    {
      CHEM_PREFETCH(ws + 118656);
      CHEM_PREFETCH(ws + 118688);
      CHEM_PREFETCH(ws + 118720);
      CHEM_PREFETCH(ws + 118752);
      double x = b[4576];
      x = fma(-CHEM_LDLU(lu + 6720), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 6752), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 6784), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 6816), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 6848), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 6880), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 6912), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 6944), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 6976), b[4288], x);
      b[4576] = x;
    }
    {
      CHEM_PREFETCH(ws + 118784);
      CHEM_PREFETCH(ws + 118816);
      CHEM_PREFETCH(ws + 118848);
      CHEM_PREFETCH(ws + 118880);
      CHEM_PREFETCH(ws + 118912);
      CHEM_PREFETCH(ws + 118944);
      CHEM_PREFETCH(ws + 118976);
      CHEM_PREFETCH(ws + 119008);
      double x = b[4608];
      x = fma(-CHEM_LDLU(lu + 7008), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 7040), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 7072), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 7104), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 7136), b[4416], x);
      b[4608] = x;
    }
    {
      CHEM_PREFETCH(ws + 119040);
      CHEM_PREFETCH(ws + 119072);
      CHEM_PREFETCH(ws + 119104);
      CHEM_PREFETCH(ws + 119136);
      CHEM_PREFETCH(ws + 119168);
      CHEM_PREFETCH(ws + 119200);
      CHEM_PREFETCH(ws + 119232);
      double x = b[4640];
      x = fma(-CHEM_LDLU(lu + 7168), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 7200), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 7232), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 7264), b[4416], x);
      b[4640] = x;
    }
    {
      CHEM_PREFETCH(ws + 119264);
      CHEM_PREFETCH(ws + 119296);
      CHEM_PREFETCH(ws + 119328);
      CHEM_PREFETCH(ws + 119360);
      CHEM_PREFETCH(ws + 119392);
      CHEM_PREFETCH(ws + 119424);
      CHEM_PREFETCH(ws + 119456);
      CHEM_PREFETCH(ws + 119488);
      CHEM_PREFETCH(ws + 119520);
      CHEM_PREFETCH(ws + 119552);
      CHEM_PREFETCH(ws + 119584);
      CHEM_PREFETCH(ws + 119616);
      double x = b[4672];
      x = fma(-CHEM_LDLU(lu + 7296), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 7328), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 7360), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 7392), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 7424), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 7456), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 7488), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 7520), b[4288], x);
      b[4672] = x;
    }
    {
      CHEM_PREFETCH(ws + 119648);
      CHEM_PREFETCH(ws + 119680);
      CHEM_PREFETCH(ws + 119712);
      CHEM_PREFETCH(ws + 119744);
      CHEM_PREFETCH(ws + 119776);
      double x = b[4704];
      x = fma(-CHEM_LDLU(lu + 7552), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 7584), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 7616), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 7648), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 7680), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 7712), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 7744), b[4640], x);
      b[4704] = x;
    }
    {
      CHEM_PREFETCH(ws + 119808);
      CHEM_PREFETCH(ws + 119840);
      CHEM_PREFETCH(ws + 119872);
      CHEM_PREFETCH(ws + 119904);
      CHEM_PREFETCH(ws + 119936);
      CHEM_PREFETCH(ws + 119968);
      double x = b[4736];
      x = fma(-CHEM_LDLU(lu + 7776), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 7808), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 7840), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 7872), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 7904), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 7936), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 7968), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 8000), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 8032), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 8064), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 8096), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 8128), b[4288], x);
      b[4736] = x;
    }
    {
      CHEM_PREFETCH(ws + 120000);
      CHEM_PREFETCH(ws + 120032);
      CHEM_PREFETCH(ws + 120064);
      CHEM_PREFETCH(ws + 120096);
      CHEM_PREFETCH(ws + 120128);
      CHEM_PREFETCH(ws + 120160);
      CHEM_PREFETCH(ws + 120192);
      CHEM_PREFETCH(ws + 120224);
      CHEM_PREFETCH(ws + 120256);
      CHEM_PREFETCH(ws + 120288);
      CHEM_PREFETCH(ws + 120320);
      double x = b[4768];
      x = fma(-CHEM_LDLU(lu + 8160), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 8192), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8224), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 8256), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 8288), b[4704], x);
      b[4768] = x;
    }
    {
      CHEM_PREFETCH(ws + 120352);
      CHEM_PREFETCH(ws + 120384);
      CHEM_PREFETCH(ws + 120416);
      CHEM_PREFETCH(ws + 120448);
      CHEM_PREFETCH(ws + 120480);
      CHEM_PREFETCH(ws + 120512);
      CHEM_PREFETCH(ws + 120544);
      CHEM_PREFETCH(ws + 120576);
      double x = b[4800];
      x = fma(-CHEM_LDLU(lu + 8320), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 8352), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 8384), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 8416), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 8448), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 8480), b[4576], x);
      b[4800] = x;
    }
    {
      CHEM_PREFETCH(ws + 120608);
      CHEM_PREFETCH(ws + 120640);
      CHEM_PREFETCH(ws + 120672);
      CHEM_PREFETCH(ws + 120704);
      CHEM_PREFETCH(ws + 120736);
      CHEM_PREFETCH(ws + 120768);
      CHEM_PREFETCH(ws + 120800);
      CHEM_PREFETCH(ws + 120832);
      CHEM_PREFETCH(ws + 120864);
      CHEM_PREFETCH(ws + 120896);
      double x = b[4832];
      x = fma(-CHEM_LDLU(lu + 8512), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 8544), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 8576), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 8608), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 8640), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 8672), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 8704), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 8736), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 8768), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8800), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 8832), b[4704], x);
      b[4832] = x;
    }
    {
      CHEM_PREFETCH(ws + 120928);
      CHEM_PREFETCH(ws + 120960);
      CHEM_PREFETCH(ws + 120992);
      CHEM_PREFETCH(ws + 121024);
      CHEM_PREFETCH(ws + 121056);
      CHEM_PREFETCH(ws + 121088);
      CHEM_PREFETCH(ws + 121120);
      CHEM_PREFETCH(ws + 121152);
      CHEM_PREFETCH(ws + 121184);
      CHEM_PREFETCH(ws + 121216);
      CHEM_PREFETCH(ws + 121248);
      CHEM_PREFETCH(ws + 121280);
      double x = b[4864];
      x = fma(-CHEM_LDLU(lu + 8864), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 8896), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 8928), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 8960), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8992), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 9024), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 9056), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 9088), b[4832], x);
      b[4864] = x;
    }
    {
      CHEM_PREFETCH(ws + 121312);
      CHEM_PREFETCH(ws + 121344);
      CHEM_PREFETCH(ws + 121376);
      CHEM_PREFETCH(ws + 121408);
      CHEM_PREFETCH(ws + 121440);
      CHEM_PREFETCH(ws + 121472);
      CHEM_PREFETCH(ws + 121504);
      CHEM_PREFETCH(ws + 121536);
      CHEM_PREFETCH(ws + 121568);
      CHEM_PREFETCH(ws + 121600);
      CHEM_PREFETCH(ws + 121632);
      CHEM_PREFETCH(ws + 121664);
      CHEM_PREFETCH(ws + 121696);
      CHEM_PREFETCH(ws + 121728);
      CHEM_PREFETCH(ws + 121760);
      CHEM_PREFETCH(ws + 121792);
      CHEM_PREFETCH(ws + 121824);
      double x = b[4896];
      x = fma(-CHEM_LDLU(lu + 9120), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 9152), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 9184), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 9216), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 9248), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 9280), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 9312), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 9344), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 9376), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 9408), b[4864], x);
      b[4896] = x;
    }
    {
      CHEM_PREFETCH(ws + 121856);
      CHEM_PREFETCH(ws + 121888);
      CHEM_PREFETCH(ws + 121920);
      CHEM_PREFETCH(ws + 121952);
      CHEM_PREFETCH(ws + 121984);
      CHEM_PREFETCH(ws + 122016);
      CHEM_PREFETCH(ws + 122048);
      CHEM_PREFETCH(ws + 122080);
      CHEM_PREFETCH(ws + 122112);
      CHEM_PREFETCH(ws + 122144);
      CHEM_PREFETCH(ws + 122176);
      CHEM_PREFETCH(ws + 122208);
      CHEM_PREFETCH(ws + 122240);
      CHEM_PREFETCH(ws + 122272);
      CHEM_PREFETCH(ws + 122304);
      CHEM_PREFETCH(ws + 122336);
      CHEM_PREFETCH(ws + 122368);
      CHEM_PREFETCH(ws + 122400);
      double x = b[4928];
      x = fma(-CHEM_LDLU(lu + 9440), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 9472), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 9504), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 9536), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 9568), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 9600), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 9632), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 9664), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 9696), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 9728), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 9760), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9792), b[4896], x);
      b[4928] = x;
    }
    {
      CHEM_PREFETCH(ws + 122432);
      CHEM_PREFETCH(ws + 122464);
      CHEM_PREFETCH(ws + 122496);
      CHEM_PREFETCH(ws + 122528);
      CHEM_PREFETCH(ws + 122560);
      CHEM_PREFETCH(ws + 122592);
      CHEM_PREFETCH(ws + 122624);
      CHEM_PREFETCH(ws + 122656);
      CHEM_PREFETCH(ws + 122688);
      CHEM_PREFETCH(ws + 122720);
      CHEM_PREFETCH(ws + 122752);
      CHEM_PREFETCH(ws + 122784);
      CHEM_PREFETCH(ws + 122816);
      CHEM_PREFETCH(ws + 122848);
      double x = b[4960];
      x = fma(-CHEM_LDLU(lu + 9824), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 9856), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 9888), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 9920), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 9952), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 9984), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 10016), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 10048), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 10080), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 10112), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 10144), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 10176), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 10208), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 10240), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 10272), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 10304), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 10336), b[4928], x);
      b[4960] = x;
    }
    {
      CHEM_PREFETCH(ws + 122880);
      CHEM_PREFETCH(ws + 122912);
      CHEM_PREFETCH(ws + 122944);
      CHEM_PREFETCH(ws + 122976);
      CHEM_PREFETCH(ws + 123008);
      CHEM_PREFETCH(ws + 123040);
      CHEM_PREFETCH(ws + 123072);
      CHEM_PREFETCH(ws + 123104);
      CHEM_PREFETCH(ws + 123136);
      CHEM_PREFETCH(ws + 123168);
      CHEM_PREFETCH(ws + 123200);
      CHEM_PREFETCH(ws + 123232);
      CHEM_PREFETCH(ws + 123264);
      CHEM_PREFETCH(ws + 123296);
      CHEM_PREFETCH(ws + 123328);
      CHEM_PREFETCH(ws + 123360);
      CHEM_PREFETCH(ws + 123392);
      CHEM_PREFETCH(ws + 123424);
      CHEM_PREFETCH(ws + 123456);
      CHEM_PREFETCH(ws + 123488);
      CHEM_PREFETCH(ws + 123520);
      CHEM_PREFETCH(ws + 123552);
      CHEM_PREFETCH(ws + 123584);
      CHEM_PREFETCH(ws + 123616);
      CHEM_PREFETCH(ws + 123648);
      CHEM_PREFETCH(ws + 123680);
      CHEM_PREFETCH(ws + 123712);
      double x = b[4992];
      x = fma(-CHEM_LDLU(lu + 10368), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 10400), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 10432), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 10464), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 10496), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 10528), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 10560), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 10592), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 10624), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 10656), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 10688), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 10720), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 10752), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 10784), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 10816), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 10848), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 10880), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10912), b[4960], x);
      b[4992] = x;
    }
    {
      CHEM_PREFETCH(ws + 123744);
      CHEM_PREFETCH(ws + 123776);
      CHEM_PREFETCH(ws + 123808);
      CHEM_PREFETCH(ws + 123840);
      CHEM_PREFETCH(ws + 123872);
      CHEM_PREFETCH(ws + 123904);
      CHEM_PREFETCH(ws + 123936);
      CHEM_PREFETCH(ws + 123968);
      CHEM_PREFETCH(ws + 124000);
      CHEM_PREFETCH(ws + 124032);
      CHEM_PREFETCH(ws + 124064);
      CHEM_PREFETCH(ws + 124096);
      CHEM_PREFETCH(ws + 124128);
      CHEM_PREFETCH(ws + 124160);
      CHEM_PREFETCH(ws + 124192);
      CHEM_PREFETCH(ws + 124224);
      CHEM_PREFETCH(ws + 124256);
      CHEM_PREFETCH(ws + 124288);
      CHEM_PREFETCH(ws + 124320);
      CHEM_PREFETCH(ws + 124352);
      CHEM_PREFETCH(ws + 124384);
      CHEM_PREFETCH(ws + 124416);
      CHEM_PREFETCH(ws + 124448);
      CHEM_PREFETCH(ws + 124480);
      CHEM_PREFETCH(ws + 124512);
      CHEM_PREFETCH(ws + 124544);
      CHEM_PREFETCH(ws + 124576);
      double x = b[5024];
      x = fma(-CHEM_LDLU(lu + 10944), b[96], x);
      x = fma(-CHEM_LDLU(lu + 10976), b[128], x);
      x = fma(-CHEM_LDLU(lu + 11008), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 11040), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 11072), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 11104), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 11136), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 11168), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 11200), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 11232), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 11264), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 11296), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 11328), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 11360), b[4288], x);
      b[5024] = x;
    }
    {
      CHEM_PREFETCH(ws + 124608);
      CHEM_PREFETCH(ws + 124640);
      CHEM_PREFETCH(ws + 124672);
      CHEM_PREFETCH(ws + 124704);
      CHEM_PREFETCH(ws + 124736);
      CHEM_PREFETCH(ws + 124768);
      CHEM_PREFETCH(ws + 124800);
      CHEM_PREFETCH(ws + 124832);
      CHEM_PREFETCH(ws + 124864);
      CHEM_PREFETCH(ws + 124896);
      CHEM_PREFETCH(ws + 124928);
      CHEM_PREFETCH(ws + 124960);
      CHEM_PREFETCH(ws + 124992);
      CHEM_PREFETCH(ws + 125024);
      CHEM_PREFETCH(ws + 125056);
      double x = b[5056];
      x = fma(-CHEM_LDLU(lu + 11392), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 11424), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 11456), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 11488), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 11520), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 11552), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 11584), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 11616), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 11648), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 11680), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 11712), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 11744), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 11776), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 11808), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 11840), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 11872), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 11904), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 11936), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 11968), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 12000), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 12032), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 12064), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 12096), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 12128), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 12160), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 12192), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 12224), b[4992], x);
      b[5056] = x;
    }
    {
      CHEM_PREFETCH(ws + 125088);
      CHEM_PREFETCH(ws + 125120);
      CHEM_PREFETCH(ws + 125152);
      CHEM_PREFETCH(ws + 125184);
      CHEM_PREFETCH(ws + 125216);
      CHEM_PREFETCH(ws + 125248);
      CHEM_PREFETCH(ws + 125280);
      CHEM_PREFETCH(ws + 125312);
      CHEM_PREFETCH(ws + 125344);
      CHEM_PREFETCH(ws + 125376);
      CHEM_PREFETCH(ws + 125408);
      CHEM_PREFETCH(ws + 125440);
      CHEM_PREFETCH(ws + 125472);
      CHEM_PREFETCH(ws + 125504);
      double x = b[5088];
      x = fma(-CHEM_LDLU(lu + 12256), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 12288), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 12320), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 12352), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 12384), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 12416), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 12448), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 12480), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 12512), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 12544), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 12576), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 12608), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 12640), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 12672), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 12704), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 12736), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 12768), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 12800), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 12832), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 12864), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 12896), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 12928), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 12960), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 12992), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 13024), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 13056), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 13088), b[4992], x);
      b[5088] = x;
    }
    {
      CHEM_PREFETCH(ws + 125536);
      CHEM_PREFETCH(ws + 125568);
      CHEM_PREFETCH(ws + 125600);
      CHEM_PREFETCH(ws + 125632);
      CHEM_PREFETCH(ws + 125664);
      CHEM_PREFETCH(ws + 125696);
      CHEM_PREFETCH(ws + 125728);
      CHEM_PREFETCH(ws + 125760);
      CHEM_PREFETCH(ws + 125792);
      CHEM_PREFETCH(ws + 125824);
      CHEM_PREFETCH(ws + 125856);
      CHEM_PREFETCH(ws + 125888);
      CHEM_PREFETCH(ws + 125920);
      CHEM_PREFETCH(ws + 125952);
      CHEM_PREFETCH(ws + 125984);
      CHEM_PREFETCH(ws + 126016);
      CHEM_PREFETCH(ws + 126048);
      CHEM_PREFETCH(ws + 126080);
      CHEM_PREFETCH(ws + 126112);
      CHEM_PREFETCH(ws + 126144);
      CHEM_PREFETCH(ws + 126176);
      CHEM_PREFETCH(ws + 126208);
      double x = b[5120];
      x = fma(-CHEM_LDLU(lu + 13120), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 13152), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 13184), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 13216), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 13248), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 13280), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 13312), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 13344), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 13376), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 13408), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 13440), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 13472), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 13504), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 13536), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 13568), b[5088], x);
      b[5120] = x;
    }
    {
      CHEM_PREFETCH(ws + 126240);
      CHEM_PREFETCH(ws + 126272);
      CHEM_PREFETCH(ws + 126304);
      CHEM_PREFETCH(ws + 126336);
      CHEM_PREFETCH(ws + 126368);
      CHEM_PREFETCH(ws + 126400);
      CHEM_PREFETCH(ws + 126432);
      CHEM_PREFETCH(ws + 126464);
      CHEM_PREFETCH(ws + 126496);
      CHEM_PREFETCH(ws + 126528);
      CHEM_PREFETCH(ws + 126560);
      CHEM_PREFETCH(ws + 126592);
      CHEM_PREFETCH(ws + 126624);
      CHEM_PREFETCH(ws + 126656);
      CHEM_PREFETCH(ws + 126688);
      CHEM_PREFETCH(ws + 126720);
      CHEM_PREFETCH(ws + 126752);
      CHEM_PREFETCH(ws + 126784);
      CHEM_PREFETCH(ws + 126816);
      CHEM_PREFETCH(ws + 126848);
      CHEM_PREFETCH(ws + 126880);
      CHEM_PREFETCH(ws + 126912);
      CHEM_PREFETCH(ws + 126944);
      CHEM_PREFETCH(ws + 126976);
      CHEM_PREFETCH(ws + 127008);
      CHEM_PREFETCH(ws + 127040);
      CHEM_PREFETCH(ws + 127072);
      CHEM_PREFETCH(ws + 127104);
      CHEM_PREFETCH(ws + 127136);
      double x = b[5152];
      x = fma(-CHEM_LDLU(lu + 13600), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 13632), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 13664), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 13696), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 13728), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 13760), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 13792), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 13824), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 13856), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 13888), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 13920), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 13952), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 13984), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 14016), b[5088], x);
      b[5152] = x;
    }
    {
      CHEM_PREFETCH(ws + 127168);
      CHEM_PREFETCH(ws + 127200);
      CHEM_PREFETCH(ws + 127232);
      CHEM_PREFETCH(ws + 127264);
      CHEM_PREFETCH(ws + 127296);
      CHEM_PREFETCH(ws + 127328);
      CHEM_PREFETCH(ws + 127360);
      CHEM_PREFETCH(ws + 127392);
      CHEM_PREFETCH(ws + 127424);
      CHEM_PREFETCH(ws + 127456);
      CHEM_PREFETCH(ws + 127488);
      CHEM_PREFETCH(ws + 127520);
      CHEM_PREFETCH(ws + 127552);
      CHEM_PREFETCH(ws + 127584);
      CHEM_PREFETCH(ws + 127616);
      CHEM_PREFETCH(ws + 127648);
      CHEM_PREFETCH(ws + 127680);
      CHEM_PREFETCH(ws + 127712);
      CHEM_PREFETCH(ws + 127744);
      CHEM_PREFETCH(ws + 127776);
      CHEM_PREFETCH(ws + 127808);
      CHEM_PREFETCH(ws + 127840);
      CHEM_PREFETCH(ws + 127872);
      CHEM_PREFETCH(ws + 127904);
      CHEM_PREFETCH(ws + 127936);
      double x = b[5184];
      x = fma(-CHEM_LDLU(lu + 14048), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 14080), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 14112), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 14144), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 14176), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 14208), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 14240), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 14272), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 14304), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 14336), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 14368), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 14400), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 14432), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 14464), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 14496), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 14528), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 14560), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 14592), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 14624), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 14656), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 14688), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 14720), b[4736], x);
      b[5184] = x;
    }
    {
      CHEM_PREFETCH(ws + 127968);
      CHEM_PREFETCH(ws + 128000);
      CHEM_PREFETCH(ws + 128032);
      CHEM_PREFETCH(ws + 128064);
      CHEM_PREFETCH(ws + 128096);
      CHEM_PREFETCH(ws + 128128);
      CHEM_PREFETCH(ws + 128160);
      CHEM_PREFETCH(ws + 128192);
      CHEM_PREFETCH(ws + 128224);
      CHEM_PREFETCH(ws + 128256);
      CHEM_PREFETCH(ws + 128288);
      CHEM_PREFETCH(ws + 128320);
      CHEM_PREFETCH(ws + 128352);
      CHEM_PREFETCH(ws + 128384);
      CHEM_PREFETCH(ws + 128416);
      CHEM_PREFETCH(ws + 128448);
      CHEM_PREFETCH(ws + 128480);
      CHEM_PREFETCH(ws + 128512);
      CHEM_PREFETCH(ws + 128544);
      CHEM_PREFETCH(ws + 128576);
      double x = b[5216];
      x = fma(-CHEM_LDLU(lu + 14752), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 14784), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 14816), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 14848), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 14880), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 14912), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 14944), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 14976), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 15008), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 15040), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 15072), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 15104), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 15136), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 15168), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 15200), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 15232), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 15264), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 15296), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 15328), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 15360), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 15392), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 15424), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 15456), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 15488), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 15520), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 15552), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 15584), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 15616), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 15648), b[5184], x);
      b[5216] = x;
    }
    {
      CHEM_PREFETCH(ws + 128608);
      CHEM_PREFETCH(ws + 128640);
      CHEM_PREFETCH(ws + 128672);
      CHEM_PREFETCH(ws + 128704);
      CHEM_PREFETCH(ws + 128736);
      CHEM_PREFETCH(ws + 128768);
      CHEM_PREFETCH(ws + 128800);
      CHEM_PREFETCH(ws + 128832);
      CHEM_PREFETCH(ws + 128864);
      CHEM_PREFETCH(ws + 128896);
      CHEM_PREFETCH(ws + 128928);
      CHEM_PREFETCH(ws + 128960);
      CHEM_PREFETCH(ws + 128992);
      CHEM_PREFETCH(ws + 129024);
      CHEM_PREFETCH(ws + 129056);
      CHEM_PREFETCH(ws + 129088);
      CHEM_PREFETCH(ws + 129120);
      CHEM_PREFETCH(ws + 129152);
      CHEM_PREFETCH(ws + 129184);
      CHEM_PREFETCH(ws + 129216);
      CHEM_PREFETCH(ws + 129248);
      CHEM_PREFETCH(ws + 129280);
      CHEM_PREFETCH(ws + 129312);
      CHEM_PREFETCH(ws + 129344);
      CHEM_PREFETCH(ws + 129376);
      CHEM_PREFETCH(ws + 129408);
      CHEM_PREFETCH(ws + 129440);
      CHEM_PREFETCH(ws + 129472);
      CHEM_PREFETCH(ws + 129504);
      double x = b[5248];
      x = fma(-CHEM_LDLU(lu + 15680), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 15712), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 15744), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 15776), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 15808), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 15840), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 15872), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 15904), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 15936), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 15968), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 16000), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 16032), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 16064), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 16096), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 16128), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 16160), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 16192), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 16224), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 16256), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 16288), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 16320), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 16352), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 16384), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 16416), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 16448), b[5184], x);
      b[5248] = x;
    }
    {
      CHEM_PREFETCH(ws + 129536);
      CHEM_PREFETCH(ws + 129568);
      CHEM_PREFETCH(ws + 129600);
      CHEM_PREFETCH(ws + 129632);
      CHEM_PREFETCH(ws + 129664);
      CHEM_PREFETCH(ws + 129696);
      CHEM_PREFETCH(ws + 129728);
      CHEM_PREFETCH(ws + 129760);
      CHEM_PREFETCH(ws + 129792);
      CHEM_PREFETCH(ws + 129824);
      CHEM_PREFETCH(ws + 129856);
      CHEM_PREFETCH(ws + 129888);
      CHEM_PREFETCH(ws + 129920);
      CHEM_PREFETCH(ws + 129952);
      CHEM_PREFETCH(ws + 129984);
      CHEM_PREFETCH(ws + 130016);
      CHEM_PREFETCH(ws + 130048);
      CHEM_PREFETCH(ws + 130080);
      CHEM_PREFETCH(ws + 130112);
      CHEM_PREFETCH(ws + 130144);
      CHEM_PREFETCH(ws + 130176);
      CHEM_PREFETCH(ws + 130208);
      CHEM_PREFETCH(ws + 130240);
      CHEM_PREFETCH(ws + 130272);
      CHEM_PREFETCH(ws + 130304);
      CHEM_PREFETCH(ws + 130336);
      CHEM_PREFETCH(ws + 130368);
      CHEM_PREFETCH(ws + 130400);
      CHEM_PREFETCH(ws + 130432);
      CHEM_PREFETCH(ws + 130464);
      CHEM_PREFETCH(ws + 130496);
      double x = b[5280];
      x = fma(-CHEM_LDLU(lu + 16480), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 16512), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 16544), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 16576), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 16608), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 16640), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 16672), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 16704), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 16736), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 16768), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 16800), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 16832), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 16864), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 16896), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 16928), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 16960), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 16992), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 17024), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 17056), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 17088), b[5184], x);
      b[5280] = x;
    }
    {
      CHEM_PREFETCH(ws + 130528);
      CHEM_PREFETCH(ws + 130560);
      CHEM_PREFETCH(ws + 130592);
      CHEM_PREFETCH(ws + 130624);
      CHEM_PREFETCH(ws + 130656);
      CHEM_PREFETCH(ws + 130688);
      CHEM_PREFETCH(ws + 130720);
      CHEM_PREFETCH(ws + 130752);
      CHEM_PREFETCH(ws + 130784);
      CHEM_PREFETCH(ws + 130816);
      CHEM_PREFETCH(ws + 130848);
      CHEM_PREFETCH(ws + 130880);
      CHEM_PREFETCH(ws + 130912);
      CHEM_PREFETCH(ws + 130944);
      CHEM_PREFETCH(ws + 130976);
      CHEM_PREFETCH(ws + 131008);
      CHEM_PREFETCH(ws + 131040);
      CHEM_PREFETCH(ws + 131072);
      CHEM_PREFETCH(ws + 131104);
      CHEM_PREFETCH(ws + 131136);
      CHEM_PREFETCH(ws + 131168);
      CHEM_PREFETCH(ws + 131200);
      double x = b[5312];
      x = fma(-CHEM_LDLU(lu + 17120), b[832], x);
      x = fma(-CHEM_LDLU(lu + 17152), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 17184), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 17216), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 17248), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 17280), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 17312), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 17344), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 17376), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 17408), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 17440), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 17472), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 17504), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 17536), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 17568), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 17600), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 17632), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 17664), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 17696), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 17728), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 17760), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 17792), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 17824), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 17856), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 17888), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 17920), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 17952), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 17984), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 18016), b[5184], x);
      b[5312] = x;
    }
    {
      CHEM_PREFETCH(ws + 131232);
      CHEM_PREFETCH(ws + 131264);
      CHEM_PREFETCH(ws + 131296);
      CHEM_PREFETCH(ws + 131328);
      CHEM_PREFETCH(ws + 131360);
      CHEM_PREFETCH(ws + 131392);
      CHEM_PREFETCH(ws + 131424);
      CHEM_PREFETCH(ws + 131456);
      CHEM_PREFETCH(ws + 131488);
      CHEM_PREFETCH(ws + 131520);
      CHEM_PREFETCH(ws + 131552);
      CHEM_PREFETCH(ws + 131584);
      CHEM_PREFETCH(ws + 131616);
      CHEM_PREFETCH(ws + 131648);
      CHEM_PREFETCH(ws + 131680);
      CHEM_PREFETCH(ws + 131712);
      CHEM_PREFETCH(ws + 131744);
      CHEM_PREFETCH(ws + 131776);
      CHEM_PREFETCH(ws + 131808);
      CHEM_PREFETCH(ws + 131840);
      double x = b[5344];
      x = fma(-CHEM_LDLU(lu + 18048), b[448], x);
      x = fma(-CHEM_LDLU(lu + 18080), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 18112), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 18144), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 18176), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 18208), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 18240), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 18272), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 18304), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 18336), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 18368), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 18400), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 18432), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 18464), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 18496), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 18528), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 18560), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 18592), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 18624), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 18656), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 18688), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 18720), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 18752), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 18784), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 18816), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 18848), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 18880), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 18912), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 18944), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 18976), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 19008), b[5312], x);
      b[5344] = x;
    }
    {
      CHEM_PREFETCH(ws + 131872);
      CHEM_PREFETCH(ws + 131904);
      CHEM_PREFETCH(ws + 131936);
      CHEM_PREFETCH(ws + 131968);
      CHEM_PREFETCH(ws + 132000);
      CHEM_PREFETCH(ws + 132032);
      CHEM_PREFETCH(ws + 132064);
      CHEM_PREFETCH(ws + 132096);
      CHEM_PREFETCH(ws + 132128);
      CHEM_PREFETCH(ws + 132160);
      CHEM_PREFETCH(ws + 132192);
      CHEM_PREFETCH(ws + 132224);
      CHEM_PREFETCH(ws + 132256);
      CHEM_PREFETCH(ws + 132288);
      CHEM_PREFETCH(ws + 132320);
      CHEM_PREFETCH(ws + 132352);
      CHEM_PREFETCH(ws + 132384);
      CHEM_PREFETCH(ws + 132416);
      CHEM_PREFETCH(ws + 132448);
      CHEM_PREFETCH(ws + 132480);
      CHEM_PREFETCH(ws + 132512);
      CHEM_PREFETCH(ws + 132544);
      CHEM_PREFETCH(ws + 132576);
      CHEM_PREFETCH(ws + 132608);
      CHEM_PREFETCH(ws + 132640);
      CHEM_PREFETCH(ws + 132672);
      CHEM_PREFETCH(ws + 132704);
      CHEM_PREFETCH(ws + 132736);
      CHEM_PREFETCH(ws + 132768);
      CHEM_PREFETCH(ws + 132800);
      CHEM_PREFETCH(ws + 132832);
      CHEM_PREFETCH(ws + 132864);
      CHEM_PREFETCH(ws + 132896);
      CHEM_PREFETCH(ws + 132928);
      CHEM_PREFETCH(ws + 132960);
      CHEM_PREFETCH(ws + 132992);
      CHEM_PREFETCH(ws + 133024);
      CHEM_PREFETCH(ws + 133056);
      CHEM_PREFETCH(ws + 133088);
      CHEM_PREFETCH(ws + 133120);
      CHEM_PREFETCH(ws + 133152);
      double x = b[5376];
      x = fma(-CHEM_LDLU(lu + 19040), b[256], x);
      x = fma(-CHEM_LDLU(lu + 19072), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 19104), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 19136), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 19168), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 19200), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 19232), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 19264), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 19296), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 19328), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 19360), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 19392), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 19424), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 19456), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 19488), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 19520), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 19552), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 19584), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 19616), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 19648), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 19680), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 19712), b[5184], x);
      b[5376] = x;
    }
}
__device__ __noinline__ void solve_1_1(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH(ws + 133184);
      CHEM_PREFETCH(ws + 133216);
      CHEM_PREFETCH(ws + 133248);
      CHEM_PREFETCH(ws + 133280);
      CHEM_PREFETCH(ws + 133312);
      CHEM_PREFETCH(ws + 133344);
      CHEM_PREFETCH(ws + 133376);
      CHEM_PREFETCH(ws + 133408);
      CHEM_PREFETCH(ws + 133440);
      CHEM_PREFETCH(ws + 133472);
      CHEM_PREFETCH(ws + 133504);
      CHEM_PREFETCH(ws + 133536);
      CHEM_PREFETCH(ws + 133568);
      CHEM_PREFETCH(ws + 133600);
      CHEM_PREFETCH(ws + 133632);
      CHEM_PREFETCH(ws + 133664);
      CHEM_PREFETCH(ws + 133696);
      CHEM_PREFETCH(ws + 133728);
      CHEM_PREFETCH(ws + 133760);
      CHEM_PREFETCH(ws + 133792);
      CHEM_PREFETCH(ws + 133824);
      CHEM_PREFETCH(ws + 133856);
      CHEM_PREFETCH(ws + 133888);
      CHEM_PREFETCH(ws + 133920);
      CHEM_PREFETCH(ws + 133952);
      double x = b[5408];
      x = fma(-CHEM_LDLU(lu + 19744), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 19776), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 19808), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 19840), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 19872), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 19904), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 19936), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 19968), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 20000), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 20032), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 20064), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 20096), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 20128), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 20160), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 20192), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 20224), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 20256), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 20288), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 20320), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 20352), b[5312], x);
      b[5408] = x;
    }
    {
      CHEM_PREFETCH(ws + 133984);
      CHEM_PREFETCH(ws + 134016);
      CHEM_PREFETCH(ws + 134048);
      CHEM_PREFETCH(ws + 134080);
      CHEM_PREFETCH(ws + 134112);
      CHEM_PREFETCH(ws + 134144);
      CHEM_PREFETCH(ws + 134176);
      CHEM_PREFETCH(ws + 134208);
      CHEM_PREFETCH(ws + 134240);
      CHEM_PREFETCH(ws + 134272);
      CHEM_PREFETCH(ws + 134304);
      CHEM_PREFETCH(ws + 134336);
      CHEM_PREFETCH(ws + 134368);
      CHEM_PREFETCH(ws + 134400);
      CHEM_PREFETCH(ws + 134432);
      CHEM_PREFETCH(ws + 134464);
      CHEM_PREFETCH(ws + 134496);
      CHEM_PREFETCH(ws + 134528);
      CHEM_PREFETCH(ws + 134560);
      CHEM_PREFETCH(ws + 134592);
      CHEM_PREFETCH(ws + 134624);
      CHEM_PREFETCH(ws + 134656);
      CHEM_PREFETCH(ws + 134688);
      CHEM_PREFETCH(ws + 134720);
      CHEM_PREFETCH(ws + 134752);
      CHEM_PREFETCH(ws + 134784);
      CHEM_PREFETCH(ws + 134816);
      CHEM_PREFETCH(ws + 134848);
      CHEM_PREFETCH(ws + 134880);
      CHEM_PREFETCH(ws + 134912);
      CHEM_PREFETCH(ws + 134944);
      CHEM_PREFETCH(ws + 134976);
      CHEM_PREFETCH(ws + 135008);
      CHEM_PREFETCH(ws + 135040);
      CHEM_PREFETCH(ws + 135072);
      double x = b[5440];
      x = fma(-CHEM_LDLU(lu + 20384), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 20416), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 20448), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 20480), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 20512), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 20544), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 20576), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 20608), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 20640), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 20672), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 20704), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 20736), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 20768), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 20800), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 20832), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 20864), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 20896), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 20928), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 20960), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 20992), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 21024), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 21056), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 21088), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 21120), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 21152), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 21184), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 21216), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 21248), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 21280), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 21312), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 21344), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 21376), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 21408), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 21440), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 21472), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 21504), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 21536), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 21568), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 21600), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 21632), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 21664), b[5408], x);
      b[5440] = x;
    }
    {
      CHEM_PREFETCH(ws + 135104);
      CHEM_PREFETCH(ws + 135136);
      CHEM_PREFETCH(ws + 135168);
      CHEM_PREFETCH(ws + 135200);
      CHEM_PREFETCH(ws + 135232);
      CHEM_PREFETCH(ws + 135264);
      CHEM_PREFETCH(ws + 135296);
      CHEM_PREFETCH(ws + 135328);
      CHEM_PREFETCH(ws + 135360);
      CHEM_PREFETCH(ws + 135392);
      CHEM_PREFETCH(ws + 135424);
      CHEM_PREFETCH(ws + 135456);
      CHEM_PREFETCH(ws + 135488);
      CHEM_PREFETCH(ws + 135520);
      CHEM_PREFETCH(ws + 135552);
      CHEM_PREFETCH(ws + 135584);
      CHEM_PREFETCH(ws + 135616);
      CHEM_PREFETCH(ws + 135648);
      CHEM_PREFETCH(ws + 135680);
      CHEM_PREFETCH(ws + 135712);
      CHEM_PREFETCH(ws + 135744);
      CHEM_PREFETCH(ws + 135776);
      CHEM_PREFETCH(ws + 135808);
      CHEM_PREFETCH(ws + 135840);
      CHEM_PREFETCH(ws + 135872);
      CHEM_PREFETCH(ws + 135904);
      CHEM_PREFETCH(ws + 135936);
      CHEM_PREFETCH(ws + 135968);
      CHEM_PREFETCH(ws + 136000);
      double x = b[5472];
      x = fma(-CHEM_LDLU(lu + 21696), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 21728), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 21760), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 21792), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 21824), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 21856), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 21888), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 21920), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 21952), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 21984), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 22016), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 22048), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 22080), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 22112), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 22144), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 22176), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 22208), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 22240), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 22272), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 22304), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 22336), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 22368), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 22400), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 22432), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 22464), b[5440], x);
      b[5472] = x;
    }
    {
      CHEM_PREFETCH(ws + 136032);
      CHEM_PREFETCH(ws + 136064);
      CHEM_PREFETCH(ws + 136096);
      CHEM_PREFETCH(ws + 136128);
      CHEM_PREFETCH(ws + 136160);
      CHEM_PREFETCH(ws + 136192);
      CHEM_PREFETCH(ws + 136224);
      CHEM_PREFETCH(ws + 136256);
      CHEM_PREFETCH(ws + 136288);
      CHEM_PREFETCH(ws + 136320);
      CHEM_PREFETCH(ws + 136352);
      CHEM_PREFETCH(ws + 136384);
      CHEM_PREFETCH(ws + 136416);
      CHEM_PREFETCH(ws + 136448);
      CHEM_PREFETCH(ws + 136480);
      CHEM_PREFETCH(ws + 136512);
      CHEM_PREFETCH(ws + 136544);
      CHEM_PREFETCH(ws + 136576);
      CHEM_PREFETCH(ws + 136608);
      CHEM_PREFETCH(ws + 136640);
      CHEM_PREFETCH(ws + 136672);
      CHEM_PREFETCH(ws + 136704);
      CHEM_PREFETCH(ws + 136736);
      CHEM_PREFETCH(ws + 136768);
      CHEM_PREFETCH(ws + 136800);
      CHEM_PREFETCH(ws + 136832);
      CHEM_PREFETCH(ws + 136864);
      CHEM_PREFETCH(ws + 136896);
      CHEM_PREFETCH(ws + 136928);
      CHEM_PREFETCH(ws + 136960);
      CHEM_PREFETCH(ws + 136992);
      CHEM_PREFETCH(ws + 137024);
      double x = b[5504];
      x = fma(-CHEM_LDLU(lu + 22496), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 22528), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 22560), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 22592), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 22624), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 22656), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 22688), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 22720), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 22752), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 22784), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 22816), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 22848), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 22880), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 22912), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 22944), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 22976), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 23008), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 23040), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 23072), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 23104), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 23136), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 23168), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 23200), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 23232), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 23264), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 23296), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 23328), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 23360), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 23392), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 23424), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 23456), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 23488), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 23520), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 23552), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 23584), b[5472], x);
      b[5504] = x;
    }
    {
      CHEM_PREFETCH(ws + 137056);
      CHEM_PREFETCH(ws + 137088);
      CHEM_PREFETCH(ws + 137120);
      CHEM_PREFETCH(ws + 137152);
      CHEM_PREFETCH(ws + 137184);
      CHEM_PREFETCH(ws + 137216);
      CHEM_PREFETCH(ws + 137248);
      CHEM_PREFETCH(ws + 137280);
      CHEM_PREFETCH(ws + 137312);
      CHEM_PREFETCH(ws + 137344);
      CHEM_PREFETCH(ws + 137376);
      CHEM_PREFETCH(ws + 137408);
      CHEM_PREFETCH(ws + 137440);
      CHEM_PREFETCH(ws + 137472);
      CHEM_PREFETCH(ws + 137504);
      CHEM_PREFETCH(ws + 137536);
      CHEM_PREFETCH(ws + 137568);
      CHEM_PREFETCH(ws + 137600);
      CHEM_PREFETCH(ws + 137632);
      CHEM_PREFETCH(ws + 137664);
      CHEM_PREFETCH(ws + 137696);
      CHEM_PREFETCH(ws + 137728);
      CHEM_PREFETCH(ws + 137760);
      CHEM_PREFETCH(ws + 137792);
      CHEM_PREFETCH(ws + 137824);
      CHEM_PREFETCH(ws + 137856);
      CHEM_PREFETCH(ws + 137888);
      CHEM_PREFETCH(ws + 137920);
      CHEM_PREFETCH(ws + 137952);
      CHEM_PREFETCH(ws + 137984);
      CHEM_PREFETCH(ws + 138016);
      CHEM_PREFETCH(ws + 138048);
      CHEM_PREFETCH(ws + 138080);
      CHEM_PREFETCH(ws + 138112);
      CHEM_PREFETCH(ws + 138144);
      CHEM_PREFETCH(ws + 138176);
      CHEM_PREFETCH(ws + 138208);
      CHEM_PREFETCH(ws + 138240);
      CHEM_PREFETCH(ws + 138272);
      CHEM_PREFETCH(ws + 138304);
      CHEM_PREFETCH(ws + 138336);
      CHEM_PREFETCH(ws + 138368);
      CHEM_PREFETCH(ws + 138400);
      CHEM_PREFETCH(ws + 138432);
      CHEM_PREFETCH(ws + 138464);
      CHEM_PREFETCH(ws + 138496);
      CHEM_PREFETCH(ws + 138528);
      CHEM_PREFETCH(ws + 138560);
      CHEM_PREFETCH(ws + 138592);
      double x = b[5536];
      x = fma(-CHEM_LDLU(lu + 23616), b[864], x);
      x = fma(-CHEM_LDLU(lu + 23648), b[896], x);
      x = fma(-CHEM_LDLU(lu + 23680), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 23712), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 23744), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 23776), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 23808), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 23840), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 23872), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 23904), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 23936), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 23968), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 24000), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 24032), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 24064), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 24096), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 24128), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 24160), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 24192), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 24224), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 24256), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 24288), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 24320), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 24352), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 24384), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 24416), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 24448), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 24480), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 24512), b[5504], x);
      b[5536] = x;
    }
    {
      CHEM_PREFETCH(ws + 138624);
      CHEM_PREFETCH(ws + 138656);
      CHEM_PREFETCH(ws + 138688);
      CHEM_PREFETCH(ws + 138720);
      CHEM_PREFETCH(ws + 138752);
      CHEM_PREFETCH(ws + 138784);
      CHEM_PREFETCH(ws + 138816);
      CHEM_PREFETCH(ws + 138848);
      CHEM_PREFETCH(ws + 138880);
      CHEM_PREFETCH(ws + 138912);
      CHEM_PREFETCH(ws + 138944);
      CHEM_PREFETCH(ws + 138976);
      CHEM_PREFETCH(ws + 139008);
      CHEM_PREFETCH(ws + 139040);
      CHEM_PREFETCH(ws + 139072);
      CHEM_PREFETCH(ws + 139104);
      CHEM_PREFETCH(ws + 139136);
      CHEM_PREFETCH(ws + 139168);
      CHEM_PREFETCH(ws + 139200);
      CHEM_PREFETCH(ws + 139232);
      CHEM_PREFETCH(ws + 139264);
      CHEM_PREFETCH(ws + 139296);
      CHEM_PREFETCH(ws + 139328);
      CHEM_PREFETCH(ws + 139360);
      CHEM_PREFETCH(ws + 139392);
      CHEM_PREFETCH(ws + 139424);
      CHEM_PREFETCH(ws + 139456);
      CHEM_PREFETCH(ws + 139488);
      CHEM_PREFETCH(ws + 139520);
      CHEM_PREFETCH(ws + 139552);
      double x = b[5568];
      x = fma(-CHEM_LDLU(lu + 24544), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 24576), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 24608), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 24640), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 24672), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 24704), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 24736), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 24768), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 24800), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 24832), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 24864), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 24896), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 24928), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 24960), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 24992), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 25024), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 25056), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 25088), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 25120), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 25152), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 25184), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 25216), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 25248), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 25280), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 25312), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 25344), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 25376), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 25408), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 25440), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 25472), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 25504), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 25536), b[5536], x);
      b[5568] = x;
    }
    {
      CHEM_PREFETCH(ws + 139584);
      CHEM_PREFETCH(ws + 139616);
      CHEM_PREFETCH(ws + 139648);
      CHEM_PREFETCH(ws + 139680);
      CHEM_PREFETCH(ws + 139712);
      CHEM_PREFETCH(ws + 139744);
      CHEM_PREFETCH(ws + 139776);
      CHEM_PREFETCH(ws + 139808);
      CHEM_PREFETCH(ws + 139840);
      CHEM_PREFETCH(ws + 139872);
      CHEM_PREFETCH(ws + 139904);
      CHEM_PREFETCH(ws + 139936);
      CHEM_PREFETCH(ws + 139968);
      CHEM_PREFETCH(ws + 140000);
      CHEM_PREFETCH(ws + 140032);
      CHEM_PREFETCH(ws + 140064);
      CHEM_PREFETCH(ws + 140096);
      CHEM_PREFETCH(ws + 140128);
      CHEM_PREFETCH(ws + 140160);
      CHEM_PREFETCH(ws + 140192);
      CHEM_PREFETCH(ws + 140224);
      CHEM_PREFETCH(ws + 140256);
      CHEM_PREFETCH(ws + 140288);
      CHEM_PREFETCH(ws + 140320);
      CHEM_PREFETCH(ws + 140352);
      CHEM_PREFETCH(ws + 140384);
      CHEM_PREFETCH(ws + 140416);
      CHEM_PREFETCH(ws + 140448);
      CHEM_PREFETCH(ws + 140480);
      CHEM_PREFETCH(ws + 140512);
      CHEM_PREFETCH(ws + 140544);
      double x = b[5600];
      x = fma(-CHEM_LDLU(lu + 25568), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 25600), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 25632), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 25664), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 25696), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 25728), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 25760), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 25792), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 25824), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 25856), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 25888), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 25920), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 25952), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 25984), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 26016), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 26048), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 26080), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 26112), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 26144), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 26176), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 26208), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 26240), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 26272), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 26304), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 26336), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 26368), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 26400), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 26432), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 26464), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 26496), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 26528), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 26560), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26592), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 26624), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 26656), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 26688), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 26720), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 26752), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 26784), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 26816), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 26848), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 26880), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 26912), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 26944), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 26976), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 27008), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 27040), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 27072), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 27104), b[5536], x);
      b[5600] = x;
    }
    {
      CHEM_PREFETCH(ws + 140576);
      CHEM_PREFETCH(ws + 140608);
      CHEM_PREFETCH(ws + 140640);
      CHEM_PREFETCH(ws + 140672);
      CHEM_PREFETCH(ws + 140704);
      CHEM_PREFETCH(ws + 140736);
      CHEM_PREFETCH(ws + 140768);
      CHEM_PREFETCH(ws + 140800);
      CHEM_PREFETCH(ws + 140832);
      CHEM_PREFETCH(ws + 140864);
      CHEM_PREFETCH(ws + 140896);
      CHEM_PREFETCH(ws + 140928);
      CHEM_PREFETCH(ws + 140960);
      CHEM_PREFETCH(ws + 140992);
      CHEM_PREFETCH(ws + 141024);
      CHEM_PREFETCH(ws + 141056);
      CHEM_PREFETCH(ws + 141088);
      CHEM_PREFETCH(ws + 141120);
      CHEM_PREFETCH(ws + 141152);
      CHEM_PREFETCH(ws + 141184);
      CHEM_PREFETCH(ws + 141216);
      CHEM_PREFETCH(ws + 141248);
      CHEM_PREFETCH(ws + 141280);
      CHEM_PREFETCH(ws + 141312);
      CHEM_PREFETCH(ws + 141344);
      CHEM_PREFETCH(ws + 141376);
      CHEM_PREFETCH(ws + 141408);
      CHEM_PREFETCH(ws + 141440);
      CHEM_PREFETCH(ws + 141472);
      CHEM_PREFETCH(ws + 141504);
      CHEM_PREFETCH(ws + 141536);
      CHEM_PREFETCH(ws + 141568);
      CHEM_PREFETCH(ws + 141600);
      CHEM_PREFETCH(ws + 141632);
      CHEM_PREFETCH(ws + 141664);
      CHEM_PREFETCH(ws + 141696);
      CHEM_PREFETCH(ws + 141728);
      CHEM_PREFETCH(ws + 141760);
      CHEM_PREFETCH(ws + 141792);
      CHEM_PREFETCH(ws + 141824);
      CHEM_PREFETCH(ws + 141856);
      CHEM_PREFETCH(ws + 141888);
      CHEM_PREFETCH(ws + 141920);
      CHEM_PREFETCH(ws + 141952);
      CHEM_PREFETCH(ws + 141984);
      CHEM_PREFETCH(ws + 142016);
      CHEM_PREFETCH(ws + 142048);
      CHEM_PREFETCH(ws + 142080);
      CHEM_PREFETCH(ws + 142112);
      CHEM_PREFETCH(ws + 142144);
      CHEM_PREFETCH(ws + 142176);
      CHEM_PREFETCH(ws + 142208);
      CHEM_PREFETCH(ws + 142240);
      CHEM_PREFETCH(ws + 142272);
      CHEM_PREFETCH(ws + 142304);
      double x = b[5632];
      x = fma(-CHEM_LDLU(lu + 27136), b[384], x);
      x = fma(-CHEM_LDLU(lu + 27168), b[416], x);
      x = fma(-CHEM_LDLU(lu + 27200), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 27232), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 27264), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 27296), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 27328), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 27360), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 27392), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 27424), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 27456), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 27488), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 27520), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 27552), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 27584), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 27616), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 27648), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 27680), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 27712), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 27744), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 27776), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 27808), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 27840), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 27872), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 27904), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 27936), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 27968), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 28000), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 28032), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 28064), b[5536], x);
      b[5632] = x;
    }
    {
      CHEM_PREFETCH(ws + 142336);
      CHEM_PREFETCH(ws + 142368);
      CHEM_PREFETCH(ws + 142400);
      CHEM_PREFETCH(ws + 142432);
      CHEM_PREFETCH(ws + 142464);
      CHEM_PREFETCH(ws + 142496);
      CHEM_PREFETCH(ws + 142528);
      CHEM_PREFETCH(ws + 142560);
      CHEM_PREFETCH(ws + 142592);
      CHEM_PREFETCH(ws + 142624);
      CHEM_PREFETCH(ws + 142656);
      CHEM_PREFETCH(ws + 142688);
      CHEM_PREFETCH(ws + 142720);
      CHEM_PREFETCH(ws + 142752);
      CHEM_PREFETCH(ws + 142784);
      CHEM_PREFETCH(ws + 142816);
      CHEM_PREFETCH(ws + 142848);
      CHEM_PREFETCH(ws + 142880);
      CHEM_PREFETCH(ws + 142912);
      CHEM_PREFETCH(ws + 142944);
      CHEM_PREFETCH(ws + 142976);
      CHEM_PREFETCH(ws + 143008);
      CHEM_PREFETCH(ws + 143040);
      CHEM_PREFETCH(ws + 143072);
      CHEM_PREFETCH(ws + 143104);
      CHEM_PREFETCH(ws + 143136);
      CHEM_PREFETCH(ws + 143168);
      CHEM_PREFETCH(ws + 143200);
      CHEM_PREFETCH(ws + 143232);
      CHEM_PREFETCH(ws + 143264);
      CHEM_PREFETCH(ws + 143296);
      CHEM_PREFETCH(ws + 143328);
      CHEM_PREFETCH(ws + 143360);
      CHEM_PREFETCH(ws + 143392);
      CHEM_PREFETCH(ws + 143424);
      CHEM_PREFETCH(ws + 143456);
      CHEM_PREFETCH(ws + 143488);
      CHEM_PREFETCH(ws + 143520);
      CHEM_PREFETCH(ws + 143552);
      CHEM_PREFETCH(ws + 143584);
      CHEM_PREFETCH(ws + 143616);
      CHEM_PREFETCH(ws + 143648);
      CHEM_PREFETCH(ws + 143680);
      CHEM_PREFETCH(ws + 143712);
      CHEM_PREFETCH(ws + 143744);
      CHEM_PREFETCH(ws + 143776);
      CHEM_PREFETCH(ws + 143808);
      CHEM_PREFETCH(ws + 143840);
      CHEM_PREFETCH(ws + 143872);
      CHEM_PREFETCH(ws + 143904);
      CHEM_PREFETCH(ws + 143936);
      CHEM_PREFETCH(ws + 143968);
      CHEM_PREFETCH(ws + 144000);
      CHEM_PREFETCH(ws + 144032);
      CHEM_PREFETCH(ws + 144064);
      CHEM_PREFETCH(ws + 144096);
      CHEM_PREFETCH(ws + 144128);
      CHEM_PREFETCH(ws + 144160);
      double x = b[5664];
      x = fma(-CHEM_LDLU(lu + 28096), b[256], x);
      x = fma(-CHEM_LDLU(lu + 28128), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 28160), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 28192), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 28224), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 28256), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 28288), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 28320), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 28352), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 28384), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 28416), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 28448), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 28480), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 28512), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 28544), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 28576), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 28608), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 28640), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 28672), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 28704), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 28736), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 28768), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 28800), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 28832), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 28864), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 28896), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 28928), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 28960), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 28992), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 29024), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 29056), b[5536], x);
      b[5664] = x;
    }
    {
      CHEM_PREFETCH(ws + 144192);
      CHEM_PREFETCH(ws + 144224);
      CHEM_PREFETCH(ws + 144256);
      CHEM_PREFETCH(ws + 144288);
      CHEM_PREFETCH(ws + 144320);
      CHEM_PREFETCH(ws + 144352);
      CHEM_PREFETCH(ws + 144384);
      CHEM_PREFETCH(ws + 144416);
      CHEM_PREFETCH(ws + 144448);
      CHEM_PREFETCH(ws + 144480);
      CHEM_PREFETCH(ws + 144512);
      CHEM_PREFETCH(ws + 144544);
      CHEM_PREFETCH(ws + 144576);
      CHEM_PREFETCH(ws + 144608);
      CHEM_PREFETCH(ws + 144640);
      CHEM_PREFETCH(ws + 144672);
      CHEM_PREFETCH(ws + 144704);
      CHEM_PREFETCH(ws + 144736);
      CHEM_PREFETCH(ws + 144768);
      CHEM_PREFETCH(ws + 144800);
      CHEM_PREFETCH(ws + 144832);
      CHEM_PREFETCH(ws + 144864);
      CHEM_PREFETCH(ws + 144896);
      CHEM_PREFETCH(ws + 144928);
      CHEM_PREFETCH(ws + 144960);
      CHEM_PREFETCH(ws + 144992);
      CHEM_PREFETCH(ws + 145024);
      CHEM_PREFETCH(ws + 145056);
      CHEM_PREFETCH(ws + 145088);
      CHEM_PREFETCH(ws + 145120);
      CHEM_PREFETCH(ws + 145152);
      CHEM_PREFETCH(ws + 145184);
      CHEM_PREFETCH(ws + 145216);
      CHEM_PREFETCH(ws + 145248);
      CHEM_PREFETCH(ws + 145280);
      CHEM_PREFETCH(ws + 145312);
      CHEM_PREFETCH(ws + 145344);
      CHEM_PREFETCH(ws + 145376);
      CHEM_PREFETCH(ws + 145408);
      CHEM_PREFETCH(ws + 145440);
      CHEM_PREFETCH(ws + 145472);
      CHEM_PREFETCH(ws + 145504);
      CHEM_PREFETCH(ws + 145536);
      CHEM_PREFETCH(ws + 145568);
      CHEM_PREFETCH(ws + 145600);
      CHEM_PREFETCH(ws + 145632);
      CHEM_PREFETCH(ws + 145664);
      CHEM_PREFETCH(ws + 145696);
      CHEM_PREFETCH(ws + 145728);
      CHEM_PREFETCH(ws + 145760);
      double x = b[5696];
      x = fma(-CHEM_LDLU(lu + 29088), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 29120), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 29152), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 29184), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 29216), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 29248), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 29280), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 29312), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 29344), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 29376), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 29408), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 29440), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 29472), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 29504), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 29536), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 29568), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 29600), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 29632), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 29664), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 29696), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 29728), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 29760), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 29792), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 29824), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 29856), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 29888), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 29920), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 29952), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 29984), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 30016), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 30048), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 30080), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 30112), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 30144), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 30176), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 30208), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 30240), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 30272), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 30304), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 30336), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 30368), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 30400), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 30432), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 30464), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 30496), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 30528), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 30560), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 30592), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 30624), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 30656), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 30688), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 30720), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 30752), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 30784), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 30816), b[5632], x);
      b[5696] = x;
    }
    {
      CHEM_PREFETCH(ws + 145792);
      CHEM_PREFETCH(ws + 145824);
      CHEM_PREFETCH(ws + 145856);
      CHEM_PREFETCH(ws + 145888);
      CHEM_PREFETCH(ws + 145920);
      CHEM_PREFETCH(ws + 145952);
      CHEM_PREFETCH(ws + 145984);
      CHEM_PREFETCH(ws + 146016);
      CHEM_PREFETCH(ws + 146048);
      CHEM_PREFETCH(ws + 146080);
      CHEM_PREFETCH(ws + 146112);
      CHEM_PREFETCH(ws + 146144);
      CHEM_PREFETCH(ws + 146176);
      CHEM_PREFETCH(ws + 146208);
      CHEM_PREFETCH(ws + 146240);
      CHEM_PREFETCH(ws + 146272);
      CHEM_PREFETCH(ws + 146304);
      CHEM_PREFETCH(ws + 146336);
      CHEM_PREFETCH(ws + 146368);
      CHEM_PREFETCH(ws + 146400);
      CHEM_PREFETCH(ws + 146432);
      CHEM_PREFETCH(ws + 146464);
      CHEM_PREFETCH(ws + 146496);
      CHEM_PREFETCH(ws + 146528);
      CHEM_PREFETCH(ws + 146560);
      CHEM_PREFETCH(ws + 146592);
      CHEM_PREFETCH(ws + 146624);
      CHEM_PREFETCH(ws + 146656);
      CHEM_PREFETCH(ws + 146688);
      CHEM_PREFETCH(ws + 146720);
      CHEM_PREFETCH(ws + 146752);
      CHEM_PREFETCH(ws + 146784);
      CHEM_PREFETCH(ws + 146816);
      CHEM_PREFETCH(ws + 146848);
      CHEM_PREFETCH(ws + 146880);
      CHEM_PREFETCH(ws + 146912);
      CHEM_PREFETCH(ws + 146944);
      CHEM_PREFETCH(ws + 146976);
      CHEM_PREFETCH(ws + 147008);
      CHEM_PREFETCH(ws + 147040);
      CHEM_PREFETCH(ws + 147072);
      CHEM_PREFETCH(ws + 147104);
      CHEM_PREFETCH(ws + 147136);
      CHEM_PREFETCH(ws + 147168);
      CHEM_PREFETCH(ws + 147200);
      CHEM_PREFETCH(ws + 147232);
      CHEM_PREFETCH(ws + 147264);
      CHEM_PREFETCH(ws + 147296);
      CHEM_PREFETCH(ws + 147328);
      CHEM_PREFETCH(ws + 147360);
      CHEM_PREFETCH(ws + 147392);
      CHEM_PREFETCH(ws + 147424);
      CHEM_PREFETCH(ws + 147456);
      CHEM_PREFETCH(ws + 147488);
      CHEM_PREFETCH(ws + 147520);
      CHEM_PREFETCH(ws + 147552);
      CHEM_PREFETCH(ws + 147584);
      CHEM_PREFETCH(ws + 147616);
      CHEM_PREFETCH(ws + 147648);
      CHEM_PREFETCH(ws + 147680);
      CHEM_PREFETCH(ws + 147712);
      CHEM_PREFETCH(ws + 147744);
      CHEM_PREFETCH(ws + 147776);
      CHEM_PREFETCH(ws + 147808);
      CHEM_PREFETCH(ws + 147840);
      CHEM_PREFETCH(ws + 147872);
      CHEM_PREFETCH(ws + 147904);
      CHEM_PREFETCH(ws + 147936);
      CHEM_PREFETCH(ws + 147968);
      CHEM_PREFETCH(ws + 148000);
      CHEM_PREFETCH(ws + 148032);
      CHEM_PREFETCH(ws + 148064);
      CHEM_PREFETCH(ws + 148096);
      CHEM_PREFETCH(ws + 148128);
      CHEM_PREFETCH(ws + 148160);
      double x = b[5728];
      x = fma(-CHEM_LDLU(lu + 30848), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 30880), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 30912), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 30944), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 30976), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 31008), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 31040), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 31072), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 31104), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 31136), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 31168), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 31200), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 31232), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 31264), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 31296), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 31328), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 31360), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 31392), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 31424), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 31456), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 31488), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 31520), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 31552), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 31584), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 31616), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 31648), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 31680), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 31712), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 31744), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 31776), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 31808), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 31840), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 31872), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 31904), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 31936), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 31968), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 32000), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 32032), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 32064), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 32096), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 32128), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 32160), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 32192), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 32224), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 32256), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 32288), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 32320), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 32352), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 32384), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 32416), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 32448), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 32480), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 32512), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 32544), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 32576), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 32608), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 32640), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 32672), b[5696], x);
      b[5728] = x;
    }
    {
      CHEM_PREFETCH(ws + 148192);
      CHEM_PREFETCH(ws + 148224);
      CHEM_PREFETCH(ws + 148256);
      CHEM_PREFETCH(ws + 148288);
      CHEM_PREFETCH(ws + 148320);
      CHEM_PREFETCH(ws + 148352);
      CHEM_PREFETCH(ws + 148384);
      CHEM_PREFETCH(ws + 148416);
      CHEM_PREFETCH(ws + 148448);
      CHEM_PREFETCH(ws + 148480);
      CHEM_PREFETCH(ws + 148512);
      CHEM_PREFETCH(ws + 148544);
      CHEM_PREFETCH(ws + 148576);
      CHEM_PREFETCH(ws + 148608);
      CHEM_PREFETCH(ws + 148640);
      CHEM_PREFETCH(ws + 148672);
      CHEM_PREFETCH(ws + 148704);
      CHEM_PREFETCH(ws + 148736);
      CHEM_PREFETCH(ws + 148768);
      CHEM_PREFETCH(ws + 148800);
      CHEM_PREFETCH(ws + 148832);
      CHEM_PREFETCH(ws + 148864);
      CHEM_PREFETCH(ws + 148896);
      CHEM_PREFETCH(ws + 148928);
      CHEM_PREFETCH(ws + 148960);
      CHEM_PREFETCH(ws + 148992);
      CHEM_PREFETCH(ws + 149024);
      CHEM_PREFETCH(ws + 149056);
      CHEM_PREFETCH(ws + 149088);
      CHEM_PREFETCH(ws + 149120);
      CHEM_PREFETCH(ws + 149152);
      CHEM_PREFETCH(ws + 149184);
      CHEM_PREFETCH(ws + 149216);
      CHEM_PREFETCH(ws + 149248);
      CHEM_PREFETCH(ws + 149280);
      CHEM_PREFETCH(ws + 149312);
      CHEM_PREFETCH(ws + 149344);
      CHEM_PREFETCH(ws + 149376);
      CHEM_PREFETCH(ws + 149408);
      CHEM_PREFETCH(ws + 149440);
      CHEM_PREFETCH(ws + 149472);
      CHEM_PREFETCH(ws + 149504);
      CHEM_PREFETCH(ws + 149536);
      CHEM_PREFETCH(ws + 149568);
      CHEM_PREFETCH(ws + 149600);
      CHEM_PREFETCH(ws + 149632);
      CHEM_PREFETCH(ws + 149664);
      CHEM_PREFETCH(ws + 149696);
      CHEM_PREFETCH(ws + 149728);
      CHEM_PREFETCH(ws + 149760);
      CHEM_PREFETCH(ws + 149792);
      CHEM_PREFETCH(ws + 149824);
      CHEM_PREFETCH(ws + 149856);
      CHEM_PREFETCH(ws + 149888);
      CHEM_PREFETCH(ws + 149920);
      CHEM_PREFETCH(ws + 149952);
      CHEM_PREFETCH(ws + 149984);
      CHEM_PREFETCH(ws + 150016);
      CHEM_PREFETCH(ws + 150048);
      CHEM_PREFETCH(ws + 150080);
      CHEM_PREFETCH(ws + 150112);
      CHEM_PREFETCH(ws + 150144);
      CHEM_PREFETCH(ws + 150176);
      CHEM_PREFETCH(ws + 150208);
      CHEM_PREFETCH(ws + 150240);
      CHEM_PREFETCH(ws + 150272);
      CHEM_PREFETCH(ws + 150304);
      CHEM_PREFETCH(ws + 150336);
      CHEM_PREFETCH(ws + 150368);
      CHEM_PREFETCH(ws + 150400);
      CHEM_PREFETCH(ws + 150432);
      CHEM_PREFETCH(ws + 150464);
      CHEM_PREFETCH(ws + 150496);
      CHEM_PREFETCH(ws + 150528);
      CHEM_PREFETCH(ws + 150560);
      CHEM_PREFETCH(ws + 150592);
      CHEM_PREFETCH(ws + 150624);
      CHEM_PREFETCH(ws + 150656);
      CHEM_PREFETCH(ws + 150688);
      CHEM_PREFETCH(ws + 150720);
      CHEM_PREFETCH(ws + 150752);
      CHEM_PREFETCH(ws + 150784);
      CHEM_PREFETCH(ws + 150816);
      CHEM_PREFETCH(ws + 150848);
      CHEM_PREFETCH(ws + 150880);
      CHEM_PREFETCH(ws + 150912);
      CHEM_PREFETCH(ws + 150944);
      CHEM_PREFETCH(ws + 150976);
      CHEM_PREFETCH(ws + 151008);
      CHEM_PREFETCH(ws + 151040);
      CHEM_PREFETCH(ws + 151072);
      CHEM_PREFETCH(ws + 151104);
      CHEM_PREFETCH(ws + 151136);
      CHEM_PREFETCH(ws + 151168);
      CHEM_PREFETCH(ws + 151200);
      double x = b[5760];
      x = fma(-CHEM_LDLU(lu + 32704), b[448], x);
      x = fma(-CHEM_LDLU(lu + 32736), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 32768), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 32800), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 32832), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 32864), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 32896), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 32928), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 32960), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 32992), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 33024), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 33056), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 33088), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 33120), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 33152), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 33184), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 33216), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 33248), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 33280), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 33312), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 33344), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 33376), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 33408), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 33440), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 33472), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 33504), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 33536), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 33568), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 33600), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 33632), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 33664), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 33696), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 33728), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 33760), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 33792), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 33824), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 33856), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 33888), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 33920), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 33952), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 33984), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 34016), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 34048), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 34080), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 34112), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 34144), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 34176), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 34208), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 34240), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 34272), b[5728], x);
      b[5760] = x;
    }
    {
      CHEM_PREFETCH(ws + 151232);
      CHEM_PREFETCH(ws + 151264);
      CHEM_PREFETCH(ws + 151296);
      CHEM_PREFETCH(ws + 151328);
      CHEM_PREFETCH(ws + 151360);
      CHEM_PREFETCH(ws + 151392);
      CHEM_PREFETCH(ws + 151424);
      CHEM_PREFETCH(ws + 151456);
      CHEM_PREFETCH(ws + 151488);
      CHEM_PREFETCH(ws + 151520);
      CHEM_PREFETCH(ws + 151552);
      CHEM_PREFETCH(ws + 151584);
      CHEM_PREFETCH(ws + 151616);
      CHEM_PREFETCH(ws + 151648);
      CHEM_PREFETCH(ws + 151680);
      CHEM_PREFETCH(ws + 151712);
      CHEM_PREFETCH(ws + 151744);
      CHEM_PREFETCH(ws + 151776);
      CHEM_PREFETCH(ws + 151808);
      CHEM_PREFETCH(ws + 151840);
      CHEM_PREFETCH(ws + 151872);
      CHEM_PREFETCH(ws + 151904);
      CHEM_PREFETCH(ws + 151936);
      CHEM_PREFETCH(ws + 151968);
      CHEM_PREFETCH(ws + 152000);
      CHEM_PREFETCH(ws + 152032);
      CHEM_PREFETCH(ws + 152064);
      CHEM_PREFETCH(ws + 152096);
      CHEM_PREFETCH(ws + 152128);
      CHEM_PREFETCH(ws + 152160);
      CHEM_PREFETCH(ws + 152192);
      CHEM_PREFETCH(ws + 152224);
      CHEM_PREFETCH(ws + 152256);
      CHEM_PREFETCH(ws + 152288);
      CHEM_PREFETCH(ws + 152320);
      CHEM_PREFETCH(ws + 152352);
      CHEM_PREFETCH(ws + 152384);
      CHEM_PREFETCH(ws + 152416);
      CHEM_PREFETCH(ws + 152448);
      CHEM_PREFETCH(ws + 152480);
      CHEM_PREFETCH(ws + 152512);
      CHEM_PREFETCH(ws + 152544);
      CHEM_PREFETCH(ws + 152576);
      CHEM_PREFETCH(ws + 152608);
      CHEM_PREFETCH(ws + 152640);
      CHEM_PREFETCH(ws + 152672);
      CHEM_PREFETCH(ws + 152704);
      CHEM_PREFETCH(ws + 152736);
      CHEM_PREFETCH(ws + 152768);
      CHEM_PREFETCH(ws + 152800);
      CHEM_PREFETCH(ws + 152832);
      CHEM_PREFETCH(ws + 152864);
      CHEM_PREFETCH(ws + 152896);
      CHEM_PREFETCH(ws + 152928);
      CHEM_PREFETCH(ws + 152960);
      CHEM_PREFETCH(ws + 152992);
      CHEM_PREFETCH(ws + 153024);
      CHEM_PREFETCH(ws + 153056);
      CHEM_PREFETCH(ws + 153088);
      CHEM_PREFETCH(ws + 153120);
      CHEM_PREFETCH(ws + 153152);
      CHEM_PREFETCH(ws + 153184);
      CHEM_PREFETCH(ws + 153216);
      CHEM_PREFETCH(ws + 153248);
      CHEM_PREFETCH(ws + 153280);
      CHEM_PREFETCH(ws + 153312);
      CHEM_PREFETCH(ws + 153344);
      CHEM_PREFETCH(ws + 153376);
      CHEM_PREFETCH(ws + 153408);
      CHEM_PREFETCH(ws + 153440);
      CHEM_PREFETCH(ws + 153472);
      CHEM_PREFETCH(ws + 153504);
      CHEM_PREFETCH(ws + 153536);
      CHEM_PREFETCH(ws + 153568);
      CHEM_PREFETCH(ws + 153600);
      CHEM_PREFETCH(ws + 153632);
      CHEM_PREFETCH(ws + 153664);
      CHEM_PREFETCH(ws + 153696);
      CHEM_PREFETCH(ws + 153728);
      CHEM_PREFETCH(ws + 153760);
      CHEM_PREFETCH(ws + 153792);
      CHEM_PREFETCH(ws + 153824);
      CHEM_PREFETCH(ws + 153856);
      CHEM_PREFETCH(ws + 153888);
      CHEM_PREFETCH(ws + 153920);
      CHEM_PREFETCH(ws + 153952);
      CHEM_PREFETCH(ws + 153984);
      double x = b[5792];
      x = fma(-CHEM_LDLU(lu + 34304), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 34336), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 34368), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 34400), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 34432), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 34464), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 34496), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 34528), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 34560), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 34592), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 34624), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 34656), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 34688), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 34720), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 34752), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 34784), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 34816), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 34848), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 34880), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 34912), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 34944), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 34976), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 35008), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 35040), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 35072), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 35104), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 35136), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 35168), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 35200), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 35232), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 35264), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 35296), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 35328), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 35360), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 35392), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 35424), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 35456), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 35488), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 35520), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 35552), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 35584), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 35616), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 35648), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 35680), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 35712), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 35744), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 35776), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 35808), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 35840), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 35872), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 35904), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 35936), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 35968), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 36000), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 36032), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 36064), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 36096), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 36128), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 36160), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 36192), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 36224), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 36256), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 36288), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 36320), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 36352), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 36384), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 36416), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 36448), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 36480), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 36512), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 36544), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 36576), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 36608), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 36640), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 36672), b[5760], x);
      b[5792] = x;
    }
    {
      CHEM_PREFETCH(ws + 154016);
      CHEM_PREFETCH(ws + 154048);
      CHEM_PREFETCH(ws + 154080);
      CHEM_PREFETCH(ws + 154112);
      CHEM_PREFETCH(ws + 154144);
      CHEM_PREFETCH(ws + 154176);
      CHEM_PREFETCH(ws + 154208);
      CHEM_PREFETCH(ws + 154240);
      CHEM_PREFETCH(ws + 154272);
      CHEM_PREFETCH(ws + 154304);
      CHEM_PREFETCH(ws + 154336);
      CHEM_PREFETCH(ws + 154368);
      CHEM_PREFETCH(ws + 154400);
      CHEM_PREFETCH(ws + 154432);
      CHEM_PREFETCH(ws + 154464);
      CHEM_PREFETCH(ws + 154496);
      CHEM_PREFETCH(ws + 154528);
      CHEM_PREFETCH(ws + 154560);
      CHEM_PREFETCH(ws + 154592);
      CHEM_PREFETCH(ws + 154624);
      CHEM_PREFETCH(ws + 154656);
      CHEM_PREFETCH(ws + 154688);
      CHEM_PREFETCH(ws + 154720);
      CHEM_PREFETCH(ws + 154752);
      CHEM_PREFETCH(ws + 154784);
      CHEM_PREFETCH(ws + 154816);
      CHEM_PREFETCH(ws + 154848);
      CHEM_PREFETCH(ws + 154880);
      CHEM_PREFETCH(ws + 154912);
      CHEM_PREFETCH(ws + 154944);
      CHEM_PREFETCH(ws + 154976);
      CHEM_PREFETCH(ws + 155008);
      CHEM_PREFETCH(ws + 155040);
      CHEM_PREFETCH(ws + 155072);
      CHEM_PREFETCH(ws + 155104);
      CHEM_PREFETCH(ws + 155136);
      CHEM_PREFETCH(ws + 155168);
      CHEM_PREFETCH(ws + 155200);
      CHEM_PREFETCH(ws + 155232);
      CHEM_PREFETCH(ws + 155264);
      CHEM_PREFETCH(ws + 155296);
      CHEM_PREFETCH(ws + 155328);
      CHEM_PREFETCH(ws + 155360);
      CHEM_PREFETCH(ws + 155392);
      CHEM_PREFETCH(ws + 155424);
      CHEM_PREFETCH(ws + 155456);
      CHEM_PREFETCH(ws + 155488);
      CHEM_PREFETCH(ws + 155520);
      CHEM_PREFETCH(ws + 155552);
      CHEM_PREFETCH(ws + 155584);
      CHEM_PREFETCH(ws + 155616);
      CHEM_PREFETCH(ws + 155648);
      CHEM_PREFETCH(ws + 155680);
      CHEM_PREFETCH(ws + 155712);
      CHEM_PREFETCH(ws + 155744);
      CHEM_PREFETCH(ws + 155776);
      CHEM_PREFETCH(ws + 155808);
      CHEM_PREFETCH(ws + 155840);
      CHEM_PREFETCH(ws + 155872);
      CHEM_PREFETCH(ws + 155904);
      CHEM_PREFETCH(ws + 155936);
      CHEM_PREFETCH(ws + 155968);
      CHEM_PREFETCH(ws + 156000);
      CHEM_PREFETCH(ws + 156032);
      CHEM_PREFETCH(ws + 156064);
      CHEM_PREFETCH(ws + 156096);
      CHEM_PREFETCH(ws + 156128);
      CHEM_PREFETCH(ws + 156160);
      CHEM_PREFETCH(ws + 156192);
      CHEM_PREFETCH(ws + 156224);
      CHEM_PREFETCH(ws + 156256);
      CHEM_PREFETCH(ws + 156288);
      CHEM_PREFETCH(ws + 156320);
      CHEM_PREFETCH(ws + 156352);
      CHEM_PREFETCH(ws + 156384);
      CHEM_PREFETCH(ws + 156416);
      CHEM_PREFETCH(ws + 156448);
      CHEM_PREFETCH(ws + 156480);
      CHEM_PREFETCH(ws + 156512);
      CHEM_PREFETCH(ws + 156544);
      CHEM_PREFETCH(ws + 156576);
      CHEM_PREFETCH(ws + 156608);
      CHEM_PREFETCH(ws + 156640);
      CHEM_PREFETCH(ws + 156672);
      double x = b[5824];
      x = fma(-CHEM_LDLU(lu + 36704), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 36736), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 36768), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 36800), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 36832), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 36864), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 36896), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 36928), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 36960), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 36992), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 37024), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 37056), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 37088), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 37120), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 37152), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 37184), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 37216), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 37248), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 37280), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 37312), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 37344), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 37376), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 37408), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 37440), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 37472), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 37504), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 37536), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 37568), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 37600), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 37632), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 37664), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 37696), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 37728), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 37760), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 37792), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 37824), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 37856), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 37888), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 37920), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 37952), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 37984), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 38016), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 38048), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 38080), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 38112), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 38144), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 38176), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 38208), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 38240), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 38272), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 38304), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 38336), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 38368), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 38400), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 38432), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 38464), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 38496), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 38528), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 38560), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 38592), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 38624), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 38656), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 38688), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 38720), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 38752), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 38784), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 38816), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 38848), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 38880), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 38912), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 38944), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 38976), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 39008), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 39040), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 39072), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 39104), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 39136), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 39168), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 39200), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 39232), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 39264), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 39296), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 39328), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 39360), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 39392), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 39424), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 39456), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 39488), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 39520), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 39552), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 39584), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 39616), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 39648), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 39680), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 39712), b[5792], x);
      b[5824] = x;
    }
    {
      CHEM_PREFETCH(ws + 156704);
      CHEM_PREFETCH(ws + 156736);
      CHEM_PREFETCH(ws + 156768);
      CHEM_PREFETCH(ws + 156800);
      CHEM_PREFETCH(ws + 156832);
      CHEM_PREFETCH(ws + 156864);
      CHEM_PREFETCH(ws + 156896);
      CHEM_PREFETCH(ws + 156928);
      CHEM_PREFETCH(ws + 156960);
      CHEM_PREFETCH(ws + 156992);
      CHEM_PREFETCH(ws + 157024);
      CHEM_PREFETCH(ws + 157056);
      CHEM_PREFETCH(ws + 157088);
      CHEM_PREFETCH(ws + 157120);
      CHEM_PREFETCH(ws + 157152);
      CHEM_PREFETCH(ws + 157184);
      CHEM_PREFETCH(ws + 157216);
      CHEM_PREFETCH(ws + 157248);
      CHEM_PREFETCH(ws + 157280);
      CHEM_PREFETCH(ws + 157312);
      CHEM_PREFETCH(ws + 157344);
      CHEM_PREFETCH(ws + 157376);
      CHEM_PREFETCH(ws + 157408);
      CHEM_PREFETCH(ws + 157440);
      CHEM_PREFETCH(ws + 157472);
      CHEM_PREFETCH(ws + 157504);
      CHEM_PREFETCH(ws + 157536);
      CHEM_PREFETCH(ws + 157568);
      CHEM_PREFETCH(ws + 157600);
      CHEM_PREFETCH(ws + 157632);
      CHEM_PREFETCH(ws + 157664);
      CHEM_PREFETCH(ws + 157696);
      CHEM_PREFETCH(ws + 157728);
      CHEM_PREFETCH(ws + 157760);
      CHEM_PREFETCH(ws + 157792);
      CHEM_PREFETCH(ws + 157824);
      CHEM_PREFETCH(ws + 157856);
      CHEM_PREFETCH(ws + 157888);
      CHEM_PREFETCH(ws + 157920);
      CHEM_PREFETCH(ws + 157952);
      CHEM_PREFETCH(ws + 157984);
      CHEM_PREFETCH(ws + 158016);
      CHEM_PREFETCH(ws + 158048);
      CHEM_PREFETCH(ws + 158080);
      CHEM_PREFETCH(ws + 158112);
      CHEM_PREFETCH(ws + 158144);
      CHEM_PREFETCH(ws + 158176);
      CHEM_PREFETCH(ws + 158208);
      CHEM_PREFETCH(ws + 158240);
      CHEM_PREFETCH(ws + 158272);
      CHEM_PREFETCH(ws + 158304);
      CHEM_PREFETCH(ws + 158336);
      CHEM_PREFETCH(ws + 158368);
      CHEM_PREFETCH(ws + 158400);
      CHEM_PREFETCH(ws + 158432);
      CHEM_PREFETCH(ws + 158464);
      CHEM_PREFETCH(ws + 158496);
      CHEM_PREFETCH(ws + 158528);
      CHEM_PREFETCH(ws + 158560);
      CHEM_PREFETCH(ws + 158592);
      CHEM_PREFETCH(ws + 158624);
      CHEM_PREFETCH(ws + 158656);
      CHEM_PREFETCH(ws + 158688);
      CHEM_PREFETCH(ws + 158720);
      CHEM_PREFETCH(ws + 158752);
      CHEM_PREFETCH(ws + 158784);
      CHEM_PREFETCH(ws + 158816);
      CHEM_PREFETCH(ws + 158848);
      CHEM_PREFETCH(ws + 158880);
      CHEM_PREFETCH(ws + 158912);
      CHEM_PREFETCH(ws + 158944);
      CHEM_PREFETCH(ws + 158976);
      CHEM_PREFETCH(ws + 159008);
      CHEM_PREFETCH(ws + 159040);
      CHEM_PREFETCH(ws + 159072);
      CHEM_PREFETCH(ws + 159104);
      CHEM_PREFETCH(ws + 159136);
      CHEM_PREFETCH(ws + 159168);
      CHEM_PREFETCH(ws + 159200);
      CHEM_PREFETCH(ws + 159232);
      CHEM_PREFETCH(ws + 159264);
      CHEM_PREFETCH(ws + 159296);
      CHEM_PREFETCH(ws + 159328);
      CHEM_PREFETCH(ws + 159360);
      CHEM_PREFETCH(ws + 159392);
      CHEM_PREFETCH(ws + 159424);
      CHEM_PREFETCH(ws + 159456);
      CHEM_PREFETCH(ws + 159488);
      CHEM_PREFETCH(ws + 159520);
      CHEM_PREFETCH(ws + 159552);
      CHEM_PREFETCH(ws + 159584);
      CHEM_PREFETCH(ws + 159616);
      CHEM_PREFETCH(ws + 159648);
      CHEM_PREFETCH(ws + 159680);
      CHEM_PREFETCH(ws + 159712);
      CHEM_PREFETCH(ws + 159744);
      CHEM_PREFETCH(ws + 159776);
      CHEM_PREFETCH(ws + 159808);
      CHEM_PREFETCH(ws + 159840);
      CHEM_PREFETCH(ws + 159872);
      CHEM_PREFETCH(ws + 159904);
      CHEM_PREFETCH(ws + 159936);
      CHEM_PREFETCH(ws + 159968);
      CHEM_PREFETCH(ws + 160000);
      CHEM_PREFETCH(ws + 160032);
      CHEM_PREFETCH(ws + 160064);
      CHEM_PREFETCH(ws + 160096);
      CHEM_PREFETCH(ws + 160128);
      double x = b[5856];
      x = fma(-CHEM_LDLU(lu + 39744), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 39776), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 39808), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 39840), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 39872), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 39904), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 39936), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 39968), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 40000), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 40032), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 40064), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 40096), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 40128), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 40160), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 40192), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 40224), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 40256), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 40288), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 40320), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 40352), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 40384), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 40416), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 40448), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 40480), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 40512), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 40544), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 40576), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 40608), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 40640), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 40672), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 40704), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 40736), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 40768), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 40800), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 40832), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 40864), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 40896), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 40928), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 40960), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 40992), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 41024), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 41056), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 41088), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 41120), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 41152), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 41184), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 41216), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 41248), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 41280), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 41312), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 41344), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 41376), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 41408), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 41440), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 41472), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 41504), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 41536), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 41568), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 41600), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41632), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 41664), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 41696), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 41728), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 41760), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 41792), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 41824), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 41856), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 41888), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 41920), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 41952), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 41984), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 42016), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 42048), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 42080), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 42112), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 42144), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 42176), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 42208), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 42240), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 42272), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 42304), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 42336), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 42368), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 42400), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 42432), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 42464), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 42496), b[5824], x);
      b[5856] = x;
    }
}
__device__ __noinline__ void solve_1_2(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH(ws + 160160);
      CHEM_PREFETCH(ws + 160192);
      CHEM_PREFETCH(ws + 160224);
      CHEM_PREFETCH(ws + 160256);
      CHEM_PREFETCH(ws + 160288);
      CHEM_PREFETCH(ws + 160320);
      CHEM_PREFETCH(ws + 160352);
      CHEM_PREFETCH(ws + 160384);
      CHEM_PREFETCH(ws + 160416);
      CHEM_PREFETCH(ws + 160448);
      CHEM_PREFETCH(ws + 160480);
      CHEM_PREFETCH(ws + 160512);
      CHEM_PREFETCH(ws + 160544);
      CHEM_PREFETCH(ws + 160576);
      CHEM_PREFETCH(ws + 160608);
      CHEM_PREFETCH(ws + 160640);
      CHEM_PREFETCH(ws + 160672);
      CHEM_PREFETCH(ws + 160704);
      CHEM_PREFETCH(ws + 160736);
      CHEM_PREFETCH(ws + 160768);
      CHEM_PREFETCH(ws + 160800);
      CHEM_PREFETCH(ws + 160832);
      CHEM_PREFETCH(ws + 160864);
      CHEM_PREFETCH(ws + 160896);
      CHEM_PREFETCH(ws + 160928);
      CHEM_PREFETCH(ws + 160960);
      CHEM_PREFETCH(ws + 160992);
      CHEM_PREFETCH(ws + 161024);
      CHEM_PREFETCH(ws + 161056);
      CHEM_PREFETCH(ws + 161088);
      CHEM_PREFETCH(ws + 161120);
      CHEM_PREFETCH(ws + 161152);
      CHEM_PREFETCH(ws + 161184);
      CHEM_PREFETCH(ws + 161216);
      CHEM_PREFETCH(ws + 161248);
      CHEM_PREFETCH(ws + 161280);
      CHEM_PREFETCH(ws + 161312);
      CHEM_PREFETCH(ws + 161344);
      CHEM_PREFETCH(ws + 161376);
      CHEM_PREFETCH(ws + 161408);
      CHEM_PREFETCH(ws + 161440);
      CHEM_PREFETCH(ws + 161472);
      CHEM_PREFETCH(ws + 161504);
      CHEM_PREFETCH(ws + 161536);
      CHEM_PREFETCH(ws + 161568);
      CHEM_PREFETCH(ws + 161600);
      CHEM_PREFETCH(ws + 161632);
      CHEM_PREFETCH(ws + 161664);
      CHEM_PREFETCH(ws + 161696);
      CHEM_PREFETCH(ws + 161728);
      CHEM_PREFETCH(ws + 161760);
      CHEM_PREFETCH(ws + 161792);
      CHEM_PREFETCH(ws + 161824);
      CHEM_PREFETCH(ws + 161856);
      CHEM_PREFETCH(ws + 161888);
      CHEM_PREFETCH(ws + 161920);
      CHEM_PREFETCH(ws + 161952);
      CHEM_PREFETCH(ws + 161984);
      CHEM_PREFETCH(ws + 162016);
      CHEM_PREFETCH(ws + 162048);
      CHEM_PREFETCH(ws + 162080);
      CHEM_PREFETCH(ws + 162112);
      CHEM_PREFETCH(ws + 162144);
      CHEM_PREFETCH(ws + 162176);
      CHEM_PREFETCH(ws + 162208);
      CHEM_PREFETCH(ws + 162240);
      CHEM_PREFETCH(ws + 162272);
      CHEM_PREFETCH(ws + 162304);
      CHEM_PREFETCH(ws + 162336);
      CHEM_PREFETCH(ws + 162368);
      CHEM_PREFETCH(ws + 162400);
      CHEM_PREFETCH(ws + 162432);
      CHEM_PREFETCH(ws + 162464);
      CHEM_PREFETCH(ws + 162496);
      CHEM_PREFETCH(ws + 162528);
      CHEM_PREFETCH(ws + 162560);
      CHEM_PREFETCH(ws + 162592);
      CHEM_PREFETCH(ws + 162624);
      CHEM_PREFETCH(ws + 162656);
      CHEM_PREFETCH(ws + 162688);
      CHEM_PREFETCH(ws + 162720);
      CHEM_PREFETCH(ws + 162752);
      CHEM_PREFETCH(ws + 162784);
      CHEM_PREFETCH(ws + 162816);
      CHEM_PREFETCH(ws + 162848);
      CHEM_PREFETCH(ws + 162880);
      CHEM_PREFETCH(ws + 162912);
      CHEM_PREFETCH(ws + 162944);
      CHEM_PREFETCH(ws + 162976);
      CHEM_PREFETCH(ws + 163008);
      CHEM_PREFETCH(ws + 163040);
      CHEM_PREFETCH(ws + 163072);
      CHEM_PREFETCH(ws + 163104);
      CHEM_PREFETCH(ws + 163136);
      CHEM_PREFETCH(ws + 163168);
      CHEM_PREFETCH(ws + 163200);
      CHEM_PREFETCH(ws + 163232);
      CHEM_PREFETCH(ws + 163264);
      CHEM_PREFETCH(ws + 163296);
      CHEM_PREFETCH(ws + 163328);
      CHEM_PREFETCH(ws + 163360);
      CHEM_PREFETCH(ws + 163392);
      CHEM_PREFETCH(ws + 163424);
      CHEM_PREFETCH(ws + 163456);
      CHEM_PREFETCH(ws + 163488);
      CHEM_PREFETCH(ws + 163520);
      CHEM_PREFETCH(ws + 163552);
      CHEM_PREFETCH(ws + 163584);
      CHEM_PREFETCH(ws + 163616);
      CHEM_PREFETCH(ws + 163648);
      CHEM_PREFETCH(ws + 163680);
      CHEM_PREFETCH(ws + 163712);
      CHEM_PREFETCH(ws + 163744);
      double x = b[5888];
      x = fma(-CHEM_LDLU(lu + 42528), b[928], x);
      x = fma(-CHEM_LDLU(lu + 42560), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 42592), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 42624), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 42656), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 42688), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 42720), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 42752), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 42784), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 42816), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 42848), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 42880), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 42912), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 42944), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 42976), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 43008), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 43040), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 43072), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 43104), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 43136), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 43168), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 43200), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 43232), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 43264), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 43296), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 43328), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 43360), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 43392), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 43424), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 43456), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 43488), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 43520), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 43552), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 43584), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 43616), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 43648), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 43680), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 43712), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 43744), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 43776), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 43808), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 43840), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 43872), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 43904), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 43936), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 43968), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 44000), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 44032), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 44064), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 44096), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 44128), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 44160), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 44192), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 44224), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 44256), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 44288), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 44320), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 44352), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 44384), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 44416), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 44448), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 44480), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 44512), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 44544), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 44576), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 44608), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 44640), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 44672), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 44704), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 44736), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 44768), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 44800), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 44832), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 44864), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 44896), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 44928), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 44960), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 44992), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 45024), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 45056), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 45088), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 45120), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 45152), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 45184), b[5824], x);
      b[5888] = x;
    }
    {
      CHEM_PREFETCH(ws + 163776);
      CHEM_PREFETCH(ws + 163808);
      CHEM_PREFETCH(ws + 163840);
      CHEM_PREFETCH(ws + 163872);
      CHEM_PREFETCH(ws + 163904);
      CHEM_PREFETCH(ws + 163936);
      CHEM_PREFETCH(ws + 163968);
      CHEM_PREFETCH(ws + 164000);
      CHEM_PREFETCH(ws + 164032);
      CHEM_PREFETCH(ws + 164064);
      CHEM_PREFETCH(ws + 164096);
      CHEM_PREFETCH(ws + 164128);
      CHEM_PREFETCH(ws + 164160);
      CHEM_PREFETCH(ws + 164192);
      CHEM_PREFETCH(ws + 164224);
      CHEM_PREFETCH(ws + 164256);
      CHEM_PREFETCH(ws + 164288);
      CHEM_PREFETCH(ws + 164320);
      CHEM_PREFETCH(ws + 164352);
      CHEM_PREFETCH(ws + 164384);
      CHEM_PREFETCH(ws + 164416);
      CHEM_PREFETCH(ws + 164448);
      CHEM_PREFETCH(ws + 164480);
      CHEM_PREFETCH(ws + 164512);
      CHEM_PREFETCH(ws + 164544);
      CHEM_PREFETCH(ws + 164576);
      CHEM_PREFETCH(ws + 164608);
      CHEM_PREFETCH(ws + 164640);
      CHEM_PREFETCH(ws + 164672);
      CHEM_PREFETCH(ws + 164704);
      CHEM_PREFETCH(ws + 164736);
      CHEM_PREFETCH(ws + 164768);
      CHEM_PREFETCH(ws + 164800);
      CHEM_PREFETCH(ws + 164832);
      CHEM_PREFETCH(ws + 164864);
      CHEM_PREFETCH(ws + 164896);
      CHEM_PREFETCH(ws + 164928);
      CHEM_PREFETCH(ws + 164960);
      CHEM_PREFETCH(ws + 164992);
      CHEM_PREFETCH(ws + 165024);
      CHEM_PREFETCH(ws + 165056);
      CHEM_PREFETCH(ws + 165088);
      CHEM_PREFETCH(ws + 165120);
      CHEM_PREFETCH(ws + 165152);
      CHEM_PREFETCH(ws + 165184);
      CHEM_PREFETCH(ws + 165216);
      CHEM_PREFETCH(ws + 165248);
      CHEM_PREFETCH(ws + 165280);
      CHEM_PREFETCH(ws + 165312);
      CHEM_PREFETCH(ws + 165344);
      CHEM_PREFETCH(ws + 165376);
      CHEM_PREFETCH(ws + 165408);
      CHEM_PREFETCH(ws + 165440);
      CHEM_PREFETCH(ws + 165472);
      CHEM_PREFETCH(ws + 165504);
      CHEM_PREFETCH(ws + 165536);
      CHEM_PREFETCH(ws + 165568);
      CHEM_PREFETCH(ws + 165600);
      CHEM_PREFETCH(ws + 165632);
      CHEM_PREFETCH(ws + 165664);
      CHEM_PREFETCH(ws + 165696);
      CHEM_PREFETCH(ws + 165728);
      CHEM_PREFETCH(ws + 165760);
      CHEM_PREFETCH(ws + 165792);
      CHEM_PREFETCH(ws + 165824);
      CHEM_PREFETCH(ws + 165856);
      CHEM_PREFETCH(ws + 165888);
      CHEM_PREFETCH(ws + 165920);
      CHEM_PREFETCH(ws + 165952);
      CHEM_PREFETCH(ws + 165984);
      CHEM_PREFETCH(ws + 166016);
      CHEM_PREFETCH(ws + 166048);
      CHEM_PREFETCH(ws + 166080);
      CHEM_PREFETCH(ws + 166112);
      CHEM_PREFETCH(ws + 166144);
      CHEM_PREFETCH(ws + 166176);
      CHEM_PREFETCH(ws + 166208);
      CHEM_PREFETCH(ws + 166240);
      CHEM_PREFETCH(ws + 166272);
      CHEM_PREFETCH(ws + 166304);
      CHEM_PREFETCH(ws + 166336);
      CHEM_PREFETCH(ws + 166368);
      CHEM_PREFETCH(ws + 166400);
      CHEM_PREFETCH(ws + 166432);
      CHEM_PREFETCH(ws + 166464);
      CHEM_PREFETCH(ws + 166496);
      CHEM_PREFETCH(ws + 166528);
      CHEM_PREFETCH(ws + 166560);
      CHEM_PREFETCH(ws + 166592);
      CHEM_PREFETCH(ws + 166624);
      CHEM_PREFETCH(ws + 166656);
      CHEM_PREFETCH(ws + 166688);
      CHEM_PREFETCH(ws + 166720);
      CHEM_PREFETCH(ws + 166752);
      CHEM_PREFETCH(ws + 166784);
      CHEM_PREFETCH(ws + 166816);
      CHEM_PREFETCH(ws + 166848);
      CHEM_PREFETCH(ws + 166880);
      CHEM_PREFETCH(ws + 166912);
      CHEM_PREFETCH(ws + 166944);
      CHEM_PREFETCH(ws + 166976);
      CHEM_PREFETCH(ws + 167008);
      CHEM_PREFETCH(ws + 167040);
      CHEM_PREFETCH(ws + 167072);
      CHEM_PREFETCH(ws + 167104);
      CHEM_PREFETCH(ws + 167136);
      CHEM_PREFETCH(ws + 167168);
      CHEM_PREFETCH(ws + 167200);
      CHEM_PREFETCH(ws + 167232);
      CHEM_PREFETCH(ws + 167264);
      CHEM_PREFETCH(ws + 167296);
      CHEM_PREFETCH(ws + 167328);
      CHEM_PREFETCH(ws + 167360);
      CHEM_PREFETCH(ws + 167392);
      CHEM_PREFETCH(ws + 167424);
      CHEM_PREFETCH(ws + 167456);
      CHEM_PREFETCH(ws + 167488);
      CHEM_PREFETCH(ws + 167520);
      CHEM_PREFETCH(ws + 167552);
      CHEM_PREFETCH(ws + 167584);
      CHEM_PREFETCH(ws + 167616);
      CHEM_PREFETCH(ws + 167648);
      CHEM_PREFETCH(ws + 167680);
      CHEM_PREFETCH(ws + 167712);
      CHEM_PREFETCH(ws + 167744);
      CHEM_PREFETCH(ws + 167776);
      CHEM_PREFETCH(ws + 167808);
      CHEM_PREFETCH(ws + 167840);
      CHEM_PREFETCH(ws + 167872);
      CHEM_PREFETCH(ws + 167904);
      CHEM_PREFETCH(ws + 167936);
      CHEM_PREFETCH(ws + 167968);
      CHEM_PREFETCH(ws + 168000);
      double x = b[5920];
      x = fma(-CHEM_LDLU(lu + 45216), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 45248), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 45280), b[1184], x);
      x = fma(-CHEM_LDLU(lu + 45312), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 45344), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 45376), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 45408), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 45440), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 45472), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 45504), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 45536), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 45568), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 45600), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 45632), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 45664), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 45696), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 45728), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 45760), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 45792), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 45824), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 45856), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 45888), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 45920), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 45952), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 45984), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 46016), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 46048), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 46080), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 46112), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 46144), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 46176), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 46208), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 46240), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 46272), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 46304), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 46336), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 46368), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 46400), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 46432), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 46464), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 46496), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 46528), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 46560), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 46592), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 46624), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 46656), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 46688), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 46720), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 46752), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 46784), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 46816), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 46848), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 46880), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 46912), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 46944), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 46976), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 47008), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 47040), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 47072), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 47104), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 47136), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 47168), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 47200), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 47232), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 47264), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 47296), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 47328), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 47360), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 47392), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 47424), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 47456), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 47488), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 47520), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 47552), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 47584), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 47616), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 47648), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 47680), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 47712), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 47744), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 47776), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 47808), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 47840), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 47872), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 47904), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 47936), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 47968), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 48000), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 48032), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 48064), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 48096), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 48128), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 48160), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 48192), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 48224), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 48256), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 48288), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 48320), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 48352), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 48384), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 48416), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 48448), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 48480), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 48512), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 48544), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 48576), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 48608), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 48640), b[5888], x);
      b[5920] = x;
    }
    {
      CHEM_PREFETCH(ws + 168032);
      CHEM_PREFETCH(ws + 168064);
      CHEM_PREFETCH(ws + 168096);
      CHEM_PREFETCH(ws + 168128);
      CHEM_PREFETCH(ws + 168160);
      CHEM_PREFETCH(ws + 168192);
      CHEM_PREFETCH(ws + 168224);
      CHEM_PREFETCH(ws + 168256);
      CHEM_PREFETCH(ws + 168288);
      CHEM_PREFETCH(ws + 168320);
      CHEM_PREFETCH(ws + 168352);
      CHEM_PREFETCH(ws + 168384);
      CHEM_PREFETCH(ws + 168416);
      CHEM_PREFETCH(ws + 168448);
      CHEM_PREFETCH(ws + 168480);
      CHEM_PREFETCH(ws + 168512);
      CHEM_PREFETCH(ws + 168544);
      CHEM_PREFETCH(ws + 168576);
      CHEM_PREFETCH(ws + 168608);
      CHEM_PREFETCH(ws + 168640);
      CHEM_PREFETCH(ws + 168672);
      CHEM_PREFETCH(ws + 168704);
      CHEM_PREFETCH(ws + 168736);
      CHEM_PREFETCH(ws + 168768);
      CHEM_PREFETCH(ws + 168800);
      CHEM_PREFETCH(ws + 168832);
      CHEM_PREFETCH(ws + 168864);
      CHEM_PREFETCH(ws + 168896);
      CHEM_PREFETCH(ws + 168928);
      CHEM_PREFETCH(ws + 168960);
      CHEM_PREFETCH(ws + 168992);
      CHEM_PREFETCH(ws + 169024);
      CHEM_PREFETCH(ws + 169056);
      CHEM_PREFETCH(ws + 169088);
      CHEM_PREFETCH(ws + 169120);
      CHEM_PREFETCH(ws + 169152);
      CHEM_PREFETCH(ws + 169184);
      CHEM_PREFETCH(ws + 169216);
      CHEM_PREFETCH(ws + 169248);
      CHEM_PREFETCH(ws + 169280);
      CHEM_PREFETCH(ws + 169312);
      CHEM_PREFETCH(ws + 169344);
      CHEM_PREFETCH(ws + 169376);
      CHEM_PREFETCH(ws + 169408);
      CHEM_PREFETCH(ws + 169440);
      CHEM_PREFETCH(ws + 169472);
      CHEM_PREFETCH(ws + 169504);
      CHEM_PREFETCH(ws + 169536);
      CHEM_PREFETCH(ws + 169568);
      CHEM_PREFETCH(ws + 169600);
      CHEM_PREFETCH(ws + 169632);
      CHEM_PREFETCH(ws + 169664);
      CHEM_PREFETCH(ws + 169696);
      CHEM_PREFETCH(ws + 169728);
      CHEM_PREFETCH(ws + 169760);
      CHEM_PREFETCH(ws + 169792);
      CHEM_PREFETCH(ws + 169824);
      CHEM_PREFETCH(ws + 169856);
      CHEM_PREFETCH(ws + 169888);
      CHEM_PREFETCH(ws + 169920);
      CHEM_PREFETCH(ws + 169952);
      CHEM_PREFETCH(ws + 169984);
      CHEM_PREFETCH(ws + 170016);
      CHEM_PREFETCH(ws + 170048);
      CHEM_PREFETCH(ws + 170080);
      CHEM_PREFETCH(ws + 170112);
      CHEM_PREFETCH(ws + 170144);
      CHEM_PREFETCH(ws + 170176);
      CHEM_PREFETCH(ws + 170208);
      CHEM_PREFETCH(ws + 170240);
      CHEM_PREFETCH(ws + 170272);
      CHEM_PREFETCH(ws + 170304);
      CHEM_PREFETCH(ws + 170336);
      CHEM_PREFETCH(ws + 170368);
      CHEM_PREFETCH(ws + 170400);
      CHEM_PREFETCH(ws + 170432);
      CHEM_PREFETCH(ws + 170464);
      CHEM_PREFETCH(ws + 170496);
      CHEM_PREFETCH(ws + 170528);
      CHEM_PREFETCH(ws + 170560);
      CHEM_PREFETCH(ws + 170592);
      CHEM_PREFETCH(ws + 170624);
      CHEM_PREFETCH(ws + 170656);
      CHEM_PREFETCH(ws + 170688);
      CHEM_PREFETCH(ws + 170720);
      CHEM_PREFETCH(ws + 170752);
      CHEM_PREFETCH(ws + 170784);
      CHEM_PREFETCH(ws + 170816);
      CHEM_PREFETCH(ws + 170848);
      CHEM_PREFETCH(ws + 170880);
      CHEM_PREFETCH(ws + 170912);
      CHEM_PREFETCH(ws + 170944);
      CHEM_PREFETCH(ws + 170976);
      CHEM_PREFETCH(ws + 171008);
      CHEM_PREFETCH(ws + 171040);
      CHEM_PREFETCH(ws + 171072);
      CHEM_PREFETCH(ws + 171104);
      CHEM_PREFETCH(ws + 171136);
      CHEM_PREFETCH(ws + 171168);
      CHEM_PREFETCH(ws + 171200);
      CHEM_PREFETCH(ws + 171232);
      CHEM_PREFETCH(ws + 171264);
      CHEM_PREFETCH(ws + 171296);
      CHEM_PREFETCH(ws + 171328);
      CHEM_PREFETCH(ws + 171360);
      CHEM_PREFETCH(ws + 171392);
      CHEM_PREFETCH(ws + 171424);
      CHEM_PREFETCH(ws + 171456);
      CHEM_PREFETCH(ws + 171488);
      CHEM_PREFETCH(ws + 171520);
      CHEM_PREFETCH(ws + 171552);
      CHEM_PREFETCH(ws + 171584);
      CHEM_PREFETCH(ws + 171616);
      CHEM_PREFETCH(ws + 171648);
      CHEM_PREFETCH(ws + 171680);
      CHEM_PREFETCH(ws + 171712);
      CHEM_PREFETCH(ws + 171744);
      CHEM_PREFETCH(ws + 171776);
      CHEM_PREFETCH(ws + 171808);
      CHEM_PREFETCH(ws + 171840);
      CHEM_PREFETCH(ws + 171872);
      CHEM_PREFETCH(ws + 171904);
      CHEM_PREFETCH(ws + 171936);
      CHEM_PREFETCH(ws + 171968);
      CHEM_PREFETCH(ws + 172000);
      CHEM_PREFETCH(ws + 172032);
      CHEM_PREFETCH(ws + 172064);
      CHEM_PREFETCH(ws + 172096);
      CHEM_PREFETCH(ws + 172128);
      CHEM_PREFETCH(ws + 172160);
      CHEM_PREFETCH(ws + 172192);
      CHEM_PREFETCH(ws + 172224);
      double x = b[5952];
      x = fma(-CHEM_LDLU(lu + 48672), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 48704), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 48736), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 48768), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 48800), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 48832), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 48864), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 48896), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 48928), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 48960), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 48992), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 49024), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 49056), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 49088), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 49120), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 49152), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 49184), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 49216), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 49248), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 49280), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 49312), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 49344), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 49376), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 49408), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 49440), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 49472), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 49504), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 49536), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 49568), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 49600), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 49632), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 49664), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 49696), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 49728), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 49760), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 49792), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 49824), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 49856), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 49888), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 49920), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 49952), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 49984), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 50016), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 50048), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 50080), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 50112), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 50144), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 50176), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 50208), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 50240), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 50272), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 50304), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 50336), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 50368), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 50400), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 50432), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 50464), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 50496), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 50528), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 50560), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 50592), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 50624), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 50656), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 50688), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 50720), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 50752), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 50784), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 50816), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 50848), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 50880), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 50912), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 50944), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 50976), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 51008), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 51040), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 51072), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 51104), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 51136), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 51168), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 51200), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 51232), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 51264), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 51296), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 51328), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 51360), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 51392), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 51424), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 51456), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 51488), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 51520), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 51552), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 51584), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 51616), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 51648), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 51680), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 51712), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 51744), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 51776), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 51808), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 51840), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 51872), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 51904), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 51936), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 51968), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 52000), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 52032), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 52064), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 52096), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 52128), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 52160), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 52192), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 52224), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 52256), b[5920], x);
      b[5952] = x;
    }
    {
      CHEM_PREFETCH(ws + 222624);
      double x = b[5984];
      x = fma(-CHEM_LDLU(lu + 52288), b[160], x);
      x = fma(-CHEM_LDLU(lu + 52320), b[256], x);
      x = fma(-CHEM_LDLU(lu + 52352), b[288], x);
      x = fma(-CHEM_LDLU(lu + 52384), b[320], x);
      x = fma(-CHEM_LDLU(lu + 52416), b[352], x);
      x = fma(-CHEM_LDLU(lu + 52448), b[448], x);
      x = fma(-CHEM_LDLU(lu + 52480), b[832], x);
      x = fma(-CHEM_LDLU(lu + 52512), b[864], x);
      x = fma(-CHEM_LDLU(lu + 52544), b[896], x);
      x = fma(-CHEM_LDLU(lu + 52576), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 52608), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 52640), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 52672), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 52704), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 52736), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 52768), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 52800), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 52832), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 52864), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 52896), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 52928), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 52960), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 52992), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 53024), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 53056), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 53088), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 53120), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 53152), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 53184), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 53216), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 53248), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 53280), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 53312), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 53344), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 53376), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 53408), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 53440), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 53472), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 53504), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 53536), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 53568), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 53600), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 53632), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 53664), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 53696), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 53728), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 53760), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 53792), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 53824), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 53856), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 53888), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 53920), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 53952), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 53984), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 54016), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 54048), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 54080), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 54112), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 54144), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 54176), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 54208), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 54240), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 54272), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 54304), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 54336), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 54368), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 54400), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 54432), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 54464), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 54496), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 54528), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 54560), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 54592), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 54624), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 54656), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 54688), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 54720), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 54752), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 54784), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 54816), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 54848), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 54880), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 54912), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 54944), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 54976), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 55008), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 55040), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 55072), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 55104), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 55136), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 55168), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 55200), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 55232), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 55264), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 55296), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 55328), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 55360), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 55392), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 55424), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 55456), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 55488), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 55520), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 55552), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 55584), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 55616), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 55648), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 55680), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 55712), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 55744), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 55776), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 55808), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 55840), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 55872), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 55904), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 55936), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 55968), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 56000), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 56032), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 56064), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 56096), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 56128), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 56160), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 56192), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 56224), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 56256), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 56288), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 56320), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 56352), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 56384), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 56416), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 56448), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 56480), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 56512), b[5952], x);
      b[5984] = x;
    }
    {
      CHEM_PREFETCH(ws + 172256);
      CHEM_PREFETCH(ws + 222592);
      double x = b[6016];
      x = fma(-CHEM_LDLU(lu + 56544), b[160], x);
      x = fma(-CHEM_LDLU(lu + 56576), b[256], x);
      x = fma(-CHEM_LDLU(lu + 56608), b[288], x);
      x = fma(-CHEM_LDLU(lu + 56640), b[320], x);
      x = fma(-CHEM_LDLU(lu + 56672), b[352], x);
      x = fma(-CHEM_LDLU(lu + 56704), b[384], x);
      x = fma(-CHEM_LDLU(lu + 56736), b[416], x);
      x = fma(-CHEM_LDLU(lu + 56768), b[448], x);
      x = fma(-CHEM_LDLU(lu + 56800), b[576], x);
      x = fma(-CHEM_LDLU(lu + 56832), b[608], x);
      x = fma(-CHEM_LDLU(lu + 56864), b[640], x);
      x = fma(-CHEM_LDLU(lu + 56896), b[672], x);
      x = fma(-CHEM_LDLU(lu + 56928), b[704], x);
      x = fma(-CHEM_LDLU(lu + 56960), b[736], x);
      x = fma(-CHEM_LDLU(lu + 56992), b[768], x);
      x = fma(-CHEM_LDLU(lu + 57024), b[800], x);
      x = fma(-CHEM_LDLU(lu + 57056), b[832], x);
      x = fma(-CHEM_LDLU(lu + 57088), b[864], x);
      x = fma(-CHEM_LDLU(lu + 57120), b[896], x);
      x = fma(-CHEM_LDLU(lu + 57152), b[928], x);
      x = fma(-CHEM_LDLU(lu + 57184), b[992], x);
      x = fma(-CHEM_LDLU(lu + 57216), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 57248), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 57280), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 57312), b[1184], x);
      x = fma(-CHEM_LDLU(lu + 57344), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 57376), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 57408), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 57440), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 57472), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 57504), b[1376], x);
      x = fma(-CHEM_LDLU(lu + 57536), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 57568), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 57600), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 57632), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 57664), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 57696), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 57728), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 57760), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 57792), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 57824), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 57856), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 57888), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 57920), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 57952), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 57984), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 58016), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 58048), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 58080), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 58112), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 58144), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 58176), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 58208), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 58240), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 58272), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 58304), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 58336), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 58368), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 58400), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 58432), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 58464), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 58496), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 58528), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 58560), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 58592), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 58624), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 58656), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 58688), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 58720), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 58752), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 58784), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 58816), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 58848), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 58880), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 58912), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 58944), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 58976), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 59008), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 59040), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 59072), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 59104), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 59136), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 59168), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 59200), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 59232), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 59264), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 59296), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 59328), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 59360), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 59392), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 59424), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 59456), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 59488), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 59520), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 59552), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 59584), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 59616), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 59648), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 59680), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 59712), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 59744), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 59776), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 59808), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 59840), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 59872), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 59904), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 59936), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 59968), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 60000), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 60032), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 60064), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 60096), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 60128), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 60160), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 60192), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 60224), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 60256), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 60288), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 60320), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 60352), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 60384), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 60416), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 60448), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 60480), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 60512), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 60544), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 60576), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 60608), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 60640), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 60672), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 60704), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 60736), b[5984], x);
      b[6016] = x;
    }
    {
      CHEM_PREFETCH(ws + 172288);
      CHEM_PREFETCH(ws + 172320);
      CHEM_PREFETCH(ws + 222560);
      double x = b[6016];
      b[6016] = x * CHEM_LDLU(vd + 6016);
    }
    {
      CHEM_PREFETCH(ws + 172352);
      CHEM_PREFETCH(ws + 172384);
      CHEM_PREFETCH(ws + 172416);
      CHEM_PREFETCH(ws + 222528);
      double x = b[5984];
      x = fma(-CHEM_LDLU(lu + 60768), b[6016], x);
      b[5984] = x * CHEM_LDLU(vd + 5984);
    }
    {
      CHEM_PREFETCH(ws + 172448);
      CHEM_PREFETCH(ws + 172480);
      CHEM_PREFETCH(ws + 172512);
      CHEM_PREFETCH(ws + 172544);
      CHEM_PREFETCH(ws + 222496);
      double x = b[5952];
      x = fma(-CHEM_LDLU(lu + 60800), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60832), b[6016], x);
      b[5952] = x * CHEM_LDLU(vd + 5952);
    }
    {
      CHEM_PREFETCH(ws + 172576);
      CHEM_PREFETCH(ws + 172608);
      CHEM_PREFETCH(ws + 172640);
      CHEM_PREFETCH(ws + 172672);
      CHEM_PREFETCH(ws + 172704);
      CHEM_PREFETCH(ws + 222464);
      double x = b[5920];
      x = fma(-CHEM_LDLU(lu + 60864), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 60896), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60928), b[6016], x);
      b[5920] = x * CHEM_LDLU(vd + 5920);
    }
    {
      CHEM_PREFETCH(ws + 172736);
      CHEM_PREFETCH(ws + 172768);
      CHEM_PREFETCH(ws + 172800);
      CHEM_PREFETCH(ws + 172832);
      CHEM_PREFETCH(ws + 172864);
      CHEM_PREFETCH(ws + 222432);
      double x = b[5888];
      x = fma(-CHEM_LDLU(lu + 60960), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 60992), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 61024), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 61056), b[6016], x);
      b[5888] = x * CHEM_LDLU(vd + 5888);
    }
    {
      CHEM_PREFETCH(ws + 172896);
      CHEM_PREFETCH(ws + 172928);
      CHEM_PREFETCH(ws + 172960);
      CHEM_PREFETCH(ws + 172992);
      CHEM_PREFETCH(ws + 173024);
      CHEM_PREFETCH(ws + 173056);
      CHEM_PREFETCH(ws + 222400);
      double x = b[5856];
      x = fma(-CHEM_LDLU(lu + 61088), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 61120), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 61152), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 61184), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 61216), b[6016], x);
      b[5856] = x * CHEM_LDLU(vd + 5856);
    }
    {
      CHEM_PREFETCH(ws + 173088);
      CHEM_PREFETCH(ws + 173120);
      CHEM_PREFETCH(ws + 173152);
      CHEM_PREFETCH(ws + 173184);
      CHEM_PREFETCH(ws + 173216);
      CHEM_PREFETCH(ws + 173248);
      CHEM_PREFETCH(ws + 173280);
      CHEM_PREFETCH(ws + 222368);
      double x = b[5824];
      x = fma(-CHEM_LDLU(lu + 61248), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 61280), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 61312), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 61344), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 61376), b[6016], x);
      b[5824] = x * CHEM_LDLU(vd + 5824);
    }
    {
      CHEM_PREFETCH(ws + 173312);
      CHEM_PREFETCH(ws + 173344);
      CHEM_PREFETCH(ws + 173376);
      CHEM_PREFETCH(ws + 173408);
      CHEM_PREFETCH(ws + 173440);
      CHEM_PREFETCH(ws + 173472);
      CHEM_PREFETCH(ws + 173504);
      CHEM_PREFETCH(ws + 173536);
      CHEM_PREFETCH(ws + 222336);
      double x = b[5792];
      x = fma(-CHEM_LDLU(lu + 61408), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61440), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 61472), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 61504), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 61536), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 61568), b[6016], x);
      b[5792] = x * CHEM_LDLU(vd + 5792);
    }
    {
      CHEM_PREFETCH(ws + 173568);
      CHEM_PREFETCH(ws + 173600);
      CHEM_PREFETCH(ws + 173632);
      CHEM_PREFETCH(ws + 173664);
      CHEM_PREFETCH(ws + 173696);
      CHEM_PREFETCH(ws + 173728);
      CHEM_PREFETCH(ws + 173760);
      CHEM_PREFETCH(ws + 173792);
      CHEM_PREFETCH(ws + 173824);
      CHEM_PREFETCH(ws + 222304);
      double x = b[5760];
      x = fma(-CHEM_LDLU(lu + 61600), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61632), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61664), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 61696), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 61728), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 61760), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 61792), b[6016], x);
      b[5760] = x * CHEM_LDLU(vd + 5760);
    }
    {
      CHEM_PREFETCH(ws + 173856);
      CHEM_PREFETCH(ws + 173888);
      CHEM_PREFETCH(ws + 173920);
      CHEM_PREFETCH(ws + 173952);
      CHEM_PREFETCH(ws + 173984);
      CHEM_PREFETCH(ws + 174016);
      CHEM_PREFETCH(ws + 174048);
      CHEM_PREFETCH(ws + 174080);
      CHEM_PREFETCH(ws + 174112);
      CHEM_PREFETCH(ws + 174144);
      CHEM_PREFETCH(ws + 222272);
      double x = b[5728];
      x = fma(-CHEM_LDLU(lu + 61824), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61856), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61888), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61920), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 61952), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 61984), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 62016), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 62048), b[6016], x);
      b[5728] = x * CHEM_LDLU(vd + 5728);
    }
    {
      CHEM_PREFETCH(ws + 174176);
      CHEM_PREFETCH(ws + 174208);
      CHEM_PREFETCH(ws + 174240);
      CHEM_PREFETCH(ws + 174272);
      CHEM_PREFETCH(ws + 174304);
      CHEM_PREFETCH(ws + 174336);
      CHEM_PREFETCH(ws + 174368);
      CHEM_PREFETCH(ws + 174400);
      CHEM_PREFETCH(ws + 174432);
      CHEM_PREFETCH(ws + 222240);
      double x = b[5696];
      x = fma(-CHEM_LDLU(lu + 62080), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 62112), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 62144), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 62176), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 62208), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 62240), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 62272), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 62304), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 62336), b[6016], x);
      b[5696] = x * CHEM_LDLU(vd + 5696);
    }
    {
      CHEM_PREFETCH(ws + 174464);
      CHEM_PREFETCH(ws + 174496);
      CHEM_PREFETCH(ws + 174528);
      CHEM_PREFETCH(ws + 174560);
      CHEM_PREFETCH(ws + 174592);
      CHEM_PREFETCH(ws + 174624);
      CHEM_PREFETCH(ws + 174656);
      CHEM_PREFETCH(ws + 174688);
      CHEM_PREFETCH(ws + 174720);
      CHEM_PREFETCH(ws + 222208);
      double x = b[5664];
      x = fma(-CHEM_LDLU(lu + 62368), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 62400), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 62432), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 62464), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 62496), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 62528), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 62560), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 62592), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 62624), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 62656), b[6016], x);
      b[5664] = x * CHEM_LDLU(vd + 5664);
    }
    {
      CHEM_PREFETCH(ws + 174752);
      CHEM_PREFETCH(ws + 174784);
      CHEM_PREFETCH(ws + 174816);
      CHEM_PREFETCH(ws + 174848);
      CHEM_PREFETCH(ws + 174880);
      CHEM_PREFETCH(ws + 174912);
      CHEM_PREFETCH(ws + 174944);
      CHEM_PREFETCH(ws + 174976);
      CHEM_PREFETCH(ws + 175008);
      CHEM_PREFETCH(ws + 222176);
      double x = b[5632];
      x = fma(-CHEM_LDLU(lu + 62688), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 62720), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 62752), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 62784), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 62816), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 62848), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 62880), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 62912), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 62944), b[6016], x);
      b[5632] = x * CHEM_LDLU(vd + 5632);
    }
    {
      CHEM_PREFETCH(ws + 175040);
      CHEM_PREFETCH(ws + 175072);
      CHEM_PREFETCH(ws + 175104);
      CHEM_PREFETCH(ws + 175136);
      CHEM_PREFETCH(ws + 175168);
      CHEM_PREFETCH(ws + 175200);
      CHEM_PREFETCH(ws + 175232);
      CHEM_PREFETCH(ws + 175264);
      CHEM_PREFETCH(ws + 222144);
      double x = b[5600];
      x = fma(-CHEM_LDLU(lu + 62976), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 63008), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 63040), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 63072), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 63104), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 63136), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 63168), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 63200), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 63232), b[6016], x);
      b[5600] = x * CHEM_LDLU(vd + 5600);
    }
    {
      CHEM_PREFETCH(ws + 175296);
      CHEM_PREFETCH(ws + 175328);
      CHEM_PREFETCH(ws + 175360);
      CHEM_PREFETCH(ws + 175392);
      CHEM_PREFETCH(ws + 175424);
      CHEM_PREFETCH(ws + 175456);
      CHEM_PREFETCH(ws + 175488);
      CHEM_PREFETCH(ws + 175520);
      CHEM_PREFETCH(ws + 175552);
      CHEM_PREFETCH(ws + 222112);
      double x = b[5568];
      x = fma(-CHEM_LDLU(lu + 63264), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 63296), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 63328), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 63360), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 63392), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 63424), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 63456), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 63488), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 63520), b[6016], x);
      b[5568] = x * CHEM_LDLU(vd + 5568);
    }
    {
      CHEM_PREFETCH(ws + 175584);
      CHEM_PREFETCH(ws + 175616);
      CHEM_PREFETCH(ws + 175648);
      CHEM_PREFETCH(ws + 175680);
      CHEM_PREFETCH(ws + 175712);
      CHEM_PREFETCH(ws + 175744);
      CHEM_PREFETCH(ws + 175776);
      CHEM_PREFETCH(ws + 175808);
      CHEM_PREFETCH(ws + 175840);
      CHEM_PREFETCH(ws + 175872);
      CHEM_PREFETCH(ws + 222080);
      double x = b[5536];
      x = fma(-CHEM_LDLU(lu + 63552), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 63584), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 63616), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 63648), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 63680), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 63712), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 63744), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 63776), b[6016], x);
      b[5536] = x * CHEM_LDLU(vd + 5536);
    }
    {
      CHEM_PREFETCH(ws + 175904);
      CHEM_PREFETCH(ws + 175936);
      CHEM_PREFETCH(ws + 175968);
      CHEM_PREFETCH(ws + 176000);
      CHEM_PREFETCH(ws + 176032);
      CHEM_PREFETCH(ws + 176064);
      CHEM_PREFETCH(ws + 176096);
      CHEM_PREFETCH(ws + 176128);
      CHEM_PREFETCH(ws + 176160);
      CHEM_PREFETCH(ws + 176192);
      CHEM_PREFETCH(ws + 222048);
      double x = b[5504];
      x = fma(-CHEM_LDLU(lu + 63808), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63840), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 63872), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 63904), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 63936), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 63968), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 64000), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 64032), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 64064), b[6016], x);
      b[5504] = x * CHEM_LDLU(vd + 5504);
    }
    {
      CHEM_PREFETCH(ws + 176224);
      CHEM_PREFETCH(ws + 176256);
      CHEM_PREFETCH(ws + 176288);
      CHEM_PREFETCH(ws + 176320);
      CHEM_PREFETCH(ws + 176352);
      CHEM_PREFETCH(ws + 176384);
      CHEM_PREFETCH(ws + 176416);
      CHEM_PREFETCH(ws + 176448);
      CHEM_PREFETCH(ws + 176480);
      CHEM_PREFETCH(ws + 176512);
      CHEM_PREFETCH(ws + 176544);
      CHEM_PREFETCH(ws + 222016);
      double x = b[5472];
      x = fma(-CHEM_LDLU(lu + 64096), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 64128), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 64160), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 64192), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 64224), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 64256), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 64288), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 64320), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 64352), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 64384), b[6016], x);
      b[5472] = x * CHEM_LDLU(vd + 5472);
    }
    {
      CHEM_PREFETCH(ws + 176576);
      CHEM_PREFETCH(ws + 176608);
      CHEM_PREFETCH(ws + 176640);
      CHEM_PREFETCH(ws + 176672);
      CHEM_PREFETCH(ws + 176704);
      CHEM_PREFETCH(ws + 176736);
      CHEM_PREFETCH(ws + 176768);
      CHEM_PREFETCH(ws + 176800);
      CHEM_PREFETCH(ws + 176832);
      CHEM_PREFETCH(ws + 176864);
      CHEM_PREFETCH(ws + 221984);
      double x = b[5440];
      x = fma(-CHEM_LDLU(lu + 64416), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 64448), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 64480), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 64512), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 64544), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 64576), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 64608), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 64640), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 64672), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 64704), b[6016], x);
      b[5440] = x * CHEM_LDLU(vd + 5440);
    }
    {
      CHEM_PREFETCH(ws + 176896);
      CHEM_PREFETCH(ws + 176928);
      CHEM_PREFETCH(ws + 176960);
      CHEM_PREFETCH(ws + 176992);
      CHEM_PREFETCH(ws + 177024);
      CHEM_PREFETCH(ws + 177056);
      CHEM_PREFETCH(ws + 177088);
      CHEM_PREFETCH(ws + 177120);
      CHEM_PREFETCH(ws + 177152);
      CHEM_PREFETCH(ws + 221952);
      double x = b[5408];
      x = fma(-CHEM_LDLU(lu + 64736), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64768), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 64800), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 64832), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 64864), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 64896), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 64928), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 64960), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 64992), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 65024), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 65056), b[6016], x);
      b[5408] = x * CHEM_LDLU(vd + 5408);
    }
    {
      CHEM_PREFETCH(ws + 177184);
      CHEM_PREFETCH(ws + 177216);
      CHEM_PREFETCH(ws + 177248);
      CHEM_PREFETCH(ws + 177280);
      CHEM_PREFETCH(ws + 177312);
      CHEM_PREFETCH(ws + 177344);
      CHEM_PREFETCH(ws + 177376);
      CHEM_PREFETCH(ws + 177408);
      CHEM_PREFETCH(ws + 177440);
      CHEM_PREFETCH(ws + 221920);
      double x = b[5376];
      x = fma(-CHEM_LDLU(lu + 65088), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 65120), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 65152), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 65184), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 65216), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 65248), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 65280), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 65312), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 65344), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 65376), b[6016], x);
      b[5376] = x * CHEM_LDLU(vd + 5376);
    }
    {
      CHEM_PREFETCH(ws + 177472);
      CHEM_PREFETCH(ws + 177504);
      CHEM_PREFETCH(ws + 177536);
      CHEM_PREFETCH(ws + 177568);
      CHEM_PREFETCH(ws + 177600);
      CHEM_PREFETCH(ws + 177632);
      CHEM_PREFETCH(ws + 177664);
      CHEM_PREFETCH(ws + 177696);
      CHEM_PREFETCH(ws + 177728);
      CHEM_PREFETCH(ws + 177760);
      CHEM_PREFETCH(ws + 177792);
      CHEM_PREFETCH(ws + 221888);
      double x = b[5344];
      x = fma(-CHEM_LDLU(lu + 65408), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 65440), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 65472), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 65504), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 65536), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 65568), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 65600), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 65632), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 65664), b[6016], x);
      b[5344] = x * CHEM_LDLU(vd + 5344);
    }
    {
      CHEM_PREFETCH(ws + 177824);
      CHEM_PREFETCH(ws + 177856);
      CHEM_PREFETCH(ws + 177888);
      CHEM_PREFETCH(ws + 177920);
      CHEM_PREFETCH(ws + 177952);
      CHEM_PREFETCH(ws + 177984);
      CHEM_PREFETCH(ws + 178016);
      CHEM_PREFETCH(ws + 178048);
      CHEM_PREFETCH(ws + 178080);
      CHEM_PREFETCH(ws + 178112);
      CHEM_PREFETCH(ws + 178144);
      CHEM_PREFETCH(ws + 178176);
      CHEM_PREFETCH(ws + 221856);
      double x = b[5312];
      x = fma(-CHEM_LDLU(lu + 65696), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 65728), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 65760), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 65792), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 65824), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 65856), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 65888), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 65920), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 65952), b[6016], x);
      b[5312] = x * CHEM_LDLU(vd + 5312);
    }
    {
      CHEM_PREFETCH(ws + 178208);
      CHEM_PREFETCH(ws + 178240);
      CHEM_PREFETCH(ws + 178272);
      CHEM_PREFETCH(ws + 178304);
      CHEM_PREFETCH(ws + 178336);
      CHEM_PREFETCH(ws + 178368);
      CHEM_PREFETCH(ws + 178400);
      CHEM_PREFETCH(ws + 178432);
      CHEM_PREFETCH(ws + 178464);
      CHEM_PREFETCH(ws + 178496);
      CHEM_PREFETCH(ws + 178528);
      CHEM_PREFETCH(ws + 178560);
      CHEM_PREFETCH(ws + 178592);
      CHEM_PREFETCH(ws + 178624);
      CHEM_PREFETCH(ws + 221824);
      double x = b[5280];
      x = fma(-CHEM_LDLU(lu + 65984), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 66016), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 66048), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 66080), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 66112), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 66144), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 66176), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 66208), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 66240), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 66272), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 66304), b[6016], x);
      b[5280] = x * CHEM_LDLU(vd + 5280);
    }
    {
      CHEM_PREFETCH(ws + 178656);
      CHEM_PREFETCH(ws + 178688);
      CHEM_PREFETCH(ws + 178720);
      CHEM_PREFETCH(ws + 178752);
      CHEM_PREFETCH(ws + 178784);
      CHEM_PREFETCH(ws + 178816);
      CHEM_PREFETCH(ws + 178848);
      CHEM_PREFETCH(ws + 178880);
      CHEM_PREFETCH(ws + 221792);
      double x = b[5248];
      x = fma(-CHEM_LDLU(lu + 66336), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 66368), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 66400), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 66432), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 66464), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 66496), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 66528), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 66560), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 66592), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 66624), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 66656), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 66688), b[6016], x);
      b[5248] = x * CHEM_LDLU(vd + 5248);
    }
}
__device__ __noinline__ void solve_1_3(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH(ws + 178912);
      CHEM_PREFETCH(ws + 178944);
      CHEM_PREFETCH(ws + 178976);
      CHEM_PREFETCH(ws + 179008);
      CHEM_PREFETCH(ws + 179040);
      CHEM_PREFETCH(ws + 179072);
      CHEM_PREFETCH(ws + 179104);
      CHEM_PREFETCH(ws + 179136);
      CHEM_PREFETCH(ws + 179168);
      CHEM_PREFETCH(ws + 179200);
      CHEM_PREFETCH(ws + 221760);
      double x = b[5216];
      x = fma(-CHEM_LDLU(lu + 66720), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 66752), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 66784), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 66816), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 66848), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 66880), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 66912), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 66944), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 66976), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 67008), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 67040), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 67072), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 67104), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 67136), b[6016], x);
      b[5216] = x * CHEM_LDLU(vd + 5216);
    }
    {
      CHEM_PREFETCH(ws + 179232);
      CHEM_PREFETCH(ws + 179264);
      CHEM_PREFETCH(ws + 179296);
      CHEM_PREFETCH(ws + 179328);
      CHEM_PREFETCH(ws + 179360);
      CHEM_PREFETCH(ws + 179392);
      CHEM_PREFETCH(ws + 179424);
      CHEM_PREFETCH(ws + 179456);
      CHEM_PREFETCH(ws + 179488);
      CHEM_PREFETCH(ws + 221728);
      double x = b[5184];
      x = fma(-CHEM_LDLU(lu + 67168), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 67200), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 67232), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 67264), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 67296), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 67328), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 67360), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 67392), b[6016], x);
      b[5184] = x * CHEM_LDLU(vd + 5184);
    }
    {
      CHEM_PREFETCH(ws + 179520);
      CHEM_PREFETCH(ws + 179552);
      CHEM_PREFETCH(ws + 179584);
      CHEM_PREFETCH(ws + 179616);
      CHEM_PREFETCH(ws + 179648);
      CHEM_PREFETCH(ws + 179680);
      CHEM_PREFETCH(ws + 179712);
      CHEM_PREFETCH(ws + 179744);
      CHEM_PREFETCH(ws + 179776);
      CHEM_PREFETCH(ws + 221696);
      double x = b[5152];
      x = fma(-CHEM_LDLU(lu + 67424), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67456), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 67488), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 67520), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 67552), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 67584), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 67616), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 67648), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 67680), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 67712), b[6016], x);
      b[5152] = x * CHEM_LDLU(vd + 5152);
    }
    {
      CHEM_PREFETCH(ws + 179808);
      CHEM_PREFETCH(ws + 179840);
      CHEM_PREFETCH(ws + 179872);
      CHEM_PREFETCH(ws + 179904);
      CHEM_PREFETCH(ws + 179936);
      CHEM_PREFETCH(ws + 179968);
      CHEM_PREFETCH(ws + 180000);
      CHEM_PREFETCH(ws + 180032);
      CHEM_PREFETCH(ws + 180064);
      CHEM_PREFETCH(ws + 180096);
      CHEM_PREFETCH(ws + 180128);
      CHEM_PREFETCH(ws + 180160);
      CHEM_PREFETCH(ws + 180192);
      CHEM_PREFETCH(ws + 180224);
      CHEM_PREFETCH(ws + 180256);
      CHEM_PREFETCH(ws + 221664);
      double x = b[5120];
      x = fma(-CHEM_LDLU(lu + 67744), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67776), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 67808), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 67840), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 67872), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 67904), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 67936), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 67968), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 68000), b[6016], x);
      b[5120] = x * CHEM_LDLU(vd + 5120);
    }
    {
      CHEM_PREFETCH(ws + 180288);
      CHEM_PREFETCH(ws + 180320);
      CHEM_PREFETCH(ws + 180352);
      CHEM_PREFETCH(ws + 180384);
      CHEM_PREFETCH(ws + 180416);
      CHEM_PREFETCH(ws + 180448);
      CHEM_PREFETCH(ws + 180480);
      CHEM_PREFETCH(ws + 180512);
      CHEM_PREFETCH(ws + 180544);
      CHEM_PREFETCH(ws + 180576);
      CHEM_PREFETCH(ws + 180608);
      CHEM_PREFETCH(ws + 180640);
      CHEM_PREFETCH(ws + 180672);
      CHEM_PREFETCH(ws + 221632);
      double x = b[5088];
      x = fma(-CHEM_LDLU(lu + 68032), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 68064), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 68096), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 68128), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 68160), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 68192), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 68224), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 68256), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 68288), b[6016], x);
      b[5088] = x * CHEM_LDLU(vd + 5088);
    }
    {
      CHEM_PREFETCH(ws + 180704);
      CHEM_PREFETCH(ws + 180736);
      CHEM_PREFETCH(ws + 180768);
      CHEM_PREFETCH(ws + 180800);
      CHEM_PREFETCH(ws + 180832);
      CHEM_PREFETCH(ws + 180864);
      CHEM_PREFETCH(ws + 180896);
      CHEM_PREFETCH(ws + 180928);
      CHEM_PREFETCH(ws + 180960);
      CHEM_PREFETCH(ws + 180992);
      CHEM_PREFETCH(ws + 221600);
      double x = b[5056];
      x = fma(-CHEM_LDLU(lu + 68320), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 68352), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 68384), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 68416), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 68448), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 68480), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 68512), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 68544), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 68576), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 68608), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 68640), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 68672), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 68704), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 68736), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 68768), b[6016], x);
      b[5056] = x * CHEM_LDLU(vd + 5056);
    }
    {
      CHEM_PREFETCH(ws + 181024);
      CHEM_PREFETCH(ws + 181056);
      CHEM_PREFETCH(ws + 181088);
      CHEM_PREFETCH(ws + 181120);
      CHEM_PREFETCH(ws + 181152);
      CHEM_PREFETCH(ws + 181184);
      CHEM_PREFETCH(ws + 181216);
      CHEM_PREFETCH(ws + 181248);
      CHEM_PREFETCH(ws + 181280);
      CHEM_PREFETCH(ws + 181312);
      CHEM_PREFETCH(ws + 181344);
      CHEM_PREFETCH(ws + 221568);
      double x = b[5024];
      x = fma(-CHEM_LDLU(lu + 68800), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 68832), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 68864), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 68896), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 68928), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 68960), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 68992), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 69024), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 69056), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 69088), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 69120), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 69152), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 69184), b[6016], x);
      b[5024] = x * CHEM_LDLU(vd + 5024);
    }
    {
      CHEM_PREFETCH(ws + 181376);
      CHEM_PREFETCH(ws + 181408);
      CHEM_PREFETCH(ws + 181440);
      CHEM_PREFETCH(ws + 181472);
      CHEM_PREFETCH(ws + 181504);
      CHEM_PREFETCH(ws + 181536);
      CHEM_PREFETCH(ws + 181568);
      CHEM_PREFETCH(ws + 181600);
      CHEM_PREFETCH(ws + 181632);
      CHEM_PREFETCH(ws + 181664);
      CHEM_PREFETCH(ws + 181696);
      CHEM_PREFETCH(ws + 181728);
      CHEM_PREFETCH(ws + 221536);
      double x = b[4992];
      x = fma(-CHEM_LDLU(lu + 69216), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 69248), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 69280), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 69312), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 69344), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 69376), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 69408), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 69440), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 69472), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 69504), b[6016], x);
      b[4992] = x * CHEM_LDLU(vd + 4992);
    }
    {
      CHEM_PREFETCH(ws + 181760);
      CHEM_PREFETCH(ws + 181792);
      CHEM_PREFETCH(ws + 181824);
      CHEM_PREFETCH(ws + 181856);
      CHEM_PREFETCH(ws + 181888);
      CHEM_PREFETCH(ws + 181920);
      CHEM_PREFETCH(ws + 181952);
      CHEM_PREFETCH(ws + 181984);
      CHEM_PREFETCH(ws + 182016);
      CHEM_PREFETCH(ws + 182048);
      CHEM_PREFETCH(ws + 182080);
      CHEM_PREFETCH(ws + 182112);
      CHEM_PREFETCH(ws + 182144);
      CHEM_PREFETCH(ws + 221504);
      double x = b[4960];
      x = fma(-CHEM_LDLU(lu + 69536), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 69568), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 69600), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 69632), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 69664), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 69696), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 69728), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 69760), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 69792), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 69824), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 69856), b[6016], x);
      b[4960] = x * CHEM_LDLU(vd + 4960);
    }
    {
      CHEM_PREFETCH(ws + 182176);
      CHEM_PREFETCH(ws + 182208);
      CHEM_PREFETCH(ws + 182240);
      CHEM_PREFETCH(ws + 182272);
      CHEM_PREFETCH(ws + 182304);
      CHEM_PREFETCH(ws + 182336);
      CHEM_PREFETCH(ws + 182368);
      CHEM_PREFETCH(ws + 182400);
      CHEM_PREFETCH(ws + 182432);
      CHEM_PREFETCH(ws + 182464);
      CHEM_PREFETCH(ws + 182496);
      CHEM_PREFETCH(ws + 182528);
      CHEM_PREFETCH(ws + 182560);
      CHEM_PREFETCH(ws + 182592);
      CHEM_PREFETCH(ws + 221472);
      double x = b[4928];
      x = fma(-CHEM_LDLU(lu + 69888), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69920), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 69952), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 69984), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 70016), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 70048), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 70080), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 70112), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 70144), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 70176), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 70208), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 70240), b[6016], x);
      b[4928] = x * CHEM_LDLU(vd + 4928);
    }
    {
      CHEM_PREFETCH(ws + 182624);
      CHEM_PREFETCH(ws + 182656);
      CHEM_PREFETCH(ws + 182688);
      CHEM_PREFETCH(ws + 182720);
      CHEM_PREFETCH(ws + 182752);
      CHEM_PREFETCH(ws + 182784);
      CHEM_PREFETCH(ws + 182816);
      CHEM_PREFETCH(ws + 182848);
      CHEM_PREFETCH(ws + 182880);
      CHEM_PREFETCH(ws + 182912);
      CHEM_PREFETCH(ws + 182944);
      CHEM_PREFETCH(ws + 182976);
      CHEM_PREFETCH(ws + 183008);
      CHEM_PREFETCH(ws + 183040);
      CHEM_PREFETCH(ws + 221440);
      double x = b[4896];
      x = fma(-CHEM_LDLU(lu + 70272), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 70304), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 70336), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 70368), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 70400), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 70432), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 70464), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 70496), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 70528), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 70560), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 70592), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 70624), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 70656), b[6016], x);
      b[4896] = x * CHEM_LDLU(vd + 4896);
    }
    {
      CHEM_PREFETCH(ws + 183072);
      CHEM_PREFETCH(ws + 183104);
      CHEM_PREFETCH(ws + 183136);
      CHEM_PREFETCH(ws + 183168);
      CHEM_PREFETCH(ws + 183200);
      CHEM_PREFETCH(ws + 183232);
      CHEM_PREFETCH(ws + 183264);
      CHEM_PREFETCH(ws + 183296);
      CHEM_PREFETCH(ws + 183328);
      CHEM_PREFETCH(ws + 183360);
      CHEM_PREFETCH(ws + 183392);
      CHEM_PREFETCH(ws + 221408);
      double x = b[4864];
      x = fma(-CHEM_LDLU(lu + 70688), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70720), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 70752), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 70784), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 70816), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 70848), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 70880), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 70912), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 70944), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 70976), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 71008), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 71040), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 71072), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 71104), b[6016], x);
      b[4864] = x * CHEM_LDLU(vd + 4864);
    }
    {
      CHEM_PREFETCH(ws + 183424);
      CHEM_PREFETCH(ws + 183456);
      CHEM_PREFETCH(ws + 183488);
      CHEM_PREFETCH(ws + 183520);
      CHEM_PREFETCH(ws + 183552);
      CHEM_PREFETCH(ws + 183584);
      CHEM_PREFETCH(ws + 183616);
      CHEM_PREFETCH(ws + 183648);
      CHEM_PREFETCH(ws + 183680);
      CHEM_PREFETCH(ws + 183712);
      CHEM_PREFETCH(ws + 183744);
      CHEM_PREFETCH(ws + 183776);
      CHEM_PREFETCH(ws + 183808);
      CHEM_PREFETCH(ws + 183840);
      CHEM_PREFETCH(ws + 183872);
      CHEM_PREFETCH(ws + 221376);
      double x = b[4832];
      x = fma(-CHEM_LDLU(lu + 71136), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 71168), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 71200), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 71232), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 71264), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 71296), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 71328), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 71360), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 71392), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 71424), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 71456), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 71488), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 71520), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 71552), b[6016], x);
      b[4832] = x * CHEM_LDLU(vd + 4832);
    }
    {
      CHEM_PREFETCH(ws + 183904);
      CHEM_PREFETCH(ws + 183936);
      CHEM_PREFETCH(ws + 183968);
      CHEM_PREFETCH(ws + 184000);
      CHEM_PREFETCH(ws + 184032);
      CHEM_PREFETCH(ws + 184064);
      CHEM_PREFETCH(ws + 184096);
      CHEM_PREFETCH(ws + 221344);
      double x = b[4800];
      x = fma(-CHEM_LDLU(lu + 71584), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 71616), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 71648), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 71680), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 71712), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 71744), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 71776), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 71808), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 71840), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 71872), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 71904), b[6016], x);
      b[4800] = x * CHEM_LDLU(vd + 4800);
    }
    {
      CHEM_PREFETCH(ws + 184128);
      CHEM_PREFETCH(ws + 184160);
      CHEM_PREFETCH(ws + 184192);
      CHEM_PREFETCH(ws + 184224);
      CHEM_PREFETCH(ws + 184256);
      CHEM_PREFETCH(ws + 184288);
      CHEM_PREFETCH(ws + 184320);
      CHEM_PREFETCH(ws + 184352);
      CHEM_PREFETCH(ws + 184384);
      CHEM_PREFETCH(ws + 184416);
      CHEM_PREFETCH(ws + 184448);
      CHEM_PREFETCH(ws + 184480);
      CHEM_PREFETCH(ws + 184512);
      CHEM_PREFETCH(ws + 184544);
      CHEM_PREFETCH(ws + 221312);
      double x = b[4768];
      x = fma(-CHEM_LDLU(lu + 71936), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 71968), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 72000), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 72032), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 72064), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 72096), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 72128), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 72160), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 72192), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 72224), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 72256), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 72288), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 72320), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 72352), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 72384), b[6016], x);
      b[4768] = x * CHEM_LDLU(vd + 4768);
    }
    {
      CHEM_PREFETCH(ws + 184576);
      CHEM_PREFETCH(ws + 184608);
      CHEM_PREFETCH(ws + 184640);
      CHEM_PREFETCH(ws + 184672);
      CHEM_PREFETCH(ws + 184704);
      CHEM_PREFETCH(ws + 184736);
      CHEM_PREFETCH(ws + 184768);
      CHEM_PREFETCH(ws + 184800);
      CHEM_PREFETCH(ws + 221280);
      double x = b[4736];
      x = fma(-CHEM_LDLU(lu + 72416), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 72448), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 72480), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 72512), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 72544), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 72576), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 72608), b[6016], x);
      b[4736] = x * CHEM_LDLU(vd + 4736);
    }
    {
      CHEM_PREFETCH(ws + 184832);
      CHEM_PREFETCH(ws + 184864);
      CHEM_PREFETCH(ws + 184896);
      CHEM_PREFETCH(ws + 184928);
      CHEM_PREFETCH(ws + 184960);
      CHEM_PREFETCH(ws + 184992);
      CHEM_PREFETCH(ws + 185024);
      CHEM_PREFETCH(ws + 185056);
      CHEM_PREFETCH(ws + 185088);
      CHEM_PREFETCH(ws + 185120);
      CHEM_PREFETCH(ws + 185152);
      CHEM_PREFETCH(ws + 185184);
      CHEM_PREFETCH(ws + 185216);
      CHEM_PREFETCH(ws + 185248);
      CHEM_PREFETCH(ws + 185280);
      CHEM_PREFETCH(ws + 221248);
      double x = b[4704];
      x = fma(-CHEM_LDLU(lu + 72640), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 72672), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 72704), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 72736), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 72768), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 72800), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 72832), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 72864), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 72896), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 72928), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 72960), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 72992), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 73024), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 73056), b[6016], x);
      b[4704] = x * CHEM_LDLU(vd + 4704);
    }
    {
      CHEM_PREFETCH(ws + 185312);
      CHEM_PREFETCH(ws + 185344);
      CHEM_PREFETCH(ws + 185376);
      CHEM_PREFETCH(ws + 185408);
      CHEM_PREFETCH(ws + 185440);
      CHEM_PREFETCH(ws + 185472);
      CHEM_PREFETCH(ws + 185504);
      CHEM_PREFETCH(ws + 185536);
      CHEM_PREFETCH(ws + 185568);
      CHEM_PREFETCH(ws + 185600);
      CHEM_PREFETCH(ws + 185632);
      CHEM_PREFETCH(ws + 185664);
      CHEM_PREFETCH(ws + 185696);
      CHEM_PREFETCH(ws + 185728);
      CHEM_PREFETCH(ws + 185760);
      CHEM_PREFETCH(ws + 221216);
      double x = b[4672];
      x = fma(-CHEM_LDLU(lu + 73088), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 73120), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 73152), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 73184), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 73216), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 73248), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 73280), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 73312), b[6016], x);
      b[4672] = x * CHEM_LDLU(vd + 4672);
    }
    {
      CHEM_PREFETCH(ws + 185792);
      CHEM_PREFETCH(ws + 185824);
      CHEM_PREFETCH(ws + 185856);
      CHEM_PREFETCH(ws + 185888);
      CHEM_PREFETCH(ws + 185920);
      CHEM_PREFETCH(ws + 185952);
      CHEM_PREFETCH(ws + 185984);
      CHEM_PREFETCH(ws + 221184);
      double x = b[4640];
      x = fma(-CHEM_LDLU(lu + 73344), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 73376), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 73408), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 73440), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 73472), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 73504), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 73536), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 73568), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 73600), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 73632), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 73664), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 73696), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 73728), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 73760), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 73792), b[6016], x);
      b[4640] = x * CHEM_LDLU(vd + 4640);
    }
    {
      CHEM_PREFETCH(ws + 186016);
      CHEM_PREFETCH(ws + 186048);
      CHEM_PREFETCH(ws + 186080);
      CHEM_PREFETCH(ws + 186112);
      CHEM_PREFETCH(ws + 186144);
      CHEM_PREFETCH(ws + 186176);
      CHEM_PREFETCH(ws + 186208);
      CHEM_PREFETCH(ws + 186240);
      CHEM_PREFETCH(ws + 221152);
      double x = b[4608];
      x = fma(-CHEM_LDLU(lu + 73824), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73856), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 73888), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 73920), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 73952), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 73984), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 74016), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 74048), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 74080), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 74112), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 74144), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 74176), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 74208), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 74240), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 74272), b[6016], x);
      b[4608] = x * CHEM_LDLU(vd + 4608);
    }
    {
      CHEM_PREFETCH(ws + 186272);
      CHEM_PREFETCH(ws + 186304);
      CHEM_PREFETCH(ws + 186336);
      CHEM_PREFETCH(ws + 186368);
      CHEM_PREFETCH(ws + 186400);
      CHEM_PREFETCH(ws + 186432);
      CHEM_PREFETCH(ws + 186464);
      CHEM_PREFETCH(ws + 221120);
      double x = b[4576];
      x = fma(-CHEM_LDLU(lu + 74304), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 74336), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 74368), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 74400), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 74432), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 74464), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 74496), b[6016], x);
      b[4576] = x * CHEM_LDLU(vd + 4576);
    }
    {
      CHEM_PREFETCH(ws + 186496);
      CHEM_PREFETCH(ws + 186528);
      CHEM_PREFETCH(ws + 186560);
      CHEM_PREFETCH(ws + 186592);
      CHEM_PREFETCH(ws + 186624);
      CHEM_PREFETCH(ws + 186656);
      CHEM_PREFETCH(ws + 186688);
      CHEM_PREFETCH(ws + 186720);
      CHEM_PREFETCH(ws + 186752);
      CHEM_PREFETCH(ws + 221088);
      double x = b[4544];
      x = fma(-CHEM_LDLU(lu + 74528), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74560), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 74592), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 74624), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 74656), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 74688), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 74720), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 74752), b[6016], x);
      b[4544] = x * CHEM_LDLU(vd + 4544);
    }
    {
      CHEM_PREFETCH(ws + 186784);
      CHEM_PREFETCH(ws + 186816);
      CHEM_PREFETCH(ws + 186848);
      CHEM_PREFETCH(ws + 186880);
      CHEM_PREFETCH(ws + 186912);
      CHEM_PREFETCH(ws + 186944);
      CHEM_PREFETCH(ws + 186976);
      CHEM_PREFETCH(ws + 221056);
      double x = b[4512];
      x = fma(-CHEM_LDLU(lu + 74784), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 74816), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 74848), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 74880), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 74912), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 74944), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 74976), b[6016], x);
      b[4512] = x * CHEM_LDLU(vd + 4512);
    }
    {
      CHEM_PREFETCH(ws + 187008);
      CHEM_PREFETCH(ws + 187040);
      CHEM_PREFETCH(ws + 187072);
      CHEM_PREFETCH(ws + 187104);
      CHEM_PREFETCH(ws + 187136);
      CHEM_PREFETCH(ws + 187168);
      CHEM_PREFETCH(ws + 187200);
      CHEM_PREFETCH(ws + 187232);
      CHEM_PREFETCH(ws + 221024);
      double x = b[4480];
      x = fma(-CHEM_LDLU(lu + 75008), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 75040), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 75072), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 75104), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 75136), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 75168), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 75200), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 75232), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 75264), b[6016], x);
      b[4480] = x * CHEM_LDLU(vd + 4480);
    }
    {
      CHEM_PREFETCH(ws + 187264);
      CHEM_PREFETCH(ws + 187296);
      CHEM_PREFETCH(ws + 187328);
      CHEM_PREFETCH(ws + 187360);
      CHEM_PREFETCH(ws + 187392);
      CHEM_PREFETCH(ws + 187424);
      CHEM_PREFETCH(ws + 187456);
      CHEM_PREFETCH(ws + 187488);
      CHEM_PREFETCH(ws + 187520);
      CHEM_PREFETCH(ws + 220992);
      double x = b[4448];
      x = fma(-CHEM_LDLU(lu + 75296), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 75328), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 75360), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 75392), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 75424), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 75456), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 75488), b[6016], x);
      b[4448] = x * CHEM_LDLU(vd + 4448);
    }
    {
      CHEM_PREFETCH(ws + 187552);
      CHEM_PREFETCH(ws + 187584);
      CHEM_PREFETCH(ws + 187616);
      CHEM_PREFETCH(ws + 187648);
      CHEM_PREFETCH(ws + 187680);
      CHEM_PREFETCH(ws + 187712);
      CHEM_PREFETCH(ws + 187744);
      CHEM_PREFETCH(ws + 187776);
      CHEM_PREFETCH(ws + 187808);
      CHEM_PREFETCH(ws + 220960);
      double x = b[4416];
      x = fma(-CHEM_LDLU(lu + 75520), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 75552), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 75584), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 75616), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 75648), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 75680), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 75712), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 75744), b[6016], x);
      b[4416] = x * CHEM_LDLU(vd + 4416);
    }
    {
      CHEM_PREFETCH(ws + 187840);
      CHEM_PREFETCH(ws + 187872);
      CHEM_PREFETCH(ws + 187904);
      CHEM_PREFETCH(ws + 187936);
      CHEM_PREFETCH(ws + 187968);
      CHEM_PREFETCH(ws + 188000);
      CHEM_PREFETCH(ws + 188032);
      CHEM_PREFETCH(ws + 220928);
      double x = b[4384];
      x = fma(-CHEM_LDLU(lu + 75776), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 75808), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 75840), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 75872), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 75904), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 75936), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 75968), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 76000), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 76032), b[6016], x);
      b[4384] = x * CHEM_LDLU(vd + 4384);
    }
    {
      CHEM_PREFETCH(ws + 188064);
      CHEM_PREFETCH(ws + 188096);
      CHEM_PREFETCH(ws + 188128);
      CHEM_PREFETCH(ws + 188160);
      CHEM_PREFETCH(ws + 188192);
      CHEM_PREFETCH(ws + 188224);
      CHEM_PREFETCH(ws + 188256);
      CHEM_PREFETCH(ws + 220896);
      double x = b[4352];
      x = fma(-CHEM_LDLU(lu + 76064), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 76096), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 76128), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 76160), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 76192), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 76224), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 76256), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 76288), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 76320), b[6016], x);
      b[4352] = x * CHEM_LDLU(vd + 4352);
    }
    {
      CHEM_PREFETCH(ws + 188288);
      CHEM_PREFETCH(ws + 188320);
      CHEM_PREFETCH(ws + 188352);
      CHEM_PREFETCH(ws + 188384);
      CHEM_PREFETCH(ws + 188416);
      CHEM_PREFETCH(ws + 188448);
      CHEM_PREFETCH(ws + 188480);
      CHEM_PREFETCH(ws + 188512);
      CHEM_PREFETCH(ws + 188544);
      CHEM_PREFETCH(ws + 188576);
      CHEM_PREFETCH(ws + 220864);
      double x = b[4320];
      x = fma(-CHEM_LDLU(lu + 76352), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 76384), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 76416), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 76448), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 76480), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 76512), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 76544), b[6016], x);
      b[4320] = x * CHEM_LDLU(vd + 4320);
    }
    {
      CHEM_PREFETCH(ws + 188608);
      CHEM_PREFETCH(ws + 188640);
      CHEM_PREFETCH(ws + 188672);
      CHEM_PREFETCH(ws + 188704);
      CHEM_PREFETCH(ws + 188736);
      CHEM_PREFETCH(ws + 188768);
      CHEM_PREFETCH(ws + 188800);
      CHEM_PREFETCH(ws + 188832);
      CHEM_PREFETCH(ws + 188864);
      CHEM_PREFETCH(ws + 188896);
      CHEM_PREFETCH(ws + 220832);
      double x = b[4288];
      x = fma(-CHEM_LDLU(lu + 76576), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 76608), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 76640), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 76672), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 76704), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 76736), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 76768), b[6016], x);
      b[4288] = x * CHEM_LDLU(vd + 4288);
    }
    {
      CHEM_PREFETCH(ws + 188928);
      CHEM_PREFETCH(ws + 188960);
      CHEM_PREFETCH(ws + 188992);
      CHEM_PREFETCH(ws + 189024);
      CHEM_PREFETCH(ws + 189056);
      CHEM_PREFETCH(ws + 189088);
      CHEM_PREFETCH(ws + 189120);
      CHEM_PREFETCH(ws + 189152);
      CHEM_PREFETCH(ws + 220800);
      double x = b[4256];
      x = fma(-CHEM_LDLU(lu + 76800), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76832), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 76864), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 76896), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 76928), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 76960), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 76992), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 77024), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 77056), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 77088), b[6016], x);
      b[4256] = x * CHEM_LDLU(vd + 4256);
    }
    {
      CHEM_PREFETCH(ws + 189184);
      CHEM_PREFETCH(ws + 189216);
      CHEM_PREFETCH(ws + 189248);
      CHEM_PREFETCH(ws + 189280);
      CHEM_PREFETCH(ws + 189312);
      CHEM_PREFETCH(ws + 189344);
      CHEM_PREFETCH(ws + 189376);
      CHEM_PREFETCH(ws + 189408);
      CHEM_PREFETCH(ws + 189440);
      CHEM_PREFETCH(ws + 220768);
      double x = b[4224];
      x = fma(-CHEM_LDLU(lu + 77120), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 77152), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 77184), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 77216), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 77248), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 77280), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 77312), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 77344), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 77376), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 77408), b[6016], x);
      b[4224] = x * CHEM_LDLU(vd + 4224);
    }
    {
      CHEM_PREFETCH(ws + 189472);
      CHEM_PREFETCH(ws + 189504);
      CHEM_PREFETCH(ws + 189536);
      CHEM_PREFETCH(ws + 189568);
      CHEM_PREFETCH(ws + 189600);
      CHEM_PREFETCH(ws + 189632);
      CHEM_PREFETCH(ws + 189664);
      CHEM_PREFETCH(ws + 189696);
      CHEM_PREFETCH(ws + 220736);
      double x = b[4192];
      x = fma(-CHEM_LDLU(lu + 77440), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 77472), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 77504), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 77536), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 77568), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 77600), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 77632), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 77664), b[6016], x);
      b[4192] = x * CHEM_LDLU(vd + 4192);
    }
    {
      CHEM_PREFETCH(ws + 189728);
      CHEM_PREFETCH(ws + 189760);
      CHEM_PREFETCH(ws + 189792);
      CHEM_PREFETCH(ws + 189824);
      CHEM_PREFETCH(ws + 189856);
      CHEM_PREFETCH(ws + 189888);
      CHEM_PREFETCH(ws + 189920);
      CHEM_PREFETCH(ws + 189952);
      CHEM_PREFETCH(ws + 189984);
      CHEM_PREFETCH(ws + 190016);
      CHEM_PREFETCH(ws + 190048);
      CHEM_PREFETCH(ws + 220704);
      double x = b[4160];
      x = fma(-CHEM_LDLU(lu + 77696), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 77728), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 77760), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 77792), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 77824), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 77856), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 77888), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 77920), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 77952), b[6016], x);
      b[4160] = x * CHEM_LDLU(vd + 4160);
    }
    {
      CHEM_PREFETCH(ws + 190080);
      CHEM_PREFETCH(ws + 190112);
      CHEM_PREFETCH(ws + 190144);
      CHEM_PREFETCH(ws + 190176);
      CHEM_PREFETCH(ws + 190208);
      CHEM_PREFETCH(ws + 190240);
      CHEM_PREFETCH(ws + 190272);
      CHEM_PREFETCH(ws + 220672);
      double x = b[4128];
      x = fma(-CHEM_LDLU(lu + 77984), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 78016), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 78048), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 78080), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 78112), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 78144), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 78176), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 78208), b[6016], x);
      b[4128] = x * CHEM_LDLU(vd + 4128);
    }
    {
      CHEM_PREFETCH(ws + 190304);
      CHEM_PREFETCH(ws + 190336);
      CHEM_PREFETCH(ws + 190368);
      CHEM_PREFETCH(ws + 190400);
      CHEM_PREFETCH(ws + 190432);
      CHEM_PREFETCH(ws + 190464);
      CHEM_PREFETCH(ws + 190496);
      CHEM_PREFETCH(ws + 190528);
      CHEM_PREFETCH(ws + 220640);
      double x = b[4096];
      x = fma(-CHEM_LDLU(lu + 78240), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 78272), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 78304), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 78336), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 78368), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 78400), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 78432), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 78464), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 78496), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 78528), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 78560), b[6016], x);
      b[4096] = x * CHEM_LDLU(vd + 4096);
    }
    {
      CHEM_PREFETCH(ws + 190560);
      CHEM_PREFETCH(ws + 190592);
      CHEM_PREFETCH(ws + 190624);
      CHEM_PREFETCH(ws + 190656);
      CHEM_PREFETCH(ws + 190688);
      CHEM_PREFETCH(ws + 190720);
      CHEM_PREFETCH(ws + 190752);
      CHEM_PREFETCH(ws + 190784);
      CHEM_PREFETCH(ws + 220608);
      double x = b[4064];
      x = fma(-CHEM_LDLU(lu + 78592), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 78624), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 78656), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 78688), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 78720), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 78752), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 78784), b[6016], x);
      b[4064] = x * CHEM_LDLU(vd + 4064);
    }
    {
      CHEM_PREFETCH(ws + 190816);
      CHEM_PREFETCH(ws + 190848);
      CHEM_PREFETCH(ws + 190880);
      CHEM_PREFETCH(ws + 190912);
      CHEM_PREFETCH(ws + 190944);
      CHEM_PREFETCH(ws + 190976);
      CHEM_PREFETCH(ws + 191008);
      CHEM_PREFETCH(ws + 191040);
      CHEM_PREFETCH(ws + 191072);
      CHEM_PREFETCH(ws + 220576);
      double x = b[4032];
      x = fma(-CHEM_LDLU(lu + 78816), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78848), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 78880), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 78912), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 78944), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 78976), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 79008), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 79040), b[6016], x);
      b[4032] = x * CHEM_LDLU(vd + 4032);
    }
    {
      CHEM_PREFETCH(ws + 191104);
      CHEM_PREFETCH(ws + 191136);
      CHEM_PREFETCH(ws + 191168);
      CHEM_PREFETCH(ws + 191200);
      CHEM_PREFETCH(ws + 191232);
      CHEM_PREFETCH(ws + 191264);
      CHEM_PREFETCH(ws + 191296);
      CHEM_PREFETCH(ws + 191328);
      CHEM_PREFETCH(ws + 191360);
      CHEM_PREFETCH(ws + 191392);
      CHEM_PREFETCH(ws + 220544);
      double x = b[4000];
      x = fma(-CHEM_LDLU(lu + 79072), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 79104), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 79136), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 79168), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 79200), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 79232), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 79264), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 79296), b[6016], x);
      b[4000] = x * CHEM_LDLU(vd + 4000);
    }
    {
      CHEM_PREFETCH(ws + 191424);
      CHEM_PREFETCH(ws + 191456);
      CHEM_PREFETCH(ws + 191488);
      CHEM_PREFETCH(ws + 191520);
      CHEM_PREFETCH(ws + 191552);
      CHEM_PREFETCH(ws + 191584);
      CHEM_PREFETCH(ws + 220512);
      double x = b[3968];
      x = fma(-CHEM_LDLU(lu + 79328), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 79360), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 79392), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 79424), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 79456), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 79488), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 79520), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 79552), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 79584), b[6016], x);
      b[3968] = x * CHEM_LDLU(vd + 3968);
    }
    {
      CHEM_PREFETCH(ws + 191616);
      CHEM_PREFETCH(ws + 191648);
      CHEM_PREFETCH(ws + 191680);
      CHEM_PREFETCH(ws + 191712);
      CHEM_PREFETCH(ws + 191744);
      CHEM_PREFETCH(ws + 191776);
      CHEM_PREFETCH(ws + 191808);
      CHEM_PREFETCH(ws + 220480);
      double x = b[3936];
      x = fma(-CHEM_LDLU(lu + 79616), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 79648), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 79680), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 79712), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 79744), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 79776), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 79808), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 79840), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 79872), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 79904), b[6016], x);
      b[3936] = x * CHEM_LDLU(vd + 3936);
    }
    {
      CHEM_PREFETCH(ws + 191840);
      CHEM_PREFETCH(ws + 191872);
      CHEM_PREFETCH(ws + 191904);
      CHEM_PREFETCH(ws + 191936);
      CHEM_PREFETCH(ws + 191968);
      CHEM_PREFETCH(ws + 192000);
      CHEM_PREFETCH(ws + 192032);
      CHEM_PREFETCH(ws + 192064);
      CHEM_PREFETCH(ws + 192096);
      CHEM_PREFETCH(ws + 192128);
      CHEM_PREFETCH(ws + 220448);
      double x = b[3904];
      x = fma(-CHEM_LDLU(lu + 79936), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 79968), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 80000), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 80032), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 80064), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 80096), b[6016], x);
      b[3904] = x * CHEM_LDLU(vd + 3904);
    }
    {
      CHEM_PREFETCH(ws + 192160);
      CHEM_PREFETCH(ws + 192192);
      CHEM_PREFETCH(ws + 192224);
      CHEM_PREFETCH(ws + 192256);
      CHEM_PREFETCH(ws + 192288);
      CHEM_PREFETCH(ws + 192320);
      CHEM_PREFETCH(ws + 192352);
      CHEM_PREFETCH(ws + 192384);
      CHEM_PREFETCH(ws + 220416);
      double x = b[3872];
      x = fma(-CHEM_LDLU(lu + 80128), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 80160), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 80192), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 80224), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 80256), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 80288), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 80320), b[6016], x);
      b[3872] = x * CHEM_LDLU(vd + 3872);
    }
    {
      CHEM_PREFETCH(ws + 192416);
      CHEM_PREFETCH(ws + 192448);
      CHEM_PREFETCH(ws + 192480);
      CHEM_PREFETCH(ws + 192512);
      CHEM_PREFETCH(ws + 192544);
      CHEM_PREFETCH(ws + 192576);
      CHEM_PREFETCH(ws + 192608);
      CHEM_PREFETCH(ws + 192640);
      CHEM_PREFETCH(ws + 192672);
      CHEM_PREFETCH(ws + 220384);
      double x = b[3840];
      x = fma(-CHEM_LDLU(lu + 80352), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 80384), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 80416), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 80448), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 80480), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 80512), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 80544), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 80576), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 80608), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 80640), b[6016], x);
      b[3840] = x * CHEM_LDLU(vd + 3840);
    }
    {
      CHEM_PREFETCH(ws + 192704);
      CHEM_PREFETCH(ws + 192736);
      CHEM_PREFETCH(ws + 192768);
      CHEM_PREFETCH(ws + 192800);
      CHEM_PREFETCH(ws + 192832);
      CHEM_PREFETCH(ws + 192864);
      CHEM_PREFETCH(ws + 192896);
      CHEM_PREFETCH(ws + 192928);
      CHEM_PREFETCH(ws + 192960);
      CHEM_PREFETCH(ws + 192992);
      CHEM_PREFETCH(ws + 220352);
      double x = b[3808];
      x = fma(-CHEM_LDLU(lu + 80672), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 80704), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 80736), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 80768), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 80800), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 80832), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 80864), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 80896), b[6016], x);
      b[3808] = x * CHEM_LDLU(vd + 3808);
    }
    {
      CHEM_PREFETCH(ws + 193024);
      CHEM_PREFETCH(ws + 193056);
      CHEM_PREFETCH(ws + 193088);
      CHEM_PREFETCH(ws + 193120);
      CHEM_PREFETCH(ws + 193152);
      CHEM_PREFETCH(ws + 193184);
      CHEM_PREFETCH(ws + 193216);
      CHEM_PREFETCH(ws + 193248);
      CHEM_PREFETCH(ws + 193280);
      CHEM_PREFETCH(ws + 193312);
      CHEM_PREFETCH(ws + 220320);
      double x = b[3776];
      x = fma(-CHEM_LDLU(lu + 80928), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 80960), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 80992), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 81024), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 81056), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 81088), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 81120), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 81152), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 81184), b[6016], x);
      b[3776] = x * CHEM_LDLU(vd + 3776);
    }
    {
      CHEM_PREFETCH(ws + 193344);
      CHEM_PREFETCH(ws + 193376);
      CHEM_PREFETCH(ws + 193408);
      CHEM_PREFETCH(ws + 193440);
      CHEM_PREFETCH(ws + 193472);
      CHEM_PREFETCH(ws + 193504);
      CHEM_PREFETCH(ws + 193536);
      CHEM_PREFETCH(ws + 193568);
      CHEM_PREFETCH(ws + 193600);
      CHEM_PREFETCH(ws + 220288);
      double x = b[3744];
      x = fma(-CHEM_LDLU(lu + 81216), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 81248), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 81280), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 81312), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 81344), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 81376), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 81408), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 81440), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 81472), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 81504), b[6016], x);
      b[3744] = x * CHEM_LDLU(vd + 3744);
    }
    {
      CHEM_PREFETCH(ws + 193632);
      CHEM_PREFETCH(ws + 193664);
      CHEM_PREFETCH(ws + 193696);
      CHEM_PREFETCH(ws + 193728);
      CHEM_PREFETCH(ws + 193760);
      CHEM_PREFETCH(ws + 193792);
      CHEM_PREFETCH(ws + 193824);
      CHEM_PREFETCH(ws + 193856);
      CHEM_PREFETCH(ws + 220256);
      double x = b[3712];
      x = fma(-CHEM_LDLU(lu + 81536), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 81568), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 81600), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 81632), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 81664), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 81696), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 81728), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 81760), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 81792), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 81824), b[6016], x);
      b[3712] = x * CHEM_LDLU(vd + 3712);
    }
    {
      CHEM_PREFETCH(ws + 193888);
      CHEM_PREFETCH(ws + 193920);
      CHEM_PREFETCH(ws + 193952);
      CHEM_PREFETCH(ws + 193984);
      CHEM_PREFETCH(ws + 194016);
      CHEM_PREFETCH(ws + 194048);
      CHEM_PREFETCH(ws + 194080);
      CHEM_PREFETCH(ws + 194112);
      CHEM_PREFETCH(ws + 194144);
      CHEM_PREFETCH(ws + 220224);
      double x = b[3680];
      x = fma(-CHEM_LDLU(lu + 81856), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 81888), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 81920), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 81952), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 81984), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 82016), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 82048), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 82080), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 82112), b[6016], x);
      b[3680] = x * CHEM_LDLU(vd + 3680);
    }
    {
      CHEM_PREFETCH(ws + 194176);
      CHEM_PREFETCH(ws + 194208);
      CHEM_PREFETCH(ws + 194240);
      CHEM_PREFETCH(ws + 194272);
      CHEM_PREFETCH(ws + 194304);
      CHEM_PREFETCH(ws + 194336);
      CHEM_PREFETCH(ws + 194368);
      CHEM_PREFETCH(ws + 220192);
      double x = b[3648];
      x = fma(-CHEM_LDLU(lu + 82144), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 82176), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 82208), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 82240), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 82272), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 82304), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 82336), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 82368), b[6016], x);
      b[3648] = x * CHEM_LDLU(vd + 3648);
    }
    {
      CHEM_PREFETCH(ws + 194400);
      CHEM_PREFETCH(ws + 194432);
      CHEM_PREFETCH(ws + 194464);
      CHEM_PREFETCH(ws + 194496);
      CHEM_PREFETCH(ws + 194528);
      CHEM_PREFETCH(ws + 194560);
      CHEM_PREFETCH(ws + 194592);
      CHEM_PREFETCH(ws + 220160);
      double x = b[3616];
      x = fma(-CHEM_LDLU(lu + 82400), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 82432), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 82464), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 82496), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 82528), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 82560), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 82592), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 82624), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 82656), b[6016], x);
      b[3616] = x * CHEM_LDLU(vd + 3616);
    }
    {
      CHEM_PREFETCH(ws + 194624);
      CHEM_PREFETCH(ws + 194656);
      CHEM_PREFETCH(ws + 194688);
      CHEM_PREFETCH(ws + 194720);
      CHEM_PREFETCH(ws + 194752);
      CHEM_PREFETCH(ws + 194784);
      CHEM_PREFETCH(ws + 194816);
      CHEM_PREFETCH(ws + 194848);
      CHEM_PREFETCH(ws + 220128);
      double x = b[3584];
      x = fma(-CHEM_LDLU(lu + 82688), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 82720), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 82752), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 82784), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 82816), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 82848), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 82880), b[6016], x);
      b[3584] = x * CHEM_LDLU(vd + 3584);
    }
    {
      CHEM_PREFETCH(ws + 194880);
      CHEM_PREFETCH(ws + 194912);
      CHEM_PREFETCH(ws + 194944);
      CHEM_PREFETCH(ws + 194976);
      CHEM_PREFETCH(ws + 195008);
      CHEM_PREFETCH(ws + 195040);
      CHEM_PREFETCH(ws + 220096);
      double x = b[3552];
      x = fma(-CHEM_LDLU(lu + 82912), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 82944), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 82976), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 83008), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 83040), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 83072), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 83104), b[6016], x);
      b[3552] = x * CHEM_LDLU(vd + 3552);
    }
    {
      CHEM_PREFETCH(ws + 195072);
      CHEM_PREFETCH(ws + 195104);
      CHEM_PREFETCH(ws + 195136);
      CHEM_PREFETCH(ws + 195168);
      CHEM_PREFETCH(ws + 195200);
      CHEM_PREFETCH(ws + 195232);
      CHEM_PREFETCH(ws + 220064);
      double x = b[3520];
      x = fma(-CHEM_LDLU(lu + 83136), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 83168), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 83200), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 83232), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 83264), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 83296), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 83328), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 83360), b[6016], x);
      b[3520] = x * CHEM_LDLU(vd + 3520);
    }
    {
      CHEM_PREFETCH(ws + 195264);
      CHEM_PREFETCH(ws + 195296);
      CHEM_PREFETCH(ws + 195328);
      CHEM_PREFETCH(ws + 195360);
      CHEM_PREFETCH(ws + 195392);
      CHEM_PREFETCH(ws + 195424);
      CHEM_PREFETCH(ws + 220032);
      double x = b[3488];
      x = fma(-CHEM_LDLU(lu + 83392), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 83424), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 83456), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 83488), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 83520), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 83552), b[6016], x);
      b[3488] = x * CHEM_LDLU(vd + 3488);
    }
    {
      CHEM_PREFETCH(ws + 195456);
      CHEM_PREFETCH(ws + 195488);
      CHEM_PREFETCH(ws + 195520);
      CHEM_PREFETCH(ws + 195552);
      CHEM_PREFETCH(ws + 195584);
      CHEM_PREFETCH(ws + 195616);
      CHEM_PREFETCH(ws + 220000);
      double x = b[3456];
      x = fma(-CHEM_LDLU(lu + 83584), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 83616), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 83648), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 83680), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 83712), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 83744), b[6016], x);
      b[3456] = x * CHEM_LDLU(vd + 3456);
    }
    {
      CHEM_PREFETCH(ws + 195648);
      CHEM_PREFETCH(ws + 195680);
      CHEM_PREFETCH(ws + 195712);
      CHEM_PREFETCH(ws + 195744);
      CHEM_PREFETCH(ws + 195776);
      CHEM_PREFETCH(ws + 195808);
      CHEM_PREFETCH(ws + 195840);
      CHEM_PREFETCH(ws + 219968);
      double x = b[3424];
      x = fma(-CHEM_LDLU(lu + 83776), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 83808), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 83840), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 83872), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 83904), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 83936), b[6016], x);
      b[3424] = x * CHEM_LDLU(vd + 3424);
    }
    {
      CHEM_PREFETCH(ws + 195872);
      CHEM_PREFETCH(ws + 195904);
      CHEM_PREFETCH(ws + 195936);
      CHEM_PREFETCH(ws + 195968);
      CHEM_PREFETCH(ws + 196000);
      CHEM_PREFETCH(ws + 196032);
      CHEM_PREFETCH(ws + 196064);
      CHEM_PREFETCH(ws + 219936);
      double x = b[3392];
      x = fma(-CHEM_LDLU(lu + 83968), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 84000), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 84032), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 84064), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 84096), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 84128), b[6016], x);
      b[3392] = x * CHEM_LDLU(vd + 3392);
    }
    {
      CHEM_PREFETCH(ws + 196096);
      CHEM_PREFETCH(ws + 196128);
      CHEM_PREFETCH(ws + 196160);
      CHEM_PREFETCH(ws + 196192);
      CHEM_PREFETCH(ws + 196224);
      CHEM_PREFETCH(ws + 196256);
      CHEM_PREFETCH(ws + 219904);
      double x = b[3360];
      x = fma(-CHEM_LDLU(lu + 84160), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 84192), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 84224), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 84256), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 84288), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 84320), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 84352), b[6016], x);
      b[3360] = x * CHEM_LDLU(vd + 3360);
    }
    {
      CHEM_PREFETCH(ws + 196288);
      CHEM_PREFETCH(ws + 196320);
      CHEM_PREFETCH(ws + 196352);
      CHEM_PREFETCH(ws + 196384);
      CHEM_PREFETCH(ws + 196416);
      CHEM_PREFETCH(ws + 196448);
      CHEM_PREFETCH(ws + 219872);
      double x = b[3328];
      x = fma(-CHEM_LDLU(lu + 84384), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 84416), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 84448), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 84480), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 84512), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 84544), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 84576), b[6016], x);
      b[3328] = x * CHEM_LDLU(vd + 3328);
    }
    {
      CHEM_PREFETCH(ws + 196480);
      CHEM_PREFETCH(ws + 196512);
      CHEM_PREFETCH(ws + 196544);
      CHEM_PREFETCH(ws + 196576);
      CHEM_PREFETCH(ws + 196608);
      CHEM_PREFETCH(ws + 196640);
      CHEM_PREFETCH(ws + 196672);
      CHEM_PREFETCH(ws + 196704);
      CHEM_PREFETCH(ws + 219840);
      double x = b[3296];
      x = fma(-CHEM_LDLU(lu + 84608), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 84640), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 84672), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 84704), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 84736), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 84768), b[6016], x);
      b[3296] = x * CHEM_LDLU(vd + 3296);
    }
    {
      CHEM_PREFETCH(ws + 196736);
      CHEM_PREFETCH(ws + 196768);
      CHEM_PREFETCH(ws + 196800);
      CHEM_PREFETCH(ws + 196832);
      CHEM_PREFETCH(ws + 196864);
      CHEM_PREFETCH(ws + 196896);
      CHEM_PREFETCH(ws + 196928);
      CHEM_PREFETCH(ws + 219808);
      double x = b[3264];
      x = fma(-CHEM_LDLU(lu + 84800), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 84832), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 84864), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 84896), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 84928), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 84960), b[6016], x);
      b[3264] = x * CHEM_LDLU(vd + 3264);
    }
    {
      CHEM_PREFETCH(ws + 196960);
      CHEM_PREFETCH(ws + 196992);
      CHEM_PREFETCH(ws + 197024);
      CHEM_PREFETCH(ws + 197056);
      CHEM_PREFETCH(ws + 197088);
      CHEM_PREFETCH(ws + 197120);
      CHEM_PREFETCH(ws + 197152);
      CHEM_PREFETCH(ws + 219776);
      double x = b[3232];
      x = fma(-CHEM_LDLU(lu + 84992), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 85024), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 85056), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 85088), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 85120), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 85152), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 85184), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 85216), b[6016], x);
      b[3232] = x * CHEM_LDLU(vd + 3232);
    }
    {
      CHEM_PREFETCH(ws + 197184);
      CHEM_PREFETCH(ws + 197216);
      CHEM_PREFETCH(ws + 197248);
      CHEM_PREFETCH(ws + 197280);
      CHEM_PREFETCH(ws + 197312);
      CHEM_PREFETCH(ws + 197344);
      CHEM_PREFETCH(ws + 197376);
      CHEM_PREFETCH(ws + 219744);
      double x = b[3200];
      x = fma(-CHEM_LDLU(lu + 85248), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 85280), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 85312), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 85344), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 85376), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 85408), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 85440), b[6016], x);
      b[3200] = x * CHEM_LDLU(vd + 3200);
    }
    {
      CHEM_PREFETCH(ws + 197408);
      CHEM_PREFETCH(ws + 197440);
      CHEM_PREFETCH(ws + 197472);
      CHEM_PREFETCH(ws + 197504);
      CHEM_PREFETCH(ws + 197536);
      CHEM_PREFETCH(ws + 197568);
      CHEM_PREFETCH(ws + 219712);
      double x = b[3168];
      x = fma(-CHEM_LDLU(lu + 85472), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 85504), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 85536), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 85568), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 85600), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 85632), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 85664), b[6016], x);
      b[3168] = x * CHEM_LDLU(vd + 3168);
    }
    {
      CHEM_PREFETCH(ws + 197600);
      CHEM_PREFETCH(ws + 197632);
      CHEM_PREFETCH(ws + 197664);
      CHEM_PREFETCH(ws + 197696);
      CHEM_PREFETCH(ws + 197728);
      CHEM_PREFETCH(ws + 197760);
      CHEM_PREFETCH(ws + 197792);
      CHEM_PREFETCH(ws + 197824);
      CHEM_PREFETCH(ws + 197856);
      CHEM_PREFETCH(ws + 219680);
      double x = b[3136];
      x = fma(-CHEM_LDLU(lu + 85696), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 85728), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 85760), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 85792), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 85824), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 85856), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 85888), b[6016], x);
      b[3136] = x * CHEM_LDLU(vd + 3136);
    }
    {
      CHEM_PREFETCH(ws + 197888);
      CHEM_PREFETCH(ws + 197920);
      CHEM_PREFETCH(ws + 197952);
      CHEM_PREFETCH(ws + 197984);
      CHEM_PREFETCH(ws + 198016);
      CHEM_PREFETCH(ws + 198048);
      CHEM_PREFETCH(ws + 198080);
      CHEM_PREFETCH(ws + 219648);
      double x = b[3104];
      x = fma(-CHEM_LDLU(lu + 85920), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 85952), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 85984), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 86016), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 86048), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 86080), b[6016], x);
      b[3104] = x * CHEM_LDLU(vd + 3104);
    }
    {
      CHEM_PREFETCH(ws + 198112);
      CHEM_PREFETCH(ws + 198144);
      CHEM_PREFETCH(ws + 198176);
      CHEM_PREFETCH(ws + 198208);
      CHEM_PREFETCH(ws + 198240);
      CHEM_PREFETCH(ws + 198272);
      CHEM_PREFETCH(ws + 198304);
      CHEM_PREFETCH(ws + 219616);
      double x = b[3072];
      x = fma(-CHEM_LDLU(lu + 86112), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 86144), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 86176), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 86208), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 86240), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 86272), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 86304), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 86336), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 86368), b[6016], x);
      b[3072] = x * CHEM_LDLU(vd + 3072);
    }
    {
      CHEM_PREFETCH(ws + 198336);
      CHEM_PREFETCH(ws + 198368);
      CHEM_PREFETCH(ws + 198400);
      CHEM_PREFETCH(ws + 198432);
      CHEM_PREFETCH(ws + 198464);
      CHEM_PREFETCH(ws + 198496);
      CHEM_PREFETCH(ws + 198528);
      CHEM_PREFETCH(ws + 219584);
      double x = b[3040];
      x = fma(-CHEM_LDLU(lu + 86400), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 86432), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 86464), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 86496), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 86528), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 86560), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 86592), b[5984], x);
      b[3040] = x * CHEM_LDLU(vd + 3040);
    }
    {
      CHEM_PREFETCH(ws + 198560);
      CHEM_PREFETCH(ws + 198592);
      CHEM_PREFETCH(ws + 198624);
      CHEM_PREFETCH(ws + 198656);
      CHEM_PREFETCH(ws + 219552);
      double x = b[3008];
      x = fma(-CHEM_LDLU(lu + 86624), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 86656), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 86688), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 86720), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 86752), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 86784), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 86816), b[6016], x);
      b[3008] = x * CHEM_LDLU(vd + 3008);
    }
    {
      CHEM_PREFETCH(ws + 198688);
      CHEM_PREFETCH(ws + 198720);
      CHEM_PREFETCH(ws + 198752);
      CHEM_PREFETCH(ws + 198784);
      CHEM_PREFETCH(ws + 198816);
      CHEM_PREFETCH(ws + 198848);
      CHEM_PREFETCH(ws + 198880);
      CHEM_PREFETCH(ws + 219520);
      double x = b[2976];
      x = fma(-CHEM_LDLU(lu + 86848), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 86880), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 86912), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 86944), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 86976), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 87008), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 87040), b[6016], x);
      b[2976] = x * CHEM_LDLU(vd + 2976);
    }
    {
      CHEM_PREFETCH(ws + 198912);
      CHEM_PREFETCH(ws + 198944);
      CHEM_PREFETCH(ws + 198976);
      CHEM_PREFETCH(ws + 199008);
      CHEM_PREFETCH(ws + 199040);
      CHEM_PREFETCH(ws + 199072);
      CHEM_PREFETCH(ws + 199104);
      CHEM_PREFETCH(ws + 219488);
      double x = b[2944];
      x = fma(-CHEM_LDLU(lu + 87072), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 87104), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 87136), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 87168), b[6016], x);
      b[2944] = x * CHEM_LDLU(vd + 2944);
    }
    {
      CHEM_PREFETCH(ws + 199136);
      CHEM_PREFETCH(ws + 199168);
      CHEM_PREFETCH(ws + 199200);
      CHEM_PREFETCH(ws + 199232);
      CHEM_PREFETCH(ws + 199264);
      CHEM_PREFETCH(ws + 199296);
      CHEM_PREFETCH(ws + 199328);
      CHEM_PREFETCH(ws + 219456);
      double x = b[2912];
      x = fma(-CHEM_LDLU(lu + 87200), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 87232), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 87264), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 87296), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 87328), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 87360), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 87392), b[6016], x);
      b[2912] = x * CHEM_LDLU(vd + 2912);
    }
    {
      CHEM_PREFETCH(ws + 199360);
      CHEM_PREFETCH(ws + 199392);
      CHEM_PREFETCH(ws + 199424);
      CHEM_PREFETCH(ws + 199456);
      CHEM_PREFETCH(ws + 199488);
      CHEM_PREFETCH(ws + 199520);
      CHEM_PREFETCH(ws + 219424);
      double x = b[2880];
      x = fma(-CHEM_LDLU(lu + 87424), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 87456), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 87488), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 87520), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 87552), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 87584), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 87616), b[6016], x);
      b[2880] = x * CHEM_LDLU(vd + 2880);
    }
    {
      CHEM_PREFETCH(ws + 199552);
      CHEM_PREFETCH(ws + 199584);
      CHEM_PREFETCH(ws + 199616);
      CHEM_PREFETCH(ws + 199648);
      CHEM_PREFETCH(ws + 199680);
      CHEM_PREFETCH(ws + 199712);
      CHEM_PREFETCH(ws + 219392);
      double x = b[2848];
      x = fma(-CHEM_LDLU(lu + 87648), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 87680), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 87712), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 87744), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 87776), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 87808), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 87840), b[6016], x);
      b[2848] = x * CHEM_LDLU(vd + 2848);
    }
    {
      CHEM_PREFETCH(ws + 199744);
      CHEM_PREFETCH(ws + 199776);
      CHEM_PREFETCH(ws + 199808);
      CHEM_PREFETCH(ws + 199840);
      CHEM_PREFETCH(ws + 199872);
      CHEM_PREFETCH(ws + 219360);
      double x = b[2816];
      x = fma(-CHEM_LDLU(lu + 87872), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 87904), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 87936), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 87968), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 88000), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 88032), b[6016], x);
      b[2816] = x * CHEM_LDLU(vd + 2816);
    }
    {
      CHEM_PREFETCH(ws + 199904);
      CHEM_PREFETCH(ws + 199936);
      CHEM_PREFETCH(ws + 199968);
      CHEM_PREFETCH(ws + 200000);
      CHEM_PREFETCH(ws + 200032);
      CHEM_PREFETCH(ws + 200064);
      CHEM_PREFETCH(ws + 200096);
      CHEM_PREFETCH(ws + 219328);
      double x = b[2784];
      x = fma(-CHEM_LDLU(lu + 88064), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 88096), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 88128), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 88160), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 88192), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 88224), b[6016], x);
      b[2784] = x * CHEM_LDLU(vd + 2784);
    }
    {
      CHEM_PREFETCH(ws + 200128);
      CHEM_PREFETCH(ws + 200160);
      CHEM_PREFETCH(ws + 200192);
      CHEM_PREFETCH(ws + 200224);
      CHEM_PREFETCH(ws + 200256);
      CHEM_PREFETCH(ws + 200288);
      CHEM_PREFETCH(ws + 200320);
      CHEM_PREFETCH(ws + 219296);
      double x = b[2752];
      x = fma(-CHEM_LDLU(lu + 88256), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 88288), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 88320), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 88352), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 88384), b[6016], x);
      b[2752] = x * CHEM_LDLU(vd + 2752);
    }
    {
      CHEM_PREFETCH(ws + 200352);
      CHEM_PREFETCH(ws + 200384);
      CHEM_PREFETCH(ws + 200416);
      CHEM_PREFETCH(ws + 200448);
      CHEM_PREFETCH(ws + 200480);
      CHEM_PREFETCH(ws + 200512);
      CHEM_PREFETCH(ws + 200544);
      CHEM_PREFETCH(ws + 219264);
      double x = b[2720];
      x = fma(-CHEM_LDLU(lu + 88416), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 88448), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 88480), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 88512), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 88544), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 88576), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 88608), b[4288], x);
      b[2720] = x * CHEM_LDLU(vd + 2720);
    }
    {
      CHEM_PREFETCH(ws + 200576);
      CHEM_PREFETCH(ws + 200608);
      CHEM_PREFETCH(ws + 200640);
      CHEM_PREFETCH(ws + 200672);
      CHEM_PREFETCH(ws + 200704);
      CHEM_PREFETCH(ws + 200736);
      CHEM_PREFETCH(ws + 200768);
      CHEM_PREFETCH(ws + 219232);
      double x = b[2688];
      x = fma(-CHEM_LDLU(lu + 88640), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 88672), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 88704), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 88736), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 88768), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 88800), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 88832), b[6016], x);
      b[2688] = x * CHEM_LDLU(vd + 2688);
    }
    {
      CHEM_PREFETCH(ws + 200800);
      CHEM_PREFETCH(ws + 200832);
      CHEM_PREFETCH(ws + 200864);
      CHEM_PREFETCH(ws + 200896);
      CHEM_PREFETCH(ws + 200928);
      CHEM_PREFETCH(ws + 200960);
      CHEM_PREFETCH(ws + 219200);
      double x = b[2656];
      x = fma(-CHEM_LDLU(lu + 88864), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 88896), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 88928), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 88960), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 88992), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 89024), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 89056), b[6016], x);
      b[2656] = x * CHEM_LDLU(vd + 2656);
    }
    {
      CHEM_PREFETCH(ws + 200992);
      CHEM_PREFETCH(ws + 201024);
      CHEM_PREFETCH(ws + 201056);
      CHEM_PREFETCH(ws + 201088);
      CHEM_PREFETCH(ws + 201120);
      CHEM_PREFETCH(ws + 201152);
      CHEM_PREFETCH(ws + 219168);
      double x = b[2624];
      x = fma(-CHEM_LDLU(lu + 89088), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 89120), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 89152), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 89184), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 89216), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 89248), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 89280), b[6016], x);
      b[2624] = x * CHEM_LDLU(vd + 2624);
    }
    {
      CHEM_PREFETCH(ws + 201184);
      CHEM_PREFETCH(ws + 201216);
      CHEM_PREFETCH(ws + 201248);
      CHEM_PREFETCH(ws + 201280);
      CHEM_PREFETCH(ws + 219136);
      double x = b[2592];
      x = fma(-CHEM_LDLU(lu + 89312), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 89344), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 89376), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 89408), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 89440), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 89472), b[6016], x);
      b[2592] = x * CHEM_LDLU(vd + 2592);
    }
}
__device__ __noinline__ void solve_1_4(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH(ws + 201312);
      CHEM_PREFETCH(ws + 201344);
      CHEM_PREFETCH(ws + 201376);
      CHEM_PREFETCH(ws + 201408);
      CHEM_PREFETCH(ws + 219104);
      double x = b[2560];
      x = fma(-CHEM_LDLU(lu + 89504), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 89536), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 89568), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 89600), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 89632), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 89664), b[6016], x);
      b[2560] = x * CHEM_LDLU(vd + 2560);
    }
    {
      CHEM_PREFETCH(ws + 201440);
      CHEM_PREFETCH(ws + 201472);
      CHEM_PREFETCH(ws + 201504);
      CHEM_PREFETCH(ws + 201536);
      CHEM_PREFETCH(ws + 219072);
      double x = b[2528];
      x = fma(-CHEM_LDLU(lu + 89696), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 89728), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 89760), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 89792), b[6016], x);
      b[2528] = x * CHEM_LDLU(vd + 2528);
    }
    {
      CHEM_PREFETCH(ws + 201568);
      CHEM_PREFETCH(ws + 201600);
      CHEM_PREFETCH(ws + 201632);
      CHEM_PREFETCH(ws + 201664);
      CHEM_PREFETCH(ws + 219040);
      double x = b[2496];
      x = fma(-CHEM_LDLU(lu + 89824), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 89856), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 89888), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 89920), b[6016], x);
      b[2496] = x * CHEM_LDLU(vd + 2496);
    }
    {
      CHEM_PREFETCH(ws + 201696);
      CHEM_PREFETCH(ws + 201728);
      CHEM_PREFETCH(ws + 201760);
      CHEM_PREFETCH(ws + 201792);
      CHEM_PREFETCH(ws + 219008);
      double x = b[2464];
      x = fma(-CHEM_LDLU(lu + 89952), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 89984), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 90016), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 90048), b[6016], x);
      b[2464] = x * CHEM_LDLU(vd + 2464);
    }
    {
      CHEM_PREFETCH(ws + 201824);
      CHEM_PREFETCH(ws + 201856);
      CHEM_PREFETCH(ws + 201888);
      CHEM_PREFETCH(ws + 201920);
      CHEM_PREFETCH(ws + 218976);
      double x = b[2432];
      x = fma(-CHEM_LDLU(lu + 90080), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 90112), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 90144), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 90176), b[6016], x);
      b[2432] = x * CHEM_LDLU(vd + 2432);
    }
    {
      CHEM_PREFETCH(ws + 201952);
      CHEM_PREFETCH(ws + 201984);
      CHEM_PREFETCH(ws + 202016);
      CHEM_PREFETCH(ws + 218944);
      double x = b[2400];
      x = fma(-CHEM_LDLU(lu + 90208), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 90240), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 90272), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 90304), b[6016], x);
      b[2400] = x * CHEM_LDLU(vd + 2400);
    }
    {
      CHEM_PREFETCH(ws + 202048);
      CHEM_PREFETCH(ws + 202080);
      CHEM_PREFETCH(ws + 202112);
      CHEM_PREFETCH(ws + 202144);
      CHEM_PREFETCH(ws + 202176);
      CHEM_PREFETCH(ws + 218912);
      double x = b[2368];
      x = fma(-CHEM_LDLU(lu + 90336), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 90368), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 90400), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 90432), b[6016], x);
      b[2368] = x * CHEM_LDLU(vd + 2368);
    }
    {
      CHEM_PREFETCH(ws + 202208);
      CHEM_PREFETCH(ws + 202240);
      CHEM_PREFETCH(ws + 202272);
      CHEM_PREFETCH(ws + 202304);
      CHEM_PREFETCH(ws + 202336);
      CHEM_PREFETCH(ws + 218880);
      double x = b[2336];
      x = fma(-CHEM_LDLU(lu + 90464), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 90496), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 90528), b[5920], x);
      b[2336] = x * CHEM_LDLU(vd + 2336);
    }
    {
      CHEM_PREFETCH(ws + 202368);
      CHEM_PREFETCH(ws + 202400);
      CHEM_PREFETCH(ws + 202432);
      CHEM_PREFETCH(ws + 218848);
      double x = b[2304];
      x = fma(-CHEM_LDLU(lu + 90560), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 90592), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 90624), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 90656), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 90688), b[6016], x);
      b[2304] = x * CHEM_LDLU(vd + 2304);
    }
    {
      CHEM_PREFETCH(ws + 202464);
      CHEM_PREFETCH(ws + 202496);
      CHEM_PREFETCH(ws + 202528);
      CHEM_PREFETCH(ws + 202560);
      CHEM_PREFETCH(ws + 202592);
      CHEM_PREFETCH(ws + 202624);
      CHEM_PREFETCH(ws + 218816);
      double x = b[2272];
      x = fma(-CHEM_LDLU(lu + 90720), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 90752), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 90784), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 90816), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 90848), b[5952], x);
      b[2272] = x * CHEM_LDLU(vd + 2272);
    }
    {
      CHEM_PREFETCH(ws + 202656);
      CHEM_PREFETCH(ws + 202688);
      CHEM_PREFETCH(ws + 202720);
      CHEM_PREFETCH(ws + 202752);
      CHEM_PREFETCH(ws + 218784);
      double x = b[2240];
      x = fma(-CHEM_LDLU(lu + 90880), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 90912), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 90944), b[6016], x);
      b[2240] = x * CHEM_LDLU(vd + 2240);
    }
    {
      CHEM_PREFETCH(ws + 202784);
      CHEM_PREFETCH(ws + 202816);
      CHEM_PREFETCH(ws + 202848);
      CHEM_PREFETCH(ws + 202880);
      CHEM_PREFETCH(ws + 218752);
      double x = b[2208];
      x = fma(-CHEM_LDLU(lu + 90976), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 91008), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 91040), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 91072), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91104), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 91136), b[6016], x);
      b[2208] = x * CHEM_LDLU(vd + 2208);
    }
    {
      CHEM_PREFETCH(ws + 202912);
      CHEM_PREFETCH(ws + 202944);
      CHEM_PREFETCH(ws + 202976);
      CHEM_PREFETCH(ws + 203008);
      CHEM_PREFETCH(ws + 218720);
      double x = b[2176];
      x = fma(-CHEM_LDLU(lu + 91168), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 91200), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 91232), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91264), b[6016], x);
      b[2176] = x * CHEM_LDLU(vd + 2176);
    }
    {
      CHEM_PREFETCH(ws + 203040);
      CHEM_PREFETCH(ws + 203072);
      CHEM_PREFETCH(ws + 203104);
      CHEM_PREFETCH(ws + 203136);
      CHEM_PREFETCH(ws + 218688);
      double x = b[2144];
      x = fma(-CHEM_LDLU(lu + 91296), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 91328), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 91360), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91392), b[5984], x);
      b[2144] = x * CHEM_LDLU(vd + 2144);
    }
    {
      CHEM_PREFETCH(ws + 203168);
      CHEM_PREFETCH(ws + 203200);
      CHEM_PREFETCH(ws + 203232);
      CHEM_PREFETCH(ws + 203264);
      CHEM_PREFETCH(ws + 218656);
      double x = b[2112];
      x = fma(-CHEM_LDLU(lu + 91424), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 91456), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 91488), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91520), b[5984], x);
      b[2112] = x * CHEM_LDLU(vd + 2112);
    }
    {
      CHEM_PREFETCH(ws + 203296);
      CHEM_PREFETCH(ws + 203328);
      CHEM_PREFETCH(ws + 203360);
      CHEM_PREFETCH(ws + 203392);
      CHEM_PREFETCH(ws + 218624);
      double x = b[2080];
      x = fma(-CHEM_LDLU(lu + 91552), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 91584), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 91616), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91648), b[5984], x);
      b[2080] = x * CHEM_LDLU(vd + 2080);
    }
    {
      CHEM_PREFETCH(ws + 203424);
      CHEM_PREFETCH(ws + 203456);
      CHEM_PREFETCH(ws + 203488);
      CHEM_PREFETCH(ws + 203520);
      CHEM_PREFETCH(ws + 218592);
      double x = b[2048];
      x = fma(-CHEM_LDLU(lu + 91680), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 91712), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 91744), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91776), b[5984], x);
      b[2048] = x * CHEM_LDLU(vd + 2048);
    }
    {
      CHEM_PREFETCH(ws + 203552);
      CHEM_PREFETCH(ws + 203584);
      CHEM_PREFETCH(ws + 203616);
      CHEM_PREFETCH(ws + 203648);
      CHEM_PREFETCH(ws + 218560);
      double x = b[2016];
      x = fma(-CHEM_LDLU(lu + 91808), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 91840), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 91872), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 91904), b[5984], x);
      b[2016] = x * CHEM_LDLU(vd + 2016);
    }
    {
      CHEM_PREFETCH(ws + 203680);
      CHEM_PREFETCH(ws + 203712);
      CHEM_PREFETCH(ws + 203744);
      CHEM_PREFETCH(ws + 203776);
      CHEM_PREFETCH(ws + 203808);
      CHEM_PREFETCH(ws + 218528);
      double x = b[1984];
      x = fma(-CHEM_LDLU(lu + 91936), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 91968), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 92000), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 92032), b[5984], x);
      b[1984] = x * CHEM_LDLU(vd + 1984);
    }
    {
      CHEM_PREFETCH(ws + 203840);
      CHEM_PREFETCH(ws + 203872);
      CHEM_PREFETCH(ws + 203904);
      CHEM_PREFETCH(ws + 203936);
      CHEM_PREFETCH(ws + 218496);
      double x = b[1952];
      x = fma(-CHEM_LDLU(lu + 92064), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 92096), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 92128), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 92160), b[5984], x);
      b[1952] = x * CHEM_LDLU(vd + 1952);
    }
    {
      CHEM_PREFETCH(ws + 203968);
      CHEM_PREFETCH(ws + 204000);
      CHEM_PREFETCH(ws + 204032);
      CHEM_PREFETCH(ws + 204064);
      CHEM_PREFETCH(ws + 218464);
      double x = b[1920];
      x = fma(-CHEM_LDLU(lu + 92192), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 92224), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 92256), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 92288), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 92320), b[6016], x);
      b[1920] = x * CHEM_LDLU(vd + 1920);
    }
    {
      CHEM_PREFETCH(ws + 204096);
      CHEM_PREFETCH(ws + 204128);
      CHEM_PREFETCH(ws + 204160);
      CHEM_PREFETCH(ws + 204192);
      CHEM_PREFETCH(ws + 218432);
      double x = b[1888];
      x = fma(-CHEM_LDLU(lu + 92352), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 92384), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 92416), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 92448), b[6016], x);
      b[1888] = x * CHEM_LDLU(vd + 1888);
    }
    {
      CHEM_PREFETCH(ws + 204224);
      CHEM_PREFETCH(ws + 204256);
      CHEM_PREFETCH(ws + 204288);
      CHEM_PREFETCH(ws + 204320);
      CHEM_PREFETCH(ws + 218400);
      double x = b[1856];
      x = fma(-CHEM_LDLU(lu + 92480), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 92512), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 92544), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 92576), b[6016], x);
      b[1856] = x * CHEM_LDLU(vd + 1856);
    }
    {
      CHEM_PREFETCH(ws + 204352);
      CHEM_PREFETCH(ws + 204384);
      CHEM_PREFETCH(ws + 204416);
      CHEM_PREFETCH(ws + 204448);
      CHEM_PREFETCH(ws + 204480);
      CHEM_PREFETCH(ws + 218368);
      double x = b[1824];
      x = fma(-CHEM_LDLU(lu + 92608), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 92640), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 92672), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 92704), b[6016], x);
      b[1824] = x * CHEM_LDLU(vd + 1824);
    }
    {
      CHEM_PREFETCH(ws + 204512);
      CHEM_PREFETCH(ws + 204544);
      CHEM_PREFETCH(ws + 204576);
      CHEM_PREFETCH(ws + 204608);
      CHEM_PREFETCH(ws + 218336);
      double x = b[1792];
      x = fma(-CHEM_LDLU(lu + 92736), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 92768), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 92800), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 92832), b[6016], x);
      b[1792] = x * CHEM_LDLU(vd + 1792);
    }
    {
      CHEM_PREFETCH(ws + 204640);
      CHEM_PREFETCH(ws + 204672);
      CHEM_PREFETCH(ws + 204704);
      CHEM_PREFETCH(ws + 204736);
      CHEM_PREFETCH(ws + 218304);
      double x = b[1760];
      x = fma(-CHEM_LDLU(lu + 92864), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 92896), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 92928), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 92960), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 92992), b[6016], x);
      b[1760] = x * CHEM_LDLU(vd + 1760);
    }
    {
      CHEM_PREFETCH(ws + 204768);
      CHEM_PREFETCH(ws + 204800);
      CHEM_PREFETCH(ws + 204832);
      CHEM_PREFETCH(ws + 204864);
      CHEM_PREFETCH(ws + 204896);
      CHEM_PREFETCH(ws + 204928);
      CHEM_PREFETCH(ws + 218272);
      double x = b[1728];
      x = fma(-CHEM_LDLU(lu + 93024), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 93056), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 93088), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 93120), b[6016], x);
      b[1728] = x * CHEM_LDLU(vd + 1728);
    }
    {
      CHEM_PREFETCH(ws + 204960);
      CHEM_PREFETCH(ws + 204992);
      CHEM_PREFETCH(ws + 205024);
      CHEM_PREFETCH(ws + 205056);
      CHEM_PREFETCH(ws + 205088);
      CHEM_PREFETCH(ws + 218240);
      double x = b[1696];
      x = fma(-CHEM_LDLU(lu + 93152), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 93184), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 93216), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 93248), b[6016], x);
      b[1696] = x * CHEM_LDLU(vd + 1696);
    }
    {
      CHEM_PREFETCH(ws + 205120);
      CHEM_PREFETCH(ws + 205152);
      CHEM_PREFETCH(ws + 205184);
      CHEM_PREFETCH(ws + 218208);
      double x = b[1664];
      x = fma(-CHEM_LDLU(lu + 93280), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 93312), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 93344), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 93376), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 93408), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 93440), b[6016], x);
      b[1664] = x * CHEM_LDLU(vd + 1664);
    }
    {
      CHEM_PREFETCH(ws + 205216);
      CHEM_PREFETCH(ws + 205248);
      CHEM_PREFETCH(ws + 205280);
      CHEM_PREFETCH(ws + 218176);
      double x = b[1632];
      x = fma(-CHEM_LDLU(lu + 93472), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 93504), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 93536), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 93568), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 93600), b[6016], x);
      b[1632] = x * CHEM_LDLU(vd + 1632);
    }
    {
      CHEM_PREFETCH(ws + 205312);
      CHEM_PREFETCH(ws + 205344);
      CHEM_PREFETCH(ws + 205376);
      CHEM_PREFETCH(ws + 218144);
      double x = b[1600];
      x = fma(-CHEM_LDLU(lu + 93632), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 93664), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 93696), b[6016], x);
      b[1600] = x * CHEM_LDLU(vd + 1600);
    }
    {
      CHEM_PREFETCH(ws + 205408);
      CHEM_PREFETCH(ws + 205440);
      CHEM_PREFETCH(ws + 205472);
      CHEM_PREFETCH(ws + 218112);
      double x = b[1568];
      x = fma(-CHEM_LDLU(lu + 93728), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 93760), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 93792), b[6016], x);
      b[1568] = x * CHEM_LDLU(vd + 1568);
    }
    {
      CHEM_PREFETCH(ws + 205504);
      CHEM_PREFETCH(ws + 205536);
      CHEM_PREFETCH(ws + 205568);
      CHEM_PREFETCH(ws + 218080);
      double x = b[1536];
      x = fma(-CHEM_LDLU(lu + 93824), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 93856), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 93888), b[6016], x);
      b[1536] = x * CHEM_LDLU(vd + 1536);
    }
    {
      CHEM_PREFETCH(ws + 205600);
      CHEM_PREFETCH(ws + 205632);
      CHEM_PREFETCH(ws + 205664);
      CHEM_PREFETCH(ws + 218048);
      double x = b[1504];
      x = fma(-CHEM_LDLU(lu + 93920), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 93952), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 93984), b[6016], x);
      b[1504] = x * CHEM_LDLU(vd + 1504);
    }
    {
      CHEM_PREFETCH(ws + 205696);
      CHEM_PREFETCH(ws + 205728);
      CHEM_PREFETCH(ws + 205760);
      CHEM_PREFETCH(ws + 218016);
      double x = b[1472];
      x = fma(-CHEM_LDLU(lu + 94016), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 94048), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 94080), b[6016], x);
      b[1472] = x * CHEM_LDLU(vd + 1472);
    }
    {
      CHEM_PREFETCH(ws + 205792);
      CHEM_PREFETCH(ws + 205824);
      CHEM_PREFETCH(ws + 205856);
      CHEM_PREFETCH(ws + 205888);
      CHEM_PREFETCH(ws + 217984);
      double x = b[1440];
      x = fma(-CHEM_LDLU(lu + 94112), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 94144), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 94176), b[6016], x);
      b[1440] = x * CHEM_LDLU(vd + 1440);
    }
    {
      CHEM_PREFETCH(ws + 205920);
      CHEM_PREFETCH(ws + 205952);
      CHEM_PREFETCH(ws + 205984);
      CHEM_PREFETCH(ws + 217952);
      double x = b[1408];
      x = fma(-CHEM_LDLU(lu + 94208), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 94240), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 94272), b[6016], x);
      b[1408] = x * CHEM_LDLU(vd + 1408);
    }
    {
      CHEM_PREFETCH(ws + 206016);
      CHEM_PREFETCH(ws + 206048);
      CHEM_PREFETCH(ws + 206080);
      CHEM_PREFETCH(ws + 217920);
      double x = b[1376];
      x = fma(-CHEM_LDLU(lu + 94304), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 94336), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 94368), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 94400), b[6016], x);
      b[1376] = x * CHEM_LDLU(vd + 1376);
    }
    {
      CHEM_PREFETCH(ws + 206112);
      CHEM_PREFETCH(ws + 206144);
      CHEM_PREFETCH(ws + 206176);
      CHEM_PREFETCH(ws + 217888);
      double x = b[1344];
      x = fma(-CHEM_LDLU(lu + 94432), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 94464), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 94496), b[6016], x);
      b[1344] = x * CHEM_LDLU(vd + 1344);
    }
    {
      CHEM_PREFETCH(ws + 206208);
      CHEM_PREFETCH(ws + 206240);
      CHEM_PREFETCH(ws + 206272);
      CHEM_PREFETCH(ws + 206304);
      CHEM_PREFETCH(ws + 217856);
      double x = b[1312];
      x = fma(-CHEM_LDLU(lu + 94528), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 94560), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 94592), b[6016], x);
      b[1312] = x * CHEM_LDLU(vd + 1312);
    }
    {
      CHEM_PREFETCH(ws + 206336);
      CHEM_PREFETCH(ws + 206368);
      CHEM_PREFETCH(ws + 206400);
      CHEM_PREFETCH(ws + 217824);
      double x = b[1280];
      x = fma(-CHEM_LDLU(lu + 94624), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 94656), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 94688), b[6016], x);
      b[1280] = x * CHEM_LDLU(vd + 1280);
    }
    {
      CHEM_PREFETCH(ws + 206432);
      CHEM_PREFETCH(ws + 206464);
      CHEM_PREFETCH(ws + 206496);
      CHEM_PREFETCH(ws + 217792);
      double x = b[1248];
      x = fma(-CHEM_LDLU(lu + 94720), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 94752), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 94784), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 94816), b[6016], x);
      b[1248] = x * CHEM_LDLU(vd + 1248);
    }
    {
      CHEM_PREFETCH(ws + 206528);
      CHEM_PREFETCH(ws + 206560);
      CHEM_PREFETCH(ws + 206592);
      CHEM_PREFETCH(ws + 217760);
      double x = b[1216];
      x = fma(-CHEM_LDLU(lu + 94848), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 94880), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 94912), b[6016], x);
      b[1216] = x * CHEM_LDLU(vd + 1216);
    }
    {
      CHEM_PREFETCH(ws + 206624);
      CHEM_PREFETCH(ws + 206656);
      CHEM_PREFETCH(ws + 206688);
      CHEM_PREFETCH(ws + 217728);
      double x = b[1184];
      x = fma(-CHEM_LDLU(lu + 94944), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 94976), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 95008), b[6016], x);
      b[1184] = x * CHEM_LDLU(vd + 1184);
    }
    {
      CHEM_PREFETCH(ws + 206720);
      CHEM_PREFETCH(ws + 206752);
      CHEM_PREFETCH(ws + 206784);
      CHEM_PREFETCH(ws + 217696);
      double x = b[1152];
      x = fma(-CHEM_LDLU(lu + 95040), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 95072), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 95104), b[6016], x);
      b[1152] = x * CHEM_LDLU(vd + 1152);
    }
    {
      CHEM_PREFETCH(ws + 206816);
      CHEM_PREFETCH(ws + 217664);
      double x = b[1120];
      x = fma(-CHEM_LDLU(lu + 95136), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 95168), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 95200), b[6016], x);
      b[1120] = x * CHEM_LDLU(vd + 1120);
    }
    {
      CHEM_PREFETCH(ws + 206848);
      CHEM_PREFETCH(ws + 206880);
      CHEM_PREFETCH(ws + 217632);
      double x = b[1088];
      x = fma(-CHEM_LDLU(lu + 95232), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 95264), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 95296), b[6016], x);
      b[1088] = x * CHEM_LDLU(vd + 1088);
    }
    {
      CHEM_PREFETCH(ws + 206912);
      CHEM_PREFETCH(ws + 217600);
      double x = b[1056];
      x = fma(-CHEM_LDLU(lu + 95328), b[1376], x);
      b[1056] = x * CHEM_LDLU(vd + 1056);
    }
    {
      CHEM_PREFETCH(ws + 217568);
      double x = b[1024];
      x = fma(-CHEM_LDLU(lu + 95360), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 95392), b[5952], x);
      b[1024] = x * CHEM_LDLU(vd + 1024);
    }
    {
      CHEM_PREFETCH(ws + 206944);
      CHEM_PREFETCH(ws + 217536);
      double x = b[992];
      x = fma(-CHEM_LDLU(lu + 95424), b[6016], x);
      b[992] = x * CHEM_LDLU(vd + 992);
    }
    {
      CHEM_PREFETCH(ws + 206976);
      CHEM_PREFETCH(ws + 217504);
      double x = b[960];
      b[960] = x * CHEM_LDLU(vd + 960);
    }
    {
      CHEM_PREFETCH(ws + 207008);
      CHEM_PREFETCH(ws + 217472);
      double x = b[928];
      x = fma(-CHEM_LDLU(lu + 95456), b[6016], x);
      b[928] = x * CHEM_LDLU(vd + 928);
    }
    {
      CHEM_PREFETCH(ws + 207040);
      CHEM_PREFETCH(ws + 217440);
      double x = b[896];
      x = fma(-CHEM_LDLU(lu + 95488), b[6016], x);
      b[896] = x * CHEM_LDLU(vd + 896);
    }
    {
      CHEM_PREFETCH(ws + 207072);
      CHEM_PREFETCH(ws + 217408);
      double x = b[864];
      x = fma(-CHEM_LDLU(lu + 95520), b[6016], x);
      b[864] = x * CHEM_LDLU(vd + 864);
    }
    {
      CHEM_PREFETCH(ws + 207104);
      CHEM_PREFETCH(ws + 217376);
      double x = b[832];
      x = fma(-CHEM_LDLU(lu + 95552), b[6016], x);
      b[832] = x * CHEM_LDLU(vd + 832);
    }
    {
      CHEM_PREFETCH(ws + 207136);
      CHEM_PREFETCH(ws + 217344);
      double x = b[800];
      x = fma(-CHEM_LDLU(lu + 95584), b[6016], x);
      b[800] = x * CHEM_LDLU(vd + 800);
    }
    {
      CHEM_PREFETCH(ws + 207168);
      CHEM_PREFETCH(ws + 217312);
      double x = b[768];
      x = fma(-CHEM_LDLU(lu + 95616), b[6016], x);
      b[768] = x * CHEM_LDLU(vd + 768);
    }
    {
      CHEM_PREFETCH(ws + 207200);
      CHEM_PREFETCH(ws + 217280);
      double x = b[736];
      x = fma(-CHEM_LDLU(lu + 95648), b[6016], x);
      b[736] = x * CHEM_LDLU(vd + 736);
    }
    {
      CHEM_PREFETCH(ws + 207232);
      CHEM_PREFETCH(ws + 217248);
      double x = b[704];
      x = fma(-CHEM_LDLU(lu + 95680), b[6016], x);
      b[704] = x * CHEM_LDLU(vd + 704);
    }
    {
      CHEM_PREFETCH(ws + 207264);
      CHEM_PREFETCH(ws + 217216);
      double x = b[672];
      x = fma(-CHEM_LDLU(lu + 95712), b[6016], x);
      b[672] = x * CHEM_LDLU(vd + 672);
    }
    {
      CHEM_PREFETCH(ws + 217184);
      double x = b[640];
      x = fma(-CHEM_LDLU(lu + 95744), b[6016], x);
      b[640] = x * CHEM_LDLU(vd + 640);
    }
    {
      CHEM_PREFETCH(ws + 207296);
      CHEM_PREFETCH(ws + 217152);
      double x = b[608];
      x = fma(-CHEM_LDLU(lu + 95776), b[6016], x);
      b[608] = x * CHEM_LDLU(vd + 608);
    }
    {
      CHEM_PREFETCH(ws + 207328);
      CHEM_PREFETCH(ws + 217120);
      double x = b[576];
      b[576] = x * CHEM_LDLU(vd + 576);
    }
    {
      CHEM_PREFETCH(ws + 207360);
      CHEM_PREFETCH(ws + 207392);
      CHEM_PREFETCH(ws + 217088);
      double x = b[544];
      x = fma(-CHEM_LDLU(lu + 95808), b[1056], x);
      b[544] = x * CHEM_LDLU(vd + 544);
    }
    {
      CHEM_PREFETCH(ws + 207424);
      CHEM_PREFETCH(ws + 217056);
      double x = b[512];
      x = fma(-CHEM_LDLU(lu + 95840), b[1056], x);
      b[512] = x * CHEM_LDLU(vd + 512);
    }
    {
      CHEM_PREFETCH(ws + 207456);
      CHEM_PREFETCH(ws + 217024);
      double x = b[480];
      x = fma(-CHEM_LDLU(lu + 95872), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 95904), b[5376], x);
      b[480] = x * CHEM_LDLU(vd + 480);
    }
    {
      CHEM_PREFETCH(ws + 207488);
      CHEM_PREFETCH(ws + 216992);
      double x = b[448];
      x = fma(-CHEM_LDLU(lu + 95936), b[6016], x);
      b[448] = x * CHEM_LDLU(vd + 448);
    }
    {
      CHEM_PREFETCH(ws + 207520);
      CHEM_PREFETCH(ws + 216960);
      double x = b[416];
      x = fma(-CHEM_LDLU(lu + 95968), b[6016], x);
      b[416] = x * CHEM_LDLU(vd + 416);
    }
    {
      CHEM_PREFETCH(ws + 207552);
      CHEM_PREFETCH(ws + 216928);
      double x = b[384];
      x = fma(-CHEM_LDLU(lu + 96000), b[6016], x);
      b[384] = x * CHEM_LDLU(vd + 384);
    }
    {
      CHEM_PREFETCH(ws + 207584);
      CHEM_PREFETCH(ws + 216896);
      double x = b[352];
      x = fma(-CHEM_LDLU(lu + 96032), b[6016], x);
      b[352] = x * CHEM_LDLU(vd + 352);
    }
    {
      CHEM_PREFETCH(ws + 207616);
      CHEM_PREFETCH(ws + 216864);
      double x = b[320];
      x = fma(-CHEM_LDLU(lu + 96064), b[6016], x);
      b[320] = x * CHEM_LDLU(vd + 320);
    }
    {
      CHEM_PREFETCH(ws + 207648);
      CHEM_PREFETCH(ws + 216832);
      double x = b[288];
      x = fma(-CHEM_LDLU(lu + 96096), b[6016], x);
      b[288] = x * CHEM_LDLU(vd + 288);
    }
    {
      CHEM_PREFETCH(ws + 207680);
      CHEM_PREFETCH(ws + 216800);
      double x = b[256];
      x = fma(-CHEM_LDLU(lu + 96128), b[6016], x);
      b[256] = x * CHEM_LDLU(vd + 256);
    }
    {
      CHEM_PREFETCH(ws + 207712);
      CHEM_PREFETCH(ws + 216768);
      double x = b[224];
      x = fma(-CHEM_LDLU(lu + 96160), b[6016], x);
      b[224] = x * CHEM_LDLU(vd + 224);
    }
    {
      CHEM_PREFETCH(ws + 216736);
      double x = b[192];
      x = fma(-CHEM_LDLU(lu + 96192), b[6016], x);
      b[192] = x * CHEM_LDLU(vd + 192);
    }
    {
      CHEM_PREFETCH(ws + 216704);
      double x = b[160];
      x = fma(-CHEM_LDLU(lu + 96224), b[6016], x);
      b[160] = x * CHEM_LDLU(vd + 160);
    }
    {
      CHEM_PREFETCH(ws + 207744);
      CHEM_PREFETCH(ws + 216672);
      double x = b[128];
      b[128] = x * CHEM_LDLU(vd + 128);
    }
    {
      CHEM_PREFETCH(ws + 207776);
      CHEM_PREFETCH(ws + 216640);
      double x = b[96];
      b[96] = x * CHEM_LDLU(vd + 96);
    }
    {
      CHEM_PREFETCH(ws + 207808);
      CHEM_PREFETCH(ws + 216608);
      double x = b[64];
      x = fma(-CHEM_LDLU(lu + 96256), b[2208], x);
      b[64] = x * CHEM_LDLU(vd + 64);
    }
    {
      double x = b[32];
      x = fma(-CHEM_LDLU(lu + 96288), b[1664], x);
      b[32] = x * CHEM_LDLU(vd + 32);
    }
    {
      double x = b[0];
      x = fma(-CHEM_LDLU(lu + 96320), b[1056], x);
      b[0] = x * CHEM_LDLU(vd + 0);
    }
}
}  // namespace mech_cracmm2
