// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void solve_1_0(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 77632;
    const double* __restrict__ vd = ws + 131712;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH_L1(ws + 77664);
      double x = b[0];
      b[0] = x;
    }
    {
      double x = b[32];
      x = fma(-CHEM_LDLU(lu + 32), b[0], x);
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
      b[192] = x;
    }
    {
      double x = b[224];
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
      CHEM_PREFETCH(ws + 77696);
      double x = b[544];
      b[544] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 77696);
      double x = b[576];
      b[576] = x;
    }
    {
      double x = b[608];
      x = fma(-CHEM_LDLU(lu + 64), b[576], x);
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
      CHEM_PREFETCH(ws + 77728);
      double x = b[736];
      b[736] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 77728);
      double x = b[768];
      b[768] = x;
    }
    {
      double x = b[800];
      x = fma(-CHEM_LDLU(lu + 96), b[768], x);
      b[800] = x;
    }
    {
      double x = b[832];
      b[832] = x;
    }
    {
      CHEM_PREFETCH(ws + 77760);
      double x = b[864];
      b[864] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 77760);
      double x = b[896];
      b[896] = x;
    }
    {
      double x = b[928];
      x = fma(-CHEM_LDLU(lu + 128), b[896], x);
      b[928] = x;
    }
    {
      double x = b[960];
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
      CHEM_PREFETCH(ws + 77792);
      double x = b[1184];
      b[1184] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 77792);
      double x = b[1216];
      b[1216] = x;
    }
    {
      CHEM_PREFETCH(ws + 77824);
      CHEM_PREFETCH(ws + 77856);
      double x = b[1248];
      x = fma(-CHEM_LDLU(lu + 160), b[544], x);
      b[1248] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 77824);
      CHEM_PREFETCH_L1(ws + 77856);
      double x = b[1280];
      b[1280] = x;
    }
    {
      CHEM_PREFETCH(ws + 77888);
      CHEM_PREFETCH(ws + 77920);
      CHEM_PREFETCH(ws + 77952);
      double x = b[1312];
      x = fma(-CHEM_LDLU(lu + 192), b[576], x);
      x = fma(-CHEM_LDLU(lu + 224), b[1056], x);
      b[1312] = x;
    }
    {
      CHEM_PREFETCH(ws + 77984);
      CHEM_PREFETCH(ws + 78016);
      CHEM_PREFETCH(ws + 78048);
      CHEM_PREFETCH_L1(ws + 77888);
      CHEM_PREFETCH_L1(ws + 77920);
      CHEM_PREFETCH_L1(ws + 77952);
      double x = b[1344];
      b[1344] = x;
    }
    {
      CHEM_PREFETCH(ws + 78080);
      CHEM_PREFETCH_L1(ws + 77984);
      CHEM_PREFETCH_L1(ws + 78016);
      CHEM_PREFETCH_L1(ws + 78048);
      double x = b[1376];
      x = fma(-CHEM_LDLU(lu + 256), b[64], x);
      x = fma(-CHEM_LDLU(lu + 288), b[96], x);
      x = fma(-CHEM_LDLU(lu + 320), b[128], x);
      b[1376] = x;
    }
    {
      CHEM_PREFETCH(ws + 78112);
      CHEM_PREFETCH_L1(ws + 78080);
      double x = b[1408];
      x = fma(-CHEM_LDLU(lu + 352), b[160], x);
      x = fma(-CHEM_LDLU(lu + 384), b[192], x);
      x = fma(-CHEM_LDLU(lu + 416), b[224], x);
      b[1408] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78112);
      double x = b[1440];
      x = fma(-CHEM_LDLU(lu + 448), b[704], x);
      b[1440] = x;
    }
    {
      double x = b[1472];
      x = fma(-CHEM_LDLU(lu + 480), b[736], x);
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
      b[1632] = x;
    }
    {
      double x = b[1664];
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
      CHEM_PREFETCH(ws + 78144);
      double x = b[1760];
      b[1760] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78144);
      double x = b[1792];
      b[1792] = x;
    }
    {
      CHEM_PREFETCH(ws + 78176);
      double x = b[1824];
      x = fma(-CHEM_LDLU(lu + 512), b[1216], x);
      b[1824] = x;
    }
    {
      CHEM_PREFETCH(ws + 78208);
      CHEM_PREFETCH(ws + 78240);
      CHEM_PREFETCH(ws + 78272);
      CHEM_PREFETCH_L1(ws + 78176);
      double x = b[1856];
      b[1856] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78208);
      CHEM_PREFETCH_L1(ws + 78240);
      CHEM_PREFETCH_L1(ws + 78272);
      double x = b[1888];
      x = fma(-CHEM_LDLU(lu + 544), b[1856], x);
      b[1888] = x;
    }
    {
      double x = b[1920];
      x = fma(-CHEM_LDLU(lu + 576), b[480], x);
      x = fma(-CHEM_LDLU(lu + 608), b[512], x);
      x = fma(-CHEM_LDLU(lu + 640), b[1280], x);
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
      CHEM_PREFETCH(ws + 78304);
      double x = b[2016];
      b[2016] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78304);
      double x = b[2048];
      b[2048] = x;
    }
    {
      CHEM_PREFETCH(ws + 78336);
      double x = b[2080];
      x = fma(-CHEM_LDLU(lu + 672), b[2048], x);
      b[2080] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78336);
      double x = b[2112];
      b[2112] = x;
    }
    {
      CHEM_PREFETCH(ws + 78368);
      double x = b[2144];
      x = fma(-CHEM_LDLU(lu + 704), b[384], x);
      b[2144] = x;
    }
    {
      CHEM_PREFETCH(ws + 78400);
      CHEM_PREFETCH_L1(ws + 78368);
      double x = b[2176];
      b[2176] = x;
    }
    {
      CHEM_PREFETCH(ws + 78432);
      CHEM_PREFETCH_L1(ws + 78400);
      double x = b[2208];
      x = fma(-CHEM_LDLU(lu + 736), b[2016], x);
      b[2208] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78432);
      double x = b[2240];
      x = fma(-CHEM_LDLU(lu + 768), b[2144], x);
      b[2240] = x;
    }
    {
      double x = b[2272];
      x = fma(-CHEM_LDLU(lu + 800), b[1728], x);
      b[2272] = x;
    }
    {
      double x = b[2304];
      b[2304] = x;
    }
    {
      double x = b[2336];
      b[2336] = x;
    }
    {
      double x = b[2368];
      b[2368] = x;
    }
    {
      double x = b[2400];
      b[2400] = x;
    }
    {
      CHEM_PREFETCH(ws + 78464);
      double x = b[2432];
      b[2432] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78464);
      double x = b[2464];
      b[2464] = x;
    }
    {
      CHEM_PREFETCH(ws + 78496);
      double x = b[2496];
      x = fma(-CHEM_LDLU(lu + 832), b[1120], x);
      b[2496] = x;
    }
    {
      CHEM_PREFETCH(ws + 78528);
      CHEM_PREFETCH(ws + 78560);
      CHEM_PREFETCH(ws + 78592);
      CHEM_PREFETCH(ws + 78624);
      CHEM_PREFETCH(ws + 78656);
      CHEM_PREFETCH(ws + 78688);
      CHEM_PREFETCH_L1(ws + 78496);
      double x = b[2528];
      b[2528] = x;
    }
    {
      CHEM_PREFETCH(ws + 78720);
      CHEM_PREFETCH(ws + 78752);
      CHEM_PREFETCH(ws + 78784);
      CHEM_PREFETCH_L1(ws + 78528);
      CHEM_PREFETCH_L1(ws + 78560);
      CHEM_PREFETCH_L1(ws + 78592);
      CHEM_PREFETCH_L1(ws + 78624);
      CHEM_PREFETCH_L1(ws + 78656);
      CHEM_PREFETCH_L1(ws + 78688);
      double x = b[2560];
      x = fma(-CHEM_LDLU(lu + 864), b[1152], x);
      b[2560] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 78720);
      CHEM_PREFETCH_L1(ws + 78752);
      CHEM_PREFETCH_L1(ws + 78784);
      double x = b[2592];
      x = fma(-CHEM_LDLU(lu + 896), b[480], x);
      x = fma(-CHEM_LDLU(lu + 928), b[512], x);
      x = fma(-CHEM_LDLU(lu + 960), b[544], x);
      x = fma(-CHEM_LDLU(lu + 992), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 1024), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 1056), b[1920], x);
      b[2592] = x;
    }
    {
      double x = b[2624];
      x = fma(-CHEM_LDLU(lu + 1088), b[448], x);
      x = fma(-CHEM_LDLU(lu + 1120), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 1152), b[2560], x);
      b[2624] = x;
    }
    {
      double x = b[2656];
      b[2656] = x;
    }
    {
      CHEM_PREFETCH(ws + 78816);
      CHEM_PREFETCH(ws + 78848);
      double x = b[2688];
      b[2688] = x;
    }
    {
      CHEM_PREFETCH(ws + 78880);
      CHEM_PREFETCH(ws + 78912);
      CHEM_PREFETCH(ws + 78944);
      CHEM_PREFETCH_L1(ws + 78816);
      CHEM_PREFETCH_L1(ws + 78848);
      double x = b[2720];
      b[2720] = x;
    }
    {
      CHEM_PREFETCH(ws + 78976);
      CHEM_PREFETCH(ws + 79008);
      CHEM_PREFETCH(ws + 79040);
      CHEM_PREFETCH(ws + 79072);
      CHEM_PREFETCH_L1(ws + 78880);
      CHEM_PREFETCH_L1(ws + 78912);
      CHEM_PREFETCH_L1(ws + 78944);
      double x = b[2752];
      x = fma(-CHEM_LDLU(lu + 1184), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 1216), b[2304], x);
      b[2752] = x;
    }
    {
      CHEM_PREFETCH(ws + 79104);
      CHEM_PREFETCH_L1(ws + 78976);
      CHEM_PREFETCH_L1(ws + 79008);
      CHEM_PREFETCH_L1(ws + 79040);
      CHEM_PREFETCH_L1(ws + 79072);
      double x = b[2784];
      x = fma(-CHEM_LDLU(lu + 1248), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 1280), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 1312), b[2752], x);
      b[2784] = x;
    }
    {
      CHEM_PREFETCH_L1(ws + 79104);
      double x = b[2816];
      x = fma(-CHEM_LDLU(lu + 1344), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 1376), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 1408), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1440), b[2784], x);
      b[2816] = x;
    }
    {
      double x = b[2848];
      x = fma(-CHEM_LDLU(lu + 1472), b[2048], x);
      b[2848] = x;
    }
    {
      CHEM_PREFETCH(ws + 79136);
      double x = b[2880];
      b[2880] = x;
    }
    {
      CHEM_PREFETCH(ws + 79168);
      CHEM_PREFETCH_L1(ws + 79136);
      double x = b[2912];
      b[2912] = x;
    }
    {
      CHEM_PREFETCH(ws + 79200);
      CHEM_PREFETCH_L1(ws + 79168);
      double x = b[2944];
      x = fma(-CHEM_LDLU(lu + 1504), b[1088], x);
      b[2944] = x;
    }
    {
      CHEM_PREFETCH(ws + 79232);
      CHEM_PREFETCH(ws + 79264);
      CHEM_PREFETCH_L1(ws + 79200);
      double x = b[2976];
      x = fma(-CHEM_LDLU(lu + 1536), b[2400], x);
      b[2976] = x;
    }
    {
      CHEM_PREFETCH(ws + 79296);
      CHEM_PREFETCH(ws + 79328);
      CHEM_PREFETCH(ws + 79360);
      CHEM_PREFETCH(ws + 79392);
      CHEM_PREFETCH(ws + 79424);
      CHEM_PREFETCH_L1(ws + 79232);
      CHEM_PREFETCH_L1(ws + 79264);
      double x = b[3008];
      x = fma(-CHEM_LDLU(lu + 1568), b[1184], x);
      b[3008] = x;
    }
    {
      CHEM_PREFETCH(ws + 79456);
      CHEM_PREFETCH_L1(ws + 79296);
      CHEM_PREFETCH_L1(ws + 79328);
      CHEM_PREFETCH_L1(ws + 79360);
      CHEM_PREFETCH_L1(ws + 79392);
      CHEM_PREFETCH_L1(ws + 79424);
      double x = b[3040];
      x = fma(-CHEM_LDLU(lu + 1600), b[1184], x);
      x = fma(-CHEM_LDLU(lu + 1632), b[3008], x);
      b[3040] = x;
    }
    {
      CHEM_PREFETCH(ws + 79488);
      CHEM_PREFETCH_L1(ws + 79456);
      double x = b[3072];
      x = fma(-CHEM_LDLU(lu + 1664), b[448], x);
      x = fma(-CHEM_LDLU(lu + 1696), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 1728), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 1760), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 1792), b[2944], x);
      b[3072] = x;
    }
    {
      CHEM_PREFETCH(ws + 79520);
      CHEM_PREFETCH(ws + 79552);
      CHEM_PREFETCH(ws + 79584);
      CHEM_PREFETCH(ws + 79616);
      CHEM_PREFETCH_L1(ws + 79488);
      double x = b[3104];
      x = fma(-CHEM_LDLU(lu + 1824), b[384], x);
      b[3104] = x;
    }
    {
      CHEM_PREFETCH(ws + 79648);
      CHEM_PREFETCH(ws + 79680);
      CHEM_PREFETCH(ws + 79712);
      CHEM_PREFETCH(ws + 79744);
      CHEM_PREFETCH(ws + 79776);
      CHEM_PREFETCH_L1(ws + 79520);
      CHEM_PREFETCH_L1(ws + 79552);
      CHEM_PREFETCH_L1(ws + 79584);
      CHEM_PREFETCH_L1(ws + 79616);
      double x = b[3136];
      x = fma(-CHEM_LDLU(lu + 1856), b[1664], x);
      b[3136] = x;
    }
    {
      CHEM_PREFETCH(ws + 79808);
      CHEM_PREFETCH(ws + 79840);
      CHEM_PREFETCH(ws + 79872);
      CHEM_PREFETCH_L1(ws + 79648);
      CHEM_PREFETCH_L1(ws + 79680);
      CHEM_PREFETCH_L1(ws + 79712);
      CHEM_PREFETCH_L1(ws + 79744);
      CHEM_PREFETCH_L1(ws + 79776);
      double x = b[3168];
      x = fma(-CHEM_LDLU(lu + 1888), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1920), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 1952), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 1984), b[2912], x);
      b[3168] = x;
    }
    {
      CHEM_PREFETCH(ws + 79904);
      CHEM_PREFETCH(ws + 79936);
      CHEM_PREFETCH(ws + 79968);
      CHEM_PREFETCH(ws + 80000);
      CHEM_PREFETCH(ws + 80032);
      CHEM_PREFETCH_L1(ws + 79808);
      CHEM_PREFETCH_L1(ws + 79840);
      CHEM_PREFETCH_L1(ws + 79872);
      double x = b[3200];
      x = fma(-CHEM_LDLU(lu + 2016), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 2048), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 2080), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 2112), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 2144), b[3168], x);
      b[3200] = x;
    }
    {
      CHEM_PREFETCH(ws + 80064);
      CHEM_PREFETCH(ws + 80096);
      CHEM_PREFETCH_L1(ws + 79904);
      CHEM_PREFETCH_L1(ws + 79936);
      CHEM_PREFETCH_L1(ws + 79968);
      CHEM_PREFETCH_L1(ws + 80000);
      CHEM_PREFETCH_L1(ws + 80032);
      double x = b[3232];
      x = fma(-CHEM_LDLU(lu + 2176), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 2208), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 2240), b[3136], x);
      b[3232] = x;
    }
    {
      CHEM_PREFETCH(ws + 80128);
      CHEM_PREFETCH(ws + 80160);
      CHEM_PREFETCH_L1(ws + 80064);
      CHEM_PREFETCH_L1(ws + 80096);
      double x = b[3264];
      x = fma(-CHEM_LDLU(lu + 2272), b[448], x);
      x = fma(-CHEM_LDLU(lu + 2304), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 2336), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 2368), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 2400), b[2944], x);
      b[3264] = x;
    }
    {
      CHEM_PREFETCH(ws + 80192);
      CHEM_PREFETCH_L1(ws + 80128);
      CHEM_PREFETCH_L1(ws + 80160);
      double x = b[3296];
      x = fma(-CHEM_LDLU(lu + 2432), b[1056], x);
      x = fma(-CHEM_LDLU(lu + 2464), b[1664], x);
      b[3296] = x;
    }
    {
      CHEM_PREFETCH(ws + 80224);
      CHEM_PREFETCH(ws + 80256);
      CHEM_PREFETCH(ws + 80288);
      CHEM_PREFETCH(ws + 80320);
      CHEM_PREFETCH_L1(ws + 80192);
      double x = b[3328];
      x = fma(-CHEM_LDLU(lu + 2496), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 2528), b[2176], x);
      b[3328] = x;
    }
    {
      CHEM_PREFETCH(ws + 80352);
      CHEM_PREFETCH(ws + 80384);
      CHEM_PREFETCH_L1(ws + 80224);
      CHEM_PREFETCH_L1(ws + 80256);
      CHEM_PREFETCH_L1(ws + 80288);
      CHEM_PREFETCH_L1(ws + 80320);
      double x = b[3360];
      x = fma(-CHEM_LDLU(lu + 2560), b[2848], x);
      b[3360] = x;
    }
    {
      CHEM_PREFETCH(ws + 80416);
      CHEM_PREFETCH(ws + 80448);
      CHEM_PREFETCH(ws + 80480);
      CHEM_PREFETCH_L1(ws + 80352);
      CHEM_PREFETCH_L1(ws + 80384);
      double x = b[3392];
      x = fma(-CHEM_LDLU(lu + 2592), b[896], x);
      x = fma(-CHEM_LDLU(lu + 2624), b[928], x);
      x = fma(-CHEM_LDLU(lu + 2656), b[960], x);
      x = fma(-CHEM_LDLU(lu + 2688), b[1984], x);
      b[3392] = x;
    }
    {
      CHEM_PREFETCH(ws + 80512);
      CHEM_PREFETCH_L1(ws + 80416);
      CHEM_PREFETCH_L1(ws + 80448);
      CHEM_PREFETCH_L1(ws + 80480);
      double x = b[3424];
      x = fma(-CHEM_LDLU(lu + 2720), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 2752), b[2528], x);
      b[3424] = x;
    }
    {
      CHEM_PREFETCH(ws + 80544);
      CHEM_PREFETCH_L1(ws + 80512);
      double x = b[3456];
      x = fma(-CHEM_LDLU(lu + 2784), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 2816), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 2848), b[3424], x);
      b[3456] = x;
    }
    {
      CHEM_PREFETCH(ws + 80576);
      CHEM_PREFETCH(ws + 80608);
      CHEM_PREFETCH(ws + 80640);
      CHEM_PREFETCH_L1(ws + 80544);
      double x = b[3488];
      x = fma(-CHEM_LDLU(lu + 2880), b[1088], x);
      b[3488] = x;
    }
    {
      CHEM_PREFETCH(ws + 80672);
      CHEM_PREFETCH(ws + 80704);
      CHEM_PREFETCH_L1(ws + 80576);
      CHEM_PREFETCH_L1(ws + 80608);
      CHEM_PREFETCH_L1(ws + 80640);
      double x = b[3520];
      x = fma(-CHEM_LDLU(lu + 2912), b[2016], x);
      b[3520] = x;
    }
    {
      CHEM_PREFETCH(ws + 80736);
      CHEM_PREFETCH(ws + 80768);
      CHEM_PREFETCH(ws + 80800);
      CHEM_PREFETCH(ws + 80832);
      CHEM_PREFETCH(ws + 80864);
      CHEM_PREFETCH_L1(ws + 80672);
      CHEM_PREFETCH_L1(ws + 80704);
      double x = b[3552];
      x = fma(-CHEM_LDLU(lu + 2944), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 2976), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 3008), b[3424], x);
      b[3552] = x;
    }
    {
      CHEM_PREFETCH(ws + 80896);
      CHEM_PREFETCH(ws + 80928);
      CHEM_PREFETCH(ws + 80960);
      CHEM_PREFETCH(ws + 80992);
      CHEM_PREFETCH(ws + 81024);
      CHEM_PREFETCH(ws + 81056);
      CHEM_PREFETCH_L1(ws + 80736);
      CHEM_PREFETCH_L1(ws + 80768);
      CHEM_PREFETCH_L1(ws + 80800);
      CHEM_PREFETCH_L1(ws + 80832);
      CHEM_PREFETCH_L1(ws + 80864);
      double x = b[3584];
      x = fma(-CHEM_LDLU(lu + 3040), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 3072), b[1152], x);
      b[3584] = x;
    }
    {
      CHEM_PREFETCH(ws + 81088);
      CHEM_PREFETCH(ws + 81120);
      CHEM_PREFETCH(ws + 81152);
      CHEM_PREFETCH(ws + 81184);
      CHEM_PREFETCH(ws + 81216);
      CHEM_PREFETCH(ws + 81248);
      CHEM_PREFETCH(ws + 81280);
      CHEM_PREFETCH(ws + 81312);
      CHEM_PREFETCH_L1(ws + 80896);
      CHEM_PREFETCH_L1(ws + 80928);
      CHEM_PREFETCH_L1(ws + 80960);
      CHEM_PREFETCH_L1(ws + 80992);
      CHEM_PREFETCH_L1(ws + 81024);
      CHEM_PREFETCH_L1(ws + 81056);
      double x = b[3616];
      x = fma(-CHEM_LDLU(lu + 3104), b[384], x);
      x = fma(-CHEM_LDLU(lu + 3136), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 3168), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 3200), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 3232), b[3328], x);
      b[3616] = x;
    }
    {
      CHEM_PREFETCH(ws + 81344);
      CHEM_PREFETCH(ws + 81376);
      CHEM_PREFETCH(ws + 81408);
      CHEM_PREFETCH(ws + 81440);
      CHEM_PREFETCH(ws + 81472);
      CHEM_PREFETCH(ws + 81504);
      CHEM_PREFETCH(ws + 81536);
      CHEM_PREFETCH(ws + 81568);
      CHEM_PREFETCH(ws + 81600);
      CHEM_PREFETCH_L1(ws + 81088);
      CHEM_PREFETCH_L1(ws + 81120);
      CHEM_PREFETCH_L1(ws + 81152);
      CHEM_PREFETCH_L1(ws + 81184);
      CHEM_PREFETCH_L1(ws + 81216);
      CHEM_PREFETCH_L1(ws + 81248);
      CHEM_PREFETCH_L1(ws + 81280);
      CHEM_PREFETCH_L1(ws + 81312);
      double x = b[3648];
      x = fma(-CHEM_LDLU(lu + 3264), b[960], x);
      x = fma(-CHEM_LDLU(lu + 3296), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 3328), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 3360), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 3392), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 3424), b[3552], x);
      b[3648] = x;
    }
    {
      CHEM_PREFETCH(ws + 81632);
      CHEM_PREFETCH(ws + 81664);
      CHEM_PREFETCH_L1(ws + 81344);
      CHEM_PREFETCH_L1(ws + 81376);
      CHEM_PREFETCH_L1(ws + 81408);
      CHEM_PREFETCH_L1(ws + 81440);
      CHEM_PREFETCH_L1(ws + 81472);
      CHEM_PREFETCH_L1(ws + 81504);
      CHEM_PREFETCH_L1(ws + 81536);
      CHEM_PREFETCH_L1(ws + 81568);
      CHEM_PREFETCH_L1(ws + 81600);
      double x = b[3680];
      x = fma(-CHEM_LDLU(lu + 3456), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 3488), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 3520), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 3552), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 3584), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 3616), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 3648), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 3680), b[3200], x);
      b[3680] = x;
    }
    {
      CHEM_PREFETCH(ws + 81696);
      CHEM_PREFETCH(ws + 81728);
      CHEM_PREFETCH(ws + 81760);
      CHEM_PREFETCH(ws + 81792);
      CHEM_PREFETCH(ws + 81824);
      CHEM_PREFETCH(ws + 81856);
      CHEM_PREFETCH(ws + 81888);
      CHEM_PREFETCH_L1(ws + 81632);
      CHEM_PREFETCH_L1(ws + 81664);
      double x = b[3712];
      x = fma(-CHEM_LDLU(lu + 3712), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 3744), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 3776), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 3808), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 3840), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 3872), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 3904), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 3936), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 3968), b[3680], x);
      b[3712] = x;
    }
    {
      CHEM_PREFETCH(ws + 81920);
      CHEM_PREFETCH(ws + 81952);
      CHEM_PREFETCH(ws + 81984);
      CHEM_PREFETCH(ws + 82016);
      CHEM_PREFETCH_L1(ws + 81696);
      CHEM_PREFETCH_L1(ws + 81728);
      CHEM_PREFETCH_L1(ws + 81760);
      CHEM_PREFETCH_L1(ws + 81792);
      CHEM_PREFETCH_L1(ws + 81824);
      CHEM_PREFETCH_L1(ws + 81856);
      CHEM_PREFETCH_L1(ws + 81888);
      double x = b[3744];
      x = fma(-CHEM_LDLU(lu + 4000), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 4032), b[3616], x);
      b[3744] = x;
    }
    {
      CHEM_PREFETCH(ws + 82048);
      CHEM_PREFETCH(ws + 82080);
      CHEM_PREFETCH(ws + 82112);
      CHEM_PREFETCH(ws + 82144);
      CHEM_PREFETCH(ws + 82176);
      CHEM_PREFETCH_L1(ws + 81920);
      CHEM_PREFETCH_L1(ws + 81952);
      CHEM_PREFETCH_L1(ws + 81984);
      CHEM_PREFETCH_L1(ws + 82016);
      double x = b[3776];
      x = fma(-CHEM_LDLU(lu + 4064), b[352], x);
      x = fma(-CHEM_LDLU(lu + 4096), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 4128), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 4160), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 4192), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 4224), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 4256), b[3552], x);
      b[3776] = x;
    }
    {
      CHEM_PREFETCH(ws + 82208);
      CHEM_PREFETCH(ws + 82240);
      CHEM_PREFETCH(ws + 82272);
      CHEM_PREFETCH_L1(ws + 82048);
      CHEM_PREFETCH_L1(ws + 82080);
      CHEM_PREFETCH_L1(ws + 82112);
      CHEM_PREFETCH_L1(ws + 82144);
      CHEM_PREFETCH_L1(ws + 82176);
      double x = b[3808];
      x = fma(-CHEM_LDLU(lu + 4288), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 4320), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 4352), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 4384), b[3584], x);
      b[3808] = x;
    }
    {
      CHEM_PREFETCH(ws + 82304);
      CHEM_PREFETCH(ws + 82336);
      CHEM_PREFETCH(ws + 82368);
      CHEM_PREFETCH(ws + 82400);
      CHEM_PREFETCH(ws + 82432);
      CHEM_PREFETCH(ws + 82464);
      CHEM_PREFETCH_L1(ws + 82208);
      CHEM_PREFETCH_L1(ws + 82240);
      CHEM_PREFETCH_L1(ws + 82272);
      double x = b[3840];
      x = fma(-CHEM_LDLU(lu + 4416), b[864], x);
      x = fma(-CHEM_LDLU(lu + 4448), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 4480), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 4512), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 4544), b[3424], x);
      b[3840] = x;
    }
    {
      CHEM_PREFETCH(ws + 82496);
      CHEM_PREFETCH(ws + 82528);
      CHEM_PREFETCH(ws + 82560);
      CHEM_PREFETCH(ws + 82592);
      CHEM_PREFETCH(ws + 82624);
      CHEM_PREFETCH(ws + 82656);
      CHEM_PREFETCH(ws + 82688);
      CHEM_PREFETCH_L1(ws + 82304);
      CHEM_PREFETCH_L1(ws + 82336);
      CHEM_PREFETCH_L1(ws + 82368);
      CHEM_PREFETCH_L1(ws + 82400);
      CHEM_PREFETCH_L1(ws + 82432);
      CHEM_PREFETCH_L1(ws + 82464);
      double x = b[3872];
      x = fma(-CHEM_LDLU(lu + 4576), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 4608), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 4640), b[3424], x);
      b[3872] = x;
    }
    {
      CHEM_PREFETCH(ws + 82720);
      CHEM_PREFETCH(ws + 82752);
      CHEM_PREFETCH(ws + 82784);
      CHEM_PREFETCH(ws + 82816);
      CHEM_PREFETCH(ws + 82848);
      CHEM_PREFETCH(ws + 82880);
      CHEM_PREFETCH(ws + 82912);
      CHEM_PREFETCH(ws + 82944);
      CHEM_PREFETCH(ws + 82976);
      CHEM_PREFETCH(ws + 83008);
      CHEM_PREFETCH_L1(ws + 82496);
      CHEM_PREFETCH_L1(ws + 82528);
      CHEM_PREFETCH_L1(ws + 82560);
      CHEM_PREFETCH_L1(ws + 82592);
      CHEM_PREFETCH_L1(ws + 82624);
      CHEM_PREFETCH_L1(ws + 82656);
      CHEM_PREFETCH_L1(ws + 82688);
      double x = b[3904];
      x = fma(-CHEM_LDLU(lu + 4672), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 4704), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 4736), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 4768), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 4800), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 4832), b[3872], x);
      b[3904] = x;
    }
    {
      CHEM_PREFETCH(ws + 83040);
      CHEM_PREFETCH(ws + 83072);
      CHEM_PREFETCH(ws + 83104);
      CHEM_PREFETCH(ws + 83136);
      CHEM_PREFETCH(ws + 83168);
      CHEM_PREFETCH(ws + 83200);
      CHEM_PREFETCH(ws + 83232);
      CHEM_PREFETCH(ws + 83264);
      CHEM_PREFETCH(ws + 83296);
      CHEM_PREFETCH(ws + 83328);
      CHEM_PREFETCH_L1(ws + 82720);
      CHEM_PREFETCH_L1(ws + 82752);
      CHEM_PREFETCH_L1(ws + 82784);
      CHEM_PREFETCH_L1(ws + 82816);
      CHEM_PREFETCH_L1(ws + 82848);
      CHEM_PREFETCH_L1(ws + 82880);
      CHEM_PREFETCH_L1(ws + 82912);
      CHEM_PREFETCH_L1(ws + 82944);
      CHEM_PREFETCH_L1(ws + 82976);
      CHEM_PREFETCH_L1(ws + 83008);
      double x = b[3936];
      x = fma(-CHEM_LDLU(lu + 4864), b[384], x);
      x = fma(-CHEM_LDLU(lu + 4896), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 4928), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 4960), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 4992), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 5024), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 5056), b[3808], x);
      b[3936] = x;
    }
    {
      CHEM_PREFETCH(ws + 83360);
      CHEM_PREFETCH(ws + 83392);
      CHEM_PREFETCH(ws + 83424);
      CHEM_PREFETCH(ws + 83456);
      CHEM_PREFETCH(ws + 83488);
      CHEM_PREFETCH(ws + 83520);
      CHEM_PREFETCH(ws + 83552);
      CHEM_PREFETCH(ws + 83584);
      CHEM_PREFETCH(ws + 83616);
      CHEM_PREFETCH(ws + 83648);
      CHEM_PREFETCH(ws + 83680);
      CHEM_PREFETCH(ws + 83712);
      CHEM_PREFETCH(ws + 83744);
      CHEM_PREFETCH(ws + 83776);
      CHEM_PREFETCH(ws + 83808);
      CHEM_PREFETCH(ws + 83840);
      CHEM_PREFETCH(ws + 83872);
      CHEM_PREFETCH_L1(ws + 83040);
      CHEM_PREFETCH_L1(ws + 83072);
      CHEM_PREFETCH_L1(ws + 83104);
      CHEM_PREFETCH_L1(ws + 83136);
      CHEM_PREFETCH_L1(ws + 83168);
      CHEM_PREFETCH_L1(ws + 83200);
      CHEM_PREFETCH_L1(ws + 83232);
      CHEM_PREFETCH_L1(ws + 83264);
      CHEM_PREFETCH_L1(ws + 83296);
      CHEM_PREFETCH_L1(ws + 83328);
      double x = b[3968];
      x = fma(-CHEM_LDLU(lu + 5088), b[832], x);
      x = fma(-CHEM_LDLU(lu + 5120), b[864], x);
      x = fma(-CHEM_LDLU(lu + 5152), b[896], x);
      x = fma(-CHEM_LDLU(lu + 5184), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 5216), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 5248), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 5280), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 5312), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 5344), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 5376), b[3424], x);
      b[3968] = x;
    }
    {
      CHEM_PREFETCH(ws + 83904);
      CHEM_PREFETCH(ws + 83936);
      CHEM_PREFETCH(ws + 83968);
      CHEM_PREFETCH(ws + 84000);
      CHEM_PREFETCH(ws + 84032);
      CHEM_PREFETCH(ws + 84064);
      CHEM_PREFETCH(ws + 84096);
      CHEM_PREFETCH(ws + 84128);
      CHEM_PREFETCH(ws + 84160);
      CHEM_PREFETCH(ws + 84192);
      CHEM_PREFETCH(ws + 84224);
      CHEM_PREFETCH(ws + 84256);
      CHEM_PREFETCH(ws + 84288);
      CHEM_PREFETCH(ws + 84320);
      CHEM_PREFETCH_L1(ws + 83360);
      CHEM_PREFETCH_L1(ws + 83392);
      CHEM_PREFETCH_L1(ws + 83424);
      CHEM_PREFETCH_L1(ws + 83456);
      CHEM_PREFETCH_L1(ws + 83488);
      CHEM_PREFETCH_L1(ws + 83520);
      CHEM_PREFETCH_L1(ws + 83552);
      CHEM_PREFETCH_L1(ws + 83584);
      CHEM_PREFETCH_L1(ws + 83616);
      CHEM_PREFETCH_L1(ws + 83648);
      CHEM_PREFETCH_L1(ws + 83680);
      CHEM_PREFETCH_L1(ws + 83712);
      CHEM_PREFETCH_L1(ws + 83744);
      CHEM_PREFETCH_L1(ws + 83776);
      CHEM_PREFETCH_L1(ws + 83808);
      CHEM_PREFETCH_L1(ws + 83840);
      CHEM_PREFETCH_L1(ws + 83872);
      double x = b[4000];
      x = fma(-CHEM_LDLU(lu + 5408), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 5440), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 5472), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 5504), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 5536), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 5568), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 5600), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 5632), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 5664), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 5696), b[3936], x);
      b[4000] = x;
    }
    {
      CHEM_PREFETCH(ws + 84352);
      CHEM_PREFETCH(ws + 84384);
      CHEM_PREFETCH(ws + 84416);
      CHEM_PREFETCH(ws + 84448);
      CHEM_PREFETCH(ws + 84480);
      CHEM_PREFETCH(ws + 84512);
      CHEM_PREFETCH(ws + 84544);
      CHEM_PREFETCH(ws + 84576);
      CHEM_PREFETCH_L1(ws + 83904);
      CHEM_PREFETCH_L1(ws + 83936);
      CHEM_PREFETCH_L1(ws + 83968);
      CHEM_PREFETCH_L1(ws + 84000);
      CHEM_PREFETCH_L1(ws + 84032);
      CHEM_PREFETCH_L1(ws + 84064);
      CHEM_PREFETCH_L1(ws + 84096);
      CHEM_PREFETCH_L1(ws + 84128);
      CHEM_PREFETCH_L1(ws + 84160);
      CHEM_PREFETCH_L1(ws + 84192);
      CHEM_PREFETCH_L1(ws + 84224);
      CHEM_PREFETCH_L1(ws + 84256);
      CHEM_PREFETCH_L1(ws + 84288);
      CHEM_PREFETCH_L1(ws + 84320);
      double x = b[4032];
      x = fma(-CHEM_LDLU(lu + 5728), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 5760), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 5792), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 5824), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 5856), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 5888), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 5920), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 5952), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 5984), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 6016), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 6048), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 6080), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 6112), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 6144), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 6176), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 6208), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 6240), b[3936], x);
      b[4032] = x;
    }
    {
      CHEM_PREFETCH(ws + 84608);
      CHEM_PREFETCH(ws + 84640);
      CHEM_PREFETCH(ws + 84672);
      CHEM_PREFETCH(ws + 84704);
      CHEM_PREFETCH(ws + 84736);
      CHEM_PREFETCH(ws + 84768);
      CHEM_PREFETCH(ws + 84800);
      CHEM_PREFETCH(ws + 84832);
      CHEM_PREFETCH(ws + 84864);
      CHEM_PREFETCH(ws + 84896);
      CHEM_PREFETCH(ws + 84928);
      CHEM_PREFETCH(ws + 84960);
      CHEM_PREFETCH_L1(ws + 84352);
      CHEM_PREFETCH_L1(ws + 84384);
      CHEM_PREFETCH_L1(ws + 84416);
      CHEM_PREFETCH_L1(ws + 84448);
      CHEM_PREFETCH_L1(ws + 84480);
      CHEM_PREFETCH_L1(ws + 84512);
      CHEM_PREFETCH_L1(ws + 84544);
      CHEM_PREFETCH_L1(ws + 84576);
      double x = b[4064];
      x = fma(-CHEM_LDLU(lu + 6272), b[928], x);
      x = fma(-CHEM_LDLU(lu + 6304), b[960], x);
      x = fma(-CHEM_LDLU(lu + 6336), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 6368), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 6400), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 6432), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 6464), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 6496), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 6528), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 6560), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 6592), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 6624), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 6656), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 6688), b[3936], x);
      b[4064] = x;
    }
    {
      CHEM_PREFETCH(ws + 84992);
      CHEM_PREFETCH(ws + 85024);
      CHEM_PREFETCH(ws + 85056);
      CHEM_PREFETCH(ws + 85088);
      CHEM_PREFETCH(ws + 85120);
      CHEM_PREFETCH(ws + 85152);
      CHEM_PREFETCH(ws + 85184);
      CHEM_PREFETCH(ws + 85216);
      CHEM_PREFETCH(ws + 85248);
      CHEM_PREFETCH(ws + 85280);
      CHEM_PREFETCH(ws + 85312);
      CHEM_PREFETCH(ws + 85344);
      CHEM_PREFETCH(ws + 85376);
      CHEM_PREFETCH(ws + 85408);
      CHEM_PREFETCH_L1(ws + 84608);
      CHEM_PREFETCH_L1(ws + 84640);
      CHEM_PREFETCH_L1(ws + 84672);
      CHEM_PREFETCH_L1(ws + 84704);
      CHEM_PREFETCH_L1(ws + 84736);
      CHEM_PREFETCH_L1(ws + 84768);
      CHEM_PREFETCH_L1(ws + 84800);
      CHEM_PREFETCH_L1(ws + 84832);
      CHEM_PREFETCH_L1(ws + 84864);
      CHEM_PREFETCH_L1(ws + 84896);
      CHEM_PREFETCH_L1(ws + 84928);
      CHEM_PREFETCH_L1(ws + 84960);
      double x = b[4096];
      x = fma(-CHEM_LDLU(lu + 6720), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 6752), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 6784), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 6816), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 6848), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 6880), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 6912), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 6944), b[4064], x);
      b[4096] = x;
    }
    {
      CHEM_PREFETCH(ws + 85440);
      CHEM_PREFETCH(ws + 85472);
      CHEM_PREFETCH(ws + 85504);
      CHEM_PREFETCH(ws + 85536);
      CHEM_PREFETCH(ws + 85568);
      CHEM_PREFETCH(ws + 85600);
      CHEM_PREFETCH(ws + 85632);
      CHEM_PREFETCH(ws + 85664);
      CHEM_PREFETCH(ws + 85696);
      CHEM_PREFETCH(ws + 85728);
      CHEM_PREFETCH(ws + 85760);
      CHEM_PREFETCH(ws + 85792);
      CHEM_PREFETCH(ws + 85824);
      CHEM_PREFETCH(ws + 85856);
      CHEM_PREFETCH(ws + 85888);
      CHEM_PREFETCH(ws + 85920);
      CHEM_PREFETCH(ws + 85952);
      CHEM_PREFETCH(ws + 85984);
      CHEM_PREFETCH(ws + 86016);
      CHEM_PREFETCH(ws + 86048);
      CHEM_PREFETCH_L1(ws + 84992);
      CHEM_PREFETCH_L1(ws + 85024);
      CHEM_PREFETCH_L1(ws + 85056);
      CHEM_PREFETCH_L1(ws + 85088);
      CHEM_PREFETCH_L1(ws + 85120);
      CHEM_PREFETCH_L1(ws + 85152);
      CHEM_PREFETCH_L1(ws + 85184);
      CHEM_PREFETCH_L1(ws + 85216);
      CHEM_PREFETCH_L1(ws + 85248);
      CHEM_PREFETCH_L1(ws + 85280);
      CHEM_PREFETCH_L1(ws + 85312);
      CHEM_PREFETCH_L1(ws + 85344);
      CHEM_PREFETCH_L1(ws + 85376);
      CHEM_PREFETCH_L1(ws + 85408);
      double x = b[4128];
      x = fma(-CHEM_LDLU(lu + 6976), b[832], x);
      x = fma(-CHEM_LDLU(lu + 7008), b[864], x);
      x = fma(-CHEM_LDLU(lu + 7040), b[960], x);
      x = fma(-CHEM_LDLU(lu + 7072), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 7104), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 7136), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 7168), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 7200), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 7232), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 7264), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 7296), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 7328), b[4096], x);
      b[4128] = x;
    }
    {
      CHEM_PREFETCH(ws + 86080);
      CHEM_PREFETCH(ws + 86112);
      CHEM_PREFETCH(ws + 86144);
      CHEM_PREFETCH(ws + 86176);
      CHEM_PREFETCH(ws + 86208);
      CHEM_PREFETCH(ws + 86240);
      CHEM_PREFETCH(ws + 86272);
      CHEM_PREFETCH(ws + 86304);
      CHEM_PREFETCH(ws + 86336);
      CHEM_PREFETCH(ws + 86368);
      CHEM_PREFETCH(ws + 86400);
      CHEM_PREFETCH(ws + 86432);
      CHEM_PREFETCH(ws + 86464);
      CHEM_PREFETCH_L1(ws + 85440);
      CHEM_PREFETCH_L1(ws + 85472);
      CHEM_PREFETCH_L1(ws + 85504);
      CHEM_PREFETCH_L1(ws + 85536);
      CHEM_PREFETCH_L1(ws + 85568);
      CHEM_PREFETCH_L1(ws + 85600);
      CHEM_PREFETCH_L1(ws + 85632);
      CHEM_PREFETCH_L1(ws + 85664);
      CHEM_PREFETCH_L1(ws + 85696);
      CHEM_PREFETCH_L1(ws + 85728);
      CHEM_PREFETCH_L1(ws + 85760);
      CHEM_PREFETCH_L1(ws + 85792);
      CHEM_PREFETCH_L1(ws + 85824);
      CHEM_PREFETCH_L1(ws + 85856);
      CHEM_PREFETCH_L1(ws + 85888);
      CHEM_PREFETCH_L1(ws + 85920);
      CHEM_PREFETCH_L1(ws + 85952);
      CHEM_PREFETCH_L1(ws + 85984);
      CHEM_PREFETCH_L1(ws + 86016);
      CHEM_PREFETCH_L1(ws + 86048);
      double x = b[4160];
      x = fma(-CHEM_LDLU(lu + 7360), b[672], x);
      x = fma(-CHEM_LDLU(lu + 7392), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 7424), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 7456), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 7488), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 7520), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 7552), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 7584), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 7616), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 7648), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 7680), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 7712), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 7744), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 7776), b[4128], x);
      b[4160] = x;
    }
    {
      CHEM_PREFETCH(ws + 86496);
      CHEM_PREFETCH(ws + 86528);
      CHEM_PREFETCH(ws + 86560);
      CHEM_PREFETCH(ws + 86592);
      CHEM_PREFETCH(ws + 86624);
      CHEM_PREFETCH(ws + 86656);
      CHEM_PREFETCH(ws + 86688);
      CHEM_PREFETCH(ws + 86720);
      CHEM_PREFETCH(ws + 86752);
      CHEM_PREFETCH(ws + 86784);
      CHEM_PREFETCH(ws + 86816);
      CHEM_PREFETCH(ws + 86848);
      CHEM_PREFETCH(ws + 86880);
      CHEM_PREFETCH(ws + 86912);
      CHEM_PREFETCH(ws + 86944);
      CHEM_PREFETCH(ws + 86976);
      CHEM_PREFETCH(ws + 87008);
      CHEM_PREFETCH_L1(ws + 86080);
      CHEM_PREFETCH_L1(ws + 86112);
      CHEM_PREFETCH_L1(ws + 86144);
      CHEM_PREFETCH_L1(ws + 86176);
      CHEM_PREFETCH_L1(ws + 86208);
      CHEM_PREFETCH_L1(ws + 86240);
      CHEM_PREFETCH_L1(ws + 86272);
      CHEM_PREFETCH_L1(ws + 86304);
      CHEM_PREFETCH_L1(ws + 86336);
      CHEM_PREFETCH_L1(ws + 86368);
      CHEM_PREFETCH_L1(ws + 86400);
      CHEM_PREFETCH_L1(ws + 86432);
      CHEM_PREFETCH_L1(ws + 86464);
      double x = b[4192];
      x = fma(-CHEM_LDLU(lu + 7808), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 7840), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 7872), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 7904), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 7936), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 7968), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 8000), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 8032), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 8064), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 8096), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 8128), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 8160), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 8192), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 8224), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 8256), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 8288), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 8320), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 8352), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 8384), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 8416), b[4160], x);
      b[4192] = x;
    }
    {
      CHEM_PREFETCH(ws + 87040);
      CHEM_PREFETCH(ws + 87072);
      CHEM_PREFETCH(ws + 87104);
      CHEM_PREFETCH(ws + 87136);
      CHEM_PREFETCH(ws + 87168);
      CHEM_PREFETCH(ws + 87200);
      CHEM_PREFETCH(ws + 87232);
      CHEM_PREFETCH(ws + 87264);
      CHEM_PREFETCH(ws + 87296);
      CHEM_PREFETCH(ws + 87328);
      CHEM_PREFETCH(ws + 87360);
      CHEM_PREFETCH(ws + 87392);
      CHEM_PREFETCH(ws + 87424);
      CHEM_PREFETCH(ws + 87456);
      CHEM_PREFETCH(ws + 87488);
      CHEM_PREFETCH(ws + 87520);
      CHEM_PREFETCH(ws + 87552);
      CHEM_PREFETCH_L1(ws + 86496);
      CHEM_PREFETCH_L1(ws + 86528);
      CHEM_PREFETCH_L1(ws + 86560);
      CHEM_PREFETCH_L1(ws + 86592);
      CHEM_PREFETCH_L1(ws + 86624);
      CHEM_PREFETCH_L1(ws + 86656);
      CHEM_PREFETCH_L1(ws + 86688);
      CHEM_PREFETCH_L1(ws + 86720);
      CHEM_PREFETCH_L1(ws + 86752);
      CHEM_PREFETCH_L1(ws + 86784);
      CHEM_PREFETCH_L1(ws + 86816);
      CHEM_PREFETCH_L1(ws + 86848);
      CHEM_PREFETCH_L1(ws + 86880);
      CHEM_PREFETCH_L1(ws + 86912);
      CHEM_PREFETCH_L1(ws + 86944);
      CHEM_PREFETCH_L1(ws + 86976);
      CHEM_PREFETCH_L1(ws + 87008);
      double x = b[4224];
      x = fma(-CHEM_LDLU(lu + 8448), b[928], x);
      x = fma(-CHEM_LDLU(lu + 8480), b[960], x);
      x = fma(-CHEM_LDLU(lu + 8512), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 8544), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 8576), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 8608), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 8640), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 8672), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 8704), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 8736), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 8768), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 8800), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 8832), b[4160], x);
      b[4224] = x;
    }
    {
      CHEM_PREFETCH(ws + 87584);
      CHEM_PREFETCH(ws + 87616);
      CHEM_PREFETCH(ws + 87648);
      CHEM_PREFETCH(ws + 87680);
      CHEM_PREFETCH(ws + 87712);
      CHEM_PREFETCH(ws + 87744);
      CHEM_PREFETCH(ws + 87776);
      CHEM_PREFETCH(ws + 87808);
      CHEM_PREFETCH(ws + 87840);
      CHEM_PREFETCH(ws + 87872);
      CHEM_PREFETCH(ws + 87904);
      CHEM_PREFETCH(ws + 87936);
      CHEM_PREFETCH(ws + 87968);
      CHEM_PREFETCH(ws + 88000);
      CHEM_PREFETCH(ws + 88032);
      CHEM_PREFETCH(ws + 88064);
      CHEM_PREFETCH(ws + 88096);
      CHEM_PREFETCH(ws + 88128);
      CHEM_PREFETCH(ws + 88160);
      CHEM_PREFETCH(ws + 88192);
      CHEM_PREFETCH(ws + 88224);
      CHEM_PREFETCH_L1(ws + 87040);
      CHEM_PREFETCH_L1(ws + 87072);
      CHEM_PREFETCH_L1(ws + 87104);
      CHEM_PREFETCH_L1(ws + 87136);
      CHEM_PREFETCH_L1(ws + 87168);
      CHEM_PREFETCH_L1(ws + 87200);
      CHEM_PREFETCH_L1(ws + 87232);
      CHEM_PREFETCH_L1(ws + 87264);
      CHEM_PREFETCH_L1(ws + 87296);
      CHEM_PREFETCH_L1(ws + 87328);
      CHEM_PREFETCH_L1(ws + 87360);
      CHEM_PREFETCH_L1(ws + 87392);
      CHEM_PREFETCH_L1(ws + 87424);
      CHEM_PREFETCH_L1(ws + 87456);
      CHEM_PREFETCH_L1(ws + 87488);
      CHEM_PREFETCH_L1(ws + 87520);
      CHEM_PREFETCH_L1(ws + 87552);
      double x = b[4256];
      x = fma(-CHEM_LDLU(lu + 8864), b[352], x);
      x = fma(-CHEM_LDLU(lu + 8896), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 8928), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 8960), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 8992), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 9024), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 9056), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 9088), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 9120), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 9152), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 9184), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 9216), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 9248), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 9280), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 9312), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 9344), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 9376), b[4224], x);
      b[4256] = x;
    }
    {
      CHEM_PREFETCH(ws + 88256);
      CHEM_PREFETCH(ws + 88288);
      CHEM_PREFETCH(ws + 88320);
      CHEM_PREFETCH(ws + 88352);
      CHEM_PREFETCH(ws + 88384);
      CHEM_PREFETCH(ws + 88416);
      CHEM_PREFETCH(ws + 88448);
      CHEM_PREFETCH(ws + 88480);
      CHEM_PREFETCH(ws + 88512);
      CHEM_PREFETCH(ws + 88544);
      CHEM_PREFETCH(ws + 88576);
      CHEM_PREFETCH(ws + 88608);
      CHEM_PREFETCH(ws + 88640);
      CHEM_PREFETCH(ws + 88672);
      CHEM_PREFETCH(ws + 88704);
      CHEM_PREFETCH(ws + 88736);
      CHEM_PREFETCH(ws + 88768);
      CHEM_PREFETCH(ws + 88800);
      CHEM_PREFETCH(ws + 88832);
      CHEM_PREFETCH(ws + 88864);
      CHEM_PREFETCH_L1(ws + 87584);
      CHEM_PREFETCH_L1(ws + 87616);
      CHEM_PREFETCH_L1(ws + 87648);
      CHEM_PREFETCH_L1(ws + 87680);
      CHEM_PREFETCH_L1(ws + 87712);
      CHEM_PREFETCH_L1(ws + 87744);
      CHEM_PREFETCH_L1(ws + 87776);
      CHEM_PREFETCH_L1(ws + 87808);
      CHEM_PREFETCH_L1(ws + 87840);
      CHEM_PREFETCH_L1(ws + 87872);
      CHEM_PREFETCH_L1(ws + 87904);
      CHEM_PREFETCH_L1(ws + 87936);
      CHEM_PREFETCH_L1(ws + 87968);
      CHEM_PREFETCH_L1(ws + 88000);
      CHEM_PREFETCH_L1(ws + 88032);
      CHEM_PREFETCH_L1(ws + 88064);
      CHEM_PREFETCH_L1(ws + 88096);
      CHEM_PREFETCH_L1(ws + 88128);
      CHEM_PREFETCH_L1(ws + 88160);
      CHEM_PREFETCH_L1(ws + 88192);
      CHEM_PREFETCH_L1(ws + 88224);
      double x = b[4288];
      x = fma(-CHEM_LDLU(lu + 9408), b[832], x);
      x = fma(-CHEM_LDLU(lu + 9440), b[896], x);
      x = fma(-CHEM_LDLU(lu + 9472), b[928], x);
      x = fma(-CHEM_LDLU(lu + 9504), b[960], x);
      x = fma(-CHEM_LDLU(lu + 9536), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 9568), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 9600), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 9632), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 9664), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 9696), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 9728), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 9760), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 9792), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 9824), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 9856), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 9888), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 9920), b[4224], x);
      b[4288] = x;
    }
    {
      CHEM_PREFETCH(ws + 88896);
      CHEM_PREFETCH(ws + 88928);
      CHEM_PREFETCH(ws + 88960);
      CHEM_PREFETCH(ws + 88992);
      CHEM_PREFETCH(ws + 89024);
      CHEM_PREFETCH(ws + 89056);
      CHEM_PREFETCH(ws + 89088);
      CHEM_PREFETCH(ws + 89120);
      CHEM_PREFETCH(ws + 89152);
      CHEM_PREFETCH(ws + 89184);
      CHEM_PREFETCH(ws + 89216);
      CHEM_PREFETCH(ws + 89248);
      CHEM_PREFETCH(ws + 89280);
      CHEM_PREFETCH(ws + 89312);
      CHEM_PREFETCH(ws + 89344);
      CHEM_PREFETCH(ws + 89376);
      CHEM_PREFETCH(ws + 89408);
      CHEM_PREFETCH(ws + 89440);
      CHEM_PREFETCH(ws + 89472);
      CHEM_PREFETCH(ws + 89504);
      CHEM_PREFETCH(ws + 89536);
      CHEM_PREFETCH(ws + 89568);
      CHEM_PREFETCH_L1(ws + 88256);
      CHEM_PREFETCH_L1(ws + 88288);
      CHEM_PREFETCH_L1(ws + 88320);
      CHEM_PREFETCH_L1(ws + 88352);
      CHEM_PREFETCH_L1(ws + 88384);
      CHEM_PREFETCH_L1(ws + 88416);
      CHEM_PREFETCH_L1(ws + 88448);
      CHEM_PREFETCH_L1(ws + 88480);
      CHEM_PREFETCH_L1(ws + 88512);
      CHEM_PREFETCH_L1(ws + 88544);
      CHEM_PREFETCH_L1(ws + 88576);
      CHEM_PREFETCH_L1(ws + 88608);
      CHEM_PREFETCH_L1(ws + 88640);
      CHEM_PREFETCH_L1(ws + 88672);
      CHEM_PREFETCH_L1(ws + 88704);
      CHEM_PREFETCH_L1(ws + 88736);
      CHEM_PREFETCH_L1(ws + 88768);
      CHEM_PREFETCH_L1(ws + 88800);
      CHEM_PREFETCH_L1(ws + 88832);
      CHEM_PREFETCH_L1(ws + 88864);
      double x = b[4320];
      x = fma(-CHEM_LDLU(lu + 9952), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 9984), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 10016), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 10048), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 10080), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 10112), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 10144), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 10176), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 10208), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 10240), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 10272), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 10304), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 10336), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 10368), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 10400), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 10432), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 10464), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 10496), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 10528), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 10560), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 10592), b[4224], x);
      b[4320] = x;
    }
    {
      CHEM_PREFETCH(ws + 89600);
      CHEM_PREFETCH(ws + 89632);
      CHEM_PREFETCH(ws + 89664);
      CHEM_PREFETCH(ws + 89696);
      CHEM_PREFETCH(ws + 89728);
      CHEM_PREFETCH(ws + 89760);
      CHEM_PREFETCH(ws + 89792);
      CHEM_PREFETCH(ws + 89824);
      CHEM_PREFETCH(ws + 89856);
      CHEM_PREFETCH(ws + 89888);
      CHEM_PREFETCH(ws + 89920);
      CHEM_PREFETCH(ws + 89952);
      CHEM_PREFETCH(ws + 89984);
      CHEM_PREFETCH(ws + 90016);
      CHEM_PREFETCH(ws + 90048);
      CHEM_PREFETCH(ws + 90080);
      CHEM_PREFETCH(ws + 90112);
      CHEM_PREFETCH(ws + 90144);
      CHEM_PREFETCH(ws + 90176);
      CHEM_PREFETCH(ws + 90208);
      CHEM_PREFETCH_L1(ws + 88896);
      CHEM_PREFETCH_L1(ws + 88928);
      CHEM_PREFETCH_L1(ws + 88960);
      CHEM_PREFETCH_L1(ws + 88992);
      CHEM_PREFETCH_L1(ws + 89024);
      CHEM_PREFETCH_L1(ws + 89056);
      CHEM_PREFETCH_L1(ws + 89088);
      CHEM_PREFETCH_L1(ws + 89120);
      CHEM_PREFETCH_L1(ws + 89152);
      CHEM_PREFETCH_L1(ws + 89184);
      CHEM_PREFETCH_L1(ws + 89216);
      CHEM_PREFETCH_L1(ws + 89248);
      CHEM_PREFETCH_L1(ws + 89280);
      CHEM_PREFETCH_L1(ws + 89312);
      CHEM_PREFETCH_L1(ws + 89344);
      CHEM_PREFETCH_L1(ws + 89376);
      CHEM_PREFETCH_L1(ws + 89408);
      CHEM_PREFETCH_L1(ws + 89440);
      CHEM_PREFETCH_L1(ws + 89472);
      CHEM_PREFETCH_L1(ws + 89504);
      CHEM_PREFETCH_L1(ws + 89536);
      CHEM_PREFETCH_L1(ws + 89568);
      double x = b[4352];
      x = fma(-CHEM_LDLU(lu + 10624), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 10656), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 10688), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 10720), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 10752), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 10784), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 10816), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 10848), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 10880), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 10912), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 10944), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 10976), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 11008), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 11040), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 11072), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 11104), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 11136), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 11168), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 11200), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 11232), b[4320], x);
      b[4352] = x;
    }
    {
      CHEM_PREFETCH(ws + 90240);
      CHEM_PREFETCH(ws + 90272);
      CHEM_PREFETCH(ws + 90304);
      CHEM_PREFETCH(ws + 90336);
      CHEM_PREFETCH(ws + 90368);
      CHEM_PREFETCH(ws + 90400);
      CHEM_PREFETCH(ws + 90432);
      CHEM_PREFETCH(ws + 90464);
      CHEM_PREFETCH(ws + 90496);
      CHEM_PREFETCH(ws + 90528);
      CHEM_PREFETCH(ws + 90560);
      CHEM_PREFETCH(ws + 90592);
      CHEM_PREFETCH(ws + 90624);
      CHEM_PREFETCH(ws + 90656);
      CHEM_PREFETCH(ws + 90688);
      CHEM_PREFETCH(ws + 90720);
      CHEM_PREFETCH(ws + 90752);
      CHEM_PREFETCH(ws + 90784);
      CHEM_PREFETCH(ws + 90816);
      CHEM_PREFETCH(ws + 90848);
      CHEM_PREFETCH(ws + 90880);
      CHEM_PREFETCH(ws + 90912);
      CHEM_PREFETCH(ws + 90944);
      CHEM_PREFETCH_L1(ws + 89600);
      CHEM_PREFETCH_L1(ws + 89632);
      CHEM_PREFETCH_L1(ws + 89664);
      CHEM_PREFETCH_L1(ws + 89696);
      CHEM_PREFETCH_L1(ws + 89728);
      CHEM_PREFETCH_L1(ws + 89760);
      CHEM_PREFETCH_L1(ws + 89792);
      CHEM_PREFETCH_L1(ws + 89824);
      CHEM_PREFETCH_L1(ws + 89856);
      CHEM_PREFETCH_L1(ws + 89888);
      CHEM_PREFETCH_L1(ws + 89920);
      CHEM_PREFETCH_L1(ws + 89952);
      CHEM_PREFETCH_L1(ws + 89984);
      CHEM_PREFETCH_L1(ws + 90016);
      CHEM_PREFETCH_L1(ws + 90048);
      CHEM_PREFETCH_L1(ws + 90080);
      CHEM_PREFETCH_L1(ws + 90112);
      CHEM_PREFETCH_L1(ws + 90144);
      CHEM_PREFETCH_L1(ws + 90176);
      CHEM_PREFETCH_L1(ws + 90208);
      double x = b[4384];
      x = fma(-CHEM_LDLU(lu + 11264), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 11296), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 11328), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 11360), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 11392), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 11424), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 11456), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 11488), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 11520), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 11552), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 11584), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 11616), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 11648), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 11680), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 11712), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 11744), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 11776), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 11808), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 11840), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 11872), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 11904), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 11936), b[4352], x);
      b[4384] = x;
    }
    {
      CHEM_PREFETCH(ws + 90976);
      CHEM_PREFETCH(ws + 91008);
      CHEM_PREFETCH(ws + 91040);
      CHEM_PREFETCH(ws + 91072);
      CHEM_PREFETCH(ws + 91104);
      CHEM_PREFETCH(ws + 91136);
      CHEM_PREFETCH(ws + 91168);
      CHEM_PREFETCH(ws + 91200);
      CHEM_PREFETCH(ws + 91232);
      CHEM_PREFETCH(ws + 91264);
      CHEM_PREFETCH(ws + 91296);
      CHEM_PREFETCH(ws + 91328);
      CHEM_PREFETCH(ws + 91360);
      CHEM_PREFETCH(ws + 91392);
      CHEM_PREFETCH(ws + 91424);
      CHEM_PREFETCH(ws + 91456);
      CHEM_PREFETCH(ws + 91488);
      CHEM_PREFETCH(ws + 91520);
      CHEM_PREFETCH(ws + 91552);
      CHEM_PREFETCH(ws + 91584);
      CHEM_PREFETCH(ws + 91616);
      CHEM_PREFETCH(ws + 91648);
      CHEM_PREFETCH(ws + 91680);
      CHEM_PREFETCH_L1(ws + 90240);
      CHEM_PREFETCH_L1(ws + 90272);
      CHEM_PREFETCH_L1(ws + 90304);
      CHEM_PREFETCH_L1(ws + 90336);
      CHEM_PREFETCH_L1(ws + 90368);
      CHEM_PREFETCH_L1(ws + 90400);
      CHEM_PREFETCH_L1(ws + 90432);
      CHEM_PREFETCH_L1(ws + 90464);
      CHEM_PREFETCH_L1(ws + 90496);
      CHEM_PREFETCH_L1(ws + 90528);
      CHEM_PREFETCH_L1(ws + 90560);
      CHEM_PREFETCH_L1(ws + 90592);
      CHEM_PREFETCH_L1(ws + 90624);
      CHEM_PREFETCH_L1(ws + 90656);
      CHEM_PREFETCH_L1(ws + 90688);
      CHEM_PREFETCH_L1(ws + 90720);
      CHEM_PREFETCH_L1(ws + 90752);
      CHEM_PREFETCH_L1(ws + 90784);
      CHEM_PREFETCH_L1(ws + 90816);
      CHEM_PREFETCH_L1(ws + 90848);
      CHEM_PREFETCH_L1(ws + 90880);
      CHEM_PREFETCH_L1(ws + 90912);
      CHEM_PREFETCH_L1(ws + 90944);
      double x = b[4416];
      x = fma(-CHEM_LDLU(lu + 11968), b[416], x);
      x = fma(-CHEM_LDLU(lu + 12000), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 12032), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 12064), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 12096), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 12128), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 12160), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 12192), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 12224), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 12256), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 12288), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 12320), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 12352), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 12384), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 12416), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 12448), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 12480), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 12512), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 12544), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 12576), b[4384], x);
      b[4416] = x;
    }
    {
      CHEM_PREFETCH(ws + 91712);
      CHEM_PREFETCH(ws + 91744);
      CHEM_PREFETCH(ws + 91776);
      CHEM_PREFETCH(ws + 91808);
      CHEM_PREFETCH(ws + 91840);
      CHEM_PREFETCH(ws + 91872);
      CHEM_PREFETCH(ws + 91904);
      CHEM_PREFETCH(ws + 91936);
      CHEM_PREFETCH(ws + 91968);
      CHEM_PREFETCH(ws + 92000);
      CHEM_PREFETCH(ws + 92032);
      CHEM_PREFETCH(ws + 92064);
      CHEM_PREFETCH(ws + 92096);
      CHEM_PREFETCH(ws + 92128);
      CHEM_PREFETCH(ws + 92160);
      CHEM_PREFETCH(ws + 92192);
      CHEM_PREFETCH(ws + 92224);
      CHEM_PREFETCH(ws + 92256);
      CHEM_PREFETCH(ws + 92288);
      CHEM_PREFETCH(ws + 92320);
      CHEM_PREFETCH(ws + 92352);
      CHEM_PREFETCH(ws + 92384);
      CHEM_PREFETCH(ws + 92416);
      CHEM_PREFETCH(ws + 92448);
      CHEM_PREFETCH(ws + 92480);
      CHEM_PREFETCH(ws + 92512);
      CHEM_PREFETCH_L1(ws + 90976);
      CHEM_PREFETCH_L1(ws + 91008);
      CHEM_PREFETCH_L1(ws + 91040);
      CHEM_PREFETCH_L1(ws + 91072);
      CHEM_PREFETCH_L1(ws + 91104);
      CHEM_PREFETCH_L1(ws + 91136);
      CHEM_PREFETCH_L1(ws + 91168);
      CHEM_PREFETCH_L1(ws + 91200);
      CHEM_PREFETCH_L1(ws + 91232);
      CHEM_PREFETCH_L1(ws + 91264);
      CHEM_PREFETCH_L1(ws + 91296);
      CHEM_PREFETCH_L1(ws + 91328);
      CHEM_PREFETCH_L1(ws + 91360);
      CHEM_PREFETCH_L1(ws + 91392);
      CHEM_PREFETCH_L1(ws + 91424);
      CHEM_PREFETCH_L1(ws + 91456);
      CHEM_PREFETCH_L1(ws + 91488);
      CHEM_PREFETCH_L1(ws + 91520);
      CHEM_PREFETCH_L1(ws + 91552);
      CHEM_PREFETCH_L1(ws + 91584);
      CHEM_PREFETCH_L1(ws + 91616);
      CHEM_PREFETCH_L1(ws + 91648);
      CHEM_PREFETCH_L1(ws + 91680);
      double x = b[4448];
      x = fma(-CHEM_LDLU(lu + 12608), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 12640), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 12672), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 12704), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 12736), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 12768), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 12800), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 12832), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 12864), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 12896), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 12928), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 12960), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 12992), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 13024), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 13056), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 13088), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 13120), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 13152), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 13184), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 13216), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 13248), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 13280), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 13312), b[4416], x);
      b[4448] = x;
    }
    {
      CHEM_PREFETCH(ws + 92544);
      CHEM_PREFETCH(ws + 92576);
      CHEM_PREFETCH(ws + 92608);
      CHEM_PREFETCH(ws + 92640);
      CHEM_PREFETCH(ws + 92672);
      CHEM_PREFETCH(ws + 92704);
      CHEM_PREFETCH(ws + 92736);
      CHEM_PREFETCH(ws + 92768);
      CHEM_PREFETCH(ws + 92800);
      CHEM_PREFETCH(ws + 92832);
      CHEM_PREFETCH(ws + 92864);
      CHEM_PREFETCH(ws + 92896);
      CHEM_PREFETCH(ws + 92928);
      CHEM_PREFETCH(ws + 92960);
      CHEM_PREFETCH(ws + 92992);
      CHEM_PREFETCH(ws + 93024);
      CHEM_PREFETCH(ws + 93056);
      CHEM_PREFETCH(ws + 93088);
      CHEM_PREFETCH(ws + 93120);
      CHEM_PREFETCH(ws + 93152);
      CHEM_PREFETCH(ws + 93184);
      CHEM_PREFETCH(ws + 93216);
      CHEM_PREFETCH(ws + 93248);
      CHEM_PREFETCH(ws + 93280);
      CHEM_PREFETCH(ws + 93312);
      CHEM_PREFETCH(ws + 93344);
      CHEM_PREFETCH(ws + 93376);
      CHEM_PREFETCH(ws + 93408);
      CHEM_PREFETCH(ws + 93440);
      CHEM_PREFETCH(ws + 93472);
      CHEM_PREFETCH(ws + 93504);
      CHEM_PREFETCH(ws + 93536);
      CHEM_PREFETCH(ws + 93568);
      CHEM_PREFETCH(ws + 93600);
      CHEM_PREFETCH_L1(ws + 91712);
      CHEM_PREFETCH_L1(ws + 91744);
      CHEM_PREFETCH_L1(ws + 91776);
      CHEM_PREFETCH_L1(ws + 91808);
      CHEM_PREFETCH_L1(ws + 91840);
      CHEM_PREFETCH_L1(ws + 91872);
      CHEM_PREFETCH_L1(ws + 91904);
      CHEM_PREFETCH_L1(ws + 91936);
      CHEM_PREFETCH_L1(ws + 91968);
      CHEM_PREFETCH_L1(ws + 92000);
      CHEM_PREFETCH_L1(ws + 92032);
      CHEM_PREFETCH_L1(ws + 92064);
      CHEM_PREFETCH_L1(ws + 92096);
      CHEM_PREFETCH_L1(ws + 92128);
      CHEM_PREFETCH_L1(ws + 92160);
      CHEM_PREFETCH_L1(ws + 92192);
      CHEM_PREFETCH_L1(ws + 92224);
      CHEM_PREFETCH_L1(ws + 92256);
      CHEM_PREFETCH_L1(ws + 92288);
      CHEM_PREFETCH_L1(ws + 92320);
      CHEM_PREFETCH_L1(ws + 92352);
      CHEM_PREFETCH_L1(ws + 92384);
      CHEM_PREFETCH_L1(ws + 92416);
      CHEM_PREFETCH_L1(ws + 92448);
      CHEM_PREFETCH_L1(ws + 92480);
      CHEM_PREFETCH_L1(ws + 92512);
      double x = b[4480];
      x = fma(-CHEM_LDLU(lu + 13344), b[352], x);
      x = fma(-CHEM_LDLU(lu + 13376), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 13408), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 13440), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 13472), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 13504), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 13536), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 13568), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 13600), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 13632), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 13664), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 13696), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 13728), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 13760), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 13792), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 13824), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 13856), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 13888), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 13920), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 13952), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 13984), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 14016), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 14048), b[4448], x);
      b[4480] = x;
    }
    {
      CHEM_PREFETCH(ws + 93632);
      CHEM_PREFETCH(ws + 93664);
      CHEM_PREFETCH(ws + 93696);
      CHEM_PREFETCH(ws + 93728);
      CHEM_PREFETCH(ws + 93760);
      CHEM_PREFETCH(ws + 93792);
      CHEM_PREFETCH(ws + 93824);
      CHEM_PREFETCH(ws + 93856);
      CHEM_PREFETCH(ws + 93888);
      CHEM_PREFETCH(ws + 93920);
      CHEM_PREFETCH(ws + 93952);
      CHEM_PREFETCH(ws + 93984);
      CHEM_PREFETCH(ws + 94016);
      CHEM_PREFETCH(ws + 94048);
      CHEM_PREFETCH(ws + 94080);
      CHEM_PREFETCH(ws + 94112);
      CHEM_PREFETCH(ws + 94144);
      CHEM_PREFETCH(ws + 94176);
      CHEM_PREFETCH(ws + 94208);
      CHEM_PREFETCH(ws + 94240);
      CHEM_PREFETCH(ws + 94272);
      CHEM_PREFETCH(ws + 94304);
      CHEM_PREFETCH(ws + 94336);
      CHEM_PREFETCH(ws + 94368);
      CHEM_PREFETCH(ws + 94400);
      CHEM_PREFETCH(ws + 94432);
      CHEM_PREFETCH(ws + 94464);
      CHEM_PREFETCH(ws + 94496);
      CHEM_PREFETCH(ws + 94528);
      CHEM_PREFETCH(ws + 94560);
      CHEM_PREFETCH(ws + 94592);
      CHEM_PREFETCH(ws + 94624);
      CHEM_PREFETCH(ws + 94656);
      CHEM_PREFETCH(ws + 94688);
      CHEM_PREFETCH_L1(ws + 92544);
      CHEM_PREFETCH_L1(ws + 92576);
      CHEM_PREFETCH_L1(ws + 92608);
      CHEM_PREFETCH_L1(ws + 92640);
      CHEM_PREFETCH_L1(ws + 92672);
      CHEM_PREFETCH_L1(ws + 92704);
      CHEM_PREFETCH_L1(ws + 92736);
      CHEM_PREFETCH_L1(ws + 92768);
      CHEM_PREFETCH_L1(ws + 92800);
      CHEM_PREFETCH_L1(ws + 92832);
      CHEM_PREFETCH_L1(ws + 92864);
      CHEM_PREFETCH_L1(ws + 92896);
      CHEM_PREFETCH_L1(ws + 92928);
      CHEM_PREFETCH_L1(ws + 92960);
      CHEM_PREFETCH_L1(ws + 92992);
      CHEM_PREFETCH_L1(ws + 93024);
      CHEM_PREFETCH_L1(ws + 93056);
      CHEM_PREFETCH_L1(ws + 93088);
      CHEM_PREFETCH_L1(ws + 93120);
      CHEM_PREFETCH_L1(ws + 93152);
      CHEM_PREFETCH_L1(ws + 93184);
      CHEM_PREFETCH_L1(ws + 93216);
      CHEM_PREFETCH_L1(ws + 93248);
      CHEM_PREFETCH_L1(ws + 93280);
      CHEM_PREFETCH_L1(ws + 93312);
      CHEM_PREFETCH_L1(ws + 93344);
      CHEM_PREFETCH_L1(ws + 93376);
      CHEM_PREFETCH_L1(ws + 93408);
      CHEM_PREFETCH_L1(ws + 93440);
      CHEM_PREFETCH_L1(ws + 93472);
      CHEM_PREFETCH_L1(ws + 93504);
      CHEM_PREFETCH_L1(ws + 93536);
      CHEM_PREFETCH_L1(ws + 93568);
      CHEM_PREFETCH_L1(ws + 93600);
      double x = b[4512];
      x = fma(-CHEM_LDLU(lu + 14080), b[864], x);
      x = fma(-CHEM_LDLU(lu + 14112), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 14144), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 14176), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 14208), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 14240), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 14272), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 14304), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 14336), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 14368), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 14400), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 14432), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 14464), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 14496), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 14528), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 14560), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 14592), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 14624), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 14656), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 14688), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 14720), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 14752), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 14784), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 14816), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 14848), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 14880), b[4448], x);
      b[4512] = x;
    }
    {
      CHEM_PREFETCH(ws + 94720);
      CHEM_PREFETCH(ws + 94752);
      CHEM_PREFETCH(ws + 94784);
      CHEM_PREFETCH(ws + 94816);
      CHEM_PREFETCH(ws + 94848);
      CHEM_PREFETCH(ws + 94880);
      CHEM_PREFETCH(ws + 94912);
      CHEM_PREFETCH(ws + 94944);
      CHEM_PREFETCH(ws + 94976);
      CHEM_PREFETCH(ws + 95008);
      CHEM_PREFETCH(ws + 95040);
      CHEM_PREFETCH(ws + 95072);
      CHEM_PREFETCH(ws + 95104);
      CHEM_PREFETCH(ws + 95136);
      CHEM_PREFETCH(ws + 95168);
      CHEM_PREFETCH(ws + 95200);
      CHEM_PREFETCH(ws + 95232);
      CHEM_PREFETCH(ws + 95264);
      CHEM_PREFETCH(ws + 95296);
      CHEM_PREFETCH(ws + 95328);
      CHEM_PREFETCH(ws + 95360);
      CHEM_PREFETCH(ws + 95392);
      CHEM_PREFETCH(ws + 95424);
      CHEM_PREFETCH(ws + 95456);
      CHEM_PREFETCH(ws + 95488);
      CHEM_PREFETCH(ws + 95520);
      CHEM_PREFETCH(ws + 95552);
      CHEM_PREFETCH(ws + 95584);
      CHEM_PREFETCH(ws + 95616);
      CHEM_PREFETCH(ws + 95648);
      CHEM_PREFETCH(ws + 95680);
      CHEM_PREFETCH(ws + 95712);
      CHEM_PREFETCH(ws + 95744);
      CHEM_PREFETCH(ws + 95776);
      CHEM_PREFETCH(ws + 95808);
      CHEM_PREFETCH(ws + 95840);
      CHEM_PREFETCH(ws + 95872);
      CHEM_PREFETCH(ws + 95904);
      CHEM_PREFETCH(ws + 95936);
      CHEM_PREFETCH_L1(ws + 93632);
      CHEM_PREFETCH_L1(ws + 93664);
      CHEM_PREFETCH_L1(ws + 93696);
      CHEM_PREFETCH_L1(ws + 93728);
      CHEM_PREFETCH_L1(ws + 93760);
      CHEM_PREFETCH_L1(ws + 93792);
      CHEM_PREFETCH_L1(ws + 93824);
      CHEM_PREFETCH_L1(ws + 93856);
      CHEM_PREFETCH_L1(ws + 93888);
      CHEM_PREFETCH_L1(ws + 93920);
      CHEM_PREFETCH_L1(ws + 93952);
      CHEM_PREFETCH_L1(ws + 93984);
      CHEM_PREFETCH_L1(ws + 94016);
      CHEM_PREFETCH_L1(ws + 94048);
      CHEM_PREFETCH_L1(ws + 94080);
      CHEM_PREFETCH_L1(ws + 94112);
      CHEM_PREFETCH_L1(ws + 94144);
      CHEM_PREFETCH_L1(ws + 94176);
      CHEM_PREFETCH_L1(ws + 94208);
      CHEM_PREFETCH_L1(ws + 94240);
      CHEM_PREFETCH_L1(ws + 94272);
      CHEM_PREFETCH_L1(ws + 94304);
      CHEM_PREFETCH_L1(ws + 94336);
      CHEM_PREFETCH_L1(ws + 94368);
      CHEM_PREFETCH_L1(ws + 94400);
      CHEM_PREFETCH_L1(ws + 94432);
      CHEM_PREFETCH_L1(ws + 94464);
      CHEM_PREFETCH_L1(ws + 94496);
      CHEM_PREFETCH_L1(ws + 94528);
      CHEM_PREFETCH_L1(ws + 94560);
      CHEM_PREFETCH_L1(ws + 94592);
      CHEM_PREFETCH_L1(ws + 94624);
      CHEM_PREFETCH_L1(ws + 94656);
      CHEM_PREFETCH_L1(ws + 94688);
      double x = b[4544];
      x = fma(-CHEM_LDLU(lu + 14912), b[832], x);
      x = fma(-CHEM_LDLU(lu + 14944), b[864], x);
      x = fma(-CHEM_LDLU(lu + 14976), b[896], x);
      x = fma(-CHEM_LDLU(lu + 15008), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 15040), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 15072), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 15104), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 15136), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 15168), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 15200), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 15232), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 15264), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 15296), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 15328), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 15360), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 15392), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 15424), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 15456), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 15488), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 15520), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 15552), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 15584), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 15616), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 15648), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 15680), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 15712), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 15744), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 15776), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 15808), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 15840), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 15872), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 15904), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 15936), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 15968), b[4512], x);
      b[4544] = x;
    }
    {
      CHEM_PREFETCH(ws + 95968);
      CHEM_PREFETCH(ws + 96000);
      CHEM_PREFETCH(ws + 96032);
      CHEM_PREFETCH(ws + 96064);
      CHEM_PREFETCH(ws + 96096);
      CHEM_PREFETCH(ws + 96128);
      CHEM_PREFETCH(ws + 96160);
      CHEM_PREFETCH(ws + 96192);
      CHEM_PREFETCH(ws + 96224);
      CHEM_PREFETCH(ws + 96256);
      CHEM_PREFETCH(ws + 96288);
      CHEM_PREFETCH(ws + 96320);
      CHEM_PREFETCH(ws + 96352);
      CHEM_PREFETCH(ws + 96384);
      CHEM_PREFETCH(ws + 96416);
      CHEM_PREFETCH(ws + 96448);
      CHEM_PREFETCH(ws + 96480);
      CHEM_PREFETCH(ws + 96512);
      CHEM_PREFETCH(ws + 96544);
      CHEM_PREFETCH(ws + 96576);
      CHEM_PREFETCH(ws + 96608);
      CHEM_PREFETCH(ws + 96640);
      CHEM_PREFETCH(ws + 96672);
      CHEM_PREFETCH(ws + 96704);
      CHEM_PREFETCH(ws + 96736);
      CHEM_PREFETCH(ws + 96768);
      CHEM_PREFETCH(ws + 96800);
      CHEM_PREFETCH(ws + 96832);
      CHEM_PREFETCH(ws + 96864);
      CHEM_PREFETCH(ws + 96896);
      CHEM_PREFETCH(ws + 96928);
      CHEM_PREFETCH(ws + 96960);
      CHEM_PREFETCH(ws + 96992);
      CHEM_PREFETCH(ws + 97024);
      CHEM_PREFETCH(ws + 97056);
      CHEM_PREFETCH(ws + 97088);
      CHEM_PREFETCH(ws + 97120);
      CHEM_PREFETCH(ws + 97152);
      CHEM_PREFETCH(ws + 97184);
      CHEM_PREFETCH(ws + 97216);
      CHEM_PREFETCH(ws + 97248);
      CHEM_PREFETCH(ws + 97280);
      CHEM_PREFETCH(ws + 97312);
      CHEM_PREFETCH_L1(ws + 94720);
      CHEM_PREFETCH_L1(ws + 94752);
      CHEM_PREFETCH_L1(ws + 94784);
      CHEM_PREFETCH_L1(ws + 94816);
      CHEM_PREFETCH_L1(ws + 94848);
      CHEM_PREFETCH_L1(ws + 94880);
      CHEM_PREFETCH_L1(ws + 94912);
      CHEM_PREFETCH_L1(ws + 94944);
      CHEM_PREFETCH_L1(ws + 94976);
      CHEM_PREFETCH_L1(ws + 95008);
      CHEM_PREFETCH_L1(ws + 95040);
      CHEM_PREFETCH_L1(ws + 95072);
      CHEM_PREFETCH_L1(ws + 95104);
      CHEM_PREFETCH_L1(ws + 95136);
      CHEM_PREFETCH_L1(ws + 95168);
      CHEM_PREFETCH_L1(ws + 95200);
      CHEM_PREFETCH_L1(ws + 95232);
      CHEM_PREFETCH_L1(ws + 95264);
      CHEM_PREFETCH_L1(ws + 95296);
      CHEM_PREFETCH_L1(ws + 95328);
      CHEM_PREFETCH_L1(ws + 95360);
      CHEM_PREFETCH_L1(ws + 95392);
      CHEM_PREFETCH_L1(ws + 95424);
      CHEM_PREFETCH_L1(ws + 95456);
      CHEM_PREFETCH_L1(ws + 95488);
      CHEM_PREFETCH_L1(ws + 95520);
      CHEM_PREFETCH_L1(ws + 95552);
      CHEM_PREFETCH_L1(ws + 95584);
      CHEM_PREFETCH_L1(ws + 95616);
      CHEM_PREFETCH_L1(ws + 95648);
      CHEM_PREFETCH_L1(ws + 95680);
      CHEM_PREFETCH_L1(ws + 95712);
      CHEM_PREFETCH_L1(ws + 95744);
      CHEM_PREFETCH_L1(ws + 95776);
      CHEM_PREFETCH_L1(ws + 95808);
      CHEM_PREFETCH_L1(ws + 95840);
      CHEM_PREFETCH_L1(ws + 95872);
      CHEM_PREFETCH_L1(ws + 95904);
      CHEM_PREFETCH_L1(ws + 95936);
      double x = b[4576];
      x = fma(-CHEM_LDLU(lu + 16000), b[832], x);
      x = fma(-CHEM_LDLU(lu + 16032), b[864], x);
      x = fma(-CHEM_LDLU(lu + 16064), b[896], x);
      x = fma(-CHEM_LDLU(lu + 16096), b[928], x);
      x = fma(-CHEM_LDLU(lu + 16128), b[960], x);
      x = fma(-CHEM_LDLU(lu + 16160), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 16192), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 16224), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 16256), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 16288), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 16320), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 16352), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 16384), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 16416), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 16448), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 16480), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 16512), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 16544), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 16576), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 16608), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 16640), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 16672), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 16704), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 16736), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 16768), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 16800), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 16832), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 16864), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 16896), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 16928), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 16960), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 16992), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 17024), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 17056), b[4544], x);
      b[4576] = x;
    }
    {
      CHEM_PREFETCH(ws + 97344);
      CHEM_PREFETCH(ws + 97376);
      CHEM_PREFETCH(ws + 97408);
      CHEM_PREFETCH(ws + 97440);
      CHEM_PREFETCH(ws + 97472);
      CHEM_PREFETCH(ws + 97504);
      CHEM_PREFETCH(ws + 97536);
      CHEM_PREFETCH(ws + 97568);
      CHEM_PREFETCH(ws + 97600);
      CHEM_PREFETCH(ws + 97632);
      CHEM_PREFETCH(ws + 97664);
      CHEM_PREFETCH(ws + 97696);
      CHEM_PREFETCH(ws + 97728);
      CHEM_PREFETCH(ws + 97760);
      CHEM_PREFETCH(ws + 97792);
      CHEM_PREFETCH(ws + 97824);
      CHEM_PREFETCH(ws + 97856);
      CHEM_PREFETCH(ws + 97888);
      CHEM_PREFETCH(ws + 97920);
      CHEM_PREFETCH(ws + 97952);
      CHEM_PREFETCH(ws + 97984);
      CHEM_PREFETCH(ws + 98016);
      CHEM_PREFETCH(ws + 98048);
      CHEM_PREFETCH(ws + 98080);
      CHEM_PREFETCH(ws + 98112);
      CHEM_PREFETCH(ws + 98144);
      CHEM_PREFETCH(ws + 98176);
      CHEM_PREFETCH(ws + 98208);
      CHEM_PREFETCH(ws + 98240);
      CHEM_PREFETCH(ws + 98272);
      CHEM_PREFETCH(ws + 98304);
      CHEM_PREFETCH(ws + 98336);
      CHEM_PREFETCH(ws + 98368);
      CHEM_PREFETCH(ws + 98400);
      CHEM_PREFETCH(ws + 98432);
      CHEM_PREFETCH(ws + 98464);
      CHEM_PREFETCH(ws + 98496);
      CHEM_PREFETCH(ws + 98528);
      CHEM_PREFETCH(ws + 98560);
      CHEM_PREFETCH(ws + 98592);
      CHEM_PREFETCH(ws + 98624);
      CHEM_PREFETCH(ws + 98656);
      CHEM_PREFETCH(ws + 98688);
      CHEM_PREFETCH(ws + 98720);
      CHEM_PREFETCH(ws + 98752);
      CHEM_PREFETCH(ws + 98784);
      CHEM_PREFETCH(ws + 98816);
      CHEM_PREFETCH(ws + 98848);
      CHEM_PREFETCH(ws + 98880);
      CHEM_PREFETCH(ws + 98912);
      CHEM_PREFETCH(ws + 98944);
      CHEM_PREFETCH_L1(ws + 95968);
      CHEM_PREFETCH_L1(ws + 96000);
      CHEM_PREFETCH_L1(ws + 96032);
      CHEM_PREFETCH_L1(ws + 96064);
      CHEM_PREFETCH_L1(ws + 96096);
      CHEM_PREFETCH_L1(ws + 96128);
      CHEM_PREFETCH_L1(ws + 96160);
      CHEM_PREFETCH_L1(ws + 96192);
      CHEM_PREFETCH_L1(ws + 96224);
      CHEM_PREFETCH_L1(ws + 96256);
      CHEM_PREFETCH_L1(ws + 96288);
      CHEM_PREFETCH_L1(ws + 96320);
      CHEM_PREFETCH_L1(ws + 96352);
      CHEM_PREFETCH_L1(ws + 96384);
      CHEM_PREFETCH_L1(ws + 96416);
      CHEM_PREFETCH_L1(ws + 96448);
      CHEM_PREFETCH_L1(ws + 96480);
      CHEM_PREFETCH_L1(ws + 96512);
      CHEM_PREFETCH_L1(ws + 96544);
      CHEM_PREFETCH_L1(ws + 96576);
      CHEM_PREFETCH_L1(ws + 96608);
      CHEM_PREFETCH_L1(ws + 96640);
      CHEM_PREFETCH_L1(ws + 96672);
      CHEM_PREFETCH_L1(ws + 96704);
      CHEM_PREFETCH_L1(ws + 96736);
      CHEM_PREFETCH_L1(ws + 96768);
      CHEM_PREFETCH_L1(ws + 96800);
      CHEM_PREFETCH_L1(ws + 96832);
      CHEM_PREFETCH_L1(ws + 96864);
      CHEM_PREFETCH_L1(ws + 96896);
      CHEM_PREFETCH_L1(ws + 96928);
      CHEM_PREFETCH_L1(ws + 96960);
      CHEM_PREFETCH_L1(ws + 96992);
      CHEM_PREFETCH_L1(ws + 97024);
      CHEM_PREFETCH_L1(ws + 97056);
      CHEM_PREFETCH_L1(ws + 97088);
      CHEM_PREFETCH_L1(ws + 97120);
      CHEM_PREFETCH_L1(ws + 97152);
      CHEM_PREFETCH_L1(ws + 97184);
      CHEM_PREFETCH_L1(ws + 97216);
      CHEM_PREFETCH_L1(ws + 97248);
      CHEM_PREFETCH_L1(ws + 97280);
      CHEM_PREFETCH_L1(ws + 97312);
      double x = b[4608];
      x = fma(-CHEM_LDLU(lu + 17088), b[960], x);
      x = fma(-CHEM_LDLU(lu + 17120), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 17152), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 17184), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 17216), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 17248), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 17280), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 17312), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 17344), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 17376), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 17408), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 17440), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 17472), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 17504), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 17536), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 17568), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 17600), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 17632), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 17664), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 17696), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 17728), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 17760), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 17792), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 17824), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 17856), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 17888), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 17920), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 17952), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 17984), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 18016), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 18048), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 18080), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 18112), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 18144), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 18176), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 18208), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 18240), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 18272), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 18304), b[4576], x);
      b[4608] = x;
    }
    {
      CHEM_PREFETCH(ws + 98976);
      CHEM_PREFETCH(ws + 99008);
      CHEM_PREFETCH(ws + 99040);
      CHEM_PREFETCH(ws + 99072);
      CHEM_PREFETCH(ws + 99104);
      CHEM_PREFETCH(ws + 99136);
      CHEM_PREFETCH(ws + 99168);
      CHEM_PREFETCH(ws + 99200);
      CHEM_PREFETCH(ws + 99232);
      CHEM_PREFETCH(ws + 99264);
      CHEM_PREFETCH(ws + 99296);
      CHEM_PREFETCH(ws + 99328);
      CHEM_PREFETCH(ws + 99360);
      CHEM_PREFETCH(ws + 99392);
      CHEM_PREFETCH(ws + 99424);
      CHEM_PREFETCH(ws + 99456);
      CHEM_PREFETCH(ws + 99488);
      CHEM_PREFETCH(ws + 99520);
      CHEM_PREFETCH(ws + 99552);
      CHEM_PREFETCH(ws + 99584);
      CHEM_PREFETCH(ws + 99616);
      CHEM_PREFETCH(ws + 99648);
      CHEM_PREFETCH(ws + 99680);
      CHEM_PREFETCH(ws + 99712);
      CHEM_PREFETCH(ws + 99744);
      CHEM_PREFETCH(ws + 99776);
      CHEM_PREFETCH(ws + 99808);
      CHEM_PREFETCH(ws + 99840);
      CHEM_PREFETCH(ws + 99872);
      CHEM_PREFETCH(ws + 99904);
      CHEM_PREFETCH(ws + 99936);
      CHEM_PREFETCH(ws + 99968);
      CHEM_PREFETCH(ws + 100000);
      CHEM_PREFETCH(ws + 100032);
      CHEM_PREFETCH(ws + 100064);
      CHEM_PREFETCH(ws + 100096);
      CHEM_PREFETCH(ws + 100128);
      CHEM_PREFETCH(ws + 100160);
      CHEM_PREFETCH(ws + 100192);
      CHEM_PREFETCH(ws + 100224);
      CHEM_PREFETCH(ws + 100256);
      CHEM_PREFETCH(ws + 100288);
      CHEM_PREFETCH(ws + 100320);
      CHEM_PREFETCH(ws + 100352);
      CHEM_PREFETCH(ws + 100384);
      CHEM_PREFETCH(ws + 100416);
      CHEM_PREFETCH(ws + 100448);
      CHEM_PREFETCH(ws + 100480);
      CHEM_PREFETCH(ws + 100512);
      CHEM_PREFETCH(ws + 100544);
      CHEM_PREFETCH(ws + 100576);
      CHEM_PREFETCH(ws + 100608);
      CHEM_PREFETCH(ws + 100640);
      CHEM_PREFETCH_L1(ws + 97344);
      CHEM_PREFETCH_L1(ws + 97376);
      CHEM_PREFETCH_L1(ws + 97408);
      CHEM_PREFETCH_L1(ws + 97440);
      CHEM_PREFETCH_L1(ws + 97472);
      CHEM_PREFETCH_L1(ws + 97504);
      CHEM_PREFETCH_L1(ws + 97536);
      CHEM_PREFETCH_L1(ws + 97568);
      CHEM_PREFETCH_L1(ws + 97600);
      CHEM_PREFETCH_L1(ws + 97632);
      CHEM_PREFETCH_L1(ws + 97664);
      CHEM_PREFETCH_L1(ws + 97696);
      CHEM_PREFETCH_L1(ws + 97728);
      CHEM_PREFETCH_L1(ws + 97760);
      CHEM_PREFETCH_L1(ws + 97792);
      CHEM_PREFETCH_L1(ws + 97824);
      CHEM_PREFETCH_L1(ws + 97856);
      CHEM_PREFETCH_L1(ws + 97888);
      CHEM_PREFETCH_L1(ws + 97920);
      CHEM_PREFETCH_L1(ws + 97952);
      CHEM_PREFETCH_L1(ws + 97984);
      CHEM_PREFETCH_L1(ws + 98016);
      CHEM_PREFETCH_L1(ws + 98048);
      CHEM_PREFETCH_L1(ws + 98080);
      CHEM_PREFETCH_L1(ws + 98112);
      CHEM_PREFETCH_L1(ws + 98144);
      CHEM_PREFETCH_L1(ws + 98176);
      CHEM_PREFETCH_L1(ws + 98208);
      CHEM_PREFETCH_L1(ws + 98240);
      CHEM_PREFETCH_L1(ws + 98272);
      CHEM_PREFETCH_L1(ws + 98304);
      CHEM_PREFETCH_L1(ws + 98336);
      CHEM_PREFETCH_L1(ws + 98368);
      CHEM_PREFETCH_L1(ws + 98400);
      CHEM_PREFETCH_L1(ws + 98432);
      CHEM_PREFETCH_L1(ws + 98464);
      CHEM_PREFETCH_L1(ws + 98496);
      CHEM_PREFETCH_L1(ws + 98528);
      CHEM_PREFETCH_L1(ws + 98560);
      CHEM_PREFETCH_L1(ws + 98592);
      CHEM_PREFETCH_L1(ws + 98624);
      CHEM_PREFETCH_L1(ws + 98656);
      CHEM_PREFETCH_L1(ws + 98688);
      CHEM_PREFETCH_L1(ws + 98720);
      CHEM_PREFETCH_L1(ws + 98752);
      CHEM_PREFETCH_L1(ws + 98784);
      CHEM_PREFETCH_L1(ws + 98816);
      CHEM_PREFETCH_L1(ws + 98848);
      CHEM_PREFETCH_L1(ws + 98880);
      CHEM_PREFETCH_L1(ws + 98912);
      CHEM_PREFETCH_L1(ws + 98944);
      double x = b[4640];
      x = fma(-CHEM_LDLU(lu + 18336), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 18368), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 18400), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 18432), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 18464), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 18496), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 18528), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 18560), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 18592), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 18624), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 18656), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 18688), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 18720), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 18752), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 18784), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 18816), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 18848), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 18880), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 18912), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 18944), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 18976), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 19008), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 19040), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 19072), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 19104), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 19136), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 19168), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 19200), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 19232), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 19264), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 19296), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 19328), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 19360), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 19392), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 19424), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 19456), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 19488), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 19520), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 19552), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 19584), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 19616), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 19648), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 19680), b[4608], x);
      b[4640] = x;
    }
}
__device__ __noinline__ void solve_1_1(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 77632;
    const double* __restrict__ vd = ws + 131712;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH(ws + 100672);
      CHEM_PREFETCH(ws + 100704);
      CHEM_PREFETCH(ws + 100736);
      CHEM_PREFETCH(ws + 100768);
      CHEM_PREFETCH(ws + 100800);
      CHEM_PREFETCH(ws + 100832);
      CHEM_PREFETCH(ws + 100864);
      CHEM_PREFETCH(ws + 100896);
      CHEM_PREFETCH(ws + 100928);
      CHEM_PREFETCH(ws + 100960);
      CHEM_PREFETCH(ws + 100992);
      CHEM_PREFETCH(ws + 101024);
      CHEM_PREFETCH(ws + 101056);
      CHEM_PREFETCH(ws + 101088);
      CHEM_PREFETCH(ws + 101120);
      CHEM_PREFETCH(ws + 101152);
      CHEM_PREFETCH(ws + 101184);
      CHEM_PREFETCH(ws + 101216);
      CHEM_PREFETCH(ws + 101248);
      CHEM_PREFETCH(ws + 101280);
      CHEM_PREFETCH(ws + 101312);
      CHEM_PREFETCH(ws + 101344);
      CHEM_PREFETCH(ws + 101376);
      CHEM_PREFETCH(ws + 101408);
      CHEM_PREFETCH(ws + 101440);
      CHEM_PREFETCH(ws + 101472);
      CHEM_PREFETCH(ws + 101504);
      CHEM_PREFETCH(ws + 101536);
      CHEM_PREFETCH(ws + 101568);
      CHEM_PREFETCH(ws + 101600);
      CHEM_PREFETCH(ws + 101632);
      CHEM_PREFETCH(ws + 101664);
      CHEM_PREFETCH(ws + 101696);
      CHEM_PREFETCH(ws + 101728);
      CHEM_PREFETCH(ws + 101760);
      CHEM_PREFETCH(ws + 101792);
      CHEM_PREFETCH(ws + 101824);
      CHEM_PREFETCH(ws + 101856);
      CHEM_PREFETCH(ws + 101888);
      CHEM_PREFETCH(ws + 101920);
      CHEM_PREFETCH(ws + 101952);
      CHEM_PREFETCH(ws + 101984);
      CHEM_PREFETCH(ws + 102016);
      CHEM_PREFETCH(ws + 102048);
      CHEM_PREFETCH(ws + 102080);
      CHEM_PREFETCH(ws + 102112);
      CHEM_PREFETCH(ws + 102144);
      CHEM_PREFETCH(ws + 102176);
      CHEM_PREFETCH(ws + 102208);
      CHEM_PREFETCH(ws + 102240);
      CHEM_PREFETCH(ws + 102272);
      CHEM_PREFETCH(ws + 102304);
      CHEM_PREFETCH(ws + 102336);
      CHEM_PREFETCH(ws + 102368);
      CHEM_PREFETCH(ws + 102400);
      CHEM_PREFETCH(ws + 102432);
      CHEM_PREFETCH(ws + 102464);
      CHEM_PREFETCH(ws + 102496);
      CHEM_PREFETCH(ws + 102528);
      CHEM_PREFETCH(ws + 102560);
      CHEM_PREFETCH(ws + 102592);
      CHEM_PREFETCH(ws + 102624);
      CHEM_PREFETCH(ws + 102656);
      CHEM_PREFETCH(ws + 102688);
      CHEM_PREFETCH(ws + 102720);
      CHEM_PREFETCH(ws + 102752);
      CHEM_PREFETCH(ws + 102784);
      CHEM_PREFETCH(ws + 102816);
      CHEM_PREFETCH(ws + 102848);
      CHEM_PREFETCH(ws + 102880);
      CHEM_PREFETCH(ws + 102912);
      CHEM_PREFETCH(ws + 102944);
      CHEM_PREFETCH(ws + 102976);
      CHEM_PREFETCH(ws + 103008);
      CHEM_PREFETCH(ws + 103040);
      CHEM_PREFETCH(ws + 103072);
      CHEM_PREFETCH(ws + 103104);
      CHEM_PREFETCH(ws + 103136);
      CHEM_PREFETCH(ws + 103168);
      CHEM_PREFETCH(ws + 103200);
      CHEM_PREFETCH(ws + 103232);
      CHEM_PREFETCH(ws + 103264);
      CHEM_PREFETCH(ws + 103296);
      CHEM_PREFETCH(ws + 103328);
      CHEM_PREFETCH(ws + 103360);
      CHEM_PREFETCH(ws + 103392);
      CHEM_PREFETCH(ws + 103424);
      CHEM_PREFETCH(ws + 103456);
      CHEM_PREFETCH(ws + 103488);
      CHEM_PREFETCH(ws + 103520);
      CHEM_PREFETCH(ws + 103552);
      CHEM_PREFETCH(ws + 103584);
      CHEM_PREFETCH(ws + 103616);
      CHEM_PREFETCH(ws + 103648);
      CHEM_PREFETCH(ws + 103680);
      CHEM_PREFETCH(ws + 103712);
      CHEM_PREFETCH_L1(ws + 98976);
      CHEM_PREFETCH_L1(ws + 99008);
      CHEM_PREFETCH_L1(ws + 99040);
      CHEM_PREFETCH_L1(ws + 99072);
      CHEM_PREFETCH_L1(ws + 99104);
      CHEM_PREFETCH_L1(ws + 99136);
      CHEM_PREFETCH_L1(ws + 99168);
      CHEM_PREFETCH_L1(ws + 99200);
      CHEM_PREFETCH_L1(ws + 99232);
      CHEM_PREFETCH_L1(ws + 99264);
      CHEM_PREFETCH_L1(ws + 99296);
      CHEM_PREFETCH_L1(ws + 99328);
      CHEM_PREFETCH_L1(ws + 99360);
      CHEM_PREFETCH_L1(ws + 99392);
      CHEM_PREFETCH_L1(ws + 99424);
      CHEM_PREFETCH_L1(ws + 99456);
      CHEM_PREFETCH_L1(ws + 99488);
      CHEM_PREFETCH_L1(ws + 99520);
      CHEM_PREFETCH_L1(ws + 99552);
      CHEM_PREFETCH_L1(ws + 99584);
      CHEM_PREFETCH_L1(ws + 99616);
      CHEM_PREFETCH_L1(ws + 99648);
      CHEM_PREFETCH_L1(ws + 99680);
      CHEM_PREFETCH_L1(ws + 99712);
      CHEM_PREFETCH_L1(ws + 99744);
      CHEM_PREFETCH_L1(ws + 99776);
      CHEM_PREFETCH_L1(ws + 99808);
      CHEM_PREFETCH_L1(ws + 99840);
      CHEM_PREFETCH_L1(ws + 99872);
      CHEM_PREFETCH_L1(ws + 99904);
      CHEM_PREFETCH_L1(ws + 99936);
      CHEM_PREFETCH_L1(ws + 99968);
      CHEM_PREFETCH_L1(ws + 100000);
      CHEM_PREFETCH_L1(ws + 100032);
      CHEM_PREFETCH_L1(ws + 100064);
      CHEM_PREFETCH_L1(ws + 100096);
      CHEM_PREFETCH_L1(ws + 100128);
      CHEM_PREFETCH_L1(ws + 100160);
      CHEM_PREFETCH_L1(ws + 100192);
      CHEM_PREFETCH_L1(ws + 100224);
      CHEM_PREFETCH_L1(ws + 100256);
      CHEM_PREFETCH_L1(ws + 100288);
      CHEM_PREFETCH_L1(ws + 100320);
      CHEM_PREFETCH_L1(ws + 100352);
      CHEM_PREFETCH_L1(ws + 100384);
      CHEM_PREFETCH_L1(ws + 100416);
      CHEM_PREFETCH_L1(ws + 100448);
      CHEM_PREFETCH_L1(ws + 100480);
      CHEM_PREFETCH_L1(ws + 100512);
      CHEM_PREFETCH_L1(ws + 100544);
      CHEM_PREFETCH_L1(ws + 100576);
      CHEM_PREFETCH_L1(ws + 100608);
      CHEM_PREFETCH_L1(ws + 100640);
      double x = b[4672];
      x = fma(-CHEM_LDLU(lu + 19712), b[384], x);
      x = fma(-CHEM_LDLU(lu + 19744), b[416], x);
      x = fma(-CHEM_LDLU(lu + 19776), b[832], x);
      x = fma(-CHEM_LDLU(lu + 19808), b[864], x);
      x = fma(-CHEM_LDLU(lu + 19840), b[896], x);
      x = fma(-CHEM_LDLU(lu + 19872), b[928], x);
      x = fma(-CHEM_LDLU(lu + 19904), b[960], x);
      x = fma(-CHEM_LDLU(lu + 19936), b[1056], x);
      x = fma(-CHEM_LDLU(lu + 19968), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 20000), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 20032), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 20064), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 20096), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 20128), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 20160), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 20192), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 20224), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 20256), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 20288), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 20320), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 20352), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 20384), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 20416), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 20448), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 20480), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 20512), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 20544), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 20576), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 20608), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 20640), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 20672), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 20704), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 20736), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 20768), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 20800), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 20832), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 20864), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 20896), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 20928), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 20960), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 20992), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 21024), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 21056), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 21088), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 21120), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 21152), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 21184), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 21216), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 21248), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 21280), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 21312), b[4640], x);
      b[4672] = x;
    }
    {
      CHEM_PREFETCH(ws + 136448);
      CHEM_PREFETCH_L1(ws + 100672);
      CHEM_PREFETCH_L1(ws + 100704);
      CHEM_PREFETCH_L1(ws + 100736);
      CHEM_PREFETCH_L1(ws + 100768);
      CHEM_PREFETCH_L1(ws + 100800);
      CHEM_PREFETCH_L1(ws + 100832);
      CHEM_PREFETCH_L1(ws + 100864);
      CHEM_PREFETCH_L1(ws + 100896);
      CHEM_PREFETCH_L1(ws + 100928);
      CHEM_PREFETCH_L1(ws + 100960);
      CHEM_PREFETCH_L1(ws + 100992);
      CHEM_PREFETCH_L1(ws + 101024);
      CHEM_PREFETCH_L1(ws + 101056);
      CHEM_PREFETCH_L1(ws + 101088);
      CHEM_PREFETCH_L1(ws + 101120);
      CHEM_PREFETCH_L1(ws + 101152);
      CHEM_PREFETCH_L1(ws + 101184);
      CHEM_PREFETCH_L1(ws + 101216);
      CHEM_PREFETCH_L1(ws + 101248);
      CHEM_PREFETCH_L1(ws + 101280);
      CHEM_PREFETCH_L1(ws + 101312);
      CHEM_PREFETCH_L1(ws + 101344);
      CHEM_PREFETCH_L1(ws + 101376);
      CHEM_PREFETCH_L1(ws + 101408);
      CHEM_PREFETCH_L1(ws + 101440);
      CHEM_PREFETCH_L1(ws + 101472);
      CHEM_PREFETCH_L1(ws + 101504);
      CHEM_PREFETCH_L1(ws + 101536);
      CHEM_PREFETCH_L1(ws + 101568);
      CHEM_PREFETCH_L1(ws + 101600);
      CHEM_PREFETCH_L1(ws + 101632);
      CHEM_PREFETCH_L1(ws + 101664);
      CHEM_PREFETCH_L1(ws + 101696);
      CHEM_PREFETCH_L1(ws + 101728);
      CHEM_PREFETCH_L1(ws + 101760);
      CHEM_PREFETCH_L1(ws + 101792);
      CHEM_PREFETCH_L1(ws + 101824);
      CHEM_PREFETCH_L1(ws + 101856);
      CHEM_PREFETCH_L1(ws + 101888);
      CHEM_PREFETCH_L1(ws + 101920);
      CHEM_PREFETCH_L1(ws + 101952);
      CHEM_PREFETCH_L1(ws + 101984);
      CHEM_PREFETCH_L1(ws + 102016);
      CHEM_PREFETCH_L1(ws + 102048);
      CHEM_PREFETCH_L1(ws + 102080);
      CHEM_PREFETCH_L1(ws + 102112);
      CHEM_PREFETCH_L1(ws + 102144);
      CHEM_PREFETCH_L1(ws + 102176);
      CHEM_PREFETCH_L1(ws + 102208);
      CHEM_PREFETCH_L1(ws + 102240);
      CHEM_PREFETCH_L1(ws + 102272);
      CHEM_PREFETCH_L1(ws + 102304);
      CHEM_PREFETCH_L1(ws + 102336);
      CHEM_PREFETCH_L1(ws + 102368);
      CHEM_PREFETCH_L1(ws + 102400);
      CHEM_PREFETCH_L1(ws + 102432);
      CHEM_PREFETCH_L1(ws + 102464);
      CHEM_PREFETCH_L1(ws + 102496);
      CHEM_PREFETCH_L1(ws + 102528);
      CHEM_PREFETCH_L1(ws + 102560);
      CHEM_PREFETCH_L1(ws + 102592);
      CHEM_PREFETCH_L1(ws + 102624);
      CHEM_PREFETCH_L1(ws + 102656);
      CHEM_PREFETCH_L1(ws + 102688);
      CHEM_PREFETCH_L1(ws + 102720);
      CHEM_PREFETCH_L1(ws + 102752);
      CHEM_PREFETCH_L1(ws + 102784);
      CHEM_PREFETCH_L1(ws + 102816);
      CHEM_PREFETCH_L1(ws + 102848);
      CHEM_PREFETCH_L1(ws + 102880);
      CHEM_PREFETCH_L1(ws + 102912);
      CHEM_PREFETCH_L1(ws + 102944);
      CHEM_PREFETCH_L1(ws + 102976);
      CHEM_PREFETCH_L1(ws + 103008);
      CHEM_PREFETCH_L1(ws + 103040);
      CHEM_PREFETCH_L1(ws + 103072);
      CHEM_PREFETCH_L1(ws + 103104);
      CHEM_PREFETCH_L1(ws + 103136);
      CHEM_PREFETCH_L1(ws + 103168);
      CHEM_PREFETCH_L1(ws + 103200);
      CHEM_PREFETCH_L1(ws + 103232);
      CHEM_PREFETCH_L1(ws + 103264);
      CHEM_PREFETCH_L1(ws + 103296);
      CHEM_PREFETCH_L1(ws + 103328);
      CHEM_PREFETCH_L1(ws + 103360);
      CHEM_PREFETCH_L1(ws + 103392);
      CHEM_PREFETCH_L1(ws + 103424);
      CHEM_PREFETCH_L1(ws + 103456);
      CHEM_PREFETCH_L1(ws + 103488);
      CHEM_PREFETCH_L1(ws + 103520);
      CHEM_PREFETCH_L1(ws + 103552);
      CHEM_PREFETCH_L1(ws + 103584);
      CHEM_PREFETCH_L1(ws + 103616);
      CHEM_PREFETCH_L1(ws + 103648);
      CHEM_PREFETCH_L1(ws + 103680);
      CHEM_PREFETCH_L1(ws + 103712);
      double x = b[4704];
      x = fma(-CHEM_LDLU(lu + 21344), b[352], x);
      x = fma(-CHEM_LDLU(lu + 21376), b[384], x);
      x = fma(-CHEM_LDLU(lu + 21408), b[864], x);
      x = fma(-CHEM_LDLU(lu + 21440), b[960], x);
      x = fma(-CHEM_LDLU(lu + 21472), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 21504), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 21536), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 21568), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 21600), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 21632), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 21664), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 21696), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 21728), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 21760), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 21792), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 21824), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 21856), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 21888), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 21920), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 21952), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 21984), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 22016), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 22048), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 22080), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 22112), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 22144), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 22176), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 22208), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 22240), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 22272), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 22304), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 22336), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 22368), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 22400), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 22432), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 22464), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 22496), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 22528), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 22560), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 22592), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 22624), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 22656), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 22688), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 22720), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 22752), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 22784), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 22816), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 22848), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 22880), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 22912), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 22944), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 22976), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 23008), b[4672], x);
      b[4704] = x;
    }
    {
      CHEM_PREFETCH(ws + 103744);
      CHEM_PREFETCH(ws + 136416);
      CHEM_PREFETCH_L1(ws + 136448);
      double x = b[4736];
      x = fma(-CHEM_LDLU(lu + 23040), b[352], x);
      x = fma(-CHEM_LDLU(lu + 23072), b[384], x);
      x = fma(-CHEM_LDLU(lu + 23104), b[416], x);
      x = fma(-CHEM_LDLU(lu + 23136), b[448], x);
      x = fma(-CHEM_LDLU(lu + 23168), b[672], x);
      x = fma(-CHEM_LDLU(lu + 23200), b[704], x);
      x = fma(-CHEM_LDLU(lu + 23232), b[736], x);
      x = fma(-CHEM_LDLU(lu + 23264), b[768], x);
      x = fma(-CHEM_LDLU(lu + 23296), b[832], x);
      x = fma(-CHEM_LDLU(lu + 23328), b[864], x);
      x = fma(-CHEM_LDLU(lu + 23360), b[896], x);
      x = fma(-CHEM_LDLU(lu + 23392), b[1056], x);
      x = fma(-CHEM_LDLU(lu + 23424), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 23456), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 23488), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 23520), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 23552), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 23584), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 23616), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 23648), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 23680), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 23712), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 23744), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 23776), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 23808), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 23840), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 23872), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 23904), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 23936), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 23968), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 24000), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 24032), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 24064), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 24096), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 24128), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 24160), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 24192), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 24224), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 24256), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 24288), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 24320), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 24352), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 24384), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 24416), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 24448), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 24480), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 24512), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 24544), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 24576), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 24608), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 24640), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 24672), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 24704), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 24736), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 24768), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 24800), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 24832), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 24864), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 24896), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 24928), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 24960), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 24992), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 25024), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 25056), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 25088), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 25120), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 25152), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 25184), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 25216), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 25248), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 25280), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 25312), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 25344), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 25376), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 25408), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 25440), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 25472), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 25504), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 25536), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 25568), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 25600), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 25632), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 25664), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 25696), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 25728), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 25760), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 25792), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 25824), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 25856), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 25888), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 25920), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 25952), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 25984), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 26016), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 26048), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26080), b[4704], x);
      b[4736] = x;
    }
    {
      CHEM_PREFETCH(ws + 103776);
      CHEM_PREFETCH(ws + 103808);
      CHEM_PREFETCH(ws + 136384);
      CHEM_PREFETCH_L1(ws + 103744);
      CHEM_PREFETCH_L1(ws + 136416);
      double x = b[4736];
      b[4736] = x * CHEM_LDLU(vd + 4736);
    }
    {
      CHEM_PREFETCH(ws + 103840);
      CHEM_PREFETCH(ws + 103872);
      CHEM_PREFETCH(ws + 103904);
      CHEM_PREFETCH(ws + 136352);
      CHEM_PREFETCH_L1(ws + 103776);
      CHEM_PREFETCH_L1(ws + 103808);
      CHEM_PREFETCH_L1(ws + 136384);
      double x = b[4704];
      x = fma(-CHEM_LDLU(lu + 26112), b[4736], x);
      b[4704] = x * CHEM_LDLU(vd + 4704);
    }
    {
      CHEM_PREFETCH(ws + 103936);
      CHEM_PREFETCH(ws + 103968);
      CHEM_PREFETCH(ws + 104000);
      CHEM_PREFETCH(ws + 104032);
      CHEM_PREFETCH(ws + 136320);
      CHEM_PREFETCH_L1(ws + 103840);
      CHEM_PREFETCH_L1(ws + 103872);
      CHEM_PREFETCH_L1(ws + 103904);
      CHEM_PREFETCH_L1(ws + 136352);
      double x = b[4672];
      x = fma(-CHEM_LDLU(lu + 26144), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 26176), b[4736], x);
      b[4672] = x * CHEM_LDLU(vd + 4672);
    }
    {
      CHEM_PREFETCH(ws + 104064);
      CHEM_PREFETCH(ws + 104096);
      CHEM_PREFETCH(ws + 104128);
      CHEM_PREFETCH(ws + 104160);
      CHEM_PREFETCH(ws + 104192);
      CHEM_PREFETCH(ws + 136288);
      CHEM_PREFETCH_L1(ws + 103936);
      CHEM_PREFETCH_L1(ws + 103968);
      CHEM_PREFETCH_L1(ws + 104000);
      CHEM_PREFETCH_L1(ws + 104032);
      CHEM_PREFETCH_L1(ws + 136320);
      double x = b[4640];
      x = fma(-CHEM_LDLU(lu + 26208), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26240), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 26272), b[4736], x);
      b[4640] = x * CHEM_LDLU(vd + 4640);
    }
    {
      CHEM_PREFETCH(ws + 104224);
      CHEM_PREFETCH(ws + 104256);
      CHEM_PREFETCH(ws + 104288);
      CHEM_PREFETCH(ws + 104320);
      CHEM_PREFETCH(ws + 104352);
      CHEM_PREFETCH(ws + 104384);
      CHEM_PREFETCH(ws + 136256);
      CHEM_PREFETCH_L1(ws + 104064);
      CHEM_PREFETCH_L1(ws + 104096);
      CHEM_PREFETCH_L1(ws + 104128);
      CHEM_PREFETCH_L1(ws + 104160);
      CHEM_PREFETCH_L1(ws + 104192);
      CHEM_PREFETCH_L1(ws + 136288);
      double x = b[4608];
      x = fma(-CHEM_LDLU(lu + 26304), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 26336), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26368), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 26400), b[4736], x);
      b[4608] = x * CHEM_LDLU(vd + 4608);
    }
    {
      CHEM_PREFETCH(ws + 104416);
      CHEM_PREFETCH(ws + 104448);
      CHEM_PREFETCH(ws + 104480);
      CHEM_PREFETCH(ws + 104512);
      CHEM_PREFETCH(ws + 104544);
      CHEM_PREFETCH(ws + 104576);
      CHEM_PREFETCH(ws + 104608);
      CHEM_PREFETCH(ws + 136224);
      CHEM_PREFETCH_L1(ws + 104224);
      CHEM_PREFETCH_L1(ws + 104256);
      CHEM_PREFETCH_L1(ws + 104288);
      CHEM_PREFETCH_L1(ws + 104320);
      CHEM_PREFETCH_L1(ws + 104352);
      CHEM_PREFETCH_L1(ws + 104384);
      CHEM_PREFETCH_L1(ws + 136256);
      double x = b[4576];
      x = fma(-CHEM_LDLU(lu + 26432), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 26464), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 26496), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26528), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 26560), b[4736], x);
      b[4576] = x * CHEM_LDLU(vd + 4576);
    }
    {
      CHEM_PREFETCH(ws + 104640);
      CHEM_PREFETCH(ws + 104672);
      CHEM_PREFETCH(ws + 104704);
      CHEM_PREFETCH(ws + 104736);
      CHEM_PREFETCH(ws + 104768);
      CHEM_PREFETCH(ws + 104800);
      CHEM_PREFETCH(ws + 104832);
      CHEM_PREFETCH(ws + 104864);
      CHEM_PREFETCH(ws + 136192);
      CHEM_PREFETCH_L1(ws + 104416);
      CHEM_PREFETCH_L1(ws + 104448);
      CHEM_PREFETCH_L1(ws + 104480);
      CHEM_PREFETCH_L1(ws + 104512);
      CHEM_PREFETCH_L1(ws + 104544);
      CHEM_PREFETCH_L1(ws + 104576);
      CHEM_PREFETCH_L1(ws + 104608);
      CHEM_PREFETCH_L1(ws + 136224);
      double x = b[4544];
      x = fma(-CHEM_LDLU(lu + 26592), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 26624), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 26656), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 26688), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26720), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 26752), b[4736], x);
      b[4544] = x * CHEM_LDLU(vd + 4544);
    }
    {
      CHEM_PREFETCH(ws + 104896);
      CHEM_PREFETCH(ws + 104928);
      CHEM_PREFETCH(ws + 104960);
      CHEM_PREFETCH(ws + 104992);
      CHEM_PREFETCH(ws + 105024);
      CHEM_PREFETCH(ws + 105056);
      CHEM_PREFETCH(ws + 105088);
      CHEM_PREFETCH(ws + 105120);
      CHEM_PREFETCH(ws + 136160);
      CHEM_PREFETCH_L1(ws + 104640);
      CHEM_PREFETCH_L1(ws + 104672);
      CHEM_PREFETCH_L1(ws + 104704);
      CHEM_PREFETCH_L1(ws + 104736);
      CHEM_PREFETCH_L1(ws + 104768);
      CHEM_PREFETCH_L1(ws + 104800);
      CHEM_PREFETCH_L1(ws + 104832);
      CHEM_PREFETCH_L1(ws + 104864);
      CHEM_PREFETCH_L1(ws + 136192);
      double x = b[4512];
      x = fma(-CHEM_LDLU(lu + 26784), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 26816), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 26848), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 26880), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 26912), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 26944), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 26976), b[4736], x);
      b[4512] = x * CHEM_LDLU(vd + 4512);
    }
    {
      CHEM_PREFETCH(ws + 105152);
      CHEM_PREFETCH(ws + 105184);
      CHEM_PREFETCH(ws + 105216);
      CHEM_PREFETCH(ws + 105248);
      CHEM_PREFETCH(ws + 105280);
      CHEM_PREFETCH(ws + 105312);
      CHEM_PREFETCH(ws + 105344);
      CHEM_PREFETCH(ws + 105376);
      CHEM_PREFETCH(ws + 105408);
      CHEM_PREFETCH(ws + 136128);
      CHEM_PREFETCH_L1(ws + 104896);
      CHEM_PREFETCH_L1(ws + 104928);
      CHEM_PREFETCH_L1(ws + 104960);
      CHEM_PREFETCH_L1(ws + 104992);
      CHEM_PREFETCH_L1(ws + 105024);
      CHEM_PREFETCH_L1(ws + 105056);
      CHEM_PREFETCH_L1(ws + 105088);
      CHEM_PREFETCH_L1(ws + 105120);
      CHEM_PREFETCH_L1(ws + 136160);
      double x = b[4480];
      x = fma(-CHEM_LDLU(lu + 27008), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 27040), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 27072), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 27104), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 27136), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 27168), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 27200), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 27232), b[4736], x);
      b[4480] = x * CHEM_LDLU(vd + 4480);
    }
    {
      CHEM_PREFETCH(ws + 105440);
      CHEM_PREFETCH(ws + 105472);
      CHEM_PREFETCH(ws + 105504);
      CHEM_PREFETCH(ws + 105536);
      CHEM_PREFETCH(ws + 105568);
      CHEM_PREFETCH(ws + 105600);
      CHEM_PREFETCH(ws + 105632);
      CHEM_PREFETCH(ws + 105664);
      CHEM_PREFETCH(ws + 105696);
      CHEM_PREFETCH(ws + 105728);
      CHEM_PREFETCH(ws + 136096);
      CHEM_PREFETCH_L1(ws + 105152);
      CHEM_PREFETCH_L1(ws + 105184);
      CHEM_PREFETCH_L1(ws + 105216);
      CHEM_PREFETCH_L1(ws + 105248);
      CHEM_PREFETCH_L1(ws + 105280);
      CHEM_PREFETCH_L1(ws + 105312);
      CHEM_PREFETCH_L1(ws + 105344);
      CHEM_PREFETCH_L1(ws + 105376);
      CHEM_PREFETCH_L1(ws + 105408);
      CHEM_PREFETCH_L1(ws + 136128);
      double x = b[4448];
      x = fma(-CHEM_LDLU(lu + 27264), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 27296), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 27328), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 27360), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 27392), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 27424), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 27456), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 27488), b[4736], x);
      b[4448] = x * CHEM_LDLU(vd + 4448);
    }
    {
      CHEM_PREFETCH(ws + 105760);
      CHEM_PREFETCH(ws + 105792);
      CHEM_PREFETCH(ws + 105824);
      CHEM_PREFETCH(ws + 105856);
      CHEM_PREFETCH(ws + 105888);
      CHEM_PREFETCH(ws + 105920);
      CHEM_PREFETCH(ws + 105952);
      CHEM_PREFETCH(ws + 105984);
      CHEM_PREFETCH(ws + 106016);
      CHEM_PREFETCH(ws + 106048);
      CHEM_PREFETCH(ws + 136064);
      CHEM_PREFETCH_L1(ws + 105440);
      CHEM_PREFETCH_L1(ws + 105472);
      CHEM_PREFETCH_L1(ws + 105504);
      CHEM_PREFETCH_L1(ws + 105536);
      CHEM_PREFETCH_L1(ws + 105568);
      CHEM_PREFETCH_L1(ws + 105600);
      CHEM_PREFETCH_L1(ws + 105632);
      CHEM_PREFETCH_L1(ws + 105664);
      CHEM_PREFETCH_L1(ws + 105696);
      CHEM_PREFETCH_L1(ws + 105728);
      CHEM_PREFETCH_L1(ws + 136096);
      double x = b[4416];
      x = fma(-CHEM_LDLU(lu + 27520), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 27552), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 27584), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 27616), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 27648), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 27680), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 27712), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 27744), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 27776), b[4736], x);
      b[4416] = x * CHEM_LDLU(vd + 4416);
    }
    {
      CHEM_PREFETCH(ws + 106080);
      CHEM_PREFETCH(ws + 106112);
      CHEM_PREFETCH(ws + 106144);
      CHEM_PREFETCH(ws + 106176);
      CHEM_PREFETCH(ws + 106208);
      CHEM_PREFETCH(ws + 106240);
      CHEM_PREFETCH(ws + 106272);
      CHEM_PREFETCH(ws + 106304);
      CHEM_PREFETCH(ws + 106336);
      CHEM_PREFETCH(ws + 106368);
      CHEM_PREFETCH(ws + 136032);
      CHEM_PREFETCH_L1(ws + 105760);
      CHEM_PREFETCH_L1(ws + 105792);
      CHEM_PREFETCH_L1(ws + 105824);
      CHEM_PREFETCH_L1(ws + 105856);
      CHEM_PREFETCH_L1(ws + 105888);
      CHEM_PREFETCH_L1(ws + 105920);
      CHEM_PREFETCH_L1(ws + 105952);
      CHEM_PREFETCH_L1(ws + 105984);
      CHEM_PREFETCH_L1(ws + 106016);
      CHEM_PREFETCH_L1(ws + 106048);
      CHEM_PREFETCH_L1(ws + 136064);
      double x = b[4384];
      x = fma(-CHEM_LDLU(lu + 27808), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 27840), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 27872), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 27904), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 27936), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 27968), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 28000), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 28032), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 28064), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 28096), b[4736], x);
      b[4384] = x * CHEM_LDLU(vd + 4384);
    }
    {
      CHEM_PREFETCH(ws + 106400);
      CHEM_PREFETCH(ws + 106432);
      CHEM_PREFETCH(ws + 106464);
      CHEM_PREFETCH(ws + 106496);
      CHEM_PREFETCH(ws + 106528);
      CHEM_PREFETCH(ws + 106560);
      CHEM_PREFETCH(ws + 106592);
      CHEM_PREFETCH(ws + 106624);
      CHEM_PREFETCH(ws + 106656);
      CHEM_PREFETCH(ws + 106688);
      CHEM_PREFETCH(ws + 106720);
      CHEM_PREFETCH(ws + 106752);
      CHEM_PREFETCH(ws + 106784);
      CHEM_PREFETCH(ws + 136000);
      CHEM_PREFETCH_L1(ws + 106080);
      CHEM_PREFETCH_L1(ws + 106112);
      CHEM_PREFETCH_L1(ws + 106144);
      CHEM_PREFETCH_L1(ws + 106176);
      CHEM_PREFETCH_L1(ws + 106208);
      CHEM_PREFETCH_L1(ws + 106240);
      CHEM_PREFETCH_L1(ws + 106272);
      CHEM_PREFETCH_L1(ws + 106304);
      CHEM_PREFETCH_L1(ws + 106336);
      CHEM_PREFETCH_L1(ws + 106368);
      CHEM_PREFETCH_L1(ws + 136032);
      double x = b[4352];
      x = fma(-CHEM_LDLU(lu + 28128), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 28160), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 28192), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 28224), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 28256), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 28288), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 28320), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 28352), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 28384), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 28416), b[4736], x);
      b[4352] = x * CHEM_LDLU(vd + 4352);
    }
    {
      CHEM_PREFETCH(ws + 106816);
      CHEM_PREFETCH(ws + 106848);
      CHEM_PREFETCH(ws + 106880);
      CHEM_PREFETCH(ws + 106912);
      CHEM_PREFETCH(ws + 106944);
      CHEM_PREFETCH(ws + 106976);
      CHEM_PREFETCH(ws + 107008);
      CHEM_PREFETCH(ws + 107040);
      CHEM_PREFETCH(ws + 107072);
      CHEM_PREFETCH(ws + 107104);
      CHEM_PREFETCH(ws + 107136);
      CHEM_PREFETCH(ws + 135968);
      CHEM_PREFETCH_L1(ws + 106400);
      CHEM_PREFETCH_L1(ws + 106432);
      CHEM_PREFETCH_L1(ws + 106464);
      CHEM_PREFETCH_L1(ws + 106496);
      CHEM_PREFETCH_L1(ws + 106528);
      CHEM_PREFETCH_L1(ws + 106560);
      CHEM_PREFETCH_L1(ws + 106592);
      CHEM_PREFETCH_L1(ws + 106624);
      CHEM_PREFETCH_L1(ws + 106656);
      CHEM_PREFETCH_L1(ws + 106688);
      CHEM_PREFETCH_L1(ws + 106720);
      CHEM_PREFETCH_L1(ws + 106752);
      CHEM_PREFETCH_L1(ws + 106784);
      CHEM_PREFETCH_L1(ws + 136000);
      double x = b[4320];
      x = fma(-CHEM_LDLU(lu + 28448), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 28480), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 28512), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 28544), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 28576), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 28608), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 28640), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 28672), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 28704), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 28736), b[4736], x);
      b[4320] = x * CHEM_LDLU(vd + 4320);
    }
    {
      CHEM_PREFETCH(ws + 107168);
      CHEM_PREFETCH(ws + 107200);
      CHEM_PREFETCH(ws + 107232);
      CHEM_PREFETCH(ws + 107264);
      CHEM_PREFETCH(ws + 107296);
      CHEM_PREFETCH(ws + 107328);
      CHEM_PREFETCH(ws + 107360);
      CHEM_PREFETCH(ws + 107392);
      CHEM_PREFETCH(ws + 107424);
      CHEM_PREFETCH(ws + 107456);
      CHEM_PREFETCH(ws + 107488);
      CHEM_PREFETCH(ws + 135936);
      CHEM_PREFETCH_L1(ws + 106816);
      CHEM_PREFETCH_L1(ws + 106848);
      CHEM_PREFETCH_L1(ws + 106880);
      CHEM_PREFETCH_L1(ws + 106912);
      CHEM_PREFETCH_L1(ws + 106944);
      CHEM_PREFETCH_L1(ws + 106976);
      CHEM_PREFETCH_L1(ws + 107008);
      CHEM_PREFETCH_L1(ws + 107040);
      CHEM_PREFETCH_L1(ws + 107072);
      CHEM_PREFETCH_L1(ws + 107104);
      CHEM_PREFETCH_L1(ws + 107136);
      CHEM_PREFETCH_L1(ws + 135968);
      double x = b[4288];
      x = fma(-CHEM_LDLU(lu + 28768), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 28800), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 28832), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 28864), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 28896), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 28928), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 28960), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 28992), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 29024), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 29056), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 29088), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 29120), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 29152), b[4736], x);
      b[4288] = x * CHEM_LDLU(vd + 4288);
    }
    {
      CHEM_PREFETCH(ws + 107520);
      CHEM_PREFETCH(ws + 107552);
      CHEM_PREFETCH(ws + 107584);
      CHEM_PREFETCH(ws + 107616);
      CHEM_PREFETCH(ws + 107648);
      CHEM_PREFETCH(ws + 107680);
      CHEM_PREFETCH(ws + 107712);
      CHEM_PREFETCH(ws + 107744);
      CHEM_PREFETCH(ws + 107776);
      CHEM_PREFETCH(ws + 107808);
      CHEM_PREFETCH(ws + 107840);
      CHEM_PREFETCH(ws + 107872);
      CHEM_PREFETCH(ws + 107904);
      CHEM_PREFETCH(ws + 107936);
      CHEM_PREFETCH(ws + 135904);
      CHEM_PREFETCH_L1(ws + 107168);
      CHEM_PREFETCH_L1(ws + 107200);
      CHEM_PREFETCH_L1(ws + 107232);
      CHEM_PREFETCH_L1(ws + 107264);
      CHEM_PREFETCH_L1(ws + 107296);
      CHEM_PREFETCH_L1(ws + 107328);
      CHEM_PREFETCH_L1(ws + 107360);
      CHEM_PREFETCH_L1(ws + 107392);
      CHEM_PREFETCH_L1(ws + 107424);
      CHEM_PREFETCH_L1(ws + 107456);
      CHEM_PREFETCH_L1(ws + 107488);
      CHEM_PREFETCH_L1(ws + 135936);
      double x = b[4256];
      x = fma(-CHEM_LDLU(lu + 29184), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 29216), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 29248), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 29280), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 29312), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 29344), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 29376), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 29408), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 29440), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 29472), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 29504), b[4736], x);
      b[4256] = x * CHEM_LDLU(vd + 4256);
    }
    {
      CHEM_PREFETCH(ws + 107968);
      CHEM_PREFETCH(ws + 108000);
      CHEM_PREFETCH(ws + 108032);
      CHEM_PREFETCH(ws + 108064);
      CHEM_PREFETCH(ws + 108096);
      CHEM_PREFETCH(ws + 108128);
      CHEM_PREFETCH(ws + 108160);
      CHEM_PREFETCH(ws + 108192);
      CHEM_PREFETCH(ws + 108224);
      CHEM_PREFETCH(ws + 108256);
      CHEM_PREFETCH(ws + 108288);
      CHEM_PREFETCH(ws + 108320);
      CHEM_PREFETCH(ws + 135872);
      CHEM_PREFETCH_L1(ws + 107520);
      CHEM_PREFETCH_L1(ws + 107552);
      CHEM_PREFETCH_L1(ws + 107584);
      CHEM_PREFETCH_L1(ws + 107616);
      CHEM_PREFETCH_L1(ws + 107648);
      CHEM_PREFETCH_L1(ws + 107680);
      CHEM_PREFETCH_L1(ws + 107712);
      CHEM_PREFETCH_L1(ws + 107744);
      CHEM_PREFETCH_L1(ws + 107776);
      CHEM_PREFETCH_L1(ws + 107808);
      CHEM_PREFETCH_L1(ws + 107840);
      CHEM_PREFETCH_L1(ws + 107872);
      CHEM_PREFETCH_L1(ws + 107904);
      CHEM_PREFETCH_L1(ws + 107936);
      CHEM_PREFETCH_L1(ws + 135904);
      double x = b[4224];
      x = fma(-CHEM_LDLU(lu + 29536), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 29568), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 29600), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 29632), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 29664), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 29696), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 29728), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 29760), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 29792), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 29824), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 29856), b[4736], x);
      b[4224] = x * CHEM_LDLU(vd + 4224);
    }
    {
      CHEM_PREFETCH(ws + 108352);
      CHEM_PREFETCH(ws + 108384);
      CHEM_PREFETCH(ws + 108416);
      CHEM_PREFETCH(ws + 108448);
      CHEM_PREFETCH(ws + 108480);
      CHEM_PREFETCH(ws + 108512);
      CHEM_PREFETCH(ws + 108544);
      CHEM_PREFETCH(ws + 108576);
      CHEM_PREFETCH(ws + 108608);
      CHEM_PREFETCH(ws + 108640);
      CHEM_PREFETCH(ws + 108672);
      CHEM_PREFETCH(ws + 135840);
      CHEM_PREFETCH_L1(ws + 107968);
      CHEM_PREFETCH_L1(ws + 108000);
      CHEM_PREFETCH_L1(ws + 108032);
      CHEM_PREFETCH_L1(ws + 108064);
      CHEM_PREFETCH_L1(ws + 108096);
      CHEM_PREFETCH_L1(ws + 108128);
      CHEM_PREFETCH_L1(ws + 108160);
      CHEM_PREFETCH_L1(ws + 108192);
      CHEM_PREFETCH_L1(ws + 108224);
      CHEM_PREFETCH_L1(ws + 108256);
      CHEM_PREFETCH_L1(ws + 108288);
      CHEM_PREFETCH_L1(ws + 108320);
      CHEM_PREFETCH_L1(ws + 135872);
      double x = b[4192];
      x = fma(-CHEM_LDLU(lu + 29888), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 29920), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 29952), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 29984), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 30016), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 30048), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 30080), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 30112), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 30144), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 30176), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 30208), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 30240), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 30272), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 30304), b[4736], x);
      b[4192] = x * CHEM_LDLU(vd + 4192);
    }
    {
      CHEM_PREFETCH(ws + 108704);
      CHEM_PREFETCH(ws + 108736);
      CHEM_PREFETCH(ws + 108768);
      CHEM_PREFETCH(ws + 108800);
      CHEM_PREFETCH(ws + 108832);
      CHEM_PREFETCH(ws + 108864);
      CHEM_PREFETCH(ws + 108896);
      CHEM_PREFETCH(ws + 108928);
      CHEM_PREFETCH(ws + 108960);
      CHEM_PREFETCH(ws + 108992);
      CHEM_PREFETCH(ws + 109024);
      CHEM_PREFETCH(ws + 135808);
      CHEM_PREFETCH_L1(ws + 108352);
      CHEM_PREFETCH_L1(ws + 108384);
      CHEM_PREFETCH_L1(ws + 108416);
      CHEM_PREFETCH_L1(ws + 108448);
      CHEM_PREFETCH_L1(ws + 108480);
      CHEM_PREFETCH_L1(ws + 108512);
      CHEM_PREFETCH_L1(ws + 108544);
      CHEM_PREFETCH_L1(ws + 108576);
      CHEM_PREFETCH_L1(ws + 108608);
      CHEM_PREFETCH_L1(ws + 108640);
      CHEM_PREFETCH_L1(ws + 108672);
      CHEM_PREFETCH_L1(ws + 135840);
      double x = b[4160];
      x = fma(-CHEM_LDLU(lu + 30336), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 30368), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 30400), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 30432), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 30464), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 30496), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 30528), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 30560), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 30592), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 30624), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 30656), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 30688), b[4736], x);
      b[4160] = x * CHEM_LDLU(vd + 4160);
    }
    {
      CHEM_PREFETCH(ws + 109056);
      CHEM_PREFETCH(ws + 109088);
      CHEM_PREFETCH(ws + 109120);
      CHEM_PREFETCH(ws + 109152);
      CHEM_PREFETCH(ws + 109184);
      CHEM_PREFETCH(ws + 109216);
      CHEM_PREFETCH(ws + 109248);
      CHEM_PREFETCH(ws + 109280);
      CHEM_PREFETCH(ws + 109312);
      CHEM_PREFETCH(ws + 109344);
      CHEM_PREFETCH(ws + 109376);
      CHEM_PREFETCH(ws + 135776);
      CHEM_PREFETCH_L1(ws + 108704);
      CHEM_PREFETCH_L1(ws + 108736);
      CHEM_PREFETCH_L1(ws + 108768);
      CHEM_PREFETCH_L1(ws + 108800);
      CHEM_PREFETCH_L1(ws + 108832);
      CHEM_PREFETCH_L1(ws + 108864);
      CHEM_PREFETCH_L1(ws + 108896);
      CHEM_PREFETCH_L1(ws + 108928);
      CHEM_PREFETCH_L1(ws + 108960);
      CHEM_PREFETCH_L1(ws + 108992);
      CHEM_PREFETCH_L1(ws + 109024);
      CHEM_PREFETCH_L1(ws + 135808);
      double x = b[4128];
      x = fma(-CHEM_LDLU(lu + 30720), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 30752), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 30784), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 30816), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 30848), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 30880), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 30912), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 30944), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 30976), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 31008), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 31040), b[4736], x);
      b[4128] = x * CHEM_LDLU(vd + 4128);
    }
    {
      CHEM_PREFETCH(ws + 109408);
      CHEM_PREFETCH(ws + 109440);
      CHEM_PREFETCH(ws + 109472);
      CHEM_PREFETCH(ws + 109504);
      CHEM_PREFETCH(ws + 109536);
      CHEM_PREFETCH(ws + 109568);
      CHEM_PREFETCH(ws + 109600);
      CHEM_PREFETCH(ws + 109632);
      CHEM_PREFETCH(ws + 109664);
      CHEM_PREFETCH(ws + 109696);
      CHEM_PREFETCH(ws + 109728);
      CHEM_PREFETCH(ws + 109760);
      CHEM_PREFETCH(ws + 135744);
      CHEM_PREFETCH_L1(ws + 109056);
      CHEM_PREFETCH_L1(ws + 109088);
      CHEM_PREFETCH_L1(ws + 109120);
      CHEM_PREFETCH_L1(ws + 109152);
      CHEM_PREFETCH_L1(ws + 109184);
      CHEM_PREFETCH_L1(ws + 109216);
      CHEM_PREFETCH_L1(ws + 109248);
      CHEM_PREFETCH_L1(ws + 109280);
      CHEM_PREFETCH_L1(ws + 109312);
      CHEM_PREFETCH_L1(ws + 109344);
      CHEM_PREFETCH_L1(ws + 109376);
      CHEM_PREFETCH_L1(ws + 135776);
      double x = b[4096];
      x = fma(-CHEM_LDLU(lu + 31072), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 31104), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 31136), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 31168), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 31200), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 31232), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 31264), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 31296), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 31328), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 31360), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 31392), b[4736], x);
      b[4096] = x * CHEM_LDLU(vd + 4096);
    }
    {
      CHEM_PREFETCH(ws + 109792);
      CHEM_PREFETCH(ws + 109824);
      CHEM_PREFETCH(ws + 109856);
      CHEM_PREFETCH(ws + 109888);
      CHEM_PREFETCH(ws + 109920);
      CHEM_PREFETCH(ws + 109952);
      CHEM_PREFETCH(ws + 109984);
      CHEM_PREFETCH(ws + 110016);
      CHEM_PREFETCH(ws + 110048);
      CHEM_PREFETCH(ws + 110080);
      CHEM_PREFETCH(ws + 135712);
      CHEM_PREFETCH_L1(ws + 109408);
      CHEM_PREFETCH_L1(ws + 109440);
      CHEM_PREFETCH_L1(ws + 109472);
      CHEM_PREFETCH_L1(ws + 109504);
      CHEM_PREFETCH_L1(ws + 109536);
      CHEM_PREFETCH_L1(ws + 109568);
      CHEM_PREFETCH_L1(ws + 109600);
      CHEM_PREFETCH_L1(ws + 109632);
      CHEM_PREFETCH_L1(ws + 109664);
      CHEM_PREFETCH_L1(ws + 109696);
      CHEM_PREFETCH_L1(ws + 109728);
      CHEM_PREFETCH_L1(ws + 109760);
      CHEM_PREFETCH_L1(ws + 135744);
      double x = b[4064];
      x = fma(-CHEM_LDLU(lu + 31424), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 31456), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 31488), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 31520), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 31552), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 31584), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 31616), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 31648), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 31680), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 31712), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 31744), b[4736], x);
      b[4064] = x * CHEM_LDLU(vd + 4064);
    }
    {
      CHEM_PREFETCH(ws + 110112);
      CHEM_PREFETCH(ws + 110144);
      CHEM_PREFETCH(ws + 110176);
      CHEM_PREFETCH(ws + 110208);
      CHEM_PREFETCH(ws + 110240);
      CHEM_PREFETCH(ws + 110272);
      CHEM_PREFETCH(ws + 110304);
      CHEM_PREFETCH(ws + 110336);
      CHEM_PREFETCH(ws + 110368);
      CHEM_PREFETCH(ws + 110400);
      CHEM_PREFETCH(ws + 110432);
      CHEM_PREFETCH(ws + 110464);
      CHEM_PREFETCH(ws + 110496);
      CHEM_PREFETCH(ws + 110528);
      CHEM_PREFETCH(ws + 135680);
      CHEM_PREFETCH_L1(ws + 109792);
      CHEM_PREFETCH_L1(ws + 109824);
      CHEM_PREFETCH_L1(ws + 109856);
      CHEM_PREFETCH_L1(ws + 109888);
      CHEM_PREFETCH_L1(ws + 109920);
      CHEM_PREFETCH_L1(ws + 109952);
      CHEM_PREFETCH_L1(ws + 109984);
      CHEM_PREFETCH_L1(ws + 110016);
      CHEM_PREFETCH_L1(ws + 110048);
      CHEM_PREFETCH_L1(ws + 110080);
      CHEM_PREFETCH_L1(ws + 135712);
      double x = b[4032];
      x = fma(-CHEM_LDLU(lu + 31776), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 31808), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 31840), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 31872), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 31904), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 31936), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 31968), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 32000), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 32032), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 32064), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 32096), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 32128), b[4736], x);
      b[4032] = x * CHEM_LDLU(vd + 4032);
    }
    {
      CHEM_PREFETCH(ws + 110560);
      CHEM_PREFETCH(ws + 110592);
      CHEM_PREFETCH(ws + 110624);
      CHEM_PREFETCH(ws + 110656);
      CHEM_PREFETCH(ws + 110688);
      CHEM_PREFETCH(ws + 110720);
      CHEM_PREFETCH(ws + 110752);
      CHEM_PREFETCH(ws + 110784);
      CHEM_PREFETCH(ws + 110816);
      CHEM_PREFETCH(ws + 135648);
      CHEM_PREFETCH_L1(ws + 110112);
      CHEM_PREFETCH_L1(ws + 110144);
      CHEM_PREFETCH_L1(ws + 110176);
      CHEM_PREFETCH_L1(ws + 110208);
      CHEM_PREFETCH_L1(ws + 110240);
      CHEM_PREFETCH_L1(ws + 110272);
      CHEM_PREFETCH_L1(ws + 110304);
      CHEM_PREFETCH_L1(ws + 110336);
      CHEM_PREFETCH_L1(ws + 110368);
      CHEM_PREFETCH_L1(ws + 110400);
      CHEM_PREFETCH_L1(ws + 110432);
      CHEM_PREFETCH_L1(ws + 110464);
      CHEM_PREFETCH_L1(ws + 110496);
      CHEM_PREFETCH_L1(ws + 110528);
      CHEM_PREFETCH_L1(ws + 135680);
      double x = b[4000];
      x = fma(-CHEM_LDLU(lu + 32160), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 32192), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 32224), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 32256), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 32288), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 32320), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 32352), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 32384), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 32416), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 32448), b[4736], x);
      b[4000] = x * CHEM_LDLU(vd + 4000);
    }
    {
      CHEM_PREFETCH(ws + 110848);
      CHEM_PREFETCH(ws + 110880);
      CHEM_PREFETCH(ws + 110912);
      CHEM_PREFETCH(ws + 110944);
      CHEM_PREFETCH(ws + 110976);
      CHEM_PREFETCH(ws + 111008);
      CHEM_PREFETCH(ws + 111040);
      CHEM_PREFETCH(ws + 111072);
      CHEM_PREFETCH(ws + 111104);
      CHEM_PREFETCH(ws + 111136);
      CHEM_PREFETCH(ws + 111168);
      CHEM_PREFETCH(ws + 111200);
      CHEM_PREFETCH(ws + 111232);
      CHEM_PREFETCH(ws + 111264);
      CHEM_PREFETCH(ws + 111296);
      CHEM_PREFETCH(ws + 111328);
      CHEM_PREFETCH(ws + 135616);
      CHEM_PREFETCH_L1(ws + 110560);
      CHEM_PREFETCH_L1(ws + 110592);
      CHEM_PREFETCH_L1(ws + 110624);
      CHEM_PREFETCH_L1(ws + 110656);
      CHEM_PREFETCH_L1(ws + 110688);
      CHEM_PREFETCH_L1(ws + 110720);
      CHEM_PREFETCH_L1(ws + 110752);
      CHEM_PREFETCH_L1(ws + 110784);
      CHEM_PREFETCH_L1(ws + 110816);
      CHEM_PREFETCH_L1(ws + 135648);
      double x = b[3968];
      x = fma(-CHEM_LDLU(lu + 32480), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 32512), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 32544), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 32576), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 32608), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 32640), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 32672), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 32704), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 32736), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 32768), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 32800), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 32832), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 32864), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 32896), b[4736], x);
      b[3968] = x * CHEM_LDLU(vd + 3968);
    }
    {
      CHEM_PREFETCH(ws + 111360);
      CHEM_PREFETCH(ws + 111392);
      CHEM_PREFETCH(ws + 111424);
      CHEM_PREFETCH(ws + 111456);
      CHEM_PREFETCH(ws + 111488);
      CHEM_PREFETCH(ws + 111520);
      CHEM_PREFETCH(ws + 111552);
      CHEM_PREFETCH(ws + 111584);
      CHEM_PREFETCH(ws + 111616);
      CHEM_PREFETCH(ws + 135584);
      CHEM_PREFETCH_L1(ws + 110848);
      CHEM_PREFETCH_L1(ws + 110880);
      CHEM_PREFETCH_L1(ws + 110912);
      CHEM_PREFETCH_L1(ws + 110944);
      CHEM_PREFETCH_L1(ws + 110976);
      CHEM_PREFETCH_L1(ws + 111008);
      CHEM_PREFETCH_L1(ws + 111040);
      CHEM_PREFETCH_L1(ws + 111072);
      CHEM_PREFETCH_L1(ws + 111104);
      CHEM_PREFETCH_L1(ws + 111136);
      CHEM_PREFETCH_L1(ws + 111168);
      CHEM_PREFETCH_L1(ws + 111200);
      CHEM_PREFETCH_L1(ws + 111232);
      CHEM_PREFETCH_L1(ws + 111264);
      CHEM_PREFETCH_L1(ws + 111296);
      CHEM_PREFETCH_L1(ws + 111328);
      CHEM_PREFETCH_L1(ws + 135616);
      double x = b[3936];
      x = fma(-CHEM_LDLU(lu + 32928), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 32960), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 32992), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 33024), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 33056), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 33088), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 33120), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 33152), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 33184), b[4736], x);
      b[3936] = x * CHEM_LDLU(vd + 3936);
    }
    {
      CHEM_PREFETCH(ws + 111648);
      CHEM_PREFETCH(ws + 111680);
      CHEM_PREFETCH(ws + 111712);
      CHEM_PREFETCH(ws + 111744);
      CHEM_PREFETCH(ws + 111776);
      CHEM_PREFETCH(ws + 111808);
      CHEM_PREFETCH(ws + 111840);
      CHEM_PREFETCH(ws + 111872);
      CHEM_PREFETCH(ws + 111904);
      CHEM_PREFETCH(ws + 111936);
      CHEM_PREFETCH(ws + 135552);
      CHEM_PREFETCH_L1(ws + 111360);
      CHEM_PREFETCH_L1(ws + 111392);
      CHEM_PREFETCH_L1(ws + 111424);
      CHEM_PREFETCH_L1(ws + 111456);
      CHEM_PREFETCH_L1(ws + 111488);
      CHEM_PREFETCH_L1(ws + 111520);
      CHEM_PREFETCH_L1(ws + 111552);
      CHEM_PREFETCH_L1(ws + 111584);
      CHEM_PREFETCH_L1(ws + 111616);
      CHEM_PREFETCH_L1(ws + 135584);
      double x = b[3904];
      x = fma(-CHEM_LDLU(lu + 33216), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 33248), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 33280), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 33312), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 33344), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 33376), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 33408), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 33440), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 33472), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 33504), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 33536), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 33568), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 33600), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 33632), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 33664), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 33696), b[4736], x);
      b[3904] = x * CHEM_LDLU(vd + 3904);
    }
    {
      CHEM_PREFETCH(ws + 111968);
      CHEM_PREFETCH(ws + 112000);
      CHEM_PREFETCH(ws + 112032);
      CHEM_PREFETCH(ws + 112064);
      CHEM_PREFETCH(ws + 112096);
      CHEM_PREFETCH(ws + 112128);
      CHEM_PREFETCH(ws + 112160);
      CHEM_PREFETCH(ws + 112192);
      CHEM_PREFETCH(ws + 135520);
      CHEM_PREFETCH_L1(ws + 111648);
      CHEM_PREFETCH_L1(ws + 111680);
      CHEM_PREFETCH_L1(ws + 111712);
      CHEM_PREFETCH_L1(ws + 111744);
      CHEM_PREFETCH_L1(ws + 111776);
      CHEM_PREFETCH_L1(ws + 111808);
      CHEM_PREFETCH_L1(ws + 111840);
      CHEM_PREFETCH_L1(ws + 111872);
      CHEM_PREFETCH_L1(ws + 111904);
      CHEM_PREFETCH_L1(ws + 111936);
      CHEM_PREFETCH_L1(ws + 135552);
      double x = b[3872];
      x = fma(-CHEM_LDLU(lu + 33728), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 33760), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 33792), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 33824), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 33856), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 33888), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 33920), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 33952), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 33984), b[4736], x);
      b[3872] = x * CHEM_LDLU(vd + 3872);
    }
    {
      CHEM_PREFETCH(ws + 112224);
      CHEM_PREFETCH(ws + 112256);
      CHEM_PREFETCH(ws + 112288);
      CHEM_PREFETCH(ws + 112320);
      CHEM_PREFETCH(ws + 112352);
      CHEM_PREFETCH(ws + 112384);
      CHEM_PREFETCH(ws + 112416);
      CHEM_PREFETCH(ws + 112448);
      CHEM_PREFETCH(ws + 112480);
      CHEM_PREFETCH(ws + 112512);
      CHEM_PREFETCH(ws + 112544);
      CHEM_PREFETCH(ws + 135488);
      CHEM_PREFETCH_L1(ws + 111968);
      CHEM_PREFETCH_L1(ws + 112000);
      CHEM_PREFETCH_L1(ws + 112032);
      CHEM_PREFETCH_L1(ws + 112064);
      CHEM_PREFETCH_L1(ws + 112096);
      CHEM_PREFETCH_L1(ws + 112128);
      CHEM_PREFETCH_L1(ws + 112160);
      CHEM_PREFETCH_L1(ws + 112192);
      CHEM_PREFETCH_L1(ws + 135520);
      double x = b[3840];
      x = fma(-CHEM_LDLU(lu + 34016), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 34048), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 34080), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 34112), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 34144), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 34176), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 34208), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 34240), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 34272), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 34304), b[4736], x);
      b[3840] = x * CHEM_LDLU(vd + 3840);
    }
    {
      CHEM_PREFETCH(ws + 112576);
      CHEM_PREFETCH(ws + 112608);
      CHEM_PREFETCH(ws + 112640);
      CHEM_PREFETCH(ws + 112672);
      CHEM_PREFETCH(ws + 112704);
      CHEM_PREFETCH(ws + 112736);
      CHEM_PREFETCH(ws + 112768);
      CHEM_PREFETCH(ws + 112800);
      CHEM_PREFETCH(ws + 112832);
      CHEM_PREFETCH(ws + 112864);
      CHEM_PREFETCH(ws + 135456);
      CHEM_PREFETCH_L1(ws + 112224);
      CHEM_PREFETCH_L1(ws + 112256);
      CHEM_PREFETCH_L1(ws + 112288);
      CHEM_PREFETCH_L1(ws + 112320);
      CHEM_PREFETCH_L1(ws + 112352);
      CHEM_PREFETCH_L1(ws + 112384);
      CHEM_PREFETCH_L1(ws + 112416);
      CHEM_PREFETCH_L1(ws + 112448);
      CHEM_PREFETCH_L1(ws + 112480);
      CHEM_PREFETCH_L1(ws + 112512);
      CHEM_PREFETCH_L1(ws + 112544);
      CHEM_PREFETCH_L1(ws + 135488);
      double x = b[3808];
      x = fma(-CHEM_LDLU(lu + 34336), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 34368), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 34400), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 34432), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 34464), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 34496), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 34528), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 34560), b[4736], x);
      b[3808] = x * CHEM_LDLU(vd + 3808);
    }
    {
      CHEM_PREFETCH(ws + 112896);
      CHEM_PREFETCH(ws + 135424);
      CHEM_PREFETCH_L1(ws + 112576);
      CHEM_PREFETCH_L1(ws + 112608);
      CHEM_PREFETCH_L1(ws + 112640);
      CHEM_PREFETCH_L1(ws + 112672);
      CHEM_PREFETCH_L1(ws + 112704);
      CHEM_PREFETCH_L1(ws + 112736);
      CHEM_PREFETCH_L1(ws + 112768);
      CHEM_PREFETCH_L1(ws + 112800);
      CHEM_PREFETCH_L1(ws + 112832);
      CHEM_PREFETCH_L1(ws + 112864);
      CHEM_PREFETCH_L1(ws + 135456);
      double x = b[3776];
      x = fma(-CHEM_LDLU(lu + 34592), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 34624), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 34656), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 34688), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 34720), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 34752), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 34784), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 34816), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 34848), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 34880), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 34912), b[4736], x);
      b[3776] = x * CHEM_LDLU(vd + 3776);
    }
    {
      CHEM_PREFETCH(ws + 112928);
      CHEM_PREFETCH(ws + 112960);
      CHEM_PREFETCH(ws + 135392);
      CHEM_PREFETCH_L1(ws + 112896);
      CHEM_PREFETCH_L1(ws + 135424);
      double x = b[3744];
      x = fma(-CHEM_LDLU(lu + 34944), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 34976), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 35008), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 35040), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 35072), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 35104), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 35136), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 35168), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 35200), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 35232), b[4736], x);
      b[3744] = x * CHEM_LDLU(vd + 3744);
    }
    {
      CHEM_PREFETCH(ws + 112992);
      CHEM_PREFETCH(ws + 113024);
      CHEM_PREFETCH(ws + 113056);
      CHEM_PREFETCH(ws + 113088);
      CHEM_PREFETCH(ws + 113120);
      CHEM_PREFETCH(ws + 113152);
      CHEM_PREFETCH(ws + 113184);
      CHEM_PREFETCH(ws + 113216);
      CHEM_PREFETCH(ws + 113248);
      CHEM_PREFETCH(ws + 113280);
      CHEM_PREFETCH(ws + 113312);
      CHEM_PREFETCH(ws + 113344);
      CHEM_PREFETCH(ws + 135360);
      CHEM_PREFETCH_L1(ws + 112928);
      CHEM_PREFETCH_L1(ws + 112960);
      CHEM_PREFETCH_L1(ws + 135392);
      double x = b[3712];
      x = fma(-CHEM_LDLU(lu + 35264), b[4736], x);
      b[3712] = x * CHEM_LDLU(vd + 3712);
    }
    {
      CHEM_PREFETCH(ws + 113376);
      CHEM_PREFETCH(ws + 113408);
      CHEM_PREFETCH(ws + 113440);
      CHEM_PREFETCH(ws + 113472);
      CHEM_PREFETCH(ws + 113504);
      CHEM_PREFETCH(ws + 135328);
      CHEM_PREFETCH_L1(ws + 112992);
      CHEM_PREFETCH_L1(ws + 113024);
      CHEM_PREFETCH_L1(ws + 113056);
      CHEM_PREFETCH_L1(ws + 113088);
      CHEM_PREFETCH_L1(ws + 113120);
      CHEM_PREFETCH_L1(ws + 113152);
      CHEM_PREFETCH_L1(ws + 113184);
      CHEM_PREFETCH_L1(ws + 113216);
      CHEM_PREFETCH_L1(ws + 113248);
      CHEM_PREFETCH_L1(ws + 113280);
      CHEM_PREFETCH_L1(ws + 113312);
      CHEM_PREFETCH_L1(ws + 113344);
      CHEM_PREFETCH_L1(ws + 135360);
      double x = b[3680];
      x = fma(-CHEM_LDLU(lu + 35296), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 35328), b[4736], x);
      b[3680] = x * CHEM_LDLU(vd + 3680);
    }
    {
      CHEM_PREFETCH(ws + 113536);
      CHEM_PREFETCH(ws + 113568);
      CHEM_PREFETCH(ws + 113600);
      CHEM_PREFETCH(ws + 113632);
      CHEM_PREFETCH(ws + 113664);
      CHEM_PREFETCH(ws + 113696);
      CHEM_PREFETCH(ws + 135296);
      CHEM_PREFETCH_L1(ws + 113376);
      CHEM_PREFETCH_L1(ws + 113408);
      CHEM_PREFETCH_L1(ws + 113440);
      CHEM_PREFETCH_L1(ws + 113472);
      CHEM_PREFETCH_L1(ws + 113504);
      CHEM_PREFETCH_L1(ws + 135328);
      double x = b[3648];
      x = fma(-CHEM_LDLU(lu + 35360), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 35392), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 35424), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 35456), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 35488), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 35520), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 35552), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 35584), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 35616), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 35648), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 35680), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 35712), b[4736], x);
      b[3648] = x * CHEM_LDLU(vd + 3648);
    }
    {
      CHEM_PREFETCH(ws + 113728);
      CHEM_PREFETCH(ws + 113760);
      CHEM_PREFETCH(ws + 113792);
      CHEM_PREFETCH(ws + 113824);
      CHEM_PREFETCH(ws + 113856);
      CHEM_PREFETCH(ws + 113888);
      CHEM_PREFETCH(ws + 113920);
      CHEM_PREFETCH(ws + 113952);
      CHEM_PREFETCH(ws + 113984);
      CHEM_PREFETCH(ws + 135264);
      CHEM_PREFETCH_L1(ws + 113536);
      CHEM_PREFETCH_L1(ws + 113568);
      CHEM_PREFETCH_L1(ws + 113600);
      CHEM_PREFETCH_L1(ws + 113632);
      CHEM_PREFETCH_L1(ws + 113664);
      CHEM_PREFETCH_L1(ws + 113696);
      CHEM_PREFETCH_L1(ws + 135296);
      double x = b[3616];
      x = fma(-CHEM_LDLU(lu + 35744), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 35776), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 35808), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 35840), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 35872), b[4736], x);
      b[3616] = x * CHEM_LDLU(vd + 3616);
    }
    {
      CHEM_PREFETCH(ws + 114016);
      CHEM_PREFETCH(ws + 114048);
      CHEM_PREFETCH(ws + 114080);
      CHEM_PREFETCH(ws + 114112);
      CHEM_PREFETCH(ws + 114144);
      CHEM_PREFETCH(ws + 114176);
      CHEM_PREFETCH(ws + 114208);
      CHEM_PREFETCH(ws + 114240);
      CHEM_PREFETCH(ws + 135232);
      CHEM_PREFETCH_L1(ws + 113728);
      CHEM_PREFETCH_L1(ws + 113760);
      CHEM_PREFETCH_L1(ws + 113792);
      CHEM_PREFETCH_L1(ws + 113824);
      CHEM_PREFETCH_L1(ws + 113856);
      CHEM_PREFETCH_L1(ws + 113888);
      CHEM_PREFETCH_L1(ws + 113920);
      CHEM_PREFETCH_L1(ws + 113952);
      CHEM_PREFETCH_L1(ws + 113984);
      CHEM_PREFETCH_L1(ws + 135264);
      double x = b[3584];
      x = fma(-CHEM_LDLU(lu + 35904), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 35936), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 35968), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 36000), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 36032), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 36064), b[4736], x);
      b[3584] = x * CHEM_LDLU(vd + 3584);
    }
    {
      CHEM_PREFETCH(ws + 114272);
      CHEM_PREFETCH(ws + 114304);
      CHEM_PREFETCH(ws + 114336);
      CHEM_PREFETCH(ws + 114368);
      CHEM_PREFETCH(ws + 114400);
      CHEM_PREFETCH(ws + 114432);
      CHEM_PREFETCH(ws + 135200);
      CHEM_PREFETCH_L1(ws + 114016);
      CHEM_PREFETCH_L1(ws + 114048);
      CHEM_PREFETCH_L1(ws + 114080);
      CHEM_PREFETCH_L1(ws + 114112);
      CHEM_PREFETCH_L1(ws + 114144);
      CHEM_PREFETCH_L1(ws + 114176);
      CHEM_PREFETCH_L1(ws + 114208);
      CHEM_PREFETCH_L1(ws + 114240);
      CHEM_PREFETCH_L1(ws + 135232);
      double x = b[3552];
      x = fma(-CHEM_LDLU(lu + 36096), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 36128), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 36160), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 36192), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 36224), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 36256), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 36288), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 36320), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 36352), b[4736], x);
      b[3552] = x * CHEM_LDLU(vd + 3552);
    }
    {
      CHEM_PREFETCH(ws + 114464);
      CHEM_PREFETCH(ws + 114496);
      CHEM_PREFETCH(ws + 114528);
      CHEM_PREFETCH(ws + 114560);
      CHEM_PREFETCH(ws + 114592);
      CHEM_PREFETCH(ws + 114624);
      CHEM_PREFETCH(ws + 114656);
      CHEM_PREFETCH(ws + 114688);
      CHEM_PREFETCH(ws + 114720);
      CHEM_PREFETCH(ws + 114752);
      CHEM_PREFETCH(ws + 114784);
      CHEM_PREFETCH(ws + 135168);
      CHEM_PREFETCH_L1(ws + 114272);
      CHEM_PREFETCH_L1(ws + 114304);
      CHEM_PREFETCH_L1(ws + 114336);
      CHEM_PREFETCH_L1(ws + 114368);
      CHEM_PREFETCH_L1(ws + 114400);
      CHEM_PREFETCH_L1(ws + 114432);
      CHEM_PREFETCH_L1(ws + 135200);
      double x = b[3520];
      x = fma(-CHEM_LDLU(lu + 36384), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 36416), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 36448), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 36480), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 36512), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 36544), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 36576), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 36608), b[4736], x);
      b[3520] = x * CHEM_LDLU(vd + 3520);
    }
    {
      CHEM_PREFETCH(ws + 114816);
      CHEM_PREFETCH(ws + 114848);
      CHEM_PREFETCH(ws + 114880);
      CHEM_PREFETCH(ws + 114912);
      CHEM_PREFETCH(ws + 114944);
      CHEM_PREFETCH(ws + 114976);
      CHEM_PREFETCH(ws + 115008);
      CHEM_PREFETCH(ws + 115040);
      CHEM_PREFETCH(ws + 115072);
      CHEM_PREFETCH(ws + 135136);
      CHEM_PREFETCH_L1(ws + 114464);
      CHEM_PREFETCH_L1(ws + 114496);
      CHEM_PREFETCH_L1(ws + 114528);
      CHEM_PREFETCH_L1(ws + 114560);
      CHEM_PREFETCH_L1(ws + 114592);
      CHEM_PREFETCH_L1(ws + 114624);
      CHEM_PREFETCH_L1(ws + 114656);
      CHEM_PREFETCH_L1(ws + 114688);
      CHEM_PREFETCH_L1(ws + 114720);
      CHEM_PREFETCH_L1(ws + 114752);
      CHEM_PREFETCH_L1(ws + 114784);
      CHEM_PREFETCH_L1(ws + 135168);
      double x = b[3488];
      x = fma(-CHEM_LDLU(lu + 36640), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 36672), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 36704), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 36736), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 36768), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 36800), b[4736], x);
      b[3488] = x * CHEM_LDLU(vd + 3488);
    }
    {
      CHEM_PREFETCH(ws + 115104);
      CHEM_PREFETCH(ws + 115136);
      CHEM_PREFETCH(ws + 115168);
      CHEM_PREFETCH(ws + 115200);
      CHEM_PREFETCH(ws + 115232);
      CHEM_PREFETCH(ws + 115264);
      CHEM_PREFETCH(ws + 135104);
      CHEM_PREFETCH_L1(ws + 114816);
      CHEM_PREFETCH_L1(ws + 114848);
      CHEM_PREFETCH_L1(ws + 114880);
      CHEM_PREFETCH_L1(ws + 114912);
      CHEM_PREFETCH_L1(ws + 114944);
      CHEM_PREFETCH_L1(ws + 114976);
      CHEM_PREFETCH_L1(ws + 115008);
      CHEM_PREFETCH_L1(ws + 115040);
      CHEM_PREFETCH_L1(ws + 115072);
      CHEM_PREFETCH_L1(ws + 135136);
      double x = b[3456];
      x = fma(-CHEM_LDLU(lu + 36832), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 36864), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 36896), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 36928), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 36960), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 36992), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 37024), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 37056), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 37088), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 37120), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 37152), b[4736], x);
      b[3456] = x * CHEM_LDLU(vd + 3456);
    }
    {
      CHEM_PREFETCH(ws + 115296);
      CHEM_PREFETCH(ws + 115328);
      CHEM_PREFETCH(ws + 115360);
      CHEM_PREFETCH(ws + 115392);
      CHEM_PREFETCH(ws + 115424);
      CHEM_PREFETCH(ws + 115456);
      CHEM_PREFETCH(ws + 115488);
      CHEM_PREFETCH(ws + 115520);
      CHEM_PREFETCH(ws + 135072);
      CHEM_PREFETCH_L1(ws + 115104);
      CHEM_PREFETCH_L1(ws + 115136);
      CHEM_PREFETCH_L1(ws + 115168);
      CHEM_PREFETCH_L1(ws + 115200);
      CHEM_PREFETCH_L1(ws + 115232);
      CHEM_PREFETCH_L1(ws + 115264);
      CHEM_PREFETCH_L1(ws + 135104);
      double x = b[3424];
      x = fma(-CHEM_LDLU(lu + 37184), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 37216), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 37248), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 37280), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 37312), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 37344), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 37376), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 37408), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 37440), b[4736], x);
      b[3424] = x * CHEM_LDLU(vd + 3424);
    }
    {
      CHEM_PREFETCH(ws + 115552);
      CHEM_PREFETCH(ws + 115584);
      CHEM_PREFETCH(ws + 115616);
      CHEM_PREFETCH(ws + 115648);
      CHEM_PREFETCH(ws + 115680);
      CHEM_PREFETCH(ws + 135040);
      CHEM_PREFETCH_L1(ws + 115296);
      CHEM_PREFETCH_L1(ws + 115328);
      CHEM_PREFETCH_L1(ws + 115360);
      CHEM_PREFETCH_L1(ws + 115392);
      CHEM_PREFETCH_L1(ws + 115424);
      CHEM_PREFETCH_L1(ws + 115456);
      CHEM_PREFETCH_L1(ws + 115488);
      CHEM_PREFETCH_L1(ws + 115520);
      CHEM_PREFETCH_L1(ws + 135072);
      double x = b[3392];
      x = fma(-CHEM_LDLU(lu + 37472), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 37504), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 37536), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 37568), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 37600), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 37632), b[4736], x);
      b[3392] = x * CHEM_LDLU(vd + 3392);
    }
    {
      CHEM_PREFETCH(ws + 115712);
      CHEM_PREFETCH(ws + 115744);
      CHEM_PREFETCH(ws + 115776);
      CHEM_PREFETCH(ws + 115808);
      CHEM_PREFETCH(ws + 115840);
      CHEM_PREFETCH(ws + 115872);
      CHEM_PREFETCH(ws + 135008);
      CHEM_PREFETCH_L1(ws + 115552);
      CHEM_PREFETCH_L1(ws + 115584);
      CHEM_PREFETCH_L1(ws + 115616);
      CHEM_PREFETCH_L1(ws + 115648);
      CHEM_PREFETCH_L1(ws + 115680);
      CHEM_PREFETCH_L1(ws + 135040);
      double x = b[3360];
      x = fma(-CHEM_LDLU(lu + 37664), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 37696), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 37728), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 37760), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 37792), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 37824), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 37856), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 37888), b[4736], x);
      b[3360] = x * CHEM_LDLU(vd + 3360);
    }
    {
      CHEM_PREFETCH(ws + 115904);
      CHEM_PREFETCH(ws + 115936);
      CHEM_PREFETCH(ws + 115968);
      CHEM_PREFETCH(ws + 116000);
      CHEM_PREFETCH(ws + 134976);
      CHEM_PREFETCH_L1(ws + 115712);
      CHEM_PREFETCH_L1(ws + 115744);
      CHEM_PREFETCH_L1(ws + 115776);
      CHEM_PREFETCH_L1(ws + 115808);
      CHEM_PREFETCH_L1(ws + 115840);
      CHEM_PREFETCH_L1(ws + 115872);
      CHEM_PREFETCH_L1(ws + 135008);
      double x = b[3328];
      x = fma(-CHEM_LDLU(lu + 37920), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 37952), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 37984), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 38016), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 38048), b[4736], x);
      b[3328] = x * CHEM_LDLU(vd + 3328);
    }
    {
      CHEM_PREFETCH(ws + 116032);
      CHEM_PREFETCH(ws + 116064);
      CHEM_PREFETCH(ws + 116096);
      CHEM_PREFETCH(ws + 116128);
      CHEM_PREFETCH(ws + 116160);
      CHEM_PREFETCH(ws + 116192);
      CHEM_PREFETCH(ws + 116224);
      CHEM_PREFETCH(ws + 116256);
      CHEM_PREFETCH(ws + 134944);
      CHEM_PREFETCH_L1(ws + 115904);
      CHEM_PREFETCH_L1(ws + 115936);
      CHEM_PREFETCH_L1(ws + 115968);
      CHEM_PREFETCH_L1(ws + 116000);
      CHEM_PREFETCH_L1(ws + 134976);
      double x = b[3296];
      x = fma(-CHEM_LDLU(lu + 38080), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 38112), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 38144), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 38176), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 38208), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 38240), b[4736], x);
      b[3296] = x * CHEM_LDLU(vd + 3296);
    }
    {
      CHEM_PREFETCH(ws + 116288);
      CHEM_PREFETCH(ws + 116320);
      CHEM_PREFETCH(ws + 116352);
      CHEM_PREFETCH(ws + 134912);
      CHEM_PREFETCH_L1(ws + 116032);
      CHEM_PREFETCH_L1(ws + 116064);
      CHEM_PREFETCH_L1(ws + 116096);
      CHEM_PREFETCH_L1(ws + 116128);
      CHEM_PREFETCH_L1(ws + 116160);
      CHEM_PREFETCH_L1(ws + 116192);
      CHEM_PREFETCH_L1(ws + 116224);
      CHEM_PREFETCH_L1(ws + 116256);
      CHEM_PREFETCH_L1(ws + 134944);
      double x = b[3264];
      x = fma(-CHEM_LDLU(lu + 38272), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 38304), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 38336), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 38368), b[4736], x);
      b[3264] = x * CHEM_LDLU(vd + 3264);
    }
    {
      CHEM_PREFETCH(ws + 116384);
      CHEM_PREFETCH(ws + 116416);
      CHEM_PREFETCH(ws + 116448);
      CHEM_PREFETCH(ws + 116480);
      CHEM_PREFETCH(ws + 134880);
      CHEM_PREFETCH_L1(ws + 116288);
      CHEM_PREFETCH_L1(ws + 116320);
      CHEM_PREFETCH_L1(ws + 116352);
      CHEM_PREFETCH_L1(ws + 134912);
      double x = b[3232];
      x = fma(-CHEM_LDLU(lu + 38400), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 38432), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 38464), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 38496), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 38528), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 38560), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 38592), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 38624), b[4736], x);
      b[3232] = x * CHEM_LDLU(vd + 3232);
    }
    {
      CHEM_PREFETCH(ws + 116512);
      CHEM_PREFETCH(ws + 116544);
      CHEM_PREFETCH(ws + 116576);
      CHEM_PREFETCH(ws + 116608);
      CHEM_PREFETCH(ws + 116640);
      CHEM_PREFETCH(ws + 116672);
      CHEM_PREFETCH(ws + 116704);
      CHEM_PREFETCH(ws + 134848);
      CHEM_PREFETCH_L1(ws + 116384);
      CHEM_PREFETCH_L1(ws + 116416);
      CHEM_PREFETCH_L1(ws + 116448);
      CHEM_PREFETCH_L1(ws + 116480);
      CHEM_PREFETCH_L1(ws + 134880);
      double x = b[3200];
      x = fma(-CHEM_LDLU(lu + 38656), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 38688), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 38720), b[4736], x);
      b[3200] = x * CHEM_LDLU(vd + 3200);
    }
    {
      CHEM_PREFETCH(ws + 116736);
      CHEM_PREFETCH(ws + 116768);
      CHEM_PREFETCH(ws + 116800);
      CHEM_PREFETCH(ws + 116832);
      CHEM_PREFETCH(ws + 116864);
      CHEM_PREFETCH(ws + 134816);
      CHEM_PREFETCH_L1(ws + 116512);
      CHEM_PREFETCH_L1(ws + 116544);
      CHEM_PREFETCH_L1(ws + 116576);
      CHEM_PREFETCH_L1(ws + 116608);
      CHEM_PREFETCH_L1(ws + 116640);
      CHEM_PREFETCH_L1(ws + 116672);
      CHEM_PREFETCH_L1(ws + 116704);
      CHEM_PREFETCH_L1(ws + 134848);
      double x = b[3168];
      x = fma(-CHEM_LDLU(lu + 38752), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 38784), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 38816), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 38848), b[4736], x);
      b[3168] = x * CHEM_LDLU(vd + 3168);
    }
    {
      CHEM_PREFETCH(ws + 116896);
      CHEM_PREFETCH(ws + 116928);
      CHEM_PREFETCH(ws + 116960);
      CHEM_PREFETCH(ws + 116992);
      CHEM_PREFETCH(ws + 134784);
      CHEM_PREFETCH_L1(ws + 116736);
      CHEM_PREFETCH_L1(ws + 116768);
      CHEM_PREFETCH_L1(ws + 116800);
      CHEM_PREFETCH_L1(ws + 116832);
      CHEM_PREFETCH_L1(ws + 116864);
      CHEM_PREFETCH_L1(ws + 134816);
      double x = b[3136];
      x = fma(-CHEM_LDLU(lu + 38880), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 38912), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 38944), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 38976), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 39008), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 39040), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 39072), b[4736], x);
      b[3136] = x * CHEM_LDLU(vd + 3136);
    }
    {
      CHEM_PREFETCH(ws + 117024);
      CHEM_PREFETCH(ws + 117056);
      CHEM_PREFETCH(ws + 117088);
      CHEM_PREFETCH(ws + 117120);
      CHEM_PREFETCH(ws + 117152);
      CHEM_PREFETCH(ws + 134752);
      CHEM_PREFETCH_L1(ws + 116896);
      CHEM_PREFETCH_L1(ws + 116928);
      CHEM_PREFETCH_L1(ws + 116960);
      CHEM_PREFETCH_L1(ws + 116992);
      CHEM_PREFETCH_L1(ws + 134784);
      double x = b[3104];
      x = fma(-CHEM_LDLU(lu + 39104), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 39136), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 39168), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 39200), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 39232), b[4736], x);
      b[3104] = x * CHEM_LDLU(vd + 3104);
    }
    {
      CHEM_PREFETCH(ws + 117184);
      CHEM_PREFETCH(ws + 117216);
      CHEM_PREFETCH(ws + 117248);
      CHEM_PREFETCH(ws + 117280);
      CHEM_PREFETCH(ws + 117312);
      CHEM_PREFETCH(ws + 134720);
      CHEM_PREFETCH_L1(ws + 117024);
      CHEM_PREFETCH_L1(ws + 117056);
      CHEM_PREFETCH_L1(ws + 117088);
      CHEM_PREFETCH_L1(ws + 117120);
      CHEM_PREFETCH_L1(ws + 117152);
      CHEM_PREFETCH_L1(ws + 134752);
      double x = b[3072];
      x = fma(-CHEM_LDLU(lu + 39264), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 39296), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 39328), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 39360), b[4736], x);
      b[3072] = x * CHEM_LDLU(vd + 3072);
    }
    {
      CHEM_PREFETCH(ws + 117344);
      CHEM_PREFETCH(ws + 117376);
      CHEM_PREFETCH(ws + 117408);
      CHEM_PREFETCH(ws + 117440);
      CHEM_PREFETCH(ws + 134688);
      CHEM_PREFETCH_L1(ws + 117184);
      CHEM_PREFETCH_L1(ws + 117216);
      CHEM_PREFETCH_L1(ws + 117248);
      CHEM_PREFETCH_L1(ws + 117280);
      CHEM_PREFETCH_L1(ws + 117312);
      CHEM_PREFETCH_L1(ws + 134720);
      double x = b[3040];
      x = fma(-CHEM_LDLU(lu + 39392), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 39424), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 39456), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 39488), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 39520), b[4736], x);
      b[3040] = x * CHEM_LDLU(vd + 3040);
    }
    {
      CHEM_PREFETCH(ws + 117472);
      CHEM_PREFETCH(ws + 117504);
      CHEM_PREFETCH(ws + 117536);
      CHEM_PREFETCH(ws + 117568);
      CHEM_PREFETCH(ws + 134656);
      CHEM_PREFETCH_L1(ws + 117344);
      CHEM_PREFETCH_L1(ws + 117376);
      CHEM_PREFETCH_L1(ws + 117408);
      CHEM_PREFETCH_L1(ws + 117440);
      CHEM_PREFETCH_L1(ws + 134688);
      double x = b[3008];
      x = fma(-CHEM_LDLU(lu + 39552), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 39584), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 39616), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 39648), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 39680), b[4736], x);
      b[3008] = x * CHEM_LDLU(vd + 3008);
    }
    {
      CHEM_PREFETCH(ws + 117600);
      CHEM_PREFETCH(ws + 117632);
      CHEM_PREFETCH(ws + 117664);
      CHEM_PREFETCH(ws + 117696);
      CHEM_PREFETCH(ws + 117728);
      CHEM_PREFETCH(ws + 134624);
      CHEM_PREFETCH_L1(ws + 117472);
      CHEM_PREFETCH_L1(ws + 117504);
      CHEM_PREFETCH_L1(ws + 117536);
      CHEM_PREFETCH_L1(ws + 117568);
      CHEM_PREFETCH_L1(ws + 134656);
      double x = b[2976];
      x = fma(-CHEM_LDLU(lu + 39712), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 39744), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 39776), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 39808), b[4736], x);
      b[2976] = x * CHEM_LDLU(vd + 2976);
    }
    {
      CHEM_PREFETCH(ws + 117760);
      CHEM_PREFETCH(ws + 117792);
      CHEM_PREFETCH(ws + 117824);
      CHEM_PREFETCH(ws + 117856);
      CHEM_PREFETCH(ws + 117888);
      CHEM_PREFETCH(ws + 134592);
      CHEM_PREFETCH_L1(ws + 117600);
      CHEM_PREFETCH_L1(ws + 117632);
      CHEM_PREFETCH_L1(ws + 117664);
      CHEM_PREFETCH_L1(ws + 117696);
      CHEM_PREFETCH_L1(ws + 117728);
      CHEM_PREFETCH_L1(ws + 134624);
      double x = b[2944];
      x = fma(-CHEM_LDLU(lu + 39840), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 39872), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 39904), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 39936), b[4736], x);
      b[2944] = x * CHEM_LDLU(vd + 2944);
    }
    {
      CHEM_PREFETCH(ws + 117920);
      CHEM_PREFETCH(ws + 117952);
      CHEM_PREFETCH(ws + 117984);
      CHEM_PREFETCH(ws + 118016);
      CHEM_PREFETCH(ws + 118048);
      CHEM_PREFETCH(ws + 118080);
      CHEM_PREFETCH(ws + 118112);
      CHEM_PREFETCH(ws + 134560);
      CHEM_PREFETCH_L1(ws + 117760);
      CHEM_PREFETCH_L1(ws + 117792);
      CHEM_PREFETCH_L1(ws + 117824);
      CHEM_PREFETCH_L1(ws + 117856);
      CHEM_PREFETCH_L1(ws + 117888);
      CHEM_PREFETCH_L1(ws + 134592);
      double x = b[2912];
      x = fma(-CHEM_LDLU(lu + 39968), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 40000), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 40032), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 40064), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 40096), b[4736], x);
      b[2912] = x * CHEM_LDLU(vd + 2912);
    }
    {
      CHEM_PREFETCH(ws + 118144);
      CHEM_PREFETCH(ws + 134528);
      CHEM_PREFETCH_L1(ws + 117920);
      CHEM_PREFETCH_L1(ws + 117952);
      CHEM_PREFETCH_L1(ws + 117984);
      CHEM_PREFETCH_L1(ws + 118016);
      CHEM_PREFETCH_L1(ws + 118048);
      CHEM_PREFETCH_L1(ws + 118080);
      CHEM_PREFETCH_L1(ws + 118112);
      CHEM_PREFETCH_L1(ws + 134560);
      double x = b[2880];
      x = fma(-CHEM_LDLU(lu + 40128), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 40160), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 40192), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 40224), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 40256), b[4736], x);
      b[2880] = x * CHEM_LDLU(vd + 2880);
    }
    {
      CHEM_PREFETCH(ws + 118176);
      CHEM_PREFETCH(ws + 118208);
      CHEM_PREFETCH(ws + 134496);
      CHEM_PREFETCH_L1(ws + 118144);
      CHEM_PREFETCH_L1(ws + 134528);
      double x = b[2848];
      x = fma(-CHEM_LDLU(lu + 40288), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 40320), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 40352), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 40384), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 40416), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 40448), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 40480), b[4736], x);
      b[2848] = x * CHEM_LDLU(vd + 2848);
    }
    {
      CHEM_PREFETCH(ws + 118240);
      CHEM_PREFETCH(ws + 118272);
      CHEM_PREFETCH(ws + 118304);
      CHEM_PREFETCH(ws + 134464);
      CHEM_PREFETCH_L1(ws + 118176);
      CHEM_PREFETCH_L1(ws + 118208);
      CHEM_PREFETCH_L1(ws + 134496);
      double x = b[2816];
      x = fma(-CHEM_LDLU(lu + 40512), b[4736], x);
      b[2816] = x * CHEM_LDLU(vd + 2816);
    }
    {
      CHEM_PREFETCH(ws + 118336);
      CHEM_PREFETCH(ws + 118368);
      CHEM_PREFETCH(ws + 118400);
      CHEM_PREFETCH(ws + 118432);
      CHEM_PREFETCH(ws + 134432);
      CHEM_PREFETCH_L1(ws + 118240);
      CHEM_PREFETCH_L1(ws + 118272);
      CHEM_PREFETCH_L1(ws + 118304);
      CHEM_PREFETCH_L1(ws + 134464);
      double x = b[2784];
      x = fma(-CHEM_LDLU(lu + 40544), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 40576), b[4736], x);
      b[2784] = x * CHEM_LDLU(vd + 2784);
    }
    {
      CHEM_PREFETCH(ws + 118464);
      CHEM_PREFETCH(ws + 118496);
      CHEM_PREFETCH(ws + 118528);
      CHEM_PREFETCH(ws + 118560);
      CHEM_PREFETCH(ws + 118592);
      CHEM_PREFETCH(ws + 134400);
      CHEM_PREFETCH_L1(ws + 118336);
      CHEM_PREFETCH_L1(ws + 118368);
      CHEM_PREFETCH_L1(ws + 118400);
      CHEM_PREFETCH_L1(ws + 118432);
      CHEM_PREFETCH_L1(ws + 134432);
      double x = b[2752];
      x = fma(-CHEM_LDLU(lu + 40608), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 40640), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 40672), b[4736], x);
      b[2752] = x * CHEM_LDLU(vd + 2752);
    }
    {
      CHEM_PREFETCH(ws + 118624);
      CHEM_PREFETCH(ws + 118656);
      CHEM_PREFETCH(ws + 118688);
      CHEM_PREFETCH(ws + 118720);
      CHEM_PREFETCH(ws + 118752);
      CHEM_PREFETCH(ws + 134368);
      CHEM_PREFETCH_L1(ws + 118464);
      CHEM_PREFETCH_L1(ws + 118496);
      CHEM_PREFETCH_L1(ws + 118528);
      CHEM_PREFETCH_L1(ws + 118560);
      CHEM_PREFETCH_L1(ws + 118592);
      CHEM_PREFETCH_L1(ws + 134400);
      double x = b[2720];
      x = fma(-CHEM_LDLU(lu + 40704), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 40736), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 40768), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 40800), b[4736], x);
      b[2720] = x * CHEM_LDLU(vd + 2720);
    }
    {
      CHEM_PREFETCH(ws + 118784);
      CHEM_PREFETCH(ws + 118816);
      CHEM_PREFETCH(ws + 118848);
      CHEM_PREFETCH(ws + 118880);
      CHEM_PREFETCH(ws + 118912);
      CHEM_PREFETCH(ws + 134336);
      CHEM_PREFETCH_L1(ws + 118624);
      CHEM_PREFETCH_L1(ws + 118656);
      CHEM_PREFETCH_L1(ws + 118688);
      CHEM_PREFETCH_L1(ws + 118720);
      CHEM_PREFETCH_L1(ws + 118752);
      CHEM_PREFETCH_L1(ws + 134368);
      double x = b[2688];
      x = fma(-CHEM_LDLU(lu + 40832), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 40864), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 40896), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 40928), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 40960), b[4736], x);
      b[2688] = x * CHEM_LDLU(vd + 2688);
    }
    {
      CHEM_PREFETCH(ws + 118944);
      CHEM_PREFETCH(ws + 118976);
      CHEM_PREFETCH(ws + 134304);
      CHEM_PREFETCH_L1(ws + 118784);
      CHEM_PREFETCH_L1(ws + 118816);
      CHEM_PREFETCH_L1(ws + 118848);
      CHEM_PREFETCH_L1(ws + 118880);
      CHEM_PREFETCH_L1(ws + 118912);
      CHEM_PREFETCH_L1(ws + 134336);
      double x = b[2656];
      x = fma(-CHEM_LDLU(lu + 40992), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 41024), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 41056), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41088), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 41120), b[4736], x);
      b[2656] = x * CHEM_LDLU(vd + 2656);
    }
    {
      CHEM_PREFETCH(ws + 119008);
      CHEM_PREFETCH(ws + 119040);
      CHEM_PREFETCH(ws + 119072);
      CHEM_PREFETCH(ws + 119104);
      CHEM_PREFETCH(ws + 134272);
      CHEM_PREFETCH_L1(ws + 118944);
      CHEM_PREFETCH_L1(ws + 118976);
      CHEM_PREFETCH_L1(ws + 134304);
      double x = b[2624];
      x = fma(-CHEM_LDLU(lu + 41152), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 41184), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 41216), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41248), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 41280), b[4736], x);
      b[2624] = x * CHEM_LDLU(vd + 2624);
    }
    {
      CHEM_PREFETCH(ws + 119136);
      CHEM_PREFETCH(ws + 119168);
      CHEM_PREFETCH(ws + 119200);
      CHEM_PREFETCH(ws + 119232);
      CHEM_PREFETCH(ws + 119264);
      CHEM_PREFETCH(ws + 134240);
      CHEM_PREFETCH_L1(ws + 119008);
      CHEM_PREFETCH_L1(ws + 119040);
      CHEM_PREFETCH_L1(ws + 119072);
      CHEM_PREFETCH_L1(ws + 119104);
      CHEM_PREFETCH_L1(ws + 134272);
      double x = b[2592];
      x = fma(-CHEM_LDLU(lu + 41312), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 41344), b[4640], x);
      b[2592] = x * CHEM_LDLU(vd + 2592);
    }
    {
      CHEM_PREFETCH(ws + 119296);
      CHEM_PREFETCH(ws + 119328);
      CHEM_PREFETCH(ws + 119360);
      CHEM_PREFETCH(ws + 119392);
      CHEM_PREFETCH(ws + 134208);
      CHEM_PREFETCH_L1(ws + 119136);
      CHEM_PREFETCH_L1(ws + 119168);
      CHEM_PREFETCH_L1(ws + 119200);
      CHEM_PREFETCH_L1(ws + 119232);
      CHEM_PREFETCH_L1(ws + 119264);
      CHEM_PREFETCH_L1(ws + 134240);
      double x = b[2560];
      x = fma(-CHEM_LDLU(lu + 41376), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 41408), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41440), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 41472), b[4736], x);
      b[2560] = x * CHEM_LDLU(vd + 2560);
    }
    {
      CHEM_PREFETCH(ws + 119424);
      CHEM_PREFETCH(ws + 119456);
      CHEM_PREFETCH(ws + 119488);
      CHEM_PREFETCH(ws + 134176);
      CHEM_PREFETCH_L1(ws + 119296);
      CHEM_PREFETCH_L1(ws + 119328);
      CHEM_PREFETCH_L1(ws + 119360);
      CHEM_PREFETCH_L1(ws + 119392);
      CHEM_PREFETCH_L1(ws + 134208);
      double x = b[2528];
      x = fma(-CHEM_LDLU(lu + 41504), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 41536), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 41568), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41600), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 41632), b[4736], x);
      b[2528] = x * CHEM_LDLU(vd + 2528);
    }
    {
      CHEM_PREFETCH(ws + 119520);
      CHEM_PREFETCH(ws + 119552);
      CHEM_PREFETCH(ws + 119584);
      CHEM_PREFETCH(ws + 119616);
      CHEM_PREFETCH(ws + 134144);
      CHEM_PREFETCH_L1(ws + 119424);
      CHEM_PREFETCH_L1(ws + 119456);
      CHEM_PREFETCH_L1(ws + 119488);
      CHEM_PREFETCH_L1(ws + 134176);
      double x = b[2496];
      x = fma(-CHEM_LDLU(lu + 41664), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 41696), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41728), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 41760), b[4736], x);
      b[2496] = x * CHEM_LDLU(vd + 2496);
    }
    {
      CHEM_PREFETCH(ws + 119648);
      CHEM_PREFETCH(ws + 119680);
      CHEM_PREFETCH(ws + 119712);
      CHEM_PREFETCH(ws + 119744);
      CHEM_PREFETCH(ws + 134112);
      CHEM_PREFETCH_L1(ws + 119520);
      CHEM_PREFETCH_L1(ws + 119552);
      CHEM_PREFETCH_L1(ws + 119584);
      CHEM_PREFETCH_L1(ws + 119616);
      CHEM_PREFETCH_L1(ws + 134144);
      double x = b[2464];
      x = fma(-CHEM_LDLU(lu + 41792), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 41824), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 41856), b[4736], x);
      b[2464] = x * CHEM_LDLU(vd + 2464);
    }
    {
      CHEM_PREFETCH(ws + 119776);
      CHEM_PREFETCH(ws + 119808);
      CHEM_PREFETCH(ws + 119840);
      CHEM_PREFETCH(ws + 119872);
      CHEM_PREFETCH(ws + 134080);
      CHEM_PREFETCH_L1(ws + 119648);
      CHEM_PREFETCH_L1(ws + 119680);
      CHEM_PREFETCH_L1(ws + 119712);
      CHEM_PREFETCH_L1(ws + 119744);
      CHEM_PREFETCH_L1(ws + 134112);
      double x = b[2432];
      x = fma(-CHEM_LDLU(lu + 41888), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 41920), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 41952), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 41984), b[4736], x);
      b[2432] = x * CHEM_LDLU(vd + 2432);
    }
    {
      CHEM_PREFETCH(ws + 119904);
      CHEM_PREFETCH(ws + 119936);
      CHEM_PREFETCH(ws + 119968);
      CHEM_PREFETCH(ws + 120000);
      CHEM_PREFETCH(ws + 134048);
      CHEM_PREFETCH_L1(ws + 119776);
      CHEM_PREFETCH_L1(ws + 119808);
      CHEM_PREFETCH_L1(ws + 119840);
      CHEM_PREFETCH_L1(ws + 119872);
      CHEM_PREFETCH_L1(ws + 134080);
      double x = b[2400];
      x = fma(-CHEM_LDLU(lu + 42016), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 42048), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 42080), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 42112), b[4736], x);
      b[2400] = x * CHEM_LDLU(vd + 2400);
    }
    {
      CHEM_PREFETCH(ws + 120032);
      CHEM_PREFETCH(ws + 120064);
      CHEM_PREFETCH(ws + 120096);
      CHEM_PREFETCH(ws + 120128);
      CHEM_PREFETCH(ws + 134016);
      CHEM_PREFETCH_L1(ws + 119904);
      CHEM_PREFETCH_L1(ws + 119936);
      CHEM_PREFETCH_L1(ws + 119968);
      CHEM_PREFETCH_L1(ws + 120000);
      CHEM_PREFETCH_L1(ws + 134048);
      double x = b[2368];
      x = fma(-CHEM_LDLU(lu + 42144), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 42176), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 42208), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 42240), b[4736], x);
      b[2368] = x * CHEM_LDLU(vd + 2368);
    }
    {
      CHEM_PREFETCH(ws + 120160);
      CHEM_PREFETCH(ws + 120192);
      CHEM_PREFETCH(ws + 120224);
      CHEM_PREFETCH(ws + 120256);
      CHEM_PREFETCH(ws + 120288);
      CHEM_PREFETCH(ws + 133984);
      CHEM_PREFETCH_L1(ws + 120032);
      CHEM_PREFETCH_L1(ws + 120064);
      CHEM_PREFETCH_L1(ws + 120096);
      CHEM_PREFETCH_L1(ws + 120128);
      CHEM_PREFETCH_L1(ws + 134016);
      double x = b[2336];
      x = fma(-CHEM_LDLU(lu + 42272), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 42304), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 42336), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 42368), b[4736], x);
      b[2336] = x * CHEM_LDLU(vd + 2336);
    }
    {
      CHEM_PREFETCH(ws + 120320);
      CHEM_PREFETCH(ws + 120352);
      CHEM_PREFETCH(ws + 120384);
      CHEM_PREFETCH(ws + 120416);
      CHEM_PREFETCH(ws + 120448);
      CHEM_PREFETCH(ws + 120480);
      CHEM_PREFETCH(ws + 133952);
      CHEM_PREFETCH_L1(ws + 120160);
      CHEM_PREFETCH_L1(ws + 120192);
      CHEM_PREFETCH_L1(ws + 120224);
      CHEM_PREFETCH_L1(ws + 120256);
      CHEM_PREFETCH_L1(ws + 120288);
      CHEM_PREFETCH_L1(ws + 133984);
      double x = b[2304];
      x = fma(-CHEM_LDLU(lu + 42400), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 42432), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 42464), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 42496), b[4736], x);
      b[2304] = x * CHEM_LDLU(vd + 2304);
    }
    {
      CHEM_PREFETCH(ws + 120512);
      CHEM_PREFETCH(ws + 120544);
      CHEM_PREFETCH(ws + 120576);
      CHEM_PREFETCH(ws + 133920);
      CHEM_PREFETCH_L1(ws + 120320);
      CHEM_PREFETCH_L1(ws + 120352);
      CHEM_PREFETCH_L1(ws + 120384);
      CHEM_PREFETCH_L1(ws + 120416);
      CHEM_PREFETCH_L1(ws + 120448);
      CHEM_PREFETCH_L1(ws + 120480);
      CHEM_PREFETCH_L1(ws + 133952);
      double x = b[2272];
      x = fma(-CHEM_LDLU(lu + 42528), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 42560), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 42592), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 42624), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 42656), b[4736], x);
      b[2272] = x * CHEM_LDLU(vd + 2272);
    }
}
__device__ __noinline__ void solve_1_2(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 77632;
    const double* __restrict__ vd = ws + 131712;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      CHEM_PREFETCH(ws + 120608);
      CHEM_PREFETCH(ws + 120640);
      CHEM_PREFETCH(ws + 120672);
      CHEM_PREFETCH(ws + 120704);
      CHEM_PREFETCH(ws + 133888);
      CHEM_PREFETCH_L1(ws + 120512);
      CHEM_PREFETCH_L1(ws + 120544);
      CHEM_PREFETCH_L1(ws + 120576);
      CHEM_PREFETCH_L1(ws + 133920);
      double x = b[2240];
      x = fma(-CHEM_LDLU(lu + 42688), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 42720), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 42752), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 42784), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 42816), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 42848), b[4736], x);
      b[2240] = x * CHEM_LDLU(vd + 2240);
    }
    {
      CHEM_PREFETCH(ws + 120736);
      CHEM_PREFETCH(ws + 120768);
      CHEM_PREFETCH(ws + 120800);
      CHEM_PREFETCH(ws + 133856);
      CHEM_PREFETCH_L1(ws + 120608);
      CHEM_PREFETCH_L1(ws + 120640);
      CHEM_PREFETCH_L1(ws + 120672);
      CHEM_PREFETCH_L1(ws + 120704);
      CHEM_PREFETCH_L1(ws + 133888);
      double x = b[2208];
      x = fma(-CHEM_LDLU(lu + 42880), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 42912), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 42944), b[4736], x);
      b[2208] = x * CHEM_LDLU(vd + 2208);
    }
    {
      CHEM_PREFETCH(ws + 120832);
      CHEM_PREFETCH(ws + 120864);
      CHEM_PREFETCH(ws + 120896);
      CHEM_PREFETCH(ws + 120928);
      CHEM_PREFETCH(ws + 133824);
      CHEM_PREFETCH_L1(ws + 120736);
      CHEM_PREFETCH_L1(ws + 120768);
      CHEM_PREFETCH_L1(ws + 120800);
      CHEM_PREFETCH_L1(ws + 133856);
      double x = b[2176];
      x = fma(-CHEM_LDLU(lu + 42976), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 43008), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 43040), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 43072), b[4736], x);
      b[2176] = x * CHEM_LDLU(vd + 2176);
    }
    {
      CHEM_PREFETCH(ws + 120960);
      CHEM_PREFETCH(ws + 120992);
      CHEM_PREFETCH(ws + 121024);
      CHEM_PREFETCH(ws + 121056);
      CHEM_PREFETCH(ws + 121088);
      CHEM_PREFETCH(ws + 133792);
      CHEM_PREFETCH_L1(ws + 120832);
      CHEM_PREFETCH_L1(ws + 120864);
      CHEM_PREFETCH_L1(ws + 120896);
      CHEM_PREFETCH_L1(ws + 120928);
      CHEM_PREFETCH_L1(ws + 133824);
      double x = b[2144];
      x = fma(-CHEM_LDLU(lu + 43104), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 43136), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 43168), b[4736], x);
      b[2144] = x * CHEM_LDLU(vd + 2144);
    }
    {
      CHEM_PREFETCH(ws + 121120);
      CHEM_PREFETCH(ws + 121152);
      CHEM_PREFETCH(ws + 121184);
      CHEM_PREFETCH(ws + 121216);
      CHEM_PREFETCH(ws + 133760);
      CHEM_PREFETCH_L1(ws + 120960);
      CHEM_PREFETCH_L1(ws + 120992);
      CHEM_PREFETCH_L1(ws + 121024);
      CHEM_PREFETCH_L1(ws + 121056);
      CHEM_PREFETCH_L1(ws + 121088);
      CHEM_PREFETCH_L1(ws + 133792);
      double x = b[2112];
      x = fma(-CHEM_LDLU(lu + 43200), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 43232), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 43264), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 43296), b[4736], x);
      b[2112] = x * CHEM_LDLU(vd + 2112);
    }
    {
      CHEM_PREFETCH(ws + 121248);
      CHEM_PREFETCH(ws + 121280);
      CHEM_PREFETCH(ws + 121312);
      CHEM_PREFETCH(ws + 133728);
      CHEM_PREFETCH_L1(ws + 121120);
      CHEM_PREFETCH_L1(ws + 121152);
      CHEM_PREFETCH_L1(ws + 121184);
      CHEM_PREFETCH_L1(ws + 121216);
      CHEM_PREFETCH_L1(ws + 133760);
      double x = b[2080];
      x = fma(-CHEM_LDLU(lu + 43328), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 43360), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 43392), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 43424), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 43456), b[4736], x);
      b[2080] = x * CHEM_LDLU(vd + 2080);
    }
    {
      CHEM_PREFETCH(ws + 121344);
      CHEM_PREFETCH(ws + 121376);
      CHEM_PREFETCH(ws + 121408);
      CHEM_PREFETCH(ws + 133696);
      CHEM_PREFETCH_L1(ws + 121248);
      CHEM_PREFETCH_L1(ws + 121280);
      CHEM_PREFETCH_L1(ws + 121312);
      CHEM_PREFETCH_L1(ws + 133728);
      double x = b[2048];
      x = fma(-CHEM_LDLU(lu + 43488), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 43520), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 43552), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 43584), b[4736], x);
      b[2048] = x * CHEM_LDLU(vd + 2048);
    }
    {
      CHEM_PREFETCH(ws + 121440);
      CHEM_PREFETCH(ws + 121472);
      CHEM_PREFETCH(ws + 121504);
      CHEM_PREFETCH(ws + 133664);
      CHEM_PREFETCH_L1(ws + 121344);
      CHEM_PREFETCH_L1(ws + 121376);
      CHEM_PREFETCH_L1(ws + 121408);
      CHEM_PREFETCH_L1(ws + 133696);
      double x = b[2016];
      x = fma(-CHEM_LDLU(lu + 43616), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 43648), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 43680), b[4736], x);
      b[2016] = x * CHEM_LDLU(vd + 2016);
    }
    {
      CHEM_PREFETCH(ws + 121536);
      CHEM_PREFETCH(ws + 121568);
      CHEM_PREFETCH(ws + 133632);
      CHEM_PREFETCH_L1(ws + 121440);
      CHEM_PREFETCH_L1(ws + 121472);
      CHEM_PREFETCH_L1(ws + 121504);
      CHEM_PREFETCH_L1(ws + 133664);
      double x = b[1984];
      x = fma(-CHEM_LDLU(lu + 43712), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 43744), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 43776), b[4736], x);
      b[1984] = x * CHEM_LDLU(vd + 1984);
    }
    {
      CHEM_PREFETCH(ws + 121600);
      CHEM_PREFETCH(ws + 121632);
      CHEM_PREFETCH(ws + 121664);
      CHEM_PREFETCH(ws + 133600);
      CHEM_PREFETCH_L1(ws + 121536);
      CHEM_PREFETCH_L1(ws + 121568);
      CHEM_PREFETCH_L1(ws + 133632);
      double x = b[1952];
      x = fma(-CHEM_LDLU(lu + 43808), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 43840), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 43872), b[4736], x);
      b[1952] = x * CHEM_LDLU(vd + 1952);
    }
    {
      CHEM_PREFETCH(ws + 121696);
      CHEM_PREFETCH(ws + 121728);
      CHEM_PREFETCH(ws + 121760);
      CHEM_PREFETCH(ws + 133568);
      CHEM_PREFETCH_L1(ws + 121600);
      CHEM_PREFETCH_L1(ws + 121632);
      CHEM_PREFETCH_L1(ws + 121664);
      CHEM_PREFETCH_L1(ws + 133600);
      double x = b[1920];
      x = fma(-CHEM_LDLU(lu + 43904), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 43936), b[4640], x);
      b[1920] = x * CHEM_LDLU(vd + 1920);
    }
    {
      CHEM_PREFETCH(ws + 121792);
      CHEM_PREFETCH(ws + 121824);
      CHEM_PREFETCH(ws + 121856);
      CHEM_PREFETCH(ws + 133536);
      CHEM_PREFETCH_L1(ws + 121696);
      CHEM_PREFETCH_L1(ws + 121728);
      CHEM_PREFETCH_L1(ws + 121760);
      CHEM_PREFETCH_L1(ws + 133568);
      double x = b[1888];
      x = fma(-CHEM_LDLU(lu + 43968), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 44000), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 44032), b[4736], x);
      b[1888] = x * CHEM_LDLU(vd + 1888);
    }
    {
      CHEM_PREFETCH(ws + 121888);
      CHEM_PREFETCH(ws + 121920);
      CHEM_PREFETCH(ws + 121952);
      CHEM_PREFETCH(ws + 133504);
      CHEM_PREFETCH_L1(ws + 121792);
      CHEM_PREFETCH_L1(ws + 121824);
      CHEM_PREFETCH_L1(ws + 121856);
      CHEM_PREFETCH_L1(ws + 133536);
      double x = b[1856];
      x = fma(-CHEM_LDLU(lu + 44064), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 44096), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 44128), b[4736], x);
      b[1856] = x * CHEM_LDLU(vd + 1856);
    }
    {
      CHEM_PREFETCH(ws + 121984);
      CHEM_PREFETCH(ws + 122016);
      CHEM_PREFETCH(ws + 122048);
      CHEM_PREFETCH(ws + 133472);
      CHEM_PREFETCH_L1(ws + 121888);
      CHEM_PREFETCH_L1(ws + 121920);
      CHEM_PREFETCH_L1(ws + 121952);
      CHEM_PREFETCH_L1(ws + 133504);
      double x = b[1824];
      x = fma(-CHEM_LDLU(lu + 44160), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 44192), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 44224), b[4704], x);
      b[1824] = x * CHEM_LDLU(vd + 1824);
    }
    {
      CHEM_PREFETCH(ws + 122080);
      CHEM_PREFETCH(ws + 122112);
      CHEM_PREFETCH(ws + 122144);
      CHEM_PREFETCH(ws + 133440);
      CHEM_PREFETCH_L1(ws + 121984);
      CHEM_PREFETCH_L1(ws + 122016);
      CHEM_PREFETCH_L1(ws + 122048);
      CHEM_PREFETCH_L1(ws + 133472);
      double x = b[1792];
      x = fma(-CHEM_LDLU(lu + 44256), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 44288), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 44320), b[4736], x);
      b[1792] = x * CHEM_LDLU(vd + 1792);
    }
    {
      CHEM_PREFETCH(ws + 122176);
      CHEM_PREFETCH(ws + 122208);
      CHEM_PREFETCH(ws + 122240);
      CHEM_PREFETCH(ws + 133408);
      CHEM_PREFETCH_L1(ws + 122080);
      CHEM_PREFETCH_L1(ws + 122112);
      CHEM_PREFETCH_L1(ws + 122144);
      CHEM_PREFETCH_L1(ws + 133440);
      double x = b[1760];
      x = fma(-CHEM_LDLU(lu + 44352), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 44384), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 44416), b[4736], x);
      b[1760] = x * CHEM_LDLU(vd + 1760);
    }
    {
      CHEM_PREFETCH(ws + 122272);
      CHEM_PREFETCH(ws + 122304);
      CHEM_PREFETCH(ws + 122336);
      CHEM_PREFETCH(ws + 133376);
      CHEM_PREFETCH_L1(ws + 122176);
      CHEM_PREFETCH_L1(ws + 122208);
      CHEM_PREFETCH_L1(ws + 122240);
      CHEM_PREFETCH_L1(ws + 133408);
      double x = b[1728];
      x = fma(-CHEM_LDLU(lu + 44448), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 44480), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 44512), b[4704], x);
      b[1728] = x * CHEM_LDLU(vd + 1728);
    }
    {
      CHEM_PREFETCH(ws + 122368);
      CHEM_PREFETCH(ws + 122400);
      CHEM_PREFETCH(ws + 122432);
      CHEM_PREFETCH(ws + 133344);
      CHEM_PREFETCH_L1(ws + 122272);
      CHEM_PREFETCH_L1(ws + 122304);
      CHEM_PREFETCH_L1(ws + 122336);
      CHEM_PREFETCH_L1(ws + 133376);
      double x = b[1696];
      x = fma(-CHEM_LDLU(lu + 44544), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 44576), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 44608), b[4736], x);
      b[1696] = x * CHEM_LDLU(vd + 1696);
    }
    {
      CHEM_PREFETCH(ws + 122464);
      CHEM_PREFETCH(ws + 122496);
      CHEM_PREFETCH(ws + 122528);
      CHEM_PREFETCH(ws + 133312);
      CHEM_PREFETCH_L1(ws + 122368);
      CHEM_PREFETCH_L1(ws + 122400);
      CHEM_PREFETCH_L1(ws + 122432);
      CHEM_PREFETCH_L1(ws + 133344);
      double x = b[1664];
      x = fma(-CHEM_LDLU(lu + 44640), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 44672), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 44704), b[4736], x);
      b[1664] = x * CHEM_LDLU(vd + 1664);
    }
    {
      CHEM_PREFETCH(ws + 122560);
      CHEM_PREFETCH(ws + 122592);
      CHEM_PREFETCH(ws + 122624);
      CHEM_PREFETCH(ws + 133280);
      CHEM_PREFETCH_L1(ws + 122464);
      CHEM_PREFETCH_L1(ws + 122496);
      CHEM_PREFETCH_L1(ws + 122528);
      CHEM_PREFETCH_L1(ws + 133312);
      double x = b[1632];
      x = fma(-CHEM_LDLU(lu + 44736), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 44768), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 44800), b[4736], x);
      b[1632] = x * CHEM_LDLU(vd + 1632);
    }
    {
      CHEM_PREFETCH(ws + 122656);
      CHEM_PREFETCH(ws + 122688);
      CHEM_PREFETCH(ws + 133248);
      CHEM_PREFETCH_L1(ws + 122560);
      CHEM_PREFETCH_L1(ws + 122592);
      CHEM_PREFETCH_L1(ws + 122624);
      CHEM_PREFETCH_L1(ws + 133280);
      double x = b[1600];
      x = fma(-CHEM_LDLU(lu + 44832), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 44864), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 44896), b[4736], x);
      b[1600] = x * CHEM_LDLU(vd + 1600);
    }
    {
      CHEM_PREFETCH(ws + 122720);
      CHEM_PREFETCH(ws + 122752);
      CHEM_PREFETCH(ws + 133216);
      CHEM_PREFETCH_L1(ws + 122656);
      CHEM_PREFETCH_L1(ws + 122688);
      CHEM_PREFETCH_L1(ws + 133248);
      double x = b[1568];
      x = fma(-CHEM_LDLU(lu + 44928), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 44960), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 44992), b[4736], x);
      b[1568] = x * CHEM_LDLU(vd + 1568);
    }
    {
      CHEM_PREFETCH(ws + 122784);
      CHEM_PREFETCH(ws + 133184);
      CHEM_PREFETCH_L1(ws + 122720);
      CHEM_PREFETCH_L1(ws + 122752);
      CHEM_PREFETCH_L1(ws + 133216);
      double x = b[1536];
      x = fma(-CHEM_LDLU(lu + 45024), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 45056), b[4736], x);
      b[1536] = x * CHEM_LDLU(vd + 1536);
    }
    {
      CHEM_PREFETCH(ws + 122816);
      CHEM_PREFETCH(ws + 133152);
      CHEM_PREFETCH_L1(ws + 122784);
      CHEM_PREFETCH_L1(ws + 133184);
      double x = b[1504];
      x = fma(-CHEM_LDLU(lu + 45088), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 45120), b[4736], x);
      b[1504] = x * CHEM_LDLU(vd + 1504);
    }
    {
      CHEM_PREFETCH(ws + 133120);
      CHEM_PREFETCH_L1(ws + 122816);
      CHEM_PREFETCH_L1(ws + 133152);
      double x = b[1472];
      x = fma(-CHEM_LDLU(lu + 45152), b[4736], x);
      b[1472] = x * CHEM_LDLU(vd + 1472);
    }
    {
      CHEM_PREFETCH(ws + 133088);
      CHEM_PREFETCH_L1(ws + 133120);
      double x = b[1440];
      x = fma(-CHEM_LDLU(lu + 45184), b[4736], x);
      b[1440] = x * CHEM_LDLU(vd + 1440);
    }
    {
      CHEM_PREFETCH(ws + 122848);
      CHEM_PREFETCH(ws + 122880);
      CHEM_PREFETCH(ws + 133056);
      CHEM_PREFETCH_L1(ws + 133088);
      double x = b[1408];
      b[1408] = x * CHEM_LDLU(vd + 1408);
    }
    {
      CHEM_PREFETCH(ws + 122912);
      CHEM_PREFETCH(ws + 122944);
      CHEM_PREFETCH(ws + 133024);
      CHEM_PREFETCH_L1(ws + 122848);
      CHEM_PREFETCH_L1(ws + 122880);
      CHEM_PREFETCH_L1(ws + 133056);
      double x = b[1376];
      b[1376] = x * CHEM_LDLU(vd + 1376);
    }
    {
      CHEM_PREFETCH(ws + 122976);
      CHEM_PREFETCH(ws + 123008);
      CHEM_PREFETCH(ws + 132992);
      CHEM_PREFETCH_L1(ws + 122912);
      CHEM_PREFETCH_L1(ws + 122944);
      CHEM_PREFETCH_L1(ws + 133024);
      double x = b[1344];
      x = fma(-CHEM_LDLU(lu + 45216), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 45248), b[4608], x);
      b[1344] = x * CHEM_LDLU(vd + 1344);
    }
    {
      CHEM_PREFETCH(ws + 123040);
      CHEM_PREFETCH(ws + 132960);
      CHEM_PREFETCH_L1(ws + 122976);
      CHEM_PREFETCH_L1(ws + 123008);
      CHEM_PREFETCH_L1(ws + 132992);
      double x = b[1312];
      x = fma(-CHEM_LDLU(lu + 45280), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 45312), b[4736], x);
      b[1312] = x * CHEM_LDLU(vd + 1312);
    }
    {
      CHEM_PREFETCH(ws + 123072);
      CHEM_PREFETCH(ws + 123104);
      CHEM_PREFETCH(ws + 132928);
      CHEM_PREFETCH_L1(ws + 123040);
      CHEM_PREFETCH_L1(ws + 132960);
      double x = b[1280];
      x = fma(-CHEM_LDLU(lu + 45344), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 45376), b[4640], x);
      b[1280] = x * CHEM_LDLU(vd + 1280);
    }
    {
      CHEM_PREFETCH(ws + 123136);
      CHEM_PREFETCH(ws + 123168);
      CHEM_PREFETCH(ws + 132896);
      CHEM_PREFETCH_L1(ws + 123072);
      CHEM_PREFETCH_L1(ws + 123104);
      CHEM_PREFETCH_L1(ws + 132928);
      double x = b[1248];
      x = fma(-CHEM_LDLU(lu + 45408), b[1280], x);
      b[1248] = x * CHEM_LDLU(vd + 1248);
    }
    {
      CHEM_PREFETCH(ws + 123200);
      CHEM_PREFETCH(ws + 123232);
      CHEM_PREFETCH(ws + 132864);
      CHEM_PREFETCH_L1(ws + 123136);
      CHEM_PREFETCH_L1(ws + 123168);
      CHEM_PREFETCH_L1(ws + 132896);
      double x = b[1216];
      x = fma(-CHEM_LDLU(lu + 45440), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 45472), b[4608], x);
      b[1216] = x * CHEM_LDLU(vd + 1216);
    }
    {
      CHEM_PREFETCH(ws + 123264);
      CHEM_PREFETCH(ws + 123296);
      CHEM_PREFETCH(ws + 132832);
      CHEM_PREFETCH_L1(ws + 123200);
      CHEM_PREFETCH_L1(ws + 123232);
      CHEM_PREFETCH_L1(ws + 132864);
      double x = b[1184];
      x = fma(-CHEM_LDLU(lu + 45504), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 45536), b[3520], x);
      b[1184] = x * CHEM_LDLU(vd + 1184);
    }
    {
      CHEM_PREFETCH(ws + 123328);
      CHEM_PREFETCH(ws + 123360);
      CHEM_PREFETCH(ws + 132800);
      CHEM_PREFETCH_L1(ws + 123264);
      CHEM_PREFETCH_L1(ws + 123296);
      CHEM_PREFETCH_L1(ws + 132832);
      double x = b[1152];
      x = fma(-CHEM_LDLU(lu + 45568), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 45600), b[4736], x);
      b[1152] = x * CHEM_LDLU(vd + 1152);
    }
    {
      CHEM_PREFETCH(ws + 123392);
      CHEM_PREFETCH(ws + 123424);
      CHEM_PREFETCH(ws + 132768);
      CHEM_PREFETCH_L1(ws + 123328);
      CHEM_PREFETCH_L1(ws + 123360);
      CHEM_PREFETCH_L1(ws + 132800);
      double x = b[1120];
      x = fma(-CHEM_LDLU(lu + 45632), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 45664), b[4736], x);
      b[1120] = x * CHEM_LDLU(vd + 1120);
    }
    {
      CHEM_PREFETCH(ws + 123456);
      CHEM_PREFETCH(ws + 123488);
      CHEM_PREFETCH(ws + 132736);
      CHEM_PREFETCH_L1(ws + 123392);
      CHEM_PREFETCH_L1(ws + 123424);
      CHEM_PREFETCH_L1(ws + 132768);
      double x = b[1088];
      x = fma(-CHEM_LDLU(lu + 45696), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 45728), b[4736], x);
      b[1088] = x * CHEM_LDLU(vd + 1088);
    }
    {
      CHEM_PREFETCH(ws + 123520);
      CHEM_PREFETCH(ws + 123552);
      CHEM_PREFETCH(ws + 123584);
      CHEM_PREFETCH(ws + 132704);
      CHEM_PREFETCH_L1(ws + 123456);
      CHEM_PREFETCH_L1(ws + 123488);
      CHEM_PREFETCH_L1(ws + 132736);
      double x = b[1056];
      x = fma(-CHEM_LDLU(lu + 45760), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 45792), b[4736], x);
      b[1056] = x * CHEM_LDLU(vd + 1056);
    }
    {
      CHEM_PREFETCH(ws + 123616);
      CHEM_PREFETCH(ws + 123648);
      CHEM_PREFETCH(ws + 132672);
      CHEM_PREFETCH_L1(ws + 123520);
      CHEM_PREFETCH_L1(ws + 123552);
      CHEM_PREFETCH_L1(ws + 123584);
      CHEM_PREFETCH_L1(ws + 132704);
      double x = b[1024];
      x = fma(-CHEM_LDLU(lu + 45824), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 45856), b[4640], x);
      b[1024] = x * CHEM_LDLU(vd + 1024);
    }
    {
      CHEM_PREFETCH(ws + 123680);
      CHEM_PREFETCH(ws + 123712);
      CHEM_PREFETCH(ws + 132640);
      CHEM_PREFETCH_L1(ws + 123616);
      CHEM_PREFETCH_L1(ws + 123648);
      CHEM_PREFETCH_L1(ws + 132672);
      double x = b[992];
      x = fma(-CHEM_LDLU(lu + 45888), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 45920), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 45952), b[4736], x);
      b[992] = x * CHEM_LDLU(vd + 992);
    }
    {
      CHEM_PREFETCH(ws + 123744);
      CHEM_PREFETCH(ws + 123776);
      CHEM_PREFETCH(ws + 132608);
      CHEM_PREFETCH_L1(ws + 123680);
      CHEM_PREFETCH_L1(ws + 123712);
      CHEM_PREFETCH_L1(ws + 132640);
      double x = b[960];
      x = fma(-CHEM_LDLU(lu + 45984), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 46016), b[4608], x);
      b[960] = x * CHEM_LDLU(vd + 960);
    }
    {
      CHEM_PREFETCH(ws + 123808);
      CHEM_PREFETCH(ws + 123840);
      CHEM_PREFETCH(ws + 132576);
      CHEM_PREFETCH_L1(ws + 123744);
      CHEM_PREFETCH_L1(ws + 123776);
      CHEM_PREFETCH_L1(ws + 132608);
      double x = b[928];
      x = fma(-CHEM_LDLU(lu + 46048), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 46080), b[4736], x);
      b[928] = x * CHEM_LDLU(vd + 928);
    }
    {
      CHEM_PREFETCH(ws + 123872);
      CHEM_PREFETCH(ws + 123904);
      CHEM_PREFETCH(ws + 132544);
      CHEM_PREFETCH_L1(ws + 123808);
      CHEM_PREFETCH_L1(ws + 123840);
      CHEM_PREFETCH_L1(ws + 132576);
      double x = b[896];
      x = fma(-CHEM_LDLU(lu + 46112), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 46144), b[4736], x);
      b[896] = x * CHEM_LDLU(vd + 896);
    }
    {
      CHEM_PREFETCH(ws + 123936);
      CHEM_PREFETCH(ws + 132512);
      CHEM_PREFETCH_L1(ws + 123872);
      CHEM_PREFETCH_L1(ws + 123904);
      CHEM_PREFETCH_L1(ws + 132544);
      double x = b[864];
      x = fma(-CHEM_LDLU(lu + 46176), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 46208), b[4736], x);
      b[864] = x * CHEM_LDLU(vd + 864);
    }
    {
      CHEM_PREFETCH(ws + 123968);
      CHEM_PREFETCH(ws + 132480);
      CHEM_PREFETCH_L1(ws + 123936);
      CHEM_PREFETCH_L1(ws + 132512);
      double x = b[832];
      x = fma(-CHEM_LDLU(lu + 46240), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 46272), b[4736], x);
      b[832] = x * CHEM_LDLU(vd + 832);
    }
    {
      CHEM_PREFETCH(ws + 124000);
      CHEM_PREFETCH(ws + 132448);
      CHEM_PREFETCH_L1(ws + 123968);
      CHEM_PREFETCH_L1(ws + 132480);
      double x = b[800];
      x = fma(-CHEM_LDLU(lu + 46304), b[4736], x);
      b[800] = x * CHEM_LDLU(vd + 800);
    }
    {
      CHEM_PREFETCH(ws + 124032);
      CHEM_PREFETCH(ws + 132416);
      CHEM_PREFETCH_L1(ws + 124000);
      CHEM_PREFETCH_L1(ws + 132448);
      double x = b[768];
      x = fma(-CHEM_LDLU(lu + 46336), b[4736], x);
      b[768] = x * CHEM_LDLU(vd + 768);
    }
    {
      CHEM_PREFETCH(ws + 132384);
      CHEM_PREFETCH_L1(ws + 124032);
      CHEM_PREFETCH_L1(ws + 132416);
      double x = b[736];
      x = fma(-CHEM_LDLU(lu + 46368), b[4736], x);
      b[736] = x * CHEM_LDLU(vd + 736);
    }
    {
      CHEM_PREFETCH(ws + 124064);
      CHEM_PREFETCH(ws + 124096);
      CHEM_PREFETCH(ws + 132352);
      CHEM_PREFETCH_L1(ws + 132384);
      double x = b[704];
      x = fma(-CHEM_LDLU(lu + 46400), b[4736], x);
      b[704] = x * CHEM_LDLU(vd + 704);
    }
    {
      CHEM_PREFETCH(ws + 124128);
      CHEM_PREFETCH(ws + 132320);
      CHEM_PREFETCH_L1(ws + 124064);
      CHEM_PREFETCH_L1(ws + 124096);
      CHEM_PREFETCH_L1(ws + 132352);
      double x = b[672];
      b[672] = x * CHEM_LDLU(vd + 672);
    }
    {
      CHEM_PREFETCH(ws + 124160);
      CHEM_PREFETCH(ws + 132288);
      CHEM_PREFETCH_L1(ws + 124128);
      CHEM_PREFETCH_L1(ws + 132320);
      double x = b[640];
      x = fma(-CHEM_LDLU(lu + 46432), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 46464), b[4256], x);
      b[640] = x * CHEM_LDLU(vd + 640);
    }
    {
      CHEM_PREFETCH(ws + 124192);
      CHEM_PREFETCH(ws + 132256);
      CHEM_PREFETCH_L1(ws + 124160);
      CHEM_PREFETCH_L1(ws + 132288);
      double x = b[608];
      x = fma(-CHEM_LDLU(lu + 46496), b[1312], x);
      b[608] = x * CHEM_LDLU(vd + 608);
    }
    {
      CHEM_PREFETCH(ws + 124224);
      CHEM_PREFETCH(ws + 132224);
      CHEM_PREFETCH_L1(ws + 124192);
      CHEM_PREFETCH_L1(ws + 132256);
      double x = b[576];
      x = fma(-CHEM_LDLU(lu + 46528), b[1312], x);
      b[576] = x * CHEM_LDLU(vd + 576);
    }
    {
      CHEM_PREFETCH(ws + 124256);
      CHEM_PREFETCH(ws + 132192);
      CHEM_PREFETCH_L1(ws + 124224);
      CHEM_PREFETCH_L1(ws + 132224);
      double x = b[544];
      x = fma(-CHEM_LDLU(lu + 46560), b[1248], x);
      b[544] = x * CHEM_LDLU(vd + 544);
    }
    {
      CHEM_PREFETCH(ws + 124288);
      CHEM_PREFETCH(ws + 132160);
      CHEM_PREFETCH_L1(ws + 124256);
      CHEM_PREFETCH_L1(ws + 132192);
      double x = b[512];
      x = fma(-CHEM_LDLU(lu + 46592), b[1920], x);
      b[512] = x * CHEM_LDLU(vd + 512);
    }
    {
      CHEM_PREFETCH(ws + 124320);
      CHEM_PREFETCH(ws + 132128);
      CHEM_PREFETCH_L1(ws + 124288);
      CHEM_PREFETCH_L1(ws + 132160);
      double x = b[480];
      x = fma(-CHEM_LDLU(lu + 46624), b[1920], x);
      b[480] = x * CHEM_LDLU(vd + 480);
    }
    {
      CHEM_PREFETCH(ws + 124352);
      CHEM_PREFETCH(ws + 132096);
      CHEM_PREFETCH_L1(ws + 124320);
      CHEM_PREFETCH_L1(ws + 132128);
      double x = b[448];
      x = fma(-CHEM_LDLU(lu + 46656), b[4736], x);
      b[448] = x * CHEM_LDLU(vd + 448);
    }
    {
      CHEM_PREFETCH(ws + 124384);
      CHEM_PREFETCH(ws + 132064);
      CHEM_PREFETCH_L1(ws + 124352);
      CHEM_PREFETCH_L1(ws + 132096);
      double x = b[416];
      x = fma(-CHEM_LDLU(lu + 46688), b[4736], x);
      b[416] = x * CHEM_LDLU(vd + 416);
    }
    {
      CHEM_PREFETCH(ws + 124416);
      CHEM_PREFETCH(ws + 132032);
      CHEM_PREFETCH_L1(ws + 124384);
      CHEM_PREFETCH_L1(ws + 132064);
      double x = b[384];
      x = fma(-CHEM_LDLU(lu + 46720), b[4736], x);
      b[384] = x * CHEM_LDLU(vd + 384);
    }
    {
      CHEM_PREFETCH(ws + 124448);
      CHEM_PREFETCH(ws + 124480);
      CHEM_PREFETCH(ws + 132000);
      CHEM_PREFETCH_L1(ws + 124416);
      CHEM_PREFETCH_L1(ws + 132032);
      double x = b[352];
      x = fma(-CHEM_LDLU(lu + 46752), b[4736], x);
      b[352] = x * CHEM_LDLU(vd + 352);
    }
    {
      CHEM_PREFETCH(ws + 124512);
      CHEM_PREFETCH(ws + 124544);
      CHEM_PREFETCH(ws + 131968);
      CHEM_PREFETCH_L1(ws + 124448);
      CHEM_PREFETCH_L1(ws + 124480);
      CHEM_PREFETCH_L1(ws + 132000);
      double x = b[320];
      x = fma(-CHEM_LDLU(lu + 46784), b[960], x);
      b[320] = x * CHEM_LDLU(vd + 320);
    }
    {
      CHEM_PREFETCH(ws + 131936);
      CHEM_PREFETCH_L1(ws + 124512);
      CHEM_PREFETCH_L1(ws + 124544);
      CHEM_PREFETCH_L1(ws + 131968);
      double x = b[288];
      x = fma(-CHEM_LDLU(lu + 46816), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 46848), b[4736], x);
      b[288] = x * CHEM_LDLU(vd + 288);
    }
    {
      CHEM_PREFETCH(ws + 131904);
      CHEM_PREFETCH_L1(ws + 131936);
      double x = b[256];
      x = fma(-CHEM_LDLU(lu + 46880), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 46912), b[4736], x);
      b[256] = x * CHEM_LDLU(vd + 256);
    }
    {
      CHEM_PREFETCH(ws + 131872);
      CHEM_PREFETCH_L1(ws + 131904);
      double x = b[224];
      b[224] = x * CHEM_LDLU(vd + 224);
    }
    {
      CHEM_PREFETCH(ws + 131840);
      CHEM_PREFETCH_L1(ws + 131872);
      double x = b[192];
      b[192] = x * CHEM_LDLU(vd + 192);
    }
    {
      CHEM_PREFETCH(ws + 131808);
      CHEM_PREFETCH_L1(ws + 131840);
      double x = b[160];
      b[160] = x * CHEM_LDLU(vd + 160);
    }
    {
      CHEM_PREFETCH(ws + 131776);
      CHEM_PREFETCH_L1(ws + 131808);
      double x = b[128];
      b[128] = x * CHEM_LDLU(vd + 128);
    }
    {
      CHEM_PREFETCH(ws + 131744);
      CHEM_PREFETCH_L1(ws + 131776);
      double x = b[96];
      b[96] = x * CHEM_LDLU(vd + 96);
    }
    {
      CHEM_PREFETCH(ws + 131712);
      CHEM_PREFETCH_L1(ws + 131744);
      double x = b[64];
      b[64] = x * CHEM_LDLU(vd + 64);
    }
    {
      CHEM_PREFETCH_L1(ws + 131712);
      double x = b[32];
      b[32] = x * CHEM_LDLU(vd + 32);
    }
    {
      double x = b[0];
      b[0] = x * CHEM_LDLU(vd + 0);
    }
}
}  // namespace mech_cb6r5_ae7_aq
