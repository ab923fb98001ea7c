// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void solve_t_1_0(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[0];
      b[0] = x * CHEM_LDLU(vd + 0);
    }
    {
      double x = b[32];
      b[32] = x * CHEM_LDLU(vd + 32);
    }
    {
      double x = b[64];
      b[64] = x * CHEM_LDLU(vd + 64);
    }
    {
      double x = b[96];
      b[96] = x * CHEM_LDLU(vd + 96);
    }
    {
      double x = b[128];
      b[128] = x * CHEM_LDLU(vd + 128);
    }
    {
      double x = b[160];
      b[160] = x * CHEM_LDLU(vd + 160);
    }
    {
      double x = b[192];
      b[192] = x * CHEM_LDLU(vd + 192);
    }
    {
      double x = b[224];
      b[224] = x * CHEM_LDLU(vd + 224);
    }
    {
      double x = b[256];
      b[256] = x * CHEM_LDLU(vd + 256);
    }
    {
      double x = b[288];
      b[288] = x * CHEM_LDLU(vd + 288);
    }
    {
      double x = b[320];
      b[320] = x * CHEM_LDLU(vd + 320);
    }
    {
      double x = b[352];
      b[352] = x * CHEM_LDLU(vd + 352);
    }
    {
      double x = b[384];
      b[384] = x * CHEM_LDLU(vd + 384);
    }
    {
      double x = b[416];
      b[416] = x * CHEM_LDLU(vd + 416);
    }
    {
      double x = b[448];
      b[448] = x * CHEM_LDLU(vd + 448);
    }
    {
      double x = b[480];
      b[480] = x * CHEM_LDLU(vd + 480);
    }
    {
      double x = b[512];
      b[512] = x * CHEM_LDLU(vd + 512);
    }
    {
      double x = b[544];
      b[544] = x * CHEM_LDLU(vd + 544);
    }
    {
      double x = b[576];
      b[576] = x * CHEM_LDLU(vd + 576);
    }
    {
      double x = b[608];
      b[608] = x * CHEM_LDLU(vd + 608);
    }
    {
      double x = b[640];
      b[640] = x * CHEM_LDLU(vd + 640);
    }
    {
      double x = b[672];
      b[672] = x * CHEM_LDLU(vd + 672);
    }
    {
      double x = b[704];
      b[704] = x * CHEM_LDLU(vd + 704);
    }
    {
      double x = b[736];
      b[736] = x * CHEM_LDLU(vd + 736);
    }
    {
      double x = b[768];
      b[768] = x * CHEM_LDLU(vd + 768);
    }
    {
      double x = b[800];
      b[800] = x * CHEM_LDLU(vd + 800);
    }
    {
      double x = b[832];
      b[832] = x * CHEM_LDLU(vd + 832);
    }
    {
      double x = b[864];
      b[864] = x * CHEM_LDLU(vd + 864);
    }
    {
      double x = b[896];
      b[896] = x * CHEM_LDLU(vd + 896);
    }
    {
      double x = b[928];
      b[928] = x * CHEM_LDLU(vd + 928);
    }
    {
      double x = b[960];
      b[960] = x * CHEM_LDLU(vd + 960);
    }
    {
      double x = b[992];
      b[992] = x * CHEM_LDLU(vd + 992);
    }
    {
      double x = b[1024];
      b[1024] = x * CHEM_LDLU(vd + 1024);
    }
    {
      double x = b[1056];
      x = fma(-CHEM_LDLU(lu + 96320), b[0], x);
      x = fma(-CHEM_LDLU(lu + 95840), b[512], x);
      x = fma(-CHEM_LDLU(lu + 95808), b[544], x);
      b[1056] = x * CHEM_LDLU(vd + 1056);
    }
    {
      double x = b[1088];
      b[1088] = x * CHEM_LDLU(vd + 1088);
    }
    {
      double x = b[1120];
      b[1120] = x * CHEM_LDLU(vd + 1120);
    }
    {
      double x = b[1152];
      b[1152] = x * CHEM_LDLU(vd + 1152);
    }
    {
      double x = b[1184];
      b[1184] = x * CHEM_LDLU(vd + 1184);
    }
    {
      double x = b[1216];
      b[1216] = x * CHEM_LDLU(vd + 1216);
    }
    {
      double x = b[1248];
      b[1248] = x * CHEM_LDLU(vd + 1248);
    }
    {
      double x = b[1280];
      b[1280] = x * CHEM_LDLU(vd + 1280);
    }
    {
      double x = b[1312];
      b[1312] = x * CHEM_LDLU(vd + 1312);
    }
    {
      double x = b[1344];
      b[1344] = x * CHEM_LDLU(vd + 1344);
    }
    {
      double x = b[1376];
      x = fma(-CHEM_LDLU(lu + 95328), b[1056], x);
      b[1376] = x * CHEM_LDLU(vd + 1376);
    }
    {
      double x = b[1408];
      b[1408] = x * CHEM_LDLU(vd + 1408);
    }
    {
      double x = b[1440];
      b[1440] = x * CHEM_LDLU(vd + 1440);
    }
    {
      double x = b[1472];
      b[1472] = x * CHEM_LDLU(vd + 1472);
    }
    {
      double x = b[1504];
      b[1504] = x * CHEM_LDLU(vd + 1504);
    }
    {
      double x = b[1536];
      b[1536] = x * CHEM_LDLU(vd + 1536);
    }
    {
      double x = b[1568];
      b[1568] = x * CHEM_LDLU(vd + 1568);
    }
    {
      double x = b[1600];
      b[1600] = x * CHEM_LDLU(vd + 1600);
    }
    {
      double x = b[1632];
      b[1632] = x * CHEM_LDLU(vd + 1632);
    }
    {
      double x = b[1664];
      x = fma(-CHEM_LDLU(lu + 96288), b[32], x);
      b[1664] = x * CHEM_LDLU(vd + 1664);
    }
    {
      double x = b[1696];
      b[1696] = x * CHEM_LDLU(vd + 1696);
    }
    {
      double x = b[1728];
      b[1728] = x * CHEM_LDLU(vd + 1728);
    }
    {
      double x = b[1760];
      b[1760] = x * CHEM_LDLU(vd + 1760);
    }
    {
      double x = b[1792];
      b[1792] = x * CHEM_LDLU(vd + 1792);
    }
    {
      double x = b[1824];
      b[1824] = x * CHEM_LDLU(vd + 1824);
    }
    {
      double x = b[1856];
      b[1856] = x * CHEM_LDLU(vd + 1856);
    }
    {
      double x = b[1888];
      b[1888] = x * CHEM_LDLU(vd + 1888);
    }
    {
      double x = b[1920];
      b[1920] = x * CHEM_LDLU(vd + 1920);
    }
    {
      double x = b[1952];
      b[1952] = x * CHEM_LDLU(vd + 1952);
    }
    {
      double x = b[1984];
      b[1984] = x * CHEM_LDLU(vd + 1984);
    }
    {
      double x = b[2016];
      b[2016] = x * CHEM_LDLU(vd + 2016);
    }
    {
      double x = b[2048];
      b[2048] = x * CHEM_LDLU(vd + 2048);
    }
    {
      double x = b[2080];
      b[2080] = x * CHEM_LDLU(vd + 2080);
    }
    {
      double x = b[2112];
      b[2112] = x * CHEM_LDLU(vd + 2112);
    }
    {
      double x = b[2144];
      b[2144] = x * CHEM_LDLU(vd + 2144);
    }
    {
      double x = b[2176];
      b[2176] = x * CHEM_LDLU(vd + 2176);
    }
    {
      double x = b[2208];
      x = fma(-CHEM_LDLU(lu + 96256), b[64], x);
      b[2208] = x * CHEM_LDLU(vd + 2208);
    }
    {
      double x = b[2240];
      b[2240] = x * CHEM_LDLU(vd + 2240);
    }
    {
      double x = b[2272];
      b[2272] = x * CHEM_LDLU(vd + 2272);
    }
    {
      double x = b[2304];
      b[2304] = x * CHEM_LDLU(vd + 2304);
    }
    {
      double x = b[2336];
      b[2336] = x * CHEM_LDLU(vd + 2336);
    }
    {
      double x = b[2368];
      x = fma(-CHEM_LDLU(lu + 92064), b[1952], x);
      b[2368] = x * CHEM_LDLU(vd + 2368);
    }
    {
      double x = b[2400];
      x = fma(-CHEM_LDLU(lu + 91936), b[1984], x);
      b[2400] = x * CHEM_LDLU(vd + 2400);
    }
    {
      double x = b[2432];
      x = fma(-CHEM_LDLU(lu + 91808), b[2016], x);
      b[2432] = x * CHEM_LDLU(vd + 2432);
    }
    {
      double x = b[2464];
      x = fma(-CHEM_LDLU(lu + 91680), b[2048], x);
      b[2464] = x * CHEM_LDLU(vd + 2464);
    }
    {
      double x = b[2496];
      x = fma(-CHEM_LDLU(lu + 91552), b[2080], x);
      b[2496] = x * CHEM_LDLU(vd + 2496);
    }
    {
      double x = b[2528];
      x = fma(-CHEM_LDLU(lu + 91424), b[2112], x);
      b[2528] = x * CHEM_LDLU(vd + 2528);
    }
    {
      double x = b[2560];
      b[2560] = x * CHEM_LDLU(vd + 2560);
    }
    {
      double x = b[2592];
      x = fma(-CHEM_LDLU(lu + 90720), b[2272], x);
      b[2592] = x * CHEM_LDLU(vd + 2592);
    }
    {
      double x = b[2624];
      b[2624] = x * CHEM_LDLU(vd + 2624);
    }
    {
      double x = b[2656];
      b[2656] = x * CHEM_LDLU(vd + 2656);
    }
    {
      double x = b[2688];
      b[2688] = x * CHEM_LDLU(vd + 2688);
    }
    {
      double x = b[2720];
      b[2720] = x * CHEM_LDLU(vd + 2720);
    }
    {
      double x = b[2752];
      x = fma(-CHEM_LDLU(lu + 95136), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 94848), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 94720), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 92864), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 92352), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 91168), b[2176], x);
      b[2752] = x * CHEM_LDLU(vd + 2752);
    }
    {
      double x = b[2784];
      x = fma(-CHEM_LDLU(lu + 94304), b[1376], x);
      x = fma(-CHEM_LDLU(lu + 90976), b[2208], x);
      b[2784] = x * CHEM_LDLU(vd + 2784);
    }
    {
      double x = b[2816];
      b[2816] = x * CHEM_LDLU(vd + 2816);
    }
    {
      double x = b[2848];
      b[2848] = x * CHEM_LDLU(vd + 2848);
    }
    {
      double x = b[2880];
      b[2880] = x * CHEM_LDLU(vd + 2880);
    }
    {
      double x = b[2912];
      b[2912] = x * CHEM_LDLU(vd + 2912);
    }
    {
      double x = b[2944];
      x = fma(-CHEM_LDLU(lu + 92896), b[1760], x);
      b[2944] = x * CHEM_LDLU(vd + 2944);
    }
    {
      double x = b[2976];
      b[2976] = x * CHEM_LDLU(vd + 2976);
    }
    {
      double x = b[3008];
      x = fma(-CHEM_LDLU(lu + 93920), b[1504], x);
      b[3008] = x * CHEM_LDLU(vd + 3008);
    }
    {
      double x = b[3040];
      b[3040] = x * CHEM_LDLU(vd + 3040);
    }
    {
      double x = b[3072];
      b[3072] = x * CHEM_LDLU(vd + 3072);
    }
    {
      double x = b[3104];
      b[3104] = x * CHEM_LDLU(vd + 3104);
    }
    {
      double x = b[3136];
      x = fma(-CHEM_LDLU(lu + 88256), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 86112), b[3072], x);
      b[3136] = x * CHEM_LDLU(vd + 3136);
    }
    {
      double x = b[3168];
      x = fma(-CHEM_LDLU(lu + 92480), b[1856], x);
      b[3168] = x * CHEM_LDLU(vd + 3168);
    }
    {
      double x = b[3200];
      b[3200] = x * CHEM_LDLU(vd + 3200);
    }
    {
      double x = b[3232];
      x = fma(-CHEM_LDLU(lu + 87072), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 86144), b[3072], x);
      b[3232] = x * CHEM_LDLU(vd + 3232);
    }
    {
      double x = b[3264];
      b[3264] = x * CHEM_LDLU(vd + 3264);
    }
    {
      double x = b[3296];
      b[3296] = x * CHEM_LDLU(vd + 3296);
    }
    {
      double x = b[3328];
      b[3328] = x * CHEM_LDLU(vd + 3328);
    }
    {
      double x = b[3360];
      b[3360] = x * CHEM_LDLU(vd + 3360);
    }
    {
      double x = b[3392];
      b[3392] = x * CHEM_LDLU(vd + 3392);
    }
    {
      double x = b[3424];
      b[3424] = x * CHEM_LDLU(vd + 3424);
    }
    {
      double x = b[3456];
      b[3456] = x * CHEM_LDLU(vd + 3456);
    }
    {
      double x = b[3488];
      b[3488] = x * CHEM_LDLU(vd + 3488);
    }
    {
      double x = b[3520];
      x = fma(-CHEM_LDLU(lu + 92736), b[1792], x);
      b[3520] = x * CHEM_LDLU(vd + 3520);
    }
    {
      double x = b[3552];
      x = fma(-CHEM_LDLU(lu + 83136), b[3520], x);
      b[3552] = x * CHEM_LDLU(vd + 3552);
    }
    {
      double x = b[3584];
      b[3584] = x * CHEM_LDLU(vd + 3584);
    }
    {
      double x = b[3616];
      b[3616] = x * CHEM_LDLU(vd + 3616);
    }
    {
      double x = b[3648];
      b[3648] = x * CHEM_LDLU(vd + 3648);
    }
    {
      double x = b[3680];
      b[3680] = x * CHEM_LDLU(vd + 3680);
    }
    {
      double x = b[3712];
      x = fma(-CHEM_LDLU(lu + 88416), b[2720], x);
      b[3712] = x * CHEM_LDLU(vd + 3712);
    }
    {
      double x = b[3744];
      x = fma(-CHEM_LDLU(lu + 88448), b[2720], x);
      b[3744] = x * CHEM_LDLU(vd + 3744);
    }
    {
      double x = b[3776];
      b[3776] = x * CHEM_LDLU(vd + 3776);
    }
    {
      double x = b[3808];
      x = fma(-CHEM_LDLU(lu + 86400), b[3040], x);
      b[3808] = x * CHEM_LDLU(vd + 3808);
    }
    {
      double x = b[3840];
      x = fma(-CHEM_LDLU(lu + 88480), b[2720], x);
      b[3840] = x * CHEM_LDLU(vd + 3840);
    }
    {
      double x = b[3872];
      x = fma(-CHEM_LDLU(lu + 87200), b[2912], x);
      b[3872] = x * CHEM_LDLU(vd + 3872);
    }
    {
      double x = b[3904];
      x = fma(-CHEM_LDLU(lu + 91296), b[2144], x);
      b[3904] = x * CHEM_LDLU(vd + 3904);
    }
    {
      double x = b[3936];
      x = fma(-CHEM_LDLU(lu + 88512), b[2720], x);
      b[3936] = x * CHEM_LDLU(vd + 3936);
    }
    {
      double x = b[3968];
      b[3968] = x * CHEM_LDLU(vd + 3968);
    }
    {
      double x = b[4000];
      b[4000] = x * CHEM_LDLU(vd + 4000);
    }
    {
      double x = b[4032];
      b[4032] = x * CHEM_LDLU(vd + 4032);
    }
    {
      double x = b[4064];
      x = fma(-CHEM_LDLU(lu + 78816), b[4032], x);
      b[4064] = x * CHEM_LDLU(vd + 4064);
    }
    {
      double x = b[4096];
      x = fma(-CHEM_LDLU(lu + 79936), b[3904], x);
      b[4096] = x * CHEM_LDLU(vd + 4096);
    }
    {
      double x = b[4128];
      x = fma(-CHEM_LDLU(lu + 83168), b[3520], x);
      b[4128] = x * CHEM_LDLU(vd + 4128);
    }
    {
      double x = b[4160];
      x = fma(-CHEM_LDLU(lu + 88544), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 81536), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81216), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 80352), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 79616), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 78240), b[4096], x);
      b[4160] = x * CHEM_LDLU(vd + 4160);
    }
    {
      double x = b[4192];
      x = fma(-CHEM_LDLU(lu + 88576), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 81568), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81248), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 80384), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 79648), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 78272), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 77696), b[4160], x);
      b[4192] = x * CHEM_LDLU(vd + 4192);
    }
    {
      double x = b[4224];
      x = fma(-CHEM_LDLU(lu + 79328), b[3968], x);
      b[4224] = x * CHEM_LDLU(vd + 4224);
    }
    {
      double x = b[4256];
      b[4256] = x * CHEM_LDLU(vd + 4256);
    }
    {
      double x = b[4288];
      x = fma(-CHEM_LDLU(lu + 94432), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 94336), b[1376], x);
      x = fma(-CHEM_LDLU(lu + 93280), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 88608), b[2720], x);
      x = fma(-CHEM_LDLU(lu + 88064), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 81600), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81280), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 80416), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 79680), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 77984), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77728), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77440), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 76800), b[4256], x);
      b[4288] = x * CHEM_LDLU(vd + 4288);
    }
    {
      double x = b[4320];
      b[4320] = x * CHEM_LDLU(vd + 4320);
    }
    {
      double x = b[4352];
      b[4352] = x * CHEM_LDLU(vd + 4352);
    }
    {
      double x = b[4384];
      x = fma(-CHEM_LDLU(lu + 93152), b[1696], x);
      b[4384] = x * CHEM_LDLU(vd + 4384);
    }
    {
      double x = b[4416];
      x = fma(-CHEM_LDLU(lu + 79360), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77120), b[4224], x);
      b[4416] = x * CHEM_LDLU(vd + 4416);
    }
    {
      double x = b[4448];
      x = fma(-CHEM_LDLU(lu + 89312), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 88640), b[2688], x);
      b[4448] = x * CHEM_LDLU(vd + 4448);
    }
    {
      double x = b[4480];
      x = fma(-CHEM_LDLU(lu + 87648), b[2848], x);
      b[4480] = x * CHEM_LDLU(vd + 4480);
    }
    {
      double x = b[4512];
      x = fma(-CHEM_LDLU(lu + 82400), b[3616], x);
      b[4512] = x * CHEM_LDLU(vd + 4512);
    }
    {
      double x = b[4544];
      x = fma(-CHEM_LDLU(lu + 89504), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 78304), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 76832), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 75776), b[4384], x);
      b[4544] = x * CHEM_LDLU(vd + 4544);
    }
    {
      double x = b[4576];
      x = fma(-CHEM_LDLU(lu + 93024), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 87872), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 81856), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 79072), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 78336), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 76864), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76064), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 75808), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 74528), b[4544], x);
      b[4576] = x * CHEM_LDLU(vd + 4576);
    }
    {
      double x = b[4608];
      x = fma(-CHEM_LDLU(lu + 79968), b[3904], x);
      b[4608] = x * CHEM_LDLU(vd + 4608);
    }
    {
      double x = b[4640];
      x = fma(-CHEM_LDLU(lu + 77152), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 73824), b[4608], x);
      b[4640] = x * CHEM_LDLU(vd + 4640);
    }
    {
      double x = b[4672];
      x = fma(-CHEM_LDLU(lu + 92768), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 92608), b[1824], x);
      b[4672] = x * CHEM_LDLU(vd + 4672);
    }
    {
      double x = b[4704];
      x = fma(-CHEM_LDLU(lu + 79392), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77184), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 75520), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 73856), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73344), b[4640], x);
      b[4704] = x * CHEM_LDLU(vd + 4704);
    }
    {
      double x = b[4736];
      x = fma(-CHEM_LDLU(lu + 87424), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 76096), b[4352], x);
      b[4736] = x * CHEM_LDLU(vd + 4736);
    }
    {
      double x = b[4768];
      b[4768] = x * CHEM_LDLU(vd + 4768);
    }
    {
      double x = b[4800];
      x = fma(-CHEM_LDLU(lu + 93824), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 81888), b[3680], x);
      b[4800] = x * CHEM_LDLU(vd + 4800);
    }
    {
      double x = b[4832];
      x = fma(-CHEM_LDLU(lu + 79424), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77216), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 75552), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 73888), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73376), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72640), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 71936), b[4768], x);
      b[4832] = x * CHEM_LDLU(vd + 4832);
    }
    {
      double x = b[4864];
      x = fma(-CHEM_LDLU(lu + 80928), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 73920), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73408), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72672), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 71968), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71136), b[4832], x);
      b[4864] = x * CHEM_LDLU(vd + 4864);
    }
    {
      double x = b[4896];
      x = fma(-CHEM_LDLU(lu + 72000), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 70688), b[4864], x);
      b[4896] = x * CHEM_LDLU(vd + 4896);
    }
    {
      double x = b[4928];
      x = fma(-CHEM_LDLU(lu + 80960), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 73440), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72704), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72032), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71168), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70720), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70272), b[4896], x);
      b[4928] = x * CHEM_LDLU(vd + 4928);
    }
    {
      double x = b[4960];
      x = fma(-CHEM_LDLU(lu + 79456), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77248), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 75584), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 73952), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73472), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72736), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72064), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71200), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70752), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70304), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 69888), b[4928], x);
      b[4960] = x * CHEM_LDLU(vd + 4960);
    }
    {
      double x = b[4992];
      x = fma(-CHEM_LDLU(lu + 77280), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 73984), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73504), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72768), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72096), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71232), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70784), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70336), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 69920), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69536), b[4960], x);
      b[4992] = x * CHEM_LDLU(vd + 4992);
    }
    {
      double x = b[5024];
      b[5024] = x * CHEM_LDLU(vd + 5024);
    }
    {
      double x = b[5056];
      b[5056] = x * CHEM_LDLU(vd + 5056);
    }
    {
      double x = b[5088];
      x = fma(-CHEM_LDLU(lu + 79488), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77312), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 75616), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 74016), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73536), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72800), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72128), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71264), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70816), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70368), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 69952), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69568), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69216), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 68320), b[5056], x);
      b[5088] = x * CHEM_LDLU(vd + 5088);
    }
    {
      double x = b[5120];
      x = fma(-CHEM_LDLU(lu + 75008), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 68352), b[5056], x);
      b[5120] = x * CHEM_LDLU(vd + 5120);
    }
    {
      double x = b[5152];
      x = fma(-CHEM_LDLU(lu + 68384), b[5056], x);
      b[5152] = x * CHEM_LDLU(vd + 5152);
    }
    {
      double x = b[5184];
      x = fma(-CHEM_LDLU(lu + 95168), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 95040), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 94880), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 94752), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 94528), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 94208), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 94112), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 93728), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 93632), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 93472), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 93312), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 93184), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 92928), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 92384), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 92192), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 91200), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 91008), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 90880), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 90560), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 90464), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 89536), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 89088), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 88864), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88288), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 88096), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 87904), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 86624), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86432), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 86176), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 85696), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85472), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85248), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 84992), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84384), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84160), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 82912), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82688), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82432), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82144), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 81920), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81632), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81312), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 80672), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80448), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80128), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 79712), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79104), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 78848), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78592), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78368), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78016), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77760), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77472), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 76896), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76576), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76352), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76128), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 75840), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75296), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75040), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74784), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74560), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74304), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 73088), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 72416), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 71584), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71296), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70848), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70400), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 69984), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69600), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69248), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 68800), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68416), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68032), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67744), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67424), b[5152], x);
      b[5184] = x * CHEM_LDLU(vd + 5184);
    }
    {
      double x = b[5216];
      x = fma(-CHEM_LDLU(lu + 71616), b[4800], x);
      b[5216] = x * CHEM_LDLU(vd + 5216);
    }
    {
      double x = b[5248];
      x = fma(-CHEM_LDLU(lu + 95872), b[480], x);
      x = fma(-CHEM_LDLU(lu + 68832), b[5024], x);
      b[5248] = x * CHEM_LDLU(vd + 5248);
    }
    {
      double x = b[5280];
      x = fma(-CHEM_LDLU(lu + 67456), b[5152], x);
      b[5280] = x * CHEM_LDLU(vd + 5280);
    }
    {
      double x = b[5312];
      x = fma(-CHEM_LDLU(lu + 79520), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77344), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 74048), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73568), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72832), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72160), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71328), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70880), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70432), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70016), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69632), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69280), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 68448), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68064), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67776), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67488), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 66720), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66336), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 65984), b[5280], x);
      b[5312] = x * CHEM_LDLU(vd + 5312);
    }
    {
      double x = b[5344];
      x = fma(-CHEM_LDLU(lu + 66368), b[5248], x);
      b[5344] = x * CHEM_LDLU(vd + 5344);
    }
    {
      double x = b[5376];
      x = fma(-CHEM_LDLU(lu + 95904), b[480], x);
      x = fma(-CHEM_LDLU(lu + 68864), b[5024], x);
      b[5376] = x * CHEM_LDLU(vd + 5376);
    }
    {
      double x = b[5408];
      x = fma(-CHEM_LDLU(lu + 75072), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 68480), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 66752), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66016), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65088), b[5376], x);
      b[5408] = x * CHEM_LDLU(vd + 5408);
    }
    {
      double x = b[5440];
      x = fma(-CHEM_LDLU(lu + 64736), b[5408], x);
      b[5440] = x * CHEM_LDLU(vd + 5440);
    }
    {
      double x = b[5472];
      x = fma(-CHEM_LDLU(lu + 71648), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 67168), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 66784), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66400), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66048), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65696), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65408), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65120), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 64768), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64416), b[5440], x);
      b[5472] = x * CHEM_LDLU(vd + 5472);
    }
    {
      double x = b[5504];
      x = fma(-CHEM_LDLU(lu + 80992), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 68512), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 66816), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66432), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 64096), b[5472], x);
      b[5504] = x * CHEM_LDLU(vd + 5504);
    }
    {
      double x = b[5536];
      x = fma(-CHEM_LDLU(lu + 79552), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 77376), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 74080), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73600), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 72864), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72192), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71360), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70912), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70464), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70048), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69664), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69312), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 68544), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68096), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67808), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67520), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 66848), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66464), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66080), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65728), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65440), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 64800), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64448), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64128), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 63808), b[5504], x);
      b[5536] = x * CHEM_LDLU(vd + 5536);
    }
    {
      double x = b[5568];
      x = fma(-CHEM_LDLU(lu + 68896), b[5024], x);
      b[5568] = x * CHEM_LDLU(vd + 5568);
    }
    {
      double x = b[5600];
      b[5600] = x * CHEM_LDLU(vd + 5600);
    }
    {
      double x = b[5632];
      x = fma(-CHEM_LDLU(lu + 94016), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 63264), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 62976), b[5600], x);
      b[5632] = x * CHEM_LDLU(vd + 5632);
    }
    {
      double x = b[5664];
      b[5664] = x * CHEM_LDLU(vd + 5664);
    }
    {
      double x = b[5696];
      x = fma(-CHEM_LDLU(lu + 86848), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 65152), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 62368), b[5664], x);
      b[5696] = x * CHEM_LDLU(vd + 5696);
    }
    {
      double x = b[5728];
      x = fma(-CHEM_LDLU(lu + 66880), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 64832), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64480), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64160), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 63840), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63552), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63296), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63008), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62688), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62400), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62080), b[5696], x);
      b[5728] = x * CHEM_LDLU(vd + 5728);
    }
    {
      double x = b[5760];
      x = fma(-CHEM_LDLU(lu + 71680), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 68928), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 66912), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 62720), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62112), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 61824), b[5728], x);
      b[5760] = x * CHEM_LDLU(vd + 5760);
    }
    {
      double x = b[5792];
      x = fma(-CHEM_LDLU(lu + 95232), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 90752), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 89344), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 89120), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 88896), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88672), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 87680), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 87456), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 87232), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 86880), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 86656), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86464), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 86208), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 85920), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 85728), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85504), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85280), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 85024), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84800), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 84608), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 84416), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84192), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 83968), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 83776), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 83584), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 83392), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 83200), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 82944), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82720), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82464), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82176), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 81952), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81664), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81344), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 81024), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 80704), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80480), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80160), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 79744), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79136), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 78880), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78624), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78400), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78048), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77792), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77504), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 76928), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76608), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76384), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76160), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 75872), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75328), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75104), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74816), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74592), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74336), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74112), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73632), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73120), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 72896), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72448), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 72224), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71712), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71392), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70944), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70496), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70080), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69696), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69344), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 68960), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68576), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68128), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67840), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67552), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 67200), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 66944), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66496), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66112), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65760), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65472), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65184), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 64864), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64512), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64192), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 63872), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63584), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63328), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63040), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62752), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62432), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62144), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 61856), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61600), b[5760], x);
      b[5792] = x * CHEM_LDLU(vd + 5792);
    }
    {
      double x = b[5824];
      x = fma(-CHEM_LDLU(lu + 94944), b[1184], x);
      x = fma(-CHEM_LDLU(lu + 93504), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 93344), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 93056), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 92512), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 92224), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 92096), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 91968), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 91840), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 91712), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 91584), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 91456), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 91328), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 91040), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 90784), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 90592), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 90496), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 90336), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 90208), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 90080), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 89952), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 89824), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 89696), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 89568), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 89376), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 89152), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 88928), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88704), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 88128), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 87712), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 87488), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 87264), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 86912), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 86688), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86496), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 86240), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 85952), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 85760), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85536), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85312), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 85056), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84832), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 84640), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 84448), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84224), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 84000), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 83808), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 83616), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 83424), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 83232), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 82976), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82752), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82496), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82208), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 81984), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81696), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81376), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 81056), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 80736), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80512), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80192), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 80000), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 79776), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79168), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 78912), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78656), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78432), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78080), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77824), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77536), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 76960), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76640), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76416), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76192), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 75904), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75648), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 75360), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75136), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74848), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74624), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74368), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74144), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73664), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73152), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 72928), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72480), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 72256), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71744), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71424), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 70976), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70528), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70112), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69728), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69376), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 68992), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68608), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68160), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67872), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67584), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 67232), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 66976), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66528), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66144), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65792), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65504), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65216), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 64896), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64544), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64224), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 63904), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63616), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63360), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63072), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62784), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62464), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62176), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 61888), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61632), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61408), b[5792], x);
      b[5824] = x * CHEM_LDLU(vd + 5824);
    }
    {
      double x = b[5856];
      x = fma(-CHEM_LDLU(lu + 69024), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 62496), b[5664], x);
      b[5856] = x * CHEM_LDLU(vd + 5856);
    }
}
__device__ __noinline__ void solve_t_1_1(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[5888];
      x = fma(-CHEM_LDLU(lu + 94048), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 93952), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 90816), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 89408), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 89184), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 88960), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88736), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 88320), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 87936), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 87744), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 87520), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 87296), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 86944), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 86720), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86528), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 86272), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 85984), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 85792), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85568), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85344), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 85088), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84864), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 84672), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 84480), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84256), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 84032), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 83840), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 83648), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 83456), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 83264), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 83008), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82784), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82528), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82240), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 82016), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81728), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81408), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 81088), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 80768), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80544), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80224), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 79808), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79200), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 78944), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78688), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78464), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78112), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77856), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77568), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 76992), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76672), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76448), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76224), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 75936), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75392), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75168), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74880), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74656), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74400), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74176), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73696), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73184), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 72960), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72512), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 72288), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71776), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71456), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 71008), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70560), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70144), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69760), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69408), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 69056), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68640), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68192), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67904), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67616), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 67264), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67008), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66560), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66176), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65824), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65536), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65248), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 64928), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64576), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64256), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 63936), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63648), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63392), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63104), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62816), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62528), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62208), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 61920), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61664), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61440), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61248), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61088), b[5856], x);
      b[5888] = x * CHEM_LDLU(vd + 5888);
    }
    {
      double x = b[5920];
      x = fma(-CHEM_LDLU(lu + 95360), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 95264), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 94976), b[1184], x);
      x = fma(-CHEM_LDLU(lu + 94624), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 93856), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 92640), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 90528), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 88768), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 85120), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 82560), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82272), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 80800), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 73216), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 71808), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 69088), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68672), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 67296), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67040), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66592), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66208), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65856), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65568), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65280), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 64960), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64608), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64288), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 63968), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63680), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63424), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63136), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62848), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62560), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62240), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 61952), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61696), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61472), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61280), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61120), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 60960), b[5888], x);
      b[5920] = x * CHEM_LDLU(vd + 5920);
    }
    {
      double x = b[5952];
      x = fma(-CHEM_LDLU(lu + 95392), b[1024], x);
      x = fma(-CHEM_LDLU(lu + 95072), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 94784), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 94560), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 94240), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 94144), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 93760), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 93664), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 93536), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 93376), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 93216), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 92960), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 92672), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 92416), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 92256), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 92128), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 92000), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 91872), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 91744), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 91616), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 91488), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 91360), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 91232), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 91072), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 90912), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 90848), b[2272], x);
      x = fma(-CHEM_LDLU(lu + 90624), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 90368), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 90240), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 90112), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 89984), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 89856), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 89728), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 89600), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 89440), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 89216), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 88992), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88800), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 88352), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 88160), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 87968), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 87776), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 87552), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 87328), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 87104), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 86976), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 86752), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86560), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 86304), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 86016), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 85824), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85600), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85376), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 85152), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84896), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 84704), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 84512), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84288), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 84064), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 83872), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 83680), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 83488), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 83296), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 83040), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82816), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82592), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82304), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 82048), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81760), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81440), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 81120), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 80832), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80576), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80256), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 80032), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 79840), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79232), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 78976), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78720), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78496), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78144), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77888), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77600), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 77024), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76704), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76480), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76256), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 75968), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75680), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 75424), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75200), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74912), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74688), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74432), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74208), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73728), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73248), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 72992), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72544), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 72320), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71840), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71488), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 71040), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70592), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70176), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69792), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69440), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 69120), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68704), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68224), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67936), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67648), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 67328), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67072), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66624), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66240), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65888), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65600), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65312), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 64992), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64640), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64320), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 64000), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63712), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63456), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63168), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62880), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62592), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62272), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 61984), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61728), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61504), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61312), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61152), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 60992), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 60864), b[5920], x);
      b[5952] = x * CHEM_LDLU(vd + 5952);
    }
    {
      double x = b[5984];
      x = fma(-CHEM_LDLU(lu + 94656), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 94464), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 94368), b[1376], x);
      x = fma(-CHEM_LDLU(lu + 93568), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 93408), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 93088), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 92800), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 92544), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 92288), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 92160), b[1952], x);
      x = fma(-CHEM_LDLU(lu + 92032), b[1984], x);
      x = fma(-CHEM_LDLU(lu + 91904), b[2016], x);
      x = fma(-CHEM_LDLU(lu + 91776), b[2048], x);
      x = fma(-CHEM_LDLU(lu + 91648), b[2080], x);
      x = fma(-CHEM_LDLU(lu + 91520), b[2112], x);
      x = fma(-CHEM_LDLU(lu + 91392), b[2144], x);
      x = fma(-CHEM_LDLU(lu + 91104), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 90656), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 90400), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 90272), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 90144), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 90016), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 89888), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 89760), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 89632), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 89248), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 89024), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88192), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 88000), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 87808), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 87584), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 87360), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 87136), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 87008), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 86784), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86592), b[3040], x);
      x = fma(-CHEM_LDLU(lu + 86336), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 86048), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 85856), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85632), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85408), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 85184), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84928), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 84736), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 84544), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84320), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 84096), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 83904), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 83712), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 83520), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 83328), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 83072), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82848), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82624), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82336), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 82080), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81792), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81472), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 81152), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 80864), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80608), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80288), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 80064), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 79872), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79264), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 79008), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78752), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78528), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78176), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77920), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77632), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 77056), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76736), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76512), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76288), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 76000), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75712), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 75456), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75232), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74944), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74720), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74464), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74240), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73760), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73280), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 73024), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72576), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 72352), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71872), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71520), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 71072), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70624), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70208), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69824), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69472), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 69152), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68736), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68256), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 67968), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67680), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 67360), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67104), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66656), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66272), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65920), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65632), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65344), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 65024), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64672), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64352), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 64032), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63744), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63488), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63200), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62912), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62624), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62304), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 62016), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61760), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61536), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61344), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61184), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 61024), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 60896), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 60800), b[5952], x);
      b[5984] = x * CHEM_LDLU(vd + 5984);
    }
    {
      double x = b[6016];
      x = fma(-CHEM_LDLU(lu + 96224), b[160], x);
      x = fma(-CHEM_LDLU(lu + 96192), b[192], x);
      x = fma(-CHEM_LDLU(lu + 96160), b[224], x);
      x = fma(-CHEM_LDLU(lu + 96128), b[256], x);
      x = fma(-CHEM_LDLU(lu + 96096), b[288], x);
      x = fma(-CHEM_LDLU(lu + 96064), b[320], x);
      x = fma(-CHEM_LDLU(lu + 96032), b[352], x);
      x = fma(-CHEM_LDLU(lu + 96000), b[384], x);
      x = fma(-CHEM_LDLU(lu + 95968), b[416], x);
      x = fma(-CHEM_LDLU(lu + 95936), b[448], x);
      x = fma(-CHEM_LDLU(lu + 95776), b[608], x);
      x = fma(-CHEM_LDLU(lu + 95744), b[640], x);
      x = fma(-CHEM_LDLU(lu + 95712), b[672], x);
      x = fma(-CHEM_LDLU(lu + 95680), b[704], x);
      x = fma(-CHEM_LDLU(lu + 95648), b[736], x);
      x = fma(-CHEM_LDLU(lu + 95616), b[768], x);
      x = fma(-CHEM_LDLU(lu + 95584), b[800], x);
      x = fma(-CHEM_LDLU(lu + 95552), b[832], x);
      x = fma(-CHEM_LDLU(lu + 95520), b[864], x);
      x = fma(-CHEM_LDLU(lu + 95488), b[896], x);
      x = fma(-CHEM_LDLU(lu + 95456), b[928], x);
      x = fma(-CHEM_LDLU(lu + 95424), b[992], x);
      x = fma(-CHEM_LDLU(lu + 95296), b[1088], x);
      x = fma(-CHEM_LDLU(lu + 95200), b[1120], x);
      x = fma(-CHEM_LDLU(lu + 95104), b[1152], x);
      x = fma(-CHEM_LDLU(lu + 95008), b[1184], x);
      x = fma(-CHEM_LDLU(lu + 94912), b[1216], x);
      x = fma(-CHEM_LDLU(lu + 94816), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 94688), b[1280], x);
      x = fma(-CHEM_LDLU(lu + 94592), b[1312], x);
      x = fma(-CHEM_LDLU(lu + 94496), b[1344], x);
      x = fma(-CHEM_LDLU(lu + 94400), b[1376], x);
      x = fma(-CHEM_LDLU(lu + 94272), b[1408], x);
      x = fma(-CHEM_LDLU(lu + 94176), b[1440], x);
      x = fma(-CHEM_LDLU(lu + 94080), b[1472], x);
      x = fma(-CHEM_LDLU(lu + 93984), b[1504], x);
      x = fma(-CHEM_LDLU(lu + 93888), b[1536], x);
      x = fma(-CHEM_LDLU(lu + 93792), b[1568], x);
      x = fma(-CHEM_LDLU(lu + 93696), b[1600], x);
      x = fma(-CHEM_LDLU(lu + 93600), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 93440), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 93248), b[1696], x);
      x = fma(-CHEM_LDLU(lu + 93120), b[1728], x);
      x = fma(-CHEM_LDLU(lu + 92992), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 92832), b[1792], x);
      x = fma(-CHEM_LDLU(lu + 92704), b[1824], x);
      x = fma(-CHEM_LDLU(lu + 92576), b[1856], x);
      x = fma(-CHEM_LDLU(lu + 92448), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 92320), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 91264), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 91136), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 90944), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 90688), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 90432), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 90304), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 90176), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 90048), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 89920), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 89792), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 89664), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 89472), b[2592], x);
      x = fma(-CHEM_LDLU(lu + 89280), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 89056), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 88832), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 88384), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 88224), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 88032), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 87840), b[2848], x);
      x = fma(-CHEM_LDLU(lu + 87616), b[2880], x);
      x = fma(-CHEM_LDLU(lu + 87392), b[2912], x);
      x = fma(-CHEM_LDLU(lu + 87168), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 87040), b[2976], x);
      x = fma(-CHEM_LDLU(lu + 86816), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 86368), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 86080), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 85888), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 85664), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 85440), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 85216), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 84960), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 84768), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 84576), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 84352), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 84128), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 83936), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 83744), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 83552), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 83360), b[3520], x);
      x = fma(-CHEM_LDLU(lu + 83104), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 82880), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 82656), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 82368), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 82112), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 81824), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 81504), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 81184), b[3776], x);
      x = fma(-CHEM_LDLU(lu + 80896), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 80640), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 80320), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 80096), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 79904), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 79584), b[3968], x);
      x = fma(-CHEM_LDLU(lu + 79296), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 79040), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 78784), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 78560), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 78208), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 77952), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 77664), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 77408), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 77088), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 76768), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 76544), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 76320), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 76032), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 75744), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 75488), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 75264), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 74976), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 74752), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 74496), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 74272), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 73792), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 73312), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 73056), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 72608), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 72384), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 71904), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 71552), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 71104), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 70656), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 70240), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 69856), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 69504), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 69184), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 68768), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 68288), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 68000), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 67712), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 67392), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 67136), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 66688), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 66304), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 65952), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 65664), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 65376), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 65056), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 64704), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 64384), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 64064), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 63776), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 63520), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 63232), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 62944), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 62656), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 62336), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 62048), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 61792), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 61568), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 61376), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 61216), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 61056), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 60928), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 60832), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 60768), b[5984], x);
      b[6016] = x * CHEM_LDLU(vd + 6016);
    }
    {
      double x = b[5984];
      x = fma(-CHEM_LDLU(lu + 60736), b[6016], x);
      b[5984] = x;
    }
    {
      double x = b[5952];
      x = fma(-CHEM_LDLU(lu + 56512), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60704), b[6016], x);
      b[5952] = x;
    }
    {
      double x = b[5920];
      x = fma(-CHEM_LDLU(lu + 52256), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56480), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60672), b[6016], x);
      b[5920] = x;
    }
    {
      double x = b[5888];
      x = fma(-CHEM_LDLU(lu + 48640), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52224), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56448), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60640), b[6016], x);
      b[5888] = x;
    }
    {
      double x = b[5856];
      x = fma(-CHEM_LDLU(lu + 52192), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56416), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60608), b[6016], x);
      b[5856] = x;
    }
    {
      double x = b[5824];
      x = fma(-CHEM_LDLU(lu + 42496), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45184), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48608), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52160), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56384), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60576), b[6016], x);
      b[5824] = x;
    }
    {
      double x = b[5792];
      x = fma(-CHEM_LDLU(lu + 39712), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42464), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45152), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48576), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52128), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56352), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60544), b[6016], x);
      b[5792] = x;
    }
    {
      double x = b[5760];
      x = fma(-CHEM_LDLU(lu + 36672), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39680), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42432), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45120), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48544), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52096), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56320), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60512), b[6016], x);
      b[5760] = x;
    }
    {
      double x = b[5728];
      x = fma(-CHEM_LDLU(lu + 34272), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36640), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39648), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42400), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45088), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48512), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52064), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56288), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60480), b[6016], x);
      b[5728] = x;
    }
    {
      double x = b[5696];
      x = fma(-CHEM_LDLU(lu + 32672), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 36608), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39616), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42368), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45056), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48480), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52032), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56256), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60448), b[6016], x);
      b[5696] = x;
    }
    {
      double x = b[5664];
      x = fma(-CHEM_LDLU(lu + 56224), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60416), b[6016], x);
      b[5664] = x;
    }
    {
      double x = b[5632];
      x = fma(-CHEM_LDLU(lu + 30816), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32640), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 36576), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39584), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42336), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45024), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48448), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52000), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56192), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60384), b[6016], x);
      b[5632] = x;
    }
    {
      double x = b[5600];
      x = fma(-CHEM_LDLU(lu + 42304), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 56160), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60352), b[6016], x);
      b[5600] = x;
    }
    {
      double x = b[5568];
      x = fma(-CHEM_LDLU(lu + 36544), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 51968), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 60320), b[6016], x);
      b[5568] = x;
    }
    {
      double x = b[5536];
      x = fma(-CHEM_LDLU(lu + 25536), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27104), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28064), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 29056), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30784), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32608), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34240), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36512), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39552), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42272), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44992), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48416), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51936), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56128), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60288), b[6016], x);
      b[5536] = x;
    }
    {
      double x = b[5504];
      x = fma(-CHEM_LDLU(lu + 24512), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25504), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27072), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28032), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 29024), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30752), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32576), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34208), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36480), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39520), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42240), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44960), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48384), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51904), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56096), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60256), b[6016], x);
      b[5504] = x;
    }
    {
      double x = b[5472];
      x = fma(-CHEM_LDLU(lu + 23584), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24480), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25472), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27040), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28000), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28992), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30720), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32544), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34176), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36448), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39488), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42208), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44928), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48352), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51872), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56064), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60224), b[6016], x);
      b[5472] = x;
    }
    {
      double x = b[5440];
      x = fma(-CHEM_LDLU(lu + 22464), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23552), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 25440), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27008), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27968), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28960), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30688), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32512), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34144), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36416), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39456), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42176), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44896), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48320), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51840), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56032), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60192), b[6016], x);
      b[5440] = x;
    }
    {
      double x = b[5408];
      x = fma(-CHEM_LDLU(lu + 21664), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22432), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23520), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 25408), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26976), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27936), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28928), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30656), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32480), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34112), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36384), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39424), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42144), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44864), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48288), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51808), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 56000), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60160), b[6016], x);
      b[5408] = x;
    }
    {
      double x = b[5376];
      x = fma(-CHEM_LDLU(lu + 28896), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 51776), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55968), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60128), b[6016], x);
      b[5376] = x;
    }
    {
      double x = b[5344];
      x = fma(-CHEM_LDLU(lu + 28864), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 36352), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 51744), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55936), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60096), b[6016], x);
      b[5344] = x;
    }
    {
      double x = b[5312];
      x = fma(-CHEM_LDLU(lu + 19008), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20352), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21632), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22400), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23488), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24448), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25376), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26944), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27904), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28832), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30624), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32448), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34080), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36320), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39392), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42112), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44832), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48256), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51712), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55904), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60064), b[6016], x);
      b[5312] = x;
    }
    {
      double x = b[5280];
      x = fma(-CHEM_LDLU(lu + 22368), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 25344), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26912), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 30592), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32416), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34048), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36288), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39360), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42080), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44800), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48224), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51680), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55872), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 60032), b[6016], x);
      b[5280] = x;
    }
    {
      double x = b[5248];
      x = fma(-CHEM_LDLU(lu + 28800), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 36256), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 51648), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 60000), b[6016], x);
      b[5248] = x;
    }
}
__device__ __noinline__ void solve_t_1_2(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[5216];
      x = fma(-CHEM_LDLU(lu + 27872), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30560), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32384), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 36224), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39328), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42048), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44768), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48192), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51616), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55840), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59968), b[6016], x);
      b[5216] = x;
    }
    {
      double x = b[5184];
      x = fma(-CHEM_LDLU(lu + 15648), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16448), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17088), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 18016), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18976), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19712), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20320), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21600), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22336), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23456), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24416), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25312), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26880), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27840), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28768), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30528), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32352), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34016), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36192), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39296), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42016), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44736), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48160), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51584), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55808), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59936), b[6016], x);
      b[5184] = x;
    }
    {
      double x = b[5152];
      x = fma(-CHEM_LDLU(lu + 22304), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 25280), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26848), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 30496), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32320), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33984), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36160), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39264), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41984), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44704), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48128), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51552), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55776), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59904), b[6016], x);
      b[5152] = x;
    }
    {
      double x = b[5120];
      x = fma(-CHEM_LDLU(lu + 15616), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 17056), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 18944), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 21568), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 23424), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 25248), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26816), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27808), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30464), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32288), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33952), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36128), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39232), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41952), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44672), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48096), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51520), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55744), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59872), b[6016], x);
      b[5120] = x;
    }
    {
      double x = b[5088];
      x = fma(-CHEM_LDLU(lu + 13568), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 14016), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15584), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16416), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17024), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17984), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18912), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20288), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21536), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22272), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23392), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24384), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25216), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26784), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27776), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30432), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32256), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33920), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36096), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39200), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41920), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44640), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48064), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51488), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55712), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59840), b[6016], x);
      b[5088] = x;
    }
    {
      double x = b[5056];
      x = fma(-CHEM_LDLU(lu + 25184), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 33888), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 55680), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59808), b[6016], x);
      b[5056] = x;
    }
    {
      double x = b[5024];
      x = fma(-CHEM_LDLU(lu + 51456), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 59776), b[6016], x);
      b[5024] = x;
    }
    {
      double x = b[4992];
      x = fma(-CHEM_LDLU(lu + 12224), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 13088), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13536), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13984), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15552), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16384), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 16992), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17952), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18880), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20256), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21504), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22240), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23360), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24352), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25152), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26752), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27744), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30400), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32224), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33856), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36064), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39168), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41888), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44608), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48032), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51424), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55648), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59744), b[6016], x);
      b[4992] = x;
    }
    {
      double x = b[4960];
      x = fma(-CHEM_LDLU(lu + 10912), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12192), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 13056), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13504), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13952), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15520), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16352), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 16960), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17920), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18848), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20224), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21472), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22208), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23328), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24320), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25120), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26720), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27712), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30368), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32192), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33824), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36032), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39136), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41856), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44576), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48000), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51392), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55616), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59712), b[6016], x);
      b[4960] = x;
    }
    {
      double x = b[4928];
      x = fma(-CHEM_LDLU(lu + 10336), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10880), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12160), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 13024), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13472), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13920), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15488), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16320), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 16928), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17888), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18816), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20192), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21440), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22176), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23296), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24288), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25088), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26688), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27680), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30336), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32160), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33792), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 36000), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39104), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41824), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44544), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47968), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51360), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55584), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59680), b[6016], x);
      b[4928] = x;
    }
    {
      double x = b[4896];
      x = fma(-CHEM_LDLU(lu + 9792), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10304), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10848), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12128), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 12992), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13440), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13888), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15456), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16288), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 16896), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17856), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18784), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20160), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21408), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22144), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23264), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24256), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25056), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26656), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27648), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30304), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32128), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33760), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35968), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39072), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41792), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44512), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47936), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51328), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55552), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59648), b[6016], x);
      b[4896] = x;
    }
    {
      double x = b[4864];
      x = fma(-CHEM_LDLU(lu + 9408), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9760), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10272), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10816), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12096), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 12960), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13408), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13856), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15424), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16256), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 16864), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17824), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18752), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20128), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21376), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22112), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23232), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24224), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25024), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26624), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27616), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30272), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32096), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33728), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35936), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39040), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41760), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44480), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47904), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51296), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55520), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59616), b[6016], x);
      b[4864] = x;
    }
    {
      double x = b[4832];
      x = fma(-CHEM_LDLU(lu + 9088), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9376), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9728), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10240), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10784), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12928), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13376), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13824), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15392), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16832), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17792), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18720), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20096), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21344), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22080), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23200), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24192), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 24992), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27584), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 32064), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33696), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 39008), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 44448), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47872), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51264), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55488), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59584), b[6016], x);
      b[4832] = x;
    }
    {
      double x = b[4800];
      x = fma(-CHEM_LDLU(lu + 15360), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 27552), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 30240), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35904), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38976), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41728), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44416), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47840), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51232), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55456), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59552), b[6016], x);
      b[4800] = x;
    }
    {
      double x = b[4768];
      x = fma(-CHEM_LDLU(lu + 13792), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 16800), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 20064), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 22048), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 24960), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27520), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 33664), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 44384), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 59520), b[6016], x);
      b[4768] = x;
    }
    {
      double x = b[4736];
      x = fma(-CHEM_LDLU(lu + 12064), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 14720), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15328), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16224), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 26592), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28736), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30208), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32032), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33632), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35872), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38944), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41696), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44352), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47808), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51200), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55424), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59488), b[6016], x);
      b[4736] = x;
    }
    {
      double x = b[4704];
      x = fma(-CHEM_LDLU(lu + 8288), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 8832), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 9056), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9344), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9696), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10208), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10752), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12896), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13344), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13760), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15296), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16768), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17760), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18688), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20032), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21312), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22016), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23168), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24160), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 24928), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27488), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 32000), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33600), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 38912), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 44320), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47776), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51168), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55392), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59456), b[6016], x);
      b[4704] = x;
    }
    {
      double x = b[4672];
      x = fma(-CHEM_LDLU(lu + 12032), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 18656), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 26560), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28704), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30176), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35840), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38880), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41664), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44288), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47744), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51136), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55360), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59424), b[6016], x);
      b[4672] = x;
    }
    {
      double x = b[4640];
      x = fma(-CHEM_LDLU(lu + 7744), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 8256), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 8800), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 9024), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9312), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9664), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10176), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10720), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12864), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13312), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13728), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15264), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16736), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17728), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18624), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20000), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21280), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 21984), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23136), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24128), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 24896), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27456), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 31968), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33568), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 38848), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 44256), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47712), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51104), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55328), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59392), b[6016], x);
      b[4640] = x;
    }
    {
      double x = b[4608];
      x = fma(-CHEM_LDLU(lu + 8224), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 8992), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9280), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9632), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 12832), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13696), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 15232), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16704), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17696), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 19968), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21248), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 21952), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 23104), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24864), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27424), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 31936), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33536), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 38816), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 44224), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47680), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51072), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55296), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59360), b[6016], x);
      b[4608] = x;
    }
    {
      double x = b[4576];
      x = fma(-CHEM_LDLU(lu + 8480), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 12800), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 14688), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15200), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 17664), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18592), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 21216), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 23072), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 31904), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33504), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35808), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38784), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41632), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44192), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47648), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51040), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55264), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59328), b[6016], x);
      b[4576] = x;
    }
    {
      double x = b[4544];
      x = fma(-CHEM_LDLU(lu + 8448), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 12768), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 14656), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15168), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 17632), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18560), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 21184), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 23040), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 31872), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33472), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 38752), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41600), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 47616), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 51008), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55232), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59296), b[6016], x);
      b[4544] = x;
    }
    {
      double x = b[4512];
      x = fma(-CHEM_LDLU(lu + 19680), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 23008), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 28672), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 44160), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 55200), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59264), b[6016], x);
      b[4512] = x;
    }
    {
      double x = b[4480];
      x = fma(-CHEM_LDLU(lu + 12000), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 26528), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 30144), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31840), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 35776), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38720), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41568), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44128), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47584), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50976), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55168), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59232), b[6016], x);
      b[4480] = x;
    }
    {
      double x = b[4448];
      x = fma(-CHEM_LDLU(lu + 21152), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 35744), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38688), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41536), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44096), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47552), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50944), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55136), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59200), b[6016], x);
      b[4448] = x;
    }
    {
      double x = b[4416];
      x = fma(-CHEM_LDLU(lu + 7136), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 7264), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 7712), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 8192), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 8768), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 8960), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9248), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9600), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10144), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10688), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12736), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13280), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13664), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 16672), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17600), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18528), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19936), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21920), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 24096), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 24832), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27392), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 31808), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33440), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 44064), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 59168), b[6016], x);
      b[4416] = x;
    }
    {
      double x = b[4384];
      x = fma(-CHEM_LDLU(lu + 6688), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 14624), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 18496), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 22976), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 33408), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 41504), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 47520), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50912), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 59136), b[6016], x);
      b[4384] = x;
    }
    {
      double x = b[4352];
      x = fma(-CHEM_LDLU(lu + 55104), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59104), b[6016], x);
      b[4352] = x;
    }
    {
      double x = b[4320];
      x = fma(-CHEM_LDLU(lu + 8416), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 14592), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15136), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16192), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 16640), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 19648), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 21888), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 28640), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 31776), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 41472), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 55072), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59072), b[6016], x);
      b[4320] = x;
    }
    {
      double x = b[4288];
      x = fma(-CHEM_LDLU(lu + 5120), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 5344), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 6080), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 6656), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6976), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 7520), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 8128), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11360), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 11968), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 12704), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 14560), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15104), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16160), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17568), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18464), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19616), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 21120), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22944), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 26496), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28608), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30112), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31744), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33376), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35712), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38656), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41440), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 44032), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47488), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50880), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55040), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 59040), b[6016], x);
      b[4288] = x;
    }
    {
      double x = b[4224];
      x = fma(-CHEM_LDLU(lu + 7104), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 7232), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 7680), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 8736), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 8928), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 9216), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9568), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10112), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10656), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12672), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13248), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13632), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 16608), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17536), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18432), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19904), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21856), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 24064), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 24800), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27360), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 31712), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33344), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 44000), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 59008), b[6016], x);
      b[4224] = x;
    }
    {
      double x = b[4192];
      x = fma(-CHEM_LDLU(lu + 4352), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 4608), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 5312), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 6048), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 6624), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6944), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 8096), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11936), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 12640), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 15072), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 17504), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 21088), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22912), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 26464), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 30080), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31680), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33312), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35680), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38624), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41408), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43968), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47456), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50848), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 55008), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58976), b[6016], x);
      b[4192] = x;
    }
    {
      double x = b[4160];
      x = fma(-CHEM_LDLU(lu + 4064), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 4320), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 4576), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 5280), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 6016), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 6592), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6912), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 8064), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11904), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 12608), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 15040), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 17472), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 21056), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22880), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 26432), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 30048), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31648), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33280), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35648), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38592), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41376), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43936), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47424), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50816), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54976), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58944), b[6016], x);
      b[4160] = x;
    }
    {
      double x = b[4128];
      x = fma(-CHEM_LDLU(lu + 5088), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 7488), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 11328), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 11872), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 14528), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15008), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16128), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 18400), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 26400), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28576), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 30016), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35616), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38560), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41344), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43904), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47392), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50784), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54944), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58912), b[6016], x);
      b[4128] = x;
    }
    {
      double x = b[4096];
      x = fma(-CHEM_LDLU(lu + 12576), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 14976), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 17440), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 21024), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22848), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 31616), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33248), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 38528), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 47360), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50752), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54912), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58880), b[6016], x);
      b[4096] = x;
    }
    {
      double x = b[4064];
      x = fma(-CHEM_LDLU(lu + 11840), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 20992), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22816), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 26368), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29984), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 33216), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35584), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38496), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41312), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43872), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47328), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50720), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54880), b[5984], x);
      b[4064] = x;
    }
    {
      double x = b[4032];
      x = fma(-CHEM_LDLU(lu + 3552), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 20960), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22784), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 33184), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35552), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38464), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41280), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43840), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47296), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50688), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54848), b[5984], x);
      b[4032] = x;
    }
    {
      double x = b[4000];
      x = fma(-CHEM_LDLU(lu + 54816), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58848), b[6016], x);
      b[4000] = x;
    }
    {
      double x = b[3968];
      x = fma(-CHEM_LDLU(lu + 4096), b[4224], x);
      x = fma(-CHEM_LDLU(lu + 7072), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 7200), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 7648), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 9184), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 9536), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 10624), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12544), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 13216), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 13600), b[5152], x);
      x = fma(-CHEM_LDLU(lu + 16576), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 17408), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 18368), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19872), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 21824), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 24032), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 24768), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27328), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 31584), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33152), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 43808), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 58816), b[6016], x);
      b[3968] = x;
    }
    {
      double x = b[3936];
      x = fma(-CHEM_LDLU(lu + 3872), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 4032), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 4288), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 4544), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 6560), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6880), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 8032), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11808), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 26336), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29952), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35520), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38432), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41248), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43776), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47264), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 54784), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58784), b[6016], x);
      b[3936] = x;
    }
    {
      double x = b[3904];
      x = fma(-CHEM_LDLU(lu + 12512), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 17376), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 20928), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22752), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 31552), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 38400), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 47232), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50656), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54752), b[5984], x);
      b[3904] = x;
    }
    {
      double x = b[3872];
      x = fma(-CHEM_LDLU(lu + 5056), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 11776), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 14496), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 14944), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16096), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 19584), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20896), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22720), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24736), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 26304), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28544), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29920), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31520), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33120), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35488), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38368), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41216), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43744), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47200), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50624), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54720), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58752), b[6016], x);
      b[3872] = x;
    }
}
__device__ __noinline__ void solve_t_1_3(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[3840];
      x = fma(-CHEM_LDLU(lu + 3840), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 4000), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 4256), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 4512), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 6528), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6848), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 8000), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11744), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 26272), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29888), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35456), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38336), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41184), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43712), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47168), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 54688), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58720), b[6016], x);
      b[3840] = x;
    }
    {
      double x = b[3808];
      x = fma(-CHEM_LDLU(lu + 14464), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 20864), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 31488), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 35424), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38304), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41152), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43680), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47136), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50592), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54656), b[5984], x);
      b[3808] = x;
    }
    {
      double x = b[3776];
      x = fma(-CHEM_LDLU(lu + 11712), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 14912), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16064), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 21792), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 26240), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29856), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31456), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33088), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35392), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38272), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41120), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43648), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47104), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50560), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54624), b[5984], x);
      b[3776] = x;
    }
    {
      double x = b[3744];
      x = fma(-CHEM_LDLU(lu + 3808), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 3968), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 4224), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 4480), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 6496), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6816), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 7968), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11680), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 26208), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29824), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35360), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38240), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41088), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43616), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47072), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 54592), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58688), b[6016], x);
      b[3744] = x;
    }
    {
      double x = b[3712];
      x = fma(-CHEM_LDLU(lu + 3776), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 3936), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 4192), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 4448), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 6464), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 6784), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 7936), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11648), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 26176), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29792), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35328), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38208), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 41056), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43584), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47040), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 54560), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58656), b[6016], x);
      b[3712] = x;
    }
    {
      double x = b[3680];
      x = fma(-CHEM_LDLU(lu + 14880), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 35296), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 41024), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 58624), b[6016], x);
      b[3680] = x;
    }
    {
      double x = b[3648];
      x = fma(-CHEM_LDLU(lu + 18336), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19552), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 31424), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 35264), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38176), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40992), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43552), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 47008), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50528), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54528), b[5984], x);
      b[3648] = x;
    }
    {
      double x = b[3584];
      x = fma(-CHEM_LDLU(lu + 2592), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 5024), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 7456), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 14432), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 16032), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 19520), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 21760), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 28512), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29760), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31392), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 54496), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58592), b[6016], x);
      b[3584] = x;
    }
    {
      double x = b[3552];
      x = fma(-CHEM_LDLU(lu + 7424), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 11296), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 11616), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 14400), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 14848), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 16000), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 18304), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19488), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 26144), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28480), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29728), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35232), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38144), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40960), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43520), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46976), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50496), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54464), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58560), b[6016], x);
      b[3552] = x;
    }
    {
      double x = b[3520];
      x = fma(-CHEM_LDLU(lu + 7392), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 11584), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 18272), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 26112), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29696), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35200), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38112), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40928), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43488), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46944), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50464), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54432), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58528), b[6016], x);
      b[3520] = x;
    }
    {
      double x = b[3488];
      x = fma(-CHEM_LDLU(lu + 5824), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 24000), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 26080), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29664), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35168), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38080), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40896), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43456), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46912), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50432), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54400), b[5984], x);
      b[3488] = x;
    }
    {
      double x = b[3456];
      x = fma(-CHEM_LDLU(lu + 4800), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 6368), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 8160), b[4768], x);
      x = fma(-CHEM_LDLU(lu + 10592), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12480), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 15968), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17344), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 19456), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 23968), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 26048), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29632), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35136), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38048), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40864), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43424), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46880), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50400), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54368), b[5984], x);
      b[3456] = x;
    }
    {
      double x = b[3424];
      x = fma(-CHEM_LDLU(lu + 4768), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 6336), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 8896), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 10080), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10560), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 15936), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17312), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 19424), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 23936), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 26016), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29600), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35104), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 38016), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40832), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43392), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46848), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50368), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54336), b[5984], x);
      b[3424] = x;
    }
    {
      double x = b[3392];
      x = fma(-CHEM_LDLU(lu + 4736), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 5792), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 6304), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 7168), b[4640], x);
      x = fma(-CHEM_LDLU(lu + 8864), b[4864], x);
      x = fma(-CHEM_LDLU(lu + 10528), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12448), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 15904), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17280), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 19392), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 25984), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29568), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 35072), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37984), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40800), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43360), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46816), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50336), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54304), b[5984], x);
      b[3392] = x;
    }
    {
      double x = b[3360];
      x = fma(-CHEM_LDLU(lu + 2080), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 4704), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 5760), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 6272), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 9152), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 17248), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 19360), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20832), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 25952), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29536), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31360), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 35040), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37952), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40768), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43328), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46784), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50304), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54272), b[5984], x);
      b[3360] = x;
    }
    {
      double x = b[3328];
      x = fma(-CHEM_LDLU(lu + 5984), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 11552), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 18240), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 20800), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22688), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24704), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 25920), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29504), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31328), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33056), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 35008), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37920), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40736), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43296), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46752), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50272), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54240), b[5984], x);
      b[3328] = x;
    }
    {
      double x = b[3296];
      x = fma(-CHEM_LDLU(lu + 5728), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 6240), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 9120), b[4896], x);
      x = fma(-CHEM_LDLU(lu + 15872), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 17216), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 19328), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20768), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 21728), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 25888), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29472), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31296), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34976), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37888), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40704), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43264), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46720), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50240), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54208), b[5984], x);
      b[3296] = x;
    }
    {
      double x = b[3264];
      x = fma(-CHEM_LDLU(lu + 4672), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 5696), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 6208), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 7040), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 9504), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 15840), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 19296), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20736), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 23904), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25856), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29440), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31264), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34944), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37856), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40672), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43232), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46688), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50208), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54176), b[5984], x);
      b[3264] = x;
    }
    {
      double x = b[3232];
      x = fma(-CHEM_LDLU(lu + 2368), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 2528), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 2848), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 11264), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 19264), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20704), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 31232), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34912), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37824), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40640), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43200), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46656), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50176), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54144), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58496), b[6016], x);
      b[3232] = x;
    }
    {
      double x = b[3200];
      x = fma(-CHEM_LDLU(lu + 5952), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 11520), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 16544), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 20672), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22656), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24672), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 25824), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29408), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31200), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 33024), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34880), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37792), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40608), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43168), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46624), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50144), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54112), b[5984], x);
      b[3200] = x;
    }
    {
      double x = b[3168];
      x = fma(-CHEM_LDLU(lu + 2048), b[3584], x);
      x = fma(-CHEM_LDLU(lu + 6176), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 14368), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 20640), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 21696), b[5472], x);
      x = fma(-CHEM_LDLU(lu + 31168), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 32992), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 37760), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 43136), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46592), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50112), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54080), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58464), b[6016], x);
      b[3168] = x;
    }
    {
      double x = b[3136];
      x = fma(-CHEM_LDLU(lu + 1440), b[3168], x);
      x = fma(-CHEM_LDLU(lu + 1504), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 1632), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 1824), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 2016), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 2336), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 2496), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 2816), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 2944), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 3200), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 3360), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 3520), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 4992), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 5664), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 5920), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 7904), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 11232), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 13184), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 14336), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 16512), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 18208), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19232), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 19840), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 20608), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 24640), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 25792), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 27296), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28448), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29376), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31136), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 32960), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34848), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37728), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40576), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43104), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46560), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50080), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54048), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58432), b[6016], x);
      b[3136] = x;
    }
    {
      double x = b[3104];
      x = fma(-CHEM_LDLU(lu + 4640), b[4320], x);
      x = fma(-CHEM_LDLU(lu + 5632), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 6144), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 7008), b[4608], x);
      x = fma(-CHEM_LDLU(lu + 9472), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 15808), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 19200), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20576), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 23872), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 25760), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29344), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31104), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34816), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37696), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40544), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43072), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46528), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50048), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 54016), b[5984], x);
      b[3104] = x;
    }
    {
      double x = b[3072];
      x = fma(-CHEM_LDLU(lu + 19168), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 20544), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 31072), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34784), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37664), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40512), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43040), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46496), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 50016), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53984), b[5984], x);
      b[3072] = x;
    }
    {
      double x = b[3040];
      x = fma(-CHEM_LDLU(lu + 2784), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 31040), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34752), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37632), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40480), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 43008), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46464), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49984), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53952), b[5984], x);
      b[3040] = x;
    }
    {
      double x = b[3008];
      x = fma(-CHEM_LDLU(lu + 25728), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29312), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 31008), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 32928), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34720), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37600), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40448), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42976), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46432), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49952), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53920), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58400), b[6016], x);
      b[3008] = x;
    }
    {
      double x = b[2976];
      x = fma(-CHEM_LDLU(lu + 19136), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 30976), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34688), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37568), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40416), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42944), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46400), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49920), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53888), b[5984], x);
      b[2976] = x;
    }
    {
      double x = b[2944];
      x = fma(-CHEM_LDLU(lu + 1344), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 1600), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 2304), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 2464), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 2752), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 11200), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 49888), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53856), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58368), b[6016], x);
      b[2944] = x;
    }
    {
      double x = b[2912];
      x = fma(-CHEM_LDLU(lu + 11488), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 15776), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 19104), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 22624), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 25696), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 28416), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29280), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 30944), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 32896), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34656), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37536), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40384), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42912), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46368), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49856), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53824), b[5984], x);
      b[2912] = x;
    }
    {
      double x = b[2880];
      x = fma(-CHEM_LDLU(lu + 11456), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 14816), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 15744), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 25664), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29248), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 30912), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 32864), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34624), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37504), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40352), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42880), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46336), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49824), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53792), b[5984], x);
      b[2880] = x;
    }
    {
      double x = b[2848];
      x = fma(-CHEM_LDLU(lu + 11424), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 25632), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 29216), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 30880), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 34592), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37472), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40320), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42848), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46304), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49792), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53760), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58336), b[6016], x);
      b[2848] = x;
    }
    {
      double x = b[2816];
      x = fma(-CHEM_LDLU(lu + 40288), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42816), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 58304), b[6016], x);
      b[2816] = x;
    }
    {
      double x = b[2784];
      x = fma(-CHEM_LDLU(lu + 11168), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 11392), b[5056], x);
      x = fma(-CHEM_LDLU(lu + 28384), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 40256), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 46272), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 53728), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58272), b[6016], x);
      b[2784] = x;
    }
    {
      double x = b[2752];
      x = fma(-CHEM_LDLU(lu + 1312), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 1472), b[3200], x);
      x = fma(-CHEM_LDLU(lu + 1568), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 1792), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 2272), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 2432), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 2720), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 3168), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 3328), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 3488), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 4960), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 5600), b[4448], x);
      x = fma(-CHEM_LDLU(lu + 5888), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 11136), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 13152), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 14304), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 16480), b[5280], x);
      x = fma(-CHEM_LDLU(lu + 18176), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19808), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 24608), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27264), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28352), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29184), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32832), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 40224), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42784), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 49760), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53696), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58240), b[6016], x);
      b[2752] = x;
    }
    {
      double x = b[2688];
      x = fma(-CHEM_LDLU(lu + 20512), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 46240), b[5920], x);
      b[2688] = x;
    }
    {
      double x = b[2656];
      x = fma(-CHEM_LDLU(lu + 5248), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 6752), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 20480), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 25600), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 34560), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37440), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40192), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42752), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46208), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49728), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53664), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58208), b[6016], x);
      b[2656] = x;
    }
    {
      double x = b[2624];
      x = fma(-CHEM_LDLU(lu + 5216), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 6432), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 20448), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22592), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 25568), b[5600], x);
      x = fma(-CHEM_LDLU(lu + 32800), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34528), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37408), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40160), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42720), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46176), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49696), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53632), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58176), b[6016], x);
      b[2624] = x;
    }
    {
      double x = b[2592];
      x = fma(-CHEM_LDLU(lu + 992), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 34496), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37376), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40128), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42688), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 46144), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49664), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53600), b[5984], x);
      b[2592] = x;
    }
    {
      double x = b[2560];
      x = fma(-CHEM_LDLU(lu + 3616), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 4160), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 5184), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 37344), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 46112), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 53568), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58144), b[6016], x);
      b[2560] = x;
    }
    {
      double x = b[2528];
      x = fma(-CHEM_LDLU(lu + 5568), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8704), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 37312), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 46080), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49632), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53536), b[5984], x);
      b[2528] = x;
    }
    {
      double x = b[2496];
      x = fma(-CHEM_LDLU(lu + 5536), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8672), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 10048), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 37280), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 46048), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49600), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53504), b[5984], x);
      b[2496] = x;
    }
    {
      double x = b[2464];
      x = fma(-CHEM_LDLU(lu + 5504), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 7616), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 8640), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 10016), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 37248), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 46016), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49568), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53472), b[5984], x);
      b[2464] = x;
    }
    {
      double x = b[2432];
      x = fma(-CHEM_LDLU(lu + 5472), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 7584), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 9984), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 12416), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 37216), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45984), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49536), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53440), b[5984], x);
      b[2432] = x;
    }
    {
      double x = b[2400];
      x = fma(-CHEM_LDLU(lu + 9952), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10496), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12384), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 23840), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 37184), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45952), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49504), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53408), b[5984], x);
      b[2400] = x;
    }
    {
      double x = b[2368];
      x = fma(-CHEM_LDLU(lu + 10464), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12352), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 17184), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 23808), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 37152), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45920), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49472), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53376), b[5984], x);
      b[2368] = x;
    }
    {
      double x = b[2336];
      x = fma(-CHEM_LDLU(lu + 14272), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 37120), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45888), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49440), b[5952], x);
      b[2336] = x;
    }
    {
      double x = b[2304];
      x = fma(-CHEM_LDLU(lu + 9920), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10432), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 23776), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 37088), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45856), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49408), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53344), b[5984], x);
      b[2304] = x;
    }
    {
      double x = b[2272];
      x = fma(-CHEM_LDLU(lu + 960), b[2688], x);
      x = fma(-CHEM_LDLU(lu + 34464), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 37056), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40096), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42656), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 45824), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49376), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53312), b[5984], x);
      b[2272] = x;
    }
    {
      double x = b[2240];
      x = fma(-CHEM_LDLU(lu + 1248), b[3008], x);
      x = fma(-CHEM_LDLU(lu + 3296), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 3456), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 4928), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 14240), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 28320), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 40064), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 49344), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53280), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58112), b[6016], x);
      b[2240] = x;
    }
    {
      double x = b[2208];
      x = fma(-CHEM_LDLU(lu + 11104), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 28288), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 40032), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45792), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 53248), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 58080), b[6016], x);
      b[2208] = x;
    }
    {
      double x = b[2176];
      x = fma(-CHEM_LDLU(lu + 2240), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 19776), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 58048), b[6016], x);
      b[2176] = x;
    }
    {
      double x = b[2144];
      x = fma(-CHEM_LDLU(lu + 12320), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 17152), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 20416), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 22560), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 37024), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45760), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49312), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53216), b[5984], x);
      b[2144] = x;
    }
    {
      double x = b[2112];
      x = fma(-CHEM_LDLU(lu + 8608), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 36992), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45728), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49280), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53184), b[5984], x);
      b[2112] = x;
    }
    {
      double x = b[2080];
      x = fma(-CHEM_LDLU(lu + 5440), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8576), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 36960), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45696), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49248), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53152), b[5984], x);
      b[2080] = x;
    }
    {
      double x = b[2048];
      x = fma(-CHEM_LDLU(lu + 5408), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 8544), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 9888), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 36928), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45664), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49216), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53120), b[5984], x);
      b[2048] = x;
    }
    {
      double x = b[2016];
      x = fma(-CHEM_LDLU(lu + 5376), b[4416], x);
      x = fma(-CHEM_LDLU(lu + 7552), b[4704], x);
      x = fma(-CHEM_LDLU(lu + 9856), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 36896), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45632), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49184), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53088), b[5984], x);
      b[2016] = x;
    }
    {
      double x = b[1984];
      x = fma(-CHEM_LDLU(lu + 9824), b[4960], x);
      x = fma(-CHEM_LDLU(lu + 10400), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12288), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 36864), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45600), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49152), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53056), b[5984], x);
      b[1984] = x;
    }
    {
      double x = b[1952];
      x = fma(-CHEM_LDLU(lu + 10368), b[4992], x);
      x = fma(-CHEM_LDLU(lu + 12256), b[5088], x);
      x = fma(-CHEM_LDLU(lu + 23744), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 36832), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45568), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49120), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 53024), b[5984], x);
      b[1952] = x;
    }
    {
      double x = b[1920];
      x = fma(-CHEM_LDLU(lu + 9440), b[4928], x);
      x = fma(-CHEM_LDLU(lu + 23712), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 36800), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 45536), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49088), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 52992), b[5984], x);
      b[1920] = x;
    }
    {
      double x = b[1888];
      x = fma(-CHEM_LDLU(lu + 27232), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 58016), b[6016], x);
      b[1888] = x;
    }
    {
      double x = b[1856];
      x = fma(-CHEM_LDLU(lu + 6112), b[4512], x);
      x = fma(-CHEM_LDLU(lu + 20384), b[5440], x);
      x = fma(-CHEM_LDLU(lu + 30848), b[5728], x);
      x = fma(-CHEM_LDLU(lu + 36768), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 42624), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 45504), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52960), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57984), b[6016], x);
      b[1856] = x;
    }
    {
      double x = b[1824];
      x = fma(-CHEM_LDLU(lu + 7360), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 18144), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 45472), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 49056), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57952), b[6016], x);
      b[1824] = x;
    }
    {
      double x = b[1792];
      x = fma(-CHEM_LDLU(lu + 7328), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 57920), b[6016], x);
      b[1792] = x;
    }
    {
      double x = b[1760];
      x = fma(-CHEM_LDLU(lu + 2688), b[3808], x);
      x = fma(-CHEM_LDLU(lu + 11072), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 49024), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57888), b[6016], x);
      b[1760] = x;
    }
    {
      double x = b[1728];
      x = fma(-CHEM_LDLU(lu + 2560), b[3680], x);
      x = fma(-CHEM_LDLU(lu + 3584), b[4096], x);
      x = fma(-CHEM_LDLU(lu + 4128), b[4256], x);
      x = fma(-CHEM_LDLU(lu + 5152), b[4384], x);
      x = fma(-CHEM_LDLU(lu + 36736), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 40000), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45440), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52928), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57856), b[6016], x);
      b[1728] = x;
    }
    {
      double x = b[1696];
      x = fma(-CHEM_LDLU(lu + 18112), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 48992), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57824), b[6016], x);
      b[1696] = x;
    }
    {
      double x = b[1664];
      x = fma(-CHEM_LDLU(lu + 3712), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 7872), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 57792), b[6016], x);
      b[1664] = x;
    }
    {
      double x = b[1632];
      x = fma(-CHEM_LDLU(lu + 352), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 544), b[2208], x);
      x = fma(-CHEM_LDLU(lu + 1088), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 7840), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 36704), b[5824], x);
      x = fma(-CHEM_LDLU(lu + 39968), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45408), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52896), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57760), b[6016], x);
      b[1632] = x;
    }
}
__device__ __noinline__ void solve_t_1_4(double* __restrict__ ws, int rhs)
{
    const double* __restrict__ lu = ws + 111488;
    const double* __restrict__ vd = ws + 216608;
    double* __restrict__ b = ws + rhs * 32;
    (void)vd;
    {
      double x = b[1600];
      x = fma(-CHEM_LDLU(lu + 448), b[1920], x);
      x = fma(-CHEM_LDLU(lu + 608), b[2304], x);
      x = fma(-CHEM_LDLU(lu + 8512), b[4832], x);
      x = fma(-CHEM_LDLU(lu + 14208), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 23680), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 48960), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57728), b[6016], x);
      b[1600] = x;
    }
    {
      double x = b[1568];
      x = fma(-CHEM_LDLU(lu + 576), b[2240], x);
      x = fma(-CHEM_LDLU(lu + 1408), b[3136], x);
      x = fma(-CHEM_LDLU(lu + 1984), b[3552], x);
      x = fma(-CHEM_LDLU(lu + 2912), b[3872], x);
      x = fma(-CHEM_LDLU(lu + 3264), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 3424), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 14176), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 28256), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 39936), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 48928), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 52864), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57696), b[6016], x);
      b[1568] = x;
    }
    {
      double x = b[1536];
      x = fma(-CHEM_LDLU(lu + 8384), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 14784), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 39904), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45376), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 48896), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57664), b[6016], x);
      b[1536] = x;
    }
    {
      double x = b[1504];
      x = fma(-CHEM_LDLU(lu + 32768), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 52832), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57632), b[6016], x);
      b[1504] = x;
    }
    {
      double x = b[1472];
      x = fma(-CHEM_LDLU(lu + 24576), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 52800), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57600), b[6016], x);
      b[1472] = x;
    }
    {
      double x = b[1440];
      x = fma(-CHEM_LDLU(lu + 928), b[2656], x);
      x = fma(-CHEM_LDLU(lu + 2624), b[3712], x);
      x = fma(-CHEM_LDLU(lu + 3008), b[3936], x);
      x = fma(-CHEM_LDLU(lu + 3136), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 3904), b[4192], x);
      x = fma(-CHEM_LDLU(lu + 6720), b[4576], x);
      x = fma(-CHEM_LDLU(lu + 8352), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 14144), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 29152), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 34432), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39872), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 48864), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57568), b[6016], x);
      b[1440] = x;
    }
    {
      double x = b[1408];
      x = fma(-CHEM_LDLU(lu + 512), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 864), b[2560], x);
      x = fma(-CHEM_LDLU(lu + 896), b[2624], x);
      x = fma(-CHEM_LDLU(lu + 1120), b[2816], x);
      x = fma(-CHEM_LDLU(lu + 2656), b[3744], x);
      x = fma(-CHEM_LDLU(lu + 2880), b[3840], x);
      x = fma(-CHEM_LDLU(lu + 3104), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 3744), b[4160], x);
      x = fma(-CHEM_LDLU(lu + 4896), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 6400), b[4544], x);
      x = fma(-CHEM_LDLU(lu + 8320), b[4800], x);
      x = fma(-CHEM_LDLU(lu + 14112), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 22528), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 28224), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29120), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 39840), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 48832), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 52768), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57536), b[6016], x);
      b[1408] = x;
    }
    {
      double x = b[1376];
      x = fma(-CHEM_LDLU(lu + 57504), b[6016], x);
      b[1376] = x;
    }
    {
      double x = b[1344];
      x = fma(-CHEM_LDLU(lu + 256), b[1376], x);
      x = fma(-CHEM_LDLU(lu + 320), b[1664], x);
      x = fma(-CHEM_LDLU(lu + 3680), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 4416), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 7808), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 15712), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 19072), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 28192), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 34400), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 52736), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57472), b[6016], x);
      b[1344] = x;
    }
    {
      double x = b[1312];
      x = fma(-CHEM_LDLU(lu + 288), b[1632], x);
      x = fma(-CHEM_LDLU(lu + 1024), b[2752], x);
      x = fma(-CHEM_LDLU(lu + 1056), b[2784], x);
      x = fma(-CHEM_LDLU(lu + 3072), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 3648), b[4128], x);
      x = fma(-CHEM_LDLU(lu + 4384), b[4288], x);
      x = fma(-CHEM_LDLU(lu + 4864), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 7296), b[4672], x);
      x = fma(-CHEM_LDLU(lu + 7776), b[4736], x);
      x = fma(-CHEM_LDLU(lu + 14080), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 15680), b[5248], x);
      x = fma(-CHEM_LDLU(lu + 28160), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 34368), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39808), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42592), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 45344), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 48800), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 52704), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57440), b[6016], x);
      b[1312] = x;
    }
    {
      double x = b[1280];
      x = fma(-CHEM_LDLU(lu + 45312), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 52672), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57408), b[6016], x);
      b[1280] = x;
    }
    {
      double x = b[1248];
      x = fma(-CHEM_LDLU(lu + 384), b[1760], x);
      x = fma(-CHEM_LDLU(lu + 1280), b[3072], x);
      x = fma(-CHEM_LDLU(lu + 1536), b[3232], x);
      x = fma(-CHEM_LDLU(lu + 2208), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 2400), b[3648], x);
      x = fma(-CHEM_LDLU(lu + 11040), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 48768), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 52640), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57376), b[6016], x);
      b[1248] = x;
    }
    {
      double x = b[1216];
      x = fma(-CHEM_LDLU(lu + 224), b[1248], x);
      x = fma(-CHEM_LDLU(lu + 1760), b[3360], x);
      x = fma(-CHEM_LDLU(lu + 52608), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57344), b[6016], x);
      b[1216] = x;
    }
    {
      double x = b[1184];
      x = fma(-CHEM_LDLU(lu + 45280), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 57312), b[6016], x);
      b[1184] = x;
    }
    {
      double x = b[1152];
      x = fma(-CHEM_LDLU(lu + 416), b[1888], x);
      x = fma(-CHEM_LDLU(lu + 480), b[2176], x);
      x = fma(-CHEM_LDLU(lu + 1728), b[3328], x);
      x = fma(-CHEM_LDLU(lu + 3040), b[4000], x);
      x = fma(-CHEM_LDLU(lu + 3232), b[4032], x);
      x = fma(-CHEM_LDLU(lu + 3392), b[4064], x);
      x = fma(-CHEM_LDLU(lu + 5856), b[4480], x);
      x = fma(-CHEM_LDLU(lu + 14048), b[5184], x);
      x = fma(-CHEM_LDLU(lu + 18080), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 19744), b[5408], x);
      x = fma(-CHEM_LDLU(lu + 22496), b[5504], x);
      x = fma(-CHEM_LDLU(lu + 24544), b[5568], x);
      x = fma(-CHEM_LDLU(lu + 27200), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 28128), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 29088), b[5696], x);
      x = fma(-CHEM_LDLU(lu + 32736), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 34336), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39776), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 42560), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 48736), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 52576), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57280), b[6016], x);
      b[1152] = x;
    }
    {
      double x = b[1120];
      x = fma(-CHEM_LDLU(lu + 2176), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 13120), b[5120], x);
      x = fma(-CHEM_LDLU(lu + 57248), b[6016], x);
      b[1120] = x;
    }
    {
      double x = b[1088];
      x = fma(-CHEM_LDLU(lu + 14752), b[5216], x);
      x = fma(-CHEM_LDLU(lu + 34304), b[5792], x);
      x = fma(-CHEM_LDLU(lu + 39744), b[5856], x);
      x = fma(-CHEM_LDLU(lu + 45248), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 48704), b[5952], x);
      x = fma(-CHEM_LDLU(lu + 57216), b[6016], x);
      b[1088] = x;
    }
    {
      double x = b[1024];
      x = fma(-CHEM_LDLU(lu + 11008), b[5024], x);
      x = fma(-CHEM_LDLU(lu + 45216), b[5920], x);
      x = fma(-CHEM_LDLU(lu + 48672), b[5952], x);
      b[1024] = x;
    }
    {
      double x = b[992];
      x = fma(-CHEM_LDLU(lu + 1952), b[3488], x);
      x = fma(-CHEM_LDLU(lu + 57184), b[6016], x);
      b[992] = x;
    }
    {
      double x = b[928];
      x = fma(-CHEM_LDLU(lu + 42528), b[5888], x);
      x = fma(-CHEM_LDLU(lu + 57152), b[6016], x);
      b[928] = x;
    }
    {
      double x = b[896];
      x = fma(-CHEM_LDLU(lu + 1920), b[3456], x);
      x = fma(-CHEM_LDLU(lu + 23648), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 52544), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57120), b[6016], x);
      b[896] = x;
    }
    {
      double x = b[864];
      x = fma(-CHEM_LDLU(lu + 1888), b[3424], x);
      x = fma(-CHEM_LDLU(lu + 23616), b[5536], x);
      x = fma(-CHEM_LDLU(lu + 52512), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57088), b[6016], x);
      b[864] = x;
    }
    {
      double x = b[832];
      x = fma(-CHEM_LDLU(lu + 1856), b[3392], x);
      x = fma(-CHEM_LDLU(lu + 17120), b[5312], x);
      x = fma(-CHEM_LDLU(lu + 52480), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 57056), b[6016], x);
      b[832] = x;
    }
    {
      double x = b[800];
      x = fma(-CHEM_LDLU(lu + 2976), b[3904], x);
      x = fma(-CHEM_LDLU(lu + 57024), b[6016], x);
      b[800] = x;
    }
    {
      double x = b[768];
      x = fma(-CHEM_LDLU(lu + 832), b[2528], x);
      x = fma(-CHEM_LDLU(lu + 56992), b[6016], x);
      b[768] = x;
    }
    {
      double x = b[736];
      x = fma(-CHEM_LDLU(lu + 800), b[2496], x);
      x = fma(-CHEM_LDLU(lu + 56960), b[6016], x);
      b[736] = x;
    }
    {
      double x = b[704];
      x = fma(-CHEM_LDLU(lu + 768), b[2464], x);
      x = fma(-CHEM_LDLU(lu + 56928), b[6016], x);
      b[704] = x;
    }
    {
      double x = b[672];
      x = fma(-CHEM_LDLU(lu + 736), b[2432], x);
      x = fma(-CHEM_LDLU(lu + 56896), b[6016], x);
      b[672] = x;
    }
    {
      double x = b[640];
      x = fma(-CHEM_LDLU(lu + 704), b[2400], x);
      x = fma(-CHEM_LDLU(lu + 56864), b[6016], x);
      b[640] = x;
    }
    {
      double x = b[608];
      x = fma(-CHEM_LDLU(lu + 672), b[2368], x);
      x = fma(-CHEM_LDLU(lu + 56832), b[6016], x);
      b[608] = x;
    }
    {
      double x = b[576];
      x = fma(-CHEM_LDLU(lu + 640), b[2336], x);
      x = fma(-CHEM_LDLU(lu + 56800), b[6016], x);
      b[576] = x;
    }
    {
      double x = b[512];
      x = fma(-CHEM_LDLU(lu + 96), b[544], x);
      x = fma(-CHEM_LDLU(lu + 192), b[1056], x);
      b[512] = x;
    }
    {
      double x = b[448];
      x = fma(-CHEM_LDLU(lu + 18048), b[5344], x);
      x = fma(-CHEM_LDLU(lu + 32704), b[5760], x);
      x = fma(-CHEM_LDLU(lu + 52448), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 56768), b[6016], x);
      b[448] = x;
    }
    {
      double x = b[416];
      x = fma(-CHEM_LDLU(lu + 2144), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 27168), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 56736), b[6016], x);
      b[416] = x;
    }
    {
      double x = b[384];
      x = fma(-CHEM_LDLU(lu + 2112), b[3616], x);
      x = fma(-CHEM_LDLU(lu + 27136), b[5632], x);
      x = fma(-CHEM_LDLU(lu + 56704), b[6016], x);
      b[384] = x;
    }
    {
      double x = b[352];
      x = fma(-CHEM_LDLU(lu + 1216), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 1664), b[3264], x);
      x = fma(-CHEM_LDLU(lu + 52416), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 56672), b[6016], x);
      b[352] = x;
    }
    {
      double x = b[320];
      x = fma(-CHEM_LDLU(lu + 1184), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 1376), b[3104], x);
      x = fma(-CHEM_LDLU(lu + 52384), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 56640), b[6016], x);
      b[320] = x;
    }
    {
      double x = b[288];
      x = fma(-CHEM_LDLU(lu + 1152), b[2944], x);
      x = fma(-CHEM_LDLU(lu + 1696), b[3296], x);
      x = fma(-CHEM_LDLU(lu + 52352), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 56608), b[6016], x);
      b[288] = x;
    }
    {
      double x = b[256];
      x = fma(-CHEM_LDLU(lu + 4832), b[4352], x);
      x = fma(-CHEM_LDLU(lu + 19040), b[5376], x);
      x = fma(-CHEM_LDLU(lu + 28096), b[5664], x);
      x = fma(-CHEM_LDLU(lu + 52320), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 56576), b[6016], x);
      b[256] = x;
    }
    {
      double x = b[160];
      x = fma(-CHEM_LDLU(lu + 32), b[192], x);
      x = fma(-CHEM_LDLU(lu + 64), b[224], x);
      x = fma(-CHEM_LDLU(lu + 52288), b[5984], x);
      x = fma(-CHEM_LDLU(lu + 56544), b[6016], x);
      b[160] = x;
    }
    {
      double x = b[128];
      x = fma(-CHEM_LDLU(lu + 160), b[960], x);
      x = fma(-CHEM_LDLU(lu + 10976), b[5024], x);
      b[128] = x;
    }
    {
      double x = b[96];
      x = fma(-CHEM_LDLU(lu + 128), b[960], x);
      x = fma(-CHEM_LDLU(lu + 10944), b[5024], x);
      b[96] = x;
    }
}
}  // namespace mech_cracmm2
