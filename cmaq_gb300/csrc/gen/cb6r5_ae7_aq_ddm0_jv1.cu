// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void ddm_jv_0_4(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[40928] * fma(y[896], v[4544], y[4544] * v[896]);
      out[4544] = out[4544] - dr;
      out[896] = out[896] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[3392] = fma(1.0, dr, out[3392]);
      out[4576] = fma(0.97, dr, out[4576]);
      out[4288] = fma(0.03, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40960] * fma(y[832], v[4544], y[4544] * v[832]);
      out[4544] = out[4544] - dr;
      out[832] = out[832] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4128] = fma(0.991, dr, out[4128]);
      out[4576] = fma(0.991, dr, out[4576]);
      out[4288] = fma(0.009, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40992] * fma(y[2656], v[4544], y[4544] * v[2656]);
      out[4544] = out[4544] - dr;
      out[2656] = out[2656] - dr;
      out[3232] = fma(1.0, dr, out[3232]);
      out[4352] = fma(2.0, dr, out[4352]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4512] = fma(1.0, dr, out[4512]);
    }
    {
      const double dr = ws[41024] * fma(y[3552], v[4544], y[4544] * v[3552]);
      out[4544] = out[4544] - dr;
      out[3552] = out[3552] - dr;
      out[3232] = fma(1.0, dr, out[3232]);
      out[4128] = fma(0.33, dr, out[4128]);
      out[4064] = fma(0.67, dr, out[4064]);
      out[4352] = fma(2.0, dr, out[4352]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4224] = fma(-1.0, dr, out[4224]);
    }
    {
      const double dr = ws[41056] * fma(y[3136], v[4544], y[4544] * v[3136]);
      out[4544] = out[4544] - dr;
      out[3136] = out[3136] - dr;
      out[3968] = fma(0.3, dr, out[3968]);
      out[3232] = fma(0.7, dr, out[3232]);
      out[4128] = fma(0.45, dr, out[4128]);
      out[4064] = fma(0.55, dr, out[4064]);
      out[3552] = fma(0.3, dr, out[3552]);
      out[4224] = fma(0.3, dr, out[4224]);
      out[4352] = fma(1.7, dr, out[4352]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[41088] * fma(y[2528], v[4544], y[4544] * v[2528]);
      out[4544] = out[4544] - dr;
      out[2528] = out[2528] - dr;
      out[3232] = fma(1.0, dr, out[3232]);
      out[3872] = fma(1.0, dr, out[3872]);
      out[4576] = fma(0.96, dr, out[4576]);
      out[4288] = fma(0.04, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[41120] * fma(y[4512], v[4544], y[4544] * v[4512]);
      out[4544] = out[4544] - dr;
      out[4512] = out[4512] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[41152] * fma(y[4128], v[4544], y[4544] * v[4128]);
      out[4544] = out[4544] - dr;
      out[4128] = out[4128] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[41184] * fma(y[4064], v[4544], y[4544] * v[4064]);
      out[4544] = out[4544] - dr;
      out[4064] = out[4064] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4096] = fma(1.0, dr, out[4096]);
    }
    {
      const double dr = ws[41216] * fma(y[2720], v[4544], y[4544] * v[2720]);
      out[4544] = out[4544] - dr;
      out[2720] = out[2720] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4512] = fma(1.0, dr, out[4512]);
    }
    {
      const double dr = ws[41248] * fma(y[864], v[4544], y[4544] * v[864]);
      out[4544] = out[4544] - dr;
      out[864] = out[864] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4128] = fma(1.0, dr, out[4128]);
    }
    {
      const double dr = ws[41280] * fma(y[4736], v[3968], y[3968] * v[4736]);
      out[3968] = out[3968] - dr;
      out[4736] = out[4736] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[41312] * fma(y[1088], v[4544], y[4544] * v[1088]);
      out[4544] = out[4544] - dr;
      out[1088] = out[1088] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[3616] = fma(0.18, dr, out[3616]);
      out[3488] = fma(0.65, dr, out[3488]);
      out[4672] = fma(0.72, dr, out[4672]);
      out[3936] = fma(0.1, dr, out[3936]);
      out[4736] = fma(0.1, dr, out[4736]);
      out[4576] = fma(0.07, dr, out[4576]);
      out[4704] = fma(0.18, dr, out[4704]);
      out[2944] = fma(1.0, dr, out[2944]);
    }
    {
      const double dr = ws[41344] * fma(y[1120], v[4544], y[4544] * v[1120]);
      out[4544] = out[4544] - dr;
      out[1120] = out[1120] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[3616] = fma(0.155, dr, out[3616]);
      out[3584] = fma(0.544, dr, out[3584]);
      out[4672] = fma(0.602, dr, out[4672]);
      out[3808] = fma(0.244, dr, out[3808]);
      out[4736] = fma(0.244, dr, out[4736]);
      out[4576] = fma(0.058, dr, out[4576]);
      out[4704] = fma(0.155, dr, out[4704]);
      out[2496] = fma(1.0, dr, out[2496]);
    }
    {
      const double dr = ws[41376] * fma(y[1152], v[4544], y[4544] * v[1152]);
      out[4544] = out[4544] - dr;
      out[1152] = out[1152] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[3616] = fma(0.155, dr, out[3616]);
      out[3584] = fma(0.544, dr, out[3584]);
      out[4672] = fma(0.602, dr, out[4672]);
      out[3808] = fma(0.244, dr, out[3808]);
      out[4736] = fma(0.244, dr, out[4736]);
      out[4576] = fma(0.058, dr, out[4576]);
      out[4704] = fma(0.155, dr, out[4704]);
      out[2560] = fma(1.0, dr, out[2560]);
    }
    {
      const double dr = ws[41408] * v[2592];
      out[2592] = out[2592] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[41440] * fma(y[4608], v[3520], y[3520] * v[4608]);
      out[3520] = out[3520] - dr;
      out[4608] = out[4608] - dr;
      out[1216] = fma(1.0, dr, out[1216]);
    }
    {
      const double dr = ws[41472] * v[1216];
      out[1216] = out[1216] - dr;
      out[3520] = fma(1.0, dr, out[3520]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[41504] * v[1216];
      out[1216] = out[1216] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[41536] * v[1216];
      out[1216] = out[1216] - dr;
      out[1824] = fma(1.0, dr, out[1824]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[41568] * v[1216];
      out[1216] = out[1216] - dr;
      out[1824] = fma(1.0, dr, out[1824]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[41600] * fma(y[4384], v[2944], y[2944] * v[4384]);
      out[2944] = out[2944] - dr;
      out[4384] = out[4384] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[3264] = fma(0.016, dr, out[3264]);
      out[2624] = fma(0.051, dr, out[2624]);
      out[3072] = fma(0.047, dr, out[3072]);
    }
    {
      const double dr = ws[41632] * fma(y[4704], v[2944], y[2944] * v[4704]);
      out[2944] = out[2944] - dr;
      out[4704] = out[4704] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[2240] = fma(0.14, dr, out[2240]);
    }
    {
      const double dr = ws[41664] * fma(y[4384], v[2496], y[2496] * v[4384]);
      out[2496] = out[2496] - dr;
      out[4384] = out[4384] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[3264] = fma(0.015, dr, out[3264]);
      out[2624] = fma(0.023, dr, out[2624]);
      out[3072] = fma(0.06, dr, out[3072]);
    }
    {
      const double dr = ws[41696] * fma(y[4704], v[2496], y[2496] * v[4704]);
      out[2496] = out[2496] - dr;
      out[4704] = out[4704] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[2240] = fma(0.193, dr, out[2240]);
    }
    {
      const double dr = ws[41728] * fma(y[4384], v[2144], y[2144] * v[4384]);
      out[2144] = out[2144] - dr;
      out[4384] = out[4384] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[3264] = fma(0.034, dr, out[3264]);
      out[3072] = fma(0.392, dr, out[3072]);
    }
    {
      const double dr = ws[41760] * fma(y[4704], v[2144], y[2144] * v[4704]);
      out[2144] = out[2144] - dr;
      out[4704] = out[4704] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[2240] = fma(0.146, dr, out[2240]);
    }
    {
      const double dr = ws[41792] * fma(y[4320], v[1856], y[1856] * v[4320]);
      out[1856] = out[1856] - dr;
      out[4320] = out[4320] - dr;
      out[4320] = fma(1.0, dr, out[4320]);
      out[1888] = fma(1.0, dr, out[1888]);
    }
    {
      const double dr = ws[41824] * fma(y[4736], v[1856], y[1856] * v[4736]);
      out[1856] = out[1856] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[1888] = fma(1.0, dr, out[1888]);
    }
    {
      const double dr = ws[41856] * fma(y[4640], v[1856], y[1856] * v[4640]);
      out[1856] = out[1856] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
      out[1888] = fma(1.0, dr, out[1888]);
    }
    {
      const double dr = ws[41888] * fma(y[4384], v[2560], y[2560] * v[4384]);
      out[2560] = out[2560] - dr;
      out[4384] = out[4384] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[3264] = fma(0.028, dr, out[3264]);
      out[2624] = fma(0.225, dr, out[2624]);
      out[3072] = fma(0.191, dr, out[3072]);
    }
    {
      const double dr = ws[41920] * fma(y[4704], v[2560], y[2560] * v[4704]);
      out[2560] = out[2560] - dr;
      out[4704] = out[4704] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[2240] = fma(0.473, dr, out[2240]);
    }
    {
      const double dr = ws[41952] * fma(y[4736], v[448], y[448] * v[4736]);
      out[448] = out[448] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3264] = fma(0.006, dr, out[3264]);
      out[2624] = fma(0.052, dr, out[2624]);
      out[3072] = fma(0.081, dr, out[3072]);
    }
    {
      const double dr = ws[41984] * v[4032];
      out[4032] = out[4032] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[42016] * v[1280];
      out[1280] = out[1280] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[1920] = fma(1.0, dr, out[1920]);
    }
    {
      const double dr = ws[42048] * v[1280];
      out[1280] = out[1280] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[1248] = fma(1.0, dr, out[1248]);
    }
    {
      const double dr = ws[42080] * v[1920];
      out[1920] = out[1920] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[42112] * v[1248];
      out[1248] = out[1248] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[42144] * fma(y[480], v[1920], y[1920] * v[480]);
      out[1920] = out[1920] - dr;
      out[480] = out[480] - dr;
      out[2592] = fma(1.0, dr, out[2592]);
    }
    {
      const double dr = ws[42176] * fma(y[512], v[1920], y[1920] * v[512]);
      out[1920] = out[1920] - dr;
      out[512] = out[512] - dr;
      out[2592] = fma(1.0, dr, out[2592]);
    }
    {
      const double dr = ws[42208] * fma(y[544], v[1248], y[1248] * v[544]);
      out[1248] = out[1248] - dr;
      out[544] = out[544] - dr;
      out[2592] = fma(1.0, dr, out[2592]);
    }
    {
      const double dr = ws[42240] * v[4608];
      out[4608] = out[4608] - dr;
      out[2464] = fma(0.5, dr, out[2464]);
      out[4192] = fma(0.5, dr, out[4192]);
    }
    {
      const double dr = ws[42272] * v[4320];
      out[4320] = out[4320] - dr;
    }
    {
      const double dr = ws[42304] * v[1056];
      out[1056] = out[1056] - dr;
      out[1312] = fma(1.0, dr, out[1312]);
    }
    {
      const double dr = ws[42336] * fma(y[576], v[1312], y[1312] * v[576]);
      out[1312] = out[1312] - dr;
      out[576] = out[576] - dr;
      out[608] = fma(1.0, dr, out[608]);
    }
    {
      const double dr = ws[42368] * v[1312];
      out[1312] = out[1312] - dr;
      out[608] = fma(1.0, dr, out[608]);
    }
    {
      const double dr = ws[42400] * v[4256];
      out[4256] = out[4256] - dr;
      out[640] = fma(1.0, dr, out[640]);
    }
    {
      const double dr = ws[42432] * v[4000];
      out[4000] = out[4000] - dr;
      out[640] = fma(1.0, dr, out[640]);
    }
    {
      const double dr = ws[42464] * fma(y[4384], v[2848], y[2848] * v[4384]);
      out[2848] = out[2848] - dr;
      out[4384] = out[4384] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[3360] = fma(0.688, dr, out[3360]);
    }
    {
      const double dr = ws[42496] * fma(y[4704], v[2848], y[2848] * v[4704]);
      out[2848] = out[2848] - dr;
      out[4704] = out[4704] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[3360] = fma(1.0, dr, out[3360]);
    }
    {
      const double dr = ws[42528] * fma(y[4640], v[2848], y[2848] * v[4640]);
      out[2848] = out[2848] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
      out[3360] = fma(0.422, dr, out[3360]);
    }
    {
      const double dr = ws[42560] * fma(y[4672], v[2848], y[2848] * v[4672]);
      out[2848] = out[2848] - dr;
      out[4672] = out[4672] - dr;
      out[4672] = fma(1.0, dr, out[4672]);
      out[3360] = fma(0.711, dr, out[3360]);
    }
    {
      const double dr = ws[42592] * fma(y[4544], v[3360], y[3360] * v[4544]);
      out[3360] = out[3360] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[3360] = fma(0.37, dr, out[3360]);
    }
    {
      const double dr = ws[42624] * fma(y[4736], v[3360], y[3360] * v[4736]);
      out[3360] = out[3360] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3360] = fma(0.24, dr, out[3360]);
    }
    {
      const double dr = ws[42656] * v[3360];
      out[3360] = out[3360] - dr;
    }
    {
      const double dr = ws[42688] * v[0];
      out[0] = out[0] - dr;
      out[32] = fma(1.0, dr, out[32]);
    }
    {
      const double dr = ws[42720] * v[64];
      out[64] = out[64] - dr;
      out[1376] = fma(0.907, dr, out[1376]);
    }
    {
      const double dr = ws[42752] * v[96];
      out[96] = out[96] - dr;
      out[1376] = fma(0.925, dr, out[1376]);
    }
    {
      const double dr = ws[42784] * v[128];
      out[128] = out[128] - dr;
      out[1376] = fma(0.943, dr, out[1376]);
    }
    {
      const double dr = ws[42816] * v[160];
      out[160] = out[160] - dr;
      out[1408] = fma(0.5, dr, out[1408]);
    }
    {
      const double dr = ws[42848] * v[192];
      out[192] = out[192] - dr;
      out[1408] = fma(0.5, dr, out[1408]);
    }
    {
      const double dr = ws[42880] * v[224];
      out[224] = out[224] - dr;
      out[1408] = fma(1.5, dr, out[1408]);
    }
    {
      const double dr = ws[42912] * fma(y[4736], v[704], y[704] * v[4736]);
      out[704] = out[704] - dr;
      out[4736] = out[4736] - dr;
      out[1440] = fma(1.25, dr, out[1440]);
      out[704] = fma(1.0, dr, out[704]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[42944] * fma(y[4736], v[1440], y[1440] * v[4736]);
      out[1440] = out[1440] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[42976] * fma(y[4736], v[736], y[736] * v[4736]);
      out[736] = out[736] - dr;
      out[4736] = out[4736] - dr;
      out[1472] = fma(1.25, dr, out[1472]);
      out[736] = fma(1.0, dr, out[736]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[43008] * fma(y[4736], v[1472], y[1472] * v[4736]);
      out[1472] = out[1472] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[43040] * fma(y[4736], v[768], y[768] * v[4736]);
      out[768] = out[768] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[800] = fma(1.0, dr, out[800]);
    }
    {
      const double dr = ws[43072] * fma(y[4736], v[2752], y[2752] * v[4736]);
      out[2752] = out[2752] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[2752] = fma(0.4857, dr, out[2752]);
      out[2784] = fma(0.0062, dr, out[2784]);
      out[2816] = fma(0.0025, dr, out[2816]);
      out[2304] = fma(0.0026, dr, out[2304]);
      out[1504] = fma(0.0023, dr, out[1504]);
      out[3680] = fma(0.2944, dr, out[3680]);
      out[3712] = fma(0.2021, dr, out[3712]);
      out[3168] = fma(0.0019, dr, out[3168]);
      out[3200] = fma(0.0023, dr, out[3200]);
    }
}
__device__ __noinline__ void ddm_jv_0_5(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[43104] * fma(y[4736], v[2784], y[2784] * v[4736]);
      out[2784] = out[2784] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[2752] = fma(0.3003, dr, out[2752]);
      out[2784] = fma(0.2862, dr, out[2784]);
      out[2816] = fma(0.0041, dr, out[2816]);
      out[2304] = fma(0.0035, dr, out[2304]);
      out[3680] = fma(0.2239, dr, out[3680]);
      out[3712] = fma(0.182, dr, out[3712]);
    }
    {
      const double dr = ws[43136] * fma(y[4736], v[2816], y[2816] * v[4736]);
      out[2816] = out[2816] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[2752] = fma(0.3856, dr, out[2752]);
      out[2784] = fma(0.095, dr, out[2784]);
      out[2816] = fma(0.1373, dr, out[2816]);
      out[2304] = fma(0.0005, dr, out[2304]);
      out[3680] = fma(0.2051, dr, out[3680]);
      out[3712] = fma(0.1764, dr, out[3712]);
    }
    {
      const double dr = ws[43168] * fma(y[4736], v[2304], y[2304] * v[4736]);
      out[2304] = out[2304] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[2752] = fma(0.2181, dr, out[2752]);
      out[2784] = fma(0.3063, dr, out[2784]);
      out[2816] = fma(0.0153, dr, out[2816]);
      out[2304] = fma(0.1043, dr, out[2304]);
      out[3680] = fma(0.1893, dr, out[3680]);
      out[3712] = fma(0.1668, dr, out[3712]);
    }
    {
      const double dr = ws[43200] * fma(y[4736], v[1504], y[1504] * v[4736]);
      out[1504] = out[1504] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[2752] = fma(0.2412, dr, out[2752]);
      out[2784] = fma(0.2089, dr, out[2784]);
      out[2816] = fma(0.3, dr, out[2816]);
      out[3680] = fma(0.2028, dr, out[3680]);
      out[3712] = fma(0.0471, dr, out[3712]);
    }
    {
      const double dr = ws[43232] * fma(y[4736], v[3680], y[3680] * v[4736]);
      out[3680] = out[3680] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3680] = fma(0.6664, dr, out[3680]);
      out[3712] = fma(0.0143, dr, out[3712]);
      out[2912] = fma(0.0123, dr, out[2912]);
      out[3168] = fma(0.1239, dr, out[3168]);
      out[3200] = fma(0.1831, dr, out[3200]);
    }
    {
      const double dr = ws[43264] * fma(y[4736], v[3712], y[3712] * v[4736]);
      out[3712] = out[3712] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3680] = fma(0.2858, dr, out[3680]);
      out[3712] = fma(0.3931, dr, out[3712]);
      out[2912] = fma(0.0139, dr, out[2912]);
      out[3168] = fma(0.1027, dr, out[3168]);
      out[3200] = fma(0.2045, dr, out[3200]);
    }
    {
      const double dr = ws[43296] * fma(y[4736], v[2912], y[2912] * v[4736]);
      out[2912] = out[2912] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3680] = fma(0.3303, dr, out[3680]);
      out[3712] = fma(0.2272, dr, out[3712]);
      out[2912] = fma(0.2607, dr, out[2912]);
      out[3168] = fma(0.0702, dr, out[3168]);
      out[3200] = fma(0.1116, dr, out[3200]);
    }
    {
      const double dr = ws[43328] * fma(y[4736], v[3168], y[3168] * v[4736]);
      out[3168] = out[3168] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3680] = fma(0.3444, dr, out[3680]);
      out[3712] = fma(0.2749, dr, out[3712]);
      out[2912] = fma(0.0491, dr, out[2912]);
      out[3168] = fma(0.2577, dr, out[3168]);
      out[3200] = fma(0.0739, dr, out[3200]);
    }
    {
      const double dr = ws[43360] * fma(y[4736], v[3200], y[3200] * v[4736]);
      out[3200] = out[3200] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3680] = fma(0.3886, dr, out[3680]);
      out[3712] = fma(0.2421, dr, out[3712]);
      out[2912] = fma(0.064, dr, out[2912]);
      out[3168] = fma(0.0385, dr, out[3168]);
      out[3200] = fma(0.2667, dr, out[3200]);
    }
    {
      const double dr = ws[43392] * fma(y[4736], v[2336], y[2336] * v[4736]);
      out[2336] = out[2336] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[43424] * fma(y[4640], v[2336], y[2336] * v[4640]);
      out[2336] = out[2336] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[43456] * fma(y[4160], v[2336], y[2336] * v[4160]);
      out[2336] = out[2336] - dr;
      out[4160] = out[4160] - dr;
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[43488] * v[2336];
      out[2336] = out[2336] - dr;
    }
    {
      const double dr = ws[43520] * v[2336];
      out[2336] = out[2336] - dr;
    }
    {
      const double dr = ws[43552] * fma(y[4544], v[2336], y[2336] * v[4544]);
      out[2336] = out[2336] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[43584] * fma(y[4736], v[2368], y[2368] * v[4736]);
      out[2368] = out[2368] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[43616] * fma(y[4640], v[2368], y[2368] * v[4640]);
      out[2368] = out[2368] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[43648] * fma(y[4160], v[2368], y[2368] * v[4160]);
      out[2368] = out[2368] - dr;
      out[4160] = out[4160] - dr;
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[43680] * v[2368];
      out[2368] = out[2368] - dr;
    }
    {
      const double dr = ws[43712] * fma(y[4544], v[2368], y[2368] * v[4544]);
      out[2368] = out[2368] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[43744] * fma(y[4736], v[2400], y[2400] * v[4736]);
      out[2400] = out[2400] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[2976] = fma(0.58, dr, out[2976]);
    }
    {
      const double dr = ws[43776] * fma(y[4320], v[2400], y[2400] * v[4320]);
      out[2400] = out[2400] - dr;
      out[4320] = out[4320] - dr;
      out[4320] = fma(1.0, dr, out[4320]);
      out[2976] = fma(0.52, dr, out[2976]);
    }
    {
      const double dr = ws[43808] * fma(y[4640], v[2400], y[2400] * v[4640]);
      out[2400] = out[2400] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
      out[2976] = fma(0.045, dr, out[2976]);
    }
    {
      const double dr = ws[43840] * fma(y[4544], v[2400], y[2400] * v[4544]);
      out[2400] = out[2400] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[2976] = fma(0.58, dr, out[2976]);
    }
    {
      const double dr = ws[43872] * fma(y[4736], v[2432], y[2432] * v[4736]);
      out[2432] = out[2432] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[43904] * fma(y[4320], v[2432], y[2432] * v[4320]);
      out[2432] = out[2432] - dr;
      out[4320] = out[4320] - dr;
      out[4320] = fma(1.0, dr, out[4320]);
    }
    {
      const double dr = ws[43936] * fma(y[4640], v[2432], y[2432] * v[4640]);
      out[2432] = out[2432] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[43968] * v[2432];
      out[2432] = out[2432] - dr;
    }
    {
      const double dr = ws[44000] * fma(y[4544], v[2432], y[2432] * v[4544]);
      out[2432] = out[2432] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[44032] * fma(y[4736], v[2976], y[2976] * v[4736]);
      out[2976] = out[2976] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[44064] * fma(y[4320], v[2976], y[2976] * v[4320]);
      out[2976] = out[2976] - dr;
      out[4320] = out[4320] - dr;
      out[4320] = fma(1.0, dr, out[4320]);
    }
    {
      const double dr = ws[44096] * fma(y[4640], v[2976], y[2976] * v[4640]);
      out[2976] = out[2976] - dr;
      out[4640] = out[4640] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[44128] * v[2976];
      out[2976] = out[2976] - dr;
    }
    {
      const double dr = ws[44160] * fma(y[4544], v[2976], y[2976] * v[4544]);
      out[2976] = out[2976] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[44192] * fma(y[4736], v[1536], y[1536] * v[4736]);
      out[1536] = out[1536] - dr;
      out[4736] = out[4736] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[44224] * fma(y[4544], v[1536], y[1536] * v[4544]);
      out[1536] = out[1536] - dr;
      out[4544] = out[4544] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[44256] * fma(y[4320], v[3008], y[3008] * v[4320]);
      out[3008] = out[3008] - dr;
      out[4320] = out[4320] - dr;
      out[1568] = fma(0.5, dr, out[1568]);
      out[3040] = fma(0.5, dr, out[3040]);
      out[4320] = fma(1.0, dr, out[4320]);
    }
    {
      const double dr = ws[44288] * fma(y[1184], v[3008], y[3008] * v[1184]);
      out[3008] = out[3008] - dr;
      out[1184] = out[1184] - dr;
      out[3040] = fma(1.0, dr, out[3040]);
      out[1184] = fma(1.0, dr, out[1184]);
    }
    {
      const double dr = ws[44320] * fma(y[3456], v[3008], y[3008] * v[3456]);
      out[3008] = out[3008] - dr;
      out[3456] = out[3456] - dr;
      out[3040] = fma(1.0, dr, out[3040]);
      out[3456] = fma(1.0, dr, out[3456]);
    }
    {
      const double dr = ws[44352] * fma(y[4736], v[3008], y[3008] * v[4736]);
      out[3008] = out[3008] - dr;
      out[4736] = out[4736] - dr;
      out[1568] = fma(0.5, dr, out[1568]);
      out[3040] = fma(0.5, dr, out[3040]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[44384] * fma(y[4544], v[3008], y[3008] * v[4544]);
      out[3008] = out[3008] - dr;
      out[4544] = out[4544] - dr;
      out[3008] = fma(0.5, dr, out[3008]);
      out[3040] = fma(0.5, dr, out[3040]);
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[44416] * fma(y[4736], v[2016], y[2016] * v[4736]);
      out[2016] = out[2016] - dr;
      out[4736] = out[4736] - dr;
      out[2208] = fma(1.0, dr, out[2208]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4512] = fma(1.0, dr, out[4512]);
    }
    {
      const double dr = ws[44448] * fma(y[4736], v[2016], y[2016] * v[4736]);
      out[2016] = out[2016] - dr;
      out[4736] = out[4736] - dr;
      out[2208] = fma(0.75, dr, out[2208]);
      out[1600] = fma(0.25, dr, out[1600]);
      out[4416] = fma(1.0, dr, out[4416]);
    }
    {
      const double dr = ws[44480] * fma(y[4640], v[2016], y[2016] * v[4640]);
      out[2016] = out[2016] - dr;
      out[4640] = out[4640] - dr;
      out[2208] = fma(1.0, dr, out[2208]);
      out[4192] = fma(1.0, dr, out[4192]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4512] = fma(1.0, dr, out[4512]);
    }
    {
      const double dr = ws[44512] * fma(y[4544], v[2016], y[2016] * v[4544]);
      out[2016] = out[2016] - dr;
      out[4544] = out[4544] - dr;
      out[2208] = fma(0.86, dr, out[2208]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4512] = fma(0.45, dr, out[4512]);
      out[3968] = fma(0.45, dr, out[3968]);
      out[1600] = fma(0.14, dr, out[1600]);
      out[3520] = fma(0.55, dr, out[3520]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
