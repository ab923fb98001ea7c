// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void ddm_src_0_4(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
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
    if (mask[251]) {
      const double q = scale * ws[52576];
      out[2592] = out[2592] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[252]) {
      const double q = scale * ws[52608];
      out[3520] = out[3520] - q;
      out[4608] = out[4608] - q;
      out[1216] = fma(1.0, q, out[1216]);
    }
    if (mask[253]) {
      const double q = scale * ws[52640];
      out[1216] = out[1216] - q;
      out[3520] = fma(1.0, q, out[3520]);
      out[4608] = fma(1.0, q, out[4608]);
    }
    if (mask[254]) {
      const double q = scale * ws[52672];
      out[1216] = out[1216] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[4640] = fma(1.0, q, out[4640]);
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
    if (mask[268]) {
      const double q = scale * ws[53120];
      out[448] = out[448] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3264] = fma(0.006, q, out[3264]);
      out[2624] = fma(0.052, q, out[2624]);
      out[3072] = fma(0.081, q, out[3072]);
    }
    if (mask[269]) {
      const double q = scale * ws[53152];
      out[4032] = out[4032] - q;
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[270]) {
      const double q = scale * ws[53184];
      out[1280] = out[1280] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[1920] = fma(1.0, q, out[1920]);
    }
    if (mask[271]) {
      const double q = scale * ws[53216];
      out[1280] = out[1280] - q;
      out[4192] = fma(1.0, q, out[4192]);
      out[1248] = fma(1.0, q, out[1248]);
    }
    if (mask[272]) {
      const double q = scale * ws[53248];
      out[1920] = out[1920] - q;
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[273]) {
      const double q = scale * ws[53280];
      out[1248] = out[1248] - q;
      out[4192] = fma(1.0, q, out[4192]);
    }
    if (mask[274]) {
      const double q = scale * ws[53312];
      out[1920] = out[1920] - q;
      out[480] = out[480] - q;
      out[2592] = fma(1.0, q, out[2592]);
    }
    if (mask[275]) {
      const double q = scale * ws[53344];
      out[1920] = out[1920] - q;
      out[512] = out[512] - q;
      out[2592] = fma(1.0, q, out[2592]);
    }
    if (mask[276]) {
      const double q = scale * ws[53376];
      out[1248] = out[1248] - q;
      out[544] = out[544] - q;
      out[2592] = fma(1.0, q, out[2592]);
    }
    if (mask[277]) {
      const double q = scale * ws[53408];
      out[4608] = out[4608] - q;
      out[2464] = fma(0.5, q, out[2464]);
      out[4192] = fma(0.5, q, out[4192]);
    }
    if (mask[278]) {
      const double q = scale * ws[53440];
      out[4320] = out[4320] - q;
    }
    if (mask[279]) {
      const double q = scale * ws[53472];
      out[1056] = out[1056] - q;
      out[1312] = fma(1.0, q, out[1312]);
    }
    if (mask[280]) {
      const double q = scale * ws[53504];
      out[1312] = out[1312] - q;
      out[576] = out[576] - q;
      out[608] = fma(1.0, q, out[608]);
    }
    if (mask[281]) {
      const double q = scale * ws[53536];
      out[1312] = out[1312] - q;
      out[608] = fma(1.0, q, out[608]);
    }
    if (mask[282]) {
      const double q = scale * ws[53568];
      out[4256] = out[4256] - q;
      out[640] = fma(1.0, q, out[640]);
    }
    if (mask[283]) {
      const double q = scale * ws[53600];
      out[4000] = out[4000] - q;
      out[640] = fma(1.0, q, out[640]);
    }
    if (mask[284]) {
      const double q = scale * ws[53632];
      out[2848] = out[2848] - q;
      out[4384] = out[4384] - q;
      out[4384] = fma(1.0, q, out[4384]);
      out[3360] = fma(0.688, q, out[3360]);
    }
    if (mask[285]) {
      const double q = scale * ws[53664];
      out[2848] = out[2848] - q;
      out[4704] = out[4704] - q;
      out[4704] = fma(1.0, q, out[4704]);
      out[3360] = fma(1.0, q, out[3360]);
    }
    if (mask[286]) {
      const double q = scale * ws[53696];
      out[2848] = out[2848] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
      out[3360] = fma(0.422, q, out[3360]);
    }
    if (mask[287]) {
      const double q = scale * ws[53728];
      out[2848] = out[2848] - q;
      out[4672] = out[4672] - q;
      out[4672] = fma(1.0, q, out[4672]);
      out[3360] = fma(0.711, q, out[3360]);
    }
    if (mask[288]) {
      const double q = scale * ws[53760];
      out[3360] = out[3360] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[3360] = fma(0.37, q, out[3360]);
    }
    if (mask[289]) {
      const double q = scale * ws[53792];
      out[3360] = out[3360] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3360] = fma(0.24, q, out[3360]);
    }
    if (mask[290]) {
      const double q = scale * ws[53824];
      out[3360] = out[3360] - q;
    }
    if (mask[291]) {
      const double q = scale * ws[53856];
      out[0] = out[0] - q;
      out[32] = fma(1.0, q, out[32]);
    }
    if (mask[292]) {
      const double q = scale * ws[53888];
      out[64] = out[64] - q;
      out[1376] = fma(0.907, q, out[1376]);
    }
    if (mask[293]) {
      const double q = scale * ws[53920];
      out[96] = out[96] - q;
      out[1376] = fma(0.925, q, out[1376]);
    }
    if (mask[294]) {
      const double q = scale * ws[53952];
      out[128] = out[128] - q;
      out[1376] = fma(0.943, q, out[1376]);
    }
    if (mask[295]) {
      const double q = scale * ws[53984];
      out[160] = out[160] - q;
      out[1408] = fma(0.5, q, out[1408]);
    }
    if (mask[296]) {
      const double q = scale * ws[54016];
      out[192] = out[192] - q;
      out[1408] = fma(0.5, q, out[1408]);
    }
    if (mask[297]) {
      const double q = scale * ws[54048];
      out[224] = out[224] - q;
      out[1408] = fma(1.5, q, out[1408]);
    }
    if (mask[298]) {
      const double q = scale * ws[54080];
      out[704] = out[704] - q;
      out[4736] = out[4736] - q;
      out[1440] = fma(1.25, q, out[1440]);
      out[704] = fma(1.0, q, out[704]);
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[299]) {
      const double q = scale * ws[54112];
      out[1440] = out[1440] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[300]) {
      const double q = scale * ws[54144];
      out[736] = out[736] - q;
      out[4736] = out[4736] - q;
      out[1472] = fma(1.25, q, out[1472]);
      out[736] = fma(1.0, q, out[736]);
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[301]) {
      const double q = scale * ws[54176];
      out[1472] = out[1472] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[302]) {
      const double q = scale * ws[54208];
      out[768] = out[768] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[800] = fma(1.0, q, out[800]);
    }
    if (mask[303]) {
      const double q = scale * ws[54240];
      out[2752] = out[2752] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[2752] = fma(0.4857, q, out[2752]);
      out[2784] = fma(0.0062, q, out[2784]);
      out[2816] = fma(0.0025, q, out[2816]);
      out[2304] = fma(0.0026, q, out[2304]);
      out[1504] = fma(0.0023, q, out[1504]);
      out[3680] = fma(0.2944, q, out[3680]);
      out[3712] = fma(0.2021, q, out[3712]);
      out[3168] = fma(0.0019, q, out[3168]);
      out[3200] = fma(0.0023, q, out[3200]);
    }
}
__device__ __noinline__ void ddm_src_0_5(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[304]) {
      const double q = scale * ws[54272];
      out[2784] = out[2784] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[2752] = fma(0.3003, q, out[2752]);
      out[2784] = fma(0.2862, q, out[2784]);
      out[2816] = fma(0.0041, q, out[2816]);
      out[2304] = fma(0.0035, q, out[2304]);
      out[3680] = fma(0.2239, q, out[3680]);
      out[3712] = fma(0.182, q, out[3712]);
    }
    if (mask[305]) {
      const double q = scale * ws[54304];
      out[2816] = out[2816] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[2752] = fma(0.3856, q, out[2752]);
      out[2784] = fma(0.095, q, out[2784]);
      out[2816] = fma(0.1373, q, out[2816]);
      out[2304] = fma(0.0005, q, out[2304]);
      out[3680] = fma(0.2051, q, out[3680]);
      out[3712] = fma(0.1764, q, out[3712]);
    }
    if (mask[306]) {
      const double q = scale * ws[54336];
      out[2304] = out[2304] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[2752] = fma(0.2181, q, out[2752]);
      out[2784] = fma(0.3063, q, out[2784]);
      out[2816] = fma(0.0153, q, out[2816]);
      out[2304] = fma(0.1043, q, out[2304]);
      out[3680] = fma(0.1893, q, out[3680]);
      out[3712] = fma(0.1668, q, out[3712]);
    }
    if (mask[307]) {
      const double q = scale * ws[54368];
      out[1504] = out[1504] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[2752] = fma(0.2412, q, out[2752]);
      out[2784] = fma(0.2089, q, out[2784]);
      out[2816] = fma(0.3, q, out[2816]);
      out[3680] = fma(0.2028, q, out[3680]);
      out[3712] = fma(0.0471, q, out[3712]);
    }
    if (mask[308]) {
      const double q = scale * ws[54400];
      out[3680] = out[3680] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3680] = fma(0.6664, q, out[3680]);
      out[3712] = fma(0.0143, q, out[3712]);
      out[2912] = fma(0.0123, q, out[2912]);
      out[3168] = fma(0.1239, q, out[3168]);
      out[3200] = fma(0.1831, q, out[3200]);
    }
    if (mask[309]) {
      const double q = scale * ws[54432];
      out[3712] = out[3712] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3680] = fma(0.2858, q, out[3680]);
      out[3712] = fma(0.3931, q, out[3712]);
      out[2912] = fma(0.0139, q, out[2912]);
      out[3168] = fma(0.1027, q, out[3168]);
      out[3200] = fma(0.2045, q, out[3200]);
    }
    if (mask[310]) {
      const double q = scale * ws[54464];
      out[2912] = out[2912] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3680] = fma(0.3303, q, out[3680]);
      out[3712] = fma(0.2272, q, out[3712]);
      out[2912] = fma(0.2607, q, out[2912]);
      out[3168] = fma(0.0702, q, out[3168]);
      out[3200] = fma(0.1116, q, out[3200]);
    }
    if (mask[311]) {
      const double q = scale * ws[54496];
      out[3168] = out[3168] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3680] = fma(0.3444, q, out[3680]);
      out[3712] = fma(0.2749, q, out[3712]);
      out[2912] = fma(0.0491, q, out[2912]);
      out[3168] = fma(0.2577, q, out[3168]);
      out[3200] = fma(0.0739, q, out[3200]);
    }
    if (mask[312]) {
      const double q = scale * ws[54528];
      out[3200] = out[3200] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[3680] = fma(0.3886, q, out[3680]);
      out[3712] = fma(0.2421, q, out[3712]);
      out[2912] = fma(0.064, q, out[2912]);
      out[3168] = fma(0.0385, q, out[3168]);
      out[3200] = fma(0.2667, q, out[3200]);
    }
    if (mask[313]) {
      const double q = scale * ws[54560];
      out[2336] = out[2336] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[314]) {
      const double q = scale * ws[54592];
      out[2336] = out[2336] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[315]) {
      const double q = scale * ws[54624];
      out[2336] = out[2336] - q;
      out[4160] = out[4160] - q;
      out[4160] = fma(1.0, q, out[4160]);
    }
    if (mask[316]) {
      const double q = scale * ws[54656];
      out[2336] = out[2336] - q;
    }
    if (mask[317]) {
      const double q = scale * ws[54688];
      out[2336] = out[2336] - q;
    }
    if (mask[318]) {
      const double q = scale * ws[54720];
      out[2336] = out[2336] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[319]) {
      const double q = scale * ws[54752];
      out[2368] = out[2368] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[320]) {
      const double q = scale * ws[54784];
      out[2368] = out[2368] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[321]) {
      const double q = scale * ws[54816];
      out[2368] = out[2368] - q;
      out[4160] = out[4160] - q;
      out[4160] = fma(1.0, q, out[4160]);
    }
    if (mask[322]) {
      const double q = scale * ws[54848];
      out[2368] = out[2368] - q;
    }
    if (mask[323]) {
      const double q = scale * ws[54880];
      out[2368] = out[2368] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[324]) {
      const double q = scale * ws[54912];
      out[2400] = out[2400] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
      out[2976] = fma(0.58, q, out[2976]);
    }
    if (mask[325]) {
      const double q = scale * ws[54944];
      out[2400] = out[2400] - q;
      out[4320] = out[4320] - q;
      out[4320] = fma(1.0, q, out[4320]);
      out[2976] = fma(0.52, q, out[2976]);
    }
    if (mask[326]) {
      const double q = scale * ws[54976];
      out[2400] = out[2400] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
      out[2976] = fma(0.045, q, out[2976]);
    }
    if (mask[327]) {
      const double q = scale * ws[55008];
      out[2400] = out[2400] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
      out[2976] = fma(0.58, q, out[2976]);
    }
    if (mask[328]) {
      const double q = scale * ws[55040];
      out[2432] = out[2432] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[329]) {
      const double q = scale * ws[55072];
      out[2432] = out[2432] - q;
      out[4320] = out[4320] - q;
      out[4320] = fma(1.0, q, out[4320]);
    }
    if (mask[330]) {
      const double q = scale * ws[55104];
      out[2432] = out[2432] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[331]) {
      const double q = scale * ws[55136];
      out[2432] = out[2432] - q;
    }
    if (mask[332]) {
      const double q = scale * ws[55168];
      out[2432] = out[2432] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[333]) {
      const double q = scale * ws[55200];
      out[2976] = out[2976] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[334]) {
      const double q = scale * ws[55232];
      out[2976] = out[2976] - q;
      out[4320] = out[4320] - q;
      out[4320] = fma(1.0, q, out[4320]);
    }
    if (mask[335]) {
      const double q = scale * ws[55264];
      out[2976] = out[2976] - q;
      out[4640] = out[4640] - q;
      out[4640] = fma(1.0, q, out[4640]);
    }
    if (mask[336]) {
      const double q = scale * ws[55296];
      out[2976] = out[2976] - q;
    }
    if (mask[337]) {
      const double q = scale * ws[55328];
      out[2976] = out[2976] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[338]) {
      const double q = scale * ws[55360];
      out[1536] = out[1536] - q;
      out[4736] = out[4736] - q;
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[339]) {
      const double q = scale * ws[55392];
      out[1536] = out[1536] - q;
      out[4544] = out[4544] - q;
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[340]) {
      const double q = scale * ws[55424];
      out[3008] = out[3008] - q;
      out[4320] = out[4320] - q;
      out[1568] = fma(0.5, q, out[1568]);
      out[3040] = fma(0.5, q, out[3040]);
      out[4320] = fma(1.0, q, out[4320]);
    }
    if (mask[341]) {
      const double q = scale * ws[55456];
      out[3008] = out[3008] - q;
      out[1184] = out[1184] - q;
      out[3040] = fma(1.0, q, out[3040]);
      out[1184] = fma(1.0, q, out[1184]);
    }
    if (mask[342]) {
      const double q = scale * ws[55488];
      out[3008] = out[3008] - q;
      out[3456] = out[3456] - q;
      out[3040] = fma(1.0, q, out[3040]);
      out[3456] = fma(1.0, q, out[3456]);
    }
    if (mask[343]) {
      const double q = scale * ws[55520];
      out[3008] = out[3008] - q;
      out[4736] = out[4736] - q;
      out[1568] = fma(0.5, q, out[1568]);
      out[3040] = fma(0.5, q, out[3040]);
      out[4736] = fma(1.0, q, out[4736]);
    }
    if (mask[344]) {
      const double q = scale * ws[55552];
      out[3008] = out[3008] - q;
      out[4544] = out[4544] - q;
      out[3008] = fma(0.5, q, out[3008]);
      out[3040] = fma(0.5, q, out[3040]);
      out[4544] = fma(1.0, q, out[4544]);
    }
    if (mask[345]) {
      const double q = scale * ws[55584];
      out[2016] = out[2016] - q;
      out[4736] = out[4736] - q;
      out[2208] = fma(1.0, q, out[2208]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4512] = fma(1.0, q, out[4512]);
    }
    if (mask[346]) {
      const double q = scale * ws[55616];
      out[2016] = out[2016] - q;
      out[4736] = out[4736] - q;
      out[2208] = fma(0.75, q, out[2208]);
      out[1600] = fma(0.25, q, out[1600]);
      out[4416] = fma(1.0, q, out[4416]);
    }
    if (mask[347]) {
      const double q = scale * ws[55648];
      out[2016] = out[2016] - q;
      out[4640] = out[4640] - q;
      out[2208] = fma(1.0, q, out[2208]);
      out[4192] = fma(1.0, q, out[4192]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4512] = fma(1.0, q, out[4512]);
    }
    if (mask[348]) {
      const double q = scale * ws[55680];
      out[2016] = out[2016] - q;
      out[4544] = out[4544] - q;
      out[2208] = fma(0.86, q, out[2208]);
      out[4416] = fma(1.0, q, out[4416]);
      out[4512] = fma(0.45, q, out[4512]);
      out[3968] = fma(0.45, q, out[3968]);
      out[1600] = fma(0.14, q, out[1600]);
      out[3520] = fma(0.55, q, out[3520]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
