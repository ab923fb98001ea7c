// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void ddm_src_1_4(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[276]) {
      const double q = scale * ws[68160];
      out[2624] = out[2624] - q;
      out[5888] = out[5888] - q;
      out[4384] = fma(0.341, q, out[4384]);
      out[5856] = fma(0.964, q, out[5856]);
      out[5600] = fma(0.043, q, out[5600]);
      out[5984] = fma(0.918, q, out[5984]);
      out[5920] = fma(0.659, q, out[5920]);
      out[4544] = fma(0.533, q, out[4544]);
      out[5504] = fma(0.007, q, out[5504]);
      out[5760] = fma(0.119, q, out[5760]);
    }
    if (mask[277]) {
      const double q = scale * ws[68192];
      out[3840] = out[3840] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.75, q, out[5984]);
      out[5920] = fma(0.75, q, out[5920]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5856] = fma(0.75, q, out[5856]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[278]) {
      const double q = scale * ws[68224];
      out[4192] = out[4192] - q;
      out[5888] = out[5888] - q;
      out[5600] = fma(0.25, q, out[5600]);
      out[4576] = fma(1.0, q, out[4576]);
      out[5856] = fma(1.03, q, out[5856]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[279]) {
      const double q = scale * ws[68256];
      out[3936] = out[3936] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(0.75, q, out[5856]);
      out[5600] = fma(0.25, q, out[5600]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[280]) {
      const double q = scale * ws[68288];
      out[2656] = out[2656] - q;
      out[5888] = out[5888] - q;
      out[4384] = fma(0.69, q, out[4384]);
      out[5856] = fma(0.91, q, out[5856]);
      out[5600] = fma(0.09, q, out[5600]);
      out[5984] = fma(1.01, q, out[5984]);
      out[4576] = fma(0.31, q, out[4576]);
      out[5920] = fma(0.31, q, out[5920]);
    }
    if (mask[281]) {
      const double q = scale * ws[68320];
      out[3712] = out[3712] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.75, q, out[5984]);
      out[5856] = fma(0.75, q, out[5856]);
      out[5920] = fma(0.75, q, out[5920]);
      out[5600] = fma(0.25, q, out[5600]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[282]) {
      const double q = scale * ws[68352];
      out[5792] = out[5792] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.9, q, out[5984]);
      out[5888] = fma(0.9, q, out[5888]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5696] = fma(0.1, q, out[5696]);
    }
    if (mask[283]) {
      const double q = scale * ws[68384];
      out[4800] = out[4800] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.9, q, out[5984]);
      out[5888] = fma(0.9, q, out[5888]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5696] = fma(0.1, q, out[5696]);
    }
    if (mask[284]) {
      const double q = scale * ws[68416];
      out[2848] = out[2848] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5792] = fma(0.5, q, out[5792]);
      out[5856] = fma(1.5, q, out[5856]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
      out[5696] = fma(0.125, q, out[5696]);
    }
    if (mask[285]) {
      const double q = scale * ws[68448];
      out[5152] = out[5152] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.834, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5472] = fma(0.334, q, out[5472]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
    }
    if (mask[286]) {
      const double q = scale * ws[68480];
      out[3776] = out[3776] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(0.75, q, out[5856]);
      out[5472] = fma(0.5, q, out[5472]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
    }
    if (mask[287]) {
      const double q = scale * ws[68512];
      out[4672] = out[4672] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5792] = fma(0.269, q, out[5792]);
      out[5664] = fma(0.5, q, out[5664]);
      out[5856] = fma(1.66, q, out[5856]);
      out[5696] = fma(0.067, q, out[5696]);
      out[5888] = fma(0.25, q, out[5888]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
    }
    if (mask[288]) {
      const double q = scale * ws[68544];
      out[3520] = out[3520] - q;
      out[5888] = out[5888] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.5, q, out[5856]);
      out[5344] = fma(0.5, q, out[5344]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
    }
    if (mask[289]) {
      const double q = scale * ws[68576];
      out[2880] = out[2880] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5792] = fma(1.16, q, out[5792]);
      out[5216] = fma(1.16, q, out[5216]);
      out[5856] = fma(1.5, q, out[5856]);
      out[5760] = fma(1.75, q, out[5760]);
      out[5248] = fma(0.5, q, out[5248]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
      out[5696] = fma(0.292, q, out[5696]);
    }
    if (mask[290]) {
      const double q = scale * ws[68608];
      out[2912] = out[2912] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5664] = fma(0.305, q, out[5664]);
      out[5856] = fma(0.773, q, out[5856]);
      out[5760] = fma(0.203, q, out[5760]);
      out[5504] = fma(0.525, q, out[5504]);
      out[5376] = fma(0.135, q, out[5376]);
      out[5248] = fma(0.105, q, out[5248]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
    }
    if (mask[291]) {
      const double q = scale * ws[68640];
      out[2592] = out[2592] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[2272] = fma(1.0, q, out[2272]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[292]) {
      const double q = scale * ws[68672];
      out[2272] = out[2272] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[2688] = fma(1.0, q, out[2688]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[293]) {
      const double q = scale * ws[68704];
      out[3648] = out[3648] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(2.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5344] = fma(0.32, q, out[5344]);
      out[5376] = fma(0.68, q, out[5376]);
      out[5728] = fma(0.68, q, out[5728]);
    }
    if (mask[294]) {
      const double q = scale * ws[68736];
      out[3040] = out[3040] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[3808] = fma(1.0, q, out[3808]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[295]) {
      const double q = scale * ws[68768];
      out[2976] = out[2976] - q;
      out[5888] = out[5888] - q;
      out[5856] = fma(1.0, q, out[5856]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5376] = fma(1.0, q, out[5376]);
    }
    if (mask[296]) {
      const double q = scale * ws[68800];
      out[4032] = out[4032] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(2.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[297]) {
      const double q = scale * ws[68832];
      out[4064] = out[4064] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5920] = fma(0.5, q, out[5920]);
      out[5856] = fma(0.965, q, out[5856]);
      out[5760] = fma(0.93, q, out[5760]);
      out[5504] = fma(0.348, q, out[5504]);
      out[5600] = fma(0.25, q, out[5600]);
      out[5056] = fma(0.25, q, out[5056]);
      out[5440] = fma(0.5, q, out[5440]);
    }
    if (mask[298]) {
      const double q = scale * ws[68864];
      out[3072] = out[3072] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(0.7, q, out[5920]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5376] = fma(0.7, q, out[5376]);
      out[5728] = fma(0.7, q, out[5728]);
      out[5440] = fma(0.3, q, out[5440]);
    }
    if (mask[299]) {
      const double q = scale * ws[68896];
      out[5216] = out[5216] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[300]) {
      const double q = scale * ws[68928];
      out[5632] = out[5632] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5568] = fma(1.0, q, out[5568]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[301]) {
      const double q = scale * ws[68960];
      out[5408] = out[5408] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.394, q, out[5984]);
      out[5888] = fma(0.58, q, out[5888]);
      out[5632] = fma(0.026, q, out[5632]);
      out[5216] = fma(0.026, q, out[5216]);
      out[5856] = fma(0.13, q, out[5856]);
      out[5760] = fma(0.273, q, out[5760]);
      out[5504] = fma(0.662, q, out[5504]);
      out[5376] = fma(0.067, q, out[5376]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[302]) {
      const double q = scale * ws[68992];
      out[5120] = out[5120] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.342, q, out[5984]);
      out[5888] = fma(0.518, q, out[5888]);
      out[5632] = fma(0.14, q, out[5632]);
      out[5216] = fma(0.191, q, out[5216]);
      out[5856] = fma(0.042, q, out[5856]);
      out[5760] = fma(0.381, q, out[5760]);
      out[5504] = fma(0.824, q, out[5504]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[303]) {
      const double q = scale * ws[69024];
      out[3008] = out[3008] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5856] = fma(1.6, q, out[5856]);
      out[5760] = fma(0.2, q, out[5760]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[304]) {
      const double q = scale * ws[69056];
      out[3200] = out[3200] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5760] = fma(0.94, q, out[5760]);
      out[5504] = fma(0.06, q, out[5504]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[305]) {
      const double q = scale * ws[69088];
      out[3328] = out[3328] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5760] = fma(1.71, q, out[5760]);
      out[5504] = fma(0.29, q, out[5504]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[306]) {
      const double q = scale * ws[69120];
      out[3360] = out[3360] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5696] = fma(0.3, q, out[5696]);
      out[4448] = fma(0.0, q, out[4448]);
      out[5376] = fma(1.0, q, out[5376]);
      out[4512] = fma(0.5, q, out[4512]);
      out[4320] = fma(0.25, q, out[4320]);
      out[3584] = fma(0.25, q, out[3584]);
    }
    if (mask[307]) {
      const double q = scale * ws[69152];
      out[3296] = out[3296] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5984] = fma(0.9146, q, out[5984]);
      out[5696] = fma(0.3, q, out[5696]);
      out[4448] = fma(0.0854, q, out[4448]);
      out[5376] = fma(0.5488, q, out[5376]);
      out[5248] = fma(0.3659, q, out[5248]);
      out[4512] = fma(0.3659, q, out[4512]);
      out[5472] = fma(0.5488, q, out[5472]);
    }
    if (mask[308]) {
      const double q = scale * ws[69184];
      out[3104] = out[3104] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5984] = fma(0.9518, q, out[5984]);
      out[5696] = fma(0.3, q, out[5696]);
      out[4448] = fma(0.0482, q, out[4448]);
      out[5376] = fma(0.7043, q, out[5376]);
      out[5248] = fma(0.2475, q, out[5248]);
      out[4512] = fma(0.3522, q, out[4512]);
      out[4320] = fma(0.5996, q, out[4320]);
    }
    if (mask[309]) {
      const double q = scale * ws[69216];
      out[3264] = out[3264] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5984] = fma(0.9146, q, out[5984]);
      out[5696] = fma(0.3, q, out[5696]);
      out[4448] = fma(0.0854, q, out[4448]);
      out[5376] = fma(0.5488, q, out[5376]);
      out[5248] = fma(0.3659, q, out[5248]);
      out[4512] = fma(0.4573, q, out[4512]);
      out[4320] = fma(0.4573, q, out[4320]);
    }
    if (mask[310]) {
      const double q = scale * ws[69248];
      out[4288] = out[4288] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5856] = fma(1.048, q, out[5856]);
      out[4128] = fma(0.219, q, out[4128]);
      out[4736] = fma(0.305, q, out[4736]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[311]) {
      const double q = scale * ws[69280];
      out[4160] = out[4160] - q;
      out[5792] = out[5792] - q;
      out[4544] = fma(0.2535, q, out[4544]);
      out[5760] = fma(0.371, q, out[5760]);
      out[4096] = fma(0.091, q, out[4096]);
      out[4480] = fma(0.1165, q, out[4480]);
      out[4576] = fma(0.1725, q, out[4576]);
      out[5856] = fma(0.403, q, out[5856]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
      out[5504] = fma(0.112, q, out[5504]);
    }
    if (mask[312]) {
      const double q = scale * ws[69312];
      out[3744] = out[3744] - q;
      out[5792] = out[5792] - q;
      out[6016] = fma(0.5, q, out[6016]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5696] = fma(0.5, q, out[5696]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[313]) {
      const double q = scale * ws[69344];
      out[2624] = out[2624] - q;
      out[5792] = out[5792] - q;
      out[5920] = fma(0.825, q, out[5920]);
      out[4544] = fma(0.65, q, out[4544]);
      out[5888] = fma(1.0, q, out[5888]);
      out[4384] = fma(0.175, q, out[4384]);
      out[5760] = fma(0.168, q, out[5760]);
      out[5504] = fma(0.007, q, out[5504]);
      out[5856] = fma(0.007, q, out[5856]);
      out[5984] = fma(0.175, q, out[5984]);
    }
    if (mask[314]) {
      const double q = scale * ws[69376];
      out[3840] = out[3840] - q;
      out[5792] = out[5792] - q;
      out[5920] = fma(0.5, q, out[5920]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5696] = fma(0.5, q, out[5696]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[315]) {
      const double q = scale * ws[69408];
      out[4192] = out[4192] - q;
      out[5792] = out[5792] - q;
      out[4576] = fma(1.0, q, out[4576]);
      out[5856] = fma(0.56, q, out[5856]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
    }
    if (mask[316]) {
      const double q = scale * ws[69440];
      out[3936] = out[3936] - q;
      out[5792] = out[5792] - q;
      out[6016] = fma(0.5, q, out[6016]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5696] = fma(0.5, q, out[5696]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[317]) {
      const double q = scale * ws[69472];
      out[2656] = out[2656] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5920] = fma(0.46, q, out[5920]);
      out[4576] = fma(0.46, q, out[4576]);
      out[4384] = fma(0.54, q, out[4384]);
      out[5984] = fma(0.54, q, out[5984]);
    }
    if (mask[318]) {
      const double q = scale * ws[69504];
      out[3712] = out[3712] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.5, q, out[5888]);
      out[5920] = fma(0.5, q, out[5920]);
      out[5696] = fma(0.5, q, out[5696]);
      out[4256] = fma(1.0, q, out[4256]);
    }
    if (mask[319]) {
      const double q = scale * ws[69536];
      out[5792] = out[5792] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(2.0, q, out[5888]);
    }
    if (mask[320]) {
      const double q = scale * ws[69568];
      out[4800] = out[4800] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5632] = fma(1.0, q, out[5632]);
    }
    if (mask[321]) {
      const double q = scale * ws[69600];
      out[2848] = out[2848] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.5, q, out[5888]);
      out[5792] = fma(0.5, q, out[5792]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5696] = fma(0.75, q, out[5696]);
    }
    if (mask[322]) {
      const double q = scale * ws[69632];
      out[5152] = out[5152] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.33, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5856] = fma(0.33, q, out[5856]);
      out[5472] = fma(0.334, q, out[5472]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[323]) {
      const double q = scale * ws[69664];
      out[3776] = out[3776] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5472] = fma(0.5, q, out[5472]);
      out[5696] = fma(0.5, q, out[5696]);
    }
}
__device__ __noinline__ void ddm_src_1_5(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[324]) {
      const double q = scale * ws[69696];
      out[4672] = out[4672] - q;
      out[5792] = out[5792] - q;
      out[5696] = fma(0.635, q, out[5696]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5792] = fma(0.269, q, out[5792]);
      out[5664] = fma(0.5, q, out[5664]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[325]) {
      const double q = scale * ws[69728];
      out[3520] = out[3520] - q;
      out[5792] = out[5792] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.5, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5344] = fma(0.5, q, out[5344]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[326]) {
      const double q = scale * ws[69760];
      out[2880] = out[2880] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5792] = fma(1.16, q, out[5792]);
      out[5216] = fma(1.16, q, out[5216]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5760] = fma(2.3, q, out[5760]);
      out[5248] = fma(0.5, q, out[5248]);
      out[5696] = fma(1.083, q, out[5696]);
    }
    if (mask[327]) {
      const double q = scale * ws[69792];
      out[2912] = out[2912] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5888] = fma(0.5, q, out[5888]);
      out[5664] = fma(0.5, q, out[5664]);
      out[5856] = fma(0.03, q, out[5856]);
      out[5760] = fma(0.27, q, out[5760]);
      out[5504] = fma(0.7, q, out[5504]);
      out[5376] = fma(0.18, q, out[5376]);
      out[5248] = fma(0.105, q, out[5248]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[328]) {
      const double q = scale * ws[69824];
      out[2592] = out[2592] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[2272] = fma(1.0, q, out[2272]);
    }
    if (mask[329]) {
      const double q = scale * ws[69856];
      out[2272] = out[2272] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[2688] = fma(1.0, q, out[2688]);
    }
    if (mask[330]) {
      const double q = scale * ws[69888];
      out[3648] = out[3648] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(2.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
      out[5344] = fma(0.32, q, out[5344]);
      out[5376] = fma(0.68, q, out[5376]);
      out[5728] = fma(0.68, q, out[5728]);
    }
    if (mask[331]) {
      const double q = scale * ws[69920];
      out[3040] = out[3040] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
      out[3808] = fma(1.0, q, out[3808]);
    }
    if (mask[332]) {
      const double q = scale * ws[69952];
      out[2976] = out[2976] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5376] = fma(1.0, q, out[5376]);
    }
    if (mask[333]) {
      const double q = scale * ws[69984];
      out[4032] = out[4032] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[334]) {
      const double q = scale * ws[70016];
      out[4064] = out[4064] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.5, q, out[5888]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.287, q, out[5856]);
      out[5760] = fma(1.24, q, out[5760]);
      out[5504] = fma(0.464, q, out[5504]);
      out[5696] = fma(0.5, q, out[5696]);
    }
    if (mask[335]) {
      const double q = scale * ws[70048];
      out[3072] = out[3072] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5888] = fma(1.0, q, out[5888]);
      out[5920] = fma(0.7, q, out[5920]);
      out[5376] = fma(0.7, q, out[5376]);
      out[5728] = fma(0.7, q, out[5728]);
      out[5440] = fma(0.3, q, out[5440]);
    }
    if (mask[336]) {
      const double q = scale * ws[70080];
      out[5216] = out[5216] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(1.0, q, out[5888]);
    }
    if (mask[337]) {
      const double q = scale * ws[70112];
      out[4800] = out[4800] - q;
      out[4800] = out[4800] - q;
      out[5632] = fma(2.0, q, out[5632]);
    }
    if (mask[338]) {
      const double q = scale * ws[70144];
      out[5888] = out[5888] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[339]) {
      const double q = scale * ws[70176];
      out[5632] = out[5632] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5568] = fma(1.0, q, out[5568]);
    }
    if (mask[340]) {
      const double q = scale * ws[70208];
      out[5408] = out[5408] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(0.254, q, out[5984]);
      out[5888] = fma(0.14, q, out[5888]);
      out[5216] = fma(0.092, q, out[5216]);
      out[5632] = fma(0.503, q, out[5632]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5568] = fma(0.519, q, out[5568]);
      out[5760] = fma(0.147, q, out[5760]);
      out[5280] = fma(0.075, q, out[5280]);
      out[4480] = fma(0.095, q, out[4480]);
    }
    if (mask[341]) {
      const double q = scale * ws[70240];
      out[5120] = out[5120] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(0.488, q, out[5984]);
      out[5888] = fma(0.055, q, out[5888]);
      out[5632] = fma(0.28, q, out[5632]);
      out[5216] = fma(0.485, q, out[5216]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.024, q, out[5856]);
      out[5760] = fma(0.241, q, out[5760]);
      out[5504] = fma(0.06, q, out[5504]);
      out[5280] = fma(0.063, q, out[5280]);
      out[4480] = fma(0.247, q, out[4480]);
      out[5568] = fma(0.048, q, out[5568]);
      out[5344] = fma(0.275, q, out[5344]);
    }
    if (mask[342]) {
      const double q = scale * ws[70272];
      out[3008] = out[3008] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(1.6, q, out[5856]);
      out[5760] = fma(0.2, q, out[5760]);
    }
    if (mask[343]) {
      const double q = scale * ws[70304];
      out[3200] = out[3200] - q;
      out[5952] = out[5952] - q;
      out[5760] = fma(0.47, q, out[5760]);
      out[5856] = fma(0.79, q, out[5856]);
      out[5984] = fma(0.79, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5280] = fma(0.18, q, out[5280]);
      out[5568] = fma(0.02, q, out[5568]);
      out[4480] = fma(0.09, q, out[4480]);
    }
    if (mask[344]) {
      const double q = scale * ws[70336];
      out[3328] = out[3328] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(0.86, q, out[5984]);
      out[5760] = fma(0.72, q, out[5760]);
      out[5504] = fma(0.11, q, out[5504]);
      out[5920] = fma(1.0, q, out[5920]);
      out[4480] = fma(0.2, q, out[4480]);
      out[5568] = fma(0.85, q, out[5568]);
      out[5344] = fma(0.04, q, out[5344]);
    }
    if (mask[345]) {
      const double q = scale * ws[70368];
      out[3360] = out[3360] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[4448] = fma(0.0, q, out[4448]);
      out[5376] = fma(1.0, q, out[5376]);
      out[4512] = fma(0.5, q, out[4512]);
      out[4320] = fma(0.25, q, out[4320]);
      out[3584] = fma(0.25, q, out[3584]);
    }
    if (mask[346]) {
      const double q = scale * ws[70400];
      out[3296] = out[3296] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.9146, q, out[5984]);
      out[4448] = fma(0.0854, q, out[4448]);
      out[5376] = fma(0.5488, q, out[5376]);
      out[5248] = fma(0.3659, q, out[5248]);
      out[4512] = fma(0.3659, q, out[4512]);
      out[5472] = fma(0.5488, q, out[5472]);
    }
    if (mask[347]) {
      const double q = scale * ws[70432];
      out[3104] = out[3104] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.9518, q, out[5984]);
      out[4448] = fma(0.0482, q, out[4448]);
      out[5376] = fma(0.7043, q, out[5376]);
      out[5248] = fma(0.2475, q, out[5248]);
      out[4512] = fma(0.3522, q, out[4512]);
      out[4320] = fma(0.5996, q, out[4320]);
    }
    if (mask[348]) {
      const double q = scale * ws[70464];
      out[3264] = out[3264] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.9146, q, out[5984]);
      out[4448] = fma(0.0854, q, out[4448]);
      out[5376] = fma(0.5488, q, out[5376]);
      out[5248] = fma(0.3659, q, out[5248]);
      out[4512] = fma(0.4573, q, out[4512]);
      out[4320] = fma(0.4573, q, out[4320]);
    }
    if (mask[349]) {
      const double q = scale * ws[70496];
      out[4288] = out[4288] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.75, q, out[5856]);
      out[4128] = fma(0.318, q, out[4128]);
      out[4736] = fma(0.5, q, out[4736]);
      out[5376] = fma(0.024, q, out[5376]);
      out[5344] = fma(0.033, q, out[5344]);
      out[5760] = fma(0.031, q, out[5760]);
    }
    if (mask[350]) {
      const double q = scale * ws[70528];
      out[4160] = out[4160] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[4544] = fma(0.2535, q, out[4544]);
      out[5760] = fma(0.371, q, out[5760]);
      out[4480] = fma(0.1165, q, out[4480]);
      out[4576] = fma(0.1725, q, out[4576]);
      out[5856] = fma(0.403, q, out[5856]);
      out[4096] = fma(0.091, q, out[4096]);
      out[5504] = fma(0.112, q, out[5504]);
    }
    if (mask[351]) {
      const double q = scale * ws[70560];
      out[4192] = out[4192] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[4576] = fma(1.0, q, out[4576]);
      out[5856] = fma(0.56, q, out[5856]);
    }
    if (mask[352]) {
      const double q = scale * ws[70592];
      out[2624] = out[2624] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.825, q, out[5920]);
      out[4544] = fma(0.65, q, out[4544]);
      out[4384] = fma(0.175, q, out[4384]);
      out[5760] = fma(0.168, q, out[5760]);
      out[5504] = fma(0.007, q, out[5504]);
      out[5856] = fma(0.007, q, out[5856]);
      out[5984] = fma(0.175, q, out[5984]);
    }
    if (mask[353]) {
      const double q = scale * ws[70624];
      out[2656] = out[2656] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.46, q, out[5920]);
      out[4576] = fma(0.46, q, out[4576]);
      out[4384] = fma(0.54, q, out[4384]);
      out[5984] = fma(0.54, q, out[5984]);
    }
    if (mask[354]) {
      const double q = scale * ws[70656];
      out[5792] = out[5792] - q;
      out[5952] = out[5952] - q;
      out[5888] = fma(1.0, q, out[5888]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[355]) {
      const double q = scale * ws[70688];
      out[4800] = out[4800] - q;
      out[5952] = out[5952] - q;
      out[5632] = fma(1.0, q, out[5632]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[356]) {
      const double q = scale * ws[70720];
      out[2848] = out[2848] - q;
      out[5952] = out[5952] - q;
      out[5792] = fma(1.0, q, out[5792]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(1.0, q, out[5856]);
    }
    if (mask[357]) {
      const double q = scale * ws[70752];
      out[5152] = out[5152] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(0.67, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.33, q, out[5856]);
      out[5472] = fma(0.67, q, out[5472]);
    }
    if (mask[358]) {
      const double q = scale * ws[70784];
      out[3776] = out[3776] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5472] = fma(1.0, q, out[5472]);
    }
    if (mask[359]) {
      const double q = scale * ws[70816];
      out[4672] = out[4672] - q;
      out[5952] = out[5952] - q;
      out[5856] = fma(1.0, q, out[5856]);
      out[5792] = fma(0.538, q, out[5792]);
      out[5664] = fma(1.0, q, out[5664]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[360]) {
      const double q = scale * ws[70848];
      out[3520] = out[3520] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[5344] = fma(1.0, q, out[5344]);
    }
    if (mask[361]) {
      const double q = scale * ws[70880];
      out[2880] = out[2880] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(0.3, q, out[5984]);
      out[5792] = fma(0.7, q, out[5792]);
      out[5216] = fma(0.7, q, out[5216]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.3, q, out[5856]);
      out[5760] = fma(0.7, q, out[5760]);
      out[5248] = fma(0.3, q, out[5248]);
    }
    if (mask[362]) {
      const double q = scale * ws[70912];
      out[2912] = out[2912] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5664] = fma(0.61, q, out[5664]);
      out[5856] = fma(0.03, q, out[5856]);
      out[5760] = fma(0.27, q, out[5760]);
      out[5504] = fma(0.7, q, out[5504]);
      out[5376] = fma(0.18, q, out[5376]);
      out[5248] = fma(0.21, q, out[5248]);
    }
    if (mask[363]) {
      const double q = scale * ws[70944];
      out[2592] = out[2592] - q;
      out[5952] = out[5952] - q;
      out[2272] = fma(1.0, q, out[2272]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[364]) {
      const double q = scale * ws[70976];
      out[2272] = out[2272] - q;
      out[5952] = out[5952] - q;
      out[2688] = fma(1.0, q, out[2688]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[365]) {
      const double q = scale * ws[71008];
      out[3648] = out[3648] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5344] = fma(0.32, q, out[5344]);
      out[5376] = fma(0.68, q, out[5376]);
      out[5728] = fma(0.68, q, out[5728]);
    }
    if (mask[366]) {
      const double q = scale * ws[71040];
      out[3040] = out[3040] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[3808] = fma(1.0, q, out[3808]);
    }
    if (mask[367]) {
      const double q = scale * ws[71072];
      out[2976] = out[2976] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5376] = fma(1.0, q, out[5376]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[368]) {
      const double q = scale * ws[71104];
      out[4032] = out[4032] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[369]) {
      const double q = scale * ws[71136];
      out[4064] = out[4064] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(2.0, q, out[5920]);
      out[5856] = fma(0.287, q, out[5856]);
      out[5760] = fma(1.24, q, out[5760]);
      out[5504] = fma(0.464, q, out[5504]);
    }
    if (mask[370]) {
      const double q = scale * ws[71168];
      out[3072] = out[3072] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(2.0, q, out[5920]);
      out[5376] = fma(1.0, q, out[5376]);
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[371]) {
      const double q = scale * ws[71200];
      out[4032] = out[4032] - q;
      out[4032] = out[4032] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5440] = fma(2.0, q, out[5440]);
    }
    if (mask[372]) {
      const double q = scale * ws[71232];
      out[4032] = out[4032] - q;
      out[4064] = out[4064] - q;
      out[5984] = fma(0.5, q, out[5984]);
      out[5920] = fma(0.5, q, out[5920]);
      out[5856] = fma(0.202, q, out[5856]);
      out[5760] = fma(0.64, q, out[5760]);
      out[5504] = fma(0.149, q, out[5504]);
      out[5440] = fma(1.5, q, out[5440]);
    }
    if (mask[373]) {
      const double q = scale * ws[71264];
      out[4064] = out[4064] - q;
      out[4064] = out[4064] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5856] = fma(0.504, q, out[5856]);
      out[5760] = fma(1.21, q, out[5760]);
      out[5504] = fma(0.285, q, out[5504]);
      out[5440] = fma(1.0, q, out[5440]);
    }
    if (mask[374]) {
      const double q = scale * ws[71296];
      out[5216] = out[5216] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[375]) {
      const double q = scale * ws[71328];
      out[5216] = out[5216] - q;
      out[4800] = out[4800] - q;
      out[5632] = fma(1.0, q, out[5632]);
    }
}
__device__ __noinline__ void ddm_src_1_6(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[376]) {
      const double q = scale * ws[71360];
      out[5216] = out[5216] - q;
      out[5216] = out[5216] - q;
    }
    if (mask[377]) {
      const double q = scale * ws[71392];
      out[3744] = out[3744] - q;
      out[4160] = out[4160] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4544] = fma(0.48, q, out[4544]);
      out[6016] = fma(0.48, q, out[6016]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[378]) {
      const double q = scale * ws[71424];
      out[3744] = out[3744] - q;
      out[4192] = out[4192] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4576] = fma(0.48, q, out[4576]);
      out[6016] = fma(0.48, q, out[6016]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[379]) {
      const double q = scale * ws[71456];
      out[3744] = out[3744] - q;
      out[4288] = out[4288] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[5856] = fma(0.48, q, out[5856]);
      out[4736] = fma(0.48, q, out[4736]);
      out[6016] = fma(0.48, q, out[6016]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[380]) {
      const double q = scale * ws[71488];
      out[3936] = out[3936] - q;
      out[4160] = out[4160] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4544] = fma(0.48, q, out[4544]);
      out[6016] = fma(0.48, q, out[6016]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[381]) {
      const double q = scale * ws[71520];
      out[3936] = out[3936] - q;
      out[4192] = out[4192] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4576] = fma(0.48, q, out[4576]);
      out[6016] = fma(0.48, q, out[6016]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[382]) {
      const double q = scale * ws[71552];
      out[3936] = out[3936] - q;
      out[4288] = out[4288] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[5856] = fma(0.48, q, out[5856]);
      out[4736] = fma(0.48, q, out[4736]);
      out[6016] = fma(0.48, q, out[6016]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[383]) {
      const double q = scale * ws[71584];
      out[3840] = out[3840] - q;
      out[4160] = out[4160] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4544] = fma(0.48, q, out[4544]);
      out[5920] = fma(0.48, q, out[5920]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[384]) {
      const double q = scale * ws[71616];
      out[3840] = out[3840] - q;
      out[4192] = out[4192] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4576] = fma(0.48, q, out[4576]);
      out[5920] = fma(0.48, q, out[5920]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[385]) {
      const double q = scale * ws[71648];
      out[3840] = out[3840] - q;
      out[4288] = out[4288] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[5856] = fma(0.48, q, out[5856]);
      out[4736] = fma(0.48, q, out[4736]);
      out[5920] = fma(0.48, q, out[5920]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[386]) {
      const double q = scale * ws[71680];
      out[3712] = out[3712] - q;
      out[4160] = out[4160] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4544] = fma(0.48, q, out[4544]);
      out[5920] = fma(0.48, q, out[5920]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[387]) {
      const double q = scale * ws[71712];
      out[3712] = out[3712] - q;
      out[4192] = out[4192] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[4576] = fma(0.48, q, out[4576]);
      out[5920] = fma(0.48, q, out[5920]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[388]) {
      const double q = scale * ws[71744];
      out[3712] = out[3712] - q;
      out[4288] = out[4288] - q;
      out[4256] = fma(0.96, q, out[4256]);
      out[5056] = fma(0.48, q, out[5056]);
      out[5856] = fma(0.48, q, out[5856]);
      out[4736] = fma(0.48, q, out[4736]);
      out[5920] = fma(0.48, q, out[5920]);
      out[5984] = fma(0.48, q, out[5984]);
      out[2720] = fma(0.04, q, out[2720]);
    }
    if (mask[389]) {
      const double q = scale * ws[71776];
      out[1376] = out[1376] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
    }
    if (mask[390]) {
      const double q = scale * ws[71808];
      out[384] = out[384] - q;
      out[6016] = out[6016] - q;
      out[5632] = fma(0.852, q, out[5632]);
      out[3616] = fma(0.149, q, out[3616]);
    }
    if (mask[391]) {
      const double q = scale * ws[71840];
      out[416] = out[416] - q;
      out[6016] = out[6016] - q;
      out[5632] = fma(1.0, q, out[5632]);
      out[3616] = fma(0.00101, q, out[3616]);
    }
    if (mask[392]) {
      const double q = scale * ws[71872];
      out[3552] = out[3552] - q;
      out[6016] = out[6016] - q;
      out[4672] = fma(0.57, q, out[4672]);
      out[3520] = fma(0.43, q, out[3520]);
    }
    if (mask[393]) {
      const double q = scale * ws[71904];
      out[3552] = out[3552] - q;
      out[5184] = out[5184] - q;
      out[5664] = fma(0.84, q, out[5664]);
      out[5984] = fma(0.56, q, out[5984]);
      out[6016] = fma(0.28, q, out[6016]);
      out[5856] = fma(0.72, q, out[5856]);
      out[5376] = fma(0.62, q, out[5376]);
    }
    if (mask[394]) {
      const double q = scale * ws[71936];
      out[3552] = out[3552] - q;
      out[5952] = out[5952] - q;
      out[5856] = fma(0.68, q, out[5856]);
      out[4672] = fma(0.32, q, out[4672]);
      out[5216] = fma(0.68, q, out[5216]);
      out[5248] = fma(0.68, q, out[5248]);
      out[5024] = fma(0.32, q, out[5024]);
      out[5920] = fma(0.68, q, out[5920]);
    }
    if (mask[396]) {
      const double q = scale * ws[72000];
      out[1568] = out[1568] - q;
      out[6016] = out[6016] - q;
      out[3136] = fma(0.667, q, out[3136]);
      out[3872] = fma(0.333, q, out[3872]);
      out[5984] = fma(0.333, q, out[5984]);
    }
    if (mask[397]) {
      const double q = scale * ws[72032];
      out[3136] = out[3136] - q;
      out[5824] = out[5824] - q;
      out[5984] = fma(0.968, q, out[5984]);
      out[5920] = fma(0.968, q, out[5920]);
      out[3552] = fma(0.895, q, out[3552]);
      out[5856] = fma(0.895, q, out[5856]);
      out[3168] = fma(0.072, q, out[3168]);
      out[5440] = fma(0.032, q, out[5440]);
    }
    if (mask[398]) {
      const double q = scale * ws[72064];
      out[3136] = out[3136] - q;
      out[5952] = out[5952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5920] = fma(1.0, q, out[5920]);
      out[3552] = fma(0.925, q, out[3552]);
      out[5856] = fma(0.925, q, out[5856]);
      out[3168] = fma(0.075, q, out[3168]);
    }
    if (mask[399]) {
      const double q = scale * ws[72096];
      out[3136] = out[3136] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[400]) {
      const double q = scale * ws[72128];
      out[3136] = out[3136] - q;
      out[5888] = out[5888] - q;
      out[5600] = fma(0.32, q, out[5600]);
      out[5856] = fma(1.143, q, out[5856]);
      out[5984] = fma(0.87, q, out[5984]);
      out[3552] = fma(0.463, q, out[3552]);
      out[2752] = fma(0.25, q, out[2752]);
      out[4736] = fma(0.231, q, out[4736]);
      out[3168] = fma(0.037, q, out[3168]);
      out[3872] = fma(0.019, q, out[3872]);
    }
    if (mask[401]) {
      const double q = scale * ws[72160];
      out[3136] = out[3136] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5696] = fma(0.3, q, out[5696]);
      out[5984] = fma(0.8, q, out[5984]);
      out[3552] = fma(0.74, q, out[3552]);
      out[5856] = fma(0.74, q, out[5856]);
      out[4736] = fma(0.185, q, out[4736]);
      out[3168] = fma(0.06, q, out[3168]);
      out[3872] = fma(0.015, q, out[3872]);
    }
    if (mask[402]) {
      const double q = scale * ws[72192];
      out[1568] = out[1568] - q;
      out[5184] = out[5184] - q;
      out[3552] = fma(0.62, q, out[3552]);
      out[5664] = fma(0.63, q, out[5664]);
      out[5984] = fma(0.42, q, out[5984]);
      out[6016] = fma(0.08, q, out[6016]);
      out[5856] = fma(0.83, q, out[5856]);
      out[2240] = fma(0.17, q, out[2240]);
    }
    if (mask[403]) {
      const double q = scale * ws[72224];
      out[1568] = out[1568] - q;
      out[5952] = out[5952] - q;
      out[4032] = fma(0.9, q, out[4032]);
      out[4064] = fma(0.1, q, out[4064]);
      out[3552] = fma(0.9, q, out[3552]);
    }
    if (mask[404]) {
      const double q = scale * ws[72256];
      out[3168] = out[3168] - q;
      out[6016] = out[6016] - q;
      out[5472] = fma(0.49, q, out[5472]);
      out[5984] = fma(0.49, q, out[5984]);
      out[1856] = fma(0.51, q, out[1856]);
    }
    if (mask[405]) {
      const double q = scale * ws[72288];
      out[1856] = out[1856] - q;
      out[5824] = out[5824] - q;
      out[5440] = fma(0.08, q, out[5440]);
      out[5920] = fma(0.92, q, out[5920]);
      out[4512] = fma(0.92, q, out[4512]);
      out[5984] = fma(0.75, q, out[5984]);
      out[5888] = fma(0.17, q, out[5888]);
    }
    if (mask[406]) {
      const double q = scale * ws[72320];
      out[1856] = out[1856] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(0.6, q, out[5728]);
      out[4512] = fma(0.4, q, out[4512]);
      out[6016] = fma(0.4, q, out[6016]);
      out[5984] = fma(0.32, q, out[5984]);
      out[5888] = fma(0.08, q, out[5888]);
    }
    if (mask[407]) {
      const double q = scale * ws[72352];
      out[4512] = out[4512] - q;
      out[6016] = out[6016] - q;
      out[5504] = fma(0.65, q, out[5504]);
      out[5376] = fma(0.31, q, out[5376]);
      out[5984] = fma(0.66, q, out[5984]);
      out[5888] = fma(0.34, q, out[5888]);
      out[5664] = fma(0.43, q, out[5664]);
      out[3616] = fma(0.04, q, out[3616]);
    }
    if (mask[408]) {
      const double q = scale * ws[72384];
      out[3168] = out[3168] - q;
      out[5184] = out[5184] - q;
      out[6016] = fma(0.02, q, out[6016]);
      out[5760] = fma(1.0, q, out[5760]);
    }
    if (mask[409]) {
      const double q = scale * ws[72416];
      out[3168] = out[3168] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5472] = fma(0.8, q, out[5472]);
      out[3584] = fma(0.2, q, out[3584]);
    }
    if (mask[410]) {
      const double q = scale * ws[72448];
      out[448] = out[448] - q;
      out[6016] = out[6016] - q;
      out[5344] = fma(0.613, q, out[5344]);
      out[5760] = fma(0.387, q, out[5760]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[411]) {
      const double q = scale * ws[72480];
      out[1600] = out[1600] - q;
      out[5952] = out[5952] - q;
      out[1920] = fma(1.0, q, out[1920]);
    }
    if (mask[412]) {
      const double q = scale * ws[72512];
      out[1920] = out[1920] - q;
      out[5984] = out[5984] - q;
      out[4928] = fma(1.0, q, out[4928]);
    }
    if (mask[413]) {
      const double q = scale * ws[72544];
      out[1920] = out[1920] - q;
      out[5824] = out[5824] - q;
      out[5536] = fma(1.0, q, out[5536]);
      out[5920] = fma(2.0, q, out[5920]);
    }
    if (mask[414]) {
      const double q = scale * ws[72576];
      out[1920] = out[1920] - q;
      out[5952] = out[5952] - q;
      out[5536] = fma(1.0, q, out[5536]);
      out[5920] = fma(2.0, q, out[5920]);
    }
    if (mask[415]) {
      const double q = scale * ws[72608];
      out[1600] = out[1600] - q;
      out[5184] = out[5184] - q;
      out[5536] = fma(0.982, q, out[5536]);
      out[4832] = fma(0.018, q, out[4832]);
    }
    if (mask[416]) {
      const double q = scale * ws[72640];
      out[1600] = out[1600] - q;
      out[6016] = out[6016] - q;
      out[2304] = fma(1.0, q, out[2304]);
    }
    if (mask[417]) {
      const double q = scale * ws[72672];
      out[2304] = out[2304] - q;
      out[5984] = out[5984] - q;
      out[4960] = fma(1.0, q, out[4960]);
    }
    if (mask[418]) {
      const double q = scale * ws[72704];
      out[2304] = out[2304] - q;
      out[5952] = out[5952] - q;
      out[5536] = fma(1.0, q, out[5536]);
    }
    if (mask[419]) {
      const double q = scale * ws[72736];
      out[2304] = out[2304] - q;
      out[5824] = out[5824] - q;
      out[4992] = fma(0.247, q, out[4992]);
      out[5536] = fma(0.753, q, out[5536]);
      out[5920] = fma(0.753, q, out[5920]);
    }
    if (mask[420]) {
      const double q = scale * ws[72768];
      out[5376] = out[5376] - q;
      out[480] = fma(1.0, q, out[480]);
    }
    if (mask[421]) {
      const double q = scale * ws[72800];
      out[5248] = out[5248] - q;
      out[480] = fma(1.0, q, out[480]);
    }
    if (mask[422]) {
      const double q = scale * ws[72832];
      out[1024] = out[1024] - q;
      out[5024] = fma(2.0, q, out[5024]);
    }
    if (mask[423]) {
      const double q = scale * ws[72864];
      out[5920] = out[5920] - q;
      out[1184] = fma(0.5, q, out[1184]);
      out[5024] = fma(0.5, q, out[5024]);
    }
    if (mask[424]) {
      const double q = scale * ws[72896];
      out[5984] = out[5984] - q;
    }
    if (mask[425]) {
      const double q = scale * ws[72928];
      out[5952] = out[5952] - q;
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[427]) {
      const double q = scale * ws[72992];
      out[1376] = out[1376] - q;
      out[1056] = fma(1.0, q, out[1056]);
    }
    if (mask[428]) {
      const double q = scale * ws[73024];
      out[1056] = out[1056] - q;
      out[0] = fma(1.0, q, out[0]);
    }
    if (mask[429]) {
      const double q = scale * ws[73056];
      out[1056] = out[1056] - q;
      out[512] = out[512] - q;
      out[544] = fma(1.0, q, out[544]);
    }
    if (mask[430]) {
      const double q = scale * ws[73088];
      out[1664] = out[1664] - q;
      out[32] = fma(1.0, q, out[32]);
    }
    if (mask[431]) {
      const double q = scale * ws[73120];
      out[2208] = out[2208] - q;
      out[64] = fma(1.0, q, out[64]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[432]) {
      const double q = scale * ws[73152];
      out[608] = out[608] - q;
      out[6016] = out[6016] - q;
      out[2368] = fma(1.0, q, out[2368]);
    }
    if (mask[433]) {
      const double q = scale * ws[73184];
      out[640] = out[640] - q;
      out[6016] = out[6016] - q;
      out[2400] = fma(1.0, q, out[2400]);
    }
    if (mask[434]) {
      const double q = scale * ws[73216];
      out[672] = out[672] - q;
      out[6016] = out[6016] - q;
      out[2432] = fma(1.0, q, out[2432]);
    }
    if (mask[435]) {
      const double q = scale * ws[73248];
      out[704] = out[704] - q;
      out[6016] = out[6016] - q;
      out[2464] = fma(1.0, q, out[2464]);
    }
    if (mask[436]) {
      const double q = scale * ws[73280];
      out[736] = out[736] - q;
      out[6016] = out[6016] - q;
      out[2496] = fma(1.0, q, out[2496]);
    }
    if (mask[437]) {
      const double q = scale * ws[73312];
      out[768] = out[768] - q;
      out[6016] = out[6016] - q;
      out[2528] = fma(1.0, q, out[2528]);
    }
    if (mask[438]) {
      const double q = scale * ws[73344];
      out[800] = out[800] - q;
      out[6016] = out[6016] - q;
      out[3904] = fma(1.0, q, out[3904]);
    }
    if (mask[439]) {
      const double q = scale * ws[73376];
      out[2368] = out[2368] - q;
      out[5824] = out[5824] - q;
      out[1952] = fma(0.72, q, out[1952]);
      out[5312] = fma(0.28, q, out[5312]);
      out[5920] = fma(0.72, q, out[5920]);
    }
}
__device__ __noinline__ void ddm_src_1_7(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[440]) {
      const double q = scale * ws[73408];
      out[2400] = out[2400] - q;
      out[5824] = out[5824] - q;
      out[1984] = fma(0.72, q, out[1984]);
      out[5536] = fma(0.28, q, out[5536]);
      out[5920] = fma(0.72, q, out[5920]);
    }
    if (mask[441]) {
      const double q = scale * ws[73440];
      out[2432] = out[2432] - q;
      out[5824] = out[5824] - q;
      out[2016] = fma(0.72, q, out[2016]);
      out[5088] = fma(0.28, q, out[5088]);
      out[5920] = fma(0.72, q, out[5920]);
    }
    if (mask[442]) {
      const double q = scale * ws[73472];
      out[2464] = out[2464] - q;
      out[5824] = out[5824] - q;
      out[2048] = fma(0.72, q, out[2048]);
      out[4704] = fma(0.28, q, out[4704]);
      out[5920] = fma(0.72, q, out[5920]);
    }
    if (mask[443]) {
      const double q = scale * ws[73504];
      out[2496] = out[2496] - q;
      out[5824] = out[5824] - q;
      out[2080] = fma(0.72, q, out[2080]);
      out[4960] = fma(0.28, q, out[4960]);
      out[5920] = fma(0.72, q, out[5920]);
    }
    if (mask[444]) {
      const double q = scale * ws[73536];
      out[2528] = out[2528] - q;
      out[5824] = out[5824] - q;
      out[2112] = fma(0.72, q, out[2112]);
      out[4416] = fma(0.28, q, out[4416]);
      out[5920] = fma(0.72, q, out[5920]);
    }
    if (mask[445]) {
      const double q = scale * ws[73568];
      out[3904] = out[3904] - q;
      out[5824] = out[5824] - q;
      out[2144] = fma(0.74, q, out[2144]);
      out[5440] = fma(0.26, q, out[5440]);
      out[5920] = fma(0.74, q, out[5920]);
    }
    if (mask[446]) {
      const double q = scale * ws[73600];
      out[2368] = out[2368] - q;
      out[5952] = out[5952] - q;
      out[1952] = fma(1.0, q, out[1952]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[447]) {
      const double q = scale * ws[73632];
      out[2400] = out[2400] - q;
      out[5952] = out[5952] - q;
      out[1984] = fma(1.0, q, out[1984]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[448]) {
      const double q = scale * ws[73664];
      out[2432] = out[2432] - q;
      out[5952] = out[5952] - q;
      out[2016] = fma(1.0, q, out[2016]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[449]) {
      const double q = scale * ws[73696];
      out[2464] = out[2464] - q;
      out[5952] = out[5952] - q;
      out[2048] = fma(1.0, q, out[2048]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[450]) {
      const double q = scale * ws[73728];
      out[2496] = out[2496] - q;
      out[5952] = out[5952] - q;
      out[2080] = fma(1.0, q, out[2080]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[451]) {
      const double q = scale * ws[73760];
      out[2528] = out[2528] - q;
      out[5952] = out[5952] - q;
      out[2112] = fma(1.0, q, out[2112]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[452]) {
      const double q = scale * ws[73792];
      out[3904] = out[3904] - q;
      out[5952] = out[5952] - q;
      out[2144] = fma(1.0, q, out[2144]);
      out[5920] = fma(1.0, q, out[5920]);
    }
    if (mask[453]) {
      const double q = scale * ws[73824];
      out[2368] = out[2368] - q;
      out[5984] = out[5984] - q;
      out[5536] = fma(1.0, q, out[5536]);
    }
    if (mask[454]) {
      const double q = scale * ws[73856];
      out[2400] = out[2400] - q;
      out[5984] = out[5984] - q;
      out[5088] = fma(1.0, q, out[5088]);
    }
    if (mask[455]) {
      const double q = scale * ws[73888];
      out[2432] = out[2432] - q;
      out[5984] = out[5984] - q;
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[456]) {
      const double q = scale * ws[73920];
      out[2464] = out[2464] - q;
      out[5984] = out[5984] - q;
      out[4960] = fma(1.0, q, out[4960]);
    }
    if (mask[457]) {
      const double q = scale * ws[73952];
      out[2496] = out[2496] - q;
      out[5984] = out[5984] - q;
      out[4416] = fma(1.0, q, out[4416]);
    }
    if (mask[458]) {
      const double q = scale * ws[73984];
      out[2528] = out[2528] - q;
      out[5984] = out[5984] - q;
      out[4832] = fma(1.0, q, out[4832]);
    }
    if (mask[459]) {
      const double q = scale * ws[74016];
      out[3904] = out[3904] - q;
      out[5984] = out[5984] - q;
      out[5728] = fma(1.0, q, out[5728]);
    }
    if (mask[460]) {
      const double q = scale * ws[74048];
      out[1952] = out[1952] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5536] = fma(1.0, q, out[5536]);
    }
    if (mask[461]) {
      const double q = scale * ws[74080];
      out[1984] = out[1984] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5088] = fma(1.0, q, out[5088]);
    }
    if (mask[462]) {
      const double q = scale * ws[74112];
      out[2016] = out[2016] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[4704] = fma(1.0, q, out[4704]);
    }
    if (mask[463]) {
      const double q = scale * ws[74144];
      out[2048] = out[2048] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[4960] = fma(1.0, q, out[4960]);
    }
    if (mask[464]) {
      const double q = scale * ws[74176];
      out[2080] = out[2080] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[4416] = fma(1.0, q, out[4416]);
    }
    if (mask[465]) {
      const double q = scale * ws[74208];
      out[2112] = out[2112] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[4832] = fma(1.0, q, out[4832]);
    }
    if (mask[466]) {
      const double q = scale * ws[74240];
      out[2144] = out[2144] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5312] = fma(1.0, q, out[5312]);
    }
    if (mask[467]) {
      const double q = scale * ws[74272];
      out[1952] = out[1952] - q;
      out[5824] = out[5824] - q;
      out[5088] = fma(0.14, q, out[5088]);
      out[5920] = fma(0.86, q, out[5920]);
      out[5536] = fma(0.86, q, out[5536]);
      out[5984] = fma(0.86, q, out[5984]);
    }
    if (mask[468]) {
      const double q = scale * ws[74304];
      out[1984] = out[1984] - q;
      out[5824] = out[5824] - q;
      out[4992] = fma(0.14, q, out[4992]);
      out[5920] = fma(0.86, q, out[5920]);
      out[5088] = fma(0.86, q, out[5088]);
      out[5984] = fma(0.86, q, out[5984]);
    }
    if (mask[469]) {
      const double q = scale * ws[74336];
      out[2016] = out[2016] - q;
      out[5824] = out[5824] - q;
      out[4960] = fma(0.14, q, out[4960]);
      out[5920] = fma(0.86, q, out[5920]);
      out[4704] = fma(0.86, q, out[4704]);
      out[5984] = fma(0.86, q, out[5984]);
    }
    if (mask[470]) {
      const double q = scale * ws[74368];
      out[2048] = out[2048] - q;
      out[5824] = out[5824] - q;
      out[4416] = fma(0.14, q, out[4416]);
      out[5920] = fma(0.86, q, out[5920]);
      out[4960] = fma(0.86, q, out[4960]);
      out[5984] = fma(0.86, q, out[5984]);
    }
    if (mask[471]) {
      const double q = scale * ws[74400];
      out[2080] = out[2080] - q;
      out[5824] = out[5824] - q;
      out[4832] = fma(0.14, q, out[4832]);
      out[5920] = fma(0.86, q, out[5920]);
      out[4416] = fma(0.86, q, out[4416]);
      out[5984] = fma(0.86, q, out[5984]);
    }
    if (mask[472]) {
      const double q = scale * ws[74432];
      out[2112] = out[2112] - q;
      out[5824] = out[5824] - q;
      out[4832] = fma(1.0, q, out[4832]);
      out[5920] = fma(0.86, q, out[5920]);
      out[5984] = fma(0.86, q, out[5984]);
    }
    if (mask[473]) {
      const double q = scale * ws[74464];
      out[2144] = out[2144] - q;
      out[5824] = out[5824] - q;
      out[5440] = fma(0.12, q, out[5440]);
      out[5920] = fma(0.88, q, out[5920]);
      out[5504] = fma(0.88, q, out[5504]);
      out[5984] = fma(0.88, q, out[5984]);
    }
    if (mask[474]) {
      const double q = scale * ws[74496];
      out[1952] = out[1952] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5536] = fma(1.0, q, out[5536]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[475]) {
      const double q = scale * ws[74528];
      out[1984] = out[1984] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5088] = fma(1.0, q, out[5088]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[476]) {
      const double q = scale * ws[74560];
      out[2016] = out[2016] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[4704] = fma(1.0, q, out[4704]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[477]) {
      const double q = scale * ws[74592];
      out[2048] = out[2048] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[4960] = fma(1.0, q, out[4960]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[478]) {
      const double q = scale * ws[74624];
      out[2080] = out[2080] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[4416] = fma(1.0, q, out[4416]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[479]) {
      const double q = scale * ws[74656];
      out[2112] = out[2112] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[4832] = fma(1.0, q, out[4832]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[480]) {
      const double q = scale * ws[74688];
      out[2144] = out[2144] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5504] = fma(1.0, q, out[5504]);
      out[5984] = fma(1.0, q, out[5984]);
    }
    if (mask[481]) {
      const double q = scale * ws[74720];
      out[1952] = out[1952] - q;
      out[5984] = out[5984] - q;
      out[4992] = fma(1.0, q, out[4992]);
    }
    if (mask[482]) {
      const double q = scale * ws[74752];
      out[1984] = out[1984] - q;
      out[5984] = out[5984] - q;
      out[4960] = fma(1.0, q, out[4960]);
    }
    if (mask[483]) {
      const double q = scale * ws[74784];
      out[2016] = out[2016] - q;
      out[5984] = out[5984] - q;
      out[4416] = fma(1.0, q, out[4416]);
    }
    if (mask[484]) {
      const double q = scale * ws[74816];
      out[2048] = out[2048] - q;
      out[5984] = out[5984] - q;
      out[4832] = fma(1.0, q, out[4832]);
    }
    if (mask[485]) {
      const double q = scale * ws[74848];
      out[2080] = out[2080] - q;
      out[5984] = out[5984] - q;
      out[4832] = fma(1.0, q, out[4832]);
    }
    if (mask[486]) {
      const double q = scale * ws[74880];
      out[2112] = out[2112] - q;
      out[5984] = out[5984] - q;
      out[4832] = fma(1.0, q, out[4832]);
    }
    if (mask[487]) {
      const double q = scale * ws[74912];
      out[2144] = out[2144] - q;
      out[5984] = out[5984] - q;
      out[5088] = fma(1.0, q, out[5088]);
    }
    if (mask[488]) {
      const double q = scale * ws[74944];
      out[832] = out[832] - q;
      out[6016] = out[6016] - q;
      out[3392] = fma(0.84, q, out[3392]);
      out[5984] = fma(0.16, q, out[5984]);
      out[5312] = fma(0.16, q, out[5312]);
    }
    if (mask[489]) {
      const double q = scale * ws[74976];
      out[3392] = out[3392] - q;
      out[5984] = out[5984] - q;
      out[5312] = fma(0.0595, q, out[5312]);
      out[4992] = fma(0.9048, q, out[4992]);
      out[4864] = fma(0.0357, q, out[4864]);
    }
    if (mask[490]) {
      const double q = scale * ws[75008];
      out[3392] = out[3392] - q;
      out[5824] = out[5824] - q;
      out[5312] = fma(0.0001, q, out[5312]);
      out[5088] = fma(0.0018, q, out[5088]);
      out[4640] = fma(0.0001, q, out[4640]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[4448] = fma(0.0594, q, out[4448]);
      out[5376] = fma(0.4693, q, out[5376]);
      out[5248] = fma(0.4693, q, out[5248]);
      out[4512] = fma(0.4693, q, out[4512]);
      out[4320] = fma(0.4693, q, out[4320]);
    }
    if (mask[491]) {
      const double q = scale * ws[75040];
      out[3392] = out[3392] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.9405, q, out[5984]);
      out[4448] = fma(0.0595, q, out[4448]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[492]) {
      const double q = scale * ws[75072];
      out[3392] = out[3392] - q;
      out[5888] = out[5888] - q;
      out[5856] = fma(0.68, q, out[5856]);
      out[5984] = fma(1.3105, q, out[5984]);
      out[5600] = fma(0.32, q, out[5600]);
      out[4448] = fma(0.0595, q, out[4448]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[493]) {
      const double q = scale * ws[75104];
      out[3392] = out[3392] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5984] = fma(0.9405, q, out[5984]);
      out[5696] = fma(0.3, q, out[5696]);
      out[4448] = fma(0.0595, q, out[4448]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[494]) {
      const double q = scale * ws[75136];
      out[864] = out[864] - q;
      out[6016] = out[6016] - q;
      out[3424] = fma(0.84, q, out[3424]);
      out[5984] = fma(0.16, q, out[5984]);
      out[5536] = fma(0.16, q, out[5536]);
    }
    if (mask[495]) {
      const double q = scale * ws[75168];
      out[3424] = out[3424] - q;
      out[5984] = out[5984] - q;
      out[5536] = fma(0.0595, q, out[5536]);
      out[4960] = fma(0.9048, q, out[4960]);
      out[4864] = fma(0.0357, q, out[4864]);
    }
    if (mask[496]) {
      const double q = scale * ws[75200];
      out[3424] = out[3424] - q;
      out[5824] = out[5824] - q;
      out[5536] = fma(0.0001, q, out[5536]);
      out[4992] = fma(0.0018, q, out[4992]);
      out[4864] = fma(0.0001, q, out[4864]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[5312] = fma(0.0594, q, out[5312]);
      out[5376] = fma(0.4693, q, out[5376]);
      out[5248] = fma(0.4693, q, out[5248]);
      out[4512] = fma(0.4693, q, out[4512]);
      out[4320] = fma(0.4693, q, out[4320]);
    }
    if (mask[497]) {
      const double q = scale * ws[75232];
      out[3424] = out[3424] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.9405, q, out[5984]);
      out[5312] = fma(0.0595, q, out[5312]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[498]) {
      const double q = scale * ws[75264];
      out[3424] = out[3424] - q;
      out[5888] = out[5888] - q;
      out[5856] = fma(0.68, q, out[5856]);
      out[5984] = fma(1.3105, q, out[5984]);
      out[5600] = fma(0.32, q, out[5600]);
      out[5312] = fma(0.0595, q, out[5312]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[499]) {
      const double q = scale * ws[75296];
      out[3424] = out[3424] - q;
      out[5792] = out[5792] - q;
      out[5888] = fma(0.7, q, out[5888]);
      out[5984] = fma(0.9405, q, out[5984]);
      out[5696] = fma(0.3, q, out[5696]);
      out[5312] = fma(0.0595, q, out[5312]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[500]) {
      const double q = scale * ws[75328];
      out[896] = out[896] - q;
      out[6016] = out[6016] - q;
      out[3456] = fma(0.84, q, out[3456]);
      out[5984] = fma(0.16, q, out[5984]);
      out[5536] = fma(0.16, q, out[5536]);
    }
    if (mask[501]) {
      const double q = scale * ws[75360];
      out[3456] = out[3456] - q;
      out[5984] = out[5984] - q;
      out[5536] = fma(0.0595, q, out[5536]);
      out[4992] = fma(0.9048, q, out[4992]);
      out[4768] = fma(0.0357, q, out[4768]);
    }
}
}  // namespace mech_cracmm2
