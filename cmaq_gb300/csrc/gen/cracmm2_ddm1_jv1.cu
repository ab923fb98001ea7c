// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void ddm_jv_1_4(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[51168] * fma(y[5888], v[2624], y[2624] * v[5888]);
      out[2624] = out[2624] - dr;
      out[5888] = out[5888] - dr;
      out[4384] = fma(0.341, dr, out[4384]);
      out[5856] = fma(0.964, dr, out[5856]);
      out[5600] = fma(0.043, dr, out[5600]);
      out[5984] = fma(0.918, dr, out[5984]);
      out[5920] = fma(0.659, dr, out[5920]);
      out[4544] = fma(0.533, dr, out[4544]);
      out[5504] = fma(0.007, dr, out[5504]);
      out[5760] = fma(0.119, dr, out[5760]);
    }
    {
      const double dr = ws[51200] * fma(y[5888], v[3840], y[3840] * v[5888]);
      out[3840] = out[3840] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.75, dr, out[5984]);
      out[5920] = fma(0.75, dr, out[5920]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[51232] * fma(y[5888], v[4192], y[4192] * v[5888]);
      out[4192] = out[4192] - dr;
      out[5888] = out[5888] - dr;
      out[5600] = fma(0.25, dr, out[5600]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[5856] = fma(1.03, dr, out[5856]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[51264] * fma(y[5888], v[3936], y[3936] * v[5888]);
      out[3936] = out[3936] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[51296] * fma(y[5888], v[2656], y[2656] * v[5888]);
      out[2656] = out[2656] - dr;
      out[5888] = out[5888] - dr;
      out[4384] = fma(0.69, dr, out[4384]);
      out[5856] = fma(0.91, dr, out[5856]);
      out[5600] = fma(0.09, dr, out[5600]);
      out[5984] = fma(1.01, dr, out[5984]);
      out[4576] = fma(0.31, dr, out[4576]);
      out[5920] = fma(0.31, dr, out[5920]);
    }
    {
      const double dr = ws[51328] * fma(y[5888], v[3712], y[3712] * v[5888]);
      out[3712] = out[3712] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.75, dr, out[5984]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[5920] = fma(0.75, dr, out[5920]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[51360] * fma(y[5888], v[5792], y[5792] * v[5888]);
      out[5792] = out[5792] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.9, dr, out[5984]);
      out[5888] = fma(0.9, dr, out[5888]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5696] = fma(0.1, dr, out[5696]);
    }
    {
      const double dr = ws[51392] * fma(y[5888], v[4800], y[4800] * v[5888]);
      out[4800] = out[4800] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.9, dr, out[5984]);
      out[5888] = fma(0.9, dr, out[5888]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5696] = fma(0.1, dr, out[5696]);
    }
    {
      const double dr = ws[51424] * fma(y[5888], v[2848], y[2848] * v[5888]);
      out[2848] = out[2848] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5792] = fma(0.5, dr, out[5792]);
      out[5856] = fma(1.5, dr, out[5856]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
      out[5696] = fma(0.125, dr, out[5696]);
    }
    {
      const double dr = ws[51456] * fma(y[5888], v[5152], y[5152] * v[5888]);
      out[5152] = out[5152] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.834, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5472] = fma(0.334, dr, out[5472]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[51488] * fma(y[5888], v[3776], y[3776] * v[5888]);
      out[3776] = out[3776] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[5472] = fma(0.5, dr, out[5472]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[51520] * fma(y[5888], v[4672], y[4672] * v[5888]);
      out[4672] = out[4672] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5792] = fma(0.269, dr, out[5792]);
      out[5664] = fma(0.5, dr, out[5664]);
      out[5856] = fma(1.66, dr, out[5856]);
      out[5696] = fma(0.067, dr, out[5696]);
      out[5888] = fma(0.25, dr, out[5888]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[51552] * fma(y[5888], v[3520], y[3520] * v[5888]);
      out[3520] = out[3520] - dr;
      out[5888] = out[5888] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.5, dr, out[5856]);
      out[5344] = fma(0.5, dr, out[5344]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[51584] * fma(y[5888], v[2880], y[2880] * v[5888]);
      out[2880] = out[2880] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5792] = fma(1.16, dr, out[5792]);
      out[5216] = fma(1.16, dr, out[5216]);
      out[5856] = fma(1.5, dr, out[5856]);
      out[5760] = fma(1.75, dr, out[5760]);
      out[5248] = fma(0.5, dr, out[5248]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
      out[5696] = fma(0.292, dr, out[5696]);
    }
    {
      const double dr = ws[51616] * fma(y[5888], v[2912], y[2912] * v[5888]);
      out[2912] = out[2912] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5664] = fma(0.305, dr, out[5664]);
      out[5856] = fma(0.773, dr, out[5856]);
      out[5760] = fma(0.203, dr, out[5760]);
      out[5504] = fma(0.525, dr, out[5504]);
      out[5376] = fma(0.135, dr, out[5376]);
      out[5248] = fma(0.105, dr, out[5248]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
    }
    {
      const double dr = ws[51648] * fma(y[5888], v[2592], y[2592] * v[5888]);
      out[2592] = out[2592] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[2272] = fma(1.0, dr, out[2272]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[51680] * fma(y[5888], v[2272], y[2272] * v[5888]);
      out[2272] = out[2272] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[2688] = fma(1.0, dr, out[2688]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[51712] * fma(y[5888], v[3648], y[3648] * v[5888]);
      out[3648] = out[3648] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(2.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5344] = fma(0.32, dr, out[5344]);
      out[5376] = fma(0.68, dr, out[5376]);
      out[5728] = fma(0.68, dr, out[5728]);
    }
    {
      const double dr = ws[51744] * fma(y[5888], v[3040], y[3040] * v[5888]);
      out[3040] = out[3040] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[3808] = fma(1.0, dr, out[3808]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[51776] * fma(y[5888], v[2976], y[2976] * v[5888]);
      out[2976] = out[2976] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(1.0, dr, out[5856]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5376] = fma(1.0, dr, out[5376]);
    }
    {
      const double dr = ws[51808] * fma(y[5888], v[4032], y[4032] * v[5888]);
      out[4032] = out[4032] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(2.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[51840] * fma(y[5888], v[4064], y[4064] * v[5888]);
      out[4064] = out[4064] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5920] = fma(0.5, dr, out[5920]);
      out[5856] = fma(0.965, dr, out[5856]);
      out[5760] = fma(0.93, dr, out[5760]);
      out[5504] = fma(0.348, dr, out[5504]);
      out[5600] = fma(0.25, dr, out[5600]);
      out[5056] = fma(0.25, dr, out[5056]);
      out[5440] = fma(0.5, dr, out[5440]);
    }
    {
      const double dr = ws[51872] * fma(y[5888], v[3072], y[3072] * v[5888]);
      out[3072] = out[3072] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(0.7, dr, out[5920]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5376] = fma(0.7, dr, out[5376]);
      out[5728] = fma(0.7, dr, out[5728]);
      out[5440] = fma(0.3, dr, out[5440]);
    }
    {
      const double dr = ws[51904] * fma(y[5888], v[5216], y[5216] * v[5888]);
      out[5216] = out[5216] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[51936] * fma(y[5792], v[5632], y[5632] * v[5792]);
      out[5632] = out[5632] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5568] = fma(1.0, dr, out[5568]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[51968] * fma(y[5792], v[5408], y[5408] * v[5792]);
      out[5408] = out[5408] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.394, dr, out[5984]);
      out[5888] = fma(0.58, dr, out[5888]);
      out[5632] = fma(0.026, dr, out[5632]);
      out[5216] = fma(0.026, dr, out[5216]);
      out[5856] = fma(0.13, dr, out[5856]);
      out[5760] = fma(0.273, dr, out[5760]);
      out[5504] = fma(0.662, dr, out[5504]);
      out[5376] = fma(0.067, dr, out[5376]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52000] * fma(y[5792], v[5120], y[5120] * v[5792]);
      out[5120] = out[5120] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.342, dr, out[5984]);
      out[5888] = fma(0.518, dr, out[5888]);
      out[5632] = fma(0.14, dr, out[5632]);
      out[5216] = fma(0.191, dr, out[5216]);
      out[5856] = fma(0.042, dr, out[5856]);
      out[5760] = fma(0.381, dr, out[5760]);
      out[5504] = fma(0.824, dr, out[5504]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52032] * fma(y[5792], v[3008], y[3008] * v[5792]);
      out[3008] = out[3008] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5856] = fma(1.6, dr, out[5856]);
      out[5760] = fma(0.2, dr, out[5760]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52064] * fma(y[5792], v[3200], y[3200] * v[5792]);
      out[3200] = out[3200] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5760] = fma(0.94, dr, out[5760]);
      out[5504] = fma(0.06, dr, out[5504]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52096] * fma(y[5792], v[3328], y[3328] * v[5792]);
      out[3328] = out[3328] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5760] = fma(1.71, dr, out[5760]);
      out[5504] = fma(0.29, dr, out[5504]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52128] * fma(y[5792], v[3360], y[3360] * v[5792]);
      out[3360] = out[3360] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[4448] = fma(0.0, dr, out[4448]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[4512] = fma(0.5, dr, out[4512]);
      out[4320] = fma(0.25, dr, out[4320]);
      out[3584] = fma(0.25, dr, out[3584]);
    }
    {
      const double dr = ws[52160] * fma(y[5792], v[3296], y[3296] * v[5792]);
      out[3296] = out[3296] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5984] = fma(0.9146, dr, out[5984]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[4448] = fma(0.0854, dr, out[4448]);
      out[5376] = fma(0.5488, dr, out[5376]);
      out[5248] = fma(0.3659, dr, out[5248]);
      out[4512] = fma(0.3659, dr, out[4512]);
      out[5472] = fma(0.5488, dr, out[5472]);
    }
    {
      const double dr = ws[52192] * fma(y[5792], v[3104], y[3104] * v[5792]);
      out[3104] = out[3104] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5984] = fma(0.9518, dr, out[5984]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[4448] = fma(0.0482, dr, out[4448]);
      out[5376] = fma(0.7043, dr, out[5376]);
      out[5248] = fma(0.2475, dr, out[5248]);
      out[4512] = fma(0.3522, dr, out[4512]);
      out[4320] = fma(0.5996, dr, out[4320]);
    }
    {
      const double dr = ws[52224] * fma(y[5792], v[3264], y[3264] * v[5792]);
      out[3264] = out[3264] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5984] = fma(0.9146, dr, out[5984]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[4448] = fma(0.0854, dr, out[4448]);
      out[5376] = fma(0.5488, dr, out[5376]);
      out[5248] = fma(0.3659, dr, out[5248]);
      out[4512] = fma(0.4573, dr, out[4512]);
      out[4320] = fma(0.4573, dr, out[4320]);
    }
    {
      const double dr = ws[52256] * fma(y[5792], v[4288], y[4288] * v[5792]);
      out[4288] = out[4288] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5856] = fma(1.048, dr, out[5856]);
      out[4128] = fma(0.219, dr, out[4128]);
      out[4736] = fma(0.305, dr, out[4736]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52288] * fma(y[5792], v[4160], y[4160] * v[5792]);
      out[4160] = out[4160] - dr;
      out[5792] = out[5792] - dr;
      out[4544] = fma(0.2535, dr, out[4544]);
      out[5760] = fma(0.371, dr, out[5760]);
      out[4096] = fma(0.091, dr, out[4096]);
      out[4480] = fma(0.1165, dr, out[4480]);
      out[4576] = fma(0.1725, dr, out[4576]);
      out[5856] = fma(0.403, dr, out[5856]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5888] = fma(1.0, dr, out[5888]);
      out[5504] = fma(0.112, dr, out[5504]);
    }
    {
      const double dr = ws[52320] * fma(y[5792], v[3744], y[3744] * v[5792]);
      out[3744] = out[3744] - dr;
      out[5792] = out[5792] - dr;
      out[6016] = fma(0.5, dr, out[6016]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5696] = fma(0.5, dr, out[5696]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[52352] * fma(y[5792], v[2624], y[2624] * v[5792]);
      out[2624] = out[2624] - dr;
      out[5792] = out[5792] - dr;
      out[5920] = fma(0.825, dr, out[5920]);
      out[4544] = fma(0.65, dr, out[4544]);
      out[5888] = fma(1.0, dr, out[5888]);
      out[4384] = fma(0.175, dr, out[4384]);
      out[5760] = fma(0.168, dr, out[5760]);
      out[5504] = fma(0.007, dr, out[5504]);
      out[5856] = fma(0.007, dr, out[5856]);
      out[5984] = fma(0.175, dr, out[5984]);
    }
    {
      const double dr = ws[52384] * fma(y[5792], v[3840], y[3840] * v[5792]);
      out[3840] = out[3840] - dr;
      out[5792] = out[5792] - dr;
      out[5920] = fma(0.5, dr, out[5920]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5696] = fma(0.5, dr, out[5696]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[52416] * fma(y[5792], v[4192], y[4192] * v[5792]);
      out[4192] = out[4192] - dr;
      out[5792] = out[5792] - dr;
      out[4576] = fma(1.0, dr, out[4576]);
      out[5856] = fma(0.56, dr, out[5856]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5888] = fma(1.0, dr, out[5888]);
    }
    {
      const double dr = ws[52448] * fma(y[5792], v[3936], y[3936] * v[5792]);
      out[3936] = out[3936] - dr;
      out[5792] = out[5792] - dr;
      out[6016] = fma(0.5, dr, out[6016]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5696] = fma(0.5, dr, out[5696]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[52480] * fma(y[5792], v[2656], y[2656] * v[5792]);
      out[2656] = out[2656] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[5920] = fma(0.46, dr, out[5920]);
      out[4576] = fma(0.46, dr, out[4576]);
      out[4384] = fma(0.54, dr, out[4384]);
      out[5984] = fma(0.54, dr, out[5984]);
    }
    {
      const double dr = ws[52512] * fma(y[5792], v[3712], y[3712] * v[5792]);
      out[3712] = out[3712] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.5, dr, out[5888]);
      out[5920] = fma(0.5, dr, out[5920]);
      out[5696] = fma(0.5, dr, out[5696]);
      out[4256] = fma(1.0, dr, out[4256]);
    }
    {
      const double dr = ws[52544] * fma(y[5792], v[5792], y[5792] * v[5792]);
      out[5792] = out[5792] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(2.0, dr, out[5888]);
    }
    {
      const double dr = ws[52576] * fma(y[5792], v[4800], y[4800] * v[5792]);
      out[4800] = out[4800] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[5632] = fma(1.0, dr, out[5632]);
    }
    {
      const double dr = ws[52608] * fma(y[5792], v[2848], y[2848] * v[5792]);
      out[2848] = out[2848] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.5, dr, out[5888]);
      out[5792] = fma(0.5, dr, out[5792]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5696] = fma(0.75, dr, out[5696]);
    }
    {
      const double dr = ws[52640] * fma(y[5792], v[5152], y[5152] * v[5792]);
      out[5152] = out[5152] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.33, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5856] = fma(0.33, dr, out[5856]);
      out[5472] = fma(0.334, dr, out[5472]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52672] * fma(y[5792], v[3776], y[3776] * v[5792]);
      out[3776] = out[3776] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5472] = fma(0.5, dr, out[5472]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
}
__device__ __noinline__ void ddm_jv_1_5(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[52704] * fma(y[5792], v[4672], y[4672] * v[5792]);
      out[4672] = out[4672] - dr;
      out[5792] = out[5792] - dr;
      out[5696] = fma(0.635, dr, out[5696]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5792] = fma(0.269, dr, out[5792]);
      out[5664] = fma(0.5, dr, out[5664]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[52736] * fma(y[5792], v[3520], y[3520] * v[5792]);
      out[3520] = out[3520] - dr;
      out[5792] = out[5792] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.5, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5344] = fma(0.5, dr, out[5344]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52768] * fma(y[5792], v[2880], y[2880] * v[5792]);
      out[2880] = out[2880] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5792] = fma(1.16, dr, out[5792]);
      out[5216] = fma(1.16, dr, out[5216]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5760] = fma(2.3, dr, out[5760]);
      out[5248] = fma(0.5, dr, out[5248]);
      out[5696] = fma(1.083, dr, out[5696]);
    }
    {
      const double dr = ws[52800] * fma(y[5792], v[2912], y[2912] * v[5792]);
      out[2912] = out[2912] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5888] = fma(0.5, dr, out[5888]);
      out[5664] = fma(0.5, dr, out[5664]);
      out[5856] = fma(0.03, dr, out[5856]);
      out[5760] = fma(0.27, dr, out[5760]);
      out[5504] = fma(0.7, dr, out[5504]);
      out[5376] = fma(0.18, dr, out[5376]);
      out[5248] = fma(0.105, dr, out[5248]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[52832] * fma(y[5792], v[2592], y[2592] * v[5792]);
      out[2592] = out[2592] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[2272] = fma(1.0, dr, out[2272]);
    }
    {
      const double dr = ws[52864] * fma(y[5792], v[2272], y[2272] * v[5792]);
      out[2272] = out[2272] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[2688] = fma(1.0, dr, out[2688]);
    }
    {
      const double dr = ws[52896] * fma(y[5792], v[3648], y[3648] * v[5792]);
      out[3648] = out[3648] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(2.0, dr, out[5984]);
      out[5888] = fma(1.0, dr, out[5888]);
      out[5344] = fma(0.32, dr, out[5344]);
      out[5376] = fma(0.68, dr, out[5376]);
      out[5728] = fma(0.68, dr, out[5728]);
    }
    {
      const double dr = ws[52928] * fma(y[5792], v[3040], y[3040] * v[5792]);
      out[3040] = out[3040] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5888] = fma(1.0, dr, out[5888]);
      out[3808] = fma(1.0, dr, out[3808]);
    }
    {
      const double dr = ws[52960] * fma(y[5792], v[2976], y[2976] * v[5792]);
      out[2976] = out[2976] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[5376] = fma(1.0, dr, out[5376]);
    }
    {
      const double dr = ws[52992] * fma(y[5792], v[4032], y[4032] * v[5792]);
      out[4032] = out[4032] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5888] = fma(1.0, dr, out[5888]);
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[53024] * fma(y[5792], v[4064], y[4064] * v[5792]);
      out[4064] = out[4064] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.5, dr, out[5888]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.287, dr, out[5856]);
      out[5760] = fma(1.24, dr, out[5760]);
      out[5504] = fma(0.464, dr, out[5504]);
      out[5696] = fma(0.5, dr, out[5696]);
    }
    {
      const double dr = ws[53056] * fma(y[5792], v[3072], y[3072] * v[5792]);
      out[3072] = out[3072] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5888] = fma(1.0, dr, out[5888]);
      out[5920] = fma(0.7, dr, out[5920]);
      out[5376] = fma(0.7, dr, out[5376]);
      out[5728] = fma(0.7, dr, out[5728]);
      out[5440] = fma(0.3, dr, out[5440]);
    }
    {
      const double dr = ws[53088] * fma(y[5792], v[5216], y[5216] * v[5792]);
      out[5216] = out[5216] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
    }
    {
      const double dr = ws[53120] * fma(y[4800], v[4800], y[4800] * v[4800]);
      out[4800] = out[4800] - dr;
      out[4800] = out[4800] - dr;
      out[5632] = fma(2.0, dr, out[5632]);
    }
    {
      const double dr = ws[53152] * fma(y[5952], v[5888], y[5888] * v[5952]);
      out[5888] = out[5888] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[53184] * fma(y[5952], v[5632], y[5632] * v[5952]);
      out[5632] = out[5632] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5568] = fma(1.0, dr, out[5568]);
    }
    {
      const double dr = ws[53216] * fma(y[5952], v[5408], y[5408] * v[5952]);
      out[5408] = out[5408] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(0.254, dr, out[5984]);
      out[5888] = fma(0.14, dr, out[5888]);
      out[5216] = fma(0.092, dr, out[5216]);
      out[5632] = fma(0.503, dr, out[5632]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5568] = fma(0.519, dr, out[5568]);
      out[5760] = fma(0.147, dr, out[5760]);
      out[5280] = fma(0.075, dr, out[5280]);
      out[4480] = fma(0.095, dr, out[4480]);
    }
    {
      const double dr = ws[53248] * fma(y[5952], v[5120], y[5120] * v[5952]);
      out[5120] = out[5120] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(0.488, dr, out[5984]);
      out[5888] = fma(0.055, dr, out[5888]);
      out[5632] = fma(0.28, dr, out[5632]);
      out[5216] = fma(0.485, dr, out[5216]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.024, dr, out[5856]);
      out[5760] = fma(0.241, dr, out[5760]);
      out[5504] = fma(0.06, dr, out[5504]);
      out[5280] = fma(0.063, dr, out[5280]);
      out[4480] = fma(0.247, dr, out[4480]);
      out[5568] = fma(0.048, dr, out[5568]);
      out[5344] = fma(0.275, dr, out[5344]);
    }
    {
      const double dr = ws[53280] * fma(y[5952], v[3008], y[3008] * v[5952]);
      out[3008] = out[3008] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(1.6, dr, out[5856]);
      out[5760] = fma(0.2, dr, out[5760]);
    }
    {
      const double dr = ws[53312] * fma(y[5952], v[3200], y[3200] * v[5952]);
      out[3200] = out[3200] - dr;
      out[5952] = out[5952] - dr;
      out[5760] = fma(0.47, dr, out[5760]);
      out[5856] = fma(0.79, dr, out[5856]);
      out[5984] = fma(0.79, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5280] = fma(0.18, dr, out[5280]);
      out[5568] = fma(0.02, dr, out[5568]);
      out[4480] = fma(0.09, dr, out[4480]);
    }
    {
      const double dr = ws[53344] * fma(y[5952], v[3328], y[3328] * v[5952]);
      out[3328] = out[3328] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(0.86, dr, out[5984]);
      out[5760] = fma(0.72, dr, out[5760]);
      out[5504] = fma(0.11, dr, out[5504]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[4480] = fma(0.2, dr, out[4480]);
      out[5568] = fma(0.85, dr, out[5568]);
      out[5344] = fma(0.04, dr, out[5344]);
    }
    {
      const double dr = ws[53376] * fma(y[5952], v[3360], y[3360] * v[5952]);
      out[3360] = out[3360] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[4448] = fma(0.0, dr, out[4448]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[4512] = fma(0.5, dr, out[4512]);
      out[4320] = fma(0.25, dr, out[4320]);
      out[3584] = fma(0.25, dr, out[3584]);
    }
    {
      const double dr = ws[53408] * fma(y[5952], v[3296], y[3296] * v[5952]);
      out[3296] = out[3296] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.9146, dr, out[5984]);
      out[4448] = fma(0.0854, dr, out[4448]);
      out[5376] = fma(0.5488, dr, out[5376]);
      out[5248] = fma(0.3659, dr, out[5248]);
      out[4512] = fma(0.3659, dr, out[4512]);
      out[5472] = fma(0.5488, dr, out[5472]);
    }
    {
      const double dr = ws[53440] * fma(y[5952], v[3104], y[3104] * v[5952]);
      out[3104] = out[3104] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.9518, dr, out[5984]);
      out[4448] = fma(0.0482, dr, out[4448]);
      out[5376] = fma(0.7043, dr, out[5376]);
      out[5248] = fma(0.2475, dr, out[5248]);
      out[4512] = fma(0.3522, dr, out[4512]);
      out[4320] = fma(0.5996, dr, out[4320]);
    }
    {
      const double dr = ws[53472] * fma(y[5952], v[3264], y[3264] * v[5952]);
      out[3264] = out[3264] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.9146, dr, out[5984]);
      out[4448] = fma(0.0854, dr, out[4448]);
      out[5376] = fma(0.5488, dr, out[5376]);
      out[5248] = fma(0.3659, dr, out[5248]);
      out[4512] = fma(0.4573, dr, out[4512]);
      out[4320] = fma(0.4573, dr, out[4320]);
    }
    {
      const double dr = ws[53504] * fma(y[5952], v[4288], y[4288] * v[5952]);
      out[4288] = out[4288] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.75, dr, out[5856]);
      out[4128] = fma(0.318, dr, out[4128]);
      out[4736] = fma(0.5, dr, out[4736]);
      out[5376] = fma(0.024, dr, out[5376]);
      out[5344] = fma(0.033, dr, out[5344]);
      out[5760] = fma(0.031, dr, out[5760]);
    }
    {
      const double dr = ws[53536] * fma(y[5952], v[4160], y[4160] * v[5952]);
      out[4160] = out[4160] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[4544] = fma(0.2535, dr, out[4544]);
      out[5760] = fma(0.371, dr, out[5760]);
      out[4480] = fma(0.1165, dr, out[4480]);
      out[4576] = fma(0.1725, dr, out[4576]);
      out[5856] = fma(0.403, dr, out[5856]);
      out[4096] = fma(0.091, dr, out[4096]);
      out[5504] = fma(0.112, dr, out[5504]);
    }
    {
      const double dr = ws[53568] * fma(y[5952], v[4192], y[4192] * v[5952]);
      out[4192] = out[4192] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[5856] = fma(0.56, dr, out[5856]);
    }
    {
      const double dr = ws[53600] * fma(y[5952], v[2624], y[2624] * v[5952]);
      out[2624] = out[2624] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.825, dr, out[5920]);
      out[4544] = fma(0.65, dr, out[4544]);
      out[4384] = fma(0.175, dr, out[4384]);
      out[5760] = fma(0.168, dr, out[5760]);
      out[5504] = fma(0.007, dr, out[5504]);
      out[5856] = fma(0.007, dr, out[5856]);
      out[5984] = fma(0.175, dr, out[5984]);
    }
    {
      const double dr = ws[53632] * fma(y[5952], v[2656], y[2656] * v[5952]);
      out[2656] = out[2656] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.46, dr, out[5920]);
      out[4576] = fma(0.46, dr, out[4576]);
      out[4384] = fma(0.54, dr, out[4384]);
      out[5984] = fma(0.54, dr, out[5984]);
    }
    {
      const double dr = ws[53664] * fma(y[5952], v[5792], y[5792] * v[5952]);
      out[5792] = out[5792] - dr;
      out[5952] = out[5952] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[53696] * fma(y[5952], v[4800], y[4800] * v[5952]);
      out[4800] = out[4800] - dr;
      out[5952] = out[5952] - dr;
      out[5632] = fma(1.0, dr, out[5632]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[53728] * fma(y[5952], v[2848], y[2848] * v[5952]);
      out[2848] = out[2848] - dr;
      out[5952] = out[5952] - dr;
      out[5792] = fma(1.0, dr, out[5792]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(1.0, dr, out[5856]);
    }
    {
      const double dr = ws[53760] * fma(y[5952], v[5152], y[5152] * v[5952]);
      out[5152] = out[5152] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(0.67, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.33, dr, out[5856]);
      out[5472] = fma(0.67, dr, out[5472]);
    }
    {
      const double dr = ws[53792] * fma(y[5952], v[3776], y[3776] * v[5952]);
      out[3776] = out[3776] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5472] = fma(1.0, dr, out[5472]);
    }
    {
      const double dr = ws[53824] * fma(y[5952], v[4672], y[4672] * v[5952]);
      out[4672] = out[4672] - dr;
      out[5952] = out[5952] - dr;
      out[5856] = fma(1.0, dr, out[5856]);
      out[5792] = fma(0.538, dr, out[5792]);
      out[5664] = fma(1.0, dr, out[5664]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[53856] * fma(y[5952], v[3520], y[3520] * v[5952]);
      out[3520] = out[3520] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[5344] = fma(1.0, dr, out[5344]);
    }
    {
      const double dr = ws[53888] * fma(y[5952], v[2880], y[2880] * v[5952]);
      out[2880] = out[2880] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(0.3, dr, out[5984]);
      out[5792] = fma(0.7, dr, out[5792]);
      out[5216] = fma(0.7, dr, out[5216]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.3, dr, out[5856]);
      out[5760] = fma(0.7, dr, out[5760]);
      out[5248] = fma(0.3, dr, out[5248]);
    }
    {
      const double dr = ws[53920] * fma(y[5952], v[2912], y[2912] * v[5952]);
      out[2912] = out[2912] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5664] = fma(0.61, dr, out[5664]);
      out[5856] = fma(0.03, dr, out[5856]);
      out[5760] = fma(0.27, dr, out[5760]);
      out[5504] = fma(0.7, dr, out[5504]);
      out[5376] = fma(0.18, dr, out[5376]);
      out[5248] = fma(0.21, dr, out[5248]);
    }
    {
      const double dr = ws[53952] * fma(y[5952], v[2592], y[2592] * v[5952]);
      out[2592] = out[2592] - dr;
      out[5952] = out[5952] - dr;
      out[2272] = fma(1.0, dr, out[2272]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[53984] * fma(y[5952], v[2272], y[2272] * v[5952]);
      out[2272] = out[2272] - dr;
      out[5952] = out[5952] - dr;
      out[2688] = fma(1.0, dr, out[2688]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[54016] * fma(y[5952], v[3648], y[3648] * v[5952]);
      out[3648] = out[3648] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5344] = fma(0.32, dr, out[5344]);
      out[5376] = fma(0.68, dr, out[5376]);
      out[5728] = fma(0.68, dr, out[5728]);
    }
    {
      const double dr = ws[54048] * fma(y[5952], v[3040], y[3040] * v[5952]);
      out[3040] = out[3040] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[3808] = fma(1.0, dr, out[3808]);
    }
    {
      const double dr = ws[54080] * fma(y[5952], v[2976], y[2976] * v[5952]);
      out[2976] = out[2976] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[54112] * fma(y[5952], v[4032], y[4032] * v[5952]);
      out[4032] = out[4032] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[54144] * fma(y[5952], v[4064], y[4064] * v[5952]);
      out[4064] = out[4064] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
      out[5856] = fma(0.287, dr, out[5856]);
      out[5760] = fma(1.24, dr, out[5760]);
      out[5504] = fma(0.464, dr, out[5504]);
    }
    {
      const double dr = ws[54176] * fma(y[5952], v[3072], y[3072] * v[5952]);
      out[3072] = out[3072] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(2.0, dr, out[5920]);
      out[5376] = fma(1.0, dr, out[5376]);
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[54208] * fma(y[4032], v[4032], y[4032] * v[4032]);
      out[4032] = out[4032] - dr;
      out[4032] = out[4032] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5440] = fma(2.0, dr, out[5440]);
    }
    {
      const double dr = ws[54240] * fma(y[4064], v[4032], y[4032] * v[4064]);
      out[4032] = out[4032] - dr;
      out[4064] = out[4064] - dr;
      out[5984] = fma(0.5, dr, out[5984]);
      out[5920] = fma(0.5, dr, out[5920]);
      out[5856] = fma(0.202, dr, out[5856]);
      out[5760] = fma(0.64, dr, out[5760]);
      out[5504] = fma(0.149, dr, out[5504]);
      out[5440] = fma(1.5, dr, out[5440]);
    }
    {
      const double dr = ws[54272] * fma(y[4064], v[4064], y[4064] * v[4064]);
      out[4064] = out[4064] - dr;
      out[4064] = out[4064] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5856] = fma(0.504, dr, out[5856]);
      out[5760] = fma(1.21, dr, out[5760]);
      out[5504] = fma(0.285, dr, out[5504]);
      out[5440] = fma(1.0, dr, out[5440]);
    }
    {
      const double dr = ws[54304] * fma(y[5952], v[5216], y[5216] * v[5952]);
      out[5216] = out[5216] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[54336] * fma(y[4800], v[5216], y[5216] * v[4800]);
      out[5216] = out[5216] - dr;
      out[4800] = out[4800] - dr;
      out[5632] = fma(1.0, dr, out[5632]);
    }
}
__device__ __noinline__ void ddm_jv_1_6(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[54368] * fma(y[5216], v[5216], y[5216] * v[5216]);
      out[5216] = out[5216] - dr;
      out[5216] = out[5216] - dr;
    }
    {
      const double dr = ws[54400] * fma(y[4160], v[3744], y[3744] * v[4160]);
      out[3744] = out[3744] - dr;
      out[4160] = out[4160] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4544] = fma(0.48, dr, out[4544]);
      out[6016] = fma(0.48, dr, out[6016]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54432] * fma(y[4192], v[3744], y[3744] * v[4192]);
      out[3744] = out[3744] - dr;
      out[4192] = out[4192] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4576] = fma(0.48, dr, out[4576]);
      out[6016] = fma(0.48, dr, out[6016]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54464] * fma(y[4288], v[3744], y[3744] * v[4288]);
      out[3744] = out[3744] - dr;
      out[4288] = out[4288] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[5856] = fma(0.48, dr, out[5856]);
      out[4736] = fma(0.48, dr, out[4736]);
      out[6016] = fma(0.48, dr, out[6016]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54496] * fma(y[4160], v[3936], y[3936] * v[4160]);
      out[3936] = out[3936] - dr;
      out[4160] = out[4160] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4544] = fma(0.48, dr, out[4544]);
      out[6016] = fma(0.48, dr, out[6016]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54528] * fma(y[4192], v[3936], y[3936] * v[4192]);
      out[3936] = out[3936] - dr;
      out[4192] = out[4192] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4576] = fma(0.48, dr, out[4576]);
      out[6016] = fma(0.48, dr, out[6016]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54560] * fma(y[4288], v[3936], y[3936] * v[4288]);
      out[3936] = out[3936] - dr;
      out[4288] = out[4288] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[5856] = fma(0.48, dr, out[5856]);
      out[4736] = fma(0.48, dr, out[4736]);
      out[6016] = fma(0.48, dr, out[6016]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54592] * fma(y[4160], v[3840], y[3840] * v[4160]);
      out[3840] = out[3840] - dr;
      out[4160] = out[4160] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4544] = fma(0.48, dr, out[4544]);
      out[5920] = fma(0.48, dr, out[5920]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54624] * fma(y[4192], v[3840], y[3840] * v[4192]);
      out[3840] = out[3840] - dr;
      out[4192] = out[4192] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4576] = fma(0.48, dr, out[4576]);
      out[5920] = fma(0.48, dr, out[5920]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54656] * fma(y[4288], v[3840], y[3840] * v[4288]);
      out[3840] = out[3840] - dr;
      out[4288] = out[4288] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[5856] = fma(0.48, dr, out[5856]);
      out[4736] = fma(0.48, dr, out[4736]);
      out[5920] = fma(0.48, dr, out[5920]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54688] * fma(y[4160], v[3712], y[3712] * v[4160]);
      out[3712] = out[3712] - dr;
      out[4160] = out[4160] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4544] = fma(0.48, dr, out[4544]);
      out[5920] = fma(0.48, dr, out[5920]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54720] * fma(y[4192], v[3712], y[3712] * v[4192]);
      out[3712] = out[3712] - dr;
      out[4192] = out[4192] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[4576] = fma(0.48, dr, out[4576]);
      out[5920] = fma(0.48, dr, out[5920]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54752] * fma(y[4288], v[3712], y[3712] * v[4288]);
      out[3712] = out[3712] - dr;
      out[4288] = out[4288] - dr;
      out[4256] = fma(0.96, dr, out[4256]);
      out[5056] = fma(0.48, dr, out[5056]);
      out[5856] = fma(0.48, dr, out[5856]);
      out[4736] = fma(0.48, dr, out[4736]);
      out[5920] = fma(0.48, dr, out[5920]);
      out[5984] = fma(0.48, dr, out[5984]);
      out[2720] = fma(0.04, dr, out[2720]);
    }
    {
      const double dr = ws[54784] * fma(y[6016], v[1376], y[1376] * v[6016]);
      out[1376] = out[1376] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
    }
    {
      const double dr = ws[54816] * fma(y[6016], v[384], y[384] * v[6016]);
      out[384] = out[384] - dr;
      out[6016] = out[6016] - dr;
      out[5632] = fma(0.852, dr, out[5632]);
      out[3616] = fma(0.149, dr, out[3616]);
    }
    {
      const double dr = ws[54848] * fma(y[6016], v[416], y[416] * v[6016]);
      out[416] = out[416] - dr;
      out[6016] = out[6016] - dr;
      out[5632] = fma(1.0, dr, out[5632]);
      out[3616] = fma(0.00101, dr, out[3616]);
    }
    {
      const double dr = ws[54880] * fma(y[6016], v[3552], y[3552] * v[6016]);
      out[3552] = out[3552] - dr;
      out[6016] = out[6016] - dr;
      out[4672] = fma(0.57, dr, out[4672]);
      out[3520] = fma(0.43, dr, out[3520]);
    }
    {
      const double dr = ws[54912] * fma(y[5184], v[3552], y[3552] * v[5184]);
      out[3552] = out[3552] - dr;
      out[5184] = out[5184] - dr;
      out[5664] = fma(0.84, dr, out[5664]);
      out[5984] = fma(0.56, dr, out[5984]);
      out[6016] = fma(0.28, dr, out[6016]);
      out[5856] = fma(0.72, dr, out[5856]);
      out[5376] = fma(0.62, dr, out[5376]);
    }
    {
      const double dr = ws[54944] * fma(y[5952], v[3552], y[3552] * v[5952]);
      out[3552] = out[3552] - dr;
      out[5952] = out[5952] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[4672] = fma(0.32, dr, out[4672]);
      out[5216] = fma(0.68, dr, out[5216]);
      out[5248] = fma(0.68, dr, out[5248]);
      out[5024] = fma(0.32, dr, out[5024]);
      out[5920] = fma(0.68, dr, out[5920]);
    }
    {
      const double dr = ws[55008] * fma(y[6016], v[1568], y[1568] * v[6016]);
      out[1568] = out[1568] - dr;
      out[6016] = out[6016] - dr;
      out[3136] = fma(0.667, dr, out[3136]);
      out[3872] = fma(0.333, dr, out[3872]);
      out[5984] = fma(0.333, dr, out[5984]);
    }
    {
      const double dr = ws[55040] * fma(y[5824], v[3136], y[3136] * v[5824]);
      out[3136] = out[3136] - dr;
      out[5824] = out[5824] - dr;
      out[5984] = fma(0.968, dr, out[5984]);
      out[5920] = fma(0.968, dr, out[5920]);
      out[3552] = fma(0.895, dr, out[3552]);
      out[5856] = fma(0.895, dr, out[5856]);
      out[3168] = fma(0.072, dr, out[3168]);
      out[5440] = fma(0.032, dr, out[5440]);
    }
    {
      const double dr = ws[55072] * fma(y[5952], v[3136], y[3136] * v[5952]);
      out[3136] = out[3136] - dr;
      out[5952] = out[5952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5920] = fma(1.0, dr, out[5920]);
      out[3552] = fma(0.925, dr, out[3552]);
      out[5856] = fma(0.925, dr, out[5856]);
      out[3168] = fma(0.075, dr, out[3168]);
    }
    {
      const double dr = ws[55104] * fma(y[5984], v[3136], y[3136] * v[5984]);
      out[3136] = out[3136] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[55136] * fma(y[5888], v[3136], y[3136] * v[5888]);
      out[3136] = out[3136] - dr;
      out[5888] = out[5888] - dr;
      out[5600] = fma(0.32, dr, out[5600]);
      out[5856] = fma(1.143, dr, out[5856]);
      out[5984] = fma(0.87, dr, out[5984]);
      out[3552] = fma(0.463, dr, out[3552]);
      out[2752] = fma(0.25, dr, out[2752]);
      out[4736] = fma(0.231, dr, out[4736]);
      out[3168] = fma(0.037, dr, out[3168]);
      out[3872] = fma(0.019, dr, out[3872]);
    }
    {
      const double dr = ws[55168] * fma(y[5792], v[3136], y[3136] * v[5792]);
      out[3136] = out[3136] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[5984] = fma(0.8, dr, out[5984]);
      out[3552] = fma(0.74, dr, out[3552]);
      out[5856] = fma(0.74, dr, out[5856]);
      out[4736] = fma(0.185, dr, out[4736]);
      out[3168] = fma(0.06, dr, out[3168]);
      out[3872] = fma(0.015, dr, out[3872]);
    }
    {
      const double dr = ws[55200] * fma(y[5184], v[1568], y[1568] * v[5184]);
      out[1568] = out[1568] - dr;
      out[5184] = out[5184] - dr;
      out[3552] = fma(0.62, dr, out[3552]);
      out[5664] = fma(0.63, dr, out[5664]);
      out[5984] = fma(0.42, dr, out[5984]);
      out[6016] = fma(0.08, dr, out[6016]);
      out[5856] = fma(0.83, dr, out[5856]);
      out[2240] = fma(0.17, dr, out[2240]);
    }
    {
      const double dr = ws[55232] * fma(y[5952], v[1568], y[1568] * v[5952]);
      out[1568] = out[1568] - dr;
      out[5952] = out[5952] - dr;
      out[4032] = fma(0.9, dr, out[4032]);
      out[4064] = fma(0.1, dr, out[4064]);
      out[3552] = fma(0.9, dr, out[3552]);
    }
    {
      const double dr = ws[55264] * fma(y[6016], v[3168], y[3168] * v[6016]);
      out[3168] = out[3168] - dr;
      out[6016] = out[6016] - dr;
      out[5472] = fma(0.49, dr, out[5472]);
      out[5984] = fma(0.49, dr, out[5984]);
      out[1856] = fma(0.51, dr, out[1856]);
    }
    {
      const double dr = ws[55296] * fma(y[5824], v[1856], y[1856] * v[5824]);
      out[1856] = out[1856] - dr;
      out[5824] = out[5824] - dr;
      out[5440] = fma(0.08, dr, out[5440]);
      out[5920] = fma(0.92, dr, out[5920]);
      out[4512] = fma(0.92, dr, out[4512]);
      out[5984] = fma(0.75, dr, out[5984]);
      out[5888] = fma(0.17, dr, out[5888]);
    }
    {
      const double dr = ws[55328] * fma(y[5984], v[1856], y[1856] * v[5984]);
      out[1856] = out[1856] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(0.6, dr, out[5728]);
      out[4512] = fma(0.4, dr, out[4512]);
      out[6016] = fma(0.4, dr, out[6016]);
      out[5984] = fma(0.32, dr, out[5984]);
      out[5888] = fma(0.08, dr, out[5888]);
    }
    {
      const double dr = ws[55360] * fma(y[6016], v[4512], y[4512] * v[6016]);
      out[4512] = out[4512] - dr;
      out[6016] = out[6016] - dr;
      out[5504] = fma(0.65, dr, out[5504]);
      out[5376] = fma(0.31, dr, out[5376]);
      out[5984] = fma(0.66, dr, out[5984]);
      out[5888] = fma(0.34, dr, out[5888]);
      out[5664] = fma(0.43, dr, out[5664]);
      out[3616] = fma(0.04, dr, out[3616]);
    }
    {
      const double dr = ws[55392] * fma(y[5184], v[3168], y[3168] * v[5184]);
      out[3168] = out[3168] - dr;
      out[5184] = out[5184] - dr;
      out[6016] = fma(0.02, dr, out[6016]);
      out[5760] = fma(1.0, dr, out[5760]);
    }
    {
      const double dr = ws[55424] * fma(y[5952], v[3168], y[3168] * v[5952]);
      out[3168] = out[3168] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5472] = fma(0.8, dr, out[5472]);
      out[3584] = fma(0.2, dr, out[3584]);
    }
    {
      const double dr = ws[55456] * fma(y[6016], v[448], y[448] * v[6016]);
      out[448] = out[448] - dr;
      out[6016] = out[6016] - dr;
      out[5344] = fma(0.613, dr, out[5344]);
      out[5760] = fma(0.387, dr, out[5760]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[55488] * fma(y[5952], v[1600], y[1600] * v[5952]);
      out[1600] = out[1600] - dr;
      out[5952] = out[5952] - dr;
      out[1920] = fma(1.0, dr, out[1920]);
    }
    {
      const double dr = ws[55520] * fma(y[5984], v[1920], y[1920] * v[5984]);
      out[1920] = out[1920] - dr;
      out[5984] = out[5984] - dr;
      out[4928] = fma(1.0, dr, out[4928]);
    }
    {
      const double dr = ws[55552] * fma(y[5824], v[1920], y[1920] * v[5824]);
      out[1920] = out[1920] - dr;
      out[5824] = out[5824] - dr;
      out[5536] = fma(1.0, dr, out[5536]);
      out[5920] = fma(2.0, dr, out[5920]);
    }
    {
      const double dr = ws[55584] * fma(y[5952], v[1920], y[1920] * v[5952]);
      out[1920] = out[1920] - dr;
      out[5952] = out[5952] - dr;
      out[5536] = fma(1.0, dr, out[5536]);
      out[5920] = fma(2.0, dr, out[5920]);
    }
    {
      const double dr = ws[55616] * fma(y[5184], v[1600], y[1600] * v[5184]);
      out[1600] = out[1600] - dr;
      out[5184] = out[5184] - dr;
      out[5536] = fma(0.982, dr, out[5536]);
      out[4832] = fma(0.018, dr, out[4832]);
    }
    {
      const double dr = ws[55648] * fma(y[6016], v[1600], y[1600] * v[6016]);
      out[1600] = out[1600] - dr;
      out[6016] = out[6016] - dr;
      out[2304] = fma(1.0, dr, out[2304]);
    }
    {
      const double dr = ws[55680] * fma(y[5984], v[2304], y[2304] * v[5984]);
      out[2304] = out[2304] - dr;
      out[5984] = out[5984] - dr;
      out[4960] = fma(1.0, dr, out[4960]);
    }
    {
      const double dr = ws[55712] * fma(y[5952], v[2304], y[2304] * v[5952]);
      out[2304] = out[2304] - dr;
      out[5952] = out[5952] - dr;
      out[5536] = fma(1.0, dr, out[5536]);
    }
    {
      const double dr = ws[55744] * fma(y[5824], v[2304], y[2304] * v[5824]);
      out[2304] = out[2304] - dr;
      out[5824] = out[5824] - dr;
      out[4992] = fma(0.247, dr, out[4992]);
      out[5536] = fma(0.753, dr, out[5536]);
      out[5920] = fma(0.753, dr, out[5920]);
    }
    {
      const double dr = ws[55776] * v[5376];
      out[5376] = out[5376] - dr;
      out[480] = fma(1.0, dr, out[480]);
    }
    {
      const double dr = ws[55808] * v[5248];
      out[5248] = out[5248] - dr;
      out[480] = fma(1.0, dr, out[480]);
    }
    {
      const double dr = ws[55840] * v[1024];
      out[1024] = out[1024] - dr;
      out[5024] = fma(2.0, dr, out[5024]);
    }
    {
      const double dr = ws[55872] * v[5920];
      out[5920] = out[5920] - dr;
      out[1184] = fma(0.5, dr, out[1184]);
      out[5024] = fma(0.5, dr, out[5024]);
    }
    {
      const double dr = ws[55904] * v[5984];
      out[5984] = out[5984] - dr;
    }
    {
      const double dr = ws[55936] * v[5952];
      out[5952] = out[5952] - dr;
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[56000] * v[1376];
      out[1376] = out[1376] - dr;
      out[1056] = fma(1.0, dr, out[1056]);
    }
    {
      const double dr = ws[56032] * v[1056];
      out[1056] = out[1056] - dr;
      out[0] = fma(1.0, dr, out[0]);
    }
    {
      const double dr = ws[56064] * fma(y[512], v[1056], y[1056] * v[512]);
      out[1056] = out[1056] - dr;
      out[512] = out[512] - dr;
      out[544] = fma(1.0, dr, out[544]);
    }
    {
      const double dr = ws[56096] * v[1664];
      out[1664] = out[1664] - dr;
      out[32] = fma(1.0, dr, out[32]);
    }
    {
      const double dr = ws[56128] * v[2208];
      out[2208] = out[2208] - dr;
      out[64] = fma(1.0, dr, out[64]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[56160] * fma(y[6016], v[608], y[608] * v[6016]);
      out[608] = out[608] - dr;
      out[6016] = out[6016] - dr;
      out[2368] = fma(1.0, dr, out[2368]);
    }
    {
      const double dr = ws[56192] * fma(y[6016], v[640], y[640] * v[6016]);
      out[640] = out[640] - dr;
      out[6016] = out[6016] - dr;
      out[2400] = fma(1.0, dr, out[2400]);
    }
    {
      const double dr = ws[56224] * fma(y[6016], v[672], y[672] * v[6016]);
      out[672] = out[672] - dr;
      out[6016] = out[6016] - dr;
      out[2432] = fma(1.0, dr, out[2432]);
    }
    {
      const double dr = ws[56256] * fma(y[6016], v[704], y[704] * v[6016]);
      out[704] = out[704] - dr;
      out[6016] = out[6016] - dr;
      out[2464] = fma(1.0, dr, out[2464]);
    }
    {
      const double dr = ws[56288] * fma(y[6016], v[736], y[736] * v[6016]);
      out[736] = out[736] - dr;
      out[6016] = out[6016] - dr;
      out[2496] = fma(1.0, dr, out[2496]);
    }
    {
      const double dr = ws[56320] * fma(y[6016], v[768], y[768] * v[6016]);
      out[768] = out[768] - dr;
      out[6016] = out[6016] - dr;
      out[2528] = fma(1.0, dr, out[2528]);
    }
    {
      const double dr = ws[56352] * fma(y[6016], v[800], y[800] * v[6016]);
      out[800] = out[800] - dr;
      out[6016] = out[6016] - dr;
      out[3904] = fma(1.0, dr, out[3904]);
    }
    {
      const double dr = ws[56384] * fma(y[5824], v[2368], y[2368] * v[5824]);
      out[2368] = out[2368] - dr;
      out[5824] = out[5824] - dr;
      out[1952] = fma(0.72, dr, out[1952]);
      out[5312] = fma(0.28, dr, out[5312]);
      out[5920] = fma(0.72, dr, out[5920]);
    }
}
__device__ __noinline__ void ddm_jv_1_7(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[56416] * fma(y[5824], v[2400], y[2400] * v[5824]);
      out[2400] = out[2400] - dr;
      out[5824] = out[5824] - dr;
      out[1984] = fma(0.72, dr, out[1984]);
      out[5536] = fma(0.28, dr, out[5536]);
      out[5920] = fma(0.72, dr, out[5920]);
    }
    {
      const double dr = ws[56448] * fma(y[5824], v[2432], y[2432] * v[5824]);
      out[2432] = out[2432] - dr;
      out[5824] = out[5824] - dr;
      out[2016] = fma(0.72, dr, out[2016]);
      out[5088] = fma(0.28, dr, out[5088]);
      out[5920] = fma(0.72, dr, out[5920]);
    }
    {
      const double dr = ws[56480] * fma(y[5824], v[2464], y[2464] * v[5824]);
      out[2464] = out[2464] - dr;
      out[5824] = out[5824] - dr;
      out[2048] = fma(0.72, dr, out[2048]);
      out[4704] = fma(0.28, dr, out[4704]);
      out[5920] = fma(0.72, dr, out[5920]);
    }
    {
      const double dr = ws[56512] * fma(y[5824], v[2496], y[2496] * v[5824]);
      out[2496] = out[2496] - dr;
      out[5824] = out[5824] - dr;
      out[2080] = fma(0.72, dr, out[2080]);
      out[4960] = fma(0.28, dr, out[4960]);
      out[5920] = fma(0.72, dr, out[5920]);
    }
    {
      const double dr = ws[56544] * fma(y[5824], v[2528], y[2528] * v[5824]);
      out[2528] = out[2528] - dr;
      out[5824] = out[5824] - dr;
      out[2112] = fma(0.72, dr, out[2112]);
      out[4416] = fma(0.28, dr, out[4416]);
      out[5920] = fma(0.72, dr, out[5920]);
    }
    {
      const double dr = ws[56576] * fma(y[5824], v[3904], y[3904] * v[5824]);
      out[3904] = out[3904] - dr;
      out[5824] = out[5824] - dr;
      out[2144] = fma(0.74, dr, out[2144]);
      out[5440] = fma(0.26, dr, out[5440]);
      out[5920] = fma(0.74, dr, out[5920]);
    }
    {
      const double dr = ws[56608] * fma(y[5952], v[2368], y[2368] * v[5952]);
      out[2368] = out[2368] - dr;
      out[5952] = out[5952] - dr;
      out[1952] = fma(1.0, dr, out[1952]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56640] * fma(y[5952], v[2400], y[2400] * v[5952]);
      out[2400] = out[2400] - dr;
      out[5952] = out[5952] - dr;
      out[1984] = fma(1.0, dr, out[1984]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56672] * fma(y[5952], v[2432], y[2432] * v[5952]);
      out[2432] = out[2432] - dr;
      out[5952] = out[5952] - dr;
      out[2016] = fma(1.0, dr, out[2016]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56704] * fma(y[5952], v[2464], y[2464] * v[5952]);
      out[2464] = out[2464] - dr;
      out[5952] = out[5952] - dr;
      out[2048] = fma(1.0, dr, out[2048]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56736] * fma(y[5952], v[2496], y[2496] * v[5952]);
      out[2496] = out[2496] - dr;
      out[5952] = out[5952] - dr;
      out[2080] = fma(1.0, dr, out[2080]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56768] * fma(y[5952], v[2528], y[2528] * v[5952]);
      out[2528] = out[2528] - dr;
      out[5952] = out[5952] - dr;
      out[2112] = fma(1.0, dr, out[2112]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56800] * fma(y[5952], v[3904], y[3904] * v[5952]);
      out[3904] = out[3904] - dr;
      out[5952] = out[5952] - dr;
      out[2144] = fma(1.0, dr, out[2144]);
      out[5920] = fma(1.0, dr, out[5920]);
    }
    {
      const double dr = ws[56832] * fma(y[5984], v[2368], y[2368] * v[5984]);
      out[2368] = out[2368] - dr;
      out[5984] = out[5984] - dr;
      out[5536] = fma(1.0, dr, out[5536]);
    }
    {
      const double dr = ws[56864] * fma(y[5984], v[2400], y[2400] * v[5984]);
      out[2400] = out[2400] - dr;
      out[5984] = out[5984] - dr;
      out[5088] = fma(1.0, dr, out[5088]);
    }
    {
      const double dr = ws[56896] * fma(y[5984], v[2432], y[2432] * v[5984]);
      out[2432] = out[2432] - dr;
      out[5984] = out[5984] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[56928] * fma(y[5984], v[2464], y[2464] * v[5984]);
      out[2464] = out[2464] - dr;
      out[5984] = out[5984] - dr;
      out[4960] = fma(1.0, dr, out[4960]);
    }
    {
      const double dr = ws[56960] * fma(y[5984], v[2496], y[2496] * v[5984]);
      out[2496] = out[2496] - dr;
      out[5984] = out[5984] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
    }
    {
      const double dr = ws[56992] * fma(y[5984], v[2528], y[2528] * v[5984]);
      out[2528] = out[2528] - dr;
      out[5984] = out[5984] - dr;
      out[4832] = fma(1.0, dr, out[4832]);
    }
    {
      const double dr = ws[57024] * fma(y[5984], v[3904], y[3904] * v[5984]);
      out[3904] = out[3904] - dr;
      out[5984] = out[5984] - dr;
      out[5728] = fma(1.0, dr, out[5728]);
    }
    {
      const double dr = ws[57056] * v[1952];
      out[1952] = out[1952] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5536] = fma(1.0, dr, out[5536]);
    }
    {
      const double dr = ws[57088] * v[1984];
      out[1984] = out[1984] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5088] = fma(1.0, dr, out[5088]);
    }
    {
      const double dr = ws[57120] * v[2016];
      out[2016] = out[2016] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[57152] * v[2048];
      out[2048] = out[2048] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[4960] = fma(1.0, dr, out[4960]);
    }
    {
      const double dr = ws[57184] * v[2080];
      out[2080] = out[2080] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[4416] = fma(1.0, dr, out[4416]);
    }
    {
      const double dr = ws[57216] * v[2112];
      out[2112] = out[2112] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[4832] = fma(1.0, dr, out[4832]);
    }
    {
      const double dr = ws[57248] * v[2144];
      out[2144] = out[2144] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5312] = fma(1.0, dr, out[5312]);
    }
    {
      const double dr = ws[57280] * fma(y[5824], v[1952], y[1952] * v[5824]);
      out[1952] = out[1952] - dr;
      out[5824] = out[5824] - dr;
      out[5088] = fma(0.14, dr, out[5088]);
      out[5920] = fma(0.86, dr, out[5920]);
      out[5536] = fma(0.86, dr, out[5536]);
      out[5984] = fma(0.86, dr, out[5984]);
    }
    {
      const double dr = ws[57312] * fma(y[5824], v[1984], y[1984] * v[5824]);
      out[1984] = out[1984] - dr;
      out[5824] = out[5824] - dr;
      out[4992] = fma(0.14, dr, out[4992]);
      out[5920] = fma(0.86, dr, out[5920]);
      out[5088] = fma(0.86, dr, out[5088]);
      out[5984] = fma(0.86, dr, out[5984]);
    }
    {
      const double dr = ws[57344] * fma(y[5824], v[2016], y[2016] * v[5824]);
      out[2016] = out[2016] - dr;
      out[5824] = out[5824] - dr;
      out[4960] = fma(0.14, dr, out[4960]);
      out[5920] = fma(0.86, dr, out[5920]);
      out[4704] = fma(0.86, dr, out[4704]);
      out[5984] = fma(0.86, dr, out[5984]);
    }
    {
      const double dr = ws[57376] * fma(y[5824], v[2048], y[2048] * v[5824]);
      out[2048] = out[2048] - dr;
      out[5824] = out[5824] - dr;
      out[4416] = fma(0.14, dr, out[4416]);
      out[5920] = fma(0.86, dr, out[5920]);
      out[4960] = fma(0.86, dr, out[4960]);
      out[5984] = fma(0.86, dr, out[5984]);
    }
    {
      const double dr = ws[57408] * fma(y[5824], v[2080], y[2080] * v[5824]);
      out[2080] = out[2080] - dr;
      out[5824] = out[5824] - dr;
      out[4832] = fma(0.14, dr, out[4832]);
      out[5920] = fma(0.86, dr, out[5920]);
      out[4416] = fma(0.86, dr, out[4416]);
      out[5984] = fma(0.86, dr, out[5984]);
    }
    {
      const double dr = ws[57440] * fma(y[5824], v[2112], y[2112] * v[5824]);
      out[2112] = out[2112] - dr;
      out[5824] = out[5824] - dr;
      out[4832] = fma(1.0, dr, out[4832]);
      out[5920] = fma(0.86, dr, out[5920]);
      out[5984] = fma(0.86, dr, out[5984]);
    }
    {
      const double dr = ws[57472] * fma(y[5824], v[2144], y[2144] * v[5824]);
      out[2144] = out[2144] - dr;
      out[5824] = out[5824] - dr;
      out[5440] = fma(0.12, dr, out[5440]);
      out[5920] = fma(0.88, dr, out[5920]);
      out[5504] = fma(0.88, dr, out[5504]);
      out[5984] = fma(0.88, dr, out[5984]);
    }
    {
      const double dr = ws[57504] * fma(y[5952], v[1952], y[1952] * v[5952]);
      out[1952] = out[1952] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5536] = fma(1.0, dr, out[5536]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57536] * fma(y[5952], v[1984], y[1984] * v[5952]);
      out[1984] = out[1984] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5088] = fma(1.0, dr, out[5088]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57568] * fma(y[5952], v[2016], y[2016] * v[5952]);
      out[2016] = out[2016] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57600] * fma(y[5952], v[2048], y[2048] * v[5952]);
      out[2048] = out[2048] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[4960] = fma(1.0, dr, out[4960]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57632] * fma(y[5952], v[2080], y[2080] * v[5952]);
      out[2080] = out[2080] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57664] * fma(y[5952], v[2112], y[2112] * v[5952]);
      out[2112] = out[2112] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[4832] = fma(1.0, dr, out[4832]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57696] * fma(y[5952], v[2144], y[2144] * v[5952]);
      out[2144] = out[2144] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5504] = fma(1.0, dr, out[5504]);
      out[5984] = fma(1.0, dr, out[5984]);
    }
    {
      const double dr = ws[57728] * fma(y[5984], v[1952], y[1952] * v[5984]);
      out[1952] = out[1952] - dr;
      out[5984] = out[5984] - dr;
      out[4992] = fma(1.0, dr, out[4992]);
    }
    {
      const double dr = ws[57760] * fma(y[5984], v[1984], y[1984] * v[5984]);
      out[1984] = out[1984] - dr;
      out[5984] = out[5984] - dr;
      out[4960] = fma(1.0, dr, out[4960]);
    }
    {
      const double dr = ws[57792] * fma(y[5984], v[2016], y[2016] * v[5984]);
      out[2016] = out[2016] - dr;
      out[5984] = out[5984] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
    }
    {
      const double dr = ws[57824] * fma(y[5984], v[2048], y[2048] * v[5984]);
      out[2048] = out[2048] - dr;
      out[5984] = out[5984] - dr;
      out[4832] = fma(1.0, dr, out[4832]);
    }
    {
      const double dr = ws[57856] * fma(y[5984], v[2080], y[2080] * v[5984]);
      out[2080] = out[2080] - dr;
      out[5984] = out[5984] - dr;
      out[4832] = fma(1.0, dr, out[4832]);
    }
    {
      const double dr = ws[57888] * fma(y[5984], v[2112], y[2112] * v[5984]);
      out[2112] = out[2112] - dr;
      out[5984] = out[5984] - dr;
      out[4832] = fma(1.0, dr, out[4832]);
    }
    {
      const double dr = ws[57920] * fma(y[5984], v[2144], y[2144] * v[5984]);
      out[2144] = out[2144] - dr;
      out[5984] = out[5984] - dr;
      out[5088] = fma(1.0, dr, out[5088]);
    }
    {
      const double dr = ws[57952] * fma(y[6016], v[832], y[832] * v[6016]);
      out[832] = out[832] - dr;
      out[6016] = out[6016] - dr;
      out[3392] = fma(0.84, dr, out[3392]);
      out[5984] = fma(0.16, dr, out[5984]);
      out[5312] = fma(0.16, dr, out[5312]);
    }
    {
      const double dr = ws[57984] * fma(y[5984], v[3392], y[3392] * v[5984]);
      out[3392] = out[3392] - dr;
      out[5984] = out[5984] - dr;
      out[5312] = fma(0.0595, dr, out[5312]);
      out[4992] = fma(0.9048, dr, out[4992]);
      out[4864] = fma(0.0357, dr, out[4864]);
    }
    {
      const double dr = ws[58016] * fma(y[5824], v[3392], y[3392] * v[5824]);
      out[3392] = out[3392] - dr;
      out[5824] = out[5824] - dr;
      out[5312] = fma(0.0001, dr, out[5312]);
      out[5088] = fma(0.0018, dr, out[5088]);
      out[4640] = fma(0.0001, dr, out[4640]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[4448] = fma(0.0594, dr, out[4448]);
      out[5376] = fma(0.4693, dr, out[5376]);
      out[5248] = fma(0.4693, dr, out[5248]);
      out[4512] = fma(0.4693, dr, out[4512]);
      out[4320] = fma(0.4693, dr, out[4320]);
    }
    {
      const double dr = ws[58048] * fma(y[5952], v[3392], y[3392] * v[5952]);
      out[3392] = out[3392] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.9405, dr, out[5984]);
      out[4448] = fma(0.0595, dr, out[4448]);
      out[5376] = fma(0.4702, dr, out[5376]);
      out[5248] = fma(0.4702, dr, out[5248]);
      out[4512] = fma(0.4702, dr, out[4512]);
      out[4320] = fma(0.4702, dr, out[4320]);
    }
    {
      const double dr = ws[58080] * fma(y[5888], v[3392], y[3392] * v[5888]);
      out[3392] = out[3392] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[5984] = fma(1.3105, dr, out[5984]);
      out[5600] = fma(0.32, dr, out[5600]);
      out[4448] = fma(0.0595, dr, out[4448]);
      out[5376] = fma(0.4702, dr, out[5376]);
      out[5248] = fma(0.4702, dr, out[5248]);
      out[4512] = fma(0.4702, dr, out[4512]);
      out[4320] = fma(0.4702, dr, out[4320]);
    }
    {
      const double dr = ws[58112] * fma(y[5792], v[3392], y[3392] * v[5792]);
      out[3392] = out[3392] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5984] = fma(0.9405, dr, out[5984]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[4448] = fma(0.0595, dr, out[4448]);
      out[5376] = fma(0.4702, dr, out[5376]);
      out[5248] = fma(0.4702, dr, out[5248]);
      out[4512] = fma(0.4702, dr, out[4512]);
      out[4320] = fma(0.4702, dr, out[4320]);
    }
    {
      const double dr = ws[58144] * fma(y[6016], v[864], y[864] * v[6016]);
      out[864] = out[864] - dr;
      out[6016] = out[6016] - dr;
      out[3424] = fma(0.84, dr, out[3424]);
      out[5984] = fma(0.16, dr, out[5984]);
      out[5536] = fma(0.16, dr, out[5536]);
    }
    {
      const double dr = ws[58176] * fma(y[5984], v[3424], y[3424] * v[5984]);
      out[3424] = out[3424] - dr;
      out[5984] = out[5984] - dr;
      out[5536] = fma(0.0595, dr, out[5536]);
      out[4960] = fma(0.9048, dr, out[4960]);
      out[4864] = fma(0.0357, dr, out[4864]);
    }
    {
      const double dr = ws[58208] * fma(y[5824], v[3424], y[3424] * v[5824]);
      out[3424] = out[3424] - dr;
      out[5824] = out[5824] - dr;
      out[5536] = fma(0.0001, dr, out[5536]);
      out[4992] = fma(0.0018, dr, out[4992]);
      out[4864] = fma(0.0001, dr, out[4864]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[5312] = fma(0.0594, dr, out[5312]);
      out[5376] = fma(0.4693, dr, out[5376]);
      out[5248] = fma(0.4693, dr, out[5248]);
      out[4512] = fma(0.4693, dr, out[4512]);
      out[4320] = fma(0.4693, dr, out[4320]);
    }
    {
      const double dr = ws[58240] * fma(y[5952], v[3424], y[3424] * v[5952]);
      out[3424] = out[3424] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(0.9405, dr, out[5984]);
      out[5312] = fma(0.0595, dr, out[5312]);
      out[5376] = fma(0.4702, dr, out[5376]);
      out[5248] = fma(0.4702, dr, out[5248]);
      out[4512] = fma(0.4702, dr, out[4512]);
      out[4320] = fma(0.4702, dr, out[4320]);
    }
    {
      const double dr = ws[58272] * fma(y[5888], v[3424], y[3424] * v[5888]);
      out[3424] = out[3424] - dr;
      out[5888] = out[5888] - dr;
      out[5856] = fma(0.68, dr, out[5856]);
      out[5984] = fma(1.3105, dr, out[5984]);
      out[5600] = fma(0.32, dr, out[5600]);
      out[5312] = fma(0.0595, dr, out[5312]);
      out[5376] = fma(0.4702, dr, out[5376]);
      out[5248] = fma(0.4702, dr, out[5248]);
      out[4512] = fma(0.4702, dr, out[4512]);
      out[4320] = fma(0.4702, dr, out[4320]);
    }
    {
      const double dr = ws[58304] * fma(y[5792], v[3424], y[3424] * v[5792]);
      out[3424] = out[3424] - dr;
      out[5792] = out[5792] - dr;
      out[5888] = fma(0.7, dr, out[5888]);
      out[5984] = fma(0.9405, dr, out[5984]);
      out[5696] = fma(0.3, dr, out[5696]);
      out[5312] = fma(0.0595, dr, out[5312]);
      out[5376] = fma(0.4702, dr, out[5376]);
      out[5248] = fma(0.4702, dr, out[5248]);
      out[4512] = fma(0.4702, dr, out[4512]);
      out[4320] = fma(0.4702, dr, out[4320]);
    }
    {
      const double dr = ws[58336] * fma(y[6016], v[896], y[896] * v[6016]);
      out[896] = out[896] - dr;
      out[6016] = out[6016] - dr;
      out[3456] = fma(0.84, dr, out[3456]);
      out[5984] = fma(0.16, dr, out[5984]);
      out[5536] = fma(0.16, dr, out[5536]);
    }
    {
      const double dr = ws[58368] * fma(y[5984], v[3456], y[3456] * v[5984]);
      out[3456] = out[3456] - dr;
      out[5984] = out[5984] - dr;
      out[5536] = fma(0.0595, dr, out[5536]);
      out[4992] = fma(0.9048, dr, out[4992]);
      out[4768] = fma(0.0357, dr, out[4768]);
    }
}
}  // namespace mech_cracmm2
