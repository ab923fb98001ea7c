// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void ddm_jv_1_8(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[58400] * fma(y[5824], v[3456], y[3456] * v[5824]);
      out[3456] = out[3456] - dr;
      out[5824] = out[5824] - dr;
      out[5312] = fma(0.0595, dr, out[5312]);
      out[5088] = fma(0.0018, dr, out[5088]);
      out[4768] = fma(0.0001, dr, out[4768]);
      out[5920] = fma(0.998, dr, out[5920]);
      out[5984] = fma(0.998, dr, out[5984]);
      out[5376] = fma(0.4693, dr, out[5376]);
      out[5248] = fma(0.4693, dr, out[5248]);
      out[4512] = fma(0.4693, dr, out[4512]);
      out[4320] = fma(0.4693, dr, out[4320]);
    }
    {
      const double dr = ws[58432] * fma(y[5952], v[3456], y[3456] * v[5952]);
      out[3456] = out[3456] - dr;
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
      const double dr = ws[58464] * fma(y[5888], v[3456], y[3456] * v[5888]);
      out[3456] = out[3456] - dr;
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
      const double dr = ws[58496] * fma(y[5792], v[3456], y[3456] * v[5792]);
      out[3456] = out[3456] - dr;
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
      const double dr = ws[58528] * fma(y[6016], v[4768], y[4768] * v[6016]);
      out[4768] = out[4768] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0854, dr, out[4768]);
      out[5472] = fma(0.2581, dr, out[5472]);
      out[5280] = fma(0.2581, dr, out[5280]);
      out[5568] = fma(0.2581, dr, out[5568]);
      out[5760] = fma(0.2581, dr, out[5760]);
      out[5888] = fma(0.2581, dr, out[5888]);
      out[5632] = fma(0.2581, dr, out[5632]);
      out[5408] = fma(0.2581, dr, out[5408]);
      out[5152] = fma(0.2581, dr, out[5152]);
    }
    {
      const double dr = ws[58560] * fma(y[6016], v[4864], y[4864] * v[6016]);
      out[4864] = out[4864] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.464, dr, out[4768]);
      out[4864] = fma(0.1977, dr, out[4864]);
      out[4896] = fma(0.0121, dr, out[4896]);
      out[4640] = fma(0.0152, dr, out[4640]);
      out[4928] = fma(0.0624, dr, out[4928]);
      out[4992] = fma(0.0388, dr, out[4992]);
      out[5088] = fma(0.0491, dr, out[5088]);
      out[5536] = fma(0.0398, dr, out[5536]);
      out[5312] = fma(0.0183, dr, out[5312]);
      out[4608] = fma(0.0308, dr, out[4608]);
      out[5728] = fma(0.004, dr, out[5728]);
      out[5472] = fma(0.0794, dr, out[5472]);
      out[5280] = fma(0.0794, dr, out[5280]);
      out[5504] = fma(0.0794, dr, out[5504]);
      out[5568] = fma(0.0794, dr, out[5568]);
      out[5760] = fma(0.0794, dr, out[5760]);
      out[5888] = fma(0.0794, dr, out[5888]);
      out[5632] = fma(0.0794, dr, out[5632]);
      out[5408] = fma(0.0794, dr, out[5408]);
      out[5152] = fma(0.0794, dr, out[5152]);
      out[5120] = fma(0.0794, dr, out[5120]);
      out[3776] = fma(0.0794, dr, out[3776]);
    }
    {
      const double dr = ws[58592] * fma(y[6016], v[4832], y[4832] * v[6016]);
      out[4832] = out[4832] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.1041, dr, out[4768]);
      out[4864] = fma(0.5638, dr, out[4864]);
      out[4832] = fma(0.2141, dr, out[4832]);
      out[4896] = fma(0.0153, dr, out[4896]);
      out[4640] = fma(0.0298, dr, out[4640]);
      out[4416] = fma(0.0096, dr, out[4416]);
      out[4928] = fma(0.0189, dr, out[4928]);
      out[4960] = fma(0.0456, dr, out[4960]);
      out[4992] = fma(0.0314, dr, out[4992]);
      out[4704] = fma(0.0199, dr, out[4704]);
      out[5088] = fma(0.0459, dr, out[5088]);
      out[5536] = fma(0.0452, dr, out[5536]);
      out[5312] = fma(0.0455, dr, out[5312]);
      out[4224] = fma(0.0325, dr, out[4224]);
      out[3968] = fma(0.0369, dr, out[3968]);
      out[4608] = fma(0.0026, dr, out[4608]);
      out[5472] = fma(0.039, dr, out[5472]);
      out[5344] = fma(0.039, dr, out[5344]);
      out[5280] = fma(0.039, dr, out[5280]);
      out[5568] = fma(0.039, dr, out[5568]);
      out[5760] = fma(0.039, dr, out[5760]);
      out[5888] = fma(0.039, dr, out[5888]);
      out[5632] = fma(0.039, dr, out[5632]);
      out[5408] = fma(0.039, dr, out[5408]);
      out[5152] = fma(0.039, dr, out[5152]);
      out[5120] = fma(0.0925, dr, out[5120]);
    }
    {
      const double dr = ws[58624] * fma(y[6016], v[4896], y[4896] * v[6016]);
      out[4896] = out[4896] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.2036, dr, out[4768]);
      out[4864] = fma(0.0071, dr, out[4864]);
      out[5472] = fma(0.184, dr, out[5472]);
      out[5280] = fma(0.184, dr, out[5280]);
      out[5504] = fma(0.184, dr, out[5504]);
      out[5568] = fma(0.184, dr, out[5568]);
      out[5760] = fma(0.184, dr, out[5760]);
      out[5888] = fma(0.184, dr, out[5888]);
      out[5632] = fma(0.184, dr, out[5632]);
      out[5408] = fma(0.184, dr, out[5408]);
      out[5152] = fma(0.184, dr, out[5152]);
      out[5120] = fma(0.184, dr, out[5120]);
    }
    {
      const double dr = ws[58656] * fma(y[6016], v[4640], y[4640] * v[6016]);
      out[4640] = out[4640] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.2792, dr, out[4768]);
      out[4864] = fma(0.4025, dr, out[4864]);
      out[4832] = fma(0.0088, dr, out[4832]);
      out[4896] = fma(0.0319, dr, out[4896]);
      out[4640] = fma(0.0076, dr, out[4640]);
      out[4928] = fma(0.0194, dr, out[4928]);
      out[4960] = fma(0.0104, dr, out[4960]);
      out[4992] = fma(0.051, dr, out[4992]);
      out[4704] = fma(0.0075, dr, out[4704]);
      out[5088] = fma(0.0512, dr, out[5088]);
      out[5536] = fma(0.0462, dr, out[5536]);
      out[5312] = fma(0.0512, dr, out[5312]);
      out[4224] = fma(0.0138, dr, out[4224]);
      out[5728] = fma(0.0135, dr, out[5728]);
      out[5472] = fma(0.0646, dr, out[5472]);
      out[5344] = fma(0.0646, dr, out[5344]);
      out[5280] = fma(0.0646, dr, out[5280]);
      out[5568] = fma(0.0646, dr, out[5568]);
      out[5760] = fma(0.0646, dr, out[5760]);
      out[5888] = fma(0.0646, dr, out[5888]);
      out[5632] = fma(0.0646, dr, out[5632]);
      out[5408] = fma(0.0646, dr, out[5408]);
      out[5152] = fma(0.0646, dr, out[5152]);
      out[5120] = fma(0.1753, dr, out[5120]);
    }
    {
      const double dr = ws[58688] * fma(y[6016], v[4416], y[4416] * v[6016]);
      out[4416] = out[4416] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0074, dr, out[4768]);
      out[4864] = fma(0.119, dr, out[4864]);
      out[4832] = fma(0.7261, dr, out[4832]);
      out[4896] = fma(0.0122, dr, out[4896]);
      out[4640] = fma(0.0305, dr, out[4640]);
      out[4416] = fma(0.007, dr, out[4416]);
      out[4928] = fma(0.0291, dr, out[4928]);
      out[4960] = fma(0.0454, dr, out[4960]);
      out[4992] = fma(0.0234, dr, out[4992]);
      out[4704] = fma(0.0352, dr, out[4704]);
      out[5088] = fma(0.0624, dr, out[5088]);
      out[5536] = fma(0.0518, dr, out[5536]);
      out[5312] = fma(0.0509, dr, out[5312]);
      out[4224] = fma(0.0347, dr, out[4224]);
      out[3968] = fma(0.0748, dr, out[3968]);
      out[4608] = fma(0.0163, dr, out[4608]);
      out[5728] = fma(0.0062, dr, out[5728]);
      out[5472] = fma(0.0244, dr, out[5472]);
      out[5344] = fma(0.0244, dr, out[5344]);
      out[5280] = fma(0.0244, dr, out[5280]);
      out[5568] = fma(0.0244, dr, out[5568]);
      out[5760] = fma(0.0244, dr, out[5760]);
      out[5888] = fma(0.0244, dr, out[5888]);
      out[5632] = fma(0.0244, dr, out[5632]);
      out[5408] = fma(0.0244, dr, out[5408]);
      out[5152] = fma(0.0244, dr, out[5152]);
      out[5120] = fma(0.0537, dr, out[5120]);
    }
    {
      const double dr = ws[58720] * fma(y[6016], v[4928], y[4928] * v[6016]);
      out[4928] = out[4928] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.2822, dr, out[4768]);
      out[4864] = fma(0.1165, dr, out[4864]);
      out[4896] = fma(0.032, dr, out[4896]);
      out[4640] = fma(0.0183, dr, out[4640]);
      out[4928] = fma(0.0011, dr, out[4928]);
      out[5088] = fma(0.066, dr, out[5088]);
      out[5536] = fma(0.0535, dr, out[5536]);
      out[5312] = fma(0.0246, dr, out[5312]);
      out[5728] = fma(0.0054, dr, out[5728]);
      out[5472] = fma(0.1068, dr, out[5472]);
      out[5280] = fma(0.1068, dr, out[5280]);
      out[5504] = fma(0.1068, dr, out[5504]);
      out[5568] = fma(0.1068, dr, out[5568]);
      out[5760] = fma(0.1068, dr, out[5760]);
      out[5888] = fma(0.1068, dr, out[5888]);
      out[5632] = fma(0.1068, dr, out[5632]);
      out[5408] = fma(0.1068, dr, out[5408]);
      out[5152] = fma(0.1068, dr, out[5152]);
      out[5120] = fma(0.1068, dr, out[5120]);
      out[3776] = fma(0.1068, dr, out[3776]);
    }
    {
      const double dr = ws[58752] * fma(y[6016], v[4960], y[4960] * v[6016]);
      out[4960] = out[4960] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0659, dr, out[4768]);
      out[4864] = fma(0.4579, dr, out[4864]);
      out[4832] = fma(0.1156, dr, out[4832]);
      out[4896] = fma(0.0325, dr, out[4896]);
      out[4640] = fma(0.0657, dr, out[4640]);
      out[4416] = fma(0.0046, dr, out[4416]);
      out[4928] = fma(0.0307, dr, out[4928]);
      out[4960] = fma(0.0024, dr, out[4960]);
      out[4992] = fma(0.0395, dr, out[4992]);
      out[4704] = fma(0.0215, dr, out[4704]);
      out[5088] = fma(0.0539, dr, out[5088]);
      out[5536] = fma(0.0516, dr, out[5536]);
      out[5312] = fma(0.0519, dr, out[5312]);
      out[4224] = fma(0.0371, dr, out[4224]);
      out[3968] = fma(0.0421, dr, out[3968]);
      out[4608] = fma(0.0105, dr, out[4608]);
      out[5472] = fma(0.0445, dr, out[5472]);
      out[5344] = fma(0.0445, dr, out[5344]);
      out[5280] = fma(0.0445, dr, out[5280]);
      out[5568] = fma(0.0445, dr, out[5568]);
      out[5760] = fma(0.0445, dr, out[5760]);
      out[5888] = fma(0.0445, dr, out[5888]);
      out[5632] = fma(0.0445, dr, out[5632]);
      out[5408] = fma(0.0445, dr, out[5408]);
      out[5152] = fma(0.0445, dr, out[5152]);
      out[5120] = fma(0.1055, dr, out[5120]);
    }
    {
      const double dr = ws[58784] * fma(y[6016], v[4992], y[4992] * v[6016]);
      out[4992] = out[4992] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.1778, dr, out[4768]);
      out[4864] = fma(0.1924, dr, out[4864]);
      out[4832] = fma(0.0004, dr, out[4832]);
      out[4896] = fma(0.074, dr, out[4896]);
      out[4640] = fma(0.0452, dr, out[4640]);
      out[4928] = fma(0.0631, dr, out[4928]);
      out[4960] = fma(0.0007, dr, out[4960]);
      out[4992] = fma(0.0006, dr, out[4992]);
      out[5088] = fma(0.0227, dr, out[5088]);
      out[5536] = fma(0.0585, dr, out[5536]);
      out[5312] = fma(0.0649, dr, out[5312]);
      out[4224] = fma(0.0174, dr, out[4224]);
      out[4608] = fma(0.0154, dr, out[4608]);
      out[5728] = fma(0.017, dr, out[5728]);
      out[5472] = fma(0.0818, dr, out[5472]);
      out[5344] = fma(0.0818, dr, out[5344]);
      out[5280] = fma(0.0818, dr, out[5280]);
      out[5568] = fma(0.0818, dr, out[5568]);
      out[5760] = fma(0.0818, dr, out[5760]);
      out[5888] = fma(0.0818, dr, out[5888]);
      out[5632] = fma(0.0818, dr, out[5632]);
      out[5408] = fma(0.0818, dr, out[5408]);
      out[5152] = fma(0.0818, dr, out[5152]);
      out[5120] = fma(0.222, dr, out[5120]);
    }
    {
      const double dr = ws[58816] * fma(y[6016], v[4704], y[4704] * v[6016]);
      out[4704] = out[4704] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0023, dr, out[4768]);
      out[4864] = fma(0.134, dr, out[4864]);
      out[4832] = fma(0.3349, dr, out[4832]);
      out[4896] = fma(0.008, dr, out[4896]);
      out[4640] = fma(0.1193, dr, out[4640]);
      out[4416] = fma(0.0758, dr, out[4416]);
      out[4928] = fma(0.0292, dr, out[4928]);
      out[4960] = fma(0.0766, dr, out[4960]);
      out[4992] = fma(0.0277, dr, out[4992]);
      out[4704] = fma(0.0118, dr, out[4704]);
      out[5088] = fma(0.0651, dr, out[5088]);
      out[5536] = fma(0.0709, dr, out[5536]);
      out[5312] = fma(0.0668, dr, out[5312]);
      out[4224] = fma(0.0423, dr, out[4224]);
      out[3968] = fma(0.0911, dr, out[3968]);
      out[4608] = fma(0.0066, dr, out[4608]);
      out[5728] = fma(0.0025, dr, out[5728]);
      out[5472] = fma(0.0297, dr, out[5472]);
      out[5344] = fma(0.0297, dr, out[5344]);
      out[5280] = fma(0.0297, dr, out[5280]);
      out[5568] = fma(0.0297, dr, out[5568]);
      out[5760] = fma(0.0297, dr, out[5760]);
      out[5888] = fma(0.0297, dr, out[5888]);
      out[5632] = fma(0.0297, dr, out[5632]);
      out[5408] = fma(0.0297, dr, out[5408]);
      out[5152] = fma(0.0297, dr, out[5152]);
      out[5120] = fma(0.0654, dr, out[5120]);
    }
    {
      const double dr = ws[58848] * fma(y[6016], v[5088], y[5088] * v[6016]);
      out[5088] = out[5088] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0445, dr, out[4768]);
      out[4864] = fma(0.1726, dr, out[4864]);
      out[4832] = fma(0.0104, dr, out[4832]);
      out[4896] = fma(0.0513, dr, out[4896]);
      out[4640] = fma(0.1118, dr, out[4640]);
      out[4416] = fma(0.0013, dr, out[4416]);
      out[4928] = fma(0.1337, dr, out[4928]);
      out[4960] = fma(0.0403, dr, out[4960]);
      out[4992] = fma(0.0511, dr, out[4992]);
      out[4704] = fma(0.0068, dr, out[4704]);
      out[5088] = fma(0.0236, dr, out[5088]);
      out[5536] = fma(0.0293, dr, out[5536]);
      out[5312] = fma(0.0733, dr, out[5312]);
      out[4224] = fma(0.0523, dr, out[4224]);
      out[3968] = fma(0.0595, dr, out[3968]);
      out[4608] = fma(0.0041, dr, out[4608]);
      out[5728] = fma(0.0023, dr, out[5728]);
      out[5472] = fma(0.0628, dr, out[5472]);
      out[5344] = fma(0.0628, dr, out[5344]);
      out[5280] = fma(0.0628, dr, out[5280]);
      out[5568] = fma(0.0628, dr, out[5568]);
      out[5760] = fma(0.0628, dr, out[5760]);
      out[5888] = fma(0.0628, dr, out[5888]);
      out[5632] = fma(0.0628, dr, out[5632]);
      out[5408] = fma(0.0628, dr, out[5408]);
      out[5152] = fma(0.0628, dr, out[5152]);
      out[5120] = fma(0.1489, dr, out[5120]);
    }
    {
      const double dr = ws[58880] * fma(y[6016], v[5536], y[5536] * v[6016]);
      out[5536] = out[5536] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0317, dr, out[4768]);
      out[4864] = fma(0.0765, dr, out[4864]);
      out[4832] = fma(0.0009, dr, out[4832]);
      out[4896] = fma(0.0526, dr, out[4896]);
      out[4640] = fma(0.0489, dr, out[4640]);
      out[4928] = fma(0.155, dr, out[4928]);
      out[4960] = fma(0.0155, dr, out[4960]);
      out[4992] = fma(0.1051, dr, out[4992]);
      out[4704] = fma(0.0013, dr, out[4704]);
      out[5088] = fma(0.0535, dr, out[5088]);
      out[5536] = fma(0.0086, dr, out[5536]);
      out[5312] = fma(0.0426, dr, out[5312]);
      out[4224] = fma(0.0582, dr, out[4224]);
      out[3968] = fma(0.0661, dr, out[3968]);
      out[4608] = fma(0.0506, dr, out[4608]);
      out[5728] = fma(0.0114, dr, out[5728]);
      out[5472] = fma(0.0698, dr, out[5472]);
      out[5344] = fma(0.0698, dr, out[5344]);
      out[5280] = fma(0.0698, dr, out[5280]);
      out[5568] = fma(0.0698, dr, out[5568]);
      out[5760] = fma(0.0698, dr, out[5760]);
      out[5888] = fma(0.0698, dr, out[5888]);
      out[5632] = fma(0.0698, dr, out[5632]);
      out[5408] = fma(0.0698, dr, out[5408]);
      out[5152] = fma(0.0698, dr, out[5152]);
      out[5120] = fma(0.1656, dr, out[5120]);
    }
    {
      const double dr = ws[58912] * fma(y[6016], v[5312], y[5312] * v[6016]);
      out[5312] = out[5312] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.0117, dr, out[4768]);
      out[4864] = fma(0.0167, dr, out[4864]);
      out[4896] = fma(0.048, dr, out[4896]);
      out[4640] = fma(0.0246, dr, out[4640]);
      out[4928] = fma(0.0881, dr, out[4928]);
      out[4992] = fma(0.0916, dr, out[4992]);
      out[4704] = fma(0.0073, dr, out[4704]);
      out[5088] = fma(0.0972, dr, out[5088]);
      out[5536] = fma(0.0456, dr, out[5536]);
      out[5312] = fma(0.0024, dr, out[5312]);
      out[4224] = fma(0.0479, dr, out[4224]);
      out[3968] = fma(0.0745, dr, out[3968]);
      out[4608] = fma(0.0607, dr, out[4608]);
      out[5728] = fma(0.0155, dr, out[5728]);
      out[5472] = fma(0.0786, dr, out[5472]);
      out[5344] = fma(0.0786, dr, out[5344]);
      out[5280] = fma(0.0786, dr, out[5280]);
      out[5568] = fma(0.0786, dr, out[5568]);
      out[5760] = fma(0.0786, dr, out[5760]);
      out[5888] = fma(0.0786, dr, out[5888]);
      out[5632] = fma(0.0786, dr, out[5632]);
      out[5408] = fma(0.0786, dr, out[5408]);
      out[5152] = fma(0.0786, dr, out[5152]);
      out[5120] = fma(0.173, dr, out[5120]);
    }
    {
      const double dr = ws[58944] * fma(y[6016], v[4224], y[4224] * v[6016]);
      out[4224] = out[4224] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4864] = fma(0.0103, dr, out[4864]);
      out[4832] = fma(0.0006, dr, out[4832]);
      out[4896] = fma(0.009, dr, out[4896]);
      out[4640] = fma(0.0146, dr, out[4640]);
      out[4928] = fma(0.0702, dr, out[4928]);
      out[4960] = fma(0.0153, dr, out[4960]);
      out[4992] = fma(0.1038, dr, out[4992]);
      out[4704] = fma(0.0031, dr, out[4704]);
      out[5088] = fma(0.165, dr, out[5088]);
      out[5536] = fma(0.1566, dr, out[5536]);
      out[5312] = fma(0.0724, dr, out[5312]);
      out[4224] = fma(0.0062, dr, out[4224]);
      out[3968] = fma(0.1398, dr, out[3968]);
      out[4608] = fma(0.0216, dr, out[4608]);
      out[5728] = fma(0.0384, dr, out[5728]);
      out[5472] = fma(0.0526, dr, out[5472]);
      out[5344] = fma(0.0526, dr, out[5344]);
      out[5280] = fma(0.0526, dr, out[5280]);
      out[5568] = fma(0.0526, dr, out[5568]);
      out[5760] = fma(0.0526, dr, out[5760]);
      out[5888] = fma(0.0526, dr, out[5888]);
      out[5632] = fma(0.0526, dr, out[5632]);
      out[5408] = fma(0.0526, dr, out[5408]);
      out[5152] = fma(0.0526, dr, out[5152]);
      out[5120] = fma(0.128, dr, out[5120]);
    }
    {
      const double dr = ws[58976] * fma(y[6016], v[3968], y[3968] * v[6016]);
      out[3968] = out[3968] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4896] = fma(0.0061, dr, out[4896]);
      out[4640] = fma(0.0049, dr, out[4640]);
      out[4928] = fma(0.0224, dr, out[4928]);
      out[4992] = fma(0.0503, dr, out[4992]);
      out[4704] = fma(0.0022, dr, out[4704]);
      out[5088] = fma(0.0879, dr, out[5088]);
      out[5536] = fma(0.1384, dr, out[5536]);
      out[5312] = fma(0.1463, dr, out[5312]);
      out[4224] = fma(0.0432, dr, out[4224]);
      out[3968] = fma(0.0957, dr, out[3968]);
      out[4608] = fma(0.0316, dr, out[4608]);
      out[5728] = fma(0.0585, dr, out[5728]);
      out[5472] = fma(0.0571, dr, out[5472]);
      out[5344] = fma(0.0571, dr, out[5344]);
      out[5280] = fma(0.0571, dr, out[5280]);
      out[5568] = fma(0.0571, dr, out[5568]);
      out[5760] = fma(0.0571, dr, out[5760]);
      out[5888] = fma(0.0571, dr, out[5888]);
      out[5632] = fma(0.0571, dr, out[5632]);
      out[5408] = fma(0.0571, dr, out[5408]);
      out[5152] = fma(0.0571, dr, out[5152]);
      out[5120] = fma(0.1544, dr, out[5120]);
    }
}
__device__ __noinline__ void ddm_jv_1_9(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[59008] * fma(y[6016], v[4608], y[4608] * v[6016]);
      out[4608] = out[4608] - dr;
      out[6016] = out[6016] - dr;
      out[6016] = fma(1.0, dr, out[6016]);
      out[4768] = fma(0.1188, dr, out[4768]);
      out[4864] = fma(0.0008, dr, out[4864]);
      out[4896] = fma(0.039, dr, out[4896]);
      out[4928] = fma(0.0114, dr, out[4928]);
      out[5472] = fma(0.2266, dr, out[5472]);
      out[5280] = fma(0.2266, dr, out[5280]);
      out[5568] = fma(0.2266, dr, out[5568]);
      out[5760] = fma(0.2266, dr, out[5760]);
      out[5888] = fma(0.2266, dr, out[5888]);
      out[5632] = fma(0.2266, dr, out[5632]);
      out[5408] = fma(0.2266, dr, out[5408]);
      out[5152] = fma(0.2266, dr, out[5152]);
    }
    {
      const double dr = ws[59040] * fma(y[6016], v[928], y[928] * v[6016]);
      out[928] = out[928] - dr;
      out[6016] = out[6016] - dr;
      out[5888] = fma(1.0, dr, out[5888]);
    }
    {
      const double dr = ws[59072] * v[96];
      out[96] = out[96] - dr;
      out[960] = fma(1.0, dr, out[960]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[59104] * v[128];
      out[128] = out[128] - dr;
      out[960] = fma(1.0, dr, out[960]);
      out[5024] = fma(1.0, dr, out[5024]);
    }
    {
      const double dr = ws[59136] * fma(y[6016], v[992], y[992] * v[6016]);
      out[992] = out[992] - dr;
      out[6016] = out[6016] - dr;
      out[3488] = fma(1.0, dr, out[3488]);
    }
    {
      const double dr = ws[59168] * fma(y[5984], v[3488], y[3488] * v[5984]);
      out[3488] = out[3488] - dr;
      out[5984] = out[5984] - dr;
      out[5536] = fma(1.0, dr, out[5536]);
    }
    {
      const double dr = ws[59200] * fma(y[5824], v[3488], y[3488] * v[5824]);
      out[3488] = out[3488] - dr;
      out[5824] = out[5824] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[59232] * fma(y[5952], v[3488], y[3488] * v[5952]);
      out[3488] = out[3488] - dr;
      out[5952] = out[5952] - dr;
      out[5920] = fma(1.0, dr, out[5920]);
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[59264] * fma(y[5888], v[3488], y[3488] * v[5888]);
      out[3488] = out[3488] - dr;
      out[5888] = out[5888] - dr;
      out[5984] = fma(1.37, dr, out[5984]);
      out[5856] = fma(1.68, dr, out[5856]);
      out[4448] = fma(1.0, dr, out[4448]);
      out[5600] = fma(0.32, dr, out[5600]);
    }
    {
      const double dr = ws[59296] * fma(y[5792], v[3488], y[3488] * v[5792]);
      out[3488] = out[3488] - dr;
      out[5792] = out[5792] - dr;
      out[5984] = fma(1.0, dr, out[5984]);
      out[5856] = fma(1.0, dr, out[5856]);
      out[4448] = fma(1.0, dr, out[4448]);
      out[5888] = fma(0.7, dr, out[5888]);
      out[5696] = fma(0.3, dr, out[5696]);
    }
}
}  // namespace mech_cracmm2
