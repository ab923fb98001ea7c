// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void ddm_src_1_8(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[502]) {
      const double q = scale * ws[75392];
      out[3456] = out[3456] - q;
      out[5824] = out[5824] - q;
      out[5312] = fma(0.0595, q, out[5312]);
      out[5088] = fma(0.0018, q, out[5088]);
      out[4768] = fma(0.0001, q, out[4768]);
      out[5920] = fma(0.998, q, out[5920]);
      out[5984] = fma(0.998, q, out[5984]);
      out[5376] = fma(0.4693, q, out[5376]);
      out[5248] = fma(0.4693, q, out[5248]);
      out[4512] = fma(0.4693, q, out[4512]);
      out[4320] = fma(0.4693, q, out[4320]);
    }
    if (mask[503]) {
      const double q = scale * ws[75424];
      out[3456] = out[3456] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(0.9405, q, out[5984]);
      out[5312] = fma(0.0595, q, out[5312]);
      out[5376] = fma(0.4702, q, out[5376]);
      out[5248] = fma(0.4702, q, out[5248]);
      out[4512] = fma(0.4702, q, out[4512]);
      out[4320] = fma(0.4702, q, out[4320]);
    }
    if (mask[504]) {
      const double q = scale * ws[75456];
      out[3456] = out[3456] - q;
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
    if (mask[505]) {
      const double q = scale * ws[75488];
      out[3456] = out[3456] - q;
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
    if (mask[506]) {
      const double q = scale * ws[75520];
      out[4768] = out[4768] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0854, q, out[4768]);
      out[5472] = fma(0.2581, q, out[5472]);
      out[5280] = fma(0.2581, q, out[5280]);
      out[5568] = fma(0.2581, q, out[5568]);
      out[5760] = fma(0.2581, q, out[5760]);
      out[5888] = fma(0.2581, q, out[5888]);
      out[5632] = fma(0.2581, q, out[5632]);
      out[5408] = fma(0.2581, q, out[5408]);
      out[5152] = fma(0.2581, q, out[5152]);
    }
    if (mask[507]) {
      const double q = scale * ws[75552];
      out[4864] = out[4864] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.464, q, out[4768]);
      out[4864] = fma(0.1977, q, out[4864]);
      out[4896] = fma(0.0121, q, out[4896]);
      out[4640] = fma(0.0152, q, out[4640]);
      out[4928] = fma(0.0624, q, out[4928]);
      out[4992] = fma(0.0388, q, out[4992]);
      out[5088] = fma(0.0491, q, out[5088]);
      out[5536] = fma(0.0398, q, out[5536]);
      out[5312] = fma(0.0183, q, out[5312]);
      out[4608] = fma(0.0308, q, out[4608]);
      out[5728] = fma(0.004, q, out[5728]);
      out[5472] = fma(0.0794, q, out[5472]);
      out[5280] = fma(0.0794, q, out[5280]);
      out[5504] = fma(0.0794, q, out[5504]);
      out[5568] = fma(0.0794, q, out[5568]);
      out[5760] = fma(0.0794, q, out[5760]);
      out[5888] = fma(0.0794, q, out[5888]);
      out[5632] = fma(0.0794, q, out[5632]);
      out[5408] = fma(0.0794, q, out[5408]);
      out[5152] = fma(0.0794, q, out[5152]);
      out[5120] = fma(0.0794, q, out[5120]);
      out[3776] = fma(0.0794, q, out[3776]);
    }
    if (mask[508]) {
      const double q = scale * ws[75584];
      out[4832] = out[4832] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.1041, q, out[4768]);
      out[4864] = fma(0.5638, q, out[4864]);
      out[4832] = fma(0.2141, q, out[4832]);
      out[4896] = fma(0.0153, q, out[4896]);
      out[4640] = fma(0.0298, q, out[4640]);
      out[4416] = fma(0.0096, q, out[4416]);
      out[4928] = fma(0.0189, q, out[4928]);
      out[4960] = fma(0.0456, q, out[4960]);
      out[4992] = fma(0.0314, q, out[4992]);
      out[4704] = fma(0.0199, q, out[4704]);
      out[5088] = fma(0.0459, q, out[5088]);
      out[5536] = fma(0.0452, q, out[5536]);
      out[5312] = fma(0.0455, q, out[5312]);
      out[4224] = fma(0.0325, q, out[4224]);
      out[3968] = fma(0.0369, q, out[3968]);
      out[4608] = fma(0.0026, q, out[4608]);
      out[5472] = fma(0.039, q, out[5472]);
      out[5344] = fma(0.039, q, out[5344]);
      out[5280] = fma(0.039, q, out[5280]);
      out[5568] = fma(0.039, q, out[5568]);
      out[5760] = fma(0.039, q, out[5760]);
      out[5888] = fma(0.039, q, out[5888]);
      out[5632] = fma(0.039, q, out[5632]);
      out[5408] = fma(0.039, q, out[5408]);
      out[5152] = fma(0.039, q, out[5152]);
      out[5120] = fma(0.0925, q, out[5120]);
    }
    if (mask[509]) {
      const double q = scale * ws[75616];
      out[4896] = out[4896] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.2036, q, out[4768]);
      out[4864] = fma(0.0071, q, out[4864]);
      out[5472] = fma(0.184, q, out[5472]);
      out[5280] = fma(0.184, q, out[5280]);
      out[5504] = fma(0.184, q, out[5504]);
      out[5568] = fma(0.184, q, out[5568]);
      out[5760] = fma(0.184, q, out[5760]);
      out[5888] = fma(0.184, q, out[5888]);
      out[5632] = fma(0.184, q, out[5632]);
      out[5408] = fma(0.184, q, out[5408]);
      out[5152] = fma(0.184, q, out[5152]);
      out[5120] = fma(0.184, q, out[5120]);
    }
    if (mask[510]) {
      const double q = scale * ws[75648];
      out[4640] = out[4640] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.2792, q, out[4768]);
      out[4864] = fma(0.4025, q, out[4864]);
      out[4832] = fma(0.0088, q, out[4832]);
      out[4896] = fma(0.0319, q, out[4896]);
      out[4640] = fma(0.0076, q, out[4640]);
      out[4928] = fma(0.0194, q, out[4928]);
      out[4960] = fma(0.0104, q, out[4960]);
      out[4992] = fma(0.051, q, out[4992]);
      out[4704] = fma(0.0075, q, out[4704]);
      out[5088] = fma(0.0512, q, out[5088]);
      out[5536] = fma(0.0462, q, out[5536]);
      out[5312] = fma(0.0512, q, out[5312]);
      out[4224] = fma(0.0138, q, out[4224]);
      out[5728] = fma(0.0135, q, out[5728]);
      out[5472] = fma(0.0646, q, out[5472]);
      out[5344] = fma(0.0646, q, out[5344]);
      out[5280] = fma(0.0646, q, out[5280]);
      out[5568] = fma(0.0646, q, out[5568]);
      out[5760] = fma(0.0646, q, out[5760]);
      out[5888] = fma(0.0646, q, out[5888]);
      out[5632] = fma(0.0646, q, out[5632]);
      out[5408] = fma(0.0646, q, out[5408]);
      out[5152] = fma(0.0646, q, out[5152]);
      out[5120] = fma(0.1753, q, out[5120]);
    }
    if (mask[511]) {
      const double q = scale * ws[75680];
      out[4416] = out[4416] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0074, q, out[4768]);
      out[4864] = fma(0.119, q, out[4864]);
      out[4832] = fma(0.7261, q, out[4832]);
      out[4896] = fma(0.0122, q, out[4896]);
      out[4640] = fma(0.0305, q, out[4640]);
      out[4416] = fma(0.007, q, out[4416]);
      out[4928] = fma(0.0291, q, out[4928]);
      out[4960] = fma(0.0454, q, out[4960]);
      out[4992] = fma(0.0234, q, out[4992]);
      out[4704] = fma(0.0352, q, out[4704]);
      out[5088] = fma(0.0624, q, out[5088]);
      out[5536] = fma(0.0518, q, out[5536]);
      out[5312] = fma(0.0509, q, out[5312]);
      out[4224] = fma(0.0347, q, out[4224]);
      out[3968] = fma(0.0748, q, out[3968]);
      out[4608] = fma(0.0163, q, out[4608]);
      out[5728] = fma(0.0062, q, out[5728]);
      out[5472] = fma(0.0244, q, out[5472]);
      out[5344] = fma(0.0244, q, out[5344]);
      out[5280] = fma(0.0244, q, out[5280]);
      out[5568] = fma(0.0244, q, out[5568]);
      out[5760] = fma(0.0244, q, out[5760]);
      out[5888] = fma(0.0244, q, out[5888]);
      out[5632] = fma(0.0244, q, out[5632]);
      out[5408] = fma(0.0244, q, out[5408]);
      out[5152] = fma(0.0244, q, out[5152]);
      out[5120] = fma(0.0537, q, out[5120]);
    }
    if (mask[512]) {
      const double q = scale * ws[75712];
      out[4928] = out[4928] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.2822, q, out[4768]);
      out[4864] = fma(0.1165, q, out[4864]);
      out[4896] = fma(0.032, q, out[4896]);
      out[4640] = fma(0.0183, q, out[4640]);
      out[4928] = fma(0.0011, q, out[4928]);
      out[5088] = fma(0.066, q, out[5088]);
      out[5536] = fma(0.0535, q, out[5536]);
      out[5312] = fma(0.0246, q, out[5312]);
      out[5728] = fma(0.0054, q, out[5728]);
      out[5472] = fma(0.1068, q, out[5472]);
      out[5280] = fma(0.1068, q, out[5280]);
      out[5504] = fma(0.1068, q, out[5504]);
      out[5568] = fma(0.1068, q, out[5568]);
      out[5760] = fma(0.1068, q, out[5760]);
      out[5888] = fma(0.1068, q, out[5888]);
      out[5632] = fma(0.1068, q, out[5632]);
      out[5408] = fma(0.1068, q, out[5408]);
      out[5152] = fma(0.1068, q, out[5152]);
      out[5120] = fma(0.1068, q, out[5120]);
      out[3776] = fma(0.1068, q, out[3776]);
    }
    if (mask[513]) {
      const double q = scale * ws[75744];
      out[4960] = out[4960] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0659, q, out[4768]);
      out[4864] = fma(0.4579, q, out[4864]);
      out[4832] = fma(0.1156, q, out[4832]);
      out[4896] = fma(0.0325, q, out[4896]);
      out[4640] = fma(0.0657, q, out[4640]);
      out[4416] = fma(0.0046, q, out[4416]);
      out[4928] = fma(0.0307, q, out[4928]);
      out[4960] = fma(0.0024, q, out[4960]);
      out[4992] = fma(0.0395, q, out[4992]);
      out[4704] = fma(0.0215, q, out[4704]);
      out[5088] = fma(0.0539, q, out[5088]);
      out[5536] = fma(0.0516, q, out[5536]);
      out[5312] = fma(0.0519, q, out[5312]);
      out[4224] = fma(0.0371, q, out[4224]);
      out[3968] = fma(0.0421, q, out[3968]);
      out[4608] = fma(0.0105, q, out[4608]);
      out[5472] = fma(0.0445, q, out[5472]);
      out[5344] = fma(0.0445, q, out[5344]);
      out[5280] = fma(0.0445, q, out[5280]);
      out[5568] = fma(0.0445, q, out[5568]);
      out[5760] = fma(0.0445, q, out[5760]);
      out[5888] = fma(0.0445, q, out[5888]);
      out[5632] = fma(0.0445, q, out[5632]);
      out[5408] = fma(0.0445, q, out[5408]);
      out[5152] = fma(0.0445, q, out[5152]);
      out[5120] = fma(0.1055, q, out[5120]);
    }
    if (mask[514]) {
      const double q = scale * ws[75776];
      out[4992] = out[4992] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.1778, q, out[4768]);
      out[4864] = fma(0.1924, q, out[4864]);
      out[4832] = fma(0.0004, q, out[4832]);
      out[4896] = fma(0.074, q, out[4896]);
      out[4640] = fma(0.0452, q, out[4640]);
      out[4928] = fma(0.0631, q, out[4928]);
      out[4960] = fma(0.0007, q, out[4960]);
      out[4992] = fma(0.0006, q, out[4992]);
      out[5088] = fma(0.0227, q, out[5088]);
      out[5536] = fma(0.0585, q, out[5536]);
      out[5312] = fma(0.0649, q, out[5312]);
      out[4224] = fma(0.0174, q, out[4224]);
      out[4608] = fma(0.0154, q, out[4608]);
      out[5728] = fma(0.017, q, out[5728]);
      out[5472] = fma(0.0818, q, out[5472]);
      out[5344] = fma(0.0818, q, out[5344]);
      out[5280] = fma(0.0818, q, out[5280]);
      out[5568] = fma(0.0818, q, out[5568]);
      out[5760] = fma(0.0818, q, out[5760]);
      out[5888] = fma(0.0818, q, out[5888]);
      out[5632] = fma(0.0818, q, out[5632]);
      out[5408] = fma(0.0818, q, out[5408]);
      out[5152] = fma(0.0818, q, out[5152]);
      out[5120] = fma(0.222, q, out[5120]);
    }
    if (mask[515]) {
      const double q = scale * ws[75808];
      out[4704] = out[4704] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0023, q, out[4768]);
      out[4864] = fma(0.134, q, out[4864]);
      out[4832] = fma(0.3349, q, out[4832]);
      out[4896] = fma(0.008, q, out[4896]);
      out[4640] = fma(0.1193, q, out[4640]);
      out[4416] = fma(0.0758, q, out[4416]);
      out[4928] = fma(0.0292, q, out[4928]);
      out[4960] = fma(0.0766, q, out[4960]);
      out[4992] = fma(0.0277, q, out[4992]);
      out[4704] = fma(0.0118, q, out[4704]);
      out[5088] = fma(0.0651, q, out[5088]);
      out[5536] = fma(0.0709, q, out[5536]);
      out[5312] = fma(0.0668, q, out[5312]);
      out[4224] = fma(0.0423, q, out[4224]);
      out[3968] = fma(0.0911, q, out[3968]);
      out[4608] = fma(0.0066, q, out[4608]);
      out[5728] = fma(0.0025, q, out[5728]);
      out[5472] = fma(0.0297, q, out[5472]);
      out[5344] = fma(0.0297, q, out[5344]);
      out[5280] = fma(0.0297, q, out[5280]);
      out[5568] = fma(0.0297, q, out[5568]);
      out[5760] = fma(0.0297, q, out[5760]);
      out[5888] = fma(0.0297, q, out[5888]);
      out[5632] = fma(0.0297, q, out[5632]);
      out[5408] = fma(0.0297, q, out[5408]);
      out[5152] = fma(0.0297, q, out[5152]);
      out[5120] = fma(0.0654, q, out[5120]);
    }
    if (mask[516]) {
      const double q = scale * ws[75840];
      out[5088] = out[5088] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0445, q, out[4768]);
      out[4864] = fma(0.1726, q, out[4864]);
      out[4832] = fma(0.0104, q, out[4832]);
      out[4896] = fma(0.0513, q, out[4896]);
      out[4640] = fma(0.1118, q, out[4640]);
      out[4416] = fma(0.0013, q, out[4416]);
      out[4928] = fma(0.1337, q, out[4928]);
      out[4960] = fma(0.0403, q, out[4960]);
      out[4992] = fma(0.0511, q, out[4992]);
      out[4704] = fma(0.0068, q, out[4704]);
      out[5088] = fma(0.0236, q, out[5088]);
      out[5536] = fma(0.0293, q, out[5536]);
      out[5312] = fma(0.0733, q, out[5312]);
      out[4224] = fma(0.0523, q, out[4224]);
      out[3968] = fma(0.0595, q, out[3968]);
      out[4608] = fma(0.0041, q, out[4608]);
      out[5728] = fma(0.0023, q, out[5728]);
      out[5472] = fma(0.0628, q, out[5472]);
      out[5344] = fma(0.0628, q, out[5344]);
      out[5280] = fma(0.0628, q, out[5280]);
      out[5568] = fma(0.0628, q, out[5568]);
      out[5760] = fma(0.0628, q, out[5760]);
      out[5888] = fma(0.0628, q, out[5888]);
      out[5632] = fma(0.0628, q, out[5632]);
      out[5408] = fma(0.0628, q, out[5408]);
      out[5152] = fma(0.0628, q, out[5152]);
      out[5120] = fma(0.1489, q, out[5120]);
    }
    if (mask[517]) {
      const double q = scale * ws[75872];
      out[5536] = out[5536] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0317, q, out[4768]);
      out[4864] = fma(0.0765, q, out[4864]);
      out[4832] = fma(0.0009, q, out[4832]);
      out[4896] = fma(0.0526, q, out[4896]);
      out[4640] = fma(0.0489, q, out[4640]);
      out[4928] = fma(0.155, q, out[4928]);
      out[4960] = fma(0.0155, q, out[4960]);
      out[4992] = fma(0.1051, q, out[4992]);
      out[4704] = fma(0.0013, q, out[4704]);
      out[5088] = fma(0.0535, q, out[5088]);
      out[5536] = fma(0.0086, q, out[5536]);
      out[5312] = fma(0.0426, q, out[5312]);
      out[4224] = fma(0.0582, q, out[4224]);
      out[3968] = fma(0.0661, q, out[3968]);
      out[4608] = fma(0.0506, q, out[4608]);
      out[5728] = fma(0.0114, q, out[5728]);
      out[5472] = fma(0.0698, q, out[5472]);
      out[5344] = fma(0.0698, q, out[5344]);
      out[5280] = fma(0.0698, q, out[5280]);
      out[5568] = fma(0.0698, q, out[5568]);
      out[5760] = fma(0.0698, q, out[5760]);
      out[5888] = fma(0.0698, q, out[5888]);
      out[5632] = fma(0.0698, q, out[5632]);
      out[5408] = fma(0.0698, q, out[5408]);
      out[5152] = fma(0.0698, q, out[5152]);
      out[5120] = fma(0.1656, q, out[5120]);
    }
    if (mask[518]) {
      const double q = scale * ws[75904];
      out[5312] = out[5312] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.0117, q, out[4768]);
      out[4864] = fma(0.0167, q, out[4864]);
      out[4896] = fma(0.048, q, out[4896]);
      out[4640] = fma(0.0246, q, out[4640]);
      out[4928] = fma(0.0881, q, out[4928]);
      out[4992] = fma(0.0916, q, out[4992]);
      out[4704] = fma(0.0073, q, out[4704]);
      out[5088] = fma(0.0972, q, out[5088]);
      out[5536] = fma(0.0456, q, out[5536]);
      out[5312] = fma(0.0024, q, out[5312]);
      out[4224] = fma(0.0479, q, out[4224]);
      out[3968] = fma(0.0745, q, out[3968]);
      out[4608] = fma(0.0607, q, out[4608]);
      out[5728] = fma(0.0155, q, out[5728]);
      out[5472] = fma(0.0786, q, out[5472]);
      out[5344] = fma(0.0786, q, out[5344]);
      out[5280] = fma(0.0786, q, out[5280]);
      out[5568] = fma(0.0786, q, out[5568]);
      out[5760] = fma(0.0786, q, out[5760]);
      out[5888] = fma(0.0786, q, out[5888]);
      out[5632] = fma(0.0786, q, out[5632]);
      out[5408] = fma(0.0786, q, out[5408]);
      out[5152] = fma(0.0786, q, out[5152]);
      out[5120] = fma(0.173, q, out[5120]);
    }
    if (mask[519]) {
      const double q = scale * ws[75936];
      out[4224] = out[4224] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4864] = fma(0.0103, q, out[4864]);
      out[4832] = fma(0.0006, q, out[4832]);
      out[4896] = fma(0.009, q, out[4896]);
      out[4640] = fma(0.0146, q, out[4640]);
      out[4928] = fma(0.0702, q, out[4928]);
      out[4960] = fma(0.0153, q, out[4960]);
      out[4992] = fma(0.1038, q, out[4992]);
      out[4704] = fma(0.0031, q, out[4704]);
      out[5088] = fma(0.165, q, out[5088]);
      out[5536] = fma(0.1566, q, out[5536]);
      out[5312] = fma(0.0724, q, out[5312]);
      out[4224] = fma(0.0062, q, out[4224]);
      out[3968] = fma(0.1398, q, out[3968]);
      out[4608] = fma(0.0216, q, out[4608]);
      out[5728] = fma(0.0384, q, out[5728]);
      out[5472] = fma(0.0526, q, out[5472]);
      out[5344] = fma(0.0526, q, out[5344]);
      out[5280] = fma(0.0526, q, out[5280]);
      out[5568] = fma(0.0526, q, out[5568]);
      out[5760] = fma(0.0526, q, out[5760]);
      out[5888] = fma(0.0526, q, out[5888]);
      out[5632] = fma(0.0526, q, out[5632]);
      out[5408] = fma(0.0526, q, out[5408]);
      out[5152] = fma(0.0526, q, out[5152]);
      out[5120] = fma(0.128, q, out[5120]);
    }
    if (mask[520]) {
      const double q = scale * ws[75968];
      out[3968] = out[3968] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4896] = fma(0.0061, q, out[4896]);
      out[4640] = fma(0.0049, q, out[4640]);
      out[4928] = fma(0.0224, q, out[4928]);
      out[4992] = fma(0.0503, q, out[4992]);
      out[4704] = fma(0.0022, q, out[4704]);
      out[5088] = fma(0.0879, q, out[5088]);
      out[5536] = fma(0.1384, q, out[5536]);
      out[5312] = fma(0.1463, q, out[5312]);
      out[4224] = fma(0.0432, q, out[4224]);
      out[3968] = fma(0.0957, q, out[3968]);
      out[4608] = fma(0.0316, q, out[4608]);
      out[5728] = fma(0.0585, q, out[5728]);
      out[5472] = fma(0.0571, q, out[5472]);
      out[5344] = fma(0.0571, q, out[5344]);
      out[5280] = fma(0.0571, q, out[5280]);
      out[5568] = fma(0.0571, q, out[5568]);
      out[5760] = fma(0.0571, q, out[5760]);
      out[5888] = fma(0.0571, q, out[5888]);
      out[5632] = fma(0.0571, q, out[5632]);
      out[5408] = fma(0.0571, q, out[5408]);
      out[5152] = fma(0.0571, q, out[5152]);
      out[5120] = fma(0.1544, q, out[5120]);
    }
}
__device__ __noinline__ void ddm_src_1_9(double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff)
{
    double* __restrict__ out = ws + outoff * 32;
    if (mask[521]) {
      const double q = scale * ws[76000];
      out[4608] = out[4608] - q;
      out[6016] = out[6016] - q;
      out[6016] = fma(1.0, q, out[6016]);
      out[4768] = fma(0.1188, q, out[4768]);
      out[4864] = fma(0.0008, q, out[4864]);
      out[4896] = fma(0.039, q, out[4896]);
      out[4928] = fma(0.0114, q, out[4928]);
      out[5472] = fma(0.2266, q, out[5472]);
      out[5280] = fma(0.2266, q, out[5280]);
      out[5568] = fma(0.2266, q, out[5568]);
      out[5760] = fma(0.2266, q, out[5760]);
      out[5888] = fma(0.2266, q, out[5888]);
      out[5632] = fma(0.2266, q, out[5632]);
      out[5408] = fma(0.2266, q, out[5408]);
      out[5152] = fma(0.2266, q, out[5152]);
    }
    if (mask[522]) {
      const double q = scale * ws[76032];
      out[928] = out[928] - q;
      out[6016] = out[6016] - q;
      out[5888] = fma(1.0, q, out[5888]);
    }
    if (mask[523]) {
      const double q = scale * ws[76064];
      out[96] = out[96] - q;
      out[960] = fma(1.0, q, out[960]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[524]) {
      const double q = scale * ws[76096];
      out[128] = out[128] - q;
      out[960] = fma(1.0, q, out[960]);
      out[5024] = fma(1.0, q, out[5024]);
    }
    if (mask[525]) {
      const double q = scale * ws[76128];
      out[992] = out[992] - q;
      out[6016] = out[6016] - q;
      out[3488] = fma(1.0, q, out[3488]);
    }
    if (mask[526]) {
      const double q = scale * ws[76160];
      out[3488] = out[3488] - q;
      out[5984] = out[5984] - q;
      out[5536] = fma(1.0, q, out[5536]);
    }
    if (mask[527]) {
      const double q = scale * ws[76192];
      out[3488] = out[3488] - q;
      out[5824] = out[5824] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[528]) {
      const double q = scale * ws[76224];
      out[3488] = out[3488] - q;
      out[5952] = out[5952] - q;
      out[5920] = fma(1.0, q, out[5920]);
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[4448] = fma(1.0, q, out[4448]);
    }
    if (mask[529]) {
      const double q = scale * ws[76256];
      out[3488] = out[3488] - q;
      out[5888] = out[5888] - q;
      out[5984] = fma(1.37, q, out[5984]);
      out[5856] = fma(1.68, q, out[5856]);
      out[4448] = fma(1.0, q, out[4448]);
      out[5600] = fma(0.32, q, out[5600]);
    }
    if (mask[530]) {
      const double q = scale * ws[76288];
      out[3488] = out[3488] - q;
      out[5792] = out[5792] - q;
      out[5984] = fma(1.0, q, out[5984]);
      out[5856] = fma(1.0, q, out[5856]);
      out[4448] = fma(1.0, q, out[4448]);
      out[5888] = fma(0.7, q, out[5888]);
      out[5696] = fma(0.3, q, out[5696]);
    }
}
}  // namespace mech_cracmm2
