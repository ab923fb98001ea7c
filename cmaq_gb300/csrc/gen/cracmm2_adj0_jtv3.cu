// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_jtv_0_12(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[6016];
      w = fma(0.2822, phi[4768], w);
      w = fma(0.1165, phi[4864], w);
      w = fma(0.032, phi[4896], w);
      w = fma(0.0183, phi[4640], w);
      w = fma(0.0011, phi[4928], w);
      w = fma(0.066, phi[5088], w);
      w = fma(0.0535, phi[5536], w);
      w = fma(0.0246, phi[5312], w);
      w = fma(0.0054, phi[5728], w);
      w = fma(0.1068, phi[5472], w);
      w = fma(0.1068, phi[5280], w);
      w = fma(0.1068, phi[5504], w);
      w = fma(0.1068, phi[5568], w);
      w = fma(0.1068, phi[5760], w);
      w = fma(0.1068, phi[5888], w);
      w = fma(0.1068, phi[5632], w);
      w = fma(0.1068, phi[5408], w);
      w = fma(0.1068, phi[5152], w);
      w = fma(0.1068, phi[5120], w);
      w = fma(0.1068, phi[3776], w);
      w = w - phi[4928];
      w = w - phi[6016];
      const double kw = ws[58720] * w;
      out[4928] = fma(kw, y[6016], out[4928]);
      out[6016] = fma(kw, y[4928], out[6016]);
      ws[287424] = fma(kw * y[4928], y[6016], ws[287424]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0659, phi[4768], w);
      w = fma(0.4579, phi[4864], w);
      w = fma(0.1156, phi[4832], w);
      w = fma(0.0325, phi[4896], w);
      w = fma(0.0657, phi[4640], w);
      w = fma(0.0046, phi[4416], w);
      w = fma(0.0307, phi[4928], w);
      w = fma(0.0024, phi[4960], w);
      w = fma(0.0395, phi[4992], w);
      w = fma(0.0215, phi[4704], w);
      w = fma(0.0539, phi[5088], w);
      w = fma(0.0516, phi[5536], w);
      w = fma(0.0519, phi[5312], w);
      w = fma(0.0371, phi[4224], w);
      w = fma(0.0421, phi[3968], w);
      w = fma(0.0105, phi[4608], w);
      w = fma(0.0445, phi[5472], w);
      w = fma(0.0445, phi[5344], w);
      w = fma(0.0445, phi[5280], w);
      w = fma(0.0445, phi[5568], w);
      w = fma(0.0445, phi[5760], w);
      w = fma(0.0445, phi[5888], w);
      w = fma(0.0445, phi[5632], w);
      w = fma(0.0445, phi[5408], w);
      w = fma(0.0445, phi[5152], w);
      w = fma(0.1055, phi[5120], w);
      w = w - phi[4960];
      w = w - phi[6016];
      const double kw = ws[58752] * w;
      out[4960] = fma(kw, y[6016], out[4960]);
      out[6016] = fma(kw, y[4960], out[6016]);
      ws[287456] = fma(kw * y[4960], y[6016], ws[287456]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.1778, phi[4768], w);
      w = fma(0.1924, phi[4864], w);
      w = fma(0.0004, phi[4832], w);
      w = fma(0.074, phi[4896], w);
      w = fma(0.0452, phi[4640], w);
      w = fma(0.0631, phi[4928], w);
      w = fma(0.0007, phi[4960], w);
      w = fma(0.0006, phi[4992], w);
      w = fma(0.0227, phi[5088], w);
      w = fma(0.0585, phi[5536], w);
      w = fma(0.0649, phi[5312], w);
      w = fma(0.0174, phi[4224], w);
      w = fma(0.0154, phi[4608], w);
      w = fma(0.017, phi[5728], w);
      w = fma(0.0818, phi[5472], w);
      w = fma(0.0818, phi[5344], w);
      w = fma(0.0818, phi[5280], w);
      w = fma(0.0818, phi[5568], w);
      w = fma(0.0818, phi[5760], w);
      w = fma(0.0818, phi[5888], w);
      w = fma(0.0818, phi[5632], w);
      w = fma(0.0818, phi[5408], w);
      w = fma(0.0818, phi[5152], w);
      w = fma(0.222, phi[5120], w);
      w = w - phi[4992];
      w = w - phi[6016];
      const double kw = ws[58784] * w;
      out[4992] = fma(kw, y[6016], out[4992]);
      out[6016] = fma(kw, y[4992], out[6016]);
      ws[287488] = fma(kw * y[4992], y[6016], ws[287488]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0023, phi[4768], w);
      w = fma(0.134, phi[4864], w);
      w = fma(0.3349, phi[4832], w);
      w = fma(0.008, phi[4896], w);
      w = fma(0.1193, phi[4640], w);
      w = fma(0.0758, phi[4416], w);
      w = fma(0.0292, phi[4928], w);
      w = fma(0.0766, phi[4960], w);
      w = fma(0.0277, phi[4992], w);
      w = fma(0.0118, phi[4704], w);
      w = fma(0.0651, phi[5088], w);
      w = fma(0.0709, phi[5536], w);
      w = fma(0.0668, phi[5312], w);
      w = fma(0.0423, phi[4224], w);
      w = fma(0.0911, phi[3968], w);
      w = fma(0.0066, phi[4608], w);
      w = fma(0.0025, phi[5728], w);
      w = fma(0.0297, phi[5472], w);
      w = fma(0.0297, phi[5344], w);
      w = fma(0.0297, phi[5280], w);
      w = fma(0.0297, phi[5568], w);
      w = fma(0.0297, phi[5760], w);
      w = fma(0.0297, phi[5888], w);
      w = fma(0.0297, phi[5632], w);
      w = fma(0.0297, phi[5408], w);
      w = fma(0.0297, phi[5152], w);
      w = fma(0.0654, phi[5120], w);
      w = w - phi[4704];
      w = w - phi[6016];
      const double kw = ws[58816] * w;
      out[4704] = fma(kw, y[6016], out[4704]);
      out[6016] = fma(kw, y[4704], out[6016]);
      ws[287520] = fma(kw * y[4704], y[6016], ws[287520]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0445, phi[4768], w);
      w = fma(0.1726, phi[4864], w);
      w = fma(0.0104, phi[4832], w);
      w = fma(0.0513, phi[4896], w);
      w = fma(0.1118, phi[4640], w);
      w = fma(0.0013, phi[4416], w);
      w = fma(0.1337, phi[4928], w);
      w = fma(0.0403, phi[4960], w);
      w = fma(0.0511, phi[4992], w);
      w = fma(0.0068, phi[4704], w);
      w = fma(0.0236, phi[5088], w);
      w = fma(0.0293, phi[5536], w);
      w = fma(0.0733, phi[5312], w);
      w = fma(0.0523, phi[4224], w);
      w = fma(0.0595, phi[3968], w);
      w = fma(0.0041, phi[4608], w);
      w = fma(0.0023, phi[5728], w);
      w = fma(0.0628, phi[5472], w);
      w = fma(0.0628, phi[5344], w);
      w = fma(0.0628, phi[5280], w);
      w = fma(0.0628, phi[5568], w);
      w = fma(0.0628, phi[5760], w);
      w = fma(0.0628, phi[5888], w);
      w = fma(0.0628, phi[5632], w);
      w = fma(0.0628, phi[5408], w);
      w = fma(0.0628, phi[5152], w);
      w = fma(0.1489, phi[5120], w);
      w = w - phi[5088];
      w = w - phi[6016];
      const double kw = ws[58848] * w;
      out[5088] = fma(kw, y[6016], out[5088]);
      out[6016] = fma(kw, y[5088], out[6016]);
      ws[287552] = fma(kw * y[5088], y[6016], ws[287552]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0317, phi[4768], w);
      w = fma(0.0765, phi[4864], w);
      w = fma(0.0009, phi[4832], w);
      w = fma(0.0526, phi[4896], w);
      w = fma(0.0489, phi[4640], w);
      w = fma(0.155, phi[4928], w);
      w = fma(0.0155, phi[4960], w);
      w = fma(0.1051, phi[4992], w);
      w = fma(0.0013, phi[4704], w);
      w = fma(0.0535, phi[5088], w);
      w = fma(0.0086, phi[5536], w);
      w = fma(0.0426, phi[5312], w);
      w = fma(0.0582, phi[4224], w);
      w = fma(0.0661, phi[3968], w);
      w = fma(0.0506, phi[4608], w);
      w = fma(0.0114, phi[5728], w);
      w = fma(0.0698, phi[5472], w);
      w = fma(0.0698, phi[5344], w);
      w = fma(0.0698, phi[5280], w);
      w = fma(0.0698, phi[5568], w);
      w = fma(0.0698, phi[5760], w);
      w = fma(0.0698, phi[5888], w);
      w = fma(0.0698, phi[5632], w);
      w = fma(0.0698, phi[5408], w);
      w = fma(0.0698, phi[5152], w);
      w = fma(0.1656, phi[5120], w);
      w = w - phi[5536];
      w = w - phi[6016];
      const double kw = ws[58880] * w;
      out[5536] = fma(kw, y[6016], out[5536]);
      out[6016] = fma(kw, y[5536], out[6016]);
      ws[287584] = fma(kw * y[5536], y[6016], ws[287584]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0117, phi[4768], w);
      w = fma(0.0167, phi[4864], w);
      w = fma(0.048, phi[4896], w);
      w = fma(0.0246, phi[4640], w);
      w = fma(0.0881, phi[4928], w);
      w = fma(0.0916, phi[4992], w);
      w = fma(0.0073, phi[4704], w);
      w = fma(0.0972, phi[5088], w);
      w = fma(0.0456, phi[5536], w);
      w = fma(0.0024, phi[5312], w);
      w = fma(0.0479, phi[4224], w);
      w = fma(0.0745, phi[3968], w);
      w = fma(0.0607, phi[4608], w);
      w = fma(0.0155, phi[5728], w);
      w = fma(0.0786, phi[5472], w);
      w = fma(0.0786, phi[5344], w);
      w = fma(0.0786, phi[5280], w);
      w = fma(0.0786, phi[5568], w);
      w = fma(0.0786, phi[5760], w);
      w = fma(0.0786, phi[5888], w);
      w = fma(0.0786, phi[5632], w);
      w = fma(0.0786, phi[5408], w);
      w = fma(0.0786, phi[5152], w);
      w = fma(0.173, phi[5120], w);
      w = w - phi[5312];
      w = w - phi[6016];
      const double kw = ws[58912] * w;
      out[5312] = fma(kw, y[6016], out[5312]);
      out[6016] = fma(kw, y[5312], out[6016]);
      ws[287616] = fma(kw * y[5312], y[6016], ws[287616]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0103, phi[4864], w);
      w = fma(0.0006, phi[4832], w);
      w = fma(0.009, phi[4896], w);
      w = fma(0.0146, phi[4640], w);
      w = fma(0.0702, phi[4928], w);
      w = fma(0.0153, phi[4960], w);
      w = fma(0.1038, phi[4992], w);
      w = fma(0.0031, phi[4704], w);
      w = fma(0.165, phi[5088], w);
      w = fma(0.1566, phi[5536], w);
      w = fma(0.0724, phi[5312], w);
      w = fma(0.0062, phi[4224], w);
      w = fma(0.1398, phi[3968], w);
      w = fma(0.0216, phi[4608], w);
      w = fma(0.0384, phi[5728], w);
      w = fma(0.0526, phi[5472], w);
      w = fma(0.0526, phi[5344], w);
      w = fma(0.0526, phi[5280], w);
      w = fma(0.0526, phi[5568], w);
      w = fma(0.0526, phi[5760], w);
      w = fma(0.0526, phi[5888], w);
      w = fma(0.0526, phi[5632], w);
      w = fma(0.0526, phi[5408], w);
      w = fma(0.0526, phi[5152], w);
      w = fma(0.128, phi[5120], w);
      w = w - phi[4224];
      w = w - phi[6016];
      const double kw = ws[58944] * w;
      out[4224] = fma(kw, y[6016], out[4224]);
      out[6016] = fma(kw, y[4224], out[6016]);
      ws[287648] = fma(kw * y[4224], y[6016], ws[287648]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0061, phi[4896], w);
      w = fma(0.0049, phi[4640], w);
      w = fma(0.0224, phi[4928], w);
      w = fma(0.0503, phi[4992], w);
      w = fma(0.0022, phi[4704], w);
      w = fma(0.0879, phi[5088], w);
      w = fma(0.1384, phi[5536], w);
      w = fma(0.1463, phi[5312], w);
      w = fma(0.0432, phi[4224], w);
      w = fma(0.0957, phi[3968], w);
      w = fma(0.0316, phi[4608], w);
      w = fma(0.0585, phi[5728], w);
      w = fma(0.0571, phi[5472], w);
      w = fma(0.0571, phi[5344], w);
      w = fma(0.0571, phi[5280], w);
      w = fma(0.0571, phi[5568], w);
      w = fma(0.0571, phi[5760], w);
      w = fma(0.0571, phi[5888], w);
      w = fma(0.0571, phi[5632], w);
      w = fma(0.0571, phi[5408], w);
      w = fma(0.0571, phi[5152], w);
      w = fma(0.1544, phi[5120], w);
      w = w - phi[3968];
      w = w - phi[6016];
      const double kw = ws[58976] * w;
      out[3968] = fma(kw, y[6016], out[3968]);
      out[6016] = fma(kw, y[3968], out[6016]);
      ws[287680] = fma(kw * y[3968], y[6016], ws[287680]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.1188, phi[4768], w);
      w = fma(0.0008, phi[4864], w);
      w = fma(0.039, phi[4896], w);
      w = fma(0.0114, phi[4928], w);
      w = fma(0.2266, phi[5472], w);
      w = fma(0.2266, phi[5280], w);
      w = fma(0.2266, phi[5568], w);
      w = fma(0.2266, phi[5760], w);
      w = fma(0.2266, phi[5888], w);
      w = fma(0.2266, phi[5632], w);
      w = fma(0.2266, phi[5408], w);
      w = fma(0.2266, phi[5152], w);
      w = w - phi[4608];
      w = w - phi[6016];
      const double kw = ws[59008] * w;
      out[4608] = fma(kw, y[6016], out[4608]);
      out[6016] = fma(kw, y[4608], out[6016]);
      ws[287712] = fma(kw * y[4608], y[6016], ws[287712]);
    }
    {
      double w = 1.0 * phi[5888];
      w = w - phi[928];
      w = w - phi[6016];
      const double kw = ws[59040] * w;
      out[928] = fma(kw, y[6016], out[928]);
      out[6016] = fma(kw, y[928], out[6016]);
      ws[287744] = fma(kw * y[928], y[6016], ws[287744]);
    }
    {
      double w = 1.0 * phi[960];
      w = fma(1.0, phi[5024], w);
      w = w - phi[96];
      const double kw = ws[59072] * w;
      out[96] = out[96] + kw;
      ws[287776] = fma(kw, y[96], ws[287776]);
    }
    {
      double w = 1.0 * phi[960];
      w = fma(1.0, phi[5024], w);
      w = w - phi[128];
      const double kw = ws[59104] * w;
      out[128] = out[128] + kw;
      ws[287808] = fma(kw, y[128], ws[287808]);
    }
    {
      double w = 1.0 * phi[3488];
      w = w - phi[992];
      w = w - phi[6016];
      const double kw = ws[59136] * w;
      out[992] = fma(kw, y[6016], out[992]);
      out[6016] = fma(kw, y[992], out[6016]);
      ws[287840] = fma(kw * y[992], y[6016], ws[287840]);
    }
    {
      double w = 1.0 * phi[5536];
      w = w - phi[3488];
      w = w - phi[5984];
      const double kw = ws[59168] * w;
      out[3488] = fma(kw, y[5984], out[3488]);
      out[5984] = fma(kw, y[3488], out[5984]);
      ws[287872] = fma(kw * y[3488], y[5984], ws[287872]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = w - phi[3488];
      w = w - phi[5824];
      const double kw = ws[59200] * w;
      out[3488] = fma(kw, y[5824], out[3488]);
      out[5824] = fma(kw, y[3488], out[5824]);
      ws[287904] = fma(kw * y[3488], y[5824], ws[287904]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = w - phi[3488];
      w = w - phi[5952];
      const double kw = ws[59232] * w;
      out[3488] = fma(kw, y[5952], out[3488]);
      out[5952] = fma(kw, y[3488], out[5952]);
      ws[287936] = fma(kw * y[3488], y[5952], ws[287936]);
    }
    {
      double w = 1.37 * phi[5984];
      w = fma(1.68, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = fma(0.32, phi[5600], w);
      w = w - phi[3488];
      w = w - phi[5888];
      const double kw = ws[59264] * w;
      out[3488] = fma(kw, y[5888], out[3488]);
      out[5888] = fma(kw, y[3488], out[5888]);
      ws[287968] = fma(kw * y[3488], y[5888], ws[287968]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = fma(0.7, phi[5888], w);
      w = fma(0.3, phi[5696], w);
      w = w - phi[3488];
      w = w - phi[5792];
      const double kw = ws[59296] * w;
      out[3488] = fma(kw, y[5792], out[3488]);
      out[5792] = fma(kw, y[3488], out[5792]);
      ws[288000] = fma(kw * y[3488], y[5792], ws[288000]);
    }
}
}  // namespace mech_cracmm2
