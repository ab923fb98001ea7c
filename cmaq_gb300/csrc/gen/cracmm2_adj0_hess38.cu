// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_hess3_0_32(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    double* __restrict__ lam = ws + 222656;
    const double* __restrict__ n1 = ws + 228704;
    const double* __restrict__ k1 = ws + 24192;
    const double* __restrict__ n2 = ws + 234752;
    const double* __restrict__ k2 = ws + 30240;
    const double* __restrict__ n3 = ws + 240800;
    const double* __restrict__ k3 = ws + 36288;
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(0.1188, n1[4768], w1);
      w1 = fma(0.0008, n1[4864], w1);
      w1 = fma(0.039, n1[4896], w1);
      w1 = fma(0.0114, n1[4928], w1);
      w1 = fma(0.2266, n1[5472], w1);
      w1 = fma(0.2266, n1[5280], w1);
      w1 = fma(0.2266, n1[5568], w1);
      w1 = fma(0.2266, n1[5760], w1);
      w1 = fma(0.2266, n1[5888], w1);
      w1 = fma(0.2266, n1[5632], w1);
      w1 = fma(0.2266, n1[5408], w1);
      w1 = fma(0.2266, n1[5152], w1);
      w1 = w1 - n1[4608];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[6016];
      w2 = fma(0.1188, n2[4768], w2);
      w2 = fma(0.0008, n2[4864], w2);
      w2 = fma(0.039, n2[4896], w2);
      w2 = fma(0.0114, n2[4928], w2);
      w2 = fma(0.2266, n2[5472], w2);
      w2 = fma(0.2266, n2[5280], w2);
      w2 = fma(0.2266, n2[5568], w2);
      w2 = fma(0.2266, n2[5760], w2);
      w2 = fma(0.2266, n2[5888], w2);
      w2 = fma(0.2266, n2[5632], w2);
      w2 = fma(0.2266, n2[5408], w2);
      w2 = fma(0.2266, n2[5152], w2);
      w2 = w2 - n2[4608];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[6016];
      w3 = fma(0.1188, n3[4768], w3);
      w3 = fma(0.0008, n3[4864], w3);
      w3 = fma(0.039, n3[4896], w3);
      w3 = fma(0.0114, n3[4928], w3);
      w3 = fma(0.2266, n3[5472], w3);
      w3 = fma(0.2266, n3[5280], w3);
      w3 = fma(0.2266, n3[5568], w3);
      w3 = fma(0.2266, n3[5760], w3);
      w3 = fma(0.2266, n3[5888], w3);
      w3 = fma(0.2266, n3[5632], w3);
      w3 = fma(0.2266, n3[5408], w3);
      w3 = fma(0.2266, n3[5152], w3);
      w3 = w3 - n3[4608];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[4608];
      wk0 = fma(w2, k2[4608], wk0);
      wk0 = fma(w3, k3[4608], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[59008];
      ws[287712] = fma(-kk, fma(y[6016], wk0, y[4608] * wk1), ws[287712]);
      lam[4608] = fma(-kk, wk1, lam[4608]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5888];
      w1 = w1 - n1[928];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5888];
      w2 = w2 - n2[928];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5888];
      w3 = w3 - n3[928];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[928];
      wk0 = fma(w2, k2[928], wk0);
      wk0 = fma(w3, k3[928], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[59040];
      ws[287744] = fma(-kk, fma(y[6016], wk0, y[928] * wk1), ws[287744]);
      lam[928] = fma(-kk, wk1, lam[928]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[960];
      w1 = fma(1.0, n1[5024], w1);
      w1 = w1 - n1[96];
      double w2 = 1.0 * n2[960];
      w2 = fma(1.0, n2[5024], w2);
      w2 = w2 - n2[96];
      double w3 = 1.0 * n3[960];
      w3 = fma(1.0, n3[5024], w3);
      w3 = w3 - n3[96];
      double wk0 = w1 * k1[96];
      wk0 = fma(w2, k2[96], wk0);
      wk0 = fma(w3, k3[96], wk0);
      const double kk = ws[59072];
      ws[287776] = fma(-kk, wk0, ws[287776]);
    }
    {
      double w1 = 1.0 * n1[960];
      w1 = fma(1.0, n1[5024], w1);
      w1 = w1 - n1[128];
      double w2 = 1.0 * n2[960];
      w2 = fma(1.0, n2[5024], w2);
      w2 = w2 - n2[128];
      double w3 = 1.0 * n3[960];
      w3 = fma(1.0, n3[5024], w3);
      w3 = w3 - n3[128];
      double wk0 = w1 * k1[128];
      wk0 = fma(w2, k2[128], wk0);
      wk0 = fma(w3, k3[128], wk0);
      const double kk = ws[59104];
      ws[287808] = fma(-kk, wk0, ws[287808]);
    }
    {
      double w1 = 1.0 * n1[3488];
      w1 = w1 - n1[992];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[3488];
      w2 = w2 - n2[992];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[3488];
      w3 = w3 - n3[992];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[992];
      wk0 = fma(w2, k2[992], wk0);
      wk0 = fma(w3, k3[992], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[59136];
      ws[287840] = fma(-kk, fma(y[6016], wk0, y[992] * wk1), ws[287840]);
      lam[992] = fma(-kk, wk1, lam[992]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5536];
      w1 = w1 - n1[3488];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[5536];
      w2 = w2 - n2[3488];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[5536];
      w3 = w3 - n3[3488];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[3488];
      wk0 = fma(w2, k2[3488], wk0);
      wk0 = fma(w3, k3[3488], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[59168];
      ws[287872] = fma(-kk, fma(y[5984], wk0, y[3488] * wk1), ws[287872]);
      lam[3488] = fma(-kk, wk1, lam[3488]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5856], w1);
      w1 = fma(1.0, n1[4448], w1);
      w1 = w1 - n1[3488];
      w1 = w1 - n1[5824];
      double w2 = 1.0 * n2[5920];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5856], w2);
      w2 = fma(1.0, n2[4448], w2);
      w2 = w2 - n2[3488];
      w2 = w2 - n2[5824];
      double w3 = 1.0 * n3[5920];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5856], w3);
      w3 = fma(1.0, n3[4448], w3);
      w3 = w3 - n3[3488];
      w3 = w3 - n3[5824];
      double wk0 = w1 * k1[3488];
      wk0 = fma(w2, k2[3488], wk0);
      wk0 = fma(w3, k3[3488], wk0);
      double wk1 = w1 * k1[5824];
      wk1 = fma(w2, k2[5824], wk1);
      wk1 = fma(w3, k3[5824], wk1);
      const double kk = ws[59200];
      ws[287904] = fma(-kk, fma(y[5824], wk0, y[3488] * wk1), ws[287904]);
      lam[3488] = fma(-kk, wk1, lam[3488]);
      lam[5824] = fma(-kk, wk0, lam[5824]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5856], w1);
      w1 = fma(1.0, n1[4448], w1);
      w1 = w1 - n1[3488];
      w1 = w1 - n1[5952];
      double w2 = 1.0 * n2[5920];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5856], w2);
      w2 = fma(1.0, n2[4448], w2);
      w2 = w2 - n2[3488];
      w2 = w2 - n2[5952];
      double w3 = 1.0 * n3[5920];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5856], w3);
      w3 = fma(1.0, n3[4448], w3);
      w3 = w3 - n3[3488];
      w3 = w3 - n3[5952];
      double wk0 = w1 * k1[3488];
      wk0 = fma(w2, k2[3488], wk0);
      wk0 = fma(w3, k3[3488], wk0);
      double wk1 = w1 * k1[5952];
      wk1 = fma(w2, k2[5952], wk1);
      wk1 = fma(w3, k3[5952], wk1);
      const double kk = ws[59232];
      ws[287936] = fma(-kk, fma(y[5952], wk0, y[3488] * wk1), ws[287936]);
      lam[3488] = fma(-kk, wk1, lam[3488]);
      lam[5952] = fma(-kk, wk0, lam[5952]);
    }
    {
      double w1 = 1.37 * n1[5984];
      w1 = fma(1.68, n1[5856], w1);
      w1 = fma(1.0, n1[4448], w1);
      w1 = fma(0.32, n1[5600], w1);
      w1 = w1 - n1[3488];
      w1 = w1 - n1[5888];
      double w2 = 1.37 * n2[5984];
      w2 = fma(1.68, n2[5856], w2);
      w2 = fma(1.0, n2[4448], w2);
      w2 = fma(0.32, n2[5600], w2);
      w2 = w2 - n2[3488];
      w2 = w2 - n2[5888];
      double w3 = 1.37 * n3[5984];
      w3 = fma(1.68, n3[5856], w3);
      w3 = fma(1.0, n3[4448], w3);
      w3 = fma(0.32, n3[5600], w3);
      w3 = w3 - n3[3488];
      w3 = w3 - n3[5888];
      double wk0 = w1 * k1[3488];
      wk0 = fma(w2, k2[3488], wk0);
      wk0 = fma(w3, k3[3488], wk0);
      double wk1 = w1 * k1[5888];
      wk1 = fma(w2, k2[5888], wk1);
      wk1 = fma(w3, k3[5888], wk1);
      const double kk = ws[59264];
      ws[287968] = fma(-kk, fma(y[5888], wk0, y[3488] * wk1), ws[287968]);
      lam[3488] = fma(-kk, wk1, lam[3488]);
      lam[5888] = fma(-kk, wk0, lam[5888]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5856], w1);
      w1 = fma(1.0, n1[4448], w1);
      w1 = fma(0.7, n1[5888], w1);
      w1 = fma(0.3, n1[5696], w1);
      w1 = w1 - n1[3488];
      w1 = w1 - n1[5792];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5856], w2);
      w2 = fma(1.0, n2[4448], w2);
      w2 = fma(0.7, n2[5888], w2);
      w2 = fma(0.3, n2[5696], w2);
      w2 = w2 - n2[3488];
      w2 = w2 - n2[5792];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5856], w3);
      w3 = fma(1.0, n3[4448], w3);
      w3 = fma(0.7, n3[5888], w3);
      w3 = fma(0.3, n3[5696], w3);
      w3 = w3 - n3[3488];
      w3 = w3 - n3[5792];
      double wk0 = w1 * k1[3488];
      wk0 = fma(w2, k2[3488], wk0);
      wk0 = fma(w3, k3[3488], wk0);
      double wk1 = w1 * k1[5792];
      wk1 = fma(w2, k2[5792], wk1);
      wk1 = fma(w3, k3[5792], wk1);
      const double kk = ws[59296];
      ws[288000] = fma(-kk, fma(y[5792], wk0, y[3488] * wk1), ws[288000]);
      lam[3488] = fma(-kk, wk1, lam[3488]);
      lam[5792] = fma(-kk, wk0, lam[5792]);
    }
}
}  // namespace mech_cracmm2
