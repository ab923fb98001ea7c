// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_hess3_0_0(double* __restrict__ ws)
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
      double w1 = 1.0 * n1[2336];
      w1 = w1 - n1[5184];
      double w2 = 1.0 * n2[2336];
      w2 = w2 - n2[5184];
      double w3 = 1.0 * n3[2336];
      w3 = w3 - n3[5184];
      double wk0 = w1 * k1[5184];
      wk0 = fma(w2, k2[5184], wk0);
      wk0 = fma(w3, k3[5184], wk0);
      const double kk = ws[42336];
      ws[271040] = fma(-kk, wk0, ws[271040]);
    }
    {
      double w1 = 1.0 * n1[576];
      w1 = w1 - n1[5184];
      double w2 = 1.0 * n2[576];
      w2 = w2 - n2[5184];
      double w3 = 1.0 * n3[576];
      w3 = w3 - n3[5184];
      double wk0 = w1 * k1[5184];
      wk0 = fma(w2, k2[5184], wk0);
      wk0 = fma(w3, k3[5184], wk0);
      const double kk = ws[42368];
      ws[271072] = fma(-kk, wk0, ws[271072]);
    }
    {
      double w1 = 2.0 * n1[6016];
      w1 = w1 - n1[4000];
      double w2 = 2.0 * n2[6016];
      w2 = w2 - n2[4000];
      double w3 = 2.0 * n3[6016];
      w3 = w3 - n3[4000];
      double wk0 = w1 * k1[4000];
      wk0 = fma(w2, k2[4000], wk0);
      wk0 = fma(w3, k3[4000], wk0);
      const double kk = ws[42400];
      ws[271104] = fma(-kk, wk0, ws[271104]);
    }
    {
      double w1 = 1.0 * n1[2336];
      w1 = fma(1.0, n1[5824], w1);
      w1 = w1 - n1[5920];
      double w2 = 1.0 * n2[2336];
      w2 = fma(1.0, n2[5824], w2);
      w2 = w2 - n2[5920];
      double w3 = 1.0 * n3[2336];
      w3 = fma(1.0, n3[5824], w3);
      w3 = w3 - n3[5920];
      double wk0 = w1 * k1[5920];
      wk0 = fma(w2, k2[5920], wk0);
      wk0 = fma(w3, k3[5920], wk0);
      const double kk = ws[42432];
      ws[271136] = fma(-kk, wk0, ws[271136]);
    }
    {
      double w1 = 1.0 * n1[5824];
      w1 = w1 - n1[5952];
      double w2 = 1.0 * n2[5824];
      w2 = w2 - n2[5952];
      double w3 = 1.0 * n3[5824];
      w3 = w3 - n3[5952];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      const double kk = ws[42464];
      ws[271168] = fma(-kk, wk0, ws[271168]);
    }
    {
      double w1 = 1.0 * n1[2336];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[5952];
      double w2 = 1.0 * n2[2336];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[5952];
      double w3 = 1.0 * n3[2336];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[5952];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      const double kk = ws[42496];
      ws[271200] = fma(-kk, wk0, ws[271200]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5824], w1);
      w1 = w1 - n1[1184];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5824], w2);
      w2 = w2 - n2[1184];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5824], w3);
      w3 = w3 - n3[1184];
      double wk0 = w1 * k1[1184];
      wk0 = fma(w2, k2[1184], wk0);
      wk0 = fma(w3, k3[1184], wk0);
      const double kk = ws[42528];
      ws[271232] = fma(-kk, wk0, ws[271232]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[5024];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[5024];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[5024];
      double wk0 = w1 * k1[5024];
      wk0 = fma(w2, k2[5024], wk0);
      wk0 = fma(w3, k3[5024], wk0);
      const double kk = ws[42560];
      ws[271264] = fma(-kk, wk0, ws[271264]);
    }
    {
      double w1 = 0.2 * n1[6016];
      w1 = fma(0.8, n1[5984], w1);
      w1 = fma(0.8, n1[5920], w1);
      w1 = fma(0.2, n1[5952], w1);
      w1 = w1 - n1[1280];
      double w2 = 0.2 * n2[6016];
      w2 = fma(0.8, n2[5984], w2);
      w2 = fma(0.8, n2[5920], w2);
      w2 = fma(0.2, n2[5952], w2);
      w2 = w2 - n2[1280];
      double w3 = 0.2 * n3[6016];
      w3 = fma(0.8, n3[5984], w3);
      w3 = fma(0.8, n3[5920], w3);
      w3 = fma(0.2, n3[5952], w3);
      w3 = w3 - n3[1280];
      double wk0 = w1 * k1[1280];
      wk0 = fma(w2, k2[1280], wk0);
      wk0 = fma(w3, k3[1280], wk0);
      const double kk = ws[42592];
      ws[271296] = fma(-kk, wk0, ws[271296]);
    }
    {
      double w1 = 1.0 * n1[5664];
      w1 = w1 - n1[5856];
      double w2 = 1.0 * n2[5664];
      w2 = w2 - n2[5856];
      double w3 = 1.0 * n3[5664];
      w3 = w3 - n3[5856];
      double wk0 = w1 * k1[5856];
      wk0 = fma(w2, k2[5856], wk0);
      wk0 = fma(w3, k3[5856], wk0);
      const double kk = ws[42624];
      ws[271328] = fma(-kk, wk0, ws[271328]);
    }
    {
      double w1 = 2.0 * n1[5984];
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[5856];
      double w2 = 2.0 * n2[5984];
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[5856];
      double w3 = 2.0 * n3[5984];
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[5856];
      double wk0 = w1 * k1[5856];
      wk0 = fma(w2, k2[5856], wk0);
      wk0 = fma(w3, k3[5856], wk0);
      const double kk = ws[42656];
      ws[271360] = fma(-kk, wk0, ws[271360]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5888], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[5568];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5888], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[5568];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5888], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[5568];
      double wk0 = w1 * k1[5568];
      wk0 = fma(w2, k2[5568], wk0);
      wk0 = fma(w3, k3[5568], wk0);
      const double kk = ws[42688];
      ws[271392] = fma(-kk, wk0, ws[271392]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5632], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[5760];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5632], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[5760];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5632], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[5760];
      double wk0 = w1 * k1[5760];
      wk0 = fma(w2, k2[5760], wk0);
      wk0 = fma(w3, k3[5760], wk0);
      const double kk = ws[42720];
      ws[271424] = fma(-kk, wk0, ws[271424]);
    }
    {
      double w1 = 1.0 * n1[5888];
      w1 = fma(1.0, n1[5792], w1);
      w1 = w1 - n1[4480];
      double w2 = 1.0 * n2[5888];
      w2 = fma(1.0, n2[5792], w2);
      w2 = w2 - n2[4480];
      double w3 = 1.0 * n3[5888];
      w3 = fma(1.0, n3[5792], w3);
      w3 = w3 - n3[4480];
      double wk0 = w1 * k1[4480];
      wk0 = fma(w2, k2[4480], wk0);
      wk0 = fma(w3, k3[4480], wk0);
      const double kk = ws[42752];
      ws[271456] = fma(-kk, wk0, ws[271456]);
    }
    {
      double w1 = 2.0 * n1[5888];
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[4480];
      double w2 = 2.0 * n2[5888];
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[4480];
      double w3 = 2.0 * n3[5888];
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[4480];
      double wk0 = w1 * k1[4480];
      wk0 = fma(w2, k2[4480], wk0);
      wk0 = fma(w3, k3[4480], wk0);
      const double kk = ws[42784];
      ws[271488] = fma(-kk, wk0, ws[271488]);
    }
    {
      double w1 = 1.22 * n1[5984];
      w1 = fma(0.784, n1[5792], w1);
      w1 = fma(1.22, n1[5664], w1);
      w1 = fma(0.35, n1[5856], w1);
      w1 = fma(0.434, n1[5760], w1);
      w1 = fma(0.216, n1[5504], w1);
      w1 = w1 - n1[3872];
      double w2 = 1.22 * n2[5984];
      w2 = fma(0.784, n2[5792], w2);
      w2 = fma(1.22, n2[5664], w2);
      w2 = fma(0.35, n2[5856], w2);
      w2 = fma(0.434, n2[5760], w2);
      w2 = fma(0.216, n2[5504], w2);
      w2 = w2 - n2[3872];
      double w3 = 1.22 * n3[5984];
      w3 = fma(0.784, n3[5792], w3);
      w3 = fma(1.22, n3[5664], w3);
      w3 = fma(0.35, n3[5856], w3);
      w3 = fma(0.434, n3[5760], w3);
      w3 = fma(0.216, n3[5504], w3);
      w3 = w3 - n3[3872];
      double wk0 = w1 * k1[3872];
      wk0 = fma(w2, k2[3872], wk0);
      wk0 = fma(w3, k3[3872], wk0);
      const double kk = ws[42816];
      ws[271520] = fma(-kk, wk0, ws[271520]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[3904], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[4544];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[3904], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[4544];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[3904], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[4544];
      double wk0 = w1 * k1[4544];
      wk0 = fma(w2, k2[4544], wk0);
      wk0 = fma(w3, k3[4544], wk0);
      const double kk = ws[42848];
      ws[271552] = fma(-kk, wk0, ws[271552]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[3904], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[4576];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[3904], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[4576];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[3904], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[4576];
      double wk0 = w1 * k1[4576];
      wk0 = fma(w2, k2[4576], wk0);
      wk0 = fma(w3, k3[4576], wk0);
      const double kk = ws[42880];
      ws[271584] = fma(-kk, wk0, ws[271584]);
    }
    {
      double w1 = 0.1 * n1[5888];
      w1 = fma(1.0, n1[5632], w1);
      w1 = fma(0.9, n1[5792], w1);
      w1 = fma(0.1, n1[5664], w1);
      w1 = w1 - n1[5280];
      double w2 = 0.1 * n2[5888];
      w2 = fma(1.0, n2[5632], w2);
      w2 = fma(0.9, n2[5792], w2);
      w2 = fma(0.1, n2[5664], w2);
      w2 = w2 - n2[5280];
      double w3 = 0.1 * n3[5888];
      w3 = fma(1.0, n3[5632], w3);
      w3 = fma(0.9, n3[5792], w3);
      w3 = fma(0.1, n3[5664], w3);
      w3 = w3 - n3[5280];
      double wk0 = w1 * k1[5280];
      wk0 = fma(w2, k2[5280], wk0);
      wk0 = fma(w3, k3[5280], wk0);
      const double kk = ws[42912];
      ws[271616] = fma(-kk, wk0, ws[271616]);
    }
    {
      double w1 = 1.5 * n1[5632];
      w1 = fma(0.5, n1[5792], w1);
      w1 = fma(0.5, n1[5664], w1);
      w1 = w1 - n1[5504];
      double w2 = 1.5 * n2[5632];
      w2 = fma(0.5, n2[5792], w2);
      w2 = fma(0.5, n2[5664], w2);
      w2 = w2 - n2[5504];
      double w3 = 1.5 * n3[5632];
      w3 = fma(0.5, n3[5792], w3);
      w3 = fma(0.5, n3[5664], w3);
      w3 = w3 - n3[5504];
      double wk0 = w1 * k1[5504];
      wk0 = fma(w2, k2[5504], wk0);
      wk0 = fma(w3, k3[5504], wk0);
      const double kk = ws[42944];
      ws[271648] = fma(-kk, wk0, ws[271648]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5792], w1);
      w1 = fma(1.0, n1[5856], w1);
      w1 = w1 - n1[5344];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5792], w2);
      w2 = fma(1.0, n2[5856], w2);
      w2 = w2 - n2[5344];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5792], w3);
      w3 = fma(1.0, n3[5856], w3);
      w3 = w3 - n3[5344];
      double wk0 = w1 * k1[5344];
      wk0 = fma(w2, k2[5344], wk0);
      wk0 = fma(w3, k3[5344], wk0);
      const double kk = ws[42976];
      ws[271680] = fma(-kk, wk0, ws[271680]);
    }
    {
      double w1 = 0.34 * n1[6016];
      w1 = fma(0.66, n1[5984], w1);
      w1 = fma(0.67, n1[5792], w1);
      w1 = fma(0.33, n1[4672], w1);
      w1 = fma(0.34, n1[5216], w1);
      w1 = fma(0.67, n1[5664], w1);
      w1 = fma(0.67, n1[5856], w1);
      w1 = w1 - n1[4128];
      double w2 = 0.34 * n2[6016];
      w2 = fma(0.66, n2[5984], w2);
      w2 = fma(0.67, n2[5792], w2);
      w2 = fma(0.33, n2[4672], w2);
      w2 = fma(0.34, n2[5216], w2);
      w2 = fma(0.67, n2[5664], w2);
      w2 = fma(0.67, n2[5856], w2);
      w2 = w2 - n2[4128];
      double w3 = 0.34 * n3[6016];
      w3 = fma(0.66, n3[5984], w3);
      w3 = fma(0.67, n3[5792], w3);
      w3 = fma(0.33, n3[4672], w3);
      w3 = fma(0.34, n3[5216], w3);
      w3 = fma(0.67, n3[5664], w3);
      w3 = fma(0.67, n3[5856], w3);
      w3 = w3 - n3[4128];
      double wk0 = w1 * k1[4128];
      wk0 = fma(w2, k2[4128], wk0);
      wk0 = fma(w3, k3[4128], wk0);
      const double kk = ws[43008];
      ws[271712] = fma(-kk, wk0, ws[271712]);
    }
    {
      double w1 = 0.3 * n1[5888];
      w1 = fma(0.3, n1[4672], w1);
      w1 = fma(0.7, n1[5664], w1);
      w1 = fma(0.7, n1[3872], w1);
      w1 = w1 - n1[4736];
      double w2 = 0.3 * n2[5888];
      w2 = fma(0.3, n2[4672], w2);
      w2 = fma(0.7, n2[5664], w2);
      w2 = fma(0.7, n2[3872], w2);
      w2 = w2 - n2[4736];
      double w3 = 0.3 * n3[5888];
      w3 = fma(0.3, n3[4672], w3);
      w3 = fma(0.7, n3[5664], w3);
      w3 = fma(0.7, n3[3872], w3);
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[4736];
      wk0 = fma(w2, k2[4736], wk0);
      wk0 = fma(w3, k3[4736], wk0);
      const double kk = ws[43040];
      ws[271744] = fma(-kk, wk0, ws[271744]);
    }
    {
      double w1 = 2.0 * n1[5664];
      w1 = w1 - n1[5376];
      double w2 = 2.0 * n2[5664];
      w2 = w2 - n2[5376];
      double w3 = 2.0 * n3[5664];
      w3 = w3 - n3[5376];
      double wk0 = w1 * k1[5376];
      wk0 = fma(w2, k2[5376], wk0);
      wk0 = fma(w3, k3[5376], wk0);
      const double kk = ws[43072];
      ws[271776] = fma(-kk, wk0, ws[271776]);
    }
    {
      double w1 = 1.0 * n1[5856];
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[5376];
      double w2 = 1.0 * n2[5856];
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[5376];
      double w3 = 1.0 * n3[5856];
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[5376];
      double wk0 = w1 * k1[5376];
      wk0 = fma(w2, k2[5376], wk0);
      wk0 = fma(w3, k3[5376], wk0);
      const double kk = ws[43104];
      ws[271808] = fma(-kk, wk0, ws[271808]);
    }
    {
      double w1 = 2.0 * n1[5984];
      w1 = fma(2.0, n1[5664], w1);
      w1 = w1 - n1[5376];
      double w2 = 2.0 * n2[5984];
      w2 = fma(2.0, n2[5664], w2);
      w2 = w2 - n2[5376];
      double w3 = 2.0 * n3[5984];
      w3 = fma(2.0, n3[5664], w3);
      w3 = w3 - n3[5376];
      double wk0 = w1 * k1[5376];
      wk0 = fma(w2, k2[5376], wk0);
      wk0 = fma(w3, k3[5376], wk0);
      const double kk = ws[43136];
      ws[271840] = fma(-kk, wk0, ws[271840]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5792], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[5248];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5792], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[5248];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5792], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[5248];
      double wk0 = w1 * k1[5248];
      wk0 = fma(w2, k2[5248], wk0);
      wk0 = fma(w3, k3[5248], wk0);
      const double kk = ws[43168];
      ws[271872] = fma(-kk, wk0, ws[271872]);
    }
}
__device__ __noinline__ void adj_hess3_0_1(double* __restrict__ ws)
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
      double w1 = 1.5 * n1[5984];
      w1 = fma(0.25, n1[5792], w1);
      w1 = fma(0.2, n1[5216], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = fma(0.5, n1[5376], w1);
      w1 = fma(0.5, n1[5248], w1);
      w1 = w1 - n1[5472];
      double w2 = 1.5 * n2[5984];
      w2 = fma(0.25, n2[5792], w2);
      w2 = fma(0.2, n2[5216], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = fma(0.5, n2[5376], w2);
      w2 = fma(0.5, n2[5248], w2);
      w2 = w2 - n2[5472];
      double w3 = 1.5 * n3[5984];
      w3 = fma(0.25, n3[5792], w3);
      w3 = fma(0.2, n3[5216], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = fma(0.5, n3[5376], w3);
      w3 = fma(0.5, n3[5248], w3);
      w3 = w3 - n3[5472];
      double wk0 = w1 * k1[5472];
      wk0 = fma(w2, k2[5472], wk0);
      wk0 = fma(w3, k3[5472], wk0);
      const double kk = ws[43200];
      ws[271904] = fma(-kk, wk0, ws[271904]);
    }
    {
      double w1 = 1.5 * n1[5984];
      w1 = fma(0.25, n1[5792], w1);
      w1 = fma(0.2, n1[5216], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = fma(0.5, n1[5376], w1);
      w1 = fma(0.5, n1[5248], w1);
      w1 = w1 - n1[4320];
      double w2 = 1.5 * n2[5984];
      w2 = fma(0.25, n2[5792], w2);
      w2 = fma(0.2, n2[5216], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = fma(0.5, n2[5376], w2);
      w2 = fma(0.5, n2[5248], w2);
      w2 = w2 - n2[4320];
      double w3 = 1.5 * n3[5984];
      w3 = fma(0.25, n3[5792], w3);
      w3 = fma(0.2, n3[5216], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = fma(0.5, n3[5376], w3);
      w3 = fma(0.5, n3[5248], w3);
      w3 = w3 - n3[4320];
      double wk0 = w1 * k1[4320];
      wk0 = fma(w2, k2[4320], wk0);
      wk0 = fma(w3, k3[4320], wk0);
      const double kk = ws[43232];
      ws[271936] = fma(-kk, wk0, ws[271936]);
    }
    {
      double w1 = 1.0 * n1[3232];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5664], w1);
      w1 = w1 - n1[4448];
      double w2 = 1.0 * n2[3232];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5664], w2);
      w2 = w2 - n2[4448];
      double w3 = 1.0 * n3[3232];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5664], w3);
      w3 = w3 - n3[4448];
      double wk0 = w1 * k1[4448];
      wk0 = fma(w2, k2[4448], wk0);
      wk0 = fma(w3, k3[4448], wk0);
      const double kk = ws[43264];
      ws[271968] = fma(-kk, wk0, ws[271968]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5856], w1);
      w1 = w1 - n1[2816];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5856], w2);
      w2 = w2 - n2[2816];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5856], w3);
      w3 = w3 - n3[2816];
      double wk0 = w1 * k1[2816];
      wk0 = fma(w2, k2[2816], wk0);
      wk0 = fma(w3, k3[2816], wk0);
      const double kk = ws[43296];
      ws[272000] = fma(-kk, wk0, ws[272000]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5760], w1);
      w1 = w1 - n1[5728];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5760], w2);
      w2 = w2 - n2[5728];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5760], w3);
      w3 = w3 - n3[5728];
      double wk0 = w1 * k1[5728];
      wk0 = fma(w2, k2[5728], wk0);
      wk0 = fma(w3, k3[5728], wk0);
      const double kk = ws[43328];
      ws[272032] = fma(-kk, wk0, ws[272032]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5760], w1);
      w1 = w1 - n1[4096];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5760], w2);
      w2 = w2 - n2[4096];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5760], w3);
      w3 = w3 - n3[4096];
      double wk0 = w1 * k1[4096];
      wk0 = fma(w2, k2[4096], wk0);
      wk0 = fma(w3, k3[4096], wk0);
      const double kk = ws[43360];
      ws[272064] = fma(-kk, wk0, ws[272064]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5984], w1);
      w1 = fma(1.0, n1[5760], w1);
      w1 = w1 - n1[4608];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5984], w2);
      w2 = fma(1.0, n2[5760], w2);
      w2 = w2 - n2[4608];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5984], w3);
      w3 = fma(1.0, n3[5760], w3);
      w3 = w3 - n3[4608];
      double wk0 = w1 * k1[4608];
      wk0 = fma(w2, k2[4608], wk0);
      wk0 = fma(w3, k3[4608], wk0);
      const double kk = ws[43392];
      ws[272096] = fma(-kk, wk0, ws[272096]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = fma(1.0, n1[5888], w1);
      w1 = w1 - n1[3680];
      double w2 = 1.0 * n2[6016];
      w2 = fma(1.0, n2[5888], w2);
      w2 = w2 - n2[3680];
      double w3 = 1.0 * n3[6016];
      w3 = fma(1.0, n3[5888], w3);
      w3 = w3 - n3[3680];
      double wk0 = w1 * k1[3680];
      wk0 = fma(w2, k2[3680], wk0);
      wk0 = fma(w3, k3[3680], wk0);
      const double kk = ws[43424];
      ws[272128] = fma(-kk, wk0, ws[272128]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5920], w1);
      w1 = fma(0.2, n1[5760], w1);
      w1 = fma(0.8, n1[5504], w1);
      w1 = w1 - n1[5440];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5920], w2);
      w2 = fma(0.2, n2[5760], w2);
      w2 = fma(0.8, n2[5504], w2);
      w2 = w2 - n2[5440];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5920], w3);
      w3 = fma(0.2, n3[5760], w3);
      w3 = fma(0.8, n3[5504], w3);
      w3 = w3 - n3[5440];
      double wk0 = w1 * k1[5440];
      wk0 = fma(w2, k2[5440], wk0);
      wk0 = fma(w3, k3[5440], wk0);
      const double kk = ws[43456];
      ws[272160] = fma(-kk, wk0, ws[272160]);
    }
    {
      double w1 = 1.0 * n1[5792];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[1088];
      double w2 = 1.0 * n2[5792];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[1088];
      double w3 = 1.0 * n3[5792];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[1088];
      double wk0 = w1 * k1[1088];
      wk0 = fma(w2, k2[1088], wk0);
      wk0 = fma(w3, k3[1088], wk0);
      const double kk = ws[43488];
      ws[272192] = fma(-kk, wk0, ws[272192]);
    }
    {
      double w1 = 1.0 * n1[5888];
      w1 = fma(1.0, n1[5952], w1);
      w1 = w1 - n1[1088];
      double w2 = 1.0 * n2[5888];
      w2 = fma(1.0, n2[5952], w2);
      w2 = w2 - n2[1088];
      double w3 = 1.0 * n3[5888];
      w3 = fma(1.0, n3[5952], w3);
      w3 = w3 - n3[1088];
      double wk0 = w1 * k1[1088];
      wk0 = fma(w2, k2[1088], wk0);
      wk0 = fma(w3, k3[1088], wk0);
      const double kk = ws[43520];
      ws[272224] = fma(-kk, wk0, ws[272224]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = fma(0.67, n1[5504], w1);
      w1 = fma(0.33, n1[3872], w1);
      w1 = w1 - n1[4384];
      double w2 = 1.0 * n2[5920];
      w2 = fma(0.67, n2[5504], w2);
      w2 = fma(0.33, n2[3872], w2);
      w2 = w2 - n2[4384];
      double w3 = 1.0 * n3[5920];
      w3 = fma(0.67, n3[5504], w3);
      w3 = fma(0.33, n3[3872], w3);
      w3 = w3 - n3[4384];
      double wk0 = w1 * k1[4384];
      wk0 = fma(w2, k2[4384], wk0);
      wk0 = fma(w3, k3[4384], wk0);
      const double kk = ws[43552];
      ws[272256] = fma(-kk, wk0, ws[272256]);
    }
    {
      double w1 = 1.0 * n1[5344];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[1696];
      double w2 = 1.0 * n2[5344];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[1696];
      double w3 = 1.0 * n3[5344];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[1696];
      double wk0 = w1 * k1[1696];
      wk0 = fma(w2, k2[1696], wk0);
      wk0 = fma(w3, k3[1696], wk0);
      const double kk = ws[43584];
      ws[272288] = fma(-kk, wk0, ws[272288]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = w1 - n1[5184];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5984];
      w2 = w2 - n2[5184];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5984];
      w3 = w3 - n3[5184];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[5184];
      wk0 = fma(w2, k2[5184], wk0);
      wk0 = fma(w3, k3[5184], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[43616];
      ws[272320] = fma(-kk, fma(y[6016], wk0, y[5184] * wk1), ws[272320]);
      lam[5184] = fma(-kk, wk1, lam[5184]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[6016];
      w1 = w1 - n1[5184];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[6016];
      w2 = w2 - n2[5184];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[6016];
      w3 = w3 - n3[5184];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5184];
      wk0 = fma(w2, k2[5184], wk0);
      wk0 = fma(w3, k3[5184], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[43648];
      ws[272352] = fma(-kk, fma(y[5984], wk0, y[5184] * wk1), ws[272352]);
      lam[5184] = fma(-kk, wk1, lam[5184]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = w1 - n1[5184];
      w1 = w1 - n1[5824];
      double w2 = 1.0 * n2[5920];
      w2 = w2 - n2[5184];
      w2 = w2 - n2[5824];
      double w3 = 1.0 * n3[5920];
      w3 = w3 - n3[5184];
      w3 = w3 - n3[5824];
      double wk0 = w1 * k1[5184];
      wk0 = fma(w2, k2[5184], wk0);
      wk0 = fma(w3, k3[5184], wk0);
      double wk1 = w1 * k1[5824];
      wk1 = fma(w2, k2[5824], wk1);
      wk1 = fma(w3, k3[5824], wk1);
      const double kk = ws[43680];
      ws[272384] = fma(-kk, fma(y[5824], wk0, y[5184] * wk1), ws[272384]);
      lam[5184] = fma(-kk, wk1, lam[5184]);
      lam[5824] = fma(-kk, wk0, lam[5824]);
    }
    {
      double w1 = 1.0 * n1[5952];
      w1 = w1 - n1[5184];
      w1 = w1 - n1[5920];
      double w2 = 1.0 * n2[5952];
      w2 = w2 - n2[5184];
      w2 = w2 - n2[5920];
      double w3 = 1.0 * n3[5952];
      w3 = w3 - n3[5184];
      w3 = w3 - n3[5920];
      double wk0 = w1 * k1[5184];
      wk0 = fma(w2, k2[5184], wk0);
      wk0 = fma(w3, k3[5184], wk0);
      double wk1 = w1 * k1[5920];
      wk1 = fma(w2, k2[5920], wk1);
      wk1 = fma(w3, k3[5920], wk1);
      const double kk = ws[43712];
      ws[272416] = fma(-kk, fma(y[5920], wk0, y[5184] * wk1), ws[272416]);
      lam[5184] = fma(-kk, wk1, lam[5184]);
      lam[5920] = fma(-kk, wk0, lam[5920]);
    }
    {
      double w1 = 1.0 * n1[5184];
      w1 = w1 - n1[2336];
      double w2 = 1.0 * n2[5184];
      w2 = w2 - n2[2336];
      double w3 = 1.0 * n3[5184];
      w3 = w3 - n3[2336];
      double wk0 = w1 * k1[2336];
      wk0 = fma(w2, k2[2336], wk0);
      wk0 = fma(w3, k3[2336], wk0);
      const double kk = ws[43744];
      ws[272448] = fma(-kk, wk0, ws[272448]);
    }
    {
      double w1 = -n1[2336];
      w1 = w1 - n1[5184];
      double w2 = -n2[2336];
      w2 = w2 - n2[5184];
      double w3 = -n3[2336];
      w3 = w3 - n3[5184];
      double wk0 = w1 * k1[2336];
      wk0 = fma(w2, k2[2336], wk0);
      wk0 = fma(w3, k3[2336], wk0);
      double wk1 = w1 * k1[5184];
      wk1 = fma(w2, k2[5184], wk1);
      wk1 = fma(w3, k3[5184], wk1);
      const double kk = ws[43776];
      ws[272480] = fma(-kk, fma(y[5184], wk0, y[2336] * wk1), ws[272480]);
      lam[2336] = fma(-kk, wk1, lam[2336]);
      lam[5184] = fma(-kk, wk0, lam[5184]);
    }
    {
      double w1 = 1.0 * n1[2336];
      w1 = w1 - n1[576];
      double w2 = 1.0 * n2[2336];
      w2 = w2 - n2[576];
      double w3 = 1.0 * n3[2336];
      w3 = w3 - n3[576];
      double wk0 = w1 * k1[576];
      wk0 = fma(w2, k2[576], wk0);
      wk0 = fma(w3, k3[576], wk0);
      const double kk = ws[43808];
      ws[272512] = fma(-kk, wk0, ws[272512]);
    }
    {
      double w1 = 1.0 * n1[2336];
      w1 = w1 - n1[576];
      double w2 = 1.0 * n2[2336];
      w2 = w2 - n2[576];
      double w3 = 1.0 * n3[2336];
      w3 = w3 - n3[576];
      double wk0 = w1 * k1[576];
      wk0 = fma(w2, k2[576], wk0);
      wk0 = fma(w3, k3[576], wk0);
      const double kk = ws[43840];
      ws[272544] = fma(-kk, wk0, ws[272544]);
    }
    {
      double w1 = 2.0 * n1[6016];
      w1 = w1 - n1[576];
      double w2 = 2.0 * n2[6016];
      w2 = w2 - n2[576];
      double w3 = 2.0 * n3[6016];
      w3 = w3 - n3[576];
      double wk0 = w1 * k1[576];
      wk0 = fma(w2, k2[576], wk0);
      wk0 = fma(w3, k3[576], wk0);
      const double kk = ws[43872];
      ws[272576] = fma(-kk, wk0, ws[272576]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5984];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5984];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[6016];
      wk0 = fma(w2, k2[6016], wk0);
      wk0 = fma(w3, k3[6016], wk0);
      const double kk = ws[43904];
      ws[272608] = fma(-kk, wk0, ws[272608]);
    }
    {
      double w1 = -n1[6016];
      w1 = w1 - n1[5984];
      double w2 = -n2[6016];
      w2 = w2 - n2[5984];
      double w3 = -n3[6016];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[6016];
      wk0 = fma(w2, k2[6016], wk0);
      wk0 = fma(w3, k3[6016], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[43936];
      ws[272640] = fma(-kk, fma(y[5984], wk0, y[6016] * wk1), ws[272640]);
      lam[6016] = fma(-kk, wk1, lam[6016]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 1.0 * n1[4000];
      w1 = w1 - n1[5984];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[4000];
      w2 = w2 - n2[5984];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[4000];
      w3 = w3 - n3[5984];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5984];
      wk0 = fma(w2, k2[5984], wk0);
      wk0 = fma(w3, k3[5984], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[43968];
      ws[272672] = fma(-kk, fma(y[5984], wk0, y[5984] * wk1), ws[272672]);
      lam[5984] = fma(-kk, wk1, lam[5984]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 1.0 * n1[4000];
      w1 = w1 - n1[5984];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[4000];
      w2 = w2 - n2[5984];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[4000];
      w3 = w3 - n3[5984];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5984];
      wk0 = fma(w2, k2[5984], wk0);
      wk0 = fma(w3, k3[5984], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[44000];
      ws[272704] = fma(-kk, fma(y[5984], wk0, y[5984] * wk1), ws[272704]);
      lam[5984] = fma(-kk, wk1, lam[5984]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
}
__device__ __noinline__ void adj_hess3_0_2(double* __restrict__ ws)
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
      double w1 = 1.0 * n1[5984];
      w1 = w1 - n1[4000];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5984];
      w2 = w2 - n2[4000];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5984];
      w3 = w3 - n3[4000];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[4000];
      wk0 = fma(w2, k2[4000], wk0);
      wk0 = fma(w3, k3[4000], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44032];
      ws[272736] = fma(-kk, fma(y[6016], wk0, y[4000] * wk1), ws[272736]);
      lam[4000] = fma(-kk, wk1, lam[4000]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = w1 - n1[5824];
      w1 = w1 - n1[2336];
      double w2 = 1.0 * n2[5920];
      w2 = w2 - n2[5824];
      w2 = w2 - n2[2336];
      double w3 = 1.0 * n3[5920];
      w3 = w3 - n3[5824];
      w3 = w3 - n3[2336];
      double wk0 = w1 * k1[5824];
      wk0 = fma(w2, k2[5824], wk0);
      wk0 = fma(w3, k3[5824], wk0);
      double wk1 = w1 * k1[2336];
      wk1 = fma(w2, k2[2336], wk1);
      wk1 = fma(w3, k3[2336], wk1);
      const double kk = ws[44064];
      ws[272768] = fma(-kk, fma(y[2336], wk0, y[5824] * wk1), ws[272768]);
      lam[5824] = fma(-kk, wk1, lam[5824]);
      lam[2336] = fma(-kk, wk0, lam[2336]);
    }
    {
      double w1 = 1.0 * n1[1184];
      w1 = w1 - n1[5824];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[1184];
      w2 = w2 - n2[5824];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[1184];
      w3 = w3 - n3[5824];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[5824];
      wk0 = fma(w2, k2[5824], wk0);
      wk0 = fma(w3, k3[5824], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44096];
      ws[272800] = fma(-kk, fma(y[6016], wk0, y[5824] * wk1), ws[272800]);
      lam[5824] = fma(-kk, wk1, lam[5824]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = fma(1.0, n1[6016], w1);
      w1 = w1 - n1[5824];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[5920];
      w2 = fma(1.0, n2[6016], w2);
      w2 = w2 - n2[5824];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[5920];
      w3 = fma(1.0, n3[6016], w3);
      w3 = w3 - n3[5824];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5824];
      wk0 = fma(w2, k2[5824], wk0);
      wk0 = fma(w3, k3[5824], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[44128];
      ws[272832] = fma(-kk, fma(y[5984], wk0, y[5824] * wk1), ws[272832]);
      lam[5824] = fma(-kk, wk1, lam[5824]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 1.0 * n1[5024];
      w1 = w1 - n1[5824];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[5024];
      w2 = w2 - n2[5824];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[5024];
      w3 = w3 - n3[5824];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5824];
      wk0 = fma(w2, k2[5824], wk0);
      wk0 = fma(w3, k3[5824], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[44160];
      ws[272864] = fma(-kk, fma(y[5984], wk0, y[5824] * wk1), ws[272864]);
      lam[5824] = fma(-kk, wk1, lam[5824]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 2.0 * n1[5920];
      w1 = w1 - n1[5824];
      w1 = w1 - n1[5824];
      double w2 = 2.0 * n2[5920];
      w2 = w2 - n2[5824];
      w2 = w2 - n2[5824];
      double w3 = 2.0 * n3[5920];
      w3 = w3 - n3[5824];
      w3 = w3 - n3[5824];
      double wk0 = w1 * k1[5824];
      wk0 = fma(w2, k2[5824], wk0);
      wk0 = fma(w3, k3[5824], wk0);
      double wk1 = w1 * k1[5824];
      wk1 = fma(w2, k2[5824], wk1);
      wk1 = fma(w3, k3[5824], wk1);
      const double kk = ws[44192];
      ws[272896] = fma(-kk, fma(y[5824], wk0, y[5824] * wk1), ws[272896]);
      lam[5824] = fma(-kk, wk1, lam[5824]);
      lam[5824] = fma(-kk, wk0, lam[5824]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = w1 - n1[1184];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5920];
      w2 = w2 - n2[1184];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5920];
      w3 = w3 - n3[1184];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1184];
      wk0 = fma(w2, k2[1184], wk0);
      wk0 = fma(w3, k3[1184], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44224];
      ws[272928] = fma(-kk, fma(y[6016], wk0, y[1184] * wk1), ws[272928]);
      lam[1184] = fma(-kk, wk1, lam[1184]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5824];
      w1 = w1 - n1[5920];
      w1 = w1 - n1[2336];
      double w2 = 1.0 * n2[5824];
      w2 = w2 - n2[5920];
      w2 = w2 - n2[2336];
      double w3 = 1.0 * n3[5824];
      w3 = w3 - n3[5920];
      w3 = w3 - n3[2336];
      double wk0 = w1 * k1[5920];
      wk0 = fma(w2, k2[5920], wk0);
      wk0 = fma(w3, k3[5920], wk0);
      double wk1 = w1 * k1[2336];
      wk1 = fma(w2, k2[2336], wk1);
      wk1 = fma(w3, k3[2336], wk1);
      const double kk = ws[44256];
      ws[272960] = fma(-kk, fma(y[2336], wk0, y[5920] * wk1), ws[272960]);
      lam[5920] = fma(-kk, wk1, lam[5920]);
      lam[2336] = fma(-kk, wk0, lam[2336]);
    }
    {
      double w1 = 1.0 * n1[5952];
      w1 = w1 - n1[5920];
      w1 = w1 - n1[2336];
      double w2 = 1.0 * n2[5952];
      w2 = w2 - n2[5920];
      w2 = w2 - n2[2336];
      double w3 = 1.0 * n3[5952];
      w3 = w3 - n3[5920];
      w3 = w3 - n3[2336];
      double wk0 = w1 * k1[5920];
      wk0 = fma(w2, k2[5920], wk0);
      wk0 = fma(w3, k3[5920], wk0);
      double wk1 = w1 * k1[2336];
      wk1 = fma(w2, k2[2336], wk1);
      wk1 = fma(w3, k3[2336], wk1);
      const double kk = ws[44288];
      ws[272992] = fma(-kk, fma(y[2336], wk0, y[5920] * wk1), ws[272992]);
      lam[5920] = fma(-kk, wk1, lam[5920]);
      lam[2336] = fma(-kk, wk0, lam[2336]);
    }
    {
      double w1 = 1.0 * n1[5024];
      w1 = w1 - n1[5920];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5024];
      w2 = w2 - n2[5920];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5024];
      w3 = w3 - n3[5920];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[5920];
      wk0 = fma(w2, k2[5920], wk0);
      wk0 = fma(w3, k3[5920], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44320];
      ws[273024] = fma(-kk, fma(y[6016], wk0, y[5920] * wk1), ws[273024]);
      lam[5920] = fma(-kk, wk1, lam[5920]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5952];
      w1 = w1 - n1[5024];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5952];
      w2 = w2 - n2[5024];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5952];
      w3 = w3 - n3[5024];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[5024];
      wk0 = fma(w2, k2[5024], wk0);
      wk0 = fma(w3, k3[5024], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44352];
      ws[273056] = fma(-kk, fma(y[6016], wk0, y[5024] * wk1), ws[273056]);
      lam[5024] = fma(-kk, wk1, lam[5024]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[5952];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[5952];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[5952];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44384];
      ws[273088] = fma(-kk, fma(y[6016], wk0, y[5952] * wk1), ws[273088]);
      lam[5952] = fma(-kk, wk1, lam[5952]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.7 * n1[6016];
      w1 = fma(0.7, n1[5920], w1);
      w1 = fma(0.3, n1[5024], w1);
      w1 = w1 - n1[5952];
      w1 = w1 - n1[5984];
      double w2 = 0.7 * n2[6016];
      w2 = fma(0.7, n2[5920], w2);
      w2 = fma(0.3, n2[5024], w2);
      w2 = w2 - n2[5952];
      w2 = w2 - n2[5984];
      double w3 = 0.7 * n3[6016];
      w3 = fma(0.7, n3[5920], w3);
      w3 = fma(0.3, n3[5024], w3);
      w3 = w3 - n3[5952];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[44416];
      ws[273120] = fma(-kk, fma(y[5984], wk0, y[5952] * wk1), ws[273120]);
      lam[5952] = fma(-kk, wk1, lam[5952]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 2.0 * n1[5920];
      w1 = w1 - n1[5952];
      w1 = w1 - n1[5824];
      double w2 = 2.0 * n2[5920];
      w2 = w2 - n2[5952];
      w2 = w2 - n2[5824];
      double w3 = 2.0 * n3[5920];
      w3 = w3 - n3[5952];
      w3 = w3 - n3[5824];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      double wk1 = w1 * k1[5824];
      wk1 = fma(w2, k2[5824], wk1);
      wk1 = fma(w3, k3[5824], wk1);
      const double kk = ws[44448];
      ws[273152] = fma(-kk, fma(y[5824], wk0, y[5952] * wk1), ws[273152]);
      lam[5952] = fma(-kk, wk1, lam[5952]);
      lam[5824] = fma(-kk, wk0, lam[5824]);
    }
    {
      double w1 = 1.0 * n1[5824];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[5952];
      w1 = w1 - n1[5920];
      double w2 = 1.0 * n2[5824];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[5952];
      w2 = w2 - n2[5920];
      double w3 = 1.0 * n3[5824];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[5952];
      w3 = w3 - n3[5920];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      double wk1 = w1 * k1[5920];
      wk1 = fma(w2, k2[5920], wk1);
      wk1 = fma(w3, k3[5920], wk1);
      const double kk = ws[44480];
      ws[273184] = fma(-kk, fma(y[5920], wk0, y[5952] * wk1), ws[273184]);
      lam[5952] = fma(-kk, wk1, lam[5952]);
      lam[5920] = fma(-kk, wk0, lam[5920]);
    }
    {
      double w1 = 2.0 * n1[5920];
      w1 = w1 - n1[5952];
      w1 = w1 - n1[5952];
      double w2 = 2.0 * n2[5920];
      w2 = w2 - n2[5952];
      w2 = w2 - n2[5952];
      double w3 = 2.0 * n3[5920];
      w3 = w3 - n3[5952];
      w3 = w3 - n3[5952];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      double wk1 = w1 * k1[5952];
      wk1 = fma(w2, k2[5952], wk1);
      wk1 = fma(w3, k3[5952], wk1);
      const double kk = ws[44512];
      ws[273216] = fma(-kk, fma(y[5952], wk0, y[5952] * wk1), ws[273216]);
      lam[5952] = fma(-kk, wk1, lam[5952]);
      lam[5952] = fma(-kk, wk0, lam[5952]);
    }
    {
      double w1 = 1.0 * n1[1024];
      w1 = w1 - n1[5952];
      w1 = w1 - n1[5920];
      double w2 = 1.0 * n2[1024];
      w2 = w2 - n2[5952];
      w2 = w2 - n2[5920];
      double w3 = 1.0 * n3[1024];
      w3 = w3 - n3[5952];
      w3 = w3 - n3[5920];
      double wk0 = w1 * k1[5952];
      wk0 = fma(w2, k2[5952], wk0);
      wk0 = fma(w3, k3[5952], wk0);
      double wk1 = w1 * k1[5920];
      wk1 = fma(w2, k2[5920], wk1);
      wk1 = fma(w3, k3[5920], wk1);
      const double kk = ws[44544];
      ws[273248] = fma(-kk, fma(y[5920], wk0, y[5952] * wk1), ws[273248]);
      lam[5952] = fma(-kk, wk1, lam[5952]);
      lam[5920] = fma(-kk, wk0, lam[5920]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = fma(1.0, n1[5952], w1);
      w1 = w1 - n1[1024];
      double w2 = 1.0 * n2[5920];
      w2 = fma(1.0, n2[5952], w2);
      w2 = w2 - n2[1024];
      double w3 = 1.0 * n3[5920];
      w3 = fma(1.0, n3[5952], w3);
      w3 = w3 - n3[1024];
      double wk0 = w1 * k1[1024];
      wk0 = fma(w2, k2[1024], wk0);
      wk0 = fma(w3, k3[1024], wk0);
      const double kk = ws[44576];
      ws[273280] = fma(-kk, wk0, ws[273280]);
    }
    {
      double w1 = 2.0 * n1[5024];
      w1 = w1 - n1[1024];
      double w2 = 2.0 * n2[5024];
      w2 = w2 - n2[1024];
      double w3 = 2.0 * n3[5024];
      w3 = w3 - n3[1024];
      double wk0 = w1 * k1[1024];
      wk0 = fma(w2, k2[1024], wk0);
      wk0 = fma(w3, k3[1024], wk0);
      const double kk = ws[44608];
      ws[273312] = fma(-kk, wk0, ws[273312]);
    }
    {
      double w1 = 1.0 * n1[1280];
      w1 = w1 - n1[5920];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[1280];
      w2 = w2 - n2[5920];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[1280];
      w3 = w3 - n3[5920];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[5920];
      wk0 = fma(w2, k2[5920], wk0);
      wk0 = fma(w3, k3[5920], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[44640];
      ws[273344] = fma(-kk, fma(y[5984], wk0, y[5920] * wk1), ws[273344]);
      lam[5920] = fma(-kk, wk1, lam[5920]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[5920], w1);
      w1 = w1 - n1[1280];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[5920], w2);
      w2 = w2 - n2[1280];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[5920], w3);
      w3 = w3 - n3[1280];
      double wk0 = w1 * k1[1280];
      wk0 = fma(w2, k2[1280], wk0);
      wk0 = fma(w3, k3[1280], wk0);
      const double kk = ws[44672];
      ws[273376] = fma(-kk, wk0, ws[273376]);
    }
    {
      double w1 = 1.0 * n1[5920];
      w1 = w1 - n1[1280];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5920];
      w2 = w2 - n2[1280];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5920];
      w3 = w3 - n3[1280];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1280];
      wk0 = fma(w2, k2[1280], wk0);
      wk0 = fma(w3, k3[1280], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44704];
      ws[273408] = fma(-kk, fma(y[6016], wk0, y[1280] * wk1), ws[273408]);
      lam[1280] = fma(-kk, wk1, lam[1280]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5984];
      w1 = fma(1.0, n1[192], w1);
      w1 = fma(1.0, n1[224], w1);
      w1 = w1 - n1[160];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5984];
      w2 = fma(1.0, n2[192], w2);
      w2 = fma(1.0, n2[224], w2);
      w2 = w2 - n2[160];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5984];
      w3 = fma(1.0, n3[192], w3);
      w3 = fma(1.0, n3[224], w3);
      w3 = w3 - n3[160];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[160];
      wk0 = fma(w2, k2[160], wk0);
      wk0 = fma(w3, k3[160], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44736];
      ws[273440] = fma(-kk, fma(y[6016], wk0, y[160] * wk1), ws[273440]);
      lam[160] = fma(-kk, wk1, lam[160]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
}
__device__ __noinline__ void adj_hess3_0_3(double* __restrict__ ws)
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
      double w1 = 1.0 * n1[5984];
      w1 = w1 - n1[5664];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5984];
      w2 = w2 - n2[5664];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5984];
      w3 = w3 - n3[5664];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[5664];
      wk0 = fma(w2, k2[5664], wk0);
      wk0 = fma(w3, k3[5664], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44768];
      ws[273472] = fma(-kk, fma(y[6016], wk0, y[5664] * wk1), ws[273472]);
      lam[5664] = fma(-kk, wk1, lam[5664]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5888];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5888];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5888];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[6016];
      wk0 = fma(w2, k2[6016], wk0);
      wk0 = fma(w3, k3[6016], wk0);
      const double kk = ws[44800];
      ws[273504] = fma(-kk, wk0, ws[273504]);
    }
    {
      double w1 = 1.0 * n1[5632];
      w1 = w1 - n1[1888];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5632];
      w2 = w2 - n2[1888];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5632];
      w3 = w3 - n3[1888];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1888];
      wk0 = fma(w2, k2[1888], wk0);
      wk0 = fma(w3, k3[1888], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44832];
      ws[273536] = fma(-kk, fma(y[6016], wk0, y[1888] * wk1), ws[273536]);
      lam[1888] = fma(-kk, wk1, lam[1888]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5408];
      w1 = fma(2.81e-05, n1[3616], w1);
      w1 = w1 - n1[2176];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5408];
      w2 = fma(2.81e-05, n2[3616], w2);
      w2 = w2 - n2[2176];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5408];
      w3 = fma(2.81e-05, n3[3616], w3);
      w3 = w3 - n3[2176];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[2176];
      wk0 = fma(w2, k2[2176], wk0);
      wk0 = fma(w3, k3[2176], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44864];
      ws[273568] = fma(-kk, fma(y[6016], wk0, y[2176] * wk1), ws[273568]);
      lam[2176] = fma(-kk, wk1, lam[2176]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[5120];
      w1 = fma(0.00134, n1[3616], w1);
      w1 = w1 - n1[1120];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[5120];
      w2 = fma(0.00134, n2[3616], w2);
      w2 = w2 - n2[1120];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[5120];
      w3 = fma(0.00134, n3[3616], w3);
      w3 = w3 - n3[1120];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1120];
      wk0 = fma(w2, k2[1120], wk0);
      wk0 = fma(w3, k3[1120], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44896];
      ws[273600] = fma(-kk, fma(y[6016], wk0, y[1120] * wk1), ws[273600]);
      lam[1120] = fma(-kk, wk1, lam[1120]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[3008];
      w1 = w1 - n1[2240];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[3008];
      w2 = w2 - n2[2240];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[3008];
      w3 = w3 - n3[2240];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[2240];
      wk0 = fma(w2, k2[2240], wk0);
      wk0 = fma(w3, k3[2240], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44928];
      ws[273632] = fma(-kk, fma(y[6016], wk0, y[2240] * wk1), ws[273632]);
      lam[2240] = fma(-kk, wk1, lam[2240]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[3200];
      w1 = w1 - n1[2752];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[3200];
      w2 = w2 - n2[2752];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[3200];
      w3 = w3 - n3[2752];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[2752];
      wk0 = fma(w2, k2[2752], wk0);
      wk0 = fma(w3, k3[2752], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44960];
      ws[273664] = fma(-kk, fma(y[6016], wk0, y[2752] * wk1), ws[273664]);
      lam[2752] = fma(-kk, wk1, lam[2752]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[3328];
      w1 = w1 - n1[1152];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[3328];
      w2 = w2 - n2[1152];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[3328];
      w3 = w3 - n3[1152];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1152];
      wk0 = fma(w2, k2[1152], wk0);
      wk0 = fma(w3, k3[1152], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[44992];
      ws[273696] = fma(-kk, fma(y[6016], wk0, y[1152] * wk1), ws[273696]);
      lam[1152] = fma(-kk, wk1, lam[1152]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.65 * n1[6016];
      w1 = fma(0.35, n1[5984], w1);
      w1 = fma(0.35, n1[5664], w1);
      w1 = fma(0.65, n1[5376], w1);
      w1 = fma(0.35, n1[4352], w1);
      w1 = w1 - n1[256];
      w1 = w1 - n1[6016];
      double w2 = 0.65 * n2[6016];
      w2 = fma(0.35, n2[5984], w2);
      w2 = fma(0.35, n2[5664], w2);
      w2 = fma(0.65, n2[5376], w2);
      w2 = fma(0.35, n2[4352], w2);
      w2 = w2 - n2[256];
      w2 = w2 - n2[6016];
      double w3 = 0.65 * n3[6016];
      w3 = fma(0.35, n3[5984], w3);
      w3 = fma(0.35, n3[5664], w3);
      w3 = fma(0.65, n3[5376], w3);
      w3 = fma(0.35, n3[4352], w3);
      w3 = w3 - n3[256];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[256];
      wk0 = fma(w2, k2[256], wk0);
      wk0 = fma(w3, k3[256], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[45024];
      ws[273728] = fma(-kk, fma(y[6016], wk0, y[256] * wk1), ws[273728]);
      lam[256] = fma(-kk, wk1, lam[256]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.47 * n1[3360];
      w1 = fma(0.53, n1[1248], w1);
      w1 = fma(0.53, n1[5984], w1);
      w1 = w1 - n1[1216];
      w1 = w1 - n1[6016];
      double w2 = 0.47 * n2[3360];
      w2 = fma(0.53, n2[1248], w2);
      w2 = fma(0.53, n2[5984], w2);
      w2 = w2 - n2[1216];
      w2 = w2 - n2[6016];
      double w3 = 0.47 * n3[3360];
      w3 = fma(0.53, n3[1248], w3);
      w3 = fma(0.53, n3[5984], w3);
      w3 = w3 - n3[1216];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1216];
      wk0 = fma(w2, k2[1216], wk0);
      wk0 = fma(w3, k3[1216], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[45056];
      ws[273760] = fma(-kk, fma(y[6016], wk0, y[1216] * wk1), ws[273760]);
      lam[1216] = fma(-kk, wk1, lam[1216]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.82 * n1[3296];
      w1 = fma(0.18, n1[2944], w1);
      w1 = fma(0.18, n1[5984], w1);
      w1 = w1 - n1[288];
      w1 = w1 - n1[6016];
      double w2 = 0.82 * n2[3296];
      w2 = fma(0.18, n2[2944], w2);
      w2 = fma(0.18, n2[5984], w2);
      w2 = w2 - n2[288];
      w2 = w2 - n2[6016];
      double w3 = 0.82 * n3[3296];
      w3 = fma(0.18, n3[2944], w3);
      w3 = fma(0.18, n3[5984], w3);
      w3 = w3 - n3[288];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[288];
      wk0 = fma(w2, k2[288], wk0);
      wk0 = fma(w3, k3[288], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[45088];
      ws[273792] = fma(-kk, fma(y[6016], wk0, y[288] * wk1), ws[273792]);
      lam[288] = fma(-kk, wk1, lam[288]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.83 * n1[3104];
      w1 = fma(0.17, n1[2944], w1);
      w1 = fma(0.17, n1[5984], w1);
      w1 = w1 - n1[320];
      w1 = w1 - n1[6016];
      double w2 = 0.83 * n2[3104];
      w2 = fma(0.17, n2[2944], w2);
      w2 = fma(0.17, n2[5984], w2);
      w2 = w2 - n2[320];
      w2 = w2 - n2[6016];
      double w3 = 0.83 * n3[3104];
      w3 = fma(0.17, n3[2944], w3);
      w3 = fma(0.17, n3[5984], w3);
      w3 = w3 - n3[320];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[320];
      wk0 = fma(w2, k2[320], wk0);
      wk0 = fma(w3, k3[320], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[45120];
      ws[273824] = fma(-kk, fma(y[6016], wk0, y[320] * wk1), ws[273824]);
      lam[320] = fma(-kk, wk1, lam[320]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.82 * n1[3264];
      w1 = fma(0.18, n1[2944], w1);
      w1 = fma(0.18, n1[5984], w1);
      w1 = w1 - n1[352];
      w1 = w1 - n1[6016];
      double w2 = 0.82 * n2[3264];
      w2 = fma(0.18, n2[2944], w2);
      w2 = fma(0.18, n2[5984], w2);
      w2 = w2 - n2[352];
      w2 = w2 - n2[6016];
      double w3 = 0.82 * n3[3264];
      w3 = fma(0.18, n3[2944], w3);
      w3 = fma(0.18, n3[5984], w3);
      w3 = w3 - n3[352];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[352];
      wk0 = fma(w2, k2[352], wk0);
      wk0 = fma(w3, k3[352], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[45152];
      ws[273856] = fma(-kk, fma(y[6016], wk0, y[352] * wk1), ws[273856]);
      lam[352] = fma(-kk, wk1, lam[352]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 0.25 * n1[6016];
      w1 = fma(0.25, n1[5984], w1);
      w1 = fma(0.4, n1[5888], w1);
      w1 = fma(0.018, n1[5792], w1);
      w1 = fma(0.1, n1[4672], w1);
      w1 = fma(0.09, n1[4000], w1);
      w1 = fma(0.22, n1[5664], w1);
      w1 = fma(1.0, n1[5856], w1);
      w1 = fma(0.3, n1[4128], w1);
      w1 = fma(0.14, n1[4736], w1);
      w1 = fma(0.28, n1[4352], w1);
      w1 = fma(0.153, n1[2752], w1);
      w1 = w1 - n1[1312];
      w1 = w1 - n1[5184];
      double w2 = 0.25 * n2[6016];
      w2 = fma(0.25, n2[5984], w2);
      w2 = fma(0.4, n2[5888], w2);
      w2 = fma(0.018, n2[5792], w2);
      w2 = fma(0.1, n2[4672], w2);
      w2 = fma(0.09, n2[4000], w2);
      w2 = fma(0.22, n2[5664], w2);
      w2 = fma(1.0, n2[5856], w2);
      w2 = fma(0.3, n2[4128], w2);
      w2 = fma(0.14, n2[4736], w2);
      w2 = fma(0.28, n2[4352], w2);
      w2 = fma(0.153, n2[2752], w2);
      w2 = w2 - n2[1312];
      w2 = w2 - n2[5184];
      double w3 = 0.25 * n3[6016];
      w3 = fma(0.25, n3[5984], w3);
      w3 = fma(0.4, n3[5888], w3);
      w3 = fma(0.018, n3[5792], w3);
      w3 = fma(0.1, n3[4672], w3);
      w3 = fma(0.09, n3[4000], w3);
      w3 = fma(0.22, n3[5664], w3);
      w3 = fma(1.0, n3[5856], w3);
      w3 = fma(0.3, n3[4128], w3);
      w3 = fma(0.14, n3[4736], w3);
      w3 = fma(0.28, n3[4352], w3);
      w3 = fma(0.153, n3[2752], w3);
      w3 = w3 - n3[1312];
      w3 = w3 - n3[5184];
      double wk0 = w1 * k1[1312];
      wk0 = fma(w2, k2[1312], wk0);
      wk0 = fma(w3, k3[1312], wk0);
      double wk1 = w1 * k1[5184];
      wk1 = fma(w2, k2[5184], wk1);
      wk1 = fma(w3, k3[5184], wk1);
      const double kk = ws[45184];
      ws[273888] = fma(-kk, fma(y[5184], wk0, y[1312] * wk1), ws[273888]);
      lam[1312] = fma(-kk, wk1, lam[1312]);
      lam[5184] = fma(-kk, wk0, lam[5184]);
    }
    {
      double w1 = 0.4 * n1[5920];
      w1 = fma(0.045, n1[2784], w1);
      w1 = fma(0.35, n1[5856], w1);
      w1 = fma(0.555, n1[1632], w1);
      w1 = fma(0.26, n1[4736], w1);
      w1 = fma(0.028, n1[4128], w1);
      w1 = w1 - n1[1312];
      w1 = w1 - n1[5952];
      double w2 = 0.4 * n2[5920];
      w2 = fma(0.045, n2[2784], w2);
      w2 = fma(0.35, n2[5856], w2);
      w2 = fma(0.555, n2[1632], w2);
      w2 = fma(0.26, n2[4736], w2);
      w2 = fma(0.028, n2[4128], w2);
      w2 = w2 - n2[1312];
      w2 = w2 - n2[5952];
      double w3 = 0.4 * n3[5920];
      w3 = fma(0.045, n3[2784], w3);
      w3 = fma(0.35, n3[5856], w3);
      w3 = fma(0.555, n3[1632], w3);
      w3 = fma(0.26, n3[4736], w3);
      w3 = fma(0.028, n3[4128], w3);
      w3 = w3 - n3[1312];
      w3 = w3 - n3[5952];
      double wk0 = w1 * k1[1312];
      wk0 = fma(w2, k2[1312], wk0);
      wk0 = fma(w3, k3[1312], wk0);
      double wk1 = w1 * k1[5952];
      wk1 = fma(w2, k2[5952], wk1);
      wk1 = fma(w3, k3[5952], wk1);
      const double kk = ws[45216];
      ws[273920] = fma(-kk, fma(y[5952], wk0, y[1312] * wk1), ws[273920]);
      lam[1312] = fma(-kk, wk1, lam[1312]);
      lam[5952] = fma(-kk, wk0, lam[5952]);
    }
    {
      double w1 = 1.0 * n1[4288];
      w1 = fma(0.25, n1[5856], w1);
      w1 = fma(0.03, n1[4128], w1);
      w1 = fma(0.05, n1[5248], w1);
      w1 = w1 - n1[1312];
      w1 = w1 - n1[6016];
      double w2 = 1.0 * n2[4288];
      w2 = fma(0.25, n2[5856], w2);
      w2 = fma(0.03, n2[4128], w2);
      w2 = fma(0.05, n2[5248], w2);
      w2 = w2 - n2[1312];
      w2 = w2 - n2[6016];
      double w3 = 1.0 * n3[4288];
      w3 = fma(0.25, n3[5856], w3);
      w3 = fma(0.03, n3[4128], w3);
      w3 = fma(0.05, n3[5248], w3);
      w3 = w3 - n3[1312];
      w3 = w3 - n3[6016];
      double wk0 = w1 * k1[1312];
      wk0 = fma(w2, k2[1312], wk0);
      wk0 = fma(w3, k3[1312], wk0);
      double wk1 = w1 * k1[6016];
      wk1 = fma(w2, k2[6016], wk1);
      wk1 = fma(w3, k3[6016], wk1);
      const double kk = ws[45248];
      ws[273952] = fma(-kk, fma(y[6016], wk0, y[1312] * wk1), ws[273952]);
      lam[1312] = fma(-kk, wk1, lam[1312]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
    {
      double w1 = 1.0 * n1[1344];
      w1 = fma(0.07, n1[5984], w1);
      w1 = fma(0.5, n1[6016], w1);
      w1 = w1 - n1[4288];
      w1 = w1 - n1[5984];
      double w2 = 1.0 * n2[1344];
      w2 = fma(0.07, n2[5984], w2);
      w2 = fma(0.5, n2[6016], w2);
      w2 = w2 - n2[4288];
      w2 = w2 - n2[5984];
      double w3 = 1.0 * n3[1344];
      w3 = fma(0.07, n3[5984], w3);
      w3 = fma(0.5, n3[6016], w3);
      w3 = w3 - n3[4288];
      w3 = w3 - n3[5984];
      double wk0 = w1 * k1[4288];
      wk0 = fma(w2, k2[4288], wk0);
      wk0 = fma(w3, k3[4288], wk0);
      double wk1 = w1 * k1[5984];
      wk1 = fma(w2, k2[5984], wk1);
      wk1 = fma(w3, k3[5984], wk1);
      const double kk = ws[45280];
      ws[273984] = fma(-kk, fma(y[5984], wk0, y[4288] * wk1), ws[273984]);
      lam[4288] = fma(-kk, wk1, lam[4288]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
    {
      double w1 = 0.13 * n1[2784];
      w1 = fma(0.4, n1[5856], w1);
      w1 = fma(0.88, n1[5984], w1);
      w1 = fma(0.87, n1[5920], w1);
      w1 = fma(0.18, n1[4128], w1);
      w1 = fma(0.51, n1[4736], w1);
      w1 = w1 - n1[4288];
      w1 = w1 - n1[5824];
      double w2 = 0.13 * n2[2784];
      w2 = fma(0.4, n2[5856], w2);
      w2 = fma(0.88, n2[5984], w2);
      w2 = fma(0.87, n2[5920], w2);
      w2 = fma(0.18, n2[4128], w2);
      w2 = fma(0.51, n2[4736], w2);
      w2 = w2 - n2[4288];
      w2 = w2 - n2[5824];
      double w3 = 0.13 * n3[2784];
      w3 = fma(0.4, n3[5856], w3);
      w3 = fma(0.88, n3[5984], w3);
      w3 = fma(0.87, n3[5920], w3);
      w3 = fma(0.18, n3[4128], w3);
      w3 = fma(0.51, n3[4736], w3);
      w3 = w3 - n3[4288];
      w3 = w3 - n3[5824];
      double wk0 = w1 * k1[4288];
      wk0 = fma(w2, k2[4288], wk0);
      wk0 = fma(w3, k3[4288], wk0);
      double wk1 = w1 * k1[5824];
      wk1 = fma(w2, k2[5824], wk1);
      wk1 = fma(w3, k3[5824], wk1);
      const double kk = ws[45312];
      ws[274016] = fma(-kk, fma(y[5824], wk0, y[4288] * wk1), ws[274016]);
      lam[4288] = fma(-kk, wk1, lam[4288]);
      lam[5824] = fma(-kk, wk0, lam[5824]);
    }
}
}  // namespace mech_cracmm2
