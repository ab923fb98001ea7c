// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_hess3_0_0(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    double* __restrict__ lam = ws + 216608;
    const double* __restrict__ n1 = ws + 222656;
    const double* __restrict__ k1 = ws + 24192;
    const double* __restrict__ n2 = ws + 228704;
    const double* __restrict__ k2 = ws + 30240;
    const double* __restrict__ n3 = ws + 234752;
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
      ws[264992] = fma(-kk, wk0, ws[264992]);
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
      ws[265024] = fma(-kk, wk0, ws[265024]);
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
      ws[265056] = fma(-kk, wk0, ws[265056]);
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
      ws[265088] = fma(-kk, wk0, ws[265088]);
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
      ws[265120] = fma(-kk, wk0, ws[265120]);
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
      ws[265152] = fma(-kk, wk0, ws[265152]);
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
      ws[265184] = fma(-kk, wk0, ws[265184]);
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
      ws[265216] = fma(-kk, wk0, ws[265216]);
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
      ws[265248] = fma(-kk, wk0, ws[265248]);
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
      ws[265280] = fma(-kk, wk0, ws[265280]);
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
      ws[265312] = fma(-kk, wk0, ws[265312]);
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
      ws[265344] = fma(-kk, wk0, ws[265344]);
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
      ws[265376] = fma(-kk, wk0, ws[265376]);
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
      ws[265408] = fma(-kk, wk0, ws[265408]);
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
      ws[265440] = fma(-kk, wk0, ws[265440]);
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
      ws[265472] = fma(-kk, wk0, ws[265472]);
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
      ws[265504] = fma(-kk, wk0, ws[265504]);
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
      ws[265536] = fma(-kk, wk0, ws[265536]);
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
      ws[265568] = fma(-kk, wk0, ws[265568]);
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
      ws[265600] = fma(-kk, wk0, ws[265600]);
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
      ws[265632] = fma(-kk, wk0, ws[265632]);
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
      ws[265664] = fma(-kk, wk0, ws[265664]);
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
      ws[265696] = fma(-kk, wk0, ws[265696]);
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
      ws[265728] = fma(-kk, wk0, ws[265728]);
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
      ws[265760] = fma(-kk, wk0, ws[265760]);
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
      ws[265792] = fma(-kk, wk0, ws[265792]);
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
      ws[265824] = fma(-kk, wk0, ws[265824]);
    }
}
__device__ __noinline__ void adj_hess3_0_1(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    double* __restrict__ lam = ws + 216608;
    const double* __restrict__ n1 = ws + 222656;
    const double* __restrict__ k1 = ws + 24192;
    const double* __restrict__ n2 = ws + 228704;
    const double* __restrict__ k2 = ws + 30240;
    const double* __restrict__ n3 = ws + 234752;
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
      ws[265856] = fma(-kk, wk0, ws[265856]);
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
      ws[265888] = fma(-kk, wk0, ws[265888]);
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
      ws[265920] = fma(-kk, wk0, ws[265920]);
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
      ws[265952] = fma(-kk, wk0, ws[265952]);
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
      ws[265984] = fma(-kk, wk0, ws[265984]);
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
      ws[266016] = fma(-kk, wk0, ws[266016]);
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
      ws[266048] = fma(-kk, wk0, ws[266048]);
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
      ws[266080] = fma(-kk, wk0, ws[266080]);
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
      ws[266112] = fma(-kk, wk0, ws[266112]);
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
      ws[266144] = fma(-kk, wk0, ws[266144]);
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
      ws[266176] = fma(-kk, wk0, ws[266176]);
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
      ws[266208] = fma(-kk, wk0, ws[266208]);
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
      ws[266240] = fma(-kk, wk0, ws[266240]);
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
      ws[266272] = fma(-kk, fma(y[6016], wk0, y[5184] * wk1), ws[266272]);
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
      ws[266304] = fma(-kk, fma(y[5984], wk0, y[5184] * wk1), ws[266304]);
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
      ws[266336] = fma(-kk, fma(y[5824], wk0, y[5184] * wk1), ws[266336]);
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
      ws[266368] = fma(-kk, fma(y[5920], wk0, y[5184] * wk1), ws[266368]);
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
      ws[266400] = fma(-kk, wk0, ws[266400]);
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
      ws[266432] = fma(-kk, fma(y[5184], wk0, y[2336] * wk1), ws[266432]);
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
      ws[266464] = fma(-kk, wk0, ws[266464]);
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
      ws[266496] = fma(-kk, wk0, ws[266496]);
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
      ws[266528] = fma(-kk, wk0, ws[266528]);
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
      ws[266560] = fma(-kk, wk0, ws[266560]);
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
      ws[266592] = fma(-kk, fma(y[5984], wk0, y[6016] * wk1), ws[266592]);
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
      ws[266624] = fma(-kk, fma(y[5984], wk0, y[5984] * wk1), ws[266624]);
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
      ws[266656] = fma(-kk, fma(y[5984], wk0, y[5984] * wk1), ws[266656]);
      lam[5984] = fma(-kk, wk1, lam[5984]);
      lam[5984] = fma(-kk, wk0, lam[5984]);
    }
}
__device__ __noinline__ void adj_hess3_0_2(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    double* __restrict__ lam = ws + 216608;
    const double* __restrict__ n1 = ws + 222656;
    const double* __restrict__ k1 = ws + 24192;
    const double* __restrict__ n2 = ws + 228704;
    const double* __restrict__ k2 = ws + 30240;
    const double* __restrict__ n3 = ws + 234752;
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
      ws[266688] = fma(-kk, fma(y[6016], wk0, y[4000] * wk1), ws[266688]);
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
      ws[266720] = fma(-kk, fma(y[2336], wk0, y[5824] * wk1), ws[266720]);
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
      ws[266752] = fma(-kk, fma(y[6016], wk0, y[5824] * wk1), ws[266752]);
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
      ws[266784] = fma(-kk, fma(y[5984], wk0, y[5824] * wk1), ws[266784]);
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
      ws[266816] = fma(-kk, fma(y[5984], wk0, y[5824] * wk1), ws[266816]);
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
      ws[266848] = fma(-kk, fma(y[5824], wk0, y[5824] * wk1), ws[266848]);
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
      ws[266880] = fma(-kk, fma(y[6016], wk0, y[1184] * wk1), ws[266880]);
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
      ws[266912] = fma(-kk, fma(y[2336], wk0, y[5920] * wk1), ws[266912]);
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
      ws[266944] = fma(-kk, fma(y[2336], wk0, y[5920] * wk1), ws[266944]);
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
      ws[266976] = fma(-kk, fma(y[6016], wk0, y[5920] * wk1), ws[266976]);
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
      ws[267008] = fma(-kk, fma(y[6016], wk0, y[5024] * wk1), ws[267008]);
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
      ws[267040] = fma(-kk, fma(y[6016], wk0, y[5952] * wk1), ws[267040]);
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
      ws[267072] = fma(-kk, fma(y[5984], wk0, y[5952] * wk1), ws[267072]);
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
      ws[267104] = fma(-kk, fma(y[5824], wk0, y[5952] * wk1), ws[267104]);
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
      ws[267136] = fma(-kk, fma(y[5920], wk0, y[5952] * wk1), ws[267136]);
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
      ws[267168] = fma(-kk, fma(y[5952], wk0, y[5952] * wk1), ws[267168]);
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
      ws[267200] = fma(-kk, fma(y[5920], wk0, y[5952] * wk1), ws[267200]);
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
      ws[267232] = fma(-kk, wk0, ws[267232]);
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
      ws[267264] = fma(-kk, wk0, ws[267264]);
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
      ws[267296] = fma(-kk, fma(y[5984], wk0, y[5920] * wk1), ws[267296]);
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
      ws[267328] = fma(-kk, wk0, ws[267328]);
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
      ws[267360] = fma(-kk, fma(y[6016], wk0, y[1280] * wk1), ws[267360]);
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
      ws[267392] = fma(-kk, fma(y[6016], wk0, y[160] * wk1), ws[267392]);
      lam[160] = fma(-kk, wk1, lam[160]);
      lam[6016] = fma(-kk, wk0, lam[6016]);
    }
}
__device__ __noinline__ void adj_hess3_0_3(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    double* __restrict__ lam = ws + 216608;
    const double* __restrict__ n1 = ws + 222656;
    const double* __restrict__ k1 = ws + 24192;
    const double* __restrict__ n2 = ws + 228704;
    const double* __restrict__ k2 = ws + 30240;
    const double* __restrict__ n3 = ws + 234752;
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
      ws[267424] = fma(-kk, fma(y[6016], wk0, y[5664] * wk1), ws[267424]);
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
      ws[267456] = fma(-kk, wk0, ws[267456]);
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
      ws[267488] = fma(-kk, fma(y[6016], wk0, y[1888] * wk1), ws[267488]);
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
      ws[267520] = fma(-kk, fma(y[6016], wk0, y[2176] * wk1), ws[267520]);
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
      ws[267552] = fma(-kk, fma(y[6016], wk0, y[1120] * wk1), ws[267552]);
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
      ws[267584] = fma(-kk, fma(y[6016], wk0, y[2240] * wk1), ws[267584]);
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
      ws[267616] = fma(-kk, fma(y[6016], wk0, y[2752] * wk1), ws[267616]);
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
      ws[267648] = fma(-kk, fma(y[6016], wk0, y[1152] * wk1), ws[267648]);
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
      ws[267680] = fma(-kk, fma(y[6016], wk0, y[256] * wk1), ws[267680]);
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
      ws[267712] = fma(-kk, fma(y[6016], wk0, y[1216] * wk1), ws[267712]);
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
      ws[267744] = fma(-kk, fma(y[6016], wk0, y[288] * wk1), ws[267744]);
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
      ws[267776] = fma(-kk, fma(y[6016], wk0, y[320] * wk1), ws[267776]);
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
      ws[267808] = fma(-kk, fma(y[6016], wk0, y[352] * wk1), ws[267808]);
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
      ws[267840] = fma(-kk, fma(y[5184], wk0, y[1312] * wk1), ws[267840]);
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
      ws[267872] = fma(-kk, fma(y[5952], wk0, y[1312] * wk1), ws[267872]);
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
      ws[267904] = fma(-kk, fma(y[6016], wk0, y[1312] * wk1), ws[267904]);
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
      ws[267936] = fma(-kk, fma(y[5984], wk0, y[4288] * wk1), ws[267936]);
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
      ws[267968] = fma(-kk, fma(y[5824], wk0, y[4288] * wk1), ws[267968]);
      lam[4288] = fma(-kk, wk1, lam[4288]);
      lam[5824] = fma(-kk, wk0, lam[5824]);
    }
}
}  // namespace mech_cracmm2
