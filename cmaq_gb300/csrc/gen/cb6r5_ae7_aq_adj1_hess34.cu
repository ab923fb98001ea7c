// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void adj_hess3_1_16(double* __restrict__ ws)
{
    const double* __restrict__ y = ws + 0;
    double* __restrict__ lam = ws + 136480;
    const double* __restrict__ n1 = ws + 141248;
    const double* __restrict__ k1 = ws + 19072;
    const double* __restrict__ n2 = ws + 146016;
    const double* __restrict__ k2 = ws + 23840;
    const double* __restrict__ n3 = ws + 150784;
    const double* __restrict__ k3 = ws + 28608;
    {
      double w1 = 1.0 * n1[4736];
      w1 = w1 - n1[2432];
      w1 = w1 - n1[4736];
      double w2 = 1.0 * n2[4736];
      w2 = w2 - n2[2432];
      w2 = w2 - n2[4736];
      double w3 = 1.0 * n3[4736];
      w3 = w3 - n3[2432];
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[2432];
      wk0 = fma(w2, k2[2432], wk0);
      wk0 = fma(w3, k3[2432], wk0);
      double wk1 = w1 * k1[4736];
      wk1 = fma(w2, k2[4736], wk1);
      wk1 = fma(w3, k3[4736], wk1);
      const double kk = ws[43872];
      ws[185120] = fma(-kk, fma(y[4736], wk0, y[2432] * wk1), ws[185120]);
      lam[2432] = fma(-kk, wk1, lam[2432]);
      lam[4736] = fma(-kk, wk0, lam[4736]);
    }
    {
      double w1 = 1.0 * n1[4320];
      w1 = w1 - n1[2432];
      w1 = w1 - n1[4320];
      double w2 = 1.0 * n2[4320];
      w2 = w2 - n2[2432];
      w2 = w2 - n2[4320];
      double w3 = 1.0 * n3[4320];
      w3 = w3 - n3[2432];
      w3 = w3 - n3[4320];
      double wk0 = w1 * k1[2432];
      wk0 = fma(w2, k2[2432], wk0);
      wk0 = fma(w3, k3[2432], wk0);
      double wk1 = w1 * k1[4320];
      wk1 = fma(w2, k2[4320], wk1);
      wk1 = fma(w3, k3[4320], wk1);
      const double kk = ws[43904];
      ws[185152] = fma(-kk, fma(y[4320], wk0, y[2432] * wk1), ws[185152]);
      lam[2432] = fma(-kk, wk1, lam[2432]);
      lam[4320] = fma(-kk, wk0, lam[4320]);
    }
    {
      double w1 = 1.0 * n1[4640];
      w1 = w1 - n1[2432];
      w1 = w1 - n1[4640];
      double w2 = 1.0 * n2[4640];
      w2 = w2 - n2[2432];
      w2 = w2 - n2[4640];
      double w3 = 1.0 * n3[4640];
      w3 = w3 - n3[2432];
      w3 = w3 - n3[4640];
      double wk0 = w1 * k1[2432];
      wk0 = fma(w2, k2[2432], wk0);
      wk0 = fma(w3, k3[2432], wk0);
      double wk1 = w1 * k1[4640];
      wk1 = fma(w2, k2[4640], wk1);
      wk1 = fma(w3, k3[4640], wk1);
      const double kk = ws[43936];
      ws[185184] = fma(-kk, fma(y[4640], wk0, y[2432] * wk1), ws[185184]);
      lam[2432] = fma(-kk, wk1, lam[2432]);
      lam[4640] = fma(-kk, wk0, lam[4640]);
    }
    {
      double w1 = 1.0 * n1[4544];
      w1 = w1 - n1[2432];
      w1 = w1 - n1[4544];
      double w2 = 1.0 * n2[4544];
      w2 = w2 - n2[2432];
      w2 = w2 - n2[4544];
      double w3 = 1.0 * n3[4544];
      w3 = w3 - n3[2432];
      w3 = w3 - n3[4544];
      double wk0 = w1 * k1[2432];
      wk0 = fma(w2, k2[2432], wk0);
      wk0 = fma(w3, k3[2432], wk0);
      double wk1 = w1 * k1[4544];
      wk1 = fma(w2, k2[4544], wk1);
      wk1 = fma(w3, k3[4544], wk1);
      const double kk = ws[44000];
      ws[185248] = fma(-kk, fma(y[4544], wk0, y[2432] * wk1), ws[185248]);
      lam[2432] = fma(-kk, wk1, lam[2432]);
      lam[4544] = fma(-kk, wk0, lam[4544]);
    }
    {
      double w1 = 1.0 * n1[4736];
      w1 = w1 - n1[2976];
      w1 = w1 - n1[4736];
      double w2 = 1.0 * n2[4736];
      w2 = w2 - n2[2976];
      w2 = w2 - n2[4736];
      double w3 = 1.0 * n3[4736];
      w3 = w3 - n3[2976];
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[2976];
      wk0 = fma(w2, k2[2976], wk0);
      wk0 = fma(w3, k3[2976], wk0);
      double wk1 = w1 * k1[4736];
      wk1 = fma(w2, k2[4736], wk1);
      wk1 = fma(w3, k3[4736], wk1);
      const double kk = ws[44032];
      ws[185280] = fma(-kk, fma(y[4736], wk0, y[2976] * wk1), ws[185280]);
      lam[2976] = fma(-kk, wk1, lam[2976]);
      lam[4736] = fma(-kk, wk0, lam[4736]);
    }
    {
      double w1 = 1.0 * n1[4320];
      w1 = w1 - n1[2976];
      w1 = w1 - n1[4320];
      double w2 = 1.0 * n2[4320];
      w2 = w2 - n2[2976];
      w2 = w2 - n2[4320];
      double w3 = 1.0 * n3[4320];
      w3 = w3 - n3[2976];
      w3 = w3 - n3[4320];
      double wk0 = w1 * k1[2976];
      wk0 = fma(w2, k2[2976], wk0);
      wk0 = fma(w3, k3[2976], wk0);
      double wk1 = w1 * k1[4320];
      wk1 = fma(w2, k2[4320], wk1);
      wk1 = fma(w3, k3[4320], wk1);
      const double kk = ws[44064];
      ws[185312] = fma(-kk, fma(y[4320], wk0, y[2976] * wk1), ws[185312]);
      lam[2976] = fma(-kk, wk1, lam[2976]);
      lam[4320] = fma(-kk, wk0, lam[4320]);
    }
    {
      double w1 = 1.0 * n1[4640];
      w1 = w1 - n1[2976];
      w1 = w1 - n1[4640];
      double w2 = 1.0 * n2[4640];
      w2 = w2 - n2[2976];
      w2 = w2 - n2[4640];
      double w3 = 1.0 * n3[4640];
      w3 = w3 - n3[2976];
      w3 = w3 - n3[4640];
      double wk0 = w1 * k1[2976];
      wk0 = fma(w2, k2[2976], wk0);
      wk0 = fma(w3, k3[2976], wk0);
      double wk1 = w1 * k1[4640];
      wk1 = fma(w2, k2[4640], wk1);
      wk1 = fma(w3, k3[4640], wk1);
      const double kk = ws[44096];
      ws[185344] = fma(-kk, fma(y[4640], wk0, y[2976] * wk1), ws[185344]);
      lam[2976] = fma(-kk, wk1, lam[2976]);
      lam[4640] = fma(-kk, wk0, lam[4640]);
    }
    {
      double w1 = 1.0 * n1[4544];
      w1 = w1 - n1[2976];
      w1 = w1 - n1[4544];
      double w2 = 1.0 * n2[4544];
      w2 = w2 - n2[2976];
      w2 = w2 - n2[4544];
      double w3 = 1.0 * n3[4544];
      w3 = w3 - n3[2976];
      w3 = w3 - n3[4544];
      double wk0 = w1 * k1[2976];
      wk0 = fma(w2, k2[2976], wk0);
      wk0 = fma(w3, k3[2976], wk0);
      double wk1 = w1 * k1[4544];
      wk1 = fma(w2, k2[4544], wk1);
      wk1 = fma(w3, k3[4544], wk1);
      const double kk = ws[44160];
      ws[185408] = fma(-kk, fma(y[4544], wk0, y[2976] * wk1), ws[185408]);
      lam[2976] = fma(-kk, wk1, lam[2976]);
      lam[4544] = fma(-kk, wk0, lam[4544]);
    }
    {
      double w1 = 1.0 * n1[4736];
      w1 = w1 - n1[1536];
      w1 = w1 - n1[4736];
      double w2 = 1.0 * n2[4736];
      w2 = w2 - n2[1536];
      w2 = w2 - n2[4736];
      double w3 = 1.0 * n3[4736];
      w3 = w3 - n3[1536];
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[1536];
      wk0 = fma(w2, k2[1536], wk0);
      wk0 = fma(w3, k3[1536], wk0);
      double wk1 = w1 * k1[4736];
      wk1 = fma(w2, k2[4736], wk1);
      wk1 = fma(w3, k3[4736], wk1);
      const double kk = ws[44192];
      ws[185440] = fma(-kk, fma(y[4736], wk0, y[1536] * wk1), ws[185440]);
      lam[1536] = fma(-kk, wk1, lam[1536]);
      lam[4736] = fma(-kk, wk0, lam[4736]);
    }
    {
      double w1 = 1.0 * n1[4544];
      w1 = w1 - n1[1536];
      w1 = w1 - n1[4544];
      double w2 = 1.0 * n2[4544];
      w2 = w2 - n2[1536];
      w2 = w2 - n2[4544];
      double w3 = 1.0 * n3[4544];
      w3 = w3 - n3[1536];
      w3 = w3 - n3[4544];
      double wk0 = w1 * k1[1536];
      wk0 = fma(w2, k2[1536], wk0);
      wk0 = fma(w3, k3[1536], wk0);
      double wk1 = w1 * k1[4544];
      wk1 = fma(w2, k2[4544], wk1);
      wk1 = fma(w3, k3[4544], wk1);
      const double kk = ws[44224];
      ws[185472] = fma(-kk, fma(y[4544], wk0, y[1536] * wk1), ws[185472]);
      lam[1536] = fma(-kk, wk1, lam[1536]);
      lam[4544] = fma(-kk, wk0, lam[4544]);
    }
    {
      double w1 = 0.5 * n1[1568];
      w1 = fma(0.5, n1[3040], w1);
      w1 = fma(1.0, n1[4320], w1);
      w1 = w1 - n1[3008];
      w1 = w1 - n1[4320];
      double w2 = 0.5 * n2[1568];
      w2 = fma(0.5, n2[3040], w2);
      w2 = fma(1.0, n2[4320], w2);
      w2 = w2 - n2[3008];
      w2 = w2 - n2[4320];
      double w3 = 0.5 * n3[1568];
      w3 = fma(0.5, n3[3040], w3);
      w3 = fma(1.0, n3[4320], w3);
      w3 = w3 - n3[3008];
      w3 = w3 - n3[4320];
      double wk0 = w1 * k1[3008];
      wk0 = fma(w2, k2[3008], wk0);
      wk0 = fma(w3, k3[3008], wk0);
      double wk1 = w1 * k1[4320];
      wk1 = fma(w2, k2[4320], wk1);
      wk1 = fma(w3, k3[4320], wk1);
      const double kk = ws[44256];
      ws[185504] = fma(-kk, fma(y[4320], wk0, y[3008] * wk1), ws[185504]);
      lam[3008] = fma(-kk, wk1, lam[3008]);
      lam[4320] = fma(-kk, wk0, lam[4320]);
    }
    {
      double w1 = 1.0 * n1[3040];
      w1 = fma(1.0, n1[1184], w1);
      w1 = w1 - n1[3008];
      w1 = w1 - n1[1184];
      double w2 = 1.0 * n2[3040];
      w2 = fma(1.0, n2[1184], w2);
      w2 = w2 - n2[3008];
      w2 = w2 - n2[1184];
      double w3 = 1.0 * n3[3040];
      w3 = fma(1.0, n3[1184], w3);
      w3 = w3 - n3[3008];
      w3 = w3 - n3[1184];
      double wk0 = w1 * k1[3008];
      wk0 = fma(w2, k2[3008], wk0);
      wk0 = fma(w3, k3[3008], wk0);
      double wk1 = w1 * k1[1184];
      wk1 = fma(w2, k2[1184], wk1);
      wk1 = fma(w3, k3[1184], wk1);
      const double kk = ws[44288];
      ws[185536] = fma(-kk, fma(y[1184], wk0, y[3008] * wk1), ws[185536]);
      lam[3008] = fma(-kk, wk1, lam[3008]);
      lam[1184] = fma(-kk, wk0, lam[1184]);
    }
    {
      double w1 = 1.0 * n1[3040];
      w1 = fma(1.0, n1[3456], w1);
      w1 = w1 - n1[3008];
      w1 = w1 - n1[3456];
      double w2 = 1.0 * n2[3040];
      w2 = fma(1.0, n2[3456], w2);
      w2 = w2 - n2[3008];
      w2 = w2 - n2[3456];
      double w3 = 1.0 * n3[3040];
      w3 = fma(1.0, n3[3456], w3);
      w3 = w3 - n3[3008];
      w3 = w3 - n3[3456];
      double wk0 = w1 * k1[3008];
      wk0 = fma(w2, k2[3008], wk0);
      wk0 = fma(w3, k3[3008], wk0);
      double wk1 = w1 * k1[3456];
      wk1 = fma(w2, k2[3456], wk1);
      wk1 = fma(w3, k3[3456], wk1);
      const double kk = ws[44320];
      ws[185568] = fma(-kk, fma(y[3456], wk0, y[3008] * wk1), ws[185568]);
      lam[3008] = fma(-kk, wk1, lam[3008]);
      lam[3456] = fma(-kk, wk0, lam[3456]);
    }
    {
      double w1 = 0.5 * n1[1568];
      w1 = fma(0.5, n1[3040], w1);
      w1 = fma(1.0, n1[4736], w1);
      w1 = w1 - n1[3008];
      w1 = w1 - n1[4736];
      double w2 = 0.5 * n2[1568];
      w2 = fma(0.5, n2[3040], w2);
      w2 = fma(1.0, n2[4736], w2);
      w2 = w2 - n2[3008];
      w2 = w2 - n2[4736];
      double w3 = 0.5 * n3[1568];
      w3 = fma(0.5, n3[3040], w3);
      w3 = fma(1.0, n3[4736], w3);
      w3 = w3 - n3[3008];
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[3008];
      wk0 = fma(w2, k2[3008], wk0);
      wk0 = fma(w3, k3[3008], wk0);
      double wk1 = w1 * k1[4736];
      wk1 = fma(w2, k2[4736], wk1);
      wk1 = fma(w3, k3[4736], wk1);
      const double kk = ws[44352];
      ws[185600] = fma(-kk, fma(y[4736], wk0, y[3008] * wk1), ws[185600]);
      lam[3008] = fma(-kk, wk1, lam[3008]);
      lam[4736] = fma(-kk, wk0, lam[4736]);
    }
    {
      double w1 = 0.5 * n1[3008];
      w1 = fma(0.5, n1[3040], w1);
      w1 = fma(1.0, n1[4544], w1);
      w1 = w1 - n1[3008];
      w1 = w1 - n1[4544];
      double w2 = 0.5 * n2[3008];
      w2 = fma(0.5, n2[3040], w2);
      w2 = fma(1.0, n2[4544], w2);
      w2 = w2 - n2[3008];
      w2 = w2 - n2[4544];
      double w3 = 0.5 * n3[3008];
      w3 = fma(0.5, n3[3040], w3);
      w3 = fma(1.0, n3[4544], w3);
      w3 = w3 - n3[3008];
      w3 = w3 - n3[4544];
      double wk0 = w1 * k1[3008];
      wk0 = fma(w2, k2[3008], wk0);
      wk0 = fma(w3, k3[3008], wk0);
      double wk1 = w1 * k1[4544];
      wk1 = fma(w2, k2[4544], wk1);
      wk1 = fma(w3, k3[4544], wk1);
      const double kk = ws[44384];
      ws[185632] = fma(-kk, fma(y[4544], wk0, y[3008] * wk1), ws[185632]);
      lam[3008] = fma(-kk, wk1, lam[3008]);
      lam[4544] = fma(-kk, wk0, lam[4544]);
    }
    {
      double w1 = 1.0 * n1[2208];
      w1 = fma(1.0, n1[4416], w1);
      w1 = fma(1.0, n1[4512], w1);
      w1 = w1 - n1[2016];
      w1 = w1 - n1[4736];
      double w2 = 1.0 * n2[2208];
      w2 = fma(1.0, n2[4416], w2);
      w2 = fma(1.0, n2[4512], w2);
      w2 = w2 - n2[2016];
      w2 = w2 - n2[4736];
      double w3 = 1.0 * n3[2208];
      w3 = fma(1.0, n3[4416], w3);
      w3 = fma(1.0, n3[4512], w3);
      w3 = w3 - n3[2016];
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[2016];
      wk0 = fma(w2, k2[2016], wk0);
      wk0 = fma(w3, k3[2016], wk0);
      double wk1 = w1 * k1[4736];
      wk1 = fma(w2, k2[4736], wk1);
      wk1 = fma(w3, k3[4736], wk1);
      const double kk = ws[44416];
      ws[185664] = fma(-kk, fma(y[4736], wk0, y[2016] * wk1), ws[185664]);
      lam[2016] = fma(-kk, wk1, lam[2016]);
      lam[4736] = fma(-kk, wk0, lam[4736]);
    }
    {
      double w1 = 0.75 * n1[2208];
      w1 = fma(0.25, n1[1600], w1);
      w1 = fma(1.0, n1[4416], w1);
      w1 = w1 - n1[2016];
      w1 = w1 - n1[4736];
      double w2 = 0.75 * n2[2208];
      w2 = fma(0.25, n2[1600], w2);
      w2 = fma(1.0, n2[4416], w2);
      w2 = w2 - n2[2016];
      w2 = w2 - n2[4736];
      double w3 = 0.75 * n3[2208];
      w3 = fma(0.25, n3[1600], w3);
      w3 = fma(1.0, n3[4416], w3);
      w3 = w3 - n3[2016];
      w3 = w3 - n3[4736];
      double wk0 = w1 * k1[2016];
      wk0 = fma(w2, k2[2016], wk0);
      wk0 = fma(w3, k3[2016], wk0);
      double wk1 = w1 * k1[4736];
      wk1 = fma(w2, k2[4736], wk1);
      wk1 = fma(w3, k3[4736], wk1);
      const double kk = ws[44448];
      ws[185696] = fma(-kk, fma(y[4736], wk0, y[2016] * wk1), ws[185696]);
      lam[2016] = fma(-kk, wk1, lam[2016]);
      lam[4736] = fma(-kk, wk0, lam[4736]);
    }
    {
      double w1 = 1.0 * n1[2208];
      w1 = fma(1.0, n1[4192], w1);
      w1 = fma(1.0, n1[4416], w1);
      w1 = fma(1.0, n1[4512], w1);
      w1 = w1 - n1[2016];
      w1 = w1 - n1[4640];
      double w2 = 1.0 * n2[2208];
      w2 = fma(1.0, n2[4192], w2);
      w2 = fma(1.0, n2[4416], w2);
      w2 = fma(1.0, n2[4512], w2);
      w2 = w2 - n2[2016];
      w2 = w2 - n2[4640];
      double w3 = 1.0 * n3[2208];
      w3 = fma(1.0, n3[4192], w3);
      w3 = fma(1.0, n3[4416], w3);
      w3 = fma(1.0, n3[4512], w3);
      w3 = w3 - n3[2016];
      w3 = w3 - n3[4640];
      double wk0 = w1 * k1[2016];
      wk0 = fma(w2, k2[2016], wk0);
      wk0 = fma(w3, k3[2016], wk0);
      double wk1 = w1 * k1[4640];
      wk1 = fma(w2, k2[4640], wk1);
      wk1 = fma(w3, k3[4640], wk1);
      const double kk = ws[44480];
      ws[185728] = fma(-kk, fma(y[4640], wk0, y[2016] * wk1), ws[185728]);
      lam[2016] = fma(-kk, wk1, lam[2016]);
      lam[4640] = fma(-kk, wk0, lam[4640]);
    }
    {
      double w1 = 0.86 * n1[2208];
      w1 = fma(1.0, n1[4416], w1);
      w1 = fma(0.45, n1[4512], w1);
      w1 = fma(0.45, n1[3968], w1);
      w1 = fma(0.14, n1[1600], w1);
      w1 = fma(0.55, n1[3520], w1);
      w1 = w1 - n1[2016];
      w1 = w1 - n1[4544];
      double w2 = 0.86 * n2[2208];
      w2 = fma(1.0, n2[4416], w2);
      w2 = fma(0.45, n2[4512], w2);
      w2 = fma(0.45, n2[3968], w2);
      w2 = fma(0.14, n2[1600], w2);
      w2 = fma(0.55, n2[3520], w2);
      w2 = w2 - n2[2016];
      w2 = w2 - n2[4544];
      double w3 = 0.86 * n3[2208];
      w3 = fma(1.0, n3[4416], w3);
      w3 = fma(0.45, n3[4512], w3);
      w3 = fma(0.45, n3[3968], w3);
      w3 = fma(0.14, n3[1600], w3);
      w3 = fma(0.55, n3[3520], w3);
      w3 = w3 - n3[2016];
      w3 = w3 - n3[4544];
      double wk0 = w1 * k1[2016];
      wk0 = fma(w2, k2[2016], wk0);
      wk0 = fma(w3, k3[2016], wk0);
      double wk1 = w1 * k1[4544];
      wk1 = fma(w2, k2[4544], wk1);
      wk1 = fma(w3, k3[4544], wk1);
      const double kk = ws[44512];
      ws[185760] = fma(-kk, fma(y[4544], wk0, y[2016] * wk1), ws[185760]);
      lam[2016] = fma(-kk, wk1, lam[2016]);
      lam[4544] = fma(-kk, wk0, lam[4544]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
