// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void adj_jtv_1_4(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[4032];
      w = fma(0.5, phi[3328], w);
      w = fma(1.0, phi[4192], w);
      w = w - phi[2176];
      w = w - phi[4640];
      const double kw = ws[39744] * w;
      out[2176] = fma(kw, y[4640], out[2176]);
      out[4640] = fma(kw, y[2176], out[4640]);
      ws[180992] = fma(kw * y[2176], y[4640], ws[180992]);
    }
    {
      double w = 1.0 * phi[4000];
      w = fma(0.4, phi[4256], w);
      w = fma(2.0, phi[4576], w);
      w = fma(2.0, phi[4672], w);
      w = w - phi[3808];
      w = w - phi[4736];
      const double kw = ws[39840] * w;
      out[3808] = fma(kw, y[4736], out[3808]);
      out[4736] = fma(kw, y[3808], out[4736]);
      ws[181088] = fma(kw * y[3808], y[4736], ws[181088]);
    }
    {
      double w = 1.2 * phi[4000];
      w = fma(0.5, phi[4736], w);
      w = fma(0.6, phi[4448], w);
      w = fma(0.1, phi[4128], w);
      w = fma(0.5, phi[4480], w);
      w = fma(0.3, phi[4576], w);
      w = fma(0.3, phi[4672], w);
      w = w - phi[3808];
      w = w - phi[4320];
      const double kw = ws[39872] * w;
      out[3808] = fma(kw, y[4320], out[3808]);
      out[4320] = fma(kw, y[3808], out[4320]);
      ws[181120] = fma(kw * y[3808], y[4320], ws[181120]);
    }
    {
      double w = 0.5 * phi[4608];
      w = fma(0.5, phi[4032], w);
      w = fma(0.45, phi[4576], w);
      w = fma(0.45, phi[4352], w);
      w = fma(0.1, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = fma(0.25, phi[3936], w);
      w = fma(0.25, phi[4000], w);
      w = w - phi[3808];
      w = w - phi[4640];
      const double kw = ws[39904] * w;
      out[3808] = fma(kw, y[4640], out[3808]);
      out[4640] = fma(kw, y[3808], out[4640]);
      ws[181152] = fma(kw * y[3808], y[4640], ws[181152]);
    }
    {
      double w = 0.6 * phi[3744];
      w = fma(0.4, phi[4576], w);
      w = fma(0.4, phi[4672], w);
      w = fma(0.4, phi[4256], w);
      w = w - phi[3936];
      w = w - phi[4736];
      const double kw = ws[39968] * w;
      out[3936] = fma(kw, y[4736], out[3936]);
      out[4736] = fma(kw, y[3936], out[4736]);
      ws[181216] = fma(kw * y[3936], y[4736], ws[181216]);
    }
    {
      double w = 1.4 * phi[4256];
      w = fma(0.24, phi[4000], w);
      w = fma(0.5, phi[4736], w);
      w = fma(0.12, phi[4448], w);
      w = fma(0.08, phi[4512], w);
      w = fma(0.02, phi[4128], w);
      w = fma(1.98, phi[4480], w);
      w = fma(0.56, phi[4704], w);
      w = w - phi[3936];
      w = w - phi[4320];
      const double kw = ws[40000] * w;
      out[3936] = fma(kw, y[4320], out[3936]);
      out[4320] = fma(kw, y[3936], out[4320]);
      ws[181248] = fma(kw * y[3936], y[4320], ws[181248]);
    }
    {
      double w = 1.0 * phi[3744];
      w = fma(1.0, phi[4192], w);
      w = w - phi[3936];
      w = w - phi[4640];
      const double kw = ws[40032] * w;
      out[3936] = fma(kw, y[4640], out[3936]);
      out[4640] = fma(kw, y[3936], out[4640]);
      ws[181280] = fma(kw * y[3936], y[4640], ws[181280]);
    }
    {
      double w = 0.14 * phi[4512];
      w = fma(0.2, phi[4704], w);
      w = fma(0.5, phi[3328], w);
      w = w - phi[1760];
      w = w - phi[4736];
      const double kw = ws[40064] * w;
      out[1760] = fma(kw, y[4736], out[1760]);
      out[4736] = fma(kw, y[1760], out[4736]);
      ws[181312] = fma(kw * y[1760], y[4736], ws[181312]);
    }
    {
      double w = 1.0 * phi[3328];
      w = fma(1.0, phi[4192], w);
      w = w - phi[1760];
      w = w - phi[4640];
      const double kw = ws[40096] * w;
      out[1760] = fma(kw, y[4640], out[1760]);
      out[4640] = fma(kw, y[1760], out[4640]);
      ws[181344] = fma(kw * y[1760], y[4640], ws[181344]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(0.5, phi[4256], w);
      w = fma(0.5, phi[4480], w);
      w = fma(0.8, phi[4704], w);
      w = fma(0.2, phi[4096], w);
      w = w - phi[3744];
      w = w - phi[4384];
      const double kw = ws[40128] * w;
      out[3744] = fma(kw, y[4384], out[3744]);
      out[4384] = fma(kw, y[3744], out[4384]);
      ws[181376] = fma(kw * y[3744], y[4384], ws[181376]);
    }
    {
      double w = 1.0 * phi[1792];
      w = w - phi[3744];
      w = w - phi[4608];
      const double kw = ws[40160] * w;
      out[3744] = fma(kw, y[4608], out[3744]);
      out[4608] = fma(kw, y[3744], out[4608]);
      ws[181408] = fma(kw * y[3744], y[4608], ws[181408]);
    }
    {
      double w = 1.0 * phi[3744];
      w = fma(1.0, phi[4608], w);
      w = w - phi[1792];
      const double kw = ws[40192] * w;
      out[1792] = out[1792] + kw;
      ws[181440] = fma(kw, y[1792], ws[181440]);
    }
    {
      double w = 0.37 * phi[2688];
      w = fma(0.13, phi[3904], w);
      w = fma(0.13, phi[4320], w);
      w = fma(0.5, phi[4736], w);
      w = fma(0.5, phi[4416], w);
      w = fma(0.5, phi[4672], w);
      w = w - phi[3744];
      w = w - phi[4704];
      const double kw = ws[40224] * w;
      out[3744] = fma(kw, y[4704], out[3744]);
      out[4704] = fma(kw, y[3744], out[4704]);
      ws[181472] = fma(kw * y[3744], y[4704], ws[181472]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4352], w);
      w = fma(1.0, phi[4064], w);
      w = fma(2.0, phi[4672], w);
      w = w - phi[3744];
      w = w - phi[4448];
      const double kw = ws[40256] * w;
      out[3744] = fma(kw, y[4448], out[3744]);
      out[4448] = fma(kw, y[3744], out[4448]);
      ws[181504] = fma(kw * y[3744], y[4448], ws[181504]);
    }
    {
      double w = 0.8 * phi[4576];
      w = fma(0.8, phi[4064], w);
      w = fma(1.8, phi[4672], w);
      w = fma(0.2, phi[3904], w);
      w = w - phi[3744];
      w = w - phi[4672];
      const double kw = ws[40288] * w;
      out[3744] = fma(kw, y[4672], out[3744]);
      out[4672] = fma(kw, y[3744], out[4672]);
      ws[181536] = fma(kw * y[3744], y[4672], ws[181536]);
    }
    {
      double w = 0.5 * phi[4608];
      w = fma(0.5, phi[4256], w);
      w = fma(1.0, phi[4480], w);
      w = fma(0.5, phi[4032], w);
      w = w - phi[1792];
      w = w - phi[4736];
      const double kw = ws[40320] * w;
      out[1792] = fma(kw, y[4736], out[1792]);
      out[4736] = fma(kw, y[1792], out[4736]);
      ws[181568] = fma(kw * y[1792], y[4736], ws[181568]);
    }
    {
      double w = 1.0 * phi[4128];
      w = fma(1.0, phi[4608], w);
      w = w - phi[1952];
      w = w - phi[4736];
      const double kw = ws[40352] * w;
      out[1952] = fma(kw, y[4736], out[1952]);
      out[4736] = fma(kw, y[1952], out[4736]);
      ws[181600] = fma(kw * y[1952], y[4736], ws[181600]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4672], w);
      w = w - phi[416];
      w = w - phi[4736];
      const double kw = ws[40384] * w;
      out[416] = fma(kw, y[4736], out[416]);
      out[4736] = fma(kw, y[416], out[4736]);
      ws[181632] = fma(kw * y[416], y[4736], ws[181632]);
    }
    {
      double w = 1.0 * phi[4288];
      w = fma(1.0, phi[4672], w);
      w = w - phi[928];
      const double kw = ws[40416] * w;
      out[928] = out[928] + kw;
      ws[181664] = fma(kw, y[928], ws[181664]);
    }
    {
      double w = 0.732 * phi[3392];
      w = fma(0.268, phi[4064], w);
      w = fma(0.268, phi[4224], w);
      w = fma(1.0, phi[4576], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[928];
      const double kw = ws[40448] * w;
      out[928] = out[928] + kw;
      ws[181696] = fma(kw, y[928], ws[181696]);
    }
    {
      double w = 1.0 * phi[4288];
      w = fma(1.0, phi[4672], w);
      w = w - phi[1984];
      const double kw = ws[40480] * w;
      out[1984] = out[1984] + kw;
      ws[181728] = fma(kw, y[1984], ws[181728]);
    }
    {
      double w = 0.126 * phi[4064];
      w = fma(0.874, phi[960], w);
      w = fma(0.126, phi[4576], w);
      w = fma(0.874, phi[4352], w);
      w = fma(1.0, phi[4672], w);
      w = fma(-0.126, phi[4224], w);
      w = w - phi[1984];
      const double kw = ws[40512] * w;
      out[1984] = out[1984] + kw;
      ws[181760] = fma(kw, y[1984], ws[181760]);
    }
    {
      double w = 1.0 * phi[4192];
      w = w - phi[4608];
      w = w - phi[4736];
      const double kw = ws[40544] * w;
      out[4608] = fma(kw, y[4736], out[4608]);
      out[4736] = fma(kw, y[4608], out[4736]);
      ws[181792] = fma(kw * y[4608], y[4736], ws[181792]);
    }
    {
      double w = 1.0 * phi[3520];
      w = w - phi[4544];
      w = w - phi[4320];
      const double kw = ws[40640] * w;
      out[4544] = fma(kw, y[4320], out[4544]);
      out[4320] = fma(kw, y[4544], out[4320]);
      ws[181888] = fma(kw * y[4544], y[4320], ws[181888]);
    }
    {
      double w = 0.3 * phi[1184];
      w = fma(1.4, phi[4544], w);
      w = w - phi[3520];
      w = w - phi[3520];
      const double kw = ws[40672] * w;
      out[3520] = fma(kw, y[3520], out[3520]);
      out[3520] = fma(kw, y[3520], out[3520]);
      ws[181920] = fma(kw * y[3520], y[3520], ws[181920]);
    }
    {
      double w = 1.0 * phi[4544];
      w = fma(1.0, phi[4608], w);
      w = w - phi[3520];
      w = w - phi[4384];
      const double kw = ws[40704] * w;
      out[3520] = fma(kw, y[4384], out[3520]);
      out[4384] = fma(kw, y[3520], out[4384]);
      ws[181952] = fma(kw * y[3520], y[4384], ws[181952]);
    }
    {
      double w = 1.0 * phi[1824];
      w = w - phi[3520];
      w = w - phi[4704];
      const double kw = ws[40736] * w;
      out[3520] = fma(kw, y[4704], out[3520]);
      out[4704] = fma(kw, y[3520], out[4704]);
      ws[181984] = fma(kw * y[3520], y[4704], ws[181984]);
    }
    {
      double w = 1.0 * phi[4544];
      w = fma(1.0, phi[4512], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[3520];
      w = w - phi[4416];
      const double kw = ws[40768] * w;
      out[3520] = fma(kw, y[4416], out[3520]);
      out[4416] = fma(kw, y[3520], out[4416]);
      ws[182016] = fma(kw * y[3520], y[4416], ws[182016]);
    }
    {
      double w = 1.0 * phi[4544];
      w = fma(1.0, phi[4480], w);
      w = w - phi[4736];
      w = w - phi[3232];
      const double kw = ws[40800] * w;
      out[4736] = fma(kw, y[3232], out[4736]);
      out[3232] = fma(kw, y[4736], out[3232]);
      ws[182048] = fma(kw * y[4736], y[3232], ws[182048]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[4416], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4544];
      const double kw = ws[40864] * w;
      out[4544] = out[4544] + kw;
      ws[182112] = fma(kw, y[4544], ws[182112]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[1984], w);
      w = w - phi[4544];
      w = w - phi[4224];
      const double kw = ws[40896] * w;
      out[4544] = fma(kw, y[4224], out[4544]);
      out[4224] = fma(kw, y[4544], out[4224]);
      ws[182144] = fma(kw * y[4544], y[4224], ws[182144]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[3392], w);
      w = fma(0.97, phi[4576], w);
      w = fma(0.03, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4544];
      w = w - phi[896];
      const double kw = ws[40928] * w;
      out[4544] = fma(kw, y[896], out[4544]);
      out[896] = fma(kw, y[4544], out[896]);
      ws[182176] = fma(kw * y[4544], y[896], ws[182176]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(0.991, phi[4128], w);
      w = fma(0.991, phi[4576], w);
      w = fma(0.009, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4544];
      w = w - phi[832];
      const double kw = ws[40960] * w;
      out[4544] = fma(kw, y[832], out[4544]);
      out[832] = fma(kw, y[4544], out[832]);
      ws[182208] = fma(kw * y[4544], y[832], ws[182208]);
    }
    {
      double w = 1.0 * phi[3232];
      w = fma(2.0, phi[4352], w);
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4512], w);
      w = w - phi[4544];
      w = w - phi[2656];
      const double kw = ws[40992] * w;
      out[4544] = fma(kw, y[2656], out[4544]);
      out[2656] = fma(kw, y[4544], out[2656]);
      ws[182240] = fma(kw * y[4544], y[2656], ws[182240]);
    }
    {
      double w = 1.0 * phi[3232];
      w = fma(0.33, phi[4128], w);
      w = fma(0.67, phi[4064], w);
      w = fma(2.0, phi[4352], w);
      w = fma(1.0, phi[4704], w);
      w = fma(-1.0, phi[4224], w);
      w = w - phi[4544];
      w = w - phi[3552];
      const double kw = ws[41024] * w;
      out[4544] = fma(kw, y[3552], out[4544]);
      out[3552] = fma(kw, y[4544], out[3552]);
      ws[182272] = fma(kw * y[4544], y[3552], ws[182272]);
    }
    {
      double w = 0.3 * phi[3968];
      w = fma(0.7, phi[3232], w);
      w = fma(0.45, phi[4128], w);
      w = fma(0.55, phi[4064], w);
      w = fma(0.3, phi[3552], w);
      w = fma(0.3, phi[4224], w);
      w = fma(1.7, phi[4352], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[4544];
      w = w - phi[3136];
      const double kw = ws[41056] * w;
      out[4544] = fma(kw, y[3136], out[4544]);
      out[3136] = fma(kw, y[4544], out[3136]);
      ws[182304] = fma(kw * y[4544], y[3136], ws[182304]);
    }
    {
      double w = 1.0 * phi[3232];
      w = fma(1.0, phi[3872], w);
      w = fma(0.96, phi[4576], w);
      w = fma(0.04, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4544];
      w = w - phi[2528];
      const double kw = ws[41088] * w;
      out[4544] = fma(kw, y[2528], out[4544]);
      out[2528] = fma(kw, y[4544], out[2528]);
      ws[182336] = fma(kw * y[4544], y[2528], ws[182336]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4480], w);
      w = w - phi[4544];
      w = w - phi[4512];
      const double kw = ws[41120] * w;
      out[4544] = fma(kw, y[4512], out[4544]);
      out[4512] = fma(kw, y[4544], out[4512]);
      ws[182368] = fma(kw * y[4544], y[4512], ws[182368]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[4448], w);
      w = w - phi[4544];
      w = w - phi[4128];
      const double kw = ws[41152] * w;
      out[4544] = fma(kw, y[4128], out[4544]);
      out[4128] = fma(kw, y[4544], out[4128]);
      ws[182400] = fma(kw * y[4544], y[4128], ws[182400]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[4096], w);
      w = w - phi[4544];
      w = w - phi[4064];
      const double kw = ws[41184] * w;
      out[4544] = fma(kw, y[4064], out[4544]);
      out[4064] = fma(kw, y[4544], out[4064]);
      ws[182432] = fma(kw * y[4544], y[4064], ws[182432]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4512], w);
      w = w - phi[4544];
      w = w - phi[2720];
      const double kw = ws[41216] * w;
      out[4544] = fma(kw, y[2720], out[4544]);
      out[2720] = fma(kw, y[4544], out[2720]);
      ws[182464] = fma(kw * y[4544], y[2720], ws[182464]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4128], w);
      w = w - phi[4544];
      w = w - phi[864];
      const double kw = ws[41248] * w;
      out[4544] = fma(kw, y[864], out[4544]);
      out[864] = fma(kw, y[4544], out[864]);
      ws[182496] = fma(kw * y[4544], y[864], ws[182496]);
    }
    {
      double w = 1.0 * phi[4544];
      w = w - phi[3968];
      w = w - phi[4736];
      const double kw = ws[41280] * w;
      out[3968] = fma(kw, y[4736], out[3968]);
      out[4736] = fma(kw, y[3968], out[4736]);
      ws[182528] = fma(kw * y[3968], y[4736], ws[182528]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(0.18, phi[3616], w);
      w = fma(0.65, phi[3488], w);
      w = fma(0.72, phi[4672], w);
      w = fma(0.1, phi[3936], w);
      w = fma(0.1, phi[4736], w);
      w = fma(0.07, phi[4576], w);
      w = fma(0.18, phi[4704], w);
      w = fma(1.0, phi[2944], w);
      w = w - phi[4544];
      w = w - phi[1088];
      const double kw = ws[41312] * w;
      out[4544] = fma(kw, y[1088], out[4544]);
      out[1088] = fma(kw, y[4544], out[1088]);
      ws[182560] = fma(kw * y[4544], y[1088], ws[182560]);
    }
}
__device__ __noinline__ void adj_jtv_1_5(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[3968];
      w = fma(0.155, phi[3616], w);
      w = fma(0.544, phi[3584], w);
      w = fma(0.602, phi[4672], w);
      w = fma(0.244, phi[3808], w);
      w = fma(0.244, phi[4736], w);
      w = fma(0.058, phi[4576], w);
      w = fma(0.155, phi[4704], w);
      w = fma(1.0, phi[2496], w);
      w = w - phi[4544];
      w = w - phi[1120];
      const double kw = ws[41344] * w;
      out[4544] = fma(kw, y[1120], out[4544]);
      out[1120] = fma(kw, y[4544], out[1120]);
      ws[182592] = fma(kw * y[4544], y[1120], ws[182592]);
    }
    {
      double w = 1.0 * phi[3968];
      w = fma(0.155, phi[3616], w);
      w = fma(0.544, phi[3584], w);
      w = fma(0.602, phi[4672], w);
      w = fma(0.244, phi[3808], w);
      w = fma(0.244, phi[4736], w);
      w = fma(0.058, phi[4576], w);
      w = fma(0.155, phi[4704], w);
      w = fma(1.0, phi[2560], w);
      w = w - phi[4544];
      w = w - phi[1152];
      const double kw = ws[41376] * w;
      out[4544] = fma(kw, y[1152], out[4544]);
      out[1152] = fma(kw, y[4544], out[1152]);
      ws[182624] = fma(kw * y[4544], y[1152], ws[182624]);
    }
    {
      double w = 1.0 * phi[1216];
      w = w - phi[3520];
      w = w - phi[4608];
      const double kw = ws[41440] * w;
      out[3520] = fma(kw, y[4608], out[3520]);
      out[4608] = fma(kw, y[3520], out[4608]);
      ws[182688] = fma(kw * y[3520], y[4608], ws[182688]);
    }
    {
      double w = 1.0 * phi[1824];
      w = fma(1.0, phi[4192], w);
      w = w - phi[1216];
      const double kw = ws[41536] * w;
      out[1216] = out[1216] + kw;
      ws[182784] = fma(kw, y[1216], ws[182784]);
    }
    {
      double w = 1.0 * phi[1824];
      w = fma(1.0, phi[4192], w);
      w = w - phi[1216];
      const double kw = ws[41568] * w;
      out[1216] = out[1216] + kw;
      ws[182816] = fma(kw, y[1216], ws[182816]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(0.016, phi[3264], w);
      w = fma(0.051, phi[2624], w);
      w = fma(0.047, phi[3072], w);
      w = w - phi[2944];
      w = w - phi[4384];
      const double kw = ws[41600] * w;
      out[2944] = fma(kw, y[4384], out[2944]);
      out[4384] = fma(kw, y[2944], out[4384]);
      ws[182848] = fma(kw * y[2944], y[4384], ws[182848]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(0.14, phi[2240], w);
      w = w - phi[2944];
      w = w - phi[4704];
      const double kw = ws[41632] * w;
      out[2944] = fma(kw, y[4704], out[2944]);
      out[4704] = fma(kw, y[2944], out[4704]);
      ws[182880] = fma(kw * y[2944], y[4704], ws[182880]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(0.015, phi[3264], w);
      w = fma(0.023, phi[2624], w);
      w = fma(0.06, phi[3072], w);
      w = w - phi[2496];
      w = w - phi[4384];
      const double kw = ws[41664] * w;
      out[2496] = fma(kw, y[4384], out[2496]);
      out[4384] = fma(kw, y[2496], out[4384]);
      ws[182912] = fma(kw * y[2496], y[4384], ws[182912]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(0.193, phi[2240], w);
      w = w - phi[2496];
      w = w - phi[4704];
      const double kw = ws[41696] * w;
      out[2496] = fma(kw, y[4704], out[2496]);
      out[4704] = fma(kw, y[2496], out[4704]);
      ws[182944] = fma(kw * y[2496], y[4704], ws[182944]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(0.034, phi[3264], w);
      w = fma(0.392, phi[3072], w);
      w = w - phi[2144];
      w = w - phi[4384];
      const double kw = ws[41728] * w;
      out[2144] = fma(kw, y[4384], out[2144]);
      out[4384] = fma(kw, y[2144], out[4384]);
      ws[182976] = fma(kw * y[2144], y[4384], ws[182976]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(0.146, phi[2240], w);
      w = w - phi[2144];
      w = w - phi[4704];
      const double kw = ws[41760] * w;
      out[2144] = fma(kw, y[4704], out[2144]);
      out[4704] = fma(kw, y[2144], out[4704]);
      ws[183008] = fma(kw * y[2144], y[4704], ws[183008]);
    }
    {
      double w = 1.0 * phi[4320];
      w = fma(1.0, phi[1888], w);
      w = w - phi[1856];
      w = w - phi[4320];
      const double kw = ws[41792] * w;
      out[1856] = fma(kw, y[4320], out[1856]);
      out[4320] = fma(kw, y[1856], out[4320]);
      ws[183040] = fma(kw * y[1856], y[4320], ws[183040]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[1888], w);
      w = w - phi[1856];
      w = w - phi[4736];
      const double kw = ws[41824] * w;
      out[1856] = fma(kw, y[4736], out[1856]);
      out[4736] = fma(kw, y[1856], out[4736]);
      ws[183072] = fma(kw * y[1856], y[4736], ws[183072]);
    }
    {
      double w = 1.0 * phi[4640];
      w = fma(1.0, phi[1888], w);
      w = w - phi[1856];
      w = w - phi[4640];
      const double kw = ws[41856] * w;
      out[1856] = fma(kw, y[4640], out[1856]);
      out[4640] = fma(kw, y[1856], out[4640]);
      ws[183104] = fma(kw * y[1856], y[4640], ws[183104]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(0.028, phi[3264], w);
      w = fma(0.225, phi[2624], w);
      w = fma(0.191, phi[3072], w);
      w = w - phi[2560];
      w = w - phi[4384];
      const double kw = ws[41888] * w;
      out[2560] = fma(kw, y[4384], out[2560]);
      out[4384] = fma(kw, y[2560], out[4384]);
      ws[183136] = fma(kw * y[2560], y[4384], ws[183136]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(0.473, phi[2240], w);
      w = w - phi[2560];
      w = w - phi[4704];
      const double kw = ws[41920] * w;
      out[2560] = fma(kw, y[4704], out[2560]);
      out[4704] = fma(kw, y[2560], out[4704]);
      ws[183168] = fma(kw * y[2560], y[4704], ws[183168]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.006, phi[3264], w);
      w = fma(0.052, phi[2624], w);
      w = fma(0.081, phi[3072], w);
      w = w - phi[448];
      w = w - phi[4736];
      const double kw = ws[41952] * w;
      out[448] = fma(kw, y[4736], out[448]);
      out[4736] = fma(kw, y[448], out[4736]);
      ws[183200] = fma(kw * y[448], y[4736], ws[183200]);
    }
    {
      double w = 1.0 * phi[4192];
      w = w - phi[4032];
      const double kw = ws[41984] * w;
      out[4032] = out[4032] + kw;
      ws[183232] = fma(kw, y[4032], ws[183232]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.0, phi[1920], w);
      w = w - phi[1280];
      const double kw = ws[42016] * w;
      out[1280] = out[1280] + kw;
      ws[183264] = fma(kw, y[1280], ws[183264]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.0, phi[1248], w);
      w = w - phi[1280];
      const double kw = ws[42048] * w;
      out[1280] = out[1280] + kw;
      ws[183296] = fma(kw, y[1280], ws[183296]);
    }
    {
      double w = 1.0 * phi[4192];
      w = w - phi[1920];
      const double kw = ws[42080] * w;
      out[1920] = out[1920] + kw;
      ws[183328] = fma(kw, y[1920], ws[183328]);
    }
    {
      double w = 1.0 * phi[4192];
      w = w - phi[1248];
      const double kw = ws[42112] * w;
      out[1248] = out[1248] + kw;
      ws[183360] = fma(kw, y[1248], ws[183360]);
    }
    {
      double w = 1.0 * phi[2592];
      w = w - phi[1920];
      w = w - phi[480];
      const double kw = ws[42144] * w;
      out[1920] = fma(kw, y[480], out[1920]);
      out[480] = fma(kw, y[1920], out[480]);
      ws[183392] = fma(kw * y[1920], y[480], ws[183392]);
    }
    {
      double w = 1.0 * phi[2592];
      w = w - phi[1920];
      w = w - phi[512];
      const double kw = ws[42176] * w;
      out[1920] = fma(kw, y[512], out[1920]);
      out[512] = fma(kw, y[1920], out[512]);
      ws[183424] = fma(kw * y[1920], y[512], ws[183424]);
    }
    {
      double w = 1.0 * phi[2592];
      w = w - phi[1248];
      w = w - phi[544];
      const double kw = ws[42208] * w;
      out[1248] = fma(kw, y[544], out[1248]);
      out[544] = fma(kw, y[1248], out[544]);
      ws[183456] = fma(kw * y[1248], y[544], ws[183456]);
    }
    {
      double w = 0.5 * phi[2464];
      w = fma(0.5, phi[4192], w);
      w = w - phi[4608];
      const double kw = ws[42240] * w;
      out[4608] = out[4608] + kw;
      ws[183488] = fma(kw, y[4608], ws[183488]);
    }
    {
      double w = 1.0 * phi[1312];
      w = w - phi[1056];
      const double kw = ws[42304] * w;
      out[1056] = out[1056] + kw;
      ws[183552] = fma(kw, y[1056], ws[183552]);
    }
    {
      double w = 1.0 * phi[608];
      w = w - phi[1312];
      w = w - phi[576];
      const double kw = ws[42336] * w;
      out[1312] = fma(kw, y[576], out[1312]);
      out[576] = fma(kw, y[1312], out[576]);
      ws[183584] = fma(kw * y[1312], y[576], ws[183584]);
    }
    {
      double w = 1.0 * phi[608];
      w = w - phi[1312];
      const double kw = ws[42368] * w;
      out[1312] = out[1312] + kw;
      ws[183616] = fma(kw, y[1312], ws[183616]);
    }
    {
      double w = 1.0 * phi[640];
      w = w - phi[4256];
      const double kw = ws[42400] * w;
      out[4256] = out[4256] + kw;
      ws[183648] = fma(kw, y[4256], ws[183648]);
    }
    {
      double w = 1.0 * phi[640];
      w = w - phi[4000];
      const double kw = ws[42432] * w;
      out[4000] = out[4000] + kw;
      ws[183680] = fma(kw, y[4000], ws[183680]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(0.688, phi[3360], w);
      w = w - phi[2848];
      w = w - phi[4384];
      const double kw = ws[42464] * w;
      out[2848] = fma(kw, y[4384], out[2848]);
      out[4384] = fma(kw, y[2848], out[4384]);
      ws[183712] = fma(kw * y[2848], y[4384], ws[183712]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(1.0, phi[3360], w);
      w = w - phi[2848];
      w = w - phi[4704];
      const double kw = ws[42496] * w;
      out[2848] = fma(kw, y[4704], out[2848]);
      out[4704] = fma(kw, y[2848], out[4704]);
      ws[183744] = fma(kw * y[2848], y[4704], ws[183744]);
    }
    {
      double w = 1.0 * phi[4640];
      w = fma(0.422, phi[3360], w);
      w = w - phi[2848];
      w = w - phi[4640];
      const double kw = ws[42528] * w;
      out[2848] = fma(kw, y[4640], out[2848]);
      out[4640] = fma(kw, y[2848], out[4640]);
      ws[183776] = fma(kw * y[2848], y[4640], ws[183776]);
    }
    {
      double w = 1.0 * phi[4672];
      w = fma(0.711, phi[3360], w);
      w = w - phi[2848];
      w = w - phi[4672];
      const double kw = ws[42560] * w;
      out[2848] = fma(kw, y[4672], out[2848]);
      out[4672] = fma(kw, y[2848], out[4672]);
      ws[183808] = fma(kw * y[2848], y[4672], ws[183808]);
    }
    {
      double w = 1.0 * phi[4544];
      w = fma(0.37, phi[3360], w);
      w = w - phi[3360];
      w = w - phi[4544];
      const double kw = ws[42592] * w;
      out[3360] = fma(kw, y[4544], out[3360]);
      out[4544] = fma(kw, y[3360], out[4544]);
      ws[183840] = fma(kw * y[3360], y[4544], ws[183840]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.24, phi[3360], w);
      w = w - phi[3360];
      w = w - phi[4736];
      const double kw = ws[42624] * w;
      out[3360] = fma(kw, y[4736], out[3360]);
      out[4736] = fma(kw, y[3360], out[4736]);
      ws[183872] = fma(kw * y[3360], y[4736], ws[183872]);
    }
    {
      double w = 1.0 * phi[32];
      w = w - phi[0];
      const double kw = ws[42688] * w;
      out[0] = out[0] + kw;
      ws[183936] = fma(kw, y[0], ws[183936]);
    }
    {
      double w = 0.907 * phi[1376];
      w = w - phi[64];
      const double kw = ws[42720] * w;
      out[64] = out[64] + kw;
      ws[183968] = fma(kw, y[64], ws[183968]);
    }
    {
      double w = 0.925 * phi[1376];
      w = w - phi[96];
      const double kw = ws[42752] * w;
      out[96] = out[96] + kw;
      ws[184000] = fma(kw, y[96], ws[184000]);
    }
    {
      double w = 0.943 * phi[1376];
      w = w - phi[128];
      const double kw = ws[42784] * w;
      out[128] = out[128] + kw;
      ws[184032] = fma(kw, y[128], ws[184032]);
    }
    {
      double w = 0.5 * phi[1408];
      w = w - phi[160];
      const double kw = ws[42816] * w;
      out[160] = out[160] + kw;
      ws[184064] = fma(kw, y[160], ws[184064]);
    }
    {
      double w = 0.5 * phi[1408];
      w = w - phi[192];
      const double kw = ws[42848] * w;
      out[192] = out[192] + kw;
      ws[184096] = fma(kw, y[192], ws[184096]);
    }
    {
      double w = 1.5 * phi[1408];
      w = w - phi[224];
      const double kw = ws[42880] * w;
      out[224] = out[224] + kw;
      ws[184128] = fma(kw, y[224], ws[184128]);
    }
    {
      double w = 1.25 * phi[1440];
      w = fma(1.0, phi[704], w);
      w = fma(1.0, phi[4736], w);
      w = w - phi[704];
      w = w - phi[4736];
      const double kw = ws[42912] * w;
      out[704] = fma(kw, y[4736], out[704]);
      out[4736] = fma(kw, y[704], out[4736]);
      ws[184160] = fma(kw * y[704], y[4736], ws[184160]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[1440];
      w = w - phi[4736];
      const double kw = ws[42944] * w;
      out[1440] = fma(kw, y[4736], out[1440]);
      out[4736] = fma(kw, y[1440], out[4736]);
      ws[184192] = fma(kw * y[1440], y[4736], ws[184192]);
    }
    {
      double w = 1.25 * phi[1472];
      w = fma(1.0, phi[736], w);
      w = fma(1.0, phi[4736], w);
      w = w - phi[736];
      w = w - phi[4736];
      const double kw = ws[42976] * w;
      out[736] = fma(kw, y[4736], out[736]);
      out[4736] = fma(kw, y[736], out[4736]);
      ws[184224] = fma(kw * y[736], y[4736], ws[184224]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[1472];
      w = w - phi[4736];
      const double kw = ws[43008] * w;
      out[1472] = fma(kw, y[4736], out[1472]);
      out[4736] = fma(kw, y[1472], out[4736]);
      ws[184256] = fma(kw * y[1472], y[4736], ws[184256]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[800], w);
      w = w - phi[768];
      w = w - phi[4736];
      const double kw = ws[43040] * w;
      out[768] = fma(kw, y[4736], out[768]);
      out[4736] = fma(kw, y[768], out[4736]);
      ws[184288] = fma(kw * y[768], y[4736], ws[184288]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.4857, phi[2752], w);
      w = fma(0.0062, phi[2784], w);
      w = fma(0.0025, phi[2816], w);
      w = fma(0.0026, phi[2304], w);
      w = fma(0.0023, phi[1504], w);
      w = fma(0.2944, phi[3680], w);
      w = fma(0.2021, phi[3712], w);
      w = fma(0.0019, phi[3168], w);
      w = fma(0.0023, phi[3200], w);
      w = w - phi[2752];
      w = w - phi[4736];
      const double kw = ws[43072] * w;
      out[2752] = fma(kw, y[4736], out[2752]);
      out[4736] = fma(kw, y[2752], out[4736]);
      ws[184320] = fma(kw * y[2752], y[4736], ws[184320]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.3003, phi[2752], w);
      w = fma(0.2862, phi[2784], w);
      w = fma(0.0041, phi[2816], w);
      w = fma(0.0035, phi[2304], w);
      w = fma(0.2239, phi[3680], w);
      w = fma(0.182, phi[3712], w);
      w = w - phi[2784];
      w = w - phi[4736];
      const double kw = ws[43104] * w;
      out[2784] = fma(kw, y[4736], out[2784]);
      out[4736] = fma(kw, y[2784], out[4736]);
      ws[184352] = fma(kw * y[2784], y[4736], ws[184352]);
    }
}
__device__ __noinline__ void adj_jtv_1_6(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[4736];
      w = fma(0.3856, phi[2752], w);
      w = fma(0.095, phi[2784], w);
      w = fma(0.1373, phi[2816], w);
      w = fma(0.0005, phi[2304], w);
      w = fma(0.2051, phi[3680], w);
      w = fma(0.1764, phi[3712], w);
      w = w - phi[2816];
      w = w - phi[4736];
      const double kw = ws[43136] * w;
      out[2816] = fma(kw, y[4736], out[2816]);
      out[4736] = fma(kw, y[2816], out[4736]);
      ws[184384] = fma(kw * y[2816], y[4736], ws[184384]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.2181, phi[2752], w);
      w = fma(0.3063, phi[2784], w);
      w = fma(0.0153, phi[2816], w);
      w = fma(0.1043, phi[2304], w);
      w = fma(0.1893, phi[3680], w);
      w = fma(0.1668, phi[3712], w);
      w = w - phi[2304];
      w = w - phi[4736];
      const double kw = ws[43168] * w;
      out[2304] = fma(kw, y[4736], out[2304]);
      out[4736] = fma(kw, y[2304], out[4736]);
      ws[184416] = fma(kw * y[2304], y[4736], ws[184416]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.2412, phi[2752], w);
      w = fma(0.2089, phi[2784], w);
      w = fma(0.3, phi[2816], w);
      w = fma(0.2028, phi[3680], w);
      w = fma(0.0471, phi[3712], w);
      w = w - phi[1504];
      w = w - phi[4736];
      const double kw = ws[43200] * w;
      out[1504] = fma(kw, y[4736], out[1504]);
      out[4736] = fma(kw, y[1504], out[4736]);
      ws[184448] = fma(kw * y[1504], y[4736], ws[184448]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.6664, phi[3680], w);
      w = fma(0.0143, phi[3712], w);
      w = fma(0.0123, phi[2912], w);
      w = fma(0.1239, phi[3168], w);
      w = fma(0.1831, phi[3200], w);
      w = w - phi[3680];
      w = w - phi[4736];
      const double kw = ws[43232] * w;
      out[3680] = fma(kw, y[4736], out[3680]);
      out[4736] = fma(kw, y[3680], out[4736]);
      ws[184480] = fma(kw * y[3680], y[4736], ws[184480]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.2858, phi[3680], w);
      w = fma(0.3931, phi[3712], w);
      w = fma(0.0139, phi[2912], w);
      w = fma(0.1027, phi[3168], w);
      w = fma(0.2045, phi[3200], w);
      w = w - phi[3712];
      w = w - phi[4736];
      const double kw = ws[43264] * w;
      out[3712] = fma(kw, y[4736], out[3712]);
      out[4736] = fma(kw, y[3712], out[4736]);
      ws[184512] = fma(kw * y[3712], y[4736], ws[184512]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.3303, phi[3680], w);
      w = fma(0.2272, phi[3712], w);
      w = fma(0.2607, phi[2912], w);
      w = fma(0.0702, phi[3168], w);
      w = fma(0.1116, phi[3200], w);
      w = w - phi[2912];
      w = w - phi[4736];
      const double kw = ws[43296] * w;
      out[2912] = fma(kw, y[4736], out[2912]);
      out[4736] = fma(kw, y[2912], out[4736]);
      ws[184544] = fma(kw * y[2912], y[4736], ws[184544]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.3444, phi[3680], w);
      w = fma(0.2749, phi[3712], w);
      w = fma(0.0491, phi[2912], w);
      w = fma(0.2577, phi[3168], w);
      w = fma(0.0739, phi[3200], w);
      w = w - phi[3168];
      w = w - phi[4736];
      const double kw = ws[43328] * w;
      out[3168] = fma(kw, y[4736], out[3168]);
      out[4736] = fma(kw, y[3168], out[4736]);
      ws[184576] = fma(kw * y[3168], y[4736], ws[184576]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.3886, phi[3680], w);
      w = fma(0.2421, phi[3712], w);
      w = fma(0.064, phi[2912], w);
      w = fma(0.0385, phi[3168], w);
      w = fma(0.2667, phi[3200], w);
      w = w - phi[3200];
      w = w - phi[4736];
      const double kw = ws[43360] * w;
      out[3200] = fma(kw, y[4736], out[3200]);
      out[4736] = fma(kw, y[3200], out[4736]);
      ws[184608] = fma(kw * y[3200], y[4736], ws[184608]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[2336];
      w = w - phi[4736];
      const double kw = ws[43392] * w;
      out[2336] = fma(kw, y[4736], out[2336]);
      out[4736] = fma(kw, y[2336], out[4736]);
      ws[184640] = fma(kw * y[2336], y[4736], ws[184640]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[2336];
      w = w - phi[4640];
      const double kw = ws[43424] * w;
      out[2336] = fma(kw, y[4640], out[2336]);
      out[4640] = fma(kw, y[2336], out[4640]);
      ws[184672] = fma(kw * y[2336], y[4640], ws[184672]);
    }
    {
      double w = 1.0 * phi[4160];
      w = w - phi[2336];
      w = w - phi[4160];
      const double kw = ws[43456] * w;
      out[2336] = fma(kw, y[4160], out[2336]);
      out[4160] = fma(kw, y[2336], out[4160]);
      ws[184704] = fma(kw * y[2336], y[4160], ws[184704]);
    }
    {
      double w = 1.0 * phi[4544];
      w = w - phi[2336];
      w = w - phi[4544];
      const double kw = ws[43552] * w;
      out[2336] = fma(kw, y[4544], out[2336]);
      out[4544] = fma(kw, y[2336], out[4544]);
      ws[184800] = fma(kw * y[2336], y[4544], ws[184800]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[2368];
      w = w - phi[4736];
      const double kw = ws[43584] * w;
      out[2368] = fma(kw, y[4736], out[2368]);
      out[4736] = fma(kw, y[2368], out[4736]);
      ws[184832] = fma(kw * y[2368], y[4736], ws[184832]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[2368];
      w = w - phi[4640];
      const double kw = ws[43616] * w;
      out[2368] = fma(kw, y[4640], out[2368]);
      out[4640] = fma(kw, y[2368], out[4640]);
      ws[184864] = fma(kw * y[2368], y[4640], ws[184864]);
    }
    {
      double w = 1.0 * phi[4160];
      w = w - phi[2368];
      w = w - phi[4160];
      const double kw = ws[43648] * w;
      out[2368] = fma(kw, y[4160], out[2368]);
      out[4160] = fma(kw, y[2368], out[4160]);
      ws[184896] = fma(kw * y[2368], y[4160], ws[184896]);
    }
    {
      double w = 1.0 * phi[4544];
      w = w - phi[2368];
      w = w - phi[4544];
      const double kw = ws[43712] * w;
      out[2368] = fma(kw, y[4544], out[2368]);
      out[4544] = fma(kw, y[2368], out[4544]);
      ws[184960] = fma(kw * y[2368], y[4544], ws[184960]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(0.58, phi[2976], w);
      w = w - phi[2400];
      w = w - phi[4736];
      const double kw = ws[43744] * w;
      out[2400] = fma(kw, y[4736], out[2400]);
      out[4736] = fma(kw, y[2400], out[4736]);
      ws[184992] = fma(kw * y[2400], y[4736], ws[184992]);
    }
    {
      double w = 1.0 * phi[4320];
      w = fma(0.52, phi[2976], w);
      w = w - phi[2400];
      w = w - phi[4320];
      const double kw = ws[43776] * w;
      out[2400] = fma(kw, y[4320], out[2400]);
      out[4320] = fma(kw, y[2400], out[4320]);
      ws[185024] = fma(kw * y[2400], y[4320], ws[185024]);
    }
    {
      double w = 1.0 * phi[4640];
      w = fma(0.045, phi[2976], w);
      w = w - phi[2400];
      w = w - phi[4640];
      const double kw = ws[43808] * w;
      out[2400] = fma(kw, y[4640], out[2400]);
      out[4640] = fma(kw, y[2400], out[4640]);
      ws[185056] = fma(kw * y[2400], y[4640], ws[185056]);
    }
    {
      double w = 1.0 * phi[4544];
      w = fma(0.58, phi[2976], w);
      w = w - phi[2400];
      w = w - phi[4544];
      const double kw = ws[43840] * w;
      out[2400] = fma(kw, y[4544], out[2400]);
      out[4544] = fma(kw, y[2400], out[4544]);
      ws[185088] = fma(kw * y[2400], y[4544], ws[185088]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[2432];
      w = w - phi[4736];
      const double kw = ws[43872] * w;
      out[2432] = fma(kw, y[4736], out[2432]);
      out[4736] = fma(kw, y[2432], out[4736]);
      ws[185120] = fma(kw * y[2432], y[4736], ws[185120]);
    }
    {
      double w = 1.0 * phi[4320];
      w = w - phi[2432];
      w = w - phi[4320];
      const double kw = ws[43904] * w;
      out[2432] = fma(kw, y[4320], out[2432]);
      out[4320] = fma(kw, y[2432], out[4320]);
      ws[185152] = fma(kw * y[2432], y[4320], ws[185152]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[2432];
      w = w - phi[4640];
      const double kw = ws[43936] * w;
      out[2432] = fma(kw, y[4640], out[2432]);
      out[4640] = fma(kw, y[2432], out[4640]);
      ws[185184] = fma(kw * y[2432], y[4640], ws[185184]);
    }
    {
      double w = 1.0 * phi[4544];
      w = w - phi[2432];
      w = w - phi[4544];
      const double kw = ws[44000] * w;
      out[2432] = fma(kw, y[4544], out[2432]);
      out[4544] = fma(kw, y[2432], out[4544]);
      ws[185248] = fma(kw * y[2432], y[4544], ws[185248]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[2976];
      w = w - phi[4736];
      const double kw = ws[44032] * w;
      out[2976] = fma(kw, y[4736], out[2976]);
      out[4736] = fma(kw, y[2976], out[4736]);
      ws[185280] = fma(kw * y[2976], y[4736], ws[185280]);
    }
    {
      double w = 1.0 * phi[4320];
      w = w - phi[2976];
      w = w - phi[4320];
      const double kw = ws[44064] * w;
      out[2976] = fma(kw, y[4320], out[2976]);
      out[4320] = fma(kw, y[2976], out[4320]);
      ws[185312] = fma(kw * y[2976], y[4320], ws[185312]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[2976];
      w = w - phi[4640];
      const double kw = ws[44096] * w;
      out[2976] = fma(kw, y[4640], out[2976]);
      out[4640] = fma(kw, y[2976], out[4640]);
      ws[185344] = fma(kw * y[2976], y[4640], ws[185344]);
    }
    {
      double w = 1.0 * phi[4544];
      w = w - phi[2976];
      w = w - phi[4544];
      const double kw = ws[44160] * w;
      out[2976] = fma(kw, y[4544], out[2976]);
      out[4544] = fma(kw, y[2976], out[4544]);
      ws[185408] = fma(kw * y[2976], y[4544], ws[185408]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[1536];
      w = w - phi[4736];
      const double kw = ws[44192] * w;
      out[1536] = fma(kw, y[4736], out[1536]);
      out[4736] = fma(kw, y[1536], out[4736]);
      ws[185440] = fma(kw * y[1536], y[4736], ws[185440]);
    }
    {
      double w = 1.0 * phi[4544];
      w = w - phi[1536];
      w = w - phi[4544];
      const double kw = ws[44224] * w;
      out[1536] = fma(kw, y[4544], out[1536]);
      out[4544] = fma(kw, y[1536], out[4544]);
      ws[185472] = fma(kw * y[1536], y[4544], ws[185472]);
    }
    {
      double w = 0.5 * phi[1568];
      w = fma(0.5, phi[3040], w);
      w = fma(1.0, phi[4320], w);
      w = w - phi[3008];
      w = w - phi[4320];
      const double kw = ws[44256] * w;
      out[3008] = fma(kw, y[4320], out[3008]);
      out[4320] = fma(kw, y[3008], out[4320]);
      ws[185504] = fma(kw * y[3008], y[4320], ws[185504]);
    }
    {
      double w = 1.0 * phi[3040];
      w = fma(1.0, phi[1184], w);
      w = w - phi[3008];
      w = w - phi[1184];
      const double kw = ws[44288] * w;
      out[3008] = fma(kw, y[1184], out[3008]);
      out[1184] = fma(kw, y[3008], out[1184]);
      ws[185536] = fma(kw * y[3008], y[1184], ws[185536]);
    }
    {
      double w = 1.0 * phi[3040];
      w = fma(1.0, phi[3456], w);
      w = w - phi[3008];
      w = w - phi[3456];
      const double kw = ws[44320] * w;
      out[3008] = fma(kw, y[3456], out[3008]);
      out[3456] = fma(kw, y[3008], out[3456]);
      ws[185568] = fma(kw * y[3008], y[3456], ws[185568]);
    }
    {
      double w = 0.5 * phi[1568];
      w = fma(0.5, phi[3040], w);
      w = fma(1.0, phi[4736], w);
      w = w - phi[3008];
      w = w - phi[4736];
      const double kw = ws[44352] * w;
      out[3008] = fma(kw, y[4736], out[3008]);
      out[4736] = fma(kw, y[3008], out[4736]);
      ws[185600] = fma(kw * y[3008], y[4736], ws[185600]);
    }
    {
      double w = 0.5 * phi[3008];
      w = fma(0.5, phi[3040], w);
      w = fma(1.0, phi[4544], w);
      w = w - phi[3008];
      w = w - phi[4544];
      const double kw = ws[44384] * w;
      out[3008] = fma(kw, y[4544], out[3008]);
      out[4544] = fma(kw, y[3008], out[4544]);
      ws[185632] = fma(kw * y[3008], y[4544], ws[185632]);
    }
    {
      double w = 1.0 * phi[2208];
      w = fma(1.0, phi[4416], w);
      w = fma(1.0, phi[4512], w);
      w = w - phi[2016];
      w = w - phi[4736];
      const double kw = ws[44416] * w;
      out[2016] = fma(kw, y[4736], out[2016]);
      out[4736] = fma(kw, y[2016], out[4736]);
      ws[185664] = fma(kw * y[2016], y[4736], ws[185664]);
    }
    {
      double w = 0.75 * phi[2208];
      w = fma(0.25, phi[1600], w);
      w = fma(1.0, phi[4416], w);
      w = w - phi[2016];
      w = w - phi[4736];
      const double kw = ws[44448] * w;
      out[2016] = fma(kw, y[4736], out[2016]);
      out[4736] = fma(kw, y[2016], out[4736]);
      ws[185696] = fma(kw * y[2016], y[4736], ws[185696]);
    }
    {
      double w = 1.0 * phi[2208];
      w = fma(1.0, phi[4192], w);
      w = fma(1.0, phi[4416], w);
      w = fma(1.0, phi[4512], w);
      w = w - phi[2016];
      w = w - phi[4640];
      const double kw = ws[44480] * w;
      out[2016] = fma(kw, y[4640], out[2016]);
      out[4640] = fma(kw, y[2016], out[4640]);
      ws[185728] = fma(kw * y[2016], y[4640], ws[185728]);
    }
    {
      double w = 0.86 * phi[2208];
      w = fma(1.0, phi[4416], w);
      w = fma(0.45, phi[4512], w);
      w = fma(0.45, phi[3968], w);
      w = fma(0.14, phi[1600], w);
      w = fma(0.55, phi[3520], w);
      w = w - phi[2016];
      w = w - phi[4544];
      const double kw = ws[44512] * w;
      out[2016] = fma(kw, y[4544], out[2016]);
      out[4544] = fma(kw, y[2016], out[4544]);
      ws[185760] = fma(kw * y[2016], y[4544], ws[185760]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
