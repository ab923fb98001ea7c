// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_jtv_1_4(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.32, phi[5344], w);
      w = fma(0.68, phi[5376], w);
      w = fma(0.68, phi[5728], w);
      w = w - phi[3648];
      w = w - phi[5824];
      const double kw = ws[49184] * w;
      out[3648] = fma(kw, y[5824], out[3648]);
      out[5824] = fma(kw, y[3648], out[5824]);
      ws[277888] = fma(kw * y[3648], y[5824], ws[277888]);
    }
    {
      double w = 1.0 * phi[3808];
      w = fma(1.0, phi[5920], w);
      w = w - phi[3040];
      w = w - phi[5824];
      const double kw = ws[49216] * w;
      out[3040] = fma(kw, y[5824], out[3040]);
      out[5824] = fma(kw, y[3040], out[5824]);
      ws[277920] = fma(kw * y[3040], y[5824], ws[277920]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5376], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2976];
      w = w - phi[5824];
      const double kw = ws[49248] * w;
      out[2976] = fma(kw, y[5824], out[2976]);
      out[5824] = fma(kw, y[2976], out[5824]);
      ws[277952] = fma(kw * y[2976], y[5824], ws[277952]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5440], w);
      w = w - phi[4032];
      w = w - phi[5824];
      const double kw = ws[49280] * w;
      out[4032] = fma(kw, y[5824], out[4032]);
      out[5824] = fma(kw, y[4032], out[5824]);
      ws[277984] = fma(kw * y[4032], y[5824], ws[277984]);
    }
    {
      double w = 2.0 * phi[5920];
      w = fma(0.287, phi[5856], w);
      w = fma(1.24, phi[5760], w);
      w = fma(0.464, phi[5504], w);
      w = w - phi[4064];
      w = w - phi[5824];
      const double kw = ws[49312] * w;
      out[4064] = fma(kw, y[5824], out[4064]);
      out[5824] = fma(kw, y[4064], out[5824]);
      ws[278016] = fma(kw * y[4064], y[5824], ws[278016]);
    }
    {
      double w = 2.0 * phi[5920];
      w = fma(1.0, phi[5376], w);
      w = fma(1.0, phi[5728], w);
      w = w - phi[3072];
      w = w - phi[5824];
      const double kw = ws[49344] * w;
      out[3072] = fma(kw, y[5824], out[3072]);
      out[5824] = fma(kw, y[3072], out[5824]);
      ws[278048] = fma(kw * y[3072], y[5824], ws[278048]);
    }
    {
      double w = 1.0 * phi[5920];
      w = w - phi[5216];
      w = w - phi[5824];
      const double kw = ws[49376] * w;
      out[5216] = fma(kw, y[5824], out[5216]);
      out[5824] = fma(kw, y[5216], out[5824]);
      ws[278080] = fma(kw * y[5216], y[5824], ws[278080]);
    }
    {
      double w = 1.0 * phi[5440];
      w = w - phi[2688];
      w = w - phi[5920];
      const double kw = ws[49408] * w;
      out[2688] = fma(kw, y[5920], out[2688]);
      out[5920] = fma(kw, y[2688], out[5920]);
      ws[278112] = fma(kw * y[2688], y[5920], ws[278112]);
    }
    {
      double w = 1.0 * phi[5440];
      w = w - phi[3232];
      w = w - phi[5920];
      const double kw = ws[49440] * w;
      out[3232] = fma(kw, y[5920], out[3232]);
      out[5920] = fma(kw, y[3232], out[5920]);
      ws[278144] = fma(kw * y[3232], y[5920], ws[278144]);
    }
    {
      double w = 1.0 * phi[5440];
      w = w - phi[3808];
      w = w - phi[5920];
      const double kw = ws[49472] * w;
      out[3808] = fma(kw, y[5920], out[3808]);
      out[5920] = fma(kw, y[3808], out[5920]);
      ws[278176] = fma(kw * y[3808], y[5920], ws[278176]);
    }
    {
      double w = 1.0 * phi[2816];
      w = w - phi[5888];
      w = w - phi[5984];
      const double kw = ws[49504] * w;
      out[5888] = fma(kw, y[5984], out[5888]);
      out[5984] = fma(kw, y[5888], out[5984]);
      ws[278208] = fma(kw * y[5888], y[5984], ws[278208]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[5632];
      w = w - phi[5984];
      const double kw = ws[49536] * w;
      out[5632] = fma(kw, y[5984], out[5632]);
      out[5984] = fma(kw, y[5632], out[5984]);
      ws[278240] = fma(kw * y[5632], y[5984], ws[278240]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[5408];
      w = w - phi[5984];
      const double kw = ws[49568] * w;
      out[5408] = fma(kw, y[5984], out[5408]);
      out[5984] = fma(kw, y[5408], out[5984]);
      ws[278272] = fma(kw * y[5408], y[5984], ws[278272]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[5120];
      w = w - phi[5984];
      const double kw = ws[49600] * w;
      out[5120] = fma(kw, y[5984], out[5120]);
      out[5984] = fma(kw, y[5120], out[5984]);
      ws[278304] = fma(kw * y[5120], y[5984], ws[278304]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3008];
      w = w - phi[5984];
      const double kw = ws[49632] * w;
      out[3008] = fma(kw, y[5984], out[3008]);
      out[5984] = fma(kw, y[3008], out[5984]);
      ws[278336] = fma(kw * y[3008], y[5984], ws[278336]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3200];
      w = w - phi[5984];
      const double kw = ws[49664] * w;
      out[3200] = fma(kw, y[5984], out[3200]);
      out[5984] = fma(kw, y[3200], out[5984]);
      ws[278368] = fma(kw * y[3200], y[5984], ws[278368]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3328];
      w = w - phi[5984];
      const double kw = ws[49696] * w;
      out[3328] = fma(kw, y[5984], out[3328]);
      out[5984] = fma(kw, y[3328], out[5984]);
      ws[278400] = fma(kw * y[3328], y[5984], ws[278400]);
    }
    {
      double w = 0.6021 * phi[5728];
      w = fma(0.3979, phi[4896], w);
      w = w - phi[3360];
      w = w - phi[5984];
      const double kw = ws[49728] * w;
      out[3360] = fma(kw, y[5984], out[3360]);
      out[5984] = fma(kw, y[3360], out[5984]);
      ws[278432] = fma(kw * y[3360], y[5984], ws[278432]);
    }
    {
      double w = 0.7195 * phi[5728];
      w = fma(0.2805, phi[4896], w);
      w = w - phi[3296];
      w = w - phi[5984];
      const double kw = ws[49760] * w;
      out[3296] = fma(kw, y[5984], out[3296]);
      out[5984] = fma(kw, y[3296], out[5984]);
      ws[278464] = fma(kw * y[3296], y[5984], ws[278464]);
    }
    {
      double w = 0.0482 * phi[5728];
      w = fma(0.6747, phi[4608], w);
      w = fma(0.2771, phi[4928], w);
      w = w - phi[3104];
      w = w - phi[5984];
      const double kw = ws[49792] * w;
      out[3104] = fma(kw, y[5984], out[3104]);
      out[5984] = fma(kw, y[3104], out[5984]);
      ws[278496] = fma(kw * y[3104], y[5984], ws[278496]);
    }
    {
      double w = 0.0854 * phi[5728];
      w = fma(0.6341, phi[4608], w);
      w = fma(0.2805, phi[4928], w);
      w = w - phi[3264];
      w = w - phi[5984];
      const double kw = ws[49824] * w;
      out[3264] = fma(kw, y[5984], out[3264]);
      out[5984] = fma(kw, y[3264], out[5984]);
      ws[278528] = fma(kw * y[3264], y[5984], ws[278528]);
    }
    {
      double w = 0.039 * phi[4480];
      w = fma(0.039, phi[4576], w);
      w = fma(0.0625, phi[5856], w);
      w = fma(0.762, phi[4096], w);
      w = fma(0.3225, phi[5984], w);
      w = fma(0.1885, phi[4544], w);
      w = fma(0.238, phi[6016], w);
      w = fma(0.0105, phi[5504], w);
      w = w - phi[4160];
      w = w - phi[5984];
      const double kw = ws[49856] * w;
      out[4160] = fma(kw, y[5984], out[4160]);
      out[5984] = fma(kw, y[4160], out[5984]);
      ws[278560] = fma(kw * y[4160], y[5984], ws[278560]);
    }
    {
      double w = 1.0 * phi[4256];
      w = w - phi[3744];
      w = w - phi[5984];
      const double kw = ws[49888] * w;
      out[3744] = fma(kw, y[5984], out[3744]);
      out[5984] = fma(kw, y[3744], out[5984]);
      ws[278592] = fma(kw * y[3744], y[5984], ws[278592]);
    }
    {
      double w = 0.461 * phi[4384];
      w = fma(0.455, phi[4544], w);
      w = fma(0.539, phi[5920], w);
      w = fma(0.6195, phi[6016], w);
      w = fma(0.077, phi[5760], w);
      w = fma(0.007, phi[5504], w);
      w = fma(0.007, phi[5856], w);
      w = w - phi[2624];
      w = w - phi[5984];
      const double kw = ws[49920] * w;
      out[2624] = fma(kw, y[5984], out[2624]);
      out[5984] = fma(kw, y[2624], out[5984]);
      ws[278624] = fma(kw * y[2624], y[5984], ws[278624]);
    }
    {
      double w = 1.0 * phi[4256];
      w = w - phi[3840];
      w = w - phi[5984];
      const double kw = ws[49952] * w;
      out[3840] = fma(kw, y[5984], out[3840]);
      out[5984] = fma(kw, y[3840], out[5984]);
      ws[278656] = fma(kw * y[3840], y[5984], ws[278656]);
    }
    {
      double w = 0.9 * phi[4096];
      w = fma(0.1, phi[4576], w);
      w = fma(0.1, phi[6016], w);
      w = fma(0.1, phi[5984], w);
      w = fma(0.06, phi[5856], w);
      w = w - phi[4192];
      w = w - phi[5984];
      const double kw = ws[49984] * w;
      out[4192] = fma(kw, y[5984], out[4192]);
      out[5984] = fma(kw, y[4192], out[5984]);
      ws[278688] = fma(kw * y[4192], y[5984], ws[278688]);
    }
    {
      double w = 1.0 * phi[4256];
      w = w - phi[3936];
      w = w - phi[5984];
      const double kw = ws[50016] * w;
      out[3936] = fma(kw, y[5984], out[3936]);
      out[5984] = fma(kw, y[3936], out[5984]);
      ws[278720] = fma(kw * y[3936], y[5984], ws[278720]);
    }
    {
      double w = 0.77 * phi[4384];
      w = fma(0.5, phi[6016], w);
      w = fma(0.23, phi[4576], w);
      w = fma(0.23, phi[5920], w);
      w = fma(0.27, phi[5984], w);
      w = w - phi[2656];
      w = w - phi[5984];
      const double kw = ws[50048] * w;
      out[2656] = fma(kw, y[5984], out[2656]);
      out[5984] = fma(kw, y[2656], out[5984]);
      ws[278752] = fma(kw * y[2656], y[5984], ws[278752]);
    }
    {
      double w = 1.0 * phi[4256];
      w = w - phi[3712];
      w = w - phi[5984];
      const double kw = ws[50080] * w;
      out[3712] = fma(kw, y[5984], out[3712]);
      out[5984] = fma(kw, y[3712], out[5984]);
      ws[278784] = fma(kw * y[3712], y[5984], ws[278784]);
    }
    {
      double w = 0.75 * phi[4096];
      w = fma(0.25, phi[6016], w);
      w = fma(0.25, phi[4256], w);
      w = w - phi[2560];
      w = w - phi[5984];
      const double kw = ws[50112] * w;
      out[2560] = fma(kw, y[5984], out[2560]);
      out[5984] = fma(kw, y[2560], out[5984]);
      ws[278816] = fma(kw * y[2560], y[5984], ws[278816]);
    }
    {
      double w = 0.9 * phi[4096];
      w = fma(0.1, phi[6016], w);
      w = fma(0.1, phi[5984], w);
      w = fma(0.1, phi[5856], w);
      w = fma(0.1, phi[3680], w);
      w = w - phi[1728];
      w = w - phi[5984];
      const double kw = ws[50144] * w;
      out[1728] = fma(kw, y[5984], out[1728]);
      out[5984] = fma(kw, y[1728], out[5984]);
      ws[278848] = fma(kw * y[1728], y[5984], ws[278848]);
    }
    {
      double w = 0.44 * phi[6016];
      w = fma(0.44, phi[5888], w);
      w = fma(0.15, phi[5696], w);
      w = fma(0.41, phi[3680], w);
      w = w - phi[5792];
      w = w - phi[5984];
      const double kw = ws[50176] * w;
      out[5792] = fma(kw, y[5984], out[5792]);
      out[5984] = fma(kw, y[5792], out[5984]);
      ws[278880] = fma(kw * y[5792], y[5984], ws[278880]);
    }
    {
      double w = 0.44 * phi[6016];
      w = fma(0.44, phi[5632], w);
      w = fma(0.15, phi[5696], w);
      w = fma(0.41, phi[3680], w);
      w = w - phi[4800];
      w = w - phi[5984];
      const double kw = ws[50208] * w;
      out[4800] = fma(kw, y[5984], out[4800]);
      out[5984] = fma(kw, y[4800], out[5984]);
      ws[278912] = fma(kw * y[4800], y[5984], ws[278912]);
    }
    {
      double w = 0.15 * phi[6016];
      w = fma(0.15, phi[5792], w);
      w = fma(0.15, phi[5856], w);
      w = fma(0.85, phi[5728], w);
      w = w - phi[2848];
      w = w - phi[5984];
      const double kw = ws[50240] * w;
      out[2848] = fma(kw, y[5984], out[2848]);
      out[5984] = fma(kw, y[2848], out[5984]);
      ws[278944] = fma(kw * y[2848], y[5984], ws[278944]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[5152];
      w = w - phi[5984];
      const double kw = ws[50272] * w;
      out[5152] = fma(kw, y[5984], out[5152]);
      out[5984] = fma(kw, y[5152], out[5984]);
      ws[278976] = fma(kw * y[5152], y[5984], ws[278976]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3776];
      w = w - phi[5984];
      const double kw = ws[50304] * w;
      out[3776] = fma(kw, y[5984], out[3776]);
      out[5984] = fma(kw, y[3776], out[5984]);
      ws[279008] = fma(kw * y[3776], y[5984], ws[279008]);
    }
    {
      double w = 1.0 * phi[1792];
      w = w - phi[4672];
      w = w - phi[5984];
      const double kw = ws[50336] * w;
      out[4672] = fma(kw, y[5984], out[4672]);
      out[5984] = fma(kw, y[4672], out[5984]);
      ws[279040] = fma(kw * y[4672], y[5984], ws[279040]);
    }
    {
      double w = 1.0 * phi[1792];
      w = w - phi[3520];
      w = w - phi[5984];
      const double kw = ws[50368] * w;
      out[3520] = fma(kw, y[5984], out[3520]);
      out[5984] = fma(kw, y[3520], out[5984]);
      ws[279072] = fma(kw * y[3520], y[5984], ws[279072]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[2880];
      w = w - phi[5984];
      const double kw = ws[50400] * w;
      out[2880] = fma(kw, y[5984], out[2880]);
      out[5984] = fma(kw, y[2880], out[5984]);
      ws[279104] = fma(kw * y[2880], y[5984], ws[279104]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[2912];
      w = w - phi[5984];
      const double kw = ws[50432] * w;
      out[2912] = fma(kw, y[5984], out[2912]);
      out[5984] = fma(kw, y[2912], out[5984]);
      ws[279136] = fma(kw * y[2912], y[5984], ws[279136]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3648];
      w = w - phi[5984];
      const double kw = ws[50464] * w;
      out[3648] = fma(kw, y[5984], out[3648]);
      out[5984] = fma(kw, y[3648], out[5984]);
      ws[279168] = fma(kw * y[3648], y[5984], ws[279168]);
    }
    {
      double w = 1.0 * phi[2944];
      w = w - phi[3232];
      w = w - phi[5984];
      const double kw = ws[50496] * w;
      out[3232] = fma(kw, y[5984], out[3232]);
      out[5984] = fma(kw, y[3232], out[5984]);
      ws[279200] = fma(kw * y[3232], y[5984], ws[279200]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3040];
      w = w - phi[5984];
      const double kw = ws[50528] * w;
      out[3040] = fma(kw, y[5984], out[3040]);
      out[5984] = fma(kw, y[3040], out[5984]);
      ws[279232] = fma(kw * y[3040], y[5984], ws[279232]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[2976];
      w = w - phi[5984];
      const double kw = ws[50560] * w;
      out[2976] = fma(kw, y[5984], out[2976]);
      out[5984] = fma(kw, y[2976], out[5984]);
      ws[279264] = fma(kw * y[2976], y[5984], ws[279264]);
    }
    {
      double w = 1.0 * phi[5440];
      w = w - phi[4032];
      w = w - phi[5984];
      const double kw = ws[50592] * w;
      out[4032] = fma(kw, y[5984], out[4032]);
      out[5984] = fma(kw, y[4032], out[5984]);
      ws[279296] = fma(kw * y[4032], y[5984], ws[279296]);
    }
    {
      double w = 1.0 * phi[5440];
      w = w - phi[4064];
      w = w - phi[5984];
      const double kw = ws[50624] * w;
      out[4064] = fma(kw, y[5984], out[4064]);
      out[5984] = fma(kw, y[4064], out[5984]);
      ws[279328] = fma(kw * y[4064], y[5984], ws[279328]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3072];
      w = w - phi[5984];
      const double kw = ws[50656] * w;
      out[3072] = fma(kw, y[5984], out[3072]);
      out[5984] = fma(kw, y[3072], out[5984]);
      ws[279360] = fma(kw * y[3072], y[5984], ws[279360]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[5216];
      w = w - phi[5984];
      const double kw = ws[50688] * w;
      out[5216] = fma(kw, y[5984], out[5216]);
      out[5984] = fma(kw, y[5216], out[5984]);
      ws[279392] = fma(kw * y[5216], y[5984], ws[279392]);
    }
    {
      double w = 0.74 * phi[5984];
      w = fma(1.37, phi[5856], w);
      w = fma(0.63, phi[5600], w);
      w = w - phi[5888];
      w = w - phi[5888];
      const double kw = ws[50720] * w;
      out[5888] = fma(kw, y[5888], out[5888]);
      out[5888] = fma(kw, y[5888], out[5888]);
      ws[279424] = fma(kw * y[5888], y[5888], ws[279424]);
    }
}
__device__ __noinline__ void adj_jtv_1_5(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5984];
      w = fma(0.75, phi[5856], w);
      w = fma(0.75, phi[5568], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[1472], w);
      w = w - phi[5632];
      w = w - phi[5888];
      const double kw = ws[50752] * w;
      out[5632] = fma(kw, y[5888], out[5632]);
      out[5888] = fma(kw, y[5632], out[5888]);
      ws[279456] = fma(kw * y[5632], y[5888], ws[279456]);
    }
    {
      double w = 0.894 * phi[5984];
      w = fma(0.08, phi[5888], w);
      w = fma(0.026, phi[5632], w);
      w = fma(0.026, phi[5216], w);
      w = fma(0.827, phi[5856], w);
      w = fma(0.198, phi[5760], w);
      w = fma(0.497, phi[5504], w);
      w = fma(0.05, phi[5376], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[5408];
      w = w - phi[5888];
      const double kw = ws[50784] * w;
      out[5408] = fma(kw, y[5888], out[5408]);
      out[5888] = fma(kw, y[5408], out[5888]);
      ws[279488] = fma(kw * y[5408], y[5888], ws[279488]);
    }
    {
      double w = 0.842 * phi[5984];
      w = fma(0.018, phi[5888], w);
      w = fma(0.14, phi[5632], w);
      w = fma(0.191, phi[5216], w);
      w = fma(0.777, phi[5856], w);
      w = fma(0.251, phi[5760], w);
      w = fma(0.618, phi[5504], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[5120];
      w = w - phi[5888];
      const double kw = ws[50816] * w;
      out[5120] = fma(kw, y[5888], out[5120]);
      out[5888] = fma(kw, y[5120], out[5888]);
      ws[279520] = fma(kw * y[5120], y[5888], ws[279520]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.95, phi[5856], w);
      w = fma(0.15, phi[5760], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[1504], w);
      w = w - phi[3008];
      w = w - phi[5888];
      const double kw = ws[50848] * w;
      out[3008] = fma(kw, y[5888], out[3008]);
      out[5888] = fma(kw, y[3008], out[5888]);
      ws[279552] = fma(kw * y[3008], y[5888], ws[279552]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.5, phi[5856], w);
      w = fma(0.705, phi[5760], w);
      w = fma(0.045, phi[5504], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[3200];
      w = w - phi[5888];
      const double kw = ws[50880] * w;
      out[3200] = fma(kw, y[5888], out[3200]);
      out[5888] = fma(kw, y[3200], out[5888]);
      ws[279584] = fma(kw * y[3200], y[5888], ws[279584]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(0.75, phi[5856], w);
      w = fma(1.28, phi[5760], w);
      w = fma(0.218, phi[5504], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[3328];
      w = w - phi[5888];
      const double kw = ws[50912] * w;
      out[3328] = fma(kw, y[5888], out[3328]);
      out[5888] = fma(kw, y[3328], out[5888]);
      ws[279616] = fma(kw * y[3328], y[5888], ws[279616]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.37, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0, phi[4448], w);
      w = fma(1.0, phi[5376], w);
      w = fma(0.5, phi[4512], w);
      w = fma(0.25, phi[4320], w);
      w = fma(0.25, phi[3584], w);
      w = w - phi[3360];
      w = w - phi[5888];
      const double kw = ws[50944] * w;
      out[3360] = fma(kw, y[5888], out[3360]);
      out[5888] = fma(kw, y[3360], out[5888]);
      ws[279648] = fma(kw * y[3360], y[5888], ws[279648]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.2846, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0854, phi[4448], w);
      w = fma(0.5488, phi[5376], w);
      w = fma(0.3659, phi[5248], w);
      w = fma(0.3659, phi[4512], w);
      w = fma(0.5488, phi[5472], w);
      w = w - phi[3296];
      w = w - phi[5888];
      const double kw = ws[50976] * w;
      out[3296] = fma(kw, y[5888], out[3296]);
      out[5888] = fma(kw, y[3296], out[5888]);
      ws[279680] = fma(kw * y[3296], y[5888], ws[279680]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.3218, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0482, phi[4448], w);
      w = fma(0.7043, phi[5376], w);
      w = fma(0.2475, phi[5248], w);
      w = fma(0.3522, phi[4512], w);
      w = fma(0.5996, phi[4320], w);
      w = w - phi[3104];
      w = w - phi[5888];
      const double kw = ws[51008] * w;
      out[3104] = fma(kw, y[5888], out[3104]);
      out[5888] = fma(kw, y[3104], out[5888]);
      ws[279712] = fma(kw * y[3104], y[5888], ws[279712]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.2846, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0854, phi[4448], w);
      w = fma(0.5488, phi[5376], w);
      w = fma(0.3659, phi[5248], w);
      w = fma(0.4573, phi[4512], w);
      w = fma(0.4573, phi[4320], w);
      w = w - phi[3264];
      w = w - phi[5888];
      const double kw = ws[51040] * w;
      out[3264] = fma(kw, y[5888], out[3264]);
      out[5888] = fma(kw, y[3264], out[5888]);
      ws[279744] = fma(kw * y[3264], y[5888], ws[279744]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.31, phi[5856], w);
      w = fma(0.159, phi[4128], w);
      w = fma(0.25, phi[4736], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = fma(0.023, phi[5760], w);
      w = fma(0.018, phi[5376], w);
      w = fma(0.016, phi[5344], w);
      w = w - phi[4288];
      w = w - phi[5888];
      const double kw = ws[51072] * w;
      out[4288] = fma(kw, y[5888], out[4288]);
      out[5888] = fma(kw, y[4288], out[5888]);
      ws[279776] = fma(kw * y[4288], y[5888], ws[279776]);
    }
    {
      double w = 1.0295 * phi[5856];
      w = fma(0.2205, phi[4576], w);
      w = fma(0.273, phi[4544], w);
      w = fma(0.2385, phi[5760], w);
      w = fma(0.0845, phi[4096], w);
      w = fma(0.1105, phi[5600], w);
      w = fma(0.1835, phi[5504], w);
      w = fma(0.067, phi[4480], w);
      w = fma(1.279, phi[5984], w);
      w = w - phi[4160];
      w = w - phi[5888];
      const double kw = ws[51104] * w;
      out[4160] = fma(kw, y[5888], out[4160]);
      out[5888] = fma(kw, y[4160], out[5888]);
      ws[279808] = fma(kw * y[4160], y[5888], ws[279808]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(0.75, phi[5856], w);
      w = fma(0.25, phi[5600], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3744];
      w = w - phi[5888];
      const double kw = ws[51136] * w;
      out[3744] = fma(kw, y[5888], out[3744]);
      out[5888] = fma(kw, y[3744], out[5888]);
      ws[279840] = fma(kw * y[3744], y[5888], ws[279840]);
    }
    {
      double w = 0.341 * phi[4384];
      w = fma(0.964, phi[5856], w);
      w = fma(0.043, phi[5600], w);
      w = fma(0.918, phi[5984], w);
      w = fma(0.659, phi[5920], w);
      w = fma(0.533, phi[4544], w);
      w = fma(0.007, phi[5504], w);
      w = fma(0.119, phi[5760], w);
      w = w - phi[2624];
      w = w - phi[5888];
      const double kw = ws[51168] * w;
      out[2624] = fma(kw, y[5888], out[2624]);
      out[5888] = fma(kw, y[2624], out[5888]);
      ws[279872] = fma(kw * y[2624], y[5888], ws[279872]);
    }
    {
      double w = 0.75 * phi[5984];
      w = fma(0.75, phi[5920], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.75, phi[5856], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3840];
      w = w - phi[5888];
      const double kw = ws[51200] * w;
      out[3840] = fma(kw, y[5888], out[3840]);
      out[5888] = fma(kw, y[3840], out[5888]);
      ws[279904] = fma(kw * y[3840], y[5888], ws[279904]);
    }
    {
      double w = 0.25 * phi[5600];
      w = fma(1.0, phi[4576], w);
      w = fma(1.03, phi[5856], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[4192];
      w = w - phi[5888];
      const double kw = ws[51232] * w;
      out[4192] = fma(kw, y[5888], out[4192]);
      out[5888] = fma(kw, y[4192], out[5888]);
      ws[279936] = fma(kw * y[4192], y[5888], ws[279936]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(0.75, phi[5856], w);
      w = fma(0.25, phi[5600], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3936];
      w = w - phi[5888];
      const double kw = ws[51264] * w;
      out[3936] = fma(kw, y[5888], out[3936]);
      out[5888] = fma(kw, y[3936], out[5888]);
      ws[279968] = fma(kw * y[3936], y[5888], ws[279968]);
    }
    {
      double w = 0.69 * phi[4384];
      w = fma(0.91, phi[5856], w);
      w = fma(0.09, phi[5600], w);
      w = fma(1.01, phi[5984], w);
      w = fma(0.31, phi[4576], w);
      w = fma(0.31, phi[5920], w);
      w = w - phi[2656];
      w = w - phi[5888];
      const double kw = ws[51296] * w;
      out[2656] = fma(kw, y[5888], out[2656]);
      out[5888] = fma(kw, y[2656], out[5888]);
      ws[280000] = fma(kw * y[2656], y[5888], ws[280000]);
    }
    {
      double w = 0.75 * phi[5984];
      w = fma(0.75, phi[5856], w);
      w = fma(0.75, phi[5920], w);
      w = fma(0.25, phi[5600], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3712];
      w = w - phi[5888];
      const double kw = ws[51328] * w;
      out[3712] = fma(kw, y[5888], out[3712]);
      out[5888] = fma(kw, y[3712], out[5888]);
      ws[280032] = fma(kw * y[3712], y[5888], ws[280032]);
    }
    {
      double w = 0.9 * phi[5984];
      w = fma(0.9, phi[5888], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.1, phi[5696], w);
      w = w - phi[5792];
      w = w - phi[5888];
      const double kw = ws[51360] * w;
      out[5792] = fma(kw, y[5888], out[5792]);
      out[5888] = fma(kw, y[5792], out[5888]);
      ws[280064] = fma(kw * y[5792], y[5888], ws[280064]);
    }
    {
      double w = 0.9 * phi[5984];
      w = fma(0.9, phi[5888], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.1, phi[5696], w);
      w = w - phi[4800];
      w = w - phi[5888];
      const double kw = ws[51392] * w;
      out[4800] = fma(kw, y[5888], out[4800]);
      out[5888] = fma(kw, y[4800], out[5888]);
      ws[280096] = fma(kw * y[4800], y[5888], ws[280096]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5792], w);
      w = fma(1.5, phi[5856], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = fma(0.125, phi[5696], w);
      w = w - phi[2848];
      w = w - phi[5888];
      const double kw = ws[51424] * w;
      out[2848] = fma(kw, y[5888], out[2848]);
      out[5888] = fma(kw, y[2848], out[5888]);
      ws[280128] = fma(kw * y[2848], y[5888], ws[280128]);
    }
    {
      double w = 0.834 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = fma(0.334, phi[5472], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[5152];
      w = w - phi[5888];
      const double kw = ws[51456] * w;
      out[5152] = fma(kw, y[5888], out[5152]);
      out[5888] = fma(kw, y[5152], out[5888]);
      ws[280160] = fma(kw * y[5152], y[5888], ws[280160]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(0.75, phi[5856], w);
      w = fma(0.5, phi[5472], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[3776];
      w = w - phi[5888];
      const double kw = ws[51488] * w;
      out[3776] = fma(kw, y[5888], out[3776]);
      out[5888] = fma(kw, y[3776], out[5888]);
      ws[280192] = fma(kw * y[3776], y[5888], ws[280192]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.269, phi[5792], w);
      w = fma(0.5, phi[5664], w);
      w = fma(1.66, phi[5856], w);
      w = fma(0.067, phi[5696], w);
      w = fma(0.25, phi[5888], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[4672];
      w = w - phi[5888];
      const double kw = ws[51520] * w;
      out[4672] = fma(kw, y[5888], out[4672]);
      out[5888] = fma(kw, y[4672], out[5888]);
      ws[280224] = fma(kw * y[4672], y[5888], ws[280224]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.5, phi[5856], w);
      w = fma(0.5, phi[5344], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[3520];
      w = w - phi[5888];
      const double kw = ws[51552] * w;
      out[3520] = fma(kw, y[5888], out[3520]);
      out[5888] = fma(kw, y[3520], out[5888]);
      ws[280256] = fma(kw * y[3520], y[5888], ws[280256]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.16, phi[5792], w);
      w = fma(1.16, phi[5216], w);
      w = fma(1.5, phi[5856], w);
      w = fma(1.75, phi[5760], w);
      w = fma(0.5, phi[5248], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = fma(0.292, phi[5696], w);
      w = w - phi[2880];
      w = w - phi[5888];
      const double kw = ws[51584] * w;
      out[2880] = fma(kw, y[5888], out[2880]);
      out[5888] = fma(kw, y[2880], out[5888]);
      ws[280288] = fma(kw * y[2880], y[5888], ws[280288]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(0.305, phi[5664], w);
      w = fma(0.773, phi[5856], w);
      w = fma(0.203, phi[5760], w);
      w = fma(0.525, phi[5504], w);
      w = fma(0.135, phi[5376], w);
      w = fma(0.105, phi[5248], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = w - phi[2912];
      w = w - phi[5888];
      const double kw = ws[51616] * w;
      out[2912] = fma(kw, y[5888], out[2912]);
      out[5888] = fma(kw, y[2912], out[5888]);
      ws[280320] = fma(kw * y[2912], y[5888], ws[280320]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[2272], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[2592];
      w = w - phi[5888];
      const double kw = ws[51648] * w;
      out[2592] = fma(kw, y[5888], out[2592]);
      out[5888] = fma(kw, y[2592], out[5888]);
      ws[280352] = fma(kw * y[2592], y[5888], ws[280352]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[2688], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[2272];
      w = w - phi[5888];
      const double kw = ws[51680] * w;
      out[2272] = fma(kw, y[5888], out[2272]);
      out[5888] = fma(kw, y[2272], out[5888]);
      ws[280384] = fma(kw * y[2272], y[5888], ws[280384]);
    }
    {
      double w = 2.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = fma(0.32, phi[5344], w);
      w = fma(0.68, phi[5376], w);
      w = fma(0.68, phi[5728], w);
      w = w - phi[3648];
      w = w - phi[5888];
      const double kw = ws[51712] * w;
      out[3648] = fma(kw, y[5888], out[3648]);
      out[5888] = fma(kw, y[3648], out[5888]);
      ws[280416] = fma(kw * y[3648], y[5888], ws[280416]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[3808], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[3040];
      w = w - phi[5888];
      const double kw = ws[51744] * w;
      out[3040] = fma(kw, y[5888], out[3040]);
      out[5888] = fma(kw, y[3040], out[5888]);
      ws[280448] = fma(kw * y[3040], y[5888], ws[280448]);
    }
    {
      double w = 1.0 * phi[5856];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5376], w);
      w = w - phi[2976];
      w = w - phi[5888];
      const double kw = ws[51776] * w;
      out[2976] = fma(kw, y[5888], out[2976]);
      out[5888] = fma(kw, y[2976], out[5888]);
      ws[280480] = fma(kw * y[2976], y[5888], ws[280480]);
    }
    {
      double w = 2.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[5440], w);
      w = w - phi[4032];
      w = w - phi[5888];
      const double kw = ws[51808] * w;
      out[4032] = fma(kw, y[5888], out[4032]);
      out[5888] = fma(kw, y[4032], out[5888]);
      ws[280512] = fma(kw * y[4032], y[5888], ws[280512]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5920], w);
      w = fma(0.965, phi[5856], w);
      w = fma(0.93, phi[5760], w);
      w = fma(0.348, phi[5504], w);
      w = fma(0.25, phi[5600], w);
      w = fma(0.25, phi[5056], w);
      w = fma(0.5, phi[5440], w);
      w = w - phi[4064];
      w = w - phi[5888];
      const double kw = ws[51840] * w;
      out[4064] = fma(kw, y[5888], out[4064]);
      out[5888] = fma(kw, y[4064], out[5888]);
      ws[280544] = fma(kw * y[4064], y[5888], ws[280544]);
    }
}
__device__ __noinline__ void adj_jtv_1_6(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5984];
      w = fma(0.7, phi[5920], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.7, phi[5376], w);
      w = fma(0.7, phi[5728], w);
      w = fma(0.3, phi[5440], w);
      w = w - phi[3072];
      w = w - phi[5888];
      const double kw = ws[51872] * w;
      out[3072] = fma(kw, y[5888], out[3072]);
      out[5888] = fma(kw, y[3072], out[5888]);
      ws[280576] = fma(kw * y[3072], y[5888], ws[280576]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = w - phi[5216];
      w = w - phi[5888];
      const double kw = ws[51904] * w;
      out[5216] = fma(kw, y[5888], out[5216]);
      out[5888] = fma(kw, y[5216], out[5888]);
      ws[280608] = fma(kw * y[5216], y[5888], ws[280608]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(1.0, phi[5568], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[5632];
      w = w - phi[5792];
      const double kw = ws[51936] * w;
      out[5632] = fma(kw, y[5792], out[5632]);
      out[5792] = fma(kw, y[5632], out[5792]);
      ws[280640] = fma(kw * y[5632], y[5792], ws[280640]);
    }
    {
      double w = 0.394 * phi[5984];
      w = fma(0.58, phi[5888], w);
      w = fma(0.026, phi[5632], w);
      w = fma(0.026, phi[5216], w);
      w = fma(0.13, phi[5856], w);
      w = fma(0.273, phi[5760], w);
      w = fma(0.662, phi[5504], w);
      w = fma(0.067, phi[5376], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[5408];
      w = w - phi[5792];
      const double kw = ws[51968] * w;
      out[5408] = fma(kw, y[5792], out[5408]);
      out[5792] = fma(kw, y[5408], out[5792]);
      ws[280672] = fma(kw * y[5408], y[5792], ws[280672]);
    }
    {
      double w = 0.342 * phi[5984];
      w = fma(0.518, phi[5888], w);
      w = fma(0.14, phi[5632], w);
      w = fma(0.191, phi[5216], w);
      w = fma(0.042, phi[5856], w);
      w = fma(0.381, phi[5760], w);
      w = fma(0.824, phi[5504], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[5120];
      w = w - phi[5792];
      const double kw = ws[52000] * w;
      out[5120] = fma(kw, y[5792], out[5120]);
      out[5792] = fma(kw, y[5120], out[5792]);
      ws[280704] = fma(kw * y[5120], y[5792], ws[280704]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(1.6, phi[5856], w);
      w = fma(0.2, phi[5760], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[3008];
      w = w - phi[5792];
      const double kw = ws[52032] * w;
      out[3008] = fma(kw, y[5792], out[3008]);
      out[5792] = fma(kw, y[3008], out[5792]);
      ws[280736] = fma(kw * y[3008], y[5792], ws[280736]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.94, phi[5760], w);
      w = fma(0.06, phi[5504], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[3200];
      w = w - phi[5792];
      const double kw = ws[52064] * w;
      out[3200] = fma(kw, y[5792], out[3200]);
      out[5792] = fma(kw, y[3200], out[5792]);
      ws[280768] = fma(kw * y[3200], y[5792], ws[280768]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(1.71, phi[5760], w);
      w = fma(0.29, phi[5504], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[3328];
      w = w - phi[5792];
      const double kw = ws[52096] * w;
      out[3328] = fma(kw, y[5792], out[3328]);
      out[5792] = fma(kw, y[3328], out[5792]);
      ws[280800] = fma(kw * y[3328], y[5792], ws[280800]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(1.0, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0, phi[4448], w);
      w = fma(1.0, phi[5376], w);
      w = fma(0.5, phi[4512], w);
      w = fma(0.25, phi[4320], w);
      w = fma(0.25, phi[3584], w);
      w = w - phi[3360];
      w = w - phi[5792];
      const double kw = ws[52128] * w;
      out[3360] = fma(kw, y[5792], out[3360]);
      out[5792] = fma(kw, y[3360], out[5792]);
      ws[280832] = fma(kw * y[3360], y[5792], ws[280832]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.9146, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0854, phi[4448], w);
      w = fma(0.5488, phi[5376], w);
      w = fma(0.3659, phi[5248], w);
      w = fma(0.3659, phi[4512], w);
      w = fma(0.5488, phi[5472], w);
      w = w - phi[3296];
      w = w - phi[5792];
      const double kw = ws[52160] * w;
      out[3296] = fma(kw, y[5792], out[3296]);
      out[5792] = fma(kw, y[3296], out[5792]);
      ws[280864] = fma(kw * y[3296], y[5792], ws[280864]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.9518, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0482, phi[4448], w);
      w = fma(0.7043, phi[5376], w);
      w = fma(0.2475, phi[5248], w);
      w = fma(0.3522, phi[4512], w);
      w = fma(0.5996, phi[4320], w);
      w = w - phi[3104];
      w = w - phi[5792];
      const double kw = ws[52192] * w;
      out[3104] = fma(kw, y[5792], out[3104]);
      out[5792] = fma(kw, y[3104], out[5792]);
      ws[280896] = fma(kw * y[3104], y[5792], ws[280896]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.9146, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0854, phi[4448], w);
      w = fma(0.5488, phi[5376], w);
      w = fma(0.3659, phi[5248], w);
      w = fma(0.4573, phi[4512], w);
      w = fma(0.4573, phi[4320], w);
      w = w - phi[3264];
      w = w - phi[5792];
      const double kw = ws[52224] * w;
      out[3264] = fma(kw, y[5792], out[3264]);
      out[5792] = fma(kw, y[3264], out[5792]);
      ws[280928] = fma(kw * y[3264], y[5792], ws[280928]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(1.048, phi[5856], w);
      w = fma(0.219, phi[4128], w);
      w = fma(0.305, phi[4736], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[4288];
      w = w - phi[5792];
      const double kw = ws[52256] * w;
      out[4288] = fma(kw, y[5792], out[4288]);
      out[5792] = fma(kw, y[4288], out[5792]);
      ws[280960] = fma(kw * y[4288], y[5792], ws[280960]);
    }
    {
      double w = 0.2535 * phi[4544];
      w = fma(0.371, phi[5760], w);
      w = fma(0.091, phi[4096], w);
      w = fma(0.1165, phi[4480], w);
      w = fma(0.1725, phi[4576], w);
      w = fma(0.403, phi[5856], w);
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5888], w);
      w = fma(0.112, phi[5504], w);
      w = w - phi[4160];
      w = w - phi[5792];
      const double kw = ws[52288] * w;
      out[4160] = fma(kw, y[5792], out[4160]);
      out[5792] = fma(kw, y[4160], out[5792]);
      ws[280992] = fma(kw * y[4160], y[5792], ws[280992]);
    }
    {
      double w = 0.5 * phi[6016];
      w = fma(0.5, phi[5888], w);
      w = fma(0.5, phi[5696], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3744];
      w = w - phi[5792];
      const double kw = ws[52320] * w;
      out[3744] = fma(kw, y[5792], out[3744]);
      out[5792] = fma(kw, y[3744], out[5792]);
      ws[281024] = fma(kw * y[3744], y[5792], ws[281024]);
    }
    {
      double w = 0.825 * phi[5920];
      w = fma(0.65, phi[4544], w);
      w = fma(1.0, phi[5888], w);
      w = fma(0.175, phi[4384], w);
      w = fma(0.168, phi[5760], w);
      w = fma(0.007, phi[5504], w);
      w = fma(0.007, phi[5856], w);
      w = fma(0.175, phi[5984], w);
      w = w - phi[2624];
      w = w - phi[5792];
      const double kw = ws[52352] * w;
      out[2624] = fma(kw, y[5792], out[2624]);
      out[5792] = fma(kw, y[2624], out[5792]);
      ws[281056] = fma(kw * y[2624], y[5792], ws[281056]);
    }
    {
      double w = 0.5 * phi[5920];
      w = fma(0.5, phi[5888], w);
      w = fma(0.5, phi[5696], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3840];
      w = w - phi[5792];
      const double kw = ws[52384] * w;
      out[3840] = fma(kw, y[5792], out[3840]);
      out[5792] = fma(kw, y[3840], out[5792]);
      ws[281088] = fma(kw * y[3840], y[5792], ws[281088]);
    }
    {
      double w = 1.0 * phi[4576];
      w = fma(0.56, phi[5856], w);
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5888], w);
      w = w - phi[4192];
      w = w - phi[5792];
      const double kw = ws[52416] * w;
      out[4192] = fma(kw, y[5792], out[4192]);
      out[5792] = fma(kw, y[4192], out[5792]);
      ws[281120] = fma(kw * y[4192], y[5792], ws[281120]);
    }
    {
      double w = 0.5 * phi[6016];
      w = fma(0.5, phi[5888], w);
      w = fma(0.5, phi[5696], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3936];
      w = w - phi[5792];
      const double kw = ws[52448] * w;
      out[3936] = fma(kw, y[5792], out[3936]);
      out[5792] = fma(kw, y[3936], out[5792]);
      ws[281152] = fma(kw * y[3936], y[5792], ws[281152]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(0.46, phi[5920], w);
      w = fma(0.46, phi[4576], w);
      w = fma(0.54, phi[4384], w);
      w = fma(0.54, phi[5984], w);
      w = w - phi[2656];
      w = w - phi[5792];
      const double kw = ws[52480] * w;
      out[2656] = fma(kw, y[5792], out[2656]);
      out[5792] = fma(kw, y[2656], out[5792]);
      ws[281184] = fma(kw * y[2656], y[5792], ws[281184]);
    }
    {
      double w = 0.5 * phi[5888];
      w = fma(0.5, phi[5920], w);
      w = fma(0.5, phi[5696], w);
      w = fma(1.0, phi[4256], w);
      w = w - phi[3712];
      w = w - phi[5792];
      const double kw = ws[52512] * w;
      out[3712] = fma(kw, y[5792], out[3712]);
      out[5792] = fma(kw, y[3712], out[5792]);
      ws[281216] = fma(kw * y[3712], y[5792], ws[281216]);
    }
    {
      double w = 2.0 * phi[5888];
      w = w - phi[5792];
      w = w - phi[5792];
      const double kw = ws[52544] * w;
      out[5792] = fma(kw, y[5792], out[5792]);
      out[5792] = fma(kw, y[5792], out[5792]);
      ws[281248] = fma(kw * y[5792], y[5792], ws[281248]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[5632], w);
      w = w - phi[4800];
      w = w - phi[5792];
      const double kw = ws[52576] * w;
      out[4800] = fma(kw, y[5792], out[4800]);
      out[5792] = fma(kw, y[4800], out[5792]);
      ws[281280] = fma(kw * y[4800], y[5792], ws[281280]);
    }
    {
      double w = 0.5 * phi[5888];
      w = fma(0.5, phi[5792], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.75, phi[5696], w);
      w = w - phi[2848];
      w = w - phi[5792];
      const double kw = ws[52608] * w;
      out[2848] = fma(kw, y[5792], out[2848]);
      out[5792] = fma(kw, y[2848], out[5792]);
      ws[281312] = fma(kw * y[2848], y[5792], ws[281312]);
    }
    {
      double w = 0.33 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(0.33, phi[5856], w);
      w = fma(0.334, phi[5472], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[5152];
      w = w - phi[5792];
      const double kw = ws[52640] * w;
      out[5152] = fma(kw, y[5792], out[5152]);
      out[5792] = fma(kw, y[5152], out[5792]);
      ws[281344] = fma(kw * y[5152], y[5792], ws[281344]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(0.5, phi[5472], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[3776];
      w = w - phi[5792];
      const double kw = ws[52672] * w;
      out[3776] = fma(kw, y[5792], out[3776]);
      out[5792] = fma(kw, y[3776], out[5792]);
      ws[281376] = fma(kw * y[3776], y[5792], ws[281376]);
    }
    {
      double w = 0.635 * phi[5696];
      w = fma(0.5, phi[5888], w);
      w = fma(0.269, phi[5792], w);
      w = fma(0.5, phi[5664], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[4672];
      w = w - phi[5792];
      const double kw = ws[52704] * w;
      out[4672] = fma(kw, y[5792], out[4672]);
      out[5792] = fma(kw, y[4672], out[5792]);
      ws[281408] = fma(kw * y[4672], y[5792], ws[281408]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.5, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.5, phi[5344], w);
      w = fma(0.5, phi[5888], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[3520];
      w = w - phi[5792];
      const double kw = ws[52736] * w;
      out[3520] = fma(kw, y[5792], out[3520]);
      out[5792] = fma(kw, y[3520], out[5792]);
      ws[281440] = fma(kw * y[3520], y[5792], ws[281440]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(1.16, phi[5792], w);
      w = fma(1.16, phi[5216], w);
      w = fma(1.0, phi[5856], w);
      w = fma(2.3, phi[5760], w);
      w = fma(0.5, phi[5248], w);
      w = fma(1.083, phi[5696], w);
      w = w - phi[2880];
      w = w - phi[5792];
      const double kw = ws[52768] * w;
      out[2880] = fma(kw, y[5792], out[2880]);
      out[5792] = fma(kw, y[2880], out[5792]);
      ws[281472] = fma(kw * y[2880], y[5792], ws[281472]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5888], w);
      w = fma(0.5, phi[5664], w);
      w = fma(0.03, phi[5856], w);
      w = fma(0.27, phi[5760], w);
      w = fma(0.7, phi[5504], w);
      w = fma(0.18, phi[5376], w);
      w = fma(0.105, phi[5248], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[2912];
      w = w - phi[5792];
      const double kw = ws[52800] * w;
      out[2912] = fma(kw, y[5792], out[2912]);
      out[5792] = fma(kw, y[2912], out[5792]);
      ws[281504] = fma(kw * y[2912], y[5792], ws[281504]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[2272], w);
      w = w - phi[2592];
      w = w - phi[5792];
      const double kw = ws[52832] * w;
      out[2592] = fma(kw, y[5792], out[2592]);
      out[5792] = fma(kw, y[2592], out[5792]);
      ws[281536] = fma(kw * y[2592], y[5792], ws[281536]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[2688], w);
      w = w - phi[2272];
      w = w - phi[5792];
      const double kw = ws[52864] * w;
      out[2272] = fma(kw, y[5792], out[2272]);
      out[5792] = fma(kw, y[2272], out[5792]);
      ws[281568] = fma(kw * y[2272], y[5792], ws[281568]);
    }
    {
      double w = 2.0 * phi[5984];
      w = fma(1.0, phi[5888], w);
      w = fma(0.32, phi[5344], w);
      w = fma(0.68, phi[5376], w);
      w = fma(0.68, phi[5728], w);
      w = w - phi[3648];
      w = w - phi[5792];
      const double kw = ws[52896] * w;
      out[3648] = fma(kw, y[5792], out[3648]);
      out[5792] = fma(kw, y[3648], out[5792]);
      ws[281600] = fma(kw * y[3648], y[5792], ws[281600]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5888], w);
      w = fma(1.0, phi[3808], w);
      w = w - phi[3040];
      w = w - phi[5792];
      const double kw = ws[52928] * w;
      out[3040] = fma(kw, y[5792], out[3040]);
      out[5792] = fma(kw, y[3040], out[5792]);
      ws[281632] = fma(kw * y[3040], y[5792], ws[281632]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[5376], w);
      w = w - phi[2976];
      w = w - phi[5792];
      const double kw = ws[52960] * w;
      out[2976] = fma(kw, y[5792], out[2976]);
      out[5792] = fma(kw, y[2976], out[5792]);
      ws[281664] = fma(kw * y[2976], y[5792], ws[281664]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5888], w);
      w = fma(1.0, phi[5440], w);
      w = w - phi[4032];
      w = w - phi[5792];
      const double kw = ws[52992] * w;
      out[4032] = fma(kw, y[5792], out[4032]);
      out[5792] = fma(kw, y[4032], out[5792]);
      ws[281696] = fma(kw * y[4032], y[5792], ws[281696]);
    }
    {
      double w = 0.5 * phi[5888];
      w = fma(1.0, phi[5920], w);
      w = fma(0.287, phi[5856], w);
      w = fma(1.24, phi[5760], w);
      w = fma(0.464, phi[5504], w);
      w = fma(0.5, phi[5696], w);
      w = w - phi[4064];
      w = w - phi[5792];
      const double kw = ws[53024] * w;
      out[4064] = fma(kw, y[5792], out[4064]);
      out[5792] = fma(kw, y[4064], out[5792]);
      ws[281728] = fma(kw * y[4064], y[5792], ws[281728]);
    }
}
__device__ __noinline__ void adj_jtv_1_7(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5888], w);
      w = fma(0.7, phi[5920], w);
      w = fma(0.7, phi[5376], w);
      w = fma(0.7, phi[5728], w);
      w = fma(0.3, phi[5440], w);
      w = w - phi[3072];
      w = w - phi[5792];
      const double kw = ws[53056] * w;
      out[3072] = fma(kw, y[5792], out[3072]);
      out[5792] = fma(kw, y[3072], out[5792]);
      ws[281760] = fma(kw * y[3072], y[5792], ws[281760]);
    }
    {
      double w = 1.0 * phi[5888];
      w = w - phi[5216];
      w = w - phi[5792];
      const double kw = ws[53088] * w;
      out[5216] = fma(kw, y[5792], out[5216]);
      out[5792] = fma(kw, y[5216], out[5792]);
      ws[281792] = fma(kw * y[5216], y[5792], ws[281792]);
    }
    {
      double w = 2.0 * phi[5632];
      w = w - phi[4800];
      w = w - phi[4800];
      const double kw = ws[53120] * w;
      out[4800] = fma(kw, y[4800], out[4800]);
      out[4800] = fma(kw, y[4800], out[4800]);
      ws[281824] = fma(kw * y[4800], y[4800], ws[281824]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[5920], w);
      w = w - phi[5888];
      w = w - phi[5952];
      const double kw = ws[53152] * w;
      out[5888] = fma(kw, y[5952], out[5888]);
      out[5952] = fma(kw, y[5888], out[5952]);
      ws[281856] = fma(kw * y[5888], y[5952], ws[281856]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[5568], w);
      w = w - phi[5632];
      w = w - phi[5952];
      const double kw = ws[53184] * w;
      out[5632] = fma(kw, y[5952], out[5632]);
      out[5952] = fma(kw, y[5632], out[5952]);
      ws[281888] = fma(kw * y[5632], y[5952], ws[281888]);
    }
    {
      double w = 0.254 * phi[5984];
      w = fma(0.14, phi[5888], w);
      w = fma(0.092, phi[5216], w);
      w = fma(0.503, phi[5632], w);
      w = fma(1.0, phi[5920], w);
      w = fma(0.519, phi[5568], w);
      w = fma(0.147, phi[5760], w);
      w = fma(0.075, phi[5280], w);
      w = fma(0.095, phi[4480], w);
      w = w - phi[5408];
      w = w - phi[5952];
      const double kw = ws[53216] * w;
      out[5408] = fma(kw, y[5952], out[5408]);
      out[5952] = fma(kw, y[5408], out[5952]);
      ws[281920] = fma(kw * y[5408], y[5952], ws[281920]);
    }
    {
      double w = 0.488 * phi[5984];
      w = fma(0.055, phi[5888], w);
      w = fma(0.28, phi[5632], w);
      w = fma(0.485, phi[5216], w);
      w = fma(1.0, phi[5920], w);
      w = fma(0.024, phi[5856], w);
      w = fma(0.241, phi[5760], w);
      w = fma(0.06, phi[5504], w);
      w = fma(0.063, phi[5280], w);
      w = fma(0.247, phi[4480], w);
      w = fma(0.048, phi[5568], w);
      w = fma(0.275, phi[5344], w);
      w = w - phi[5120];
      w = w - phi[5952];
      const double kw = ws[53248] * w;
      out[5120] = fma(kw, y[5952], out[5120]);
      out[5952] = fma(kw, y[5120], out[5952]);
      ws[281952] = fma(kw * y[5120], y[5952], ws[281952]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.6, phi[5856], w);
      w = fma(0.2, phi[5760], w);
      w = w - phi[3008];
      w = w - phi[5952];
      const double kw = ws[53280] * w;
      out[3008] = fma(kw, y[5952], out[3008]);
      out[5952] = fma(kw, y[3008], out[5952]);
      ws[281984] = fma(kw * y[3008], y[5952], ws[281984]);
    }
    {
      double w = 0.47 * phi[5760];
      w = fma(0.79, phi[5856], w);
      w = fma(0.79, phi[5984], w);
      w = fma(1.0, phi[5920], w);
      w = fma(0.18, phi[5280], w);
      w = fma(0.02, phi[5568], w);
      w = fma(0.09, phi[4480], w);
      w = w - phi[3200];
      w = w - phi[5952];
      const double kw = ws[53312] * w;
      out[3200] = fma(kw, y[5952], out[3200]);
      out[5952] = fma(kw, y[3200], out[5952]);
      ws[282016] = fma(kw * y[3200], y[5952], ws[282016]);
    }
    {
      double w = 0.86 * phi[5984];
      w = fma(0.72, phi[5760], w);
      w = fma(0.11, phi[5504], w);
      w = fma(1.0, phi[5920], w);
      w = fma(0.2, phi[4480], w);
      w = fma(0.85, phi[5568], w);
      w = fma(0.04, phi[5344], w);
      w = w - phi[3328];
      w = w - phi[5952];
      const double kw = ws[53344] * w;
      out[3328] = fma(kw, y[5952], out[3328]);
      out[5952] = fma(kw, y[3328], out[5952]);
      ws[282048] = fma(kw * y[3328], y[5952], ws[282048]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(0.0, phi[4448], w);
      w = fma(1.0, phi[5376], w);
      w = fma(0.5, phi[4512], w);
      w = fma(0.25, phi[4320], w);
      w = fma(0.25, phi[3584], w);
      w = w - phi[3360];
      w = w - phi[5952];
      const double kw = ws[53376] * w;
      out[3360] = fma(kw, y[5952], out[3360]);
      out[5952] = fma(kw, y[3360], out[5952]);
      ws[282080] = fma(kw * y[3360], y[5952], ws[282080]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.9146, phi[5984], w);
      w = fma(0.0854, phi[4448], w);
      w = fma(0.5488, phi[5376], w);
      w = fma(0.3659, phi[5248], w);
      w = fma(0.3659, phi[4512], w);
      w = fma(0.5488, phi[5472], w);
      w = w - phi[3296];
      w = w - phi[5952];
      const double kw = ws[53408] * w;
      out[3296] = fma(kw, y[5952], out[3296]);
      out[5952] = fma(kw, y[3296], out[5952]);
      ws[282112] = fma(kw * y[3296], y[5952], ws[282112]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.9518, phi[5984], w);
      w = fma(0.0482, phi[4448], w);
      w = fma(0.7043, phi[5376], w);
      w = fma(0.2475, phi[5248], w);
      w = fma(0.3522, phi[4512], w);
      w = fma(0.5996, phi[4320], w);
      w = w - phi[3104];
      w = w - phi[5952];
      const double kw = ws[53440] * w;
      out[3104] = fma(kw, y[5952], out[3104]);
      out[5952] = fma(kw, y[3104], out[5952]);
      ws[282144] = fma(kw * y[3104], y[5952], ws[282144]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.9146, phi[5984], w);
      w = fma(0.0854, phi[4448], w);
      w = fma(0.5488, phi[5376], w);
      w = fma(0.3659, phi[5248], w);
      w = fma(0.4573, phi[4512], w);
      w = fma(0.4573, phi[4320], w);
      w = w - phi[3264];
      w = w - phi[5952];
      const double kw = ws[53472] * w;
      out[3264] = fma(kw, y[5952], out[3264]);
      out[5952] = fma(kw, y[3264], out[5952]);
      ws[282176] = fma(kw * y[3264], y[5952], ws[282176]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.75, phi[5856], w);
      w = fma(0.318, phi[4128], w);
      w = fma(0.5, phi[4736], w);
      w = fma(0.024, phi[5376], w);
      w = fma(0.033, phi[5344], w);
      w = fma(0.031, phi[5760], w);
      w = w - phi[4288];
      w = w - phi[5952];
      const double kw = ws[53504] * w;
      out[4288] = fma(kw, y[5952], out[4288]);
      out[5952] = fma(kw, y[4288], out[5952]);
      ws[282208] = fma(kw * y[4288], y[5952], ws[282208]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(0.2535, phi[4544], w);
      w = fma(0.371, phi[5760], w);
      w = fma(0.1165, phi[4480], w);
      w = fma(0.1725, phi[4576], w);
      w = fma(0.403, phi[5856], w);
      w = fma(0.091, phi[4096], w);
      w = fma(0.112, phi[5504], w);
      w = w - phi[4160];
      w = w - phi[5952];
      const double kw = ws[53536] * w;
      out[4160] = fma(kw, y[5952], out[4160]);
      out[5952] = fma(kw, y[4160], out[5952]);
      ws[282240] = fma(kw * y[4160], y[5952], ws[282240]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[4576], w);
      w = fma(0.56, phi[5856], w);
      w = w - phi[4192];
      w = w - phi[5952];
      const double kw = ws[53568] * w;
      out[4192] = fma(kw, y[5952], out[4192]);
      out[5952] = fma(kw, y[4192], out[5952]);
      ws[282272] = fma(kw * y[4192], y[5952], ws[282272]);
    }
    {
      double w = 1.825 * phi[5920];
      w = fma(0.65, phi[4544], w);
      w = fma(0.175, phi[4384], w);
      w = fma(0.168, phi[5760], w);
      w = fma(0.007, phi[5504], w);
      w = fma(0.007, phi[5856], w);
      w = fma(0.175, phi[5984], w);
      w = w - phi[2624];
      w = w - phi[5952];
      const double kw = ws[53600] * w;
      out[2624] = fma(kw, y[5952], out[2624]);
      out[5952] = fma(kw, y[2624], out[5952]);
      ws[282304] = fma(kw * y[2624], y[5952], ws[282304]);
    }
    {
      double w = 1.46 * phi[5920];
      w = fma(0.46, phi[4576], w);
      w = fma(0.54, phi[4384], w);
      w = fma(0.54, phi[5984], w);
      w = w - phi[2656];
      w = w - phi[5952];
      const double kw = ws[53632] * w;
      out[2656] = fma(kw, y[5952], out[2656]);
      out[5952] = fma(kw, y[2656], out[5952]);
      ws[282336] = fma(kw * y[2656], y[5952], ws[282336]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[5920], w);
      w = w - phi[5792];
      w = w - phi[5952];
      const double kw = ws[53664] * w;
      out[5792] = fma(kw, y[5952], out[5792]);
      out[5952] = fma(kw, y[5792], out[5952]);
      ws[282368] = fma(kw * y[5792], y[5952], ws[282368]);
    }
    {
      double w = 1.0 * phi[5632];
      w = fma(1.0, phi[5920], w);
      w = w - phi[4800];
      w = w - phi[5952];
      const double kw = ws[53696] * w;
      out[4800] = fma(kw, y[5952], out[4800]);
      out[5952] = fma(kw, y[4800], out[5952]);
      ws[282400] = fma(kw * y[4800], y[5952], ws[282400]);
    }
    {
      double w = 1.0 * phi[5792];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[2848];
      w = w - phi[5952];
      const double kw = ws[53728] * w;
      out[2848] = fma(kw, y[5952], out[2848]);
      out[5952] = fma(kw, y[2848], out[5952]);
      ws[282432] = fma(kw * y[2848], y[5952], ws[282432]);
    }
    {
      double w = 0.67 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.33, phi[5856], w);
      w = fma(0.67, phi[5472], w);
      w = w - phi[5152];
      w = w - phi[5952];
      const double kw = ws[53760] * w;
      out[5152] = fma(kw, y[5952], out[5152]);
      out[5952] = fma(kw, y[5152], out[5952]);
      ws[282464] = fma(kw * y[5152], y[5952], ws[282464]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[5472], w);
      w = w - phi[3776];
      w = w - phi[5952];
      const double kw = ws[53792] * w;
      out[3776] = fma(kw, y[5952], out[3776]);
      out[5952] = fma(kw, y[3776], out[5952]);
      ws[282496] = fma(kw * y[3776], y[5952], ws[282496]);
    }
    {
      double w = 1.0 * phi[5856];
      w = fma(0.538, phi[5792], w);
      w = fma(1.0, phi[5664], w);
      w = fma(1.0, phi[5920], w);
      w = w - phi[4672];
      w = w - phi[5952];
      const double kw = ws[53824] * w;
      out[4672] = fma(kw, y[5952], out[4672]);
      out[5952] = fma(kw, y[4672], out[5952]);
      ws[282528] = fma(kw * y[4672], y[5952], ws[282528]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[5344], w);
      w = w - phi[3520];
      w = w - phi[5952];
      const double kw = ws[53856] * w;
      out[3520] = fma(kw, y[5952], out[3520]);
      out[5952] = fma(kw, y[3520], out[5952]);
      ws[282560] = fma(kw * y[3520], y[5952], ws[282560]);
    }
    {
      double w = 0.3 * phi[5984];
      w = fma(0.7, phi[5792], w);
      w = fma(0.7, phi[5216], w);
      w = fma(1.0, phi[5920], w);
      w = fma(0.3, phi[5856], w);
      w = fma(0.7, phi[5760], w);
      w = fma(0.3, phi[5248], w);
      w = w - phi[2880];
      w = w - phi[5952];
      const double kw = ws[53888] * w;
      out[2880] = fma(kw, y[5952], out[2880]);
      out[5952] = fma(kw, y[2880], out[5952]);
      ws[282592] = fma(kw * y[2880], y[5952], ws[282592]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.61, phi[5664], w);
      w = fma(0.03, phi[5856], w);
      w = fma(0.27, phi[5760], w);
      w = fma(0.7, phi[5504], w);
      w = fma(0.18, phi[5376], w);
      w = fma(0.21, phi[5248], w);
      w = w - phi[2912];
      w = w - phi[5952];
      const double kw = ws[53920] * w;
      out[2912] = fma(kw, y[5952], out[2912]);
      out[5952] = fma(kw, y[2912], out[5952]);
      ws[282624] = fma(kw * y[2912], y[5952], ws[282624]);
    }
    {
      double w = 1.0 * phi[2272];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2592];
      w = w - phi[5952];
      const double kw = ws[53952] * w;
      out[2592] = fma(kw, y[5952], out[2592]);
      out[5952] = fma(kw, y[2592], out[5952]);
      ws[282656] = fma(kw * y[2592], y[5952], ws[282656]);
    }
    {
      double w = 1.0 * phi[2688];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2272];
      w = w - phi[5952];
      const double kw = ws[53984] * w;
      out[2272] = fma(kw, y[5952], out[2272]);
      out[5952] = fma(kw, y[2272], out[5952]);
      ws[282688] = fma(kw * y[2272], y[5952], ws[282688]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.32, phi[5344], w);
      w = fma(0.68, phi[5376], w);
      w = fma(0.68, phi[5728], w);
      w = w - phi[3648];
      w = w - phi[5952];
      const double kw = ws[54016] * w;
      out[3648] = fma(kw, y[5952], out[3648]);
      out[5952] = fma(kw, y[3648], out[5952]);
      ws[282720] = fma(kw * y[3648], y[5952], ws[282720]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[3808], w);
      w = w - phi[3040];
      w = w - phi[5952];
      const double kw = ws[54048] * w;
      out[3040] = fma(kw, y[5952], out[3040]);
      out[5952] = fma(kw, y[3040], out[5952]);
      ws[282752] = fma(kw * y[3040], y[5952], ws[282752]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5376], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2976];
      w = w - phi[5952];
      const double kw = ws[54080] * w;
      out[2976] = fma(kw, y[5952], out[2976]);
      out[5952] = fma(kw, y[2976], out[5952]);
      ws[282784] = fma(kw * y[2976], y[5952], ws[282784]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[5440], w);
      w = w - phi[4032];
      w = w - phi[5952];
      const double kw = ws[54112] * w;
      out[4032] = fma(kw, y[5952], out[4032]);
      out[5952] = fma(kw, y[4032], out[5952]);
      ws[282816] = fma(kw * y[4032], y[5952], ws[282816]);
    }
    {
      double w = 2.0 * phi[5920];
      w = fma(0.287, phi[5856], w);
      w = fma(1.24, phi[5760], w);
      w = fma(0.464, phi[5504], w);
      w = w - phi[4064];
      w = w - phi[5952];
      const double kw = ws[54144] * w;
      out[4064] = fma(kw, y[5952], out[4064]);
      out[5952] = fma(kw, y[4064], out[5952]);
      ws[282848] = fma(kw * y[4064], y[5952], ws[282848]);
    }
    {
      double w = 2.0 * phi[5920];
      w = fma(1.0, phi[5376], w);
      w = fma(1.0, phi[5728], w);
      w = w - phi[3072];
      w = w - phi[5952];
      const double kw = ws[54176] * w;
      out[3072] = fma(kw, y[5952], out[3072]);
      out[5952] = fma(kw, y[3072], out[5952]);
      ws[282880] = fma(kw * y[3072], y[5952], ws[282880]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(2.0, phi[5440], w);
      w = w - phi[4032];
      w = w - phi[4032];
      const double kw = ws[54208] * w;
      out[4032] = fma(kw, y[4032], out[4032]);
      out[4032] = fma(kw, y[4032], out[4032]);
      ws[282912] = fma(kw * y[4032], y[4032], ws[282912]);
    }
    {
      double w = 0.5 * phi[5984];
      w = fma(0.5, phi[5920], w);
      w = fma(0.202, phi[5856], w);
      w = fma(0.64, phi[5760], w);
      w = fma(0.149, phi[5504], w);
      w = fma(1.5, phi[5440], w);
      w = w - phi[4032];
      w = w - phi[4064];
      const double kw = ws[54240] * w;
      out[4032] = fma(kw, y[4064], out[4032]);
      out[4064] = fma(kw, y[4032], out[4064]);
      ws[282944] = fma(kw * y[4032], y[4064], ws[282944]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.504, phi[5856], w);
      w = fma(1.21, phi[5760], w);
      w = fma(0.285, phi[5504], w);
      w = fma(1.0, phi[5440], w);
      w = w - phi[4064];
      w = w - phi[4064];
      const double kw = ws[54272] * w;
      out[4064] = fma(kw, y[4064], out[4064]);
      out[4064] = fma(kw, y[4064], out[4064]);
      ws[282976] = fma(kw * y[4064], y[4064], ws[282976]);
    }
}
}  // namespace mech_cracmm2
