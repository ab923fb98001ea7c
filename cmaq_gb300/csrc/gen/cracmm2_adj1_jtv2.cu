// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_jtv_1_8(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5920];
      w = w - phi[5216];
      w = w - phi[5952];
      const double kw = ws[54304] * w;
      out[5216] = fma(kw, y[5952], out[5216]);
      out[5952] = fma(kw, y[5216], out[5952]);
      ws[283008] = fma(kw * y[5216], y[5952], ws[283008]);
    }
    {
      double w = 1.0 * phi[5632];
      w = w - phi[5216];
      w = w - phi[4800];
      const double kw = ws[54336] * w;
      out[5216] = fma(kw, y[4800], out[5216]);
      out[4800] = fma(kw, y[5216], out[4800]);
      ws[283040] = fma(kw * y[5216], y[4800], ws[283040]);
    }
    {
      double w = -phi[5216];
      w = w - phi[5216];
      const double kw = ws[54368] * w;
      out[5216] = fma(kw, y[5216], out[5216]);
      out[5216] = fma(kw, y[5216], out[5216]);
      ws[283072] = fma(kw * y[5216], y[5216], ws[283072]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4544], w);
      w = fma(0.48, phi[6016], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3744];
      w = w - phi[4160];
      const double kw = ws[54400] * w;
      out[3744] = fma(kw, y[4160], out[3744]);
      out[4160] = fma(kw, y[3744], out[4160]);
      ws[283104] = fma(kw * y[3744], y[4160], ws[283104]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4576], w);
      w = fma(0.48, phi[6016], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3744];
      w = w - phi[4192];
      const double kw = ws[54432] * w;
      out[3744] = fma(kw, y[4192], out[3744]);
      out[4192] = fma(kw, y[3744], out[4192]);
      ws[283136] = fma(kw * y[3744], y[4192], ws[283136]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[5856], w);
      w = fma(0.48, phi[4736], w);
      w = fma(0.48, phi[6016], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3744];
      w = w - phi[4288];
      const double kw = ws[54464] * w;
      out[3744] = fma(kw, y[4288], out[3744]);
      out[4288] = fma(kw, y[3744], out[4288]);
      ws[283168] = fma(kw * y[3744], y[4288], ws[283168]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4544], w);
      w = fma(0.48, phi[6016], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3936];
      w = w - phi[4160];
      const double kw = ws[54496] * w;
      out[3936] = fma(kw, y[4160], out[3936]);
      out[4160] = fma(kw, y[3936], out[4160]);
      ws[283200] = fma(kw * y[3936], y[4160], ws[283200]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4576], w);
      w = fma(0.48, phi[6016], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3936];
      w = w - phi[4192];
      const double kw = ws[54528] * w;
      out[3936] = fma(kw, y[4192], out[3936]);
      out[4192] = fma(kw, y[3936], out[4192]);
      ws[283232] = fma(kw * y[3936], y[4192], ws[283232]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[5856], w);
      w = fma(0.48, phi[4736], w);
      w = fma(0.48, phi[6016], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3936];
      w = w - phi[4288];
      const double kw = ws[54560] * w;
      out[3936] = fma(kw, y[4288], out[3936]);
      out[4288] = fma(kw, y[3936], out[4288]);
      ws[283264] = fma(kw * y[3936], y[4288], ws[283264]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4544], w);
      w = fma(0.48, phi[5920], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3840];
      w = w - phi[4160];
      const double kw = ws[54592] * w;
      out[3840] = fma(kw, y[4160], out[3840]);
      out[4160] = fma(kw, y[3840], out[4160]);
      ws[283296] = fma(kw * y[3840], y[4160], ws[283296]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4576], w);
      w = fma(0.48, phi[5920], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3840];
      w = w - phi[4192];
      const double kw = ws[54624] * w;
      out[3840] = fma(kw, y[4192], out[3840]);
      out[4192] = fma(kw, y[3840], out[4192]);
      ws[283328] = fma(kw * y[3840], y[4192], ws[283328]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[5856], w);
      w = fma(0.48, phi[4736], w);
      w = fma(0.48, phi[5920], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3840];
      w = w - phi[4288];
      const double kw = ws[54656] * w;
      out[3840] = fma(kw, y[4288], out[3840]);
      out[4288] = fma(kw, y[3840], out[4288]);
      ws[283360] = fma(kw * y[3840], y[4288], ws[283360]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4544], w);
      w = fma(0.48, phi[5920], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3712];
      w = w - phi[4160];
      const double kw = ws[54688] * w;
      out[3712] = fma(kw, y[4160], out[3712]);
      out[4160] = fma(kw, y[3712], out[4160]);
      ws[283392] = fma(kw * y[3712], y[4160], ws[283392]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[4576], w);
      w = fma(0.48, phi[5920], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3712];
      w = w - phi[4192];
      const double kw = ws[54720] * w;
      out[3712] = fma(kw, y[4192], out[3712]);
      out[4192] = fma(kw, y[3712], out[4192]);
      ws[283424] = fma(kw * y[3712], y[4192], ws[283424]);
    }
    {
      double w = 0.96 * phi[4256];
      w = fma(0.48, phi[5056], w);
      w = fma(0.48, phi[5856], w);
      w = fma(0.48, phi[4736], w);
      w = fma(0.48, phi[5920], w);
      w = fma(0.48, phi[5984], w);
      w = fma(0.04, phi[2720], w);
      w = w - phi[3712];
      w = w - phi[4288];
      const double kw = ws[54752] * w;
      out[3712] = fma(kw, y[4288], out[3712]);
      out[4288] = fma(kw, y[3712], out[4288]);
      ws[283456] = fma(kw * y[3712], y[4288], ws[283456]);
    }
    {
      double w = 1.0 * phi[6016];
      w = w - phi[1376];
      w = w - phi[6016];
      const double kw = ws[54784] * w;
      out[1376] = fma(kw, y[6016], out[1376]);
      out[6016] = fma(kw, y[1376], out[6016]);
      ws[283488] = fma(kw * y[1376], y[6016], ws[283488]);
    }
    {
      double w = 0.852 * phi[5632];
      w = fma(0.149, phi[3616], w);
      w = w - phi[384];
      w = w - phi[6016];
      const double kw = ws[54816] * w;
      out[384] = fma(kw, y[6016], out[384]);
      out[6016] = fma(kw, y[384], out[6016]);
      ws[283520] = fma(kw * y[384], y[6016], ws[283520]);
    }
    {
      double w = 1.0 * phi[5632];
      w = fma(0.00101, phi[3616], w);
      w = w - phi[416];
      w = w - phi[6016];
      const double kw = ws[54848] * w;
      out[416] = fma(kw, y[6016], out[416]);
      out[6016] = fma(kw, y[416], out[6016]);
      ws[283552] = fma(kw * y[416], y[6016], ws[283552]);
    }
    {
      double w = 0.57 * phi[4672];
      w = fma(0.43, phi[3520], w);
      w = w - phi[3552];
      w = w - phi[6016];
      const double kw = ws[54880] * w;
      out[3552] = fma(kw, y[6016], out[3552]);
      out[6016] = fma(kw, y[3552], out[6016]);
      ws[283584] = fma(kw * y[3552], y[6016], ws[283584]);
    }
    {
      double w = 0.84 * phi[5664];
      w = fma(0.56, phi[5984], w);
      w = fma(0.28, phi[6016], w);
      w = fma(0.72, phi[5856], w);
      w = fma(0.62, phi[5376], w);
      w = w - phi[3552];
      w = w - phi[5184];
      const double kw = ws[54912] * w;
      out[3552] = fma(kw, y[5184], out[3552]);
      out[5184] = fma(kw, y[3552], out[5184]);
      ws[283616] = fma(kw * y[3552], y[5184], ws[283616]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(0.32, phi[4672], w);
      w = fma(0.68, phi[5216], w);
      w = fma(0.68, phi[5248], w);
      w = fma(0.32, phi[5024], w);
      w = fma(0.68, phi[5920], w);
      w = w - phi[3552];
      w = w - phi[5952];
      const double kw = ws[54944] * w;
      out[3552] = fma(kw, y[5952], out[3552]);
      out[5952] = fma(kw, y[3552], out[5952]);
      ws[283648] = fma(kw * y[3552], y[5952], ws[283648]);
    }
    {
      double w = 0.667 * phi[3136];
      w = fma(0.333, phi[3872], w);
      w = fma(0.333, phi[5984], w);
      w = w - phi[1568];
      w = w - phi[6016];
      const double kw = ws[55008] * w;
      out[1568] = fma(kw, y[6016], out[1568]);
      out[6016] = fma(kw, y[1568], out[6016]);
      ws[283712] = fma(kw * y[1568], y[6016], ws[283712]);
    }
    {
      double w = 0.968 * phi[5984];
      w = fma(0.968, phi[5920], w);
      w = fma(0.895, phi[3552], w);
      w = fma(0.895, phi[5856], w);
      w = fma(0.072, phi[3168], w);
      w = fma(0.032, phi[5440], w);
      w = w - phi[3136];
      w = w - phi[5824];
      const double kw = ws[55040] * w;
      out[3136] = fma(kw, y[5824], out[3136]);
      out[5824] = fma(kw, y[3136], out[5824]);
      ws[283744] = fma(kw * y[3136], y[5824], ws[283744]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.925, phi[3552], w);
      w = fma(0.925, phi[5856], w);
      w = fma(0.075, phi[3168], w);
      w = w - phi[3136];
      w = w - phi[5952];
      const double kw = ws[55072] * w;
      out[3136] = fma(kw, y[5952], out[3136]);
      out[5952] = fma(kw, y[3136], out[5952]);
      ws[283776] = fma(kw * y[3136], y[5952], ws[283776]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3136];
      w = w - phi[5984];
      const double kw = ws[55104] * w;
      out[3136] = fma(kw, y[5984], out[3136]);
      out[5984] = fma(kw, y[3136], out[5984]);
      ws[283808] = fma(kw * y[3136], y[5984], ws[283808]);
    }
    {
      double w = 0.32 * phi[5600];
      w = fma(1.143, phi[5856], w);
      w = fma(0.87, phi[5984], w);
      w = fma(0.463, phi[3552], w);
      w = fma(0.25, phi[2752], w);
      w = fma(0.231, phi[4736], w);
      w = fma(0.037, phi[3168], w);
      w = fma(0.019, phi[3872], w);
      w = w - phi[3136];
      w = w - phi[5888];
      const double kw = ws[55136] * w;
      out[3136] = fma(kw, y[5888], out[3136]);
      out[5888] = fma(kw, y[3136], out[5888]);
      ws[283840] = fma(kw * y[3136], y[5888], ws[283840]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.3, phi[5696], w);
      w = fma(0.8, phi[5984], w);
      w = fma(0.74, phi[3552], w);
      w = fma(0.74, phi[5856], w);
      w = fma(0.185, phi[4736], w);
      w = fma(0.06, phi[3168], w);
      w = fma(0.015, phi[3872], w);
      w = w - phi[3136];
      w = w - phi[5792];
      const double kw = ws[55168] * w;
      out[3136] = fma(kw, y[5792], out[3136]);
      out[5792] = fma(kw, y[3136], out[5792]);
      ws[283872] = fma(kw * y[3136], y[5792], ws[283872]);
    }
    {
      double w = 0.62 * phi[3552];
      w = fma(0.63, phi[5664], w);
      w = fma(0.42, phi[5984], w);
      w = fma(0.08, phi[6016], w);
      w = fma(0.83, phi[5856], w);
      w = fma(0.17, phi[2240], w);
      w = w - phi[1568];
      w = w - phi[5184];
      const double kw = ws[55200] * w;
      out[1568] = fma(kw, y[5184], out[1568]);
      out[5184] = fma(kw, y[1568], out[5184]);
      ws[283904] = fma(kw * y[1568], y[5184], ws[283904]);
    }
    {
      double w = 0.9 * phi[4032];
      w = fma(0.1, phi[4064], w);
      w = fma(0.9, phi[3552], w);
      w = w - phi[1568];
      w = w - phi[5952];
      const double kw = ws[55232] * w;
      out[1568] = fma(kw, y[5952], out[1568]);
      out[5952] = fma(kw, y[1568], out[5952]);
      ws[283936] = fma(kw * y[1568], y[5952], ws[283936]);
    }
    {
      double w = 0.49 * phi[5472];
      w = fma(0.49, phi[5984], w);
      w = fma(0.51, phi[1856], w);
      w = w - phi[3168];
      w = w - phi[6016];
      const double kw = ws[55264] * w;
      out[3168] = fma(kw, y[6016], out[3168]);
      out[6016] = fma(kw, y[3168], out[6016]);
      ws[283968] = fma(kw * y[3168], y[6016], ws[283968]);
    }
    {
      double w = 0.08 * phi[5440];
      w = fma(0.92, phi[5920], w);
      w = fma(0.92, phi[4512], w);
      w = fma(0.75, phi[5984], w);
      w = fma(0.17, phi[5888], w);
      w = w - phi[1856];
      w = w - phi[5824];
      const double kw = ws[55296] * w;
      out[1856] = fma(kw, y[5824], out[1856]);
      out[5824] = fma(kw, y[1856], out[5824]);
      ws[284000] = fma(kw * y[1856], y[5824], ws[284000]);
    }
    {
      double w = 0.6 * phi[5728];
      w = fma(0.4, phi[4512], w);
      w = fma(0.4, phi[6016], w);
      w = fma(0.32, phi[5984], w);
      w = fma(0.08, phi[5888], w);
      w = w - phi[1856];
      w = w - phi[5984];
      const double kw = ws[55328] * w;
      out[1856] = fma(kw, y[5984], out[1856]);
      out[5984] = fma(kw, y[1856], out[5984]);
      ws[284032] = fma(kw * y[1856], y[5984], ws[284032]);
    }
    {
      double w = 0.65 * phi[5504];
      w = fma(0.31, phi[5376], w);
      w = fma(0.66, phi[5984], w);
      w = fma(0.34, phi[5888], w);
      w = fma(0.43, phi[5664], w);
      w = fma(0.04, phi[3616], w);
      w = w - phi[4512];
      w = w - phi[6016];
      const double kw = ws[55360] * w;
      out[4512] = fma(kw, y[6016], out[4512]);
      out[6016] = fma(kw, y[4512], out[6016]);
      ws[284064] = fma(kw * y[4512], y[6016], ws[284064]);
    }
    {
      double w = 0.02 * phi[6016];
      w = fma(1.0, phi[5760], w);
      w = w - phi[3168];
      w = w - phi[5184];
      const double kw = ws[55392] * w;
      out[3168] = fma(kw, y[5184], out[3168]);
      out[5184] = fma(kw, y[3168], out[5184]);
      ws[284096] = fma(kw * y[3168], y[5184], ws[284096]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.8, phi[5472], w);
      w = fma(0.2, phi[3584], w);
      w = w - phi[3168];
      w = w - phi[5952];
      const double kw = ws[55424] * w;
      out[3168] = fma(kw, y[5952], out[3168]);
      out[5952] = fma(kw, y[3168], out[5952]);
      ws[284128] = fma(kw * y[3168], y[5952], ws[284128]);
    }
    {
      double w = 0.613 * phi[5344];
      w = fma(0.387, phi[5760], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[448];
      w = w - phi[6016];
      const double kw = ws[55456] * w;
      out[448] = fma(kw, y[6016], out[448]);
      out[6016] = fma(kw, y[448], out[6016]);
      ws[284160] = fma(kw * y[448], y[6016], ws[284160]);
    }
    {
      double w = 1.0 * phi[1920];
      w = w - phi[1600];
      w = w - phi[5952];
      const double kw = ws[55488] * w;
      out[1600] = fma(kw, y[5952], out[1600]);
      out[5952] = fma(kw, y[1600], out[5952]);
      ws[284192] = fma(kw * y[1600], y[5952], ws[284192]);
    }
    {
      double w = 1.0 * phi[4928];
      w = w - phi[1920];
      w = w - phi[5984];
      const double kw = ws[55520] * w;
      out[1920] = fma(kw, y[5984], out[1920]);
      out[5984] = fma(kw, y[1920], out[5984]);
      ws[284224] = fma(kw * y[1920], y[5984], ws[284224]);
    }
    {
      double w = 1.0 * phi[5536];
      w = fma(2.0, phi[5920], w);
      w = w - phi[1920];
      w = w - phi[5824];
      const double kw = ws[55552] * w;
      out[1920] = fma(kw, y[5824], out[1920]);
      out[5824] = fma(kw, y[1920], out[5824]);
      ws[284256] = fma(kw * y[1920], y[5824], ws[284256]);
    }
    {
      double w = 1.0 * phi[5536];
      w = fma(2.0, phi[5920], w);
      w = w - phi[1920];
      w = w - phi[5952];
      const double kw = ws[55584] * w;
      out[1920] = fma(kw, y[5952], out[1920]);
      out[5952] = fma(kw, y[1920], out[5952]);
      ws[284288] = fma(kw * y[1920], y[5952], ws[284288]);
    }
    {
      double w = 0.982 * phi[5536];
      w = fma(0.018, phi[4832], w);
      w = w - phi[1600];
      w = w - phi[5184];
      const double kw = ws[55616] * w;
      out[1600] = fma(kw, y[5184], out[1600]);
      out[5184] = fma(kw, y[1600], out[5184]);
      ws[284320] = fma(kw * y[1600], y[5184], ws[284320]);
    }
}
__device__ __noinline__ void adj_jtv_1_9(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[2304];
      w = w - phi[1600];
      w = w - phi[6016];
      const double kw = ws[55648] * w;
      out[1600] = fma(kw, y[6016], out[1600]);
      out[6016] = fma(kw, y[1600], out[6016]);
      ws[284352] = fma(kw * y[1600], y[6016], ws[284352]);
    }
    {
      double w = 1.0 * phi[4960];
      w = w - phi[2304];
      w = w - phi[5984];
      const double kw = ws[55680] * w;
      out[2304] = fma(kw, y[5984], out[2304]);
      out[5984] = fma(kw, y[2304], out[5984]);
      ws[284384] = fma(kw * y[2304], y[5984], ws[284384]);
    }
    {
      double w = 1.0 * phi[5536];
      w = w - phi[2304];
      w = w - phi[5952];
      const double kw = ws[55712] * w;
      out[2304] = fma(kw, y[5952], out[2304]);
      out[5952] = fma(kw, y[2304], out[5952]);
      ws[284416] = fma(kw * y[2304], y[5952], ws[284416]);
    }
    {
      double w = 0.247 * phi[4992];
      w = fma(0.753, phi[5536], w);
      w = fma(0.753, phi[5920], w);
      w = w - phi[2304];
      w = w - phi[5824];
      const double kw = ws[55744] * w;
      out[2304] = fma(kw, y[5824], out[2304]);
      out[5824] = fma(kw, y[2304], out[5824]);
      ws[284448] = fma(kw * y[2304], y[5824], ws[284448]);
    }
    {
      double w = 1.0 * phi[480];
      w = w - phi[5376];
      const double kw = ws[55776] * w;
      out[5376] = out[5376] + kw;
      ws[284480] = fma(kw, y[5376], ws[284480]);
    }
    {
      double w = 1.0 * phi[480];
      w = w - phi[5248];
      const double kw = ws[55808] * w;
      out[5248] = out[5248] + kw;
      ws[284512] = fma(kw, y[5248], ws[284512]);
    }
    {
      double w = 2.0 * phi[5024];
      w = w - phi[1024];
      const double kw = ws[55840] * w;
      out[1024] = out[1024] + kw;
      ws[284544] = fma(kw, y[1024], ws[284544]);
    }
    {
      double w = 0.5 * phi[1184];
      w = fma(0.5, phi[5024], w);
      w = w - phi[5920];
      const double kw = ws[55872] * w;
      out[5920] = out[5920] + kw;
      ws[284576] = fma(kw, y[5920], ws[284576]);
    }
    {
      double w = -phi[5984];
      const double kw = ws[55904] * w;
      out[5984] = out[5984] + kw;
      ws[284608] = fma(kw, y[5984], ws[284608]);
    }
    {
      double w = 1.0 * phi[5024];
      w = w - phi[5952];
      const double kw = ws[55936] * w;
      out[5952] = out[5952] + kw;
      ws[284640] = fma(kw, y[5952], ws[284640]);
    }
    {
      double w = 1.0 * phi[1056];
      w = w - phi[1376];
      const double kw = ws[56000] * w;
      out[1376] = out[1376] + kw;
      ws[284704] = fma(kw, y[1376], ws[284704]);
    }
    {
      double w = 1.0 * phi[0];
      w = w - phi[1056];
      const double kw = ws[56032] * w;
      out[1056] = out[1056] + kw;
      ws[284736] = fma(kw, y[1056], ws[284736]);
    }
    {
      double w = 1.0 * phi[544];
      w = w - phi[1056];
      w = w - phi[512];
      const double kw = ws[56064] * w;
      out[1056] = fma(kw, y[512], out[1056]);
      out[512] = fma(kw, y[1056], out[512]);
      ws[284768] = fma(kw * y[1056], y[512], ws[284768]);
    }
    {
      double w = 1.0 * phi[32];
      w = w - phi[1664];
      const double kw = ws[56096] * w;
      out[1664] = out[1664] + kw;
      ws[284800] = fma(kw, y[1664], ws[284800]);
    }
    {
      double w = 1.0 * phi[64];
      w = fma(1.0, phi[5024], w);
      w = w - phi[2208];
      const double kw = ws[56128] * w;
      out[2208] = out[2208] + kw;
      ws[284832] = fma(kw, y[2208], ws[284832]);
    }
    {
      double w = 1.0 * phi[2368];
      w = w - phi[608];
      w = w - phi[6016];
      const double kw = ws[56160] * w;
      out[608] = fma(kw, y[6016], out[608]);
      out[6016] = fma(kw, y[608], out[6016]);
      ws[284864] = fma(kw * y[608], y[6016], ws[284864]);
    }
    {
      double w = 1.0 * phi[2400];
      w = w - phi[640];
      w = w - phi[6016];
      const double kw = ws[56192] * w;
      out[640] = fma(kw, y[6016], out[640]);
      out[6016] = fma(kw, y[640], out[6016]);
      ws[284896] = fma(kw * y[640], y[6016], ws[284896]);
    }
    {
      double w = 1.0 * phi[2432];
      w = w - phi[672];
      w = w - phi[6016];
      const double kw = ws[56224] * w;
      out[672] = fma(kw, y[6016], out[672]);
      out[6016] = fma(kw, y[672], out[6016]);
      ws[284928] = fma(kw * y[672], y[6016], ws[284928]);
    }
    {
      double w = 1.0 * phi[2464];
      w = w - phi[704];
      w = w - phi[6016];
      const double kw = ws[56256] * w;
      out[704] = fma(kw, y[6016], out[704]);
      out[6016] = fma(kw, y[704], out[6016]);
      ws[284960] = fma(kw * y[704], y[6016], ws[284960]);
    }
    {
      double w = 1.0 * phi[2496];
      w = w - phi[736];
      w = w - phi[6016];
      const double kw = ws[56288] * w;
      out[736] = fma(kw, y[6016], out[736]);
      out[6016] = fma(kw, y[736], out[6016]);
      ws[284992] = fma(kw * y[736], y[6016], ws[284992]);
    }
    {
      double w = 1.0 * phi[2528];
      w = w - phi[768];
      w = w - phi[6016];
      const double kw = ws[56320] * w;
      out[768] = fma(kw, y[6016], out[768]);
      out[6016] = fma(kw, y[768], out[6016]);
      ws[285024] = fma(kw * y[768], y[6016], ws[285024]);
    }
    {
      double w = 1.0 * phi[3904];
      w = w - phi[800];
      w = w - phi[6016];
      const double kw = ws[56352] * w;
      out[800] = fma(kw, y[6016], out[800]);
      out[6016] = fma(kw, y[800], out[6016]);
      ws[285056] = fma(kw * y[800], y[6016], ws[285056]);
    }
    {
      double w = 0.72 * phi[1952];
      w = fma(0.28, phi[5312], w);
      w = fma(0.72, phi[5920], w);
      w = w - phi[2368];
      w = w - phi[5824];
      const double kw = ws[56384] * w;
      out[2368] = fma(kw, y[5824], out[2368]);
      out[5824] = fma(kw, y[2368], out[5824]);
      ws[285088] = fma(kw * y[2368], y[5824], ws[285088]);
    }
    {
      double w = 0.72 * phi[1984];
      w = fma(0.28, phi[5536], w);
      w = fma(0.72, phi[5920], w);
      w = w - phi[2400];
      w = w - phi[5824];
      const double kw = ws[56416] * w;
      out[2400] = fma(kw, y[5824], out[2400]);
      out[5824] = fma(kw, y[2400], out[5824]);
      ws[285120] = fma(kw * y[2400], y[5824], ws[285120]);
    }
    {
      double w = 0.72 * phi[2016];
      w = fma(0.28, phi[5088], w);
      w = fma(0.72, phi[5920], w);
      w = w - phi[2432];
      w = w - phi[5824];
      const double kw = ws[56448] * w;
      out[2432] = fma(kw, y[5824], out[2432]);
      out[5824] = fma(kw, y[2432], out[5824]);
      ws[285152] = fma(kw * y[2432], y[5824], ws[285152]);
    }
    {
      double w = 0.72 * phi[2048];
      w = fma(0.28, phi[4704], w);
      w = fma(0.72, phi[5920], w);
      w = w - phi[2464];
      w = w - phi[5824];
      const double kw = ws[56480] * w;
      out[2464] = fma(kw, y[5824], out[2464]);
      out[5824] = fma(kw, y[2464], out[5824]);
      ws[285184] = fma(kw * y[2464], y[5824], ws[285184]);
    }
    {
      double w = 0.72 * phi[2080];
      w = fma(0.28, phi[4960], w);
      w = fma(0.72, phi[5920], w);
      w = w - phi[2496];
      w = w - phi[5824];
      const double kw = ws[56512] * w;
      out[2496] = fma(kw, y[5824], out[2496]);
      out[5824] = fma(kw, y[2496], out[5824]);
      ws[285216] = fma(kw * y[2496], y[5824], ws[285216]);
    }
    {
      double w = 0.72 * phi[2112];
      w = fma(0.28, phi[4416], w);
      w = fma(0.72, phi[5920], w);
      w = w - phi[2528];
      w = w - phi[5824];
      const double kw = ws[56544] * w;
      out[2528] = fma(kw, y[5824], out[2528]);
      out[5824] = fma(kw, y[2528], out[5824]);
      ws[285248] = fma(kw * y[2528], y[5824], ws[285248]);
    }
    {
      double w = 0.74 * phi[2144];
      w = fma(0.26, phi[5440], w);
      w = fma(0.74, phi[5920], w);
      w = w - phi[3904];
      w = w - phi[5824];
      const double kw = ws[56576] * w;
      out[3904] = fma(kw, y[5824], out[3904]);
      out[5824] = fma(kw, y[3904], out[5824]);
      ws[285280] = fma(kw * y[3904], y[5824], ws[285280]);
    }
    {
      double w = 1.0 * phi[1952];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2368];
      w = w - phi[5952];
      const double kw = ws[56608] * w;
      out[2368] = fma(kw, y[5952], out[2368]);
      out[5952] = fma(kw, y[2368], out[5952]);
      ws[285312] = fma(kw * y[2368], y[5952], ws[285312]);
    }
    {
      double w = 1.0 * phi[1984];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2400];
      w = w - phi[5952];
      const double kw = ws[56640] * w;
      out[2400] = fma(kw, y[5952], out[2400]);
      out[5952] = fma(kw, y[2400], out[5952]);
      ws[285344] = fma(kw * y[2400], y[5952], ws[285344]);
    }
    {
      double w = 1.0 * phi[2016];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2432];
      w = w - phi[5952];
      const double kw = ws[56672] * w;
      out[2432] = fma(kw, y[5952], out[2432]);
      out[5952] = fma(kw, y[2432], out[5952]);
      ws[285376] = fma(kw * y[2432], y[5952], ws[285376]);
    }
    {
      double w = 1.0 * phi[2048];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2464];
      w = w - phi[5952];
      const double kw = ws[56704] * w;
      out[2464] = fma(kw, y[5952], out[2464]);
      out[5952] = fma(kw, y[2464], out[5952]);
      ws[285408] = fma(kw * y[2464], y[5952], ws[285408]);
    }
    {
      double w = 1.0 * phi[2080];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2496];
      w = w - phi[5952];
      const double kw = ws[56736] * w;
      out[2496] = fma(kw, y[5952], out[2496]);
      out[5952] = fma(kw, y[2496], out[5952]);
      ws[285440] = fma(kw * y[2496], y[5952], ws[285440]);
    }
    {
      double w = 1.0 * phi[2112];
      w = fma(1.0, phi[5920], w);
      w = w - phi[2528];
      w = w - phi[5952];
      const double kw = ws[56768] * w;
      out[2528] = fma(kw, y[5952], out[2528]);
      out[5952] = fma(kw, y[2528], out[5952]);
      ws[285472] = fma(kw * y[2528], y[5952], ws[285472]);
    }
    {
      double w = 1.0 * phi[2144];
      w = fma(1.0, phi[5920], w);
      w = w - phi[3904];
      w = w - phi[5952];
      const double kw = ws[56800] * w;
      out[3904] = fma(kw, y[5952], out[3904]);
      out[5952] = fma(kw, y[3904], out[5952]);
      ws[285504] = fma(kw * y[3904], y[5952], ws[285504]);
    }
    {
      double w = 1.0 * phi[5536];
      w = w - phi[2368];
      w = w - phi[5984];
      const double kw = ws[56832] * w;
      out[2368] = fma(kw, y[5984], out[2368]);
      out[5984] = fma(kw, y[2368], out[5984]);
      ws[285536] = fma(kw * y[2368], y[5984], ws[285536]);
    }
    {
      double w = 1.0 * phi[5088];
      w = w - phi[2400];
      w = w - phi[5984];
      const double kw = ws[56864] * w;
      out[2400] = fma(kw, y[5984], out[2400]);
      out[5984] = fma(kw, y[2400], out[5984]);
      ws[285568] = fma(kw * y[2400], y[5984], ws[285568]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[2432];
      w = w - phi[5984];
      const double kw = ws[56896] * w;
      out[2432] = fma(kw, y[5984], out[2432]);
      out[5984] = fma(kw, y[2432], out[5984]);
      ws[285600] = fma(kw * y[2432], y[5984], ws[285600]);
    }
    {
      double w = 1.0 * phi[4960];
      w = w - phi[2464];
      w = w - phi[5984];
      const double kw = ws[56928] * w;
      out[2464] = fma(kw, y[5984], out[2464]);
      out[5984] = fma(kw, y[2464], out[5984]);
      ws[285632] = fma(kw * y[2464], y[5984], ws[285632]);
    }
    {
      double w = 1.0 * phi[4416];
      w = w - phi[2496];
      w = w - phi[5984];
      const double kw = ws[56960] * w;
      out[2496] = fma(kw, y[5984], out[2496]);
      out[5984] = fma(kw, y[2496], out[5984]);
      ws[285664] = fma(kw * y[2496], y[5984], ws[285664]);
    }
    {
      double w = 1.0 * phi[4832];
      w = w - phi[2528];
      w = w - phi[5984];
      const double kw = ws[56992] * w;
      out[2528] = fma(kw, y[5984], out[2528]);
      out[5984] = fma(kw, y[2528], out[5984]);
      ws[285696] = fma(kw * y[2528], y[5984], ws[285696]);
    }
    {
      double w = 1.0 * phi[5728];
      w = w - phi[3904];
      w = w - phi[5984];
      const double kw = ws[57024] * w;
      out[3904] = fma(kw, y[5984], out[3904]);
      out[5984] = fma(kw, y[3904], out[5984]);
      ws[285728] = fma(kw * y[3904], y[5984], ws[285728]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5536], w);
      w = w - phi[1952];
      const double kw = ws[57056] * w;
      out[1952] = out[1952] + kw;
      ws[285760] = fma(kw, y[1952], ws[285760]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5088], w);
      w = w - phi[1984];
      const double kw = ws[57088] * w;
      out[1984] = out[1984] + kw;
      ws[285792] = fma(kw, y[1984], ws[285792]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[4704], w);
      w = w - phi[2016];
      const double kw = ws[57120] * w;
      out[2016] = out[2016] + kw;
      ws[285824] = fma(kw, y[2016], ws[285824]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[4960], w);
      w = w - phi[2048];
      const double kw = ws[57152] * w;
      out[2048] = out[2048] + kw;
      ws[285856] = fma(kw, y[2048], ws[285856]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[4416], w);
      w = w - phi[2080];
      const double kw = ws[57184] * w;
      out[2080] = out[2080] + kw;
      ws[285888] = fma(kw, y[2080], ws[285888]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[4832], w);
      w = w - phi[2112];
      const double kw = ws[57216] * w;
      out[2112] = out[2112] + kw;
      ws[285920] = fma(kw, y[2112], ws[285920]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5312], w);
      w = w - phi[2144];
      const double kw = ws[57248] * w;
      out[2144] = out[2144] + kw;
      ws[285952] = fma(kw, y[2144], ws[285952]);
    }
    {
      double w = 0.14 * phi[5088];
      w = fma(0.86, phi[5920], w);
      w = fma(0.86, phi[5536], w);
      w = fma(0.86, phi[5984], w);
      w = w - phi[1952];
      w = w - phi[5824];
      const double kw = ws[57280] * w;
      out[1952] = fma(kw, y[5824], out[1952]);
      out[5824] = fma(kw, y[1952], out[5824]);
      ws[285984] = fma(kw * y[1952], y[5824], ws[285984]);
    }
    {
      double w = 0.14 * phi[4992];
      w = fma(0.86, phi[5920], w);
      w = fma(0.86, phi[5088], w);
      w = fma(0.86, phi[5984], w);
      w = w - phi[1984];
      w = w - phi[5824];
      const double kw = ws[57312] * w;
      out[1984] = fma(kw, y[5824], out[1984]);
      out[5824] = fma(kw, y[1984], out[5824]);
      ws[286016] = fma(kw * y[1984], y[5824], ws[286016]);
    }
    {
      double w = 0.14 * phi[4960];
      w = fma(0.86, phi[5920], w);
      w = fma(0.86, phi[4704], w);
      w = fma(0.86, phi[5984], w);
      w = w - phi[2016];
      w = w - phi[5824];
      const double kw = ws[57344] * w;
      out[2016] = fma(kw, y[5824], out[2016]);
      out[5824] = fma(kw, y[2016], out[5824]);
      ws[286048] = fma(kw * y[2016], y[5824], ws[286048]);
    }
    {
      double w = 0.14 * phi[4416];
      w = fma(0.86, phi[5920], w);
      w = fma(0.86, phi[4960], w);
      w = fma(0.86, phi[5984], w);
      w = w - phi[2048];
      w = w - phi[5824];
      const double kw = ws[57376] * w;
      out[2048] = fma(kw, y[5824], out[2048]);
      out[5824] = fma(kw, y[2048], out[5824]);
      ws[286080] = fma(kw * y[2048], y[5824], ws[286080]);
    }
}
__device__ __noinline__ void adj_jtv_1_10(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 0.14 * phi[4832];
      w = fma(0.86, phi[5920], w);
      w = fma(0.86, phi[4416], w);
      w = fma(0.86, phi[5984], w);
      w = w - phi[2080];
      w = w - phi[5824];
      const double kw = ws[57408] * w;
      out[2080] = fma(kw, y[5824], out[2080]);
      out[5824] = fma(kw, y[2080], out[5824]);
      ws[286112] = fma(kw * y[2080], y[5824], ws[286112]);
    }
    {
      double w = 1.0 * phi[4832];
      w = fma(0.86, phi[5920], w);
      w = fma(0.86, phi[5984], w);
      w = w - phi[2112];
      w = w - phi[5824];
      const double kw = ws[57440] * w;
      out[2112] = fma(kw, y[5824], out[2112]);
      out[5824] = fma(kw, y[2112], out[5824]);
      ws[286144] = fma(kw * y[2112], y[5824], ws[286144]);
    }
    {
      double w = 0.12 * phi[5440];
      w = fma(0.88, phi[5920], w);
      w = fma(0.88, phi[5504], w);
      w = fma(0.88, phi[5984], w);
      w = w - phi[2144];
      w = w - phi[5824];
      const double kw = ws[57472] * w;
      out[2144] = fma(kw, y[5824], out[2144]);
      out[5824] = fma(kw, y[2144], out[5824]);
      ws[286176] = fma(kw * y[2144], y[5824], ws[286176]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5536], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[1952];
      w = w - phi[5952];
      const double kw = ws[57504] * w;
      out[1952] = fma(kw, y[5952], out[1952]);
      out[5952] = fma(kw, y[1952], out[5952]);
      ws[286208] = fma(kw * y[1952], y[5952], ws[286208]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5088], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[1984];
      w = w - phi[5952];
      const double kw = ws[57536] * w;
      out[1984] = fma(kw, y[5952], out[1984]);
      out[5952] = fma(kw, y[1984], out[5952]);
      ws[286240] = fma(kw * y[1984], y[5952], ws[286240]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2016];
      w = w - phi[5952];
      const double kw = ws[57568] * w;
      out[2016] = fma(kw, y[5952], out[2016]);
      out[5952] = fma(kw, y[2016], out[5952]);
      ws[286272] = fma(kw * y[2016], y[5952], ws[286272]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[4960], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2048];
      w = w - phi[5952];
      const double kw = ws[57600] * w;
      out[2048] = fma(kw, y[5952], out[2048]);
      out[5952] = fma(kw, y[2048], out[5952]);
      ws[286304] = fma(kw * y[2048], y[5952], ws[286304]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[4416], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2080];
      w = w - phi[5952];
      const double kw = ws[57632] * w;
      out[2080] = fma(kw, y[5952], out[2080]);
      out[5952] = fma(kw, y[2080], out[5952]);
      ws[286336] = fma(kw * y[2080], y[5952], ws[286336]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[4832], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2112];
      w = w - phi[5952];
      const double kw = ws[57664] * w;
      out[2112] = fma(kw, y[5952], out[2112]);
      out[5952] = fma(kw, y[2112], out[5952]);
      ws[286368] = fma(kw * y[2112], y[5952], ws[286368]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5504], w);
      w = fma(1.0, phi[5984], w);
      w = w - phi[2144];
      w = w - phi[5952];
      const double kw = ws[57696] * w;
      out[2144] = fma(kw, y[5952], out[2144]);
      out[5952] = fma(kw, y[2144], out[5952]);
      ws[286400] = fma(kw * y[2144], y[5952], ws[286400]);
    }
    {
      double w = 1.0 * phi[4992];
      w = w - phi[1952];
      w = w - phi[5984];
      const double kw = ws[57728] * w;
      out[1952] = fma(kw, y[5984], out[1952]);
      out[5984] = fma(kw, y[1952], out[5984]);
      ws[286432] = fma(kw * y[1952], y[5984], ws[286432]);
    }
    {
      double w = 1.0 * phi[4960];
      w = w - phi[1984];
      w = w - phi[5984];
      const double kw = ws[57760] * w;
      out[1984] = fma(kw, y[5984], out[1984]);
      out[5984] = fma(kw, y[1984], out[5984]);
      ws[286464] = fma(kw * y[1984], y[5984], ws[286464]);
    }
    {
      double w = 1.0 * phi[4416];
      w = w - phi[2016];
      w = w - phi[5984];
      const double kw = ws[57792] * w;
      out[2016] = fma(kw, y[5984], out[2016]);
      out[5984] = fma(kw, y[2016], out[5984]);
      ws[286496] = fma(kw * y[2016], y[5984], ws[286496]);
    }
    {
      double w = 1.0 * phi[4832];
      w = w - phi[2048];
      w = w - phi[5984];
      const double kw = ws[57824] * w;
      out[2048] = fma(kw, y[5984], out[2048]);
      out[5984] = fma(kw, y[2048], out[5984]);
      ws[286528] = fma(kw * y[2048], y[5984], ws[286528]);
    }
    {
      double w = 1.0 * phi[4832];
      w = w - phi[2080];
      w = w - phi[5984];
      const double kw = ws[57856] * w;
      out[2080] = fma(kw, y[5984], out[2080]);
      out[5984] = fma(kw, y[2080], out[5984]);
      ws[286560] = fma(kw * y[2080], y[5984], ws[286560]);
    }
    {
      double w = 1.0 * phi[4832];
      w = w - phi[2112];
      w = w - phi[5984];
      const double kw = ws[57888] * w;
      out[2112] = fma(kw, y[5984], out[2112]);
      out[5984] = fma(kw, y[2112], out[5984]);
      ws[286592] = fma(kw * y[2112], y[5984], ws[286592]);
    }
    {
      double w = 1.0 * phi[5088];
      w = w - phi[2144];
      w = w - phi[5984];
      const double kw = ws[57920] * w;
      out[2144] = fma(kw, y[5984], out[2144]);
      out[5984] = fma(kw, y[2144], out[5984]);
      ws[286624] = fma(kw * y[2144], y[5984], ws[286624]);
    }
    {
      double w = 0.84 * phi[3392];
      w = fma(0.16, phi[5984], w);
      w = fma(0.16, phi[5312], w);
      w = w - phi[832];
      w = w - phi[6016];
      const double kw = ws[57952] * w;
      out[832] = fma(kw, y[6016], out[832]);
      out[6016] = fma(kw, y[832], out[6016]);
      ws[286656] = fma(kw * y[832], y[6016], ws[286656]);
    }
    {
      double w = 0.0595 * phi[5312];
      w = fma(0.9048, phi[4992], w);
      w = fma(0.0357, phi[4864], w);
      w = w - phi[3392];
      w = w - phi[5984];
      const double kw = ws[57984] * w;
      out[3392] = fma(kw, y[5984], out[3392]);
      out[5984] = fma(kw, y[3392], out[5984]);
      ws[286688] = fma(kw * y[3392], y[5984], ws[286688]);
    }
    {
      double w = 0.0001 * phi[5312];
      w = fma(0.0018, phi[5088], w);
      w = fma(0.0001, phi[4640], w);
      w = fma(0.998, phi[5920], w);
      w = fma(0.998, phi[5984], w);
      w = fma(0.0594, phi[4448], w);
      w = fma(0.4693, phi[5376], w);
      w = fma(0.4693, phi[5248], w);
      w = fma(0.4693, phi[4512], w);
      w = fma(0.4693, phi[4320], w);
      w = w - phi[3392];
      w = w - phi[5824];
      const double kw = ws[58016] * w;
      out[3392] = fma(kw, y[5824], out[3392]);
      out[5824] = fma(kw, y[3392], out[5824]);
      ws[286720] = fma(kw * y[3392], y[5824], ws[286720]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.9405, phi[5984], w);
      w = fma(0.0595, phi[4448], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3392];
      w = w - phi[5952];
      const double kw = ws[58048] * w;
      out[3392] = fma(kw, y[5952], out[3392]);
      out[5952] = fma(kw, y[3392], out[5952]);
      ws[286752] = fma(kw * y[3392], y[5952], ws[286752]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.3105, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0595, phi[4448], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3392];
      w = w - phi[5888];
      const double kw = ws[58080] * w;
      out[3392] = fma(kw, y[5888], out[3392]);
      out[5888] = fma(kw, y[3392], out[5888]);
      ws[286784] = fma(kw * y[3392], y[5888], ws[286784]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.9405, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0595, phi[4448], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3392];
      w = w - phi[5792];
      const double kw = ws[58112] * w;
      out[3392] = fma(kw, y[5792], out[3392]);
      out[5792] = fma(kw, y[3392], out[5792]);
      ws[286816] = fma(kw * y[3392], y[5792], ws[286816]);
    }
    {
      double w = 0.84 * phi[3424];
      w = fma(0.16, phi[5984], w);
      w = fma(0.16, phi[5536], w);
      w = w - phi[864];
      w = w - phi[6016];
      const double kw = ws[58144] * w;
      out[864] = fma(kw, y[6016], out[864]);
      out[6016] = fma(kw, y[864], out[6016]);
      ws[286848] = fma(kw * y[864], y[6016], ws[286848]);
    }
    {
      double w = 0.0595 * phi[5536];
      w = fma(0.9048, phi[4960], w);
      w = fma(0.0357, phi[4864], w);
      w = w - phi[3424];
      w = w - phi[5984];
      const double kw = ws[58176] * w;
      out[3424] = fma(kw, y[5984], out[3424]);
      out[5984] = fma(kw, y[3424], out[5984]);
      ws[286880] = fma(kw * y[3424], y[5984], ws[286880]);
    }
    {
      double w = 0.0001 * phi[5536];
      w = fma(0.0018, phi[4992], w);
      w = fma(0.0001, phi[4864], w);
      w = fma(0.998, phi[5920], w);
      w = fma(0.998, phi[5984], w);
      w = fma(0.0594, phi[5312], w);
      w = fma(0.4693, phi[5376], w);
      w = fma(0.4693, phi[5248], w);
      w = fma(0.4693, phi[4512], w);
      w = fma(0.4693, phi[4320], w);
      w = w - phi[3424];
      w = w - phi[5824];
      const double kw = ws[58208] * w;
      out[3424] = fma(kw, y[5824], out[3424]);
      out[5824] = fma(kw, y[3424], out[5824]);
      ws[286912] = fma(kw * y[3424], y[5824], ws[286912]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.9405, phi[5984], w);
      w = fma(0.0595, phi[5312], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3424];
      w = w - phi[5952];
      const double kw = ws[58240] * w;
      out[3424] = fma(kw, y[5952], out[3424]);
      out[5952] = fma(kw, y[3424], out[5952]);
      ws[286944] = fma(kw * y[3424], y[5952], ws[286944]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.3105, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0595, phi[5312], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3424];
      w = w - phi[5888];
      const double kw = ws[58272] * w;
      out[3424] = fma(kw, y[5888], out[3424]);
      out[5888] = fma(kw, y[3424], out[5888]);
      ws[286976] = fma(kw * y[3424], y[5888], ws[286976]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.9405, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0595, phi[5312], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3424];
      w = w - phi[5792];
      const double kw = ws[58304] * w;
      out[3424] = fma(kw, y[5792], out[3424]);
      out[5792] = fma(kw, y[3424], out[5792]);
      ws[287008] = fma(kw * y[3424], y[5792], ws[287008]);
    }
    {
      double w = 0.84 * phi[3456];
      w = fma(0.16, phi[5984], w);
      w = fma(0.16, phi[5536], w);
      w = w - phi[896];
      w = w - phi[6016];
      const double kw = ws[58336] * w;
      out[896] = fma(kw, y[6016], out[896]);
      out[6016] = fma(kw, y[896], out[6016]);
      ws[287040] = fma(kw * y[896], y[6016], ws[287040]);
    }
    {
      double w = 0.0595 * phi[5536];
      w = fma(0.9048, phi[4992], w);
      w = fma(0.0357, phi[4768], w);
      w = w - phi[3456];
      w = w - phi[5984];
      const double kw = ws[58368] * w;
      out[3456] = fma(kw, y[5984], out[3456]);
      out[5984] = fma(kw, y[3456], out[5984]);
      ws[287072] = fma(kw * y[3456], y[5984], ws[287072]);
    }
    {
      double w = 0.0595 * phi[5312];
      w = fma(0.0018, phi[5088], w);
      w = fma(0.0001, phi[4768], w);
      w = fma(0.998, phi[5920], w);
      w = fma(0.998, phi[5984], w);
      w = fma(0.4693, phi[5376], w);
      w = fma(0.4693, phi[5248], w);
      w = fma(0.4693, phi[4512], w);
      w = fma(0.4693, phi[4320], w);
      w = w - phi[3456];
      w = w - phi[5824];
      const double kw = ws[58400] * w;
      out[3456] = fma(kw, y[5824], out[3456]);
      out[5824] = fma(kw, y[3456], out[5824]);
      ws[287104] = fma(kw * y[3456], y[5824], ws[287104]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.9405, phi[5984], w);
      w = fma(0.0595, phi[5312], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3456];
      w = w - phi[5952];
      const double kw = ws[58432] * w;
      out[3456] = fma(kw, y[5952], out[3456]);
      out[5952] = fma(kw, y[3456], out[5952]);
      ws[287136] = fma(kw * y[3456], y[5952], ws[287136]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(1.3105, phi[5984], w);
      w = fma(0.32, phi[5600], w);
      w = fma(0.0595, phi[5312], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3456];
      w = w - phi[5888];
      const double kw = ws[58464] * w;
      out[3456] = fma(kw, y[5888], out[3456]);
      out[5888] = fma(kw, y[3456], out[5888]);
      ws[287168] = fma(kw * y[3456], y[5888], ws[287168]);
    }
    {
      double w = 0.7 * phi[5888];
      w = fma(0.9405, phi[5984], w);
      w = fma(0.3, phi[5696], w);
      w = fma(0.0595, phi[5312], w);
      w = fma(0.4702, phi[5376], w);
      w = fma(0.4702, phi[5248], w);
      w = fma(0.4702, phi[4512], w);
      w = fma(0.4702, phi[4320], w);
      w = w - phi[3456];
      w = w - phi[5792];
      const double kw = ws[58496] * w;
      out[3456] = fma(kw, y[5792], out[3456]);
      out[5792] = fma(kw, y[3456], out[5792]);
      ws[287200] = fma(kw * y[3456], y[5792], ws[287200]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0854, phi[4768], w);
      w = fma(0.2581, phi[5472], w);
      w = fma(0.2581, phi[5280], w);
      w = fma(0.2581, phi[5568], w);
      w = fma(0.2581, phi[5760], w);
      w = fma(0.2581, phi[5888], w);
      w = fma(0.2581, phi[5632], w);
      w = fma(0.2581, phi[5408], w);
      w = fma(0.2581, phi[5152], w);
      w = w - phi[4768];
      w = w - phi[6016];
      const double kw = ws[58528] * w;
      out[4768] = fma(kw, y[6016], out[4768]);
      out[6016] = fma(kw, y[4768], out[6016]);
      ws[287232] = fma(kw * y[4768], y[6016], ws[287232]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.464, phi[4768], w);
      w = fma(0.1977, phi[4864], w);
      w = fma(0.0121, phi[4896], w);
      w = fma(0.0152, phi[4640], w);
      w = fma(0.0624, phi[4928], w);
      w = fma(0.0388, phi[4992], w);
      w = fma(0.0491, phi[5088], w);
      w = fma(0.0398, phi[5536], w);
      w = fma(0.0183, phi[5312], w);
      w = fma(0.0308, phi[4608], w);
      w = fma(0.004, phi[5728], w);
      w = fma(0.0794, phi[5472], w);
      w = fma(0.0794, phi[5280], w);
      w = fma(0.0794, phi[5504], w);
      w = fma(0.0794, phi[5568], w);
      w = fma(0.0794, phi[5760], w);
      w = fma(0.0794, phi[5888], w);
      w = fma(0.0794, phi[5632], w);
      w = fma(0.0794, phi[5408], w);
      w = fma(0.0794, phi[5152], w);
      w = fma(0.0794, phi[5120], w);
      w = fma(0.0794, phi[3776], w);
      w = w - phi[4864];
      w = w - phi[6016];
      const double kw = ws[58560] * w;
      out[4864] = fma(kw, y[6016], out[4864]);
      out[6016] = fma(kw, y[4864], out[6016]);
      ws[287264] = fma(kw * y[4864], y[6016], ws[287264]);
    }
}
__device__ __noinline__ void adj_jtv_1_11(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[6016];
      w = fma(0.1041, phi[4768], w);
      w = fma(0.5638, phi[4864], w);
      w = fma(0.2141, phi[4832], w);
      w = fma(0.0153, phi[4896], w);
      w = fma(0.0298, phi[4640], w);
      w = fma(0.0096, phi[4416], w);
      w = fma(0.0189, phi[4928], w);
      w = fma(0.0456, phi[4960], w);
      w = fma(0.0314, phi[4992], w);
      w = fma(0.0199, phi[4704], w);
      w = fma(0.0459, phi[5088], w);
      w = fma(0.0452, phi[5536], w);
      w = fma(0.0455, phi[5312], w);
      w = fma(0.0325, phi[4224], w);
      w = fma(0.0369, phi[3968], w);
      w = fma(0.0026, phi[4608], w);
      w = fma(0.039, phi[5472], w);
      w = fma(0.039, phi[5344], w);
      w = fma(0.039, phi[5280], w);
      w = fma(0.039, phi[5568], w);
      w = fma(0.039, phi[5760], w);
      w = fma(0.039, phi[5888], w);
      w = fma(0.039, phi[5632], w);
      w = fma(0.039, phi[5408], w);
      w = fma(0.039, phi[5152], w);
      w = fma(0.0925, phi[5120], w);
      w = w - phi[4832];
      w = w - phi[6016];
      const double kw = ws[58592] * w;
      out[4832] = fma(kw, y[6016], out[4832]);
      out[6016] = fma(kw, y[4832], out[6016]);
      ws[287296] = fma(kw * y[4832], y[6016], ws[287296]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.2036, phi[4768], w);
      w = fma(0.0071, phi[4864], w);
      w = fma(0.184, phi[5472], w);
      w = fma(0.184, phi[5280], w);
      w = fma(0.184, phi[5504], w);
      w = fma(0.184, phi[5568], w);
      w = fma(0.184, phi[5760], w);
      w = fma(0.184, phi[5888], w);
      w = fma(0.184, phi[5632], w);
      w = fma(0.184, phi[5408], w);
      w = fma(0.184, phi[5152], w);
      w = fma(0.184, phi[5120], w);
      w = w - phi[4896];
      w = w - phi[6016];
      const double kw = ws[58624] * w;
      out[4896] = fma(kw, y[6016], out[4896]);
      out[6016] = fma(kw, y[4896], out[6016]);
      ws[287328] = fma(kw * y[4896], y[6016], ws[287328]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.2792, phi[4768], w);
      w = fma(0.4025, phi[4864], w);
      w = fma(0.0088, phi[4832], w);
      w = fma(0.0319, phi[4896], w);
      w = fma(0.0076, phi[4640], w);
      w = fma(0.0194, phi[4928], w);
      w = fma(0.0104, phi[4960], w);
      w = fma(0.051, phi[4992], w);
      w = fma(0.0075, phi[4704], w);
      w = fma(0.0512, phi[5088], w);
      w = fma(0.0462, phi[5536], w);
      w = fma(0.0512, phi[5312], w);
      w = fma(0.0138, phi[4224], w);
      w = fma(0.0135, phi[5728], w);
      w = fma(0.0646, phi[5472], w);
      w = fma(0.0646, phi[5344], w);
      w = fma(0.0646, phi[5280], w);
      w = fma(0.0646, phi[5568], w);
      w = fma(0.0646, phi[5760], w);
      w = fma(0.0646, phi[5888], w);
      w = fma(0.0646, phi[5632], w);
      w = fma(0.0646, phi[5408], w);
      w = fma(0.0646, phi[5152], w);
      w = fma(0.1753, phi[5120], w);
      w = w - phi[4640];
      w = w - phi[6016];
      const double kw = ws[58656] * w;
      out[4640] = fma(kw, y[6016], out[4640]);
      out[6016] = fma(kw, y[4640], out[6016]);
      ws[287360] = fma(kw * y[4640], y[6016], ws[287360]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.0074, phi[4768], w);
      w = fma(0.119, phi[4864], w);
      w = fma(0.7261, phi[4832], w);
      w = fma(0.0122, phi[4896], w);
      w = fma(0.0305, phi[4640], w);
      w = fma(0.007, phi[4416], w);
      w = fma(0.0291, phi[4928], w);
      w = fma(0.0454, phi[4960], w);
      w = fma(0.0234, phi[4992], w);
      w = fma(0.0352, phi[4704], w);
      w = fma(0.0624, phi[5088], w);
      w = fma(0.0518, phi[5536], w);
      w = fma(0.0509, phi[5312], w);
      w = fma(0.0347, phi[4224], w);
      w = fma(0.0748, phi[3968], w);
      w = fma(0.0163, phi[4608], w);
      w = fma(0.0062, phi[5728], w);
      w = fma(0.0244, phi[5472], w);
      w = fma(0.0244, phi[5344], w);
      w = fma(0.0244, phi[5280], w);
      w = fma(0.0244, phi[5568], w);
      w = fma(0.0244, phi[5760], w);
      w = fma(0.0244, phi[5888], w);
      w = fma(0.0244, phi[5632], w);
      w = fma(0.0244, phi[5408], w);
      w = fma(0.0244, phi[5152], w);
      w = fma(0.0537, phi[5120], w);
      w = w - phi[4416];
      w = w - phi[6016];
      const double kw = ws[58688] * w;
      out[4416] = fma(kw, y[6016], out[4416]);
      out[6016] = fma(kw, y[4416], out[6016]);
      ws[287392] = fma(kw * y[4416], y[6016], ws[287392]);
    }
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
}
}  // namespace mech_cracmm2
