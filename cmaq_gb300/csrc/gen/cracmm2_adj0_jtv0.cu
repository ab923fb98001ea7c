// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_jtv_0_0(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[2336];
      w = w - phi[5184];
      const double kw = ws[42336] * w;
      out[5184] = out[5184] + kw;
      ws[271040] = fma(kw, y[5184], ws[271040]);
    }
    {
      double w = 1.0 * phi[576];
      w = w - phi[5184];
      const double kw = ws[42368] * w;
      out[5184] = out[5184] + kw;
      ws[271072] = fma(kw, y[5184], ws[271072]);
    }
    {
      double w = 2.0 * phi[6016];
      w = w - phi[4000];
      const double kw = ws[42400] * w;
      out[4000] = out[4000] + kw;
      ws[271104] = fma(kw, y[4000], ws[271104]);
    }
    {
      double w = 1.0 * phi[2336];
      w = fma(1.0, phi[5824], w);
      w = w - phi[5920];
      const double kw = ws[42432] * w;
      out[5920] = out[5920] + kw;
      ws[271136] = fma(kw, y[5920], ws[271136]);
    }
    {
      double w = 1.0 * phi[5824];
      w = w - phi[5952];
      const double kw = ws[42464] * w;
      out[5952] = out[5952] + kw;
      ws[271168] = fma(kw, y[5952], ws[271168]);
    }
    {
      double w = 1.0 * phi[2336];
      w = fma(1.0, phi[5920], w);
      w = w - phi[5952];
      const double kw = ws[42496] * w;
      out[5952] = out[5952] + kw;
      ws[271200] = fma(kw, y[5952], ws[271200]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5824], w);
      w = w - phi[1184];
      const double kw = ws[42528] * w;
      out[1184] = out[1184] + kw;
      ws[271232] = fma(kw, y[1184], ws[271232]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5920], w);
      w = w - phi[5024];
      const double kw = ws[42560] * w;
      out[5024] = out[5024] + kw;
      ws[271264] = fma(kw, y[5024], ws[271264]);
    }
    {
      double w = 0.2 * phi[6016];
      w = fma(0.8, phi[5984], w);
      w = fma(0.8, phi[5920], w);
      w = fma(0.2, phi[5952], w);
      w = w - phi[1280];
      const double kw = ws[42592] * w;
      out[1280] = out[1280] + kw;
      ws[271296] = fma(kw, y[1280], ws[271296]);
    }
    {
      double w = 1.0 * phi[5664];
      w = w - phi[5856];
      const double kw = ws[42624] * w;
      out[5856] = out[5856] + kw;
      ws[271328] = fma(kw, y[5856], ws[271328]);
    }
    {
      double w = 2.0 * phi[5984];
      w = fma(1.0, phi[5664], w);
      w = w - phi[5856];
      const double kw = ws[42656] * w;
      out[5856] = out[5856] + kw;
      ws[271360] = fma(kw, y[5856], ws[271360]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5888], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[5568];
      const double kw = ws[42688] * w;
      out[5568] = out[5568] + kw;
      ws[271392] = fma(kw, y[5568], ws[271392]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5632], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[5760];
      const double kw = ws[42720] * w;
      out[5760] = out[5760] + kw;
      ws[271424] = fma(kw, y[5760], ws[271424]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[5792], w);
      w = w - phi[4480];
      const double kw = ws[42752] * w;
      out[4480] = out[4480] + kw;
      ws[271456] = fma(kw, y[4480], ws[271456]);
    }
    {
      double w = 2.0 * phi[5888];
      w = fma(1.0, phi[5664], w);
      w = w - phi[4480];
      const double kw = ws[42784] * w;
      out[4480] = out[4480] + kw;
      ws[271488] = fma(kw, y[4480], ws[271488]);
    }
    {
      double w = 1.22 * phi[5984];
      w = fma(0.784, phi[5792], w);
      w = fma(1.22, phi[5664], w);
      w = fma(0.35, phi[5856], w);
      w = fma(0.434, phi[5760], w);
      w = fma(0.216, phi[5504], w);
      w = w - phi[3872];
      const double kw = ws[42816] * w;
      out[3872] = out[3872] + kw;
      ws[271520] = fma(kw, y[3872], ws[271520]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[3904], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[4544];
      const double kw = ws[42848] * w;
      out[4544] = out[4544] + kw;
      ws[271552] = fma(kw, y[4544], ws[271552]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[3904], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[4576];
      const double kw = ws[42880] * w;
      out[4576] = out[4576] + kw;
      ws[271584] = fma(kw, y[4576], ws[271584]);
    }
    {
      double w = 0.1 * phi[5888];
      w = fma(1.0, phi[5632], w);
      w = fma(0.9, phi[5792], w);
      w = fma(0.1, phi[5664], w);
      w = w - phi[5280];
      const double kw = ws[42912] * w;
      out[5280] = out[5280] + kw;
      ws[271616] = fma(kw, y[5280], ws[271616]);
    }
    {
      double w = 1.5 * phi[5632];
      w = fma(0.5, phi[5792], w);
      w = fma(0.5, phi[5664], w);
      w = w - phi[5504];
      const double kw = ws[42944] * w;
      out[5504] = out[5504] + kw;
      ws[271648] = fma(kw, y[5504], ws[271648]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5792], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[5344];
      const double kw = ws[42976] * w;
      out[5344] = out[5344] + kw;
      ws[271680] = fma(kw, y[5344], ws[271680]);
    }
    {
      double w = 0.34 * phi[6016];
      w = fma(0.66, phi[5984], w);
      w = fma(0.67, phi[5792], w);
      w = fma(0.33, phi[4672], w);
      w = fma(0.34, phi[5216], w);
      w = fma(0.67, phi[5664], w);
      w = fma(0.67, phi[5856], w);
      w = w - phi[4128];
      const double kw = ws[43008] * w;
      out[4128] = out[4128] + kw;
      ws[271712] = fma(kw, y[4128], ws[271712]);
    }
    {
      double w = 0.3 * phi[5888];
      w = fma(0.3, phi[4672], w);
      w = fma(0.7, phi[5664], w);
      w = fma(0.7, phi[3872], w);
      w = w - phi[4736];
      const double kw = ws[43040] * w;
      out[4736] = out[4736] + kw;
      ws[271744] = fma(kw, y[4736], ws[271744]);
    }
    {
      double w = 2.0 * phi[5664];
      w = w - phi[5376];
      const double kw = ws[43072] * w;
      out[5376] = out[5376] + kw;
      ws[271776] = fma(kw, y[5376], ws[271776]);
    }
    {
      double w = 1.0 * phi[5856];
      w = fma(1.0, phi[5664], w);
      w = w - phi[5376];
      const double kw = ws[43104] * w;
      out[5376] = out[5376] + kw;
      ws[271808] = fma(kw, y[5376], ws[271808]);
    }
    {
      double w = 2.0 * phi[5984];
      w = fma(2.0, phi[5664], w);
      w = w - phi[5376];
      const double kw = ws[43136] * w;
      out[5376] = out[5376] + kw;
      ws[271840] = fma(kw, y[5376], ws[271840]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5792], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[5248];
      const double kw = ws[43168] * w;
      out[5248] = out[5248] + kw;
      ws[271872] = fma(kw, y[5248], ws[271872]);
    }
    {
      double w = 1.5 * phi[5984];
      w = fma(0.25, phi[5792], w);
      w = fma(0.2, phi[5216], w);
      w = fma(1.0, phi[5664], w);
      w = fma(0.5, phi[5376], w);
      w = fma(0.5, phi[5248], w);
      w = w - phi[5472];
      const double kw = ws[43200] * w;
      out[5472] = out[5472] + kw;
      ws[271904] = fma(kw, y[5472], ws[271904]);
    }
    {
      double w = 1.5 * phi[5984];
      w = fma(0.25, phi[5792], w);
      w = fma(0.2, phi[5216], w);
      w = fma(1.0, phi[5664], w);
      w = fma(0.5, phi[5376], w);
      w = fma(0.5, phi[5248], w);
      w = w - phi[4320];
      const double kw = ws[43232] * w;
      out[4320] = out[4320] + kw;
      ws[271936] = fma(kw, y[4320], ws[271936]);
    }
    {
      double w = 1.0 * phi[3232];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[4448];
      const double kw = ws[43264] * w;
      out[4448] = out[4448] + kw;
      ws[271968] = fma(kw, y[4448], ws[271968]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[2816];
      const double kw = ws[43296] * w;
      out[2816] = out[2816] + kw;
      ws[272000] = fma(kw, y[2816], ws[272000]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5760], w);
      w = w - phi[5728];
      const double kw = ws[43328] * w;
      out[5728] = out[5728] + kw;
      ws[272032] = fma(kw, y[5728], ws[272032]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5760], w);
      w = w - phi[4096];
      const double kw = ws[43360] * w;
      out[4096] = out[4096] + kw;
      ws[272064] = fma(kw, y[4096], ws[272064]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5760], w);
      w = w - phi[4608];
      const double kw = ws[43392] * w;
      out[4608] = out[4608] + kw;
      ws[272096] = fma(kw, y[4608], ws[272096]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(1.0, phi[5888], w);
      w = w - phi[3680];
      const double kw = ws[43424] * w;
      out[3680] = out[3680] + kw;
      ws[272128] = fma(kw, y[3680], ws[272128]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(0.2, phi[5760], w);
      w = fma(0.8, phi[5504], w);
      w = w - phi[5440];
      const double kw = ws[43456] * w;
      out[5440] = out[5440] + kw;
      ws[272160] = fma(kw, y[5440], ws[272160]);
    }
    {
      double w = 1.0 * phi[5792];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1088];
      const double kw = ws[43488] * w;
      out[1088] = out[1088] + kw;
      ws[272192] = fma(kw, y[1088], ws[272192]);
    }
    {
      double w = 1.0 * phi[5888];
      w = fma(1.0, phi[5952], w);
      w = w - phi[1088];
      const double kw = ws[43520] * w;
      out[1088] = out[1088] + kw;
      ws[272224] = fma(kw, y[1088], ws[272224]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(0.67, phi[5504], w);
      w = fma(0.33, phi[3872], w);
      w = w - phi[4384];
      const double kw = ws[43552] * w;
      out[4384] = out[4384] + kw;
      ws[272256] = fma(kw, y[4384], ws[272256]);
    }
    {
      double w = 1.0 * phi[5344];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1696];
      const double kw = ws[43584] * w;
      out[1696] = out[1696] + kw;
      ws[272288] = fma(kw, y[1696], ws[272288]);
    }
    {
      double w = 1.0 * phi[5984];
      w = w - phi[5184];
      w = w - phi[6016];
      const double kw = ws[43616] * w;
      out[5184] = fma(kw, y[6016], out[5184]);
      out[6016] = fma(kw, y[5184], out[6016]);
      ws[272320] = fma(kw * y[5184], y[6016], ws[272320]);
    }
    {
      double w = 1.0 * phi[6016];
      w = w - phi[5184];
      w = w - phi[5984];
      const double kw = ws[43648] * w;
      out[5184] = fma(kw, y[5984], out[5184]);
      out[5984] = fma(kw, y[5184], out[5984]);
      ws[272352] = fma(kw * y[5184], y[5984], ws[272352]);
    }
    {
      double w = 1.0 * phi[5920];
      w = w - phi[5184];
      w = w - phi[5824];
      const double kw = ws[43680] * w;
      out[5184] = fma(kw, y[5824], out[5184]);
      out[5824] = fma(kw, y[5184], out[5824]);
      ws[272384] = fma(kw * y[5184], y[5824], ws[272384]);
    }
    {
      double w = 1.0 * phi[5952];
      w = w - phi[5184];
      w = w - phi[5920];
      const double kw = ws[43712] * w;
      out[5184] = fma(kw, y[5920], out[5184]);
      out[5920] = fma(kw, y[5184], out[5920]);
      ws[272416] = fma(kw * y[5184], y[5920], ws[272416]);
    }
    {
      double w = 1.0 * phi[5184];
      w = w - phi[2336];
      const double kw = ws[43744] * w;
      out[2336] = out[2336] + kw;
      ws[272448] = fma(kw, y[2336], ws[272448]);
    }
    {
      double w = -phi[2336];
      w = w - phi[5184];
      const double kw = ws[43776] * w;
      out[2336] = fma(kw, y[5184], out[2336]);
      out[5184] = fma(kw, y[2336], out[5184]);
      ws[272480] = fma(kw * y[2336], y[5184], ws[272480]);
    }
    {
      double w = 1.0 * phi[2336];
      w = w - phi[576];
      const double kw = ws[43808] * w;
      out[576] = out[576] + kw;
      ws[272512] = fma(kw, y[576], ws[272512]);
    }
    {
      double w = 1.0 * phi[2336];
      w = w - phi[576];
      const double kw = ws[43840] * w;
      out[576] = out[576] + kw;
      ws[272544] = fma(kw, y[576], ws[272544]);
    }
    {
      double w = 2.0 * phi[6016];
      w = w - phi[576];
      const double kw = ws[43872] * w;
      out[576] = out[576] + kw;
      ws[272576] = fma(kw, y[576], ws[272576]);
    }
    {
      double w = 1.0 * phi[5984];
      w = w - phi[6016];
      const double kw = ws[43904] * w;
      out[6016] = out[6016] + kw;
      ws[272608] = fma(kw, y[6016], ws[272608]);
    }
    {
      double w = -phi[6016];
      w = w - phi[5984];
      const double kw = ws[43936] * w;
      out[6016] = fma(kw, y[5984], out[6016]);
      out[5984] = fma(kw, y[6016], out[5984]);
      ws[272640] = fma(kw * y[6016], y[5984], ws[272640]);
    }
    {
      double w = 1.0 * phi[4000];
      w = w - phi[5984];
      w = w - phi[5984];
      const double kw = ws[43968] * w;
      out[5984] = fma(kw, y[5984], out[5984]);
      out[5984] = fma(kw, y[5984], out[5984]);
      ws[272672] = fma(kw * y[5984], y[5984], ws[272672]);
    }
    {
      double w = 1.0 * phi[4000];
      w = w - phi[5984];
      w = w - phi[5984];
      const double kw = ws[44000] * w;
      out[5984] = fma(kw, y[5984], out[5984]);
      out[5984] = fma(kw, y[5984], out[5984]);
      ws[272704] = fma(kw * y[5984], y[5984], ws[272704]);
    }
    {
      double w = 1.0 * phi[5984];
      w = w - phi[4000];
      w = w - phi[6016];
      const double kw = ws[44032] * w;
      out[4000] = fma(kw, y[6016], out[4000]);
      out[6016] = fma(kw, y[4000], out[6016]);
      ws[272736] = fma(kw * y[4000], y[6016], ws[272736]);
    }
    {
      double w = 1.0 * phi[5920];
      w = w - phi[5824];
      w = w - phi[2336];
      const double kw = ws[44064] * w;
      out[5824] = fma(kw, y[2336], out[5824]);
      out[2336] = fma(kw, y[5824], out[2336]);
      ws[272768] = fma(kw * y[5824], y[2336], ws[272768]);
    }
    {
      double w = 1.0 * phi[1184];
      w = w - phi[5824];
      w = w - phi[6016];
      const double kw = ws[44096] * w;
      out[5824] = fma(kw, y[6016], out[5824]);
      out[6016] = fma(kw, y[5824], out[6016]);
      ws[272800] = fma(kw * y[5824], y[6016], ws[272800]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[6016], w);
      w = w - phi[5824];
      w = w - phi[5984];
      const double kw = ws[44128] * w;
      out[5824] = fma(kw, y[5984], out[5824]);
      out[5984] = fma(kw, y[5824], out[5984]);
      ws[272832] = fma(kw * y[5824], y[5984], ws[272832]);
    }
}
__device__ __noinline__ void adj_jtv_0_1(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5024];
      w = w - phi[5824];
      w = w - phi[5984];
      const double kw = ws[44160] * w;
      out[5824] = fma(kw, y[5984], out[5824]);
      out[5984] = fma(kw, y[5824], out[5984]);
      ws[272864] = fma(kw * y[5824], y[5984], ws[272864]);
    }
    {
      double w = 2.0 * phi[5920];
      w = w - phi[5824];
      w = w - phi[5824];
      const double kw = ws[44192] * w;
      out[5824] = fma(kw, y[5824], out[5824]);
      out[5824] = fma(kw, y[5824], out[5824]);
      ws[272896] = fma(kw * y[5824], y[5824], ws[272896]);
    }
    {
      double w = 1.0 * phi[5920];
      w = w - phi[1184];
      w = w - phi[6016];
      const double kw = ws[44224] * w;
      out[1184] = fma(kw, y[6016], out[1184]);
      out[6016] = fma(kw, y[1184], out[6016]);
      ws[272928] = fma(kw * y[1184], y[6016], ws[272928]);
    }
    {
      double w = 1.0 * phi[5824];
      w = w - phi[5920];
      w = w - phi[2336];
      const double kw = ws[44256] * w;
      out[5920] = fma(kw, y[2336], out[5920]);
      out[2336] = fma(kw, y[5920], out[2336]);
      ws[272960] = fma(kw * y[5920], y[2336], ws[272960]);
    }
    {
      double w = 1.0 * phi[5952];
      w = w - phi[5920];
      w = w - phi[2336];
      const double kw = ws[44288] * w;
      out[5920] = fma(kw, y[2336], out[5920]);
      out[2336] = fma(kw, y[5920], out[2336]);
      ws[272992] = fma(kw * y[5920], y[2336], ws[272992]);
    }
    {
      double w = 1.0 * phi[5024];
      w = w - phi[5920];
      w = w - phi[6016];
      const double kw = ws[44320] * w;
      out[5920] = fma(kw, y[6016], out[5920]);
      out[6016] = fma(kw, y[5920], out[6016]);
      ws[273024] = fma(kw * y[5920], y[6016], ws[273024]);
    }
    {
      double w = 1.0 * phi[5952];
      w = w - phi[5024];
      w = w - phi[6016];
      const double kw = ws[44352] * w;
      out[5024] = fma(kw, y[6016], out[5024]);
      out[6016] = fma(kw, y[5024], out[6016]);
      ws[273056] = fma(kw * y[5024], y[6016], ws[273056]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = w - phi[5952];
      w = w - phi[6016];
      const double kw = ws[44384] * w;
      out[5952] = fma(kw, y[6016], out[5952]);
      out[6016] = fma(kw, y[5952], out[6016]);
      ws[273088] = fma(kw * y[5952], y[6016], ws[273088]);
    }
    {
      double w = 0.7 * phi[6016];
      w = fma(0.7, phi[5920], w);
      w = fma(0.3, phi[5024], w);
      w = w - phi[5952];
      w = w - phi[5984];
      const double kw = ws[44416] * w;
      out[5952] = fma(kw, y[5984], out[5952]);
      out[5984] = fma(kw, y[5952], out[5984]);
      ws[273120] = fma(kw * y[5952], y[5984], ws[273120]);
    }
    {
      double w = 2.0 * phi[5920];
      w = w - phi[5952];
      w = w - phi[5824];
      const double kw = ws[44448] * w;
      out[5952] = fma(kw, y[5824], out[5952]);
      out[5824] = fma(kw, y[5952], out[5824]);
      ws[273152] = fma(kw * y[5952], y[5824], ws[273152]);
    }
    {
      double w = 1.0 * phi[5824];
      w = fma(1.0, phi[5920], w);
      w = w - phi[5952];
      w = w - phi[5920];
      const double kw = ws[44480] * w;
      out[5952] = fma(kw, y[5920], out[5952]);
      out[5920] = fma(kw, y[5952], out[5920]);
      ws[273184] = fma(kw * y[5952], y[5920], ws[273184]);
    }
    {
      double w = 2.0 * phi[5920];
      w = w - phi[5952];
      w = w - phi[5952];
      const double kw = ws[44512] * w;
      out[5952] = fma(kw, y[5952], out[5952]);
      out[5952] = fma(kw, y[5952], out[5952]);
      ws[273216] = fma(kw * y[5952], y[5952], ws[273216]);
    }
    {
      double w = 1.0 * phi[1024];
      w = w - phi[5952];
      w = w - phi[5920];
      const double kw = ws[44544] * w;
      out[5952] = fma(kw, y[5920], out[5952]);
      out[5920] = fma(kw, y[5952], out[5920]);
      ws[273248] = fma(kw * y[5952], y[5920], ws[273248]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5952], w);
      w = w - phi[1024];
      const double kw = ws[44576] * w;
      out[1024] = out[1024] + kw;
      ws[273280] = fma(kw, y[1024], ws[273280]);
    }
    {
      double w = 2.0 * phi[5024];
      w = w - phi[1024];
      const double kw = ws[44608] * w;
      out[1024] = out[1024] + kw;
      ws[273312] = fma(kw, y[1024], ws[273312]);
    }
    {
      double w = 1.0 * phi[1280];
      w = w - phi[5920];
      w = w - phi[5984];
      const double kw = ws[44640] * w;
      out[5920] = fma(kw, y[5984], out[5920]);
      out[5984] = fma(kw, y[5920], out[5984]);
      ws[273344] = fma(kw * y[5920], y[5984], ws[273344]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1280];
      const double kw = ws[44672] * w;
      out[1280] = out[1280] + kw;
      ws[273376] = fma(kw, y[1280], ws[273376]);
    }
    {
      double w = 1.0 * phi[5920];
      w = w - phi[1280];
      w = w - phi[6016];
      const double kw = ws[44704] * w;
      out[1280] = fma(kw, y[6016], out[1280]);
      out[6016] = fma(kw, y[1280], out[6016]);
      ws[273408] = fma(kw * y[1280], y[6016], ws[273408]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[192], w);
      w = fma(1.0, phi[224], w);
      w = w - phi[160];
      w = w - phi[6016];
      const double kw = ws[44736] * w;
      out[160] = fma(kw, y[6016], out[160]);
      out[6016] = fma(kw, y[160], out[6016]);
      ws[273440] = fma(kw * y[160], y[6016], ws[273440]);
    }
    {
      double w = 1.0 * phi[5984];
      w = w - phi[5664];
      w = w - phi[6016];
      const double kw = ws[44768] * w;
      out[5664] = fma(kw, y[6016], out[5664]);
      out[6016] = fma(kw, y[5664], out[6016]);
      ws[273472] = fma(kw * y[5664], y[6016], ws[273472]);
    }
    {
      double w = 1.0 * phi[5888];
      w = w - phi[6016];
      const double kw = ws[44800] * w;
      out[6016] = out[6016] + kw;
      ws[273504] = fma(kw, y[6016], ws[273504]);
    }
    {
      double w = 1.0 * phi[5632];
      w = w - phi[1888];
      w = w - phi[6016];
      const double kw = ws[44832] * w;
      out[1888] = fma(kw, y[6016], out[1888]);
      out[6016] = fma(kw, y[1888], out[6016]);
      ws[273536] = fma(kw * y[1888], y[6016], ws[273536]);
    }
    {
      double w = 1.0 * phi[5408];
      w = fma(2.81e-05, phi[3616], w);
      w = w - phi[2176];
      w = w - phi[6016];
      const double kw = ws[44864] * w;
      out[2176] = fma(kw, y[6016], out[2176]);
      out[6016] = fma(kw, y[2176], out[6016]);
      ws[273568] = fma(kw * y[2176], y[6016], ws[273568]);
    }
    {
      double w = 1.0 * phi[5120];
      w = fma(0.00134, phi[3616], w);
      w = w - phi[1120];
      w = w - phi[6016];
      const double kw = ws[44896] * w;
      out[1120] = fma(kw, y[6016], out[1120]);
      out[6016] = fma(kw, y[1120], out[6016]);
      ws[273600] = fma(kw * y[1120], y[6016], ws[273600]);
    }
    {
      double w = 1.0 * phi[3008];
      w = w - phi[2240];
      w = w - phi[6016];
      const double kw = ws[44928] * w;
      out[2240] = fma(kw, y[6016], out[2240]);
      out[6016] = fma(kw, y[2240], out[6016]);
      ws[273632] = fma(kw * y[2240], y[6016], ws[273632]);
    }
    {
      double w = 1.0 * phi[3200];
      w = w - phi[2752];
      w = w - phi[6016];
      const double kw = ws[44960] * w;
      out[2752] = fma(kw, y[6016], out[2752]);
      out[6016] = fma(kw, y[2752], out[6016]);
      ws[273664] = fma(kw * y[2752], y[6016], ws[273664]);
    }
    {
      double w = 1.0 * phi[3328];
      w = w - phi[1152];
      w = w - phi[6016];
      const double kw = ws[44992] * w;
      out[1152] = fma(kw, y[6016], out[1152]);
      out[6016] = fma(kw, y[1152], out[6016]);
      ws[273696] = fma(kw * y[1152], y[6016], ws[273696]);
    }
    {
      double w = 0.65 * phi[6016];
      w = fma(0.35, phi[5984], w);
      w = fma(0.35, phi[5664], w);
      w = fma(0.65, phi[5376], w);
      w = fma(0.35, phi[4352], w);
      w = w - phi[256];
      w = w - phi[6016];
      const double kw = ws[45024] * w;
      out[256] = fma(kw, y[6016], out[256]);
      out[6016] = fma(kw, y[256], out[6016]);
      ws[273728] = fma(kw * y[256], y[6016], ws[273728]);
    }
    {
      double w = 0.47 * phi[3360];
      w = fma(0.53, phi[1248], w);
      w = fma(0.53, phi[5984], w);
      w = w - phi[1216];
      w = w - phi[6016];
      const double kw = ws[45056] * w;
      out[1216] = fma(kw, y[6016], out[1216]);
      out[6016] = fma(kw, y[1216], out[6016]);
      ws[273760] = fma(kw * y[1216], y[6016], ws[273760]);
    }
    {
      double w = 0.82 * phi[3296];
      w = fma(0.18, phi[2944], w);
      w = fma(0.18, phi[5984], w);
      w = w - phi[288];
      w = w - phi[6016];
      const double kw = ws[45088] * w;
      out[288] = fma(kw, y[6016], out[288]);
      out[6016] = fma(kw, y[288], out[6016]);
      ws[273792] = fma(kw * y[288], y[6016], ws[273792]);
    }
    {
      double w = 0.83 * phi[3104];
      w = fma(0.17, phi[2944], w);
      w = fma(0.17, phi[5984], w);
      w = w - phi[320];
      w = w - phi[6016];
      const double kw = ws[45120] * w;
      out[320] = fma(kw, y[6016], out[320]);
      out[6016] = fma(kw, y[320], out[6016]);
      ws[273824] = fma(kw * y[320], y[6016], ws[273824]);
    }
    {
      double w = 0.82 * phi[3264];
      w = fma(0.18, phi[2944], w);
      w = fma(0.18, phi[5984], w);
      w = w - phi[352];
      w = w - phi[6016];
      const double kw = ws[45152] * w;
      out[352] = fma(kw, y[6016], out[352]);
      out[6016] = fma(kw, y[352], out[6016]);
      ws[273856] = fma(kw * y[352], y[6016], ws[273856]);
    }
    {
      double w = 0.25 * phi[6016];
      w = fma(0.25, phi[5984], w);
      w = fma(0.4, phi[5888], w);
      w = fma(0.018, phi[5792], w);
      w = fma(0.1, phi[4672], w);
      w = fma(0.09, phi[4000], w);
      w = fma(0.22, phi[5664], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.3, phi[4128], w);
      w = fma(0.14, phi[4736], w);
      w = fma(0.28, phi[4352], w);
      w = fma(0.153, phi[2752], w);
      w = w - phi[1312];
      w = w - phi[5184];
      const double kw = ws[45184] * w;
      out[1312] = fma(kw, y[5184], out[1312]);
      out[5184] = fma(kw, y[1312], out[5184]);
      ws[273888] = fma(kw * y[1312], y[5184], ws[273888]);
    }
    {
      double w = 0.4 * phi[5920];
      w = fma(0.045, phi[2784], w);
      w = fma(0.35, phi[5856], w);
      w = fma(0.555, phi[1632], w);
      w = fma(0.26, phi[4736], w);
      w = fma(0.028, phi[4128], w);
      w = w - phi[1312];
      w = w - phi[5952];
      const double kw = ws[45216] * w;
      out[1312] = fma(kw, y[5952], out[1312]);
      out[5952] = fma(kw, y[1312], out[5952]);
      ws[273920] = fma(kw * y[1312], y[5952], ws[273920]);
    }
    {
      double w = 1.0 * phi[4288];
      w = fma(0.25, phi[5856], w);
      w = fma(0.03, phi[4128], w);
      w = fma(0.05, phi[5248], w);
      w = w - phi[1312];
      w = w - phi[6016];
      const double kw = ws[45248] * w;
      out[1312] = fma(kw, y[6016], out[1312]);
      out[6016] = fma(kw, y[1312], out[6016]);
      ws[273952] = fma(kw * y[1312], y[6016], ws[273952]);
    }
    {
      double w = 1.0 * phi[1344];
      w = fma(0.07, phi[5984], w);
      w = fma(0.5, phi[6016], w);
      w = w - phi[4288];
      w = w - phi[5984];
      const double kw = ws[45280] * w;
      out[4288] = fma(kw, y[5984], out[4288]);
      out[5984] = fma(kw, y[4288], out[5984]);
      ws[273984] = fma(kw * y[4288], y[5984], ws[273984]);
    }
    {
      double w = 0.13 * phi[2784];
      w = fma(0.4, phi[5856], w);
      w = fma(0.88, phi[5984], w);
      w = fma(0.87, phi[5920], w);
      w = fma(0.18, phi[4128], w);
      w = fma(0.51, phi[4736], w);
      w = w - phi[4288];
      w = w - phi[5824];
      const double kw = ws[45312] * w;
      out[4288] = fma(kw, y[5824], out[4288]);
      out[5824] = fma(kw, y[4288], out[5824]);
      ws[274016] = fma(kw * y[4288], y[5824], ws[274016]);
    }
    {
      double w = 1.0 * phi[4288];
      w = w - phi[1344];
      w = w - phi[6016];
      const double kw = ws[45344] * w;
      out[1344] = fma(kw, y[6016], out[1344]);
      out[6016] = fma(kw, y[1344], out[6016]);
      ws[274048] = fma(kw * y[1344], y[6016], ws[274048]);
    }
    {
      double w = 0.04 * phi[5248];
      w = fma(0.02, phi[5376], w);
      w = fma(0.13, phi[4736], w);
      w = fma(0.44, phi[1376], w);
      w = fma(0.11, phi[5792], w);
      w = fma(0.03, phi[4128], w);
      w = fma(2.0, phi[6016], w);
      w = fma(0.34, phi[5984], w);
      w = fma(0.14, phi[1664], w);
      w = fma(1.0, phi[5664], w);
      w = w - phi[1344];
      w = w - phi[6016];
      const double kw = ws[45376] * w;
      out[1344] = fma(kw, y[6016], out[1344]);
      out[6016] = fma(kw, y[1344], out[6016]);
      ws[274080] = fma(kw * y[1344], y[6016], ws[274080]);
    }
    {
      double w = 0.45 * phi[6016];
      w = fma(0.95, phi[2208], w);
      w = fma(0.02, phi[1664], w);
      w = w - phi[1632];
      w = w - phi[5984];
      const double kw = ws[45408] * w;
      out[1632] = fma(kw, y[5984], out[1632]);
      out[5984] = fma(kw, y[1632], out[5984]);
      ws[274112] = fma(kw * y[1632], y[5984], ws[274112]);
    }
    {
      double w = 0.15 * phi[4736];
      w = fma(0.65, phi[2208], w);
      w = fma(0.05, phi[2784], w);
      w = fma(0.2, phi[5856], w);
      w = fma(1.3, phi[5920], w);
      w = w - phi[1632];
      w = w - phi[5824];
      const double kw = ws[45440] * w;
      out[1632] = fma(kw, y[5824], out[1632]);
      out[5824] = fma(kw, y[1632], out[5824]);
      ws[274144] = fma(kw * y[1632], y[5824], ws[274144]);
    }
    {
      double w = 1.0 * phi[6016];
      w = fma(0.35, phi[2208], w);
      w = fma(0.17, phi[1376], w);
      w = fma(0.65, phi[5920], w);
      w = w - phi[2784];
      w = w - phi[6016];
      const double kw = ws[45472] * w;
      out[2784] = fma(kw, y[6016], out[2784]);
      out[6016] = fma(kw, y[2784], out[6016]);
      ws[274176] = fma(kw * y[2784], y[6016], ws[274176]);
    }
    {
      double w = 1.0 * phi[5664];
      w = fma(1.0, phi[5920], w);
      w = fma(0.3, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[6016];
      w = w - phi[2208];
      const double kw = ws[45504] * w;
      out[6016] = fma(kw, y[2208], out[6016]);
      out[2208] = fma(kw, y[6016], out[2208]);
      ws[274208] = fma(kw * y[6016], y[2208], ws[274208]);
    }
    {
      double w = 1.0 * phi[5024];
      w = fma(1.0, phi[5056], w);
      w = w - phi[2784];
      const double kw = ws[45536] * w;
      out[2784] = out[2784] + kw;
      ws[274240] = fma(kw, y[2784], ws[274240]);
    }
    {
      double w = 0.57 * phi[4128];
      w = fma(0.43, phi[4736], w);
      w = w - phi[1664];
      w = w - phi[6016];
      const double kw = ws[45568] * w;
      out[1664] = fma(kw, y[6016], out[1664]);
      out[6016] = fma(kw, y[1664], out[6016]);
      ws[274272] = fma(kw * y[1664], y[6016], ws[274272]);
    }
    {
      double w = 0.975 * phi[4160];
      w = fma(0.025, phi[3744], w);
      w = w - phi[1408];
      w = w - phi[6016];
      const double kw = ws[45600] * w;
      out[1408] = fma(kw, y[6016], out[1408]);
      out[6016] = fma(kw, y[1408], out[6016]);
      ws[274304] = fma(kw * y[1408], y[6016], ws[274304]);
    }
    {
      double w = 0.945 * phi[4192];
      w = fma(0.055, phi[3936], w);
      w = w - phi[1440];
      w = w - phi[6016];
      const double kw = ws[45632] * w;
      out[1440] = fma(kw, y[6016], out[1440]);
      out[6016] = fma(kw, y[1440], out[6016]);
      ws[274336] = fma(kw * y[1440], y[6016], ws[274336]);
    }
    {
      double w = 0.23 * phi[2560];
      w = fma(0.77, phi[4800], w);
      w = w - phi[4544];
      w = w - phi[6016];
      const double kw = ws[45664] * w;
      out[4544] = fma(kw, y[6016], out[4544]);
      out[6016] = fma(kw, y[4544], out[6016]);
      ws[274368] = fma(kw * y[4544], y[6016], ws[274368]);
    }
}
__device__ __noinline__ void adj_jtv_0_2(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 0.83 * phi[1728];
      w = fma(0.17, phi[4800], w);
      w = w - phi[4576];
      w = w - phi[6016];
      const double kw = ws[45696] * w;
      out[4576] = fma(kw, y[6016], out[4576]);
      out[6016] = fma(kw, y[4576], out[6016]);
      ws[274400] = fma(kw * y[4576], y[6016], ws[274400]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5664], w);
      w = w - phi[5856];
      w = w - phi[6016];
      const double kw = ws[45728] * w;
      out[5856] = fma(kw, y[6016], out[5856]);
      out[6016] = fma(kw, y[5856], out[6016]);
      ws[274432] = fma(kw * y[5856], y[6016], ws[274432]);
    }
    {
      double w = 1.0 * phi[5792];
      w = w - phi[5568];
      w = w - phi[6016];
      const double kw = ws[45760] * w;
      out[5568] = fma(kw, y[6016], out[5568]);
      out[6016] = fma(kw, y[5568], out[6016]);
      ws[274464] = fma(kw * y[5568], y[6016], ws[274464]);
    }
    {
      double w = 1.0 * phi[4800];
      w = w - phi[5760];
      w = w - phi[6016];
      const double kw = ws[45792] * w;
      out[5760] = fma(kw, y[6016], out[5760]);
      out[6016] = fma(kw, y[5760], out[6016]);
      ws[274496] = fma(kw * y[5760], y[6016], ws[274496]);
    }
    {
      double w = 1.0 * phi[2848];
      w = w - phi[4480];
      w = w - phi[6016];
      const double kw = ws[45824] * w;
      out[4480] = fma(kw, y[6016], out[4480]);
      out[6016] = fma(kw, y[4480], out[6016]);
      ws[274528] = fma(kw * y[4480], y[6016], ws[274528]);
    }
    {
      double w = 1.0 * phi[5152];
      w = w - phi[5280];
      w = w - phi[6016];
      const double kw = ws[45856] * w;
      out[5280] = fma(kw, y[6016], out[5280]);
      out[6016] = fma(kw, y[5280], out[6016]);
      ws[274560] = fma(kw * y[5280], y[6016], ws[274560]);
    }
    {
      double w = 1.0 * phi[3776];
      w = w - phi[5504];
      w = w - phi[6016];
      const double kw = ws[45888] * w;
      out[5504] = fma(kw, y[6016], out[5504]);
      out[6016] = fma(kw, y[5504], out[6016]);
      ws[274592] = fma(kw * y[5504], y[6016], ws[274592]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5248], w);
      w = w - phi[5344];
      w = w - phi[6016];
      const double kw = ws[45920] * w;
      out[5344] = fma(kw, y[6016], out[5344]);
      out[6016] = fma(kw, y[5344], out[6016]);
      ws[274624] = fma(kw * y[5344], y[6016], ws[274624]);
    }
    {
      double w = 0.57 * phi[4672];
      w = fma(0.43, phi[3520], w);
      w = w - phi[4128];
      w = w - phi[6016];
      const double kw = ws[45952] * w;
      out[4128] = fma(kw, y[6016], out[4128]);
      out[6016] = fma(kw, y[4128], out[6016]);
      ws[274656] = fma(kw * y[4128], y[6016], ws[274656]);
    }
    {
      double w = 1.0 * phi[2880];
      w = w - phi[4736];
      w = w - phi[6016];
      const double kw = ws[45984] * w;
      out[4736] = fma(kw, y[6016], out[4736]);
      out[6016] = fma(kw, y[4736], out[6016]);
      ws[274688] = fma(kw * y[4736], y[6016], ws[274688]);
    }
    {
      double w = 0.313 * phi[5792];
      w = fma(0.687, phi[2912], w);
      w = w - phi[3872];
      w = w - phi[6016];
      const double kw = ws[46016] * w;
      out[3872] = fma(kw, y[6016], out[3872]);
      out[6016] = fma(kw, y[3872], out[6016]);
      ws[274720] = fma(kw * y[3872], y[6016], ws[274720]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(2.0, phi[5664], w);
      w = w - phi[5376];
      w = w - phi[6016];
      const double kw = ws[46048] * w;
      out[5376] = fma(kw, y[6016], out[5376]);
      out[6016] = fma(kw, y[5376], out[6016]);
      ws[274752] = fma(kw * y[5376], y[6016], ws[274752]);
    }
    {
      double w = 1.0 * phi[5792];
      w = fma(1.0, phi[5664], w);
      w = w - phi[5248];
      w = w - phi[6016];
      const double kw = ws[46080] * w;
      out[5248] = fma(kw, y[6016], out[5248]);
      out[6016] = fma(kw, y[5248], out[6016]);
      ws[274784] = fma(kw * y[5248], y[6016], ws[274784]);
    }
    {
      double w = 0.52 * phi[5984];
      w = fma(0.33, phi[5664], w);
      w = fma(0.4, phi[5760], w);
      w = fma(0.78, phi[5504], w);
      w = fma(0.1, phi[5376], w);
      w = fma(0.01, phi[5248], w);
      w = w - phi[5472];
      w = w - phi[6016];
      const double kw = ws[46112] * w;
      out[5472] = fma(kw, y[6016], out[5472]);
      out[6016] = fma(kw, y[5472], out[6016]);
      ws[274816] = fma(kw * y[5472], y[6016], ws[274816]);
    }
    {
      double w = 0.52 * phi[5984];
      w = fma(0.33, phi[5664], w);
      w = fma(0.13, phi[5280], w);
      w = fma(0.1, phi[5376], w);
      w = fma(0.01, phi[5248], w);
      w = fma(0.78, phi[5728], w);
      w = w - phi[4320];
      w = w - phi[6016];
      const double kw = ws[46144] * w;
      out[4320] = fma(kw, y[6016], out[4320]);
      out[6016] = fma(kw, y[4320], out[6016]);
      ws[274848] = fma(kw * y[4320], y[6016], ws[274848]);
    }
    {
      double w = 0.56 * phi[5984];
      w = fma(0.21, phi[4672], w);
      w = fma(0.11, phi[5664], w);
      w = fma(0.27, phi[5376], w);
      w = fma(0.01, phi[5248], w);
      w = fma(0.79, phi[5728], w);
      w = w - phi[3584];
      w = w - phi[6016];
      const double kw = ws[46176] * w;
      out[3584] = fma(kw, y[6016], out[3584]);
      out[6016] = fma(kw, y[3584], out[6016]);
      ws[274880] = fma(kw * y[3584], y[6016], ws[274880]);
    }
    {
      double w = 1.0 * phi[2592];
      w = w - phi[4448];
      w = w - phi[6016];
      const double kw = ws[46208] * w;
      out[4448] = fma(kw, y[6016], out[4448]);
      out[6016] = fma(kw, y[4448], out[6016]);
      ws[274912] = fma(kw * y[4448], y[6016], ws[274912]);
    }
    {
      double w = 0.152 * phi[3616];
      w = fma(0.619, phi[5984], w);
      w = fma(0.17, phi[3648], w);
      w = fma(0.059, phi[3232], w);
      w = fma(0.619, phi[1760], w);
      w = w - phi[1248];
      w = w - phi[6016];
      const double kw = ws[46240] * w;
      out[1248] = fma(kw, y[6016], out[1248]);
      out[6016] = fma(kw, y[1248], out[6016]);
      ws[274944] = fma(kw * y[1248], y[6016], ws[274944]);
    }
    {
      double w = 0.2 * phi[3616];
      w = fma(0.584, phi[5984], w);
      w = fma(0.16, phi[3648], w);
      w = fma(0.056, phi[3232], w);
      w = fma(0.584, phi[1760], w);
      w = w - phi[2944];
      w = w - phi[6016];
      const double kw = ws[46272] * w;
      out[2944] = fma(kw, y[6016], out[2944]);
      out[6016] = fma(kw, y[2944], out[6016]);
      ws[274976] = fma(kw * y[2944], y[6016], ws[274976]);
    }
    {
      double w = 1.0 * phi[3808];
      w = w - phi[1760];
      w = w - phi[6016];
      const double kw = ws[46304] * w;
      out[1760] = fma(kw, y[6016], out[1760]);
      out[6016] = fma(kw, y[1760], out[6016]);
      ws[275008] = fma(kw * y[1760], y[6016], ws[275008]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = w - phi[5600];
      w = w - phi[6016];
      const double kw = ws[46336] * w;
      out[5600] = fma(kw, y[6016], out[5600]);
      out[6016] = fma(kw, y[5600], out[6016]);
      ws[275040] = fma(kw * y[5600], y[6016], ws[275040]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5568], w);
      w = w - phi[1472];
      w = w - phi[6016];
      const double kw = ws[46368] * w;
      out[1472] = fma(kw, y[6016], out[1472]);
      out[6016] = fma(kw, y[1472], out[6016]);
      ws[275072] = fma(kw * y[1472], y[6016], ws[275072]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(0.719, phi[5760], w);
      w = fma(0.184, phi[5568], w);
      w = w - phi[5056];
      w = w - phi[6016];
      const double kw = ws[46400] * w;
      out[5056] = fma(kw, y[6016], out[5056]);
      out[6016] = fma(kw, y[5056], out[6016]);
      ws[275104] = fma(kw * y[5056], y[6016], ws[275104]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5760], w);
      w = w - phi[1504];
      w = w - phi[6016];
      const double kw = ws[46432] * w;
      out[1504] = fma(kw, y[6016], out[1504]);
      out[6016] = fma(kw, y[1504], out[6016]);
      ws[275136] = fma(kw * y[1504], y[6016], ws[275136]);
    }
    {
      double w = 0.35 * phi[6016];
      w = fma(0.65, phi[5888], w);
      w = fma(0.35, phi[5856], w);
      w = w - phi[2816];
      w = w - phi[6016];
      const double kw = ws[46464] * w;
      out[2816] = fma(kw, y[6016], out[2816]);
      out[6016] = fma(kw, y[2816], out[6016]);
      ws[275168] = fma(kw * y[2816], y[6016], ws[275168]);
    }
    {
      double w = 0.01 * phi[6016];
      w = fma(0.44, phi[5408], w);
      w = fma(0.07, phi[5216], w);
      w = fma(0.08, phi[5760], w);
      w = fma(0.41, phi[5504], w);
      w = w - phi[5728];
      w = w - phi[6016];
      const double kw = ws[46496] * w;
      out[5728] = fma(kw, y[6016], out[5728]);
      out[6016] = fma(kw, y[5728], out[6016]);
      ws[275200] = fma(kw * y[5728], y[6016], ws[275200]);
    }
    {
      double w = 0.01 * phi[6016];
      w = fma(0.44, phi[3904], w);
      w = fma(0.07, phi[5216], w);
      w = fma(0.08, phi[5760], w);
      w = fma(0.41, phi[5504], w);
      w = w - phi[4096];
      w = w - phi[6016];
      const double kw = ws[46528] * w;
      out[4096] = fma(kw, y[6016], out[4096]);
      out[6016] = fma(kw, y[4096], out[6016]);
      ws[275232] = fma(kw * y[4096], y[6016], ws[275232]);
    }
    {
      double w = 0.01 * phi[6016];
      w = fma(0.44, phi[3904], w);
      w = fma(0.07, phi[5216], w);
      w = fma(0.08, phi[5760], w);
      w = fma(0.41, phi[5504], w);
      w = w - phi[4608];
      w = w - phi[6016];
      const double kw = ws[46560] * w;
      out[4608] = fma(kw, y[6016], out[4608]);
      out[6016] = fma(kw, y[4608], out[6016]);
      ws[275264] = fma(kw * y[4608], y[6016], ws[275264]);
    }
    {
      double w = 1.0 * phi[4672];
      w = w - phi[1792];
      w = w - phi[6016];
      const double kw = ws[46592] * w;
      out[1792] = fma(kw, y[6016], out[1792]);
      out[6016] = fma(kw, y[1792], out[6016]);
      ws[275296] = fma(kw * y[1792], y[6016], ws[275296]);
    }
    {
      double w = 1.0 * phi[5984];
      w = w - phi[4352];
      w = w - phi[6016];
      const double kw = ws[46624] * w;
      out[4352] = fma(kw, y[6016], out[4352]);
      out[6016] = fma(kw, y[4352], out[6016]);
      ws[275328] = fma(kw * y[4352], y[6016], ws[275328]);
    }
    {
      double w = 0.64 * phi[5888];
      w = fma(0.36, phi[2976], w);
      w = w - phi[5696];
      w = w - phi[6016];
      const double kw = ws[46656] * w;
      out[5696] = fma(kw, y[6016], out[5696]);
      out[6016] = fma(kw, y[5696], out[6016]);
      ws[275360] = fma(kw * y[5696], y[6016], ws[275360]);
    }
    {
      double w = 0.35 * phi[6016];
      w = fma(0.65, phi[5792], w);
      w = fma(0.35, phi[5216], w);
      w = fma(0.35, phi[5856], w);
      w = w - phi[3680];
      w = w - phi[6016];
      const double kw = ws[46688] * w;
      out[3680] = fma(kw, y[6016], out[3680]);
      out[6016] = fma(kw, y[3680], out[6016]);
      ws[275392] = fma(kw * y[3680], y[6016], ws[275392]);
    }
    {
      double w = 1.0 * phi[5216];
      w = fma(1.0, phi[5952], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[1088];
      w = w - phi[6016];
      const double kw = ws[46720] * w;
      out[1088] = fma(kw, y[6016], out[1088]);
      out[6016] = fma(kw, y[1088], out[6016]);
      ws[275424] = fma(kw * y[1088], y[6016], ws[275424]);
    }
    {
      double w = 1.0 * phi[5216];
      w = fma(1.0, phi[5952], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[1536];
      w = w - phi[6016];
      const double kw = ws[46752] * w;
      out[1536] = fma(kw, y[6016], out[1536]);
      out[6016] = fma(kw, y[1536], out[6016]);
      ws[275456] = fma(kw * y[1536], y[6016], ws[275456]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5344], w);
      w = w - phi[1824];
      w = w - phi[6016];
      const double kw = ws[46784] * w;
      out[1824] = fma(kw, y[6016], out[1824]);
      out[6016] = fma(kw, y[1824], out[6016]);
      ws[275488] = fma(kw * y[1824], y[6016], ws[275488]);
    }
    {
      double w = 1.0 * phi[5408];
      w = fma(1.0, phi[5920], w);
      w = w - phi[5440];
      w = w - phi[6016];
      const double kw = ws[46816] * w;
      out[5440] = fma(kw, y[6016], out[5440]);
      out[6016] = fma(kw, y[5440], out[6016]);
      ws[275520] = fma(kw * y[5440], y[6016], ws[275520]);
    }
    {
      double w = 0.33 * phi[1696];
      w = fma(0.67, phi[5920], w);
      w = fma(0.27, phi[4544], w);
      w = fma(0.38, phi[5504], w);
      w = fma(0.21, phi[5856], w);
      w = fma(0.02, phi[5760], w);
      w = w - phi[4384];
      w = w - phi[6016];
      const double kw = ws[46848] * w;
      out[4384] = fma(kw, y[6016], out[4384]);
      out[6016] = fma(kw, y[4384], out[6016]);
      ws[275552] = fma(kw * y[4384], y[6016], ws[275552]);
    }
    {
      double w = 1.0 * phi[5344];
      w = fma(1.0, phi[5952], w);
      w = w - phi[1696];
      w = w - phi[6016];
      const double kw = ws[46880] * w;
      out[1696] = fma(kw, y[6016], out[1696]);
      out[6016] = fma(kw, y[1696], out[6016]);
      ws[275584] = fma(kw * y[1696], y[6016], ws[275584]);
    }
    {
      double w = 0.08 * phi[6016];
      w = fma(0.15, phi[5984], w);
      w = fma(0.43, phi[5664], w);
      w = fma(1.0, phi[5856], w);
      w = fma(0.37, phi[4352], w);
      w = w - phi[2240];
      w = w - phi[5184];
      const double kw = ws[46912] * w;
      out[2240] = fma(kw, y[5184], out[2240]);
      out[5184] = fma(kw, y[2240], out[5184]);
      ws[275616] = fma(kw * y[2240], y[5184], ws[275616]);
    }
    {
      double w = 0.22 * phi[6016];
      w = fma(0.32, phi[5984], w);
      w = fma(0.08, phi[5888], w);
      w = fma(0.06, phi[5632], w);
      w = fma(0.04, phi[5408], w);
      w = fma(0.02, phi[5120], w);
      w = fma(0.068, phi[4000], w);
      w = fma(0.43, phi[5664], w);
      w = fma(0.02, phi[1888], w);
      w = fma(0.015, phi[2176], w);
      w = fma(0.006, phi[1120], w);
      w = fma(0.032, phi[1216], w);
      w = fma(0.56, phi[5856], w);
      w = fma(0.01, phi[5568], w);
      w = fma(0.44, phi[5760], w);
      w = fma(0.03, phi[4480], w);
      w = fma(0.02, phi[4448], w);
      w = fma(0.06, phi[5280], w);
      w = fma(0.01, phi[5344], w);
      w = fma(0.03, phi[4352], w);
      w = fma(0.06, phi[5696], w);
      w = w - phi[2752];
      w = w - phi[5184];
      const double kw = ws[46944] * w;
      out[2752] = fma(kw, y[5184], out[2752]);
      out[5184] = fma(kw, y[2752], out[5184]);
      ws[275648] = fma(kw * y[2752], y[5184], ws[275648]);
    }
    {
      double w = 0.46 * phi[6016];
      w = fma(0.07, phi[5984], w);
      w = fma(0.32, phi[5888], w);
      w = fma(0.07, phi[5632], w);
      w = fma(0.04, phi[5408], w);
      w = fma(0.09, phi[5792], w);
      w = fma(0.37, phi[5664], w);
      w = fma(0.026, phi[4000], w);
      w = fma(0.01, phi[1888], w);
      w = fma(0.01, phi[2176], w);
      w = fma(0.09, phi[5856], w);
      w = fma(0.457, phi[5568], w);
      w = fma(0.73, phi[5760], w);
      w = fma(0.11, phi[4480], w);
      w = fma(0.017, phi[5504], w);
      w = fma(0.044, phi[5344], w);
      w = fma(0.017, phi[5696], w);
      w = w - phi[1152];
      w = w - phi[5184];
      const double kw = ws[46976] * w;
      out[1152] = fma(kw, y[5184], out[1152]);
      out[5184] = fma(kw, y[1152], out[5184]);
      ws[275680] = fma(kw * y[1152], y[5184], ws[275680]);
    }
    {
      double w = 0.6055 * phi[6016];
      w = fma(0.2145, phi[2560], w);
      w = fma(0.255, phi[4000], w);
      w = fma(0.2535, phi[4544], w);
      w = fma(0.0065, phi[5696], w);
      w = fma(0.1105, phi[5984], w);
      w = fma(0.1105, phi[5664], w);
      w = fma(0.459, phi[5856], w);
      w = fma(0.2805, phi[4800], w);
      w = fma(0.1785, phi[5504], w);
      w = fma(0.0665, phi[2176], w);
      w = fma(0.0385, phi[2816], w);
      w = fma(0.028, phi[4352], w);
      w = w - phi[1408];
      w = w - phi[5184];
      const double kw = ws[47008] * w;
      out[1408] = fma(kw, y[5184], out[1408]);
      out[5184] = fma(kw, y[1408], out[5184]);
      ws[275712] = fma(kw * y[1408], y[5184], ws[275712]);
    }
}
__device__ __noinline__ void adj_jtv_0_3(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 0.66 * phi[6016];
      w = fma(0.66, phi[4576], w);
      w = fma(0.33, phi[5792], w);
      w = fma(0.33, phi[5856], w);
      w = fma(0.33, phi[4800], w);
      w = fma(0.33, phi[4000], w);
      w = fma(0.01, phi[5696], w);
      w = w - phi[1440];
      w = w - phi[5184];
      const double kw = ws[47040] * w;
      out[1440] = fma(kw, y[5184], out[1440]);
      out[5184] = fma(kw, y[1440], out[5184]);
      ws[275744] = fma(kw * y[1440], y[5184], ws[275744]);
    }
    {
      double w = 0.09 * phi[6016];
      w = fma(1.0, phi[5760], w);
      w = fma(0.62, phi[5856], w);
      w = fma(0.23, phi[2816], w);
      w = fma(0.02, phi[4000], w);
      w = fma(0.15, phi[4352], w);
      w = w - phi[4576];
      w = w - phi[5184];
      const double kw = ws[47072] * w;
      out[4576] = fma(kw, y[5184], out[4576]);
      out[5184] = fma(kw, y[4576], out[5184]);
      ws[275776] = fma(kw * y[4576], y[5184], ws[275776]);
    }
    {
      double w = 0.33 * phi[1696];
      w = fma(0.67, phi[5920], w);
      w = fma(0.27, phi[4544], w);
      w = fma(0.38, phi[5504], w);
      w = fma(0.21, phi[5856], w);
      w = fma(0.02, phi[5760], w);
      w = w - phi[4384];
      w = w - phi[5184];
      const double kw = ws[47104] * w;
      out[4384] = fma(kw, y[5184], out[4384]);
      out[5184] = fma(kw, y[4384], out[5184]);
      ws[275808] = fma(kw * y[4384], y[5184], ws[275808]);
    }
    {
      double w = 0.19 * phi[6016];
      w = fma(0.14, phi[5984], w);
      w = fma(0.1, phi[5792], w);
      w = fma(0.22, phi[5664], w);
      w = fma(0.5, phi[5248], w);
      w = fma(0.45, phi[4352], w);
      w = w - phi[4128];
      w = w - phi[5184];
      const double kw = ws[47136] * w;
      out[4128] = fma(kw, y[5184], out[4128]);
      out[5184] = fma(kw, y[4128], out[5184]);
      ws[275840] = fma(kw * y[4128], y[5184], ws[275840]);
    }
    {
      double w = 0.16 * phi[6016];
      w = fma(0.11, phi[5984], w);
      w = fma(0.28, phi[5792], w);
      w = fma(0.01, phi[5216], w);
      w = fma(0.56, phi[5664], w);
      w = fma(0.1, phi[5856], w);
      w = fma(0.54, phi[5248], w);
      w = fma(0.07, phi[4352], w);
      w = fma(0.07, phi[5696], w);
      w = fma(0.1, phi[5760], w);
      w = w - phi[4736];
      w = w - phi[5184];
      const double kw = ws[47168] * w;
      out[4736] = fma(kw, y[5184], out[4736]);
      out[5184] = fma(kw, y[4736], out[5184]);
      ws[275872] = fma(kw * y[4736], y[5184], ws[275872]);
    }
    {
      double w = 0.1 * phi[6016];
      w = fma(0.072, phi[5984], w);
      w = fma(0.008, phi[5888], w);
      w = fma(0.002, phi[5792], w);
      w = fma(0.1, phi[5216], w);
      w = fma(0.243, phi[5664], w);
      w = fma(0.08, phi[5856], w);
      w = fma(0.42, phi[5568], w);
      w = fma(0.028, phi[5504], w);
      w = fma(0.491, phi[5376], w);
      w = fma(0.003, phi[5248], w);
      w = fma(0.044, phi[4352], w);
      w = w - phi[3872];
      w = w - phi[5184];
      const double kw = ws[47200] * w;
      out[3872] = fma(kw, y[5184], out[3872]);
      out[5184] = fma(kw, y[3872], out[5184]);
      ws[275904] = fma(kw * y[3872], y[5184], ws[275904]);
    }
    {
      double w = 0.05 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(0.6, phi[4800], w);
      w = fma(0.6, phi[5216], w);
      w = fma(1.5, phi[5664], w);
      w = fma(0.05, phi[5856], w);
      w = fma(0.05, phi[5376], w);
      w = fma(0.08, phi[5248], w);
      w = fma(0.65, phi[5728], w);
      w = w - phi[5472];
      w = w - phi[5184];
      const double kw = ws[47232] * w;
      out[5472] = fma(kw, y[5184], out[5472]);
      out[5184] = fma(kw, y[5472], out[5184]);
      ws[275936] = fma(kw * y[5472], y[5184], ws[275936]);
    }
    {
      double w = 0.05 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(0.6, phi[4800], w);
      w = fma(0.6, phi[5216], w);
      w = fma(1.5, phi[5664], w);
      w = fma(0.05, phi[5856], w);
      w = fma(0.05, phi[5376], w);
      w = fma(0.08, phi[5248], w);
      w = fma(0.7, phi[5472], w);
      w = fma(0.65, phi[5728], w);
      w = w - phi[4320];
      w = w - phi[5184];
      const double kw = ws[47264] * w;
      out[4320] = fma(kw, y[5184], out[4320]);
      out[5184] = fma(kw, y[4320], out[5184]);
      ws[275968] = fma(kw * y[4320], y[5184], ws[275968]);
    }
    {
      double w = 0.05 * phi[6016];
      w = fma(1.0, phi[5984], w);
      w = fma(1.5, phi[5664], w);
      w = fma(0.48, phi[5376], w);
      w = fma(0.7, phi[5472], w);
      w = fma(0.25, phi[4352], w);
      w = fma(0.25, phi[5696], w);
      w = fma(0.11, phi[3680], w);
      w = w - phi[3584];
      w = w - phi[5184];
      const double kw = ws[47296] * w;
      out[3584] = fma(kw, y[5184], out[3584]);
      out[5184] = fma(kw, y[3584], out[5184]);
      ws[276000] = fma(kw * y[3584], y[5184], ws[276000]);
    }
    {
      double w = 1.0 * phi[3040];
      w = w - phi[3808];
      w = w - phi[5184];
      const double kw = ws[47328] * w;
      out[3808] = fma(kw, y[5184], out[3808]);
      out[5184] = fma(kw, y[3808], out[5184]);
      ws[276032] = fma(kw * y[3808], y[5184], ws[276032]);
    }
    {
      double w = 0.8 * phi[4032];
      w = fma(0.2, phi[4064], w);
      w = w - phi[2240];
      w = w - phi[5952];
      const double kw = ws[47360] * w;
      out[2240] = fma(kw, y[5952], out[2240]);
      out[5952] = fma(kw, y[2240], out[5952]);
      ws[276064] = fma(kw * y[2240], y[5952], ws[276064]);
    }
    {
      double w = 0.43 * phi[4032];
      w = fma(0.57, phi[4064], w);
      w = w - phi[2752];
      w = w - phi[5952];
      const double kw = ws[47392] * w;
      out[2752] = fma(kw, y[5952], out[2752]);
      out[5952] = fma(kw, y[2752], out[5952]);
      ws[276096] = fma(kw * y[2752], y[5952], ws[276096]);
    }
    {
      double w = 0.11 * phi[4032];
      w = fma(0.89, phi[4064], w);
      w = w - phi[1152];
      w = w - phi[5952];
      const double kw = ws[47424] * w;
      out[1152] = fma(kw, y[5952], out[1152]);
      out[5952] = fma(kw, y[1152], out[5952]);
      ws[276128] = fma(kw * y[1152], y[5952], ws[276128]);
    }
    {
      double w = 0.975 * phi[2624];
      w = fma(0.025, phi[3840], w);
      w = w - phi[1408];
      w = w - phi[5952];
      const double kw = ws[47456] * w;
      out[1408] = fma(kw, y[5952], out[1408]);
      out[5952] = fma(kw, y[1408], out[5952]);
      ws[276160] = fma(kw * y[1408], y[5952], ws[276160]);
    }
    {
      double w = 0.945 * phi[2656];
      w = fma(0.055, phi[3712], w);
      w = w - phi[1440];
      w = w - phi[5952];
      const double kw = ws[47488] * w;
      out[1440] = fma(kw, y[5952], out[1440]);
      out[5952] = fma(kw, y[1440], out[5952]);
      ws[276192] = fma(kw * y[1440], y[5952], ws[276192]);
    }
    {
      double w = 0.33 * phi[1696];
      w = fma(0.67, phi[5920], w);
      w = fma(0.27, phi[4544], w);
      w = fma(0.38, phi[5504], w);
      w = fma(0.21, phi[5856], w);
      w = fma(0.02, phi[5760], w);
      w = w - phi[4384];
      w = w - phi[5952];
      const double kw = ws[47520] * w;
      out[4384] = fma(kw, y[5952], out[4384]);
      out[5952] = fma(kw, y[4384], out[5952]);
      ws[276224] = fma(kw * y[4384], y[5952], ws[276224]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5664], w);
      w = fma(1.0, phi[5024], w);
      w = w - phi[5856];
      w = w - phi[5952];
      const double kw = ws[47552] * w;
      out[5856] = fma(kw, y[5952], out[5856]);
      out[5952] = fma(kw, y[5856], out[5952]);
      ws[276256] = fma(kw * y[5856], y[5952], ws[276256]);
    }
    {
      double w = 1.0 * phi[5792];
      w = fma(1.0, phi[5024], w);
      w = w - phi[5568];
      w = w - phi[5952];
      const double kw = ws[47584] * w;
      out[5568] = fma(kw, y[5952], out[5568]);
      out[5952] = fma(kw, y[5568], out[5952]);
      ws[276288] = fma(kw * y[5568], y[5952], ws[276288]);
    }
    {
      double w = 1.0 * phi[4800];
      w = fma(1.0, phi[5024], w);
      w = w - phi[5760];
      w = w - phi[5952];
      const double kw = ws[47616] * w;
      out[5760] = fma(kw, y[5952], out[5760]);
      out[5952] = fma(kw, y[5760], out[5952]);
      ws[276320] = fma(kw * y[5760], y[5952], ws[276320]);
    }
    {
      double w = 0.68 * phi[5856];
      w = fma(0.32, phi[4672], w);
      w = fma(0.68, phi[5216], w);
      w = fma(0.68, phi[5248], w);
      w = fma(0.32, phi[5024], w);
      w = fma(0.68, phi[5920], w);
      w = w - phi[4128];
      w = w - phi[5952];
      const double kw = ws[47648] * w;
      out[4128] = fma(kw, y[5952], out[4128]);
      out[5952] = fma(kw, y[4128], out[5952]);
      ws[276352] = fma(kw * y[4128], y[5952], ws[276352]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5216], w);
      w = fma(0.668, phi[5664], w);
      w = fma(0.332, phi[5856], w);
      w = fma(0.332, phi[5760], w);
      w = fma(1.0, phi[5440], w);
      w = w - phi[3872];
      w = w - phi[5952];
      const double kw = ws[47680] * w;
      out[3872] = fma(kw, y[5952], out[3872]);
      out[5952] = fma(kw, y[3872], out[5952]);
      ws[276384] = fma(kw * y[3872], y[5952], ws[276384]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(2.0, phi[5664], w);
      w = fma(1.0, phi[5024], w);
      w = w - phi[5376];
      w = w - phi[5952];
      const double kw = ws[47712] * w;
      out[5376] = fma(kw, y[5952], out[5376]);
      out[5952] = fma(kw, y[5376], out[5952]);
      ws[276416] = fma(kw * y[5376], y[5952], ws[276416]);
    }
    {
      double w = 1.0 * phi[5792];
      w = fma(1.0, phi[5664], w);
      w = fma(1.0, phi[5024], w);
      w = w - phi[5248];
      w = w - phi[5952];
      const double kw = ws[47744] * w;
      out[5248] = fma(kw, y[5952], out[5248]);
      out[5952] = fma(kw, y[5248], out[5952]);
      ws[276448] = fma(kw * y[5248], y[5952], ws[276448]);
    }
    {
      double w = 0.152 * phi[3616];
      w = fma(0.339, phi[3232], w);
      w = fma(0.85, phi[3648], w);
      w = fma(0.424, phi[3072], w);
      w = fma(0.424, phi[5024], w);
      w = w - phi[1248];
      w = w - phi[5952];
      const double kw = ws[47776] * w;
      out[1248] = fma(kw, y[5952], out[1248]);
      out[5952] = fma(kw, y[1248], out[5952]);
      ws[276480] = fma(kw * y[1248], y[5952], ws[276480]);
    }
    {
      double w = 0.2 * phi[3616];
      w = fma(0.32, phi[3232], w);
      w = fma(0.08, phi[3648], w);
      w = fma(0.4, phi[3072], w);
      w = fma(0.4, phi[5024], w);
      w = w - phi[2944];
      w = w - phi[5952];
      const double kw = ws[47808] * w;
      out[2944] = fma(kw, y[5952], out[2944]);
      out[5952] = fma(kw, y[2944], out[5952]);
      ws[276512] = fma(kw * y[2944], y[5952], ws[276512]);
    }
    {
      double w = 1.0 * phi[3808];
      w = fma(1.0, phi[5024], w);
      w = w - phi[1760];
      w = w - phi[5952];
      const double kw = ws[47840] * w;
      out[1760] = fma(kw, y[5952], out[1760]);
      out[5952] = fma(kw, y[1760], out[5952]);
      ws[276544] = fma(kw * y[1760], y[5952], ws[276544]);
    }
    {
      double w = 1.0 * phi[4672];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1824];
      w = w - phi[5952];
      const double kw = ws[47872] * w;
      out[1824] = fma(kw, y[5952], out[1824]);
      out[5952] = fma(kw, y[1824], out[5952]);
      ws[276576] = fma(kw * y[1824], y[5952], ws[276576]);
    }
    {
      double w = 1.0 * phi[4256];
      w = w - phi[2560];
      const double kw = ws[47904] * w;
      out[2560] = out[2560] + kw;
      ws[276608] = fma(kw, y[2560], ws[276608]);
    }
    {
      double w = 1.0 * phi[4256];
      w = w - phi[1728];
      const double kw = ws[47936] * w;
      out[1728] = out[1728] + kw;
      ws[276640] = fma(kw, y[1728], ws[276640]);
    }
    {
      double w = 1.0 * phi[1088];
      w = w - phi[5792];
      w = w - phi[5920];
      const double kw = ws[47968] * w;
      out[5792] = fma(kw, y[5920], out[5792]);
      out[5920] = fma(kw, y[5792], out[5920]);
      ws[276672] = fma(kw * y[5792], y[5920], ws[276672]);
    }
    {
      double w = 1.0 * phi[5792];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1088];
      const double kw = ws[48000] * w;
      out[1088] = out[1088] + kw;
      ws[276704] = fma(kw, y[1088], ws[276704]);
    }
    {
      double w = 1.0 * phi[1536];
      w = w - phi[4800];
      w = w - phi[5920];
      const double kw = ws[48032] * w;
      out[4800] = fma(kw, y[5920], out[4800]);
      out[5920] = fma(kw, y[4800], out[5920]);
      ws[276736] = fma(kw * y[4800], y[5920], ws[276736]);
    }
    {
      double w = 1.0 * phi[4800];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1536];
      const double kw = ws[48064] * w;
      out[1536] = out[1536] + kw;
      ws[276768] = fma(kw, y[1536], ws[276768]);
    }
    {
      double w = 1.0 * phi[1824];
      w = w - phi[4672];
      w = w - phi[5920];
      const double kw = ws[48096] * w;
      out[4672] = fma(kw, y[5920], out[4672]);
      out[5920] = fma(kw, y[4672], out[5920]);
      ws[276800] = fma(kw * y[4672], y[5920], ws[276800]);
    }
    {
      double w = 1.0 * phi[4672];
      w = fma(1.0, phi[5920], w);
      w = w - phi[1824];
      const double kw = ws[48128] * w;
      out[1824] = out[1824] + kw;
      ws[276832] = fma(kw, y[1824], ws[276832]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[5856], w);
      w = w - phi[5888];
      w = w - phi[5824];
      const double kw = ws[48160] * w;
      out[5888] = fma(kw, y[5824], out[5888]);
      out[5824] = fma(kw, y[5888], out[5824]);
      ws[276864] = fma(kw * y[5888], y[5824], ws[276864]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.0, phi[5568], w);
      w = w - phi[5632];
      w = w - phi[5824];
      const double kw = ws[48192] * w;
      out[5632] = fma(kw, y[5824], out[5632]);
      out[5824] = fma(kw, y[5632], out[5824]);
      ws[276896] = fma(kw * y[5632], y[5824], ws[276896]);
    }
    {
      double w = 0.66 * phi[5984];
      w = fma(0.131, phi[5888], w);
      w = fma(0.048, phi[5632], w);
      w = fma(0.089, phi[5216], w);
      w = fma(0.935, phi[5920], w);
      w = fma(0.504, phi[5568], w);
      w = fma(0.132, phi[5760], w);
      w = fma(0.165, phi[4480], w);
      w = fma(0.042, phi[5280], w);
      w = fma(0.065, phi[5440], w);
      w = w - phi[5408];
      w = w - phi[5824];
      const double kw = ws[48224] * w;
      out[5408] = fma(kw, y[5824], out[5408]);
      out[5824] = fma(kw, y[5408], out[5824]);
      ws[276928] = fma(kw * y[5408], y[5824], ws[276928]);
    }
    {
      double w = 0.2 * phi[5984];
      w = fma(0.051, phi[5888], w);
      w = fma(0.231, phi[5632], w);
      w = fma(0.235, phi[5216], w);
      w = fma(0.864, phi[5920], w);
      w = fma(0.018, phi[5856], w);
      w = fma(0.045, phi[5568], w);
      w = fma(0.203, phi[5760], w);
      w = fma(0.033, phi[5280], w);
      w = fma(0.217, phi[4480], w);
      w = fma(0.033, phi[5504], w);
      w = fma(0.272, phi[5344], w);
      w = fma(0.136, phi[5440], w);
      w = w - phi[5120];
      w = w - phi[5824];
      const double kw = ws[48256] * w;
      out[5120] = fma(kw, y[5824], out[5120]);
      out[5824] = fma(kw, y[5120], out[5824]);
      ws[276960] = fma(kw * y[5120], y[5824], ws[276960]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5920], w);
      w = fma(1.6, phi[5856], w);
      w = fma(0.2, phi[5760], w);
      w = w - phi[3008];
      w = w - phi[5824];
      const double kw = ws[48288] * w;
      out[3008] = fma(kw, y[5824], out[3008]);
      out[5824] = fma(kw, y[3008], out[5824]);
      ws[276992] = fma(kw * y[3008], y[5824], ws[276992]);
    }
    {
      double w = 0.78 * phi[5984];
      w = fma(0.97, phi[5920], w);
      w = fma(0.78, phi[5856], w);
      w = fma(0.012, phi[5568], w);
      w = fma(0.44, phi[5760], w);
      w = fma(0.06, phi[4480], w);
      w = fma(0.13, phi[5280], w);
      w = fma(0.03, phi[5440], w);
      w = w - phi[3200];
      w = w - phi[5824];
      const double kw = ws[48320] * w;
      out[3200] = fma(kw, y[5824], out[3200]);
      out[5824] = fma(kw, y[3200], out[5824]);
      ws[277024] = fma(kw * y[3200], y[5824], ws[277024]);
    }
}
}  // namespace mech_cracmm2
