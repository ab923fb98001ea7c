// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void adj_jtv_0_0(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[4384];
      w = fma(1.0, phi[4160], w);
      w = w - phi[4608];
      const double kw = ws[33376] * w;
      out[4608] = out[4608] + kw;
      ws[174624] = fma(kw, y[4608], ws[174624]);
    }
    {
      double w = 1.0 * phi[4320];
      w = w - phi[4160];
      const double kw = ws[33408] * w;
      out[4160] = out[4160] + kw;
      ws[174656] = fma(kw, y[4160], ws[174656]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[4320];
      w = w - phi[4384];
      const double kw = ws[33440] * w;
      out[4320] = fma(kw, y[4384], out[4320]);
      out[4384] = fma(kw, y[4320], out[4384]);
      ws[174688] = fma(kw * y[4320], y[4384], ws[174688]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[4160];
      w = w - phi[4384];
      const double kw = ws[33472] * w;
      out[4160] = fma(kw, y[4384], out[4160]);
      out[4384] = fma(kw, y[4160], out[4384]);
      ws[174720] = fma(kw * y[4160], y[4384], ws[174720]);
    }
    {
      double w = 1.0 * phi[4384];
      w = w - phi[4160];
      w = w - phi[4608];
      const double kw = ws[33504] * w;
      out[4160] = fma(kw, y[4608], out[4160]);
      out[4608] = fma(kw, y[4160], out[4608]);
      ws[174752] = fma(kw * y[4160], y[4608], ws[174752]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[4160];
      w = w - phi[4608];
      const double kw = ws[33536] * w;
      out[4160] = fma(kw, y[4608], out[4160]);
      out[4608] = fma(kw, y[4160], out[4608]);
      ws[174784] = fma(kw * y[4160], y[4608], ws[174784]);
    }
    {
      double w = -phi[4160];
      w = w - phi[4320];
      const double kw = ws[33568] * w;
      out[4160] = fma(kw, y[4320], out[4160]);
      out[4320] = fma(kw, y[4160], out[4320]);
      ws[174816] = fma(kw * y[4160], y[4320], ws[174816]);
    }
    {
      double w = 1.0 * phi[4160];
      w = w - phi[4320];
      const double kw = ws[33600] * w;
      out[4320] = out[4320] + kw;
      ws[174848] = fma(kw, y[4320], ws[174848]);
    }
    {
      double w = 1.0 * phi[672];
      w = w - phi[4320];
      const double kw = ws[33632] * w;
      out[4320] = out[4320] + kw;
      ws[174880] = fma(kw, y[4320], ws[174880]);
    }
    {
      double w = 1.0 * phi[4160];
      w = w - phi[672];
      const double kw = ws[33664] * w;
      out[672] = out[672] + kw;
      ws[174912] = fma(kw, y[672], ws[174912]);
    }
    {
      double w = 2.0 * phi[4736];
      w = w - phi[672];
      const double kw = ws[33696] * w;
      out[672] = out[672] + kw;
      ws[174944] = fma(kw, y[672], ws[174944]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[4320];
      w = w - phi[4736];
      const double kw = ws[33728] * w;
      out[4320] = fma(kw, y[4736], out[4320]);
      out[4736] = fma(kw, y[4320], out[4736]);
      ws[174976] = fma(kw * y[4320], y[4736], ws[174976]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[4320];
      w = w - phi[4704];
      const double kw = ws[33760] * w;
      out[4320] = fma(kw, y[4704], out[4320]);
      out[4704] = fma(kw, y[4320], out[4704]);
      ws[175008] = fma(kw * y[4320], y[4704], ws[175008]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[4736];
      w = w - phi[4160];
      const double kw = ws[33792] * w;
      out[4736] = fma(kw, y[4160], out[4736]);
      out[4160] = fma(kw, y[4736], out[4160]);
      ws[175040] = fma(kw * y[4736], y[4160], ws[175040]);
    }
    {
      double w = 1.0 * phi[4736];
      w = w - phi[4704];
      w = w - phi[4160];
      const double kw = ws[33824] * w;
      out[4704] = fma(kw, y[4160], out[4704]);
      out[4160] = fma(kw, y[4704], out[4160]);
      ws[175072] = fma(kw * y[4704], y[4160], ws[175072]);
    }
    {
      double w = 1.0 * phi[4160];
      w = w - phi[4736];
      w = w - phi[4736];
      const double kw = ws[33856] * w;
      out[4736] = fma(kw, y[4736], out[4736]);
      out[4736] = fma(kw, y[4736], out[4736]);
      ws[175104] = fma(kw * y[4736], y[4736], ws[175104]);
    }
    {
      double w = 1.0 * phi[3456];
      w = w - phi[4736];
      w = w - phi[4736];
      const double kw = ws[33888] * w;
      out[4736] = fma(kw, y[4736], out[4736]);
      out[4736] = fma(kw, y[4736], out[4736]);
      ws[175136] = fma(kw * y[4736], y[4736], ws[175136]);
    }
    {
      double w = -phi[4736];
      w = w - phi[4704];
      const double kw = ws[33920] * w;
      out[4736] = fma(kw, y[4704], out[4736]);
      out[4704] = fma(kw, y[4736], out[4704]);
      ws[175168] = fma(kw * y[4736], y[4704], ws[175168]);
    }
    {
      double w = 1.0 * phi[3456];
      w = w - phi[4704];
      w = w - phi[4704];
      const double kw = ws[33952] * w;
      out[4704] = fma(kw, y[4704], out[4704]);
      out[4704] = fma(kw, y[4704], out[4704]);
      ws[175200] = fma(kw * y[4704], y[4704], ws[175200]);
    }
    {
      double w = 1.0 * phi[3456];
      w = w - phi[4704];
      w = w - phi[4704];
      const double kw = ws[33984] * w;
      out[4704] = fma(kw, y[4704], out[4704]);
      out[4704] = fma(kw, y[4704], out[4704]);
      ws[175232] = fma(kw * y[4704], y[4704], ws[175232]);
    }
    {
      double w = 2.0 * phi[4736];
      w = w - phi[3456];
      const double kw = ws[34016] * w;
      out[3456] = out[3456] + kw;
      ws[175264] = fma(kw, y[3456], ws[175264]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[3456];
      w = w - phi[4736];
      const double kw = ws[34048] * w;
      out[3456] = fma(kw, y[4736], out[3456]);
      out[4736] = fma(kw, y[3456], out[4736]);
      ws[175296] = fma(kw * y[3456], y[4736], ws[175296]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[4704], w);
      w = w - phi[3456];
      w = w - phi[4160];
      const double kw = ws[34080] * w;
      out[3456] = fma(kw, y[4160], out[3456]);
      out[4160] = fma(kw, y[3456], out[4160]);
      ws[175328] = fma(kw * y[3456], y[4160], ws[175328]);
    }
    {
      double w = 2.0 * phi[4608];
      w = w - phi[4384];
      w = w - phi[4384];
      const double kw = ws[34112] * w;
      out[4384] = fma(kw, y[4384], out[4384]);
      out[4384] = fma(kw, y[4384], out[4384]);
      ws[175360] = fma(kw * y[4384], y[4384], ws[175360]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[4608], w);
      w = w - phi[4704];
      w = w - phi[4384];
      const double kw = ws[34144] * w;
      out[4704] = fma(kw, y[4384], out[4704]);
      out[4384] = fma(kw, y[4704], out[4384]);
      ws[175392] = fma(kw * y[4704], y[4384], ws[175392]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[4608];
      w = w - phi[4320];
      const double kw = ws[34176] * w;
      out[4608] = fma(kw, y[4320], out[4608]);
      out[4320] = fma(kw, y[4608], out[4320]);
      ws[175424] = fma(kw * y[4608], y[4320], ws[175424]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4160], w);
      w = w - phi[4640];
      const double kw = ws[34208] * w;
      out[4640] = out[4640] + kw;
      ws[175456] = fma(kw, y[4640], ws[175456]);
    }
    {
      double w = 1.0 * phi[4384];
      w = w - phi[4640];
      const double kw = ws[34240] * w;
      out[4640] = out[4640] + kw;
      ws[175488] = fma(kw, y[4640], ws[175488]);
    }
    {
      double w = 2.0 * phi[4608];
      w = w - phi[4640];
      w = w - phi[4384];
      const double kw = ws[34272] * w;
      out[4640] = fma(kw, y[4384], out[4640]);
      out[4384] = fma(kw, y[4640], out[4384]);
      ws[175520] = fma(kw * y[4640], y[4384], ws[175520]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(1.0, phi[4608], w);
      w = w - phi[4640];
      w = w - phi[4608];
      const double kw = ws[34304] * w;
      out[4640] = fma(kw, y[4608], out[4640]);
      out[4608] = fma(kw, y[4640], out[4608]);
      ws[175552] = fma(kw * y[4640], y[4608], ws[175552]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[4640];
      w = w - phi[4160];
      const double kw = ws[34336] * w;
      out[4640] = fma(kw, y[4160], out[4640]);
      out[4160] = fma(kw, y[4640], out[4160]);
      ws[175584] = fma(kw * y[4640], y[4160], ws[175584]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(1.0, phi[4608], w);
      w = w - phi[4640];
      w = w - phi[4736];
      const double kw = ws[34368] * w;
      out[4640] = fma(kw, y[4736], out[4640]);
      out[4736] = fma(kw, y[4640], out[4736]);
      ws[175616] = fma(kw * y[4640], y[4736], ws[175616]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[4608], w);
      w = w - phi[4640];
      w = w - phi[4704];
      const double kw = ws[34400] * w;
      out[4640] = fma(kw, y[4704], out[4640]);
      out[4704] = fma(kw, y[4640], out[4704]);
      ws[175648] = fma(kw * y[4640], y[4704], ws[175648]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[4640];
      w = w - phi[4320];
      const double kw = ws[34432] * w;
      out[4640] = fma(kw, y[4320], out[4640]);
      out[4320] = fma(kw, y[4640], out[4320]);
      ws[175680] = fma(kw * y[4640], y[4320], ws[175680]);
    }
    {
      double w = 2.0 * phi[4608];
      w = w - phi[4640];
      w = w - phi[4640];
      const double kw = ws[34464] * w;
      out[4640] = fma(kw, y[4640], out[4640]);
      out[4640] = fma(kw, y[4640], out[4640]);
      ws[175712] = fma(kw * y[4640], y[4640], ws[175712]);
    }
    {
      double w = 1.0 * phi[1280];
      w = w - phi[4640];
      w = w - phi[4608];
      const double kw = ws[34496] * w;
      out[4640] = fma(kw, y[4608], out[4640]);
      out[4608] = fma(kw, y[4640], out[4608]);
      ws[175744] = fma(kw * y[4640], y[4608], ws[175744]);
    }
    {
      double w = 1.0 * phi[4640];
      w = fma(1.0, phi[4608], w);
      w = w - phi[1280];
      const double kw = ws[34528] * w;
      out[1280] = out[1280] + kw;
      ws[175776] = fma(kw, y[1280], ws[175776]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4640], w);
      w = w - phi[1280];
      const double kw = ws[34560] * w;
      out[1280] = out[1280] + kw;
      ws[175808] = fma(kw, y[1280], ws[175808]);
    }
    {
      double w = 2.0 * phi[4192];
      w = w - phi[1280];
      const double kw = ws[34592] * w;
      out[1280] = out[1280] + kw;
      ws[175840] = fma(kw, y[1280], ws[175840]);
    }
    {
      double w = 1.0 * phi[2464];
      w = w - phi[4384];
      w = w - phi[4736];
      const double kw = ws[34624] * w;
      out[4384] = fma(kw, y[4736], out[4384]);
      out[4736] = fma(kw, y[4384], out[4736]);
      ws[175872] = fma(kw * y[4384], y[4736], ws[175872]);
    }
    {
      double w = 2.0 * phi[2464];
      w = w - phi[4384];
      w = w - phi[4608];
      const double kw = ws[34656] * w;
      out[4384] = fma(kw, y[4608], out[4384]);
      out[4608] = fma(kw, y[4384], out[4608]);
      ws[175904] = fma(kw * y[4384], y[4608], ws[175904]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(1.0, phi[4608], w);
      w = w - phi[2464];
      w = w - phi[2464];
      const double kw = ws[34688] * w;
      out[2464] = fma(kw, y[2464], out[2464]);
      out[2464] = fma(kw, y[2464], out[2464]);
      ws[175936] = fma(kw * y[2464], y[2464], ws[175936]);
    }
    {
      double w = 1.0 * phi[4384];
      w = fma(1.0, phi[4736], w);
      w = w - phi[2464];
      const double kw = ws[34720] * w;
      out[2464] = out[2464] + kw;
      ws[175968] = fma(kw, y[2464], ws[175968]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[2464];
      w = w - phi[4736];
      const double kw = ws[34752] * w;
      out[2464] = fma(kw, y[4736], out[2464]);
      out[4736] = fma(kw, y[2464], out[4736]);
      ws[176000] = fma(kw * y[2464], y[4736], ws[176000]);
    }
    {
      double w = 1.0 * phi[4192];
      w = w - phi[4608];
      w = w - phi[4736];
      const double kw = ws[34784] * w;
      out[4608] = fma(kw, y[4736], out[4608]);
      out[4736] = fma(kw, y[4608], out[4736]);
      ws[176032] = fma(kw * y[4608], y[4736], ws[176032]);
    }
    {
      double w = 1.0 * phi[4640];
      w = w - phi[4192];
      w = w - phi[4736];
      const double kw = ws[34816] * w;
      out[4192] = fma(kw, y[4736], out[4192]);
      out[4736] = fma(kw, y[4192], out[4736]);
      ws[176064] = fma(kw * y[4192], y[4736], ws[176064]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[4608], w);
      w = w - phi[4192];
      const double kw = ws[34848] * w;
      out[4192] = out[4192] + kw;
      ws[176096] = fma(kw, y[4192], ws[176096]);
    }
    {
      double w = 1.0 * phi[1696];
      w = w - phi[4704];
      w = w - phi[4608];
      const double kw = ws[34880] * w;
      out[4704] = fma(kw, y[4608], out[4704]);
      out[4608] = fma(kw, y[4704], out[4608]);
      ws[176128] = fma(kw * y[4704], y[4608], ws[176128]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(1.0, phi[4608], w);
      w = w - phi[1696];
      const double kw = ws[34912] * w;
      out[1696] = out[1696] + kw;
      ws[176160] = fma(kw, y[1696], ws[176160]);
    }
    {
      double w = 0.59 * phi[4704];
      w = fma(0.59, phi[4608], w);
      w = fma(0.41, phi[4736], w);
      w = fma(0.41, phi[4640], w);
      w = w - phi[1696];
      const double kw = ws[34944] * w;
      out[1696] = out[1696] + kw;
      ws[176192] = fma(kw, y[1696], ws[176192]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[1696];
      w = w - phi[4736];
      const double kw = ws[34976] * w;
      out[1696] = fma(kw, y[4736], out[1696]);
      out[4736] = fma(kw, y[1696], out[4736]);
      ws[176224] = fma(kw * y[1696], y[4736], ws[176224]);
    }
    {
      double w = 1.0 * phi[256];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[288], w);
      w = w - phi[2208];
      w = w - phi[4736];
      const double kw = ws[35008] * w;
      out[2208] = fma(kw, y[4736], out[2208]);
      out[4736] = fma(kw, y[2208], out[4736]);
      ws[176256] = fma(kw * y[2208], y[4736], ws[176256]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4416], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4448];
      w = w - phi[4384];
      const double kw = ws[35040] * w;
      out[4448] = fma(kw, y[4384], out[4448]);
      out[4384] = fma(kw, y[4448], out[4384]);
      ws[176288] = fma(kw * y[4448], y[4384], ws[176288]);
    }
    {
      double w = 1.0 * phi[1344];
      w = w - phi[4448];
      w = w - phi[4608];
      const double kw = ws[35072] * w;
      out[4448] = fma(kw, y[4608], out[4448]);
      out[4608] = fma(kw, y[4448], out[4608]);
      ws[176320] = fma(kw * y[4448], y[4608], ws[176320]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4448], w);
      w = w - phi[1344];
      const double kw = ws[35104] * w;
      out[1344] = out[1344] + kw;
      ws[176352] = fma(kw, y[1344], ws[176352]);
    }
    {
      double w = 0.6 * phi[4608];
      w = fma(0.6, phi[4448], w);
      w = fma(0.4, phi[4640], w);
      w = fma(0.4, phi[4416], w);
      w = fma(0.4, phi[4672], w);
      w = w - phi[1344];
      const double kw = ws[35136] * w;
      out[1344] = out[1344] + kw;
      ws[176384] = fma(kw, y[1344], ws[176384]);
    }
}
__device__ __noinline__ void adj_jtv_0_1(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 0.37 * phi[2688];
      w = fma(0.13, phi[3904], w);
      w = fma(0.13, phi[4320], w);
      w = fma(0.5, phi[4416], w);
      w = fma(0.5, phi[4672], w);
      w = fma(0.5, phi[4736], w);
      w = w - phi[4448];
      w = w - phi[4704];
      const double kw = ws[35168] * w;
      out[4448] = fma(kw, y[4704], out[4448]);
      out[4704] = fma(kw, y[4448], out[4704]);
      ws[176416] = fma(kw * y[4448], y[4704], ws[176416]);
    }
    {
      double w = 1.0 * phi[4416];
      w = w - phi[4448];
      w = w - phi[4672];
      const double kw = ws[35200] * w;
      out[4448] = fma(kw, y[4672], out[4448]);
      out[4672] = fma(kw, y[4448], out[4672]);
      ws[176448] = fma(kw * y[4448], y[4672], ws[176448]);
    }
    {
      double w = 2.0 * phi[4416];
      w = fma(2.0, phi[4672], w);
      w = w - phi[4448];
      w = w - phi[4448];
      const double kw = ws[35232] * w;
      out[4448] = fma(kw, y[4448], out[4448]);
      out[4448] = fma(kw, y[4448], out[4448]);
      ws[176480] = fma(kw * y[4448], y[4448], ws[176480]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4128], w);
      w = fma(1.0, phi[4576], w);
      w = fma(2.0, phi[4672], w);
      w = w - phi[4448];
      w = w - phi[4096];
      const double kw = ws[35264] * w;
      out[4448] = fma(kw, y[4096], out[4448]);
      out[4096] = fma(kw, y[4448], out[4096]);
      ws[176512] = fma(kw * y[4448], y[4096], ws[176512]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4128], w);
      w = fma(1.0, phi[4576], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4096];
      w = w - phi[4384];
      const double kw = ws[35296] * w;
      out[4096] = fma(kw, y[4384], out[4096]);
      out[4384] = fma(kw, y[4096], out[4384]);
      ws[176544] = fma(kw * y[4096], y[4384], ws[176544]);
    }
    {
      double w = 1.0 * phi[1952];
      w = w - phi[4096];
      w = w - phi[4608];
      const double kw = ws[35328] * w;
      out[4096] = fma(kw, y[4608], out[4096]);
      out[4608] = fma(kw, y[4096], out[4608]);
      ws[176576] = fma(kw * y[4096], y[4608], ws[176576]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4096], w);
      w = w - phi[1952];
      const double kw = ws[35360] * w;
      out[1952] = out[1952] + kw;
      ws[176608] = fma(kw, y[1952], ws[176608]);
    }
    {
      double w = 0.6 * phi[4608];
      w = fma(0.6, phi[4096], w);
      w = fma(0.4, phi[4640], w);
      w = fma(0.4, phi[4128], w);
      w = fma(0.4, phi[4576], w);
      w = fma(0.4, phi[4672], w);
      w = w - phi[1952];
      const double kw = ws[35392] * w;
      out[1952] = out[1952] + kw;
      ws[176640] = fma(kw, y[1952], ws[176640]);
    }
    {
      double w = 0.37 * phi[2688];
      w = fma(0.13, phi[3904], w);
      w = fma(0.13, phi[4320], w);
      w = fma(0.5, phi[4736], w);
      w = fma(0.5, phi[4416], w);
      w = fma(0.5, phi[4672], w);
      w = w - phi[4096];
      w = w - phi[4704];
      const double kw = ws[35424] * w;
      out[4096] = fma(kw, y[4704], out[4096]);
      out[4704] = fma(kw, y[4096], out[4704]);
      ws[176672] = fma(kw * y[4096], y[4704], ws[176672]);
    }
    {
      double w = 1.0 * phi[4416];
      w = w - phi[4096];
      w = w - phi[4672];
      const double kw = ws[35456] * w;
      out[4096] = fma(kw, y[4672], out[4096]);
      out[4672] = fma(kw, y[4096], out[4672]);
      ws[176704] = fma(kw * y[4096], y[4672], ws[176704]);
    }
    {
      double w = 2.0 * phi[4416];
      w = fma(2.0, phi[4672], w);
      w = w - phi[4096];
      w = w - phi[4096];
      const double kw = ws[35488] * w;
      out[4096] = fma(kw, y[4096], out[4096]);
      out[4096] = fma(kw, y[4096], out[4096]);
      ws[176736] = fma(kw * y[4096], y[4096], ws[176736]);
    }
    {
      double w = 1.0 * phi[4384];
      w = w - phi[4672];
      w = w - phi[4384];
      const double kw = ws[35520] * w;
      out[4672] = fma(kw, y[4384], out[4672]);
      out[4384] = fma(kw, y[4672], out[4384]);
      ws[176768] = fma(kw * y[4672], y[4384], ws[176768]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[4672];
      w = w - phi[4704];
      const double kw = ws[35552] * w;
      out[4672] = fma(kw, y[4704], out[4672]);
      out[4704] = fma(kw, y[4672], out[4704]);
      ws[176800] = fma(kw * y[4672], y[4704], ws[176800]);
    }
    {
      double w = -phi[4672];
      w = w - phi[4672];
      const double kw = ws[35584] * w;
      out[4672] = fma(kw, y[4672], out[4672]);
      out[4672] = fma(kw, y[4672], out[4672]);
      ws[176832] = fma(kw * y[4672], y[4672], ws[176832]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4608], w);
      w = w - phi[4416];
      w = w - phi[4384];
      const double kw = ws[35616] * w;
      out[4416] = fma(kw, y[4384], out[4416]);
      out[4384] = fma(kw, y[4416], out[4384]);
      ws[176864] = fma(kw * y[4416], y[4384], ws[176864]);
    }
    {
      double w = 0.9 * phi[2272];
      w = fma(0.1, phi[4512], w);
      w = w - phi[4416];
      w = w - phi[4704];
      const double kw = ws[35648] * w;
      out[4416] = fma(kw, y[4704], out[4416]);
      out[4704] = fma(kw, y[4416], out[4704]);
      ws[176896] = fma(kw * y[4416], y[4704], ws[176896]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(0.9, phi[4704], w);
      w = fma(0.9, phi[4416], w);
      w = fma(0.1, phi[3904], w);
      w = fma(0.9, phi[4672], w);
      w = w - phi[4416];
      w = w - phi[4448];
      const double kw = ws[35680] * w;
      out[4416] = fma(kw, y[4448], out[4416]);
      out[4448] = fma(kw, y[4416], out[4448]);
      ws[176928] = fma(kw * y[4416], y[4448], ws[176928]);
    }
    {
      double w = 0.685 * phi[4512];
      w = fma(0.315, phi[2720], w);
      w = fma(0.37, phi[4704], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4416];
      w = w - phi[4672];
      const double kw = ws[35712] * w;
      out[4416] = fma(kw, y[4672], out[4416]);
      out[4672] = fma(kw, y[4416], out[4672]);
      ws[176960] = fma(kw * y[4416], y[4672], ws[176960]);
    }
    {
      double w = 1.0 * phi[4608];
      w = fma(1.0, phi[4704], w);
      w = w - phi[4576];
      w = w - phi[4384];
      const double kw = ws[35744] * w;
      out[4576] = fma(kw, y[4384], out[4576]);
      out[4384] = fma(kw, y[4576], out[4384]);
      ws[176992] = fma(kw * y[4576], y[4384], ws[176992]);
    }
    {
      double w = 1.0 * phi[2880];
      w = w - phi[4576];
      w = w - phi[4704];
      const double kw = ws[35776] * w;
      out[4576] = fma(kw, y[4704], out[4576]);
      out[4704] = fma(kw, y[4576], out[4704]);
      ws[177024] = fma(kw * y[4576], y[4704], ws[177024]);
    }
    {
      double w = 0.8 * phi[4704];
      w = fma(0.8, phi[4416], w);
      w = fma(0.2, phi[3904], w);
      w = fma(0.8, phi[4672], w);
      w = w - phi[4576];
      w = w - phi[4448];
      const double kw = ws[35808] * w;
      out[4576] = fma(kw, y[4448], out[4576]);
      out[4448] = fma(kw, y[4576], out[4448]);
      ws[177056] = fma(kw * y[4576], y[4448], ws[177056]);
    }
    {
      double w = 0.6 * phi[4704];
      w = fma(1.0, phi[4672], w);
      w = w - phi[4576];
      w = w - phi[4672];
      const double kw = ws[35840] * w;
      out[4576] = fma(kw, y[4672], out[4576]);
      out[4672] = fma(kw, y[4576], out[4672]);
      ws[177088] = fma(kw * y[4576], y[4672], ws[177088]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[4352];
      w = w - phi[4384];
      const double kw = ws[35872] * w;
      out[4352] = fma(kw, y[4384], out[4352]);
      out[4384] = fma(kw, y[4352], out[4384]);
      ws[177120] = fma(kw * y[4352], y[4384], ws[177120]);
    }
    {
      double w = 1.0 * phi[2880];
      w = w - phi[4352];
      w = w - phi[4704];
      const double kw = ws[35904] * w;
      out[4352] = fma(kw, y[4704], out[4352]);
      out[4704] = fma(kw, y[4352], out[4704]);
      ws[177152] = fma(kw * y[4352], y[4704], ws[177152]);
    }
    {
      double w = 0.8 * phi[4416];
      w = fma(0.2, phi[3904], w);
      w = fma(0.8, phi[4672], w);
      w = w - phi[4352];
      w = w - phi[4448];
      const double kw = ws[35936] * w;
      out[4352] = fma(kw, y[4448], out[4352]);
      out[4448] = fma(kw, y[4352], out[4448]);
      ws[177184] = fma(kw * y[4352], y[4448], ws[177184]);
    }
    {
      double w = 1.0 * phi[4672];
      w = w - phi[4352];
      w = w - phi[4672];
      const double kw = ws[35968] * w;
      out[4352] = fma(kw, y[4672], out[4352]);
      out[4672] = fma(kw, y[4352], out[4672]);
      ws[177216] = fma(kw * y[4352], y[4672], ws[177216]);
    }
    {
      double w = 0.5 * phi[3648];
      w = fma(0.5, phi[4032], w);
      w = w - phi[4288];
      w = w - phi[4384];
      const double kw = ws[36000] * w;
      out[4288] = fma(kw, y[4384], out[4288]);
      out[4384] = fma(kw, y[4288], out[4384]);
      ws[177248] = fma(kw * y[4288], y[4384], ws[177248]);
    }
    {
      double w = 1.0 * phi[2880];
      w = w - phi[4288];
      w = w - phi[4704];
      const double kw = ws[36032] * w;
      out[4288] = fma(kw, y[4704], out[4288]);
      out[4704] = fma(kw, y[4288], out[4704]);
      ws[177280] = fma(kw * y[4288], y[4704], ws[177280]);
    }
    {
      double w = 0.8 * phi[4704];
      w = fma(0.8, phi[4416], w);
      w = fma(0.2, phi[3904], w);
      w = fma(0.8, phi[4672], w);
      w = w - phi[4288];
      w = w - phi[4448];
      const double kw = ws[36064] * w;
      out[4288] = fma(kw, y[4448], out[4288]);
      out[4448] = fma(kw, y[4288], out[4448]);
      ws[177312] = fma(kw * y[4288], y[4448], ws[177312]);
    }
    {
      double w = 1.0 * phi[4672];
      w = w - phi[4288];
      w = w - phi[4672];
      const double kw = ws[36096] * w;
      out[4288] = fma(kw, y[4672], out[4288]);
      out[4672] = fma(kw, y[4288], out[4672]);
      ws[177344] = fma(kw * y[4288], y[4672], ws[177344]);
    }
    {
      double w = 0.6 * phi[4416];
      w = fma(0.6, phi[4672], w);
      w = fma(0.4, phi[4512], w);
      w = fma(0.4, phi[4736], w);
      w = w - phi[2272];
      w = w - phi[4736];
      const double kw = ws[36128] * w;
      out[2272] = fma(kw, y[4736], out[2272]);
      out[4736] = fma(kw, y[2272], out[4736]);
      ws[177376] = fma(kw * y[2272], y[4736], ws[177376]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4672], w);
      w = fma(1.0, phi[4736], w);
      w = w - phi[2272];
      const double kw = ws[36160] * w;
      out[2272] = out[2272] + kw;
      ws[177408] = fma(kw, y[2272], ws[177408]);
    }
    {
      double w = 0.54 * phi[4576];
      w = fma(0.06, phi[4288], w);
      w = fma(0.6, phi[4672], w);
      w = fma(0.4, phi[4736], w);
      w = w - phi[2880];
      w = w - phi[4736];
      const double kw = ws[36192] * w;
      out[2880] = fma(kw, y[4736], out[2880]);
      out[4736] = fma(kw, y[2880], out[4736]);
      ws[177440] = fma(kw * y[2880], y[4736], ws[177440]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(1.0, phi[4736], w);
      w = w - phi[2880];
      const double kw = ws[36224] * w;
      out[2880] = out[2880] + kw;
      ws[177472] = fma(kw, y[2880], ws[177472]);
    }
    {
      double w = 1.0 * phi[4032];
      w = w - phi[3648];
      w = w - phi[4736];
      const double kw = ws[36256] * w;
      out[3648] = fma(kw, y[4736], out[3648]);
      out[4736] = fma(kw, y[3648], out[4736]);
      ws[177504] = fma(kw * y[3648], y[4736], ws[177504]);
    }
    {
      double w = 1.0 * phi[4608];
      w = w - phi[3648];
      const double kw = ws[36288] * w;
      out[3648] = out[3648] + kw;
      ws[177536] = fma(kw, y[3648], ws[177536]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[3776];
      w = w - phi[4736];
      const double kw = ws[36320] * w;
      out[3776] = fma(kw, y[4736], out[3776]);
      out[4736] = fma(kw, y[3776], out[4736]);
      ws[177568] = fma(kw * y[3776], y[4736], ws[177568]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4672], w);
      w = w - phi[3904];
      w = w - phi[4736];
      const double kw = ws[36352] * w;
      out[3904] = fma(kw, y[4736], out[3904]);
      out[4736] = fma(kw, y[3904], out[4736]);
      ws[177600] = fma(kw * y[3904], y[4736], ws[177600]);
    }
    {
      double w = 1.0 * phi[4448];
      w = w - phi[2688];
      w = w - phi[4736];
      const double kw = ws[36384] * w;
      out[2688] = fma(kw, y[4736], out[2688]);
      out[4736] = fma(kw, y[2688], out[4736]);
      ws[177632] = fma(kw * y[2688], y[4736], ws[177632]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(1.0, phi[4480], w);
      w = w - phi[4512];
      w = w - phi[4736];
      const double kw = ws[36416] * w;
      out[4512] = fma(kw, y[4736], out[4512]);
      out[4736] = fma(kw, y[4512], out[4736]);
      ws[177664] = fma(kw * y[4512], y[4736], ws[177664]);
    }
    {
      double w = 2.0 * phi[4704];
      w = fma(1.0, phi[4480], w);
      w = w - phi[4512];
      const double kw = ws[36448] * w;
      out[4512] = out[4512] + kw;
      ws[177696] = fma(kw, y[4512], ws[177696]);
    }
    {
      double w = 1.0 * phi[4480];
      w = w - phi[4512];
      const double kw = ws[36480] * w;
      out[4512] = out[4512] + kw;
      ws[177728] = fma(kw, y[4512], ws[177728]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4480], w);
      w = w - phi[4512];
      w = w - phi[4160];
      const double kw = ws[36512] * w;
      out[4512] = fma(kw, y[4160], out[4512]);
      out[4160] = fma(kw, y[4512], out[4160]);
      ws[177760] = fma(kw * y[4512], y[4160], ws[177760]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4480], w);
      w = w - phi[4512];
      w = w - phi[4640];
      const double kw = ws[36544] * w;
      out[4512] = fma(kw, y[4640], out[4512]);
      out[4640] = fma(kw, y[4512], out[4640]);
      ws[177792] = fma(kw * y[4512], y[4640], ws[177792]);
    }
    {
      double w = 1.0 * phi[1728];
      w = w - phi[4512];
      w = w - phi[4704];
      const double kw = ws[36576] * w;
      out[4512] = fma(kw, y[4704], out[4512]);
      out[4704] = fma(kw, y[4512], out[4704]);
      ws[177824] = fma(kw * y[4512], y[4704], ws[177824]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(1.0, phi[4704], w);
      w = w - phi[1728];
      const double kw = ws[36608] * w;
      out[1728] = out[1728] + kw;
      ws[177856] = fma(kw, y[1728], ws[177856]);
    }
    {
      double w = 1.0 * phi[3776];
      w = fma(1.0, phi[4608], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[1728];
      w = w - phi[4384];
      const double kw = ws[36640] * w;
      out[1728] = fma(kw, y[4384], out[1728]);
      out[4384] = fma(kw, y[1728], out[4384]);
      ws[177888] = fma(kw * y[1728], y[4384], ws[177888]);
    }
    {
      double w = 0.5 * phi[2272];
      w = fma(0.5, phi[3776], w);
      w = fma(0.2, phi[4736], w);
      w = fma(0.2, phi[4704], w);
      w = w - phi[1728];
      w = w - phi[4704];
      const double kw = ws[36672] * w;
      out[1728] = fma(kw, y[4704], out[1728]);
      out[4704] = fma(kw, y[1728], out[4704]);
      ws[177920] = fma(kw * y[1728], y[4704], ws[177920]);
    }
    {
      double w = 1.0 * phi[4448];
      w = fma(1.0, phi[4736], w);
      w = w - phi[4128];
      w = w - phi[4160];
      const double kw = ws[36704] * w;
      out[4128] = fma(kw, y[4160], out[4128]);
      out[4160] = fma(kw, y[4128], out[4160]);
      ws[177952] = fma(kw * y[4128], y[4160], ws[177952]);
    }
}
__device__ __noinline__ void adj_jtv_0_2(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[4448];
      w = w - phi[4128];
      w = w - phi[4736];
      const double kw = ws[36736] * w;
      out[4128] = fma(kw, y[4736], out[4128]);
      out[4736] = fma(kw, y[4128], out[4736]);
      ws[177984] = fma(kw * y[4128], y[4736], ws[177984]);
    }
    {
      double w = 1.0 * phi[4448];
      w = fma(1.0, phi[4192], w);
      w = w - phi[4128];
      w = w - phi[4640];
      const double kw = ws[36768] * w;
      out[4128] = fma(kw, y[4640], out[4128]);
      out[4640] = fma(kw, y[4128], out[4640]);
      ws[178016] = fma(kw * y[4128], y[4640], ws[178016]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4672], w);
      w = fma(1.0, phi[4480], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[4128];
      const double kw = ws[36800] * w;
      out[4128] = out[4128] + kw;
      ws[178048] = fma(kw, y[4128], ws[178048]);
    }
    {
      double w = 1.0 * phi[4096];
      w = fma(1.0, phi[4736], w);
      w = w - phi[4064];
      w = w - phi[4160];
      const double kw = ws[36832] * w;
      out[4064] = fma(kw, y[4160], out[4064]);
      out[4160] = fma(kw, y[4064], out[4160]);
      ws[178080] = fma(kw * y[4064], y[4160], ws[178080]);
    }
    {
      double w = 1.0 * phi[4096];
      w = w - phi[4064];
      w = w - phi[4736];
      const double kw = ws[36864] * w;
      out[4064] = fma(kw, y[4736], out[4064]);
      out[4736] = fma(kw, y[4064], out[4736]);
      ws[178112] = fma(kw * y[4064], y[4736], ws[178112]);
    }
    {
      double w = 1.0 * phi[4096];
      w = fma(1.0, phi[4192], w);
      w = w - phi[4064];
      w = w - phi[4640];
      const double kw = ws[36896] * w;
      out[4064] = fma(kw, y[4640], out[4064]);
      out[4640] = fma(kw, y[4064], out[4640]);
      ws[178144] = fma(kw * y[4064], y[4640], ws[178144]);
    }
    {
      double w = 1.0 * phi[4128];
      w = fma(1.0, phi[4576], w);
      w = fma(1.0, phi[4672], w);
      w = fma(1.0, phi[4480], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[4064];
      const double kw = ws[36928] * w;
      out[4064] = out[4064] + kw;
      ws[178176] = fma(kw, y[4064], ws[178176]);
    }
    {
      double w = 0.2 * phi[4256];
      w = fma(0.2, phi[4704], w);
      w = fma(0.8, phi[4448], w);
      w = w - phi[3840];
      w = w - phi[4736];
      const double kw = ws[36960] * w;
      out[3840] = fma(kw, y[4736], out[3840]);
      out[4736] = fma(kw, y[3840], out[4736]);
      ws[178208] = fma(kw * y[3840], y[4736], ws[178208]);
    }
    {
      double w = 0.74 * phi[4512];
      w = fma(0.89, phi[4480], w);
      w = fma(1.4, phi[4704], w);
      w = fma(0.15, phi[2720], w);
      w = fma(0.19, phi[4736], w);
      w = fma(0.11, phi[4256], w);
      w = fma(0.11, phi[4576], w);
      w = fma(0.11, phi[4672], w);
      w = w - phi[3840];
      const double kw = ws[36992] * w;
      out[3840] = out[3840] + kw;
      ws[178240] = fma(kw, y[3840], ws[178240]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.0, phi[4448], w);
      w = w - phi[3840];
      w = w - phi[4640];
      const double kw = ws[37024] * w;
      out[3840] = fma(kw, y[4640], out[3840]);
      out[4640] = fma(kw, y[3840], out[4640]);
      ws[178272] = fma(kw * y[3840], y[4640], ws[178272]);
    }
    {
      double w = 1.8 * phi[4480];
      w = fma(0.2, phi[4352], w);
      w = fma(0.2, phi[4672], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[4256];
      w = w - phi[4736];
      const double kw = ws[37056] * w;
      out[4256] = fma(kw, y[4736], out[4256]);
      out[4736] = fma(kw, y[4256], out[4736]);
      ws[178304] = fma(kw * y[4256], y[4736], ws[178304]);
    }
    {
      double w = 2.0 * phi[4704];
      w = fma(2.0, phi[4480], w);
      w = w - phi[4256];
      const double kw = ws[37088] * w;
      out[4256] = out[4256] + kw;
      ws[178336] = fma(kw, y[4256], ws[178336]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.5, phi[4480], w);
      w = fma(0.5, phi[4352], w);
      w = fma(0.5, phi[4672], w);
      w = fma(1.0, phi[4704], w);
      w = w - phi[4256];
      w = w - phi[4640];
      const double kw = ws[37120] * w;
      out[4256] = fma(kw, y[4640], out[4256]);
      out[4640] = fma(kw, y[4256], out[4640]);
      ws[178368] = fma(kw * y[4256], y[4640], ws[178368]);
    }
    {
      double w = 1.0 * phi[4448];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4480], w);
      w = w - phi[4000];
      const double kw = ws[37152] * w;
      out[4000] = out[4000] + kw;
      ws[178400] = fma(kw, y[4000], ws[178400]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.0, phi[4448], w);
      w = fma(1.0, phi[4352], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[4000];
      w = w - phi[4640];
      const double kw = ws[37184] * w;
      out[4000] = fma(kw, y[4640], out[4000]);
      out[4640] = fma(kw, y[4000], out[4640]);
      ws[178432] = fma(kw * y[4000], y[4640], ws[178432]);
    }
    {
      double w = 1.0 * phi[4448];
      w = fma(1.0, phi[4480], w);
      w = w - phi[4000];
      w = w - phi[4736];
      const double kw = ws[37216] * w;
      out[4000] = fma(kw, y[4736], out[4000]);
      out[4736] = fma(kw, y[4000], out[4736]);
      ws[178464] = fma(kw * y[4000], y[4736], ws[178464]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[4736];
      const double kw = ws[37248] * w;
      out[4736] = out[4736] + kw;
      ws[178496] = fma(kw, y[4736], ws[178496]);
    }
    {
      double w = 1.0 * phi[4704];
      w = w - phi[4480];
      w = w - phi[4736];
      const double kw = ws[37280] * w;
      out[4480] = fma(kw, y[4736], out[4480]);
      out[4736] = fma(kw, y[4480], out[4736]);
      ws[178528] = fma(kw * y[4480], y[4736], ws[178528]);
    }
    {
      double w = 1.0 * phi[4416];
      w = fma(1.0, phi[4672], w);
      w = w - phi[4736];
      const double kw = ws[37312] * w;
      out[4736] = out[4736] + kw;
      ws[178560] = fma(kw, y[4736], ws[178560]);
    }
    {
      double w = 0.991 * phi[4128];
      w = fma(0.991, phi[4576], w);
      w = fma(0.009, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[832];
      w = w - phi[4736];
      const double kw = ws[37344] * w;
      out[832] = fma(kw, y[4736], out[832]);
      out[4736] = fma(kw, y[832], out[4736]);
      ws[178592] = fma(kw * y[832], y[4736], ws[178592]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(1.0, phi[4704], w);
      w = w - phi[2720];
      w = w - phi[4736];
      const double kw = ws[37376] * w;
      out[2720] = fma(kw, y[4736], out[2720]);
      out[4736] = fma(kw, y[2720], out[4736]);
      ws[178624] = fma(kw * y[2720], y[4736], ws[178624]);
    }
    {
      double w = 0.95 * phi[4128];
      w = fma(0.9, phi[4704], w);
      w = fma(0.1, phi[4576], w);
      w = fma(0.1, phi[4672], w);
      w = fma(0.078, phi[4512], w);
      w = fma(0.011, phi[3840], w);
      w = w - phi[864];
      w = w - phi[4736];
      const double kw = ws[37408] * w;
      out[864] = fma(kw, y[4736], out[864]);
      out[4736] = fma(kw, y[864], out[4736]);
      ws[178656] = fma(kw * y[864], y[4736], ws[178656]);
    }
    {
      double w = 0.5 * phi[4128];
      w = fma(0.5, phi[4448], w);
      w = fma(0.5, phi[4576], w);
      w = fma(0.5, phi[4096], w);
      w = fma(0.5, phi[4416], w);
      w = fma(1.0, phi[4672], w);
      w = fma(-2.5, phi[4224], w);
      w = w - phi[320];
      const double kw = ws[37440] * w;
      out[320] = out[320] + kw;
      ws[178688] = fma(kw, y[320], ws[178688]);
    }
    {
      double w = 0.38 * phi[4480];
      w = fma(1.38, phi[4416], w);
      w = fma(1.38, phi[4672], w);
      w = fma(0.62, phi[4448], w);
      w = w - phi[3392];
      const double kw = ws[37472] * w;
      out[3392] = out[3392] + kw;
      ws[178720] = fma(kw, y[3392], ws[178720]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(1.0, phi[4448], w);
      w = fma(1.0, phi[4352], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[3392];
      w = w - phi[4736];
      const double kw = ws[37504] * w;
      out[3392] = fma(kw, y[4736], out[3392]);
      out[4736] = fma(kw, y[3392], out[4736]);
      ws[178752] = fma(kw * y[3392], y[4736], ws[178752]);
    }
    {
      double w = 1.0 * phi[928];
      w = w - phi[896];
      w = w - phi[4736];
      const double kw = ws[37536] * w;
      out[896] = fma(kw, y[4736], out[896]);
      out[4736] = fma(kw, y[896], out[4736]);
      ws[178784] = fma(kw * y[896], y[4736], ws[178784]);
    }
    {
      double w = 1.0 * phi[1984];
      w = w - phi[4224];
      w = w - phi[4736];
      const double kw = ws[37568] * w;
      out[4224] = fma(kw, y[4736], out[4224]);
      out[4736] = fma(kw, y[4224], out[4736]);
      ws[178816] = fma(kw * y[4224], y[4736], ws[178816]);
    }
    {
      double w = 0.2 * phi[320];
      w = fma(0.42, phi[3392], w);
      w = fma(0.74, phi[4128], w);
      w = fma(0.37, phi[4064], w);
      w = fma(0.04, phi[4288], w);
      w = fma(0.94, phi[4576], w);
      w = fma(0.98, phi[4672], w);
      w = fma(0.02, phi[960], w);
      w = fma(-2.7, phi[4224], w);
      w = w - phi[960];
      const double kw = ws[37600] * w;
      out[960] = out[960] + kw;
      ws[178848] = fma(kw, y[960], ws[178848]);
    }
    {
      double w = 1.0 * phi[320];
      w = fma(1.0, phi[4704], w);
      w = w - phi[960];
      const double kw = ws[37632] * w;
      out[960] = out[960] + kw;
      ws[178880] = fma(kw, y[960], ws[178880]);
    }
    {
      double w = 1.0 * phi[3648];
      w = w - phi[960];
      w = w - phi[4608];
      const double kw = ws[37664] * w;
      out[960] = fma(kw, y[4608], out[960]);
      out[4608] = fma(kw, y[960], out[4608]);
      ws[178912] = fma(kw * y[960], y[4608], ws[178912]);
    }
    {
      double w = 0.7 * phi[4256];
      w = fma(0.7, phi[4736], w);
      w = fma(0.3, phi[3776], w);
      w = fma(0.3, phi[4480], w);
      w = fma(0.3, phi[4704], w);
      w = w - phi[352];
      w = w - phi[4736];
      const double kw = ws[37696] * w;
      out[352] = fma(kw, y[4736], out[352]);
      out[4736] = fma(kw, y[352], out[4736]);
      ws[178944] = fma(kw * y[352], y[4736], ws[178944]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(1.0, phi[4704], w);
      w = fma(1.0, phi[4480], w);
      w = fma(0.7, phi[4576], w);
      w = fma(0.7, phi[4672], w);
      w = fma(0.3, phi[4736], w);
      w = w - phi[2656];
      w = w - phi[4160];
      const double kw = ws[37728] * w;
      out[2656] = fma(kw, y[4160], out[2656]);
      out[4160] = fma(kw, y[2656], out[4160]);
      ws[178976] = fma(kw * y[2656], y[4160], ws[178976]);
    }
    {
      double w = 1.0 * phi[4576];
      w = fma(1.0, phi[4672], w);
      w = fma(1.56, phi[4512], w);
      w = fma(0.22, phi[3840], w);
      w = w - phi[2656];
      w = w - phi[4736];
      const double kw = ws[37760] * w;
      out[2656] = fma(kw, y[4736], out[2656]);
      out[4736] = fma(kw, y[2656], out[4736]);
      ws[179008] = fma(kw * y[2656], y[4736], ws[179008]);
    }
    {
      double w = 1.0 * phi[4512];
      w = fma(0.35, phi[4480], w);
      w = fma(0.27, phi[4704], w);
      w = fma(0.17, phi[4736], w);
      w = fma(0.42, phi[3776], w);
      w = w - phi[2656];
      w = w - phi[4320];
      const double kw = ws[37792] * w;
      out[2656] = fma(kw, y[4320], out[2656]);
      out[4320] = fma(kw, y[2656], out[4320]);
      ws[179040] = fma(kw * y[2656], y[4320], ws[179040]);
    }
    {
      double w = 0.5 * phi[4608];
      w = fma(0.5, phi[3648], w);
      w = fma(0.5, phi[4576], w);
      w = fma(0.5, phi[4352], w);
      w = fma(1.0, phi[4672], w);
      w = fma(1.125, phi[4512], w);
      w = w - phi[2656];
      w = w - phi[4640];
      const double kw = ws[37824] * w;
      out[2656] = fma(kw, y[4640], out[2656]);
      out[4640] = fma(kw, y[2656], out[4640]);
      ws[179072] = fma(kw * y[2656], y[4640], ws[179072]);
    }
    {
      double w = 0.2 * phi[4128];
      w = fma(0.3, phi[4064], w);
      w = fma(0.1, phi[4704], w);
      w = fma(0.2, phi[4576], w);
      w = fma(0.2, phi[4480], w);
      w = fma(0.2, phi[4512], w);
      w = fma(0.01, phi[4288], w);
      w = fma(0.21, phi[4672], w);
      w = fma(0.2, phi[4224], w);
      w = fma(0.1, phi[4736], w);
      w = w - phi[3552];
      w = w - phi[4160];
      const double kw = ws[37856] * w;
      out[3552] = fma(kw, y[4160], out[3552]);
      out[4160] = fma(kw, y[3552], out[4160]);
      ws[179104] = fma(kw * y[3552], y[4160], ws[179104]);
    }
    {
      double w = 0.781 * phi[4512];
      w = fma(0.488, phi[4128], w);
      w = fma(0.488, phi[4064], w);
      w = fma(0.976, phi[4576], w);
      w = fma(0.195, phi[4352], w);
      w = fma(0.024, phi[4288], w);
      w = fma(1.195, phi[4672], w);
      w = fma(-0.73, phi[4224], w);
      w = w - phi[3552];
      w = w - phi[4736];
      const double kw = ws[37888] * w;
      out[3552] = fma(kw, y[4736], out[3552]);
      out[4736] = fma(kw, y[3552], out[4736]);
      ws[179136] = fma(kw * y[3552], y[4736], ws[179136]);
    }
    {
      double w = 0.295 * phi[4128];
      w = fma(0.555, phi[4512], w);
      w = fma(0.27, phi[4064], w);
      w = fma(0.15, phi[4576], w);
      w = fma(0.15, phi[4672], w);
      w = fma(0.334, phi[4736], w);
      w = fma(0.08, phi[4704], w);
      w = fma(0.378, phi[4480], w);
      w = fma(0.075, phi[4256], w);
      w = fma(0.075, phi[4000], w);
      w = fma(0.09, phi[3776], w);
      w = fma(0.13, phi[3904], w);
      w = fma(0.04, phi[3456], w);
      w = fma(-0.79, phi[4224], w);
      w = w - phi[3552];
      w = w - phi[4320];
      const double kw = ws[37920] * w;
      out[3552] = fma(kw, y[4320], out[3552]);
      out[4320] = fma(kw, y[3552], out[4320]);
      ws[179168] = fma(kw * y[3552], y[4320], ws[179168]);
    }
    {
      double w = 0.5 * phi[4608];
      w = fma(0.5, phi[3648], w);
      w = fma(0.48, phi[4352], w);
      w = fma(0.48, phi[4576], w);
      w = fma(0.04, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = fma(0.5, phi[4512], w);
      w = fma(0.25, phi[4128], w);
      w = fma(0.375, phi[4064], w);
      w = fma(-1.0, phi[4224], w);
      w = w - phi[3552];
      w = w - phi[4640];
      const double kw = ws[37952] * w;
      out[3552] = fma(kw, y[4640], out[3552]);
      out[4640] = fma(kw, y[3552], out[4640]);
      ws[179200] = fma(kw * y[3552], y[4640], ws[179200]);
    }
    {
      double w = 1.24 * phi[4128];
      w = fma(0.66, phi[4064], w);
      w = fma(0.1, phi[4576], w);
      w = fma(0.1, phi[4672], w);
      w = fma(0.1, phi[4480], w);
      w = fma(0.1, phi[4224], w);
      w = w - phi[3136];
      w = w - phi[4160];
      const double kw = ws[37984] * w;
      out[3136] = fma(kw, y[4160], out[3136]);
      out[4160] = fma(kw, y[3136], out[4160]);
      ws[179232] = fma(kw * y[3136], y[4160], ws[179232]);
    }
    {
      double w = 1.3 * phi[4128];
      w = fma(0.7, phi[4064], w);
      w = fma(1.0, phi[4576], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[3136];
      w = w - phi[4736];
      const double kw = ws[38016] * w;
      out[3136] = fma(kw, y[4736], out[3136]);
      out[4736] = fma(kw, y[3136], out[4736]);
      ws[179264] = fma(kw * y[3136], y[4736], ws[179264]);
    }
    {
      double w = 0.732 * phi[4128];
      w = fma(0.442, phi[4064], w);
      w = fma(0.128, phi[4512], w);
      w = fma(0.245, phi[4480], w);
      w = fma(0.5, phi[4736], w);
      w = fma(0.3, phi[4576], w);
      w = fma(0.3, phi[4672], w);
      w = fma(0.24, phi[4256], w);
      w = fma(0.06, phi[4000], w);
      w = fma(0.29, phi[4224], w);
      w = fma(0.08, phi[3904], w);
      w = fma(0.08, phi[3456], w);
      w = w - phi[3136];
      w = w - phi[4320];
      const double kw = ws[38048] * w;
      out[3136] = fma(kw, y[4320], out[3136]);
      out[4320] = fma(kw, y[3136], out[4320]);
      ws[179296] = fma(kw * y[3136], y[4320], ws[179296]);
    }
}
__device__ __noinline__ void adj_jtv_0_3(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 0.5 * phi[4608];
      w = fma(0.5, phi[3648], w);
      w = fma(0.48, phi[4352], w);
      w = fma(0.48, phi[4576], w);
      w = fma(0.04, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = fma(0.5, phi[4128], w);
      w = fma(0.625, phi[4064], w);
      w = fma(1.0, phi[4224], w);
      w = w - phi[3136];
      w = w - phi[4640];
      const double kw = ws[38080] * w;
      out[3136] = fma(kw, y[4640], out[3136]);
      out[4640] = fma(kw, y[3136], out[4640]);
      ws[179328] = fma(kw * y[3136], y[4640], ws[179328]);
    }
    {
      double w = 1.0 * phi[3424];
      w = fma(1.0, phi[4672], w);
      w = fma(1.0, phi[992], w);
      w = w - phi[2528];
      w = w - phi[4736];
      const double kw = ws[38112] * w;
      out[2528] = fma(kw, y[4736], out[2528]);
      out[4736] = fma(kw, y[2528], out[4736]);
      ws[179360] = fma(kw * y[2528], y[4736], ws[179360]);
    }
    {
      double w = 0.75 * phi[3872];
      w = fma(0.5, phi[4512], w);
      w = fma(0.25, phi[4352], w);
      w = fma(0.25, phi[4672], w);
      w = fma(0.25, phi[4704], w);
      w = fma(0.25, phi[4096], w);
      w = fma(0.25, phi[4224], w);
      w = w - phi[2528];
      w = w - phi[4160];
      const double kw = ws[38144] * w;
      out[2528] = fma(kw, y[4160], out[2528]);
      out[4160] = fma(kw, y[2528], out[4160]);
      ws[179392] = fma(kw * y[2528], y[4160], ws[179392]);
    }
    {
      double w = 0.1 * phi[1632];
      w = fma(0.9, phi[4608], w);
      w = fma(0.673, phi[4512], w);
      w = fma(0.9, phi[3872], w);
      w = fma(0.818, phi[4704], w);
      w = fma(0.082, phi[4576], w);
      w = fma(0.082, phi[4672], w);
      w = w - phi[3424];
      w = w - phi[4384];
      const double kw = ws[38176] * w;
      out[3424] = fma(kw, y[4384], out[3424]);
      out[4384] = fma(kw, y[3424], out[4384]);
      ws[179424] = fma(kw * y[3424], y[4384], ws[179424]);
    }
    {
      double w = 0.88 * phi[1664];
      w = fma(0.12, phi[4736], w);
      w = fma(0.12, phi[4704], w);
      w = fma(0.12, phi[4512], w);
      w = fma(0.12, phi[3872], w);
      w = w - phi[3424];
      w = w - phi[4704];
      const double kw = ws[38208] * w;
      out[3424] = fma(kw, y[4704], out[3424]);
      out[4704] = fma(kw, y[3424], out[4704]);
      ws[179456] = fma(kw * y[3424], y[4704], ws[179456]);
    }
    {
      double w = 0.598 * phi[4512];
      w = fma(1.0, phi[3872], w);
      w = fma(0.728, phi[4704], w);
      w = fma(0.072, phi[4576], w);
      w = fma(0.8, phi[4416], w);
      w = fma(0.2, phi[3904], w);
      w = fma(0.872, phi[4672], w);
      w = w - phi[3424];
      w = w - phi[4448];
      const double kw = ws[38240] * w;
      out[3424] = fma(kw, y[4448], out[3424]);
      out[4448] = fma(kw, y[3424], out[4448]);
      ws[179488] = fma(kw * y[3424], y[4448], ws[179488]);
    }
    {
      double w = 0.598 * phi[4512];
      w = fma(1.0, phi[3872], w);
      w = fma(0.728, phi[4704], w);
      w = fma(0.072, phi[4576], w);
      w = fma(1.072, phi[4672], w);
      w = w - phi[3424];
      w = w - phi[4672];
      const double kw = ws[38272] * w;
      out[3424] = fma(kw, y[4672], out[3424]);
      out[4672] = fma(kw, y[3424], out[4672]);
      ws[179520] = fma(kw * y[3424], y[4672], ws[179520]);
    }
    {
      double w = 1.0 * phi[4704];
      w = fma(1.0, phi[1024], w);
      w = w - phi[3424];
      const double kw = ws[38304] * w;
      out[3424] = out[3424] + kw;
      ws[179552] = fma(kw, y[3424], ws[179552]);
    }
    {
      double w = 0.6 * phi[4512];
      w = fma(0.65, phi[3872], w);
      w = fma(0.15, phi[4064], w);
      w = fma(0.2, phi[4096], w);
      w = fma(0.35, phi[4224], w);
      w = fma(0.266, phi[4736], w);
      w = fma(0.2, phi[4352], w);
      w = fma(0.2, phi[4672], w);
      w = fma(0.066, phi[4704], w);
      w = fma(0.066, phi[4480], w);
      w = w - phi[2528];
      w = w - phi[4320];
      const double kw = ws[38336] * w;
      out[2528] = fma(kw, y[4320], out[2528]);
      out[4320] = fma(kw, y[2528], out[4320]);
      ws[179584] = fma(kw * y[2528], y[4320], ws[179584]);
    }
    {
      double w = 0.35 * phi[4608];
      w = fma(0.65, phi[4032], w);
      w = fma(0.64, phi[4576], w);
      w = fma(0.33, phi[4352], w);
      w = fma(0.03, phi[4288], w);
      w = fma(1.0, phi[4672], w);
      w = fma(0.35, phi[4512], w);
      w = fma(0.35, phi[3872], w);
      w = fma(1.0, phi[992], w);
      w = w - phi[2528];
      w = w - phi[4640];
      const double kw = ws[38368] * w;
      out[2528] = fma(kw, y[4640], out[2528]);
      out[4640] = fma(kw, y[2528], out[4640]);
      ws[179616] = fma(kw * y[2528], y[4640], ws[179616]);
    }
    {
      double w = 0.022 * phi[4288];
      w = fma(0.521, phi[4352], w);
      w = fma(0.115, phi[4000], w);
      w = fma(0.115, phi[4416], w);
      w = fma(0.269, phi[3840], w);
      w = fma(0.269, phi[4448], w);
      w = fma(0.457, phi[3744], w);
      w = fma(0.117, phi[4224], w);
      w = fma(0.137, phi[3392], w);
      w = fma(0.137, phi[4480], w);
      w = fma(0.137, phi[4704], w);
      w = fma(0.658, phi[4672], w);
      w = w - phi[3872];
      w = w - phi[4736];
      const double kw = ws[38400] * w;
      out[3872] = fma(kw, y[4736], out[3872]);
      out[4736] = fma(kw, y[3872], out[4736]);
      ws[179648] = fma(kw * y[3872], y[4736], ws[179648]);
    }
    {
      double w = 0.04 * phi[4128];
      w = fma(0.231, phi[4512], w);
      w = fma(0.531, phi[4000], w);
      w = fma(0.17, phi[4256], w);
      w = fma(0.17, phi[3392], w);
      w = fma(0.543, phi[4480], w);
      w = fma(0.461, phi[4736], w);
      w = fma(0.15, phi[3776], w);
      w = fma(0.398, phi[4704], w);
      w = fma(0.143, phi[4448], w);
      w = w - phi[3872];
      w = w - phi[4320];
      const double kw = ws[38432] * w;
      out[3872] = fma(kw, y[4320], out[3872]);
      out[4320] = fma(kw, y[3872], out[4320]);
      ws[179680] = fma(kw * y[3872], y[4320], ws[179680]);
    }
    {
      double w = 0.717 * phi[4192];
      w = fma(0.142, phi[4032], w);
      w = fma(0.142, phi[4608], w);
      w = fma(0.142, phi[4352], w);
      w = fma(0.142, phi[4576], w);
      w = fma(0.113, phi[3840], w);
      w = fma(0.113, phi[4000], w);
      w = fma(0.717, phi[4224], w);
      w = fma(0.717, phi[4096], w);
      w = fma(0.284, phi[4672], w);
      w = w - phi[3872];
      w = w - phi[4640];
      const double kw = ws[38464] * w;
      out[3872] = fma(kw, y[4640], out[3872]);
      out[4640] = fma(kw, y[3872], out[4640]);
      ws[179712] = fma(kw * y[3872], y[4640], ws[179712]);
    }
    {
      double w = 0.76 * phi[4704];
      w = fma(0.34, phi[4576], w);
      w = fma(0.16, phi[4352], w);
      w = fma(0.34, phi[4416], w);
      w = fma(0.208, phi[4448], w);
      w = fma(0.26, phi[4512], w);
      w = fma(0.24, phi[3552], w);
      w = fma(0.24, phi[4224], w);
      w = fma(0.17, phi[3392], w);
      w = fma(0.128, phi[3840], w);
      w = fma(0.84, phi[4672], w);
      w = w - phi[3872];
      const double kw = ws[38496] * w;
      out[3872] = out[3872] + kw;
      ws[179744] = fma(kw, y[3872], ws[179744]);
    }
    {
      double w = 0.904 * phi[1056];
      w = fma(0.933, phi[4736], w);
      w = fma(0.067, phi[3424], w);
      w = fma(0.067, phi[4672], w);
      w = fma(0.029, phi[3136], w);
      w = fma(0.029, phi[4064], w);
      w = w - phi[1664];
      w = w - phi[4736];
      const double kw = ws[38528] * w;
      out[1664] = fma(kw, y[4736], out[1664]);
      out[4736] = fma(kw, y[1664], out[4736]);
      ws[179776] = fma(kw * y[1664], y[4736], ws[179776]);
    }
    {
      double w = 1.0 * phi[4736];
      w = fma(1.0, phi[3872], w);
      w = w - phi[1024];
      const double kw = ws[38560] * w;
      out[1024] = out[1024] + kw;
      ws[179808] = fma(kw, y[1024], ws[179808]);
    }
    {
      double w = 1.0 * phi[4192];
      w = fma(1.0, phi[3872], w);
      w = w - phi[1024];
      w = w - phi[4640];
      const double kw = ws[38592] * w;
      out[1024] = fma(kw, y[4640], out[1024]);
      out[4640] = fma(kw, y[1024], out[4640]);
      ws[179840] = fma(kw * y[1024], y[4640], ws[179840]);
    }
    {
      double w = 1.0 * phi[3296];
      w = fma(1.0, phi[4672], w);
      w = w - phi[1056];
      w = w - phi[4736];
      const double kw = ws[38624] * w;
      out[1056] = fma(kw, y[4736], out[1056]);
      out[4736] = fma(kw, y[1056], out[4736]);
      ws[179872] = fma(kw * y[1056], y[4736], ws[179872]);
    }
    {
      double w = 0.275 * phi[3840];
      w = fma(0.275, phi[4256], w);
      w = fma(0.275, phi[4000], w);
      w = fma(1.125, phi[4736], w);
      w = fma(0.825, phi[4704], w);
      w = fma(0.375, phi[4512], w);
      w = fma(0.074, phi[3776], w);
      w = fma(0.251, phi[4480], w);
      w = fma(2.175, phi[4224], w);
      w = w - phi[3296];
      w = w - phi[4704];
      const double kw = ws[38656] * w;
      out[3296] = fma(kw, y[4704], out[3296]);
      out[4704] = fma(kw, y[3296], out[4704]);
      ws[179904] = fma(kw * y[3296], y[4704], ws[179904]);
    }
    {
      double w = 0.275 * phi[3840];
      w = fma(0.275, phi[4256], w);
      w = fma(0.275, phi[4000], w);
      w = fma(0.125, phi[4736], w);
      w = fma(0.825, phi[4704], w);
      w = fma(0.375, phi[4512], w);
      w = fma(1.0, phi[4608], w);
      w = fma(0.251, phi[4480], w);
      w = fma(2.175, phi[4224], w);
      w = w - phi[3296];
      w = w - phi[4384];
      const double kw = ws[38688] * w;
      out[3296] = fma(kw, y[4384], out[3296]);
      out[4384] = fma(kw, y[3296], out[4384]);
      ws[179936] = fma(kw * y[3296], y[4384], ws[179936]);
    }
    {
      double w = 0.22 * phi[3840];
      w = fma(0.22, phi[4256], w);
      w = fma(0.22, phi[4000], w);
      w = fma(0.1, phi[4736], w);
      w = fma(0.66, phi[4704], w);
      w = fma(0.3, phi[4512], w);
      w = fma(0.2, phi[4480], w);
      w = fma(1.74, phi[4224], w);
      w = fma(0.8, phi[4416], w);
      w = fma(0.2, phi[3904], w);
      w = fma(0.8, phi[4672], w);
      w = w - phi[3296];
      w = w - phi[4448];
      const double kw = ws[38720] * w;
      out[3296] = fma(kw, y[4448], out[3296]);
      out[4448] = fma(kw, y[3296], out[4448]);
      ws[179968] = fma(kw * y[3296], y[4448], ws[179968]);
    }
    {
      double w = 0.275 * phi[3840];
      w = fma(0.275, phi[4256], w);
      w = fma(0.275, phi[4000], w);
      w = fma(0.125, phi[4736], w);
      w = fma(0.825, phi[4704], w);
      w = fma(0.375, phi[4512], w);
      w = fma(0.251, phi[4480], w);
      w = fma(2.175, phi[4224], w);
      w = fma(1.0, phi[4672], w);
      w = w - phi[3296];
      w = w - phi[4672];
      const double kw = ws[38752] * w;
      out[3296] = fma(kw, y[4672], out[3296]);
      out[4672] = fma(kw, y[3296], out[4672]);
      ws[180000] = fma(kw * y[3296], y[4672], ws[180000]);
    }
    {
      double w = 0.63 * phi[4352];
      w = fma(0.37, phi[4576], w);
      w = fma(1.0, phi[4672], w);
      w = fma(0.444, phi[4608], w);
      w = fma(0.185, phi[4640], w);
      w = fma(0.104, phi[1632], w);
      w = fma(0.592, phi[4512], w);
      w = fma(0.331, phi[3840], w);
      w = fma(0.185, phi[3776], w);
      w = fma(2.7, phi[4224], w);
      w = fma(0.098, phi[3552], w);
      w = fma(0.078, phi[4064], w);
      w = fma(0.266, phi[4032], w);
      w = w - phi[1632];
      w = w - phi[4736];
      const double kw = ws[38784] * w;
      out[1632] = fma(kw, y[4736], out[1632]);
      out[4736] = fma(kw, y[1632], out[4736]);
      ws[180032] = fma(kw * y[1632], y[4736], ws[180032]);
    }
    {
      double w = 0.15 * phi[4064];
      w = fma(5.12, phi[4224], w);
      w = fma(1.0, phi[2080], w);
      w = w - phi[2048];
      w = w - phi[4160];
      const double kw = ws[38816] * w;
      out[2048] = fma(kw, y[4160], out[2048]);
      out[4160] = fma(kw, y[2048], out[4160]);
      ws[180064] = fma(kw * y[2048], y[4160], ws[180064]);
    }
    {
      double w = 0.75 * phi[4576];
      w = fma(0.5, phi[4352], w);
      w = fma(0.25, phi[4288], w);
      w = fma(1.5, phi[4672], w);
      w = fma(0.28, phi[4512], w);
      w = fma(1.66, phi[4224], w);
      w = fma(0.47, phi[4064], w);
      w = fma(1.0, phi[2080], w);
      w = w - phi[2048];
      w = w - phi[4736];
      const double kw = ws[38848] * w;
      out[2048] = fma(kw, y[4736], out[2048]);
      out[4736] = fma(kw, y[2048], out[4736]);
      ws[180096] = fma(kw * y[2048], y[4736], ws[180096]);
    }
    {
      double w = 0.57 * phi[4736];
      w = fma(0.07, phi[4576], w);
      w = fma(0.69, phi[4352], w);
      w = fma(0.18, phi[4288], w);
      w = fma(0.94, phi[4672], w);
      w = fma(0.24, phi[4512], w);
      w = fma(0.001, phi[4480], w);
      w = fma(7.0, phi[4224], w);
      w = fma(0.21, phi[4064], w);
      w = fma(0.39, phi[4096], w);
      w = fma(1.0, phi[2080], w);
      w = w - phi[2048];
      w = w - phi[4320];
      const double kw = ws[38880] * w;
      out[2048] = fma(kw, y[4320], out[2048]);
      out[4320] = fma(kw, y[2048], out[4320]);
      ws[180128] = fma(kw * y[2048], y[4320], ws[180128]);
    }
    {
      double w = 0.47 * phi[4608];
      w = fma(0.28, phi[4576], w);
      w = fma(0.75, phi[4352], w);
      w = fma(0.25, phi[4288], w);
      w = fma(1.28, phi[4672], w);
      w = fma(0.47, phi[4064], w);
      w = fma(0.53, phi[4032], w);
      w = fma(1.0, phi[2848], w);
      w = w - phi[2048];
      w = w - phi[4640];
      const double kw = ws[38912] * w;
      out[2048] = fma(kw, y[4640], out[2048]);
      out[4640] = fma(kw, y[2048], out[4640]);
      ws[180160] = fma(kw * y[2048], y[4640], ws[180160]);
    }
    {
      double w = 0.15 * phi[4064];
      w = fma(5.12, phi[4224], w);
      w = fma(1.0, phi[2080], w);
      w = w - phi[2112];
      w = w - phi[4160];
      const double kw = ws[38944] * w;
      out[2112] = fma(kw, y[4160], out[2112]);
      out[4160] = fma(kw, y[2112], out[4160]);
      ws[180192] = fma(kw * y[2112], y[4160], ws[180192]);
    }
    {
      double w = 0.75 * phi[4576];
      w = fma(0.5, phi[4352], w);
      w = fma(0.25, phi[4288], w);
      w = fma(1.5, phi[4672], w);
      w = fma(0.28, phi[4512], w);
      w = fma(1.66, phi[4224], w);
      w = fma(0.47, phi[4064], w);
      w = fma(1.0, phi[2080], w);
      w = w - phi[2112];
      w = w - phi[4736];
      const double kw = ws[38976] * w;
      out[2112] = fma(kw, y[4736], out[2112]);
      out[4736] = fma(kw, y[2112], out[4736]);
      ws[180224] = fma(kw * y[2112], y[4736], ws[180224]);
    }
    {
      double w = 0.57 * phi[4736];
      w = fma(0.07, phi[4576], w);
      w = fma(0.69, phi[4352], w);
      w = fma(0.18, phi[4288], w);
      w = fma(0.94, phi[4672], w);
      w = fma(0.24, phi[4512], w);
      w = fma(0.001, phi[4480], w);
      w = fma(7.0, phi[4224], w);
      w = fma(0.21, phi[4064], w);
      w = fma(0.39, phi[4096], w);
      w = fma(1.0, phi[2080], w);
      w = w - phi[2112];
      w = w - phi[4320];
      const double kw = ws[39008] * w;
      out[2112] = fma(kw, y[4320], out[2112]);
      out[4320] = fma(kw, y[2112], out[4320]);
      ws[180256] = fma(kw * y[2112], y[4320], ws[180256]);
    }
    {
      double w = 0.47 * phi[4608];
      w = fma(0.28, phi[4576], w);
      w = fma(0.75, phi[4352], w);
      w = fma(0.25, phi[4288], w);
      w = fma(1.28, phi[4672], w);
      w = fma(0.47, phi[4064], w);
      w = fma(0.53, phi[4032], w);
      w = w - phi[2112];
      w = w - phi[4640];
      const double kw = ws[39040] * w;
      out[2112] = fma(kw, y[4640], out[2112]);
      out[4640] = fma(kw, y[2112], out[4640]);
      ws[180288] = fma(kw * y[2112], y[4640], ws[180288]);
    }
    {
      double w = 0.53 * phi[3616];
      w = fma(0.352, phi[3104], w);
      w = fma(0.352, phi[4672], w);
      w = fma(0.118, phi[3936], w);
      w = fma(0.118, phi[4736], w);
      w = fma(0.53, phi[4704], w);
      w = fma(1.0, phi[2144], w);
      w = w - phi[384];
      w = w - phi[4736];
      const double kw = ws[39072] * w;
      out[384] = fma(kw, y[4736], out[384]);
      out[4736] = fma(kw, y[384], out[4736]);
      ws[180320] = fma(kw * y[384], y[4736], ws[180320]);
    }
    {
      double w = 0.918 * phi[4608];
      w = fma(0.082, phi[4032], w);
      w = fma(0.918, phi[4256], w);
      w = fma(0.918, phi[3936], w);
      w = fma(0.918, phi[4704], w);
      w = w - phi[3104];
      w = w - phi[4384];
      const double kw = ws[39104] * w;
      out[3104] = fma(kw, y[4384], out[3104]);
      out[4384] = fma(kw, y[3104], out[4384]);
      ws[180352] = fma(kw * y[3104], y[4384], ws[180352]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
