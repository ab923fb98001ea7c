// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 4242f44b2527a299).  Do not edit.
#include "cb6r5_ae7_aq_mech.cuh"
#include <math.h>
namespace mech_cb6r5_ae7_aq {
__device__ __noinline__ void ddm_jv_0_0(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[33376] * v[4608];
      out[4608] = out[4608] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[33408] * v[4160];
      out[4160] = out[4160] - dr;
      out[4320] = fma(1.0, dr, out[4320]);
    }
    {
      const double dr = ws[33440] * fma(y[4384], v[4320], y[4320] * v[4384]);
      out[4320] = out[4320] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[33472] * fma(y[4384], v[4160], y[4160] * v[4384]);
      out[4160] = out[4160] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[33504] * fma(y[4608], v[4160], y[4160] * v[4608]);
      out[4160] = out[4160] - dr;
      out[4608] = out[4608] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
    }
    {
      const double dr = ws[33536] * fma(y[4608], v[4160], y[4160] * v[4608]);
      out[4160] = out[4160] - dr;
      out[4608] = out[4608] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[33568] * fma(y[4320], v[4160], y[4160] * v[4320]);
      out[4160] = out[4160] - dr;
      out[4320] = out[4320] - dr;
    }
    {
      const double dr = ws[33600] * v[4320];
      out[4320] = out[4320] - dr;
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[33632] * v[4320];
      out[4320] = out[4320] - dr;
      out[672] = fma(1.0, dr, out[672]);
    }
    {
      const double dr = ws[33664] * v[672];
      out[672] = out[672] - dr;
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[33696] * v[672];
      out[672] = out[672] - dr;
      out[4736] = fma(2.0, dr, out[4736]);
    }
    {
      const double dr = ws[33728] * fma(y[4736], v[4320], y[4320] * v[4736]);
      out[4320] = out[4320] - dr;
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[33760] * fma(y[4704], v[4320], y[4320] * v[4704]);
      out[4320] = out[4320] - dr;
      out[4704] = out[4704] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[33792] * fma(y[4160], v[4736], y[4736] * v[4160]);
      out[4736] = out[4736] - dr;
      out[4160] = out[4160] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[33824] * fma(y[4160], v[4704], y[4704] * v[4160]);
      out[4704] = out[4704] - dr;
      out[4160] = out[4160] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[33856] * fma(y[4736], v[4736], y[4736] * v[4736]);
      out[4736] = out[4736] - dr;
      out[4736] = out[4736] - dr;
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[33888] * fma(y[4736], v[4736], y[4736] * v[4736]);
      out[4736] = out[4736] - dr;
      out[4736] = out[4736] - dr;
      out[3456] = fma(1.0, dr, out[3456]);
    }
    {
      const double dr = ws[33920] * fma(y[4704], v[4736], y[4736] * v[4704]);
      out[4736] = out[4736] - dr;
      out[4704] = out[4704] - dr;
    }
    {
      const double dr = ws[33952] * fma(y[4704], v[4704], y[4704] * v[4704]);
      out[4704] = out[4704] - dr;
      out[4704] = out[4704] - dr;
      out[3456] = fma(1.0, dr, out[3456]);
    }
    {
      const double dr = ws[33984] * fma(y[4704], v[4704], y[4704] * v[4704]);
      out[4704] = out[4704] - dr;
      out[4704] = out[4704] - dr;
      out[3456] = fma(1.0, dr, out[3456]);
    }
    {
      const double dr = ws[34016] * v[3456];
      out[3456] = out[3456] - dr;
      out[4736] = fma(2.0, dr, out[4736]);
    }
    {
      const double dr = ws[34048] * fma(y[4736], v[3456], y[3456] * v[4736]);
      out[3456] = out[3456] - dr;
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[34080] * fma(y[4160], v[3456], y[3456] * v[4160]);
      out[3456] = out[3456] - dr;
      out[4160] = out[4160] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[34112] * fma(y[4384], v[4384], y[4384] * v[4384]);
      out[4384] = out[4384] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(2.0, dr, out[4608]);
    }
    {
      const double dr = ws[34144] * fma(y[4384], v[4704], y[4704] * v[4384]);
      out[4704] = out[4704] - dr;
      out[4384] = out[4384] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34176] * fma(y[4320], v[4608], y[4608] * v[4320]);
      out[4608] = out[4608] - dr;
      out[4320] = out[4320] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[34208] * v[4640];
      out[4640] = out[4640] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4160] = fma(1.0, dr, out[4160]);
    }
    {
      const double dr = ws[34240] * v[4640];
      out[4640] = out[4640] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
    }
    {
      const double dr = ws[34272] * fma(y[4384], v[4640], y[4640] * v[4384]);
      out[4640] = out[4640] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(2.0, dr, out[4608]);
    }
    {
      const double dr = ws[34304] * fma(y[4608], v[4640], y[4640] * v[4608]);
      out[4640] = out[4640] - dr;
      out[4608] = out[4608] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34336] * fma(y[4160], v[4640], y[4640] * v[4160]);
      out[4640] = out[4640] - dr;
      out[4160] = out[4160] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34368] * fma(y[4736], v[4640], y[4640] * v[4736]);
      out[4640] = out[4640] - dr;
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34400] * fma(y[4704], v[4640], y[4640] * v[4704]);
      out[4640] = out[4640] - dr;
      out[4704] = out[4704] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34432] * fma(y[4320], v[4640], y[4640] * v[4320]);
      out[4640] = out[4640] - dr;
      out[4320] = out[4320] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34464] * fma(y[4640], v[4640], y[4640] * v[4640]);
      out[4640] = out[4640] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(2.0, dr, out[4608]);
    }
    {
      const double dr = ws[34496] * fma(y[4608], v[4640], y[4640] * v[4608]);
      out[4640] = out[4640] - dr;
      out[4608] = out[4608] - dr;
      out[1280] = fma(1.0, dr, out[1280]);
    }
    {
      const double dr = ws[34528] * v[1280];
      out[1280] = out[1280] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34560] * v[1280];
      out[1280] = out[1280] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[34592] * v[1280];
      out[1280] = out[1280] - dr;
      out[4192] = fma(2.0, dr, out[4192]);
    }
    {
      const double dr = ws[34624] * fma(y[4736], v[4384], y[4384] * v[4736]);
      out[4384] = out[4384] - dr;
      out[4736] = out[4736] - dr;
      out[2464] = fma(1.0, dr, out[2464]);
    }
    {
      const double dr = ws[34656] * fma(y[4608], v[4384], y[4384] * v[4608]);
      out[4384] = out[4384] - dr;
      out[4608] = out[4608] - dr;
      out[2464] = fma(2.0, dr, out[2464]);
    }
    {
      const double dr = ws[34688] * fma(y[2464], v[2464], y[2464] * v[2464]);
      out[2464] = out[2464] - dr;
      out[2464] = out[2464] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34720] * v[2464];
      out[2464] = out[2464] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[34752] * fma(y[4736], v[2464], y[2464] * v[4736]);
      out[2464] = out[2464] - dr;
      out[4736] = out[4736] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34784] * fma(y[4736], v[4608], y[4608] * v[4736]);
      out[4608] = out[4608] - dr;
      out[4736] = out[4736] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[34816] * fma(y[4736], v[4192], y[4192] * v[4736]);
      out[4192] = out[4192] - dr;
      out[4736] = out[4736] - dr;
      out[4640] = fma(1.0, dr, out[4640]);
    }
    {
      const double dr = ws[34848] * v[4192];
      out[4192] = out[4192] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34880] * fma(y[4608], v[4704], y[4704] * v[4608]);
      out[4704] = out[4704] - dr;
      out[4608] = out[4608] - dr;
      out[1696] = fma(1.0, dr, out[1696]);
    }
    {
      const double dr = ws[34912] * v[1696];
      out[1696] = out[1696] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[34944] * v[1696];
      out[1696] = out[1696] - dr;
      out[4704] = fma(0.59, dr, out[4704]);
      out[4608] = fma(0.59, dr, out[4608]);
      out[4736] = fma(0.41, dr, out[4736]);
      out[4640] = fma(0.41, dr, out[4640]);
    }
    {
      const double dr = ws[34976] * fma(y[4736], v[1696], y[1696] * v[4736]);
      out[1696] = out[1696] - dr;
      out[4736] = out[4736] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[35008] * fma(y[4736], v[2208], y[2208] * v[4736]);
      out[2208] = out[2208] - dr;
      out[4736] = out[4736] - dr;
      out[256] = fma(1.0, dr, out[256]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[288] = fma(1.0, dr, out[288]);
    }
    {
      const double dr = ws[35040] * fma(y[4384], v[4448], y[4448] * v[4384]);
      out[4448] = out[4448] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[35072] * fma(y[4608], v[4448], y[4448] * v[4608]);
      out[4448] = out[4448] - dr;
      out[4608] = out[4608] - dr;
      out[1344] = fma(1.0, dr, out[1344]);
    }
    {
      const double dr = ws[35104] * v[1344];
      out[1344] = out[1344] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[35136] * v[1344];
      out[1344] = out[1344] - dr;
      out[4608] = fma(0.6, dr, out[4608]);
      out[4448] = fma(0.6, dr, out[4448]);
      out[4640] = fma(0.4, dr, out[4640]);
      out[4416] = fma(0.4, dr, out[4416]);
      out[4672] = fma(0.4, dr, out[4672]);
    }
    {
      const double dr = ws[35168] * fma(y[4704], v[4448], y[4448] * v[4704]);
      out[4448] = out[4448] - dr;
      out[4704] = out[4704] - dr;
      out[2688] = fma(0.37, dr, out[2688]);
      out[3904] = fma(0.13, dr, out[3904]);
      out[4320] = fma(0.13, dr, out[4320]);
      out[4416] = fma(0.5, dr, out[4416]);
      out[4672] = fma(0.5, dr, out[4672]);
      out[4736] = fma(0.5, dr, out[4736]);
    }
    {
      const double dr = ws[35200] * fma(y[4672], v[4448], y[4448] * v[4672]);
      out[4448] = out[4448] - dr;
      out[4672] = out[4672] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
    }
    {
      const double dr = ws[35232] * fma(y[4448], v[4448], y[4448] * v[4448]);
      out[4448] = out[4448] - dr;
      out[4448] = out[4448] - dr;
      out[4416] = fma(2.0, dr, out[4416]);
      out[4672] = fma(2.0, dr, out[4672]);
    }
    {
      const double dr = ws[35264] * fma(y[4096], v[4448], y[4448] * v[4096]);
      out[4448] = out[4448] - dr;
      out[4096] = out[4096] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4128] = fma(1.0, dr, out[4128]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[4672] = fma(2.0, dr, out[4672]);
    }
    {
      const double dr = ws[35296] * fma(y[4384], v[4096], y[4096] * v[4384]);
      out[4096] = out[4096] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4128] = fma(1.0, dr, out[4128]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[35328] * fma(y[4608], v[4096], y[4096] * v[4608]);
      out[4096] = out[4096] - dr;
      out[4608] = out[4608] - dr;
      out[1952] = fma(1.0, dr, out[1952]);
    }
    {
      const double dr = ws[35360] * v[1952];
      out[1952] = out[1952] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4096] = fma(1.0, dr, out[4096]);
    }
    {
      const double dr = ws[35392] * v[1952];
      out[1952] = out[1952] - dr;
      out[4608] = fma(0.6, dr, out[4608]);
      out[4096] = fma(0.6, dr, out[4096]);
      out[4640] = fma(0.4, dr, out[4640]);
      out[4128] = fma(0.4, dr, out[4128]);
      out[4576] = fma(0.4, dr, out[4576]);
      out[4672] = fma(0.4, dr, out[4672]);
    }
    {
      const double dr = ws[35424] * fma(y[4704], v[4096], y[4096] * v[4704]);
      out[4096] = out[4096] - dr;
      out[4704] = out[4704] - dr;
      out[2688] = fma(0.37, dr, out[2688]);
      out[3904] = fma(0.13, dr, out[3904]);
      out[4320] = fma(0.13, dr, out[4320]);
      out[4736] = fma(0.5, dr, out[4736]);
      out[4416] = fma(0.5, dr, out[4416]);
      out[4672] = fma(0.5, dr, out[4672]);
    }
    {
      const double dr = ws[35456] * fma(y[4672], v[4096], y[4096] * v[4672]);
      out[4096] = out[4096] - dr;
      out[4672] = out[4672] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
    }
    {
      const double dr = ws[35488] * fma(y[4096], v[4096], y[4096] * v[4096]);
      out[4096] = out[4096] - dr;
      out[4096] = out[4096] - dr;
      out[4416] = fma(2.0, dr, out[4416]);
      out[4672] = fma(2.0, dr, out[4672]);
    }
    {
      const double dr = ws[35520] * fma(y[4384], v[4672], y[4672] * v[4384]);
      out[4672] = out[4672] - dr;
      out[4384] = out[4384] - dr;
      out[4384] = fma(1.0, dr, out[4384]);
    }
    {
      const double dr = ws[35552] * fma(y[4704], v[4672], y[4672] * v[4704]);
      out[4672] = out[4672] - dr;
      out[4704] = out[4704] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[35584] * fma(y[4672], v[4672], y[4672] * v[4672]);
      out[4672] = out[4672] - dr;
      out[4672] = out[4672] - dr;
    }
    {
      const double dr = ws[35616] * fma(y[4384], v[4416], y[4416] * v[4384]);
      out[4416] = out[4416] - dr;
      out[4384] = out[4384] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[35648] * fma(y[4704], v[4416], y[4416] * v[4704]);
      out[4416] = out[4416] - dr;
      out[4704] = out[4704] - dr;
      out[2272] = fma(0.9, dr, out[2272]);
      out[4512] = fma(0.1, dr, out[4512]);
    }
    {
      const double dr = ws[35680] * fma(y[4448], v[4416], y[4416] * v[4448]);
      out[4416] = out[4416] - dr;
      out[4448] = out[4448] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4704] = fma(0.9, dr, out[4704]);
      out[4416] = fma(0.9, dr, out[4416]);
      out[3904] = fma(0.1, dr, out[3904]);
      out[4672] = fma(0.9, dr, out[4672]);
    }
    {
      const double dr = ws[35712] * fma(y[4672], v[4416], y[4416] * v[4672]);
      out[4416] = out[4416] - dr;
      out[4672] = out[4672] - dr;
      out[4512] = fma(0.685, dr, out[4512]);
      out[2720] = fma(0.315, dr, out[2720]);
      out[4704] = fma(0.37, dr, out[4704]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[35744] * fma(y[4384], v[4576], y[4576] * v[4384]);
      out[4576] = out[4576] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[35776] * fma(y[4704], v[4576], y[4576] * v[4704]);
      out[4576] = out[4576] - dr;
      out[4704] = out[4704] - dr;
      out[2880] = fma(1.0, dr, out[2880]);
    }
}
__device__ __noinline__ void ddm_jv_0_1(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[35808] * fma(y[4448], v[4576], y[4576] * v[4448]);
      out[4576] = out[4576] - dr;
      out[4448] = out[4448] - dr;
      out[4704] = fma(0.8, dr, out[4704]);
      out[4416] = fma(0.8, dr, out[4416]);
      out[3904] = fma(0.2, dr, out[3904]);
      out[4672] = fma(0.8, dr, out[4672]);
    }
    {
      const double dr = ws[35840] * fma(y[4672], v[4576], y[4576] * v[4672]);
      out[4576] = out[4576] - dr;
      out[4672] = out[4672] - dr;
      out[4704] = fma(0.6, dr, out[4704]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[35872] * fma(y[4384], v[4352], y[4352] * v[4384]);
      out[4352] = out[4352] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[35904] * fma(y[4704], v[4352], y[4352] * v[4704]);
      out[4352] = out[4352] - dr;
      out[4704] = out[4704] - dr;
      out[2880] = fma(1.0, dr, out[2880]);
    }
    {
      const double dr = ws[35936] * fma(y[4448], v[4352], y[4352] * v[4448]);
      out[4352] = out[4352] - dr;
      out[4448] = out[4448] - dr;
      out[4416] = fma(0.8, dr, out[4416]);
      out[3904] = fma(0.2, dr, out[3904]);
      out[4672] = fma(0.8, dr, out[4672]);
    }
    {
      const double dr = ws[35968] * fma(y[4672], v[4352], y[4352] * v[4672]);
      out[4352] = out[4352] - dr;
      out[4672] = out[4672] - dr;
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[36000] * fma(y[4384], v[4288], y[4288] * v[4384]);
      out[4288] = out[4288] - dr;
      out[4384] = out[4384] - dr;
      out[3648] = fma(0.5, dr, out[3648]);
      out[4032] = fma(0.5, dr, out[4032]);
    }
    {
      const double dr = ws[36032] * fma(y[4704], v[4288], y[4288] * v[4704]);
      out[4288] = out[4288] - dr;
      out[4704] = out[4704] - dr;
      out[2880] = fma(1.0, dr, out[2880]);
    }
    {
      const double dr = ws[36064] * fma(y[4448], v[4288], y[4288] * v[4448]);
      out[4288] = out[4288] - dr;
      out[4448] = out[4448] - dr;
      out[4704] = fma(0.8, dr, out[4704]);
      out[4416] = fma(0.8, dr, out[4416]);
      out[3904] = fma(0.2, dr, out[3904]);
      out[4672] = fma(0.8, dr, out[4672]);
    }
    {
      const double dr = ws[36096] * fma(y[4672], v[4288], y[4288] * v[4672]);
      out[4288] = out[4288] - dr;
      out[4672] = out[4672] - dr;
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[36128] * fma(y[4736], v[2272], y[2272] * v[4736]);
      out[2272] = out[2272] - dr;
      out[4736] = out[4736] - dr;
      out[4416] = fma(0.6, dr, out[4416]);
      out[4672] = fma(0.6, dr, out[4672]);
      out[4512] = fma(0.4, dr, out[4512]);
      out[4736] = fma(0.4, dr, out[4736]);
    }
    {
      const double dr = ws[36160] * v[2272];
      out[2272] = out[2272] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[36192] * fma(y[4736], v[2880], y[2880] * v[4736]);
      out[2880] = out[2880] - dr;
      out[4736] = out[4736] - dr;
      out[4576] = fma(0.54, dr, out[4576]);
      out[4288] = fma(0.06, dr, out[4288]);
      out[4672] = fma(0.6, dr, out[4672]);
      out[4736] = fma(0.4, dr, out[4736]);
    }
    {
      const double dr = ws[36224] * v[2880];
      out[2880] = out[2880] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[36256] * fma(y[4736], v[3648], y[3648] * v[4736]);
      out[3648] = out[3648] - dr;
      out[4736] = out[4736] - dr;
      out[4032] = fma(1.0, dr, out[4032]);
    }
    {
      const double dr = ws[36288] * v[3648];
      out[3648] = out[3648] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[36320] * fma(y[4736], v[3776], y[3776] * v[4736]);
      out[3776] = out[3776] - dr;
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[36352] * fma(y[4736], v[3904], y[3904] * v[4736]);
      out[3904] = out[3904] - dr;
      out[4736] = out[4736] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[36384] * fma(y[4736], v[2688], y[2688] * v[4736]);
      out[2688] = out[2688] - dr;
      out[4736] = out[4736] - dr;
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[36416] * fma(y[4736], v[4512], y[4512] * v[4736]);
      out[4512] = out[4512] - dr;
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[36448] * v[4512];
      out[4512] = out[4512] - dr;
      out[4704] = fma(2.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[36480] * v[4512];
      out[4512] = out[4512] - dr;
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[36512] * fma(y[4160], v[4512], y[4512] * v[4160]);
      out[4512] = out[4512] - dr;
      out[4160] = out[4160] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[36544] * fma(y[4640], v[4512], y[4512] * v[4640]);
      out[4512] = out[4512] - dr;
      out[4640] = out[4640] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[36576] * fma(y[4704], v[4512], y[4512] * v[4704]);
      out[4512] = out[4512] - dr;
      out[4704] = out[4704] - dr;
      out[1728] = fma(1.0, dr, out[1728]);
    }
    {
      const double dr = ws[36608] * v[1728];
      out[1728] = out[1728] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[36640] * fma(y[4384], v[1728], y[1728] * v[4384]);
      out[1728] = out[1728] - dr;
      out[4384] = out[4384] - dr;
      out[3776] = fma(1.0, dr, out[3776]);
      out[4608] = fma(1.0, dr, out[4608]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[36672] * fma(y[4704], v[1728], y[1728] * v[4704]);
      out[1728] = out[1728] - dr;
      out[4704] = out[4704] - dr;
      out[2272] = fma(0.5, dr, out[2272]);
      out[3776] = fma(0.5, dr, out[3776]);
      out[4736] = fma(0.2, dr, out[4736]);
      out[4704] = fma(0.2, dr, out[4704]);
    }
    {
      const double dr = ws[36704] * fma(y[4160], v[4128], y[4128] * v[4160]);
      out[4128] = out[4128] - dr;
      out[4160] = out[4160] - dr;
      out[4448] = fma(1.0, dr, out[4448]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[36736] * fma(y[4736], v[4128], y[4128] * v[4736]);
      out[4128] = out[4128] - dr;
      out[4736] = out[4736] - dr;
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[36768] * fma(y[4640], v[4128], y[4128] * v[4640]);
      out[4128] = out[4128] - dr;
      out[4640] = out[4640] - dr;
      out[4448] = fma(1.0, dr, out[4448]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[36800] * v[4128];
      out[4128] = out[4128] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4480] = fma(1.0, dr, out[4480]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[36832] * fma(y[4160], v[4064], y[4064] * v[4160]);
      out[4064] = out[4064] - dr;
      out[4160] = out[4160] - dr;
      out[4096] = fma(1.0, dr, out[4096]);
      out[4736] = fma(1.0, dr, out[4736]);
    }
    {
      const double dr = ws[36864] * fma(y[4736], v[4064], y[4064] * v[4736]);
      out[4064] = out[4064] - dr;
      out[4736] = out[4736] - dr;
      out[4096] = fma(1.0, dr, out[4096]);
    }
    {
      const double dr = ws[36896] * fma(y[4640], v[4064], y[4064] * v[4640]);
      out[4064] = out[4064] - dr;
      out[4640] = out[4640] - dr;
      out[4096] = fma(1.0, dr, out[4096]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[36928] * v[4064];
      out[4064] = out[4064] - dr;
      out[4128] = fma(1.0, dr, out[4128]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4480] = fma(1.0, dr, out[4480]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[36960] * fma(y[4736], v[3840], y[3840] * v[4736]);
      out[3840] = out[3840] - dr;
      out[4736] = out[4736] - dr;
      out[4256] = fma(0.2, dr, out[4256]);
      out[4704] = fma(0.2, dr, out[4704]);
      out[4448] = fma(0.8, dr, out[4448]);
    }
    {
      const double dr = ws[36992] * v[3840];
      out[3840] = out[3840] - dr;
      out[4512] = fma(0.74, dr, out[4512]);
      out[4480] = fma(0.89, dr, out[4480]);
      out[4704] = fma(1.4, dr, out[4704]);
      out[2720] = fma(0.15, dr, out[2720]);
      out[4736] = fma(0.19, dr, out[4736]);
      out[4256] = fma(0.11, dr, out[4256]);
      out[4576] = fma(0.11, dr, out[4576]);
      out[4672] = fma(0.11, dr, out[4672]);
    }
    {
      const double dr = ws[37024] * fma(y[4640], v[3840], y[3840] * v[4640]);
      out[3840] = out[3840] - dr;
      out[4640] = out[4640] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[4448] = fma(1.0, dr, out[4448]);
    }
    {
      const double dr = ws[37056] * fma(y[4736], v[4256], y[4256] * v[4736]);
      out[4256] = out[4256] - dr;
      out[4736] = out[4736] - dr;
      out[4480] = fma(1.8, dr, out[4480]);
      out[4352] = fma(0.2, dr, out[4352]);
      out[4672] = fma(0.2, dr, out[4672]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[37088] * v[4256];
      out[4256] = out[4256] - dr;
      out[4704] = fma(2.0, dr, out[4704]);
      out[4480] = fma(2.0, dr, out[4480]);
    }
    {
      const double dr = ws[37120] * fma(y[4640], v[4256], y[4256] * v[4640]);
      out[4256] = out[4256] - dr;
      out[4640] = out[4640] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[4480] = fma(1.5, dr, out[4480]);
      out[4352] = fma(0.5, dr, out[4352]);
      out[4672] = fma(0.5, dr, out[4672]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[37152] * v[4000];
      out[4000] = out[4000] - dr;
      out[4448] = fma(1.0, dr, out[4448]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[37184] * fma(y[4640], v[4000], y[4000] * v[4640]);
      out[4000] = out[4000] - dr;
      out[4640] = out[4640] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[4448] = fma(1.0, dr, out[4448]);
      out[4352] = fma(1.0, dr, out[4352]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[37216] * fma(y[4736], v[4000], y[4000] * v[4736]);
      out[4000] = out[4000] - dr;
      out[4736] = out[4736] - dr;
      out[4448] = fma(1.0, dr, out[4448]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[37248] * v[4736];
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[37280] * fma(y[4736], v[4480], y[4480] * v[4736]);
      out[4480] = out[4480] - dr;
      out[4736] = out[4736] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[37312] * v[4736];
      out[4736] = out[4736] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[37344] * fma(y[4736], v[832], y[832] * v[4736]);
      out[832] = out[832] - dr;
      out[4736] = out[4736] - dr;
      out[4128] = fma(0.991, dr, out[4128]);
      out[4576] = fma(0.991, dr, out[4576]);
      out[4288] = fma(0.009, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[37376] * fma(y[4736], v[2720], y[2720] * v[4736]);
      out[2720] = out[2720] - dr;
      out[4736] = out[4736] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[37408] * fma(y[4736], v[864], y[864] * v[4736]);
      out[864] = out[864] - dr;
      out[4736] = out[4736] - dr;
      out[4128] = fma(0.95, dr, out[4128]);
      out[4704] = fma(0.9, dr, out[4704]);
      out[4576] = fma(0.1, dr, out[4576]);
      out[4672] = fma(0.1, dr, out[4672]);
      out[4512] = fma(0.078, dr, out[4512]);
      out[3840] = fma(0.011, dr, out[3840]);
    }
    {
      const double dr = ws[37440] * v[320];
      out[320] = out[320] - dr;
      out[4128] = fma(0.5, dr, out[4128]);
      out[4448] = fma(0.5, dr, out[4448]);
      out[4576] = fma(0.5, dr, out[4576]);
      out[4096] = fma(0.5, dr, out[4096]);
      out[4416] = fma(0.5, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4224] = fma(-2.5, dr, out[4224]);
    }
    {
      const double dr = ws[37472] * v[3392];
      out[3392] = out[3392] - dr;
      out[4480] = fma(0.38, dr, out[4480]);
      out[4416] = fma(1.38, dr, out[4416]);
      out[4672] = fma(1.38, dr, out[4672]);
      out[4448] = fma(0.62, dr, out[4448]);
    }
    {
      const double dr = ws[37504] * fma(y[4736], v[3392], y[3392] * v[4736]);
      out[3392] = out[3392] - dr;
      out[4736] = out[4736] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4448] = fma(1.0, dr, out[4448]);
      out[4352] = fma(1.0, dr, out[4352]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[37536] * fma(y[4736], v[896], y[896] * v[4736]);
      out[896] = out[896] - dr;
      out[4736] = out[4736] - dr;
      out[928] = fma(1.0, dr, out[928]);
    }
    {
      const double dr = ws[37568] * fma(y[4736], v[4224], y[4224] * v[4736]);
      out[4224] = out[4224] - dr;
      out[4736] = out[4736] - dr;
      out[1984] = fma(1.0, dr, out[1984]);
    }
    {
      const double dr = ws[37600] * v[960];
      out[960] = out[960] - dr;
      out[320] = fma(0.2, dr, out[320]);
      out[3392] = fma(0.42, dr, out[3392]);
      out[4128] = fma(0.74, dr, out[4128]);
      out[4064] = fma(0.37, dr, out[4064]);
      out[4288] = fma(0.04, dr, out[4288]);
      out[4576] = fma(0.94, dr, out[4576]);
      out[4672] = fma(0.98, dr, out[4672]);
      out[960] = fma(0.02, dr, out[960]);
      out[4224] = fma(-2.7, dr, out[4224]);
    }
    {
      const double dr = ws[37632] * v[960];
      out[960] = out[960] - dr;
      out[320] = fma(1.0, dr, out[320]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[37664] * fma(y[4608], v[960], y[960] * v[4608]);
      out[960] = out[960] - dr;
      out[4608] = out[4608] - dr;
      out[3648] = fma(1.0, dr, out[3648]);
    }
    {
      const double dr = ws[37696] * fma(y[4736], v[352], y[352] * v[4736]);
      out[352] = out[352] - dr;
      out[4736] = out[4736] - dr;
      out[4256] = fma(0.7, dr, out[4256]);
      out[4736] = fma(0.7, dr, out[4736]);
      out[3776] = fma(0.3, dr, out[3776]);
      out[4480] = fma(0.3, dr, out[4480]);
      out[4704] = fma(0.3, dr, out[4704]);
    }
    {
      const double dr = ws[37728] * fma(y[4160], v[2656], y[2656] * v[4160]);
      out[2656] = out[2656] - dr;
      out[4160] = out[4160] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
      out[4576] = fma(0.7, dr, out[4576]);
      out[4672] = fma(0.7, dr, out[4672]);
      out[4736] = fma(0.3, dr, out[4736]);
    }
    {
      const double dr = ws[37760] * fma(y[4736], v[2656], y[2656] * v[4736]);
      out[2656] = out[2656] - dr;
      out[4736] = out[4736] - dr;
      out[4576] = fma(1.0, dr, out[4576]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4512] = fma(1.56, dr, out[4512]);
      out[3840] = fma(0.22, dr, out[3840]);
    }
    {
      const double dr = ws[37792] * fma(y[4320], v[2656], y[2656] * v[4320]);
      out[2656] = out[2656] - dr;
      out[4320] = out[4320] - dr;
      out[4512] = fma(1.0, dr, out[4512]);
      out[4480] = fma(0.35, dr, out[4480]);
      out[4704] = fma(0.27, dr, out[4704]);
      out[4736] = fma(0.17, dr, out[4736]);
      out[3776] = fma(0.42, dr, out[3776]);
    }
    {
      const double dr = ws[37824] * fma(y[4640], v[2656], y[2656] * v[4640]);
      out[2656] = out[2656] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.5, dr, out[4608]);
      out[3648] = fma(0.5, dr, out[3648]);
      out[4576] = fma(0.5, dr, out[4576]);
      out[4352] = fma(0.5, dr, out[4352]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4512] = fma(1.125, dr, out[4512]);
    }
}
__device__ __noinline__ void ddm_jv_0_2(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[37856] * fma(y[4160], v[3552], y[3552] * v[4160]);
      out[3552] = out[3552] - dr;
      out[4160] = out[4160] - dr;
      out[4128] = fma(0.2, dr, out[4128]);
      out[4064] = fma(0.3, dr, out[4064]);
      out[4704] = fma(0.1, dr, out[4704]);
      out[4576] = fma(0.2, dr, out[4576]);
      out[4480] = fma(0.2, dr, out[4480]);
      out[4512] = fma(0.2, dr, out[4512]);
      out[4288] = fma(0.01, dr, out[4288]);
      out[4672] = fma(0.21, dr, out[4672]);
      out[4224] = fma(0.2, dr, out[4224]);
      out[4736] = fma(0.1, dr, out[4736]);
    }
    {
      const double dr = ws[37888] * fma(y[4736], v[3552], y[3552] * v[4736]);
      out[3552] = out[3552] - dr;
      out[4736] = out[4736] - dr;
      out[4512] = fma(0.781, dr, out[4512]);
      out[4128] = fma(0.488, dr, out[4128]);
      out[4064] = fma(0.488, dr, out[4064]);
      out[4576] = fma(0.976, dr, out[4576]);
      out[4352] = fma(0.195, dr, out[4352]);
      out[4288] = fma(0.024, dr, out[4288]);
      out[4672] = fma(1.195, dr, out[4672]);
      out[4224] = fma(-0.73, dr, out[4224]);
    }
    {
      const double dr = ws[37920] * fma(y[4320], v[3552], y[3552] * v[4320]);
      out[3552] = out[3552] - dr;
      out[4320] = out[4320] - dr;
      out[4128] = fma(0.295, dr, out[4128]);
      out[4512] = fma(0.555, dr, out[4512]);
      out[4064] = fma(0.27, dr, out[4064]);
      out[4576] = fma(0.15, dr, out[4576]);
      out[4672] = fma(0.15, dr, out[4672]);
      out[4736] = fma(0.334, dr, out[4736]);
      out[4704] = fma(0.08, dr, out[4704]);
      out[4480] = fma(0.378, dr, out[4480]);
      out[4256] = fma(0.075, dr, out[4256]);
      out[4000] = fma(0.075, dr, out[4000]);
      out[3776] = fma(0.09, dr, out[3776]);
      out[3904] = fma(0.13, dr, out[3904]);
      out[3456] = fma(0.04, dr, out[3456]);
      out[4224] = fma(-0.79, dr, out[4224]);
    }
    {
      const double dr = ws[37952] * fma(y[4640], v[3552], y[3552] * v[4640]);
      out[3552] = out[3552] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.5, dr, out[4608]);
      out[3648] = fma(0.5, dr, out[3648]);
      out[4352] = fma(0.48, dr, out[4352]);
      out[4576] = fma(0.48, dr, out[4576]);
      out[4288] = fma(0.04, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4512] = fma(0.5, dr, out[4512]);
      out[4128] = fma(0.25, dr, out[4128]);
      out[4064] = fma(0.375, dr, out[4064]);
      out[4224] = fma(-1.0, dr, out[4224]);
    }
    {
      const double dr = ws[37984] * fma(y[4160], v[3136], y[3136] * v[4160]);
      out[3136] = out[3136] - dr;
      out[4160] = out[4160] - dr;
      out[4128] = fma(1.24, dr, out[4128]);
      out[4064] = fma(0.66, dr, out[4064]);
      out[4576] = fma(0.1, dr, out[4576]);
      out[4672] = fma(0.1, dr, out[4672]);
      out[4480] = fma(0.1, dr, out[4480]);
      out[4224] = fma(0.1, dr, out[4224]);
    }
    {
      const double dr = ws[38016] * fma(y[4736], v[3136], y[3136] * v[4736]);
      out[3136] = out[3136] - dr;
      out[4736] = out[4736] - dr;
      out[4128] = fma(1.3, dr, out[4128]);
      out[4064] = fma(0.7, dr, out[4064]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[38048] * fma(y[4320], v[3136], y[3136] * v[4320]);
      out[3136] = out[3136] - dr;
      out[4320] = out[4320] - dr;
      out[4128] = fma(0.732, dr, out[4128]);
      out[4064] = fma(0.442, dr, out[4064]);
      out[4512] = fma(0.128, dr, out[4512]);
      out[4480] = fma(0.245, dr, out[4480]);
      out[4736] = fma(0.5, dr, out[4736]);
      out[4576] = fma(0.3, dr, out[4576]);
      out[4672] = fma(0.3, dr, out[4672]);
      out[4256] = fma(0.24, dr, out[4256]);
      out[4000] = fma(0.06, dr, out[4000]);
      out[4224] = fma(0.29, dr, out[4224]);
      out[3904] = fma(0.08, dr, out[3904]);
      out[3456] = fma(0.08, dr, out[3456]);
    }
    {
      const double dr = ws[38080] * fma(y[4640], v[3136], y[3136] * v[4640]);
      out[3136] = out[3136] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.5, dr, out[4608]);
      out[3648] = fma(0.5, dr, out[3648]);
      out[4352] = fma(0.48, dr, out[4352]);
      out[4576] = fma(0.48, dr, out[4576]);
      out[4288] = fma(0.04, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4128] = fma(0.5, dr, out[4128]);
      out[4064] = fma(0.625, dr, out[4064]);
      out[4224] = fma(1.0, dr, out[4224]);
    }
    {
      const double dr = ws[38112] * fma(y[4736], v[2528], y[2528] * v[4736]);
      out[2528] = out[2528] - dr;
      out[4736] = out[4736] - dr;
      out[3424] = fma(1.0, dr, out[3424]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[992] = fma(1.0, dr, out[992]);
    }
    {
      const double dr = ws[38144] * fma(y[4160], v[2528], y[2528] * v[4160]);
      out[2528] = out[2528] - dr;
      out[4160] = out[4160] - dr;
      out[3872] = fma(0.75, dr, out[3872]);
      out[4512] = fma(0.5, dr, out[4512]);
      out[4352] = fma(0.25, dr, out[4352]);
      out[4672] = fma(0.25, dr, out[4672]);
      out[4704] = fma(0.25, dr, out[4704]);
      out[4096] = fma(0.25, dr, out[4096]);
      out[4224] = fma(0.25, dr, out[4224]);
    }
    {
      const double dr = ws[38176] * fma(y[4384], v[3424], y[3424] * v[4384]);
      out[3424] = out[3424] - dr;
      out[4384] = out[4384] - dr;
      out[1632] = fma(0.1, dr, out[1632]);
      out[4608] = fma(0.9, dr, out[4608]);
      out[4512] = fma(0.673, dr, out[4512]);
      out[3872] = fma(0.9, dr, out[3872]);
      out[4704] = fma(0.818, dr, out[4704]);
      out[4576] = fma(0.082, dr, out[4576]);
      out[4672] = fma(0.082, dr, out[4672]);
    }
    {
      const double dr = ws[38208] * fma(y[4704], v[3424], y[3424] * v[4704]);
      out[3424] = out[3424] - dr;
      out[4704] = out[4704] - dr;
      out[1664] = fma(0.88, dr, out[1664]);
      out[4736] = fma(0.12, dr, out[4736]);
      out[4704] = fma(0.12, dr, out[4704]);
      out[4512] = fma(0.12, dr, out[4512]);
      out[3872] = fma(0.12, dr, out[3872]);
    }
    {
      const double dr = ws[38240] * fma(y[4448], v[3424], y[3424] * v[4448]);
      out[3424] = out[3424] - dr;
      out[4448] = out[4448] - dr;
      out[4512] = fma(0.598, dr, out[4512]);
      out[3872] = fma(1.0, dr, out[3872]);
      out[4704] = fma(0.728, dr, out[4704]);
      out[4576] = fma(0.072, dr, out[4576]);
      out[4416] = fma(0.8, dr, out[4416]);
      out[3904] = fma(0.2, dr, out[3904]);
      out[4672] = fma(0.872, dr, out[4672]);
    }
    {
      const double dr = ws[38272] * fma(y[4672], v[3424], y[3424] * v[4672]);
      out[3424] = out[3424] - dr;
      out[4672] = out[4672] - dr;
      out[4512] = fma(0.598, dr, out[4512]);
      out[3872] = fma(1.0, dr, out[3872]);
      out[4704] = fma(0.728, dr, out[4704]);
      out[4576] = fma(0.072, dr, out[4576]);
      out[4672] = fma(1.072, dr, out[4672]);
    }
    {
      const double dr = ws[38304] * v[3424];
      out[3424] = out[3424] - dr;
      out[4704] = fma(1.0, dr, out[4704]);
      out[1024] = fma(1.0, dr, out[1024]);
    }
    {
      const double dr = ws[38336] * fma(y[4320], v[2528], y[2528] * v[4320]);
      out[2528] = out[2528] - dr;
      out[4320] = out[4320] - dr;
      out[4512] = fma(0.6, dr, out[4512]);
      out[3872] = fma(0.65, dr, out[3872]);
      out[4064] = fma(0.15, dr, out[4064]);
      out[4096] = fma(0.2, dr, out[4096]);
      out[4224] = fma(0.35, dr, out[4224]);
      out[4736] = fma(0.266, dr, out[4736]);
      out[4352] = fma(0.2, dr, out[4352]);
      out[4672] = fma(0.2, dr, out[4672]);
      out[4704] = fma(0.066, dr, out[4704]);
      out[4480] = fma(0.066, dr, out[4480]);
    }
    {
      const double dr = ws[38368] * fma(y[4640], v[2528], y[2528] * v[4640]);
      out[2528] = out[2528] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.35, dr, out[4608]);
      out[4032] = fma(0.65, dr, out[4032]);
      out[4576] = fma(0.64, dr, out[4576]);
      out[4352] = fma(0.33, dr, out[4352]);
      out[4288] = fma(0.03, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4512] = fma(0.35, dr, out[4512]);
      out[3872] = fma(0.35, dr, out[3872]);
      out[992] = fma(1.0, dr, out[992]);
    }
    {
      const double dr = ws[38400] * fma(y[4736], v[3872], y[3872] * v[4736]);
      out[3872] = out[3872] - dr;
      out[4736] = out[4736] - dr;
      out[4288] = fma(0.022, dr, out[4288]);
      out[4352] = fma(0.521, dr, out[4352]);
      out[4000] = fma(0.115, dr, out[4000]);
      out[4416] = fma(0.115, dr, out[4416]);
      out[3840] = fma(0.269, dr, out[3840]);
      out[4448] = fma(0.269, dr, out[4448]);
      out[3744] = fma(0.457, dr, out[3744]);
      out[4224] = fma(0.117, dr, out[4224]);
      out[3392] = fma(0.137, dr, out[3392]);
      out[4480] = fma(0.137, dr, out[4480]);
      out[4704] = fma(0.137, dr, out[4704]);
      out[4672] = fma(0.658, dr, out[4672]);
    }
    {
      const double dr = ws[38432] * fma(y[4320], v[3872], y[3872] * v[4320]);
      out[3872] = out[3872] - dr;
      out[4320] = out[4320] - dr;
      out[4128] = fma(0.04, dr, out[4128]);
      out[4512] = fma(0.231, dr, out[4512]);
      out[4000] = fma(0.531, dr, out[4000]);
      out[4256] = fma(0.17, dr, out[4256]);
      out[3392] = fma(0.17, dr, out[3392]);
      out[4480] = fma(0.543, dr, out[4480]);
      out[4736] = fma(0.461, dr, out[4736]);
      out[3776] = fma(0.15, dr, out[3776]);
      out[4704] = fma(0.398, dr, out[4704]);
      out[4448] = fma(0.143, dr, out[4448]);
    }
    {
      const double dr = ws[38464] * fma(y[4640], v[3872], y[3872] * v[4640]);
      out[3872] = out[3872] - dr;
      out[4640] = out[4640] - dr;
      out[4192] = fma(0.717, dr, out[4192]);
      out[4032] = fma(0.142, dr, out[4032]);
      out[4608] = fma(0.142, dr, out[4608]);
      out[4352] = fma(0.142, dr, out[4352]);
      out[4576] = fma(0.142, dr, out[4576]);
      out[3840] = fma(0.113, dr, out[3840]);
      out[4000] = fma(0.113, dr, out[4000]);
      out[4224] = fma(0.717, dr, out[4224]);
      out[4096] = fma(0.717, dr, out[4096]);
      out[4672] = fma(0.284, dr, out[4672]);
    }
    {
      const double dr = ws[38496] * v[3872];
      out[3872] = out[3872] - dr;
      out[4704] = fma(0.76, dr, out[4704]);
      out[4576] = fma(0.34, dr, out[4576]);
      out[4352] = fma(0.16, dr, out[4352]);
      out[4416] = fma(0.34, dr, out[4416]);
      out[4448] = fma(0.208, dr, out[4448]);
      out[4512] = fma(0.26, dr, out[4512]);
      out[3552] = fma(0.24, dr, out[3552]);
      out[4224] = fma(0.24, dr, out[4224]);
      out[3392] = fma(0.17, dr, out[3392]);
      out[3840] = fma(0.128, dr, out[3840]);
      out[4672] = fma(0.84, dr, out[4672]);
    }
    {
      const double dr = ws[38528] * fma(y[4736], v[1664], y[1664] * v[4736]);
      out[1664] = out[1664] - dr;
      out[4736] = out[4736] - dr;
      out[1056] = fma(0.904, dr, out[1056]);
      out[4736] = fma(0.933, dr, out[4736]);
      out[3424] = fma(0.067, dr, out[3424]);
      out[4672] = fma(0.067, dr, out[4672]);
      out[3136] = fma(0.029, dr, out[3136]);
      out[4064] = fma(0.029, dr, out[4064]);
    }
    {
      const double dr = ws[38560] * v[1024];
      out[1024] = out[1024] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[3872] = fma(1.0, dr, out[3872]);
    }
    {
      const double dr = ws[38592] * fma(y[4640], v[1024], y[1024] * v[4640]);
      out[1024] = out[1024] - dr;
      out[4640] = out[4640] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
      out[3872] = fma(1.0, dr, out[3872]);
    }
    {
      const double dr = ws[38624] * fma(y[4736], v[1056], y[1056] * v[4736]);
      out[1056] = out[1056] - dr;
      out[4736] = out[4736] - dr;
      out[3296] = fma(1.0, dr, out[3296]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[38656] * fma(y[4704], v[3296], y[3296] * v[4704]);
      out[3296] = out[3296] - dr;
      out[4704] = out[4704] - dr;
      out[3840] = fma(0.275, dr, out[3840]);
      out[4256] = fma(0.275, dr, out[4256]);
      out[4000] = fma(0.275, dr, out[4000]);
      out[4736] = fma(1.125, dr, out[4736]);
      out[4704] = fma(0.825, dr, out[4704]);
      out[4512] = fma(0.375, dr, out[4512]);
      out[3776] = fma(0.074, dr, out[3776]);
      out[4480] = fma(0.251, dr, out[4480]);
      out[4224] = fma(2.175, dr, out[4224]);
    }
    {
      const double dr = ws[38688] * fma(y[4384], v[3296], y[3296] * v[4384]);
      out[3296] = out[3296] - dr;
      out[4384] = out[4384] - dr;
      out[3840] = fma(0.275, dr, out[3840]);
      out[4256] = fma(0.275, dr, out[4256]);
      out[4000] = fma(0.275, dr, out[4000]);
      out[4736] = fma(0.125, dr, out[4736]);
      out[4704] = fma(0.825, dr, out[4704]);
      out[4512] = fma(0.375, dr, out[4512]);
      out[4608] = fma(1.0, dr, out[4608]);
      out[4480] = fma(0.251, dr, out[4480]);
      out[4224] = fma(2.175, dr, out[4224]);
    }
    {
      const double dr = ws[38720] * fma(y[4448], v[3296], y[3296] * v[4448]);
      out[3296] = out[3296] - dr;
      out[4448] = out[4448] - dr;
      out[3840] = fma(0.22, dr, out[3840]);
      out[4256] = fma(0.22, dr, out[4256]);
      out[4000] = fma(0.22, dr, out[4000]);
      out[4736] = fma(0.1, dr, out[4736]);
      out[4704] = fma(0.66, dr, out[4704]);
      out[4512] = fma(0.3, dr, out[4512]);
      out[4480] = fma(0.2, dr, out[4480]);
      out[4224] = fma(1.74, dr, out[4224]);
      out[4416] = fma(0.8, dr, out[4416]);
      out[3904] = fma(0.2, dr, out[3904]);
      out[4672] = fma(0.8, dr, out[4672]);
    }
    {
      const double dr = ws[38752] * fma(y[4672], v[3296], y[3296] * v[4672]);
      out[3296] = out[3296] - dr;
      out[4672] = out[4672] - dr;
      out[3840] = fma(0.275, dr, out[3840]);
      out[4256] = fma(0.275, dr, out[4256]);
      out[4000] = fma(0.275, dr, out[4000]);
      out[4736] = fma(0.125, dr, out[4736]);
      out[4704] = fma(0.825, dr, out[4704]);
      out[4512] = fma(0.375, dr, out[4512]);
      out[4480] = fma(0.251, dr, out[4480]);
      out[4224] = fma(2.175, dr, out[4224]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[38784] * fma(y[4736], v[1632], y[1632] * v[4736]);
      out[1632] = out[1632] - dr;
      out[4736] = out[4736] - dr;
      out[4352] = fma(0.63, dr, out[4352]);
      out[4576] = fma(0.37, dr, out[4576]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4608] = fma(0.444, dr, out[4608]);
      out[4640] = fma(0.185, dr, out[4640]);
      out[1632] = fma(0.104, dr, out[1632]);
      out[4512] = fma(0.592, dr, out[4512]);
      out[3840] = fma(0.331, dr, out[3840]);
      out[3776] = fma(0.185, dr, out[3776]);
      out[4224] = fma(2.7, dr, out[4224]);
      out[3552] = fma(0.098, dr, out[3552]);
      out[4064] = fma(0.078, dr, out[4064]);
      out[4032] = fma(0.266, dr, out[4032]);
    }
    {
      const double dr = ws[38816] * fma(y[4160], v[2048], y[2048] * v[4160]);
      out[2048] = out[2048] - dr;
      out[4160] = out[4160] - dr;
      out[4064] = fma(0.15, dr, out[4064]);
      out[4224] = fma(5.12, dr, out[4224]);
      out[2080] = fma(1.0, dr, out[2080]);
    }
    {
      const double dr = ws[38848] * fma(y[4736], v[2048], y[2048] * v[4736]);
      out[2048] = out[2048] - dr;
      out[4736] = out[4736] - dr;
      out[4576] = fma(0.75, dr, out[4576]);
      out[4352] = fma(0.5, dr, out[4352]);
      out[4288] = fma(0.25, dr, out[4288]);
      out[4672] = fma(1.5, dr, out[4672]);
      out[4512] = fma(0.28, dr, out[4512]);
      out[4224] = fma(1.66, dr, out[4224]);
      out[4064] = fma(0.47, dr, out[4064]);
      out[2080] = fma(1.0, dr, out[2080]);
    }
    {
      const double dr = ws[38880] * fma(y[4320], v[2048], y[2048] * v[4320]);
      out[2048] = out[2048] - dr;
      out[4320] = out[4320] - dr;
      out[4736] = fma(0.57, dr, out[4736]);
      out[4576] = fma(0.07, dr, out[4576]);
      out[4352] = fma(0.69, dr, out[4352]);
      out[4288] = fma(0.18, dr, out[4288]);
      out[4672] = fma(0.94, dr, out[4672]);
      out[4512] = fma(0.24, dr, out[4512]);
      out[4480] = fma(0.001, dr, out[4480]);
      out[4224] = fma(7.0, dr, out[4224]);
      out[4064] = fma(0.21, dr, out[4064]);
      out[4096] = fma(0.39, dr, out[4096]);
      out[2080] = fma(1.0, dr, out[2080]);
    }
    {
      const double dr = ws[38912] * fma(y[4640], v[2048], y[2048] * v[4640]);
      out[2048] = out[2048] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.47, dr, out[4608]);
      out[4576] = fma(0.28, dr, out[4576]);
      out[4352] = fma(0.75, dr, out[4352]);
      out[4288] = fma(0.25, dr, out[4288]);
      out[4672] = fma(1.28, dr, out[4672]);
      out[4064] = fma(0.47, dr, out[4064]);
      out[4032] = fma(0.53, dr, out[4032]);
      out[2848] = fma(1.0, dr, out[2848]);
    }
    {
      const double dr = ws[38944] * fma(y[4160], v[2112], y[2112] * v[4160]);
      out[2112] = out[2112] - dr;
      out[4160] = out[4160] - dr;
      out[4064] = fma(0.15, dr, out[4064]);
      out[4224] = fma(5.12, dr, out[4224]);
      out[2080] = fma(1.0, dr, out[2080]);
    }
    {
      const double dr = ws[38976] * fma(y[4736], v[2112], y[2112] * v[4736]);
      out[2112] = out[2112] - dr;
      out[4736] = out[4736] - dr;
      out[4576] = fma(0.75, dr, out[4576]);
      out[4352] = fma(0.5, dr, out[4352]);
      out[4288] = fma(0.25, dr, out[4288]);
      out[4672] = fma(1.5, dr, out[4672]);
      out[4512] = fma(0.28, dr, out[4512]);
      out[4224] = fma(1.66, dr, out[4224]);
      out[4064] = fma(0.47, dr, out[4064]);
      out[2080] = fma(1.0, dr, out[2080]);
    }
    {
      const double dr = ws[39008] * fma(y[4320], v[2112], y[2112] * v[4320]);
      out[2112] = out[2112] - dr;
      out[4320] = out[4320] - dr;
      out[4736] = fma(0.57, dr, out[4736]);
      out[4576] = fma(0.07, dr, out[4576]);
      out[4352] = fma(0.69, dr, out[4352]);
      out[4288] = fma(0.18, dr, out[4288]);
      out[4672] = fma(0.94, dr, out[4672]);
      out[4512] = fma(0.24, dr, out[4512]);
      out[4480] = fma(0.001, dr, out[4480]);
      out[4224] = fma(7.0, dr, out[4224]);
      out[4064] = fma(0.21, dr, out[4064]);
      out[4096] = fma(0.39, dr, out[4096]);
      out[2080] = fma(1.0, dr, out[2080]);
    }
    {
      const double dr = ws[39040] * fma(y[4640], v[2112], y[2112] * v[4640]);
      out[2112] = out[2112] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.47, dr, out[4608]);
      out[4576] = fma(0.28, dr, out[4576]);
      out[4352] = fma(0.75, dr, out[4352]);
      out[4288] = fma(0.25, dr, out[4288]);
      out[4672] = fma(1.28, dr, out[4672]);
      out[4064] = fma(0.47, dr, out[4064]);
      out[4032] = fma(0.53, dr, out[4032]);
    }
    {
      const double dr = ws[39072] * fma(y[4736], v[384], y[384] * v[4736]);
      out[384] = out[384] - dr;
      out[4736] = out[4736] - dr;
      out[3616] = fma(0.53, dr, out[3616]);
      out[3104] = fma(0.352, dr, out[3104]);
      out[4672] = fma(0.352, dr, out[4672]);
      out[3936] = fma(0.118, dr, out[3936]);
      out[4736] = fma(0.118, dr, out[4736]);
      out[4704] = fma(0.53, dr, out[4704]);
      out[2144] = fma(1.0, dr, out[2144]);
    }
}
__device__ __noinline__ void ddm_jv_0_3(double* __restrict__ ws, int yoff, int voff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ v = ws + voff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      const double dr = ws[39104] * fma(y[4384], v[3104], y[3104] * v[4384]);
      out[3104] = out[3104] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(0.918, dr, out[4608]);
      out[4032] = fma(0.082, dr, out[4032]);
      out[4256] = fma(0.918, dr, out[4256]);
      out[3936] = fma(0.918, dr, out[3936]);
      out[4704] = fma(0.918, dr, out[4704]);
    }
    {
      const double dr = ws[39136] * fma(y[4448], v[3104], y[3104] * v[4448]);
      out[3104] = out[3104] - dr;
      out[4448] = out[4448] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
      out[3936] = fma(1.0, dr, out[3936]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[39168] * fma(y[4704], v[3104], y[3104] * v[4704]);
      out[3104] = out[3104] - dr;
      out[4704] = out[4704] - dr;
    }
    {
      const double dr = ws[39200] * fma(y[4672], v[3104], y[3104] * v[4672]);
      out[3104] = out[3104] - dr;
      out[4672] = out[4672] - dr;
      out[4256] = fma(1.0, dr, out[4256]);
      out[3936] = fma(1.0, dr, out[3936]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[39232] * fma(y[4736], v[1088], y[1088] * v[4736]);
      out[1088] = out[1088] - dr;
      out[4736] = out[4736] - dr;
      out[3616] = fma(0.18, dr, out[3616]);
      out[3488] = fma(0.65, dr, out[3488]);
      out[4672] = fma(0.72, dr, out[4672]);
      out[3936] = fma(0.1, dr, out[3936]);
      out[4736] = fma(0.1, dr, out[4736]);
      out[4576] = fma(0.07, dr, out[4576]);
      out[4704] = fma(0.18, dr, out[4704]);
      out[2944] = fma(1.0, dr, out[2944]);
    }
    {
      const double dr = ws[39264] * fma(y[4384], v[3488], y[3488] * v[4384]);
      out[3488] = out[3488] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(0.86, dr, out[4608]);
      out[4032] = fma(0.14, dr, out[4032]);
      out[4256] = fma(0.417, dr, out[4256]);
      out[4000] = fma(0.443, dr, out[4000]);
      out[3936] = fma(0.66, dr, out[3936]);
      out[3808] = fma(0.2, dr, out[3808]);
      out[4704] = fma(0.86, dr, out[4704]);
    }
    {
      const double dr = ws[39296] * fma(y[4448], v[3488], y[3488] * v[4448]);
      out[3488] = out[3488] - dr;
      out[4448] = out[4448] - dr;
      out[4256] = fma(0.48, dr, out[4256]);
      out[4000] = fma(0.52, dr, out[4000]);
      out[3936] = fma(0.77, dr, out[3936]);
      out[3808] = fma(0.23, dr, out[3808]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[39328] * fma(y[4704], v[3488], y[3488] * v[4704]);
      out[3488] = out[3488] - dr;
      out[4704] = out[4704] - dr;
    }
    {
      const double dr = ws[39360] * fma(y[4672], v[3488], y[3488] * v[4672]);
      out[3488] = out[3488] - dr;
      out[4672] = out[4672] - dr;
      out[4256] = fma(0.48, dr, out[4256]);
      out[4000] = fma(0.52, dr, out[4000]);
      out[3936] = fma(0.77, dr, out[3936]);
      out[3808] = fma(0.23, dr, out[3808]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[39392] * fma(y[4736], v[1120], y[1120] * v[4736]);
      out[1120] = out[1120] - dr;
      out[4736] = out[4736] - dr;
      out[3616] = fma(0.155, dr, out[3616]);
      out[3584] = fma(0.544, dr, out[3584]);
      out[4672] = fma(0.602, dr, out[4672]);
      out[3808] = fma(0.244, dr, out[3808]);
      out[4736] = fma(0.244, dr, out[4736]);
      out[4576] = fma(0.058, dr, out[4576]);
      out[4704] = fma(0.155, dr, out[4704]);
      out[2496] = fma(1.0, dr, out[2496]);
    }
    {
      const double dr = ws[39424] * fma(y[4736], v[1152], y[1152] * v[4736]);
      out[1152] = out[1152] - dr;
      out[4736] = out[4736] - dr;
      out[3616] = fma(0.155, dr, out[3616]);
      out[3584] = fma(0.544, dr, out[3584]);
      out[4672] = fma(0.602, dr, out[4672]);
      out[3808] = fma(0.244, dr, out[3808]);
      out[4736] = fma(0.244, dr, out[4736]);
      out[4576] = fma(0.058, dr, out[4576]);
      out[4704] = fma(0.155, dr, out[4704]);
      out[2560] = fma(1.0, dr, out[2560]);
    }
    {
      const double dr = ws[39456] * fma(y[4384], v[3584], y[3584] * v[4384]);
      out[3584] = out[3584] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(0.86, dr, out[4608]);
      out[4032] = fma(0.14, dr, out[4032]);
      out[4256] = fma(0.221, dr, out[4256]);
      out[4000] = fma(0.675, dr, out[4000]);
      out[3936] = fma(0.3, dr, out[3936]);
      out[3808] = fma(0.56, dr, out[3808]);
      out[4704] = fma(0.86, dr, out[4704]);
    }
    {
      const double dr = ws[39488] * fma(y[4704], v[3584], y[3584] * v[4704]);
      out[3584] = out[3584] - dr;
      out[4704] = out[4704] - dr;
    }
    {
      const double dr = ws[39520] * fma(y[4448], v[3584], y[3584] * v[4448]);
      out[3584] = out[3584] - dr;
      out[4448] = out[4448] - dr;
      out[4256] = fma(0.26, dr, out[4256]);
      out[4000] = fma(0.77, dr, out[4000]);
      out[3936] = fma(0.35, dr, out[3936]);
      out[3808] = fma(0.65, dr, out[3808]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[39552] * fma(y[4672], v[3584], y[3584] * v[4672]);
      out[3584] = out[3584] - dr;
      out[4672] = out[4672] - dr;
      out[4256] = fma(0.26, dr, out[4256]);
      out[4000] = fma(0.77, dr, out[4000]);
      out[3936] = fma(0.35, dr, out[3936]);
      out[3808] = fma(0.65, dr, out[3808]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[39584] * fma(y[4736], v[3616], y[3616] * v[4736]);
      out[3616] = out[3616] - dr;
      out[4736] = out[4736] - dr;
      out[4256] = fma(0.025, dr, out[4256]);
      out[3936] = fma(0.025, dr, out[3936]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[3328] = fma(0.2, dr, out[3328]);
      out[1760] = fma(0.732, dr, out[1760]);
      out[4288] = fma(0.02, dr, out[4288]);
      out[4672] = fma(0.02, dr, out[4672]);
    }
    {
      const double dr = ws[39616] * fma(y[4640], v[3616], y[3616] * v[4640]);
      out[3616] = out[3616] - dr;
      out[4640] = out[4640] - dr;
      out[3328] = fma(0.3, dr, out[3328]);
      out[4192] = fma(1.0, dr, out[4192]);
      out[4352] = fma(0.48, dr, out[4352]);
      out[4576] = fma(0.12, dr, out[4576]);
      out[4256] = fma(0.24, dr, out[4256]);
      out[4000] = fma(0.24, dr, out[4000]);
      out[3744] = fma(0.48, dr, out[3744]);
      out[4288] = fma(0.1, dr, out[4288]);
      out[4672] = fma(0.7, dr, out[4672]);
    }
    {
      const double dr = ws[39648] * fma(y[4608], v[3328], y[3328] * v[4608]);
      out[3328] = out[3328] - dr;
      out[4608] = out[4608] - dr;
      out[2176] = fma(1.0, dr, out[2176]);
    }
    {
      const double dr = ws[39680] * fma(y[4704], v[3328], y[3328] * v[4704]);
      out[3328] = out[3328] - dr;
      out[4704] = out[4704] - dr;
      out[3616] = fma(1.0, dr, out[3616]);
    }
    {
      const double dr = ws[39712] * fma(y[4736], v[2176], y[2176] * v[4736]);
      out[2176] = out[2176] - dr;
      out[4736] = out[4736] - dr;
      out[4032] = fma(1.0, dr, out[4032]);
      out[3328] = fma(0.5, dr, out[3328]);
    }
    {
      const double dr = ws[39744] * fma(y[4640], v[2176], y[2176] * v[4640]);
      out[2176] = out[2176] - dr;
      out[4640] = out[4640] - dr;
      out[4032] = fma(1.0, dr, out[4032]);
      out[3328] = fma(0.5, dr, out[3328]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[39776] * v[2176];
      out[2176] = out[2176] - dr;
      out[2464] = fma(1.0, dr, out[2464]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4512] = fma(1.0, dr, out[4512]);
      out[3936] = fma(1.0, dr, out[3936]);
    }
    {
      const double dr = ws[39808] * v[3808];
      out[3808] = out[3808] - dr;
      out[4256] = fma(0.4, dr, out[4256]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[4704] = fma(0.7, dr, out[4704]);
      out[4480] = fma(0.7, dr, out[4480]);
      out[4448] = fma(0.3, dr, out[4448]);
    }
    {
      const double dr = ws[39840] * fma(y[4736], v[3808], y[3808] * v[4736]);
      out[3808] = out[3808] - dr;
      out[4736] = out[4736] - dr;
      out[4000] = fma(1.0, dr, out[4000]);
      out[4256] = fma(0.4, dr, out[4256]);
      out[4576] = fma(2.0, dr, out[4576]);
      out[4672] = fma(2.0, dr, out[4672]);
    }
    {
      const double dr = ws[39872] * fma(y[4320], v[3808], y[3808] * v[4320]);
      out[3808] = out[3808] - dr;
      out[4320] = out[4320] - dr;
      out[4000] = fma(1.2, dr, out[4000]);
      out[4736] = fma(0.5, dr, out[4736]);
      out[4448] = fma(0.6, dr, out[4448]);
      out[4128] = fma(0.1, dr, out[4128]);
      out[4480] = fma(0.5, dr, out[4480]);
      out[4576] = fma(0.3, dr, out[4576]);
      out[4672] = fma(0.3, dr, out[4672]);
    }
    {
      const double dr = ws[39904] * fma(y[4640], v[3808], y[3808] * v[4640]);
      out[3808] = out[3808] - dr;
      out[4640] = out[4640] - dr;
      out[4608] = fma(0.5, dr, out[4608]);
      out[4032] = fma(0.5, dr, out[4032]);
      out[4576] = fma(0.45, dr, out[4576]);
      out[4352] = fma(0.45, dr, out[4352]);
      out[4288] = fma(0.1, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[3936] = fma(0.25, dr, out[3936]);
      out[4000] = fma(0.25, dr, out[4000]);
    }
    {
      const double dr = ws[39936] * v[3936];
      out[3936] = out[3936] - dr;
      out[3744] = fma(1.0, dr, out[3744]);
      out[4704] = fma(1.0, dr, out[4704]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[39968] * fma(y[4736], v[3936], y[3936] * v[4736]);
      out[3936] = out[3936] - dr;
      out[4736] = out[4736] - dr;
      out[3744] = fma(0.6, dr, out[3744]);
      out[4576] = fma(0.4, dr, out[4576]);
      out[4672] = fma(0.4, dr, out[4672]);
      out[4256] = fma(0.4, dr, out[4256]);
    }
    {
      const double dr = ws[40000] * fma(y[4320], v[3936], y[3936] * v[4320]);
      out[3936] = out[3936] - dr;
      out[4320] = out[4320] - dr;
      out[4256] = fma(1.4, dr, out[4256]);
      out[4000] = fma(0.24, dr, out[4000]);
      out[4736] = fma(0.5, dr, out[4736]);
      out[4448] = fma(0.12, dr, out[4448]);
      out[4512] = fma(0.08, dr, out[4512]);
      out[4128] = fma(0.02, dr, out[4128]);
      out[4480] = fma(1.98, dr, out[4480]);
      out[4704] = fma(0.56, dr, out[4704]);
    }
    {
      const double dr = ws[40032] * fma(y[4640], v[3936], y[3936] * v[4640]);
      out[3936] = out[3936] - dr;
      out[4640] = out[4640] - dr;
      out[3744] = fma(1.0, dr, out[3744]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[40064] * fma(y[4736], v[1760], y[1760] * v[4736]);
      out[1760] = out[1760] - dr;
      out[4736] = out[4736] - dr;
      out[4512] = fma(0.14, dr, out[4512]);
      out[4704] = fma(0.2, dr, out[4704]);
      out[3328] = fma(0.5, dr, out[3328]);
    }
    {
      const double dr = ws[40096] * fma(y[4640], v[1760], y[1760] * v[4640]);
      out[1760] = out[1760] - dr;
      out[4640] = out[4640] - dr;
      out[3328] = fma(1.0, dr, out[3328]);
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[40128] * fma(y[4384], v[3744], y[3744] * v[4384]);
      out[3744] = out[3744] - dr;
      out[4384] = out[4384] - dr;
      out[4608] = fma(1.0, dr, out[4608]);
      out[4256] = fma(0.5, dr, out[4256]);
      out[4480] = fma(0.5, dr, out[4480]);
      out[4704] = fma(0.8, dr, out[4704]);
      out[4096] = fma(0.2, dr, out[4096]);
    }
    {
      const double dr = ws[40160] * fma(y[4608], v[3744], y[3744] * v[4608]);
      out[3744] = out[3744] - dr;
      out[4608] = out[4608] - dr;
      out[1792] = fma(1.0, dr, out[1792]);
    }
    {
      const double dr = ws[40192] * v[1792];
      out[1792] = out[1792] - dr;
      out[3744] = fma(1.0, dr, out[3744]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[40224] * fma(y[4704], v[3744], y[3744] * v[4704]);
      out[3744] = out[3744] - dr;
      out[4704] = out[4704] - dr;
      out[2688] = fma(0.37, dr, out[2688]);
      out[3904] = fma(0.13, dr, out[3904]);
      out[4320] = fma(0.13, dr, out[4320]);
      out[4736] = fma(0.5, dr, out[4736]);
      out[4416] = fma(0.5, dr, out[4416]);
      out[4672] = fma(0.5, dr, out[4672]);
    }
    {
      const double dr = ws[40256] * fma(y[4448], v[3744], y[3744] * v[4448]);
      out[3744] = out[3744] - dr;
      out[4448] = out[4448] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4352] = fma(1.0, dr, out[4352]);
      out[4064] = fma(1.0, dr, out[4064]);
      out[4672] = fma(2.0, dr, out[4672]);
    }
    {
      const double dr = ws[40288] * fma(y[4672], v[3744], y[3744] * v[4672]);
      out[3744] = out[3744] - dr;
      out[4672] = out[4672] - dr;
      out[4576] = fma(0.8, dr, out[4576]);
      out[4064] = fma(0.8, dr, out[4064]);
      out[4672] = fma(1.8, dr, out[4672]);
      out[3904] = fma(0.2, dr, out[3904]);
    }
    {
      const double dr = ws[40320] * fma(y[4736], v[1792], y[1792] * v[4736]);
      out[1792] = out[1792] - dr;
      out[4736] = out[4736] - dr;
      out[4608] = fma(0.5, dr, out[4608]);
      out[4256] = fma(0.5, dr, out[4256]);
      out[4480] = fma(1.0, dr, out[4480]);
      out[4032] = fma(0.5, dr, out[4032]);
    }
    {
      const double dr = ws[40352] * fma(y[4736], v[1952], y[1952] * v[4736]);
      out[1952] = out[1952] - dr;
      out[4736] = out[4736] - dr;
      out[4128] = fma(1.0, dr, out[4128]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[40384] * fma(y[4736], v[416], y[416] * v[4736]);
      out[416] = out[416] - dr;
      out[4736] = out[4736] - dr;
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40416] * v[928];
      out[928] = out[928] - dr;
      out[4288] = fma(1.0, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40448] * v[928];
      out[928] = out[928] - dr;
      out[3392] = fma(0.732, dr, out[3392]);
      out[4064] = fma(0.268, dr, out[4064]);
      out[4224] = fma(0.268, dr, out[4224]);
      out[4576] = fma(1.0, dr, out[4576]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40480] * v[1984];
      out[1984] = out[1984] - dr;
      out[4288] = fma(1.0, dr, out[4288]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40512] * v[1984];
      out[1984] = out[1984] - dr;
      out[4064] = fma(0.126, dr, out[4064]);
      out[960] = fma(0.874, dr, out[960]);
      out[4576] = fma(0.126, dr, out[4576]);
      out[4352] = fma(0.874, dr, out[4352]);
      out[4672] = fma(1.0, dr, out[4672]);
      out[4224] = fma(-0.126, dr, out[4224]);
    }
    {
      const double dr = ws[40544] * fma(y[4736], v[4608], y[4608] * v[4736]);
      out[4608] = out[4608] - dr;
      out[4736] = out[4736] - dr;
      out[4192] = fma(1.0, dr, out[4192]);
    }
    {
      const double dr = ws[40576] * v[1184];
      out[1184] = out[1184] - dr;
      out[4544] = fma(2.0, dr, out[4544]);
    }
    {
      const double dr = ws[40608] * v[1824];
      out[1824] = out[1824] - dr;
      out[4736] = fma(1.0, dr, out[4736]);
      out[4544] = fma(1.0, dr, out[4544]);
    }
    {
      const double dr = ws[40640] * fma(y[4320], v[4544], y[4544] * v[4320]);
      out[4544] = out[4544] - dr;
      out[4320] = out[4320] - dr;
      out[3520] = fma(1.0, dr, out[3520]);
    }
    {
      const double dr = ws[40672] * fma(y[3520], v[3520], y[3520] * v[3520]);
      out[3520] = out[3520] - dr;
      out[3520] = out[3520] - dr;
      out[1184] = fma(0.3, dr, out[1184]);
      out[4544] = fma(1.4, dr, out[4544]);
    }
    {
      const double dr = ws[40704] * fma(y[4384], v[3520], y[3520] * v[4384]);
      out[3520] = out[3520] - dr;
      out[4384] = out[4384] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[4608] = fma(1.0, dr, out[4608]);
    }
    {
      const double dr = ws[40736] * fma(y[4704], v[3520], y[3520] * v[4704]);
      out[3520] = out[3520] - dr;
      out[4704] = out[4704] - dr;
      out[1824] = fma(1.0, dr, out[1824]);
    }
    {
      const double dr = ws[40768] * fma(y[4416], v[3520], y[3520] * v[4416]);
      out[3520] = out[3520] - dr;
      out[4416] = out[4416] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[4512] = fma(1.0, dr, out[4512]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[40800] * fma(y[3232], v[4736], y[4736] * v[3232]);
      out[4736] = out[4736] - dr;
      out[3232] = out[3232] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[4480] = fma(1.0, dr, out[4480]);
    }
    {
      const double dr = ws[40832] * v[3232];
      out[3232] = out[3232] - dr;
      out[4544] = fma(1.0, dr, out[4544]);
      out[4480] = fma(1.0, dr, out[4480]);
      out[4704] = fma(1.0, dr, out[4704]);
    }
    {
      const double dr = ws[40864] * v[4544];
      out[4544] = out[4544] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[4416] = fma(1.0, dr, out[4416]);
      out[4672] = fma(1.0, dr, out[4672]);
    }
    {
      const double dr = ws[40896] * fma(y[4224], v[4544], y[4544] * v[4224]);
      out[4544] = out[4544] - dr;
      out[4224] = out[4224] - dr;
      out[3968] = fma(1.0, dr, out[3968]);
      out[1984] = fma(1.0, dr, out[1984]);
    }
}
}  // namespace mech_cb6r5_ae7_aq
