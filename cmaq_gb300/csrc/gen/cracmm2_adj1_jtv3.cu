// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/cracmm2/RXNS_DATA_MODULE.F90
// and RXNS_FUNC_MODULE.F90 (sha256/16 61a0c9d4d7262bbb).  Do not edit.
#include "cracmm2_mech.cuh"
#include <math.h>
namespace mech_cracmm2 {
__device__ __noinline__ void adj_jtv_1_12(double* __restrict__ ws, int yoff, int phioff, int outoff)
{
    const double* __restrict__ y = ws + yoff * 32;
    const double* __restrict__ phi = ws + phioff * 32;
    double* __restrict__ out = ws + outoff * 32;
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = w - phi[3488];
      w = w - phi[5824];
      const double kw = ws[59200] * w;
      out[3488] = fma(kw, y[5824], out[3488]);
      out[5824] = fma(kw, y[3488], out[5824]);
      ws[287904] = fma(kw * y[3488], y[5824], ws[287904]);
    }
    {
      double w = 1.0 * phi[5920];
      w = fma(1.0, phi[5984], w);
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = w - phi[3488];
      w = w - phi[5952];
      const double kw = ws[59232] * w;
      out[3488] = fma(kw, y[5952], out[3488]);
      out[5952] = fma(kw, y[3488], out[5952]);
      ws[287936] = fma(kw * y[3488], y[5952], ws[287936]);
    }
    {
      double w = 1.37 * phi[5984];
      w = fma(1.68, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = fma(0.32, phi[5600], w);
      w = w - phi[3488];
      w = w - phi[5888];
      const double kw = ws[59264] * w;
      out[3488] = fma(kw, y[5888], out[3488]);
      out[5888] = fma(kw, y[3488], out[5888]);
      ws[287968] = fma(kw * y[3488], y[5888], ws[287968]);
    }
    {
      double w = 1.0 * phi[5984];
      w = fma(1.0, phi[5856], w);
      w = fma(1.0, phi[4448], w);
      w = fma(0.7, phi[5888], w);
      w = fma(0.3, phi[5696], w);
      w = w - phi[3488];
      w = w - phi[5792];
      const double kw = ws[59296] * w;
      out[3488] = fma(kw, y[5792], out[3488]);
      out[5792] = fma(kw, y[3488], out[5792]);
      ws[288000] = fma(kw * y[3488], y[5792], ws[288000]);
    }
}
}  // namespace mech_cracmm2
