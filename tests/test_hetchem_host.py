"""The HETCHEM_RATES device code (cmaq_gb300/csrc/hetchem.cuh), built for the host, against
the oracle (oracle/hetchem_oracle.c): two restatements of AEROSOL_CHEMISTRY.F's
HETCHEM_RATES and the aerosol routines it calls, written apart, with the same C math
library on the host, so every KHETERO entry must agree bit for bit; AddressSanitizer
checks every table and array index.  Both mechanisms with HETCHEM_RATES tables
(cb6r5_ae7_aq, cracmm2).  tests/test_gpu_hetchem.py holds the GPU to the oracle within
the ulps of CUDA's math functions.
"""
import numpy as np
import pytest

from conftest import run_hetchem_harness

h = pytest.importorskip("hetchem")   # oracle/hetchem.py


def _same(a, b):
    return (a == b) | (np.isnan(a) & np.isnan(b))


def test_seeded_cells_bit_for_bit(hetchem_harness, tmp_path):
    from cmaq_gb300.synthetic import make_aerosol_cells
    ae, ta, p, q, d = make_aerosol_cells(4000, seed=11)
    got = run_hetchem_harness(hetchem_harness(), ae, ta, p, q, d, tmp_path)
    want = h.rates(ae, ta, p, q, d)
    assert got.shape == want.shape == (4000, 17)
    assert _same(got, want).all()
    assert np.isfinite(want).all()


def test_edge_cells_bit_for_bit(hetchem_harness, tmp_path):
    """Clean air (every row below the minimum concentrations), cold saturated air (ice:
    N2O5_GAMMA's FREEZES branch), dry air with an ammonium-sulfate aerosol (CRYSTALIZED),
    chloride-rich wet aerosol (the ClNO2 yields), no organic aerosol (NTR2 partitioning
    off; POC and PNCOM both at extract_aero's minimum, 1e-23 ug/m3, so PNCOM_LOSS sees the
    ratio 2 and the rate stays on, as in the reference)."""
    from cmaq_gb300.synthetic import make_aerosol_cells
    t = h.tables()
    n = 6
    ae, ta, p, q, d = make_aerosol_cells(n, seed=3)
    ae[:, 0] = 0.0                                           # clean
    ta[1], q[1] = 245.0, 1.0e-3                              # cold, supersaturated over ice
    rows = {name: i for i, name in enumerate(t["ae_rows"])}
    ta[2], q[2] = 295.0, 1.0e-4                              # dry
    ae[rows["ASO4J"], 2], ae[rows["ANH4J"], 2], ae[rows["ANO3J"], 2] = 10.0, 3.7, 0.01
    ae[rows["ACLJ"], 3], ae[rows["AH2OJ"], 3] = 5.0, 40.0    # chloride-rich, wet
    for s in t["species"]:                                   # no organic aerosol
        if s["om"]:
            for r in s["row"]:
                if r >= 0:
                    ae[r, 4] = 0.0
    ae[rows["AH3OP" + "J"], 5] = 0.0                         # no H+: IEPOX uptake from HSO4- alone
    got = run_hetchem_harness(hetchem_harness(), ae, ta, p, q, d, tmp_path)
    want = h.rates(ae, ta, p, q, d)
    assert _same(got, want).all()
    col = {name: j for j, name in enumerate(t["hetero"])}
    assert want[4, col["HETERO_NTR2"]] == 0.0
    assert want[4, col["HETERO_PNCOMLJ"]] > 0.0
    assert want[3, col["HETERO_H2NO3PBIJ"]] > 0.0


def test_cracmm2_seeded_and_edge_cells_bit_for_bit(hetchem_harness, tmp_path):
    """CRACMM2's 9 KHETERO labels: CRACMM's IEPOX pair table (ISO3NOSJ / ISO3OSJ products),
    NO3 and HO2 uptake, on seeded cells plus a clean cell and one without H+."""
    from cmaq_gb300.synthetic import make_aerosol_cells
    t = h.tables("cracmm2")
    ae, ta, p, q, d = make_aerosol_cells(3000, seed=12, mech="cracmm2")
    rows = {name: i for i, name in enumerate(t["ae_rows"])}
    ae[:, 0] = 0.0
    ae[rows["AH3OPJ"], 1] = 0.0
    got = run_hetchem_harness(hetchem_harness("cracmm2"), ae, ta, p, q, d, tmp_path)
    want = h.rates(ae, ta, p, q, d, mech="cracmm2")
    assert got.shape == want.shape == (3000, 9)
    assert _same(got, want).all()
    assert np.isfinite(want).all()
    col = {name: j for j, name in enumerate(t["hetero"])}
    for lab in ("HETERO_NO3", "HETERO_HO2", "HETERO_IEPOX", "HETERO_ISO3NOSJ", "HETERO_ISO3OSJ"):
        assert (want[:, col[lab]] > 0).mean() > 0.5, lab
