"""The EBI device code (cmaq_gb300/csrc/ebi.cuh's per-cell HRSOLVER with the generated
HRRATES, HRG1-4 and HRPRODLOSS of cmaq_gb300/csrc/gen/<mech>_ebi.cu), built for the host,
against the oracle's HRSOLVER (oracle/ebi_oracle.c): the same operations in the same
order, so every concentration and iteration count must agree bit for bit, for both
mechanisms and for sync steps of 2, 5 and 15 minutes (one, two and six EBI steps);
AddressSanitizer checks every workspace and table index.  tests/test_gpu_ebi.py holds the
GPU build to the same oracle.
"""
import numpy as np
import pytest

from conftest import run_ebi_harness
from helpers import gather_cells
from cmaq_gb300.synthetic import make_grid


@pytest.mark.parametrize("mech,tstep_sec", [("cb6r5_ae7_aq", 300), ("cb6r5_ae7_aq", 120), ("cb6r5_ae7_aq", 900),
                                            ("cracmm2", 300)])
def test_host_build_equals_the_oracle_bit_for_bit(ebi_harness, tmp_path, mech, tstep_sec):
    from oracle import Oracle
    o = Oracle(mech)
    g = make_grid(mech=mech, ncols=8, nrows=6, nlays=3, seed=24, het=True, seawater_fraction=0.3)
    y, rki, _ = gather_cells(g, o)
    yc0 = np.ascontiguousarray(y[np.asarray(o.iold2new)])      # mechanism species order
    yc, st, it = run_ebi_harness(ebi_harness(mech), yc0, rki, tstep_sec, tmp_path)
    ycr, str_, itr = o.ebi_solve_cells(yc0.copy(), rki, tstep_sec, threads=4)
    assert (st == 0).all() and (str_ == 0).all()
    assert np.array_equal(it, itr), "iteration counts differ from the oracle"
    bad = np.nonzero((yc != ycr).any(axis=0))[0]
    assert len(bad) == 0, f"cells {bad[:8]} differ from the oracle"
