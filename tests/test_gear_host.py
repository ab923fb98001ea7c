"""The SMVGEAR device code (cmaq_gb300/csrc/gear.cuh's per-cell state machine with the
generated f, PDERIV, LU and solve routines of cmaq_gb300/csrc/gen/), built for the host,
against the oracle's per-cell SMVGEAR (oracle/gear_oracle.c): the same operations in the
same order, so every concentration and every step, failure, Jacobian, f and Newton count
must agree bit for bit, for both mechanisms and for day and night cells; AddressSanitizer
checks every workspace and table index.  tests/test_gpu_gear.py holds the GPU build to
the same oracle.
"""
import numpy as np
import pytest

from conftest import run_gear_harness
from helpers import gather_cells
from cmaq_gb300.synthetic import make_grid

RTOL = float(np.float32(1e-3))


@pytest.mark.parametrize("mech,dims,seed", [("cb6r5_ae7_aq", (6, 4, 2), 5), ("cracmm2", (5, 3, 2), 6)])
def test_host_build_equals_the_oracle_bit_for_bit(gear_harness, tmp_path, mech, dims, seed):
    from oracle import Oracle
    o = Oracle(mech)
    g = make_grid(mech=mech, ncols=dims[0], nrows=dims[1], nlays=dims[2], seed=seed)
    y0, rk, night = gather_cells(g, o, gear=True)
    assert 0 < night.sum() < len(night)               # day and night cells
    y, st = run_gear_harness(gear_harness(mech), y0, rk, night, 5.0, RTOL, 1e-7, 1e-9, 1e-12, tmp_path)
    yr, sr = o.gear_cells(y0, rk, night, 5.0, o.gear_cfg(rtol=RTOL))
    assert (st[:, 7] == 0).all() and (sr[:, 7] == 0).all()
    assert np.array_equal(st, sr), "step statistics differ from the oracle"
    bad = np.nonzero((y != yr).any(axis=0))[0]
    assert len(bad) == 0, f"cells {bad[:8]} differ from the oracle"
