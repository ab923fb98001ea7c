"""The ROS3 device code (cmaq_gb300/csrc/ros3.cuh with the generated rate, LU and solve
routines of cmaq_gb300/csrc/gen/), built for the host, against the oracle's per-cell
RBSOLVER (oracle/ros3_oracle.c): the generator's straight-line code and the oracle's
restatement perform the same IEEE operations in the same order, so every concentration
and step counter must agree bit for bit; AddressSanitizer checks every workspace index the
generated code touches, for both mechanisms, on day, night and mixed groups of 32 cells
and on a ragged last group.  tests/test_gpu_parity.py holds the GPU build to the same
oracle.
"""
import numpy as np
import pytest

from conftest import run_ros3_harness
from helpers import gather_cells
from cmaq_gb300.synthetic import make_grid

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


@pytest.mark.parametrize("mech,dims,seed", [("cb6r5_ae7_aq", (10, 8, 3), 21), ("cb6r5_ae7_aq", (33, 1, 1), 5),
                                            ("cracmm2", (9, 5, 2), 22)])
def test_host_build_equals_the_oracle_bit_for_bit(ros3_harness, tmp_path, mech, dims, seed):
    from oracle import Oracle
    o = Oracle(mech)
    g = make_grid(mech=mech, ncols=dims[0], nrows=dims[1], nlays=dims[2], seed=seed, het=True)
    y0, rki, night = gather_cells(g, o)
    if dims == (33, 1, 1):
        night[:] = 1                      # a dark group of 32 and a ragged dark cell: night lists
    y, ns, nf, st = run_ros3_harness(ros3_harness(mech), y0, rki, night, 5.0, RTOL, ATOL, tmp_path)
    yr, nsr, nfr, str_ = o.solve_cells(y0, rki, night, 5.0, RTOL, ATOL, threads=4)
    assert (st == 0).all() and (str_ == 0).all()
    assert np.array_equal(ns, nsr) and np.array_equal(nf, nfr), "step counts differ from the oracle"
    bad = np.nonzero((y != yr).any(axis=0))[0]
    assert len(bad) == 0, f"cells {bad[:8]} differ from the oracle"
    assert ns.sum() > 0
