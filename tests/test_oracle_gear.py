"""The SMVGEAR restatement in the oracle (CCTM/src/gas/smvgear), on the CPU.

The reference ships no test or golden vector for its Gear solver and its Fortran cannot
be compiled here, so the restatement is pinned by properties:
* convergence: against a tight ROS3 solution of the same cells (itself checked against
  the reference's structure in the ROS3 tests), the Gear error falls in proportion to
  GEAR_RTOL and the absolute-tolerance levels;
* driver and gather: one CHEM call with BLKSIZE = 1 gives exactly the per-cell solver's
  results on the separately gathered inputs (REAL(8) floor of grdriver.F:419-422);
* block semantics (BLKSIZE 50, stiffness reordering) integrate without failure and stay
  within the tolerance-level error of the per-cell solution;
* the coefficient tables: Nordsieck l0 = ASET(q, 1) of the BDF formulas of order 1-5,
  REAL(4) ENQQ1-3 of JSPARSE.
"""
import numpy as np
import pytest

from helpers import gather_cells
from cmaq_gb300.synthetic import make_grid

F32 = np.float32


@pytest.fixture(scope="module", params=["cb6r5_ae7_aq", "cracmm2"])
def case(request):
    from oracle import Oracle
    o = Oracle(request.param)
    g = make_grid(mech=request.param, ncols=6, nrows=4, nlays=2, seed=61, het=True)
    y0, rk, night = gather_cells(g, o, gear=True)
    with o.tight():
        yt, *_ = o.solve_cells(y0, rk, night, 5.0, 1e-8, 1e-14, threads=4)
    return dict(o=o, g=g, y0=y0, rk=rk, night=night, yt=yt)


def test_gear_converges_to_the_tight_solution(case):
    o, yt = case["o"], case["yt"]
    m = np.abs(yt) > 1e-6
    med, worst = [], []
    for rtol, amax, amin in [(1e-3, 1e-7, 1e-9), (1e-4, 1e-8, 1e-10), (1e-5, 1e-9, 1e-11), (1e-6, 1e-10, 1e-12)]:
        cfg = o.gear_cfg(rtol=float(F32(rtol)), max_atol=amax, min_atol=amin, conc_floor=min(1e-12, amin * 1e-3))
        y, st = o.gear_cells(case["y0"], case["rk"], case["night"], 5.0, cfg=cfg, threads=4)
        assert st[:, 7].max() == 0
        e = np.abs(y[m] - yt[m]) / np.abs(yt[m])
        med.append(float(np.median(e)))
        worst.append(float(np.max(e)))
    # the typical error falls about tenfold per decade of tolerance (measured 6-9x)
    assert all(med[k] > 4.0 * med[k + 1] for k in range(3))
    assert worst[3] < 5e-3 and med[3] < 1e-6


def test_chem_blksize1_equals_per_cell_solver(case):
    o, g = case["o"], case["g"]
    conc, tot = o.chem_gear(g, tstep_sec=300, blksize=1, threads=4)
    assert tot["rc"] == 0
    y, st = o.gear_cells(case["y0"], case["rk"], case["night"], 5.0, threads=4)
    # write-back of the per-cell results as grdriver.F:577-596 does
    from cmaq_gb300.synthetic import manifest
    man = manifest(g.mech)
    n = g.ncell
    want = g.conc.reshape(g.nspcsd, n).copy()
    dens = g.dens.reshape(n).astype(np.float64)
    for s, sp in enumerate(man["species"]):
        v = y[o.iold2new[s]]
        if sp["convert"]:
            fwd = F32(F32(F32(1.0e-3) * F32(28.9628)) / F32(sp["molwt"]))
            v = (np.float64(F32(1.0) / fwd) * dens) * v
        want[g.cgrid_index[s] - 1] = v.astype(F32)
    assert np.array_equal(conc.reshape(g.nspcsd, n), want)
    assert tot["nsteps"] == int(st[:, 0].sum())


def test_block_semantics_run_and_stay_close(case):
    o, g = case["o"], case["g"]
    c1, t1 = o.chem_gear(g, tstep_sec=300, blksize=1, threads=4)
    c50, t50 = o.chem_gear(g, tstep_sec=300, blksize=50, threads=4)
    assert t1["rc"] == 0 and t50["rc"] == 0
    m = np.abs(c1) > 1e-3 * np.abs(c1).max(axis=None)
    assert np.max(np.abs(c50[m] - c1[m]) / np.abs(c1[m])) < 5e-2


def test_gear_coefficients():
    from oracle import Oracle
    o = Oracle("cb6r5_ae7_aq")
    v = np.frombuffer(o.gear_cfg().raw, np.float64, count=80 + 21 + 35)
    aset = v[:80].reshape(10, 8)
    assert np.allclose(aset[:5, 0], [1.0, 2 / 3, 6 / 11, 12 / 25, 60 / 137], rtol=0, atol=1e-16)
    assert np.all(aset[:6, 1] == 1.0)
    enqq = v[101:122].reshape(3, 7)
    for q in range(7):
        assert enqq[0, q] == float(F32(0.5) / F32(q + 1))
        assert enqq[2, q] == float(F32(0.5) / F32(q + 3))
