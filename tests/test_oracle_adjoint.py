"""The oracle's discrete adjoint of ROS3 (CPU) against finite differences.

* central differences of the fixed-step map (the accepted step sizes of the forward
  run replayed): relative 1e-6 on random directions;
* central differences of the adaptive forward (step sizes re-chosen): relative 3e-2.
  The discrete adjoint leaves out the sensitivity of the chosen step sizes; with
  rtol 1e-3 it was measured at 5e-5 to 1e-2 of the derivative (largest in CRACMM2
  cells taking 60-80 steps in their first synchronisation step), smooth in the
  perturbation size, so it is that term and not differencing noise;
* gradients are linear in the adjoint seed.
"""
import numpy as np
import pytest

from helpers import gather_cells
from cmaq_gb300.synthetic import make_grid

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


@pytest.fixture(scope="module", params=["cb6r5_ae7_aq", "cracmm2"])
def case(request):
    from oracle import AdjointWindow, Oracle
    o = Oracle(request.param)
    g = make_grid(mech=request.param, ncols=3, nrows=2, nlays=1, seed=31, het=True)
    y0, rki, night = gather_cells(g, o)
    rng = np.random.default_rng(0)
    emis = 1e-6 * rng.random(y0.shape)
    kmult = np.exp(0.1 * rng.standard_normal(o.nrxns))
    w = AdjointWindow(o, rki, night, 3, 5.0, RTOL, ATOL, kmult=kmult, emis=emis, hcap=2048, threads=2)
    yend = w.forward(y0)
    wt = rng.standard_normal(y0.shape) / np.maximum(yend, 1e-12)
    lam, gk, ge = w.backward(wt)
    return dict(o=o, w=w, y0=y0, rki=rki, night=night, kmult=kmult, emis=emis, yend=yend, wt=wt,
                lam=lam, gk=gk, ge=ge, rng=rng)


def test_replay_reproduces_forward(case):
    c = case
    assert np.array_equal(c["w"].replay(c["y0"], c["kmult"], c["emis"]), c["yend"])


@pytest.mark.parametrize("what", ["y0", "logk", "emis"])
def test_adjoint_vs_fixed_step_differences(case, what):
    c = case
    w, y0, km, em, wt = c["w"], c["y0"], c["kmult"], c["emis"], c["wt"]
    L = lambda y: float((wt * y).sum())
    for _ in range(2):
        if what == "y0":
            d = y0 * c["rng"].standard_normal(y0.shape)
            ad = float((c["lam"] * d).sum())
            f = lambda e: L(w.replay(y0 + e * d, km, em))
        elif what == "logk":
            d = c["rng"].standard_normal(km.shape)
            ad = float((c["gk"] * d).sum())
            f = lambda e: L(w.replay(y0, km * np.exp(e * d), em))
        else:
            d = 1e-6 * c["rng"].standard_normal(em.shape)
            ad = float((c["ge"] * d).sum())
            f = lambda e: L(w.replay(y0, km, em + e * d))
        fd = (f(1e-6) - f(-1e-6)) / 2e-6
        assert abs(ad - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(c["lam"] * y0).sum())


def test_adjoint_vs_adaptive_forward_differences(case):
    from oracle import AdjointWindow
    c = case
    d = c["y0"] * c["rng"].standard_normal(c["y0"].shape)
    ad = float((c["lam"] * d).sum())

    def f(e):
        w2 = AdjointWindow(c["o"], c["rki"], c["night"], 3, 5.0, RTOL, ATOL, kmult=c["kmult"], emis=c["emis"],
                           hcap=2048, threads=2)
        return float((c["wt"] * w2.forward(c["y0"] + e * d)).sum())
    fd = (f(1e-6) - f(-1e-6)) / 2e-6
    assert abs(ad - fd) <= 3e-2 * abs(fd)


def test_adjoint_is_linear_in_the_seed(case):
    c = case
    lam2, gk2, ge2 = c["w"].backward(2.0 * c["wt"])
    assert np.allclose(lam2, 2.0 * c["lam"], rtol=1e-12, atol=0)
    assert np.allclose(gk2, 2.0 * c["gk"], rtol=1e-12, atol=1e-300)
