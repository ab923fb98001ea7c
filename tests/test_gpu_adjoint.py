"""GPU discrete adjoint of ROS3 against the oracle's restatement and finite differences.

Tolerances:
* forward window: the same accepted steps per cell and synchronisation step as the
  oracle, states within 1e-9 relative (species above 1e-10 ppmV);
* gradients (dL/dy0, dL/dlog k, dL/demis) vs the oracle adjoint: relative 1e-7 of the
  largest component (the device sums per-reaction gradients in a different order);
* gradients vs central differences of the adaptive GPU forward: relative 3e-2 on
  random directions (the discrete adjoint holds step sizes fixed; the left-out
  step-size sensitivity measured up to 1e-2 at rtol 1e-3).
"""
import numpy as np
import pytest

from helpers import gather_cells, rel_err
from cmaq_gb300.synthetic import make_grid

pytestmark = pytest.mark.gpu

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


@pytest.fixture(scope="module", params=["cb6r5_ae7_aq", "cracmm2"])
def case(request):
    import torch
    from oracle import Oracle
    from cmaq_gb300.chem import ChemSolver
    mech = request.param
    o = Oracle(mech)
    g = make_grid(mech=mech, ncols=8, nrows=5, nlays=2, seed=41, het=True)
    y0, rki, night = gather_cells(g, o)
    rng = np.random.default_rng(3)
    kmult = np.exp(0.05 * rng.standard_normal(o.nrxns))
    emis = 1e-6 * rng.random(y0.shape)
    s = ChemSolver(mech, ncols=y0.shape[1], nrows=1, nlays=1, nspcsd=g.nspcsd, rtol=1e-3, atol=1e-9)
    t = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
         dict(y0=y0, rki=rki, night=night, kmult=kmult, emis=emis).items()}
    return dict(o=o, s=s, y0=y0, rki=rki, night=night, kmult=kmult, emis=emis, t=t, rng=rng)


def _window(c, nsync=3):
    from cmaq_gb300.adjoint import Ros3Window
    return Ros3Window(c["s"], c["t"]["rki"], c["t"]["night"], nsync, 5.0)


def _rel_vec(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_adjoint_matches_oracle(case):
    import torch
    from oracle import AdjointWindow
    c = case
    wt = c["rng"].standard_normal(c["y0"].shape)
    ow = AdjointWindow(c["o"], c["rki"], c["night"], 3, 5.0, RTOL, ATOL, kmult=c["kmult"], emis=c["emis"], threads=4)
    y_ref = ow.forward(c["y0"])
    wt = wt / np.maximum(np.abs(y_ref), 1e-12)
    lam_ref, gk_ref, ge_ref = ow.backward(wt)

    y0 = c["t"]["y0"].clone().requires_grad_(True)
    logk = torch.log(c["t"]["kmult"]).clone().requires_grad_(True)
    emis = c["t"]["emis"].clone().requires_grad_(True)
    y = _window(c)(y0, logk, emis)
    assert rel_err(y.detach().cpu().numpy(), y_ref) < 1e-9
    (y * torch.from_numpy(wt).cuda()).sum().backward()
    assert _rel_vec(y0.grad.cpu().numpy(), lam_ref) < 1e-7
    assert _rel_vec(logk.grad.cpu().numpy(), gk_ref) < 1e-7
    assert _rel_vec(emis.grad.cpu().numpy(), ge_ref) < 1e-7


def test_adjoint_matches_finite_differences(case):
    import torch
    c = case
    w = _window(c, nsync=2)
    wt = torch.from_numpy(c["rng"].standard_normal(c["y0"].shape)).cuda()
    y0 = c["t"]["y0"]
    logk0 = torch.log(c["t"]["kmult"])
    emis0 = c["t"]["emis"]
    yend = w(y0, logk0, emis0)
    wt = wt / yend.abs().clamp_min(1e-12)

    def loss(y, k, e):
        return float((w(y, k, e) * wt).sum())

    a_y, a_k, a_e = (t.clone().requires_grad_(True) for t in (y0, logk0, emis0))
    (w(a_y, a_k, a_e) * wt).sum().backward()
    for _ in range(2):
        dy = y0 * torch.randn_like(y0)
        dk = torch.randn_like(logk0)
        de = 1e-6 * torch.randn_like(emis0)
        ad = float((a_y.grad * dy).sum() + (a_k.grad * dk).sum() + (a_e.grad * de).sum())
        eps = 1e-6
        fd = (loss(y0 + eps * dy, logk0 + eps * dk, emis0 + eps * de)
              - loss(y0 - eps * dy, logk0 - eps * dk, emis0 - eps * de)) / (2 * eps)
        assert abs(ad - fd) <= 3e-2 * abs(fd)


def test_per_step_rate_constants_and_no_optional_inputs(case):
    import torch
    from cmaq_gb300.adjoint import Ros3Window
    from oracle import AdjointWindow
    c = case
    rki3 = np.stack([c["rki"] * f for f in (1.0, 0.9, 1.1)])
    ow = AdjointWindow(c["o"], rki3, c["night"], 3, 5.0, RTOL, ATOL, threads=4)
    y_ref = ow.forward(c["y0"])
    lam_ref, gk_ref, _ = ow.backward(np.ones_like(y_ref))
    w = Ros3Window(c["s"], torch.from_numpy(rki3).cuda(), c["t"]["night"], 3, 5.0)
    y0 = c["t"]["y0"].clone().requires_grad_(True)
    y = w(y0)
    assert rel_err(y.detach().cpu().numpy(), y_ref) < 1e-9
    y.sum().backward()
    assert _rel_vec(y0.grad.cpu().numpy(), lam_ref) < 1e-7


def test_tape_budget_batches_give_the_same_gradients(case):
    """A tape budget far below one step's tape makes the backward pass run each step in
    batches of consecutive cells; per-cell results are unchanged (the log-k sums only
    change their order)."""
    import torch
    from cmaq_gb300.adjoint import Ros3Window
    c = case
    w = Ros3Window(c["s"], c["t"]["rki"], c["t"]["night"], 2, 5.0, tape_bytes=0)   # every step re-run
    res = []
    for mb in (0, 1):
        c["s"].set_tuning(adjoint_tape_mb=mb)
        y0 = c["t"]["y0"].clone().requires_grad_(True)
        logk = torch.log(c["t"]["kmult"]).clone().requires_grad_(True)
        emis = c["t"]["emis"].clone().requires_grad_(True)
        w(y0, logk, emis).sum().backward()
        res.append((y0.grad.cpu().numpy(), logk.grad.cpu().numpy(), emis.grad.cpu().numpy()))
    c["s"].set_tuning(adjoint_tape_mb=0)
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][2], res[1][2])
    assert _rel_vec(res[1][1], res[0][1]) < 1e-12


@pytest.mark.parametrize("ncell", [1, 33])
def test_adjoint_on_ragged_cell_counts(ncell):
    """One cell and one cell more than a warp: the queue and the tape offsets cover ragged
    sizes; gradients match the oracle."""
    import torch
    from oracle import AdjointWindow, Oracle
    from cmaq_gb300.adjoint import Ros3Window
    from cmaq_gb300.chem import ChemSolver
    o = Oracle("cb6r5_ae7_aq")
    g = make_grid(ncols=ncell, nrows=1, nlays=1, seed=42)
    y0, rki, night = gather_cells(g, o)
    ow = AdjointWindow(o, rki, night, 2, 5.0, RTOL, ATOL, threads=2)
    y_ref = ow.forward(y0)
    lam_ref, gk_ref, _ = ow.backward(np.ones_like(y_ref))
    s = ChemSolver("cb6r5_ae7_aq", ncols=ncell, nrows=1, nlays=1, nspcsd=g.nspcsd, rtol=1e-3, atol=1e-9)
    w = Ros3Window(s, torch.from_numpy(rki).cuda(), torch.from_numpy(night).cuda(), 2, 5.0)
    a = torch.from_numpy(y0).cuda().requires_grad_(True)
    k = torch.zeros(o.nrxns, dtype=torch.float64, device="cuda", requires_grad=True)
    y = w(a, k)
    assert rel_err(y.detach().cpu().numpy(), y_ref) < 1e-9
    y.sum().backward()
    assert _rel_vec(a.grad.cpu().numpy(), lam_ref) < 1e-7
    assert _rel_vec(k.grad.cpu().numpy(), gk_ref) < 1e-7


def test_forward_tape_full_partial_and_absent_agree(case):
    """The tape recorded by the forward pass (complete, partial: later steps re-run, or
    absent: every step re-run) changes nothing but the log-k summation order."""
    import torch
    from cmaq_gb300.adjoint import Ros3Window
    c = case
    res = []
    n, ischan = c["y0"].shape[1], c["s"].info.ischan
    one_step = n * 3 * 64 + 4 * n * (ischan + 1) * 8      # room for about one step's blocks
    for tb in (None, one_step, 0):
        w = Ros3Window(c["s"], c["t"]["rki"], c["t"]["night"], 3, 5.0, tape_bytes=tb)
        y0 = c["t"]["y0"].clone().requires_grad_(True)
        logk = torch.log(c["t"]["kmult"]).clone().requires_grad_(True)
        emis = c["t"]["emis"].clone().requires_grad_(True)
        y = w(y0, logk, emis)
        (y * y.detach().clamp_min(1e-12).reciprocal()).sum().backward()
        res.append((y.detach().cpu().numpy(), y0.grad.cpu().numpy(), logk.grad.cpu().numpy(),
                    emis.grad.cpu().numpy()))
    for r in res[1:]:
        assert np.array_equal(r[0], res[0][0])
        assert np.array_equal(r[1], res[0][1])
        assert np.array_equal(r[3], res[0][3])
        assert _rel_vec(r[2], res[0][2]) < 1e-12
