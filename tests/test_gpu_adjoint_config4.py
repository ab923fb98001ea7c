"""The differentiable 1-hour window of the adjoint benchmark (100x100x35 cells, 12 x 5-min
synchronisation steps, L = sum of O3 over the surface layer at the end) on slices of that
grid, checked two ways on the GPU:

* against central differences on 50 random directions (initial concentrations, the
  per-reaction log rate multipliers and the emission tendencies together) of the
  oracle's fixed-step map: the forward run's accepted step sizes replayed at perturbed
  inputs (oracle/ros3_adjoint.c: oracle_adj_replay), which is the map the discrete
  adjoint differentiates.  Tolerance: 1e-5 of the directional derivative plus 1e-6 of
  the sum of its absolute terms (central differences with a 1e-6 step in double);
* against CMAQ's own sensitivities, DDM-3D on the GPU (cmaqchem_step_ddm_device,
  CCTM/src/ddm3d/DDM3D_CHEM.F:155-511), for NOx and VOC emissions over an hour that
  follows a 1-hour spin-up.  Emissions enter between the chemistry calls, as VDIFF adds
  them (E * DT into CGRID, and DT into the emitted species' row of SENGRID for the
  parameter); the adjoint side chains one-step windows with the same injection.  DDM-3D
  linearises each synchronisation step once, at the step's time-averaged concentrations
  (a Crank-Nicolson-type update), so a pulse of emitted NO that reacts away within the
  step is followed less accurately the longer the step: measured 3.8 % for the NO
  parameter with 5-minute steps; the test uses 1-minute steps (TSTEP(2) = 000100, 60
  CHEM calls) and a tolerance of 2e-2.
"""
import numpy as np
import pytest

from helpers import gather_cells
from cmaq_gb300.synthetic import make_grid, manifest, subgrid

pytestmark = pytest.mark.gpu

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


def _slice(ncols, nrows):
    """Surface cells of the 100x100x35 benchmark grid: every (100 // ncols)-th column and
    (100 // nrows)-th row of layer 1."""
    g = make_grid(ncols=100, nrows=100, nlays=35, seed=2018)
    return subgrid(g, 100 // ncols, 100 // nrows, 35)


def test_window_gradients_match_fixed_step_differences_on_50_directions():
    import torch
    from oracle import AdjointWindow, Oracle
    from cmaq_gb300.adjoint import Ros3Window
    from cmaq_gb300.chem import ChemSolver
    sub = _slice(10, 10)
    o = Oracle(sub.mech)
    names = [sp["name"] for sp in manifest(sub.mech)["species"]]
    io3 = int(o.iold2new[names.index("O3")])
    y0, rki, night = gather_cells(sub, o)
    rng = np.random.default_rng(2018)
    logk0 = 0.02 * rng.standard_normal(o.nrxns)
    emis0 = 1e-7 * rng.random(y0.shape)
    n = y0.shape[1]
    # GPU: forward over the hour and the adjoint of L = sum of surface O3
    s = ChemSolver(sub.mech, ncols=n, nrows=1, nlays=1, nspcsd=sub.nspcsd, rtol=1e-3, atol=1e-9)
    w = Ros3Window(s, torch.from_numpy(rki).cuda(), torch.from_numpy(night).cuda(), 12, 5.0)
    a_y = torch.from_numpy(y0).cuda().requires_grad_(True)
    a_k = torch.from_numpy(logk0).cuda().requires_grad_(True)
    a_e = torch.from_numpy(emis0).cuda().requires_grad_(True)
    y = w(a_y, a_k, a_e)
    y[io3].sum().backward()
    gy, gk, ge = (t.grad.cpu().numpy() for t in (a_y, a_k, a_e))
    # the oracle's forward takes the same steps; its replay is the fixed-step map
    ow = AdjointWindow(o, rki, night, 12, 5.0, RTOL, ATOL, kmult=np.exp(logk0), emis=emis0, threads=8)
    yref = ow.forward(y0)
    big = np.abs(yref) > 1e-10
    assert np.max(np.abs(y.detach().cpu().numpy()[big] - yref[big]) / np.abs(yref[big])) < 1e-9

    def loss(yy, kk, ee):
        return float(ow.replay(yy, np.exp(kk), ee)[io3].sum())

    eps = 1e-6
    for _ in range(50):
        dy = y0 * rng.standard_normal(y0.shape)
        dk = rng.standard_normal(o.nrxns)
        de = 1e-7 * rng.standard_normal(y0.shape)
        terms = np.concatenate([(gy * dy).ravel(), gk * dk, (ge * de).ravel()])
        ad = float(terms.sum())
        fd = (loss(y0 + eps * dy, logk0 + eps * dk, emis0 + eps * de)
              - loss(y0 - eps * dy, logk0 - eps * dk, emis0 - eps * de)) / (2 * eps)
        tol = 1e-5 * abs(fd) + 1e-6 * float(np.abs(terms).sum())
        assert abs(ad - fd) <= tol, (ad, fd)
    s.close()


def test_emission_gradients_match_gpu_ddm3d():
    import torch
    from cmaq_gb300.adjoint import Ros3Window
    from cmaq_gb300.chem import ChemSolver
    from cmaq_gb300.synthetic import solver_inputs
    sub = _slice(6, 4)
    names = [sp["name"] for sp in manifest(sub.mech)["species"]]
    emitted = ["NO", "NO2"] + [v for v in ("FORM", "ISOP") if v in names]
    slots = [int(sub.cgrid_index[names.index(v)]) - 1 for v in emitted]
    dt = 1.0                                                    # minutes per synchronisation step
    nstep = 60
    tstep = (10000, 100, 100)                                   # TSTEP(2) = 000100: one minute
    e_rate = 1e-6                                               # ppm/min of each emitted species
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(sub, k))).cuda()
           for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")}
    args = [dev[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")]
    s = ChemSolver(sub.mech, ncols=sub.ncols, nrows=sub.nrows, nlays=sub.nlays, nspcsd=sub.nspcsd,
                   cgrid_index=sub.cgrid_index, rtol=1e-3, atol=1e-9)
    for _ in range(12):                                         # spin-up hour, no emissions
        s.step(*args)
    spun = subgrid(sub, 1, 1, 1)
    spun.conc = dev["conc"].cpu().numpy().copy()
    # DDM-3D on the GPU: parameter p = the emission rate of species emitted[p] in every cell
    nparam = len(emitted)
    sen = torch.zeros((sub.nspcsd, nparam) + tuple(dev["conc"].shape[1:]), dtype=torch.float32, device="cuda")
    for _ in range(nstep):
        for p, slot in enumerate(slots):
            dev["conc"][slot] += e_rate * dt                    # VDIFF adds E * DT
            sen[slot, p] += dt                                  # and DT to the parameter's own species
        s.step_ddm(sen, *args, tstep=tstep)
    io3_slot = int(sub.cgrid_index[names.index("O3")]) - 1
    ddm = sen[io3_slot].reshape(nparam, -1).sum(dim=1).double().cpu().numpy()
    s.close()
    # the adjoint of the same hour: one-step windows, the injection before each
    n = sub.ncell
    ss = ChemSolver(sub.mech, ncols=n, nrows=1, nlays=1, nspcsd=sub.nspcsd, rtol=1e-3, atol=1e-9)
    gs = ChemSolver(sub.mech, ncols=sub.ncols, nrows=sub.nrows, nlays=sub.nlays, nspcsd=sub.nspcsd,
                    cgrid_index=sub.cgrid_index, rtol=1e-3, atol=1e-9)
    y1, rki, night = solver_inputs(spun, gs)
    gs.close()
    rows = [ss.iold2new[names.index(v)] for v in emitted]
    rate = torch.full((nparam,), e_rate, dtype=torch.float64, device="cuda", requires_grad=True)
    y = y1
    for _ in range(nstep):
        inj = torch.zeros_like(y1)
        inj = inj.index_put((torch.tensor(rows, device="cuda"),), (rate * dt)[:, None].expand(nparam, n),
                            accumulate=True)
        y = Ros3Window(ss, rki, night, 1, dt)(y + inj)
    y[ss.iold2new[names.index("O3")]].sum().backward()
    adj = rate.grad.cpu().numpy()
    ss.close()
    rel = np.abs(adj - ddm) / np.abs(adj)
    assert (rel <= 2e-2).all(), list(zip(emitted, adj, ddm, rel))
