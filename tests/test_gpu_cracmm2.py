"""GPU parity of ROS3 for the larger mechanism, CRACMM2 (189 species, 531 reactions),
against the oracle; same tolerances as tests/test_gpu_parity.py."""
import numpy as np
import pytest

from helpers import gather_cells, gpu_chem, rel_err, to_cuda
from cmaq_gb300.synthetic import make_grid

pytestmark = pytest.mark.gpu

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


@pytest.fixture(scope="module")
def oracle():
    from oracle import Oracle
    return Oracle("cracmm2")


@pytest.fixture(scope="module")
def grid():
    return make_grid(mech="cracmm2", ncols=9, nrows=8, nlays=4, seed=71, het=True, seawater_fraction=0.3)


def _solver(g, **kw):
    from cmaq_gb300.chem import ChemSolver
    return ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                      cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, **kw)


def test_rconst_parity(oracle, grid):
    s = _solver(grid)
    t = to_cuda(grid)
    rki, sun = s.rconst(*[t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj",
                                         "khetero")])
    _, rki_ref, night = gather_cells(grid, oracle)
    assert np.array_equal(sun.cpu().numpy(), 1 - night)
    assert rel_err(rki.cpu().numpy(), rki_ref, floor=1e-300) < 1e-12


def test_solver_parity_same_rate_constants(oracle, grid):
    import torch
    y0, rki, night = gather_cells(grid, oracle)
    y_ref, ns_ref, nf_ref, st_ref = oracle.solve_cells(y0, rki, night, 5.0, RTOL, ATOL, threads=4)
    y = torch.from_numpy(y0.copy()).cuda()
    st, ns, nf = _solver(grid).solve(y, torch.from_numpy(rki).cuda(), torch.from_numpy(night).cuda(), 5.0,
                                     with_stats=True)
    assert (st_ref == 0).all() and (st.cpu().numpy() == 0).all()
    assert np.array_equal(ns.cpu().numpy(), ns_ref) and np.array_equal(nf.cpu().numpy(), nf_ref)
    assert rel_err(y.cpu().numpy(), y_ref) < 1e-9


def test_chem_call_parity_and_schedules(oracle, grid):
    conc_static, stats, _ = gpu_chem(grid, schedule="static")
    conc_ref, tot = oracle.chem(grid, blksize=1, rtol=RTOL, atol=ATOL, threads=4)
    assert stats[0]["failed_cells"] == 0 and tot["rc"] == 0
    assert stats[0]["accepted_steps"] == tot["nsteps"] and stats[0]["rejected_steps"] == tot["nfails"]
    assert rel_err(conc_static, conc_ref) < 1e-5
    conc_queue, _, _ = gpu_chem(grid, schedule="queue")
    assert np.array_equal(conc_queue, conc_static)


def test_step_cap_failures_are_reported(grid):
    """A cap of 3 step attempts cannot finish a 5-minute call (the first step is 0.05 min):
    every cell reports CMAQCHEM_CELL_MAXITER and keeps its last accepted state."""
    s = _solver(grid, max_iter=3)
    t = to_cuda(grid)
    st = s.step(*[t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")])
    assert st["failed_cells"] == grid.ncell
    status, attempts = s.cell_stats()
    assert (status == 2).all() and (attempts == 3).all()
    assert np.isfinite(t["conc"].cpu().numpy()).all()
