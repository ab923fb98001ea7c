"""GPU parity of the EBI solver (HRSOLVER / HRDRIVER) against the CPU oracle.

Tolerances:
* HRSOLVER on identical inputs: the same Backward-Euler iteration count per cell and
  relative 1e-12 on species above 1e-10 ppmV (the translated routines run in the same
  operation order on both sides, without contraction);
* a full EBI CHEM call: relative 1e-5 on the REAL(4) concentrations above 1e-10 ppmV
  (device and host rate constants differ by a few ulps through exp/pow).
"""
import numpy as np
import pytest

from helpers import gather_cells, rel_err, to_cuda
from cmaq_gb300.synthetic import make_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["cb6r5_ae7_aq", "cracmm2"])
def mech(request):
    return request.param


@pytest.fixture(scope="module")
def oracle(mech):
    from oracle import Oracle
    return Oracle(mech)


def _solver(g, **kw):
    from cmaq_gb300.chem import ChemSolver
    return ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                      cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, solver="ebi", **kw)


def _run(g, s, nsteps=1, tstep=(10000, 500, 500)):
    t = to_cuda(g)
    stats = [s.step(t["conc"], t["ta"], t["qv"], t["dens"], t["pres"], t["seaice"], t["ocean_szone"], t["rj"],
                    t["khetero"], tstep=tstep) for _ in range(nsteps)]
    return t["conc"].cpu().numpy(), stats


@pytest.mark.parametrize("tstep_sec", [300, 120, 900])
def test_hrsolver_parity_same_rate_constants(oracle, mech, tstep_sec):
    import torch
    g = make_grid(mech=mech, ncols=10, nrows=8, nlays=3, seed=21, het=True, seawater_fraction=0.3)
    y, rki, _ = gather_cells(g, oracle)
    yc0 = np.ascontiguousarray(y[np.asarray(oracle.iold2new)])   # mechanism species order
    yc_ref, st_ref, it_ref = oracle.ebi_solve_cells(yc0.copy(), rki, tstep_sec, threads=4)
    s = _solver(g)
    yc = torch.from_numpy(yc0.copy()).cuda()
    st, it = s.ebi_solve(yc, torch.from_numpy(rki).cuda(), tstep_sec, with_stats=True)
    assert (st_ref == 0).all() and (st.cpu().numpy() == 0).all()
    assert np.array_equal(it.cpu().numpy(), it_ref)
    assert rel_err(yc.cpu().numpy(), yc_ref) < 1e-12


def test_ebi_chem_call_parity(oracle, mech):
    g = make_grid(mech=mech, ncols=12, nrows=9, nlays=4, seed=23, het=True, seawater_fraction=0.3)
    conc_ref, tot = oracle.chem_ebi(g, threads=4)
    conc, stats = _run(g, _solver(g))
    assert tot["rc"] == 0 and stats[0]["failed_cells"] == 0
    assert rel_err(conc, conc_ref) < 1e-5
    assert stats[0]["sunlit_cells"] == int((g.rj.reshape(g.rj.shape[0], -1) > 0).any(axis=0).sum())


def test_ebi_static_and_queue_schedules_agree():
    g = make_grid(ncols=9, nrows=7, nlays=3, seed=24)
    a, sa = _run(g, _solver(g, schedule="static"), nsteps=2)
    b, sb = _run(g, _solver(g, schedule="queue"), nsteps=2)
    assert np.array_equal(a, b)
    assert [x["accepted_steps"] for x in sa] == [x["accepted_steps"] for x in sb]


@pytest.mark.parametrize("dims", [(1, 1, 1), (33, 1, 1)])
def test_ebi_ragged_grids(dims):
    from oracle import Oracle
    g = make_grid(ncols=dims[0], nrows=dims[1], nlays=dims[2], seed=25)
    conc_ref, _ = Oracle(g.mech).chem_ebi(g)
    conc, _ = _run(g, _solver(g))
    assert rel_err(conc, conc_ref) < 1e-5


def test_ebi_iteration_cap_is_reported():
    # a 5-minute step is two EBI steps, so a cap of one iteration stops every cell
    g = make_grid(ncols=4, nrows=4, nlays=1, seed=26)
    s = _solver(g, max_iter=1)
    _, stats = _run(g, s)
    assert stats[0]["failed_cells"] == g.ncell
    status, iters = s.cell_stats()
    assert (status == 2).all() and (iters == 1).all()


@pytest.mark.parametrize("mech_name", ["cb6r5_ae7_aq", "cracmm2"])
def test_warp_and_lane_ebi_kernels_are_bit_identical(mech_name):
    """One cell per warp (state in shared memory, routines spread over the lanes), one cell
    per lane, and one cell per lane handing long-running cells to the warp kernel compute
    every value with the same operations: identical output and iteration counts over two
    calls."""
    g = make_grid(mech=mech_name, ncols=10, nrows=7, nlays=3, seed=27, het=True)
    res = []
    for warp, defer in ((1, 0), (0, 0), (1, 50)):
        s = _solver(g)
        s.set_tuning(ebi_warp=warp, ebi_defer=defer)   # (1, 50): lanes, then warps past 50 iterations
        conc, stats = _run(g, s, nsteps=2)
        res.append((conc, [x["accepted_steps"] for x in stats], s.cell_stats()[1]))
    assert (res[2][2] > 50).any()                         # some cells were handed to the warp kernel
    for r in res[1:]:
        assert np.array_equal(res[0][0], r[0])
        assert res[0][1] == r[1]
        assert np.array_equal(res[0][2], r[2])
