"""GPU parity of the chemistry operator against the CPU oracle (ROS3 restatement).

Tolerances:
* rate constants: relative 1e-12 (device and host exp/pow/log10 differ by a few ulps);
* ROS3 on identical rate constants: relative 1e-9 on species above 1e-10 ppmV (same
  operation order and fma placement; only pow() in the step-size factor may differ
  by an ulp);
* a full CHEM call: relative 1e-5 on the REAL(4) concentrations above 1e-10 ppmV;
* work-queue and static schedules: bit-identical.
"""
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
    return Oracle("cb6r5_ae7_aq")


@pytest.fixture(scope="module")
def grid():
    return make_grid(ncols=12, nrows=10, nlays=5, seed=11, het=True, seawater_fraction=0.3)


def _solver(g, **kw):
    from cmaq_gb300.chem import ChemSolver
    return ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                      cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, **kw)


def test_rconst_parity(oracle, grid):
    s = _solver(grid)
    t = to_cuda(grid)
    rki, sun = s.rconst(t["conc"], t["ta"], t["qv"], t["dens"], t["pres"], t["seaice"], t["ocean_szone"],
                        t["rj"], t["khetero"])
    _, rki_ref, night = gather_cells(grid, oracle)
    assert np.array_equal(sun.cpu().numpy(), 1 - night)
    got = rki.cpu().numpy()
    assert np.isfinite(got).all()
    nz = np.abs(rki_ref) > 0
    assert np.array_equal(got != 0, nz)
    assert rel_err(got, rki_ref, floor=1e-300) < 1e-12


def test_solver_parity_same_rate_constants(oracle, grid):
    import torch
    y0, rki, night = gather_cells(grid, oracle)
    y_ref, ns_ref, nf_ref, st_ref = oracle.solve_cells(y0, rki, night, 5.0, RTOL, ATOL, threads=4)
    s = _solver(grid)
    y = torch.from_numpy(y0.copy()).cuda()
    st, ns, nf = s.solve(y, torch.from_numpy(rki).cuda(), torch.from_numpy(night).cuda(), 5.0, with_stats=True)
    assert (st_ref == 0).all() and (st.cpu().numpy() == 0).all()
    assert np.array_equal(ns.cpu().numpy(), ns_ref) and np.array_equal(nf.cpu().numpy(), nf_ref)
    assert rel_err(y.cpu().numpy(), y_ref) < 1e-9


def test_chem_call_parity_per_cell(oracle, grid):
    conc_gpu, stats, _ = gpu_chem(grid, schedule="static")
    conc_ref, tot = oracle.chem(grid, blksize=1, rtol=RTOL, atol=ATOL, threads=4)
    assert stats[0]["failed_cells"] == 0 and tot["rc"] == 0
    assert stats[0]["accepted_steps"] == tot["nsteps"]
    assert stats[0]["rejected_steps"] == tot["nfails"]
    assert rel_err(conc_gpu, conc_ref) < 1e-5


def test_queue_schedule_is_bit_identical(grid):
    a, sa, _ = gpu_chem(grid, schedule="static", nsteps=2)
    b, sb, _ = gpu_chem(grid, schedule="queue", nsteps=2)
    assert np.array_equal(a, b)
    assert [x["accepted_steps"] for x in sa] == [x["accepted_steps"] for x in sb]


@pytest.mark.parametrize("dims", [(7, 5, 3), (1, 1, 1), (33, 1, 1)])
def test_ragged_grids(oracle, dims):
    g = make_grid(ncols=dims[0], nrows=dims[1], nlays=dims[2], seed=5)
    conc_gpu, stats, _ = gpu_chem(g, schedule="queue")
    conc_ref, tot = oracle.chem(g, blksize=1, rtol=RTOL, atol=ATOL)
    assert stats[0]["failed_cells"] == 0
    assert rel_err(conc_gpu, conc_ref) < 1e-5


def test_all_dark_grid_uses_night_reactions(oracle):
    g = make_grid(ncols=8, nrows=4, nlays=2, seed=6, sza_range=(95.0, 100.0))
    assert float(g.rj.max()) == 0.0
    conc_gpu, stats, _ = gpu_chem(g)
    assert stats[0]["sunlit_cells"] == 0
    conc_ref, _ = oracle.chem(g, blksize=1, rtol=RTOL, atol=ATOL)
    assert rel_err(conc_gpu, conc_ref) < 1e-5


@pytest.mark.parametrize("tstep", [(10000, 100, 100), (10000, 1000, 1000)])
def test_sync_step_lengths(oracle, tstep):
    g = make_grid(ncols=6, nrows=6, nlays=2, seed=8)
    conc_gpu, stats, _ = gpu_chem(g, tstep=tstep)
    sec = (tstep[1] // 100) * 60 + tstep[1] % 100
    conc_ref, _ = oracle.chem(g, blksize=1, rtol=RTOL, atol=ATOL, tstep_sec=sec)
    assert rel_err(conc_gpu, conc_ref) < 1e-5


def test_host_pointer_entry_matches_device_entry(grid):
    from cmaq_gb300.chem import ChemSolver
    dev, _, _ = gpu_chem(grid, schedule="static")
    s = ChemSolver(grid.mech, ncols=grid.ncols, nrows=grid.nrows, nlays=grid.nlays, nspcsd=grid.nspcsd,
                   cgrid_index=grid.cgrid_index, rtol=1e-3, atol=1e-9, schedule="static")
    conc = grid.conc.copy()
    s.step(conc, grid.ta, grid.qv, grid.dens, grid.pres, grid.seaice, grid.ocean_szone, grid.rj, grid.khetero)
    assert np.array_equal(conc, dev)


def test_shape_errors_are_reported(grid):
    from cmaq_gb300._lib import ChemError
    s = _solver(grid)
    t = to_cuda(grid)
    with pytest.raises(ChemError):
        s.step(t["conc"][:, :1], t["ta"], t["qv"], t["dens"], t["pres"], t["seaice"], t["ocean_szone"], t["rj"],
               t["khetero"])


def test_graph_replayed_steps_match_single_calls(grid):
    from helpers import to_cuda
    a, sa, _ = gpu_chem(grid, schedule="queue", nsteps=3)
    s = _solver(grid, schedule="queue")
    t = to_cuda(grid)
    args = [t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")]
    st = s.steps(3, *args)
    assert np.array_equal(t["conc"].cpu().numpy(), a)
    assert st["accepted_steps"] == sum(x["accepted_steps"] for x in sa)
    # a second replay continues from the new state, like further single calls
    st2 = s.steps(1, *args)
    b, sb, _ = gpu_chem(grid, schedule="queue", nsteps=4)
    assert np.array_equal(t["conc"].cpu().numpy(), b)
    assert st2["accepted_steps"] == sb[3]["accepted_steps"]


@pytest.mark.parametrize("chunks", [1, 3, 16])
def test_chunked_host_path_matches_device_path(grid, chunks):
    """The host-pointer call moves the grid in chunks whose copies overlap the integration;
    results, per-cell stats and totals equal the device-pointer call's, over two calls
    (the second one ordered by the first one's step counts)."""
    from cmaq_gb300.chem import ChemSolver
    dev, sdev, _ = gpu_chem(grid, schedule="queue", nsteps=2)
    s = ChemSolver(grid.mech, ncols=grid.ncols, nrows=grid.nrows, nlays=grid.nlays, nspcsd=grid.nspcsd,
                   cgrid_index=grid.cgrid_index, rtol=1e-3, atol=1e-9, schedule="queue")
    s.set_tuning(host_chunks=chunks)
    conc = grid.conc.copy()
    st = [s.step(conc, grid.ta, grid.qv, grid.dens, grid.pres, grid.seaice, grid.ocean_szone, grid.rj,
                 grid.khetero) for _ in range(2)]
    assert np.array_equal(conc, dev)
    assert [x["accepted_steps"] for x in st] == [x["accepted_steps"] for x in sdev]
