"""Autotuner: every candidate launch shape gives the same concentrations, the best one is
returned and cached per mechanism / GPU / grid size."""
import numpy as np
import pytest

from cmaq_gb300.synthetic import make_grid

pytestmark = pytest.mark.gpu


def test_tune_returns_and_caches_a_candidate(tmp_path):
    from cmaq_gb300.autotune import candidates, tune, tuned_solver
    from helpers import to_cuda
    g = make_grid(ncols=10, nrows=8, nlays=3, seed=61)
    cache = tmp_path / "tune.json"
    res = tune(g, nsteps=1, variants=("default",), cache=cache)
    assert {"variant", "lockstep", "block_warps", "ms"} <= set(res)
    assert len(res["table"]) == len(candidates(("default",)))
    assert res["ms"] == min(r["ms"] for r in res["table"])
    again = tune(g, nsteps=1, variants=("default",), cache=cache)
    assert again == res
    # the tuned solver and the default one agree bit for bit
    outs = []
    for s in (tuned_solver(g, res, rtol=1e-3, atol=1e-9), None):
        from cmaq_gb300.chem import ChemSolver
        s = s or ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                            cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9)
        t = to_cuda(g)
        s.step(*[t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")])
        outs.append(t["conc"].cpu().numpy())
    assert np.array_equal(outs[0], outs[1])
