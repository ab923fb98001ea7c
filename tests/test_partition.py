"""Multi-process path on CPU: subdomain split over 2 gloo ranks changes no per-cell result,
and the shards' log-k gradients summed over the ranks are the whole domain's."""
import os
import socket

import numpy as np
import pytest

from cmaq_gb300.partition import balanced_ranges, subdomain


def test_subdomains_tile_the_domain():
    ncols, nrows = 17, 10
    seen = np.zeros((nrows, ncols), int)
    for r in range(3 * 2):
        c, w = subdomain(ncols, nrows, 3, 2, r)
        seen[w, c] += 1
    assert (seen == 1).all()
    with pytest.raises(ValueError):
        subdomain(2, 2, 3, 1, 0)


def test_balanced_ranges_cover_and_balance():
    rng = np.random.default_rng(0)
    cost = rng.integers(1, 100, size=1000)
    rs = balanced_ranges(cost, 4)
    assert rs[0][0] == 0 and rs[-1][1] == 1000
    assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
    sums = [cost[a:b].sum() for a, b in rs]
    assert max(sums) - min(sums) <= 2 * cost.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    sys.path.insert(0, str(root / "oracle"))
    import torch
    import torch.distributed as dist
    from cmaq_gb300.partition import sub_grid, subdomain
    from cmaq_gb300.synthetic import make_grid
    from oracle import Oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    g = make_grid(ncols=9, nrows=4, nlays=2, seed=21)
    cols, rows = subdomain(g.ncols, g.nrows, world, 1, rank)
    sub = sub_grid(g, cols, rows)
    conc, tot = Oracle(g.mech).chem(sub, blksize=1, threads=1)
    parts = [None] * world
    dist.all_gather_object(parts, (cols.start, cols.stop, conc))
    if rank == 0:
        full = np.empty_like(g.conc)
        for c0, c1, cc in parts:
            full[:, :, :, c0:c1] = cc
        out_q.put(full)
    dist.destroy_process_group()


def test_two_rank_decomposition_matches_single_domain():
    import multiprocessing as mp
    from cmaq_gb300.synthetic import make_grid
    from oracle import Oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    full = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    g = make_grid(ncols=9, nrows=4, nlays=2, seed=21)
    ref, _ = Oracle(g.mech).chem(g, blksize=1, threads=1)
    assert np.array_equal(full, ref)


NSYNC, RTOL_A, ATOL_A = 2, float(np.float32(1e-3)), float(np.float32(1e-9))


def _adjoint_case():
    """Surface O3 at the end of two 5-min steps of a 4x3x1 grid, its gradient wrt the
    per-reaction log rate multipliers (oracle adjoint)."""
    from helpers import gather_cells
    from cmaq_gb300.synthetic import make_grid, manifest
    from oracle import Oracle
    o = Oracle("cb6r5_ae7_aq")
    g = make_grid(ncols=4, nrows=3, nlays=1, seed=33, het=True)
    y0, rki, night = gather_cells(g, o)
    names = [sp["name"] for sp in manifest(g.mech)["species"]]
    lam = np.zeros_like(y0)
    lam[o.iold2new[names.index("O3")]] = 1.0
    return o, y0, rki, night, lam


def _logk_grad(o, y0, rki, night, lam):
    from oracle import AdjointWindow
    w = AdjointWindow(o, rki, night, NSYNC, 5.0, RTOL_A, ATOL_A, kmult=np.ones(o.nrxns), threads=1)
    w.forward(y0)
    return w.backward(lam)[1]


def _grad_worker(rank, world, port, out_q):
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    for p in (root, root / "oracle", root / "tests"):
        sys.path.insert(0, str(p))
    import torch
    import torch.distributed as dist
    from cmaq_gb300.partition import balanced_ranges, reduce_shard_gradient
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    o, y0, rki, night, lam = _adjoint_case()
    c0, c1 = balanced_ranges(np.ones(y0.shape[1]), world)[rank]
    gk = _logk_grad(o, np.ascontiguousarray(y0[:, c0:c1]), np.ascontiguousarray(rki[:, c0:c1]),
                    np.ascontiguousarray(night[c0:c1]), np.ascontiguousarray(lam[:, c0:c1]))
    t = torch.from_numpy(gk.copy())
    out = reduce_shard_gradient(t)
    assert out is t
    if rank == 0:
        out_q.put(t.numpy().copy())
    dist.destroy_process_group()


def test_two_rank_logk_gradient_sum_matches_single_domain():
    import multiprocessing as mp
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_grad_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    summed = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ref = _logk_grad(*_adjoint_case())
    assert np.abs(ref).max() > 0
    # the sum over cells is taken in another order (per shard, then over ranks)
    np.testing.assert_allclose(summed, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_reduce_shard_gradient_is_identity_without_a_group():
    import torch
    from cmaq_gb300.partition import reduce_shard_gradient
    t = torch.arange(5, dtype=torch.float64)
    assert reduce_shard_gradient(t) is t and t.tolist() == [0, 1, 2, 3, 4]
    assert reduce_shard_gradient(None) is None
