"""Multi-process path on CPU: subdomain split over 2 gloo ranks changes no per-cell result."""
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
