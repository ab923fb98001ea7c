"""Host-side work partitioning across GPUs (one process per GPU).

CMAQ decomposes the horizontal domain into NPCOL x NPROW subdomains, one MPI rank
each (CCTM/scripts/run_cctm_Bench_2018_12NE3_CB6R5.csh:87-91; STENEX/se), and the
gas chemistry of a rank touches only its own cells (no MPI call under
CCTM/src/gas).  The same holds here: a rank integrates its subdomain and nothing
is exchanged, so the split changes no per-cell result.

* :func:`subdomain` -- the column/row ranges of a rank in an NPCOL x NPROW split,
  remainders going to the leading subdomains.
* :func:`balanced_ranges` -- contiguous cell ranges of near-equal cost from per-cell
  costs (e.g. the previous call's step attempts), for uneven stiffness.
* :func:`reduce_shard_gradient` -- the one exchange of a sharded run: the gradient of a
  parameter every rank shares (the adjoint window's per-reaction log rate multipliers, or
  a scalar loss) summed over the ranks.
"""
from __future__ import annotations

import numpy as np


def _split(n: int, parts: int, i: int) -> tuple[int, int]:
    base, rem = divmod(n, parts)
    lo = i * base + min(i, rem)
    return lo, lo + base + (1 if i < rem else 0)


def subdomain(ncols: int, nrows: int, npcol: int, nprow: int, rank: int) -> tuple[slice, slice]:
    """(col slice, row slice) of `rank`; ranks run fastest along columns."""
    if npcol < 1 or nprow < 1 or not 0 <= rank < npcol * nprow:
        raise ValueError("bad decomposition")
    if npcol > ncols or nprow > nrows:
        raise ValueError("more subdomains than columns or rows")
    pc, pr = rank % npcol, rank // npcol
    c0, c1 = _split(ncols, npcol, pc)
    r0, r1 = _split(nrows, nprow, pr)
    return slice(c0, c1), slice(r0, r1)


def balanced_ranges(costs, parts: int) -> list[tuple[int, int]]:
    """Split cells 0..n-1 into `parts` contiguous ranges of near-equal summed cost."""
    c = np.asarray(costs, dtype=np.float64)
    n = len(c)
    if parts < 1:
        raise ValueError("parts must be >= 1")
    cum = np.concatenate([[0.0], np.cumsum(np.maximum(c, 0.0))])
    total = cum[-1]
    bounds = [0]
    for k in range(1, parts):
        target = total * k / parts
        b = int(np.searchsorted(cum, target, side="left"))
        bounds.append(min(max(b, bounds[-1]), n))
    bounds.append(n)
    return [(bounds[i], bounds[i + 1]) for i in range(parts)]


def sub_grid(g, cols: slice, rows: slice):
    """GridInputs restricted to a horizontal subdomain (all layers)."""
    from dataclasses import replace
    return replace(g, ncols=cols.stop - cols.start, nrows=rows.stop - rows.start,
                   conc=np.ascontiguousarray(g.conc[:, :, rows, cols]),
                   ta=np.ascontiguousarray(g.ta[:, rows, cols]), qv=np.ascontiguousarray(g.qv[:, rows, cols]),
                   dens=np.ascontiguousarray(g.dens[:, rows, cols]), pres=np.ascontiguousarray(g.pres[:, rows, cols]),
                   seaice=np.ascontiguousarray(g.seaice[rows, cols]),
                   ocean_szone=np.ascontiguousarray(g.ocean_szone[rows, cols]),
                   rj=np.ascontiguousarray(g.rj[:, :, rows, cols]),
                   khetero=np.ascontiguousarray(g.khetero[:, rows, cols, :]))


def reduce_shard_gradient(grad, group=None):
    """Sum, over the ranks of ``group``, of a gradient that every rank computed for its own
    cells; in place, and returned.  A parameter shared by all cells (``log_k`` of the
    adjoint window) gets one contribution per cell, so the whole domain's gradient is the
    sum of the subdomains'.  One all-reduce of the flat tensor (349 doubles for CB6r5's
    log-k, 531 for CRACMM2's) on the tensor's device: NCCL for GPU tensors, gloo for CPU
    ones.  Without an initialised process group, or with one rank, it returns ``grad``."""
    import torch.distributed as dist
    if grad is None or not dist.is_available() or not dist.is_initialized():
        return grad
    if dist.get_world_size(group) == 1:
        return grad
    if not grad.is_contiguous():
        raise ValueError("reduce_shard_gradient: the gradient must be contiguous")
    dist.all_reduce(grad, op=dist.ReduceOp.SUM, group=group)
    return grad
