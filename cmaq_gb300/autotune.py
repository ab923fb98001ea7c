"""Autotuner for the batched (work-queue) chemistry kernel.

The reference tunes its CPU chemistry by hand: BLKSIZE, the cells per vectorised
block (rbdriver.F:140-141; CCTM/src/gas/ros3/rbdata_mod.F).  On the GPU the
launch shape matters instead, and the best one depends on the mechanism (code
size, registers) and on the grid's stiffness mix.  The tuner times a few CHEM calls
of a sample of the grid for each candidate:

* cells per block: 64, 128 or 256 (``block_warps`` 2, 4, 8; one cell per thread);
* register cap and prefetch: library variants of ``cmaq_gb300.build`` (the default
  library caps the generated functions at 80 registers for 24 warps per SM and
  prefetches workspace rows; ``w16`` 128 registers and 16 warps; ``g168`` 168 registers
  and 12 warps; ``nopf`` 168 without the prefetch; ``full255`` no cap (8 warps);
  ``r168`` caps every function);
* queue granularity: whether the block's warps pass barriers between the phases of
  each step attempt (``lockstep`` 1), also between the generated chunks of the LU
  and the solves (2), or run free (0, 256-cell blocks only); a lane always refills
  from the queue as soon as its cell finishes.

Results are cached as JSON keyed by mechanism, GPU name and grid size, so later runs
on the same machine reuse them.  Every candidate computes bit-identical results (the
schedule changes no arithmetic), so the choice affects speed only.
"""
from __future__ import annotations

import json
import time
from dataclasses import asdict, dataclass
from pathlib import Path

import numpy as np

from .chem import ChemSolver

KEYS = ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")


@dataclass(frozen=True)
class Candidate:
    variant: str = "default"
    lockstep: int = 1
    block_warps: int = 4

    def knobs(self) -> dict:
        # block size first: every (lockstep, block_warps) pair is reachable from the defaults
        return {"block_warps": self.block_warps, "lockstep": self.lockstep}


def candidates(variants=("default", "w16", "g168", "nopf", "full255", "r168")) -> list[Candidate]:
    out = []
    for v in variants:
        out.append(Candidate(v, 0, 8))
        for ls in (1, 2):
            for bw in (2, 4, 8):
                out.append(Candidate(v, ls, bw))
    return out


def available_variants(build_missing: bool = False) -> list[str]:
    """Built library variants (the default library always; others if built)."""
    from . import build as cbuild
    have = []
    for v in cbuild.VARIANTS:
        if v in ("lucs", "pf255", "r128"):
            continue
        if cbuild.lib_path(v).exists():
            have.append(v)
        elif build_missing:
            cbuild.build(variant=v)
            have.append(v)
    return have


def cache_key(mechanism: str, ncell: int) -> str:
    import torch
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    bucket = 1 << max(0, int(ncell).bit_length() - 1)     # power-of-two bucket of the grid size
    return f"{mechanism}|{name}|{bucket}"


def _time_candidate(g, cand: Candidate, nsteps: int, dev: dict, conc0) -> float:
    s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                   cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, schedule="queue", variant=cand.variant)
    try:
        s.set_tuning(**cand.knobs())
        args = [dev[k] for k in KEYS]
        dev["conc"].copy_(conc0)
        s.step(*args)                    # first call from the initial state; gives the queue order
        dev["conc"].copy_(conc0)
        ms = 0.0
        for _ in range(nsteps):
            ms += s.step(*args)["device_ms"]
        return ms
    finally:
        s.close()


def tune(g, nsteps: int = 2, variants=None, cache: str | Path | None = None, verbose: bool = False) -> dict:
    """Time every candidate on grid ``g`` (GridInputs); returns the best as a dict
    {variant, lockstep, block_warps, ms, table}.  With ``cache``, a stored result for
    the same key is returned without timing, and a new one is stored."""
    import torch
    key = cache_key(g.mech, g.ncell)
    path = Path(cache) if cache else None
    db = {}
    if path and path.exists():
        db = json.loads(path.read_text())
        if key in db:
            return db[key]
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).cuda() for k in KEYS}
    conc0 = dev["conc"].clone()
    table = []
    for cand in candidates(tuple(variants or available_variants())):
        t0 = time.perf_counter()
        ms = _time_candidate(g, cand, nsteps, dev, conc0)
        table.append({**asdict(cand), "ms": ms})
        if verbose:
            print(f"autotune {cand}: {ms:.1f} ms ({time.perf_counter() - t0:.1f} s)", flush=True)
    best = min(table, key=lambda r: r["ms"])
    res = {**best, "nsteps": nsteps, "cells": g.ncell, "table": table}
    if path:
        db[key] = res
        path.write_text(json.dumps(db, indent=1))
    return res


def tuned_solver(g, result: dict, **kw) -> ChemSolver:
    """A queue-scheduled ChemSolver for grid ``g`` with the tuned variant and knobs."""
    s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd, cgrid_index=g.cgrid_index,
                   schedule="queue", variant=result["variant"], **kw)
    s.set_tuning(block_warps=result["block_warps"], lockstep=result["lockstep"])
    return s


def sweep(g, specs, ncalls: int = 12, reps: int = 2, verbose: bool = True) -> dict:
    """Launch-shape sweep: for each spec "variant:block_warps:lockstep:rconst_pass" (later
    fields optional; defaults 8, 1, 1) the device time of ``ncalls`` graph-replayed CHEM
    calls of grid ``g`` after one call from the initial state (the queue history is then
    cleared, so every spec starts from the same queue order), ``reps`` times, with the
    FP64 rate and whether the final concentrations equal the first spec's bit for bit."""
    import torch
    from . import _lib
    info, _ = _lib.mech_info(g.mech)
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).cuda() for k in KEYS}
    conc0 = dev["conc"].clone()
    args = [dev[k] for k in KEYS]
    ref, out = None, {}
    for rep in range(reps):
        for spec in specs:
            f = spec.split(":")
            knobs = dict(zip(("block_warps", "lockstep", "rconst_pass"), (int(x) for x in f[1:])))
            knobs = {"block_warps": 8, "lockstep": 1, "rconst_pass": 1, **knobs}
            s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                           cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, schedule="queue", variant=f[0])
            try:
                s.set_tuning(**knobs)
                dev["conc"].copy_(conc0)
                s.steps(1, *args)
                dev["conc"].copy_(conc0)
                s.set_tuning(queue_history=0)
                st = s.steps(ncalls, *args)
                torch.cuda.synchronize()
            finally:
                s.close()
            conc = dev["conc"].cpu().numpy()
            ref = conc.copy() if ref is None else ref
            att = st["accepted_steps"] + st["rejected_steps"]
            sun = st["sunlit_attempts"]
            tf = (sun * info.flops_step_day + (att - sun) * info.flops_step_night) / (st["device_ms"] * 1e-3) / 1e12
            r = {"ms": st["device_ms"], "tflops": tf, "same_bits": bool(np.array_equal(conc, ref)),
                 "attempts_per_cell_and_call": att / g.ncell / ncalls}
            out.setdefault(spec, []).append(r)
            if verbose:
                print(f"rep {rep} {spec}: {r['ms']:.0f} ms for {ncalls} calls, {r['tflops']:.4f} TFLOP/s, "
                      f"{r['attempts_per_cell_and_call']:.2f} attempts/cell/call, same bits: {r['same_bits']}",
                      flush=True)
    return out


if __name__ == "__main__":
    import argparse
    from . import build as cbuild
    from .synthetic import make_grid
    ap = argparse.ArgumentParser(description="launch-shape sweep of the batched ROS3 kernel (see sweep())")
    ap.add_argument("specs", help="comma-separated variant:block_warps:lockstep:rconst_pass")
    ap.add_argument("--grid", default="459x299x8", help="COLSxROWSxLAYS of the seeded grid")
    ap.add_argument("--mech", default="cb6r5_ae7_aq")
    ap.add_argument("--calls", type=int, default=12)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    specs = a.specs.split(",")
    for v in dict.fromkeys(sp.split(":")[0] for sp in specs):
        cbuild.build(variant=v)
    nc, nr, nl = map(int, a.grid.split("x"))
    sweep(make_grid(mech=a.mech, ncols=nc, nrows=nr, nlays=nl, seed=2018), specs, a.calls, a.reps)

