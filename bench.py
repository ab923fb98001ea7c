"""Benchmark: ROS3 CB6r5 grid-cells/s per 1-h chemistry step on GB300.

One step = one CHEM call (a 5-min synchronisation step) over the whole grid; a
1-hour chemistry step is 12 of them, so

    value = cells / (12 * seconds per step)     [grid-cells/s per 1-h chem step]

timed over K consecutive steps from the seeded initial state (K = 12 by default:
exactly the first simulated hour).  Workload: cb6r5_ae7_aq on the CONUS-size grid
459 x 299 x 35 (4,803,315 cells), rtol 1e-3, atol 1e-9 ppmV, FP64, seeded
synthetic inputs (cmaq_gb300/synthetic.py); CGRID (4 GB) is larger than L2, so no
L2 flush is needed between steps.

Arms and extras
* gb300 (default): the batched persistent kernel (work queue ordered by previous
  step counts, launch shape autotuned on a 4-layer slice of the grid, the K calls
  replayed from one captured CUDA graph) on device-resident arrays -> ``value``; the
  plain per-cell kernel on the same steps -> ``plain``; the host-pointer C ABI with
  copies inside the timed region -> ``e2e``; the FP64 roofline of the solver kernel;
  a bounded CPU sample of the reference algorithm (the C oracle, BLKSIZE 50 with the
  stiffness reordering) on the host cores -> ``cpu_baseline``; the differentiable
  1-hour window on 100x100x35 cells (forward and discrete-adjoint times) ->
  ``adjoint``; EBI on the workload grid -> ``ebi``; SMVGEAR against ROS3 on 100x100x10
  cells -> ``gear``; the accuracy block (GPU hour against the oracle's tight solution
  on a sample of cells) -> ``accuracy``; the KMT2 aqueous kinetics on 200,000 cloudy
  cells -> ``aqchem``; HETCHEM_RATES on the workload grid -> ``hetchem`` (CRACMM2's on
  1,000,000 cells -> ``hetchem.cracmm2``); the CONUS grid
  with skewed stiffness (30 % plume columns), batched against plain -> ``skewed``;
  CRACMM2 on 200x200x25 cells, batched hour and adjoint window -> ``cracmm2``; the
  tight-tolerance timing leg (rtol 3e-7 on every 7th layer, --tight-steps calls) ->
  ``tight``.  The whole default run takes about half an hour.
* --impl reference: the reference algorithm (C oracle; the Fortran cannot be
  compiled here) on all host cores, bounded sample per step.
* --only-hetchem: HETCHEM_RATES alone (cmaqchem_hetchem_rates_device) on the workload
  grid's cells, its own line: cells/s, HBM roofline, end to end, the oracle on a sample.
* --only-aqchem: the KMT2 aqueous kinetics kernel alone (cmaqchem_kmt2_solve_device) on
  --aqchem-cells seeded cloudy cells per call, with its own line: cells/s, FP64
  roofline, end to end through pinned host memory, the C oracle on a host sample and a
  parity summary of that sample.

Multi-GPU (torchrun): every rank integrates its own grid of the same size (CMAQ
gives each process its own subdomain; chemistry exchanges nothing), timing is the
max over ranks and ``value`` counts all ranks' cells: weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "ROS3 CB6r5 grid-cells/s per 1-h chem step"
UNIT = "grid-cells/s per 1-h chem step"
RTOL, ATOL = 1.0e-3, 1.0e-9
# tight tolerance of the accuracy block and its timing leg (DTMIN lowered to 1e-14 min)
TIGHT_RTOL, TIGHT_ATOL = 3.0e-7, 1.0e-16
TSTEP = (10000, 500, 500)          # TSTEP(3) HHMMSS: output 1 h, sync 5 min
STEPS_PER_HOUR = 12

WORKLOADS = {
    "conus": dict(ncols=459, nrows=299, nlays=35),
    "conus_skewed": dict(ncols=459, nrows=299, nlays=35, plume_fraction=0.3),
    "small": dict(ncols=100, nrows=100, nlays=10),
    "conus4": dict(ncols=459, nrows=299, nlays=4),   # a 4-layer slice of the CONUS grid (profiling)
    "cpu4k": dict(ncols=20, nrows=20, nlays=10),
}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            import tempfile
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, busy, smax, reasons = [], [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            try:
                if len(p) > 9 and float(p[9]) >= 50.0:
                    busy.append(sm[-1])
            except ValueError:
                pass
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        # the median over samples with the GPU busy (utilization >= 50 %), else over all
        use = busy if busy else sm
        return {"sm_mhz": statistics.median(use) if use else None, "sm_max_mhz": smax, "samples": len(sm),
                "samples_under_load": len(busy), "reasons": sorted(reasons)}


def make_inputs(workload: str, seed: int):
    from cmaq_gb300.synthetic import make_grid
    return make_grid(seed=seed, **WORKLOADS[workload])


def flops_of(st: dict, info) -> float:
    att = st["accepted_steps"] + st["rejected_steps"]
    sun = st["sunlit_attempts"]
    return sun * info.flops_step_day + (att - sun) * info.flops_step_night


def run_device(g, schedule: str, steps: int, warmup: int, dist, device: int, sample_clocks: bool,
               tuned: dict | None = None, graph: bool = False, solver: str = "ros3", rtol: float = RTOL,
               atol: float = ATOL, dtmin_exp: int | None = None):
    """K timed CHEM calls on device-resident arrays from the initial state.  graph: the K
    calls are replayed from one captured CUDA graph (cmaqchem_steps_device), as three
    replays (the first call, the rest of the first hour, the calls after it) whose
    statistics are kept apart.  The warm-up calls repeat the first call; the work queue's
    step-count history is cleared after them, so the timed first call is queued as a fresh
    run's first call (grid order), and later calls by the previous call's step counts."""
    import torch
    from cmaq_gb300.chem import ChemSolver
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).to(f"cuda:{device}")
           for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")}
    conc0 = dev["conc"].clone()
    s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd, cgrid_index=g.cgrid_index,
                   rtol=rtol, atol=atol, schedule=schedule, device=device, solver=solver,
                   variant=(tuned or {}).get("variant", "default"))
    if tuned:
        s.set_tuning(block_warps=tuned["block_warps"], lockstep=tuned["lockstep"])
    if dtmin_exp is not None:
        s.set_tuning(ros3_dtmin_exp=dtmin_exp)
    stream = torch.cuda.current_stream(device)
    args = [dev[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")]
    # every warm-up step is the hour's first CHEM call from the initial state, so the queue
    # order the timed hour starts from comes from the same call
    for _ in range(warmup):
        dev["conc"].copy_(conc0)
        if graph:
            s.steps(1, *args, tstep=TSTEP, stream=stream)   # also captures the graph
        else:
            s.step(*args, tstep=TSTEP, stream=stream)
    dev["conc"].copy_(conc0)
    if schedule == "queue":
        s.set_tuning(queue_history=0)
    torch.cuda.synchronize(device)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    parts = [n for n in (1, min(steps, STEPS_PER_HOUR) - 1, steps - STEPS_PER_HOUR) if n > 0]
    clocks = ClockSampler(device) if sample_clocks else None
    if clocks:
        clocks.__enter__()
    barrier(dist)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    ev0.record(stream)
    if graph:
        for n in parts:
            stats.append(s.steps(n, *args, tstep=TSTEP, stream=stream))
    else:
        for _ in range(steps):
            stats.append(s.step(*args, tstep=TSTEP, stream=stream))
    ev1.record(stream)
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - t0
    barrier(dist)
    if clocks:
        clocks.__exit__()
    ms = ev0.elapsed_time(ev1)
    s.close()
    del dev, conc0
    torch.cuda.empty_cache()
    return {"ms_total": ms, "wall_s": wall, "stats": stats, "calls": parts if graph else [1] * steps,
            "clocks": clocks.summary() if clocks else None}


def split_calls(r: dict, ncell: int) -> dict:
    """First call and first hour of a run_device result: device time and step attempts."""
    out, done, ms, att = {}, 0, 0.0, 0
    for n, st in zip(r["calls"], r["stats"]):
        done += n
        ms += st["device_ms"]
        att += st["accepted_steps"] + st["rejected_steps"]
        if done == 1:
            out["first_call_ms"] = ms
            out["first_call_attempts_per_cell"] = att / ncell
        if done == STEPS_PER_HOUR:
            out["first_hour"] = {"value": ncell / (ms * 1e-3), "ms_per_step": ms / done,
                                 "step_attempts_per_cell": att / ncell / done}
    return out


FP64_SHAPES = [(0, 8, 256, 8), (0, 16, 256, 4), (0, 4, 256, 8), (0, 1, 1024, 2), (0, 8, 128, 2),
               (0, 8, 32, 4), (1, 8, 256, 8), (2, 8, 256, 8)]   # (op, chains, threads, blocks per SM)


def fp64_peak_record(device: int) -> dict:
    """The FP64 roofline's denominator: (1) independent FMA chains on every SM for about a
    second, three times, with the SM clock sampled meanwhile (best TFLOP/s); (2) the FP64
    pipe's rate in lane operations per clock per SM over a sweep of kernel shapes (1-16
    chains per thread, 4-64 warps per SM, fma / mul / add), whose saturated value times 2 FLOP
    x SMs x the timed region's SM clock is the clock-derived peak; (3) for reference, the rate
    a one-warp clock64 probe implies (one FP64 warp instruction per 64 cycles per SM
    sub-partition: 4 x 32 / 64 = 2 per clock per SM), which no kernel shape reaches."""
    import torch
    from cmaq_gb300 import _lib
    nsm = torch.cuda.get_device_properties(device).multi_processor_count
    _lib.fp64_peak(device)
    with ClockSampler(device) as ck:
        runs = [_lib.fp64_peak_long(device, 1000.0) for _ in range(3)]
    c = ck.summary()
    best = max(r[0] for r in runs)
    sweep = {f"op{o}_ch{ch}_t{t}_b{b}": _lib.fp64_rate(device, o, ch, t, b) for o, ch, t, b in FP64_SHAPES}
    return {"measured_tflops": best, "kernel_ms": [r[1] for r in runs], "measured_sm_mhz": c.get("sm_mhz"),
            "measured_clock_samples": c.get("samples_under_load"), "measured_reasons": c.get("reasons"),
            "sms": nsm, "fp64_ops_per_clk_per_sm": sweep,
            "saturated_ops_per_clk_per_sm": max(sweep.values()),
            "measured_fma_per_clk_per_sm": None if not c.get("sm_mhz") else
            best * 1e12 / 2.0 / nsm / (c["sm_mhz"] * 1e6),
            "issue_probe_ops_per_clk_per_sm": 2.0}


def clock_peak(rec: dict, sm_mhz: float | None, per_clk: float | None = None) -> float | None:
    """FP64 ops per clock per SM (default: the saturated rate of the sweep) x 2 FLOP x SMs x
    clock, in TFLOP/s."""
    if not sm_mhz:
        return None
    r = rec["saturated_ops_per_clk_per_sm"] if per_clk is None else per_clk
    return r * 2.0 * rec["sms"] * sm_mhz * 1e6 / 1e12


def run_accuracy(g, device: int, tuned, threads: int, tight_tol=(TIGHT_RTOL, TIGHT_ATOL), col_step: int = 46,
                 row_step: int = 50, lay_step: int = 2) -> dict:
    """Accuracy of the batched GPU kernel after one simulated hour (12 CHEM calls) on a
    sample of the workload grid (every col_step-th column, row_step-th row and lay_step-th
    layer), against the oracle's tight solution (rtol 1e-8, atol 1e-16 ppmV, DTMIN lowered to
    1e-14 min; within 4e-6 of a solution at rtol 1e-9, atol 1e-17 on such a sample), on
    species above 1e-10 ppmV of the REAL(4) CGRID output: at the headline tolerance and at
    the tight one (DTMIN lowered to 1e-14 there too)."""
    import torch
    from cmaq_gb300.chem import ChemSolver
    from cmaq_gb300.synthetic import subgrid
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle
    sub = subgrid(g, col_step, row_step, lay_step)
    o = Oracle(sub.mech)
    t0 = time.perf_counter()
    truth = sub.conc.copy()
    with o.tight():
        for _ in range(STEPS_PER_HOUR):
            truth, tot = o.chem(sub, blksize=1, rtol=1.0e-8, atol=1.0e-16, threads=threads, conc=truth,
                                max_iter=10000000)
            if tot["rc"] != 0:
                return {"error": "the tight oracle solution failed"}
    truth_s = time.perf_counter() - t0
    idx = np.unique(sub.cgrid_index - 1)
    tr = truth[idx].astype(np.float64)
    mask = tr > 1.0e-10

    def gpu_hour(rtol, atol, dtmin_exp):
        dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(sub, k))).to(f"cuda:{device}")
               for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")}
        sv = ChemSolver(sub.mech, ncols=sub.ncols, nrows=sub.nrows, nlays=sub.nlays, nspcsd=sub.nspcsd,
                        cgrid_index=sub.cgrid_index, rtol=rtol, atol=atol, schedule="queue", device=device)
        if tuned:
            sv.set_tuning(block_warps=tuned["block_warps"], lockstep=tuned["lockstep"])
        if dtmin_exp is not None:
            sv.set_tuning(ros3_dtmin_exp=dtmin_exp)
        failed = 0
        for _ in range(STEPS_PER_HOUR):
            failed += sv.step(*[dev[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj",
                                                 "khetero")], tstep=TSTEP)["failed_cells"]
        sv.close()
        got = dev["conc"].cpu().numpy()[idx].astype(np.float64)
        rel = np.abs(got[mask] - tr[mask]) / tr[mask]
        return {"rtol": rtol, "atol": atol, "max": float(rel.max()), "p99_9": float(np.quantile(rel, 0.999)),
                "median": float(np.median(rel)), "failed_cells": int(failed)}

    return {"sample": f"{sub.ncols}x{sub.nrows}x{sub.nlays} ({sub.ncell} cells): every {col_step}th column, "
                      f"{row_step}th row and {lay_step}th layer of the workload grid",
            "truth": "oracle (ROS3 per cell) rtol 1e-8, atol 1e-16 ppmV, DTMIN 1e-14 min",
            "species": f"CGRID species above 1e-10 ppmV after the hour ({int(mask.sum())} values)",
            "truth_s": truth_s, "headline": gpu_hour(RTOL, ATOL, None),
            "tight": dict(gpu_hour(tight_tol[0], tight_tol[1], -14), dtmin_min=1.0e-14)}


def run_e2e(g, steps: int, warmup: int, dist, device: int):
    """Same hour through the host-pointer C ABI (cmaqchem_step): every call copies CGRID, met,
    photolysis and heterogeneous rates host->device and CGRID device->host."""
    import torch
    from cmaq_gb300.chem import ChemSolver

    def pinned(a):
        t = torch.empty(a.shape, dtype={np.float32: torch.float32, np.float64: torch.float64}[a.dtype.type],
                        pin_memory=True)
        t.numpy()[...] = a
        return t.numpy()

    h = {k: pinned(np.ascontiguousarray(getattr(g, k)))
         for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")}
    conc0 = h["conc"].copy()
    s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd, cgrid_index=g.cgrid_index,
                   rtol=RTOL, atol=ATOL, schedule="queue", device=device)
    args = [h[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")]
    for _ in range(warmup):
        h["conc"][...] = conc0
        s.step(*args, tstep=TSTEP)
    h["conc"][...] = conc0
    s.set_tuning(queue_history=0)        # the timed first call is queued as a fresh run's
    # the call copies the mechanism's CGRID planes (not all NSPCSD) and the other inputs
    plane = h["conc"].nbytes // g.nspcsd
    nplanes = len(set(int(c) for c in g.cgrid_index))
    h2d = nplanes * plane + sum(a.nbytes for a in args[1:])
    d2h = nplanes * plane
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(steps):
        s.step(*args, tstep=TSTEP)
    wall = time.perf_counter() - t0
    barrier(dist)
    s.close()
    return {"wall_s": wall, "h2d": h2d, "d2h": d2h}


def run_autotune(workload: str, seed: int, device: int) -> dict:
    """Launch-shape autotuning on a layer slice of the workload grid (same columns and
    distributions, 4 layers), 2 timed CHEM calls per candidate, over the default library
    (80 registers, 24 warps per SM) and the w16 build (128 registers, 16 warps), which is
    built here if missing."""
    from cmaq_gb300 import build as cbuild
    from cmaq_gb300.autotune import tune
    from cmaq_gb300.synthetic import make_grid
    dims = dict(WORKLOADS[workload])
    dims["nlays"] = min(4, dims["nlays"])
    g = make_grid(seed=seed, **dims)
    t0 = time.perf_counter()
    variants = ["default"]
    try:
        cbuild.build(variant="w16")
        variants.append("w16")
    except Exception as e:   # no nvcc: the default library alone
        print(f"[bench] w16 build skipped: {e}", file=sys.stderr)
    res = tune(g, nsteps=2, variants=variants)
    res["tuning_s"] = time.perf_counter() - t0
    res["sample"] = f"{g.ncols}x{g.nrows}x{g.nlays} ({g.ncell} cells)"
    return res


def run_adjoint(device: int, nsync: int = STEPS_PER_HOUR, dims=(100, 100, 35)) -> dict:
    """The differentiable 1-hour window on 100x100x35 cells: forward (checkpointed) and
    backward (discrete adjoint) of L = sum of surface O3 wrt initial concentrations,
    per-reaction log rate multipliers and emission tendencies."""
    import torch
    from cmaq_gb300.adjoint import Ros3Window
    from cmaq_gb300.chem import ChemSolver
    from cmaq_gb300.synthetic import make_grid, manifest, solver_inputs
    g = make_grid(seed=2018, ncols=dims[0], nrows=dims[1], nlays=dims[2])
    gs = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                    cgrid_index=g.cgrid_index, rtol=RTOL, atol=ATOL, device=device)
    y0, rki, night = solver_inputs(g, gs)
    gs.close()
    n = g.ncell
    s = ChemSolver(g.mech, ncols=n, nrows=1, nlays=1, nspcsd=g.nspcsd, rtol=RTOL, atol=ATOL, device=device)
    names = [sp["name"] for sp in manifest(g.mech)["species"]]
    io3 = s.iold2new[names.index("O3")]
    nsurf = g.ncols * g.nrows
    w = Ros3Window(s, rki, night, nsync, 5.0)
    logk = torch.zeros(s.info.nrxns, dtype=torch.float64, device=y0.device, requires_grad=True)
    emis = torch.zeros_like(y0).requires_grad_(True)
    times = []
    for rep in range(2):                                   # the first pass is the warm-up
        a = y0.clone().requires_grad_(True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize(device)
        e0.record()
        y = w(a, logk, emis)
        e1.record()
        y[io3, :nsurf].sum().backward()
        e2.record()
        torch.cuda.synchronize(device)
        times.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
        logk.grad = None
        emis.grad = None
    fwd, bwd = times[-1]
    s.close()
    del w, a, y, emis, logk, y0, rki, night
    torch.cuda.empty_cache()
    # the same cells' hour through the batched CHEM kernel (no tape): the forward a user
    # would run without gradients
    b = run_device(g, "queue", nsync, 1, None, device, sample_clocks=False, graph=True)
    bfwd = b["ms_total"]
    return {"workload": f"cb6r5_ae7_aq {dims[0]}x{dims[1]}x{dims[2]} ({n} cells), {nsync} x 5-min steps, solver level "
                        "(rates from CALC_RCONST of the grid, fixed over the hour)",
            "loss": "sum of O3 over the surface layer at the end of the hour",
            "gradients": "initial concentrations, 349 log rate multipliers, emission tendencies",
            "forward_ms": fwd, "backward_ms": bwd, "backward_over_forward": bwd / fwd,
            "total_over_forward": (fwd + bwd) / fwd,
            "batched_forward_ms": bfwd, "total_over_batched_forward": (fwd + bwd) / bfwd,
            "forward_note": "forward_ms records the tape (accepted steps' states and sizes); batched_forward_ms is "
                            "the same cells' hour through the batched CHEM kernel without a tape"}


def run_skewed(device: int, steps: int, tuned) -> dict:
    """Config with skewed stiffness: the CONUS grid with 10x NOx/VOC plumes in 30 % of the
    columns; batched (tuned, graph-replayed) against the plain per-cell kernel."""
    from cmaq_gb300.synthetic import make_grid
    g = make_grid(seed=2018, **WORKLOADS["conus_skewed"])
    b = run_device(g, "queue", steps, 1, None, device, sample_clocks=False, tuned=tuned, graph=True)
    p = run_device(g, "static", steps, 1, None, device, sample_clocks=False)
    bv = g.ncell / (STEPS_PER_HOUR * b["ms_total"] / steps / 1e3)
    pv = g.ncell / (STEPS_PER_HOUR * p["ms_total"] / steps / 1e3)
    att = sum(st["accepted_steps"] + st["rejected_steps"] for st in b["stats"]) / g.ncell / steps
    return {"workload": f"cb6r5_ae7_aq {g.ncols}x{g.nrows}x{g.nlays} ({g.ncell} cells), 30 % of columns with "
                        f"10x NOx/VOC, {steps} x 5-min CHEM calls from the initial state",
            "batched_value": bv, "plain_value": pv, "batched_over_plain": bv / pv,
            "step_attempts_per_cell": att}


def run_tight(g, device: int, steps: int, tuned, info, tol, peak_rec, lay_step: int = 7) -> dict:
    """The tight tolerance of the accuracy block (DTMIN lowered to 1e-14 min) on every
    lay_step-th layer of the workload grid (all columns and rows; a step there costs about
    25 times one at the headline tolerance): batched (graph-replayed) and plain, the first
    `steps` calls from the initial state without warm-up calls, with the batched kernel's
    FP64 rate."""
    from cmaq_gb300.synthetic import subgrid
    g = subgrid(g, 1, 1, lay_step)
    b = run_device(g, "queue", steps, 0, None, device, sample_clocks=True, tuned=tuned, graph=True,
                   rtol=tol[0], atol=tol[1], dtmin_exp=-14)
    p = run_device(g, "static", steps, 0, None, device, sample_clocks=False, rtol=tol[0], atol=tol[1],
                   dtmin_exp=-14)
    bv = g.ncell / (STEPS_PER_HOUR * b["ms_total"] / steps / 1e3)
    pv = g.ncell / (STEPS_PER_HOUR * p["ms_total"] / steps / 1e3)
    fl = sum(flops_of(st, info) for st in b["stats"])
    dev_ms = sum(st["device_ms"] for st in b["stats"])
    ach = fl / (dev_ms * 1e-3) / 1e12
    cp = clock_peak(peak_rec, (b["clocks"] or {}).get("sm_mhz"))
    peak = max(x for x in (peak_rec["measured_tflops"], cp) if x)
    att = sum(st["accepted_steps"] + st["rejected_steps"] for st in b["stats"]) / g.ncell / steps
    return {"workload": f"cb6r5_ae7_aq {g.ncols}x{g.nrows}x{g.nlays} ({g.ncell} cells: every {lay_step}th layer of "
                        f"the workload grid), the hour's first {steps} x 5-min CHEM calls, rtol {tol[0]:g}, "
                        f"atol {tol[1]:g} ppmV, DTMIN 1e-14 min, no warm-up call",
            "batched_value": bv, "plain_value": pv, "batched_over_plain": bv / pv,
            "step_attempts_per_cell": att, "achieved_tflops": ach, "roofline_frac": ach / peak,
            "failed_cells": int(sum(st["failed_cells"] for st in b["stats"])), "clocks": b["clocks"]}


def run_cracmm2(device: int, steps: int) -> dict:
    """The larger mechanism on 200x200x25 cells: batched CHEM hour, then the differentiable
    window (forward with checkpoints, backward) on the same grid within a 180 GB budget."""
    import torch
    from cmaq_gb300.adjoint import Ros3Window
    from cmaq_gb300.chem import ChemSolver
    from cmaq_gb300.synthetic import make_grid, manifest, solver_inputs
    g = make_grid(mech="cracmm2", seed=2018, ncols=200, nrows=200, nlays=25)
    b = run_device(g, "queue", steps, 1, None, device, sample_clocks=False, graph=True)
    out = {"workload": f"cracmm2 200x200x25 ({g.ncell} cells), {steps} x 5-min calls",
           "batched_value": g.ncell / (STEPS_PER_HOUR * b["ms_total"] / steps / 1e3),
           "batched_ms_per_step": b["ms_total"] / steps}
    gs = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                    cgrid_index=g.cgrid_index, rtol=RTOL, atol=ATOL, device=device)
    y0, rki, night = solver_inputs(g, gs)
    gs.close()
    n = g.ncell
    s = ChemSolver(g.mech, ncols=n, nrows=1, nlays=1, nspcsd=g.nspcsd, rtol=RTOL, atol=ATOL, device=device)
    ckpt = steps * s.info.ischan * n * 8
    budget = 180 << 30
    tape_mb = max(1024, (budget - ckpt - (16 << 30)) >> 20)   # 16 GB for inputs, gradients, workspaces
    s.set_tuning(adjoint_tape_mb=int(tape_mb))
    names = [sp["name"] for sp in manifest(g.mech)["species"]]
    io3 = s.iold2new[names.index("O3")]
    nsurf = g.ncols * g.nrows
    logk = torch.zeros(s.info.nrxns, dtype=torch.float64, device=y0.device, requires_grad=True)
    emis = torch.zeros_like(y0).requires_grad_(True)
    times = []
    for nsync in (1, steps):      # one-step pass first: allocates the first (largest) step's tape
        w = Ros3Window(s, rki, night, nsync, 5.0)
        a = y0.clone().requires_grad_(True)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize(device)
        e0.record()
        y = w(a, logk, emis)
        e1.record()
        y[io3, :nsurf].sum().backward()
        e2.record()
        torch.cuda.synchronize(device)
        times.append((e0.elapsed_time(e1), e1.elapsed_time(e2)))
        logk.grad = None
        emis.grad = None
    fwd, bwd = times[-1]
    peak = torch.cuda.max_memory_allocated(device)
    s.close()
    out.update({"adjoint_forward_ms": fwd, "adjoint_backward_ms": bwd, "adjoint_backward_over_forward": bwd / fwd,
                "adjoint_total_over_forward": (fwd + bwd) / fwd,
                "adjoint_memory": f"checkpoints {ckpt / 2**30:.1f} GiB, tape budget {tape_mb / 1024:.1f} GiB "
                                  f"(180 GB total budget), torch peak {peak / 2**30:.1f} GiB"})
    return out


def run_ebi(device: int, steps: int, g=None) -> dict:
    """EBI (HRSOLVER) CHEM calls on the workload grid (the CONUS grid of the headline line
    unless g is given), K calls from the initial state; ROS3 on the same grid is the
    headline's batched arm."""
    from cmaq_gb300.synthetic import make_grid
    if g is None:
        g = make_grid(seed=2018, ncols=100, nrows=100, nlays=10)
    r = run_device(g, "queue", steps, 1, None, device, sample_clocks=False, solver="ebi")
    att = sum(st["accepted_steps"] for st in r["stats"]) / g.ncell / steps
    return {"workload": f"cb6r5_ae7_aq {g.ncols}x{g.nrows}x{g.nlays} ({g.ncell} cells), {steps} x 5-min EBI CHEM "
                        "calls from the initial state",
            "ebi_ms_per_step": r["ms_total"] / steps,
            "ebi_value": g.ncell / (STEPS_PER_HOUR * r["ms_total"] / steps / 1e3),
            "ebi_iterations_per_cell_and_call": att, **{"ebi_" + k: v for k, v in split_calls(r, g.ncell).items()}}


def run_gear(device: int, steps: int) -> dict:
    """SMVGEAR against batched ROS3 on one 100x100x10 grid of the same distributions
    (GEAR_RTOL 1e-3, OPTIMAL_ATOL_PPM between 1e-9 and 1e-7 ppmV).  A Gear call lasts as
    long as its stiffest cell (tens of seconds here), so at most 3 calls are timed."""
    from cmaq_gb300.synthetic import make_grid
    steps = min(steps, 3)
    g = make_grid(seed=2018, ncols=100, nrows=100, nlays=10)
    out = {"workload": f"cb6r5_ae7_aq 100x100x10 ({g.ncell} cells), the hour's first {steps} x 5-min CHEM calls"}
    for solver in ("gear", "ros3"):
        r = run_device(g, "queue", steps, 1, None, device, sample_clocks=False, solver=solver)
        out[f"{solver}_ms_per_step"] = r["ms_total"] / steps
        out[f"{solver}_value"] = g.ncell / (STEPS_PER_HOUR * r["ms_total"] / steps / 1e3)
        if solver == "gear":
            out["gear_steps_per_cell"] = sum(st["accepted_steps"] for st in r["stats"]) / g.ncell / steps
            out["gear_failures_per_cell"] = sum(st["rejected_steps"] for st in r["stats"]) / g.ncell / steps
    return out


def aqchem_roofline(r: dict, peak_rec: dict | None) -> dict:
    """FP64 roofline of the KMT2 kernel against the measured FMA-chain rate."""
    pk = None if peak_rec is None else peak_rec["measured_tflops"]
    return {"bound": "fp64", "achieved": r["achieved_tflops"], "peak": pk, "unit": "TFLOP/s",
            "frac": None if not pk else r["achieved_tflops"] / pk, "traffic": None,
            "peak_source": "measured live (cmaqchem_diag_fp64_peak_long)"}


def run_aqchem_whole(dev, ncell: int, steps: int) -> dict:
    """The whole AQCHEM (cmaqchem_aqchem_device: GAS / AEROSOL mapping, kinetic core,
    redistribution) on ncell seeded columns; device time per call by CUDA events."""
    import torch
    from cmaq_gb300.aqchem import aqchem as aqchem_whole
    from cmaq_gb300.synthetic import make_cloud_columns
    cp, cg, ca, cidx, cfac = make_cloud_columns(ncell, seed=2018)
    tp, tg0, ta0 = (torch.from_numpy(np.ascontiguousarray(x.T)).to(dev) for x in (cp, cg, ca))
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms = []
    for rep in range(steps + 1):                      # the first call is the warm-up
        tg, ta = tg0.clone(), ta0.clone()
        ev[0].record()
        _, _, wout, wst = aqchem_whole(tp, tg, ta, cidx, cfac)
        ev[1].record()
        torch.cuda.synchronize(dev)
        if rep:
            ms.append(ev[0].elapsed_time(ev[1]))
    wo = wout.cpu().numpy()
    return {"ms_per_call": float(np.mean(ms)), "value": ncell / (float(np.mean(ms)) * 1e-3),
            "failed_cells": int((wst.cpu().numpy()[8] != 1).sum()),
            "max_abs_mass_balance_percent": float(np.abs(wo[6:10]).max())}


def run_hetchem(device: int, ncell: int, steps: int, threads: int, mech: str = "cb6r5_ae7_aq") -> dict:
    """HETCHEM_RATES (cmaqchem_hetchem_rates_device) of mechanism ``mech``: KHETERO of ncell
    seeded cells from their CGRID aerosol block and met fields (cmaq_gb300/synthetic.py:
    make_aerosol_cells).
    Device time by CUDA events around each call (inputs resident); end to end with the
    aerosol block and met copied from pinned host memory and KHETERO copied back; the HBM
    roofline of the call's algorithmic bytes (the block and met read once, KHETERO written
    once); the oracle on a host sample for the baseline and a parity summary."""
    import torch
    from cmaq_gb300.hetchem import hetchem_rates, layout
    from cmaq_gb300.synthetic import make_aerosol_cells
    nae, _, nhet = layout(mech)
    ae, ta, p, q, d = make_aerosol_cells(ncell, seed=2018, mech=mech)
    dev = torch.device(f"cuda:{device}")
    host = [torch.from_numpy(x).pin_memory() for x in (ae, ta, p, q, d)]
    dv = [x.to(dev) for x in host]
    out = hetchem_rates(*dv, mechanism=mech)
    hout = torch.empty((ncell, nhet), dtype=torch.float64).pin_memory()
    for _ in range(2):
        hetchem_rates(*dv, mechanism=mech, out=out)
    torch.cuda.synchronize(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms = []
    for _ in range(steps):
        ev[0].record()
        hetchem_rates(*dv, mechanism=mech, out=out)
        ev[1].record()
        torch.cuda.synchronize(dev)
        ms.append(ev[0].elapsed_time(ev[1]))
    dev_ms = float(np.median(ms))
    t0 = time.perf_counter()
    for _ in range(steps):
        for hx, dx in zip(host, dv):
            dx.copy_(hx, non_blocking=True)
        hetchem_rates(*dv, mechanism=mech, out=out)
        hout.copy_(out, non_blocking=True)
        torch.cuda.synchronize(dev)
    e2e_s = (time.perf_counter() - t0) / steps
    nbytes = ncell * (nae * 4 + 16 + nhet * 8)
    peak = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"] if (ROOT / "MEASURED_PEAKS.json").exists() else None
    achieved = nbytes / (dev_ms * 1e-3) / 1e9
    res = {"mechanism": mech, "ncell": ncell, "ms_per_call": dev_ms, "value": ncell / (dev_ms * 1e-3),
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": None if not peak else achieved / peak, "traffic": None,
                        "bytes_per_cell": nae * 4 + 16 + nhet * 8,
                        "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy bandwidth)"},
           "e2e": {"value": ncell / e2e_s, "unit": "cells/s",
                   "h2d_bytes_per_step": int(sum(x.numel() * x.element_size() for x in host)),
                   "d2h_bytes_per_step": int(hout.numel() * 8)}}
    if threads > 0:                                   # CPU baseline: the oracle on a sample
        sys.path.insert(0, str(ROOT / "oracle"))
        import hetchem as het_oracle
        nsample = min(ncell, 20000 * threads)
        t0 = time.perf_counter()
        want = het_oracle.rates(ae[:, :nsample], ta[:nsample], p[:nsample], q[:nsample], d[:nsample], threads=threads,
                                mech=mech)
        wall = time.perf_counter() - t0
        got = out[:nsample].cpu().numpy()
        rel = np.where(got == want, 0.0, np.abs(got - want) / np.maximum(np.abs(want), 1e-300))
        switch = [j for j, x in enumerate(het_oracle.tables(mech)["hetero"])
                  if x in ("HETERO_IEPOX", "HETERO_IEPOXOS", "HETERO_TETROL", "HETERO_ISO3NOSJ", "HETERO_ISO3OSJ")]
        rest = np.delete(rel, switch, axis=1)
        res["cpu"] = {"value": nsample / wall, "cells": nsample, "wall_s": wall, "threads": threads}
        res["parity"] = {"cells": nsample, "max_rel_diff_off_switch": float(rest.max()),
                         "cells_on_the_iepox_switch": int((rel[:, switch] > 1e-5).any(axis=1).sum()),
                         "note": "CALCISOPGAMMAS' q / TANH( q ) > 1 switch flips with an ulp of TANH for tiny q"}
    return res


def run_aqchem(device: int, ncell: int, steps: int, warmup: int, threads: int, whole: bool = True) -> dict:
    """KMT2 aqueous kinetics (cmaqchem_kmt2_solve_device): one call integrates ncell seeded
    cloudy cells over their cloud time.  Device time by CUDA events around each call
    (inputs resident); end to end with the inputs copied from pinned host memory and the
    state copied back; FLOPs from the per-cell step counts and the generated routines'
    operation counts (cmaq_gb300/mechs/kmt2/manifest.json); the oracle on a CPU sample
    for the baseline and a parity summary of that sample."""
    import torch
    from cmaq_gb300.aqchem import aqchem_kinetics
    from cmaq_gb300.synthetic import kmt2_manifest, make_cloud_cells
    fl = kmt2_manifest()["flops"]
    p, v = make_cloud_cells(ncell, seed=2018)
    dev = torch.device(f"cuda:{device}")
    hp = torch.from_numpy(np.ascontiguousarray(p.T)).pin_memory()
    hv = torch.from_numpy(np.ascontiguousarray(v.T)).pin_memory()
    hout = torch.empty((161, ncell), dtype=torch.float64).pin_memory()
    pt, vt = hp.to(dev), hv.to(dev)
    for _ in range(warmup):
        out, st = aqchem_kinetics(pt, vt)
    torch.cuda.synchronize(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ms = []
    for _ in range(steps):
        ev[0].record()
        out, st = aqchem_kinetics(pt, vt)
        ev[1].record()
        torch.cuda.synchronize(dev)
        ms.append(ev[0].elapsed_time(ev[1]))
    sd = st.cpu().numpy().astype(np.int64)
    # each routine's operation count times its own counter: f, J, factorisations (with the
    # repeats after a singular one), solves, and the vector work of every attempt
    flops = float(sd[3].sum() * fl["fun"] + sd[4].sum() * fl["jac"] + sd[5].sum() * fl["decomp"]
                  + sd[6].sum() * fl["solve"] + sd[0].sum() * fl["vector"])
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(steps):
        pt.copy_(hp, non_blocking=True)
        vt.copy_(hv, non_blocking=True)
        out, _ = aqchem_kinetics(pt, vt)
        hout.copy_(out, non_blocking=True)
        torch.cuda.synchronize(dev)
    e2e_s = (time.perf_counter() - t0) / steps
    dev_ms = float(np.mean(ms))
    # the whole AQCHEM (GAS / AEROSOL mapping, kinetic core, redistribution) on seeded columns
    res_whole = None
    if whole:
        res_whole = run_aqchem_whole(dev, ncell, steps)
    res = {"ncell": ncell, "ms_per_call": dev_ms, "value": ncell / (dev_ms * 1e-3), "whole_aqchem": res_whole,
           "achieved_tflops": flops / (dev_ms * 1e-3) / 1e12, "flops_per_call": flops,
           "steps_per_cell": float(sd[1].mean()), "max_steps_per_cell": int(sd[1].max()),
           "failed_cells": int((sd[8] != 1).sum()),
           "e2e": {"value": ncell / e2e_s, "unit": "cells/s", "h2d_bytes_per_step": int(hp.numel() + hv.numel()) * 8,
                   "d2h_bytes_per_step": int(hout.numel()) * 8}}
    if threads > 0:                                   # CPU baseline leg: the oracle on a sample
        sys.path.insert(0, str(ROOT / "oracle"))
        from kmt2 import KMT2Oracle
        o = KMT2Oracle()
        nsample = min(ncell, 4000 * threads)             # a few seconds of host time
        t0 = time.perf_counter()
        vr, _, sr, _ = o.cells(p[:nsample], v[:nsample], threads=threads)
        wall = time.perf_counter() - t0
        got = out[:, :nsample].cpu().numpy().T
        same = (sd[:, :nsample].T == sr).all(axis=1)
        big = np.abs(vr) > 1e-6 * np.abs(vr).max(axis=1, keepdims=True)
        rel = np.where(big, np.abs(got - vr) / np.maximum(np.abs(vr), 1e-300), 0.0).max(axis=1)
        res["cpu"] = {"value": nsample / wall, "cells": nsample, "wall_s": wall}
        res["parity"] = {"cells": nsample, "same_steps": float(same.mean()),
                         "bit_equal_cells": float(((got == vr).all(axis=1) & same).mean()),
                         "max_rel": float(rel.max())}
    return res


def barrier(dist):
    if dist is not None:
        import torch.distributed as tdist
        tdist.barrier()


def max_over_ranks(x: float, dist) -> float:
    if dist is None:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([x], dtype=torch.float64, device=dist)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def cpu_reference(workload_cells: int, steps: int, warmup: int, threads: int, target_s: float = 20.0,
                  solver: str = "ros3"):
    """The reference algorithm (C oracle: ROS3 with BLKSIZE 50 and the stiffness reordering,
    or EBI) on host cores, on a sample grid drawn from the same distributions; K calls from
    the initial state after W calls."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import Oracle
    from cmaq_gb300.synthetic import make_grid
    o = Oracle("cb6r5_ae7_aq")
    rt, at = float(np.float32(RTOL)), float(np.float32(ATOL))

    def call(g, conc=None):
        if solver == "ebi":
            return o.chem_ebi(g, threads=threads, conc=conc)
        if solver == "gear":
            return o.chem_gear(g, blksize=50, threads=threads, conc=conc)
        return o.chem(g, blksize=50, rtol=rt, atol=at, threads=threads, conc=conc)
    # size the sample so that the timed calls take about target_s
    ncols = 20
    g = make_grid(ncols=ncols, nrows=10, nlays=10, seed=2018)
    t0 = time.perf_counter()
    c, _ = call(g)
    first = time.perf_counter() - t0
    est_hour = first * 3.0            # later calls are cheaper than the first
    scale = max(1, min(64, int(target_s / max(est_hour, 1e-3))))
    g = make_grid(ncols=ncols * scale, nrows=10, nlays=10, seed=2018)
    conc = g.conc.copy()
    for _ in range(warmup):
        conc, _ = call(g, conc)
    conc = g.conc.copy()
    t0 = time.perf_counter()
    for _ in range(steps):
        conc, _ = call(g, conc)
    wall = time.perf_counter() - t0
    value = g.ncell / (STEPS_PER_HOUR * wall / steps)
    return {"value": value, "cells": g.ncell, "wall_s": wall, "steps": steps}


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=STEPS_PER_HOUR)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="conus", choices=sorted(WORKLOADS))
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-kernel comparison")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-ebi", action="store_true")
    ap.add_argument("--no-gear", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="only the headline arms (batched, plain, e2e, CPU baseline)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the skewed-stiffness CONUS grid and CRACMM2 on 1M cells (about 5 minutes)")
    ap.add_argument("--all-configs", action="store_true", help="accepted for compatibility: the configs run by default")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the accuracy block and the tight-tolerance leg")
    ap.add_argument("--no-aqchem", action="store_true", help="skip the KMT2 aqueous kinetics leg")
    ap.add_argument("--no-hetchem", action="store_true", help="skip the HETCHEM_RATES leg")
    ap.add_argument("--only-hetchem", action="store_true",
                    help="only the HETCHEM_RATES kernel on the workload grid's cells, its own JSON line")
    ap.add_argument("--tight-steps", type=int, default=2,
                    help="CHEM calls of the tight-tolerance leg on every 7th layer of the workload grid "
                         "(0: skip; 2 take about 14 minutes)")
    ap.add_argument("--adjoint-dims", default="100x100x35", help="grid of the adjoint window, NCOLSxNROWSxNLAYS")
    ap.add_argument("--only-adjoint", action="store_true",
                    help="time only the adjoint window and print its own line (for profiling)")
    ap.add_argument("--only-aqchem", action="store_true",
                    help="time only the KMT2 aqueous kinetics kernel and print its own line")
    ap.add_argument("--aqchem-cells", type=int, default=200000, help="cloudy cells per KMT2 call")
    ap.add_argument("--solver", default="ros3", choices=["ros3", "ebi", "gear"],
                    help="solver of the timed CHEM calls (the metric is quoted for ros3)")
    a = ap.parse_args()
    world, rank, local = dist_env()

    if a.impl == "reference":
        if rank != 0:
            return 0
        thr = host_threads()
        r = cpu_reference(0, a.steps, a.warmup, thr, target_s=60.0)
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "impl": "reference", "n_gpus": a.gpus,
                "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * r["wall_s"] / r["steps"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (seeded; cmaq_gb300/synthetic.py)",
                "config": {"workload": f"cb6r5_ae7_aq sample grid {r['cells']} cells (same distributions as "
                                       f"459x299x35), {r['steps']} x 5-min CHEM calls, rtol 1e-3 atol 1e-9",
                           "algorithm": "reference ROS3 (BLKSIZE 50, stiffness reordering) restated in C; "
                                        "the Fortran reference cannot be compiled on this image"},
                "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": thr, "kind": "port",
                                 "sample": f"{r['cells']} cells x {r['steps']} CHEM calls"},
                "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return 0

    import torch
    dist = None
    if world > 1:
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
        dist = torch.device(f"cuda:{local}")
    device = local if world > 1 else 0
    torch.cuda.set_device(device)
    from cmaq_gb300 import _lib
    try:
        _lib.lib()
    except _lib.ChemError:
        from cmaq_gb300 import build as cbuild
        cbuild.build()
        _lib.lib.cache_clear()
    info, _ = _lib.mech_info("cb6r5_ae7_aq")
    adims = tuple(int(x) for x in a.adjoint_dims.split("x"))
    if a.only_adjoint:
        r = run_adjoint(device, a.steps, adims)
        if rank == 0:
            print(json.dumps({"metric": "ROS3 CB6r5 adjoint/forward time", "value": r["backward_over_forward"],
                              "unit": "backward time / forward time", "n_gpus": 1, "steps": a.steps,
                              "warmup": 1, "ms_per_step": (r["forward_ms"] + r["backward_ms"]) / a.steps,
                              "higher_is_better": False, "dtype": "f64", "data": "synthetic", "adjoint": r}))
        return 0
    if a.only_hetchem:
        thr = 0 if (a.no_cpu or rank != 0) else host_threads()
        dims = WORKLOADS[a.workload]
        ncell = dims["ncols"] * dims["nrows"] * dims["nlays"]
        r = run_hetchem(device, ncell, min(a.steps, 5), thr)
        if not a.no_configs:                          # CRACMM2's tables on its 200x200x25 grid
            r["cracmm2"] = run_hetchem(device, 1000000, min(a.steps, 5), min(thr, 4), "cracmm2")
        if rank == 0:
            line = {"metric": "HETCHEM_RATES: grid cells of KHETERO per second", "value": r["value"],
                    "unit": "cells/s", "n_gpus": 1, "steps": min(a.steps, 5), "warmup": 3,
                    "ms_per_step": r["ms_per_call"], "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "f32+f64",
                    "data": "synthetic (seeded; cmaq_gb300/synthetic.py: make_aerosol_cells)",
                    "config": {"workload": f"{ncell} cells ({a.workload} grid), cb6r5_ae7_aq aerosol block "
                                           "(84 rows) and met, 17 KHETERO",
                               "l2": f"inputs of {ncell * 352 / 1e9:.1f} GB per call, larger than the 129 MB L2"},
                    "roofline": r["roofline"], "e2e": r["e2e"], "gpu_launches": min(a.steps, 5), "hetchem": r}
            if "cpu" in r:
                line["cpu_baseline"] = {"value": r["cpu"]["value"], "unit": "cells/s", "cores": r["cpu"]["threads"],
                                        "kind": "port", "sample": f"{r['cpu']['cells']} cells"}
            print(json.dumps(line))
        return 0
    peak_rec = fp64_peak_record(device) if rank == 0 or world == 1 else None
    if a.only_aqchem:
        thr = 0 if (a.no_cpu or rank != 0) else host_threads()
        r = run_aqchem(device, a.aqchem_cells, min(a.steps, 5), max(a.warmup, 3), thr)
        if rank == 0:
            line = {"metric": "KMT2 aqueous chemistry: cloudy cells integrated over their cloud time per second",
                    "value": r["value"], "unit": "cells/s", "n_gpus": 1, "steps": min(a.steps, 5),
                    "warmup": max(a.warmup, 3), "ms_per_step": r["ms_per_call"], "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                    "data": "synthetic (seeded; cmaq_gb300/synthetic.py: make_cloud_cells)",
                    "config": {"workload": f"{r['ncell']} cloudy cells, KMT2 aqueous mechanism "
                                           "(CCTM/src/cloud/acm_ae7_kmt2), TAUCLD 600-3600 s",
                               "l2": f"inputs of {r['ncell'] * 176 * 8 / 1e6:.0f} MB per call, larger than the "
                                     "129 MB L2, plus a 1 GB workspace"},
                    "roofline": aqchem_roofline(r, peak_rec),
                    "e2e": r["e2e"], "gpu_launches": min(a.steps, 5), "aqchem": r}
            if "cpu" in r:
                line["cpu_baseline"] = {"value": r["cpu"]["value"], "unit": "cells/s", "cores": host_threads(),
                                        "kind": "port", "sample": f"{r['cpu']['cells']} cells"}
            print(json.dumps(line))
        return 0
    issue = {f"{k}_lanes": _lib.fp64_issue(device, k) for k in (1, 32)}

    tuned = None if a.no_autotune else run_autotune(a.workload, 2018 + rank, device)
    g = make_inputs(a.workload, seed=2018 + rank)
    ncell = g.ncell
    batched = run_device(g, "queue", a.steps, a.warmup, dist, device, sample_clocks=(rank == 0), tuned=tuned,
                         graph=True, solver=a.solver)
    ms_step = max_over_ranks(batched["ms_total"] / a.steps, dist)
    value = world * ncell / (STEPS_PER_HOUR * ms_step / 1e3)
    fl = sum(flops_of(s, info) for s in batched["stats"])
    dev_ms = sum(s["device_ms"] for s in batched["stats"])
    achieved_tf = fl / (dev_ms * 1e-3) / 1e12
    attempts = sum(s["accepted_steps"] + s["rejected_steps"] for s in batched["stats"])
    calls = split_calls(batched, ncell)

    plain = None
    if not a.no_plain:
        p = run_device(g, "static", a.steps, a.warmup, dist, device, sample_clocks=False)
        p_ms = max_over_ranks(p["ms_total"] / a.steps, dist)
        p_fl = sum(flops_of(s, info) for s in p["stats"])
        p_dev = sum(s["device_ms"] for s in p["stats"])
        plain = {"value": world * ncell / (STEPS_PER_HOUR * p_ms / 1e3), "ms_per_step": p_ms,
                 "achieved_tflops": p_fl / (p_dev * 1e-3) / 1e12, **split_calls(p, ncell)}

    e2e = None
    if not a.no_e2e:
        e = run_e2e(g, a.steps, a.warmup, dist, device)
        e_s = max_over_ranks(e["wall_s"] / a.steps, dist)
        e2e = {"value": world * ncell / (STEPS_PER_HOUR * e_s), "unit": UNIT, "h2d_bytes_per_step": e["h2d"],
               "d2h_bytes_per_step": e["d2h"], "ms_per_step": 1e3 * e_s,
               "path": "cmaqchem_step (host pointers, pinned buffers; copies inside each call)"}

    cpu = None
    if rank == 0 and not a.no_cpu:
        thr = host_threads()
        r = cpu_reference(ncell, STEPS_PER_HOUR, 0, thr, target_s=15.0)
        r1 = cpu_reference(ncell, STEPS_PER_HOUR, 0, 1, target_s=8.0)
        re = cpu_reference(ncell, STEPS_PER_HOUR, 0, thr, target_s=8.0, solver="ebi")
        rg = None if a.no_gear else cpu_reference(ncell, STEPS_PER_HOUR, 0, thr, target_s=8.0, solver="gear")
        cpu = {"value": r["value"], "unit": UNIT, "cores": thr, "kind": "port",
               "sample": f"{r['cells']} cells of the same distributions x {r['steps']} CHEM calls "
                         f"(reference algorithm, BLKSIZE 50 + reordering, C restatement, {r['wall_s']:.1f} s)",
               "single_core_value": r1["value"],
               "single_core_sample": f"{r1['cells']} cells x {r1['steps']} calls, 1 thread",
               "ebi_value": re["value"],
               "ebi_sample": f"{re['cells']} cells x {re['steps']} EBI CHEM calls, {thr} threads",
               "gear_value": None if rg is None else rg["value"],
               "gear_sample": None if rg is None else
               f"{rg['cells']} cells x {rg['steps']} SMVGEAR CHEM calls (BLKSIZE 50 + reordering), {thr} threads"}

    extras = rank == 0 and not a.no_extras
    tight_tol = (TIGHT_RTOL, TIGHT_ATOL)
    legs_s = {}

    def leg(name, on, fn):
        if not on:
            return None
        t0 = time.perf_counter()
        out = fn()
        legs_s[name] = round(time.perf_counter() - t0, 1)
        print(f"[bench] {name}: {legs_s[name]} s", file=sys.stderr, flush=True)
        return out
    accuracy = leg("accuracy", extras and not a.no_accuracy,
                   lambda: run_accuracy(g, device, tuned, host_threads(), tight_tol))
    tight = leg("tight", extras and not a.no_accuracy and a.tight_steps > 0,
                lambda: run_tight(g, device, a.tight_steps, tuned, info, tight_tol, peak_rec))
    ebi = leg("ebi", extras and not a.no_ebi, lambda: run_ebi(device, STEPS_PER_HOUR, g))
    adjoint = leg("adjoint", extras and not a.no_adjoint, lambda: run_adjoint(device, STEPS_PER_HOUR, adims))
    gear = leg("gear", extras and not a.no_gear, lambda: run_gear(device, a.steps))
    skewed = leg("skewed", extras and not a.no_configs, lambda: run_skewed(device, STEPS_PER_HOUR, tuned))
    cracmm2 = leg("cracmm2", extras and not a.no_configs, lambda: run_cracmm2(device, STEPS_PER_HOUR))
    def hetchem_both():
        r = run_hetchem(device, g.ncell, 5, 0 if a.no_cpu else host_threads())
        if not a.no_configs:                          # CRACMM2's tables on its 200x200x25 grid
            r["cracmm2"] = run_hetchem(device, 1000000, 5, 0 if a.no_cpu else min(4, host_threads()), "cracmm2")
        return r
    hetchem = leg("hetchem", extras and not a.no_hetchem, hetchem_both)
    aqchem = leg("aqchem", extras and not a.no_aqchem,
                 lambda: run_aqchem(device, a.aqchem_cells, 3, 3, 0 if a.no_cpu else host_threads()))
    if aqchem is not None:
        aqchem["roofline"] = aqchem_roofline(aqchem, peak_rec)

    traffic = traffic_note = None
    tfile = ROOT / "profiles" / "traffic_per_step.json"
    if tfile.exists():
        try:
            t = json.loads(tfile.read_text()).get(a.workload)
            if t is not None:
                # DRAM bytes per cell-attempt from the ncu capture, times this run's attempts per call
                traffic = float(t["bytes_per_cell_attempt"]) * attempts / a.steps
                traffic_note = t["source"]
        except Exception:
            traffic = None
    if rank == 0:
        launches_per_step = 4   # queue ordering (hist, scan, scatter) + solve, replayed from one graph
        if a.solver != "ros3":   # EBI iterations and Gear steps have no ROS3 FLOP count
            achieved_tf = None
        bclk = (batched["clocks"] or {}).get("sm_mhz")
        cpk = clock_peak(peak_rec, bclk)
        ipk = clock_peak(peak_rec, bclk, peak_rec["issue_probe_ops_per_clk_per_sm"])
        peak_tf = max(x for x in (peak_rec["measured_tflops"], cpk) if x)
        line = {
            "metric": METRIC if a.solver == "ros3" else METRIC.replace("ROS3", a.solver.upper()), "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded; cmaq_gb300/synthetic.py)",
            "config": {"workload": f"cb6r5_ae7_aq {g.ncols}x{g.nrows}x{g.nlays} ({ncell} cells per GPU), "
                                   f"{a.steps} x 5-min CHEM calls from the initial state, rtol 1e-3, atol 1e-9 ppmV",
                       "schedule": "batched (persistent, work queue ordered by previous step counts; "
                                   "the calls replayed from one captured CUDA graph)",
                       "queue": "cold at the first timed call: the warm-up calls' step counts are cleared, so "
                                "it is queued in grid order like a fresh run's first call",
                       "tuned": None if tuned is None else {k: tuned[k] for k in
                                                            ("variant", "lockstep", "block_warps", "sample",
                                                             "tuning_s")},
                       "cells": ncell, "step_attempts_per_cell": attempts / ncell / a.steps,
                       "l2": "inputs larger than L2 (CGRID %.1f GB); no flush" % (g.conc.nbytes / 1e9),
                       "parallelism": f"replicas x{world} (own grid per GPU)"},
            **calls,
            "roofline": None if achieved_tf is None else {
                         "bound": "fp64", "achieved": achieved_tf, "peak": peak_tf, "unit": "TFLOP/s",
                         "frac": achieved_tf / peak_tf, "traffic": traffic, "traffic_source": traffic_note,
                         "traffic_per": "one CHEM call (launch) of this run: DRAM bytes per cell-attempt x this run's "
                                        "attempts per call",
                         "dram_gbs_from_traffic": None if traffic is None else traffic / (ms_step * 1e-3) / 1e9,
                         "peak_source": "the larger of the measured FP64 FMA-chain rate and the clock-derived "
                                        "rate (the saturated FP64 ops per clock per SM of a sweep of kernel "
                                        "shapes, at the timed region's median SM clock); no FP64 figure in "
                                        "MEASURED_PEAKS.json",
                         "peak_measured": peak_rec, "peak_clock_derived": cpk, "timed_sm_mhz": bclk,
                         "frac_of_measured": achieved_tf / peak_rec["measured_tflops"],
                         "frac_of_clock_derived": None if not cpk else achieved_tf / cpk,
                         "issue_probe_peak": ipk,
                         "frac_of_issue_probe_peak": None if not ipk else achieved_tf / ipk,
                         "flops": "algorithmic FLOPs of the reference's ROS3 step per attempt x attempts",
                         "fp64_chain_cycles_per_fma": issue},
            "plain": plain,
            "batched_over_plain": None if plain is None else value / plain["value"],
            "accuracy": accuracy,
            "tight": tight,
            "adjoint": adjoint,
            "ebi": ebi,
            "gear": gear,
            "skewed": skewed,
            "cracmm2": cracmm2,
            "aqchem": aqchem,
            "hetchem": hetchem,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": batched["clocks"],
            "gpu_launches": launches_per_step * a.steps,
            "extra_legs_s": legs_s,
        }
        print(json.dumps(line))
    if dist is not None:
        import torch.distributed as tdist
        tdist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
