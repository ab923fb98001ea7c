"""KMT2 aqueous cloud chemistry on the GPU: the kinetic core of CMAQ's AQCHEM
(CCTM/src/cloud/acm_ae7_kmt2/aqchem_kmt.F90:371-543) for a batch of cloudy cells.

    var_out, stats = aqchem_kinetics(params, var_mix)

``params`` [15][n] and ``var_mix`` [161][n] are float64 CUDA tensors laid out as
``include/cmaqchem.h`` (``cmaqchem_kmt2_solve_device``) describes: AQCHEM's arguments per
cell, and the KPP state as the reference's Initialize maps the gas and aerosol arrays
(mixing ratios).  ``var_out`` is the state after the cloud time TAUCLD in molec/cm3, as
KPP's VAR; ``stats`` [10][n] int32 the integrator's counters per cell (see
``STATS``).  The call runs in libcmaqchem.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib

NVAR, NFIX, NPARAM = 161, 4, 15
PARAMS = ("temp2", "pres_pa", "taucld", "prcrate", "wcavg", "wtavg", "airm", "alfa0", "alfa3", "coszen", "jh2o2",
          "ho", "ispc8", "mtpyrac", "photo")
STATS = ("nstp", "nacc", "nrej", "nfun", "njac", "ndec", "nsol", "nsng", "ierr", "npass")


def _ptr(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def aqchem_kinetics(params: torch.Tensor, var_mix: torch.Tensor, *, lanes: int | None = None, with_fix: bool = False,
                    stream: torch.cuda.Stream | None = None, variant: str = "default"):
    """Integrate n cloudy cells over their TAUCLD; returns (var_out, stats) or, with
    with_fix, (var_out, fix_out, stats).  ``lanes`` is the number of threads that take
    cells from the call's queue (the workspace holds 23 KB per lane); by default as
    many as the device holds resident (cmaqchem_kmt2_default_lanes).  ``variant``: a
    library build of ``cmaq_gb300.build`` (same bits in all)."""
    for name, t, rows in (("params", params, NPARAM), ("var_mix", var_mix, NVAR)):
        if not (t.is_cuda and t.dtype == torch.float64 and t.dim() == 2 and t.shape[0] == rows and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous float64 CUDA tensor of shape ({rows}, n)")
    n = params.shape[1]
    if var_mix.shape[1] != n or var_mix.device != params.device:
        raise ValueError("params and var_mix must describe the same cells on the same device")
    dev = params.device
    var_out = torch.empty((NVAR, n), dtype=torch.float64, device=dev)
    fix_out = torch.empty((NFIX, n), dtype=torch.float64, device=dev) if with_fix else None
    stats = torch.zeros((len(STATS), n), dtype=torch.int32, device=dev)
    if n == 0:
        return (var_out, fix_out, stats) if with_fix else (var_out, stats)
    L = _lib.lib(variant)
    if lanes is None:
        lanes = L.cmaqchem_kmt2_default_lanes(dev.index if dev.index is not None else torch.cuda.current_device())
        if lanes < 1:
            raise _lib.ChemError(_lib.last_error())
    lanes = max(1, min(int(lanes), n))
    ws = torch.empty(L.cmaqchem_kmt2_workspace_doubles(lanes), dtype=torch.float64, device=dev)
    s = stream or torch.cuda.current_stream(dev)
    with torch.cuda.device(dev):
        _lib.check(L.cmaqchem_kmt2_solve_device(n, _ptr(params), _ptr(var_mix), _ptr(var_out), _ptr(fix_out),
                                                _ptr(stats), _ptr(ws), ws.numel(), C.c_void_p(s.cuda_stream)))
    return (var_out, fix_out, stats) if with_fix else (var_out, stats)


def aqchem_kinetics_host(params, var_mix, *, device: int = 0, with_fix: bool = False):
    """The same integration on host numpy arrays, params [15][n] and var_mix [161][n]
    float64, through the host-array entry point (cmaqchem_kmt2_solve): returns numpy
    (var_out, stats) or (var_out, fix_out, stats)."""
    import numpy as np
    params = np.ascontiguousarray(params, dtype=np.float64)
    var_mix = np.ascontiguousarray(var_mix, dtype=np.float64)
    if params.ndim != 2 or params.shape[0] != NPARAM or var_mix.shape != (NVAR, params.shape[1]):
        raise ValueError(f"params must be ({NPARAM}, n) and var_mix ({NVAR}, n)")
    n = params.shape[1]
    var_out = np.empty((NVAR, n))
    fix_out = np.empty((NFIX, n)) if with_fix else None
    stats = np.zeros((len(STATS), n), dtype=np.int32)
    if n:
        L = _lib.lib()
        p = lambda a: None if a is None else C.c_void_p(a.ctypes.data)
        _lib.check(L.cmaqchem_kmt2_solve(n, p(params), p(var_mix), p(var_out), p(fix_out), p(stats), int(device)))
    return (var_out, fix_out, stats) if with_fix else (var_out, stats)


NGAS, NSURROGATE, NFACTOR, NOUT = 29, 31, 16, 10
OUTS = ("hpwdep", "betaso4", "fractr", "fracpoa", "fracpri", "fracsoa", "mbal_s", "mbal_n", "mbal_nh4", "mbal_cl")


def aqchem(params: torch.Tensor, gas: torch.Tensor, aerosol: torch.Tensor, aer_index, factors, *,
           lanes: int | None = None, stream: torch.cuda.Stream | None = None, variant: str = "default"):
    """The whole AQCHEM (mapping of GAS and AEROSOL into the KPP state, the kinetic core,
    redistribution; include/cmaqchem.h: cmaqchem_aqchem_device) for n cloudy cells.
    ``params`` [15][n], ``gas`` [29][n] and ``aerosol`` [naer * 3][n] float64 CUDA tensors
    (gas and aerosol are updated in place, as AQCHEM's INOUT arguments); ``aer_index`` the
    31 rows of AQCHEM's surrogates in the aerosol list, ``factors`` the 16 coarse crustal
    factors (the manifest's ``crustal_factors`` for the repository's mechanism).  Returns
    (gas_wdep [29][n], aer_wdep [naer * 3][n], out [10][n] (``OUTS``), stats [10][n])."""
    import numpy as np
    for name, t, rows in (("params", params, NPARAM), ("gas", gas, NGAS), ("aerosol", aerosol, None)):
        ok = t.is_cuda and t.dtype == torch.float64 and t.dim() == 2 and t.is_contiguous()
        if not ok or (rows is not None and t.shape[0] != rows):
            raise ValueError(f"{name} must be a contiguous float64 CUDA tensor of shape ({rows or 'naer*3'}, n)")
    n = params.shape[1]
    if gas.shape[1] != n or aerosol.shape[1] != n or aerosol.shape[0] % 3:
        raise ValueError("params, gas and aerosol must describe the same cells; aerosol has naer * 3 rows")
    naer = aerosol.shape[0] // 3
    idx = np.ascontiguousarray(aer_index, dtype=np.int32)
    fac = np.ascontiguousarray(factors, dtype=np.float64)
    if idx.shape != (NSURROGATE,) or fac.shape != (NFACTOR,):
        raise ValueError(f"aer_index needs {NSURROGATE} entries and factors {NFACTOR}")
    dev = params.device
    gwd = torch.empty_like(gas)
    awd = torch.empty_like(aerosol)
    out = torch.empty((NOUT, n), dtype=torch.float64, device=dev)
    stats = torch.zeros((len(STATS), n), dtype=torch.int32, device=dev)
    if n == 0:
        return gwd, awd, out, stats
    L = _lib.lib(variant)
    if lanes is None:
        lanes = L.cmaqchem_kmt2_default_lanes(dev.index if dev.index is not None else torch.cuda.current_device())
        if lanes < 1:
            raise _lib.ChemError(_lib.last_error())
    lanes = max(1, min(int(lanes), n))
    ws = torch.empty(L.cmaqchem_kmt2_workspace_doubles(lanes), dtype=torch.float64, device=dev)
    s = stream or torch.cuda.current_stream(dev)
    with torch.cuda.device(dev):
        _lib.check(L.cmaqchem_aqchem_device(n, _ptr(params), _ptr(gas), _ptr(aerosol), naer,
                                            C.c_void_p(idx.ctypes.data), C.c_void_p(fac.ctypes.data), _ptr(gwd),
                                            _ptr(awd), _ptr(out), _ptr(stats), _ptr(ws), ws.numel(),
                                            C.c_void_p(s.cuda_stream)))
    return gwd, awd, out, stats


def sweep(ncell: int, specs, reps: int = 2, seed: int = 2018) -> dict:
    """Launch-shape sweep of the kinetic core: for each spec "variant:lanes_per_sm" (a
    build of ``cmaq_gb300.build`` and the lanes per SM of the call) the device time of one
    call on ``ncell`` seeded cloudy cells (median of 3, after one untimed call), the FP64
    rate from the routines' operation counts, and whether the state equals the first
    spec's bit for bit."""
    import numpy as np
    from .synthetic import kmt2_manifest, make_cloud_cells
    fl = kmt2_manifest()["flops"]
    p, v = make_cloud_cells(ncell, seed=seed)
    pt = torch.from_numpy(np.ascontiguousarray(p.T)).cuda()
    vt = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
    nsm = torch.cuda.get_device_properties(pt.device).multi_processor_count
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    ref, out = None, {}
    for rep in range(reps):
        for spec in specs:
            variant, lps = spec.split(":")
            lanes = min(ncell, nsm * int(lps))
            aqchem_kinetics(pt, vt, lanes=lanes, variant=variant)
            ms = []
            for _ in range(3):
                ev[0].record()
                var, st = aqchem_kinetics(pt, vt, lanes=lanes, variant=variant)
                ev[1].record()
                torch.cuda.synchronize()
                ms.append(ev[0].elapsed_time(ev[1]))
            sd = st.cpu().numpy().astype(np.int64)
            flops = float(sd[3].sum() * fl["fun"] + sd[4].sum() * fl["jac"] + sd[5].sum() * fl["decomp"]
                          + sd[6].sum() * fl["solve"] + sd[0].sum() * fl["vector"])
            vo = var.cpu().numpy()
            ref = vo.copy() if ref is None else ref
            m = float(np.median(ms))
            r = {"ms": m, "cells_per_s": ncell / m * 1e3, "tflops": flops / m / 1e9,
                 "same_bits": bool(np.array_equal(vo, ref, equal_nan=True))}
            out.setdefault(spec, []).append(r)
            print(f"rep {rep} {spec}: {m:.1f} ms ({ncell} cells, {lanes} lanes), {r['cells_per_s']:.0f} cells/s, "
                  f"{r['tflops']:.4f} TFLOP/s, same bits: {r['same_bits']}", flush=True)
    return out


if __name__ == "__main__":
    import argparse
    from . import build as cbuild
    ap = argparse.ArgumentParser(description="launch-shape sweep of the KMT2 kinetic core (see sweep())")
    ap.add_argument("specs", help="comma-separated variant:lanes_per_sm, e.g. default:512,kq3:384")
    ap.add_argument("--cells", type=int, default=200000)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    specs = a.specs.split(",")
    for v in dict.fromkeys(["default"] + [sp.split(":")[0] for sp in specs]):   # variants share its objects
        cbuild.build(variant=v)
    sweep(a.cells, specs, a.reps)
