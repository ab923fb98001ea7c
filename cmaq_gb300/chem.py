"""Host-side chemistry operator: the GB300 counterpart of CMAQ's ``CHEM``.

CMAQ calls ``CHEM(CGRID, JDATE, JTIME, TSTEP)`` once per synchronisation step
(CCTM/src/driver/sciproc.F:298); the operator sets itself up on its first call
(rbdriver.F:226-371) and reads met, photolysis and heterogeneous rates through
modules.  Here:

* :class:`ChemSolver` owns a library handle (the first-call state) for one of the
  reference's solvers (``solver="ros3"``, ``"ebi"`` or ``"gear"`` for SMVGEAR) and exposes
  ``step`` (one CHEM call), ``steps`` (several, from one captured CUDA graph),
  ``step_ddm`` (a CHEM call with DDM-3D sensitivities), the solver-level ``solve``
  (RBSOLVER), ``ebi_solve`` (HRSOLVER) and ``gear_solve`` (SMVGEAR) with given rate
  constants, and ``rconst`` (CALC_RCONST);
* :func:`CHEM` keeps the reference's call signature; the implicit inputs are set
  with :func:`set_environment`, the analogue of the modules CHEM reads.

Arrays are CMAQ's Fortran layouts held as C-ordered arrays of reversed shape
(``conc[spc, lay, row, col]`` = ``CONC(col, row, lay, spc)``).  ``step`` accepts
numpy arrays (copied to and from the GPU inside the call) or CUDA torch tensors
(used in place).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import ChemError, check

SOLVERS = {"ros3": _lib.SOLVER_ROS3, "ebi": _lib.SOLVER_EBI, "gear": _lib.SOLVER_GEAR}
SCHEDULES = {"static": _lib.SCHED_STATIC, "plain": _lib.SCHED_STATIC, "queue": _lib.SCHED_QUEUE,
             "batched": _lib.SCHED_QUEUE}


def reference_tolerance(x: float) -> float:
    """RB_RTOL / RB_ATOL are REAL(4) run-time settings widened to REAL(8) (rbinit.F:250-251)."""
    return float(np.float32(x))


def _is_torch(x) -> bool:
    return hasattr(x, "data_ptr") and hasattr(x, "is_cuda")


def _ptr(x):
    if x is None:
        return None
    if _is_torch(x):
        if not x.is_cuda:
            raise ChemError("torch tensors passed to the chemistry operator must be on the GPU")
        if not x.is_contiguous():
            raise ChemError("torch tensors must be contiguous")
        return C.c_void_p(x.data_ptr())
    if not x.flags["C_CONTIGUOUS"]:
        raise ChemError("numpy arrays must be C-contiguous")
    return C.c_void_p(x.ctypes.data)


def tstep_array(tstep) -> C.Array:
    t = (C.c_int * 3)(*[int(v) for v in tstep])
    return t


class ChemSolver:
    """One chemistry handle for a fixed local domain (first-call state of CHEM)."""

    def __init__(self, mechanism: str = "cb6r5_ae7_aq", *, ncols: int, nrows: int, nlays: int, nspcsd: int,
                 cgrid_index=None, rtol: float = 1.0e-3, atol: float = 1.0e-7, schedule: str = "queue",
                 device: int = 0, max_iter: int = 0, reference_tolerances: bool = True, variant: str = "default",
                 solver: str = "ros3"):
        if solver not in SOLVERS:
            raise ChemError(f"unknown solver {solver!r}; use one of {sorted(SOLVERS)}")
        if schedule not in SCHEDULES:
            raise ChemError(f"unknown schedule {schedule!r}; use one of {sorted(SCHEDULES)}")
        self.mechanism = mechanism
        self.variant = variant
        self._L = _lib.lib(variant)
        self.info, self.inew2old = _lib.mech_info(mechanism)
        self.iold2new = [0] * len(self.inew2old)
        for i, old in enumerate(self.inew2old):
            self.iold2new[old] = i
        self.shape = (nlays, nrows, ncols)
        self.nspcsd = nspcsd
        self.rtol = reference_tolerance(rtol) if reference_tolerances else float(rtol)
        self.atol = reference_tolerance(atol) if reference_tolerances else float(atol)
        self._cgi = None
        if cgrid_index is not None:
            self._cgi = (C.c_int * self.info.nspec)(*[int(v) for v in cgrid_index])
        self.solver = solver
        cfg = _lib.Cfg(mechanism.encode(), SOLVERS[solver], SCHEDULES[schedule], self.rtol, self.atol, ncols, nrows,
                       nlays, nspcsd, self._cgi, device, max_iter)
        h = C.c_void_p()
        check(self._L.cmaqchem_init(C.byref(cfg), C.byref(h)), self._L)
        self._h = h
        self.schedule = schedule

    def set_tuning(self, **knobs) -> None:
        """Scheduling knobs (see include/cmaqchem_diag.h): night_pattern=0/1, lockstep=0/1/2,
        block_warps=2/4/8, blocks_per_sm=0 (as many as fit) or a cap."""
        for k, v in knobs.items():
            check(self._L.cmaqchem_diag_set_tuning(self._h, k.encode(), int(v)), self._L)

    @property
    def ncell(self) -> int:
        n = 1
        for s in self.shape:
            n *= s
        return n

    def close(self):
        if getattr(self, "_h", None):
            self._L.cmaqchem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def step(self, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero, jdate: int = 2018182,
             jtime: int = 0, tstep=(10000, 500, 500), stream=None) -> dict:
        """One CHEM call (rbdriver.F).  Returns totals; ``failed_cells`` > 0 when some cells stopped
        (their per-cell status is in :meth:`cell_stats`)."""
        args = [conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero]
        on_gpu = [_is_torch(a) for a in args]
        if any(on_gpu) and not all(on_gpu):
            raise ChemError("pass either all numpy arrays (host) or all CUDA tensors (device)")
        self._check_shapes(*args)
        st = _lib.Stats()
        ts = tstep_array(tstep)
        ptrs = [_ptr(a) for a in args]
        if all(on_gpu):
            s = C.c_void_p(stream) if isinstance(stream, int) else (
                C.c_void_p(stream.cuda_stream) if stream is not None else None)
            rc = self._L.cmaqchem_step_device(self._h, *ptrs, jdate, jtime, ts, s, C.byref(st))
        else:
            rc = self._L.cmaqchem_step(self._h, *ptrs, jdate, jtime, ts, C.byref(st))
        check(rc, self._L)
        return st.as_dict()

    def step_ddm(self, sengrid, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero, rate_mask=None,
                 region=None, jdate: int = 2018182, jtime: int = 0, tstep=(10000, 500, 500), stream=None) -> dict:
        """One CHEM call on CUDA tensors that also advances DDM-3D sensitivities: sengrid
        [nspcsd, nparam, nlays, nrows, ncols] float32 (SENGRID(C,R,L,NP,SPC)); rate_mask
        [nparam, nrxns] uint8 marks reaction-rate parameters' reactions; region [nparam, ...cells]
        float32 weights (IREGION)."""
        args = [conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero]
        if not all(_is_torch(a) for a in args) or not _is_torch(sengrid):
            raise ChemError("step_ddm() takes CUDA tensors")
        self._check_shapes(*args)
        nparam = int(sengrid.shape[1])
        if tuple(sengrid.shape) != (self.nspcsd, nparam) + self.shape or "float32" not in str(sengrid.dtype):
            raise ChemError(f"sengrid must be float32 [{self.nspcsd}, nparam, {self.shape}]")
        if rate_mask is not None and tuple(rate_mask.shape) != (nparam, self.info.nrxns):
            raise ChemError("rate_mask must be [nparam, nrxns] uint8")
        st = _lib.Stats()
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        rc = self._L.cmaqchem_step_ddm_device(self._h, *[_ptr(a) for a in args], jdate, jtime, tstep_array(tstep),
                                              _ptr(sengrid), nparam, _ptr(rate_mask), _ptr(region), s, C.byref(st))
        check(rc, self._L)
        return st.as_dict()

    def steps(self, nsteps: int, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero, jdate: int = 2018182,
              jtime: int = 0, tstep=(10000, 500, 500), stream=None) -> dict:
        """``nsteps`` consecutive CHEM calls on CUDA tensors, replayed from one captured
        CUDA graph without host synchronisation in between; totals over the calls."""
        args = [conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero]
        if not all(_is_torch(a) for a in args):
            raise ChemError("steps() takes CUDA tensors")
        self._check_shapes(*args)
        st = _lib.Stats()
        s = C.c_void_p(stream) if isinstance(stream, int) else (
            C.c_void_p(stream.cuda_stream) if stream is not None else None)
        rc = self._L.cmaqchem_steps_device(self._h, *[_ptr(a) for a in args], jdate, jtime, tstep_array(tstep),
                                           int(nsteps), s, C.byref(st))
        check(rc, self._L)
        return st.as_dict()

    def _check_shapes(self, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero):
        L, R, Cc = self.shape
        exp = {"conc": (self.nspcsd, L, R, Cc), "ta": (L, R, Cc), "qv": (L, R, Cc), "dens": (L, R, Cc),
               "pres": (L, R, Cc), "seaice": (R, Cc), "ocean_szone": (R, Cc),
               "rj": (self.info.nphotab, L, R, Cc), "khetero": (L, R, Cc, self.info.nhetero)}
        got = dict(conc=conc, ta=ta, qv=qv, dens=dens, pres=pres, seaice=seaice, ocean_szone=ocean_szone, rj=rj,
                   khetero=khetero)
        for k, shp in exp.items():
            a = got[k]
            if tuple(a.shape) != shp:
                raise ChemError(f"{k} has shape {tuple(a.shape)}, expected {shp}")
            want = "float64" if k == "khetero" else "float32"
            if want not in str(a.dtype):
                raise ChemError(f"{k} must be {want}, got {a.dtype}")

    def cell_stats(self):
        status = np.zeros(self.shape, np.int32)
        attempts = np.zeros(self.shape, np.int32)
        check(self._L.cmaqchem_cell_stats(self._h, C.c_void_p(status.ctypes.data),
                                          C.c_void_p(attempts.ctypes.data)), self._L)
        return status, attempts

    def solve(self, y, rki, night, chemstep_min: float, with_stats: bool = False, stream=None):
        """RBSOLVER on CUDA tensors: y [ischan, n] (solver species order) in place, rki [nrxns, n],
        night [n] uint8.  Optional per-cell status / accepted / rejected step counts."""
        import torch
        n = y.shape[1]
        st = ns = nf = None
        if with_stats:
            st, ns, nf = (torch.zeros(n, dtype=torch.int32, device=y.device) for _ in range(3))
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        check(self._L.cmaqchem_ros3_solve_device(self._h, n, _ptr(y), _ptr(rki), _ptr(night), chemstep_min,
                                                 _ptr(st), _ptr(ns), _ptr(nf), s), self._L)
        return (st, ns, nf) if with_stats else None

    def ebi_solve(self, yc, rki, tstep_sec: int, with_stats: bool = False, stream=None):
        """HRSOLVER on CUDA tensors: yc [nspec, n] (mechanism species order, ppm) in place,
        rki [nrxns, n]; tstep_sec = synchronisation step.  Optional per-cell status and
        Backward-Euler iteration counts."""
        import torch
        n = yc.shape[1]
        st = it = None
        if with_stats:
            st, it = (torch.zeros(n, dtype=torch.int32, device=yc.device) for _ in range(2))
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        check(self._L.cmaqchem_ebi_solve_device(self._h, n, _ptr(yc), _ptr(rki), int(tstep_sec), _ptr(st),
                                                _ptr(it), s), self._L)
        return (st, it) if with_stats else None

    GEAR_STATS = ("nsteps", "ncfail", "nefail", "npderiv", "nsubfun", "nnewt", "maxord", "status")

    def gear_solve(self, y, rk, night, chemstep_min: float, with_stats: bool = False, stream=None):
        """SMVGEAR (grsmvgear.F, BLKSIZE = 1) on CUDA tensors: y [nspec, n] (solver species order,
        ppm) in place, rk [nrxns, n], night [n] uint8.  Optional per-cell statistics [n, 8] with
        the columns of GEAR_STATS.  Needs a handle made with solver="gear"."""
        import torch
        n = y.shape[1]
        st = torch.zeros((n, 8), dtype=torch.int32, device=y.device) if with_stats else None
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        check(self._L.cmaqchem_gear_solve_device(self._h, n, _ptr(y), _ptr(rk), _ptr(night), chemstep_min,
                                                 _ptr(st), s), self._L)
        return st

    def gear_tolerances(self, max_atol: float = 1e-7, min_atol: float = 1e-9, conc_floor: float = 1e-12) -> None:
        """GEAR_MAX_ATOL, GEAR_MIN_ATOL, GEAR_CONC_FLOOR (ppmV) of a solver="gear" handle."""
        check(self._L.cmaqchem_gear_tolerances(self._h, max_atol, min_atol, conc_floor), self._L)

    def rconst(self, conc, ta, qv, dens, pres, seaice, ocean_szone, rj, khetero):
        """CALC_RCONST for every cell of the grid (CUDA tensors): returns rki [nrxns, ncell], sunlit [ncell]."""
        import torch
        dev = conc.device
        rki = torch.empty((self.info.nrxns, self.ncell), dtype=torch.float64, device=dev)
        sun = torch.empty(self.ncell, dtype=torch.uint8, device=dev)
        check(self._L.cmaqchem_rconst_device(self._h, *[_ptr(a) for a in (conc, ta, qv, dens, pres, seaice,
                                                                         ocean_szone, rj, khetero)],
                                             _ptr(rki), _ptr(sun), None), self._L)
        return rki, sun


# ------------------------------------------------------------------ reference-shaped entry point
@dataclass
class Environment:
    """The inputs CHEM reads through modules: met (INTERPOLATE_VAR), OCEAN+SZONE, SEAICE,
    photolysis rates (PHOT_MOD RJ) and heterogeneous rates (AEROSOL_CHEMISTRY KHETERO)."""
    ta: object
    qv: object
    dens: object
    pres: object
    seaice: object
    ocean_szone: object
    rj: object
    khetero: object
    nspcsd: int
    mechanism: str = "cb6r5_ae7_aq"
    cgrid_index: object = None
    rtol: float = 1.0e-3
    atol: float = 1.0e-7
    schedule: str = "queue"


_ENV: Environment | None = None
_SOLVER: ChemSolver | None = None


def set_environment(env: Environment) -> None:
    global _ENV, _SOLVER
    _ENV = env
    if _SOLVER is not None:
        _SOLVER.close()
        _SOLVER = None


def CHEM(conc, jdate: int, jtime: int, tstep) -> dict:
    """``CHEM(CGRID, JDATE, JTIME, TSTEP)``: integrate the gas chemistry of every cell over
    TSTEP(2) and update ``conc`` in place.  The first call sets the solver up."""
    global _SOLVER
    if _ENV is None:
        raise ChemError("CHEM: call set_environment() with the met, photolysis and heterogeneous inputs first")
    e = _ENV
    nlays, nrows, ncols = tuple(e.ta.shape)
    if _SOLVER is None:
        _SOLVER = ChemSolver(e.mechanism, ncols=ncols, nrows=nrows, nlays=nlays, nspcsd=e.nspcsd,
                             cgrid_index=e.cgrid_index, rtol=e.rtol, atol=e.atol, schedule=e.schedule)
    return _SOLVER.step(conc, e.ta, e.qv, e.dens, e.pres, e.seaice, e.ocean_szone, e.rj, e.khetero, jdate,
                        jtime, tstep)
