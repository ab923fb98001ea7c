"""ctypes binding of the CPU oracle (test infrastructure only).

Loads ``oracle/_build/liboracle_<mech>.so`` (see ``oracle/build.py``), a C
restatement of CMAQ's ROS3, EBI and SMVGEAR chemistry (CCTM/src/gas/ros3/*.F,
ebi_<mech>/*.F, smvgear/*.F).  Tests, the smoke
check and the CPU-baseline leg of the benchmark use it as the checker; nothing
in the product imports it.
"""
from __future__ import annotations

import ctypes as C
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


class OracleChemArgs(C.Structure):
    _fields_ = [("ncols", C.c_int), ("nrows", C.c_int), ("nlays", C.c_int), ("nspcsd", C.c_int),
                ("conc", C.POINTER(C.c_float)), ("cgrid_index", C.POINTER(C.c_int)),
                ("convert", C.POINTER(C.c_int)), ("ta", C.POINTER(C.c_float)), ("qv", C.POINTER(C.c_float)),
                ("dens", C.POINTER(C.c_float)), ("pres", C.POINTER(C.c_float)),
                ("seaice", C.POINTER(C.c_float)), ("ocean_szone", C.POINTER(C.c_float)),
                ("rj", C.POINTER(C.c_float)), ("khetero", C.POINTER(C.c_double)),
                ("tstep_sec", C.c_int), ("rtol", C.c_double), ("atol", C.c_double), ("blksize", C.c_int),
                ("lreorder", C.c_int), ("max_iter", C.c_int), ("threads", C.c_int),
                ("nsteps_total", C.c_longlong), ("nfails_total", C.c_longlong), ("nfailed_blocks", C.c_int)]


def _p(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


@lru_cache(maxsize=None)
def load(mech: str = "cb6r5_ae7_aq") -> C.CDLL:
    import sys
    sys.path.insert(0, str(HERE))
    try:
        import build as _b  # oracle/build.py
    finally:
        sys.path.pop(0)
    path = _b.lib_path(mech)
    if not path.exists():
        _b.build([mech])
    lib = C.CDLL(str(path))
    dp, ip, fp, u8p = C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_float), C.POINTER(C.c_uint8)
    lib.oracle_calc_rconst.argtypes = [C.c_int, dp, dp, dp, dp, dp, C.c_int, dp, dp]
    lib.oracle_feval.argtypes = [C.c_int, C.c_int, dp, dp, dp]
    lib.oracle_jac_decomp.argtypes = [C.c_int, C.c_int, dp, dp, C.c_double, dp, dp]
    lib.oracle_rbsolver_block.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, dp, dp, ip]
    lib.oracle_rbsolver_cells.argtypes = [C.c_long, C.c_double, C.c_double, C.c_double, C.c_int, dp, dp, u8p,
                                          ip, ip, ip, C.c_int]
    lib.oracle_chem.argtypes = [C.POINTER(OracleChemArgs)]
    lib.oracle_mech_name.restype = C.c_char_p
    lib.oracle_chem_ebi.argtypes = [C.POINTER(OracleChemArgs)]
    lib.oracle_ebi_solve_cells.argtypes = [C.c_long, C.c_int, dp, dp, ip, C.POINTER(C.c_long), C.c_int]
    lib.oracle_adj_forward.argtypes = [C.c_long, dp, dp, C.c_long, u8p, dp, dp, C.c_int, C.c_double, C.c_double,
                                       C.c_double, dp, ip, dp, C.c_int, C.c_int]
    lib.oracle_adj_backward.argtypes = [C.c_long, dp, dp, C.c_long, u8p, dp, dp, C.c_int, C.c_double, C.c_double,
                                        C.c_double, dp, ip, dp, dp, C.c_int]
    lib.oracle_adj_replay.argtypes = [C.c_long, dp, dp, C.c_long, u8p, dp, dp, C.c_int, ip, dp, C.c_int, C.c_int]
    lib.oracle_adj_replay.restype = None
    lib.oracle_ddm3d_window.argtypes = [C.c_long, dp, dp, C.c_long, u8p, dp, dp, C.c_int, C.c_double, C.c_double,
                                        C.c_double, C.c_int, ip, ip, dp, C.c_int, C.c_void_p, C.c_int]
    lib.oracle_ebi_gather.argtypes = [C.POINTER(OracleChemArgs), dp, dp, u8p]
    lib.oracle_ebi_gather.restype = None
    lib.oracle_gear_cfg_size.restype = C.c_size_t
    lib.oracle_gear_cfg.argtypes = [C.c_double, C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p]
    lib.oracle_gear_cfg.restype = None
    lib.oracle_gear_cells.argtypes = [C.c_long, C.c_double, C.c_void_p, dp, dp, u8p, ip, C.c_int]
    lib.oracle_gear_chem.argtypes = [C.POINTER(OracleChemArgs), C.c_void_p]
    lib.oracle_gear_pow.argtypes = [C.c_double, C.c_double]
    lib.oracle_gear_pow.restype = C.c_double
    lib.oracle_set_dtmin.argtypes = [C.c_double]
    lib.oracle_get_dtmin.restype = C.c_double
    return lib


class Oracle:
    def __init__(self, mech: str = "cb6r5_ae7_aq"):
        self.mech = mech
        self.lib = load(mech)
        self.nspec = self.lib.oracle_nspec()
        self.nrxns = self.lib.oracle_nrxns()
        self.ischan = self.lib.oracle_ischan()
        self.nphotab = self.lib.oracle_nphotab()
        self.nhetero = self.lib.oracle_nhetero()
        self.inew2old = np.zeros(self.nspec, np.int32)
        self.iold2new = np.zeros(self.nspec, np.int32)
        self.lib.oracle_inew2old(_p(self.inew2old, C.c_int))
        self.lib.oracle_iold2new(_p(self.iold2new, C.c_int))

    def tight(self):
        """Context manager for the tight truth solution: DTMIN lowered to 1e-14 min."""
        import contextlib

        @contextlib.contextmanager
        def cm():
            old = self.lib.oracle_get_dtmin()
            self.lib.oracle_set_dtmin(1.0e-14)
            try:
                yield self
            finally:
                self.lib.oracle_set_dtmin(old)
        return cm()

    def rconst(self, temp, pres_atm, h2o_ppm, rj, het, sunlit: bool, seawater) -> np.ndarray:
        n = len(temp)
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (temp, pres_atm, h2o_ppm)]
        rj = np.ascontiguousarray(rj, dtype=np.float64).reshape(self.nphotab, n)
        het = np.ascontiguousarray(het, dtype=np.float64).reshape(max(self.nhetero, 1), n)
        sw = np.ascontiguousarray(seawater, dtype=np.float64)
        out = np.zeros((self.nrxns, n))
        self.lib.oracle_calc_rconst(n, _p(a[0], C.c_double), _p(a[1], C.c_double), _p(a[2], C.c_double),
                                    _p(rj, C.c_double), _p(het, C.c_double), int(bool(sunlit)),
                                    _p(sw, C.c_double), _p(out, C.c_double))
        return out

    def feval(self, y, rki, ncsp: int = 0) -> np.ndarray:
        y = np.ascontiguousarray(y, np.float64)
        rki = np.ascontiguousarray(rki, np.float64)
        n = y.shape[1]
        out = np.zeros_like(y)
        self.lib.oracle_feval(n, ncsp, _p(y, C.c_double), _p(rki, C.c_double), _p(out, C.c_double))
        return out

    def solve_cells(self, y, rki, night, chemstep: float, rtol: float, atol: float, max_iter: int = 100000,
                    threads: int = 0):
        """Per-cell ROS3 (BLKSIZE = 1) over chemstep minutes; y (nspec, n) new order, in place copy."""
        y = np.array(y, dtype=np.float64, order="C", copy=True)
        rki = np.ascontiguousarray(rki, np.float64)
        night = np.ascontiguousarray(night, np.uint8)
        n = y.shape[1]
        ns, nf, st = (np.zeros(n, np.int32) for _ in range(3))
        self.lib.oracle_rbsolver_cells(n, chemstep, rtol, atol, max_iter, _p(y, C.c_double), _p(rki, C.c_double),
                                       _p(night, C.c_uint8), _p(ns, C.c_int), _p(nf, C.c_int), _p(st, C.c_int),
                                       threads)
        return y, ns, nf, st

    def solve_block(self, y, rki, ncsp: int, chemstep: float, rtol: float, atol: float, max_iter: int = 100000):
        y = np.array(y, dtype=np.float64, order="C", copy=True)
        rki = np.ascontiguousarray(rki, np.float64)
        stats = np.zeros(4, np.int32)
        self.lib.oracle_rbsolver_block(y.shape[1], ncsp, chemstep, rtol, atol, max_iter, _p(y, C.c_double),
                                       _p(rki, C.c_double), _p(stats, C.c_int))
        return y, stats

    def chem(self, g, tstep_sec: int = 300, rtol: float = 1e-3, atol: float = 1e-9, blksize: int = 50,
             lreorder: bool = True, max_iter: int = 100000, threads: int = 0, conc=None):
        """One CHEM call on a GridInputs-like object; returns (new conc, totals)."""
        conc = np.array(g.conc if conc is None else conc, dtype=np.float32, order="C", copy=True)
        man_cgi = np.ascontiguousarray(g.cgrid_index - 1, np.int32)
        convert = np.ascontiguousarray(self.convert_flags(g.mech), np.int32)
        keep = [conc, man_cgi, convert, g.ta, g.qv, g.dens, g.pres, g.seaice, g.ocean_szone, g.rj, g.khetero]
        a = OracleChemArgs(g.ncols, g.nrows, g.nlays, g.nspcsd, _p(conc, C.c_float), _p(man_cgi, C.c_int),
                           _p(convert, C.c_int), _p(g.ta, C.c_float), _p(g.qv, C.c_float), _p(g.dens, C.c_float),
                           _p(g.pres, C.c_float), _p(g.seaice, C.c_float), _p(g.ocean_szone, C.c_float),
                           _p(g.rj, C.c_float), _p(g.khetero, C.c_double), tstep_sec, rtol, atol, blksize,
                           int(lreorder), max_iter, threads, 0, 0, 0)
        rc = self.lib.oracle_chem(C.byref(a))
        del keep
        return conc, {"rc": rc, "nsteps": a.nsteps_total, "nfails": a.nfails_total,
                      "nfailed_blocks": a.nfailed_blocks}

    def chem_ebi(self, g, tstep_sec: int = 300, max_iter: int = 10000000, threads: int = 0, conc=None):
        """One EBI CHEM call (hrdriver.F / hrsolver.F) on a GridInputs-like object."""
        conc = np.array(g.conc if conc is None else conc, dtype=np.float32, order="C", copy=True)
        man_cgi = np.ascontiguousarray(g.cgrid_index - 1, np.int32)
        convert = np.ascontiguousarray(self.convert_flags(g.mech), np.int32)
        keep = [conc, man_cgi, convert]
        a = OracleChemArgs(g.ncols, g.nrows, g.nlays, g.nspcsd, _p(conc, C.c_float), _p(man_cgi, C.c_int),
                           _p(convert, C.c_int), _p(g.ta, C.c_float), _p(g.qv, C.c_float), _p(g.dens, C.c_float),
                           _p(g.pres, C.c_float), _p(g.seaice, C.c_float), _p(g.ocean_szone, C.c_float),
                           _p(g.rj, C.c_float), _p(g.khetero, C.c_double), tstep_sec, 0.0, 0.0, 1, 0, max_iter,
                           threads, 0, 0, 0)
        rc = self.lib.oracle_chem_ebi(C.byref(a))
        del keep
        return conc, {"rc": rc, "iterations": a.nsteps_total, "nfailed": a.nfailed_blocks}

    def ebi_solve_cells(self, yc, rki, tstep_sec: int = 300, threads: int = 0):
        """EBI (HRSOLVER) for cells with given yc [nspec, n] (mechanism order) and rki [nrxns, n]."""
        yc = np.array(yc, dtype=np.float64, order="C", copy=True)
        rki = np.ascontiguousarray(rki, np.float64)
        n = yc.shape[1]
        st = np.zeros(n, np.int32)
        it = np.zeros(n, np.int64)
        self.lib.oracle_ebi_solve_cells(n, tstep_sec, _p(yc, C.c_double), _p(rki, C.c_double), _p(st, C.c_int),
                                        it.ctypes.data_as(C.POINTER(C.c_long)), threads)
        return yc, st, it

    # ---- SMVGEAR (CCTM/src/gas/smvgear)

    GEAR_STATS = ("nsteps", "ncfail", "nefail", "npderiv", "nsubfun", "nnewt", "maxord", "status")

    def gear_cfg(self, rtol: float = float(np.float32(1e-3)), max_atol: float = 1e-7, min_atol: float = 1e-9,
                 conc_floor: float = 1e-12, max_iter: int = 100000):
        """Tolerances and Gear coefficients: rtol = REAL(GEAR_RTOL, 8); the three others are the
        REAL(4) run-time settings GEAR_MAX_ATOL, GEAR_MIN_ATOL, GEAR_CONC_FLOOR (ppmV)."""
        buf = C.create_string_buffer(self.lib.oracle_gear_cfg_size())
        self.lib.oracle_gear_cfg(rtol, max_atol, min_atol, conc_floor, max_iter, buf)
        return buf

    def gear_cells(self, y, rk, night, chemstep: float, cfg=None, threads: int = 0):
        """Per-cell SMVGEAR (BLKSIZE = 1) over chemstep minutes; y (nspec, n) solver order.
        Returns (y, stats[n, 8]) with the columns of GEAR_STATS."""
        cfg = cfg if cfg is not None else self.gear_cfg()
        y = np.array(y, dtype=np.float64, order="C", copy=True)
        rk = np.ascontiguousarray(rk, np.float64)
        night = np.ascontiguousarray(night, np.uint8)
        n = y.shape[1]
        stats = np.zeros((n, 8), np.int32)
        self.lib.oracle_gear_cells(n, chemstep, cfg, _p(y, C.c_double), _p(rk, C.c_double), _p(night, C.c_uint8),
                                   _p(stats, C.c_int), threads)
        return y, stats

    def chem_gear(self, g, tstep_sec: int = 300, blksize: int = 50, cfg=None, lreorder: bool = True,
                  threads: int = 0, conc=None):
        """One SMVGEAR CHEM call (grdriver.F) on a GridInputs-like object; returns (new conc, totals)."""
        cfg = cfg if cfg is not None else self.gear_cfg()
        conc = np.array(g.conc if conc is None else conc, dtype=np.float32, order="C", copy=True)
        man_cgi = np.ascontiguousarray(g.cgrid_index - 1, np.int32)
        convert = np.ascontiguousarray(self.convert_flags(g.mech), np.int32)
        keep = [conc, man_cgi, convert]
        a = OracleChemArgs(g.ncols, g.nrows, g.nlays, g.nspcsd, _p(conc, C.c_float), _p(man_cgi, C.c_int),
                           _p(convert, C.c_int), _p(g.ta, C.c_float), _p(g.qv, C.c_float), _p(g.dens, C.c_float),
                           _p(g.pres, C.c_float), _p(g.seaice, C.c_float), _p(g.ocean_szone, C.c_float),
                           _p(g.rj, C.c_float), _p(g.khetero, C.c_double), tstep_sec, 0.0, 0.0, blksize,
                           int(lreorder), 0, threads, 0, 0, 0)
        rc = self.lib.oracle_gear_chem(C.byref(a), cfg)
        del keep
        return conc, {"rc": rc, "nsteps": a.nsteps_total, "nfails": a.nfails_total,
                      "nfailed_blocks": a.nfailed_blocks}

    def ebi_gather(self, g):
        """The EBI driver's gather of a GridInputs-like object: (yc [nspec, n] mechanism order,
        rki [nrxns, n], night [n])."""
        conc = np.ascontiguousarray(g.conc, np.float32)
        man_cgi = np.ascontiguousarray(g.cgrid_index - 1, np.int32)
        convert = np.ascontiguousarray(self.convert_flags(g.mech), np.int32)
        a = OracleChemArgs(g.ncols, g.nrows, g.nlays, g.nspcsd, _p(conc, C.c_float), _p(man_cgi, C.c_int),
                           _p(convert, C.c_int), _p(g.ta, C.c_float), _p(g.qv, C.c_float), _p(g.dens, C.c_float),
                           _p(g.pres, C.c_float), _p(g.seaice, C.c_float), _p(g.ocean_szone, C.c_float),
                           _p(g.rj, C.c_float), _p(g.khetero, C.c_double), 300, 0.0, 0.0, 1, 0, 0, 0, 0, 0, 0)
        n = g.ncell
        yc = np.zeros((self.nspec, n))
        rki = np.zeros((self.nrxns, n))
        night = np.zeros(n, np.uint8)
        self.lib.oracle_ebi_gather(C.byref(a), _p(yc, C.c_double), _p(rki, C.c_double), _p(night, C.c_uint8))
        return yc, rki, night

    @staticmethod
    def convert_flags(mech: str) -> np.ndarray:
        import json
        man = json.loads((HERE.parent / "cmaq_gb300" / "mechs" / mech / "manifest.json").read_text())
        return np.array([1 if s["convert"] else 0 for s in man["species"]], np.int32)


def _opt(a, ct):
    return None if a is None else _p(a, ct)


class AdjointWindow:
    """Discrete adjoint of per-cell ROS3 over ``nsync`` synchronisation steps (oracle side).

    y0 [nspec, n] (solver order), rki [nrxns, n] or [nsync, nrxns, n], night [n],
    kmult [nrxns] or None, emis [nspec, n] or None."""

    def __init__(self, oracle: "Oracle", rki, night, nsync: int, chemstep: float, rtol: float, atol: float,
                 kmult=None, emis=None, hcap: int = 4096, threads: int = 0):
        self.o, self.nsync, self.chemstep, self.rtol, self.atol = oracle, nsync, chemstep, rtol, atol
        self.rki = np.ascontiguousarray(rki, np.float64)
        self.stride = 0 if self.rki.ndim == 2 else self.rki.shape[1] * self.rki.shape[2]
        self.night = np.ascontiguousarray(night, np.uint8)
        self.n = self.night.shape[0]
        self.kmult = None if kmult is None else np.ascontiguousarray(kmult, np.float64)
        self.emis = None if emis is None else np.ascontiguousarray(emis, np.float64)
        self.hcap, self.threads = hcap, threads

    def forward(self, y0):
        o, n = self.o, self.n
        y = np.array(y0, np.float64, order="C", copy=True)
        self.ck = np.zeros((self.nsync, o.nspec, n))
        self.nsteps = np.zeros((self.nsync, n), np.int32)
        self.hs = np.zeros((self.nsync, n, self.hcap))
        bad = o.lib.oracle_adj_forward(n, _p(y, C.c_double), _p(self.rki, C.c_double), self.stride,
                                       _p(self.night, C.c_uint8), _opt(self.kmult, C.c_double),
                                       _opt(self.emis, C.c_double), self.nsync, self.chemstep, self.rtol,
                                       self.atol, _p(self.ck, C.c_double), _p(self.nsteps, C.c_int),
                                       _p(self.hs, C.c_double), self.hcap, self.threads)
        if bad:
            raise RuntimeError(f"{bad} failed cell-steps in the oracle forward window")
        return y

    def backward(self, lam_end):
        o, n = self.o, self.n
        lam = np.array(lam_end, np.float64, order="C", copy=True)
        gk = np.zeros(o.nrxns)
        ge = np.zeros((o.nspec, n))
        bad = o.lib.oracle_adj_backward(n, _p(lam, C.c_double), _p(self.rki, C.c_double), self.stride,
                                        _p(self.night, C.c_uint8), _opt(self.kmult, C.c_double),
                                        _opt(self.emis, C.c_double), self.nsync, self.chemstep, self.rtol,
                                        self.atol, _p(self.ck, C.c_double), _p(self.nsteps, C.c_int),
                                        _p(gk, C.c_double), _p(ge, C.c_double), self.threads)
        if bad:
            raise RuntimeError(f"{bad} cell-steps re-ran differently in the oracle backward window")
        return lam, gk, ge

    def replay(self, y0, kmult=None, emis=None):
        """The fixed-step map of the recorded forward run at other inputs."""
        o, n = self.o, self.n
        y = np.array(y0, np.float64, order="C", copy=True)
        km = None if kmult is None else np.ascontiguousarray(kmult, np.float64)
        em = None if emis is None else np.ascontiguousarray(emis, np.float64)
        o.lib.oracle_adj_replay(n, _p(y, C.c_double), _p(self.rki, C.c_double), self.stride,
                                _p(self.night, C.c_uint8), _opt(km, C.c_double), _opt(em, C.c_double),
                                self.nsync, _p(self.nsteps, C.c_int), _p(self.hs, C.c_double), self.hcap,
                                self.threads)
        return y


def ddm3d_window(o: "Oracle", y0, rki, night, nsync: int, chemstep: float, rtol: float, atol: float, params,
                 kmult=None, emis=None, threads: int = 0, gear_cfg=None, ebi: bool = False):
    """First-order DDM-3D sensitivities (CMAQ's SOLVE_DDM3D_CHEM restated) over a window.
    params: list of ("init", species index in solver order), ("rate", reaction index) or
    ("emis", species index: the emission tendency of that species in every cell).
    gear_cfg (Oracle.gear_cfg()): the steps are SMVGEAR's and the averages its CAVEG;
    ebi: the steps are HRSOLVER's and the averages its YCDDM (no emission tendency in
    either).  Returns (y_end, s_end [nparam, nspec, n])."""
    if (gear_cfg is not None or ebi) and emis is not None:
        raise ValueError("the SMVGEAR and EBI paths have no emission tendency")
    y = np.array(y0, np.float64, order="C", copy=True)
    rki = np.ascontiguousarray(rki, np.float64)
    stride = 0 if rki.ndim == 2 else rki.shape[1] * rki.shape[2]
    night = np.ascontiguousarray(night, np.uint8)
    n = y.shape[1]
    kind = np.array([{"init": 0, "rate": 1, "emis": 2}[k] for k, _ in params], np.int32)
    idx = np.array([i for _, i in params], np.int32)
    s_end = np.zeros((len(params), o.nspec, n))
    km = None if kmult is None else np.ascontiguousarray(kmult, np.float64)
    em = None if emis is None else np.ascontiguousarray(emis, np.float64)
    bad = o.lib.oracle_ddm3d_window(n, _p(y, C.c_double), _p(rki, C.c_double), stride, _p(night, C.c_uint8),
                                    _opt(km, C.c_double), _opt(em, C.c_double), nsync, chemstep, rtol, atol,
                                    len(params),
                                    _p(kind, C.c_int), _p(idx, C.c_int), _p(s_end, C.c_double), threads,
                                    gear_cfg, int(bool(ebi)))
    if bad:
        raise RuntimeError(f"{bad} failed cell-steps in the DDM-3D window")
    return y, s_end
