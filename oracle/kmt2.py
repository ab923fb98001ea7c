"""ctypes binding of the KMT2 aqueous-chemistry oracle (test infrastructure only).

Loads ``oracle/_build/liboracle_kmt2.so`` (``oracle/kmt2_oracle.c`` with the tables of
``oracle/gen/kmt2_aq.c``), a C restatement of the kinetic core of CMAQ's KMT2 cloud
chemistry (CCTM/src/cloud/acm_ae7_kmt2: AQCHEM's set-up, the KPP rate laws, Fun,
Jac_SP, KppDecomp / KppSolve and the Rodas3 Rosenbrock integrator).  Nothing in the
product imports it.

``synthetic_cells`` gives the seeded cloudy-cell inputs of
``cmaq_gb300.synthetic.make_cloud_cells``: the AQCHEM arguments the kinetic core reads
and the state vector as Initialize maps it from the gas and aerosol arrays
(aqchem_Initialize.F90:308-421), in mixing ratios.
"""
from __future__ import annotations

import ctypes as C
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

P_TEMP2, P_PRES_PA, P_TAUCLD, P_PRCRATE, P_WCAVG, P_WTAVG, P_AIRM, P_ALFA0, P_ALFA3, P_COSZEN, P_JH2O2, P_HO, \
    P_ISPC8, P_MTPYRAC, P_PHOTO = range(15)
STATS = ("nstp", "nacc", "nrej", "nfun", "njac", "ndec", "nsol", "nsng", "ierr", "nkron")


@lru_cache(maxsize=None)
def load() -> C.CDLL:
    import sys
    sys.path.insert(0, str(HERE))
    try:
        import build as _b  # oracle/build.py
    finally:
        sys.path.pop(0)
    _b.build([])            # incremental: rebuilds the KMT2 library when its sources changed
    path = _b.kmt2_lib_path()
    lib = C.CDLL(str(path))
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
    lib.oracle_kq_sizes.argtypes = [ip]
    lib.oracle_kq_name.argtypes = [C.c_int]
    lib.oracle_kq_name.restype = C.c_char_p
    lib.oracle_kq_lu_structure.argtypes = [ip, ip, ip]
    lib.oracle_kq_setup.argtypes = [dp, dp, dp, dp, dp, dp, dp]
    lib.oracle_kq_rconst_at.argtypes = [dp, dp, dp, dp]
    lib.oracle_kq_fun.argtypes = [dp, dp, dp, dp]
    lib.oracle_kq_fun.restype = None
    lib.oracle_kq_jac.argtypes = [dp, dp, dp, dp]
    lib.oracle_kq_jac.restype = None
    lib.oracle_kq_decomp.argtypes = [dp]
    lib.oracle_kq_solve.argtypes = [dp, dp]
    lib.oracle_kq_solve.restype = None
    for name in ("oracle_kq_fun_unrolled", "oracle_kq_jac_unrolled"):
        getattr(lib, name).argtypes = [dp, dp, dp, dp]
        getattr(lib, name).restype = None
    lib.oracle_kq_decomp_unrolled.argtypes = [dp]
    lib.oracle_kq_solve_unrolled.argtypes = [dp, dp]
    lib.oracle_kq_solve_unrolled.restype = None
    lib.oracle_kq_set_rtol_scale.argtypes = [C.c_double]
    lib.oracle_kq_set_rtol_scale.restype = None
    lib.oracle_kq_cells.argtypes = [C.c_longlong, dp, dp, dp, dp, ip, C.c_int]
    lib.oracle_kq_aqchem_cells.argtypes = [C.c_longlong, dp, dp, dp, C.c_int, ip, dp, dp, dp, dp, ip, C.c_int]
    return lib


def _p(a: np.ndarray, ct=C.c_double):
    return a.ctypes.data_as(C.POINTER(ct))


class KMT2Oracle:
    def __init__(self):
        self.lib = load()
        s = (C.c_int * 8)()
        self.lib.oracle_kq_sizes(s)
        self.nvar, self.nfix, self.nreact, self.lu_nonzero, self.nb, self.nhenry, self.nparam, self.nstat = list(s)
        self.names = [self.lib.oracle_kq_name(i).decode() for i in range(self.nvar + self.nfix)]
        self.index = {n: i for i, n in enumerate(self.names)}
        icol = np.zeros(self.lu_nonzero, np.int32)
        crow = np.zeros(self.nvar + 1, np.int32)
        diag = np.zeros(self.nvar + 1, np.int32)
        self.lib.oracle_kq_lu_structure(_p(icol, C.c_int), _p(crow, C.c_int), _p(diag, C.c_int))
        self.lu_icol, self.lu_crow, self.lu_diag = icol, crow, diag
        self.lu_irow = np.repeat(np.arange(self.nvar, dtype=np.int32), np.diff(crow))

    # ------------------------------------------------------------------ pieces
    def setup(self, params, var_mix):
        params = np.ascontiguousarray(params, np.float64)
        var_mix = np.ascontiguousarray(var_mix, np.float64)
        var = np.zeros(self.nvar)
        fix = np.zeros(self.nfix)
        rconst = np.zeros(self.nreact)
        henry = np.zeros(self.nhenry)
        sc = np.zeros(8)
        rc = self.lib.oracle_kq_setup(_p(params), _p(var_mix), _p(var), _p(fix), _p(rconst), _p(henry), _p(sc))
        if rc != 0:
            raise ValueError(f"AQCHEM set-up failed ({rc})")
        keys = ("phi2", "cfactor", "stion", "gm1", "gm2", "wetfac", "delinvt", "tend")
        return var, fix, rconst, henry, dict(zip(keys, sc))

    def rconst_at(self, params, var_mix, var):
        out = np.zeros(self.nreact)
        rc = self.lib.oracle_kq_rconst_at(_p(np.ascontiguousarray(params, np.float64)),
                                          _p(np.ascontiguousarray(var_mix, np.float64)),
                                          _p(np.ascontiguousarray(var, np.float64)), _p(out))
        if rc != 0:
            raise ValueError(f"AQCHEM set-up failed ({rc})")
        return out

    def fun(self, var, fix, rconst, unrolled: bool = False):
        out = np.zeros(self.nvar)
        (self.lib.oracle_kq_fun_unrolled if unrolled else self.lib.oracle_kq_fun)(_p(np.ascontiguousarray(var, np.float64)), _p(np.ascontiguousarray(fix, np.float64)),
                               _p(np.ascontiguousarray(rconst, np.float64)), _p(out))
        return out

    def jac(self, var, fix, rconst, unrolled: bool = False):
        out = np.zeros(self.lu_nonzero)
        (self.lib.oracle_kq_jac_unrolled if unrolled else self.lib.oracle_kq_jac)(_p(np.ascontiguousarray(var, np.float64)), _p(np.ascontiguousarray(fix, np.float64)),
                               _p(np.ascontiguousarray(rconst, np.float64)), _p(out))
        return out

    def decomp(self, jvs, unrolled: bool = False):
        a = np.array(jvs, np.float64)
        ising = (self.lib.oracle_kq_decomp_unrolled if unrolled else self.lib.oracle_kq_decomp)(_p(a))
        return a, ising

    def solve(self, lu, b, unrolled: bool = False):
        x = np.array(b, np.float64)
        (self.lib.oracle_kq_solve_unrolled if unrolled else self.lib.oracle_kq_solve)(_p(np.ascontiguousarray(lu, np.float64)), _p(x))
        return x

    def dense(self, jvs):
        m = np.zeros((self.nvar, self.nvar))
        m[self.lu_irow, self.lu_icol] = jvs
        return m

    # ------------------------------------------------------------------ integration
    def cells(self, params, var_mix, threads: int = 0, rtol_scale: float = 1.0):
        """Integrate cells over their cloud time; rtol_scale multiplies the reference's
        RTOL (convergence tests only)."""
        self.lib.oracle_kq_set_rtol_scale(rtol_scale)
        params = np.ascontiguousarray(params, np.float64)
        var_mix = np.ascontiguousarray(var_mix, np.float64)
        n = params.shape[0]
        var = np.zeros((n, self.nvar))
        fix = np.zeros((n, self.nfix))
        st = np.zeros((n, self.nstat), np.int32)
        threads = threads or min(16, max(1, __import__("os").cpu_count() or 1))
        try:
            nfail = self.lib.oracle_kq_cells(n, _p(params), _p(var_mix), _p(var), _p(fix), _p(st, C.c_int), threads)
        finally:
            self.lib.oracle_kq_set_rtol_scale(1.0)
        return var, fix, st, nfail

    def aqchem(self, params, gas, aerosol, aer_index, factors, threads: int = 0):
        """The whole AQCHEM per cell (mapping, kinetic core, redistribution): params [n][15],
        gas [n][29], aerosol [n][naer * 3] (element (i, mode) at i + naer * mode), aer_index
        [31] positions of AQCHEM's surrogates in the aerosol list, factors [16] coarse
        crustal factors.  Returns (gas, aerosol, gas_wdep, aer_wdep, out [n][10], stats,
        nfail); out: HPWDEP, BETASO4, FRACTR, FRACPOA, FRACPRI, FRACSOA, MBAL(1:4)."""
        params = np.ascontiguousarray(params, np.float64)
        g = np.array(gas, np.float64, order="C", copy=True)
        a = np.array(aerosol, np.float64, order="C", copy=True)
        n = params.shape[0]
        naer = a.shape[1] // 3
        idx = np.ascontiguousarray(aer_index, np.int32)
        fac = np.ascontiguousarray(factors, np.float64)
        gw, aw = np.zeros_like(g), np.zeros_like(a)
        out = np.zeros((n, 10))
        st = np.zeros((n, self.nstat), np.int32)
        threads = threads or min(16, max(1, __import__("os").cpu_count() or 1))
        nfail = self.lib.oracle_kq_aqchem_cells(n, _p(params), _p(g), _p(a), naer, _p(idx, C.c_int), _p(fac),
                                                _p(gw), _p(aw), _p(out), _p(st, C.c_int), threads)
        return g, a, gw, aw, out, st, nfail

    # ------------------------------------------------------------------ synthetic cells
    def synthetic_cells(self, n: int, seed: int = 0, ispc8: int = 0, mtpyrac: int = 0):
        """Seeded cloudy cells (cmaq_gb300.synthetic.make_cloud_cells: the benchmark's
        inputs), params [n][15] and var_mix [n][161]."""
        import sys
        root = str(HERE.parent)
        if root not in sys.path:
            sys.path.insert(0, root)
        from cmaq_gb300.synthetic import make_cloud_cells
        return make_cloud_cells(n, seed=seed, ispc8=ispc8, mtpyrac=mtpyrac)

    def synthetic_columns(self, n: int, seed: int = 0, ispc8: int = 0, mtpyrac: int = 0):
        """Seeded AQCHEM inputs (cmaq_gb300.synthetic.make_cloud_columns): params [n][15],
        gas [n][29], aerosol [n][31 * 3], aer_index [31], factors [16]."""
        import sys
        root = str(HERE.parent)
        if root not in sys.path:
            sys.path.insert(0, root)
        from cmaq_gb300.synthetic import make_cloud_columns
        return make_cloud_columns(n, seed=seed, ispc8=ispc8, mtpyrac=mtpyrac)
