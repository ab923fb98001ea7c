"""ctypes binding of the HETCHEM_RATES oracle (test infrastructure only).

Loads ``oracle/_build/liboracle_hetchem_<mech>.so`` (``oracle/hetchem_oracle.c`` with the
tables of ``oracle/gen/<mech>_hetchem.h``), a C restatement of CMAQ's heterogeneous rate
constants (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F: HETCHEM_RATES with the aerosol-state
routines of AERO_DATA.F, getpar.f and aero_subs.F it calls).  Nothing in the product
imports it.
"""
from __future__ import annotations

import ctypes as C
import json
from functools import lru_cache
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
MECH = "cb6r5_ae7_aq"


@lru_cache(maxsize=None)
def tables(mech: str = MECH) -> dict:
    return json.loads((HERE.parent / "cmaq_gb300" / "mechs" / mech / "hetchem.json").read_text())


@lru_cache(maxsize=None)
def load(mech: str = MECH) -> C.CDLL:
    import sys
    sys.path.insert(0, str(HERE))
    try:
        import build as _b  # oracle/build.py
    finally:
        sys.path.pop(0)
    _b.build([])
    lib = C.CDLL(str(_b.hetchem_lib_path(mech)))
    fp, dp = C.POINTER(C.c_float), C.POINTER(C.c_double)
    lib.oracle_hetchem_rates.argtypes = [C.c_longlong, fp, fp, fp, fp, fp, dp, C.c_int]
    lib.oracle_hetchem_rates.restype = None
    lib.oracle_het_n2o5_gamma.argtypes = [fp, C.c_longlong, C.c_double, C.c_double, C.c_int]
    lib.oracle_het_n2o5_gamma.restype = C.c_double
    lib.oracle_het_crystalized.argtypes = [fp, C.c_longlong, C.c_double, C.c_int]
    lib.oracle_het_freezes.argtypes = [C.c_double, C.c_double]
    lib.oracle_het_pncom_loss.argtypes = [C.c_float, C.c_float]
    lib.oracle_het_pncom_loss.restype = C.c_double
    lib.oracle_het_moments.argtypes = [fp, C.c_longlong, dp, dp, dp]
    lib.oracle_het_moments.restype = None
    lib.oracle_het_isop_q.argtypes = [fp, C.c_longlong, C.c_double]
    lib.oracle_het_isop_q.restype = C.c_double
    return lib


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def rates(ae, ta, pres, qv, dens, threads: int = 1, mech: str = MECH) -> np.ndarray:
    """KHETERO [ncell][NHET] of cells given the CGRID aerosol block ae [NAE][ncell]
    (float32, ug/m3, #/m3, m2/m3) and met [ncell] (K, Pa, kg/kg, kg/m3)."""
    ae = _f(ae)
    n = ae.shape[1]
    assert ae.shape[0] == len(tables(mech)["ae_rows"]), ae.shape
    out = np.empty((n, len(tables(mech)["hetero"])), np.float64)
    args = [_f(x) for x in (ta, pres, qv, dens)]
    fp = C.POINTER(C.c_float)
    load(mech).oracle_hetchem_rates(n, ae.ctypes.data_as(fp), *[a.ctypes.data_as(fp) for a in args],
                                out.ctypes.data_as(C.POINTER(C.c_double)), int(threads))
    return out


def cell_piece(name: str, ae_col, *args, mech: str = MECH):
    """One cell's N2O5_GAMMA, CRYSTALIZED or wet moments from its aerosol column ae_col [NAE]."""
    col = _f(ae_col)
    p = col.ctypes.data_as(C.POINTER(C.c_float))
    L = load(mech)
    if name == "n2o5_gamma":
        return L.oracle_het_n2o5_gamma(p, 1, *args)
    if name == "crystalized":
        return bool(L.oracle_het_crystalized(p, 1, *args))
    if name == "isop_q":
        return L.oracle_het_isop_q(p, 1, *args)
    if name == "moments":
        m2, m3, de = (np.zeros(3) for _ in range(3))
        dp = C.POINTER(C.c_double)
        L.oracle_het_moments(p, 1, m2.ctypes.data_as(dp), m3.ctypes.data_as(dp), de.ctypes.data_as(dp))
        return m2, m3, de
    raise ValueError(name)
