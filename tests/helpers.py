"""Shared helpers of the test suite: oracle-side gathers and GPU runs of one CHEM call."""
from __future__ import annotations

import numpy as np

from cmaq_gb300.synthetic import GridInputs, manifest

F32 = np.float32


def gather_cells(g: GridInputs, o, gear: bool = False):
    """Per-cell inputs gathered like rbdriver.F:460-511 (REAL(4) arithmetic), cells in CGRID order.
    gear: SMVGEAR's REAL(8) concentration floor (grdriver.F:419-422) instead of ROS3's REAL(4) one.

    Returns y [nspec, n] (solver species order), rki [nrxns, n], night [n] via the oracle's CALC_RCONST."""
    man = manifest(g.mech)
    n = g.ncell
    conc = g.conc.reshape(g.nspcsd, n)
    dens = g.dens.reshape(n)
    svol = (F32(1.0) / dens).astype(F32)
    y = np.zeros((o.nspec, n))
    for s, sp in enumerate(man["species"]):
        v = conc[g.cgrid_index[s] - 1]
        if sp["convert"]:
            fwd = F32(F32(1.0e-3) * F32(28.9628)) / F32(sp["molwt"])
            v = (F32(fwd) * svol).astype(F32) * v
        if gear:
            y[o.iold2new[s]] = np.maximum(v.astype(F32).astype(np.float64), 1.0e-30)
        else:
            y[o.iold2new[s]] = np.maximum(v.astype(F32), F32(1.0e-30)).astype(np.float64)
    temp = g.ta.reshape(n).astype(np.float64)
    pres = (F32(F32(1.0) / F32(101325.0)) * g.pres.reshape(n)).astype(F32).astype(np.float64)
    qv2ppm = F32(F32(1.0e6) * F32(F32(28.9628) / F32(18.0153)))
    h2o = np.maximum((qv2ppm * g.qv.reshape(n)).astype(F32), F32(0.0)).astype(np.float64)
    col = np.arange(n) % (g.ncols * g.nrows)
    sea = np.maximum(F32(0.0), (g.ocean_szone.reshape(-1) - g.seaice.reshape(-1)).astype(F32))[col].astype(np.float64)
    rj = g.rj.reshape(o.nphotab, n).astype(np.float64)
    het = g.khetero.reshape(n, -1).T.astype(np.float64)
    sun = (rj > 0).any(axis=0)
    rki = np.zeros((o.nrxns, n))
    for lit in (True, False):
        idx = np.where(sun == lit)[0]
        if len(idx):
            rki[:, idx] = o.rconst(temp[idx], pres[idx], h2o[idx], rj[:, idx], het[:, idx], lit, sea[idx])
    return y, rki, (~sun).astype(np.uint8)


def to_cuda(g: GridInputs):
    import torch
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).cuda()
         for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")}
    return t


def gpu_chem(g: GridInputs, schedule="static", rtol=1e-3, atol=1e-9, tstep=(10000, 500, 500), nsteps=1,
             solver=None):
    """Run nsteps CHEM calls on the GPU; returns (conc numpy, stats list, solver)."""
    from cmaq_gb300.chem import ChemSolver
    t = to_cuda(g)
    s = solver or ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                             cgrid_index=g.cgrid_index, rtol=rtol, atol=atol, schedule=schedule)
    stats = []
    for _ in range(nsteps):
        stats.append(s.step(t["conc"], t["ta"], t["qv"], t["dens"], t["pres"], t["seaice"], t["ocean_szone"],
                            t["rj"], t["khetero"], tstep=tstep))
    return t["conc"].cpu().numpy(), stats, s


def rel_err(a, b, floor=1e-10):
    """Max relative difference over entries where either value exceeds `floor` (ppmV)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    m = (np.abs(a) > floor) | (np.abs(b) > floor)
    if not m.any():
        return 0.0
    return float(np.max(np.abs(a[m] - b[m]) / np.maximum(np.abs(b[m]), floor)))


def writeback(g: GridInputs, o, y):
    """CONC after a CHEM call whose per-cell solver results are y [nspec, n] (solver order):
    the REAL(4) write-back of rbdriver.F:577-595 / grdriver.F:577-596."""
    man = manifest(g.mech)
    n = g.ncell
    out = g.conc.reshape(g.nspcsd, n).copy()
    dens = g.dens.reshape(n).astype(np.float64)
    for s, sp in enumerate(man["species"]):
        v = y[o.iold2new[s]]
        if sp["convert"]:
            fwd = F32(F32(F32(1.0e-3) * F32(28.9628)) / F32(sp["molwt"]))
            v = (np.float64(F32(1.0) / fwd) * dens) * v
        out[g.cgrid_index[s] - 1] = v.astype(F32)
    return out.reshape(g.conc.shape)


def _fma(a: float, b: float, c: float) -> float:
    """a * b + c rounded once (exact rational arithmetic, then one round to nearest)."""
    from fractions import Fraction
    return float(Fraction(a) * Fraction(b) + Fraction(c))


_h = float.fromhex
_EXP_SERIES = [_h("0x1.6124613a86d09p-33"), _h("0x1.1eed8eff8d898p-29"), _h("0x1.ae64567f544e4p-26"), _h("0x1.27e4fb7789f5cp-22"),
               _h("0x1.71de3a556c734p-19"), _h("0x1.a01a01a01a01ap-16"), _h("0x1.a01a01a01a01ap-13"), _h("0x1.6c16c16c16c17p-10"),
               _h("0x1.1111111111111p-7"), _h("0x1.5555555555555p-5"), _h("0x1.5555555555555p-3"), 0.5, 1.0, 1.0]
_LOG_SERIES = [_h("0x1.642c8590b2164p-5"), _h("0x1.8618618618618p-5"), _h("0x1.af286bca1af28p-5"), _h("0x1.e1e1e1e1e1e1ep-5"),
               _h("0x1.1111111111111p-4"), _h("0x1.3b13b13b13b14p-4"), _h("0x1.745d1745d1746p-4"), _h("0x1.c71c71c71c71cp-4"),
               _h("0x1.2492492492492p-3"), _h("0x1.999999999999ap-3"), _h("0x1.5555555555555p-2"), 1.0]
_LN2_HI, _LN2_LO = _h("0x1.62e42fee00000p-1"), _h("0x1.a39ef35793c76p-33")


def portable_exp(t: float) -> float:
    """exp(t) of the oracle's portable series (t = n ln2 + r, Cody-Waite split of ln 2,
    Taylor series to r^13), restated in Python with exact fused multiply-adds: the bits
    the oracle and the device code compute."""
    import math
    t = float(t)
    if t > 709.0:
        return math.inf
    if t < -745.0:
        return 0.0
    n = float(round(t * _h("0x1.71547652b82fep+0")))   # round half to even, as rint
    r = _fma(-n, _LN2_LO, _fma(-n, _LN2_HI, t))
    e = _EXP_SERIES[0]
    for c in _EXP_SERIES[1:]:
        e = _fma(e, r, c)
    return math.ldexp(e, int(n))


def portable_pow(x: float, y: float) -> float:
    """x**y of the oracle's portable series (log by 2 atanh(s) to s^23 after x = m 2^k),
    restated in Python like portable_exp."""
    import math
    x, y = float(x), float(y)
    if not x > 0.0:
        return 0.0 if x == 0.0 else x
    if math.isinf(x):
        return x
    m, k = math.frexp(x)
    if m < _h("0x1.6a09e667f3bcdp-1"):
        m, k = m * 2.0, k - 1
    s = (m - 1.0) / (m + 1.0)
    z = s * s
    p = _LOG_SERIES[0]
    for c in _LOG_SERIES[1:]:
        p = _fma(p, z, c)
    lx = _fma(float(k), _LN2_HI, _fma(float(k), _LN2_LO, (2.0 * s) * p))
    return portable_exp(y * lx)
