"""KMT2 aqueous cloud chemistry oracle (CCTM/src/cloud/acm_ae7_kmt2), CPU only.

What pins the restatement to the reference, without a Fortran compiler to run it:
* the generator derives the Jacobian terms and the LU structure and checks them term
  for term against the reference's aqchem_Jacobian.F90 and aqchem_JacobianSP.F90
  (test_generator_matches_the_reference, skipped without the CMAQ sources);
* rate laws, Henry's law constants, the set-up's unit conversions and the initial
  charge balance against formulas restated here from the reference text, to the last
  bit where the operation order is the same (EXP and ** by the portable series both
  the oracle and the device code use, restated in tests/helpers.py);
* J against finite differences of f, the sparse LU against a dense solve;
* Rodas3 with the reference's tolerances against the same integration with RTOL
  scaled down (convergence), and the reference's step statistics' invariants.
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

from helpers import portable_exp as pexp, portable_pow as ppow

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
from kmt2 import (KMT2Oracle, P_AIRM, P_ALFA3, P_COSZEN, P_HO, P_ISPC8, P_JH2O2, P_MTPYRAC,  # noqa: E402
                  P_PRCRATE, P_PRES_PA, P_TAUCLD, P_TEMP2, P_WCAVG, P_WTAVG, STATS)
from conftest import cmaq_root  # noqa: E402

CMAQ = cmaq_root()
KMT2_DIR = CMAQ / "CCTM" / "src" / "cloud" / "acm_ae7_kmt2"
S = {n: i for i, n in enumerate(STATS)}


@pytest.fixture(scope="module")
def o():
    return KMT2Oracle()


@pytest.fixture(scope="module")
def cells(o):
    return o.synthetic_cells(24, seed=5)


def test_sizes(o):
    assert (o.nvar, o.nfix, o.nreact, o.lu_nonzero) == (161, 4, 269, 738)
    assert o.names[o.index["L_HPLUS"]] == "L_HPLUS" and o.index["L_HPLUS"] == 155
    assert o.names[o.nvar:] == ["L_H2O", "G_HO", "L_O2", "DUMMY"]
    assert (np.diff(o.lu_crow) > 0).all() and (o.lu_icol[o.lu_diag[:-1]] == np.arange(o.nvar)).all()


@pytest.mark.skipif(not KMT2_DIR.exists(), reason="CMAQ sources not available")
def test_generator_matches_the_reference_and_the_committed_tables():
    """kpp_aq.load raises unless the derived Jacobian terms and LU structure equal
    aqchem_Jacobian.F90 / aqchem_JacobianSP.F90; the committed oracle tables and device
    headers are its output."""
    from cmaq_gb300.mechgen import kpp_aq
    k = kpp_aq.load(str(CMAQ))
    assert len(k.lu_irow) == 738 and len(k.blist) == 364
    assert (ROOT / "oracle" / "gen" / "kmt2_aq.c").read_text() == kpp_aq.oracle_source(k)
    assert (ROOT / "oracle" / "gen" / "kmt2_aq_unrolled.c").read_text() == kpp_aq.unrolled_source(k)
    gen = ROOT / "cmaq_gb300" / "csrc" / "gen"
    assert (gen / "kmt2_aq_consts.cuh").read_text() == kpp_aq.device_consts(k)
    assert (gen / "kmt2_aq.cuh").read_text() == kpp_aq.device_source(k)


# ----------------------------------------------------------------------------- set-up
def _f32(x):
    return np.float32(x)


def test_henry_constants(o, cells):
    """HLCONST (hlconst.F:509-511) in REAL(4); GCOLH / CH3O2H in double; HCHOH = 2.5.
    numpy's float32 exp and libm's expf may differ by one ulp."""
    p, v = cells
    for c in range(4):
        _, _, _, henry, _ = o.setup(p[c], v[c])
        t = _f32(p[c, P_TEMP2])
        tfac = (_f32(298.0) - t) / (_f32(298.0) * t)
        so2 = _f32(1.4) * np.exp(_f32(2900.0) * tfac, dtype=np.float32)
        assert abs(henry[0] - float(so2)) <= float(np.spacing(so2))     # SO2H, the first one used
        assert henry[0] == float(np.float32(henry[0]))                  # a REAL(4) value
        td = float(t)
        gcol = 4.1e4 * pexp(4.6e3 * ((298.0 - td) / (298.0 * td)))
        assert gcol in henry
        assert 2.5 in henry


def test_setup_units_and_charge_balance(o, cells):
    """aqchem_Initialize.F90:252-288, 425-485 restated: CFACTOR, PHI2, fixed species,
    and H+ / OH- from the charge balance of the initial ions."""
    p, v = cells
    ix = o.index
    for c in range(6):
        var, fix, _, _, sc = o.setup(p[c], v[c])
        t, pres = float(_f32(p[c, P_TEMP2])), float(_f32(p[c, P_PRES_PA]))
        cfactor = pres / (t * float(np.float32(8.314510))) * 6.0221413e17
        assert sc["cfactor"] == cfactor
        lwcfrac = float(_f32(p[c, P_WCAVG])) * 1.0e-3
        phi2 = 1000.0 / 6.022e23 / lwcfrac
        assert sc["phi2"] == phi2
        delinvt = (298.0 - t) / (298.0 * t)
        assert fix[ix["L_H2O"] - o.nvar] == 55.5 * (1.0 / phi2)
        assert fix[ix["G_HO"] - o.nvar] == p[c, P_HO] * cfactor
        o2 = float(np.float32(0.21)) * (pres / 101325.0) * 1.3e-3 * pexp(1500.0 * delinvt) * (1.0 / phi2)
        assert fix[ix["L_O2"] - o.nvar] == o2
        kept = [i for i in range(o.nvar) if o.names[i] not in ("L_HPLUS", "L_OHMIN")]
        assert np.array_equal(var[kept], cfactor * v[c, kept])
        pos = 2.0 * (var[ix["L_CAPLUS2"]] + var[ix["L_MGPLUS2"]]) + var[ix["L_NAPLUS"]] + var[ix["L_KPLUS"]] \
            + var[ix["L_NH4PLUS"]]
        neg = 2.0 * (var[ix["L_SO4MIN2"]] + var[ix["L_OXLACMIN2"]]) + var[ix["L_NO3MIN"]] + var[ix["L_CLMIN"]]
        h, oh = var[ix["L_HPLUS"]] * phi2, var[ix["L_OHMIN"]] * phi2
        kw = 1.0e-14 * pexp(-6.955e3 * delinvt)
        assert abs((h + pos * phi2) - (oh + neg * phi2)) <= 1e-9 * (h + pos * phi2)
        assert abs(h * oh / kw - 1.0) < 1e-12


def test_wet_removal_and_cloud_thickness(o, cells):
    """TWASH / WETFAC_KPP (aqchem_Initialize.F90:270-280) from the cloud thickness of
    aqchem_kmt.F90:511, where AIRM * TEMP2 is a REAL(4) product."""
    p, v = cells
    for c in range(len(p)):
        _, _, rc, _, sc = o.setup(p[c], v[c])
        airm, t, pres = _f32(p[c, P_AIRM]), _f32(p[c, P_TEMP2]), float(_f32(p[c, P_PRES_PA]))
        cthk1 = float(np.float32(airm * t)) * 0.08206 / (pres / 101325.0 * 1000.0)
        prc = float(_f32(p[c, P_PRCRATE]))
        twash = float(_f32(p[c, P_WTAVG])) * 1000.0 * cthk1 * 3600.0 / (1000.0 * max(1.0e-20, prc))
        wet = 1.0 / twash if prc > 0 else 0.0
        assert sc["wetfac"] == wet
        assert rc[95] == wet and rc[268] == wet                  # RCONST(96), RCONST(269)
        assert rc[32] == float(_f32(p[c, P_ALFA3]))              # RCONST(33) = ALFA3_KPP
        assert sc["tend"] == float(_f32(p[c, P_TAUCLD]))


def _kmt(t, accom, dg, mw):
    rad = 1.6e-5 * 0.5
    v = np.sqrt(8.0 * 8.3145 * t * 1000.0 / float(np.float32(3.1415926536)) / mw)
    kmt = (rad * rad) / (3.0 * dg)
    kmt = kmt + (4.0 * rad / (3.0 * v * accom))
    return 1.0 / kmt


def test_rate_laws_set_once(o, cells):
    """KMTF / KMTB / HYDF / KPHOT / constants (aqchem_Initialize.F90:53-152, 491-636)."""
    p, v = cells
    for c in range(4):
        _, _, rc, henry, sc = o.setup(p[c], v[c])
        t = float(_f32(p[c, P_TEMP2]))
        lwc = float(_f32(p[c, P_WCAVG]))
        assert rc[0] == _kmt(t, 0.11, 1.28e-5, 64.064) * lwc / 1000.0           # RCONST(1)
        assert rc[16] == _kmt(t, 0.11, 1.28e-5, 64.064) / (0.08206 * t * henry[0])  # RCONST(17), SO2H
        assert rc[188] == 1.8e-1 * pexp(4.03e3 * sc["delinvt"]) * sc["phi2"]      # RCONST(189) HYDF
        assert rc[189] == 5.1e-3                                                 # RCONST(190)
        assert rc[91] == 1.1                                                     # RCONST(92)
        assert rc[192] == p[c, P_JH2O2]                                          # RCONST(193) KPHOT(J)
        assert rc[231] == 0.0                                                    # RCONST(232), PHOTO = 0
        assert rc[170] == 0.0 and rc[175] == 0.0                                 # MTPYRAC = 0


def test_pyruvic_acid_switch(o):
    p, v = o.synthetic_cells(2, seed=9, mtpyrac=1)
    _, _, rc, _, _ = o.setup(p[0], v[0])
    t = float(_f32(p[0, P_TEMP2]))
    assert rc[170] == 1.0 * (_kmt(t, 0.0322, 1.24e-5, 88.06) * float(_f32(p[0, P_WCAVG])) / 1000.0)


def test_rate_laws_refreshed_from_the_state(o, cells):
    """Update_RCONST (aqchem_Rates.F90:415-581): ionic strength, activity coefficients,
    DISF / DISB / KRXN / KIEPOX, restated here from the reference text."""
    p, v = cells
    ix = o.index
    for c in range(4):
        var, fix, rc, _, sc = o.setup(p[c], v[c])
        phi2, d = sc["phi2"], sc["delinvt"]
        x = lambda n: var[ix[n]]
        s = (x("L_HPLUS") + x("L_NH4PLUS") + x("L_OHMIN") + x("L_HCO3MIN") + x("L_O2MIN") + x("L_NO2MIN")
             + x("L_NO4MIN") + x("L_GLYACMIN") + x("L_OXLACMIN") + x("L_PYRACMIN") + x("L_GCOLACMIN")
             + x("L_CCOOHMIN") + x("L_HSO3MIN") + x("L_HCOOMIN") + x("L_NO3MIN") + x("L_HSO4MIN") + x("L_HMSMIN")
             + x("L_NAPLUS") + x("L_KPLUS") + x("L_CLMIN") + x("L_SO4MIN") + x("L_SO3MIN") + x("L_HMSMIN")
             + x("L_SO5MIN") + x("L_HSO5MIN") + x("L_CO2MIN") + 3.0 * x("L_FEPLUS3") + 2.0 * x("L_MNPLUS2")
             + 4.0 * (x("L_SO4MIN2") + x("L_CO3MIN2") + x("L_OXLACMIN2") + x("L_SO3MIN2") + x("L_MNPLUS2")
                      + x("L_CAPLUS2") + x("L_MGPLUS2")) + 9.0 * x("L_FEPLUS3"))
        stion = 0.5 * s * phi2
        assert sc["stion"] == stion
        lg1 = -0.509 * (np.sqrt(stion) / (1.0 + np.sqrt(stion)) - 0.2 * stion)
        assert sc["gm1"] == ppow(10.0, lg1)
        assert abs(sc["gm1"] / 10.0 ** lg1 - 1) < 1e-15
        gm1, gm2 = sc["gm1"], sc["gm2"]
        assert rc[40] == 2.0e8 * (1.39e-2 * pexp(1.87e3 * d))                   # DISF(.., 0)
        assert rc[41] == 5.0e10 * (6.72e-8 * pexp(3.55e2 * d)) * gm1            # DISF(.., 1)
        assert rc[54] == 2.0e8 * gm1 * gm1 * phi2                               # DISB(2.0D8, 2)
        assert rc[55] == 5.0e10 * gm1 * gm2 * phi2                              # DISB(5.0D10, 1)
        k = 7.45e7 * pexp(-4756.08 * d)                                         # KRXN(.., 1, 0, 0)
        assert rc[68] == (k / (1.0 + 13.0 * x("L_HPLUS") * phi2)) * phi2 * phi2
        k = 750.0 * pexp(0.0 * d)                                               # KRXN(750, 0, 0, 0, 1)
        svi = 1.0 + 75.0 * ppow((x("L_H2SO4") + x("L_HSO4MIN") + x("L_SO4MIN2")) * phi2, 0.67)
        assert rc[72] == (k / svi) * phi2
        assert rc[239] == 2.6e-2 * pexp(0.0 * d) / phi2 * phi2                  # KRXN(.., 4, 0, 0)
        assert rc[146] == 0.0 and rc[153] == 0.0                                # KIEPOX TYPE >= 1 off
        assert rc[150] > 0.0                                                    # KIEPOX TYPE 0 on (ISPC8 = 0)


def test_rates_follow_the_state(o, cells):
    """Rates refreshed from a changed state: more H+ -> larger ionic strength, smaller
    activity coefficients, smaller DISF(.., 1)."""
    p, v = cells
    var, _, rc0, _, _ = o.setup(p[0], v[0])
    var2 = var.copy()
    var2[o.index["L_HPLUS"]] *= 1e3
    var2[o.index["L_SO4MIN2"]] *= 1e3
    rc1 = o.rconst_at(p[0], v[0], var2)
    assert rc1[41] < rc0[41]
    assert np.array_equal(rc1[:40], rc0[:40])                                   # set once: unchanged


def test_isoprene_epoxide_switch(o):
    """ISPC8 = 1 switches KIEPOX from TYPE 0 to TYPE >= 1 rates."""
    p, v = o.synthetic_cells(2, seed=11, ispc8=1)
    _, _, rc, _, _ = o.setup(p[0], v[0])
    assert rc[146] > 0.0 and rc[153] > 0.0 and rc[150] == 0.0


# ----------------------------------------------------------------------------- f, J, LU
def test_jacobian_against_finite_differences(o, cells):
    p, v = cells
    rng = np.random.default_rng(3)
    for c in range(3):
        var, fix, rc, _, _ = o.setup(p[c], v[c])
        y = var * rng.uniform(0.5, 1.5, o.nvar) + 1e3
        jd = o.dense(o.jac(y, fix, rc))
        f0 = o.fun(y, fix, rc)
        for j in rng.choice(o.nvar, 40, replace=False):
            h = 1e-6 * abs(y[j])
            yp, ym = y.copy(), y.copy()
            yp[j] += h
            ym[j] -= h
            fp, fm = o.fun(yp, fix, rc), o.fun(ym, fix, rc)
            col = (fp - fm) / (2 * h)
            # the difference quotient resolves nothing below the rounding of f itself
            tol = 1e-6 * np.abs(jd[:, j]).max() + 64 * np.finfo(float).eps * np.maximum(abs(fp), abs(fm)) / (2 * h)
            assert (np.abs(col - jd[:, j]) <= tol).all(), (c, j)
        assert np.isfinite(f0).all()


def test_jacobian_pattern_is_the_lu_pattern(o, cells):
    """Every nonzero of J lies in the stored LU structure (the structure's fill-in entries
    start at zero)."""
    p, v = cells
    var, fix, rc, _, _ = o.setup(p[0], v[0])
    jvs = o.jac(var + 1.0, fix, rc)
    assert np.count_nonzero(jvs) <= 670                    # NONZERO of aqchem_Parameters.F90
    assert np.count_nonzero(jvs) > 500


def test_sparse_lu_against_dense_solve(o, cells):
    p, v = cells
    rng = np.random.default_rng(4)
    var, fix, rc, _, _ = o.setup(p[1], v[1])
    for h in (1e-3, 1.0, 60.0):
        jac = o.jac(var + 1.0, fix, rc)
        g = -jac
        g[o.lu_diag[:-1]] += 1.0 / (h * 0.5)               # ros_PrepareMatrix, gamma(1) = 0.5
        lu, ising = o.decomp(g)
        assert ising == 0
        b = rng.standard_normal(o.nvar)
        x = o.solve(lu, b)
        xd = np.linalg.solve(o.dense(g), b)
        assert np.abs(x - xd).max() <= 1e-9 * np.abs(xd).max()


def test_straight_line_routines_equal_the_tables_bit_for_bit(o, cells):
    """The generated straight-line f / J / LU / solve (the device code's form) against
    the table-driven routines: identical bits on states across the cells, including
    negative entries and zeros."""
    p, v = cells
    rng = np.random.default_rng(8)
    for c in range(6):
        var, fix, rc, _, _ = o.setup(p[c], v[c])
        y = var * rng.uniform(0.3, 3.0, o.nvar)
        y[rng.choice(o.nvar, 10, replace=False)] *= -1e-3
        assert np.array_equal(o.fun(y, fix, rc), o.fun(y, fix, rc, unrolled=True))
        jac = o.jac(y, fix, rc)
        assert np.array_equal(jac, o.jac(y, fix, rc, unrolled=True))
        g = -jac
        g[o.lu_diag[:-1]] += 1.0 / (rng.uniform(1e-3, 100.0) * 0.5)
        lu_t, s_t = o.decomp(g)
        lu_u, s_u = o.decomp(g, unrolled=True)
        assert s_t == s_u == 0 and np.array_equal(lu_t, lu_u)
        b = rng.standard_normal(o.nvar) * np.abs(y + 1.0)
        assert np.array_equal(o.solve(lu_t, b), o.solve(lu_u, b, unrolled=True))
    jvs = np.ones(o.lu_nonzero)
    jvs[o.lu_diag[40]] = 0.0
    assert o.decomp(jvs)[1] == o.decomp(jvs, unrolled=True)[1] == 41


def test_singular_pivot_is_reported(o):
    """KppDecomp returns the 1-based row whose diagonal is below TINY (checked on the
    row before its elimination, as the reference does)."""
    jvs = np.ones(o.lu_nonzero)
    jvs[o.lu_diag[7]] = 0.0
    _, ising = o.decomp(jvs)
    assert ising == 8


# ----------------------------------------------------------------------------- integration
def test_integration_finishes_with_consistent_statistics(o, cells):
    p, v = cells
    var, fix, st, nfail = o.cells(p, v)
    assert nfail == 0 and (st[:, S["ierr"]] == 1).all() and (st[:, S["nkron"]] == 1).all()
    assert np.isfinite(var).all()
    nacc, nstp = st[:, S["nacc"]], st[:, S["nstp"]]
    assert (nacc >= 1).all() and (nstp >= nacc).all()
    assert (st[:, S["njac"]] == nacc).all()                          # one Jacobian per accepted step
    assert (st[:, S["ndec"]] == nstp + st[:, S["nsng"]]).all()
    assert (st[:, S["nsol"]] == 4 * nstp).all()                     # four Rodas3 stages
    assert (st[:, S["nfun"]] == nacc + 2 * nstp).all()              # stages 3 and 4 evaluate f
    ph = -np.log10(var[:, o.index["L_HPLUS"]] * (1000.0 / 6.022e23 / (p[:, P_WCAVG].astype(np.float32) * 1e-3)))
    assert ((ph > 1.5) & (ph < 8.0)).all()


def test_threads_give_the_same_bits(o, cells):
    p, v = cells
    a = o.cells(p, v, threads=1)
    b = o.cells(p, v, threads=8)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


def test_rodas3_converges_to_the_tight_solution(o):
    """The reference's tolerances (RTOL 1e-2, 1e-3 for H2O2 / GLY / MGLY / IETET) against
    the same integration with RTOL x 1e-4: the error shrinks with the tolerance."""
    p, v = o.synthetic_cells(12, seed=21)
    ref, _, _, nf = o.cells(p, v, rtol_scale=1e-4)
    assert nf == 0
    errs = []
    for scale in (1.0, 1e-2):
        y, _, st, nf = o.cells(p, v, rtol_scale=scale)
        assert nf == 0
        big = np.abs(ref) > 1e-6 * np.abs(ref).max(axis=1, keepdims=True)
        errs.append(np.max(np.abs(y - ref)[big] / np.abs(ref)[big]))
    assert errs[1] < errs[0]
    assert errs[0] < 0.05 and errs[1] < 5e-3


def test_sulfate_production_and_gas_uptake(o, cells):
    """Chemistry sanity over the cloud time: SO2 is taken up and oxidised, sulfate grows,
    dissolved species exist only through uptake."""
    p, v = cells
    var, _, _, _ = o.cells(p, v)
    var0 = np.array([o.setup(p[c], v[c])[0] for c in range(len(p))])
    so2 = o.index["G_SO2"]
    assert (var[:, so2] < var0[:, so2]).all()
    s6 = [o.index[n] for n in ("L_SO4MIN2", "L_HSO4MIN", "L_H2SO4", "WD_H2SO4")]   # incl. wet deposition
    assert (var[:, s6].sum(axis=1) > var0[:, s6].sum(axis=1)).all()


def test_met_data_error_is_reported(o, cells):
    p, v = cells
    bad = p[:2].copy()
    bad[0, P_TEMP2] = 0.0
    var, _, st, nfail = o.cells(bad, v[:2])
    assert nfail == 1 and st[0, S["ierr"]] < 0 and st[1, S["ierr"]] == 1


def test_sunlit_and_dark_cells(o, cells):
    p, v = cells
    assert (p[:, P_COSZEN] > 0).any() and (p[:, P_COSZEN] <= 0).any()
    assert (p[:, P_PRCRATE] > 0).any() and (p[:, P_PRCRATE] == 0).any()


def test_manifest_flop_counts_match_the_generated_code():
    """The benchmark's algorithmic FLOPs (cmaq_gb300/mechs/kmt2/manifest.json) are the
    binary +, -, *, / of the generated straight-line routines (unary minus is not counted;
    the decomposition's count adds the diagonal shift of ros_PrepareMatrix, one add per
    species)."""
    import json
    import re
    man = json.loads((ROOT / "cmaq_gb300" / "mechs" / "kmt2" / "manifest.json").read_text())
    src = (ROOT / "oracle" / "gen" / "kmt2_aq_unrolled.c").read_text()
    counts = {}
    for name in ("fun", "jac", "decomp", "solve"):
        body = src.split(f"kqu_{name}(", 1)[1].split("\n}\n", 1)[0]
        body = re.sub(r"fabs\([^)]*\) < DBL_MIN", "", body)
        counts[name] = len(re.findall(r" [-+*/] ", body))
    fl = man["flops"]
    assert counts["fun"] == fl["fun"] and counts["jac"] == fl["jac"] and counts["solve"] == fl["solve"]
    assert counts["decomp"] + man["nvar"] == fl["decomp"]
    assert fl["per_attempt"] == fl["decomp"] + 4 * fl["solve"] + 2 * fl["fun"] + fl["vector"]
    assert man["species"][:2] and len(man["species"]) == man["nvar"] + man["nfix"]


@pytest.mark.skipif(not KMT2_DIR.exists(), reason="CMAQ sources not available")
def test_generator_check_catches_a_wrong_derivation():
    """The generator's comparison with Jac_SP rejects a Jacobian with one coefficient
    changed; the LU structure derived from the Jacobian pattern, fill-in included, is
    JacobianSP's."""
    from cmaq_gb300.mechgen import kpp_aq as K
    text = (KMT2_DIR / "aqchem_Function.F90").read_text()
    factors, vdot = K._function(text, 161, 269)
    blist, entries = K._derive_jacobian(factors, vdot, 161)
    lu = K._symbolic_lu(set(entries), 161)
    jac_text = (KMT2_DIR / "aqchem_Jacobian.F90").read_text()
    K._check_reference_jacobian(jac_text, 161, factors, blist, lu, entries)   # the derivation passes
    key = next(kk for kk, v in entries.items() if v)
    bad = dict(entries)
    bad[key] = [(2.0 * entries[key][0][0], entries[key][0][1])] + entries[key][1:]
    with pytest.raises(ValueError, match="Jac_SP"):
        K._check_reference_jacobian(jac_text, 161, factors, blist, lu, bad)
    pattern = set(entries)
    fill = sorted(set(zip(lu[0], lu[1])) - pattern)
    assert fill, "the mechanism has fill-in"
    sp = (KMT2_DIR / "aqchem_JacobianSP.F90").read_text()
    assert [v - 1 for v in K._int_array(sp, "LU_IROW")] == lu[0]
    assert [v - 1 for v in K._int_array(sp, "LU_ICOL")] == lu[1]


def test_cloud_cell_inputs_are_seeded_and_in_range():
    from cmaq_gb300.synthetic import KMT2_PARAMS, make_cloud_cells
    a = make_cloud_cells(50, seed=4)
    b = make_cloud_cells(50, seed=4)
    c = make_cloud_cells(50, seed=5)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and not np.array_equal(a[1], c[1])
    p, v = a
    col = {k: i for i, k in enumerate(KMT2_PARAMS)}
    assert ((p[:, col["temp2"]] >= 268) & (p[:, col["temp2"]] <= 298)).all()
    assert (p[:, col["wcavg"]] <= p[:, col["wtavg"]]).all()
    assert np.array_equal(p[:, col["temp2"]], p[:, col["temp2"]].astype(np.float32))   # REAL arguments
    assert (v >= 0).all() and (v.max(axis=1) > 3e-4).all()                             # CO2 present


# ----------------------------------------------------------------------------- the whole AQCHEM
def _aq_names():
    from cmaq_gb300.synthetic import kmt2_manifest
    m = kmt2_manifest()["aqchem"]
    return m["gas"], m["aerosol_surrogates"]


def _map_in(o, p, g, a):
    """Initialize's mapping of GAS and AEROSOL into the KPP state (aqchem_Initialize.F90:
    290-421), restated from the reference text for one cell."""
    gn, an = _aq_names()
    na = len(an)
    G = lambda s: g[gn.index(s)]
    A = lambda s, m: a[an.index(s) + na * m]
    f32 = lambda x: float(np.float32(x))
    v = np.zeros(o.nvar)
    x = o.index
    ispc8, mtpyrac = int(p[P_ISPC8]), int(p[P_MTPYRAC])
    for kpp, gas in (("G_SO2", "SO2"), ("G_CO2", "CO2"), ("G_NH3", "NH3"), ("G_H2O2", "H2O2"), ("G_O3", "O3"),
                     ("G_HCOOH", "FOA"), ("G_MHP", "MHP"), ("G_PAA", "PAA"), ("G_HCL", "HCL"), ("G_GLY", "GLY"),
                     ("G_MGLY", "MGLY"), ("G_IEPOX", "IEPOX"), ("G_NO2", "NO2"), ("G_HONO", "HONO"),
                     ("G_HNO4", "HNO4"), ("G_NO3", "NO3RAD"), ("G_CH3O2", "CH3O2"), ("G_GCOL", "GCOL"),
                     ("G_CCOOH", "CCOOH"), ("G_HCHO", "HCHO"), ("G_HO2", "HO2"), ("G_HCHOP", "HCHOP")):
        v[x[kpp]] = G(gas)
    v[x["G_HNO3"]] = G("HNO3") + 2.0 * G("N2O5")
    if ispc8:
        v[x["G_IMAE"]], v[x["G_IHMML"]] = G("IMAE"), G("IHMML")
    if mtpyrac:
        v[x["G_PYRAC"]] = G("PYRUV")
    for kpp, s in (("A_NO3AKN", "NO3"), ("A_NH4AKN", "NH4"), ("A_CLAKN", "CL"), ("A_NAAKN", "NA"),
                   ("A_SO4AKN", "SO4"), ("A_PECAKN", "EC"), ("A_POAAKN", "POA"), ("A_PRIAKN", "PRI")):
        v[x[kpp]] = A(s, 0)
    for kpp, s in (("L_SO4MIN2", "SO4"), ("L_NO3MIN", "NO3"), ("L_NH4PLUS", "NH4"), ("L_CLMIN", "CL")):
        v[x[kpp]] = A(s, 1) + A(s, 2)
    for kpp, s in (("L_PRIACC", "PRI"), ("L_NAPLUS", "NA"), ("L_CAPLUS2", "CAACC"), ("L_MGPLUS2", "MGACC"),
                   ("L_KPLUS", "KACC"), ("L_PECACC", "EC"), ("L_POAACC", "POA")):
        v[x[kpp]] = A(s, 1)
    v[x["L_ORGC"]] = f32(0.2) * A("ORGC", 1)
    v[x["L_OXLACMIN2"]] = f32(0.8) * A("ORGC", 1) / f32(np.float32(90.03) / np.float32(177.0))
    if ispc8:
        for s in ("IETET", "IEOS", "DIMER", "IMGA", "IMOS"):
            v[x["L_" + s]] = A(s, 1)
    else:
        v[x["L_ISO3"]] = A("ISO3", 1)
    v[x["L_SO4MIN2"]] = v[x["L_SO4MIN2"]] + G("H2SO4")
    return v


def test_whole_aqchem_conserves_mass_like_the_reference_checks(o):
    """aqchem_kmt.F90:919-973 warns when S, N (without NH3), NH3/NH4 or Cl change by more than
    0.5 % between the inputs and GAS + AEROSOL + wet deposition; the restatement stays far
    inside that on seeded cells, every output is non-negative, N2O5 and H2SO4 end at zero
    (moved to HNO3 and sulfate), and the scavenged fractions lie in [0, 1]."""
    for ispc8, mtpyrac in ((0, 0), (1, 1)):
        p, g, a, idx, fac = o.synthetic_columns(40, seed=61 + ispc8, ispc8=ispc8, mtpyrac=mtpyrac)
        g2, a2, gw, aw, out, st, nf = o.aqchem(p, g, a, idx, fac)
        assert nf == 0 and (st[:, S["ierr"]] == 1).all()
        assert np.abs(out[:, 6:10]).max() < 1e-2                     # percent
        assert (g2 >= 0).all() and (a2 >= 0).all() and (gw >= 0).all() and (aw >= 0).all()
        gn, _ = _aq_names()
        assert (g2[:, gn.index("N2O5")] == 0).all() and (g2[:, gn.index("H2SO4")] == 0).all()
        assert ((out[:, 2:6] >= 0) & (out[:, 2:6] <= 1)).all()
        assert (out[:, 1] >= 0).all()                                # BETASO4


def test_whole_aqchem_maps_into_the_kinetic_core_and_back(o):
    """The state AQCHEM hands the kinetic core is Initialize's mapping (restated here from
    the reference text), with GAS's HO as the fixed OH: the kinetic core on that state gives
    the same final state, so GAS(O3) = (G_O3 + L_O3) / CFACTOR and GAS(H2O2) = (G_H2O2 +
    L_H2O2) / CFACTOR (aqchem_kmt.F90:785-786) to the last bit."""
    p, g, a, idx, fac = o.synthetic_columns(6, seed=71)
    g2, a2, gw, aw, out, st, nf = o.aqchem(p, g, a, idx, fac)
    gn, an = _aq_names()
    ix = o.index
    for c in range(6):
        v = _map_in(o, p[c], g[c], a[c])
        na = len(an)
        fe_iii = 0.9 if np.float32(p[c, P_COSZEN]) <= 0 else 0.1
        soil, anth, seas = a[c, an.index("SOILC") + 2 * na], a[c, an.index("ANTHC") + 2 * na], a[c, an.index("SEASC") + 2 * na]
        # coarse crustal cations (aqchem_Initialize.F90:392-421)
        v[ix["L_NAPLUS"]] += fac[4] * seas + fac[5] * soil + fac[6] * anth
        v[ix["L_CAPLUS2"]] += fac[10] * seas + fac[11] * soil + fac[12] * anth
        v[ix["L_MGPLUS2"]] += fac[7] * seas + fac[8] * soil + fac[9] * anth
        v[ix["L_KPLUS"]] += fac[13] * seas + fac[14] * soil + fac[15] * anth
        v[ix["L_FEPLUS3"]] = 0.1 * fe_iii * (a[c, an.index("FEACC") + na] + (fac[0] * soil + fac[1] * anth))
        v[ix["L_MNPLUS2"]] = 0.5 * 1.0 * (a[c, an.index("MNACC") + na] + (fac[2] * soil + fac[3] * anth))
        pc = p[c].copy()
        pc[P_HO] = g[c, gn.index("HO")]
        var, fix, stc, nfc = o.cells(pc[None], v[None])
        _, _, _, _, sc = o.setup(pc, v)
        inv = 1.0 / sc["cfactor"]
        assert g2[c, gn.index("O3")] == (var[0, ix["G_O3"]] + var[0, ix["L_O3"]]) * inv
        assert g2[c, gn.index("H2O2")] == (var[0, ix["G_H2O2"]] + var[0, ix["L_H2O2"]]) * inv
        assert np.array_equal(stc[0], st[c])
