"""Pins of the HETCHEM_RATES oracle (oracle/hetchem_oracle.c).  No reference outputs exist
for this routine here (its Fortran cannot be compiled), so its pieces are checked against
the reference's formulas restated a second time, in Python, from AEROSOL_CHEMISTRY.F,
AERO_DATA.F and getpar.f; and its tables against the generator run on the reference
text."""
import json

import numpy as np
import pytest

from conftest import ROOT, cmaq_root

h = pytest.importorskip("hetchem")   # oracle/hetchem.py
f32 = np.float32


MECHS = ("cb6r5_ae7_aq", "cracmm2")


@pytest.mark.parametrize("mech", MECHS)
def test_tables_are_the_generators_output_on_the_reference(mech):
    root = cmaq_root()
    if not (root / "CCTM").exists():
        pytest.skip("CMAQ sources not present")
    from cmaq_gb300.mechgen.hetchem import tables
    committed = json.loads((ROOT / "cmaq_gb300" / "mechs" / mech / "hetchem.json").read_text())
    assert tables(root, mech) == committed


@pytest.mark.parametrize("mech", MECHS)
def test_aerosol_block_rows_match_the_mechanisms_cgrid_indices(mech):
    t = h.tables(mech)
    man = json.loads((ROOT / "cmaq_gb300" / "mechs" / mech / "manifest.json").read_text())
    n = 0
    for s in man["species"]:   # the aerosol species the gas mechanism reads or writes
        if s["type"] == "AE":
            assert t["ae_first"] + t["ae_rows"].index(s["name"]) == s["cgrid_index"], s["name"]
            n += 1
    assert n >= 1
    assert t["hetero"] == man["hetero"]
    if mech != "cb6r5_ae7_aq":
        return
    assert t["ae_rows"][:6] == ["ASO4I", "ASO4J", "ASO4K", "ANH4I", "ANH4J", "ANH4K"]
    assert "NUMATKN" in t["ae_rows"] and "SRFCOR" in t["ae_rows"] and "ASEACAT" in t["ae_rows"]
    spc = {s["bulkname"]: s for s in t["species"]}
    assert spc["ASO4"]["density"] == 1800.0 and spc["ASO4"]["charge"] == -2 and spc["ASO4"]["molwt"] == 96.0
    assert spc["AH2O"]["no_m2wet"] and not spc["AH2O"]["tracer"] and spc["AH3OP"]["tracer"]
    assert spc["APOC"]["om"] and not spc["AEC"]["om"]


def pncom_loss_py(poc, pncom):
    """AEROSOL_CHEMISTRY.F:1539-1646: 15/16 of KOHEFF above H/C 11/3, 0 below 7/6, the
    hyperbola between, all from the REAL ratio (POC + PNCOM) / POC."""
    k = 2.5e-12
    lo, hi = float(f32(7.0) / f32(6.0)), float(f32(11.0) / f32(3.0))
    if poc <= 1e-30:
        return 0.0
    r = float((f32(poc) + f32(pncom)) / f32(poc))
    if lo < r < hi:
        return 15.0 * k / (16.0 + (hi - r) / (r - lo))
    return 15.0 / 16.0 * k if r >= hi else 0.0


@pytest.mark.parametrize("pncom", [0.0, 0.1, 0.1666, 0.2, 1.0, 2.5, 2.6667, 2.7, 10.0])
def test_pncom_loss(pncom):
    assert h.load().oracle_het_pncom_loss(1.0, pncom) == pncom_loss_py(1.0, pncom)


def _column(mech="cb6r5_ae7_aq", **mass):
    """An aerosol column of the block: every species at 1e-3 ug/m3 per present mode, then
    the given 'NAMEmode' masses; number and surface area of typical modes."""
    t = h.tables(mech)
    col = np.zeros(len(t["ae_rows"]), np.float32)
    for s in t["species"]:
        for r in s["row"]:
            if r >= 0:
                col[r] = 1e-3
    rows = {n: i for i, n in enumerate(t["ae_rows"])}
    for k, v in mass.items():
        col[rows[k]] = v
    for m, (num, dg, sg) in enumerate(((5e9, 0.02e-6, 1.7), (1e9, 0.15e-6, 2.0), (1e6, 2e-6, 2.2))):
        col[t["num_rows"][m]] = num
        col[t["srf_rows"][m]] = np.pi * num * dg ** 2 * np.exp(2 * np.log(sg) ** 2)
    return col


def _logitinv(x):
    return f32(1.0) / (f32(1.0) + np.exp(-f32(x)))


def test_n2o5_gamma_davis_aqueous():
    """Davis et al. (2008), the appendix form for aqueous particles (Eqs 6, 8, 12, A1, A2)."""
    col = _column(ASO4I=0.2, ASO4J=4.0, ANO3I=0.1, ANO3J=2.0, ANH4I=0.1, ANH4J=2.0)
    temp, rh = 295.0, 0.62
    g = h.cell_piece("n2o5_gamma", col, temp, rh, 0)
    mw = {s["bulkname"]: f32(s["molwt"]) for s in h.tables()["species"]}
    nno3 = (f32(0.1) + f32(2.0)) / mw["ANO3"]
    nso4 = (f32(0.2) + f32(4.0)) / mw["ASO4"]
    nnh4 = (f32(0.1) + f32(2.0)) / mw["ANH4"]
    nani = nno3 + nso4
    x3 = nno3 / nani
    x2 = max(f32(0), min(f32(1) - x3, nnh4 / nani - f32(1)))
    x1 = f32(1) - (x2 + x3)
    gam3 = min(_logitinv(f32(-8.10774) + f32(4.902) * f32(rh)), f32(0.0154))
    t291 = max(f32(0), f32(temp) - f32(291))
    lam2 = f32(-3.64849) + f32(9.553) * min(f32(0), f32(rh) - f32(0.46))
    lam1 = lam2 + f32(0.97579) - f32(0.20427) * t291
    want = x1 * min(_logitinv(lam1), f32(0.08585)) + x2 * min(_logitinv(lam2), f32(0.053)) + x3 * gam3
    assert g == pytest.approx(float(want), rel=2e-6)


def test_n2o5_gamma_ice_and_dry_sulfate():
    col = _column(ASO4J=8.0, ANH4J=3.0, ANO3J=0.05)
    assert h.cell_piece("n2o5_gamma", col, 250.0, 0.99, 0) == 0.02            # FREEZES: Eq 14
    assert h.load().oracle_het_freezes(250.0, 0.99) == 1
    assert h.load().oracle_het_freezes(280.0, 0.99) == 0                       # above the ice point
    # dry: CRYSTALIZED (x = NH4/cations >= 0.5, y = SO4/anions >= 0.22, RH below the CRH)
    assert h.cell_piece("crystalized", col, 0.2, 1)
    g = h.cell_piece("n2o5_gamma", col, 300.0, 0.2, 0)
    mw = {s["bulkname"]: f32(s["molwt"]) for s in h.tables()["species"]}
    nno3 = (f32(1e-3) + f32(0.05)) / mw["ANO3"]
    nso4 = (f32(1e-3) + f32(8.0)) / mw["ASO4"]
    nnh4 = (f32(1e-3) + f32(3.0)) / mw["ANH4"]
    x3 = nno3 / (nno3 + nso4)
    x2 = max(f32(0), min(f32(1) - x3, nnh4 / (nno3 + nso4) - f32(1)))
    x1 = f32(1) - (x2 + x3)
    lamd = f32(-6.13376) + f32(3.592) * f32(0.2) - f32(0.19688) * (f32(300.0) - f32(293.0))
    gamd = min(_logitinv(lamd), f32(0.0124))                                   # Eqs 9, 10, 13
    gam3 = min(_logitinv(f32(-8.10774) + f32(4.902) * f32(0.2)), f32(0.0154))
    assert g == pytest.approx(float((x1 + x2) * gamd + x3 * min(gamd, gam3)), rel=2e-6)


def test_n2o5_gamma_bertram_thornton_coarse():
    """GPARAM 5: A k2f (1 - 1 / (1 + k3/k2b [H2O]/[NO3] + k4/k2b [Cl]/[NO3])), k2f =
    beta (1 - exp(-delta [H2O])), concentrations per litre of coarse particles."""
    col = _column(AH2OK=30.0, ACLK=1.5, ANO3K=0.8)
    _, m3, _ = h.cell_piece("moments", col)
    g = h.cell_piece("n2o5_gamma", col, 290.0, 0.7, 5)
    mw = {s["bulkname"]: f32(s["molwt"]) for s in h.tables()["species"]}
    inv_vol = f32(1e-9) * (f32(6.0) / f32(3.14159265)) / f32(m3[2])
    h2o = f32(30.0) * inv_vol / mw["AH2O"]
    cl = f32(1.5) * inv_vol / mw["ACL"]
    no3 = f32(0.8) * inv_vol / mw["ANO3"]
    k2f = f32(1.15e6) - f32(1.15e6) * np.exp(-f32(0.13) * h2o)
    den = f32(0.06) * (h2o / no3) + f32(1.0) + f32(29.0) * (cl / no3)
    want = f32(3.2e-8) * k2f * (f32(1.0) - f32(1.0) / den)
    assert g == pytest.approx(float(want), rel=2e-6)


def test_wet_moments_and_diameters():
    """extract_aero, calcmoments( .true. ) and getpar restated: the wet third moment is
    6/pi 1e-9 sum(m/rho) over the mode's non-tracer species, the second moment is the
    dry one (SRF / pi) scaled by (wet/dry M3)^(2/3), then getpar's ln^2(sigma_g) =
    ln(M0)/3 + 2 ln(M3)/3 - ln(M2) (within ln^2 1.05 .. ln^2 2.5001) gives M2 again and
    D_g = (M3 / (M0 exp(4.5 ln^2 sg)))^(1/3); the effective diameter is D_g exp(1.5 ln^2 sg)."""
    t = h.tables()
    col = _column(ASO4J=3.0, AH2OJ=20.0, ANO3J=1.0)
    m2, m3, de = h.cell_piece("moments", col)
    f6pi = 6.0 / float(f32(3.14159265))
    for m in range(3):
        conc = {s["bulkname"]: max(float(col[s["row"][m]]), 1e-23) for s in t["species"] if s["row"][m] >= 0}
        dens = {s["bulkname"]: s["density"] for s in t["species"]}
        tracer = {s["bulkname"]: s["tracer"] for s in t["species"]}
        nom2 = {s["bulkname"]: s["no_m2wet"] for s in t["species"]}
        wet = sum(1e-9 * f6pi / dens[k] * v for k, v in conc.items() if not tracer[k])
        dry = sum(v / dens[k] for k, v in conc.items() if not tracer[k] and not nom2[k]) * 1e-9 * f6pi
        m0 = float(col[t["num_rows"][m]])
        m2_0 = float(col[t["srf_rows"][m]]) / float(f32(3.14159265)) * (wet / dry) ** (2 / 3)
        l2 = np.log(m0) / 3 + 2 * np.log(wet) / 3 - np.log(m2_0)
        l2 = min(max(l2, np.log(1.05) ** 2), np.log(2.5001) ** 2)
        m2_1 = np.exp(np.log(m0) / 3 + 2 * np.log(wet) / 3 - l2)
        dg = (wet / (m0 * np.exp(4.5 * l2))) ** (1 / 3)
        assert m3[m] == pytest.approx(wet, rel=1e-6)
        assert m2[m] == pytest.approx(m2_1, rel=1e-5)
        assert de[m] == pytest.approx(dg * np.exp(1.5 * l2), rel=1e-5)


def test_uptake_rates_follow_the_kinetic_limit():
    """CLNO3 on Aitken and accumulation particles, NO2 on the fine surface, GLY on the
    accumulation mode: k = 60 S / (r / D + 4 / (gamma cbar)) with the wet moments above,
    the molecular speed sqrt(8 R T / (pi M)) and the diffusivity scaled by (T/273.15)^1.75
    (101325/p)."""
    t = h.tables()
    col = _column(ASO4J=3.0, AH2OJ=20.0)
    temp, pres, qv, dens = 285.0, 90000.0, 5e-3, 1.1
    k = h.rates(col[:, None], np.array([temp]), np.array([pres]), np.array([qv]), np.array([dens]))[0]
    m2, _, de = h.cell_piece("moments", col)
    adj = (temp / 273.15) ** 1.75 * (101325.0 / pres)
    cbar_coeff = np.sqrt(8.0 * 1000.0 * 8.314510 / 3.14159265 * temp)
    lab = {n: j for j, n in enumerate(t["hetero"])}
    for j, m in (("HETERO_CLNO3_WAI", 0), ("HETERO_CLNO3_WAJ", 1)):
        cbar = cbar_coeff * 1.012739360000e-1
        want = 60 * m2[m] * np.pi / (0.5 * de[m] / (0.1014e-4 * adj) + 4.0 / 0.024 / cbar)
        assert k[lab[j]] == pytest.approx(want, rel=1e-5)
    assert k[lab["HETERO_NO2"]] == pytest.approx(60 * 1e-4 * (m2[0] + m2[1]) * np.pi, rel=1e-12)
    cbar_gly = np.sqrt(8e3 * 8.314510 / (t["gas_molwt"]["GLY"] * np.pi)) * np.sqrt(temp)
    g = 2.9e-3
    want = 60 * g * m2[1] / (4 + 0.5 * de[1] * g * cbar_gly / (0.0855e-4 * adj)) * cbar_gly * np.pi
    assert k[lab["HETERO_GLY"]] == pytest.approx(want, rel=1e-5)


def test_cracmm2_no3_ho2_uptake_and_iepox_products():
    """CRACMM2's own labels: NO3 on the Aitken and accumulation modes (gamma 1e-3) and HO2
    on the accumulation mode (gamma 0.2), k = gamma S / (4 + D_e gamma cbar / (2 D)) cbar
    pi (AEROSOL_CHEMISTRY.F:954-981, 1269-1279); ISO3NOSJ and ISO3OSJ split the IEPOX
    uptake by CRACMM's pair table (:259-273): the sulfated fraction fos is the share of the
    ASO4J pairs in sum(k_pair [nuc] [acid]) with H+ from AH3OPJ, HSO4- from the charge
    balance and sulfate less the bisulfate, and ISO3NOSJ carries 1 - fos."""
    mech = "cracmm2"
    t = h.tables(mech)
    col = _column(mech, ASO4J=4.0, AH2OJ=25.0, ANO3J=1.5, ANH4J=1.0, AH3OPJ=2e-4)
    temp, pres, qv, dens = 290.0, 95000.0, 8e-3, 1.15
    k = h.rates(col[:, None], np.array([temp]), np.array([pres]), np.array([qv]), np.array([dens]), mech=mech)[0]
    m2, _, de = h.cell_piece("moments", col, mech=mech)
    lab = {n: j for j, n in enumerate(t["hetero"])}
    inv_d = 1.0 / (0.0855e-4 * (temp / 273.15) ** 1.75 * (101325.0 / pres))

    def uptake(gamma, mw, m):
        cbar = np.sqrt(8e3 * 8.314510 / (mw * np.pi)) * np.sqrt(temp)
        return gamma * m2[m] / (4 + 0.5 * de[m] * gamma * cbar * inv_d) * cbar * np.pi

    mw = t["gas_molwt"]
    assert k[lab["HETERO_NO3"]] == pytest.approx(60 * (uptake(1e-3, mw["NO3"], 0) + uptake(1e-3, mw["NO3"], 1)),
                                                 rel=1e-5)
    assert k[lab["HETERO_HO2"]] == pytest.approx(60 * uptake(0.2, mw["HO2"], 1), rel=1e-5)
    spc = t["species"]
    conc = {s["bulkname"]: float(col[s["row"][1]]) for s in spc if s["row"][1] >= 0}
    mwa = {s["bulkname"]: s["molwt"] for s in spc}
    hplus = conc["AH3OP"] / mwa["AH3OP"] * 1e-6
    charge = -sum(s["charge"] * conc[s["bulkname"]] / s["molwt"] for s in spc
                  if s["row"][1] >= 0 and not s["tracer"])
    acid = [hplus, max(charge * 1e-6 - hplus, 0.0)]
    tot = os_ = 0.0
    for p in t["nuc_pairs"]:
        nuc = conc[p["nuc"][:-1]] / mwa[p["nuc"][:-1]] * 1e-6
        if p["idx_remove"] >= 1:
            nuc = max(nuc - acid[p["idx_remove"] - 1], 0.0)
        kc = p["kchem"] * nuc * acid[p["idx_acid"] - 1]
        tot += kc
        os_ += kc if p["prod"] == "AISO3OSJ" else 0.0
    fos = os_ / tot
    assert {p["prod"] for p in t["nuc_pairs"]} == {"AISO3NOSJ", "AISO3OSJ"}
    assert k[lab["HETERO_ISO3NOSJ"]] == pytest.approx(60 * 1e9 * (1 - fos), rel=1e-9)
    aso4j_ppm = 1e-3 * (28.9628 / dens) * 4.0 / mwa["ASO4"]
    assert k[lab["HETERO_ISO3OSJ"]] == pytest.approx(60 * 1e9 * fos / aso4j_ppm, rel=1e-6)
    assert k[lab["HETERO_IEPOX"]] > 0
