"""Seeded synthetic inputs for the chemistry operator.

CMAQ's benchmark inputs (met, photolysis, initial conditions) are external data that
are not available, so workloads use seeded synthetic fields with the benchmark's
shapes and the value distributions below.  ``numpy.random.Generator(PCG64(seed))``;
the same seed gives the same arrays on every machine.

Per column:   surface temperature U(240, 310) K with a -6.5 K/km lapse (200 K floor);
              pressure on sigma levels from 1013 to 100 hPa; solar zenith angle
              U(sza_min, sza_max) deg; photolysis J_k = Jmax_k * max(cos SZA, 0);
              OCEAN+SZONE = 0, except a fraction of columns at U(0, 1); SEAICE = 0.
Per cell:     H2O U(1e-4, 2e-2) mol/mol; density from the ideal-gas law.
Initial mixing ratios (ppmV): O3 U(10, 120) ppb; NO, NO2 log-uniform 0.01-100 ppb;
              CO U(50, 300) ppb; radicals and short-lived intermediates log-uniform
              1e-12 - 1e-10 ppm (near their quasi-steady state); other gases log-uniform 0.01-50 ppb; aerosol species
              (CGRID in ug/m3) log-uniform 1e-4 - 1 ug/m3.  Optional plume columns
              multiply NO, NO2 and VOCs by `plume_factor`.
Heterogeneous rates are zero unless `het` is set (log-uniform 1e-6 - 1e-2 1/min).

The Jmax table is a project choice of representative clear-sky values [1/min]; CMAQ
holds no J climatology in source.
"""
from __future__ import annotations

import json
from dataclasses import dataclass
from pathlib import Path

import numpy as np

MECH_DIR = Path(__file__).resolve().parent / "mechs"

# representative clear-sky maxima, 1/min (project choice)
JMAX = {
    "NO2": 0.48, "O3_O3P": 0.024, "O3_O1D": 1.8e-3, "H2O2": 4.2e-4, "NO3NO2": 9.6, "NO3NO": 1.2,
    "N2O5": 1.8e-3, "HONO": 0.096, "HNO3": 3.0e-5, "PNA": 3.0e-4, "PAN": 3.0e-5, "MEPX": 3.0e-4,
    "NTR": 1.8e-4, "FORM_R": 1.8e-3, "FORM_M": 2.7e-3, "ALD2": 2.4e-4, "ALDX": 9.0e-4, "GLYD": 6.0e-4,
    "GLY": 1.8e-3, "MGLY": 7.2e-3, "KET": 1.2e-4, "ACET": 3.0e-5, "ISPD": 1.2e-3, "HPALD": 6.0e-3,
    "CL2": 0.12, "HOCL": 0.018, "FMCL": 6.0e-4, "CLNO2": 0.018, "CLONO2_1": 1.2e-3,
    "CLONO2_2": 3.0e-3, "IC3ONO2": 1.8e-4, "ACRO": 1.8e-4,
}
JMAX_DEFAULT = 1.0e-3

RADICALS = {"O", "O1D", "OH", "HO2", "NO3", "HO", "O3P", "CL", "CLO", "ROR", "CRO", "BZO2", "TO2",
            "XLO2", "ISO2", "C2O3", "CXO3", "MEO2", "RO2", "XO2", "XO2H", "XO2N", "OPO3", "EPX2",
            "HCO3", "BENZRO2", "TOLRO2", "XYLRO2", "PAHRO2", "CAT1", "CRON", "TERPNRO2", "ECH4"}


def jmax_for(photab: str) -> float:
    name = photab.upper()
    for key in sorted(JMAX, key=len, reverse=True):
        if name.startswith(key):
            return JMAX[key]
    return JMAX_DEFAULT


def manifest(mech: str) -> dict:
    return json.loads((MECH_DIR / mech / "manifest.json").read_text())


@dataclass
class GridInputs:
    """Arrays in CMAQ's Fortran layouts, held as C-ordered numpy arrays of the reversed shape."""
    mech: str
    ncols: int
    nrows: int
    nlays: int
    nspcsd: int
    conc: np.ndarray        # (nspcsd, nlays, nrows, ncols) float32  = CONC(C, R, L, S)
    ta: np.ndarray          # (nlays, nrows, ncols) float32
    qv: np.ndarray
    dens: np.ndarray
    pres: np.ndarray
    seaice: np.ndarray      # (nrows, ncols) float32
    ocean_szone: np.ndarray
    rj: np.ndarray          # (nphotab, nlays, nrows, ncols) float32
    khetero: np.ndarray     # (nlays, nrows, ncols, nhet) float64 = KHETERO(NHET, C, R, L)
    cgrid_index: np.ndarray  # (nspec,) int32, 1-based
    seed: int

    @property
    def ncell(self) -> int:
        return self.ncols * self.nrows * self.nlays


def make_grid(mech: str = "cb6r5_ae7_aq", ncols: int = 20, nrows: int = 20, nlays: int = 10, seed: int = 2018,
              sza_range=(0.0, 100.0), plume_fraction: float = 0.0, plume_factor: float = 10.0,
              seawater_fraction: float = 0.1, het: bool = False) -> GridInputs:
    man = manifest(mech)
    rng = np.random.Generator(np.random.PCG64(seed))
    nspec = man["nspec"]
    cgi = np.array([s["cgrid_index"] for s in man["species"]], dtype=np.int32)
    nspcsd = int(cgi.max()) + 1
    ncr = ncols * nrows
    shape3 = (nlays, nrows, ncols)
    # vertical structure
    sig = (np.arange(nlays) + 0.5) / nlays
    p_hpa = 1013.0 - (1013.0 - 100.0) * sig
    z_km = 7.5 * np.log(1013.0 / p_hpa)
    tsurf = rng.uniform(240.0, 310.0, size=(nrows, ncols))
    ta = np.maximum(tsurf[None] - 6.5 * z_km[:, None, None], 200.0).astype(np.float32)
    pres = np.broadcast_to((p_hpa * 100.0)[:, None, None], shape3).astype(np.float32)
    h2o = rng.uniform(1.0e-4, 2.0e-2, size=shape3)
    qv = (h2o * 18.0153 / 28.9628).astype(np.float32)
    dens = (pres.astype(np.float64) / (287.05 * ta.astype(np.float64))).astype(np.float32)
    # photolysis
    sza = rng.uniform(sza_range[0], sza_range[1], size=(nrows, ncols))
    cosz = np.maximum(np.cos(np.deg2rad(sza)), 0.0)
    jm = np.array([jmax_for(p) for p in man["photab"]])
    rj = (jm[:, None, None, None] * cosz[None, None, :, :] * np.ones((1, nlays, 1, 1))).astype(np.float32)
    # seawater
    osz = np.zeros(ncr)
    sea_cols = rng.random(ncr) < seawater_fraction
    osz[sea_cols] = rng.uniform(0.0, 1.0, size=int(sea_cols.sum()))
    osz = osz.reshape(nrows, ncols).astype(np.float32)
    seaice = np.zeros((nrows, ncols), np.float32)
    # heterogeneous rates
    nhet = man["nhetero"]
    if het:
        khet = np.exp(rng.uniform(np.log(1e-6), np.log(1e-2), size=shape3 + (nhet,)))
    else:
        khet = np.zeros(shape3 + (nhet,))
    # concentrations
    plume = rng.random((nrows, ncols)) < plume_fraction
    conc = np.zeros((nspcsd,) + shape3, np.float32)

    def logu(lo, hi):
        return np.exp(rng.uniform(np.log(lo), np.log(hi), size=shape3))

    voc_like = {"FORM", "ALD2", "ALDX", "PAR", "ETH", "OLE", "IOLE", "ISOP", "TERP", "TOL", "XYLMN", "BENZENE",
                "ETHA", "ETOH", "MEOH", "ACET", "KET", "PRPA", "ETHY", "APIN", "NAPH", "SESQ", "CRES", "GLY",
                "GLYD", "MGLY", "ISPD", "ACRO_PRIMARY", "TOLU", "DMS", "HC3", "HC5", "HC10", "OLT", "OLI", "API",
                "LIM", "TOL", "XYM", "XYE", "BEN", "ETE", "ETH", "HCHO", "ACD", "ALD", "ACT", "MEK", "KET"}
    for s, sp in enumerate(man["species"]):
        name = sp["name"]
        if sp["convert"]:
            v = logu(1.0e-4, 1.0)                       # ug/m3
        elif name == "O3":
            v = rng.uniform(0.010, 0.120, size=shape3)
        elif name in ("NO", "NO2"):
            v = logu(1.0e-5, 0.1)
        elif name == "CO":
            v = rng.uniform(0.05, 0.30, size=shape3)
        elif name in RADICALS:
            v = logu(1.0e-12, 1.0e-10)
        else:
            v = logu(1.0e-5, 0.05) if name in voc_like else logu(1.0e-12, 0.05)
        if plume.any() and (name in ("NO", "NO2") or name in voc_like):
            v = np.where(plume[None], v * plume_factor, v)
        conc[cgi[s] - 1] = v.astype(np.float32)
    return GridInputs(mech=mech, ncols=ncols, nrows=nrows, nlays=nlays, nspcsd=nspcsd, conc=conc, ta=ta,
                      qv=qv, dens=dens, pres=np.ascontiguousarray(pres), seaice=seaice, ocean_szone=osz,
                      rj=np.ascontiguousarray(rj), khetero=np.ascontiguousarray(khet), cgrid_index=cgi,
                      seed=seed)


def subgrid(g: GridInputs, col_step: int = 1, row_step: int = 1, lay_step: int = 1) -> GridInputs:
    """Every col_step-th column, row_step-th row and lay_step-th layer of a grid, with the
    same per-cell inputs: a sample of a large grid whose cells integrate exactly as they do
    inside it (chemistry couples no cells)."""
    c, r, lv = slice(None, None, col_step), slice(None, None, row_step), slice(None, None, lay_step)
    conc = np.ascontiguousarray(g.conc[:, lv, r, c])
    _, nlays, nrows, ncols = conc.shape
    return GridInputs(mech=g.mech, ncols=ncols, nrows=nrows, nlays=nlays, nspcsd=g.nspcsd, conc=conc,
                      ta=np.ascontiguousarray(g.ta[lv, r, c]), qv=np.ascontiguousarray(g.qv[lv, r, c]),
                      dens=np.ascontiguousarray(g.dens[lv, r, c]), pres=np.ascontiguousarray(g.pres[lv, r, c]),
                      seaice=np.ascontiguousarray(g.seaice[r, c]),
                      ocean_szone=np.ascontiguousarray(g.ocean_szone[r, c]),
                      rj=np.ascontiguousarray(g.rj[:, lv, r, c]), khetero=np.ascontiguousarray(g.khetero[lv, r, c]),
                      cgrid_index=g.cgrid_index, seed=g.seed)


# --- configurations of the chemistry benchmark (CB6r5 unless stated)
CONFIGS = {
    "cpu4k": dict(ncols=20, nrows=20, nlays=10),                        # 4,000 cells
    "conus": dict(ncols=459, nrows=299, nlays=35),                      # 4,803,315 cells
    "conus_skewed": dict(ncols=459, nrows=299, nlays=35, plume_fraction=0.3),
    "adjoint350k": dict(ncols=100, nrows=100, nlays=35),
    "cracmm2_1m": dict(ncols=200, nrows=200, nlays=25, mech="cracmm2"),
}


def solver_inputs(g: GridInputs, solver):
    """Solver-level inputs of a grid on the GPU, gathered as one CHEM call does
    (rbdriver.F:460-519): y0 [ischan, n] FP64 in the solver's species order from the
    REAL(4) conversions, rki [nrxns, n] from the device CALC_RCONST, night [n] uint8."""
    import torch
    man = manifest(g.mech)
    n = g.ncell
    dev = torch.device("cuda")
    conc = torch.from_numpy(np.ascontiguousarray(g.conc.reshape(g.nspcsd, n))).to(dev)
    svol = (1.0 / torch.from_numpy(g.dens.reshape(n)).to(dev)).to(torch.float32)
    y0 = torch.empty((len(man["species"]), n), dtype=torch.float64, device=dev)
    for s, sp in enumerate(man["species"]):
        v = conc[g.cgrid_index[s] - 1]
        if sp["convert"]:
            fwd = np.float32(np.float32(1.0e-3) * np.float32(28.9628)) / np.float32(sp["molwt"])
            v = (float(np.float32(fwd)) * svol).to(torch.float32) * v
        y0[solver.iold2new[s]] = torch.clamp_min(v.to(torch.float32), 1.0e-30).to(torch.float64)
    t = {k: torch.from_numpy(np.ascontiguousarray(getattr(g, k))).to(dev)
         for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")}
    rki, sun = solver.rconst(t["conc"], t["ta"], t["qv"], t["dens"], t["pres"], t["seaice"], t["ocean_szone"],
                             t["rj"], t["khetero"])
    return y0, rki, (1 - sun).to(torch.uint8)


# ----------------------------------------------------------------------------- cloudy cells
KMT2_PARAMS = ("temp2", "pres_pa", "taucld", "prcrate", "wcavg", "wtavg", "airm", "alfa0", "alfa3", "coszen", "jh2o2",
               "ho", "ispc8", "mtpyrac", "photo")

# log10 ranges of the state as AQCHEM's Initialize maps it from GAS and AEROSOL (mol/molV)
_CLOUD_RANGES = {
    "G_SO2": (-9.5, -8), "G_HNO3": (-10.5, -9), "G_CO2": (-3.45, -3.35), "G_NH3": (-10.5, -8.5),
    "G_H2O2": (-10, -8.7), "G_O3": (-7.6, -7.2), "G_HCOOH": (-10.5, -9), "G_MHP": (-10.5, -9),
    "G_PAA": (-11, -10), "G_HCL": (-11.5, -10), "G_GLY": (-11.5, -10), "G_MGLY": (-11.5, -10),
    "G_IEPOX": (-11, -9.5), "G_NO2": (-10, -8), "G_HONO": (-11.5, -10), "G_HNO4": (-12, -10.5),
    "G_NO3": (-13.5, -12), "G_CH3O2": (-12.5, -11), "G_GCOL": (-12, -10.5), "G_CCOOH": (-10.5, -9),
    "G_HCHO": (-9.5, -8.5), "G_HO2": (-12, -10.7), "G_HCHOP": (-13, -11),
    "A_NO3AKN": (-13, -11.5), "A_NH4AKN": (-12.5, -11), "A_CLAKN": (-14, -12.5), "A_NAAKN": (-14, -12.5),
    "A_SO4AKN": (-12.5, -11), "A_PECAKN": (-13, -11.5), "A_POAAKN": (-12.5, -11), "A_PRIAKN": (-13, -11.5),
    "L_SO4MIN2": (-10, -9), "L_NO3MIN": (-10.5, -9.3), "L_NH4PLUS": (-9.8, -8.8), "L_CLMIN": (-12, -10.5),
    "L_PRIACC": (-11.5, -10), "L_NAPLUS": (-12, -10.5), "L_CAPLUS2": (-12.5, -11), "L_MGPLUS2": (-13, -11.5),
    "L_KPLUS": (-13, -11.5), "L_PECACC": (-11.5, -10.5), "L_ORGC": (-12, -10.5), "L_OXLACMIN2": (-12, -10.5),
    "L_POAACC": (-11, -9.8), "L_FEPLUS3": (-14.5, -13), "L_MNPLUS2": (-15.5, -14),
}
_CLOUD_RANGES_ISPC8 = {"G_IMAE": (-12, -10.5), "G_IHMML": (-12, -10.5), "L_IETET": (-12, -10.5),
                       "L_IEOS": (-12, -10.5), "L_DIMER": (-13, -11.5), "L_IMGA": (-13, -11.5),
                       "L_IMOS": (-13, -11.5)}


def kmt2_manifest() -> dict:
    return json.loads((Path(__file__).resolve().parent / "mechs" / "kmt2" / "manifest.json").read_text())


def make_cloud_cells(n: int, seed: int = 0, ispc8: int = 0, mtpyrac: int = 0):
    """Seeded cloudy cells for the KMT2 aqueous chemistry: (params [n][15], var_mix
    [n][161]) in the order of ``KMT2_PARAMS`` and of the KPP species.  Temperature
    268-298 K, 700-1000 hPa, liquid water 0.05-1 g/m3, cloud time 600-3600 s, half of
    the cells precipitating 0.1-5 mm/h, cloudy air mass 5e3-8e4 mol/m2, Aitken
    scavenging 1e-5-1e-3 1/s, cos(zenith) -0.5-1 with J(H2O2) 3e-7-1e-5 1/s when sunlit;
    gas and aerosol species log-uniform within the decades of ``_CLOUD_RANGES``.  REAL
    arguments of AQCHEM are rounded to float32."""
    names = kmt2_manifest()["species"]
    index = {s: i for i, s in enumerate(names)}
    rng = np.random.default_rng(seed)
    p = np.zeros((n, len(KMT2_PARAMS)))
    f32 = lambda a: a.astype(np.float32).astype(np.float64)
    col = {k: i for i, k in enumerate(KMT2_PARAMS)}
    p[:, col["temp2"]] = f32(rng.uniform(268.0, 298.0, n))
    p[:, col["pres_pa"]] = f32(rng.uniform(70000.0, 100000.0, n))
    p[:, col["taucld"]] = f32(rng.choice([600.0, 1200.0, 1800.0, 3600.0], n))
    p[:, col["prcrate"]] = f32(np.where(rng.random(n) < 0.5, rng.uniform(0.1, 5.0, n), 0.0))
    wc = rng.uniform(5e-5, 1e-3, n)
    p[:, col["wcavg"]] = f32(wc)
    p[:, col["wtavg"]] = f32(wc * rng.uniform(1.0, 1.5, n))
    p[:, col["airm"]] = f32(rng.uniform(5e3, 8e4, n))
    p[:, col["alfa0"]] = f32(10 ** rng.uniform(-5, -3, n))
    p[:, col["alfa3"]] = f32(10 ** rng.uniform(-5, -3, n))
    p[:, col["coszen"]] = f32(rng.uniform(-0.5, 1.0, n))
    p[:, col["jh2o2"]] = np.where(p[:, col["coszen"]] > 0, 10 ** rng.uniform(-6.5, -5, n), 0.0)
    p[:, col["ho"]] = 10 ** rng.uniform(-14.5, -12.5, n)
    p[:, col["ispc8"]] = ispc8
    p[:, col["mtpyrac"]] = mtpyrac
    v = np.zeros((n, int(kmt2_manifest()["nvar"])))
    ranges = dict(_CLOUD_RANGES)
    if ispc8:
        ranges.update(_CLOUD_RANGES_ISPC8)
    else:
        ranges["L_ISO3"] = (-12, -10.5)
    if mtpyrac:
        ranges["G_PYRAC"] = (-12, -10.5)
    for name, (lo, hi) in ranges.items():
        v[:, index[name]] = 10 ** rng.uniform(lo, hi, n)
    return p, v


# log10 ranges of AQCHEM's GAS and AEROSOL inputs (mol/molV; the aerosol numbers per mol of air)
_GAS_RANGES = {"SO2": (-9.5, -8), "HNO3": (-10.5, -9), "N2O5": (-12, -10.5), "CO2": (-3.45, -3.35),
               "NH3": (-10.5, -8.5), "H2O2": (-10, -8.7), "O3": (-7.6, -7.2), "FOA": (-10.5, -9), "MHP": (-10.5, -9),
               "PAA": (-11, -10), "H2SO4": (-12, -10.5), "HCL": (-11.5, -10), "GLY": (-11.5, -10),
               "MGLY": (-11.5, -10), "HO": (-14.5, -12.5), "IEPOX": (-11, -9.5), "HO2": (-12, -10.7),
               "NO2": (-10, -8), "HONO": (-11.5, -10), "HNO4": (-12, -10.5), "GCOL": (-12, -10.5),
               "CCOOH": (-10.5, -9), "HCHO": (-9.5, -8.5), "NO3RAD": (-13.5, -12), "CH3O2": (-12.5, -11),
               "HCHOP": (-13, -11)}
_AER_RANGES = {  # (surrogate, mode 0 Aitken / 1 accumulation / 2 coarse)
    ("NO3", 0): (-13, -11.5), ("NH4", 0): (-12.5, -11), ("CL", 0): (-14, -12.5), ("NA", 0): (-14, -12.5),
    ("SO4", 0): (-12.5, -11), ("EC", 0): (-13, -11.5), ("POA", 0): (-12.5, -11), ("PRI", 0): (-13, -11.5),
    ("SOA", 0): (-13, -11.5), ("NUM", 0): (10, 12), ("TRACER_AKN", 0): (-14, -12), ("PHG_AKN", 0): (-15, -13),
    ("SO4", 1): (-10, -9), ("NO3", 1): (-10.5, -9.3), ("NH4", 1): (-9.8, -8.8), ("CL", 1): (-12, -10.5),
    ("PRI", 1): (-11.5, -10), ("NA", 1): (-12, -10.5), ("CAACC", 1): (-12.5, -11), ("MGACC", 1): (-13, -11.5),
    ("KACC", 1): (-13, -11.5), ("EC", 1): (-11.5, -10.5), ("ORGC", 1): (-12, -10.5), ("POA", 1): (-11, -9.8),
    ("FEACC", 1): (-13.5, -12), ("MNACC", 1): (-14.5, -13), ("SOA", 1): (-11, -9.8), ("NUM", 1): (9, 11),
    ("TRACER_ACC", 1): (-13, -11.5), ("PHG_ACC", 1): (-14, -12.5),
    ("SO4", 2): (-11.5, -10), ("NO3", 2): (-11.5, -10.5), ("NH4", 2): (-11, -10), ("CL", 2): (-11.5, -10.5),
    ("SOILC", 2): (-11, -9.5), ("SEASC", 2): (-11.5, -10), ("ANTHC", 2): (-11, -9.5), ("NUM", 2): (7, 9),
    ("TRACER_COR", 2): (-13.5, -12), ("PHG_COR", 2): (-14.5, -13)}


def make_cloud_columns(n: int, seed: int = 0, ispc8: int = 0, mtpyrac: int = 0):
    """Seeded inputs of the whole AQCHEM (mapping, kinetics, redistribution) for n cloudy
    cells: params [n][15] as ``make_cloud_cells`` draws them (the HO row is not read: GAS
    carries HO), gas [n][29] in AQ_DATA's order, aerosol [n][31 * 3] (surrogate i of mode m
    at i + 31 * m, the surrogates in the order of the manifest's ``aerosol_surrogates``),
    the identity surrogate positions [31] and the coarse crustal factors [16] of the
    manifest."""
    man = kmt2_manifest()["aqchem"]
    gas_names, aer_names = man["gas"], man["aerosol_surrogates"]
    p, _ = make_cloud_cells(n, seed=seed, ispc8=ispc8, mtpyrac=mtpyrac)
    rng = np.random.default_rng(seed + 7919)
    g = np.zeros((n, len(gas_names)))
    ranges = dict(_GAS_RANGES)
    if ispc8:
        ranges.update({"IMAE": (-12, -10.5), "IHMML": (-12, -10.5)})
    if mtpyrac:
        ranges["PYRUV"] = (-12, -10.5)
    for name, (lo, hi) in ranges.items():
        g[:, gas_names.index(name)] = 10 ** rng.uniform(lo, hi, n)
    na = len(aer_names)
    a = np.zeros((n, na * 3))
    ar = dict(_AER_RANGES)
    if ispc8:
        ar.update({(k, 1): (-12.5, -11) for k in ("IETET", "IEOS", "DIMER", "IMGA", "IMOS")})
    else:
        ar[("ISO3", 1)] = (-12, -10.5)
    for (name, mode), (lo, hi) in ar.items():
        a[:, aer_names.index(name) + na * mode] = 10 ** rng.uniform(lo, hi, n)
    return p, g, a, np.arange(na, dtype=np.int32), np.array(man["crustal_factors"])


def hetchem_tables(mech: str = "cb6r5_ae7_aq") -> dict:
    return json.loads((Path(__file__).resolve().parent / "mechs" / mech / "hetchem.json").read_text())


# log10 ranges (ug/m3) of the aerosol species' mass per mode (Aitken, accumulation, coarse)
_AE_MASS = {"ASO4": ((-2.5, -0.5), (-1.0, 1.3), (-1.5, 0.5)), "ANO3": ((-3, -1), (-2.0, 1.0), (-2.0, 0.3)),
            "ANH4": ((-3, -1), (-1.5, 0.9), (-2.0, 0.0)), "ACL": ((-4, -2), (-3.0, 0.3), (-3.0, 0.5)),
            "ANA": ((-4, -2), (-3.0, 0.0), None), "AH2O": ((-3, -0.5), (-2.0, 1.7), (-2.0, 1.3)),
            "AH3OP": ((-7, -5), (-6.0, -2.5), (-7.0, -4.0)), "AORGH2O": (None, (-3.0, 0.5), None),
            "ASOIL": (None, None, (-1.0, 1.3)), "ACORS": (None, None, (-1.0, 1.3)), "ASEACAT": (None, None, (-2.0, 0.7))}
_AE_DEFAULT = ((-3.5, -1.5), (-3.0, 0.3), (-2.5, 0.5))
# number (#/m3) and geometric mean diameter (m) ranges, sigma_g, per mode
_AE_NUM = ((9.0, 10.7), (8.0, 9.7), (4.5, 6.5))
_AE_DG = ((0.01e-6, 0.04e-6), (0.08e-6, 0.3e-6), (1.0e-6, 4.0e-6))
_AE_SG = (1.7, 2.0, 2.2)


def make_aerosol_cells(n: int, seed: int = 0, mech: str = "cb6r5_ae7_aq"):
    """Seeded inputs of HETCHEM_RATES for n grid cells: the CGRID aerosol block ae [NAE][n]
    (float32; species mass log-uniform in the decades of ``_AE_MASS`` per mode, ug/m3; the
    number per mode log-uniform, #/m3, and the surface area of a lognormal mode with a
    geometric mean diameter in ``_AE_DG`` and sigma_g of ``_AE_SG``, m2/m3, as CGRID's
    SRF rows hold it), and met [n] float32: temperature 230-310 K, pressure 200-1013 hPa,
    relative humidity 2-100 % given as the water-vapour mass mixing ratio of the same
    saturation formula, air density of the ideal gas.  Every tenth cell is clean (all
    masses at 1e-6 of their draw)."""
    t = hetchem_tables(mech)
    rows = t["ae_rows"]
    rng = np.random.default_rng(seed)
    ae = np.zeros((len(rows), n), np.float32)
    clean = np.where(np.arange(n) % 10 == 9, 1.0e-6, 1.0)
    for s in t["species"]:
        rng_s = _AE_MASS.get(s["bulkname"], _AE_DEFAULT)
        for m in range(3):
            r = s["row"][m]
            if r < 0:
                continue
            lo, hi = rng_s[m] if rng_s[m] is not None else _AE_DEFAULT[m]
            ae[r] = (10 ** rng.uniform(lo, hi, n) * clean).astype(np.float32)
    for m in range(3):
        num = 10 ** rng.uniform(*_AE_NUM[m], n)
        dg = rng.uniform(*_AE_DG[m], n)
        ae[t["num_rows"][m]] = num.astype(np.float32)
        ae[t["srf_rows"][m]] = (np.pi * num * dg ** 2 * np.exp(2.0 * np.log(_AE_SG[m]) ** 2)).astype(np.float32)
    ta = rng.uniform(230.0, 310.0, n)
    pres = rng.uniform(20000.0, 101325.0, n)
    rh = rng.uniform(0.02, 1.0, n)
    esat = 610.94 * np.exp(17.625 * (ta - 273.15) / (ta - 273.15 + 243.04))
    e = np.minimum(rh * esat, 0.5 * pres)
    eps = 18.0153 / 28.9628
    qv = eps * e / (pres - e)
    dens = pres / (287.0 * ta)
    f = lambda a: a.astype(np.float32)
    return ae, f(ta), f(pres), f(qv), f(dens)
