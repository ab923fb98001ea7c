"""Tables of HETCHEM_RATES (CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:282-1535) for one
mechanism, read from the reference's sources:

* the aerosol species of the mechanism: AERO_DATA.F's master list (``aerolist``,
  AERO_DATA.F:236-380: density, tracer and no_M2wet flags, charge, OM flag; minimum
  concentrations ``cm_*``) filtered by the mechanism's AE namelist
  (MECHS/<mech>/AE_<mech>.nml: molecular weights and modes), in the order ``map_aero``
  builds them (AERO_DATA.F:849-1292: master-list order);
* the CGRID rows of the aerosol block: the AE namelist expanded by mode as
  ``aero_nml_modes`` does (aero_nml_modes.F:140-300: Aitken, accumulation, coarse per
  species; NUM / SRF as NUMATKN ... SRFCOR; ACORS, ASOIL, ASEACAT, ADE_CORS without
  suffix), checked against the CGRID indices of the mechanism's aerosol species;
* KHETERO's order (RXNS_DATA_MODULE.F90: HETERO), the rate labels HETCHEM_RATES knows
  (AEROSOL_CHEMISTRY.F: NAMES_AERO_RATES, IA_*), the acid / nucleophile pairs of the
  epoxide uptake (ACID_NUC_PAIRS_AE, _AEI, _CRCM and their K_* constants), HLCONST's
  IEPOX and IMAE Henry's law constants (hlconst.F) and the gas species' molecular
  weights (SPECIES_MOLWT).

Writes ``cmaq_gb300/mechs/<mech>/hetchem.json`` (the tables), the device header
``cmaq_gb300/csrc/gen/<mech>_hetchem.cuh`` and the oracle's header
``oracle/gen/<mech>_hetchem.h``:

    python -m cmaq_gb300.mechgen.hetchem --cmaq <CMAQ checkout> [--mech cb6r5_ae7_aq]
"""
from __future__ import annotations

import argparse
import json
import re
from pathlib import Path

PKG = Path(__file__).resolve().parents[1]
REPO = PKG.parent
MODES = ("I", "J", "K")
CORS_NAMES = ("ACORS", "ASOIL", "ASEACAT", "ADE_CORS")
NUM_SUFFIX = ("ATKN", "ACC", "COR")
# the rate labels the device and oracle implement (AEROSOL_CHEMISTRY.F:967-1302)
IMPLEMENTED = ("HETERO_N2O5IJ", "HETERO_N2O5K", "HETERO_H2NO3PAIJ", "HETERO_H2NO3PBIJ", "HETERO_H2NO3PAK",
               "HETERO_H2NO3PBK", "HETERO_NO2", "HETERO_IEPOX", "HETERO_IEPOXOS", "HETERO_TETROL", "HETERO_GLY",
               "HETERO_MGLY", "HETERO_NTR2", "HETERO_CLNO3_WAI", "HETERO_CLNO3_WAJ", "HETERO_PNCOMLI",
               "HETERO_PNCOMLJ", "HETERO_NO3", "HETERO_HO2", "HETERO_N2O5I", "HETERO_N2O5J", "HETERO_ISO3NOSJ",
               "HETERO_ISO3OSJ")


def _split_args(s: str) -> list[str]:
    out, cur, q = [], "", False
    for ch in s:
        if ch == "'":
            q = not q
        if ch == "," and not q:
            out.append(cur.strip())
            cur = ""
        else:
            cur += ch
    out.append(cur.strip())
    return out


def _fbool(tok: str) -> bool:
    return tok.strip().upper() in ("T", ".TRUE.")


def _fnum(tok: str) -> float:
    return float(tok.strip().upper().replace("D", "E"))


def aerolist(cmaq: Path) -> list[dict]:
    """AERO_DATA.F's master list (spcs_list_type entries, in order)."""
    text = (cmaq / "CCTM/src/aero/aero6/AERO_DATA.F").read_text()
    conmin = _fnum(re.search(r"Real,\s*Parameter\s*::\s*conmin\s*=\s*([0-9.Ee+-]+)", text).group(1))
    cms = {}
    for m in re.finditer(r"Real,\s*Parameter\s*::\s*(cm_\w+)\(\s*n_mode\s*\)\s*=\s*\(/(.*?)/\)", text):
        vals = [v.strip() for v in m.group(2).split(",")]
        assert all(v == "conmin" for v in vals), m.group(0)
        cms[m.group(1)] = [conmin] * 3
    out = []
    for m in re.finditer(r"spcs_list_type\((.*?)\)\s*,?\s*(?:!|\n)", text):
        a = _split_args(m.group(1))
        if len(a) != 18 or not a[0].startswith("'"):
            continue
        out.append({"bulkname": a[0].strip("'").strip(), "lait": _fbool(a[1]), "lacc": _fbool(a[2]),
                    "lcor": _fbool(a[3]), "min_conc": cms[a[4]], "density": _fnum(a[5]),
                    "no_m2wet": _fbool(a[10]), "tracer": _fbool(a[11]), "charge": int(a[12]),
                    "om": _fbool(a[15])})
    n = int(re.search(r"n_aerolist\s*=\s*(\d+)", text).group(1))
    assert len(out) == n, (len(out), n)
    return out


def ae_namelist(cmaq: Path, mech: str) -> list[dict]:
    text = (cmaq / f"CCTM/src/MECHS/{mech}/AE_{mech}.nml").read_text()
    out = []
    for line in text.splitlines():
        line = line.strip()
        if not line.startswith("'"):
            continue
        a = _split_args(line.split("!")[0])
        out.append({"name": a[0].strip("'").strip(), "molwt": _fnum(a[1]),
                    "modes": [_fbool(a[2]), _fbool(a[3]), _fbool(a[4])]})
    return out


def ae_rows(nml: list[dict]) -> list[str]:
    """CGRID names of the aerosol block, aero_nml_modes' order."""
    rows = []
    for sp in nml:
        for m in range(3):
            if not sp["modes"][m]:
                continue
            if sp["name"] in ("NUM", "SRF"):
                rows.append(sp["name"] + NUM_SUFFIX[m])
            elif m == 2 and sp["name"] in CORS_NAMES:
                rows.append(sp["name"])
            else:
                rows.append(sp["name"] + MODES[m])
    return rows


def _aero_chem_text(cmaq: Path) -> str:
    return (cmaq / "CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F").read_text()


def nuc_pairs(cmaq: Path, mechname: str) -> list[dict]:
    """The epoxide acid / nucleophile pairs HETCHEM_RATES selects for this mechanism
    (AEROSOL_CHEMISTRY.F:790-808) with their rate constants."""
    text = _aero_chem_text(cmaq)
    ks = {m.group(1).upper(): _fnum(m.group(2)) for m in
          re.finditer(r"REAL\s*\(\s*8\s*\)\s*,\s*PARAMETER\s*::\s*(K_\w+)\s*=\s*([0-9.DdEe+-]+)", text)}
    up = mechname.upper()
    table = "AEI" if ("AE6I" in up or "AE7I" in up) else ("CRCM" if ("CRACMM1" in up or "CRACMM2" in up) else "AE")
    m = re.search(r"ACID_NUC_PAIRS_" + table + r"\(\s*N_NUCPAIRS_" + table + r"\s*\)\s*=\s*\(/(.*?)/\)", text,
                  re.S | re.I)
    out = []
    for e in re.finditer(r"acid_cat\((.*?)\)", m.group(1), re.I):
        a = _split_args(e.group(1))
        out.append({"parent": a[0].strip("'").strip(), "nuc": a[1].strip("'").strip(),
                    "acid": a[2].strip("'").strip(), "idx_acid": int(a[3]), "idx_remove": int(a[4]),
                    "kchem": ks[a[5].strip().upper()], "prod": a[6].strip("'").strip()})
    return out


def henry(cmaq: Path, name: str) -> tuple[float, float]:
    text = (cmaq / "CCTM/src/cloud/acm_ae7_kmt2/hlconst.F").read_text()
    m = re.search(r"DATA\s+SUBNAME\(\s*\d+\),\s*A\(\s*\d+\),\s*E\(\s*\d+\)\s*/\s*'" + name +
                  r"\s*'\s*,\s*([0-9.Ee+-]+)\s*,\s*([0-9.Ee+-]+)\s*/", text)
    return _fnum(m.group(1)), _fnum(m.group(2))


def tables(cmaq: str | Path, mech: str = "cb6r5_ae7_aq") -> dict:
    cmaq = Path(cmaq)
    man = json.loads((PKG / "mechs" / mech / "manifest.json").read_text())
    master = aerolist(cmaq)
    nml = ae_namelist(cmaq, mech)
    rows = ae_rows(nml)
    mw = {sp["name"]: sp["molwt"] for sp in nml}
    # the CGRID row of the block's first entry, from the mechanism's aerosol species
    firsts = {s["cgrid_index"] - rows.index(s["name"]) for s in man["species"] if s["type"] == "AE"}
    assert len(firsts) == 1, firsts
    ae_first = firsts.pop()
    spc = []
    for e in master:                                  # map_aero: master-list order
        names = []
        for m in range(3):
            sn = e["bulkname"] if (m == 2 and e["bulkname"] in CORS_NAMES) else e["bulkname"] + MODES[m]
            names.append(sn if sn in rows else None)
        if not any(names):
            continue
        spc.append({**e, "molwt": mw[e["bulkname"]], "names": names,
                    "row": [rows.index(n) if n else -1 for n in names]})
    find = lambda nm: next(i for i, s in enumerate(spc) if s["bulkname"] == nm or nm in s["names"])
    text = _aero_chem_text(cmaq)
    labels = re.search(r"NAMES_AERO_RATES\(\s*NUMB_AERO_RATES\s*\)\s*=[\s&]*\(/(.*?)/\)", text, re.S).group(1)
    labels = [x.strip() for x in re.findall(r"'([^']*)'", labels)]
    for h in man["hetero"]:
        assert h in labels, h
        assert h in IMPLEMENTED, f"{h}: not implemented"
    pairs = nuc_pairs(cmaq, man["mechname"])
    for p in pairs:
        p["nuc_spc"] = find(p["nuc"])
        assert p["parent"] == "IEPOX", p
        p["os"] = int(p["prod"] in ("AIEOSJ", "AISO3OSJ") or (p["prod"] == "AISO3J" and p["nuc"] == "ASO4J"))
        assert p["prod"] in ("AISO3J", "AISO3NOSJ", "AISO3OSJ"), p   # no dimer products in these tables
    gas_mw = {s["name"]: s["molwt"] for s in man["species"]}
    # INDEX1 misses give HETCHEM_RATES' defaults (AEROSOL_CHEMISTRY.F:738-800)
    mws = {"IEPOX": gas_mw.get("IEPOX", 118.1), "NO3": gas_mw.get("NO3", 62.01), "GLY": gas_mw.get("GLY", 58.04),
           "MGLY": gas_mw.get("MGLY", 72.07), "HO2": gas_mw.get("HO2", 33.0)}
    return {"mechanism": mech, "ae_rows": rows, "ae_first": ae_first, "species": spc,
            "num_rows": [rows.index("NUM" + s) for s in NUM_SUFFIX],
            "srf_rows": [rows.index("SRF" + s) for s in NUM_SUFFIX],
            "idx": {k: find(k) for k in ("ASO4", "ANO3", "ACL", "ANH4", "AH2O", "AH3OP", "APOC", "APNCOM")},
            "hetero": man["hetero"], "nuc_pairs": pairs, "gas_molwt": mws,
            "henry_iepox": list(henry(cmaq, "IEPOX"))}


def _m3fac(density: float) -> float:
    """REAL( 1.0E-9 * f6pi / density, 8 ) with f6pi = 6.0 / PI, each operation in float
    as the reference's REAL arithmetic rounds it."""
    import numpy as np
    f6pi = np.float32(6.0) / np.float32(3.14159265)
    return float(np.float32(np.float32(1.0e-9) * f6pi) / np.float32(density))


def _c_float(v: float) -> str:
    return repr(float(v)) + "f"


def _c_double(v: float) -> str:
    return repr(float(v))


def device_header(t: dict) -> str:
    """Tables for csrc/hetchem.cuh: sizes and indices as constants, the per-species data
    as the initializer of a HetTables (a __constant__ copy on the device, a host copy for
    the host build)."""
    sp = t["species"]
    o = [f"// Generated by cmaq_gb300/mechgen/hetchem.py from CCTM/src/aero/aero6 (AERO_DATA.F, "
         f"AEROSOL_CHEMISTRY.F) and MECHS/{t['mechanism']}.",
         "// Included inside the mechanism's namespace by csrc/hetchem.cuh.  Do not edit.", "#pragma once", "",
         f"constexpr int NAE = {len(t['ae_rows'])};      // CGRID rows of the aerosol block",
         f"constexpr int AE_FIRST = {t['ae_first']};  // its first row in the mechanism's CGRID (0-based)",
         f"constexpr int NSPC = {len(sp)};     // aerosol chemical species (map_aero order)",
         f"constexpr int NHET = {len(t['hetero'])};     // KHETERO rows",
         f"constexpr int NNUC = {len(t['nuc_pairs'])};      // epoxide acid / nucleophile pairs", ""]
    for k, v in t["idx"].items():
        o.append(f"constexpr int I_{k} = {v};")
    o.append("")
    o.append("enum HetKind { " + ", ".join(h.replace("HETERO_", "K_") + f" = {i}" for i, h in enumerate(IMPLEMENTED))
             + " };")
    g = t["gas_molwt"]
    o += ["", f"constexpr double MW_IEPOX = {_c_double(g['IEPOX'])}, MW_NO3 = {_c_double(g['NO3'])}, "
          f"MW_GLY = {_c_double(g['GLY'])}, MW_MGLY = {_c_double(g['MGLY'])}, MW_HO2 = {_c_double(g['HO2'])};",
          f"constexpr float HL_IEPOX_A = {_c_float(t['henry_iepox'][0])}, HL_IEPOX_E = "
          f"{_c_float(t['henry_iepox'][1])};", ""]
    o.append("struct HetTables {")
    o += ["    float density[NSPC];", "    float molwt[NSPC];", "    float min_conc[NSPC][3];",
          "    double m3fac[NSPC];   // REAL( 1.0E-9 * f6pi / density, 8 ), the factor of the moment sums",
          "    int charge[NSPC];", "    unsigned char tracer[NSPC], no_m2wet[NSPC], om[NSPC];",
          "    short row[NSPC][3];   // row in the aerosol block per mode, -1: missing",
          "    short num_row[3], srf_row[3];",
          "    int nuc_spc[NNUC], nuc_acid[NNUC], nuc_remove[NNUC], nuc_os[NNUC];",
          "    double nuc_kchem[NNUC];", "    int kind[NHET];   // HetKind of each KHETERO row", "};", ""]
    vec = lambda xs, f: "{" + ", ".join(f(x) for x in xs) + "}"
    p = t["nuc_pairs"]
    o.append("#define HET_TABLES_INIT \\")
    o.append("    {" + vec([s["density"] for s in sp], _c_float) + ", \\")
    o.append("     " + vec([s["molwt"] for s in sp], _c_float) + ", \\")
    o.append("     {" + ", ".join(vec(s["min_conc"], _c_float) for s in sp) + "}, \\")
    o.append("     " + vec([_m3fac(s["density"]) for s in sp], _c_double) + ", \\")
    o.append("     " + vec([s["charge"] for s in sp], str) + ", \\")
    for key in ("tracer", "no_m2wet", "om"):
        o.append("     " + vec([int(s[key]) for s in sp], str) + ", \\")
    o.append("     {" + ", ".join(vec(s["row"], str) for s in sp) + "}, \\")
    o.append("     " + vec(t["num_rows"], str) + ", " + vec(t["srf_rows"], str) + ", \\")
    o.append("     " + vec([x["nuc_spc"] for x in p], str) + ", " + vec([x["idx_acid"] for x in p], str) + ", "
             + vec([x["idx_remove"] for x in p], str) + ", " + vec([x["os"] for x in p], str) + ", \\")
    o.append("     " + vec([x["kchem"] for x in p], _c_double) + ", \\")
    o.append("     " + vec([h.replace("HETERO_", "K_") for h in t["hetero"]], str) + "}")
    o.append("")
    o.append("// CGRID names of the aerosol block, for reference: " + " ".join(t["ae_rows"]))
    return "\n".join(o) + "\n"


def oracle_header(t: dict) -> str:
    """The same tables as plain C arrays for oracle/hetchem_oracle.c."""
    sp = t["species"]
    o = [f"/* Generated by cmaq_gb300/mechgen/hetchem.py from CCTM/src/aero/aero6 and MECHS/{t['mechanism']}:",
         " * the aerosol species of map_aero, the CGRID aerosol block, KHETERO's labels and the epoxide",
         " * acid / nucleophile pairs.  Test infrastructure (the oracle).  Do not edit. */", "#pragma once", "",
         f"#define HO_NAE {len(t['ae_rows'])}", f"#define HO_NSPC {len(sp)}", f"#define HO_NHET {len(t['hetero'])}",
         f"#define HO_NNUC {len(t['nuc_pairs'])}", ""]
    for k, v in t["idx"].items():
        o.append(f"#define HO_{k} {v}")
    o.append("")
    arr = lambda ty, name, xs: f"static const {ty} {name}[] = {{" + ", ".join(xs) + "};"
    o.append(arr("float", "ho_density", [_c_float(s["density"]) for s in sp]))
    o.append(arr("float", "ho_molwt", [_c_float(s["molwt"]) for s in sp]))
    o.append(arr("float", "ho_min_conc", [_c_float(v) for s in sp for v in s["min_conc"]]))
    o.append(arr("int", "ho_charge", [str(s["charge"]) for s in sp]))
    o.append(arr("int", "ho_tracer", [str(int(s["tracer"])) for s in sp]))
    o.append(arr("int", "ho_no_m2wet", [str(int(s["no_m2wet"])) for s in sp]))
    o.append(arr("int", "ho_om", [str(int(s["om"])) for s in sp]))
    o.append(arr("int", "ho_row", [str(r) for s in sp for r in s["row"]]) + "   /* [spc][mode], -1: missing */")
    o.append(arr("int", "ho_num_row", [str(r) for r in t["num_rows"]]))
    o.append(arr("int", "ho_srf_row", [str(r) for r in t["srf_rows"]]))
    p = t["nuc_pairs"]
    o.append(arr("int", "ho_nuc_spc", [str(x["nuc_spc"]) for x in p]))
    o.append(arr("int", "ho_nuc_acid", [str(x["idx_acid"]) for x in p]))
    o.append(arr("int", "ho_nuc_remove", [str(x["idx_remove"]) for x in p]))
    o.append(arr("int", "ho_nuc_os", [str(x["os"]) for x in p]))
    o.append(arr("double", "ho_nuc_kchem", [_c_double(x["kchem"]) for x in p]))
    o.append(arr("char* const", "ho_hetero", ['"' + h + '"' for h in t["hetero"]]))
    g = t["gas_molwt"]
    o.append(f"static const double ho_mw_iepox = {_c_double(g['IEPOX'])}, ho_mw_gly = {_c_double(g['GLY'])}, "
             f"ho_mw_mgly = {_c_double(g['MGLY'])}, ho_mw_no3 = {_c_double(g['NO3'])}, "
             f"ho_mw_ho2 = {_c_double(g['HO2'])};")
    o.append(f"static const float ho_hl_iepox_a = {_c_float(t['henry_iepox'][0])}, ho_hl_iepox_e = "
             f"{_c_float(t['henry_iepox'][1])};")
    return "\n".join(o) + "\n"


def write(cmaq: str | Path, mech: str = "cb6r5_ae7_aq") -> dict:
    t = tables(cmaq, mech)
    (PKG / "mechs" / mech / "hetchem.json").write_text(json.dumps(t, indent=1) + "\n")
    (PKG / "csrc" / "gen" / f"{mech}_hetchem.cuh").write_text(device_header(t))
    (REPO / "oracle" / "gen" / f"{mech}_hetchem.h").write_text(oracle_header(t))
    return t


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--cmaq", required=True, help="CMAQ source checkout")
    ap.add_argument("--mech", default="cb6r5_ae7_aq")
    a = ap.parse_args(argv)
    t = write(a.cmaq, a.mech)
    print(a.mech, "aerosol rows", len(t["ae_rows"]), "species", len(t["species"]), "KHETERO", len(t["hetero"]),
          "first row", t["ae_first"])


if __name__ == "__main__":
    main()
