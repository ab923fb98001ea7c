"""Parse a CMAQ mechanism table module (``RXNS_DATA_MODULE.F90``).

The table module is machine-written by CMAQ's ``chemmech`` generator and uses a
small, regular subset of Fortran: ``PARAMETER`` constants, implied-do ``DATA``
statements over reaction or species indices, per-element ``DATA`` statements for
species attributes and one ``SPECIES_LIST`` constructor.  This module reads that
subset and returns plain Python lists with 1-based Fortran indices translated to
0-based ones where noted.

Reference layout (cb6r5_ae7_aq):
  * species names / weights      CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90:413-561
  * CGRID index / type / convert CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_DATA_MODULE.F90:564-712
  * KTYPE / IRXBITS              RXNS_DATA_MODULE.F90:949-1000
  * IRR (reactants + products)   RXNS_DATA_MODULE.F90:1166-1796
  * SC / NREACT / NPRDCT         RXNS_DATA_MODULE.F90:2054-2140
  * IPH / IHETERO / PHOTAB       RXNS_DATA_MODULE.F90:923-945, 3141-3175
  * third-body lists NRXW*       RXNS_DATA_MODULE.F90:1125-1163
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

_NUM = r"[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[DdEe][-+]?\d+)?"


def fnum(tok: str) -> float:
    """Fortran real literal -> float (``1.0D-3`` -> 0.001)."""
    return float(tok.replace("D", "E").replace("d", "e"))


def join_continuations(text: str) -> list[str]:
    """Return logical statements: strip ``!`` comments and join ``&`` lines."""
    out: list[str] = []
    cur = ""
    for raw in text.splitlines():
        line = raw
        # strip comments outside string literals
        in_str = None
        cut = len(line)
        for i, ch in enumerate(line):
            if in_str:
                if ch == in_str:
                    in_str = None
            elif ch in ("'", '"'):
                in_str = ch
            elif ch == "!":
                cut = i
                break
        line = line[:cut].rstrip()
        s = line.strip()
        if not s:
            continue
        if s.startswith("&"):
            s = s[1:].strip()
        cont = s.endswith("&")
        if cont:
            s = s[:-1].rstrip()
        cur = (cur + " " + s) if cur else s
        if not cont:
            out.append(cur)
            cur = ""
    if cur:
        out.append(cur)
    return out


@dataclass
class Mechanism:
    name: str
    nspec: int
    nrxns: int
    species: list[str] = field(default_factory=list)
    molwt: list[float] = field(default_factory=list)
    cgrid_index: list[int] = field(default_factory=list)      # 1-based CGRID slot
    species_type: list[str] = field(default_factory=list)
    convert_conc: list[bool] = field(default_factory=list)
    irr: list[list[int]] = field(default_factory=list)         # [rxn][3+mxprd], 1-based species, 0 = none
    sc: list[list[float]] = field(default_factory=list)        # [rxn][mxprd]
    nreact: list[int] = field(default_factory=list)
    nprdct: list[int] = field(default_factory=list)
    ktype: list[int] = field(default_factory=list)
    irxbits: list[int] = field(default_factory=list)
    mxprd: int = 0
    nphotab: int = 0
    photab: list[str] = field(default_factory=list)
    nhetero: int = 0
    hetero: list[str] = field(default_factory=list)
    iph: list[tuple[int, int, int]] = field(default_factory=list)
    ihetero: list[tuple[int, int]] = field(default_factory=list)
    third_body: dict[str, list[int]] = field(default_factory=dict)  # 'M','O2','N2','H2O','H2','CH4' -> 1-based rxns
    third_body_conc: dict[str, float] = field(default_factory=dict)
    rxlabel: list[str] = field(default_factory=list)
    nspecial_rxn: int = 0
    rtdat: list[list[float]] = field(default_factory=list)   # [rxn][3]
    rfdat: list[list[float]] = field(default_factory=list)   # [falloff][5]
    irrfall: list[int] = field(default_factory=list)          # 1-based reactions
    iorder: list[int] = field(default_factory=list)
    kunits: int = 0


_TB = {"NRXWM": "M", "NRXWO2": "O2", "NRXWN2": "N2", "NRXWW": "H2O", "NRXWH2": "H2", "NRXWCH4": "CH4"}
_TB_CONC = {"ATM_AIR": "M", "ATM_O2": "O2", "ATM_N2": "N2", "ATM_CH4": "CH4", "ATM_H2": "H2"}


def _values(blob: str) -> list[str]:
    """Split the value list of a DATA statement into tokens (strings kept quoted)."""
    toks: list[str] = []
    for m in re.finditer(r"'[^']*'|[^,\s][^,]*", blob):
        t = m.group(0).strip()
        if t:
            toks.append(t)
    return toks


def parse_rxns_data(text: str) -> Mechanism:
    stmts = join_continuations(text)
    params: dict[str, str] = {}
    arrays: dict[str, dict] = {}
    per_elem: dict[str, dict[int, str]] = {}
    member_list: list[tuple] = []
    index_vars: dict[str, int] = {}

    re_param = re.compile(r"^(INTEGER|REAL\s*\(\s*8\s*\)|CHARACTER\s*\(\s*\d+\s*\)|LOGICAL)\s*,\s*PARAMETER\s*::\s*(\w+)\s*=\s*(.+)$", re.I)
    re_idx_var = re.compile(r"^INTEGER\s*::\s*(INDEX_\w+)\s*=\s*(\d+)\s*$", re.I)
    # DATA ( NAME( IRXXN [, k] | k, IRXXN ), IRXXN = 1, N ) / values /
    re_impl = re.compile(r"^DATA\s*\(\s*(\w+)\s*\(([^)]*)\)\s*,\s*IRXXN\s*=\s*1\s*,\s*(\w+)\s*\)\s*/(.*)/\s*$", re.I)
    # DATA A( i ), B( i ) [, C( i )] / v1, v2 [, v3] /
    re_elem = re.compile(r"^DATA\s+((?:\w+\s*\(\s*\d+\s*\)\s*,?\s*)+)/(.*)/\s*$", re.I)
    re_member = re.compile(r'MEMBER\(\s*"([^"]*)"\s*,\s*(-?\d+)\s*,\s*"([^"]*)"\s*,\s*(' + _NUM + r')\s*,\s*([TF])\s*\)')

    for st in stmts:
        m = re_param.match(st)
        if m:
            params[m.group(2).upper()] = m.group(3).strip()
            continue
        m = re_idx_var.match(st)
        if m:
            index_vars[m.group(1).upper()] = int(m.group(2))
            continue
        m = re_impl.match(st)
        if m:
            name = m.group(1).upper()
            subs = [s.strip().upper() for s in m.group(2).split(",")]
            vals = _values(m.group(4))
            arrays.setdefault(name, {})[tuple(subs)] = vals
            continue
        m = re_elem.match(st)
        if m:
            lhs = re.findall(r"(\w+)\s*\(\s*(\d+)\s*\)", m.group(1))
            vals = _values(m.group(2))
            if len(lhs) == len(vals):
                for (nm, idx), v in zip(lhs, vals):
                    per_elem.setdefault(nm.upper(), {})[int(idx)] = v
            continue
        if "SPECIES_LIST" in st.upper() and "MEMBER(" in st.upper():
            member_list = re_member.findall(st)

    def pint(name: str) -> int:
        return int(params[name])

    mech = Mechanism(
        name=params["MECHNAME"].strip("'\" ").strip(),
        nspec=pint("NUMB_MECH_SPC"),
        nrxns=pint("NRXNS"),
    )
    ns, nr = mech.nspec, mech.nrxns
    mech.mxprd = pint("MXPRD")
    mech.nphotab = pint("NPHOTAB")
    mech.nhetero = pint("NHETERO")
    mech.nspecial_rxn = int(params.get("NSPECIAL_RXN", "0"))

    spc = per_elem["CHEMISTRY_SPC"]
    mw = per_elem["SPECIES_MOLWT"]
    cgi = per_elem["CGRID_INDEX"]
    sty = per_elem["SPECIES_TYPE"]
    cvt = per_elem["CONVERT_CONC"]
    for i in range(1, ns + 1):
        mech.species.append(spc[i].strip("'").strip())
        mech.molwt.append(fnum(mw[i]))
        mech.cgrid_index.append(int(cgi[i]))
        mech.species_type.append(sty[i].strip("'").strip())
        mech.convert_conc.append(cvt[i].strip().upper() == "T")

    def col(name: str, sub2: str | None = None) -> list[str]:
        tab = arrays[name]
        key = ("IRXXN",) if sub2 is None else None
        if sub2 is not None:
            for k, v in tab.items():
                if len(k) == 2 and k[0] == "IRXXN" and k[1] == sub2:
                    return v
                if len(k) == 2 and k[1] == "IRXXN" and k[0] == sub2:
                    return v
            raise KeyError((name, sub2))
        return tab[key]

    mech.ktype = [int(v) for v in col("KTYPE")]
    mech.irxbits = [int(v) for v in col("IRXBITS")]
    mech.nreact = [int(v) for v in col("NREACT")]
    mech.nprdct = [int(v) for v in col("NPRDCT")]
    assert len(mech.ktype) == nr and len(mech.nreact) == nr
    irr_cols = [[int(v) for v in col("IRR", str(k))] for k in range(1, mech.mxprd + 4)]
    mech.irr = [[irr_cols[k][r] for k in range(mech.mxprd + 3)] for r in range(nr)]
    sc_cols = [[fnum(v) for v in col("SC", str(k))] for k in range(1, mech.mxprd + 1)]
    mech.sc = [[sc_cols[k][r] for k in range(mech.mxprd)] for r in range(nr)]
    mech.rxlabel = [v.strip("'").strip() for v in col("RXLABEL")]
    rt = [[fnum(v) for v in col("RTDAT", str(k))] for k in (1, 2, 3)]
    mech.rtdat = [[rt[0][r], rt[1][r], rt[2][r]] for r in range(nr)]
    nfall = int(params.get("NFALLOFF", "0"))
    if nfall > 0:
        rf = [[fnum(v) for v in col("RFDAT", str(k))] for k in (1, 2, 3, 4, 5)]
        mech.rfdat = [[rf[k][i] for k in range(5)] for i in range(nfall)]
        mech.irrfall = [int(v) for v in col("IRRFALL")][:nfall]
    mech.iorder = [int(v) for v in col("IORDER")]
    mech.kunits = int(params.get("KUNITS", "0"))
    mech.photab = [v.strip("'").strip() for v in arrays["PHOTAB"][("IRXXN",)]]
    mech.hetero = [v.strip("'").strip() for v in arrays["HETERO"][("IRXXN",)]]
    nmphot = pint("NMPHOT")
    iph = [[int(v) for v in col("IPH", str(k))] for k in (1, 2, 3)]
    mech.iph = [(iph[0][i], iph[1][i], iph[2][i]) for i in range(nmphot)]
    mhet = pint("MHETERO")
    ih = [[int(v) for v in col("IHETERO", str(k))] for k in (1, 2)]
    mech.ihetero = [(ih[0][i], ih[1][i]) for i in range(mhet)]

    for arr, key in _TB.items():
        cnt = int(params.get({"NRXWM": "NWM", "NRXWO2": "NWO2", "NRXWN2": "NWN2", "NRXWW": "NWW",
                              "NRXWH2": "NWH2", "NRXWCH4": "NWCH4"}[arr], "0"))
        if cnt > 0:
            mech.third_body[key] = [int(v) for v in arrays[arr][("IRXXN",)]][:cnt]
        else:
            mech.third_body[key] = []
    for p, key in _TB_CONC.items():
        if p in params:
            mech.third_body_conc[key] = fnum(params[p])

    # cross-check against the SPECIES_LIST constructor when present
    if member_list:
        assert len(member_list) == ns, (len(member_list), ns)
        for i, (nm, idx, ty, w, cv) in enumerate(member_list):
            assert nm.strip() == mech.species[i], (nm, mech.species[i])
    # sanity: reactant/product counts agree with IRR
    for r in range(nr):
        nre = sum(1 for k in range(3) if mech.irr[r][k] != 0)
        npr = sum(1 for k in range(3, 3 + mech.mxprd) if mech.irr[r][k] != 0)
        assert nre == mech.nreact[r], (r, nre, mech.nreact[r])
        assert npr == mech.nprdct[r], (r, npr, mech.nprdct[r])
    return mech
