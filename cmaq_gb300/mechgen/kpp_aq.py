"""KMT2 aqueous chemistry generator: KPP mechanism files -> oracle tables.

Usage (run where the CMAQ source tree is available; the output is committed):

    python -m cmaq_gb300.mechgen.kpp_aq --cmaq <CMAQ tree>

CMAQ's KMT2 cloud chemistry (``CCTM/src/cloud/acm_ae7_kmt2``) integrates a
KPP-generated aqueous mechanism of 161 variable and 4 fixed species and 269
reactions with KPP's Rodas3 Rosenbrock solver.  This module reads that mechanism
as data and writes ``oracle/gen/kmt2_aq.c``, tables that the oracle's own
evaluation code (``oracle/kmt2_oracle.c``) walks:

* species indices                ``aqchem_Parameters.F90`` (``ind_*`` / ``indf_*``)
* reaction rate factors          ``aqchem_Function.F90`` ``A(i) = RCT(i)*V(..)*F(..)``
* species tendencies             ``aqchem_Function.F90`` ``Vdot(k) = c*A(i) ...``
* rate laws                      ``aqchem_Rates.F90`` ``Update_RCONST`` (ionic-strength
                                 dependent, refreshed during the integration) and
                                 ``aqchem_Initialize.F90`` (set once per call)
* tolerances                     ``aqchem_Initialize.F90`` ``RTOL`` / ``ATOL``
* Henry's law constants          ``aqchem_kmt.F90:371-396`` with the table of ``hlconst.F``

and, for the device code, ``cmaq_gb300/csrc/gen/kmt2_aq_consts.cuh`` (sizes, species
indices) and ``cmaq_gb300/csrc/gen/kmt2_aq.cuh`` (Henry's law constants, rate constants,
tolerances, f, J, LU factorisation and solve as strided straight-line code in functions
of about 200 operations; the rate-law functions they call are in ``csrc/kmt2.cuh``).  ``oracle/gen/kmt2_aq_unrolled.c`` holds
the same straight-line f, J, LU and solve for the oracle's bit-for-bit check, and
``cmaq_gb300/mechs/kmt2/manifest.json`` the species names and the FLOP counts of those
routines (the benchmark's algorithmic work per step).

The Jacobian terms (one partial derivative per reaction and variable reactant,
combined per Jacobian entry with the species' net coefficients) and the sparse LU
structure (the Jacobian pattern plus its symbolic fill-in in KPP's species order)
are derived here, not read; generation fails unless they equal the reference's
``aqchem_Jacobian.F90`` (``B`` / ``JVS``) and ``aqchem_JacobianSP.F90``
(``LU_IROW`` / ``LU_ICOL`` / ``LU_CROW`` / ``LU_DIAG``) term for term.

Fortran literal kinds are kept: a literal without a ``D`` exponent or ``_dp`` kind
(``0.92*A(204)``, ``0.21 * PRESS``) is a REAL(4) value widened to double.
"""
from __future__ import annotations

import argparse
import json
import os
import re
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from .fortran_tables import join_continuations

REPO = Path(__file__).resolve().parents[2]
SUBDIR = Path("CCTM") / "src" / "cloud" / "acm_ae7_kmt2"


def flit(tok: str) -> float:
    """Value of a Fortran numeric literal with its kind: D exponent or ``_dp`` ->
    double; a real literal without either -> REAL(4) widened; integer -> exact."""
    t = tok.strip()
    if t.endswith("_dp"):
        return float(t[:-3].replace("d", "e").replace("D", "e"))
    if "d" in t or "D" in t:
        return float(t.replace("d", "e").replace("D", "e"))
    if "." in t or "e" in t or "E" in t:
        return float(np.float32(float(t)))
    return float(int(t))


def c_dbl(v: float) -> str:
    return float(v).hex()


@dataclass
class KppMech:
    nvar: int
    nfix: int
    nreact: int
    names: list[str]                                   # nvar + nfix, 0-based
    index: dict[str, int]                              # ind_X -> 0-based (fixed: nvar + k)
    factors: list[list[int]] = field(default_factory=list)      # per reaction, A-order, 0-based C index
    vdot: list[list[tuple[float, int]]] = field(default_factory=list)  # per variable species
    blist: list[tuple[int, int, list[int]]] = field(default_factory=list)  # (rxn, mult, other factors)
    jvs: list[list[tuple[float, int]]] = field(default_factory=list)  # per LU entry: (coef, b index)
    lu_irow: list[int] = field(default_factory=list)
    lu_icol: list[int] = field(default_factory=list)
    lu_crow: list[int] = field(default_factory=list)
    lu_diag: list[int] = field(default_factory=list)
    rates: list[tuple] = field(default_factory=list)   # per reaction: (kind, args, refreshed, mtpyrac)
    rtol: list[float] = field(default_factory=list)
    atol: list[float] = field(default_factory=list)
    henry: list[tuple] = field(default_factory=list)   # (var name, kind, a, e)


# ----------------------------------------------------------------------------- parsing
def _params(text: str):
    vals, index = {}, {}
    for m in re.finditer(r"INTEGER,\s*PARAMETER\s*::\s*(\w+)\s*=\s*(\d+)", text):
        vals[m.group(1)] = int(m.group(2))
    nvar = vals["NVAR"]
    for k, v in vals.items():
        if k.startswith("ind_") and not k.startswith("indf_"):
            index[k[4:]] = v - 1
    return vals, index


def _function(text: str, nvar: int, nreact: int):
    factors: list[list[int] | None] = [None] * nreact
    vdot: list[list[tuple[float, int]] | None] = [None] * nvar
    for st in join_continuations(text):
        m = re.fullmatch(r"A\((\d+)\)\s*=\s*RCT\((\d+)\)((?:\*[VF]\(\d+\))*)", st.replace(" ", ""))
        if m:
            r = int(m.group(1)) - 1
            assert int(m.group(2)) - 1 == r
            facs = []
            for kind, i in re.findall(r"\*([VF])\((\d+)\)", m.group(3)):
                facs.append(int(i) - 1 if kind == "V" else nvar + int(i) - 1)
            factors[r] = facs
            continue
        m = re.fullmatch(r"Vdot\((\d+)\)=(.*)", st.replace(" ", ""))
        if m:
            k = int(m.group(1)) - 1
            terms = []
            for sign, coef, r in re.findall(r"([+-]?)(?:([0-9.]+(?:[dDeE][-+]?\d+)?)\*)?A\((\d+)\)", m.group(2)):
                c = flit(coef) if coef else 1.0
                terms.append((-c if sign == "-" else c, int(r) - 1))
            vdot[k] = terms
    assert all(f is not None for f in factors) and all(v is not None for v in vdot)
    return factors, vdot


def _derive_jacobian(factors, vdot, nvar):
    """Partial derivatives per (reaction, distinct variable reactant) in reaction and
    factor order; Jacobian entries (i, j) as the net coefficient of i times the
    derivative of reaction r with respect to j, summed in reaction order."""
    blist, bindex = [], {}
    for r, facs in enumerate(factors):
        seen = []
        for f in facs:
            if f < nvar and f not in seen:
                seen.append(f)
        for j in seen:
            others = list(facs)
            others.remove(j)
            mult = facs.count(j)
            bindex[(r, j)] = len(blist)
            blist.append((r, mult, others))
    coef = {}
    for i, terms in enumerate(vdot):
        for c, r in terms:
            coef[(i, r)] = c
    entries: dict[tuple[int, int], list[tuple[float, int]]] = {}
    for i in range(nvar):
        entries[(i, i)] = []
    for i, terms in enumerate(vdot):
        for c, r in terms:
            for (rr, j), b in ((key, v) for key, v in bindex.items() if key[0] == r):
                entries.setdefault((i, j), []).append((c, b))
    for key in entries:
        entries[key].sort(key=lambda t: t[1])
    return blist, entries


def _symbolic_lu(pattern: set[tuple[int, int]], n: int):
    """Row-wise symbolic LU without pivoting: row k gains, for every j < k in its
    pattern (in increasing order, including entries it gained), the columns > j of
    row j of U."""
    rows = [set() for _ in range(n)]
    for i, j in pattern:
        rows[i].add(j)
    for k in range(n):
        rows[k].add(k)
        done = set()
        while True:
            todo = sorted(j for j in rows[k] if j < k and j not in done)
            if not todo:
                break
            j = todo[0]
            done.add(j)
            rows[k] |= {c for c in rows[j] if c > j}
    irow, icol, crow, diag = [], [], [], []
    for k in range(n):
        crow.append(len(icol))
        for c in sorted(rows[k]):
            if c == k:
                diag.append(len(icol))
            irow.append(k)
            icol.append(c)
    crow.append(len(icol))
    diag.append(len(icol))
    return irow, icol, crow, diag


def _int_array(text: str, name: str) -> list[int]:
    """Concatenate ``NAME`` or ``NAME_0, NAME_1, ...`` PARAMETER arrays."""
    parts = []
    for st in join_continuations(text):
        m = re.match(rf"INTEGER,\s*PARAMETER,\s*DIMENSION\(\d+\)\s*::\s*{name}(_\d+)?\s*=\s*\(/(.*)/\)", st)
        if m:
            vals = [int(v) for v in m.group(2).replace(" ", "").split(",") if re.fullmatch(r"\d+", v)]
            if vals:
                parts.append((int(m.group(1)[1:]) if m.group(1) else -1, vals))
    chunks = [v for k, v in sorted(parts) if k >= 0]
    whole = [v for k, v in parts if k < 0]
    return sum(chunks, []) if chunks else whole[0]


def _check_reference_jacobian(text: str, nvar, factors, blist, lu, entries):
    """Compare the derived terms with the reference Jac_SP: B(k) bodies by their
    factors and JVS(k) by (coefficient, B body) sequences."""
    def bkey(r, mult, others):
        return (r, mult, tuple(others))
    bref = {}
    jref = {}
    for st in join_continuations(text):
        s = st.replace(" ", "")
        m = re.fullmatch(r"B\((\d+)\)=RCT\((\d+)\)((?:\*(?:\d+|[VF]\(\d+\)))*)", s)
        if m:
            mult, others = 1, []
            for tok in re.findall(r"\*(\d+|[VF]\(\d+\))", m.group(3)):
                if tok[0] in "VF":
                    i = int(tok[2:-1]) - 1
                    others.append(i if tok[0] == "V" else nvar + i)
                else:
                    mult = int(tok)
            bref[int(m.group(1))] = bkey(int(m.group(2)) - 1, mult, others)
            continue
        m = re.fullmatch(r"JVS\((\d+)\)=(.*)", s)
        if m:
            terms = []
            if m.group(2) != "0":
                for sign, coef, b in re.findall(r"([+-]?)(?:([0-9.]+(?:[dDeE][-+]?\d+)?)\*)?B\((\d+)\)", m.group(2)):
                    c = flit(coef) if coef else 1.0
                    terms.append((-c if sign == "-" else c, bref[int(b)]))
            jref[int(m.group(1)) - 1] = terms
    irow, icol = lu[0], lu[1]
    bad = []
    for k in range(len(irow)):
        mine = [(c, bkey(*blist[b])) for c, b in entries.get((irow[k], icol[k]), [])]
        if mine != jref.get(k):
            bad.append(k)
    if bad:
        raise ValueError(f"derived Jacobian differs from Jac_SP at JVS entries {bad[:10]} (+{len(bad) - 10 if len(bad) > 10 else 0})")


_RATE_FUNCS = {"DISF": 0, "DISB": 1, "KRXN": 2, "KIEPOX": 3, "KMTF": 4, "KMTB": 5, "HYDF": 6, "KPHOT": 7}
KIND_NAMES = ["DISF", "DISB", "KRXN", "KIEPOX", "KMTF", "KMTB", "HYDF", "KPHOT", "ALFA3", "WETFAC", "CONST"]


def _rate_lines(text: str, sub: str):
    body = text.split(f"SUBROUTINE {sub}", 1)[1]
    out = {}
    for st in join_continuations(body):
        m = re.fullmatch(r"RCONST\((\d+)\)\s*=\s*(.*)", st.strip())
        if m:
            out[int(m.group(1)) - 1] = m.group(2).replace(" ", "")
    return out


def _parse_rate(expr: str, henry_names: list[str]):
    """``((FN(a,b,..)))`` / ``(ALFA3_KPP)`` / ``((1.1d0))`` / ``((MTPYRAC*KMTF(..)))``."""
    e = expr
    while e.startswith("(") and e.endswith(")"):
        e = e[1:-1]
    mt = 0
    if e.startswith("MTPYRAC*"):
        mt, e = 1, e[len("MTPYRAC*"):]
    if e == "ALFA3_KPP":
        return ("ALFA3", [], mt)
    if e == "WETFAC_KPP":
        return ("WETFAC", [], mt)
    m = re.fullmatch(r"(\w+)\((.*)\)", e)
    if not m:
        return ("CONST", [flit(e)], mt)
    fn, args = m.group(1), m.group(2).split(",")
    vals = []
    for a in args:
        if re.fullmatch(r"[A-Za-z_]\w*", a):
            if a == "JH2O2":
                vals.append(-2.0)                  # KPHOT: take the caller's J(H2O2)
            else:
                if a not in henry_names:
                    henry_names.append(a)
                vals.append(float(henry_names.index(a)))
        else:
            vals.append(flit(a))
    return (fn, vals, mt)


def _henry(kmt_text: str, hl_text: str, names: list[str]):
    table = {}
    for m in re.finditer(r"DATA\s+SUBNAME\(\s*\d+\),\s*A\(\s*\d+\),\s*E\(\s*\d+\)\s*/\s*'([^']*)'\s*,\s*([^,]+),\s*([^/]+)/",
                         hl_text):
        # the first entry of a name, as HLCONST's search (hlconst.F:491-497)
        table.setdefault(m.group(1).strip(), (float(np.float32(float(m.group(2)))), float(np.float32(float(m.group(3))))))
    chars = {m.group(1): m.group(2).strip() for m in
             re.finditer(r"CHARACTER\(\s*16\s*\),\s*SAVE\s*::\s*(\w+)\s*=\s*'([^']*)'", kmt_text)}
    out = []
    for v in names:
        m = re.search(rf"^\s*{v}\s*=\s*(.*)$", kmt_text, flags=re.M)
        if not m:
            raise ValueError(f"Henry constant {v} not assigned in aqchem_kmt.F90")
        rhs = m.group(1).split("!")[0].strip()
        mh = re.match(r"HLCONST\(\s*(?:'([^']*)'|(\w+))", rhs)
        if mh:
            key = (mh.group(1) or chars[mh.group(2)]).strip()
            a, e = table[key]
            out.append((v, "hlconst", a, e))
            continue
        mx = re.fullmatch(r"([0-9.DdEe+-]+)\s*\*\s*EXP\(\s*([0-9.DdEe+-]+)\s*\*\s*\(\s*\(\s*298\.D0\s*-\s*TEMP2\s*\)"
                          r"\s*/\s*\(\s*298\.D0\s*\*\s*TEMP2\s*\)\s*\)\s*\)", rhs)
        if mx:
            out.append((v, "exp", flit(mx.group(1)), flit(mx.group(2))))
            continue
        out.append((v, "const", flit(rhs), 0.0))
    return out


def _tolerances(text: str, index: dict[str, int], nvar: int):
    body = text.split("SUBROUTINE Initialize", 1)[1]
    rtol, atol = [None] * nvar, [None] * nvar
    for st in join_continuations(body):
        s = st.replace(" ", "")
        m = re.fullmatch(r"(RTOL|ATOL)=([0-9.DdEe+-]+)", s)
        if m:
            arr = rtol if m.group(1) == "RTOL" else atol
            arr[:] = [flit(m.group(2))] * nvar
            continue
        m = re.fullmatch(r"(RTOL|ATOL)\(ind_(\w+)\)=([0-9.DdEe+-]+)", s)
        if m:
            (rtol if m.group(1) == "RTOL" else atol)[index[m.group(2)]] = flit(m.group(3))
    assert None not in rtol and None not in atol
    return rtol, atol


def load(cmaq_root: str) -> KppMech:
    d = Path(cmaq_root) / SUBDIR
    par = (d / "aqchem_Parameters.F90").read_text()
    vals, index = _params(par)
    nvar, nfix, nreact = vals["NVAR"], vals["NFIX"], vals["NREACT"]
    names = [""] * (nvar + nfix)
    for k, v in index.items():
        names[v] = k
    factors, vdot = _function((d / "aqchem_Function.F90").read_text(), nvar, nreact)
    blist, entries = _derive_jacobian(factors, vdot, nvar)
    lu = _symbolic_lu(set(entries), nvar)
    sp = (d / "aqchem_JacobianSP.F90").read_text()
    ref_lu = ([v - 1 for v in _int_array(sp, "LU_IROW")], [v - 1 for v in _int_array(sp, "LU_ICOL")],
              [v - 1 for v in _int_array(sp, "LU_CROW")], [v - 1 for v in _int_array(sp, "LU_DIAG")])
    if tuple(lu) != ref_lu:
        raise ValueError("derived LU structure differs from aqchem_JacobianSP.F90")
    if len(lu[0]) != vals["LU_NONZERO"]:
        raise ValueError("LU_NONZERO mismatch")
    _check_reference_jacobian((d / "aqchem_Jacobian.F90").read_text(), nvar, factors, blist, lu, entries)
    jvs = [entries.get((lu[0][k], lu[1][k]), []) for k in range(len(lu[0]))]

    rates_text = (d / "aqchem_Rates.F90").read_text()
    init_text = (d / "aqchem_Initialize.F90").read_text()
    upd = _rate_lines(rates_text, "Update_RCONST")
    ini = _rate_lines(init_text, "Initialize")
    if set(upd) & set(ini) or len(set(upd) | set(ini)) != nreact:
        raise ValueError("rate constants must be set exactly once, by Initialize or Update_RCONST")
    hnames: list[str] = []
    rates = []
    for r in range(nreact):
        kind, args, mt = _parse_rate(upd[r] if r in upd else ini[r], hnames)
        rates.append((kind, args, r in upd, mt))
    henry = _henry((d / "aqchem_kmt.F90").read_text(), (d / "hlconst.F").read_text(), hnames)
    rtol, atol = _tolerances(init_text, index, nvar)
    return KppMech(nvar, nfix, nreact, names, index, factors, vdot, blist, jvs, *lu, rates, rtol, atol, henry)


# ----------------------------------------------------------------------------- emission
def _arr(ctype: str, name: str, vals, fmt=str, per_line=12) -> str:
    vals = list(vals)
    lines = []
    for i in range(0, len(vals), per_line):
        lines.append("    " + ", ".join(fmt(v) for v in vals[i:i + per_line]) + ",")
    return f"static const {ctype} {name}[{max(len(vals), 1)}] = {{\n" + ("\n".join(lines) if vals else "    0") + "\n};\n"


def _csr(rows):
    ptr, flat = [0], []
    for r in rows:
        flat += r
        ptr.append(len(flat))
    return ptr, flat


def oracle_source(k: KppMech) -> str:
    out = ["/* Generated by cmaq_gb300/mechgen/kpp_aq.py from CCTM/src/cloud/acm_ae7_kmt2 (KPP aqueous",
           " * mechanism of the KMT2 cloud chemistry).  Tables only; oracle/kmt2_oracle.c evaluates them.",
           " * Do not edit. */", ""]
    out.append(f"#define KQ_NVAR {k.nvar}\n#define KQ_NFIX {k.nfix}\n#define KQ_NREACT {k.nreact}")
    out.append(f"#define KQ_LU_NONZERO {len(k.lu_irow)}\n#define KQ_NB {len(k.blist)}")
    out.append(f"#define KQ_NHENRY {len(k.henry)}\n")
    for name, i in sorted(k.index.items(), key=lambda t: t[1]):
        out.append(f"#define KQ_{name} {i if i < k.nvar else i - k.nvar}")
    out.append("")
    out.append("static const char* const kq_names[KQ_NVAR + KQ_NFIX] = {\n" +
               ",\n".join(f'    "{n}"' for n in k.names) + "\n};\n")
    ptr, flat = _csr(k.factors)
    out.append(_arr("int", "kq_fac_ptr", ptr))
    out.append(_arr("int", "kq_fac", flat))
    ptr, flat = _csr([[r for _, r in t] for t in k.vdot])
    out.append(_arr("int", "kq_f_ptr", ptr))
    out.append(_arr("int", "kq_f_rxn", flat))
    out.append(_arr("double", "kq_f_coef", [c for t in k.vdot for c, _ in t], c_dbl, 6))
    out.append(_arr("int", "kq_b_rxn", [b[0] for b in k.blist]))
    out.append(_arr("int", "kq_b_mult", [b[1] for b in k.blist]))
    ptr, flat = _csr([b[2] for b in k.blist])
    out.append(_arr("int", "kq_b_ptr", ptr))
    out.append(_arr("int", "kq_b_fac", flat))
    ptr, flat = _csr([[b for _, b in t] for t in k.jvs])
    out.append(_arr("int", "kq_j_ptr", ptr))
    out.append(_arr("int", "kq_j_b", flat))
    out.append(_arr("double", "kq_j_coef", [c for t in k.jvs for c, _ in t], c_dbl, 6))
    out.append(_arr("int", "kq_lu_icol", k.lu_icol))
    out.append(_arr("int", "kq_lu_crow", k.lu_crow))
    out.append(_arr("int", "kq_lu_diag", k.lu_diag))
    out.append("/* rate laws: kind (KQ_RATE_*), up to 5 arguments (Henry constants by their index in\n"
               " * kq_henry_*, J(H2O2) as -2), refreshed by Update_RCONST, multiplied by MTPYRAC */")
    for i, n in enumerate(KIND_NAMES):
        out.append(f"#define KQ_RATE_{n} {i}")
    kinds = [KIND_NAMES.index(r[0]) for r in k.rates]
    out.append(_arr("int", "kq_rate_kind", kinds))
    out.append(_arr("double", "kq_rate_arg", [a for r in k.rates for a in (r[1] + [0.0] * 5)[:5]], c_dbl, 5))
    out.append(_arr("unsigned char", "kq_rate_update", [int(r[2]) for r in k.rates], per_line=30))
    out.append(_arr("unsigned char", "kq_rate_mtpyrac", [r[3] for r in k.rates], per_line=30))
    out.append("/* Henry's law constants: 0 = HLCONST table entry (REAL(4) A, E), 1 = a*exp(e*dT) in\n"
               " * double, 2 = constant a */")
    out.append("static const char* const kq_henry_name[KQ_NHENRY] = {" +
               ", ".join(f'"{h[0]}"' for h in k.henry) + "};")
    out.append(_arr("int", "kq_henry_kind", [{"hlconst": 0, "exp": 1, "const": 2}[h[1]] for h in k.henry]))
    out.append(_arr("double", "kq_henry_a", [h[2] for h in k.henry], c_dbl, 6))
    out.append(_arr("double", "kq_henry_e", [h[3] for h in k.henry], c_dbl, 6))
    out.append(_arr("double", "kq_rtol", k.rtol, c_dbl, 6))
    out.append(_arr("double", "kq_atol", k.atol, c_dbl, 6))
    return "\n".join(out)


def _term(coef: float, x: str) -> str:
    if coef == 1.0:
        return f" + {x}"
    if coef == -1.0:
        return f" - {x}"
    return f" + {c_dbl(coef)} * {x}"


def _factor(f: int, nvar: int, acc) -> str:
    return acc("v", f) if f < nvar else acc("f", f - nvar)


def unrolled_routines(k: KppMech, qual: str = "static", acc=None) -> str:
    """Straight-line f, J, LU factorisation and solve with the operations, operands
    and order of the table-driven oracle (Fun, Jac_SP, KppDecomp, KppSolve): the form
    the device kernel takes, checked bit for bit against the tables on the CPU.
    ``acc(array, index)`` renders an element access (plain indexing by default)."""
    acc = acc or (lambda name, i: f"{name}[{i}]")
    n = k.nvar
    out = []
    # Fun
    out.append(f"{qual} void kqu_fun(const double* v, const double* f, const double* r, double* vdot)\n{{")
    for rx, facs in enumerate(k.factors):
        out.append(f"    const double a{rx} = " + " * ".join([acc("r", rx)] + [_factor(x, n, acc) for x in facs]) + ";")
    for i, terms in enumerate(k.vdot):
        out.append(f"    {acc('vdot', i)} = 0.0" + "".join(_term(c, f"a{rx}") for c, rx in terms) + ";")
    out.append("}\n")
    # Jac_SP
    out.append(f"{qual} void kqu_jac(const double* v, const double* f, const double* r, double* jvs)\n{{")
    for b, (rx, mult, others) in enumerate(k.blist):
        parts = [acc("r", rx)] + ([c_dbl(float(mult))] if mult > 1 else []) + [_factor(x, n, acc) for x in others]
        out.append(f"    const double b{b} = " + " * ".join(parts) + ";")
    for e, terms in enumerate(k.jvs):
        out.append(f"    {acc('jvs', e)} = 0.0" + "".join(_term(c, f"b{b}") for c, b in terms) + ";")
    out.append("}\n")
    # KppDecomp: row k's work row is row k of the stored factors itself (its pattern holds
    # every column the elimination touches)
    pos = {(k.lu_irow[e], k.lu_icol[e]): e for e in range(len(k.lu_irow))}
    out.append(f"{qual} int kqu_decomp(double* jvs)\n{{")
    for row in range(n):
        out.append(f"    if (fabs({acc('jvs', k.lu_diag[row])}) < DBL_MIN) return {row + 1};")
        for kk in range(k.lu_crow[row], k.lu_diag[row]):
            j = k.lu_icol[kk]
            out.append(f"    {{ const double a = -{acc('jvs', kk)} / {acc('jvs', k.lu_diag[j])}; {acc('jvs', kk)} = -a;")
            for jj in range(k.lu_diag[j] + 1, k.lu_crow[j + 1]):
                q = pos[(row, k.lu_icol[jj])]
                out.append(f"      {acc('jvs', q)} = {acc('jvs', q)} + a * {acc('jvs', jj)};")
            out.append("    }")
    out.append("    return 0;\n}\n")
    # KppSolve
    out.append(f"{qual} void kqu_solve(const double* jvs, double* x)\n{{")
    for row in range(n):
        terms = "".join(f" - {acc('jvs', kk)} * {acc('x', k.lu_icol[kk])}" for kk in range(k.lu_crow[row], k.lu_diag[row]))
        if terms:
            out.append(f"    {acc('x', row)} = {acc('x', row)}{terms};")
    for row in range(n - 1, -1, -1):
        terms = "".join(f" - {acc('jvs', kk)} * {acc('x', k.lu_icol[kk])}"
                        for kk in range(k.lu_diag[row] + 1, k.lu_crow[row + 1]))
        out.append(f"    {acc('x', row)} = ({acc('x', row)}{terms}) / {acc('jvs', k.lu_diag[row])};")
    out.append("}\n")
    return "\n".join(out)


def device_consts(k: KppMech) -> str:
    """Sizes and species indices for the device code (``namespace kmt2``)."""
    out = ["// Generated by cmaq_gb300/mechgen/kpp_aq.py from CCTM/src/cloud/acm_ae7_kmt2 (KPP aqueous",
           "// mechanism of the KMT2 cloud chemistry).  Included inside namespace kmt2.  Do not edit.",
           "#pragma once", "",
           f"constexpr int NVAR = {k.nvar};", f"constexpr int NFIX = {k.nfix};", f"constexpr int NREACT = {k.nreact};",
           f"constexpr int LU_NONZERO = {len(k.lu_irow)};", f"constexpr int NHENRY = {len(k.henry)};", ""]
    for name, i in sorted(k.index.items(), key=lambda t: t[1]):
        out.append(f"constexpr int {name} = {i if i < k.nvar else i - k.nvar};")
    return "\n".join(out) + "\n"


def _rate_call(kind: str, a: list[float]) -> str:
    d = c_dbl
    if kind == "DISF":
        return f"kq_disf(c, {d(a[0])}, {d(a[1])}, {d(a[2])}, {int(a[3])})"
    if kind == "DISB":
        return f"kq_disb(c, {d(a[0])}, {int(a[1])})"
    if kind == "KRXN":
        return f"kq_krxn(c, v, {d(a[0])}, {d(a[1])}, {int(a[2])}, {int(a[3])}, {int(a[4])})"
    if kind == "KIEPOX":
        return f"kq_kiepox(c, v, f, {d(a[0])}, {d(a[1])}, {int(a[2])})"
    if kind == "KMTF":
        return f"kq_kmtf(c, {d(a[0])}, {d(a[1])}, {d(a[2])})"
    if kind == "KMTB":
        return f"kq_kmtb(c, c.henry[{int(a[0])}], {d(a[1])}, {d(a[2])}, {d(a[3])})"
    if kind == "HYDF":
        return f"kq_hydf(c, {d(a[0])}, {d(a[1])})"
    if kind == "KPHOT":
        return f"kq_kphot(c, {d(a[0])}, {'c.jh2o2' if a[1] == -2.0 else d(a[1])})"
    if kind == "ALFA3":
        return "c.alfa3"
    if kind == "WETFAC":
        return "c.wetfac"
    return d(a[0])


def device_source(k: KppMech) -> str:
    """Strided straight-line routines for the device code (``namespace kmt2``, after the
    rate-law functions of csrc/kmt2.cuh): Henry's law constants, the rate constants set
    once and refreshed, RTOL, f, J, LU factorisation and solve.  Arrays live in a
    lane-interleaved workspace: element i of a lane at ``p[i * KQ_S]`` (KQ_S, the lanes
    of a warp, is a constant of csrc/kmt2.cuh)."""
    out = ["// Generated by cmaq_gb300/mechgen/kpp_aq.py from CCTM/src/cloud/acm_ae7_kmt2: Henry's law",
           "// constants (aqchem_kmt.F90:371-396), rate constants (aqchem_Initialize.F90:491-636,",
           "// aqchem_Rates.F90:456-579), tolerances, Fun, Jac_SP, KppDecomp, KppSolve as straight-line",
           "// code.  Included inside namespace kmt2 by csrc/kmt2.cuh.  Do not edit.",
           "#pragma once", ""]
    out.append("KQ_HD inline void kq_henry(Cell& c, float t2)\n{")
    for h, (name, kind, a, e) in enumerate(k.henry):
        if kind == "hlconst":
            out.append(f"    c.henry[{h}] = (double)kq_hlconst((float){c_dbl(a)}, (float){c_dbl(e)}, t2);   // {name}")
        elif kind == "exp":
            out.append(f"    c.henry[{h}] = {c_dbl(a)} * kq_exp({c_dbl(e)} * ((298.0 - (double)t2) / (298.0 * (double)t2)));"
                       f"   // {name}")
        else:
            out.append(f"    c.henry[{h}] = {c_dbl(a)};   // {name}")
    out.append("}\n")
    for fn, upd in (("kq_rates_once", False), ("kq_rates_update", True)):
        out.append(f"KQ_HD KQ_NOINLINE void {fn}(const Cell& c, const double* v, const double* f, double* r)\n{{")
        if not upd:
            out.append("    (void)v;\n    (void)f;")
        for rx, (kind, args, refreshed, mt) in enumerate(k.rates):
            if refreshed != upd:
                continue
            call = _rate_call(kind, args)
            if mt:
                call = f"(double)c.mtpyrac * {call}"
            out.append(f"    r[{rx} * KQ_S] = {call};")
        out.append("}\n")
    special = sorted({i for i in range(k.nvar) if k.rtol[i] != k.rtol[0]})
    assert len(set(k.atol)) == 1 and len({k.rtol[i] for i in special}) <= 1
    cond = " || ".join(f"i == {i}" for i in special) or "false"
    alt = c_dbl(k.rtol[special[0]]) if special else c_dbl(k.rtol[0])
    out.append(f"KQ_HD inline double kq_rtol(int i) {{ return ({cond}) ? {alt} : {c_dbl(k.rtol[0])}; }}")
    out.append(f"KQ_HD inline double kq_atol(int) {{ return {c_dbl(k.atol[0])}; }}\n")
    out.append("KQ_HD inline void kq_add_diagonal(double* g, double x)\n{")
    out += [f"    g[{d} * KQ_S] = g[{d} * KQ_S] + x;" for d in k.lu_diag[:-1]]
    out.append("}\n")
    out.append(device_routines(k))
    return "\n".join(out)


DEVICE_CHUNK_OPS = 200   # LU updates / solve terms per generated device function (bounds register spills)


def device_routines(k: KppMech, chunk_ops: int = DEVICE_CHUNK_OPS) -> str:
    """The straight-line f, J, LU and solve of ``unrolled_routines`` for the device:
    strided accesses; every tendency and Jacobian entry computed from its products
    inline (no hundreds of live temporaries; each product is formed from the same
    operands in the same order, so the bits are those of the oracle's routines); the LU
    factorisation and the two triangular solves split at row boundaries into functions of
    about ``chunk_ops`` operations."""
    acc = lambda name, i: f"{name}[{i} * KQ_S]"
    n = k.nvar
    q = "KQ_HD KQ_NOINLINE"
    out = []
    prod = lambda rx: " * ".join([acc("r", rx)] + [_factor(x, n, acc) for x in k.factors[rx]])
    def chunked(name, args, call_args, items, cost, line):
        groups, cur, ops = [], [], 0
        for it in items:
            if cur and ops + cost(it) > chunk_ops:
                groups.append(cur)
                cur, ops = [], 0
            cur.append(it)
            ops += cost(it)
        if cur:
            groups.append(cur)
        for gi, g in enumerate(groups):
            out.append(f"{q} void {name}_{gi}({args})\n{{")
            out.extend(line(it) for it in g)
            out.append("}\n")
        out.append(f"KQ_HD inline void {name}({args})\n{{")
        out.extend(f"    {name}_{gi}({call_args});" for gi in range(len(groups)))
        out.append("}\n")

    fargs = "const double* v, const double* f, const double* r, double* vdot"
    chunked("kqu_fun", fargs, "v, f, r, vdot", range(n),
            lambda i: sum(1 + len(k.factors[rx]) for _, rx in k.vdot[i]),
            lambda i: f"    {acc('vdot', i)} = 0.0" + "".join(_term(c, f"({prod(rx)})") for c, rx in k.vdot[i]) + ";")
    bprod = lambda b: " * ".join([acc("r", k.blist[b][0])] + ([c_dbl(float(k.blist[b][1]))] if k.blist[b][1] > 1 else [])
                                 + [_factor(x, n, acc) for x in k.blist[b][2]])
    jargs = "const double* v, const double* f, const double* r, double* jvs"
    chunked("kqu_jac", jargs, "v, f, r, jvs", range(len(k.jvs)),
            lambda e: sum(1 + len(k.blist[b][2]) for _, b in k.jvs[e]) + 1,
            lambda e: f"    {acc('jvs', e)} = 0.0" + "".join(_term(c, f"({bprod(b)})") for c, b in k.jvs[e]) + ";")
    pos = {(k.lu_irow[e], k.lu_icol[e]): e for e in range(len(k.lu_irow))}

    def row_cost(row):
        return sum(1 + k.lu_crow[k.lu_icol[kk] + 1] - k.lu_diag[k.lu_icol[kk]] - 1
                   for kk in range(k.lu_crow[row], k.lu_diag[row])) + 1

    def split(rows, cost):
        groups, cur, acc_ops = [], [], 0
        for row in rows:
            if cur and acc_ops + cost(row) > chunk_ops:
                groups.append(cur)
                cur, acc_ops = [], 0
            cur.append(row)
            acc_ops += cost(row)
        if cur:
            groups.append(cur)
        return groups

    dgroups = split(range(n), row_cost)
    for gi, rows in enumerate(dgroups):
        out.append(f"{q} int kqu_decomp_{gi}(double* jvs)\n{{")
        for row in rows:
            out.append(f"    if (fabs({acc('jvs', k.lu_diag[row])}) < DBL_MIN) return {row + 1};")
            for kk in range(k.lu_crow[row], k.lu_diag[row]):
                j = k.lu_icol[kk]
                out.append(f"    {{ const double a = -{acc('jvs', kk)} / {acc('jvs', k.lu_diag[j])}; {acc('jvs', kk)} = -a;")
                for jj in range(k.lu_diag[j] + 1, k.lu_crow[j + 1]):
                    qq = pos[(row, k.lu_icol[jj])]
                    out.append(f"      {acc('jvs', qq)} = {acc('jvs', qq)} + a * {acc('jvs', jj)};")
                out.append("    }")
        out.append("    return 0;\n}\n")
    out.append(f"KQ_HD inline int kqu_decomp(double* jvs)\n{{\n    int rc;")
    out += [f"    if ((rc = kqu_decomp_{gi}(jvs)) != 0) return rc;" for gi in range(len(dgroups))]
    out.append("    return 0;\n}\n")
    fgroups = split(range(n), lambda row: k.lu_diag[row] - k.lu_crow[row] + 1)
    bgroups = split(range(n - 1, -1, -1), lambda row: k.lu_crow[row + 1] - k.lu_diag[row])
    for gi, rows in enumerate(fgroups):
        out.append(f"{q} void kqu_solve_f{gi}(const double* jvs, double* x)\n{{")
        for row in rows:
            terms = "".join(f" - {acc('jvs', kk)} * {acc('x', k.lu_icol[kk])}" for kk in range(k.lu_crow[row], k.lu_diag[row]))
            if terms:
                out.append(f"    {acc('x', row)} = {acc('x', row)}{terms};")
        out.append("}\n")
    for gi, rows in enumerate(bgroups):
        out.append(f"{q} void kqu_solve_b{gi}(const double* jvs, double* x)\n{{")
        for row in rows:
            terms = "".join(f" - {acc('jvs', kk)} * {acc('x', k.lu_icol[kk])}"
                            for kk in range(k.lu_diag[row] + 1, k.lu_crow[row + 1]))
            out.append(f"    {acc('x', row)} = ({acc('x', row)}{terms}) / {acc('jvs', k.lu_diag[row])};")
        out.append("}\n")
    out.append(f"KQ_HD inline void kqu_solve(const double* jvs, double* x)\n{{")
    out += [f"    kqu_solve_f{gi}(jvs, x);" for gi in range(len(fgroups))]
    out += [f"    kqu_solve_b{gi}(jvs, x);" for gi in range(len(bgroups))]
    out.append("}\n")
    return "\n".join(out)


def flop_counts(k: KppMech) -> dict:
    """Floating-point operations of the straight-line routines as emitted (a multiply by
    a coefficient of +-1 is not emitted; divide = 1), and of one Rodas3 attempt's vector
    work (11 axpys, 2 scaled by 1, the error norm's 6 per species)."""
    unit = lambda c: abs(c) == 1.0
    fun = sum(len(f) for f in k.factors) + sum(len(t) + sum(not unit(c) for c, _ in t) for t in k.vdot)
    jac = sum((b[1] > 1) + len(b[2]) for b in k.blist) + sum(len(t) + sum(not unit(c) for c, _ in t) for t in k.jvs)
    lower = sum(k.lu_diag[r] - k.lu_crow[r] for r in range(k.nvar))
    updates = sum(k.lu_crow[k.lu_icol[kk] + 1] - k.lu_diag[k.lu_icol[kk]] - 1
                  for r in range(k.nvar) for kk in range(k.lu_crow[r], k.lu_diag[r]))
    decomp = lower + 2 * updates + k.nvar                  # divisions, multiply-adds, diagonal shift
    solve = 2 * (len(k.lu_irow) - k.nvar) + k.nvar
    vector = 11 * 2 * k.nvar + 6 * k.nvar
    return {"fun": fun, "jac": jac, "decomp": decomp, "solve": solve, "vector": vector,
            "per_step": fun + jac, "per_attempt": decomp + 4 * solve + 2 * fun + vector}


# AQCHEM's GAS array (CCTM/src/cloud/acm_ae7_kmt2/AQ_DATA.F: srggas, in that order)
AQ_GAS = ("SO2", "HNO3", "N2O5", "CO2", "NH3", "H2O2", "O3", "FOA", "MHP", "PAA", "H2SO4", "HCL", "GLY", "MGLY",
          "HO", "IEPOX", "IMAE", "IHMML", "HO2", "NO2", "HONO", "HNO4", "GCOL", "CCOOH", "HCHO", "NO3RAD", "CH3O2",
          "HCHOP", "PYRUV")
# the aerosol surrogates AQCHEM reads or writes (AQ_DATA.F's LSO4, LNH4, ... used in aqchem_kmt.F90 and
# aqchem_Initialize.F90), in the order of the library's surrogate-position array
AQ_AEROSOL = ("SO4", "NH4", "NO3", "CL", "NA", "EC", "POA", "PRI", "SOA", "NUM", "SOILC", "SEASC", "ANTHC",
              "CAACC", "MGACC", "KACC", "FEACC", "MNACC", "ORGC", "TRACER_AKN", "TRACER_ACC", "TRACER_COR",
              "PHG_AKN", "PHG_ACC", "PHG_COR", "IETET", "IEOS", "DIMER", "IMGA", "IMOS", "ISO3")
# the coarse crustal factors of aqchem_kmt.F90:329-365: (name, AERO_DATA factor, bulk species, element, renorm)
CRUSTAL = (("SOIL_FE_FAC", "asoil_fe_fac", "ASOIL", "AFE", "asoil_renorm"),
           ("CORS_FE_FAC", "acors_fe_fac", "ACORS", "AFE", "acorsem_renorm"),
           ("SOIL_MN_FAC", "asoil_mn_fac", "ASOIL", "AMN", "asoil_renorm"),
           ("CORS_MN_FAC", "acors_mn_fac", "ACORS", "AMN", "acorsem_renorm"),
           ("SEAS_NA_FAC", "ascat_na_fac", "ASEACAT", "ANA", None),
           ("SOIL_NA_FAC", "asoil_na_fac", "ASOIL", "ANA", "asoil_renorm"),
           ("CORS_NA_FAC", "acors_na_fac", "ACORS", "ANA", "acorsem_renorm"),
           ("SEAS_MG_FAC", "ascat_mg_fac", "ASEACAT", "AMG", None),
           ("SOIL_MG_FAC", "asoil_mg_fac", "ASOIL", "AMG", "asoil_renorm"),
           ("CORS_MG_FAC", "acors_mg_fac", "ACORS", "AMG", "acorsem_renorm"),
           ("SEAS_CA_FAC", "ascat_ca_fac", "ASEACAT", "ACA", None),
           ("SOIL_CA_FAC", "asoil_ca_fac", "ASOIL", "ACA", "asoil_renorm"),
           ("CORS_CA_FAC", "acors_ca_fac", "ACORS", "ACA", "acorsem_renorm"),
           ("SEAS_K_FAC", "ascat_k_fac", "ASEACAT", "AK", None),
           ("SOIL_K_FAC", "asoil_k_fac", "ASOIL", "AK", "asoil_renorm"),
           ("CORS_K_FAC", "acors_k_fac", "ACORS", "AK", "acorsem_renorm"))


def crustal_factors(cmaq_root: str, mech: str = "cb6r5_ae7_aq") -> list[float]:
    """AQCHEM's first-call coarse crustal factors (aqchem_kmt.F90:329-365): AERO_DATA's
    REAL(8) speciation factors and renormalisations (CCTM/src/aero/aero6/AERO_DATA.F:591-627)
    times the ratio of the REAL(4) molecular weights of the mechanism's AE namelist
    (MECHS/<mech>/AE_<mech>.nml), in the reference's operation order."""
    import numpy as np
    root = Path(cmaq_root) / "CCTM" / "src"
    text = (root / "aero" / "aero6" / "AERO_DATA.F").read_text()
    const = {}
    for m in re.finditer(r"Real\(\s*8\s*\),\s*Parameter\s*::\s*(\w+)\s*=\s*([^!\n]+(?:\n\s*&[^!\n]+)*)", text):
        expr = re.sub(r"\n\s*&", " ", m.group(2)).strip()
        const[m.group(1).lower()] = expr
    def value(name):
        expr = const[name]
        terms = re.findall(r"([+-]?)\s*([0-9.]+D[+-]?[0-9]+|[0-9.]+|[a-z_0-9]+)", expr.replace(" ", ""))
        acc = None
        for sign, tok in terms:
            v = value(tok.lower()) if re.match(r"[a-z_]", tok) else float(tok.replace("D", "e"))
            acc = v if acc is None else (acc - v if sign == "-" else acc + v)
        return acc
    nml = (root / "MECHS" / mech / f"AE_{mech}.nml").read_text()
    mw = {m.group(1): float(np.float32(float(m.group(2))))
          for m in re.finditer(r"^'(\w+)'\s*,\s*([0-9.]+)", nml, flags=re.M)}
    out = []
    for _, fac, bulk, elem, renorm in CRUSTAL:
        v = value(fac) * mw[bulk] / mw[elem]
        if renorm:
            v = v / value(renorm)
        out.append(v)
    return out


def manifest(k: KppMech, cmaq_root: str | None = None) -> dict:
    m = {"mechanism": "kmt2 (CCTM/src/cloud/acm_ae7_kmt2)", "nvar": k.nvar, "nfix": k.nfix, "nreact": k.nreact,
         "lu_nonzero": len(k.lu_irow), "species": k.names, "flops": flop_counts(k)}
    if cmaq_root:
        m["aqchem"] = {"gas": list(AQ_GAS), "aerosol_surrogates": list(AQ_AEROSOL),
                       "crustal_factor_names": [c[0] for c in CRUSTAL],
                       "crustal_factors": crustal_factors(cmaq_root)}
    return m


def unrolled_source(k: KppMech) -> str:
    return ("/* Generated by cmaq_gb300/mechgen/kpp_aq.py from CCTM/src/cloud/acm_ae7_kmt2: straight-line\n"
            " * f, J, LU factorisation and solve of the KMT2 aqueous mechanism, the same operations in\n"
            " * the same order as the table-driven routines of oracle/kmt2_oracle.c.  Do not edit. */\n\n"
            + unrolled_routines(k))


def write_outputs(cmaq_root: str) -> KppMech:
    k = load(cmaq_root)
    odir = REPO / "oracle" / "gen"
    odir.mkdir(parents=True, exist_ok=True)
    (odir / "kmt2_aq.c").write_text(oracle_source(k))
    (odir / "kmt2_aq_unrolled.c").write_text(unrolled_source(k))
    cdir = REPO / "cmaq_gb300" / "csrc" / "gen"
    cdir.mkdir(parents=True, exist_ok=True)
    (cdir / "kmt2_aq_consts.cuh").write_text(device_consts(k))
    (cdir / "kmt2_aq.cuh").write_text(device_source(k))
    mdir = REPO / "cmaq_gb300" / "mechs" / "kmt2"
    mdir.mkdir(parents=True, exist_ok=True)
    (mdir / "manifest.json").write_text(json.dumps(manifest(k, cmaq_root), indent=1) + "\n")
    return k


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cmaq", default=os.environ.get("CMAQ_ROOT", ""))
    a = ap.parse_args(argv)
    if not a.cmaq:
        raise SystemExit("--cmaq <CMAQ source tree> is required")
    k = write_outputs(a.cmaq)
    print("kmt2", k.nvar, k.nfix, k.nreact, len(k.lu_irow), len(k.blist), len(k.henry))


if __name__ == "__main__":
    main()
