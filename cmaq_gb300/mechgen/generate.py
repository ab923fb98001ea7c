"""Mechanism generator: CMAQ mechanism tables -> manifest, oracle tables, CUDA kernels.

Usage (run where the CMAQ source tree is available; outputs are committed):

    python -m cmaq_gb300.mechgen.generate --mech cb6r5_ae7_aq --cmaq <CMAQ tree>

Reads ``CCTM/src/MECHS/<mech>/RXNS_DATA_MODULE.F90`` and ``RXNS_FUNC_MODULE.F90``
and writes

* ``cmaq_gb300/mechs/<mech>/manifest.json``   species, reactions, sparse structure, FLOP counts
* ``oracle/gen/<mech>_mech.c``                 tables + rate constants for the CPU oracle
* ``cmaq_gb300/csrc/gen/<mech>_*.cu[h]``      unrolled device code for the kernels
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
from pathlib import Path

from .emit_common import RATE_HELPERS, c_double, emit_expr
from .fortran_tables import Mechanism, parse_rxns_data
from .rate_expr import RateProgram, parse_rate_program
from .sparse import SparseMech, build_sparse, flop_counts

REPO = Path(__file__).resolve().parents[2]


def load(cmaq_root: str, mech: str):
    d = Path(cmaq_root) / "CCTM" / "src" / "MECHS" / mech
    data_text = (d / "RXNS_DATA_MODULE.F90").read_text()
    func_text = (d / "RXNS_FUNC_MODULE.F90").read_text()
    m = parse_rxns_data(data_text)
    prog = parse_rate_program(func_text, data_text)
    sp = build_sparse(m)
    src_hash = hashlib.sha256((data_text + func_text).encode()).hexdigest()[:16]
    return m, prog, sp, src_hash


# ----------------------------------------------------------------------------- manifest
def manifest(m: Mechanism, prog: RateProgram, sp: SparseMech, mech: str, src_hash: str) -> dict:
    photo_rx = set(prog.photo) | set(prog.seawater_cond)
    return {
        "mechanism": mech,
        "mechname": m.name,
        "source_sha256_16": src_hash,
        "nspec": m.nspec, "nrxns": m.nrxns, "ischan": sp.ischan, "mxprd": m.mxprd,
        "nphotab": m.nphotab, "nhetero": m.nhetero,
        "photab": m.photab, "hetero": m.hetero,
        "species": [{"name": m.species[i], "molwt": m.molwt[i], "cgrid_index": m.cgrid_index[i],
                     "type": m.species_type[i], "convert": m.convert_conc[i]} for i in range(m.nspec)],
        "inew2old": sp.inew2old, "iold2new": sp.iold2new,
        "reactions": [{"label": m.rxlabel[r], "nreact": m.nreact[r], "nprdct": m.nprdct[r],
                       "reactants": [m.irr[r][k] - 1 for k in range(m.nreact[r])],
                       "products": [m.irr[r][3 + k] - 1 for k in range(m.nprdct[r])],
                       "sc": m.sc[r][:m.nprdct[r]], "photolytic": bool((m.irxbits[r] >> 1) & 1),
                       "sunlit_rate_block": r in photo_rx, "ktype": m.ktype[r]}
                      for r in range(m.nrxns)],
        "third_body": m.third_body, "third_body_conc": m.third_body_conc,
        "rate_tables": {"ktype": m.ktype, "rtdat": m.rtdat, "rfdat": m.rfdat, "irrfall": m.irrfall,
                        "iorder": m.iorder, "kunits": m.kunits, "iph": m.iph, "ihetero": m.ihetero,
                        "rate_block": {str(r): ("photo" if r in prog.photo else "seawater" if r in
                                                prog.seawater_cond else "thermal") for r in range(m.nrxns)}},
        "active": sp.active, "iarray": sp.iarray, "nnz_jac": sp.nnz_jac,
        "flops_per_step": {"day": flop_counts(m, sp, 0), "night": flop_counts(m, sp, 1)},
    }


# ----------------------------------------------------------------------------- rate program -> C
def rate_body(m: Mechanism, prog: RateProgram, cell: str, rki, rj, het, indent: str) -> list[str]:
    """Statements computing all rate constants of one cell, in CALC_RCONST order.

    ``rki(k)``/``rj(k)``/``het(k)`` render array references; the caller declares
    ``temp, press, h2o, seawater, lsunlight`` for the cell."""
    def leaf(e):
        k = e[0]
        if k == "var":
            return e[1].lower()
        if k == "press":
            return "press"
        if k == "blktemp":
            return "temp_in"
        if k == "h2o":
            return "h2o"
        if k == "seawater":
            return "seawater"
        if k == "rj":
            return rj(e[1])
        if k == "het":
            return het(e[1])
        if k == "rki":
            return rki(e[1])
        raise ValueError(e)

    out = []
    I = indent
    out.append(f"{I}/* RKI = 0 (RXNS_FUNC_MODULE.F90 CALC_RCONST) */")
    for r in range(m.nrxns):
        out.append(f"{I}{rki(r)} = 0.0;")
    out.append(f"{I}if (lsunlight) {{")
    for r in prog.photo_order:
        if r in prog.seawater_cond:
            thr, e = prog.seawater_cond[r]
            out.append(f"{I}    if (seawater > {c_double(thr)}) {rki(r)} = {emit_expr(e, leaf)};")
            out.append(f"{I}    else {rki(r)} = 0.0;")
        else:
            out.append(f"{I}    {rki(r)} = {emit_expr(prog.photo[r], leaf)};")
    out.append(f"{I}}}")
    out.append(f"{I}{{")
    for name, e in prog.factors:
        out.append(f"{I}    const double {name.lower()} = {emit_expr(e, leaf)};")
    used = {n.lower() for n, _ in prog.factors}
    for r in prog.thermal_order:
        out.append(f"{I}    {rki(r)} = {emit_expr(prog.thermal[r], leaf)};")
    out.append(f"{I}    " + " ".join(f"(void){u};" for u in sorted(used)))
    out.append(f"{I}}}")
    order = ["M", "O2", "N2", "H2O", "H2", "CH4"]
    for key in order:
        for r in m.third_body.get(key, []):
            r0 = r - 1
            if key == "H2O":
                out.append(f"{I}{rki(r0)} = {rki(r0)} * h2o;")
            else:
                out.append(f"{I}{rki(r0)} = {rki(r0)} * {c_double(m.third_body_conc[key])};")
    return out


# ----------------------------------------------------------------------------- oracle tables
def _arr(ctype: str, name: str, vals, per_line: int = 16) -> str:
    vals = list(vals)
    if not vals:
        vals = [0]
    lines = []
    for i in range(0, len(vals), per_line):
        lines.append("    " + ", ".join(str(v) for v in vals[i:i + per_line]) + ",")
    return f"static const {ctype} {name}[{len(vals)}] = {{\n" + "\n".join(lines) + "\n};\n"


def oracle_source(m: Mechanism, prog: RateProgram, sp: SparseMech, mech: str, src_hash: str) -> str:
    nr, ns, n = m.nrxns, m.nspec, sp.ischan
    L = []
    L.append(f"/* Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/{mech}/RXNS_DATA_MODULE.F90")
    L.append(f" * and RXNS_FUNC_MODULE.F90 (sha256/16 {src_hash}).  Do not edit.")
    L.append(" * Tables follow the reference's symbolic set-up (CCTM/src/gas/ros3/rbsparse.F);")
    L.append(" * species indices are 0-based in the reordered (new) order, CC2 storage indices")
    L.append(" * are 1-based with slot 0 the reference's scratch slot. */")
    L.append(f'#define MECH_NAME "{mech}"')
    for k, v in (("NSPEC", ns), ("NRXNS", nr), ("ISCHAN", n), ("MXPRD", m.mxprd),
                 ("NPHOTAB", m.nphotab), ("NHETERO", m.nhetero),
                 ("MXARR", max(sp.iarray) + 1)):
        L.append(f"#define MECH_{k} {v}")
    L.append("#define CHEM_HD")
    L.append(RATE_HELPERS)
    L.append(_arr("double", "mech_molwt", [c_double(x) for x in m.molwt]))
    L.append(_arr("int", "mech_cgrid_index", m.cgrid_index))
    L.append(_arr("int", "mech_convert", [1 if c else 0 for c in m.convert_conc]))
    L.append(_arr("int", "mech_inew2old", sp.inew2old))
    L.append(_arr("int", "mech_iold2new", sp.iold2new))
    L.append(_arr("int", "mech_nreact", m.nreact))
    L.append(_arr("int", "mech_nprdct", m.nprdct))
    L.append(_arr("int", "mech_irm2", [x for r in range(nr) for x in sp.irm2[r]]))
    L.append(_arr("double", "mech_sc", [c_double(x) for r in range(nr) for x in m.sc[r]]))
    L.append(_arr("int", "mech_nuserat", [len(sp.active[0]), len(sp.active[1])]))
    L.append(_arr("int", "mech_nkuserat", sp.active[0] + [0] * (nr - len(sp.active[0]))
                  + sp.active[1] + [0] * (nr - len(sp.active[1]))))
    L.append(_arr("int", "mech_iarray", sp.iarray))
    for ncsp in range(2):
        lptr, liarp, lial, pptr, piarp, pial, pic = [0], [], [], [0], [], [], []
        for r in range(nr):
            for (iar, ial) in sp.loss_pd[ncsp].get(r, []):
                liarp.append(iar); lial.append(ial)
            lptr.append(len(liarp))
            for (iar, ial, ic) in sp.prod_pd[ncsp].get(r, []):
                piarp.append(iar); pial.append(ial); pic.append(ic)
            pptr.append(len(piarp))
        L.append(_arr("int", f"mech_loss_ptr{ncsp}", lptr))
        L.append(_arr("int", f"mech_loss_iarp{ncsp}", liarp))
        L.append(_arr("int", f"mech_loss_ial{ncsp}", lial))
        L.append(_arr("int", f"mech_prod_ptr{ncsp}", pptr))
        L.append(_arr("int", f"mech_prod_iarp{ncsp}", piarp))
        L.append(_arr("int", f"mech_prod_ial{ncsp}", pial))
        L.append(_arr("int", f"mech_prod_icoeff{ncsp}", pic))
        dptr, dij, dik, dkj = [0], [], [], []
        sptr, sij = [0], []
        for j in range(n):
            for (ij, ik, kj) in sp.decomp_ops[ncsp][j]:
                dij.append(ij); dik.append(ik); dkj.append(kj)
            dptr.append(len(dij))
            sij.extend(sp.lscale[ncsp][j])
            sptr.append(len(sij))
        L.append(_arr("int", f"mech_dec_ptr{ncsp}", dptr))
        L.append(_arr("int", f"mech_dec_ij{ncsp}", dij))
        L.append(_arr("int", f"mech_dec_ik{ncsp}", dik))
        L.append(_arr("int", f"mech_dec_kj{ncsp}", dkj))
        L.append(_arr("int", f"mech_lsc_ptr{ncsp}", sptr))
        L.append(_arr("int", f"mech_lsc_ij{ncsp}", sij))
        L.append(_arr("int", f"mech_diag{ncsp}", sp.diag[ncsp]))
        # back-substitution: KZERO (column of each stored entry, 1-based storage), per-row counts
        kzero = [0] * (sp.iarray[ncsp] + 1)
        for i in range(n):
            for (st, j) in sp.lower[ncsp][i]:
                kzero[st] = j
            for (st, j) in sp.upper[ncsp][i]:
                kzero[st] = j
        L.append(_arr("int", f"mech_kzero{ncsp}", kzero))
        L.append(_arr("int", f"mech_kzilch{ncsp}", [len(sp.lower[ncsp][i]) for i in range(n)]))
        L.append(_arr("int", f"mech_mzilch{ncsp}", [len(sp.upper[ncsp][i]) for i in range(n)]))
    L.append("static const int* const mech_loss_ptr[2] = {mech_loss_ptr0, mech_loss_ptr1};")
    L.append("static const int* const mech_loss_iarp[2] = {mech_loss_iarp0, mech_loss_iarp1};")
    L.append("static const int* const mech_loss_ial[2] = {mech_loss_ial0, mech_loss_ial1};")
    L.append("static const int* const mech_prod_ptr[2] = {mech_prod_ptr0, mech_prod_ptr1};")
    L.append("static const int* const mech_prod_iarp[2] = {mech_prod_iarp0, mech_prod_iarp1};")
    L.append("static const int* const mech_prod_ial[2] = {mech_prod_ial0, mech_prod_ial1};")
    L.append("static const int* const mech_prod_icoeff[2] = {mech_prod_icoeff0, mech_prod_icoeff1};")
    L.append("static const int* const mech_dec_ptr[2] = {mech_dec_ptr0, mech_dec_ptr1};")
    L.append("static const int* const mech_dec_ij[2] = {mech_dec_ij0, mech_dec_ij1};")
    L.append("static const int* const mech_dec_ik[2] = {mech_dec_ik0, mech_dec_ik1};")
    L.append("static const int* const mech_dec_kj[2] = {mech_dec_kj0, mech_dec_kj1};")
    L.append("static const int* const mech_lsc_ptr[2] = {mech_lsc_ptr0, mech_lsc_ptr1};")
    L.append("static const int* const mech_lsc_ij[2] = {mech_lsc_ij0, mech_lsc_ij1};")
    L.append("static const int* const mech_diag[2] = {mech_diag0, mech_diag1};")
    L.append("static const int* const mech_kzero[2] = {mech_kzero0, mech_kzero1};")
    L.append("static const int* const mech_kzilch[2] = {mech_kzilch0, mech_kzilch1};")
    L.append("static const int* const mech_mzilch[2] = {mech_mzilch0, mech_mzilch1};")
    # rate constants for a block (CALC_RCONST signature, arrays cell-fastest with leading dim ld)
    L.append("")
    L.append("/* Rate constants [ppm, min units] for cells 0..ncells-1 of a block; restates")
    L.append(f" * CALC_RCONST of CCTM/src/MECHS/{mech}/RXNS_FUNC_MODULE.F90. */")
    L.append("static void mech_calc_rconst(int ncells, int ld, const double* blktemp, const double* blkpres,")
    L.append("                             const double* blkh2o, const double* rjblk, const double* blkhet,")
    L.append("                             int lsunlight, const double* blkseawater, double* rki)")
    L.append("{")
    L.append("    for (int c = 0; c < ncells; ++c) {")
    L.append("        const double temp_in = blktemp[c];")
    L.append("        const double press = blkpres[c];")
    L.append("        const double h2o = blkh2o[c];")
    L.append("        const double seawater = blkseawater[c];")
    L.append("        (void)seawater; (void)h2o; (void)temp_in;")
    body = rate_body(m, prog, "c",
                     rki=lambda k: f"rki[(size_t){k} * ld + c]",
                     rj=lambda k: f"rjblk[(size_t){k} * ld + c]",
                     het=lambda k: f"blkhet[(size_t){k} * ld + c]",
                     indent="        ")
    L.extend(body)
    L.append("    }")
    L.append("}")
    return "\n".join(L) + "\n"


def ebi_oracle_source(ebi: dict, mech: str, nspec: int) -> str:
    from .ebi_translate import c_routines
    L = [f"/* Generated by cmaq_gb300.mechgen.generate from CCTM/src/gas/ebi_{mech}/hr*.F.  Do not edit.",
         " * EBI species list and tolerances (hrinit.F) and the translated straight-line routines",
         " * HRRATES, HRPRODLOSS, HRG1-HRG4; species indices 0-based in mechanism order. */",
         f"#define EBI_N_EBISP {len(ebi['ebisp'])}",
         f"#define EBI_DELTAT {c_double(ebi['deltat'])}",
         f"#define EBI_NEBITER {ebi['nebiter']}",
         f"#define EBI_NPNEG {len(ebi['pneg_species'])}",
         _arr("int", "ebi_ebisp", ebi["ebisp"]),
         _arr("double", "ebi_rtol", [c_double(ebi["rtol"][i]) for i in range(nspec)]),
         _arr("int", "ebi_pneg_species", ebi["pneg_species"] or [-1]),
         c_routines(ebi, "static")]
    return "\n".join(L)


def ebi_warp_tables(ebi: dict) -> dict:
    """Tables of HRRATES and HRPRODLOSS for the warp-cooperative EBI kernel.  Every
    statement of both routines is a left-deep product RKI(r) * YC(a) * ... or a left-deep
    sum of terms RXRAT(r) / c * RXRAT(r) (checked here), so a loop over a statement's
    table entries performs the same operations in the same order as the straight-line
    code.  HRPRODLOSS statements are spread over the 32 lanes longest first (each lane
    gets the next statement while it has the least work)."""
    rates = []
    for lhs, rhs in ebi["routines"]["hrrates"][1]:
        fac = []
        node = rhs
        while node[0] == "bin" and node[1] == "*":
            if node[3][0] != "arr" or node[3][1] != "YC":
                raise ValueError("unsupported HRRATES statement")
            fac.append(node[3][2])
            node = node[2]
        if not (lhs[0] == "arr" and lhs[1] == "RXRAT" and node[0] == "arr" and node[1] == "RKI"
                and node[2] == lhs[2] and len(fac) <= 3):
            raise ValueError("unsupported HRRATES statement")
        rates.append((lhs[2], list(reversed(fac))))

    def terms(node):
        if node[0] == "num" and node[1] == 0.0:
            return []
        if node[0] == "arr" and node[1] == "RXRAT":
            return [(node[2], 1.0)]
        if node[0] == "bin" and node[1] == "*" and node[2][0] == "num" and node[3][0] == "arr" \
                and node[3][1] == "RXRAT":
            return [(node[3][2], node[2][1])]
        if node[0] == "bin" and node[1] == "+":
            right = terms(node[3])
            if len(right) != 1:
                raise ValueError("unsupported HRPRODLOSS statement")
            return terms(node[2]) + right
        raise ValueError("unsupported HRPRODLOSS statement")
    kinds = {"PROD": 0, "LOSS": 1, "PNEG": 2}
    stmts = []
    for lhs, rhs in ebi["routines"]["hrprodloss"][1]:
        if lhs[0] != "arr" or lhs[1] not in kinds:
            raise ValueError("unsupported HRPRODLOSS target")
        stmts.append((kinds[lhs[1]], lhs[2], terms(rhs)))
    load = [0] * 32
    lanes = [[] for _ in range(32)]
    for st in sorted(stmts, key=lambda t: -max(1, len(t[2]))):
        k = min(range(32), key=lambda q: load[q])
        lanes[k].append(st)
        load[k] += max(1, len(st[2]))
    ordered = [st for lane in lanes for st in lane]
    ptr = [0]
    for lane in lanes:
        ptr.append(ptr[-1] + len(lane))
    t0, tr, tc = [], [], []
    for st in ordered:
        t0.append(len(tr))
        for (r, c) in st[2]:
            tr.append(r)
            tc.append(c)
    t0.append(len(tr))
    return {"rates": rates, "pl": ordered, "pl_ptr": ptr, "pl_t0": t0, "term_r": tr, "term_c": tc,
            "max_lane_terms": max(load)}


def ebi_cuda_source(ebi: dict, mech: str, nspec: int) -> tuple[str, str]:
    """(declarations for the mechanism header, translation unit of device routines)."""
    from .ebi_translate import c_routines
    ns_name = f"mech_{mech}"
    wt = ebi_warp_tables(ebi)
    nrate, npl, nterm = len(wt["rates"]), len(wt["pl"]), len(wt["term_r"])
    decl = [f"constexpr int EBI_N_EBISP = {len(ebi['ebisp'])};",
            f"constexpr double EBI_DELTAT = {c_double(ebi['deltat'])};",
            f"constexpr int EBI_NEBITER = {ebi['nebiter']};",
            f"constexpr int EBI_NPNEG = {len(ebi['pneg_species'])};",
            f"extern __constant__ int c_ebi_ebisp[{len(ebi['ebisp'])}];",
            f"extern __constant__ double c_ebi_rtol[{nspec}];",
            f"extern __constant__ int c_ebi_pneg[{max(1, len(ebi['pneg_species']))}];"]
    for name in ebi["routines"]:
        args = ", double dtc" if name.startswith("hrg") else ""
        decl.append(f"__device__ void ebi_{name}(double* __restrict__ ws{args});")
    # warp-cooperative kernel: cell state in shared memory, tables of HRRATES / HRPRODLOSS
    decl += [f"constexpr int EBIW_NRATE = {nrate};", f"constexpr int EBIW_NPL = {npl};",
             f"constexpr int EBIW_NTERM = {nterm};",
             "extern __device__ const int c_ebiw_rate_r[EBIW_NRATE];",
             "extern __device__ const int c_ebiw_rate_nf[EBIW_NRATE];",
             "extern __device__ const int c_ebiw_rate_sp[EBIW_NRATE * 3];",
             "extern __device__ const int c_ebiw_pl_ptr[33];",
             "extern __device__ const int c_ebiw_pl_kind[EBIW_NPL];",
             "extern __device__ const int c_ebiw_pl_sp[EBIW_NPL];",
             "extern __device__ const int c_ebiw_pl_t0[EBIW_NPL + 1];",
             "extern __device__ const int c_ebiw_term_r[EBIW_NTERM > 0 ? EBIW_NTERM : 1];",
             "extern __device__ const double c_ebiw_term_c[EBIW_NTERM > 0 ? EBIW_NTERM : 1];",
             "namespace wsm {"]
    for name in ("hrg1", "hrg2", "hrg3", "hrg4"):
        decl.append(f"__device__ void ebi_{name}(double* __restrict__ sm, double dtc);")
    decl.append("}  // namespace wsm")
    tu = [f"// Generated by cmaq_gb300.mechgen.generate from CCTM/src/gas/ebi_{mech}/hr*.F.  Do not edit.",
          "// Translated EBI routines HRRATES, HRPRODLOSS, HRG1-HRG4 on the per-cell workspace.",
          f'#include "{mech}_mech.cuh"', "#include <math.h>", f"namespace {ns_name} {{",
          f"__constant__ int c_ebi_ebisp[{len(ebi['ebisp'])}] = {{{', '.join(map(str, ebi['ebisp']))}}};",
          f"__constant__ double c_ebi_rtol[{nspec}] = {{{', '.join(c_double(ebi['rtol'][i]) for i in range(nspec))}}};",
          f"__constant__ int c_ebi_pneg[{max(1, len(ebi['pneg_species']))}] = "
          f"{{{', '.join(map(str, ebi['pneg_species'] or [-1]))}}};",
          "#define EBI_CELL_ARGS double* __restrict__ ws",
          "#define EBI_YC(i) ws[(EBI_OFF_YC + (i)) * 32]",
          "#define EBI_YC0(i) ws[(EBI_OFF_YC0 + (i)) * 32]",
          "#define EBI_YCP(i) ws[(EBI_OFF_YCP + (i)) * 32]",
          "#define EBI_RKI(r) ws[(OFF_RKI + (r)) * 32]",
          "#define EBI_RXRAT(r) ws[(OFF_RXRAT + (r)) * 32]",
          "#define EBI_PROD(i) ws[(EBI_OFF_PROD + (i)) * 32]",
          "#define EBI_LOSS(i) ws[(EBI_OFF_LOSS + (i)) * 32]",
          "#define EBI_PNEG(i) ws[(EBI_OFF_PNEG + (i)) * 32]",
          c_routines(ebi, "__device__ __noinline__")]

    def arr(ctype, name, vals, fmt=str):
        vals = list(vals) or [0]
        return f"__device__ const {ctype} {name}[{len(vals)}] = {{{', '.join(fmt(v) for v in vals)}}};"
    tu += ["// tables of the warp-cooperative kernel (HRRATES / HRPRODLOSS as data, same operation order)",
           arr("int", "c_ebiw_rate_r", [r for r, _ in wt["rates"]]),
           arr("int", "c_ebiw_rate_nf", [len(f) for _, f in wt["rates"]]),
           arr("int", "c_ebiw_rate_sp", [x for _, f in wt["rates"] for x in (f + [0, 0, 0])[:3]]),
           arr("int", "c_ebiw_pl_ptr", wt["pl_ptr"]),
           arr("int", "c_ebiw_pl_kind", [k for k, _, _ in wt["pl"]]),
           arr("int", "c_ebiw_pl_sp", [sp for _, sp, _ in wt["pl"]]),
           arr("int", "c_ebiw_pl_t0", wt["pl_t0"]),
           arr("int", "c_ebiw_term_r", wt["term_r"]),
           arr("double", "c_ebiw_term_c", wt["term_c"], c_double),
           "// HRG1-HRG4 on the warp's shared-memory cell state (run by one lane)",
           "namespace wsm {",
           "#undef EBI_CELL_ARGS", "#undef EBI_YC", "#undef EBI_YC0", "#undef EBI_YCP", "#undef EBI_RKI",
           "#undef EBI_RXRAT", "#undef EBI_PROD", "#undef EBI_LOSS", "#undef EBI_PNEG",
           "#define EBI_CELL_ARGS double* __restrict__ sm",
           "#define EBI_YC(i) sm[EBIW_YC + (i)]",
           "#define EBI_YC0(i) sm[EBIW_YC0 + (i)]",
           "#define EBI_YCP(i) sm[EBIW_YCP + (i)]",
           "#define EBI_RKI(r) sm[EBIW_RKI + (r)]",
           "#define EBI_RXRAT(r) sm[EBIW_RXRAT + (r)]",
           "#define EBI_PROD(i) sm[EBIW_PROD + (i)]",
           "#define EBI_LOSS(i) sm[EBIW_LOSS + (i)]",
           "#define EBI_PNEG(i) sm[EBIW_PNEG + (i)]",
           c_routines({**ebi, "routines": {k: v for k, v in ebi["routines"].items() if k.startswith("hrg")}},
                      "__device__ __noinline__"),
           "}  // namespace wsm",
           f"}}  // namespace {ns_name}"]
    return "\n".join(decl), "\n".join(tu) + "\n"


def write_outputs(cmaq_root: str, mech: str, out_root: Path = REPO) -> dict:
    m, prog, sp, src_hash = load(cmaq_root, mech)
    man = manifest(m, prog, sp, mech, src_hash)
    REPO_ = Path(out_root)
    mdir = REPO_ / "cmaq_gb300" / "mechs" / mech
    mdir.mkdir(parents=True, exist_ok=True)
    (mdir / "manifest.json").write_text(json.dumps(man, indent=1) + "\n")
    odir = REPO_ / "oracle" / "gen"
    odir.mkdir(parents=True, exist_ok=True)
    (odir / f"{mech}_mech.c").write_text(oracle_source(m, prog, sp, mech, src_hash))
    from .ebi_translate import parse_ebi
    ebi = parse_ebi(Path(cmaq_root) / "CCTM" / "src" / "gas" / f"ebi_{mech}")
    (odir / f"{mech}_ebi.c").write_text(ebi_oracle_source(ebi, mech, m.nspec))
    from .emit_cuda import cuda_sources
    cdir = REPO_ / "cmaq_gb300" / "csrc" / "gen"
    cdir.mkdir(parents=True, exist_ok=True)
    for old in cdir.glob(f"{mech}_*"):
        if not old.name.endswith("_hetchem.cuh"):   # written by mechgen/hetchem.py
            old.unlink()
    ebi_decl, ebi_tu = ebi_cuda_source(ebi, mech, m.nspec)
    for fname, text in cuda_sources(m, prog, sp, mech, src_hash, ebi_decl).items():
        (cdir / fname).write_text(text)
    (cdir / f"{mech}_ebi.cu").write_text(ebi_tu)
    return man


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--mech", action="append", required=True)
    ap.add_argument("--cmaq", default=os.environ.get("CMAQ_ROOT", ""))
    a = ap.parse_args(argv)
    if not a.cmaq:
        raise SystemExit("--cmaq <CMAQ source tree> is required")
    for mech in a.mech:
        man = write_outputs(a.cmaq, mech)
        print(mech, man["nspec"], man["nrxns"], man["iarray"], man["flops_per_step"]["day"]["step_total"])


if __name__ == "__main__":
    main()
