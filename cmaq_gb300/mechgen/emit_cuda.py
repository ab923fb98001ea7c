"""Emit fully unrolled FP64 device code for one mechanism.

Per-cell working storage lives in a per-warp block ``[element][lane]`` of global
memory: element ``k`` of a cell is at ``ws[k * 32]`` from the cell's thread
pointer, so each access of a warp is one contiguous 256-byte row and every
offset is a compile-time immediate.

Generated functions (namespace ``mech_<name>``; ``d`` = 0 day, 1 night):

* ``rconst``          rate constants, restating CALC_RCONST (RXNS_FUNC_MODULE.F90)
* ``feval_d``         YDOT = f(Y), reactions in the active order of rbfeval.F:80-151
* ``explic_d``        per-reaction partial-derivative products of rbjacob.F:112-143
* ``jacdecomp_d``     Jacobian (rbjacob.F), diagonal shift (rbsolver.F:377-381) and
                      LU without pivoting (rbdecomp.F), fused and ordered by rows
* ``solve_d``         forward / backward substitution (rbsolve.F)

Every sum is accumulated in the reference's order and every ``x +/- a*b`` of the
reference is a single ``fma``; the translation unit is compiled with
``-fmad=false`` so no other contraction happens.  The CPU oracle applies the
same rule, so both compute the same sums with the same roundings.
"""
from __future__ import annotations

from .emit_common import RATE_HELPERS, c_double
from .fortran_tables import Mechanism
from .rate_expr import RateProgram
from .sparse import SparseMech, flop_counts


class Layout:
    """Element offsets of the per-cell workspace."""

    def __init__(self, m: Mechanism, sp: SparseMech):
        ns, nr = m.nspec, m.nrxns
        off = 0
        self.y = off; off += ns
        self.yp = off; off += ns
        self.ydot = off; off += ns
        self.f0 = off; off += ns
        self.k1 = off; off += ns
        self.k2 = off; off += ns
        self.k3 = off; off += ns
        self.rki = off; off += nr
        self.rxrat = off; off += nr
        # partial-derivative products of multi-reactant reactions
        self.ex = {}
        for r in sp.active[0]:
            if m.nreact[r] >= 2:
                for ial in range(m.nreact[r]):
                    self.ex[(r, ial)] = off
                    off += 1
        self.yave = off; off += ns      # DDM-3D: time integral of Y over the accepted steps
        self.lu = off; off += max(sp.iarray) + 1      # 1-based storage, slot 0 unused
        # EBI species arrays overlay the LU region (the two solvers never share a cell state)
        self.ebi_yc = self.lu
        self.vdiag = off; off += sp.ischan
        off = max(off, self.ebi_yc + 6 * ns)
        self.total = off
        # discrete-adjoint arrays behind the forward workspace; only the adjoint kernels,
        # whose per-warp stride is ADJ_WS_ELEMS, use them
        self.adj_lam = off; off += ns       # adjoint of Y
        self.adj_mu1 = off; off += ns       # adjoints of the stages K1..K3, solved in place
        self.adj_mu2 = off; off += ns
        self.adj_mu3 = off; off += ns
        self.adj_phi = off; off += ns       # adjoint of an f evaluation
        self.adj_tmp = off; off += ns
        self.adj_emis = off; off += ns      # emission tendency added to f
        self.adj_ge = off; off += ns        # gradient wrt the emission tendency
        self.adj_gk = off; off += nr        # gradient wrt log rate multipliers
        self.adj_total = off
        # SMVGEAR: CNEW, GLOSS, DTLOS, CHOLD, CEST and the gathered concentrations reuse Y,
        # YDOT, K1, K2, K3 and F0; the Nordsieck history CONC (6 x ISCHAN) lies behind the
        # forward workspace (only the Gear kernels, per-warp stride GEAR_WS_ELEMS, use it)
        self.gear_conc = self.total
        self.gear_total = self.total + 6 * sp.ischan
        # DDM-3D with SMVGEAR: CAVEG (time integral over the accepted steps) uses YAVE, CFINI
        # (the state at the previous accepted step) follows the history
        self.gear_cfini = self.gear_total
        self.gear_total += ns


def _w(k: int) -> str:
    return f"ws[{k * 32}]"


def cuda_sources(m: Mechanism, prog: RateProgram, sp: SparseMech, mech: str, src_hash: str,
                 ebi_decl: str = "") -> dict[str, str]:
    """Return {file name: text}: one header with declarations and the kernel traits,
    and several translation units of device functions that compile in parallel
    (relocatable device code)."""
    lay = Layout(m, sp)
    ns, nr, n = m.nspec, m.nrxns, sp.ischan
    ns_name = f"mech_{mech}"
    banner = [f"// Generated by cmaq_gb300.mechgen.generate from CCTM/src/MECHS/{mech}/RXNS_DATA_MODULE.F90",
              f"// and RXNS_FUNC_MODULE.F90 (sha256/16 {src_hash}).  Do not edit."]
    units: dict[str, list[str]] = {}
    units["rates"] = _rconst(m, prog, lay)
    for d in range(2):
        units["rates"] += _feval(m, sp, lay, d) + _explic(m, sp, lay, d)
    # SMVGEAR uses the day pattern for every cell (see csrc/gear.cuh); the warp-per-cell
    # kernel runs table-driven cooperative forms of its routines
    units["rates"] += _explic(m, sp, lay, 0, gear=True)
    gw_decl, gw_defs, gw_info = _gear_warp_tables(m, sp, lay)
    units["gw_tables"] = gw_defs
    decls: list[str] = ["__device__ void rconst(double* __restrict__ ws, double temp_in, double press, double h2o, "
                        "double seawater, int lsunlight, const double* __restrict__ rjv, const double* __restrict__ hetv);"]
    for d in range(2):
        decls.append(f"__device__ void feval_{d}(double* __restrict__ ws, int src, int dst);")
        decls.append(f"__device__ void explic_{d}(double* __restrict__ ws);")
    decls.append("__device__ void gear_explic_0(double* __restrict__ ws);")
    wrappers: list[str] = []
    for d in range(1):
        gchunks = _jacdecomp_chunks(m, sp, lay, d, gear=True)
        for ci, code in enumerate(gchunks):
            units.setdefault(f"glu{d}_{ci // 3}", []).extend(code)
            decls.append(f"__device__ void gear_pdecomp_{d}_{ci}(double* __restrict__ ws, double r1delt);")
        wrappers.append(f"__device__ __forceinline__ void gear_pdecomp_{d}(double* __restrict__ ws, double r1delt)")
        wrappers.append("{")
        wrappers.extend(f"    gear_pdecomp_{d}_{ci}(ws, r1delt);" for ci in range(len(gchunks)))
        wrappers.append("}")
    for d in range(2):
        chunks = _jacdecomp_chunks(m, sp, lay, d)
        for ci, code in enumerate(chunks):
            unit = f"lu{d}_{ci // 3}"
            units.setdefault(unit, []).extend(code)
            decls.append(f"__device__ void jacdecomp_{d}_{ci}(double* __restrict__ ws, double gdtinv);")
        wrappers.append(f"__device__ __forceinline__ void jacdecomp_{d}(double* __restrict__ ws, double gdtinv)")
        wrappers.append("{")
        wrappers.extend(f"    jacdecomp_{d}_{ci}(ws, gdtinv);" for ci in range(len(chunks)))
        wrappers.append("}")
        # block-synchronous form: every thread calls it, `go` lanes work, barrier after each chunk
        wrappers.append(f"__device__ __forceinline__ void jacdecomp_{d}_sync(double* __restrict__ ws, double gdtinv, bool go)")
        wrappers.append("{")
        wrappers.extend(f"    if (go) jacdecomp_{d}_{ci}(ws, gdtinv);\n    __syncthreads();" for ci in range(len(chunks)))
        wrappers.append("}")
        schunks = _solve_chunks(sp, lay, d)
        for ci, code in enumerate(schunks):
            unit = f"solve{d}"
            units.setdefault(unit, []).extend(code)
            decls.append(f"__device__ void solve_{d}_{ci}(double* __restrict__ ws, int rhs);")
        wrappers.append(f"__device__ __forceinline__ void solve_{d}(double* __restrict__ ws, int rhs)")
        wrappers.append("{")
        wrappers.extend(f"    solve_{d}_{ci}(ws, rhs);" for ci in range(len(schunks)))
        wrappers.append("}")
        wrappers.append(f"__device__ __forceinline__ void solve_{d}_sync(double* __restrict__ ws, int rhs, bool go)")
        wrappers.append("{")
        wrappers.extend(f"    if (go) solve_{d}_{ci}(ws, rhs);\n    __syncthreads();" for ci in range(len(schunks)))
        wrappers.append("}")

    for d in range(2):
        tchunks = _solve_t_chunks(sp, lay, d)
        for ci, code in enumerate(tchunks):
            units.setdefault(f"solvet{d}", []).extend(code)
            decls.append(f"__device__ void solve_t_{d}_{ci}(double* __restrict__ ws, int rhs);")
        wrappers.append(f"__device__ __forceinline__ void solve_t_{d}(double* __restrict__ ws, int rhs)")
        wrappers.append("{")
        wrappers.extend(f"    solve_t_{d}_{ci}(ws, rhs);" for ci in range(len(tchunks)))
        wrappers.append("}")
        # reaction-wise adjoint routines in bounded chunks, spread over translation units
        for kind, chunks, sig, call in (
                ("jtv", _adj_jtv(m, sp, lay, d), "double* __restrict__ ws, int yoff, int phioff, int outoff",
                 "ws, yoff, phioff, outoff"),
                ("hess3", _adj_hess3(m, sp, lay, d), "double* __restrict__ ws", "ws")):
            for ci, code in enumerate(chunks):
                units.setdefault(f"adj{d}_{kind}{ci // 4}", []).extend(code)
                decls.append(f"__device__ void adj_{kind}_{d}_{ci}({sig});")
            wrappers.append(f"__device__ __forceinline__ void adj_{kind}_{d}({sig})")
            wrappers.append("{")
            wrappers.extend(f"    adj_{kind}_{d}_{ci}({call});" for ci in range(len(chunks)))
            wrappers.append("}")

    for d in range(2):
        for kind, chunks, sig, call in (
                ("jv", _ddm_jv(m, sp, lay, d), "double* __restrict__ ws, int yoff, int voff, int outoff",
                 "ws, yoff, voff, outoff"),
                ("src", _ddm_src(m, sp, lay, d),
                 "double* __restrict__ ws, const unsigned char* __restrict__ mask, double scale, int outoff",
                 "ws, mask, scale, outoff")):
            for ci, code in enumerate(chunks):
                units.setdefault(f"ddm{d}_{kind}{ci // 4}", []).extend(code)
                decls.append(f"__device__ void ddm_{kind}_{d}_{ci}({sig});")
            wrappers.append(f"__device__ __forceinline__ void ddm_{kind}_{d}({sig})")
            wrappers.append("{")
            wrappers.extend(f"    ddm_{kind}_{d}_{ci}({call});" for ci in range(len(chunks)))
            wrappers.append("}")

    h = banner + ["#pragma once", "#include <cuda_runtime.h>", "#ifndef CHEM_HD", "#define CHEM_HD __device__",
                  "#endif",
                  "// load of an LU factor or 1/U(i,i); a build may define it as a streaming load (__ldcs)",
                  "#ifndef CHEM_LDLU", "#define CHEM_LDLU(p) (*(p))", "#endif",
                  "// L2 prefetch of workspace entries a few rows ahead (build variant 'pf'); off by default",
                  "#ifdef CHEM_USE_PREFETCH",
                  "__device__ __forceinline__ void chem_prefetch_l2(const double* p)",
                  "{",
                  '    asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(p)));',
                  "}",
                  "#define CHEM_PREFETCH(p) chem_prefetch_l2(p)",
                  "#else",
                  "#define CHEM_PREFETCH(p) ((void)0)",
                  "#endif",
                  "// L1 prefetch of the entries the next row reads (build variant 'pfl1'); off by default",
                  "#ifdef CHEM_USE_PREFETCH_L1",
                  "__device__ __forceinline__ void chem_prefetch_l1(const double* p)",
                  "{",
                  '    asm volatile("prefetch.global.L1 [%0];" ::"l"(__cvta_generic_to_global(p)));',
                  "}",
                  "#define CHEM_PREFETCH_L1(p) chem_prefetch_l1(p)",
                  "#else",
                  "#define CHEM_PREFETCH_L1(p) ((void)0)",
                  "#endif",
                  "// 1/U(i,i): IEEE division by default; a build may use the correctly rounded",
                  "// reciprocal __drcp_rn, which gives the same bits",
                  "#ifndef CHEM_RCP",
                  "#define CHEM_RCP(x) (1.0 / (x))",
                  "#endif",
                  f"namespace {ns_name} {{", f'constexpr const char* NAME = "{mech}";']
    consts = (("NSPEC", ns), ("NRXNS", nr), ("ISCHAN", n), ("NPHOTAB", m.nphotab),
              ("NHETERO", m.nhetero), ("WS_ELEMS", lay.total), ("OFF_Y", lay.y), ("OFF_YP", lay.yp),
              ("OFF_YDOT", lay.ydot), ("OFF_F0", lay.f0), ("OFF_K1", lay.k1), ("OFF_K2", lay.k2),
              ("OFF_K3", lay.k3), ("OFF_RKI", lay.rki), ("OFF_RXRAT", lay.rxrat), ("OFF_LU", lay.lu),
              ("OFF_VDIAG", lay.vdiag), ("IARRAY_DAY", sp.iarray[0]), ("IARRAY_NIGHT", sp.iarray[1]),
              # EBI cell state reuses the workspace: YC, YC0, YCP, PROD, LOSS, PNEG after RKI/RXRAT
              ("EBI_OFF_YC", lay.ebi_yc), ("EBI_OFF_YC0", lay.ebi_yc + ns), ("EBI_OFF_YCP", lay.ebi_yc + 2 * ns),
              ("EBI_OFF_PROD", lay.ebi_yc + 3 * ns), ("EBI_OFF_LOSS", lay.ebi_yc + 4 * ns),
              ("EBI_OFF_PNEG", lay.ebi_yc + 5 * ns),
              ("ADJ_WS_ELEMS", lay.adj_total), ("ADJ_LAM", lay.adj_lam), ("ADJ_MU1", lay.adj_mu1),
              ("ADJ_MU2", lay.adj_mu2), ("ADJ_MU3", lay.adj_mu3), ("ADJ_PHI", lay.adj_phi),
              ("ADJ_TMP", lay.adj_tmp), ("ADJ_EMIS", lay.adj_emis), ("ADJ_GE", lay.adj_ge),
              ("ADJ_GK", lay.adj_gk), ("OFF_YAVE", lay.yave),
              ("GEAR_WS_ELEMS", lay.gear_total), ("GEAR_CNEW", lay.y), ("GEAR_GLOSS", lay.ydot),
              ("GEAR_DTLOS", lay.k1), ("GEAR_CHOLD", lay.k2), ("GEAR_CEST", lay.k3), ("GEAR_BLKCONC", lay.f0),
              ("GEAR_CONC", lay.gear_conc), ("GEAR_E", lay.yp), ("GEAR_CAVEG", lay.yave),
              ("GEAR_CFINI", lay.gear_cfini),
              # warp-cooperative EBI: one cell's state in shared memory (doubles)
              ("EBIW_YC", 0), ("EBIW_YC0", ns), ("EBIW_YCP", 2 * ns), ("EBIW_PROD", 3 * ns),
              ("EBIW_LOSS", 4 * ns), ("EBIW_PNEG", 5 * ns), ("EBIW_NOTMAX", 6 * ns), ("EBIW_RKI", 7 * ns),
              ("EBIW_RXRAT", 7 * ns + nr), ("EBIW_ELEMS", 7 * ns + 2 * nr))
    for k, v in consts:
        h.append(f"constexpr int {k} = {v};")
    h.append(f"constexpr double FLOPS_STEP_DAY = {float(flop_counts(m, sp, 0)['step_total'])};")
    h.append(f"constexpr double FLOPS_STEP_NIGHT = {float(flop_counts(m, sp, 1)['step_total'])};")
    h.append(f"extern __constant__ int c_inew2old[{ns}];")
    h.append(f"extern __constant__ int c_iold2new[{ns}];")
    h.append(f"static const int h_inew2old[{ns}] = {{{', '.join(map(str, sp.inew2old))}}};")
    h.append(f"static const int h_iold2new[{ns}] = {{{', '.join(map(str, sp.iold2new))}}};")
    h.append(f"static const int h_cgrid_index[{ns}] = {{{', '.join(str(x - 1) for x in m.cgrid_index)}}};")
    h.append(f"static const int h_convert[{ns}] = {{{', '.join('1' if c else '0' for c in m.convert_conc)}}};")
    h.append(f"static const double h_molwt[{ns}] = {{{', '.join(c_double(x) for x in m.molwt)}}};")
    h.extend(decls)
    h.extend(gw_decl)
    if ebi_decl:
        h.append(ebi_decl)
    h.extend(wrappers)
    h.append("struct Traits {")
    for k, _ in consts:
        h.append(f"    static constexpr int {k} = {ns_name}::{k};")
    h.append(f"    static constexpr const char* name() {{ return {ns_name}::NAME; }}")
    h.append(f"    static __device__ __forceinline__ int iold2new(int s) {{ return {ns_name}::c_iold2new[s]; }}")
    h.append(f"    static __device__ __forceinline__ int inew2old(int i) {{ return {ns_name}::c_inew2old[i]; }}")
    for d in range(2):
        h.append(f"    static __device__ __forceinline__ void feval_{d}(double* ws, int s, int t) {{ {ns_name}::feval_{d}(ws, s, t); }}")
        h.append(f"    static __device__ __forceinline__ void explic_{d}(double* ws) {{ {ns_name}::explic_{d}(ws); }}")
        if d == 0:
            h.append(f"    static __device__ __forceinline__ void gear_explic_0(double* ws) {{ {ns_name}::gear_explic_0(ws); }}")
            h.append(f"    static __device__ __forceinline__ void gear_pdecomp_0(double* ws, double r) {{ {ns_name}::gear_pdecomp_0(ws, r); }}")
        h.append(f"    static __device__ __forceinline__ void jacdecomp_{d}(double* ws, double g) {{ {ns_name}::jacdecomp_{d}(ws, g); }}")
        h.append(f"    static __device__ __forceinline__ void solve_{d}(double* ws, int r) {{ {ns_name}::solve_{d}(ws, r); }}")
        h.append(f"    static __device__ __forceinline__ void jacdecomp_{d}_sync(double* ws, double g, bool go) {{ {ns_name}::jacdecomp_{d}_sync(ws, g, go); }}")
        h.append(f"    static __device__ __forceinline__ void solve_{d}_sync(double* ws, int r, bool go) {{ {ns_name}::solve_{d}_sync(ws, r, go); }}")
        h.append(f"    static __device__ __forceinline__ void solve_t_{d}(double* ws, int r) {{ {ns_name}::solve_t_{d}(ws, r); }}")
        h.append(f"    static __device__ __forceinline__ void adj_jtv_{d}(double* ws, int y, int phi, int out) {{ {ns_name}::adj_jtv_{d}(ws, y, phi, out); }}")
        h.append(f"    static __device__ __forceinline__ void adj_hess3_{d}(double* ws) {{ {ns_name}::adj_hess3_{d}(ws); }}")
        h.append(f"    static __device__ __forceinline__ void ddm_jv_{d}(double* ws, int y, int v, int out) {{ {ns_name}::ddm_jv_{d}(ws, y, v, out); }}")
        h.append(f"    static __device__ __forceinline__ void ddm_src_{d}(double* ws, const unsigned char* mk, double sc, int out) {{ {ns_name}::ddm_src_{d}(ws, mk, sc, out); }}")
    if ebi_decl:
        h.append(f"    static constexpr int EBI_N_EBISP = {ns_name}::EBI_N_EBISP;")
        h.append(f"    static constexpr int EBI_NEBITER = {ns_name}::EBI_NEBITER;")
        h.append(f"    static constexpr int EBI_NPNEG = {ns_name}::EBI_NPNEG;")
        h.append(f"    static constexpr double EBI_DELTAT = {ns_name}::EBI_DELTAT;")
        h.append(f"    static __device__ __forceinline__ int ebi_ebisp(int e) {{ return {ns_name}::c_ebi_ebisp[e]; }}")
        h.append(f"    static __device__ __forceinline__ double ebi_rtol(int i) {{ return {ns_name}::c_ebi_rtol[i]; }}")
        h.append(f"    static __device__ __forceinline__ int ebi_pneg(int k) {{ return {ns_name}::c_ebi_pneg[k]; }}")
        for nm in ("hrrates", "hrprodloss"):
            h.append(f"    static __device__ __forceinline__ void ebi_{nm}(double* ws) {{ {ns_name}::ebi_{nm}(ws); }}")
        for nm in ("hrg1", "hrg2", "hrg3", "hrg4"):
            h.append(f"    static __device__ __forceinline__ void ebi_{nm}(double* ws, double dtc) {{ {ns_name}::ebi_{nm}(ws, dtc); }}")
            h.append(f"    static __device__ __forceinline__ void ebiw_{nm}(double* sm, double dtc) {{ {ns_name}::wsm::ebi_{nm}(sm, dtc); }}")
        h.append(f"    static constexpr int EBIW_NRATE = {ns_name}::EBIW_NRATE;")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_rate_r() {{ return {ns_name}::c_ebiw_rate_r; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_rate_nf() {{ return {ns_name}::c_ebiw_rate_nf; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_rate_sp() {{ return {ns_name}::c_ebiw_rate_sp; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_pl_ptr() {{ return {ns_name}::c_ebiw_pl_ptr; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_pl_kind() {{ return {ns_name}::c_ebiw_pl_kind; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_pl_sp() {{ return {ns_name}::c_ebiw_pl_sp; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_pl_t0() {{ return {ns_name}::c_ebiw_pl_t0; }}")
        h.append(f"    static __device__ __forceinline__ const int* ebiw_term_r() {{ return {ns_name}::c_ebiw_term_r; }}")
        h.append(f"    static __device__ __forceinline__ const double* ebiw_term_c() {{ return {ns_name}::c_ebiw_term_c; }}")
    for k, v in gw_info["sizes"].items():
        h.append(f"    static constexpr int {k} = {v};")
    for k in gw_info["names"]:
        ty = "double" if k in ("sum_c", "asm_c") else "int"
        h.append(f"    static __device__ __forceinline__ const {ty}* gw_{k}() {{ return {ns_name}::c_gw_{k}; }}")
    h.append("    static __device__ __forceinline__ void rconst(double* ws, double t, double p, double h, double sw, int sun,")
    h.append(f"                                                  const double* rj, const double* het) {{ {ns_name}::rconst(ws, t, p, h, sw, sun, rj, het); }}")
    h.append("};")
    h.append(f"}}  // namespace {ns_name}")
    files = {f"{mech}_mech.cuh": "\n".join(h) + "\n"}
    for unit, body in units.items():
        t = banner + [f'#include "{mech}_mech.cuh"', "#include <math.h>", f"namespace {ns_name} {{"]
        if unit == "rates":
            t.append(RATE_HELPERS)
            t.append(f"__constant__ int c_inew2old[{ns}] = {{{', '.join(map(str, sp.inew2old))}}};")
            t.append(f"__constant__ int c_iold2new[{ns}] = {{{', '.join(map(str, sp.iold2new))}}};")
        t.extend(body)
        t.append(f"}}  // namespace {ns_name}")
        files[f"{mech}_{unit}.cu"] = "\n".join(t) + "\n"
    return files


def _gear_warp_tables(m: Mechanism, sp: SparseMech, lay: Layout) -> tuple[list[str], list[str], dict]:
    """Tables of the warp-cooperative SMVGEAR routines (day pattern), each listing the
    operations of the generated sequential routines in an order that lanes can share
    without changing any element's operation sequence:
      rates (RXRAT of each active reaction) and, per species, its derivative terms in
      RBFEVAL's order, species given to lanes longest-first;
      the partial-derivative products (EXPLIC) of 2- and 3-reactant reactions;
      per LU storage entry its P assembly terms in PDERIV's order;
      the elimination by pivot (right-looking): the L entries a pivot scales and the
      updates it makes, each entry still receiving its updates in ascending pivot order;
      forward and backward substitution rows grouped in dependency levels.
    Returns (header declarations, table definitions, sizes)."""
    d = 0
    n = sp.ischan
    act = list(sp.active[d])
    rate_sp = []
    for r in act:
        rate_sp += [sp.irm2[r][i] if i < m.nreact[r] else -1 for i in range(3)]
    contrib: dict[int, list] = {}
    for r in act:
        for i in range(m.nreact[r]):
            contrib.setdefault(sp.irm2[r][i], []).append((r, None))
        for p in range(m.nprdct[r]):
            contrib.setdefault(sp.irm2[r][3 + p], []).append((r, m.sc[r][p]))
    sum_ptr, sum_r, sum_k, sum_c = [0], [], [], []
    for s_ in range(n):
        for (r, c) in contrib.get(s_, []):
            sum_r.append(r)
            sum_k.append(0 if c is None else 1)
            sum_c.append(0.0 if c is None else c)
        sum_ptr.append(len(sum_r))
    loads = [0] * 32
    lanes: list[list[int]] = [[] for _ in range(32)]
    for s_ in sorted(range(n), key=lambda q: -(sum_ptr[q + 1] - sum_ptr[q])):
        ln = min(range(32), key=lambda q: loads[q])
        lanes[ln].append(s_)
        loads[ln] += sum_ptr[s_ + 1] - sum_ptr[s_] + 1
    lane_ptr, lane_sp = [0], []
    for ln in range(32):
        lane_sp += lanes[ln]
        lane_ptr.append(len(lane_sp))
    ex_r, ex_sp, ex_off = [], [], []
    for r in act:
        if m.nreact[r] >= 2:
            ex_r.append(r)
            ex_sp += [sp.irm2[r][i] if i < m.nreact[r] else -1 for i in range(3)]
            ex_off.append(lay.ex[(r, 0)])
    terms = _jac_terms(m, sp, d)
    iarr = sp.iarray[d]
    asm_ptr, asm_src, asm_kind, asm_c = [0, 0], [], [], []
    for st in range(1, iarr + 1):
        for (r, ial, coef, sign) in terms.get(st, []):
            asm_src.append(lay.rki + r if m.nreact[r] == 1 else lay.ex[(r, ial)])
            asm_kind.append(-1 if sign < 0 else (0 if coef is None else 1))
            asm_c.append(0.0 if coef is None else coef)
        asm_ptr.append(len(asm_src))
    jpt = sp.jarraypt[d]
    piv_diag = [jpt[(k, k)] for k in range(n)]
    lsc_ptr, lsc_st, up_ptr, up_ij, up_ik, up_kj = [0], [], [0], [], [], []
    rows_of = {k: [] for k in range(n)}
    for i in range(n):
        for (st_ik, k) in sp.lower[d][i]:
            rows_of[k].append((i, st_ik))
    for k in range(n):
        for (i, st_ik) in rows_of[k]:
            lsc_st.append(st_ik)
            for (st_kj, j) in sp.upper[d][k]:
                up_ij.append(jpt[(i, j)])
                up_ik.append(st_ik)
                up_kj.append(st_kj)
        lsc_ptr.append(len(lsc_st))
        up_ptr.append(len(up_ij))

    def levels(deps, order):
        lv = {}
        for i in order:
            lv[i] = 1 + max((lv[j] for j in deps(i)), default=0)
        nl = max(lv.values())
        ptr, rows = [0], []
        for l in range(1, nl + 1):
            rows += [i for i in order if lv[i] == l]
            ptr.append(len(rows))
        return ptr, rows
    fl_ptr, fl_row = levels(lambda i: [j for (_, j) in sp.lower[d][i]], list(range(n)))
    bl_ptr, bl_row = levels(lambda i: [j for (_, j) in sp.upper[d][i]], list(range(n - 1, -1, -1)))
    fr_ptr, fr_st, fr_col, br_ptr, br_st, br_col = [0], [], [], [0], [], []
    for i in range(n):
        for (st, j) in sp.lower[d][i]:
            fr_st.append(st); fr_col.append(j)
        fr_ptr.append(len(fr_st))
        for (st, j) in sp.upper[d][i]:
            br_st.append(st); br_col.append(j)
        br_ptr.append(len(br_st))
    ints = {"act_r": act, "act_sp": rate_sp, "sum_ptr": sum_ptr, "sum_r": sum_r, "sum_k": sum_k,
            "lane_ptr": lane_ptr, "lane_sp": lane_sp, "ex_r": ex_r, "ex_sp": ex_sp, "ex_off": ex_off,
            "asm_ptr": asm_ptr, "asm_src": asm_src, "asm_kind": asm_kind, "piv_diag": piv_diag,
            "lsc_ptr": lsc_ptr, "lsc_st": lsc_st, "up_ptr": up_ptr, "up_ij": up_ij, "up_ik": up_ik,
            "up_kj": up_kj, "fl_ptr": fl_ptr, "fl_row": fl_row, "bl_ptr": bl_ptr, "bl_row": bl_row,
            "fr_ptr": fr_ptr, "fr_st": fr_st, "fr_col": fr_col, "br_ptr": br_ptr, "br_st": br_st,
            "br_col": br_col}
    dbls = {"sum_c": sum_c, "asm_c": asm_c}
    sizes = {"GW_NACT": len(act), "GW_NEX": len(ex_r), "GW_NFL": len(fl_ptr) - 1, "GW_NBL": len(bl_ptr) - 1}
    decl, defs = [], []
    for k, v in ints.items():
        v = v or [0]
        decl.append(f"extern __device__ const int c_gw_{k}[{len(v)}];")
        defs.append(f"__device__ const int c_gw_{k}[{len(v)}] = {{{', '.join(map(str, v))}}};")
    for k, v in dbls.items():
        v = v or [0.0]
        decl.append(f"extern __device__ const double c_gw_{k}[{len(v)}];")
        defs.append(f"__device__ const double c_gw_{k}[{len(v)}] = {{{', '.join(c_double(x) for x in v)}}};")
    return decl, defs, {"sizes": sizes, "names": list(ints) + list(dbls)}


def _rconst(m: Mechanism, prog: RateProgram, lay: Layout) -> list[str]:
    from .generate import rate_body
    o = ["// Rate constants of one cell into ws[OFF_RKI + r] (CALC_RCONST, RXNS_FUNC_MODULE.F90).",
         "__device__ __noinline__ void rconst(double* __restrict__ ws, double temp_in, double press, double h2o,",
         "                                    double seawater, int lsunlight, const double* __restrict__ rjv,",
         "                                    const double* __restrict__ hetv)",
         "{"]
    body = rate_body(m, prog, "c",
                     rki=lambda k: _w(lay.rki + k),
                     rj=lambda k: f"rjv[{k}]",
                     het=lambda k: f"hetv[{k}]",
                     indent="    ")
    o.extend(body)
    o.append("}")
    return o


def _feval(m: Mechanism, sp: SparseMech, lay: Layout, d: int) -> list[str]:
    """ws[dst..] = f(ws[src..]) in two phases: reaction rates into ws (RXRAT of
    rbfeval.F:88-127), then each species' rate of change summed over its loss and
    production terms in the reference's reaction order (rbfeval.F:129-151)."""
    contrib: dict[int, list] = {}
    for r in sp.active[d]:
        for i in range(m.nreact[r]):
            contrib.setdefault(sp.irm2[r][i], []).append((r, None))
        for p in range(m.nprdct[r]):
            contrib.setdefault(sp.irm2[r][3 + p], []).append((r, m.sc[r][p]))
    o = [f"// f(y) for the {'day' if d == 0 else 'night'} reaction list (rbfeval.F:80-151).",
         f"__device__ __noinline__ void feval_{d}(double* __restrict__ ws, int src, int dst)",
         "{",
         "    const double* __restrict__ yin = ws + src * 32;",
         "    double* __restrict__ yout = ws + dst * 32;"]
    for r in sp.active[d]:
        expr = _w(lay.rki + r)
        for i in range(m.nreact[r]):
            expr = f"({expr}) * yin[{sp.irm2[r][i] * 32}]"
        o.append(f"    {_w(lay.rxrat + r)} = {expr};")
    for s_ in range(sp.ischan):
        terms = contrib.get(s_, [])
        if not terms:
            o.append(f"    yout[{s_ * 32}] = 0.0;")
            continue
        o.append("    {")
        for t, (r, scv) in enumerate(terms):
            rr = _w(lay.rxrat + r)
            if t == 0:
                o.append(f"      double a = {'-' + rr if scv is None else c_double(scv) + ' * ' + rr};")
            elif scv is None:
                o.append(f"      a = a - {rr};")
            else:
                o.append(f"      a = fma({c_double(scv)}, {rr}, a);")
        o.append(f"      yout[{s_ * 32}] = a;")
        o.append("    }")
    o.append("}")
    return o


def _ex_ref(m: Mechanism, sp: SparseMech, lay: Layout, r: int, ial: int) -> str:
    if m.nreact[r] == 1:
        return _w(lay.rki + r)
    return _w(lay.ex[(r, ial)])


def _explic(m: Mechanism, sp: SparseMech, lay: Layout, d: int, gear: bool = False) -> list[str]:
    """Partial-derivative products of 2- and 3-reactant reactions into the EX slots.  gear:
    SMVGEAR's form, with concentrations at or below ZBOUND = 1e-30 taken as zero
    (CEFF of grpderiv.F:147-155, products of :163-189)."""
    name = f"gear_explic_{d}" if gear else f"explic_{d}"
    src = "grpderiv.F:163-189" if gear else "rbjacob.F:112-143"
    o = [f"// Partial-derivative products of 2- and 3-reactant reactions ({src}).",
         f"__device__ __noinline__ void {name}(double* __restrict__ ws)",
         "{",
         f"    const double* __restrict__ y = ws + {lay.y * 32};"]
    if gear:
        o.append("#define CEFF_(v) ((v) <= 1.0e-30 ? 0.0 : (v))")
    for r in sp.active[d]:
        nre = m.nreact[r]
        k = _w(lay.rki + r)
        wrap = (lambda e: f"CEFF_({e})") if gear else (lambda e: e)
        if nre == 2:
            y1 = wrap(f"y[{sp.irm2[r][0] * 32}]")
            y2 = wrap(f"y[{sp.irm2[r][1] * 32}]")
            o.append(f"    {{ const double kk = {k}; {_w(lay.ex[(r, 0)])} = kk * {y2}; {_w(lay.ex[(r, 1)])} = kk * {y1}; }}")
        elif nre == 3:
            y1 = wrap(f"y[{sp.irm2[r][0] * 32}]")
            y2 = wrap(f"y[{sp.irm2[r][1] * 32}]")
            y3 = wrap(f"y[{sp.irm2[r][2] * 32}]")
            o.append(f"    {{ const double kk = {k}; const double cr2 = kk * {y2};"
                     f" {_w(lay.ex[(r, 0)])} = cr2 * {y3};"
                     f" {_w(lay.ex[(r, 1)])} = (kk * {y1}) * {y3};"
                     f" {_w(lay.ex[(r, 2)])} = cr2 * {y1}; }}")
    if gear:
        o.append("#undef CEFF_")
    o.append("}")
    return o


def _jac_terms(m: Mechanism, sp: SparseMech, d: int) -> dict[int, list[tuple]]:
    """storage index -> ordered PD terms [(rxn, ial, coef or None, sign)]."""
    terms: dict[int, list] = {}
    for r in sp.active[d]:
        for (iar, ial) in sp.loss_pd[d][r]:
            terms.setdefault(iar, []).append((r, ial, None, -1))
        for (iar, ial, ic) in sp.prod_pd[d][r]:
            terms.setdefault(iar, []).append((r, ial, None if ic < 0 else m.sc[r][ic], +1))
    return terms


JAC_CHUNK_OPS = 200     # elimination ops per generated function; bounds ptxas time and register spills


def _jacdecomp_chunks(m: Mechanism, sp: SparseMech, lay: Layout, d: int, gear: bool = False) -> list[list[str]]:
    """Jacobian - I/(gamma h) and its LU factors, row by row.  Each entry receives the same
    updates in the same order as the column-ordered elimination of rbdecomp.F; L is stored
    scaled by 1/U(k,k) and VDIAG = 1/U(i,i).  Rows are grouped into functions of bounded size.
    gear: SMVGEAR's predictor matrix P = I - ASN1*DELT*J instead (grpderiv.F:131-226: every
    entry starts at 0, the diagonal at 1, and takes R1DELT = -ASN1*DELT times each
    partial-derivative term in PDERIV's order), factored by the same elimination
    (grdecomp.F is rbdecomp.F)."""
    n = sp.ischan
    jpt = sp.jarraypt[d]
    terms = _jac_terms(m, sp, d)
    # workspace elements each row reads (Jacobian terms, earlier rows' U, 1/U(k,k))
    reads = []
    for i in range(n):
        r_set = []
        cols = [j for (_, j) in sp.lower[d][i]] + [i] + [j for (_, j) in sp.upper[d][i]]
        for j in cols:
            for (r, ial, _, _) in terms.get(jpt[(i, j)], []):
                r_set.append(lay.rki + r if m.nreact[r] == 1 else lay.ex[(r, ial)])
        for (_, k) in sp.lower[d][i]:
            r_set.append(lay.vdiag + k)
            r_set.extend(lay.lu + st for (st, _) in sp.upper[d][k])
        reads.append(list(dict.fromkeys(r_set)))
    rows_code = []
    for i in range(n):
        lower = sp.lower[d][i]
        upper = sp.upper[d][i]
        cols = [j for (_, j) in lower] + [i] + [j for (_, j) in upper]
        o = [f"    {{ // row {i}"]
        if i + PREFETCH_AHEAD < n:
            o.extend(f"      CHEM_PREFETCH(ws + {e * 32});" for e in reads[i + PREFETCH_AHEAD])
        if i + 1 < n:
            o.extend(f"      CHEM_PREFETCH_L1(ws + {e * 32});" for e in reads[i + 1])
        nops = 0
        for j in cols:
            st = jpt[(i, j)]
            tl = terms.get(st, [])
            var = f"a{j}"
            if gear:
                o.append(f"      double {var} = {'1.0' if j == i else '0.0'};")
                for (r, ial, coef, sign) in tl:
                    ex = _ex_ref(m, sp, lay, r, ial)
                    if sign < 0:
                        o.append(f"      {var} = fma(-r1delt, {ex}, {var});")
                    elif coef is None:
                        o.append(f"      {var} = fma(r1delt, {ex}, {var});")
                    else:
                        o.append(f"      {var} = fma({c_double(coef)} * r1delt, {ex}, {var});")
                continue
            if not tl:
                o.append(f"      double {var} = 0.0;")
                continue
            first = True
            for (r, ial, coef, sign) in tl:
                ex = _ex_ref(m, sp, lay, r, ial)
                if first:
                    if sign < 0:
                        o.append(f"      double {var} = -{ex};")
                    elif coef is None:
                        o.append(f"      double {var} = {ex};")
                    else:
                        o.append(f"      double {var} = {c_double(coef)} * {ex};")
                    first = False
                elif sign < 0:
                    o.append(f"      {var} = {var} - {ex};")
                elif coef is None:
                    o.append(f"      {var} = {var} + {ex};")
                else:
                    o.append(f"      {var} = fma({c_double(coef)}, {ex}, {var});")
        if not gear:
            o.append(f"      a{i} = a{i} - gdtinv;")
        for (st_ik, k) in lower:
            o.append(f"      a{k} = a{k} * CHEM_LDLU(vd + {k * 32});")
            o.append(f"      lu[{st_ik * 32}] = a{k};")
            for (st_kj, j) in sp.upper[d][k]:
                o.append(f"      a{j} = fma(-a{k}, CHEM_LDLU(lu + {st_kj * 32}), a{j});")
                nops += 1
        for (st_ij, j) in upper:
            o.append(f"      lu[{st_ij * 32}] = a{j};")
        o.append(f"      vd[{i * 32}] = CHEM_RCP(a{i});")
        o.append("    }")
        rows_code.append((nops + len(cols), o))
    # group rows into chunks
    chunks, cur, cost = [], [], 0
    for c, code in rows_code:
        if cur and cost + c > JAC_CHUNK_OPS:
            chunks.append(cur); cur, cost = [], 0
        cur.append(code); cost += c
    if cur:
        chunks.append(cur)
    out = []
    for ci, ch in enumerate(chunks):
        sig = f"gear_pdecomp_{d}_{ci}(double* __restrict__ ws, double r1delt)" if gear else \
            f"jacdecomp_{d}_{ci}(double* __restrict__ ws, double gdtinv)"
        f = [f"__device__ __noinline__ void {sig}", "{",
             f"    double* __restrict__ lu = ws + {lay.lu * 32};",
             f"    double* __restrict__ vd = ws + {lay.vdiag * 32};"]
        for code in ch:
            f.extend(code)
        f.append("}")
        out.append(f)
    return out


SOLVE_CHUNK_TERMS = 800
PREFETCH_AHEAD = 2      # rows ahead whose workspace reads a row prefetches (variant 'pf')


def _solve_chunks(sp: SparseMech, lay: Layout, d: int) -> list[list[str]]:
    """Forward then backward substitution in place at ws[rhs] (rbsolve.F); each row
    sums its terms in the reference's column order."""
    n = sp.ischan
    # rows in sweep order with the LU elements each reads
    sweep = [("L", i, [lay.lu + st for (st, _) in sp.lower[d][i]]) for i in range(n)]
    sweep += [("U", i, [lay.lu + st for (st, _) in sp.upper[d][i]] + [lay.vdiag + i]) for i in range(n - 1, -1, -1)]
    ahead, next1 = {}, {}
    for q in range(len(sweep) - PREFETCH_AHEAD):
        ahead[(sweep[q][0], sweep[q][1])] = sweep[q + PREFETCH_AHEAD][2]
    for q in range(len(sweep) - 1):
        next1[(sweep[q][0], sweep[q][1])] = sweep[q + 1][2]

    def pf(kind, i):
        return ([f"      CHEM_PREFETCH(ws + {e * 32});" for e in ahead.get((kind, i), [])]
                + [f"      CHEM_PREFETCH_L1(ws + {e * 32});" for e in next1.get((kind, i), [])])
    pieces = []
    for i in range(n):
        o = ["    {"] + pf("L", i) + [f"      double x = b[{i * 32}];"]
        for (st, j) in sp.lower[d][i]:
            o.append(f"      x = fma(-CHEM_LDLU(lu + {st * 32}), b[{j * 32}], x);")
        o.append(f"      b[{i * 32}] = x;")
        o.append("    }")
        pieces.append((len(sp.lower[d][i]) + 1, o))
    for i in range(n - 1, -1, -1):
        o = ["    {"] + pf("U", i) + [f"      double x = b[{i * 32}];"]
        for (st, j) in sp.upper[d][i]:
            o.append(f"      x = fma(-CHEM_LDLU(lu + {st * 32}), b[{j * 32}], x);")
        o.append(f"      b[{i * 32}] = x * CHEM_LDLU(vd + {i * 32});")
        o.append("    }")
        pieces.append((len(sp.upper[d][i]) + 1, o))
    chunks, cur, cost = [], [], 0
    for c, code in pieces:
        if cur and cost + c > SOLVE_CHUNK_TERMS:
            chunks.append(cur); cur, cost = [], 0
        cur.append(code); cost += c
    if cur:
        chunks.append(cur)
    out = []
    for ci, ch in enumerate(chunks):
        f = [f"__device__ __noinline__ void solve_{d}_{ci}(double* __restrict__ ws, int rhs)", "{",
             f"    const double* __restrict__ lu = ws + {lay.lu * 32};",
             f"    const double* __restrict__ vd = ws + {lay.vdiag * 32};",
             "    double* __restrict__ b = ws + rhs * 32;",
             "    (void)vd;"]
        for code in ch:
            f.extend(code)
        f.append("}")
        out.append(f)
    return out


def _solve_t_chunks(sp: SparseMech, lay: Layout, d: int) -> list[list[str]]:
    """Transposed solve A^T x = b in place at ws[rhs] with the LU factors of A = L U that
    jacdecomp_d leaves (unit L, U with 1/U(i,i) in VDIAG): U^T z = b by ascending rows,
    then L^T x = z by descending rows.  Each row gathers the column of U (or L) below
    (above) its diagonal in ascending column order; the discrete adjoint of the stage
    solves needs these."""
    n = sp.ischan
    col_u = {i: [] for i in range(n)}
    col_l = {i: [] for i in range(n)}
    for k in range(n):
        for (st, j) in sp.upper[d][k]:
            col_u[j].append((st, k))
        for (st, j) in sp.lower[d][k]:
            col_l[j].append((st, k))
    pieces = []
    for i in range(n):
        o = ["    {", f"      double x = b[{i * 32}];"]
        for (st, k) in sorted(col_u[i], key=lambda t: t[1]):
            o.append(f"      x = fma(-CHEM_LDLU(lu + {st * 32}), b[{k * 32}], x);")
        o.append(f"      b[{i * 32}] = x * CHEM_LDLU(vd + {i * 32});")
        o.append("    }")
        pieces.append((len(col_u[i]) + 1, o))
    for i in range(n - 1, -1, -1):
        if not col_l[i]:
            continue
        o = ["    {", f"      double x = b[{i * 32}];"]
        for (st, k) in sorted(col_l[i], key=lambda t: t[1]):
            o.append(f"      x = fma(-CHEM_LDLU(lu + {st * 32}), b[{k * 32}], x);")
        o.append(f"      b[{i * 32}] = x;")
        o.append("    }")
        pieces.append((len(col_l[i]) + 1, o))
    chunks, cur, cost = [], [], 0
    for c, code in pieces:
        if cur and cost + c > SOLVE_CHUNK_TERMS:
            chunks.append(cur); cur, cost = [], 0
        cur.append(code); cost += c
    if cur:
        chunks.append(cur)
    out = []
    for ci, ch in enumerate(chunks):
        f = [f"__device__ __noinline__ void solve_t_{d}_{ci}(double* __restrict__ ws, int rhs)", "{",
             f"    const double* __restrict__ lu = ws + {lay.lu * 32};",
             f"    const double* __restrict__ vd = ws + {lay.vdiag * 32};",
             "    double* __restrict__ b = ws + rhs * 32;",
             "    (void)vd;"]
        for code in ch:
            f.extend(code)
        f.append("}")
        out.append(f)
    return out


def _stoich_sum(m: Mechanism, sp: SparseMech, r: int, vec: str, name: str) -> list[str]:
    """``name`` = sum over reaction r's net stoichiometry of vec[]: products (SC-weighted,
    in product order), then minus each reactant."""
    o, first = [], True
    for p in range(m.nprdct[r]):
        sp_idx = sp.irm2[r][3 + p]
        term = f"{vec}[{sp_idx * 32}]"
        if first:
            o.append(f"double {name} = {c_double(m.sc[r][p])} * {term};")
            first = False
        else:
            o.append(f"{name} = fma({c_double(m.sc[r][p])}, {term}, {name});")
    for i in range(m.nreact[r]):
        term = f"{vec}[{sp.irm2[r][i] * 32}]"
        if first:
            o.append(f"double {name} = -{term};")
            first = False
        else:
            o.append(f"{name} = {name} - {term};")
    if first:
        o.append(f"double {name} = 0.0;")
    return o


ADJ_CHUNK_LINES = 500    # generated lines per reaction-wise adjoint function; bounds ptxas time


def _chunk_reactions(head: list[str], blocks: list[list[str]], name: str) -> list[list[str]]:
    """Wrap per-reaction code blocks into __noinline__ functions of bounded size."""
    out, cur, n = [], [], 0
    for b in blocks:
        if cur and n + len(b) > ADJ_CHUNK_LINES:
            out.append(cur); cur, n = [], 0
        cur.append(b); n += len(b)
    if cur or not out:
        out.append(cur)
    funcs = []
    for ci, ch in enumerate(out):
        f = [head[0].format(name=f"{name}_{ci}"), "{"] + head[1:]
        for b in ch:
            f.extend(b)
        f.append("}")
        funcs.append(f)
    return funcs


def _adj_jtv(m: Mechanism, sp: SparseMech, lay: Layout, d: int) -> list[list[str]]:
    """out += J(y)^T phi over the active reactions, and ADJ_GK[r] += w_r * R_r(y), the
    derivative of phi . f(y) with respect to log k_r; w_r is phi contracted with the
    reaction's net stoichiometry and R_r its rate.  Returned as chunk functions
    adj_jtv_d_c, called in order."""
    head = ["__device__ __noinline__ void {name}(double* __restrict__ ws, int yoff, int phioff, int outoff)",
            "    const double* __restrict__ y = ws + yoff * 32;",
            "    const double* __restrict__ phi = ws + phioff * 32;",
            "    double* __restrict__ out = ws + outoff * 32;"]
    blocks = []
    for r in sp.active[d]:
        nre = m.nreact[r]
        if nre == 0 and m.nprdct[r] == 0:
            continue
        gk = _w(lay.adj_gk + r)
        o = ["    {"]
        o.extend("      " + t for t in _stoich_sum(m, sp, r, "phi", "w"))
        o.append(f"      const double kw = {_w(lay.rki + r)} * w;")
        a = [sp.irm2[r][i] * 32 for i in range(nre)]
        if nre == 0:
            o.append(f"      {gk} = {gk} + kw;")
        elif nre == 1:
            o.append(f"      out[{a[0]}] = out[{a[0]}] + kw;")
            o.append(f"      {gk} = fma(kw, y[{a[0]}], {gk});")
        elif nre == 2:
            o.append(f"      out[{a[0]}] = fma(kw, y[{a[1]}], out[{a[0]}]);")
            o.append(f"      out[{a[1]}] = fma(kw, y[{a[0]}], out[{a[1]}]);")
            o.append(f"      {gk} = fma(kw * y[{a[0]}], y[{a[1]}], {gk});")
        else:
            o.append(f"      out[{a[0]}] = fma(kw * y[{a[1]}], y[{a[2]}], out[{a[0]}]);")
            o.append(f"      out[{a[1]}] = fma(kw * y[{a[0]}], y[{a[2]}], out[{a[1]}]);")
            o.append(f"      out[{a[2]}] = fma(kw * y[{a[0]}], y[{a[1]}], out[{a[2]}]);")
            o.append(f"      {gk} = fma((kw * y[{a[0]}]) * y[{a[1]}], y[{a[2]}], {gk});")
        o.append("    }")
        blocks.append(o)
    return _chunk_reactions(head, blocks, f"adj_jtv_{d}")


def _adj_hess3(m: Mechanism, sp: SparseMech, lay: Layout, d: int) -> list[list[str]]:
    """Second-order terms of the stage solves' adjoint: with nu_i the solved stage
    adjoints (ADJ_MU1..3) and K_i the stages, ADJ_LAM -= sum_i d/dy (nu_i . J(y) K_i)
    and ADJ_GK[r] -= sum_i d/d log k_r (nu_i . J(y) K_i), y = Y.  Per reaction the
    three contractions share WK_s = sum_i w_i K_i[s] over its reactant slots s.  Returned
    as chunk functions adj_hess3_d_c, called in order."""
    head = ["__device__ __noinline__ void {name}(double* __restrict__ ws)",
            f"    const double* __restrict__ y = ws + {lay.y * 32};",
            f"    double* __restrict__ lam = ws + {lay.adj_lam * 32};"]
    vecs = [("n1", lay.adj_mu1, "k1", lay.k1), ("n2", lay.adj_mu2, "k2", lay.k2), ("n3", lay.adj_mu3, "k3", lay.k3)]
    for nv, off_n, kv, off_k in vecs:
        head.append(f"    const double* __restrict__ {nv} = ws + {off_n * 32};")
        head.append(f"    const double* __restrict__ {kv} = ws + {off_k * 32};")
    blocks = []
    for r in sp.active[d]:
        nre = m.nreact[r]
        if nre == 0:
            continue
        gk = _w(lay.adj_gk + r)
        a = [sp.irm2[r][i] * 32 for i in range(nre)]
        o = ["    {"]
        for i, (nv, _, _, _) in enumerate(vecs):
            o.extend("      " + t for t in _stoich_sum(m, sp, r, nv, f"w{i + 1}"))
        for j in range(nre):
            o.append(f"      double wk{j} = w1 * k1[{a[j]}];")
            o.append(f"      wk{j} = fma(w2, k2[{a[j]}], wk{j});")
            o.append(f"      wk{j} = fma(w3, k3[{a[j]}], wk{j});")
        o.append(f"      const double kk = {_w(lay.rki + r)};")
        if nre == 1:
            o.append(f"      {gk} = fma(-kk, wk0, {gk});")
        elif nre == 2:
            o.append(f"      {gk} = fma(-kk, fma(y[{a[1]}], wk0, y[{a[0]}] * wk1), {gk});")
            o.append(f"      lam[{a[0]}] = fma(-kk, wk1, lam[{a[0]}]);")
            o.append(f"      lam[{a[1]}] = fma(-kk, wk0, lam[{a[1]}]);")
        else:
            o.append(f"      {gk} = fma(-kk, fma(y[{a[1]}] * y[{a[2]}], wk0, "
                     f"fma(y[{a[0]}] * y[{a[2]}], wk1, (y[{a[0]}] * y[{a[1]}]) * wk2)), {gk});")
            o.append(f"      lam[{a[0]}] = fma(-kk, fma(y[{a[2]}], wk1, y[{a[1]}] * wk2), lam[{a[0]}]);")
            o.append(f"      lam[{a[1]}] = fma(-kk, fma(y[{a[2]}], wk0, y[{a[0]}] * wk2), lam[{a[1]}]);")
            o.append(f"      lam[{a[2]}] = fma(-kk, fma(y[{a[1]}], wk0, y[{a[0]}] * wk1), lam[{a[2]}]);")
        o.append("    }")
        blocks.append(o)
    return _chunk_reactions(head, blocks, f"adj_hess3_{d}")


def _ddm_jv(m: Mechanism, sp: SparseMech, lay: Layout, d: int) -> list[list[str]]:
    """out += J(y) v over the active reactions (the Jacobian-vector product of the DDM-3D
    update, DDM3D_CHEM.F:386-396): per reaction d = grad R . v, then every species of the
    reaction's net stoichiometry gets its coefficient times d."""
    head = ["__device__ __noinline__ void {name}(double* __restrict__ ws, int yoff, int voff, int outoff)",
            "    const double* __restrict__ y = ws + yoff * 32;",
            "    const double* __restrict__ v = ws + voff * 32;",
            "    double* __restrict__ out = ws + outoff * 32;"]
    blocks = []
    for r in sp.active[d]:
        nre = m.nreact[r]
        if nre == 0:
            continue
        a = [sp.irm2[r][i] * 32 for i in range(nre)]
        k = _w(lay.rki + r)
        o = ["    {"]
        if nre == 1:
            o.append(f"      const double dr = {k} * v[{a[0]}];")
        elif nre == 2:
            o.append(f"      const double dr = {k} * fma(y[{a[1]}], v[{a[0]}], y[{a[0]}] * v[{a[1]}]);")
        else:
            o.append(f"      const double dr = {k} * fma(y[{a[1]}] * y[{a[2]}], v[{a[0]}], "
                     f"fma(y[{a[0]}] * y[{a[2]}], v[{a[1]}], (y[{a[0]}] * y[{a[1]}]) * v[{a[2]}]));")
        for i in range(nre):
            o.append(f"      out[{a[i]}] = out[{a[i]}] - dr;")
        for p in range(m.nprdct[r]):
            t = sp.irm2[r][3 + p] * 32
            o.append(f"      out[{t}] = fma({c_double(m.sc[r][p])}, dr, out[{t}]);")
        o.append("    }")
        blocks.append(o)
    return _chunk_reactions(head, blocks, f"ddm_jv_{d}")


def _ddm_src(m: Mechanism, sp: SparseMech, lay: Layout, d: int) -> list[list[str]]:
    """out += scale * sum over the reactions with mask[r] != 0 of the net stoichiometry
    times the rate RXRAT (as left by feval): the source of a reaction-rate parameter
    (DDM3D_CHEM.F:338-385).  The mask is the same for every lane, so the branches are
    uniform."""
    head = ["__device__ __noinline__ void {name}(double* __restrict__ ws, const unsigned char* __restrict__ mask, "
            "double scale, int outoff)",
            "    double* __restrict__ out = ws + outoff * 32;"]
    blocks = []
    for r in sp.active[d]:
        o = [f"    if (mask[{r}]) {{", f"      const double q = scale * {_w(lay.rxrat + r)};"]
        for i in range(m.nreact[r]):
            t = sp.irm2[r][i] * 32
            o.append(f"      out[{t}] = out[{t}] - q;")
        for p in range(m.nprdct[r]):
            t = sp.irm2[r][3 + p] * 32
            o.append(f"      out[{t}] = fma({c_double(m.sc[r][p])}, q, out[{t}]);")
        o.append("    }")
        blocks.append(o)
    return _chunk_reactions(head, blocks, f"ddm_src_{d}")
