"""Translate CMAQ's generated EBI routines (CCTM/src/gas/ebi_<mech>/hr*.F) to C / CUDA.

The EBI solver of a mechanism is written by CMAQ's create_ebi generator.  Its
mechanism-specific routines are straight-line code -- assignments over the module
arrays RKI, RXRAT, YC, YC0, YCP, PROD, LOSS, PNEG and local REAL(8) scalars, with the
intrinsics SIGN, SQRT, MAX, MIN and ABS -- so they translate statement by statement:

  HRRATES     reaction rates RXRAT = RKI * YC ...        (hrrates.F)
  HRPRODLOSS  production / loss of each EBI species       (hrprodloss.F)
  HRG1..HRG4  closed-form solutions of the coupled groups  (hrg1.F .. hrg4.F)

and HRINIT's tables: the EBI species list EBISP and the per-species convergence
tolerances RTOL (hrinit.F).  The solver's control loop (HRSOLVER) and the driver
(HRDRIVER) are restated by hand in the oracle and the kernel.

Emitted code accesses the module arrays through macros the including file defines:
``EBI_YC(i)``, ``EBI_YC0(i)``, ``EBI_YCP(i)``, ``EBI_RKI(r)``, ``EBI_RXRAT(r)``,
``EBI_PROD(i)``, ``EBI_LOSS(i)``, ``EBI_PNEG(i)`` with 0-based indices.
"""
from __future__ import annotations

import re
from pathlib import Path

from .emit_common import c_double
from .fortran_tables import fnum

ARRAYS = {"YC": "EBI_YC", "YC0": "EBI_YC0", "YCP": "EBI_YCP", "RKI": "EBI_RKI", "RXRAT": "EBI_RXRAT",
          "PROD": "EBI_PROD", "LOSS": "EBI_LOSS", "PNEG": "EBI_PNEG"}
INTRINSICS = {"SIGN": "copysign_f", "SQRT": "sqrt", "MAX": "fmax", "MIN": "fmin", "ABS": "fabs", "DBLE": ""}


def fixed_form_statements(text: str) -> list[str]:
    """Logical statements of fixed-form source: drop comment lines (c, C, *, ! in column 1),
    strip trailing ! comments, join column-6 continuations."""
    out: list[str] = []
    for raw in text.splitlines():
        if not raw.strip():
            continue
        if raw[0] in "cC*!#":
            continue
        line = raw.rstrip("\n")
        # inline comment
        if "!" in line:
            q = None
            for i, ch in enumerate(line):
                if q:
                    if ch == q:
                        q = None
                elif ch in "'\"":
                    q = ch
                elif ch == "!":
                    line = line[:i]
                    break
        if len(line) > 5 and line[5] not in " 0" and line[:5].strip() == "" and out:
            out[-1] += " " + line[6:].strip()
        else:
            out.append(line.strip())
    return [s for s in out if s]


_TOK = re.compile(r"\s*(?:(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[DdEe][-+]?\d+)?)|(?P<id>[A-Za-z_]\w*)|(?P<op>\*\*|[-+*/(),=]))")


def _tokens(s: str):
    pos, out = 0, []
    while pos < len(s):
        m = _TOK.match(s, pos)
        if not m or m.end() == pos:
            if not s[pos:].strip():
                break
            raise ValueError(f"cannot tokenize {s[pos:pos + 40]!r}")
        out.append((m.lastgroup, m.group(m.lastgroup)))
        pos = m.end()
    return out


class _P:
    def __init__(self, toks, species: dict[str, int]):
        self.t, self.i, self.sp = toks, 0, species

    def peek(self):
        return self.t[self.i][1] if self.i < len(self.t) else None

    def take(self, v=None):
        k, val = self.t[self.i]
        if v is not None and val.upper() != v:
            raise ValueError(f"expected {v} got {val}")
        self.i += 1
        return k, val

    def expr(self):
        n = self.term()
        while self.peek() in ("+", "-"):
            op = self.take()[1]
            n = ("bin", op, n, self.term())
        return n

    def term(self):
        n = self.unary()
        while self.peek() in ("*", "/"):
            op = self.take()[1]
            n = ("bin", op, n, self.unary())
        return n

    def unary(self):
        if self.peek() == "-":
            self.take()
            return ("neg", self.power())
        if self.peek() == "+":
            self.take()
        return self.power()

    def power(self):
        b = self.primary()
        if self.peek() == "**":
            self.take()
            e = self.unary()
            return ("pow", b, e)
        return b

    def index(self):
        k, v = self.take()
        if k == "num":
            return int(v) - 1
        return self.sp[v.upper()] - 1

    def primary(self):
        k, v = self.take()
        if k == "num":
            return ("num", fnum(v))
        if v == "(":
            e = self.expr()
            self.take(")")
            return e
        name = v.upper()
        if self.peek() == "(":
            self.take("(")
            if name in ARRAYS:
                idx = self.index()
                self.take(")")
                return ("arr", name, idx)
            args = [self.expr()]
            while self.peek() == ",":
                self.take()
                args.append(self.expr())
            self.take(")")
            if name not in INTRINSICS:
                raise ValueError(f"unknown function {name}")
            return ("call", name, args)
        return ("var", name)


def emit(e) -> str:
    k = e[0]
    if k == "num":
        s = c_double(e[1])
        return f"({s})" if e[1] < 0 else s
    if k == "var":
        # locals get a prefix so that they cannot collide with the including code's names
        return "dtc" if e[1] == "DTC" else "l_" + e[1].lower()
    if k == "arr":
        return f"{ARRAYS[e[1]]}({e[2]})"
    if k == "neg":
        return f"(-{emit(e[1])})"
    if k == "pow":
        ex = e[2]
        if ex[0] == "num" and ex[1] == 2.0:
            b = emit(e[1])
            return f"(({b}) * ({b}))"
        return f"pow({emit(e[1])}, {emit(ex)})"
    if k == "bin":
        a, b = emit(e[2]), emit(e[3])
        if e[2][0] == "bin":
            a = f"({a})"
        if e[3][0] == "bin":
            b = f"({b})"
        return f"{a} {e[1]} {b}"
    if k == "call":
        fn = INTRINSICS[e[1]]
        args = [emit(a) for a in e[2]]
        if e[1] == "SIGN":
            # Fortran SIGN(A, B): |A| with the sign of B
            return f"copysign(fabs({args[0]}), {args[1]})"
        if e[1] in ("MAX", "MIN") and len(args) > 2:
            acc = args[0]
            for a in args[1:]:
                acc = f"{fn}({acc}, {a})"
            return acc
        if fn == "":
            return f"({args[0]})"
        return f"{fn}({', '.join(args)})"
    raise ValueError(e)


_SKIP = re.compile(r"^(SUBROUTINE|USE|IMPLICIT|REAL|INTEGER|LOGICAL|CHARACTER|RETURN|END\b|INCLUDE)", re.I)


def routine(text: str, species: dict[str, int]) -> tuple[list[str], list[tuple]]:
    """(local scalar names, statements [(lhs node, rhs node)]) of one straight-line routine."""
    stmts = []
    locals_ = []
    for st in fixed_form_statements(text):
        if _SKIP.match(st):
            continue
        if "=" not in st:
            raise ValueError(f"unsupported statement: {st[:60]}")
        lhs_s, rhs_s = st.split("=", 1)
        lhs = _P(_tokens(lhs_s), species).primary()
        p = _P(_tokens(rhs_s), species)
        rhs = p.expr()
        if p.i != len(p.t):
            raise ValueError(f"trailing tokens in {st[:60]}")
        if lhs[0] == "var" and lhs[1] not in locals_ and lhs[1] != "DTC":
            locals_.append(lhs[1])
        stmts.append((lhs, rhs))
    return locals_, stmts


def parse_ebi(ebi_dir: Path) -> dict:
    d = Path(ebi_dir)
    data = (d / "hrdata_mod.F").read_text()
    species = {m.group(1).upper(): int(m.group(2)) for m in
               re.finditer(r"INTEGER,\s*PARAMETER\s*::\s*(\w+)\s*=\s*(\d+)", data)}
    for k in ("NEBITER", "MAX_CELLS_EBI"):
        species.pop(k, None)
    deltat = fnum(re.search(r"DELTAT\s*=\s*([0-9.DdEe+-]+)", data).group(1))
    nebiter = int(re.search(r"NEBITER\s*=\s*(\d+)", data).group(1))
    init = (d / "hrinit.F").read_text()
    n_ebisp = int(re.search(r"N_EBISP\s*=\s*(\d+)", init).group(1))
    ebisp = [None] * n_ebisp
    for m in re.finditer(r"EBISP\(\s*(\d+)\s*\)\s*=\s*(\w+)", init):
        ebisp[int(m.group(1)) - 1] = species[m.group(2).upper()] - 1
    rtol = {}
    for m in re.finditer(r"RTOL\(\s*(\w+)\s*\)\s*=\s*([0-9.DdEe+-]+)", init):
        rtol[species[m.group(1).upper()] - 1] = fnum(m.group(2))
    routines = {}
    for name in ("hrrates", "hrprodloss", "hrg1", "hrg2", "hrg3", "hrg4"):
        routines[name] = routine((d / f"{name}.F").read_text(), species)
    pneg_species = sorted({lhs[2] for (lhs, _) in routines["hrprodloss"][1] if lhs[0] == "arr" and lhs[1] == "PNEG"})
    return {"species": species, "ebisp": ebisp, "rtol": rtol, "deltat": deltat, "nebiter": nebiter,
            "routines": routines, "pneg_species": pneg_species}


def c_routines(ebi: dict, qualifier: str) -> str:
    """C/CUDA text of the translated routines; ``qualifier`` prefixes each function."""
    out = []
    for name, (locals_, stmts) in ebi["routines"].items():
        args = "double dtc" if name.startswith("hrg") else "void"
        out.append(f"{qualifier} void ebi_{name}(EBI_CELL_ARGS{', ' + args if args != 'void' else ''})")
        out.append("{")
        if locals_:
            out.append("    double " + ", ".join("l_" + v.lower() for v in locals_) + ";")
        for lhs, rhs in stmts:
            out.append(f"    {emit(lhs)} = {emit(rhs)};")
        if name.startswith("hrg"):
            out.append("    (void)dtc;")
        out.append("}")
    return "\n".join(out) + "\n"
