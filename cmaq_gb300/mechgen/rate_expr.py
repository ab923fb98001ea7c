"""Parse ``CALC_RCONST`` of a CMAQ ``RXNS_FUNC_MODULE.F90`` into expression trees.

``CALC_RCONST`` (cb6r5_ae7_aq: CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_FUNC_MODULE.F90:204-1116)
is generated code with three parts:

1. a sunlit-only block that sets photolysis rates ``RKI = [coef *] RJBLK(IJ_x)``
   and the seawater-conditioned halogen rate (``:271-366``);
2. a thermal block that sets per-cell unit factors (``INV_TEMP``, ``CAIR``,
   ``CFACT`` ...; ``:368-379``) and one assignment per thermal / heterogeneous
   reaction built from the rate functions ``POWER_T02``, ``ARRHENUIS_T03/T04``,
   ``FALLOFF_T08..T11`` and ``HALOGEN_FALLOFF`` (``:15-160``);
3. third-body multiplications by [M], [O2], [N2], [H2O], [H2], [CH4]
   (``:1065-1114``), which come from the table module's ``NRXW*`` lists.

Expressions are kept as trees so that the oracle (C) and the device code (CUDA)
evaluate them in the same written order: binary chains associate to the left,
as the Fortran source is written.

Node forms (tuples):
  ('num', float, text)            literal
  ('var', NAME)                   per-cell factor: INV_TEMP TEMPOT300 CAIR CFACT CFACT_SQU SFACT RFACT ...
  ('press',)                      BLKPRES(NCELL) [atm]
  ('blktemp',)                    BLKTEMP(NCELL) [K]
  ('h2o',)                        BLKH2O(NCELL) [ppm]
  ('seawater',)                   SEAWATER(NCELL)
  ('rj', k)                       RJBLK(NCELL, k)   k 0-based photolysis table
  ('het', k)                      BLKHET(NCELL, k)  k 0-based heterogeneous table
  ('rki', m)                      RKI(NCELL, m)     m 0-based reaction
  ('call', FNAME, [args])         rate function or DEXP
  ('bin', op, a, b)               op in + - * /
  ('neg', a)
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

from .fortran_tables import join_continuations, fnum

_TOKEN = re.compile(r"\s*(?:(?P<num>(?:\d+\.\d*|\.\d+|\d+)(?:[DdEe][-+]?\d+)?)|(?P<id>[A-Za-z_]\w*)|(?P<op>\*\*|[-+*/(),]))")

RATE_FUNCS = {"POWER_T02", "ARRHENUIS_T03", "ARRHENUIS_T04", "FALLOFF_T08", "FALLOFF_T09",
              "FALLOFF_T10", "FALLOFF_T11", "HALOGEN_FALLOFF", "DEXP"}
CELL_VARS = {"INV_TEMP", "TEMPOT300", "CAIR", "CFACT", "CFACT_SQU", "SFACT", "RFACT",
             "RFACT_SQU", "INV_CAIR", "INV_CFACT", "TEMP", "PRESS", "H2O"}


def tokenize(s: str) -> list[tuple[str, str]]:
    pos, out = 0, []
    s = s.rstrip()
    while pos < len(s):
        m = _TOKEN.match(s, pos)
        if not m or m.end() == pos:
            if s[pos:].strip() == "":
                break
            raise ValueError(f"cannot tokenize at {s[pos:pos+30]!r}")
        kind = m.lastgroup
        out.append((kind, m.group(kind)))
        pos = m.end()
    return out


class _Parser:
    def __init__(self, toks, ij: dict[str, int], ik: dict[str, int], consts: dict[str, float]):
        self.t = toks
        self.i = 0
        self.ij = ij
        self.ik = ik
        self.consts = consts

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1].upper() != val:
            raise ValueError(f"expected {val}, got {tok}")
        self.i += 1
        return tok

    def expr(self):
        node = self.term()
        while self.peek()[1] in ("+", "-"):
            op = self.take()[1]
            node = ("bin", op, node, self.term())
        return node

    def term(self):
        node = self.power()
        while self.peek()[1] in ("*", "/"):
            op = self.take()[1]
            node = ("bin", op, node, self.power())
        return node

    def power(self):
        base = self.unary()
        if self.peek()[1] == "**":
            self.take()
            return ("call", "POW", [base, self.power()])
        return base

    def unary(self):
        k, v = self.peek()
        if v == "-":
            self.take()
            inner = self.unary()
            if inner[0] == "num":
                return ("num", -inner[1], "-" + inner[2])
            return ("neg", inner)
        if v == "+":
            self.take()
            return self.unary()
        return self.primary()

    def args(self):
        self.take("(")
        out = [self.expr()]
        while self.peek()[1] == ",":
            self.take()
            out.append(self.expr())
        self.take(")")
        return out

    def primary(self):
        k, v = self.peek()
        if k == "num":
            self.take()
            return ("num", fnum(v), v)
        if v == "(":
            self.take()
            e = self.expr()
            self.take(")")
            return e
        if k == "id":
            name = v.upper()
            self.take()
            if name in ("RJBLK", "BLKHET", "RKI", "BLKPRES", "SEAWATER", "BLKTEMP", "BLKH2O"):
                self.take("(")
                self.take("NCELL")
                if name in ("BLKPRES", "SEAWATER", "BLKTEMP", "BLKH2O"):
                    self.take(")")
                    return {"BLKPRES": ("press",), "SEAWATER": ("seawater",),
                            "BLKTEMP": ("blktemp",), "BLKH2O": ("h2o",)}[name]
                self.take(",")
                kk, vv = self.take()
                self.take(")")
                if name == "RJBLK":
                    return ("rj", self.ij[vv.upper()] - 1)
                if name == "BLKHET":
                    return ("het", self.ik[vv.upper()] - 1)
                return ("rki", int(vv) - 1)
            if name in RATE_FUNCS:
                return ("call", name, self.args())
            if name in self.consts:
                return ("num", self.consts[name], name)
            if name in CELL_VARS:
                return ("var", name)
            raise ValueError(f"unknown identifier {name}")
        raise ValueError(f"unexpected token {v!r}")


@dataclass
class RateProgram:
    photo: dict[int, tuple] = field(default_factory=dict)       # rxn(0-based) -> expr (sunlit block)
    photo_order: list[int] = field(default_factory=list)
    seawater_cond: dict[int, tuple[float, tuple]] = field(default_factory=dict)  # rxn -> (threshold, expr)
    thermal: dict[int, tuple] = field(default_factory=dict)
    thermal_order: list[int] = field(default_factory=list)
    factors: list[tuple[str, tuple]] = field(default_factory=list)  # per-cell factor definitions in order
    constants: dict[str, float] = field(default_factory=dict)


def parse_rate_program(func_text: str, data_text: str) -> RateProgram:
    """Parse CALC_RCONST from the function module; IJ_/IK_ names from the table module."""
    ij = {m.group(1).upper(): int(m.group(2))
          for m in re.finditer(r"INTEGER,\s*PARAMETER\s*::\s*(IJ_\w+)\s*=\s*(\d+)", data_text)}
    ik = {m.group(1).upper(): int(m.group(2))
          for m in re.finditer(r"INTEGER,\s*PARAMETER\s*::\s*(IK_\w+)\s*=\s*(\d+)", data_text)}
    start = re.search(r"SUBROUTINE\s+CALC_RCONST", func_text, re.I).start()
    end = re.search(r"END\s+SUBROUTINE\s+CALC_RCONST", func_text, re.I).end()
    body = join_continuations(func_text[start:end])
    prog = RateProgram()
    section = None          # 'photo' | 'thermal'
    pending_cond = None     # threshold of an open IF ( SEAWATER > thr )
    re_assign = re.compile(r"^RKI\s*\(\s*NCELL\s*,\s*(\d+)\s*\)\s*=\s*(.+)$", re.I)
    re_param = re.compile(r"^REAL\s*\(\s*8\s*\)\s*,\s*PARAMETER\s*::\s*(\w+)\s*=\s*(.+)$", re.I)
    re_factor = re.compile(r"^(INV_TEMP|CAIR|CFACT|CFACT_SQU|INV_CAIR|INV_CFACT|TEMP|TEMPOT300|RFACT|RFACT_SQU)\s*=\s*(.+)$", re.I)
    re_if_sea = re.compile(r"^IF\s*\(\s*SEAWATER\s*\(\s*NCELL\s*\)\s*\.GT\.\s*(\S+)\s*\)\s*THEN$", re.I)
    in_else = False
    for st in body:
        u = st.upper().replace(" ", "")
        m = re_param.match(st)
        if m:
            val = m.group(2).strip()
            if val.upper() == "1.0D+0/300.0D+0":
                prog.constants[m.group(1).upper()] = 1.0 / 300.0
            else:
                prog.constants[m.group(1).upper()] = fnum(val)
            continue
        if u.startswith("IF(LSUNLIGHT)THEN"):
            section = "photo"
            continue
        if u == "DONCELL=1,NUMCELLS" and section == "photo_done":
            section = "thermal"
            continue
        if u == "ENDIF" and section == "photo" and pending_cond is None:
            section = "photo_done"
            continue
        if u.startswith("ENDDO") and section == "thermal":
            section = "done"
            continue
        m = re_if_sea.match(st)
        if m:
            pending_cond = fnum(m.group(1))
            in_else = False
            continue
        if u == "ELSE" and pending_cond is not None:
            in_else = True
            continue
        if u == "ENDIF" and pending_cond is not None:
            pending_cond = None
            in_else = False
            continue
        m = re_factor.match(st)
        if m and section == "thermal":
            expr = _Parser(tokenize(m.group(2)), ij, ik, prog.constants).expr()
            prog.factors.append((m.group(1).upper(), expr))
            continue
        m = re_assign.match(st)
        if m:
            rx = int(m.group(1)) - 1
            rhs = m.group(2)
            p = _Parser(tokenize(rhs), ij, ik, prog.constants)
            expr = p.expr()
            if p.i != len(p.t):
                raise ValueError(f"trailing tokens in {st}")
            if pending_cond is not None:
                if in_else:
                    assert expr[0] == "num" and expr[1] == 0.0
                else:
                    prog.seawater_cond[rx] = (pending_cond, expr)
                    prog.photo_order.append(rx)
                continue
            if section == "photo":
                prog.photo[rx] = expr
                prog.photo_order.append(rx)
            elif section == "thermal":
                prog.thermal[rx] = expr
                prog.thermal_order.append(rx)
            else:
                raise ValueError(f"assignment outside known section: {st}")
    return prog


def expr_refs(expr, kind: str) -> set:
    """Collect leaves of a given kind ('rki', 'rj', 'het', ...)."""
    out = set()

    def walk(e):
        if e[0] == kind:
            out.add(e[1] if len(e) > 1 else True)
        if e[0] == "bin":
            walk(e[2]); walk(e[3])
        elif e[0] == "neg":
            walk(e[1])
        elif e[0] == "call":
            for a in e[2]:
                walk(a)
    walk(expr)
    return out
