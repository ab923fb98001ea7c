"""Shared emitters: rate-expression trees -> C/CUDA source text.

The rate functions below restate the formulas of CMAQ's generated rate-constant
helpers (CCTM/src/MECHS/cb6r5_ae7_aq/RXNS_FUNC_MODULE.F90:15-160) as C
functions that compile both for the host (oracle) and the device (kernels).
Operation order follows the Fortran source, left to right; ``x ** 2.0D0`` is
written as ``x * x`` and ``DMIN1`` as ``fmin``.
"""
from __future__ import annotations

RATE_HELPERS = r"""
/* Rate-constant helpers, one per CMAQ rate form (RXNS_FUNC_MODULE.F90:15-160). */
CHEM_HD static inline double chem_power_t02(double tempot300, double a0, double b0)
{
    return a0 * pow(tempot300, b0);
}
CHEM_HD static inline double chem_arrhenius_t03(double inv_temp, double a0, double b0)
{
    return a0 * exp(b0 * inv_temp);
}
CHEM_HD static inline double chem_arrhenius_t04(double inv_temp, double tempot300, double a0, double b0, double c0)
{
    return a0 * exp(b0 * inv_temp) * pow(tempot300, c0);
}
CHEM_HD static inline double chem_falloff_t08(double inv_temp, double cair, double a0, double c0,
                                              double a2, double c2, double a3, double c3)
{
    double k0 = a0 * exp(c0 * inv_temp);
    double k2 = a2 * exp(c2 * inv_temp);
    double k3 = a3 * exp(c3 * inv_temp);
    k3 = k3 * cair;
    return k0 + k3 / (1.0 + k3 / k2);
}
CHEM_HD static inline double chem_falloff_t09(double inv_temp, double cair, double a1, double c1,
                                              double a2, double c2)
{
    double k1 = a1 * exp(c1 * inv_temp);
    double k2 = a2 * exp(c2 * inv_temp);
    return k1 + k2 * cair;
}
CHEM_HD static inline double chem_falloff_t10(double inv_temp, double tempot300, double cair,
                                              double a0, double b0, double c0, double a1, double b1,
                                              double c1, double ce, double cf)
{
    double k0 = a0 * cair * exp(b0 * inv_temp) * pow(tempot300, c0);
    double k1 = a1 * exp(b1 * inv_temp) * pow(tempot300, c1);
    double x = (1.0 / ce) * log10(k0 / k1);
    double kend = 1.0 + x * x;
    kend = 1.0 / kend;
    return (k0 / (1.0 + k0 / k1)) * pow(cf, kend);
}
CHEM_HD static inline double chem_falloff_t11(double inv_temp, double tempot300, double cair,
                                              double a1, double b1, double c1, double a2, double b2,
                                              double c2, double d1, double d2)
{
    double k1 = a1 * exp(c1 * inv_temp) * pow(tempot300, b1);
    double k2 = a2 * exp(c2 * inv_temp) * pow(tempot300, b2);
    double k3 = d1 * exp(d2 * inv_temp);
    return k1 + k2 * cair + k3;
}
CHEM_HD static inline double chem_halogen_falloff(double press, double a1, double b1, double a2,
                                                  double b2, double a3)
{
    double k = a1 * exp(b1 * press) + a2 * exp(b2 * press);
    return fmin(a3, k);
}
"""

_FUNC = {"POWER_T02": "chem_power_t02", "ARRHENUIS_T03": "chem_arrhenius_t03",
         "ARRHENUIS_T04": "chem_arrhenius_t04", "FALLOFF_T08": "chem_falloff_t08",
         "FALLOFF_T09": "chem_falloff_t09", "FALLOFF_T10": "chem_falloff_t10",
         "FALLOFF_T11": "chem_falloff_t11", "HALOGEN_FALLOFF": "chem_halogen_falloff",
         "DEXP": "exp", "POW": "pow"}


def c_double(v: float) -> str:
    r = repr(float(v))
    if "e" not in r and "." not in r and "inf" not in r and "nan" not in r:
        r += ".0"
    return r


def emit_expr(e, leaf) -> str:
    """Translate an expression tree; ``leaf(node)`` renders non-arithmetic leaves."""
    kind = e[0]
    if kind == "num":
        s = c_double(e[1])
        return f"({s})" if e[1] < 0 else s
    if kind == "bin":
        # every binary operand is parenthesised, so C evaluates exactly the parsed tree
        a = emit_expr(e[2], leaf)
        b = emit_expr(e[3], leaf)
        if e[2][0] == "bin":
            a = f"({a})"
        if e[3][0] == "bin":
            b = f"({b})"
        return f"{a} {e[1]} {b}"
    if kind == "neg":
        return f"(-{emit_expr(e[1], leaf)})"
    if kind == "call":
        args = ", ".join(emit_expr(a, leaf) for a in e[2])
        return f"{_FUNC[e[1]]}({args})"
    return leaf(e)
