"""Rate constants: two encodings in the reference must agree.

CMAQ's table module holds every reaction's rate law as KTYPE / RTDAT / RFDAT
(RXNS_DATA_MODULE.F90), from which chemmech writes CALC_RCONST
(UTIL/chemmech/src/wrt_reactions_module.f:654-801; numbers printed with 5
significant digits, formats :1314-1363).  The oracle evaluates the parsed
CALC_RCONST; here the rate laws are evaluated independently from the tables and
the two must agree to round-off (the tables' values print exactly in 5 digits for
these mechanisms).  KTYPE 12 (seawater halogen) and the few KTYPE 5/9 forms of
cracmm2 that use other falloff variants are not re-derived.
"""
import math

import numpy as np
import pytest

from cmaq_gb300.synthetic import manifest


def _falloff_t10(inv_t, t300, cair, a0, b0, c0, a1, b1, c1, ce, cf):
    k0 = a0 * cair * math.exp(b0 * inv_t) * t300 ** c0
    k1 = a1 * math.exp(b1 * inv_t) * t300 ** c1
    x = (1.0 / ce) * math.log10(k0 / k1)
    return (k0 / (1.0 + k0 / k1)) * cf ** (1.0 / (1.0 + x * x))


def table_rates(man, temp, press, h2o, rj, het, sunlit):
    rt = man["rate_tables"]
    kt, rtd, rfd, irrfall, iorder = rt["ktype"], rt["rtdat"], rt["rfdat"], rt["irrfall"], rt["iorder"]
    inv_t = 1.0 / temp
    cair = 1.0e6 * 7.33981e15 * press * inv_t
    conv = {0: 6.0e7 / cair, 1: 60.0, 2: 6.0e-5 * cair, 3: 6.0e-11 * cair * cair}
    t300 = temp / 300.0
    iph = {r - 1: (j, flag) for (r, j, flag) in rt["iph"]}
    ihet = {r - 1: j for (r, j) in rt["ihetero"]}
    fall = {r - 1: i for i, r in enumerate(irrfall)}
    k = [None] * man["nrxns"]
    checked = set()
    for r in range(man["nrxns"]):
        t = kt[r]
        a = rtd[r]
        c = conv.get(iorder[r], 1.0)
        if t == 0:
            j, flag = iph[r]
            k[r] = a[0] * rj[j - 1] if (sunlit and flag != 0) else 0.0
        elif t == -1:
            k[r] = a[0] * het[ihet[r] - 1]
        elif t == 1:
            k[r] = a[0] * c
        elif t == 2:
            k[r] = c * a[0] * t300 ** a[1]
        elif t == 3:
            k[r] = c * a[0] * math.exp(a[2] * inv_t)
        elif t == 4:
            k[r] = c * a[0] * math.exp(a[2] * inv_t) * t300 ** a[1]
        elif t == 8:
            f = rfd[fall[r]]
            k0, k2, k3 = a[0] * math.exp(a[1] * inv_t), a[2] * math.exp(f[0] * inv_t), f[1] * math.exp(f[2] * inv_t)
            k3 *= cair
            k[r] = c * (k0 + k3 / (1.0 + k3 / k2))
        elif t == 9 and rfd[fall[r]][1] == 0.0 and rfd[fall[r]][2] == 0.0:
            f = rfd[fall[r]]
            k[r] = c * (a[0] * math.exp(a[1] * inv_t) + a[2] * math.exp(f[0] * inv_t) * cair)
        elif t == 10:
            f = rfd[fall[r]]
            k[r] = c * _falloff_t10(inv_t, t300, cair, a[0], a[2], a[1], f[0], f[2], f[1], f[4], f[3])
        else:
            continue
        checked.add(r)
    # reactions proportional to another reaction (KTYPE 6, same order)
    for r in range(man["nrxns"]):
        if kt[r] == 6:
            irx = int(rtd[r][1]) - 1
            if k[irx] is not None and iorder[irx] == iorder[r]:
                k[r] = rtd[r][0] * k[irx]
                checked.add(r)
    mult = {"M": 1.0e6, "O2": 2.095e5, "N2": 7.808e5, "H2": 0.56, "CH4": 1.85}
    for key, rxns in man["third_body"].items():
        for r1 in rxns:
            if k[r1 - 1] is not None:
                k[r1 - 1] *= h2o if key == "H2O" else mult[key]
    return k, checked


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_calc_rconst_matches_rate_tables(mech):
    from oracle import Oracle
    o = Oracle(mech)
    man = manifest(mech)
    assert man["rate_tables"]["kunits"] == 2
    rng = np.random.default_rng(7)
    n = 16
    temp = rng.uniform(220.0, 320.0, n)
    press = rng.uniform(0.1, 1.05, n)
    h2o = rng.uniform(1.0e2, 3.0e4, n)
    rj = rng.uniform(1e-5, 0.5, (o.nphotab, n))
    het = rng.uniform(1e-6, 1e-2, (max(o.nhetero, 1), n))
    got = o.rconst(temp, press, h2o, rj, het, True, np.zeros(n))
    worst, nchecked = 0.0, 0
    for c in range(n):
        ref, checked = table_rates(man, temp[c], press[c], h2o[c], rj[:, c], het[:, c], True)
        for r in checked:
            if ref[r] == 0.0:
                assert got[r, c] == 0.0
                continue
            worst = max(worst, abs(got[r, c] - ref[r]) / abs(ref[r]))
        nchecked = len(checked)
    assert nchecked >= 0.9 * man["nrxns"], nchecked
    assert worst < 1e-12, worst
