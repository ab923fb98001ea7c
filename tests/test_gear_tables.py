"""Schedules of the warp-cooperative SMVGEAR routines (the generator's gw tables).

The one-cell-per-warp Gear kernel spreads a cell's work over the lanes with table-driven
routines; its results equal the generated sequential routines' bit for bit only if every
element receives the same operations in the same order.  Checked here on the tables the
generator emits, against the symbolic LU of the mechanism:
* elimination by pivot (right-looking): each LU entry receives exactly the updates of the
  sequential row-by-row elimination, in the same (ascending pivot) order; within a pivot
  the update targets are distinct and none is read by another update of that pivot;
* every L entry is scaled once, at its column's pivot;
* forward / backward substitution levels respect the row dependencies;
* every species' derivative sum is assigned to exactly one lane.
"""
import re
from pathlib import Path

import pytest
from conftest import cmaq_root  # noqa: E402

CMAQ = cmaq_root()
pytestmark = pytest.mark.skipif(not (CMAQ / "CCTM").exists(), reason="needs the CMAQ sources")


def _tables(mech):
    from cmaq_gb300.mechgen import generate
    from cmaq_gb300.mechgen.emit_cuda import Layout, _gear_warp_tables
    m, prog, sp, _ = generate.load(str(CMAQ), mech)
    _, defs, _ = _gear_warp_tables(m, sp, Layout(m, sp))
    tab = {}
    for line in defs:
        mm = re.match(r"__device__ const (int|double) c_gw_(\w+)\[\d+\] = \{(.*)\};", line)
        conv = float if mm.group(1) == "double" else int
        tab[mm.group(2)] = [conv(x) for x in mm.group(3).split(", ")]
    return sp, tab


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_gear_cooperative_schedules(mech):
    sp, tab = _tables(mech)
    d, n, jpt = 0, sp.ischan, sp.jarraypt[0]
    sequential = {}
    for i in range(n):
        for (st_ik, k) in sp.lower[d][i]:
            for (st_kj, j) in sp.upper[d][k]:
                sequential.setdefault(jpt[(i, j)], []).append((st_ik, st_kj))
    by_pivot = {}
    for k in range(n):
        lo, hi = tab["up_ptr"][k], tab["up_ptr"][k + 1]
        targets = tab["up_ij"][lo:hi]
        sources = set(tab["up_ik"][lo:hi]) | set(tab["up_kj"][lo:hi])
        assert len(targets) == len(set(targets)) and not set(targets) & sources
        for t in range(lo, hi):
            by_pivot.setdefault(tab["up_ij"][t], []).append((tab["up_ik"][t], tab["up_kj"][t]))
        assert tab["piv_diag"][k] == jpt[(k, k)]
    assert by_pivot == sequential
    assert sorted(tab["lsc_st"]) == sorted(st for i in range(n) for (st, _) in sp.lower[d][i])
    for kind, deps in (("f", sp.lower[d]), ("b", sp.upper[d])):
        level = {}
        ptr, rows = tab[f"{kind}l_ptr"], tab[f"{kind}l_row"]
        for lv in range(len(ptr) - 1):
            for u in range(ptr[lv], ptr[lv + 1]):
                level[rows[u]] = lv
        assert len(level) == n
        assert all(level[j] < level[i] for i in range(n) for (_, j) in deps[i])
    assert sorted(tab["lane_sp"]) == list(range(n)) and len(tab["lane_ptr"]) == 33
