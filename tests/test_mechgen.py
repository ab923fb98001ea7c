"""Mechanism generator: parsed sizes, symbolic LU, rate-program coverage, reproducibility."""
import ctypes as C
import filecmp
from pathlib import Path

import numpy as np
import pytest

from cmaq_gb300.synthetic import manifest
from conftest import cmaq_root  # noqa: E402

ROOT = Path(__file__).resolve().parents[1]
CMAQ = cmaq_root()


@pytest.mark.parametrize("mech,ns,nr,iarray,nnzj", [
    ("cb6r5_ae7_aq", 149, 349, [1689, 1615], [1417, 1365]),
    ("cracmm2", 189, 531, [3284, 3199], [2601, 2548]),
])
def test_manifest_sizes(mech, ns, nr, iarray, nnzj):
    m = manifest(mech)
    assert (m["nspec"], m["nrxns"], m["ischan"]) == (ns, nr, ns)
    assert m["iarray"] == iarray and m["nnz_jac"] == nnzj
    # night list = day list minus photolytic reactions (rbsparse.F:275-279)
    day, night = m["active"]
    assert set(night) == {r for r in day if not m["reactions"][r]["photolytic"]}


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_every_reaction_has_one_rate_expression(mech):
    m = manifest(mech)
    blocks = m["rate_tables"]["rate_block"]
    assert len(blocks) == m["nrxns"]
    photo = {int(r) for r, b in blocks.items() if b in ("photo", "seawater")}
    # CALC_RCONST's sunlit block holds exactly the photolysis (KTYPE 0) reactions and the
    # seawater-conditioned halogen reaction (KTYPE 12)
    kt = m["rate_tables"]["ktype"]
    assert photo == {r for r in range(m["nrxns"]) if kt[r] in (0, 12)}


def test_lu_factors_reproduce_jacobian():
    """L U = J - g I with J from central differences of the oracle's f(y) (day pattern)."""
    from oracle import Oracle
    o = Oracle("cb6r5_ae7_aq")
    man = manifest("cb6r5_ae7_aq")
    rng = np.random.default_rng(0)
    n = 1
    k = o.rconst(np.array([290.0]), np.array([1.0]), np.array([1.0e4]), np.full((o.nphotab, n), 1e-3),
                 np.zeros((o.nhetero, n)), True, np.zeros(n))
    y = np.exp(rng.uniform(np.log(1e-8), np.log(1e-2), size=(o.nspec, n)))
    N = o.ischan
    J = np.zeros((N, N))
    for j in range(N):
        h = y[j, 0] * 1e-5
        yp, ym = y.copy(), y.copy()
        yp[j, 0] += h
        ym[j, 0] -= h
        J[:, j] = (o.feval(yp, k)[:, 0] - o.feval(ym, k)[:, 0]) / (2 * h)
    g = 100.0
    iar = man["iarray"][0]
    cc2 = np.zeros((iar + 1, n))
    vd = np.zeros((N, n))
    dp = C.POINTER(C.c_double)
    o.lib.oracle_jac_decomp(n, 0, y.ctypes.data_as(dp), k.ctypes.data_as(dp), g, cc2.ctypes.data_as(dp),
                            vd.ctypes.data_as(dp))
    from cmaq_gb300.mechgen.sparse import build_sparse  # structure from the committed manifest order
    inew = man["inew2old"]
    assert inew == list(o.inew2old)
    # rebuild L and U from storage using the generator's storage map
    jpt = _storage_map(man)
    L = np.eye(N)
    U = np.zeros((N, N))
    for (i, j), st in jpt.items():
        if i > j:
            L[i, j] = cc2[st, 0]
        elif i < j:
            U[i, j] = cc2[st, 0]
    U[np.arange(N), np.arange(N)] = 1.0 / vd[:, 0]
    A = J - g * np.eye(N)
    rel = np.abs(L @ U - A) / np.maximum(np.abs(A), 1e-6 * np.abs(A).max())
    assert rel.max() < 1e-4


def _storage_map(man):
    """Storage index of each LU entry, recomputed from the manifest's reaction lists."""
    from cmaq_gb300.mechgen.fortran_tables import Mechanism
    from cmaq_gb300.mechgen.sparse import build_sparse
    m = Mechanism(name=man["mechname"], nspec=man["nspec"], nrxns=man["nrxns"])
    m.mxprd = man["mxprd"]
    m.irr = []
    for r in man["reactions"]:
        row = [0] * (3 + m.mxprd)
        for i, s in enumerate(r["reactants"]):
            row[i] = s + 1
        for i, s in enumerate(r["products"]):
            row[3 + i] = s + 1
        m.irr.append(row)
    m.nreact = [r["nreact"] for r in man["reactions"]]
    m.nprdct = [r["nprdct"] for r in man["reactions"]]
    m.sc = [r["sc"] + [0.0] * (m.mxprd - len(r["sc"])) for r in man["reactions"]]
    m.irxbits = [2 if r["photolytic"] else 0 for r in man["reactions"]]
    sp = build_sparse(m)
    assert sp.iarray == man["iarray"]
    return sp.jarraypt[0]


@pytest.mark.skipif(not (CMAQ / "CCTM" / "src" / "MECHS" / "cb6r5_ae7_aq").exists(),
                    reason="CMAQ source tree not available")
def test_generator_reproduces_committed_outputs(tmp_path):
    from cmaq_gb300.mechgen.generate import write_outputs
    write_outputs(str(CMAQ), "cb6r5_ae7_aq", out_root=tmp_path)
    for rel in ["cmaq_gb300/mechs/cb6r5_ae7_aq/manifest.json", "oracle/gen/cb6r5_ae7_aq_mech.c",
                "cmaq_gb300/csrc/gen/cb6r5_ae7_aq_mech.cuh", "cmaq_gb300/csrc/gen/cb6r5_ae7_aq_rates.cu",
                "cmaq_gb300/csrc/gen/cb6r5_ae7_aq_solve0.cu"]:
        assert filecmp.cmp(tmp_path / rel, ROOT / rel, shallow=False), rel
