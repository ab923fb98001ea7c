"""The KMT2 device code (cmaq_gb300/csrc/kmt2.cuh), built for the host, against the oracle.

kmt2.cuh is host/device code: tests/kmt2_host_harness.cpp compiles it with g++ under
AddressSanitizer and UndefinedBehaviorSanitizer and runs the kernels' cell queue serially
(one Rodas3 attempt per busy lane per pass, same interleaved workspace, same
[element][cell] arrays), so these CPU
tests check the product's arithmetic bit for bit against the oracle (same libm on both
sides, exp and pow by the portable series of both) and every array index for the sizes
below.  tests/test_gpu_kmt2.py holds the GPU to the same bits.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
from kmt2 import KMT2Oracle, P_TEMP2, STATS  # noqa: E402

from conftest import run_aqchem_harness, run_kmt2_harness  # noqa: E402


@pytest.fixture(scope="module")
def o():
    return KMT2Oracle()


def run(harness, o, params, var_mix, nlanes, tmp_path):
    var, fix, st, nfail, ws_elems = run_kmt2_harness(harness, params.T, var_mix.T, nlanes, tmp_path)
    return var.T, fix.T, st.T, nfail, ws_elems


@pytest.mark.parametrize("ncell,nlanes", [(37, 8), (5, 5), (1, 1), (12, 32)])
def test_device_code_equals_the_oracle(kmt2_harness, o, tmp_path, ncell, nlanes):
    p, v = o.synthetic_cells(ncell, seed=100 + ncell)
    var, fix, st, nfail, ws_elems = run(kmt2_harness, o, p, v, nlanes, tmp_path)
    vr, fr, sr, nf_r = o.cells(p, v)
    assert nfail == nf_r == 0
    assert ws_elems == 7 * o.nvar + 2 * o.lu_nonzero + o.nreact + o.nfix
    assert np.array_equal(st, sr)
    assert np.array_equal(var, vr)
    assert np.array_equal(fix, fr)


def test_switches_and_failed_cells(kmt2_harness, o, tmp_path):
    """ISPC8 / MTPYRAC paths, and a cell with the reference's MET DATA ERROR next to good
    ones: status -101, the others unaffected."""
    p1, v1 = o.synthetic_cells(6, seed=7, ispc8=1, mtpyrac=1)
    p2, v2 = o.synthetic_cells(6, seed=8)
    p, v = np.concatenate([p1, p2]), np.concatenate([v1, v2])
    p[3, P_TEMP2] = 0.0
    var, _, st, nfail, _ = run(kmt2_harness, o, p, v, 4, tmp_path)
    vr, _, sr, nf_r = o.cells(p, v)
    assert nfail == nf_r == 1
    ierr = STATS.index("ierr")
    assert st[3, ierr] == sr[3, ierr] == -101
    assert np.array_equal(st, sr)
    good = np.arange(len(p)) != 3
    assert np.array_equal(var[good], vr[good])
    assert np.isnan(var[3]).all() and np.isnan(vr[3]).all()     # a failed set-up leaves NaN, not stale memory


@pytest.mark.parametrize("ncell,nlanes,ispc8,mtpyrac", [(23, 5, 0, 0), (9, 9, 1, 1)])
def test_whole_aqchem_device_code_equals_the_oracle(kmt2_harness, o, tmp_path, ncell, nlanes, ispc8, mtpyrac):
    """The whole AQCHEM (kq_aq_map, the queued kinetic core, kq_aq_finish) built for the host against the
    oracle's restatement: every output bit for bit, with a shuffled surrogate order (the
    positions array maps AQCHEM's surrogates into the caller's aerosol list) and a failed
    set-up next to good cells."""
    p, g, a, idx, fac = o.synthetic_columns(ncell, seed=200 + ncell, ispc8=ispc8, mtpyrac=mtpyrac)
    naer = len(idx)
    perm = np.random.default_rng(1).permutation(naer)          # surrogate k lives at row perm[k]
    a2 = np.zeros_like(a)
    for m in range(3):
        a2[:, perm + naer * m] = a[:, np.arange(naer) + naer * m]
    p[2, P_TEMP2] = 0.0
    hg, ha, hgw, haw, ho, hs, hnf = run_aqchem_harness(kmt2_harness, p.T, g.T, a2.T, perm, fac, nlanes, tmp_path)
    rg, ra, rgw, raw_, ro, rs, rnf = o.aqchem(p, g, a2, perm, fac)
    assert hnf == rnf >= 1
    assert np.array_equal(hs.T, rs)
    for h, r in ((hg, rg), (ha, ra), (hgw, rgw), (haw, raw_), (ho, ro)):
        assert np.array_equal(h.T, r, equal_nan=True)
    assert np.isnan(rg[2]).all() and np.isfinite(rg[np.arange(ncell) != 2]).all()
