"""GPU parity of the KMT2 aqueous cloud chemistry kernel (CCTM/src/cloud/acm_ae7_kmt2)
against the CPU oracle, through the C ABI (cmaqchem_kmt2_solve_device).

The device code and the oracle perform the same IEEE operations in the same order:
-fmad=false on the device and -ffp-contract=off in the oracle, explicit fma where the
reference's a*b+c becomes one, and every exp and x**y by the same portable series
(kq_exp / kq_pow, portable_exp / portable_pow), because CUDA's and libm's exp and pow
differ by ulps and Rodas3's step control amplifies one ulp in a rate constant to 1e-5
in the final state.  The bar is therefore bit equality: every state element, fixed
species and step counter of every cell equals the oracle's.
"""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
from kmt2 import KMT2Oracle, P_TEMP2, STATS  # noqa: E402

pytestmark = pytest.mark.gpu
IERR, NSTP, NACC = STATS.index("ierr"), STATS.index("nstp"), STATS.index("nacc")


@pytest.fixture(scope="module")
def o():
    return KMT2Oracle()


def _gpu(p, v, **kw):
    import torch
    from cmaq_gb300.aqchem import aqchem_kinetics
    pt = torch.from_numpy(np.ascontiguousarray(p.T)).cuda()
    vt = torch.from_numpy(np.ascontiguousarray(v.T)).cuda()
    var, fix, st = aqchem_kinetics(pt, vt, with_fix=True, **kw)
    torch.cuda.synchronize()
    return var.cpu().numpy().T, fix.cpu().numpy().T, st.cpu().numpy().T


def _rel(a, b):
    big = np.abs(b) > 1e-6 * np.abs(b).max(axis=1, keepdims=True)
    return np.where(big, np.abs(a - b) / np.maximum(np.abs(b), 1e-300), 0.0).max(axis=1)


@pytest.mark.parametrize("seed,ispc8,mtpyrac", [(31, 0, 0), (32, 1, 1)])
def test_kmt2_kernel_parity(o, seed, ispc8, mtpyrac):
    p, v = o.synthetic_cells(200, seed=seed, ispc8=ispc8, mtpyrac=mtpyrac)
    var, fix, st = _gpu(p, v)
    vr, fr, sr, nfail = o.cells(p, v)
    assert nfail == 0 and (st[:, IERR] == 1).all()
    assert np.array_equal(st, sr), "step counters differ from the oracle"
    bad = np.where((var != vr).any(axis=1))[0]
    assert len(bad) == 0, f"cells {bad[:8]} differ from the oracle (max rel {_rel(var, vr).max():.3e})"
    assert np.array_equal(fix, fr)


def test_kmt2_lanes_do_not_change_the_bits(o):
    """Fewer lanes than cells (each lane integrates several cells in turn) gives the same
    bits as one lane per cell."""
    p, v = o.synthetic_cells(45, seed=33)
    a = _gpu(p, v)
    b = _gpu(p, v, lanes=7)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[2], b[2])


def test_kmt2_failed_cell_and_empty_call(o):
    import torch
    from cmaq_gb300.aqchem import aqchem_kinetics
    p, v = o.synthetic_cells(4, seed=34)
    p[1, P_TEMP2] = 0.0
    var, fix, st = _gpu(p, v)
    assert st[1, IERR] == -101 and (st[[0, 2, 3], IERR] == 1).all()
    assert np.isnan(var[1]).all() and np.isnan(fix[1]).all()     # no state: NaN, not stale memory
    assert np.isfinite(var[[0, 2, 3]]).all()
    out, stats = aqchem_kinetics(torch.zeros((15, 0), dtype=torch.float64, device="cuda"),
                                 torch.zeros((161, 0), dtype=torch.float64, device="cuda"))
    assert out.shape == (161, 0) and stats.shape == (10, 0)


def test_kmt2_rejects_bad_arguments():
    import torch
    from cmaq_gb300 import _lib
    from cmaq_gb300.aqchem import aqchem_kinetics
    with pytest.raises(ValueError):
        aqchem_kinetics(torch.zeros((15, 3), dtype=torch.float32, device="cuda"),
                        torch.zeros((161, 3), dtype=torch.float64, device="cuda"))
    L = _lib.lib()
    ws = torch.empty(10, dtype=torch.float64, device="cuda")
    x = torch.zeros((161, 2), dtype=torch.float64, device="cuda")
    import ctypes as C
    rc = L.cmaqchem_kmt2_solve_device(2, C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()), C.c_void_p(x.data_ptr()),
                                      None, C.c_void_p(ws.data_ptr()), C.c_void_p(ws.data_ptr()), ws.numel(), None)
    assert rc == -1 and "workspace" in _lib.last_error()


def test_kmt2_host_array_entry_equals_the_device_entry(o):
    """cmaqchem_kmt2_solve (host arrays, copies inside the call) gives the device entry's bits."""
    from cmaq_gb300.aqchem import aqchem_kinetics_host
    p, v = o.synthetic_cells(37, seed=35)
    var, fix, st = _gpu(p, v)
    hv, hf, hs = aqchem_kinetics_host(p.T, v.T, with_fix=True)
    assert np.array_equal(hv.T, var) and np.array_equal(hf.T, fix) and np.array_equal(hs.T, st)
    empty = aqchem_kinetics_host(np.zeros((15, 0)), np.zeros((161, 0)))
    assert empty[0].shape == (161, 0)


@pytest.mark.parametrize("seed,ispc8,mtpyrac", [(41, 0, 0), (42, 1, 1)])
def test_whole_aqchem_equals_the_oracle(o, seed, ispc8, mtpyrac):
    """cmaqchem_aqchem_device (mapping, kinetic core, redistribution) against the oracle's
    restatement: every output bit for bit, with AQCHEM's surrogates at shuffled rows of the
    aerosol list and a failed set-up among the cells."""
    import torch
    from cmaq_gb300.aqchem import aqchem
    p, g, a, idx, fac = o.synthetic_columns(150, seed=seed, ispc8=ispc8, mtpyrac=mtpyrac)
    naer = len(idx)
    perm = np.random.default_rng(seed).permutation(naer)
    a2 = np.zeros_like(a)
    for m in range(3):
        a2[:, perm + naer * m] = a[:, np.arange(naer) + naer * m]
    p[7, P_TEMP2] = 0.0
    rg, ra, rgw, raw_, ro, rs, rnf = o.aqchem(p, g, a2, perm, fac)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    pg, gg, ga = t(p), t(g), t(a2)
    gwd, awd, out, st = aqchem(pg, gg, ga, perm, fac)
    torch.cuda.synchronize()
    assert np.array_equal(st.cpu().numpy().T, rs)
    for got, ref in ((gg, rg), (ga, ra), (gwd, rgw), (awd, raw_), (out, ro)):
        assert np.array_equal(got.cpu().numpy().T, ref, equal_nan=True)
    assert np.isnan(rg[7]).all() and np.abs(ro[np.arange(150) != 7, 6:10]).max() < 1e-2
