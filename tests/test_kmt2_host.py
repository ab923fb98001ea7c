"""The KMT2 device code (cmaq_gb300/csrc/kmt2.cuh), built for the host, against the oracle.

kmt2.cuh is host/device code: tests/kmt2_host_harness.cpp compiles it with g++ under
AddressSanitizer and UndefinedBehaviorSanitizer and runs the kernel's lane loop over the
cells serially (same interleaved workspace, same [element][cell] arrays), so these CPU
tests check the product's arithmetic bit for bit against the oracle (same libm on both
sides) and every array index for the sizes below.  On the GPU only CUDA's exp / pow /
expf differ (tests/test_gpu_kmt2.py).
"""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
from kmt2 import KMT2Oracle, P_TEMP2, STATS  # noqa: E402

GXX = shutil.which("g++")
pytestmark = pytest.mark.skipif(GXX is None, reason="no C++ compiler")


@pytest.fixture(scope="module")
def o():
    return KMT2Oracle()


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = tmp_path_factory.mktemp("kmt2") / "kmt2_host_harness"
    cmd = [GXX, "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-o", str(exe), str(ROOT / "tests" / "kmt2_host_harness.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("sanitizer runtime not available")
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def run(harness, o, params, var_mix, nlanes, tmp_path):
    n = params.shape[0]
    inp = tmp_path / "in.bin"
    out = tmp_path / "out.bin"
    np.concatenate([params.T.ravel(), var_mix.T.ravel()]).astype(np.float64).tofile(inp)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(harness), str(inp), str(out), str(n), str(nlanes)], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    raw = out.read_bytes()
    nv, nf = o.nvar * n, o.nfix * n
    var = np.frombuffer(raw[:8 * nv], np.float64).reshape(o.nvar, n).T
    fix = np.frombuffer(raw[8 * nv:8 * (nv + nf)], np.float64).reshape(o.nfix, n).T
    st = np.frombuffer(raw[8 * (nv + nf):], np.int32).reshape(o.nstat, n).T
    nfail, ws_elems = map(int, r.stdout.split())
    return var, fix, st, nfail, ws_elems


@pytest.mark.parametrize("ncell,nlanes", [(37, 8), (5, 5), (1, 1), (12, 32)])
def test_device_code_equals_the_oracle(harness, o, tmp_path, ncell, nlanes):
    p, v = o.synthetic_cells(ncell, seed=100 + ncell)
    var, fix, st, nfail, ws_elems = run(harness, o, p, v, nlanes, tmp_path)
    vr, fr, sr, nf_r = o.cells(p, v)
    assert nfail == nf_r == 0
    assert ws_elems == 9 * o.nvar + 2 * o.lu_nonzero + o.nreact + o.nfix
    assert np.array_equal(st, sr)
    assert np.array_equal(var, vr)
    assert np.array_equal(fix, fr)


def test_switches_and_failed_cells(harness, o, tmp_path):
    """ISPC8 / MTPYRAC paths, and a cell with the reference's MET DATA ERROR next to good
    ones: status -101, the others unaffected."""
    p1, v1 = o.synthetic_cells(6, seed=7, ispc8=1, mtpyrac=1)
    p2, v2 = o.synthetic_cells(6, seed=8)
    p, v = np.concatenate([p1, p2]), np.concatenate([v1, v2])
    p[3, P_TEMP2] = 0.0
    var, _, st, nfail, _ = run(harness, o, p, v, 4, tmp_path)
    vr, _, sr, nf_r = o.cells(p, v)
    assert nfail == nf_r == 1
    ierr = STATS.index("ierr")
    assert st[3, ierr] == sr[3, ierr] == -101
    assert np.array_equal(st, sr)
    good = np.arange(len(p)) != 3
    assert np.array_equal(var[good], vr[good])
