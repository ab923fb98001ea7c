import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def cmaq_root() -> Path:
    """The CMAQ source tree the generator checks read: $CMAQ_ROOT, else a checkout named
    ``reference`` beside this repository.  Tests that need it skip when neither holds
    ``CCTM``."""
    import os
    env = os.environ.get("CMAQ_ROOT")
    return Path(env) if env else ROOT.parent / "reference"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libcmaqchem.so")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if gpu_available():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def kmt2_harness(tmp_path_factory):
    """tests/kmt2_host_harness.cpp (the KMT2 device code built for the host) compiled with
    g++ under AddressSanitizer and UndefinedBehaviorSanitizer; skipped without g++."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path_factory.mktemp("kmt2") / "kmt2_host_harness"
    cmd = [gxx, "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-o", str(exe), str(ROOT / "tests" / "kmt2_host_harness.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("sanitizer runtime not available")
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.fixture(scope="session")
def hetchem_harness(tmp_path_factory):
    """tests/hetchem_host_harness.cpp (the HETCHEM_RATES device code built for the host)
    compiled with g++ under AddressSanitizer and UndefinedBehaviorSanitizer: a function of
    the mechanism returning its executable (built once per mechanism)."""
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    built = {}

    def get(mech="cb6r5_ae7_aq"):
        if mech not in built:
            exe = tmp_path_factory.mktemp("hetchem") / f"hetchem_host_harness_{mech}"
            defs = [] if mech == "cb6r5_ae7_aq" else [f"-DHET_NS=het_{mech}", f'-DHET_GEN="gen/{mech}_hetchem.cuh"']
            cmd = [gxx, "-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-fsanitize=address,undefined",
                   "-fno-sanitize-recover=all", *defs, "-o", str(exe), str(ROOT / "tests" / "hetchem_host_harness.cpp")]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0 and "sanitize" in r.stderr:
                pytest.skip("sanitizer runtime not available")
            assert r.returncode == 0, r.stderr[-3000:]
            built[mech] = exe
        return built[mech]
    return get


def _host_build(tmp_path_factory, name, mech, srcs):
    """g++ build of a host harness with the mechanism's generated device files (csrc/gen)
    under AddressSanitizer and UndefinedBehaviorSanitizer, one object per file in
    parallel; CUDA qualifiers shimmed by tests/cuda_host_shim.h."""
    import os
    import shutil
    import subprocess
    from concurrent.futures import ThreadPoolExecutor
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp(f"{name}_{mech}")
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    flags = ["-std=c++17", "-O1", "-ffp-contract=off", "-fno-fast-math", "-fsanitize=address,undefined",
             "-fno-sanitize-recover=all", "-I", str(cuda_inc), "-include", str(ROOT / "tests" / "cuda_host_shim.h"),
             f'-DMECH_HEADER="../cmaq_gb300/csrc/gen/{mech}_mech.cuh"', f"-DMECH_NS=mech_{mech}"]

    def cc(src):
        obj = d / (src.stem + ".o")
        r = subprocess.run([gxx, *flags, "-x", "c++", "-c", str(src), "-o", str(obj)], capture_output=True, text=True)
        return obj, r

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        res = list(ex.map(cc, srcs))
    for _, r in res:
        if r.returncode != 0 and "sanitize" in r.stderr:
            pytest.skip("sanitizer runtime not available")
        assert r.returncode == 0, r.stderr[-3000:]
    exe = d / name
    r = subprocess.run([gxx, "-fsanitize=address,undefined", *[str(o) for o, _ in res], "-o", str(exe), "-lm"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.fixture(scope="session")
def ros3_harness(tmp_path_factory):
    """tests/ros3_host_harness.cpp with the mechanism's generated rate, LU and solve files
    (the ROS3 device code built for the host): a function of the mechanism returning its
    executable (built once per mechanism)."""
    gen = ROOT / "cmaq_gb300" / "csrc" / "gen"
    built = {}

    def get(mech="cb6r5_ae7_aq"):
        if mech not in built:
            srcs = ([ROOT / "tests" / "ros3_host_harness.cpp"] + sorted(gen.glob(f"{mech}_lu*.cu"))
                    + [gen / f"{mech}_solve0.cu", gen / f"{mech}_solve1.cu", gen / f"{mech}_rates.cu"])
            built[mech] = _host_build(tmp_path_factory, "ros3_host_harness", mech, srcs)
        return built[mech]
    return get


@pytest.fixture(scope="session")
def ebi_harness(tmp_path_factory):
    """tests/ebi_host_harness.cpp with the mechanism's generated EBI routines (the EBI
    device code built for the host): a function of the mechanism returning its executable."""
    gen = ROOT / "cmaq_gb300" / "csrc" / "gen"
    built = {}

    def get(mech="cb6r5_ae7_aq"):
        if mech not in built:
            srcs = [ROOT / "tests" / "ebi_host_harness.cpp", gen / f"{mech}_ebi.cu", gen / f"{mech}_rates.cu"]
            built[mech] = _host_build(tmp_path_factory, "ebi_host_harness", mech, srcs)
        return built[mech]
    return get


@pytest.fixture(scope="session")
def gear_harness(tmp_path_factory):
    """tests/gear_host_harness.cpp with the mechanism's generated f, PDERIV, LU and solve
    routines and the cooperative kernel's tables (the SMVGEAR device code built for the
    host): a function of the mechanism returning its executable."""
    gen = ROOT / "cmaq_gb300" / "csrc" / "gen"
    built = {}

    def get(mech="cb6r5_ae7_aq"):
        if mech not in built:
            srcs = ([ROOT / "tests" / "gear_host_harness.cpp"] + sorted(gen.glob(f"{mech}_glu*.cu"))
                    + [gen / f"{mech}_solve0.cu", gen / f"{mech}_rates.cu", gen / f"{mech}_gw_tables.cu"])
            built[mech] = _host_build(tmp_path_factory, "gear_host_harness", mech, srcs)
        return built[mech]
    return get


def run_gear_harness(exe, y0, rk, night, chemstep, rtol, max_atol, min_atol, conc_floor, workdir):
    """The host build's SMVGEAR over chemstep minutes: y [NSPEC][n] (solver order), rk
    [NRXNS][n], night [n]; returns (y, stats [n][8])."""
    import os
    import subprocess
    import numpy as np
    n = y0.shape[1]
    inp, out = workdir / "gear_in.bin", workdir / "gear_out.bin"
    np.concatenate([np.ascontiguousarray(y0, np.float64).view(np.uint8).ravel(),
                    np.ascontiguousarray(rk, np.float64).view(np.uint8).ravel(),
                    np.ascontiguousarray(night, np.uint8).ravel()]).tofile(inp)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), str(inp), str(out), str(n), repr(float(chemstep)), repr(float(rtol)),
                        repr(float(max_atol)), repr(float(min_atol)), repr(float(conc_floor))],
                       capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    raw = np.fromfile(out, np.uint8)
    ny = y0.size * 8
    return raw[:ny].view(np.float64).reshape(y0.shape), raw[ny:].view(np.int32).reshape(n, 8)


def run_ebi_harness(exe, yc0, rki, tstep_sec, workdir):
    """The host build's HRSOLVER over tstep_sec: yc [NSPEC][n] (mechanism order), rki
    [NRXNS][n]; returns (yc, status, iterations)."""
    import os
    import subprocess
    import numpy as np
    n = yc0.shape[1]
    inp, out = workdir / "ebi_in.bin", workdir / "ebi_out.bin"
    np.concatenate([np.ascontiguousarray(yc0, np.float64).view(np.uint8).ravel(),
                    np.ascontiguousarray(rki, np.float64).view(np.uint8).ravel()]).tofile(inp)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), str(inp), str(out), str(n), str(int(tstep_sec))], capture_output=True, text=True,
                       timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    raw = np.fromfile(out, np.uint8)
    ny = yc0.size * 8
    yc = raw[:ny].view(np.float64).reshape(yc0.shape)
    st = raw[ny:].view(np.int32).reshape(2, n)
    return yc, st[0], st[1]


def run_ros3_harness(exe, y0, rki, night, chemstep, rtol, atol, workdir):
    """The host build's per-cell ROS3 over chemstep minutes: y [ISCHAN][n] (new species
    order), rki [NRXNS][n], night [n]; returns (y, nsteps, nfails, status)."""
    import os
    import subprocess
    import numpy as np
    n = y0.shape[1]
    inp, out = workdir / "ros3_in.bin", workdir / "ros3_out.bin"
    np.concatenate([np.ascontiguousarray(y0, np.float64).view(np.uint8).ravel(),
                    np.ascontiguousarray(rki, np.float64).view(np.uint8).ravel(),
                    np.ascontiguousarray(night, np.uint8).ravel()]).tofile(inp)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), str(inp), str(out), str(n), repr(float(chemstep)), repr(float(rtol)),
                        repr(float(atol))], capture_output=True, text=True, timeout=900, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    raw = np.fromfile(out, np.uint8)
    ny = y0.size * 8
    y = raw[:ny].view(np.float64).reshape(y0.shape)
    st = raw[ny:].view(np.int32).reshape(3, n)
    return y, st[0], st[1], st[2]


def run_hetchem_harness(exe, ae, ta, pres, qv, dens, workdir):
    """KHETERO [ncell][NHET] of the host build for the aerosol block ae [NAE][ncell] and met."""
    import os
    import subprocess
    import numpy as np
    n = ae.shape[1]
    inp, out = workdir / "het_in.bin", workdir / "het_out.bin"
    np.concatenate([np.asarray(ae, np.float32).ravel()] + [np.asarray(x, np.float32).ravel()
                                                           for x in (ta, pres, qv, dens)]).tofile(inp)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), str(inp), str(out), str(n)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    return np.fromfile(out, np.float64).reshape(n, -1)


def run_kmt2_harness(exe, params_t, var_mix_t, nlanes, workdir):
    """Run the host build on [element][cell] arrays; returns var_out [161][n], fix_out
    [4][n], stats [10][n], the number of failed cells and the per-lane workspace size."""
    import os
    import subprocess
    import numpy as np
    n = params_t.shape[1]
    inp, out = workdir / "in.bin", workdir / "out.bin"
    np.concatenate([params_t.ravel(), var_mix_t.ravel()]).astype(np.float64).tofile(inp)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), str(inp), str(out), str(n), str(nlanes)], capture_output=True, text=True,
                       timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    raw = out.read_bytes()
    nv, nf = 161 * n, 4 * n
    var = np.frombuffer(raw[:8 * nv], np.float64).reshape(161, n)
    fix = np.frombuffer(raw[8 * nv:8 * (nv + nf)], np.float64).reshape(4, n)
    st = np.frombuffer(raw[8 * (nv + nf):], np.int32).reshape(10, n)
    nfail, ws_elems = map(int, r.stdout.split())
    return var, fix, st, nfail, ws_elems


def run_aqchem_harness(exe, params_t, gas_t, aer_t, aer_index, factors, nlanes, workdir):
    """The whole AQCHEM of the host build on [element][cell] arrays; returns gas, aerosol,
    gas_wdep, aer_wdep, out [10][n], stats [10][n] ([element][cell]) and the failed cells."""
    import os
    import subprocess
    import numpy as np
    n = params_t.shape[1]
    naer = aer_t.shape[0] // 3
    inp, out = workdir / "aq_in.bin", workdir / "aq_out.bin"
    with open(inp, "wb") as f:
        np.concatenate([params_t.ravel(), gas_t.ravel(), aer_t.ravel(), np.asarray(factors, np.float64)]).astype(
            np.float64).tofile(f)
        np.asarray(aer_index, np.int32).tofile(f)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0", UBSAN_OPTIONS="halt_on_error=1")
    r = subprocess.run([str(exe), "aqchem", str(inp), str(out), str(n), str(nlanes), str(naer)], capture_output=True,
                       text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-3000:]
    assert "runtime error" not in r.stderr, r.stderr[-3000:]
    raw = np.fromfile(out, dtype=np.uint8)
    ng, na = 29 * n, naer * 3 * n
    d = raw[:8 * (2 * ng + 2 * na + 10 * n)].view(np.float64)
    g, a = d[:ng].reshape(29, n), d[ng:ng + na].reshape(naer * 3, n)
    gw, aw = d[ng + na:2 * ng + na].reshape(29, n), d[2 * ng + na:2 * ng + 2 * na].reshape(naer * 3, n)
    o = d[2 * ng + 2 * na:].reshape(10, n)
    st = raw[8 * (2 * ng + 2 * na + 10 * n):].view(np.int32).reshape(10, n)
    return g, a, gw, aw, o, st, int(r.stdout.split()[0])
