"""The C ABI library exports every entry point its headers declare (no GPU needed)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
LIB = ROOT / "cmaq_gb300" / "_build" / "libcmaqchem.so"


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:int|void|long long)\s+(cmaqchem_\w+)\s*\(", text, flags=re.M)
    return names


@pytest.mark.skipif(not LIB.exists(), reason="libcmaqchem.so not built (python -m cmaq_gb300.build)")
def test_library_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 10
    lib = C.CDLL(str(LIB))
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


@pytest.mark.skipif(not LIB.exists(), reason="libcmaqchem.so not built")
def test_host_only_entry_points_work_without_gpu():
    from cmaq_gb300 import _lib
    info, order = _lib.mech_info("cb6r5_ae7_aq")
    assert (info.nspec, info.nrxns, info.iarray_day, info.iarray_night) == (149, 349, 1689, 1615)
    assert sorted(order) == list(range(149))
    with pytest.raises(_lib.ChemError, match="unknown mechanism"):
        _lib.mech_info("not_a_mechanism")


def _c_struct_fields(header: str, name: str):
    """(kind, field) pairs of `typedef struct {...} name;` in the C header, in order."""
    body = re.search(r"typedef struct \{([^}]*)\}\s*" + name + ";", header).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    out = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        m = re.match(r"(const\s+)?(long long|double|int|char)\s*(\*?)\s*(.*)", decl)
        kind = "ptr" if m.group(3) else {"long long": "llong", "double": "double", "int": "int"}[m.group(2)]
        out += [(kind, f.strip().lower()) for f in m.group(4).split(",")]
    return out


def _f_type_fields(shim: str, name: str):
    """(kind, field) pairs of `TYPE, BIND(C) :: name` in the Fortran source, in order."""
    body = re.search(r"TYPE, BIND\(C\) :: " + name + r"\n(.*?)END TYPE", shim, flags=re.S).group(1)
    kinds = {"TYPE(C_PTR)": "ptr", "INTEGER(C_INT)": "int", "REAL(C_DOUBLE)": "double",
             "INTEGER(C_LONG_LONG)": "llong"}
    out = []
    for line in body.strip().splitlines():
        t, fields = line.split("::")
        out += [(kinds[t.strip()], f.strip().lower()) for f in fields.split(",")]
    return out


def test_fortran_shim_binds_the_header_names():
    """include/chem_gpu.F (the drop-in CHEM for the Fortran host) binds the header's entry
    points by name, and its BIND(C) types have the C structs' fields in the same order
    with the same kinds (no Fortran compiler exists here to build it)."""
    shim = (ROOT / "include" / "chem_gpu.F").read_text()
    header = (ROOT / "include" / "cmaqchem.h").read_text()
    for n in ("cmaqchem_init", "cmaqchem_step", "cmaqchem_last_error"):
        assert f"NAME='{n}'" in shim and f" {n}(" in header
    cfg_c, cfg_f = _c_struct_fields(header, "cmaqchem_cfg"), _f_type_fields(shim, "CMAQCHEM_CFG")
    assert [k for k, _ in cfg_c] == [k for k, _ in cfg_f]
    assert [f for _, f in cfg_c][1:] == [f for _, f in cfg_f][1:]   # MECHANISM <-> mechanism
    st_c, st_f = _c_struct_fields(header, "cmaqchem_stats"), _f_type_fields(shim, "CMAQCHEM_STATS")
    assert [k for k, _ in st_c] == [k for k, _ in st_f] and len(st_c) == 6
    assert "SUBROUTINE CHEM( CONC, JDATE, JTIME, TSTEP )" in shim


HOST_PROGRAM = r"""
#include <stdio.h>
#include <stdlib.h>
#include "cmaqchem.h"

int main(void) {
    cmaqchem_mech_info info;
    int* order;
    int i, sum = 0;
    char msg[256];
    if (cmaqchem_mech_info_get("cb6r5_ae7_aq", &info, NULL) != 0) return 2;
    order = (int*)malloc(sizeof(int) * (size_t)info.nspec);
    if (cmaqchem_mech_info_get("cb6r5_ae7_aq", NULL, order) != 0) return 3;
    for (i = 0; i < info.nspec; ++i) sum += order[i];
    free(order);
    if (cmaqchem_mech_info_get("not_a_mechanism", &info, NULL) == 0) return 4;
    cmaqchem_last_error(msg, sizeof msg);
    printf("%d %d %d %d %d\n%s\n", info.nspec, info.nrxns, info.iarray_day, info.iarray_night, sum, msg);
    return 0;
}
"""


def _gcc():
    import shutil
    return shutil.which("gcc")


@pytest.mark.skipif(_gcc() is None, reason="no C compiler")
@pytest.mark.parametrize("lang,std", [("c", "-std=c99"), ("c++", "-std=c++11")])
def test_headers_compile_standalone(lang, std):
    """Each public header compiles on its own, as C for a Fortran/C host and as C++."""
    import subprocess
    for h in sorted((ROOT / "include").glob("*.h")):
        r = subprocess.run([_gcc(), std, "-Wall", "-Wextra", "-Werror", "-pedantic", "-fsyntax-only", "-x", lang,
                            str(h)], capture_output=True, text=True)
        assert r.returncode == 0, (h.name, r.stderr)


@pytest.mark.skipif(_gcc() is None or not LIB.exists(), reason="no C compiler or libcmaqchem.so not built")
def test_c_host_program_links_and_calls(tmp_path):
    """A plain C program built against include/cmaqchem.h links libcmaqchem.so and calls
    the host-only entry points, the way a non-Python host model binds the library."""
    import subprocess
    src = tmp_path / "host.c"
    src.write_text(HOST_PROGRAM)
    exe = tmp_path / "host"
    subprocess.run([_gcc(), "-std=c99", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(LIB.parent), "-lcmaqchem", f"-Wl,-rpath,{LIB.parent}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    first, msg = r.stdout.splitlines()[:2]
    assert first.split() == ["149", "349", "1689", "1615", str(sum(range(149)))]
    assert "unknown mechanism" in msg


@pytest.mark.skipif(not LIB.exists(), reason="libcmaqchem.so not built")
def test_kmt2_entry_checks_arguments_before_any_cuda_call():
    """cmaqchem_kmt2_* reject bad arguments on the host (no GPU needed)."""
    from cmaq_gb300 import _lib
    L = _lib.lib()
    per_lane = 7 * 161 + 2 * 738 + 269 + 4
    tail = L.cmaqchem_kmt2_workspace_doubles(1) - 32 * per_lane   # whole warps, then the queue's counter
    assert 1 <= tail <= 64
    assert L.cmaqchem_kmt2_workspace_doubles(32) == 32 * per_lane + tail
    assert L.cmaqchem_kmt2_workspace_doubles(1000) == 1024 * per_lane + tail
    assert L.cmaqchem_kmt2_workspace_doubles(0) == 0
    assert L.cmaqchem_kmt2_solve_device(0, None, None, None, None, None, None, 0, None) == 0
    assert L.cmaqchem_kmt2_solve_device(-1, None, None, None, None, None, None, 0, None) == -1
    assert "ncell" in _lib.last_error()
    assert L.cmaqchem_kmt2_solve_device(4, None, None, None, None, None, None, 0, None) == -1
    assert "null" in _lib.last_error()
    buf = (C.c_double * 8)()
    p = C.cast(buf, C.c_void_p)
    assert L.cmaqchem_kmt2_solve_device(4, p, p, p, None, p, p, 8, None) == -1
    assert "workspace" in _lib.last_error()


def test_aqchem_wrapper_rejects_host_tensors():
    torch = pytest.importorskip("torch")
    from cmaq_gb300.aqchem import aqchem_kinetics
    with pytest.raises(ValueError, match="CUDA tensor"):
        aqchem_kinetics(torch.zeros((15, 2), dtype=torch.float64), torch.zeros((161, 2), dtype=torch.float64))
