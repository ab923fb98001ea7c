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
        names += re.findall(r"^\s*(?:int|void)\s+(cmaqchem_\w+)\s*\(", text, flags=re.M)
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


def test_fortran_shim_binds_the_header_names():
    shim = (ROOT / "INTEGRATION.md").read_text() if (ROOT / "INTEGRATION.md").exists() else ""
    if not shim:
        pytest.skip("INTEGRATION.md not written yet")
    for n in ("cmaqchem_init", "cmaqchem_step", "cmaqchem_last_error"):
        assert n in shim
