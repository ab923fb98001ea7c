"""The library's FP64 measurement helpers (include/cmaqchem_diag.h) on the GPU.

The FP64 throughput probe must report a plausible peak, and the chain probe shows the
property the one-cell-per-warp kernels are built around: a dependent FP64 FMA costs the
same clock cycles whether 1 or 32 lanes of the warp are active.
"""
import pytest

pytestmark = pytest.mark.gpu


def test_fp64_peak_and_chain_latency():
    from cmaq_gb300 import _lib
    tf, ms = _lib.fp64_peak(0)
    assert tf > 0.1 and ms > 0.0
    one, full = _lib.fp64_issue(0, 1), _lib.fp64_issue(0, 32)
    assert one >= 4.0 and full >= 4.0
    assert 0.8 < one / full < 1.25
    with pytest.raises(_lib.ChemError):
        _lib.fp64_issue(0, 0)
