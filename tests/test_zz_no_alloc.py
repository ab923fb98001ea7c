"""The allocation-free solver entry point (cmaqchem_ros3_solve_noalloc) against the
handle-based one (cmaqchem_ros3_solve_device).

The allocation-free entry is for callers that cannot allocate device memory where
they call the chemistry (host models that own all device memory through their own
pool, fixed memory budgets, loops that cannot take cudaMalloc's device-wide
synchronisation).  It keeps its workspace in a static device array shared by all
calls, so the test makes two calls in a row on different inputs and checks both
against the handle-based entry, within the tolerance of the other solver tests
(relative 1e-9 on species above 1e-10 ppmV).  This file sorts last so that a run
stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import gather_cells, rel_err
from cmaq_gb300.synthetic import make_grid

pytestmark = pytest.mark.gpu

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


def _noalloc(lib, y, rki, night, chemstep):
    import torch
    st = torch.full((y.shape[1],), -1, dtype=torch.int32, device=y.device)
    fn = lib.cmaqchem_ros3_solve_noalloc
    fn.argtypes = [C.c_char_p, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                   C.c_double, C.c_void_p, C.c_void_p]
    rc = fn(b"cb6r5_ae7_aq", y.shape[1], y.data_ptr(), rki.data_ptr(), night.data_ptr(), chemstep, RTOL, ATOL,
            st.data_ptr(), None)
    if rc != 0:
        buf = C.create_string_buffer(1024)
        lib.cmaqchem_last_error(buf, len(buf))
        raise AssertionError(buf.value.decode())
    return st


def test_noalloc_entry_matches_handle_entry_on_two_calls_in_a_row():
    import torch
    from oracle import Oracle
    from cmaq_gb300 import _lib
    from cmaq_gb300.chem import ChemSolver
    o = Oracle("cb6r5_ae7_aq")
    lib = _lib.lib()
    for call, seed in enumerate((31, 32)):
        g = make_grid(ncols=9, nrows=7, nlays=3, seed=seed)
        y0, rki, night = gather_cells(g, o)
        rk = torch.from_numpy(rki).cuda()
        nt = torch.from_numpy(night).cuda()
        y_ref = torch.from_numpy(y0.copy()).cuda()
        s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd, rtol=1e-3, atol=1e-9)
        st_ref, _, _ = s.solve(y_ref, rk, nt, 5.0, with_stats=True)
        s.close()
        y = torch.from_numpy(y0.copy()).cuda()
        st = _noalloc(lib, y, rk, nt, 5.0)
        assert (st.cpu().numpy() == st_ref.cpu().numpy()).all(), f"status differs on call {call}"
        assert rel_err(y.cpu().numpy(), y_ref.cpu().numpy()) < 1e-9, f"call {call}"


def test_noalloc_entry_rejects_bad_sizes():
    import torch
    from cmaq_gb300 import _lib
    lib = _lib.lib()
    fn = lib.cmaqchem_ros3_solve_noalloc
    fn.argtypes = [C.c_char_p, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_double,
                   C.c_double, C.c_void_p, C.c_void_p]
    y = torch.zeros((149, 4), dtype=torch.float64, device="cuda")
    assert fn(b"cb6r5_ae7_aq", (1 << 31) + 1, y.data_ptr(), y.data_ptr(), y.data_ptr(), 5.0, RTOL, ATOL, None,
              None) == -1
    buf = C.create_string_buffer(256)
    lib.cmaqchem_last_error(buf, len(buf))
    assert b"ncell must be in" in buf.value
    assert fn(b"no_such_mech", 4, y.data_ptr(), y.data_ptr(), y.data_ptr(), 5.0, RTOL, ATOL, None, None) == -1
