"""bench.py's KMT2 line (--only-aqchem: run_aqchem) exercised on the CPU.

The kernel call is replaced by the host build of the same device code
(tests/kmt2_host_harness.cpp, see tests/test_kmt2_host.py) and the CUDA plumbing (pinned
memory, device copies, events) by host stand-ins, so the bench's bookkeeping (inputs,
FLOP accounting from the manifest, end-to-end bytes, the CPU-oracle leg and its parity
summary) runs without a GPU.  Host build and oracle agree bit for bit, so the parity
summary must be exact here.
"""
import sys
import time
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
torch = pytest.importorskip("torch")

from conftest import run_kmt2_harness  # noqa: E402


class _HostEvent:
    def __init__(self, **kw):
        self.t = 0.0

    def record(self, *a):
        self.t = time.perf_counter()

    def elapsed_time(self, other):
        return (other.t - self.t) * 1e3


def test_run_aqchem_bookkeeping_on_the_host(kmt2_harness, tmp_path, monkeypatch):
    import cmaq_gb300.aqchem as aq

    def host_kinetics(params, var_mix, *, lanes=None, with_fix=False, stream=None):
        var, fix, st, _, _ = run_kmt2_harness(kmt2_harness, params.numpy(), var_mix.numpy(),
                                              lanes or params.shape[1], tmp_path)
        out = (torch.from_numpy(var.copy()), torch.from_numpy(st.copy()))
        return (out[0], torch.from_numpy(fix.copy()), out[1]) if with_fix else out

    to = torch.Tensor.to
    monkeypatch.setattr(aq, "aqchem_kinetics", host_kinetics)
    monkeypatch.setattr(torch.cuda, "Event", _HostEvent)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(torch.Tensor, "pin_memory", lambda self: self)
    monkeypatch.setattr(torch.Tensor, "to", lambda self, *a, **k: self if a and str(a[0]).startswith("cuda")
                        else to(self, *a, **k))
    sys.path.insert(0, str(ROOT))
    import bench
    r = bench.run_aqchem(0, 40, 2, 1, 2, whole=False)
    assert r["ncell"] == 40 and r["failed_cells"] == 0 and r["value"] > 0
    assert 20 < r["steps_per_cell"] < 100
    fl = bench_manifest_flops()
    assert r["flops_per_call"] > 40 * 20 * fl["per_attempt"]
    # each routine's count times its own counter: four solves per attempt, f at stages 3 and 4
    # plus once per accepted step, one J per accepted step, at least one factorisation per attempt
    per_cell = 20 * (fl["decomp"] + 4 * fl["solve"] + 2 * fl["fun"] + fl["vector"])
    assert r["flops_per_call"] > 40 * per_cell
    assert r["e2e"]["h2d_bytes_per_step"] == 40 * (15 + 161) * 8 and r["e2e"]["d2h_bytes_per_step"] == 40 * 161 * 8
    assert r["parity"] == {"cells": 40, "same_steps": 1.0, "bit_equal_cells": 1.0, "max_rel": 0.0}
    assert r["cpu"]["cells"] == 40 and r["cpu"]["value"] > 0


def bench_manifest_flops():
    from cmaq_gb300.synthetic import kmt2_manifest
    return kmt2_manifest()["flops"]
