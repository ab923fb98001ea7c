"""bench.py's HETCHEM_RATES leg (run_hetchem) exercised on the CPU: the kernel call is
replaced by the host build of the same device code (tests/hetchem_host_harness.cpp) and
the CUDA plumbing by host stand-ins, so the leg's bookkeeping (inputs, the HBM roofline's
bytes, end-to-end bytes, the CPU-oracle leg and its parity summary) runs without a GPU.
Host build and oracle agree bit for bit, so the parity summary must be exact here."""
import sys
import time
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
torch = pytest.importorskip("torch")

from conftest import run_hetchem_harness  # noqa: E402


class _HostEvent:
    def __init__(self, **kw):
        self.t = 0.0

    def record(self, *a):
        self.t = time.perf_counter()

    def elapsed_time(self, other):
        return (other.t - self.t) * 1e3


@pytest.mark.parametrize("mech,nae,nhet", [("cb6r5_ae7_aq", 84, 17), ("cracmm2", 90, 9)])
def test_run_hetchem_bookkeeping_on_the_host(hetchem_harness, tmp_path, monkeypatch, mech, nae, nhet):
    import cmaq_gb300.hetchem as het

    def host_rates(ae, ta, pres, qv, dens, *, mechanism="cb6r5_ae7_aq", out=None, stream=None):
        k = torch.from_numpy(run_hetchem_harness(hetchem_harness(mechanism), ae.numpy(), ta.numpy(), pres.numpy(), qv.numpy(),
                                                 dens.numpy(), tmp_path).copy())
        if out is not None:
            out.copy_(k)
            return out
        return k

    to = torch.Tensor.to
    monkeypatch.setattr(het, "hetchem_rates", host_rates)
    monkeypatch.setattr(torch.cuda, "Event", _HostEvent)
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)
    monkeypatch.setattr(torch.Tensor, "pin_memory", lambda self: self)
    monkeypatch.setattr(torch.Tensor, "to", lambda self, *a, **k: self if a and str(a[0]).startswith("cuda")
                        else to(self, *a, **k))
    sys.path.insert(0, str(ROOT))
    import bench
    r = bench.run_hetchem(0, 300, 2, 2, mech)
    assert r["ncell"] == 300 and r["value"] > 0 and r["mechanism"] == mech
    assert r["roofline"]["bound"] == "hbm" and r["roofline"]["bytes_per_cell"] == nae * 4 + 16 + nhet * 8
    assert r["e2e"]["h2d_bytes_per_step"] == 300 * (nae + 4) * 4 and r["e2e"]["d2h_bytes_per_step"] == 300 * nhet * 8
    assert r["parity"]["cells"] == 300 and r["parity"]["max_rel_diff_off_switch"] == 0.0
    assert r["parity"]["cells_on_the_iepox_switch"] == 0
    assert r["cpu"]["cells"] == 300 and r["cpu"]["value"] > 0
