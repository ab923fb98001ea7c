"""Heterogeneous rate constants KHETERO on the GPU: HETCHEM_RATES of CMAQ
(CCTM/src/aero/aero6/AEROSOL_CHEMISTRY.F:282-1535) through the C ABI
(include/cmaqchem.h: cmaqchem_hetchem_*).

The input is the aerosol block of CGRID (the AE namelist's species expanded by mode,
``layout()`` gives its rows and its first row in the mechanism's CGRID) and the met
fields of the cells; the output is KHETERO(NHETERO, cell), the array the CHEM entries
take (``cmaq_gb300.chem.ChemSolver.step``'s ``khetero``, cell index slowest).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


def _ptr(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


def layout(mechanism: str = "cb6r5_ae7_aq") -> tuple[int, int, int]:
    """(rows of the aerosol block, its first row in the mechanism's CGRID, NHETERO)."""
    nae, first, nhet = C.c_int(), C.c_int(), C.c_int()
    _lib.check(_lib.lib().cmaqchem_hetchem_layout(mechanism.encode(), C.byref(nae), C.byref(first), C.byref(nhet)))
    return nae.value, first.value, nhet.value


def hetchem_rates(ae: torch.Tensor, ta: torch.Tensor, pres: torch.Tensor, qv: torch.Tensor, dens: torch.Tensor, *,
                  mechanism: str = "cb6r5_ae7_aq", out: torch.Tensor | None = None,
                  stream: torch.cuda.Stream | None = None) -> torch.Tensor:
    """KHETERO [ncell][NHETERO] (float64) of ncell cells: ``ae`` the CGRID aerosol block as a
    contiguous float32 CUDA tensor (NAE, ncell) (ug/m3, #/m3, m2/m3), ``ta``, ``pres``,
    ``qv``, ``dens`` float32 (ncell,) (K, Pa, kg/kg, kg/m3)."""
    nae, _, nhet = layout(mechanism)
    if not (ae.is_cuda and ae.dtype == torch.float32 and ae.dim() == 2 and ae.shape[0] == nae and ae.is_contiguous()):
        raise ValueError(f"ae must be a contiguous float32 CUDA tensor of shape ({nae}, ncell)")
    n = ae.shape[1]
    met = []
    for name, t in (("ta", ta), ("pres", pres), ("qv", qv), ("dens", dens)):
        t = t.reshape(-1)
        if not (t.is_cuda and t.dtype == torch.float32 and t.numel() == n and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous float32 CUDA tensor of {n} cells")
        met.append(t)
    if out is None:
        out = torch.empty((n, nhet), dtype=torch.float64, device=ae.device)
    elif not (out.dtype == torch.float64 and out.is_contiguous() and out.numel() == n * nhet):
        raise ValueError(f"out must be a contiguous float64 tensor of {n} x {nhet}")
    s = stream or torch.cuda.current_stream(ae.device)
    with torch.cuda.device(ae.device):
        _lib.check(_lib.lib().cmaqchem_hetchem_rates_device(mechanism.encode(), n, _ptr(ae), *[_ptr(t) for t in met],
                                                            _ptr(out), C.c_void_p(s.cuda_stream)))
    return out


def hetchem_rates_host(ae, ta, pres, qv, dens, *, mechanism: str = "cb6r5_ae7_aq", device: int = 0):
    """The same on host numpy arrays through the host-array entry (cmaqchem_hetchem_rates)."""
    import numpy as np
    f = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    ae = f(ae)
    n = ae.shape[1]
    met = [f(x).reshape(-1) for x in (ta, pres, qv, dens)]
    nhet = layout(mechanism)[2]
    out = np.empty((n, nhet))
    p = lambda a: C.c_void_p(a.ctypes.data)
    _lib.check(_lib.lib().cmaqchem_hetchem_rates(mechanism.encode(), n, p(ae), *[p(x) for x in met], p(out),
                                                 int(device)))
    return out
