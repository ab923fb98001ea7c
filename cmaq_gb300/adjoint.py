"""Gradients of the ROS3 chemistry: a ``torch.autograd.Function`` over the library's
discrete adjoint (``cmaqchem_adj_forward`` / ``cmaqchem_adj_backward``).

The forward map is the solver-level RBSOLVER (CCTM/src/gas/ros3/rbsolver.F) applied
to every cell for ``nsync`` synchronisation steps of ``chemstep`` minutes, with two
inputs that the reference keeps fixed made differentiable:

* ``log_k`` [nrxns]: per-reaction log rate multipliers, RKI = rki * exp(log_k);
* ``emis`` [ischan, ncell]: an emission tendency (ppm/min) added to f(y).

Gradients come back for ``y0``, ``log_k`` and ``emis``.  The adjoint is that of the
steps the forward pass took (accepted step sizes held fixed); it differs from the
derivative of the adaptive integrator by the step-size sensitivity, which is of the
order of the error tolerance.  The reference's own sensitivity tool is the forward
DDM-3D (CCTM/src/ddm3d/DDM3D_CHEM.F), which propagates one parameter at a time.

Species are in the solver's order (``ChemSolver.inew2old`` maps them back), as for
``ChemSolver.solve``.
"""
from __future__ import annotations

import ctypes as C

import torch

from ._lib import ChemError, check
from .chem import ChemSolver, _ptr


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Ros3Window:
    """The inputs of one differentiable chemistry window that are not differentiated:
    the solver handle, rate constants rki [nrxns, n] (or [nsync, nrxns, n], one plane per
    synchronisation step) and the night flags [n] (uint8, night reaction list)."""

    def __init__(self, solver: ChemSolver, rki, night, nsync: int, chemstep: float = 5.0, tape_bytes=None):
        """tape_bytes: device memory for the tape the forward pass records (None: up to half
        the free memory, sized for about 16 accepted steps per cell and step; 0: no tape,
        the backward pass re-runs every step from its checkpoint)."""
        if rki.dtype != torch.float64 or night.dtype != torch.uint8:
            raise ChemError("rki must be float64 and night uint8")
        if rki.dim() not in (2, 3) or not rki.is_contiguous():
            raise ChemError("rki must be a contiguous [nrxns, n] or [nsync, nrxns, n] tensor")
        if rki.dim() == 3 and rki.shape[0] != nsync:
            raise ChemError("per-step rki needs nsync planes")
        self.solver, self.rki, self.night = solver, rki, night.contiguous()
        self.nsync, self.chemstep = int(nsync), float(chemstep)
        self.n = rki.shape[-1]
        self.stride = 0 if rki.dim() == 2 else rki.shape[1] * rki.shape[2]
        if tape_bytes is None:
            free, _ = torch.cuda.mem_get_info(rki.device)
            want = self.n * self.nsync * (16 * (solver.info.ischan + 1) * 8 + 64)
            tape_bytes = min(want, free // 2)
        self.tape_bytes = int(tape_bytes)

    def __call__(self, y0, log_k=None, emis=None):
        return Ros3WindowFn.apply(y0, log_k, emis, self)


class Ros3WindowFn(torch.autograd.Function):
    """autograd node of one window: forward = cmaqchem_adj_forward (checkpoints the state
    at each synchronisation step), backward = cmaqchem_adj_backward."""

    @staticmethod
    def forward(ctx, y0, log_k, emis, w: Ros3Window):
        s = w.solver
        ischan = s.info.ischan
        if tuple(y0.shape) != (ischan, w.n) or y0.dtype != torch.float64:
            raise ChemError(f"y0 must be float64 [{ischan}, {w.n}]")
        y = y0.detach().contiguous().clone()
        kmult = None if log_k is None else torch.exp(log_k.detach().to(torch.float64)).contiguous()
        e = None if emis is None else emis.detach().to(torch.float64).contiguous()
        ck = torch.empty((w.nsync, ischan, w.n), dtype=torch.float64, device=y.device)
        nsteps = torch.empty((w.nsync, w.n), dtype=torch.int32, device=y.device)
        tape = torch.empty(w.tape_bytes, dtype=torch.uint8, device=y.device) if w.tape_bytes > 0 else None
        rc = s._L.cmaqchem_adj_forward(s._h, w.n, _ptr(y), _ptr(w.rki), w.stride, _ptr(w.night), _ptr(kmult),
                                       _ptr(e), w.nsync, w.chemstep, _ptr(ck), _ptr(nsteps), _ptr(tape),
                                       w.tape_bytes, _stream())
        check(rc, s._L)
        if rc > 0:
            raise ChemError(f"{rc} cell-steps failed in the chemistry window")
        ctx.w = w
        ctx.has_k, ctx.has_e = log_k is not None, emis is not None
        ctx.tape = tape
        ctx.save_for_backward(ck, nsteps, *(t for t in (kmult, e) if t is not None))
        return y

    @staticmethod
    def backward(ctx, gy):
        w = ctx.w
        s = w.solver
        saved = list(ctx.saved_tensors)
        ck, nsteps, rest = saved[0], saved[1], saved[2:]
        kmult = rest.pop(0) if ctx.has_k else None
        e = rest.pop(0) if ctx.has_e else None
        lam = gy.detach().to(torch.float64).contiguous().clone()
        gk = torch.zeros(s.info.nrxns, dtype=torch.float64, device=lam.device)
        ge = torch.zeros_like(e) if (e is not None and ctx.needs_input_grad[2]) else None
        rc = s._L.cmaqchem_adj_backward(s._h, w.n, _ptr(lam), _ptr(w.rki), w.stride, _ptr(w.night), _ptr(kmult),
                                        _ptr(e), w.nsync, w.chemstep, _ptr(ck), _ptr(nsteps), _ptr(ctx.tape),
                                        w.tape_bytes if ctx.tape is not None else 0, _ptr(gk), _ptr(ge), _stream())
        check(rc, s._L)
        ctx.tape = None
        return (lam if ctx.needs_input_grad[0] else None,
                gk if ctx.has_k and ctx.needs_input_grad[1] else None,
                ge, None)


def ros3_window(solver: ChemSolver, y0, rki, night, nsync: int, chemstep: float = 5.0, log_k=None, emis=None,
                tape_bytes=None):
    """y at the end of ``nsync`` synchronisation steps; differentiable in y0, log_k, emis."""
    return Ros3Window(solver, rki, night, nsync, chemstep, tape_bytes)(y0, log_k, emis)
