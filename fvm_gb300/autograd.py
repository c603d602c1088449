"""torch.autograd binding of the discrete adjoint: the mean drag coefficient over
a window of time steps as a differentiable function of the wall rotation rate and
the wall-normal blowing speeds.

    J = window_drag(omega, blow, solver, window, ckpt)

solver is a capi.Context whose current state is the start of the window (for
example after a spin-up); every evaluation starts from that state (it is saved on
first use and restored before each call) and leaves it unchanged.  The forward
call runs fvm_adjoint_drag_grad, which returns J and its gradient together; the
backward pass scales the stored gradient.  Tensors are FP64 on the CPU."""
from __future__ import annotations

import numpy as np
import torch

_STATE = ("U", "V", "P", "T", "NLX", "NLY", "ADV")


class _Start:
    """The state of a context at the start of the window (host copy)."""

    def __init__(self, solver):
        self.arrays = {nm: solver.get(nm).copy() for nm in _STATE}

    def restore(self, solver):
        a = self.arrays
        solver.upload(a["U"], a["V"], a["P"], a["T"], a["NLX"], a["NLY"], a["ADV"])


class WindowDrag(torch.autograd.Function):
    @staticmethod
    def forward(ctx, omega, blow, solver, window, ckpt, start):
        start.restore(solver)
        solver.set_controls(float(omega.item()), blow.detach().cpu().numpy().astype(np.float64))
        J, dw, db = solver.adjoint_drag_grad(window, ckpt)
        start.restore(solver)
        ctx.save_for_backward(torch.tensor(dw, dtype=torch.float64), torch.from_numpy(db.copy()))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        dw, db = ctx.saved_tensors
        return grad * dw, grad * db, None, None, None, None


def window_drag(omega, blow, solver, window, ckpt=50, start=None):
    """Mean drag coefficient over `window` steps from the solver's current state,
    differentiable in omega (0-d tensor) and blow (NJ-1 tensor)."""
    if start is None:
        start = getattr(solver, "_window_start", None)
        if start is None:
            start = _Start(solver)
            solver._window_start = start
    return WindowDrag.apply(omega, blow, solver, window, ckpt, start)
