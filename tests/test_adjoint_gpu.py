"""Discrete adjoint of the time step (fvm_adjoint_*).

1. One step transposed, checked by the dot-product identity against central
   differences of the GPU step: with the Poisson equation converged the step is a
   quadratic map of (state, controls), so the central difference is exact up to
   rounding and the convergence tolerance.
2. The window gradient d(mean Cd)/d(rotation, blowing) against central finite
   differences (h = 1e-6) of the FP64 oracle run from the same state, at the
   1e-5 relative bar, with checkpointed recomputation over several segments.
3. The torch.autograd binding returns the same gradient."""
import numpy as np
import pytest

import oracle
from fvm_gb300 import capi
from tests.helpers import copy_oracle_state_to_gpu, make_case, make_gpu, make_oracle

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _case(**kw):
    base = dict(n_theta=32, n_r=24, re=100.0, dt=0.005, skew=0.25, resimax=TOL, nswpp=200000, vel_rot=0.2)
    base.update(kw)
    return make_case(**base)


def _state(ctx):
    return {nm: ctx.get(nm) for nm in ("U", "V", "P", "T", "NLX", "NLY", "ADV")}


def _upload(ctx, s):
    ctx.upload(s["U"], s["V"], s["P"], s["T"], s["NLX"], s["NLY"], s["ADV"])


def test_one_step_transpose_dot_product():
    case = _case()
    ctx = make_gpu(case, capi.FP64)
    rng = np.random.default_rng(5)
    nj1 = case["g"].nj - 1
    blow0 = 0.02 * rng.standard_normal(nj1)
    ctx.set_controls(0.2, blow0)
    ctx.step(3)
    x0 = _state(ctx)
    shape = x0["U"].shape
    # direction in state and controls, adjoint weights of the outputs
    v = {nm: rng.standard_normal(shape) for nm in ("U", "V", "P", "NLX", "NLY")}
    for nm in ("NLX", "NLY"):      # NL arrays are interior quantities
        v[nm][0, :] = v[nm][-1, :] = 0.0
        v[nm][:, 0] = v[nm][:, -1] = 0.0
    vw, vb = rng.standard_normal(), rng.standard_normal(nj1)
    lam = {nm: rng.standard_normal(shape) for nm in ("U", "V", "P", "NLX", "NLY")}
    eps = 1e-4

    def step_from(sign):
        s = dict(x0)
        for nm in v:
            s[nm] = x0[nm] + sign * eps * v[nm]
        _upload(ctx, s)
        ctx.set_controls(0.2 + sign * eps * vw, blow0 + sign * eps * vb)
        ctx.step(1)
        return {nm: ctx.get(nm) for nm in lam}

    fp, fm = step_from(+1), step_from(-1)
    lhs = sum(float(np.sum(lam[nm] * (fp[nm] - fm[nm]))) for nm in lam) / (2 * eps)
    _upload(ctx, x0)
    ctx.set_controls(0.2, blow0)
    adj, dw, db = ctx.adjoint_vjp(lam)
    rhs = sum(float(np.sum(adj[nm] * v[nm])) for nm in v) + dw * vw + float(np.dot(db, vb))
    assert abs(lhs - rhs) <= 1e-7 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def _oracle_window_cd(o, start, omega, blow, window):
    o.restore_state(start)
    o.set_controls(omega, blow)
    cds = []
    for _ in range(window):
        o.step(1)
        cds.append(o.coeffs()["cd"])
    return float(np.mean(cds))


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED], ids=["fp64", "mixed"])
def test_window_gradient_matches_oracle_finite_differences(precision):
    case = _case()
    nj1 = case["g"].nj - 1
    rng = np.random.default_rng(11)
    omega = 0.2
    blow = 0.01 * rng.standard_normal(nj1)
    # spin-up on the oracle (GPU order, FP64); the window starts from its state
    o = make_oracle(case, order=oracle.GPU, res_every=1)
    o.set_controls(omega, blow)
    o.step(4)
    start = o.save_state()
    ctx = make_gpu(case, precision, refine_sweeps=8)
    copy_oracle_state_to_gpu(o, ctx)
    ctx.set_controls(omega, blow)
    window, ckpt = 6, 4
    J, dw, db = ctx.adjoint_drag_grad(window, ckpt)
    J0 = _oracle_window_cd(o, start, omega, blow, window)
    assert abs(J - J0) <= (1e-9 if precision == capi.FP64 else 1e-5) * abs(J0)
    h = 1e-6
    fd_w = (_oracle_window_cd(o, start, omega + h, blow, window)
            - _oracle_window_cd(o, start, omega - h, blow, window)) / (2 * h)
    tol = 1e-5 if precision == capi.FP64 else 1e-4
    assert abs(dw - fd_w) <= tol * abs(fd_w), (dw, fd_w)
    for j in (0, nj1 // 3, nj1 // 2, nj1 - 1):
        e = np.zeros(nj1)
        e[j] = h
        fd = (_oracle_window_cd(o, start, omega, blow + e, window)
              - _oracle_window_cd(o, start, omega, blow - e, window)) / (2 * h)
        scale = max(abs(fd), 1e-3 * np.max(np.abs(db)))
        assert abs(db[j] - fd) <= tol * scale, (j, db[j], fd)


def test_autograd_binding():
    torch = pytest.importorskip("torch")
    from fvm_gb300.autograd import window_drag
    case = _case(resimax=1e-12)
    nj1 = case["g"].nj - 1
    ctx = make_gpu(case, capi.FP64)
    ctx.step(3)
    omega = torch.tensor(0.1, dtype=torch.float64, requires_grad=True)
    blow = torch.zeros(nj1, dtype=torch.float64, requires_grad=True)
    J = window_drag(omega, blow, ctx, window=4, ckpt=2)
    J.backward()
    ctx2 = make_gpu(case, capi.FP64)
    ctx2.step(3)
    ctx2.set_controls(0.1, np.zeros(nj1))
    J2, dw2, db2 = ctx2.adjoint_drag_grad(4, 2)
    assert J.item() == pytest.approx(J2, rel=1e-12)
    assert omega.grad.item() == pytest.approx(dw2, rel=1e-10)
    assert np.allclose(blow.grad.numpy(), db2, rtol=1e-10, atol=1e-14)
    # the start state is kept: a second evaluation gives the same value
    J3 = window_drag(omega.detach(), blow.detach(), ctx, window=4, ckpt=2)
    assert J3.item() == pytest.approx(J.item(), rel=1e-12)
