"""GPU test of the allocation-free residual entry point.

Some callers cannot allocate device memory (a stream being captured into a CUDA
graph, or a program whose device memory is owned by a pool allocator);
fvm_poisson_residual_static serves them with a fixed static scratch array.  This
test calls it through the C-ABI on device arrays prepared outside the library and
checks it against an FP64 numpy evaluation of the same arrays and against the
residual the solver context reports for the same pressure field (the existing
fvm_step entry point), twice in a row so that the shared scratch is reused.  It
runs last and needs nothing from the other tests.
"""
import ctypes

import numpy as np
import pytest

from fvm_gb300 import capi
from tests.helpers import make_case, make_gpu

pytestmark = pytest.mark.gpu


def _poisson_system(ctx, g):
    """Coefficients of the pressure equation with the wall/far-field folding
    (iter_p.f90:12-17, bcp.f90:16-26) and SU = DIV/dt - DD(P) (iter_p.f90:24-30),
    DD paired by position
    for the context's current pressure."""
    get = ctx.get
    DE, DW, DN, DS = get("DE"), get("DW"), get("DN"), get("DS")
    AP = ((-DE) - DW - DN) - DS
    AE, AW, AN, AS = -DE, -DW, -DN, -DS
    AP[:, 1] = AP[:, 1] - AW[:, 1]
    AW[:, 1] = 0.0
    AE[:, g.ni - 1] = 0.0
    K = get("DJAC") * get("Q12")
    P = get("P")
    ni, nj = g.ni, g.nj
    SU = np.zeros_like(P)
    i = np.arange(1, ni)[None, :]
    j = np.arange(1, nj)[:, None]
    ke, kw, kn, ks = K[j, i + 1], K[j, i - 1], K[j + 1, i], K[j - 1, i]
    dd = ((0.25 * (ke + kn)) * P[j + 1, i + 1] + (-(0.25 * (ke + ks))) * P[j - 1, i + 1]
          + (-(0.25 * (kw + kn))) * P[j + 1, i - 1] + (0.25 * (kw + ks)) * P[j - 1, i - 1])
    # cell (I,J) takes the cross term of cell (I-1,J-1), zero on row/column 1
    # (the positional whole-array DD of iter_p.f90:27-30)
    dds = np.zeros_like(dd)
    dds[1:, 1:] = dd[:-1, :-1]
    SU[1:nj, 1:ni] = get("DIVDT")[1:nj, 1:ni] - dds
    return P, SU, AP, AE, AW, AN, AS


def test_static_residual_matches_the_step_residual():
    torch = pytest.importorskip("torch")
    # A capped (unconverged) Poisson solve keeps the residual well above rounding.
    # The FP64 evaluation of the same arrays agrees to the suites' FP64 tolerance;
    # the context's own norm (double-float residual, FP32 sums within a warp) to 1e-5.
    case = make_case(32, 24, skew=0.3, resimax=1e-14, nswpp=4)
    g = case["g"]
    ctx = make_gpu(case, precision=capi.MIXED, refine_sweeps=4)
    ctx.step(1)
    step_resid = ctx.step(1)["resid"]
    system = _poisson_system(ctx, g)
    ref = _numpy_residual(*system, g.ni, g.nj)
    assert abs(step_resid - ref) <= 1e-5 * ref, (step_resid, ref)
    arrays = [torch.tensor(np.ascontiguousarray(a).ravel(), dtype=torch.float64, device="cuda")
              for a in system]
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    L = capi.load()
    ptrs = [ctypes.c_void_p(a.data_ptr()) for a in arrays]
    for k in range(2):
        rc = L.fvm_poisson_residual_static(g.ni, g.nj, *ptrs, ctypes.c_void_p(out[k:].data_ptr()), None)
        assert rc == capi.FVM_OK
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert np.all(np.isfinite(got))
    assert abs(got[0] - ref) <= 1e-12 * abs(ref), (got, ref)
    assert abs(got[1] - ref) <= 1e-12 * abs(ref), (got, ref)


def _numpy_residual(P, SU, AP, AE, AW, AN, AS, ni, nj):
    """sum|r| / sum|AP*P| over the interior in float64, circumferential neighbours
    through the periodic branch cut (the entry point's documented formula)."""
    i = np.arange(1, ni)[None, :]
    j = np.arange(1, nj)[:, None]
    jn = np.where(j == nj - 1, 1, j + 1)
    js = np.where(j == 1, nj - 1, j - 1)
    r = ((((AE[j, i] * P[j, i + 1] + AW[j, i] * P[j, i - 1]) + AN[j, i] * P[jn, i]) + AS[j, i] * P[js, i])
         + SU[j, i]) - AP[j, i] * P[j, i]
    return np.abs(r).sum() / np.abs(AP[j, i] * P[j, i]).sum()


def test_static_residual_at_the_size_limit():
    """1024 x 1024 interior cells, the largest grid accepted: every one of the 2048
    scratch slots and the arrival ticket behind them are in use."""
    torch = pytest.importorskip("torch")
    ni = nj = 1025
    rng = np.random.default_rng(7)
    arrays = [rng.uniform(-1.0, 1.0, size=(nj + 1, ni + 1)) for _ in range(7)]
    arrays[2] = arrays[2] + 4.0   # AP dominant, as in the pressure equation
    want = _numpy_residual(*arrays, ni, nj)
    dev = [torch.tensor(a.ravel(), dtype=torch.float64, device="cuda") for a in arrays]
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    L = capi.load()
    ptrs = [ctypes.c_void_p(a.data_ptr()) for a in dev]
    for k in range(2):
        rc = L.fvm_poisson_residual_static(ni, nj, *ptrs, ctypes.c_void_p(out[k:].data_ptr()), None)
        assert rc == capi.FVM_OK
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    assert abs(got[0] - want) <= 1e-12 * want, (got, want)
    assert abs(got[1] - want) <= 1e-12 * want, (got, want)


def test_static_residual_rejects_oversized_grids():
    # Null pointers throughout: the size check must refuse these before any
    # pointer is used, so a broken check can never reach a kernel launch.
    L = capi.load()
    null = [None] * 8
    assert L.fvm_poisson_residual_static(1025, 1026, *null, None) == capi.FVM_ERR_ARG   # one row too many
    assert L.fvm_poisson_residual_static(2000, 2000, *null, None) == capi.FVM_ERR_ARG
    assert L.fvm_poisson_residual_static(97, 129, *null, None) == capi.FVM_ERR_ARG
