"""ctypes binding of the C-ABI in include/fvm.h.

This is the Python face of the same entry points a Fortran driver binds through
ISO_C_BINDING.  The CUDA library must be present: loading raises if it is not
(there is no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

FVM_OK, FVM_ERR_ARG, FVM_ERR_CUDA, FVM_ERR_NOCONV, FVM_ERR_TIMEOUT, FVM_ERR_NAN, FVM_ERR_NOMEM = range(7)
FP64, MIXED = 0, 1
FIELD_U, FIELD_V, FIELD_T = 0, 1, 2

STATUS_NAMES = {0: "FVM_OK", 1: "FVM_ERR_ARG", 2: "FVM_ERR_CUDA", 3: "FVM_ERR_NOCONV",
                4: "FVM_ERR_TIMEOUT", 5: "FVM_ERR_NAN", 6: "FVM_ERR_NOMEM"}

# Every symbol include/fvm.h declares (checked by the CPU tests).
EXPORTS = ["fvm_default_params", "fvm_create", "fvm_destroy", "fvm_last_error", "fvm_set_grid",
           "fvm_init", "fvm_upload_state", "fvm_download_state", "fvm_get_array", "fvm_set_array",
           "fvm_set_time", "fvm_set_controls", "fvm_adjoint_drag_grad", "fvm_adjoint_vjp", "fvm_begin_step", "fvm_contra_vel", "fvm_nl", "fvm_dif", "fvm_p_source",
           "fvm_iter_u", "fvm_iter_v", "fvm_remove_grad", "fvm_iter_p", "fvm_correct", "fvm_iter_t",
           "fvm_calccoef", "fvm_step", "fvm_history", "fvm_synchronize", "fvm_get_stream",
           "fvm_timing_reset", "fvm_get_timing", "fvm_time_sweeps", "fvm_resident_wait_test",
           "fvm_resident_info",
           "fvm_poisson_residual_static",
           "fvm_batch_create", "fvm_batch_destroy", "fvm_batch_last_error", "fvm_batch_case",
           "fvm_batch_tiles", "fvm_batch_set_tiles", "fvm_batch_autotune", "fvm_batch_time_sweeps",
           "fvm_batch_step", "fvm_batch_get_timing", "fvm_post_begin", "fvm_post_get", "fvm_post_final",
           "fvm_post_end", "fvm_calc_vor"]


class Params(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int),
                ("re", ctypes.c_double), ("pr", ctypes.c_double), ("dt", ctypes.c_double),
                ("vel_rot", ctypes.c_double), ("uin", ctypes.c_double), ("vin", ctypes.c_double),
                ("tin", ctypes.c_double), ("t_wall", ctypes.c_double), ("resimax", ctypes.c_double),
                ("nswpp", ctypes.c_int), ("precision", ctypes.c_int), ("thermal", ctypes.c_int),
                ("iter_t_bug", ctypes.c_int), ("res_every", ctypes.c_int),
                ("refine_sweeps", ctypes.c_int), ("adi_refine", ctypes.c_int), ("device", ctypes.c_int),
                ("poisson_groups", ctypes.c_int), ("poisson_host_loop", ctypes.c_int),
                ("dd_positional", ctypes.c_int),
                ("tile_r_warps", ctypes.c_int), ("tile_r_m", ctypes.c_int),
                ("tile_t_warps", ctypes.c_int), ("tile_t_m", ctypes.c_int),
                ("poisson_resident", ctypes.c_int), ("resident_depth", ctypes.c_int)]


class Coeffs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "cfl", "cpb", "cd", "cl", "cd_p", "cd_v", "cl_p", "cl_v", "nu")] + \
               [("sweeps", ctypes.c_int), ("resid", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Post(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "nu", "cd", "cl", "cl_amp", "cpb", "st", "rms_cd", "rms_cl", "st_last", "cl_amp_last")] + \
               [("niter", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Timing(ctypes.Structure):
    _fields_ = [("sweep_span_ms", ctypes.c_double), ("sweep_span_launches", ctypes.c_longlong),
                ("kernel_launches", ctypes.c_longlong), ("sweeps", ctypes.c_longlong),
                ("steps", ctypes.c_longlong)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class FvmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libfvm_gb300.so (building it in-tree first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise ImportError(f"CUDA library {path} is missing; run fvm_gb300.build.build()")
        _build.build()
    L = ctypes.CDLL(path)
    D = ctypes.POINTER(ctypes.c_double)
    V = ctypes.c_void_p
    L.fvm_default_params.argtypes = [ctypes.POINTER(Params)]
    L.fvm_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(V)]
    L.fvm_destroy.argtypes = [V]
    L.fvm_last_error.argtypes = [V]
    L.fvm_last_error.restype = ctypes.c_char_p
    L.fvm_set_grid.argtypes = [V, D, D]
    L.fvm_init.argtypes = [V, D, D]
    L.fvm_upload_state.argtypes = [V] + [D] * 7
    L.fvm_download_state.argtypes = [V] + [D] * 7
    L.fvm_get_array.argtypes = [V, ctypes.c_char_p, D]
    L.fvm_set_array.argtypes = [V, ctypes.c_char_p, D]
    L.fvm_set_time.argtypes = [V, ctypes.c_double, ctypes.c_int]
    L.fvm_set_controls.argtypes = [V, ctypes.c_double, D]
    L.fvm_adjoint_drag_grad.argtypes = [V, ctypes.c_int, ctypes.c_int, D, D, D]
    for f in ("fvm_post_begin", "fvm_post_end", "fvm_calc_vor"):
        getattr(L, f).argtypes = [V]
    L.fvm_post_get.argtypes = [V, ctypes.POINTER(Post)]
    L.fvm_post_final.argtypes = [V, ctypes.POINTER(Post), D, D, D, D, D]
    L.fvm_adjoint_vjp.argtypes = [V, D, D, D, D, D, D]
    for f in ("fvm_begin_step", "fvm_contra_vel", "fvm_p_source", "fvm_iter_u", "fvm_iter_v",
              "fvm_remove_grad", "fvm_correct", "fvm_iter_t", "fvm_synchronize"):
        getattr(L, f).argtypes = [V]
    L.fvm_nl.argtypes = [V, ctypes.c_int]
    L.fvm_dif.argtypes = [V, ctypes.c_int]
    L.fvm_iter_p.argtypes = [V, D, ctypes.POINTER(ctypes.c_int)]
    L.fvm_calccoef.argtypes = [V, ctypes.POINTER(Coeffs)]
    L.fvm_step.argtypes = [V, ctypes.c_int, ctypes.POINTER(Coeffs)]
    L.fvm_history.argtypes = [V, ctypes.POINTER(Coeffs), ctypes.c_int]
    L.fvm_get_stream.argtypes = [V, ctypes.POINTER(ctypes.c_void_p)]
    L.fvm_timing_reset.argtypes = [V]
    L.fvm_get_timing.argtypes = [V, ctypes.POINTER(Timing)]
    L.fvm_time_sweeps.argtypes = [V, ctypes.c_int, D, ctypes.POINTER(ctypes.c_longlong)]
    L.fvm_resident_wait_test.argtypes = [V, ctypes.c_int]
    L.fvm_resident_info.argtypes = [V] + [ctypes.POINTER(ctypes.c_int)] * 3
    L.fvm_poisson_residual_static.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 8 + [V]
    I = ctypes.POINTER(ctypes.c_int)
    L.fvm_batch_create.argtypes = [ctypes.c_int, ctypes.POINTER(Params), ctypes.POINTER(V)]
    L.fvm_batch_destroy.argtypes = [V]
    L.fvm_batch_last_error.argtypes = [V]
    L.fvm_batch_last_error.restype = ctypes.c_char_p
    L.fvm_batch_case.argtypes = [V, ctypes.c_int, ctypes.POINTER(V)]
    L.fvm_batch_tiles.argtypes = [V, I]
    L.fvm_batch_set_tiles.argtypes = [V, I]
    L.fvm_batch_autotune.argtypes = [V, ctypes.c_int, I, D]
    L.fvm_batch_time_sweeps.argtypes = [V, ctypes.c_int, D]
    L.fvm_batch_step.argtypes = [V, ctypes.c_int, ctypes.POINTER(Coeffs)]
    L.fvm_batch_get_timing.argtypes = [V, ctypes.POINTER(Timing)]
    _lib = L
    return L


def default_params(**kw) -> Params:
    p = Params()
    load().fvm_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _arr(a, n):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float64).ravel()
    if a.size != n:
        raise ValueError(f"array has {a.size} elements, expected {n}")
    return a


class Context:
    """One solver context (one CUDA stream on one GPU).  Field arrays are numpy
    arrays shaped (NJ+1, NI+1): a[j, i] is the reference's (I, J)."""

    def __init__(self, params: Params, _handle=None, _owner=None):
        self.L = load()
        self.p = params
        self.ni, self.nj = params.ni, params.nj
        self.n = (self.ni + 1) * (self.nj + 1)
        self._owner = _owner          # a Batch owns the contexts of its cases
        if _handle is not None:
            self.h = _handle
            return
        h = ctypes.c_void_p()
        rc = self.L.fvm_create(ctypes.byref(params), ctypes.byref(h))
        if rc != FVM_OK:
            raise FvmError(rc, "fvm_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self._owner is None:
            self.L.fvm_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, allow=()):
        if rc != FVM_OK and rc not in allow:
            raise FvmError(rc, self.L.fvm_last_error(self.h).decode())
        return rc

    def last_error(self) -> str:
        return self.L.fvm_last_error(self.h).decode()

    # set-up ------------------------------------------------------------------
    def set_grid(self, xg, yg):
        x, y = _arr(xg, self.n), _arr(yg, self.n)
        self._ok(self.L.fvm_set_grid(self.h, _dp(x), _dp(y)))

    def init(self, du=None, dv=None):
        a, b = _arr(du, self.n), _arr(dv, self.n)
        self._ok(self.L.fvm_init(self.h, _dp(a), _dp(b)))

    # state -------------------------------------------------------------------
    def upload(self, u=None, v=None, p=None, t=None, nlx=None, nly=None, adv=None):
        arrs = [_arr(a, self.n) for a in (u, v, p, t, nlx, nly, adv)]
        self._ok(self.L.fvm_upload_state(self.h, *[_dp(a) for a in arrs]))

    def download(self, names=("U", "V", "P", "T")):
        return {nm: self.get(nm) for nm in names}

    def get(self, name) -> np.ndarray:
        out = np.empty(self.n)
        self._ok(self.L.fvm_get_array(self.h, name.encode(), _dp(out)))
        return out.reshape(self.nj + 1, self.ni + 1)

    def set(self, name, a):
        a = _arr(a, self.n)
        self._ok(self.L.fvm_set_array(self.h, name.encode(), _dp(a)))

    def set_time(self, t, niter=0):
        self._ok(self.L.fvm_set_time(self.h, t, niter))

    def set_controls(self, omega=0.0, blow=None):
        """Wall rotation rate and wall-normal blowing speeds (NJ-1 values)."""
        b = None if blow is None else _arr(blow, self.nj - 1)
        self._ok(self.L.fvm_set_controls(self.h, omega, _dp(b)))

    def post_begin(self):
        """POST_PROCESS with IPOST=0: time averaging from the next step on."""
        self._ok(self.L.fvm_post_begin(self.h))

    def post_get(self) -> dict:
        """The POST_NU_CD_CL.PLT record of the last step."""
        r = Post()
        self._ok(self.L.fvm_post_get(self.h, ctypes.byref(r)))
        return r.as_dict()

    def post_final(self):
        """POST_PROCESS with IPOST=1: averaged coefficients and fields (the state
        is left unchanged)."""
        r = Post()
        f = {nm: np.zeros((self.nj + 1, self.ni + 1)) for nm in ("U", "V", "P", "T", "VOR")}
        self._ok(self.L.fvm_post_final(self.h, ctypes.byref(r), *[_dp(f[nm]) for nm in ("U", "V", "P", "T", "VOR")]))
        return r.as_dict(), f

    def post_end(self):
        self._ok(self.L.fvm_post_end(self.h))

    def calc_vor(self) -> np.ndarray:
        """CALC_VOR of the current state."""
        self._ok(self.L.fvm_calc_vor(self.h))
        return self.get("VOR")

    def adjoint_drag_grad(self, window, ckpt=50):
        """Runs `window` steps from the current state; returns (J, dJ/domega,
        dJ/dblow) with J the mean drag coefficient over the window."""
        J = ctypes.c_double()
        dw = ctypes.c_double()
        db = np.zeros(self.nj - 1)
        self._ok(self.L.fvm_adjoint_drag_grad(self.h, window, ckpt, ctypes.byref(J), ctypes.byref(dw), _dp(db)),
                 allow=(FVM_ERR_NOCONV,))
        return J.value, dw.value, db

    def adjoint_vjp(self, lam):
        """One step transposed at the current state: lam maps U, V, P, NLX, NLY to
        adjoints of the state after the step (arrays shaped like get()); returns the
        adjoints of the state before it and the control adjoints (rotation, blowing)."""
        names = ("U", "V", "P", "NLX", "NLY")
        arrs = [np.ascontiguousarray(lam[nm], dtype=np.float64).ravel().copy() for nm in names]
        ctrl = np.zeros(self.nj)
        self._ok(self.L.fvm_adjoint_vjp(self.h, *[_dp(a) for a in arrs], _dp(ctrl)))
        out = {nm: a.reshape(self.nj + 1, self.ni + 1) for nm, a in zip(names, arrs)}
        return out, ctrl[0], ctrl[1:]

    # reference call points -----------------------------------------------------
    def begin_step(self): self._ok(self.L.fvm_begin_step(self.h))
    def contra_vel(self): self._ok(self.L.fvm_contra_vel(self.h))
    def nl(self, field): self._ok(self.L.fvm_nl(self.h, field))
    def dif(self, field): self._ok(self.L.fvm_dif(self.h, field))
    def p_source(self): self._ok(self.L.fvm_p_source(self.h))
    def iter_u(self): self._ok(self.L.fvm_iter_u(self.h))
    def iter_v(self): self._ok(self.L.fvm_iter_v(self.h))
    def remove_grad(self): self._ok(self.L.fvm_remove_grad(self.h))
    def correct(self): self._ok(self.L.fvm_correct(self.h))
    def iter_t(self): self._ok(self.L.fvm_iter_t(self.h))

    def iter_p(self):
        r = ctypes.c_double()
        s = ctypes.c_int()
        rc = self._ok(self.L.fvm_iter_p(self.h, ctypes.byref(r), ctypes.byref(s)), allow=(FVM_ERR_NOCONV,))
        return r.value, s.value, rc

    def calccoef(self) -> dict:
        c = Coeffs()
        self._ok(self.L.fvm_calccoef(self.h, ctypes.byref(c)))
        return c.as_dict()

    def step(self, n=1) -> dict:
        c = Coeffs()
        self._ok(self.L.fvm_step(self.h, n, ctypes.byref(c)), allow=(FVM_ERR_NOCONV,))
        return c.as_dict()

    def history(self, n):
        arr = (Coeffs * n)()
        self._ok(self.L.fvm_history(self.h, arr, n))
        return [a.as_dict() for a in arr]

    def synchronize(self):
        self._ok(self.L.fvm_synchronize(self.h))

    # instrumentation -----------------------------------------------------------
    def stream_handle(self) -> int:
        s = ctypes.c_void_p()
        self._ok(self.L.fvm_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def timing_reset(self):
        self._ok(self.L.fvm_timing_reset(self.h))

    def time_sweeps(self, sweeps=200):
        ms = ctypes.c_double()
        n = ctypes.c_longlong()
        self._ok(self.L.fvm_time_sweeps(self.h, sweeps, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def resident_wait_test(self, max_polls=4096) -> int:
        """fvm_resident_wait_test: status code (FVM_ERR_TIMEOUT when the bounded
        waits of the resident sweeps reported running out)."""
        return self.L.fvm_resident_wait_test(self.h, max_polls)

    def resident_info(self) -> dict:
        """fvm_resident_info: lines per block (0: per-colour path), blocks and sweeps
        per boundary-line exchange of the resident Poisson sweeps."""
        v = [ctypes.c_int() for _ in range(3)]
        self._ok(self.L.fvm_resident_info(self.h, *[ctypes.byref(x) for x in v]))
        return {"lines_per_block": v[0].value, "blocks": v[1].value, "sweeps_per_exchange": v[2].value}

    def timing(self) -> dict:
        t = Timing()
        self._ok(self.L.fvm_get_timing(self.h, ctypes.byref(t)))
        return t.as_dict()

    def upload_ptrs(self, ptrs):
        """fvm_upload_state from raw host addresses (e.g. pinned buffers)."""
        P = ctypes.POINTER(ctypes.c_double)
        args = [ctypes.cast(p, P) if p else None for p in ptrs]
        self._ok(self.L.fvm_upload_state(self.h, *args))

    def download_ptrs(self, ptrs):
        P = ctypes.POINTER(ctypes.c_double)
        args = [ctypes.cast(p, P) if p else None for p in ptrs]
        self._ok(self.L.fvm_download_state(self.h, *args))


class Batch:
    """Independent cases advanced together (fvm_batch_*).  cases[k] is the
    Context of case k (owned by the batch): set its grid and initial state with the
    Context methods, then step the batch."""

    def __init__(self, params_list):
        self.L = load()
        self.params = list(params_list)
        arr = (Params * len(self.params))(*self.params)
        h = ctypes.c_void_p()
        rc = self.L.fvm_batch_create(len(self.params), arr, ctypes.byref(h))
        if rc != FVM_OK:
            raise FvmError(rc, "fvm_batch_create failed (run options and tiles must agree across cases)")
        self.h = h
        self.cases = []
        for k, p in enumerate(self.params):
            ch = ctypes.c_void_p()
            self._ok(self.L.fvm_batch_case(self.h, k, ctypes.byref(ch)))
            q = Params()
            ctypes.pointer(q)[0] = p
            self.cases.append(Context(q, _handle=ch, _owner=self))

    def __len__(self):
        return len(self.cases)

    def close(self):
        if getattr(self, "h", None):
            for c in self.cases:
                c.h = None
            self.L.fvm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, allow=()):
        if rc != FVM_OK and rc not in allow:
            raise FvmError(rc, self.L.fvm_batch_last_error(self.h).decode())
        return rc

    def tiles(self):
        t = (ctypes.c_int * 4)()
        self._ok(self.L.fvm_batch_tiles(self.h, t))
        return tuple(t)

    def set_tiles(self, tiles):
        t = (ctypes.c_int * 4)(*tiles)
        self._ok(self.L.fvm_batch_set_tiles(self.h, t))

    def autotune(self, sweeps=50):
        """Times the candidate line tiles on this batch and keeps the fastest;
        returns (tiles, ms per sweep of the radial and circumferential families)."""
        t = (ctypes.c_int * 4)()
        ms = (ctypes.c_double * 2)()
        self._ok(self.L.fvm_batch_autotune(self.h, sweeps, t, ms))
        return tuple(t), (ms[0], ms[1])

    def time_sweeps(self, sweeps=100):
        ms = ctypes.c_double()
        self._ok(self.L.fvm_batch_time_sweeps(self.h, sweeps, ctypes.byref(ms)))
        return ms.value

    def step(self, n=1):
        """n steps of every case; returns records[s][k] (dicts)."""
        k = len(self.cases)
        arr = (Coeffs * (n * k))()
        self._ok(self.L.fvm_batch_step(self.h, n, arr), allow=(FVM_ERR_NOCONV,))
        return [[arr[s * k + j].as_dict() for j in range(k)] for s in range(n)]

    def resident_wait_test(self, max_polls=4096) -> int:
        """fvm_resident_wait_test: status code (FVM_ERR_TIMEOUT when the bounded
        waits of the resident sweeps reported running out)."""
        return self.L.fvm_resident_wait_test(self.h, max_polls)

    def timing(self) -> dict:
        t = Timing()
        self._ok(self.L.fvm_batch_get_timing(self.h, ctypes.byref(t)))
        return t.as_dict()
