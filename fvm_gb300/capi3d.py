"""ctypes binding of the 3-D LES C-ABI (include/fvm3d.h).  Field arrays are numpy
arrays shaped (NK+1, NJ+1, NI+1): a[k, j, i] is the reference's (I, J, K)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import capi

ROUTINES = ["fvm3_begin_step", "fvm3_contra_vel", "fvm3_nl", "fvm3_stress_tensor", "fvm3_dif", "fvm3_p_source",
            "fvm3_remove_grad", "fvm3_correct", "fvm3_iter_t"]
EXPORTS = ["fvm3_default_params", "fvm3_create", "fvm3_destroy", "fvm3_last_error", "fvm3_set_grid", "fvm3_init",
           "fvm3_step", "fvm3_get_array", "fvm3_set_array", "fvm3_upload_state", "fvm3_download_state",
           "fvm3_sgs", "fvm3_time_sweeps", "fvm3_get_stream",
           "fvm3_iter_u", "fvm3_iter_p", "fvm3_calccoef", "fvm3_test_filter", "fvm3_post_begin", "fvm3_post_get",
           "fvm3_post_steps", "fvm3_post_end"] + ROUTINES


class Params3(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("re", ctypes.c_double), ("pr", ctypes.c_double), ("dt", ctypes.c_double),
                ("tin", ctypes.c_double), ("t_wall", ctypes.c_double), ("resimax", ctypes.c_double),
                ("nswpp", ctypes.c_int), ("use_les", ctypes.c_int), ("les_zavg", ctypes.c_int),
                ("thermal", ctypes.c_int), ("res_every", ctypes.c_int), ("ref_a", ctypes.c_double),
                ("precision", ctypes.c_int), ("refine_sweeps", ctypes.c_int), ("device", ctypes.c_int),
                ("tile_i_warps", ctypes.c_int), ("tile_i_m", ctypes.c_int), ("poisson_host_loop", ctypes.c_int)]


class Coeffs3(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "cfl", "cpb", "cd", "cl", "cd_p", "cd_v", "cl_p", "cl_v", "nu", "cs2", "ct2")] + \
               [("sweeps", ctypes.c_int), ("resid", ctypes.c_double)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


_ready = False


def load():
    global _ready
    L = capi.load()
    if not _ready:
        D = ctypes.POINTER(ctypes.c_double)
        V = ctypes.c_void_p
        L.fvm3_default_params.argtypes = [ctypes.POINTER(Params3)]
        L.fvm3_create.argtypes = [ctypes.POINTER(Params3), ctypes.POINTER(V)]
        L.fvm3_destroy.argtypes = [V]
        L.fvm3_last_error.argtypes = [V]
        L.fvm3_last_error.restype = ctypes.c_char_p
        L.fvm3_set_grid.argtypes = [V, D, D, D]
        L.fvm3_init.argtypes = [V, D, D, D]
        L.fvm3_step.argtypes = [V, ctypes.c_int, ctypes.POINTER(Coeffs3)]
        L.fvm3_get_array.argtypes = [V, ctypes.c_char_p, D]
        L.fvm3_set_array.argtypes = [V, ctypes.c_char_p, D]
        L.fvm3_upload_state.argtypes = [V] + [D] * 9
        L.fvm3_download_state.argtypes = [V] + [D] * 9
        L.fvm3_sgs.argtypes = [V, ctypes.POINTER(Coeffs3)]
        L.fvm3_time_sweeps.argtypes = [V, ctypes.c_int, D]
        L.fvm3_get_stream.argtypes = [V, ctypes.POINTER(V)]
        for f in ROUTINES:
            getattr(L, f).argtypes = [V]
        L.fvm3_iter_u.argtypes = [V, ctypes.c_int]
        L.fvm3_iter_p.argtypes = [V, D, ctypes.POINTER(ctypes.c_int)]
        L.fvm3_calccoef.argtypes = [V, ctypes.POINTER(Coeffs3)]
        L.fvm3_test_filter.argtypes = [V, D, D]
        L.fvm3_post_begin.argtypes = [V]
        L.fvm3_post_end.argtypes = [V]
        L.fvm3_post_steps.argtypes = [V, ctypes.POINTER(ctypes.c_int)]
        L.fvm3_post_get.argtypes = [V, ctypes.c_char_p, D]
        _ready = True
    return L


def default_params(**kw) -> Params3:
    p = Params3()
    load().fvm3_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Context3:
    """One 3-D LES solver context (one CUDA stream)."""

    def __init__(self, params: Params3):
        self.L = load()
        self.p = params
        self.ni, self.nj, self.nk = params.ni, params.nj, params.nk
        self.shape = (self.nk + 1, self.nj + 1, self.ni + 1)
        self.n = int(np.prod(self.shape))
        h = ctypes.c_void_p()
        rc = self.L.fvm3_create(ctypes.byref(params), ctypes.byref(h))
        if rc != capi.FVM_OK:
            raise capi.FvmError(rc, "fvm3_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.fvm3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ok(self, rc, allow=()):
        if rc != capi.FVM_OK and rc not in allow:
            raise capi.FvmError(rc, self.L.fvm3_last_error(self.h).decode())
        return rc

    def _arr(self, a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64).ravel()
        if a.size != self.n:
            raise ValueError(f"array has {a.size} elements, expected {self.n}")
        return a

    def set_grid(self, g):
        x, y, z = self._arr(g.xg), self._arr(g.yg), self._arr(g.zg)
        self._ok(self.L.fvm3_set_grid(self.h, _dp(x), _dp(y), _dp(z)))

    def init(self, du=None, dv=None, dw=None):
        a, b, c = self._arr(du), self._arr(dv), self._arr(dw)
        self._ok(self.L.fvm3_init(self.h, _dp(a), _dp(b), _dp(c)))

    def step(self, n=1) -> dict:
        c = Coeffs3()
        self._ok(self.L.fvm3_step(self.h, n, ctypes.byref(c)), allow=(capi.FVM_ERR_NOCONV,))
        return c.as_dict()

    def call(self, name):
        """One per-routine call point without arguments, e.g. call("begin_step")."""
        f = "fvm3_" + name
        if f not in ROUTINES:
            raise KeyError(name)
        self._ok(getattr(self.L, f)(self.h))

    def iter_u(self, component):
        self._ok(self.L.fvm3_iter_u(self.h, component))

    def iter_p(self):
        """CONTRA_VEL, ITER_P, BCP; returns (scaled residual, sweeps)."""
        r = ctypes.c_double()
        n = ctypes.c_int()
        self._ok(self.L.fvm3_iter_p(self.h, ctypes.byref(r), ctypes.byref(n)), allow=(capi.FVM_ERR_NOCONV,))
        return r.value, n.value

    def calccoef(self) -> dict:
        c = Coeffs3()
        self._ok(self.L.fvm3_calccoef(self.h, ctypes.byref(c)))
        return c.as_dict()

    def test_filter(self, a, out=None) -> np.ndarray:
        """TEST_FILTER(IN, OUT): the box filter of a into the interior of out."""
        src = self._arr(a)
        dst = np.zeros(self.n) if out is None else self._arr(out).copy()
        self._ok(self.L.fvm3_test_filter(self.h, _dp(src), _dp(dst)))
        return dst.reshape(self.shape)

    WALL_STATS = ("CF_WALL", "CP_WALL", "NU_WALL")

    def post_begin(self):
        """POST_PROCESS with IPOST=0: averaging from the next step on."""
        self._ok(self.L.fvm3_post_begin(self.h))

    def post_end(self):
        self._ok(self.L.fvm3_post_end(self.h))

    def post_steps(self) -> int:
        n = ctypes.c_int()
        self._ok(self.L.fvm3_post_steps(self.h, ctypes.byref(n)))
        return n.value

    def post_get(self, name) -> np.ndarray:
        """An average of POST_PROCESS with IPOST=1: a field shaped like the state, or
        for the wall statistics an array shaped (NK+1, NJ+1)."""
        shape = (self.nk + 1, self.nj + 1) if name in self.WALL_STATS else self.shape
        out = np.zeros(shape)
        self._ok(self.L.fvm3_post_get(self.h, name.encode(), _dp(out)))
        return out

    def sgs(self) -> dict:
        c = Coeffs3()
        self._ok(self.L.fvm3_sgs(self.h, ctypes.byref(c)))
        return c.as_dict()

    def get(self, name) -> np.ndarray:
        out = np.empty(self.n)
        self._ok(self.L.fvm3_get_array(self.h, name.encode(), _dp(out)))
        return out.reshape(self.shape)

    STATE = ("U", "V", "W", "P", "T", "NLX", "NLY", "NLZ", "ADV")

    def upload_ptrs(self, ptrs):
        """fvm3_upload_state from nine raw host addresses in STATE order (0 skips an
        array); page-locked buffers make each copy one DMA transfer."""
        P = ctypes.POINTER(ctypes.c_double)
        self._ok(self.L.fvm3_upload_state(self.h, *[ctypes.cast(p, P) if p else None for p in ptrs]))

    def download_ptrs(self, ptrs):
        P = ctypes.POINTER(ctypes.c_double)
        self._ok(self.L.fvm3_download_state(self.h, *[ctypes.cast(p, P) if p else None for p in ptrs]))

    def upload(self, **arrays):
        """fvm3_upload_state from numpy arrays named as in STATE (missing: skipped)."""
        arrs = [None if arrays.get(nm) is None else self._arr(arrays[nm]) for nm in self.STATE]
        self._ok(self.L.fvm3_upload_state(self.h, *[None if a is None else _dp(a) for a in arrs]))

    def download(self, names=STATE) -> dict:
        """fvm3_download_state into fresh arrays shaped like the state."""
        out = {nm: np.empty(self.shape) for nm in names}
        self._ok(self.L.fvm3_download_state(self.h, *[_dp(out[nm]) if nm in out else None for nm in self.STATE]))
        return out

    def set(self, name, a):
        a = self._arr(a)
        self._ok(self.L.fvm3_set_array(self.h, name.encode(), _dp(a)))

    def time_sweeps(self, sweeps=50) -> float:
        ms = ctypes.c_double()
        self._ok(self.L.fvm3_time_sweeps(self.h, sweeps, ctypes.byref(ms)))
        return ms.value

    def stream_handle(self) -> int:
        s = ctypes.c_void_p()
        self._ok(self.L.fvm3_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0
