"""ctypes binding of the CPU restatement (test infrastructure only).

Only the tests, the smoke check and the CPU-baseline leg of bench.py use this
module, as the checker.  The product never imports it.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
# Builds of the same sources (oracle/Makefile): "check" is the serial checker;
# "par" adds OpenMP to the GPU-order line sweeps and stencil loops with results
# bit-identical to "check"; "fast" is a serial timing copy with FMA contraction.
VARIANTS = {"check": LIB, "par": os.path.join(HERE, "_build", "liboracle_par.so"),
            "fast": os.path.join(HERE, "_build", "liboracle_fast.so")}
SOURCES = ("fvm_oracle.c", "fvm_oracle.h", "fvm3d_oracle.c", "fvm3d_oracle.h", "Makefile")

FAITHFUL, GPU = 0, 1


class Params(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int),
                ("re", ctypes.c_double), ("pr", ctypes.c_double), ("dt", ctypes.c_double),
                ("vel_rot", ctypes.c_double), ("uin", ctypes.c_double), ("vin", ctypes.c_double),
                ("tin", ctypes.c_double), ("t_wall", ctypes.c_double), ("resimax", ctypes.c_double),
                ("nswpp", ctypes.c_int), ("order", ctypes.c_int), ("iter_t_bug", ctypes.c_int),
                ("thermal", ctypes.c_int), ("res_every", ctypes.c_int), ("dd_positional", ctypes.c_int)]


class Coeffs(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "cfl", "cpb", "cd", "cl", "cd_p", "cd_v", "cl_p", "cl_v", "nu")] + \
               [("sweeps", ctypes.c_int), ("resid", ctypes.c_double)]


class Post(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "nu", "cd", "cl", "cl_amp", "cpb", "st", "rms_cd", "rms_cl", "st_last", "cl_amp_last")] + \
               [("niter", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


def _stale(path: str) -> bool:
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    return any(os.path.getmtime(os.path.join(HERE, f)) > t for f in SOURCES)


def build(force: bool = False) -> str:
    """Compile every variant of the restatement with its Makefile when any source,
    header or the Makefile itself is newer than a library."""
    if force or any(_stale(v) for v in VARIANTS.values()):
        subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []), check=True)
    return LIB


_libs = {}


def lib(variant: str = "check"):
    """The ctypes handle of one build variant ("check", "par" or "fast")."""
    if variant not in _libs:
        build()
        L = ctypes.CDLL(VARIANTS[variant])
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(Params)]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        P = ctypes.POINTER(ctypes.c_double)
        L.orc_set_grid.argtypes = [ctypes.c_void_p, P, P]
        L.orc_init.argtypes = [ctypes.c_void_p, P, P]
        L.orc_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_last_coeffs.restype = ctypes.POINTER(Coeffs)
        L.orc_last_coeffs.argtypes = [ctypes.c_void_p]
        L.orc_array.restype = P
        L.orc_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc_time.restype = ctypes.c_double
        L.orc_time.argtypes = [ctypes.c_void_p]
        L.orc_set_time.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        L.orc_set_controls.argtypes = [ctypes.c_void_p, ctypes.c_double, P]
        L.orc_sum_area.restype = ctypes.c_double
        L.orc_sum_area.argtypes = [ctypes.c_void_p]
        L.orc_iter_p.restype = ctypes.c_int
        L.orc_post_begin.argtypes = [ctypes.c_void_p]
        L.orc_calc_vor.argtypes = [ctypes.c_void_p]
        L.orc_post_record.restype = ctypes.POINTER(Post)
        L.orc_post_record.argtypes = [ctypes.c_void_p]
        L.orc_post_final.argtypes = [ctypes.c_void_p, ctypes.POINTER(Post), P, P, P, P, P]
        for f in ("orc_begin_step", "orc_contra_vel", "orc_explicit", "orc_iter_u", "orc_iter_v",
                  "orc_remove_grad", "orc_iter_p", "orc_correct", "orc_iter_t", "orc_calccoef"):
            getattr(L, f).argtypes = [ctypes.c_void_p]
        _libs[variant] = L
    return _libs[variant]


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """One case of the CPU restatement.  Arrays are numpy views shaped
    (NJ+1, NI+1): a[j, i] is the reference's (I, J)."""

    def __init__(self, ni, nj, re=100.0, pr=0.71, dt=0.005, vel_rot=0.0, order=GPU,
                 resimax=1e-10, nswpp=100000, thermal=True, iter_t_bug=True, res_every=1,
                 uin=1.0, vin=0.0, tin=0.0, t_wall=1.0, dd_positional=True, variant="check"):
        self.ni, self.nj = ni, nj
        self._L = lib(variant)
        p = Params(ni=ni, nj=nj, re=re, pr=pr, dt=dt, vel_rot=vel_rot, uin=uin, vin=vin, tin=tin,
                   t_wall=t_wall, resimax=resimax, nswpp=nswpp, order=order,
                   iter_t_bug=int(iter_t_bug), thermal=int(thermal), res_every=res_every,
                   dd_positional=int(dd_positional))
        self._p = p
        self._h = self._L.orc_create(ctypes.byref(p))
        if not self._h:
            raise ValueError("orc_create failed")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            self._L.orc_destroy(h)
            self._h = None

    def set_grid(self, xg, yg):
        xg = np.ascontiguousarray(xg, dtype=np.float64).ravel()
        yg = np.ascontiguousarray(yg, dtype=np.float64).ravel()
        rc = self._L.orc_set_grid(self._h, _dptr(xg), _dptr(yg))
        if rc != 0:
            raise ValueError(f"orc_set_grid failed ({rc})")

    def init(self, du=None, dv=None):
        a = None if du is None else np.ascontiguousarray(du, dtype=np.float64).ravel()
        b = None if dv is None else np.ascontiguousarray(dv, dtype=np.float64).ravel()
        self._L.orc_init(self._h, None if a is None else _dptr(a), None if b is None else _dptr(b))

    def step(self, n=1):
        rc = self._L.orc_step(self._h, n)
        if rc != 0:
            raise FloatingPointError(f"orc_step failed ({rc})")

    def call(self, name):
        return getattr(self._L, "orc_" + name)(self._h)

    def set_controls(self, omega=0.0, blow=None):
        """Wall rotation rate and wall-normal blowing speeds (NJ-1 values)."""
        b = None if blow is None else np.ascontiguousarray(blow, dtype=np.float64).ravel()
        if b is not None and b.size != self.nj - 1:
            raise ValueError(f"blow needs {self.nj - 1} values")
        self._L.orc_set_controls(self._h, ctypes.c_double(omega), None if b is None else _dptr(b))

    STATE = ("U", "V", "P", "T", "U_N", "V_N", "T_N", "NLX", "NLY", "ADV", "NLX_NM1", "NLY_NM1", "ADV_NM1")

    def save_state(self):
        return {nm: self.array(nm).copy() for nm in self.STATE}, self.time

    def restore_state(self, saved):
        arrs, t = saved
        for nm, a in arrs.items():
            self.array(nm)[...] = a
        self.set_time(t)

    def array(self, name) -> np.ndarray:
        p = self._L.orc_array(self._h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(self.nj + 1, self.ni + 1))

    def coeffs(self) -> dict:
        c = self._L.orc_last_coeffs(self._h).contents
        return {n: getattr(c, n) for n, _ in Coeffs._fields_}

    def post_begin(self):
        """POST_PROCESS with IPOST=0: time averaging from the next step on."""
        self._L.orc_post_begin(self._h)

    def post_record(self) -> dict:
        """The POST_NU_CD_CL.PLT record of the last step."""
        return self._L.orc_post_record(self._h).contents.as_dict()

    def post_final(self):
        """POST_PROCESS with IPOST=1: averaged coefficients and fields."""
        out = Post()
        shape = (self.nj + 1, self.ni + 1)
        f = {nm: np.zeros(shape) for nm in ("U", "V", "P", "T", "VOR")}
        self._L.orc_post_final(self._h, ctypes.byref(out), *[_dptr(f[nm]) for nm in ("U", "V", "P", "T", "VOR")])
        return out.as_dict(), f

    @property
    def time(self):
        return self._L.orc_time(self._h)

    def set_time(self, t, niter=0):
        self._L.orc_set_time(self._h, t, niter)


# ---------------------------------------------------------------------------
# 3-D LES restatement (fvm3d_oracle.c)
# ---------------------------------------------------------------------------
O3_FAITHFUL, O3_GPU = 0, 1


class Params3D(ctypes.Structure):
    _fields_ = [("ni", ctypes.c_int), ("nj", ctypes.c_int), ("nk", ctypes.c_int),
                ("re", ctypes.c_double), ("pr", ctypes.c_double), ("dt", ctypes.c_double),
                ("tin", ctypes.c_double), ("t_wall", ctypes.c_double), ("resimax", ctypes.c_double),
                ("nswpp", ctypes.c_int), ("order", ctypes.c_int), ("use_les", ctypes.c_int),
                ("les_zavg", ctypes.c_int), ("thermal", ctypes.c_int), ("res_every", ctypes.c_int),
                ("ref_a", ctypes.c_double)]


class Coeffs3D(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("time", "cfl", "cpb", "cd", "cl", "cd_p", "cd_v", "cl_p", "cl_v", "nu", "cs2", "ct2")] + \
               [("sweeps", ctypes.c_int), ("resid", ctypes.c_double)]


class Oracle3D:
    """The 3-D LES step of the reference restated in C (test infrastructure).
    Arrays are numpy views shaped (NK+1, NJ+1, NI+1)."""

    def __init__(self, ni, nj, nk, re=3900.0, pr=0.71, dt=0.002, order=O3_GPU, resimax=1e-10, nswpp=100000,
                 use_les=True, les_zavg=False, thermal=True, res_every=2, ref_a=None, lz=math.pi,
                 tin=0.0, t_wall=1.0):
        L = lib()
        if not hasattr(L, "_o3_ready"):
            P = ctypes.POINTER(ctypes.c_double)
            L.o3_create.restype = ctypes.c_void_p
            L.o3_create.argtypes = [ctypes.POINTER(Params3D)]
            L.o3_destroy.argtypes = [ctypes.c_void_p]
            L.o3_set_grid.argtypes = [ctypes.c_void_p, P, P, P]
            L.o3_init.argtypes = [ctypes.c_void_p, P, P, P]
            L.o3_step.argtypes = [ctypes.c_void_p, ctypes.c_int]
            L.o3_last_coeffs.restype = ctypes.POINTER(Coeffs3D)
            L.o3_last_coeffs.argtypes = [ctypes.c_void_p]
            L.o3_array.restype = P
            L.o3_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
            L.o3_sgs.argtypes = [ctypes.c_void_p]
            L.o3_test_filter.argtypes = [ctypes.c_void_p, P, P]
            L.o3_post_begin.argtypes = [ctypes.c_void_p]
            L.o3_post_steps.argtypes = [ctypes.c_void_p]
            L.o3_post_steps.restype = ctypes.c_int
            L.o3_post_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, P]
            L.o3_post_get.restype = ctypes.c_int
            L._o3_ready = True
        self.ni, self.nj, self.nk = ni, nj, nk
        if ref_a is None:
            ref_a = 1.0 * lz          # diameter x span
        p = Params3D(ni=ni, nj=nj, nk=nk, re=re, pr=pr, dt=dt, tin=tin, t_wall=t_wall, resimax=resimax,
                     nswpp=nswpp, order=order, use_les=int(use_les), les_zavg=int(les_zavg), thermal=int(thermal),
                     res_every=res_every, ref_a=ref_a)
        self._h = L.o3_create(ctypes.byref(p))
        if not self._h:
            raise MemoryError("o3_create failed")

    def __del__(self):
        try:
            if self._h:
                lib().o3_destroy(self._h)
                self._h = None
        except Exception:
            pass

    def set_grid(self, g):
        arrs = [np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (g.xg, g.yg, g.zg)]
        rc = lib().o3_set_grid(self._h, *[_dptr(a) for a in arrs])
        if rc != 0:
            raise ValueError(f"o3_set_grid failed ({rc})")

    def init(self, du=None, dv=None, dw=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64).ravel() for a in (du, dv, dw)]
        lib().o3_init(self._h, *[None if a is None else _dptr(a) for a in arrs])

    def step(self, n=1):
        rc = lib().o3_step(self._h, n)
        if rc != 0:
            raise FloatingPointError(f"o3_step failed ({rc})")

    def sgs(self):
        lib().o3_sgs(self._h)

    WALL_STATS = ("CF_WALL", "CP_WALL", "NU_WALL")

    def post_begin(self):
        """POST_PROCESS with IPOST=0: averaging from the next step on."""
        lib().o3_post_begin(self._h)

    def post_steps(self):
        return lib().o3_post_steps(self._h)

    def post_get(self, name):
        """An average of POST_PROCESS with IPOST=1: a field shaped (NK+1, NJ+1, NI+1),
        or for the wall statistics an array shaped (NK+1, NJ+1)."""
        shape = (self.nk + 1, self.nj + 1) if name in self.WALL_STATS else (self.nk + 1, self.nj + 1, self.ni + 1)
        out = np.zeros(shape)
        if lib().o3_post_get(self._h, name.encode(), _dptr(out)) != 0:
            raise KeyError(name)
        return out

    def test_filter(self, a, out=None):
        """TEST_FILTER(IN, OUT) of a into the interior of out (test_filter.f90)."""
        shape = (self.nk + 1, self.nj + 1, self.ni + 1)
        src = np.ascontiguousarray(a, dtype=np.float64).reshape(shape)
        dst = np.zeros(shape) if out is None else np.array(out, dtype=np.float64).reshape(shape)
        lib().o3_test_filter(self._h, _dptr(src), _dptr(dst))
        return dst

    def array(self, name) -> np.ndarray:
        p = lib().o3_array(self._h, name.encode())
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, shape=(self.nk + 1, self.nj + 1, self.ni + 1))

    def coeffs(self) -> dict:
        c = lib().o3_last_coeffs(self._h).contents
        return {n: getattr(c, n) for n, _ in Coeffs3D._fields_}
