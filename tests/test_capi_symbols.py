"""CPU tests: the CUDA library loads without a GPU and exports every function the
public header declares; argument errors are reported as status codes."""
import ctypes
import os
import re

from fvm_gb300 import capi

HDR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    names = set()
    for f in os.listdir(HDR):
        if f.endswith(".h"):
            txt = open(os.path.join(HDR, f)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(fvm3?_[a-z0-9_]+)\s*\(", txt, re.M))
    return names


def test_header_declares_the_binding_list():
    from fvm_gb300 import capi3d
    assert declared_functions() == set(capi.EXPORTS) | set(capi3d.EXPORTS)


def test_library_exports_every_declared_symbol():
    L = capi.load()
    for name in declared_functions():
        assert hasattr(L, name), name


def test_default_params_are_the_reference_parameters():
    p = capi.default_params()
    assert p.resimax == 1e-4 and p.nswpp == 20 and p.uin == 1.0 and p.t_wall == 1.0
    assert p.precision == capi.FP64


def test_create_rejects_bad_parameters_without_a_gpu():
    L = capi.load()
    h = ctypes.c_void_p()
    p = capi.default_params(nj=128)          # NJ-1 odd: the zebra order needs an even count
    assert L.fvm_create(ctypes.byref(p), ctypes.byref(h)) == capi.FVM_ERR_ARG
    p = capi.default_params(dt=0.0)
    assert L.fvm_create(ctypes.byref(p), ctypes.byref(h)) == capi.FVM_ERR_ARG
    assert L.fvm_create(None, ctypes.byref(h)) == capi.FVM_ERR_ARG
    assert L.fvm_destroy(None) == capi.FVM_ERR_ARG
    assert L.fvm_step(None, 1, None) == capi.FVM_ERR_ARG


def test_batch_rejects_mismatched_options_without_a_gpu():
    L = capi.load()
    h = ctypes.c_void_p()
    ps = (capi.Params * 2)(capi.default_params(), capi.default_params(precision=capi.MIXED))
    assert L.fvm_batch_create(2, ps, ctypes.byref(h)) == capi.FVM_ERR_ARG
    assert L.fvm_batch_create(0, ps, ctypes.byref(h)) == capi.FVM_ERR_ARG
    assert L.fvm_batch_destroy(None) == capi.FVM_ERR_ARG
    assert L.fvm_batch_step(None, 1, None) == capi.FVM_ERR_ARG


def test_create_rejects_a_tile_that_does_not_cover_the_line():
    L = capi.load()
    h = ctypes.c_void_p()
    p = capi.default_params(ni=97, tile_r_warps=1, tile_r_m=2)     # 64 < 96 radial cells
    assert L.fvm_create(ctypes.byref(p), ctypes.byref(h)) == capi.FVM_ERR_ARG
    p = capi.default_params(tile_r_warps=3, tile_r_m=1)
    assert L.fvm_create(ctypes.byref(p), ctypes.byref(h)) == capi.FVM_ERR_ARG
