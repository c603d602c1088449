"""CPU checks of the benchmark script's pure parts: the roofline arithmetic of the
Poisson sweep kernels (algorithmic bytes per launch / launch time against the
measured HBM copy rate, the fallback when no measurement exists), the command-line
contract, and the 3-D defaults the bench builds on."""
import subprocess
import sys
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def test_2d_roofline_bytes_and_fraction():
    w = dict(bench.WORKLOAD)
    n_active = bench.cells(w) // 2
    r = bench.roofline_sweep(w, 2e-3, {"hbm_gbs": 6000.0}, True)   # 2 us per launch
    assert r["bytes_per_launch"] == 32.0 * n_active
    assert r["achieved"] == pytest.approx(32.0 * n_active / 2e-6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6000.0) and r["peak_source"] == "measured"
    r64 = bench.roofline_sweep(w, 2e-3, {}, False)
    assert r64["bytes_per_launch"] == 100.0 * n_active and r64["peak"] == 6800.0
    assert r64["peak_source"] == "fallback" and r64["kernel"] == "k_pois64"
    assert bench.roofline_sweep(w, 0.0, {}, True) is None


def test_3d_roofline_bytes():
    n_int = 256 * 192 * 48
    r = bench.roofline_sweep3d(n_int, 7e-3, {"hbm_gbs": 6693.5}, True)
    assert r["bytes_per_launch"] == 40.0 * (n_int // 2) and r["kernel"] == "k3_line32"
    assert r["achieved"] == pytest.approx(40.0 * (n_int // 2) / 7e-6 / 1e9)
    r64 = bench.roofline_sweep3d(n_int, 36e-3, {"hbm_gbs": 6693.5}, False)
    assert r64["bytes_per_launch"] == 80.0 * (n_int // 2)


def test_command_line_contract():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--poisson-loop"):
        assert flag in out.stdout, flag


def test_3d_default_params():
    from fvm_gb300 import capi, capi3d
    p = capi3d.default_params()
    assert (p.ni, p.nj, p.nk) == (241, 201, 121) and p.nswpp == 20 and p.resimax == 1e-4
    assert p.precision == capi.FP64 and p.poisson_host_loop == 1 and p.tile_i_warps == 0
