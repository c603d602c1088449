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


def test_resident_roofline_names_the_kernel_it_timed():
    w = dict(bench.WORKLOAD)
    spl = w["refine_sweeps"]
    two = bench.roofline_sweep(w, 0.7e-3, {"hbm_gbs": 6790.0}, True, True,
                               {"lines_per_block": 4, "blocks": 128, "sweeps_per_exchange": 2})
    one = bench.roofline_sweep(w, 0.8e-3, {"hbm_gbs": 6790.0}, True, True,
                               {"lines_per_block": 4, "blocks": 128, "sweeps_per_exchange": 1})
    assert two["kernel"] == "k_pois32_resident2" and one["kernel"] == "k_pois32_resident"
    assert two["per_sweep_us"] == pytest.approx(1.4) and two["sweeps_per_launch"] == spl
    assert two["bytes_per_sweep"] == 32.0 * bench.cells(w)
    assert two["avg_launch_us"] == pytest.approx(1.4 * spl)


def test_clock_sampler_counts_only_readings_inside_timed_windows(tmp_path, monkeypatch):
    """A stand-in nvidia-smi prints a reading every 50 ms, SM clock 1000 MHz outside
    and 2070 inside the two windows the test opens; only the latter may count."""
    flag = tmp_path / "inside"
    fake = tmp_path / "nvidia-smi"
    fake.write_text("#!/bin/sh\nwhile true; do\n  if [ -e '%s' ]; then c=2070; r='Active'; else c=1000; r='Not Active'; fi\n"
                    "  echo \"0, $c, 2070, 500.0, 0x0, Not Active, Not Active, Not Active, $r\"\n"
                    "  sleep 0.05\ndone\n" % flag)
    fake.chmod(0o755)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))
    import time
    clk = bench.ClockSampler(0)
    clk.open()
    time.sleep(0.3)
    for _ in range(2):
        flag.write_text("1")
        time.sleep(0.15)
        clk.begin()
        time.sleep(0.5)
        clk.end()
        flag.unlink()
        time.sleep(0.4)
    out = clk.close()
    assert out["samples"] >= 8
    assert out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]
    assert out["timed_s"] == pytest.approx(1.0, abs=0.1)
