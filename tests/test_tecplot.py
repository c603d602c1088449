"""The Tecplot writers (fvm_gb300.tecplot) reproduce the numeric rows of the
files the reference wrote in the golden program runs: the 2-D time-averaged field
and the 3-D averaged, rms, Reynolds-stress and wall files (written by the
reference with D16.9, so to 9 significant digits)."""
import json
import math
import os

import numpy as np
import pytest

import oracle
from fvm_gb300 import tecplot
from fvm_gb300.grid import o_grid, o_grid_3d, perturbation_3d

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _manifest():
    path = os.path.join(GOLD, "manifest.json")
    return json.load(open(path)) if os.path.exists(path) else {}


@pytest.mark.parametrize("entry", _manifest().get("program_cases", []), ids=lambda e: e["name"])
def test_averaged_field_file_2d(entry, tmp_path):
    data = np.load(os.path.join(GOLD, entry["file"]))
    g = o_grid(entry["n_theta"], entry["n_r"], dr1=entry["dr1"], r_out=entry["r_out"], skew=entry["skew"])
    o = oracle.Oracle(g.ni, g.nj, re=entry["re"], pr=entry["pr"], dt=entry["dt"], vel_rot=entry["vel_rot"],
                      order=oracle.FAITHFUL, resimax=entry["resimax"], nswpp=entry["nswpp"], thermal=True)
    o.set_grid(g.xg, g.yg)
    o.init()
    o.step(entry["steps_before"])
    o.post_begin()
    o.step(entry["steps_post"])
    _, f = o.post_final()
    path = tmp_path / "TIME-AVERAGED FIELD.PLT"
    tecplot.write_averaged_file_2d(str(path), o.array("X"), o.array("Y"), f, o.time)
    rows = tecplot.read_rows(str(path))
    ref = data["AVG_FIELD"]
    assert rows.shape == ref.shape
    assert np.abs(rows - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("entry", _manifest().get("program_cases_3d", []), ids=lambda e: e["name"])
def test_averaged_and_wall_files_3d(entry, tmp_path):
    data = np.load(os.path.join(GOLD, entry["file"]))
    g = o_grid_3d(entry["n_theta"], entry["n_r"], entry["n_z"], lz=math.pi, dr1=entry["dr1"], skew=entry["skew"])
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, entry["amp"], entry["seed"])
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=entry["re"], pr=entry["pr"], dt=entry["dt"], order=oracle.O3_FAITHFUL,
                        resimax=entry["resimax"], nswpp=entry["nswpp"], use_les=True, thermal=True,
                        ref_a=entry["ref_a"])
    o.set_grid(g)
    o.init(du, dv, dw)
    o.step(entry["steps_before"])
    o.post_begin()
    o.step(entry["steps_post"])
    names = ("U_AVG", "V_AVG", "W_AVG", "P_AVG", "T_AVG", "UU", "UV", "UW", "VV", "VW", "WW", "U_RMS", "V_RMS",
             "W_RMS")
    post = {nm: o.post_get(nm) for nm in names}
    tecplot.write_averaged_files_3d(str(tmp_path), g, post, o.coeffs()["time"], entry["re"], entry["pr"])
    for fn, key in (("Avrg000.PLT", "AVRG"), ("Urms000.PLT", "URMS"), ("Strs000.PLT", "STRS")):
        rows = tecplot.read_rows(str(tmp_path / fn))
        ref = data[key]
        assert rows.shape == ref.shape, fn
        for col in range(ref.shape[1]):   # 9 significant digits per value
            assert np.allclose(rows[:, col], ref[:, col], rtol=1e-8, atol=1e-8 * np.abs(ref[:, col]).max()), (fn, col)
    wall = tmp_path / "Surf000.PLT"
    tecplot.write_wall_file_3d(str(wall), o.array("X"), o.array("Y"), o.array("Z"), o.array("THETA"),
                               o.post_get("CF_WALL"), o.post_get("CP_WALL"), o.post_get("NU_WALL"))
    rows = tecplot.read_rows(str(wall))
    ref = data["SURF"]
    assert rows.shape == ref.shape
    for col in range(ref.shape[1]):
        assert np.allclose(rows[:, col], ref[:, col], rtol=1e-8, atol=1e-8 * np.abs(ref[:, col]).max()), col


def test_d16_9_edit_descriptor():
    assert tecplot._d169(1.0) == " 0.100000000D+01"
    assert tecplot._d169(-0.000123456789) == "-0.123456789D-03"
    assert tecplot._d169(0.0) == " 0.000000000D+00"
    assert len(tecplot._d169(123456.7)) == 16
