"""CPU tests: the O-grid generator, the CPU restatement's own invariants, its
faithful/GPU orderings against each other, and the committed golden fixtures."""
import json
import math
import os

import numpy as np
import pytest

import oracle
from fvm_gb300.grid import (grid_file_name, o_grid, perturbation, read_grid_file, stretch_ratio,
                            write_grid_file)
from tests.helpers import make_case, make_oracle, rel_l2

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_stretch_ratio_reaches_outer_radius():
    for n, dr1, q_expect in ((96, 0.005, 1.0706), (384, 0.005, 1.0127), (192, 0.001, 1.0404)):
        q = stretch_ratio(n, dr1, 0.5, 50.0)
        assert abs(q - q_expect) < 5e-4
        r = 0.5 + dr1 * (q ** n - 1) / (q - 1)
        assert abs(r - 50.0) < 1e-9


def test_o_grid_closure_and_orientation():
    g = o_grid(32, 16)
    assert g.ni == 17 and g.nj == 33
    assert np.array_equal(g.xg[g.nj, 1:], g.xg[1, 1:])
    assert np.array_equal(g.yg[g.nj, 1:], g.yg[1, 1:])
    # node J=1 on the downstream axis, J increasing counter-clockwise
    assert g.xg[1, 1] == pytest.approx(0.5) and g.yg[1, 1] == 0.0
    assert g.yg[2, 1] > 0.0


def test_grid_file_roundtrip(tmp_path):
    g = o_grid(16, 8, skew=0.3)
    f = tmp_path / grid_file_name(g.ni, g.nj)
    write_grid_file(str(f), g)
    assert f.name == "009x017.dat"
    h = read_grid_file(str(f), g.ni, g.nj)
    assert np.array_equal(h.xg, g.xg) and np.array_equal(h.yg, g.yg)


def test_perturbation_is_seeded_and_interior_only():
    du, dv = perturbation(9, 17, 1e-3, 7)
    du2, _ = perturbation(9, 17, 1e-3, 7)
    assert np.array_equal(du, du2)
    assert np.all(du[0, :] == 0) and np.all(du[:, 0] == 0) and np.all(du[17, :] == 0) and np.all(du[:, 9] == 0)
    assert np.abs(du).max() <= 1e-3 and np.abs(dv).max() > 0


def test_metrics_of_polar_grid():
    case = make_case(32, 24)
    o = make_oracle(case)
    J = o.array("DJAC")
    assert np.all(J > 0)
    q12 = o.array("Q12")[1:-1, 1:-1]
    q11 = o.array("Q11")[1:-1, 1:-1]
    assert np.abs(q12).max() < 1e-9 * np.abs(q11).max()   # orthogonal polar grid
    area = o.array("AREA")[1:case["g"].nj, 1]
    assert area.sum() == pytest.approx(math.pi * 1.0, rel=2e-3)   # circumference of D=1


def test_theta_quadrants():
    case = make_case(32, 24)
    o = make_oracle(case)
    th = o.array("THETA")
    assert np.all(th >= 0) and np.all(th < 2 * math.pi)
    # first interior cell centre sits at half a theta spacing above the x axis
    assert th[1, 1] == pytest.approx(math.pi / 32, rel=1e-9)


@pytest.mark.parametrize("order", [oracle.FAITHFUL, oracle.GPU])
def test_poisson_converges_and_projection_reduces_divergence(order):
    case = make_case(32, 24, resimax=1e-12)
    o = make_oracle(case, order=order)
    o.step(2)
    c = o.coeffs()
    assert c["resid"] <= 1e-12 and c["sweeps"] > 10
    assert np.isfinite(c["cd"]) and c["cd"] > 0


def test_gpu_order_tracks_faithful_order():
    """The zebra/cyclic reordering changes the predictor's splitting error only;
    after a few steps the two orders stay close."""
    case = make_case(32, 24, resimax=1e-12)
    a = make_oracle(case, order=oracle.FAITHFUL)
    b = make_oracle(case, order=oracle.GPU)
    a.step(5)
    b.step(5)
    ni, nj = case["g"].ni, case["g"].nj
    for nm in ("U", "V"):
        assert rel_l2(b.array(nm), a.array(nm), (ni, nj)) < 1e-2
    assert rel_l2(b.array("P"), a.array("P"), (ni, nj)) < 5e-2
    assert abs(b.coeffs()["cd"] - a.coeffs()["cd"]) < 2e-2 * abs(a.coeffs()["cd"])


def test_res_every_only_adds_sweeps():
    case = make_case(32, 24, resimax=1e-10)
    a = make_oracle(case, res_every=1)
    b = make_oracle(case, res_every=4)
    a.step(1)
    b.step(1)
    sa, sb = a.coeffs()["sweeps"], b.coeffs()["sweeps"]
    assert sb >= sa and sb % 4 == 0 and sb - sa < 4
    assert b.coeffs()["resid"] <= 1e-10


def test_sweep_cap_is_honoured():
    case = make_case(32, 24, resimax=1e-14, nswpp=7)
    o = make_oracle(case)
    o.step(1)
    assert o.coeffs()["sweeps"] == 7


def test_iter_t_bug_switch_changes_only_temperature():
    case = make_case(32, 24, resimax=1e-12)
    a = make_oracle(case)
    g = case["g"]
    b = oracle.Oracle(g.ni, g.nj, re=100, pr=0.71, dt=0.005, order=oracle.GPU, resimax=1e-12, nswpp=200000,
                      thermal=True, iter_t_bug=False)
    b.set_grid(g.xg, g.yg)
    b.init(case["du"], case["dv"])
    a.step(2)
    b.step(2)
    assert np.array_equal(a.array("U"), b.array("U"))
    assert not np.array_equal(a.array("T"), b.array("T"))


# record layout of the coefficient file written by CALCCOEF
GOLD_COEFFS = ("time", "nu", "cd", "cl", "cpb", "cd_p", "cd_v", "cl_p", "cl_v", "cfl")


def _golden_cases():
    path = os.path.join(GOLD, "manifest.json")
    if not os.path.exists(path):
        return []
    return json.load(open(path))["cases"]


@pytest.mark.parametrize("entry", _golden_cases(), ids=lambda e: e["name"])
def test_oracle_against_golden_fixtures(entry):
    """Replays each committed fixture case and compares every stored field."""
    data = np.load(os.path.join(GOLD, entry["file"]))
    g = o_grid(entry["n_theta"], entry["n_r"], dr1=entry["dr1"], r_out=entry["r_out"], skew=entry["skew"])
    du, dv = perturbation(g.ni, g.nj, entry["amp"], entry["seed"])
    o = oracle.Oracle(g.ni, g.nj, re=entry["re"], pr=entry["pr"], dt=entry["dt"], vel_rot=entry["vel_rot"],
                      order=entry["order"], resimax=entry["resimax"], nswpp=entry["nswpp"],
                      thermal=True, iter_t_bug=True)
    o.set_grid(g.xg, g.yg)
    o.init(du, dv)
    recs = []
    for _ in range(entry["steps"]):
        o.step(1)
        c = o.coeffs()
        recs.append([c[k] for k in GOLD_COEFFS])
    tol = entry["tol"]
    for nm in entry["fields"]:
        ref = data[nm]
        got = o.array(nm)
        assert rel_l2(got, ref) <= tol, nm
    # one NU_CD_CL.PLT record per step (calccoef.f90:122-123)
    ref = data["COEFFS"]
    assert ref.shape == (entry["steps"], len(GOLD_COEFFS))
    np.testing.assert_allclose(np.array(recs), ref, rtol=1e-11, atol=1e-11)
