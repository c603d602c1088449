"""CPU tests of the 3-D LES restatement: geometry invariants of the extruded
O-grid, the test filter, the two line orders tracking each other, and the
committed golden fixtures (the reference's LES solver executed from its own
sources by tests/golden/ftn_interp.py)."""
import json
import math
import os

import numpy as np
import pytest

import oracle
from fvm_gb300.grid import o_grid_3d, perturbation_3d, read_grid_file_3d, write_grid_file_3d


def _oracle(order=oracle.O3_GPU, skew=0.0, les=True, **kw):
    g = o_grid_3d(16, 12, 8, lz=math.pi, dr1=0.01, skew=skew)
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=3900.0, dt=0.002, order=order, resimax=1e-10, nswpp=4000,
                        use_les=les, ref_a=math.pi, **kw)
    o.set_grid(g)
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, 0.05, 1)
    o.init(du, dv, dw)
    return g, o


def test_jacobian_sums_to_the_annulus_volume():
    g, o = _oracle()
    J = o.array("DJAC")[1:g.nk, 1:g.nj, 1:g.ni]
    assert (J > 0).all()
    # cell volumes of the 16-sided polygonal annulus times the span, within the
    # accuracy of the centred metric differences on this coarse grid
    poly = 0.5 * 16 * math.sin(2 * math.pi / 16) * (50.0 ** 2 - 0.5 ** 2) * math.pi
    assert abs(J.sum() / poly - 1.0) < 0.15


def test_polar_grid_is_orthogonal_and_spanwise_uniform():
    g, o = _oracle()
    # xi is radial, zeta is spanwise: no xi or eta dependence of z and vice versa
    assert np.max(np.abs(o.array("XIZ")[1:g.nk, 1:g.nj, 1:g.ni])) < 1e-12
    assert np.max(np.abs(o.array("ZTX")[1:g.nk, 1:g.nj, 1:g.ni])) < 1e-12
    zt = o.array("ZTZ")[1:g.nk, 1:g.nj, 1:g.ni]
    assert np.allclose(zt, (g.nk - 1) / math.pi, rtol=1e-9)     # 1 / (dz per index)


def test_grid_file_round_trip(tmp_path):
    g = o_grid_3d(8, 6, 4, lz=1.5)
    path = tmp_path / "g.dat"
    write_grid_file_3d(str(path), g)
    h = read_grid_file_3d(str(path), g.ni, g.nj, g.nk)
    assert np.array_equal(h.xg, g.xg) and np.array_equal(h.zg, g.zg)


def test_orders_track_each_other():
    _, a = _oracle(oracle.O3_FAITHFUL, skew=0.3)
    _, b = _oracle(oracle.O3_GPU, skew=0.3)
    a.step(3)
    b.step(3)
    for nm in ("U", "V", "W"):
        x, y = a.array(nm), b.array(nm)
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 2e-2, nm
    assert abs(a.coeffs()["cd"] - b.coeffs()["cd"]) < 0.05 * abs(b.coeffs()["cd"])


def test_dynamic_coefficient_is_positive_and_small():
    _, o = _oracle(skew=0.2)
    o.step(2)
    c = o.coeffs()
    assert 0.0 < c["cs2"] < 0.1 and np.isfinite(c["ct2"])


GOLD = os.path.join(os.path.dirname(__file__), "golden")
# record layout of the coefficient file written by CALCCOEF (calccoef.f90)
GOLD_COEFFS = ("time", "nu", "cd", "cl", "cpb", "cd_p", "cd_v", "cl_p", "cl_v", "cfl")


def _golden_cases_3d():
    path = os.path.join(GOLD, "manifest.json")
    if not os.path.exists(path):
        return []
    return json.load(open(path)).get("cases3d", [])


@pytest.mark.parametrize("entry", _golden_cases_3d(), ids=lambda e: e["name"])
def test_oracle_against_golden_fixtures_3d(entry):
    """Replays each committed 3-D case in the reference's own (lexicographic) order
    and compares every stored field and every coefficient record."""
    data = np.load(os.path.join(GOLD, entry["file"]))
    g = o_grid_3d(entry["n_theta"], entry["n_r"], entry["n_z"], lz=math.pi, dr1=entry["dr1"], skew=entry["skew"])
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, entry["amp"], entry["seed"])
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=entry["re"], pr=entry["pr"], dt=entry["dt"], order=oracle.O3_FAITHFUL,
                        resimax=entry["resimax"], nswpp=entry["nswpp"], use_les=bool(entry["use_les"]),
                        thermal=True, ref_a=entry["ref_a"])
    o.set_grid(g)
    o.init(du, dv, dw)
    recs = []
    for _ in range(entry["steps"]):
        o.step(1)
        c = o.coeffs()
        recs.append([c[k] for k in GOLD_COEFFS])
    for nm in entry["fields"]:
        ref = data[nm]
        got = o.array(nm)
        scale = max(np.linalg.norm(ref), 1e-300)
        assert np.linalg.norm(got - ref) / scale <= entry["tol"] or np.abs(got - ref).max() <= 1e-15, nm
    ref = data["COEFFS"]
    assert ref.shape == (entry["steps"], len(GOLD_COEFFS))
    np.testing.assert_allclose(np.array(recs), ref, rtol=1e-11, atol=1e-11)


def _program3d_cases():
    path = os.path.join(GOLD, "manifest.json")
    if not os.path.exists(path):
        return []
    return json.load(open(path)).get("program_cases_3d", [])


def _nodal(a, g):
    """The node values the reference writes: the mean of the 8 cells around node
    (i, j, k), i = 1..NI, j = 1..NJ, k = 1..NK (post_process.f90:120-132)."""
    out = []
    for k in range(1, g.nk + 1):
        for j in range(1, g.nj + 1):
            for i in range(1, g.ni + 1):
                out.append(0.125 * (((((((a[k, j, i] + a[k, j - 1, i]) + a[k, j, i - 1]) + a[k, j - 1, i - 1]) +
                                       a[k - 1, j, i]) + a[k - 1, j - 1, i]) + a[k - 1, j, i - 1]) +
                                    a[k - 1, j - 1, i - 1]))
    return np.array(out)


@pytest.mark.parametrize("entry", _program3d_cases(), ids=lambda e: e["name"])
def test_post_processing_against_the_reference_program_3d(entry, tmp_path):
    """The whole LES program with its averaging phase: per-step coefficient and
    dynamic-coefficient records, the averaged, rms, Reynolds-stress and wall files,
    and the restart file, replayed by the oracle in the reference's order."""
    from fvm_gb300 import restart
    data = np.load(os.path.join(GOLD, entry["file"]))
    g = o_grid_3d(entry["n_theta"], entry["n_r"], entry["n_z"], lz=math.pi, dr1=entry["dr1"], skew=entry["skew"])
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, entry["amp"], entry["seed"])
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=entry["re"], pr=entry["pr"], dt=entry["dt"], order=oracle.O3_FAITHFUL,
                        resimax=entry["resimax"], nswpp=entry["nswpp"], use_les=True, thermal=True,
                        ref_a=entry["ref_a"])
    o.set_grid(g)
    o.init(du, dv, dw)
    recs, cs, ct, state = [], [], [], None
    for s in range(1, entry["steps_before"] + entry["steps_post"] + 1):
        o.step(1)
        c = o.coeffs()
        recs.append([c[k] for k in GOLD_COEFFS])
        cs.append([c["time"], math.sqrt(c["cs2"])])
        ct.append([c["time"], math.sqrt(c["ct2"])])
        if s % entry["niter_r"] == 0:
            state = {nm: o.array(nm).copy() for nm in restart.STATE_3D}
        if s == entry["steps_before"]:
            o.post_begin()
    assert o.post_steps() == entry["steps_post"]
    np.testing.assert_allclose(np.array(recs), data["COEFFS"], rtol=1e-11, atol=1e-11)
    np.testing.assert_allclose(np.array(cs), data["CS"], rtol=1e-11, atol=1e-14)
    np.testing.assert_allclose(np.array(ct), data["CT"], rtol=1e-11, atol=1e-14)

    def close(got, ref, nm):
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), nm

    for col, nm in ((3, "P_AVG"), (4, "U_AVG"), (5, "V_AVG"), (6, "W_AVG"), (7, "T_AVG")):
        close(_nodal(o.post_get(nm), g), data["AVRG"][:, col], nm)
    for col, nm in ((3, "U_RMS"), (4, "V_RMS"), (5, "W_RMS")):
        close(_nodal(o.post_get(nm), g), data["URMS"][:, col], nm)
    for col, nm in ((3, "UU"), (4, "UV"), (5, "UW"), (6, "VV"), (7, "VW"), (8, "WW")):
        close(_nodal(o.post_get(nm), g), data["STRS"][:, col], nm)
    for col, nm in ((4, "CF_WALL"), (5, "CP_WALL"), (6, "NU_WALL")):
        w = o.post_get(nm)
        close(np.array([w[k, j] for k in range(1, g.nk) for j in range(1, g.nj)]), data["SURF"][:, col], nm)
    # the reference's one write past THETA's end is the only dropped write
    assert data["OOB_WRITES"].tolist() == [[g.ni + 1, g.nj + 1, g.nk + 1]]
    # RESTART000.DAT: the state of the last multiple of NITER_R, and this package's
    # writer reproduces the reference's E24.16 fields
    head = data["RESTART_HEAD"]
    assert head[4] == entry["niter_r"] * (len(recs) // entry["niter_r"])
    for q, nm in enumerate(("NLX", "NLY", "NLZ", "ADV")):
        close(state[nm].ravel(), data["RESTART_NL"][:, q], nm)
    for q, nm in enumerate(("U", "V", "W", "P", "T")):
        close(state[nm].ravel(), data["RESTART_STATE"][:, q], nm)
    path = tmp_path / "RESTART000.DAT"
    restart.write_restart_3d(str(path), state, head[0], head[1], head[2], head[3], int(head[4]))
    h, back = restart.read_restart_3d(str(path), g.ni, g.nj, g.nk)
    assert h["niter_time"] == int(head[4]) and h["rtime"] == float(restart.format_e(head[3]).replace("E", "e"))
    for nm in restart.STATE_3D:
        ref16 = np.vectorize(lambda x: restart._num(restart.format_e(x)))(state[nm])
        assert np.array_equal(back[nm], ref16), nm
