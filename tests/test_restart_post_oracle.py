"""CPU tests of the post-processing phase and of the restart files.

The fixture `program_*` is the reference's whole 2-D program (time loop,
POST_PROCESS with IPOST=0 then 1, RESTART.DAT every NITER_R steps) executed from
its own sources by tests/golden/ftn_interp.py.  The oracle replays it: the
coefficient records, the POST_NU_CD_CL.PLT records, the final averages, the
time-averaged field file and the restart records must agree."""
import json
import os

import numpy as np
import pytest

import oracle
from fvm_gb300 import restart
from fvm_gb300.grid import o_grid

GOLD = os.path.join(os.path.dirname(__file__), "golden")
COEFF_KEYS = ("time", "nu", "cd", "cl", "cpb", "cd_p", "cd_v", "cl_p", "cl_v", "cfl")
POST_KEYS = ("time", "nu", "cd", "cl", "cl_amp", "cpb", "st", "rms_cd", "rms_cl")


def _program_cases():
    path = os.path.join(GOLD, "manifest.json")
    if not os.path.exists(path):
        return []
    return json.load(open(path)).get("program_cases", [])


def _replay(entry):
    g = o_grid(entry["n_theta"], entry["n_r"], dr1=entry["dr1"], r_out=entry["r_out"], skew=entry["skew"])
    o = oracle.Oracle(g.ni, g.nj, re=entry["re"], pr=entry["pr"], dt=entry["dt"], vel_rot=entry["vel_rot"],
                      order=oracle.FAITHFUL, resimax=entry["resimax"], nswpp=entry["nswpp"], thermal=True,
                      iter_t_bug=True)
    o.set_grid(g.xg, g.yg)
    o.init()
    coeffs, post, restart_state = [], [], None
    total = entry["steps_before"] + entry["steps_post"]
    for s in range(1, total + 1):
        o.step(1)
        c = o.coeffs()
        coeffs.append([c[k] for k in COEFF_KEYS])
        if s > entry["steps_before"]:
            r = o.post_record()
            post.append([r[k] for k in POST_KEYS])
        if s % entry["niter_r"] == 0:
            restart_state = {nm: o.array(nm).copy() for nm in restart.STATE_2D}
        if s == entry["steps_before"]:
            o.post_begin()     # POST_PROCESS, IPOST=0, after the loop reaches RTIME_MAX
    return g, o, np.array(coeffs), np.array(post), restart_state


@pytest.mark.parametrize("entry", _program_cases(), ids=lambda e: e["name"])
def test_post_processing_against_the_reference_program(entry):
    data = np.load(os.path.join(GOLD, entry["file"]))
    g, o, coeffs, post, restart_state = _replay(entry)
    np.testing.assert_allclose(coeffs, data["COEFFS"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(post, data["POST"], rtol=1e-12, atol=1e-12)
    fin, fields = o.post_final()
    np.testing.assert_allclose([fin[k] for k in POST_KEYS], data["FINAL"][0], rtol=1e-12, atol=1e-12)
    # TIME-AVERAGED FIELD.PLT: x, y, u, v, P, vorticity, T for J = 0..NJ, I = 0..NI
    avg = data["AVG_FIELD"]
    cols = {"X": o.array("X"), "Y": o.array("Y"), "U": fields["U"], "V": fields["V"], "P": fields["P"],
            "VOR": fields["VOR"], "T": fields["T"]}
    for q, nm in enumerate(("X", "Y", "U", "V", "P", "VOR", "T")):
        ref = avg[:, q]
        got = cols[nm].ravel()
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), nm
    # the extremum test fired in this window (rotating cylinder): St and the
    # lift amplitude are non-zero
    assert fin["st_last"] > 0 and fin["cl_amp_last"] > 0
    # the last RESTART.DAT: the state after the last multiple of NITER_R steps
    head = data["RESTART_HEAD"]
    assert head[:4].tolist() == [entry["re"], entry["pr"], entry["dt"], entry["vel_rot"]]
    nl, st = data["RESTART_NL"], data["RESTART_STATE"]
    for q, nm in enumerate(("NLX", "NLY", "ADV")):
        assert np.array_equal(nl[:, q], restart_state[nm].ravel()), nm
    for q, nm in enumerate(("U", "V", "P", "T")):
        assert np.array_equal(st[:, q], restart_state[nm].ravel()), nm


def test_calc_vor_of_solid_rotation():
    """u = -w y, v = w x has vorticity 2w in the interior of any grid."""
    g = o_grid(32, 16, skew=0.2)
    o = oracle.Oracle(g.ni, g.nj)
    o.set_grid(g.xg, g.yg)
    o.init()
    X, Y = o.array("X"), o.array("Y")
    o.array("U")[...] = -0.7 * Y
    o.array("V")[...] = 0.7 * X
    o.call("calc_vor")
    w = o.array("VOR")
    assert np.allclose(w[1:g.nj, 1:g.ni], 1.4, rtol=1e-12, atol=1e-12)
    assert np.array_equal(w[0, :], w[g.nj - 1, :]) and np.array_equal(w[g.nj, :], w[1, :])


def test_format_e_matches_fortran_edit_descriptor():
    assert restart.format_e(1.0) == "  0.1000000000000000E+01"
    assert restart.format_e(-0.5) == " -0.5000000000000000E+00"
    assert restart.format_e(0.0) == "  0.0000000000000000E+00"
    assert restart.format_e(123.456) == "  0.1234560000000000E+03"
    assert restart.format_e(2.5e-120) == "  0.2500000000000000-119"
    assert restart.format_e(0.9999999999999999999) == "  0.1000000000000000E+01"
    assert restart._num("0.2500000000000000-119") == 2.5e-120
    assert restart._num("1.5D-3") == 1.5e-3


def test_restart_2d_round_trip_is_exact(tmp_path):
    rng = np.random.default_rng(4)
    ni, nj = 9, 13
    st = {nm: rng.standard_normal((nj + 1, ni + 1)) * 10.0 ** rng.integers(-8, 8) for nm in restart.STATE_2D}
    path = tmp_path / "RESTART.DAT"
    restart.write_restart_2d(str(path), st, 100.0, 0.71, 0.005, 0.3, 1.25, 250)
    head, back = restart.read_restart_2d(str(path), ni, nj)
    assert head == dict(re=100.0, pr=0.71, dt=0.005, vel_rot=0.3, rtime=1.25, niter_time=250)
    for nm in restart.STATE_2D:
        assert np.array_equal(back[nm], st[nm]), nm


def test_restart_2d_reads_list_directed_forms(tmp_path):
    """Blank- or comma-separated values, D exponents and repeat counts."""
    ni, nj = 2, 2
    lines = ["  100.0D0, 0.71 5.0D-3 0.0", " 2.5 40"]
    for q in range((ni + 1) * (nj + 1)):
        lines.append(" 3*0.0")
        lines.append(f" {q}.0 , {q}.5D0 2*-1.0")
    path = tmp_path / "RESTART.DAT"
    path.write_text("\n".join(lines) + "\n")
    head, st = restart.read_restart_2d(str(path), ni, nj)
    assert head["dt"] == 5e-3 and head["niter_time"] == 40
    assert st["U"][1, 2] == 5.0 and st["V"][1, 2] == 5.5 and st["T"][2, 2] == -1.0 and st["NLX"].max() == 0.0


def test_restart_3d_round_trip_in_fixed_format(tmp_path):
    rng = np.random.default_rng(5)
    ni, nj, nk = 5, 7, 3
    shape = (nk + 1, nj + 1, ni + 1)
    st = {nm: rng.standard_normal(shape) for nm in restart.STATE_3D}
    path = tmp_path / "RESTART000.DAT"
    restart.write_restart_3d(str(path), st, 3900.0, 2769.0, 0.002, 0.5, 250)
    text = path.read_text().splitlines()
    assert len(text[0]) == 4 * 25 + 17 and all(len(t) in (100, 125) for t in text[1:])
    head, back = restart.read_restart_3d(str(path), ni, nj, nk)
    assert head["niter_time"] == 250 and head["pe"] == 2769.0
    for nm in restart.STATE_3D:
        assert np.allclose(back[nm], st[nm], rtol=1e-15, atol=0), nm
