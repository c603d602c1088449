"""Generate the golden fixtures by running the reference's own Fortran sources.

Usage (only where the reference tree exists; its root directory is required):
    python tests/golden/make_golden.py REFERENCE_ROOT [--3d-only | --program-only]

For each case the R2D snapshot (cylinder/cylinder_v3.0.3_AF_original 4step_face_nl)
is executed by ftn_interp with NI, NJ (and where stated NSWPP, RESIMAX) replaced in
ComDat_Param; the grid file that GRID reads is served from fvm_gb300.grid; the
values Main.f90 reads from standard input (restart flag, Re, Pr, rotation, dt) are
fed in.  Main's statements up to CALL INIT run once, then the statements between
label 777 and the time-loop test run once per step.  Saved: U, V, P, T and the
NLX/NLY/ADV history after the last step, and every record CALCCOEF appends to
NU_CD_CL.PLT (time, Nu, Cd, Cl, Cpb, Cd_p, Cd_v, Cl_p, Cl_v, CFL).

The 3-D cases run the LES solver (LES/v2.3_LES-Reynolds stresses) the same way on
one rank (NDIMJ = NDIMK = 1; the MPI calls are served by ftn_interp's one-rank
stubs): GRID reads the node triples of fvm_gb300.grid.o_grid_3d from unit 10, the
seeded perturbation_3d is added to U, V, W after INIT, and the statements of the
time loop run once per step.  Saved: U, V, W, P, T, NLX, NLY, NLZ, ADV in
(NK+1, NJ+1, NI+1) order and the CALCCOEF records.  With USE_LES = 0 the
reference still writes YPLUS in CALCCOEF although INIT allocates it only for LES
(calccoef.f90:121, init.f90:79-81); the harness allocates it so that the run
proceeds (YPLUS is written, never read, on the path).
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import ftn_interp as F  # noqa: E402
from fvm_gb300.grid import o_grid  # noqa: E402

SNAPSHOT = os.path.join("cylinder", "cylinder_v3.0.3_AF_original 4step_face_nl")
FILES = ["comdat_param.f90", "comdat_shared.f90", "grid.f90", "metric.f90", "init.f90", "contra_vel.f90",
         "nl.f90", "dif.f90", "dif_diagonal.f90", "p_source.f90", "iter_u.f90", "iter_v.f90", "iter_p.f90",
         "lisolv.f90", "bcu.f90", "bcv.f90", "bcp.f90", "bct.f90", "iter_T.f90", "calccoef.f90", "calc_vor.f90",
         "writedata.f90", "post_process.f90", "Main.f90"]

CASES = [
    # the reference's own Poisson settings (RESIMAX=1e-4, NSWPP=20)
    dict(name="polar_32x16_re100_ref", n_theta=32, n_r=16, skew=0.0, re=100.0, pr=0.71, vel_rot=0.0, dt=0.005,
         steps=6, over={}),
    # non-orthogonal grid (non-zero cross terms) with a rotating wall
    dict(name="skew_32x16_re150_rot", n_theta=32, n_r=16, skew=0.35, re=150.0, pr=1.0, vel_rot=0.3, dt=0.004,
         steps=4, over={}),
    # Poisson converged far below the default tolerance
    dict(name="polar_16x12_re80_tight", n_theta=16, n_r=12, skew=0.0, re=80.0, pr=0.71, vel_rot=0.0, dt=0.005,
         steps=3, over={"NSWPP": 100000, "RESIMAX": 1e-12}),
]


# The whole 2-D program, time loop included: the loop runs to RTIME_MAX, POST_PROCESS
# (IPOST=0) switches the averaging on and the loop continues to RTIME_END, with the
# CALCCOEF post-processing block active; POST_PROCESS (IPOST=1) writes the averages.
# RESTART.DAT is written every NITER_R steps.
PROGRAM_CASES = [
    dict(name="program_32x16_re100_rot_post", n_theta=32, n_r=16, skew=0.0, re=100.0, pr=0.71, vel_rot=0.3,
         dt=0.005, steps_before=5, steps_post=8, niter_r=5),
]


def run_program_case(ref_root, c):
    g = o_grid(c["n_theta"], c["n_r"], skew=c["skew"])
    dt = c["dt"]
    # half-step margins keep the RTIME comparisons of Main.f90:118 away from ties
    over = {"NI": g.ni, "NJ": g.nj, "RTIME_MAX": (c["steps_before"] - 0.5) * dt,
            "RTIME_END": (c["steps_before"] + c["steps_post"] - 0.5) * dt, "NITER_R": c["niter_r"]}
    M = F.load_program(os.path.join(ref_root, SNAPSHOT), FILES, over)
    M.stdin = [0, c["re"], c["pr"], c["vel_rot"], dt]
    vals = []
    for j in range(1, g.nj + 1):
        for i in range(1, g.ni + 1):
            vals += [float(g.xg[j, i]), float(g.yg[j, i])]
    M.unit_in[10] = vals
    F.run_stmts(M, M.subs["__MAIN__"].body, None)
    out = {nm: M.g[nm].a[:, :, 0].T.copy() for nm in ("U", "V", "P", "T", "NLX", "NLY", "ADV")}

    def numeric(unit, skip):
        return np.array([r for r in M.unit_out.get(unit, [])[skip:]], dtype=np.float64)

    out["COEFFS"] = numeric(11, 1)        # NU_CD_CL.PLT
    out["POST"] = numeric(12, 1)          # POST_NU_CD_CL.PLT
    out["FINAL"] = numeric(13, 1)         # TIME_AVERAGED_RESULTS.DAT
    out["AVG_FIELD"] = numeric(41, 3)     # TIME-AVERAGED FIELD.PLT: x, y, u, v, P, vorticity, T
    r16 = M.unit_out.get(16, [])          # RESTART.DAT of the last multiple of NITER_R
    out["RESTART_HEAD"] = np.array(r16[0] + r16[1], dtype=np.float64)
    out["RESTART_NL"] = np.array(r16[2::2], dtype=np.float64)
    out["RESTART_STATE"] = np.array(r16[3::2], dtype=np.float64)
    return g, out


SNAPSHOT3D = os.path.join("LES", "v2.3_LES-Reynolds stresses")
FILES3D = ["comdat_param.f90", "comdat_shared.f90", "define.f90", "mpi_x.f90", "grid.f90", "metric.f90", "init.f90",
           "contra_vel.f90", "nl.f90", "dif.f90", "dif_diagonal.f90", "p_source.f90", "iter_u.f90", "iter_p.f90",
           "lisolv.f90", "bcu.f90", "bcp.f90", "bct.f90", "iter_t.f90", "test_filter.f90", "stress_tensor_dy.f90",
           "calccoef.f90", "main.f90"]
FIELDS3D = ["U", "V", "W", "P", "T", "NLX", "NLY", "NLZ", "ADV"]

CASES3D = [
    # the reference's own settings (LES on, NSWPP=20, RESIMAX=1e-4) on a skewed grid
    dict(name="les3d_12x8x6_re3900", n_theta=12, n_r=8, n_z=6, skew=0.2, re=3900.0, pr=0.71, dt=0.002, amp=0.05,
         seed=1, steps=3, use_les=1, over={}),
    # stronger skew, lower Reynolds number, unit Prandtl number
    dict(name="les3d_16x12x8_re1000_skew", n_theta=16, n_r=12, n_z=8, skew=0.3, re=1000.0, pr=1.0, dt=0.003,
         amp=0.05, seed=3, steps=2, use_les=1, over={}),
    # no SGS model, circular section
    dict(name="dns3d_12x8x6_re300_polar", n_theta=12, n_r=8, n_z=6, skew=0.0, re=300.0, pr=0.71, dt=0.004,
         amp=0.05, seed=2, steps=2, use_les=0, over={}),
]


# The whole 3-D program: the loop to RTIME_MAX, POST_PROCESS (IPOST=0), the loop to
# RTIME_END with the averaging of CALCCOEF, POST_PROCESS (IPOST=1) writing the
# averaged, rms, Reynolds-stress and wall files; RESTART000.DAT every NITER_R steps.
# DTIME_POST is set to DTIME (the reference switches the time step there).  After
# its last loops POST_PROCESS writes THETA(IE+1,JE+1,KE+1), one element past the
# array (post_process.f90:250, undefined in the compiled program): the interpreter
# drops that write and the fixture records it.
PROGRAM3D_CASES = [
    dict(name="program3d_12x8x6_re3900_post", n_theta=12, n_r=8, n_z=6, skew=0.2, re=3900.0, pr=0.71, dt=0.002,
         amp=0.05, seed=1, steps_before=3, steps_post=3, niter_r=4),
]


def run_program_case_3d(ref_root, c):
    import math
    from fvm_gb300.grid import o_grid_3d, perturbation_3d
    g = o_grid_3d(c["n_theta"], c["n_r"], c["n_z"], lz=math.pi, dr1=0.01, skew=c["skew"])
    dt = c["dt"]
    over = {"NI": g.ni, "NJ": g.nj, "NK": g.nk, "NDIMJ": 1, "NDIMK": 1, "RE": c["re"], "PR": c["pr"],
            "PE": c["re"] * c["pr"], "DTIME": dt, "DTIME_POST": dt, "RTIME_MAX": (c["steps_before"] - 0.5) * dt,
            "RTIME_END": (c["steps_before"] + c["steps_post"] - 0.5) * dt, "NITER_R": c["niter_r"]}
    M = F.load_program(os.path.join(ref_root, SNAPSHOT3D), FILES3D[:-1] + ["post_process.f90", "writedata.f90",
                                                                         "main.f90"], over)
    vals = []
    for k in range(1, g.nk + 1):
        for j in range(1, g.nj + 1):
            for i in range(1, g.ni + 1):
                vals += [float(g.xg[k, j, i]), float(g.yg[k, j, i]), float(g.zg[k, j, i])]
    M.unit_in[10] = vals
    main = M.subs["__MAIN__"].body
    k_init = next(k for k, s in enumerate(main) if s[0] == "call" and s[2] == "INIT")
    F.run_stmts(M, main[:k_init + 1], None)
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, c["amp"], c["seed"])
    for nm, dd in (("U", du), ("V", dv), ("W", dw)):
        M.g[nm].a[...] += dd.transpose(2, 1, 0)
    M.drop_oob_writes = True
    F.run_stmts(M, main[k_init + 1:], None)
    files = {name: recs for _, name, recs in M.archive}
    for u, recs in M.unit_out.items():
        files[M.units_open.get(u)] = recs

    def numeric(recs, skip):
        return np.array(recs[skip:], dtype=np.float64)

    out = {nm: M.g[nm].a.transpose(2, 1, 0).copy() for nm in FIELDS3D}
    out["COEFFS"] = numeric(files["NU_CD_CL.PLT"], 1)
    out["CS"] = numeric(files["CS.PLT"], 1)          # time, sqrt of the volume-averaged coefficient
    out["CT"] = numeric(files["CT.PLT"], 1)
    out["AVRG"] = numeric(files["Avrg000.PLT"], 3)   # x, y, z, p, u, v, w, T at the nodes
    out["URMS"] = numeric(files["Urms000.PLT"], 3)   # x, y, z, u_rms, v_rms, w_rms
    out["STRS"] = numeric(files["Strs000.PLT"], 3)   # x, y, z, uu, uv, uw, vv, vw, ww
    out["SURF"] = numeric(files["Surf000.PLT"], 3)   # x, y, z, theta, Cf, Cp, Nu at the wall cells
    r16 = files["RESTART000.DAT"]
    out["RESTART_HEAD"] = np.array(r16[0], dtype=np.float64)
    out["RESTART_NL"] = np.array(r16[1::2], dtype=np.float64)
    out["RESTART_STATE"] = np.array(r16[2::2], dtype=np.float64)
    out["OOB_WRITES"] = np.array([list(ix) for _, ix in M.oob_log], dtype=np.int64)
    return g, out


def run_case_3d(ref_root, c):
    import math
    from fvm_gb300.grid import o_grid_3d, perturbation_3d
    g = o_grid_3d(c["n_theta"], c["n_r"], c["n_z"], lz=math.pi, dr1=0.01, skew=c["skew"])
    over = {"NI": g.ni, "NJ": g.nj, "NK": g.nk, "NDIMJ": 1, "NDIMK": 1, "RE": c["re"], "PR": c["pr"],
            "PE": c["re"] * c["pr"], "DTIME": c["dt"], "USE_LES": c["use_les"]}
    over.update(c["over"])
    M = F.load_program(os.path.join(ref_root, SNAPSHOT3D), FILES3D, over)
    vals = []
    for k in range(1, g.nk + 1):          # grid.f90: one (x, y, z) record per node, I fastest
        for j in range(1, g.nj + 1):
            for i in range(1, g.ni + 1):
                vals += [float(g.xg[k, j, i]), float(g.yg[k, j, i]), float(g.zg[k, j, i])]
    M.unit_in[10] = vals
    main = M.subs["__MAIN__"].body
    k_init = next(k for k, s in enumerate(main) if s[0] == "call" and s[2] == "INIT")
    F.run_stmts(M, main[:k_init + 1], None)
    if M.g.get("YPLUS") is None:
        M.g["YPLUS"] = F.FArray([1, 1, 1], [1, g.nj - 1, g.nk - 1])
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, c["amp"], c["seed"])
    for nm, dd in (("U", du), ("V", dv), ("W", dw)):
        M.g[nm].a[...] += dd.transpose(2, 1, 0)
    k777 = next(k for k, s in enumerate(main) if s[1] == 777)
    kend = next(k for k, s in enumerate(main) if s[0] == "lif" and s[3] and s[3][0][0] == "goto")
    # the loop body without the output routines this restatement does not cover
    keep = set(M.subs)
    step = [s for s in main[k777:kend] if not (s[0] == "call" and s[2] not in keep and not s[2].startswith("MPI_"))]
    step[0] = ("assign", None) + step[0][2:] if step[0][0] == "assign" else ("nop", None)
    for _ in range(c["steps"]):
        F.run_stmts(M, step, None)
    out = {nm: M.g[nm].a.transpose(2, 1, 0).copy() for nm in FIELDS3D}
    recs = [r for r in M.unit_out.get(11, []) if r and not isinstance(r[0], str)]
    out["COEFFS"] = np.array(recs, dtype=np.float64)
    return g, out


def run_case(ref_root, c):
    g = o_grid(c["n_theta"], c["n_r"], skew=c["skew"])
    over = {"NI": g.ni, "NJ": g.nj}
    over.update(c["over"])
    M = F.load_program(os.path.join(ref_root, SNAPSHOT), FILES, over)
    M.stdin = [0, c["re"], c["pr"], c["vel_rot"], c["dt"]]
    vals = []
    for j in range(1, g.nj + 1):          # grid.f90:36-42: K, J, I loops, one pair per record
        for i in range(1, g.ni + 1):
            vals += [float(g.xg[j, i]), float(g.yg[j, i])]
    M.unit_in[10] = vals
    main = M.subs["__MAIN__"].body
    k_init = next(k for k, s in enumerate(main) if s[0] == "call" and s[2] == "INIT")
    F.run_stmts(M, main[:k_init + 1], None)
    k777 = next(k for k, s in enumerate(main) if s[1] == 777)
    kend = next(k for k, s in enumerate(main) if s[0] == "lif" and s[3] and s[3][0][0] == "goto")
    step = [s for s in main[k777:kend]]
    step[0] = ("assign", None) + step[0][2:]   # the label only marks the loop head
    for _ in range(c["steps"]):
        F.run_stmts(M, step, None)
    out = {nm: M.g[nm].a[:, :, 0].T.copy() for nm in ("U", "V", "P", "T", "NLX", "NLY", "ADV")}
    recs = [r for r in M.unit_out.get(11, []) if r and not isinstance(r[0], str)]
    out["COEFFS"] = np.array(recs, dtype=np.float64)
    return g, out


def main():
    pos = [a for a in sys.argv[1:] if not a.startswith("--")]
    if not pos or not os.path.isdir(pos[0]):
        sys.exit("usage: make_golden.py REFERENCE_ROOT [--3d-only | --program-only]  "
                 "(the root directory of the reference source tree)")
    ref_root = pos[0]
    only3d = "--3d-only" in sys.argv
    only_prog = "--program-only" in sys.argv
    manifest = []
    if only3d or only_prog:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest = json.load(f)["cases"]
    for c in ([] if (only3d or only_prog) else CASES):
        t0 = time.time()
        g, out = run_case(ref_root, c)
        fn = f"{c['name']}.npz"
        np.savez_compressed(os.path.join(HERE, fn), **out)
        manifest.append(dict(name=c["name"], file=fn, n_theta=c["n_theta"], n_r=c["n_r"], skew=c["skew"],
                             dr1=0.005, r_out=50.0, re=c["re"], pr=c["pr"], vel_rot=c["vel_rot"], dt=c["dt"],
                             steps=c["steps"], nswpp=int(c["over"].get("NSWPP", 20)),
                             resimax=float(c["over"].get("RESIMAX", 1e-4)), amp=0.0, seed=0,
                             fields=["U", "V", "P", "T", "NLX", "NLY", "ADV"], order=0, tol=1e-12))
        print(f"{c['name']}: {time.time() - t0:.1f} s, {len(out['COEFFS'])} coefficient records", flush=True)
    manifest_prog = []
    for c in ([] if only3d else PROGRAM_CASES):
        t0 = time.time()
        g, out = run_program_case(ref_root, c)
        fn = f"{c['name']}.npz"
        np.savez_compressed(os.path.join(HERE, fn), **out)
        manifest_prog.append(dict(c, file=fn, dr1=0.005, r_out=50.0, nswpp=20, resimax=1e-4))
        print(f"{c['name']}: {time.time() - t0:.1f} s, {len(out['POST'])} post records", flush=True)
    if only3d:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest_prog = json.load(f).get("program_cases", [])
    manifest_prog3d = []
    for c in ([] if only3d else PROGRAM3D_CASES):
        t0 = time.time()
        g, out = run_program_case_3d(ref_root, c)
        fn = f"{c['name']}.npz"
        np.savez_compressed(os.path.join(HERE, fn), **out)
        manifest_prog3d.append(dict(c, file=fn, dr1=0.01, lz="pi", nswpp=20, resimax=1e-4, use_les=1,
                                    ref_a=6.283185307))
        print(f"{c['name']}: {time.time() - t0:.1f} s", flush=True)
    if only3d:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest_prog3d = json.load(f).get("program_cases_3d", [])
    manifest3d = []
    if only_prog:
        with open(os.path.join(HERE, "manifest.json")) as f:
            manifest3d = json.load(f).get("cases3d", [])
    for c in ([] if only_prog else CASES3D):
        t0 = time.time()
        g, out = run_case_3d(ref_root, c)
        fn = f"{c['name']}.npz"
        np.savez_compressed(os.path.join(HERE, fn), **out)
        manifest3d.append(dict(name=c["name"], file=fn, n_theta=c["n_theta"], n_r=c["n_r"], n_z=c["n_z"],
                               skew=c["skew"], dr1=0.01, lz="pi", re=c["re"], pr=c["pr"], dt=c["dt"],
                               steps=c["steps"], nswpp=int(c["over"].get("NSWPP", 20)),
                               resimax=float(c["over"].get("RESIMAX", 1e-4)), amp=c["amp"], seed=c["seed"],
                               use_les=c["use_les"], ref_a=6.283185307, fields=FIELDS3D, tol=1e-12))
        print(f"{c['name']}: {time.time() - t0:.1f} s, {len(out['COEFFS'])} coefficient records", flush=True)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py (reference sources executed by ftn_interp)",
                   "cases": manifest, "program_cases": manifest_prog, "cases3d": manifest3d,
                   "program_cases_3d": manifest_prog3d}, f, indent=1)


if __name__ == "__main__":
    main()
