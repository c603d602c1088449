"""Generate the golden fixtures by running the reference's own Fortran sources.

Usage (only where the reference tree exists):
    python tests/golden/make_golden.py /root/reference

For each case the R2D snapshot (cylinder/cylinder_v3.0.3_AF_original 4step_face_nl)
is executed by ftn_interp with NI, NJ (and where stated NSWPP, RESIMAX) replaced in
ComDat_Param; the grid file that GRID reads is served from fvm_gb300.grid; the
values Main.f90 reads from standard input (restart flag, Re, Pr, rotation, dt) are
fed in.  Main's statements up to CALL INIT run once, then the statements between
label 777 and the time-loop test run once per step.  Saved: U, V, P, T and the
NLX/NLY/ADV history after the last step, and every record CALCCOEF appends to
NU_CD_CL.PLT (time, Nu, Cd, Cl, Cpb, Cd_p, Cd_v, Cl_p, Cl_v, CFL).
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
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    manifest = []
    for c in CASES:
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
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py (reference sources executed by ftn_interp)",
                   "cases": manifest}, f, indent=1)


if __name__ == "__main__":
    main()
