"""The 3-D LES configuration (256 x 192 x 48 O-grid, first radial spacing 0.001,
Re 3900, dt 0.002, seeded 5 % start, volume-averaged dynamic Smagorinsky, Poisson
capped at 200 sweeps) stepped by the CPU restatement in the reference's own order
(lexicographic line Gauss-Seidel, lagged ghosts), printing the CFL number and the
drag every few steps until the run ends or goes non-finite.  Test infrastructure:
it shows whether the reference's algorithm itself stays stable at this time step.

    python oracle/les3d_cfl_check.py --steps 700 --every 10
"""
from __future__ import annotations

import argparse
import json
import math
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from fvm_gb300.grid import o_grid_3d, perturbation_3d  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=700)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--nswpp", type=int, default=200)
    args = ap.parse_args()
    g = o_grid_3d(256, 192, 48, lz=math.pi, dr1=0.001)
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, 0.05, 0)
    o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=3900.0, pr=0.71, dt=0.002, order=oracle.O3_FAITHFUL, resimax=1e-10,
                        nswpp=args.nswpp, use_les=True, les_zavg=False, thermal=True,
                        ref_a=float(g.zg[g.nk, 1, 1] - g.zg[1, 1, 1]))
    o.set_grid(g)
    o.init(du, dv, dw)
    t0 = time.perf_counter()
    for s in range(1, args.steps + 1):
        try:
            o.step(1)
        except FloatingPointError as e:
            print(json.dumps({"step": s, "error": str(e), "elapsed_s": round(time.perf_counter() - t0, 1)}),
                  flush=True)
            return
        c = o.coeffs()
        if s % args.every == 0 or c["cfl"] > 1.0:
            print(json.dumps({"step": s, "time": c["time"], "cfl": c["cfl"], "cd": c["cd"], "cs2": c["cs2"],
                              "elapsed_s": round(time.perf_counter() - t0, 1)}), flush=True)


if __name__ == "__main__":
    main()
