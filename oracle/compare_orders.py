"""The GPU order against the reference's order, on the CPU restatement.

The GPU runs the reference's algorithm with three changes (zebra line order,
periodic wrap across the branch cut inside sweeps and residuals, cyclic
circumferential predictor lines); the GPU-order restatement reproduces the FP64
GPU path to ~1e-13 (the parity tests and bench.py's vs_oracle).  This script runs
the 128 x 96 Re=100 case (first radial spacing 0.005, outer radius 50, dt 0.005,
seeded 1e-3 start, Poisson to the scaled-L1 tolerance 1e-10) in both orders of the
restatement for a number of steps and reports how far the drag and lift records of
the two orders drift apart, step by step.  It is test infrastructure: CPU only,
serial checker build for the reference's order, the OpenMP build for the GPU order.

    python oracle/compare_orders.py --steps 2000 --out orders.jsonl
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from fvm_gb300.grid import o_grid, perturbation  # noqa: E402

CASE = dict(n_theta=128, n_r=96, re=100.0, dt=0.005, resimax=1e-10, amp=1e-3, seed=0)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=50, help="print a summary every this many steps")
    ap.add_argument("--out", default=None, help="JSON lines: one record per step")
    args = ap.parse_args()
    c = CASE
    g = o_grid(c["n_theta"], c["n_r"])
    du, dv = perturbation(g.ni, g.nj, c["amp"], c["seed"])
    runs = {}
    for name, order, variant, res_every in (("reference_order", oracle.FAITHFUL, "check", 1),
                                            ("gpu_order", oracle.GPU, "par", 8)):
        o = oracle.Oracle(g.ni, g.nj, re=c["re"], dt=c["dt"], order=order, resimax=c["resimax"], nswpp=10 ** 7,
                          thermal=False, res_every=res_every, variant=variant)
        o.set_grid(g.xg, g.yg)
        o.init(du, dv)
        runs[name] = o
    out = open(args.out, "w") if args.out else None
    worst = {"cd": 0.0, "cl": 0.0}
    t0 = time.perf_counter()
    for s in range(1, args.steps + 1):
        rec = {"step": s}
        for name, o in runs.items():
            o.step(1)
            co = o.coeffs()
            rec[name] = {k: co[k] for k in ("time", "cd", "cl", "sweeps", "resid")}
        a, b = rec["reference_order"], rec["gpu_order"]
        rec["cd_rel"] = abs(b["cd"] - a["cd"]) / abs(a["cd"])
        rec["cl_abs"] = abs(b["cl"] - a["cl"])
        worst["cd"] = max(worst["cd"], rec["cd_rel"])
        worst["cl"] = max(worst["cl"], rec["cl_abs"])
        if out:
            out.write(json.dumps(rec) + "\n")
            out.flush()
        if s % args.every == 0 or s == args.steps:
            ua, ub = runs["reference_order"].array("U"), runs["gpu_order"].array("U")
            urel = float(np.linalg.norm(ub - ua) / np.linalg.norm(ua))
            print(json.dumps({"step": s, "time": a["time"], "cd": [a["cd"], b["cd"]], "cd_rel": rec["cd_rel"],
                              "max_cd_rel_so_far": worst["cd"], "max_cl_abs_so_far": worst["cl"],
                              "u_rel_l2": urel, "sweeps": [a["sweeps"], b["sweeps"]],
                              "elapsed_s": round(time.perf_counter() - t0, 1)}), flush=True)


if __name__ == "__main__":
    main()
