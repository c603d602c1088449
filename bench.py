#!/usr/bin/env python3
"""Throughput of the cylinder time step on GB300 (Mcell-steps/s).

Workload (one GPU): the 2-D Re=200 cylinder with passive temperature (Pr=0.71,
wall T=1, inflow T=0) on the 512 (theta) x 384 (r) O-grid, wall radius 0.5 to
50, first radial spacing 0.005 with the geometric ratio solved for the outer
radius, dt=0.002, uniform start with a seeded +-1e-3 perturbation.  The Poisson
iteration runs to the scaled-L1 tolerance 1e-10 under the reference's sweep cap
NSWPP, set to 2048 so that every step does the same, reported, amount of line
Gauss-Seidel work (both paths check the residual every 8 or 32 sweeps, which
divide the cap).  A step is one complete time step (Main.f90:48-114).

value: the mixed-precision path (FP32 zebra sweeps in FP64 refinement); the FP64
path is timed in the same run.  e2e: the same metric through the C-ABI with the
state uploaded from and downloaded to pinned host memory every step.

--impl reference times the CPU restatement of the reference in its own order
(line sweeps sequential, as the reference's; stencil loops on every host thread)
on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(name="cylinder2d-re200-thermal-512x384", n_theta=512, n_r=384, re=200.0, pr=0.71, dt=0.002,
                resimax=1e-10, nswpp=2048, thermal=1, amp=1e-3, seed=0, dr1=0.005, r_out=50.0,
                res_every=8, refine_sweeps=32)
METRIC = "Mcell-steps/s mixed vs FP64 GPU at <=1e-6 rel field error; adjoint/forward time"


def cells(w):
    return w["n_theta"] * w["n_r"]


def case_inputs(w):
    from fvm_gb300.grid import o_grid, perturbation
    g = o_grid(w["n_theta"], w["n_r"], dr1=w["dr1"], r_out=w["r_out"])
    du, dv = perturbation(g.ni, g.nj, w["amp"], w["seed"])
    return g, du, dv


# ---------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi every 100 ms in the background; only the samples that arrive
    inside a timed window (begin() .. end(), several windows allowed) count.  open()
    waits for the first sample, so that a short timed region does not start before
    the sampler does."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []          # (arrival time, csv line)
        self.windows = []
        self.t = None

    def open(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()
        t0 = time.monotonic()
        while not self.lines and time.monotonic() - t0 < 5.0 and self.proc.poll() is None:
            time.sleep(0.01)

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.monotonic(), ln.strip()))

    def begin(self):
        self.windows.append([time.monotonic(), None])

    def end(self):
        if self.windows and self.windows[-1][1] is None:
            self.windows[-1][1] = time.monotonic()

    def start(self):
        self.open()
        self.begin()

    def stop(self):
        self.end()
        return self.close()

    def close(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        inside = [ln for t, ln in self.lines if any(a <= t <= b for a, b in self.windows if b is not None)]
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in inside:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "timed_s": round(sum(b - a for a, b in self.windows if b is not None), 3)}


# ---------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------
# The Poisson loop of a step: "device" (a graph while node ends it, no host round trip
# per outer iteration) or "host" (the host replays the body until the control block
# reports completion; ncu lists only the kernels of this form).  Set from --poisson-loop.
POISSON_LOOP = {"mode": "device"}


def make_ctx(w, precision, device, g, du, dv):
    from fvm_gb300 import capi
    p = capi.default_params(ni=g.ni, nj=g.nj, re=w["re"], pr=w["pr"], dt=w["dt"], resimax=w["resimax"],
                            nswpp=w["nswpp"], thermal=w["thermal"], precision=precision,
                            res_every=w["res_every"], refine_sweeps=w["refine_sweeps"], adi_refine=2, device=device,
                            poisson_host_loop=1 if POISSON_LOOP["mode"] == "host" else 0)
    ctx = capi.Context(p)
    ctx.set_grid(g.xg, g.yg)
    ctx.init(du, dv)
    return ctx


def timed_steps(ctx, steps, flush, torch, ext):
    """Time `steps` steps one at a time with CUDA events on the context's stream,
    writing a buffer larger than L2 between steps (outside the events)."""
    total = 0.0
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(ext)
        ctx.step(1)
        b.record(ext)
        b.synchronize()
        total += a.elapsed_time(b)
    return total


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline(w, g, du, dv, steps=3):
    """Serial CPU restatement (reference order) on a bounded sample: the first
    `steps` steps of the same workload, timing build of the restatement (-O3 with
    FMA contraction; portable flags, no -march=native)."""
    import oracle
    o = oracle.Oracle(g.ni, g.nj, re=w["re"], pr=w["pr"], dt=w["dt"], order=oracle.FAITHFUL,
                      resimax=w["resimax"], nswpp=w["nswpp"], thermal=bool(w["thermal"]), variant="fast")
    o.set_grid(g.xg, g.yg)
    o.init(du, dv)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    sw = o.coeffs()["sweeps"]
    return {"value": cells(w) * steps / dt / 1e6, "unit": "Mcell-steps/s", "cores": 1, "kind": "port",
            "sample": f"first {steps} time steps of the same workload ({sw} Poisson sweeps in the last), "
                      f"serial restatement in the reference's lexicographic order (-O3, FMA contraction), "
                      f"{dt:.1f} s"}


def oracle_gpu_order(w, g, du, dv, steps):
    """The restatement in GPU order (zebra sweeps, periodic wrap, cyclic circumferential
    lines) over the same `steps` steps, sweep cap and residual interval as the FP64
    GPU path, on all host threads (the OpenMP build, bit-identical to the serial
    checker).  Returns the final fields, the last step's coefficients and the time."""
    import oracle
    o = oracle.Oracle(g.ni, g.nj, re=w["re"], pr=w["pr"], dt=w["dt"], order=oracle.GPU, resimax=w["resimax"],
                      nswpp=w["nswpp"], thermal=bool(w["thermal"]), res_every=w["res_every"], variant="par")
    o.set_grid(g.xg, g.yg)
    o.init(du, dv)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return {nm: o.array(nm).copy() for nm in ("U", "V", "P", "T")}, o.coeffs(), dt


def vs_oracle(res, ofields, oco, w):
    """rel-L2 of the fields and relative coefficient errors of each GPU path against
    the GPU-order restatement after the same steps."""
    import numpy as np
    ni, nj = w["n_r"] + 1, w["n_theta"] + 1

    def rel(a, b):
        a, b = a[1:nj, 1:ni], b[1:nj, 1:ni]
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    out = {}
    for path, r in res.items():
        out[path] = {"field_rel_l2": {nm: rel(r["fields"][nm], ofields[nm]) for nm in ("U", "V", "P", "T")},
                     "coeff_rel": {k: abs(r[k] - oco[k]) / abs(oco[k]) for k in ("cd", "cl", "nu")},
                     "sweeps": {"gpu": r["sweeps"], "oracle": oco["sweeps"]}}
    return out


def roofline_sweep(w, ms_per_colour, peaks, mixed, resident=False, layout=None):
    """Roofline of the Poisson sweep kernel from its measured time per zebra colour.
    Algorithmic bytes per colour (half the cells active):
    FP32 sweep: per active cell RF, ANf, ASf, invDf, faf, fbf read and DF written
    (28 B) plus the other colour's DF read once (4 B): 32 B x active cells.
    FP64 sweep: per active cell DIVDT, 4 cross-term weights, AN, AS, 3 factors read
    (80 B) and P written (8 B), plus the other colour's lagged P (8 B) and, for the
    second colour, its new P (8 B): 100 B x active cells on average.
    The per-colour kernels launch once per colour.  The resident kernel runs the
    refine_sweeps sweeps of a refinement interval in one launch with its lines'
    operands held on chip: its algorithmic bytes per launch are the same per-sweep
    figure times the sweeps it runs, so achieved = 32 B x cells / time per sweep."""
    n_active = cells(w) // 2
    if not ms_per_colour or ms_per_colour <= 0:
        return None
    per_colour = (32.0 if mixed else 100.0) * n_active
    achieved = per_colour / (ms_per_colour * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs") if peaks else None
    peak_src = "measured" if peak else "fallback"
    if not peak:
        peak = 6800.0
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "traffic": None, "kernel": "k_pois32" if mixed else "k_pois64",
           "avg_launch_us": ms_per_colour * 1e3, "bytes_per_launch": per_colour, "peak_source": peak_src}
    if resident:
        spl = w["refine_sweeps"]
        pairs = bool(layout) and layout.get("sweeps_per_exchange") == 2
        out.update({"kernel": "k_pois32_resident2" if pairs else "k_pois32_resident", "sweeps_per_launch": spl,
                    "avg_launch_us": 2 * ms_per_colour * 1e3 * spl, "bytes_per_launch": 2 * per_colour * spl,
                    "per_sweep_us": 2 * ms_per_colour * 1e3, "bytes_per_sweep": 2 * per_colour,
                    "note": "lines' factors, couplings, right-hand side and correction stay on chip for the "
                            "interval; one launch per refine_sweeps sweeps" +
                            ("; boundary lines exchanged once per two sweeps (three lines per block solved "
                             "again)" if pairs else ""),
                    "layout": layout})
    return out


def fp64_pipe(profile, kernel):
    """FP64-pipe figures of an FP64 kernel from a committed ncu summary
    (profiles/<profile>.json): the pipe's busy fraction of the active cycles — how
    close the kernel runs to GB300's FP64 issue rate — and FP64 instructions per
    active cell.  None when the summary is absent."""
    path = os.path.join(ROOT, "profiles", profile + ".json")
    try:
        k = json.load(open(path))["kernels"][kernel]
    except Exception:
        return None
    return {"pipe_busy_frac": k["fp64_pipe_busy_pct"] / 100.0, "fp64_instr_per_cell": k.get("fp64_instr_per_cell"),
            "source": f"profiles/{profile}.json (ncu, sm__pipe_fp64_cycles_active)"}


def run_ours(args):
    import numpy as np
    import torch
    from fvm_gb300 import capi, dist

    rank, world = dist.init("nccl")
    local = dist.rank_world()[2]
    torch.cuda.set_device(local)
    w = dict(WORKLOAD)
    g, du, dv = case_inputs(w)
    capi.load()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MiB > L2
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))

    res = {}
    parts = {"all": (("mixed", capi.MIXED), ("fp64", capi.FP64)), "mixed": (("mixed", capi.MIXED),),
             "fp64": (("fp64", capi.FP64),)}[args.parts]
    # one sampler over every timed region of this run (mixed, FP64, end to end)
    clk = ClockSampler(local)
    clk.open()
    for name, prec in parts:
        ctx = make_ctx(w, prec, local, g, du, dv)
        ext = torch.cuda.ExternalStream(ctx.stream_handle())
        ctx.step(args.warmup)
        ctx.timing_reset()
        dist.barrier()
        clk.begin()
        ms = timed_steps(ctx, args.steps, flush, torch, ext)
        clk.end()
        clocks = None
        dist.barrier()
        ms_max = dist.max_over_ranks(ms, device="cuda")
        tm = ctx.timing()
        # average launch time of the sweep kernel: CUDA events on the context's
        # stream around a replay of 200 zebra sweeps of the same kernel on the
        # state just reached (scratch arrays only)
        sweep_ms, sweep_launches = ctx.time_sweeps(200)
        hist = ctx.history(1)
        fields = {nm: ctx.get(nm).copy() for nm in ("U", "V", "P", "T")}
        res[name] = dict(ms=ms_max, timing=tm, clocks=clocks, sweeps=hist[0]["sweeps"], fields=fields,
                         cd=hist[0]["cd"], cl=hist[0]["cl"], nu=hist[0]["nu"], resid=hist[0]["resid"],
                         sweep_ms=sweep_ms, resident=(sweep_launches == 1), layout=ctx.resident_info())
        ctx.close()

    if args.parts != "all":   # profiling runs: one path only
        clk.close()
        nm = parts[0][0]
        if rank == 0:
            print(json.dumps({"metric": METRIC, "parts": nm, "ms_per_step": res[nm]["ms"] / args.steps,
                              "sweep_us": res[nm]["sweep_ms"] * 1e3}), flush=True)
        dist.finalize()
        return
    # e2e through the C-ABI with host buffers (mixed path)
    ctx = make_ctx(w, capi.MIXED, local, g, du, dv)
    ext = torch.cuda.ExternalStream(ctx.stream_handle())
    ctx.step(args.warmup)
    n = (g.ni + 1) * (g.nj + 1)
    host = [torch.empty(n, dtype=torch.float64, pin_memory=True) for _ in range(7)]
    ptrs = [h.data_ptr() for h in host]
    ctx.download_ptrs(ptrs)
    e2e_ms = 0.0
    dist.barrier()
    clk.begin()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(ext)
        ctx.upload_ptrs(ptrs)
        ctx.step(1)
        ctx.download_ptrs(ptrs)
        b.record(ext)
        b.synchronize()
        e2e_ms += a.elapsed_time(b)
    clk.end()
    clocks = clk.close()
    clocks["regions"] = "mixed, fp64 and e2e timed loops"
    dist.barrier()
    e2e_ms = dist.max_over_ranks(e2e_ms, device="cuda")
    ctx.close()

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    field_err = {nm: rel(res["mixed"]["fields"][nm], res["fp64"]["fields"][nm]) for nm in ("U", "V", "P", "T")}
    units = world * cells(w) * args.steps
    value = units / (res["mixed"]["ms"] * 1e-3) / 1e6
    fp64_value = units / (res["fp64"]["ms"] * 1e-3) / 1e6
    e2e_value = units / (e2e_ms * 1e-3) / 1e6
    roof = roofline_sweep(w, res["mixed"]["sweep_ms"], peaks, True, res["mixed"]["resident"],
                          res["mixed"]["layout"])
    roof64 = roofline_sweep(w, res["fp64"]["sweep_ms"], peaks, False)
    if roof64:
        roof64["fp64_issue"] = fp64_pipe("fp64_pipe_cylinder2d_512x384", "k_pois64")
        roof64["fp64_issue_residual"] = fp64_pipe("fp64_pipe_cylinder2d_512x384", "k_pres64")
    traffic_file = os.path.join(ROOT, "profiles", (roof["kernel"] if roof else "k_pois32") +
                                "_cylinder2d_512x384.json")
    if roof and os.path.exists(traffic_file):
        try:
            roof["traffic"] = json.load(open(traffic_file)).get("dram_bytes_per_launch")
        except Exception:
            roof["traffic"] = None

    out = {
        "metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["mixed"]["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
        "config": {"workload": w["name"], "grid": f"{w['n_theta']} theta x {w['n_r']} r cells",
                   "cells": cells(w), "re": w["re"], "pr": w["pr"], "dt": w["dt"],
                   "poisson": f"zebra line GS to scaled-L1 {w['resimax']:g}, cap NSWPP={w['nswpp']}",
                   "sweeps_per_step": res["mixed"]["sweeps"], "precision": "mixed: FP32 zebra sweeps in FP64 "
                   f"refinement every {w['refine_sweeps']} sweeps, FP32 predictor lines with 2 FP64 "
                   "defect-correction passes; state and metrics FP64, Poisson residual in double-float "
                   "(FP32 pairs) from the FP64 pressure",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "poisson_loop": POISSON_LOOP["mode"],
                   "l2": "256 MiB buffer written between timed steps (outside the events)"},
        "fp64": {"value": fp64_value, "ms_per_step": res["fp64"]["ms"] / args.steps,
                 "sweeps_per_step": res["fp64"]["sweeps"], "roofline": roof64},
        "mixed_vs_fp64": {"speedup": value / fp64_value, "field_rel_l2": field_err,
                          "cd_rel": abs(res["mixed"]["cd"] - res["fp64"]["cd"]) / abs(res["fp64"]["cd"])},
        "roofline": roof,
        "e2e": {"value": e2e_value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 7 * n * 8,
                "d2h_bytes_per_step": 7 * n * 8 + 96},
        "gpu_launches": int(res["mixed"]["timing"]["kernel_launches"]),
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(w, g, du, dv)
        # the GPU-order restatement over the same warm-up + timed steps: the parity
        # of both GPU paths at this configuration, and a second (labelled) CPU figure
        nst = args.warmup + args.steps
        ofields, oco, odt = oracle_gpu_order(w, g, du, dv, nst)
        out["vs_oracle"] = vs_oracle({"mixed": res["mixed"], "fp64": res["fp64"]}, ofields, oco, w)
        out["vs_oracle"]["steps"] = nst
        out["vs_oracle"]["oracle"] = (f"CPU restatement in GPU order, residual every {w['res_every']} sweeps, "
                                      f"cap {w['nswpp']}, the same {nst} steps from the same inputs")
        out["cpu_gpu_order_omp"] = {
            "value": cells(w) * nst / odt / 1e6, "unit": "Mcell-steps/s", "cores": host_threads(), "kind": "port",
            "sample": f"{nst} steps of the workload, restatement in GPU order (zebra sweeps of one colour and "
                      f"the stencil loops on {host_threads()} OpenMP threads), {odt:.1f} s; not the reference's "
                      f"order, reported beside the serial baseline"}
    elif rank == 0:
        out["cpu_baseline"] = None
    if rank == 0:
        print(json.dumps(out), flush=True)
    dist.finalize()


# ---------------------------------------------------------------------------------
# discrete adjoint: d(mean Cd over a window)/d(rotation, blowing) on the 128 x 96 grid
# ---------------------------------------------------------------------------------
ADJOINT = dict(name="adjoint-cylinder2d-re100-128x96", n_theta=128, n_r=96, re=100.0, pr=0.71, dt=0.005,
               resimax=1e-10, nswpp=100000, amp=1e-3, seed=0, dr1=0.005, r_out=50.0, window=100, ckpt=10,
               omega=0.0, blow_sigma=0.01)


def adjoint_measure(spinup, precision, device, fd_check=True, window=None, ckpt=None, fd_blow=0):
    """Spin-up, then the window forward alone and the adjoint call (its own
    forward pass, the recomputation of every segment and the reverse pass), both
    timed; the rotation gradient is compared with a central difference (h=1e-6) of
    the same solver when fd_check."""
    import numpy as np
    import torch
    from fvm_gb300 import capi
    a = dict(ADJOINT)
    if window:
        a["window"] = window
    if ckpt:
        a["ckpt"] = ckpt
    g, du, dv = case_inputs(a)
    p = capi.default_params(ni=g.ni, nj=g.nj, re=a["re"], pr=a["pr"], dt=a["dt"], resimax=a["resimax"],
                            nswpp=a["nswpp"], thermal=0, precision=precision, res_every=8, refine_sweeps=16,
                            device=device)
    ctx = capi.Context(p)
    ctx.set_grid(g.xg, g.yg)
    ctx.init(du, dv)
    blow = a["blow_sigma"] * np.random.default_rng(a["seed"]).standard_normal(g.nj - 1)
    ctx.set_controls(a["omega"], blow)
    t0 = time.perf_counter()
    ctx.step(spinup)
    torch.cuda.synchronize()
    print(f"adjoint workload: spin-up {spinup} steps {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
    start = {nm: ctx.get(nm) for nm in ("U", "V", "P", "T", "NLX", "NLY", "ADV")}

    def restore():
        ctx.upload(start["U"], start["V"], start["P"], start["T"], start["NLX"], start["NLY"], start["ADV"])

    def window_cd(omega, b=None):
        restore()
        ctx.set_controls(omega, blow if b is None else b)
        ctx.step(a["window"])
        return float(np.mean([h["cd"] for h in ctx.history(a["window"])]))

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    j_fwd = window_cd(a["omega"])
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    restore()
    ctx.set_controls(a["omega"], blow)
    t0 = time.perf_counter()
    J, dw, db = ctx.adjoint_drag_grad(a["window"], a["ckpt"])
    torch.cuda.synchronize()
    t_adj = time.perf_counter() - t0
    print(f"adjoint workload: window forward {t_fwd:.2f} s, adjoint {t_adj:.2f} s", file=sys.stderr, flush=True)
    out = {"J": J, "dJ_domega": dw, "dJ_dblow_norm": float(np.linalg.norm(db)), "forward_s": t_fwd,
           "adjoint_s": t_adj, "adjoint_over_forward": t_adj / t_fwd, "J_vs_forward": abs(J - j_fwd) / abs(j_fwd),
           "spinup_steps": spinup}
    if fd_check:
        h = 1e-6
        fd = (window_cd(a["omega"] + h) - window_cd(a["omega"] - h)) / (2 * h)
        out["fd_dJ_domega"] = fd
        out["rel_err_vs_fd"] = abs(dw - fd) / abs(fd)
    if fd_blow:
        # central differences of the same solver for the blowing speeds with the
        # largest gradients
        h = 1e-6
        ks = [int(k) for k in np.argsort(-np.abs(db))[:fd_blow]]
        errs = []
        for k in ks:
            bp, bm = blow.copy(), blow.copy()
            bp[k] += h
            bm[k] -= h
            fdk = (window_cd(a["omega"], bp) - window_cd(a["omega"], bm)) / (2 * h)
            errs.append({"j": k + 1, "adjoint": float(db[k]), "fd": fdk, "rel_err": abs(db[k] - fdk) / abs(fdk)})
        out["fd_dJ_dblow"] = errs
    out["window"] = a["window"]
    out["checkpoint_every"] = a["ckpt"]
    ctx.close()
    return out


def run_adjoint_bench(args):
    import torch
    from fvm_gb300 import capi, dist
    rank, world = dist.init("nccl")
    local = dist.rank_world()[2]
    torch.cuda.set_device(local)
    which = {"all": (("fp64", capi.FP64), ("mixed", capi.MIXED)), "fp64": (("fp64", capi.FP64),),
             "mixed": (("mixed", capi.MIXED),)}[args.parts]
    res = {nm: adjoint_measure(args.spinup, prec, local, window=args.window, ckpt=args.ckpt, fd_blow=args.fd_blow)
           for nm, prec in which}
    first = res[which[0][0]]
    a = dict(ADJOINT, window=first["window"], ckpt=first["checkpoint_every"])
    out = {"metric": METRIC, "workload": a["name"], "value": first["adjoint_over_forward"],
           "unit": "adjoint/forward time", "n_gpus": world, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": a["name"], "grid": f"{a['n_theta']} theta x {a['n_r']} r", "re": a["re"],
                      "dt": a["dt"], "window": a["window"], "checkpoint_every": a["ckpt"],
                      "spinup_steps": args.spinup, "poisson": f"scaled-L1 {a['resimax']:g}",
                      "controls": "rotation omega=0 and 128 blowing speeds ~ N(0, 0.01^2), seeded"},
           "fp64": res.get("fp64"), "mixed": res.get("mixed")}
    if rank == 0:
        print(json.dumps(out), flush=True)
    dist.finalize()


# ---------------------------------------------------------------------------------
# 3-D LES (include/fvm3d.h) on the 256 theta x 192 r x 48 z O-grid, FP64 and mixed
# ---------------------------------------------------------------------------------
LES3D = dict(name="les3d-re3900-256x192x48", n_theta=256, n_r=192, n_z=48, re=3900.0, pr=0.71, dt=0.002,
             dr1=0.001, amp=0.05, seed=0, resimax=1e-10, nswpp=200, res_every=4, refine_sweeps=20, zavg=0,
             thermal=1)
# the same case on a smaller grid, for ncu captures that replay kernels many times
LES3D_PROFILE = dict(LES3D, name="les3d-re3900-192x160x32", n_theta=192, n_r=160, n_z=32)
FIELDS3D = ("U", "V", "W", "P", "T", "NLX", "NLY", "NLZ", "ADV")


def les3d_inputs(w):
    import math
    from fvm_gb300.grid import o_grid_3d, perturbation_3d
    g = o_grid_3d(w["n_theta"], w["n_r"], w["n_z"], lz=math.pi, dr1=w["dr1"])
    du, dv, dw = perturbation_3d(g.ni, g.nj, g.nk, w["amp"], w["seed"])
    return g, du, dv, dw


def make_ctx3(w, precision, device, g, du, dv, dw):
    from fvm_gb300 import capi3d
    p = capi3d.default_params(ni=g.ni, nj=g.nj, nk=g.nk, re=w["re"], pr=w["pr"], dt=w["dt"], resimax=w["resimax"],
                              nswpp=w["nswpp"], use_les=1, les_zavg=w["zavg"], thermal=w["thermal"],
                              res_every=w["res_every"], refine_sweeps=w["refine_sweeps"], precision=precision,
                              ref_a=float(g.zg[g.nk, 1, 1] - g.zg[1, 1, 1]), device=device,
                              poisson_host_loop=1 if POISSON_LOOP["mode"] == "host" else 0)
    ctx = capi3d.Context3(p)
    ctx.set_grid(g)
    ctx.init(du, dv, dw)
    return ctx


def roofline_sweep3d(n_int, ms_per_launch, peaks, mixed):
    """Roofline of the 3-D Poisson line kernel from its average launch time (one
    colour = half the I lines).  Algorithmic bytes per active cell:
    FP32 (k3_line32): RF, the north and top couplings of its own lines and of the
    south and bottom neighbour lines (ANf, ATf: the operator is symmetric), invDf,
    faf, fbf read, DF written, the other colour's DF read once: 40 B (the two colour
    launches of a sweep share the coupling arrays, 8 B of the 40, through L2).
    FP64 (k3_line): SU, AN, AS, AT, AB, invD, fa, fb read, P written, the other
    colour's P read once: 80 B."""
    if not ms_per_launch or ms_per_launch <= 0:
        return None
    per_launch = (40.0 if mixed else 80.0) * (n_int // 2)
    achieved = per_launch / (ms_per_launch * 1e-3) / 1e9
    peak = peaks.get("hbm_gbs") if peaks else None
    src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "k3_line32" if mixed else "k3_line<fam 0>",
            "avg_launch_us": ms_per_launch * 1e3, "bytes_per_launch": per_launch, "peak_source": src}


def roofline3d_with_traffic(n_int, ms_per_launch, peaks):
    """The FP32 sweep's roofline with `traffic` from the committed ncu capture on the
    profiling grid, scaled to this grid by the active cells per launch (the
    capture's traffic is 1.08 x its algorithmic bytes, no re-reads)."""
    roof = roofline_sweep3d(n_int, ms_per_launch, peaks, True)
    path = os.path.join(ROOT, "profiles", "k3_line32_les3d_192x160x32.json")
    if roof and os.path.exists(path):
        try:
            prof = json.load(open(path))
            roof["traffic"] = prof["dram_bytes_per_launch"] * (n_int // 2) / prof["active_cells_per_launch"]
            roof["traffic_note"] = "ncu capture on the 192x160x32 grid, scaled by the active cells"
        except Exception:
            roof["traffic"] = None
    return roof


def cpu_baseline_3d(w, g, du, dv, dw, sweeps_gpu):
    """Serial CPU restatement (reference order) on a bounded sample: one step with
    the Poisson capped at 20 sweeps and one capped at 120 give the fixed cost of a
    step and the cost of one sweep; the rate is extrapolated to the GPU run's
    sweeps per step and labelled as such."""
    import oracle
    t = {}
    for cap in (20, 120):
        o = oracle.Oracle3D(g.ni, g.nj, g.nk, re=w["re"], pr=w["pr"], dt=w["dt"], order=oracle.O3_FAITHFUL,
                            resimax=w["resimax"], nswpp=cap, use_les=True, les_zavg=bool(w["zavg"]),
                            thermal=bool(w["thermal"]), ref_a=float(g.zg[g.nk, 1, 1] - g.zg[1, 1, 1]))
        o.set_grid(g)
        o.init(du, dv, dw)
        t0 = time.perf_counter()
        o.step(1)
        t[cap] = time.perf_counter() - t0
        del o
    per_sweep = max((t[120] - t[20]) / 100.0, 0.0)
    fixed = max(t[20] - 20 * per_sweep, 0.0)
    est = fixed + per_sweep * sweeps_gpu
    n_int = (g.ni - 1) * (g.nj - 1) * (g.nk - 1)
    return {"value": n_int / est / 1e6, "unit": "Mcell-steps/s", "cores": 1, "kind": "port",
            "sample": f"first step twice, Poisson capped at 20 and 120 sweeps ({t[20]:.1f} s, {t[120]:.1f} s): "
                      f"{fixed:.2f} s fixed + {per_sweep * 1e3:.1f} ms per sweep, extrapolated to "
                      f"{sweeps_gpu} sweeps per step; serial restatement in the reference's order"}


def run_les3d_bench(args):
    import numpy as np
    import torch
    from fvm_gb300 import capi, dist

    rank, world = dist.init("nccl")
    local = dist.rank_world()[2]
    torch.cuda.set_device(local)
    w = dict(LES3D_PROFILE if args.les3d_grid == "profile" else LES3D)
    g, du, dv, dw = les3d_inputs(w)
    n_int = (g.ni - 1) * (g.nj - 1) * (g.nk - 1)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    res = {}
    parts = {"all": (("mixed", capi.MIXED), ("fp64", capi.FP64)), "mixed": (("mixed", capi.MIXED),),
             "fp64": (("fp64", capi.FP64),)}[args.parts]
    for name, prec in parts:
        ctx = make_ctx3(w, prec, local, g, du, dv, dw)
        ext = torch.cuda.ExternalStream(ctx.stream_handle())
        t0 = time.perf_counter()
        ctx.step(args.warmup)
        print(f"les3d {name}: {args.warmup} warm-up steps {time.perf_counter() - t0:.1f} s", file=sys.stderr,
              flush=True)
        dist.barrier()
        clk = ClockSampler(local) if name == "mixed" else None
        if clk:
            clk.start()
        ms, sweeps = 0.0, []
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(ext)
            c = ctx.step(1)
            b.record(ext)
            b.synchronize()
            ms += a.elapsed_time(b)
            sweeps.append(c["sweeps"])
        clocks = clk.stop() if clk else None
        dist.barrier()
        ms = dist.max_over_ranks(ms, device="cuda")
        sweep_ms = ctx.time_sweeps(50)
        fields = {nm: ctx.get(nm) for nm in ("U", "V", "W", "P", "T")}
        res[name] = dict(ms=ms, sweeps=sweeps, clocks=clocks, cd=c["cd"], resid=c["resid"], sweep_ms=sweep_ms,
                         fields=fields, u_max=float(np.abs(fields["U"]).max()))
        print(f"les3d {name}: {ms / args.steps:.1f} ms/step, sweeps {sweeps}, sweep pair {sweep_ms * 1e3:.1f} us",
              file=sys.stderr, flush=True)
        ctx.close()
    if args.parts != "all":   # profiling runs: one precision only
        if rank == 0:
            nm = parts[0][0]
            print(json.dumps({"metric": METRIC, "workload": w["name"], "parts": nm,
                              "ms_per_step": res[nm]["ms"] / args.steps,
                              "sweep_pair_us": res[nm]["sweep_ms"] * 1e3}), flush=True)
        dist.finalize()
        return
    # e2e through the C-ABI with pinned host buffers (mixed path)
    ctx = make_ctx3(w, capi.MIXED, local, g, du, dv, dw)
    ext = torch.cuda.ExternalStream(ctx.stream_handle())
    ctx.step(args.warmup)
    # pinned host buffers handed straight to fvm3_upload_state / fvm3_download_state
    # (one DMA per array, one synchronisation per call)
    host = [torch.empty(ctx.n, dtype=torch.float64, pin_memory=True) for _ in FIELDS3D]
    ptrs = [h.data_ptr() for h in host]
    ctx.download_ptrs(ptrs)
    e2e_ms = 0.0
    dist.barrier()
    clk.begin()
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(ext)
        ctx.upload_ptrs(ptrs)
        ctx.step(1)
        ctx.download_ptrs(ptrs)
        b.record(ext)
        b.synchronize()
        e2e_ms += a.elapsed_time(b)
    clk.end()
    clocks = clk.close()
    clocks["regions"] = "mixed, fp64 and e2e timed loops"
    dist.barrier()
    e2e_ms = dist.max_over_ranks(e2e_ms, device="cuda")
    ctx.close()

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))

    units = world * n_int * args.steps
    value = units / (res["mixed"]["ms"] * 1e-3) / 1e6
    fp64_value = units / (res["fp64"]["ms"] * 1e-3) / 1e6
    nbytes = (g.ni + 1) * (g.nj + 1) * (g.nk + 1) * 8
    out = {
        "metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["mixed"]["ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32pair+f32", "data": "synthetic",
        "config": {"workload": w["name"], "grid": f"{w['n_theta']} theta x {w['n_r']} r x {w['n_z']} z cells",
                   "cells": n_int, "re": w["re"], "dt": w["dt"], "lz": "pi", "dr1": w["dr1"],
                   "les": "dynamic Smagorinsky, coefficient averaged over the volume (the reference's); the "
                          "z-averaged Lilly coefficient diverges with the reference's explicit SGS term at this dt "
                          "and wall spacing",
                   "poisson": f"red-black I-line GS to scaled-L1 {w['resimax']:g}, cap NSWPP={w['nswpp']}",
                   "sweeps_per_step": res["mixed"]["sweeps"],
                   "precision": f"mixed: FP32 red-black Poisson sweeps in FP64 refinement every "
                                f"{w['refine_sweeps']} sweeps; SGS model, DIF, NL, P_SOURCE, the AF right-hand "
                                "sides and predictor line solves in double-float (FP32 pairs, ~48-bit "
                                "significands); metrics, Poisson residual, divergence, CALCCOEF and the state "
                                "FP64",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "poisson_loop": POISSON_LOOP["mode"],
                   "l2": "256 MiB buffer written between timed steps (outside the events)"},
        "fp64": {"value": fp64_value, "ms_per_step": res["fp64"]["ms"] / args.steps,
                 "sweeps_per_step": res["fp64"]["sweeps"],
                 "roofline": dict(roofline_sweep3d(n_int, res["fp64"]["sweep_ms"] / 2, peaks, False) or {},
                                  fp64_issue=fp64_pipe("fp64_pipe_les3d_192x160x32", "k3_line"),
                                  fp64_issue_residual=fp64_pipe("fp64_pipe_les3d_192x160x32", "k3_pres"))},
        "mixed_vs_fp64": {"speedup": value / fp64_value,
                          "field_rel_l2": {nm: rel(res["mixed"]["fields"][nm], res["fp64"]["fields"][nm])
                                           for nm in ("U", "V", "W", "P", "T")},
                          "cd_rel": abs(res["mixed"]["cd"] - res["fp64"]["cd"]) / abs(res["fp64"]["cd"]),
                          "cd": {"mixed": res["mixed"]["cd"], "fp64": res["fp64"]["cd"]},
                          "u_max": {"mixed": res["mixed"]["u_max"], "fp64": res["fp64"]["u_max"]}},
        "roofline": roofline3d_with_traffic(n_int, res["mixed"]["sweep_ms"] / 2, peaks),
        "e2e": {"value": units / (e2e_ms * 1e-3) / 1e6, "unit": "Mcell-steps/s",
                "h2d_bytes_per_step": len(FIELDS3D) * nbytes, "d2h_bytes_per_step": len(FIELDS3D) * nbytes},
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_3d(w, g, du, dv, dw, int(np.mean(res["fp64"]["sweeps"])))
    if rank == 0:
        print(json.dumps(out), flush=True)
    dist.finalize()


# ---------------------------------------------------------------------------------
# sweep of 64 ragged cases (fvm_batch_*), sharded over the ranks by estimated cost
# ---------------------------------------------------------------------------------
SWEEP = dict(name="sweep64-ragged-mixed", n=64, seed=0, resimax=1e-10, nswpp=2048, refine_sweeps=32)


def run_sweep_bench(args):
    import numpy as np
    import torch
    from fvm_gb300 import batch, capi, dist

    rank, world = dist.init("nccl")
    local = dist.rank_world()[2]
    torch.cuda.set_device(local)
    sw = dict(SWEEP)
    specs = batch.sweep_cases(sw["n"], seed=sw["seed"])
    parts = batch.partition([batch.case_cost(s) for s in specs], world)
    mine = [specs[k] for k in parts[rank]]
    kw = dict(resimax=sw["resimax"], nswpp=sw["nswpp"], refine_sweeps=sw["refine_sweeps"], device=local)
    t0 = time.perf_counter()
    b = batch.build_batch(mine, capi.MIXED, autotune_sweeps=20, **kw)
    setup_s = time.perf_counter() - t0
    b.step(args.warmup)
    tl0 = b.timing()["kernel_launches"]
    dist.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(local)
    clk.start()
    t0 = time.perf_counter()
    recs = b.step(args.steps)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    clocks = clk.stop()
    dist.barrier()
    dt_max = dist.max_over_ranks(dt, device="cuda")
    launches = b.timing()["kernel_launches"] - tl0
    units = sum(s.cells for s in specs) * args.steps
    value = units / dt_max / 1e6
    sweeps = [r["sweeps"] for r in recs[-1]]
    tiles_used = list(b.tiles())
    # the same cases one by one (separate contexts, same tiles), rank 0 of a
    # single-GPU run: warm-up, then 2 timed steps per case
    one = None
    if world == 1:
        tiles = b.tiles()
        t_one, ones_equal = 0.0, True
        tk = dict(tile_r_warps=tiles[0], tile_r_m=tiles[1], tile_t_warps=tiles[2], tile_t_m=tiles[3])
        for k, s in enumerate(mine):
            ctx = capi.Context(batch.case_params(s, capi.MIXED, **kw, **tk))
            g, du, dv = batch.case_inputs(s)
            ctx.set_grid(g.xg, g.yg)
            ctx.init(du, dv)
            ctx.step(args.warmup)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            ctx.step(2)
            torch.cuda.synchronize()
            t_one += time.perf_counter() - t1
            ctx.close()
        one = {"value": sum(s.cells for s in mine) * 2 / t_one / 1e6, "unit": "Mcell-steps/s",
               "note": "same cases as independent contexts stepped one after another, 2 steps each"}
    # bit-identity of the batch with the same cases run one by one over the same
    # warm-up + timed steps (the first check_cases cases of this rank, the batch's tiles)
    check = None
    if args.check_cases > 0:
        tiles = b.tiles()
        tk = dict(tile_r_warps=tiles[0], tile_r_m=tiles[1], tile_t_warps=tiles[2], tile_t_m=tiles[3])
        nst = args.warmup + args.steps
        same, cases = True, []
        for k, s in enumerate(mine[:args.check_cases]):
            want = {nm: b.cases[k].get(nm) for nm in ("U", "V", "P")}
            ctx = capi.Context(batch.case_params(s, capi.MIXED, **kw, **tk))
            g, du, dv = batch.case_inputs(s)
            ctx.set_grid(g.xg, g.yg)
            ctx.init(du, dv)
            ctx.step(nst)
            eq = all(np.array_equal(ctx.get(nm), want[nm]) for nm in want)
            same = same and eq
            cases.append({"n_theta": s.n_theta, "n_r": s.n_r, "re": s.re, "bit_identical": eq})
            ctx.close()
        check = {"steps": nst, "cases": cases, "all_bit_identical": same,
                 "note": "the batch's fields after all its steps against the same cases stepped one by one "
                         "with the batch's tiles"}
    b.close()
    out = {"metric": METRIC, "workload": sw["name"], "value": value, "unit": "Mcell-steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt_max / args.steps,
           "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f64+f32",
           "data": "synthetic",
           "config": {"workload": sw["name"], "cases": len(specs), "cells": sum(s.cells for s in specs),
                      "grids": "theta cells uniform in {64..256} step 16, radial cells uniform in 48..192, "
                               "Re log-uniform in [60, 300], dt 0.004, seeded",
                      "poisson": f"zebra line GS to scaled-L1 {sw['resimax']:g}, cap NSWPP={sw['nswpp']}",
                      "sweeps_per_step": {"min": min(sweeps), "max": max(sweeps)},
                      "tiles": {"radial": tiles_used[:2], "circumferential": tiles_used[2:],
                                "chosen_by": "autotuner (timed on this batch)"},
                      "partition": [len(p) for p in parts],
                      "setup_s_rank": setup_s,
                      "l2": "inputs larger than L2 (about 0.5 GB of case state)"},
           "one_by_one": one, "batch_vs_one_by_one": check, "gpu_launches": int(launches), "clocks": clocks}
    if rank == 0:
        print(json.dumps(out), flush=True)
    dist.finalize()


# ---------------------------------------------------------------------------------
# acceptance on the 128 x 96 Re=100 case: mean Cd, rms Cl and St of the FP64 and the
# mixed path over whole shedding periods from the same developed state
# ---------------------------------------------------------------------------------
ACCEPT = dict(name="acceptance-cylinder2d-re100-128x96", n_theta=128, n_r=96, re=100.0, pr=0.71, dt=0.005,
              resimax=1e-10, nswpp=1000000, amp=1e-3, seed=0, dr1=0.005, r_out=50.0, res_every=8,
              refine_sweeps=32)


def shedding_stats(hist):
    """Mean Cd, rms Cl (about its mean) and the Strouhal number from the upward zero
    crossings of Cl - mean(Cl) (linear interpolation in time; D = U = 1) over a
    record list."""
    import numpy as np
    t = np.array([h["time"] for h in hist])
    cd = np.array([h["cd"] for h in hist])
    cl = np.array([h["cl"] for h in hist])
    c = cl - cl.mean()
    up = np.nonzero((c[:-1] < 0.0) & (c[1:] >= 0.0))[0]
    tc = t[up] + (t[up + 1] - t[up]) * (-c[up]) / (c[up + 1] - c[up])
    st = (len(tc) - 1) / (tc[-1] - tc[0]) if len(tc) >= 2 else float("nan")
    return {"cd_mean": float(cd.mean()), "cl_rms": float(np.sqrt(np.mean(c * c))), "st": float(st),
            "cl_amp": float(0.5 * (cl.max() - cl.min())), "periods": int(max(len(tc) - 1, 0))}


def run_acceptance(args):
    import numpy as np
    import torch
    from fvm_gb300 import capi, dist
    rank, world = dist.init("nccl")
    local = dist.rank_world()[2]
    torch.cuda.set_device(local)
    a = dict(ACCEPT)
    g, du, dv = case_inputs(a)

    def make(precision):
        p = capi.default_params(ni=g.ni, nj=g.nj, re=a["re"], pr=a["pr"], dt=a["dt"], resimax=a["resimax"],
                                nswpp=a["nswpp"], thermal=0, precision=precision, res_every=a["res_every"],
                                refine_sweeps=a["refine_sweeps"], adi_refine=2, device=local, poisson_host_loop=0)
        ctx = capi.Context(p)
        ctx.set_grid(g.xg, g.yg)
        return ctx

    # spin-up (mixed path) from the seeded start, one shedding period (~1212 steps) per
    # chunk, until the lift amplitude of two consecutive chunks agrees to 1 % (or the
    # time limit); the lift amplitudes of the chunks are reported
    per = 1212
    ctx = make(capi.MIXED)
    ctx.init(du, dv)
    amps, t0, sweeps = [], time.perf_counter(), []
    while True:
        ctx.step(per)
        h = ctx.history(per)
        cl = np.array([r["cl"] for r in h])
        amps.append(float(0.5 * (cl.max() - cl.min())))
        sweeps.append(float(np.mean([r["sweeps"] for r in h])))
        tnow = h[-1]["time"]
        print(f"acceptance spin-up: t={tnow:.1f} cl_amp={amps[-1]:.4f} sweeps/step={sweeps[-1]:.0f} "
              f"{time.perf_counter() - t0:.0f} s", file=sys.stderr, flush=True)
        if (tnow >= args.spinup_min and len(amps) >= 2 and amps[-1] > 0.05
                and abs(amps[-1] - amps[-2]) <= 0.01 * amps[-1]) or tnow >= args.spinup_max:
            break
    spin_s = time.perf_counter() - t0
    state = ctx.download(("U", "V", "P", "T", "NLX", "NLY", "ADV"))
    t_start = h[-1]["time"]
    ctx.close()

    # the window: the same number of steps from the same state in each precision
    steps = int(round(args.window_periods * per))
    res = {}
    for name, prec in (("mixed", capi.MIXED), ("fp64", capi.FP64)):
        c = make(prec)
        c.upload(state["U"], state["V"], state["P"], state["T"], state["NLX"], state["NLY"], state["ADV"])
        c.set_time(t_start)
        c.post_begin()
        clk = ClockSampler(local)
        clk.start()
        hist, t1, done = [], time.perf_counter(), 0
        while done < steps:
            n = min(1000, steps - done)
            c.step(n)
            hist += c.history(n)
            done += n
        torch.cuda.synchronize()
        wall = time.perf_counter() - t1
        clocks = clk.stop()
        post = c.post_get()
        st = shedding_stats(hist)
        res[name] = dict(st, post_record={k: post[k] for k in ("cd", "rms_cl", "st", "st_last", "cl_amp", "niter")},
                         sweeps_per_step=float(np.mean([r["sweeps"] for r in hist])),
                         max_resid=float(max(r["resid"] for r in hist)), ms_per_step=1e3 * wall / steps,
                         clocks=clocks)
        print(f"acceptance {name}: {wall:.0f} s, {json.dumps(st)}", file=sys.stderr, flush=True)
        c.close()
    rel = {k: abs(res["mixed"][k] - res["fp64"][k]) / abs(res["fp64"][k]) for k in ("cd_mean", "cl_rms", "st")}
    out = {"metric": "mean Cd, rms Cl, St: mixed vs FP64 GPU (bar 0.1 %)", "workload": a["name"],
           "config": {"grid": "128 theta x 96 r", "re": a["re"], "dt": a["dt"],
                      "poisson": f"scaled-L1 {a['resimax']:g} (no sweep cap in effect)",
                      "start": f"seeded {a['amp']:g} perturbation, spin-up on the mixed path until the lift "
                               f"amplitude of two consecutive {per}-step chunks agreed to 1 %",
                      "spinup": {"t_end": t_start, "chunk_cl_amp": amps, "sweeps_per_step": sweeps,
                                 "seconds": spin_s},
                      "window": {"steps": steps, "t": [t_start, t_start + steps * a["dt"]],
                                 "from": "the same downloaded state (U, V, P, NLX, NLY) in both precisions"}},
           "fp64": res["fp64"], "mixed": res["mixed"], "mixed_vs_fp64_rel": rel,
           "within_0.1_percent": bool(all(v <= 1e-3 for v in rel.values()))}
    if rank == 0:
        print(json.dumps(out), flush=True)
    dist.finalize()


# ---------------------------------------------------------------------------------
# reference arm
# ---------------------------------------------------------------------------------
def run_reference(args):
    from fvm_gb300 import dist
    rank, world, _ = dist.rank_world()
    if rank != 0:
        return
    import oracle
    w = dict(WORKLOAD)
    g, du, dv = case_inputs(w)
    # The reference's algorithm: lexicographic line Gauss-Seidel, sequential over the
    # lines; the OpenMP build runs its stencil loops on every host thread (results
    # bit-identical to the serial restatement).
    o = oracle.Oracle(g.ni, g.nj, re=w["re"], pr=w["pr"], dt=w["dt"], order=oracle.FAITHFUL,
                      resimax=w["resimax"], nswpp=w["nswpp"], thermal=bool(w["thermal"]), variant="par")
    o.set_grid(g.xg, g.yg)
    o.init(du, dv)
    # Each step is timed by sub-step so that a long run can sample fewer Poisson
    # sweeps per step and scale the Poisson part to the full sweep count.
    budget_s = 200.0
    est_step = None
    sample_sweeps = w["nswpp"]

    def one_step(nswpp_sample):
        t0 = time.perf_counter()
        for f in ("begin_step", "contra_vel", "explicit", "iter_u", "iter_v", "remove_grad"):
            o.call(f)
        t1 = time.perf_counter()
        sw = o.call("iter_p")
        t2 = time.perf_counter()
        o.call("correct")
        if w["thermal"]:
            o.call("iter_t")
        o.call("calccoef")
        t3 = time.perf_counter()
        return (t1 - t0) + (t3 - t2), t2 - t1, sw

    # the oracle reads its parameters at creation: rebuild with the sample cap when needed
    def rebuild(cap):
        nonlocal o
        o = oracle.Oracle(g.ni, g.nj, re=w["re"], pr=w["pr"], dt=w["dt"], order=oracle.FAITHFUL,
                          resimax=w["resimax"], nswpp=cap, thermal=bool(w["thermal"]), variant="par")
        o.set_grid(g.xg, g.yg)
        o.init(du, dv)

    t_fix, t_p, sw = one_step(w["nswpp"])   # probe step (counts as warm-up)
    est_step = t_fix + t_p
    total_steps = args.warmup + args.steps
    if total_steps * est_step > budget_s:
        sample_sweeps = max(20, int(w["nswpp"] * budget_s / (total_steps * est_step)))
        rebuild(sample_sweeps)
    for _ in range(max(0, args.warmup - 1)):
        one_step(sample_sweeps)
    tot = 0.0
    for _ in range(args.steps):
        tf, tp, swn = one_step(sample_sweeps)
        tot += tf + tp * (w["nswpp"] / max(swn, 1))
    value = cells(w) * args.steps / tot / 1e6
    sample = (f"CPU restatement, reference (lexicographic) order: line sweeps sequential as in the reference, "
              f"stencil loops on {host_threads()} OpenMP threads; {args.steps} steps of the workload"
              + ("" if sample_sweeps == w["nswpp"] else
                 f", Poisson sampled at {sample_sweeps} of {w['nswpp']} sweeps per step and scaled"))
    out = {"metric": METRIC, "value": value, "unit": "Mcell-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": w["name"], "cells": cells(w),
                      "poisson": f"line GS to scaled-L1 {w['resimax']:g}, cap NSWPP={w['nswpp']}"},
           "cpu_baseline": {"value": value, "unit": "Mcell-steps/s", "cores": host_threads(), "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--parts", choices=["all", "mixed", "fp64"], default="all",
                    help="'mixed' / 'fp64' time one precision only (profiler runs)")
    ap.add_argument("--workload", choices=["cylinder2d", "sweep64", "adjoint", "les3d", "acceptance"],
                    default="cylinder2d",
                    help="sweep64: 64 ragged cases advanced as batches, sharded over the ranks; "
                         "adjoint: window-drag gradient on the 128x96 grid; "
                         "les3d: 3-D LES on the 256x192x48 grid, FP64 and mixed")
    ap.add_argument("--spinup", type=int, default=200, help="adjoint workload: steps before the window")
    ap.add_argument("--window", type=int, default=0, help="adjoint: drag-averaging window in steps (0: 100)")
    ap.add_argument("--ckpt", type=int, default=0, help="adjoint: checkpoint interval in steps (0: 10)")
    ap.add_argument("--fd-blow", type=int, default=0,
                    help="adjoint: also check this many blowing components against central differences")
    ap.add_argument("--check-cases", type=int, default=0,
                    help="sweep64: compare this many cases with one-by-one runs of the same steps, bit for bit")
    ap.add_argument("--spinup-min", type=float, default=100.0, help="acceptance: earliest end of the spin-up (time)")
    ap.add_argument("--spinup-max", type=float, default=300.0, help="acceptance: latest end of the spin-up (time)")
    ap.add_argument("--window-periods", type=float, default=5.0,
                    help="acceptance: window length in shedding periods of ~1212 steps")
    ap.add_argument("--poisson-loop", choices=["device", "host"], default="device",
                    help="cylinder2d and les3d: the Poisson loop on the device (graph while node) or replayed by "
                         "the host (kernels listed by ncu)")
    ap.add_argument("--les3d-grid", choices=["full", "profile"], default="full",
                    help="les3d: the 256x192x48 grid, or 192x160x32 for profiler captures")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    POISSON_LOOP["mode"] = args.poisson_loop
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "sweep64":
        run_sweep_bench(args)
    elif args.workload == "adjoint":
        run_adjoint_bench(args)
    elif args.workload == "les3d":
        run_les3d_bench(args)
    elif args.workload == "acceptance":
        run_acceptance(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
