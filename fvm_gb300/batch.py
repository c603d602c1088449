"""Sweeps of independent cylinder cases: seeded case sets with uneven grids and
Reynolds numbers, cost-balanced sharding of the cases over GPUs (one process per
GPU, no collective on the data path: each rank advances its own cases, the host
gathers the records at the end), and the batched run of one shard through
fvm_batch_* (all of a shard's cases advanced together, each sub-step one launch).

The reference runs one case per process (Main.f90:40-118); a sweep is a set of such
runs."""
from __future__ import annotations

import math
import time
from dataclasses import asdict, dataclass

import numpy as np


@dataclass(frozen=True)
class CaseSpec:
    """One case: O-grid of n_theta x n_r cells (grid law of fvm_gb300.grid.o_grid),
    flow parameters, and the seed of its initial perturbation."""
    n_theta: int
    n_r: int
    re: float
    dt: float = 0.004
    pr: float = 0.71
    vel_rot: float = 0.0
    amp: float = 1e-3
    seed: int = 0
    thermal: bool = False

    @property
    def cells(self) -> int:
        return self.n_theta * self.n_r


def sweep_cases(n=64, seed=0, dt=0.004, theta=(64, 256, 16), radial=(48, 192), re=(60.0, 300.0),
                thermal=False):
    """n seeded cases: theta cells uniform over {theta[0], theta[0]+theta[2], ...,
    theta[1]}, radial cells uniform over radial[0]..radial[1], Re log-uniform over
    re, one perturbation seed per case."""
    rng = np.random.default_rng(seed)
    thetas = np.arange(theta[0], theta[1] + 1, theta[2])
    out = []
    for k in range(n):
        nt = int(rng.choice(thetas))
        nr = int(rng.integers(radial[0], radial[1] + 1))
        r = float(math.exp(rng.uniform(math.log(re[0]), math.log(re[1]))))
        out.append(CaseSpec(n_theta=nt, n_r=nr, re=r, dt=dt, seed=seed * 1000 + k, thermal=thermal))
    return out


def case_cost(spec: CaseSpec) -> float:
    """Estimated work of one step: cells x Poisson sweeps, with the sweeps of the
    radial-line Gauss-Seidel growing with the circumferential line count (the
    direction it couples explicitly)."""
    return float(spec.cells) * spec.n_theta


def partition(costs, world: int):
    """Cases split over `world` ranks by longest-processing-time: cases in
    decreasing cost, each to the least-loaded rank (ties to the lower rank).
    Returns one sorted index list per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda k: (-costs[k], k))
    loads = [0.0] * world
    parts = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(k)
        loads[r] += costs[k]
    return [sorted(p) for p in parts]


def case_inputs(spec: CaseSpec):
    """Grid and initial perturbation of a case (host arrays shared by every
    implementation that runs it)."""
    from .grid import o_grid, perturbation
    g = o_grid(spec.n_theta, spec.n_r)
    du, dv = perturbation(g.ni, g.nj, spec.amp, spec.seed)
    return g, du, dv


def case_params(spec: CaseSpec, precision, resimax=1e-10, nswpp=100000, refine_sweeps=32, **extra):
    from . import capi
    from .grid import o_grid
    g = o_grid(spec.n_theta, spec.n_r)
    return capi.default_params(ni=g.ni, nj=g.nj, re=spec.re, pr=spec.pr, dt=spec.dt, vel_rot=spec.vel_rot,
                               resimax=resimax, nswpp=nswpp, thermal=int(spec.thermal), precision=precision,
                               refine_sweeps=refine_sweeps, **extra)


def build_batch(specs, precision, autotune_sweeps=20, tiles=None, **kw):
    """A capi.Batch of the cases with grids and initial states set; the line tiles
    are given or chosen by the autotuner (timed on the batch itself)."""
    from . import capi
    b = capi.Batch([case_params(s, precision, **kw) for s in specs])
    for ctx, s in zip(b.cases, specs):
        g, du, dv = case_inputs(s)
        ctx.set_grid(g.xg, g.yg)
    if tiles is not None:
        b.set_tiles(tiles)
    elif autotune_sweeps:
        b.autotune(autotune_sweeps)
    for ctx, s in zip(b.cases, specs):
        g, du, dv = case_inputs(s)
        ctx.init(du, dv)
    return b


def run_shard(specs, indices, steps, precision=None, **kw):
    """Advance the cases `indices` of specs by `steps` steps as one batch on this
    process's GPU; returns {case index: list of per-step coefficient records}."""
    from . import capi
    if not indices:
        return {}
    precision = capi.MIXED if precision is None else precision
    b = build_batch([specs[k] for k in indices], precision, **kw)
    recs = b.step(steps)
    out = {k: [recs[s][j] for s in range(steps)] for j, k in enumerate(indices)}
    b.close()
    return out


def run_sweep(specs, steps, runner=run_shard, **kw):
    """The whole sweep over all ranks of the process group (or this process alone):
    each rank runs its share (partition by case_cost), rank 0 gathers every case's
    records in case order and returns them; the other ranks return None."""
    from . import dist
    rank, world, _ = dist.rank_world()
    parts = partition([case_cost(s) for s in specs], world)
    t0 = time.perf_counter()
    mine = runner(specs, parts[rank], steps, **kw)
    elapsed = time.perf_counter() - t0
    gathered = _gather_to_root((mine, elapsed), rank, world)
    if rank != 0:
        return None
    recs, times = {}, []
    for part, t in gathered:
        recs.update(part)
        times.append(t)
    return {"records": [recs[k] for k in range(len(specs))], "partition": parts, "rank_seconds": times,
            "specs": [asdict(s) for s in specs]}


def _gather_to_root(obj, rank, world):
    if world == 1:
        return [obj]
    import torch.distributed as tdist
    out = [None] * world if rank == 0 else None
    tdist.gather_object(obj, out, dst=0)
    return out
