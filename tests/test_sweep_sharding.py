"""CPU tests of the sweep layer: seeded case sets, cost-balanced partition over
ranks, and a two-rank gloo run of a whole sweep (each rank runs its share with the
oracle as the runner, rank 0 gathers) against the same sweep in one process."""
import os
import pickle
import socket

import numpy as np
import pytest

import oracle
from fvm_gb300 import batch


def test_sweep_cases_are_seeded_and_in_range():
    a = batch.sweep_cases(64, seed=3)
    b = batch.sweep_cases(64, seed=3)
    assert a == b and len(a) == 64
    assert all(64 <= s.n_theta <= 256 and s.n_theta % 16 == 0 for s in a)
    assert all(48 <= s.n_r <= 192 and 60.0 <= s.re <= 300.0 and s.dt == 0.004 for s in a)
    assert len({s.seed for s in a}) == 64
    assert batch.sweep_cases(64, seed=4) != a


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_partition_is_complete_disjoint_and_balanced(world):
    specs = batch.sweep_cases(64, seed=0)
    costs = [batch.case_cost(s) for s in specs]
    parts = batch.partition(costs, world)
    flat = sorted(k for p in parts for k in p)
    assert flat == list(range(64))
    loads = [sum(costs[k] for k in p) for p in parts]
    assert max(loads) <= 1.10 * (sum(costs) / world) + max(costs) * (world > 16)
    assert batch.partition(costs, world) == parts          # deterministic


def oracle_runner(specs, indices, steps, **kw):
    """The CPU restatement as the per-rank runner (test stand-in for the GPU batch)."""
    out = {}
    for k in indices:
        s = specs[k]
        g, du, dv = batch.case_inputs(s)
        o = oracle.Oracle(g.ni, g.nj, re=s.re, pr=s.pr, dt=s.dt, vel_rot=s.vel_rot, order=oracle.GPU,
                          resimax=1e-8, nswpp=3000, thermal=s.thermal)
        o.set_grid(g.xg, g.yg)
        o.init(du, dv)
        recs = []
        for _ in range(steps):
            o.step(1)
            recs.append(dict(o.coeffs()))
        out[k] = recs
    return out


def small_specs():
    return batch.sweep_cases(6, seed=7, theta=(16, 32, 8), radial=(10, 14))


def _worker(rank, world, port, outdir):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from fvm_gb300 import dist
    dist.init("gloo")
    try:
        res = batch.run_sweep(small_specs(), 2, runner=oracle_runner)
        with open(os.path.join(outdir, f"rank{rank}.pkl"), "wb") as f:
            pickle.dump(res, f)
    finally:
        dist.finalize()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_gloo_sweep_matches_one_process(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    one = batch.run_sweep(small_specs(), 2, runner=oracle_runner)
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    r0 = pickle.load(open(tmp_path / "rank0.pkl", "rb"))
    r1 = pickle.load(open(tmp_path / "rank1.pkl", "rb"))
    assert r1 is None
    assert len(r0["partition"]) == 2 and all(r0["partition"])
    assert r0["specs"] == one["specs"]
    for a, b in zip(r0["records"], one["records"]):
        assert [x["cd"] for x in a] == [x["cd"] for x in b]
        assert [x["sweeps"] for x in a] == [x["sweeps"] for x in b]
    assert np.isfinite([x["cd"] for rec in r0["records"] for x in rec]).all()
