"""The N > 1 path on CPU: two `gloo` ranks (world size 2) run bench.py's rank logic -- the
environment, the barrier, the max over ranks of the step time that the whole-job rate is made
from -- and draw their own ensemble members (each rank runs an independent ensemble: replicas,
no per-step collective)."""

import multiprocessing as mp
import os
import socket
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))  # fmt: skip
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    from pydyn_gb300.ensemble import member_specs

    n, r, local = bench.dist_env()
    slowest = bench.max_over_ranks(0.1 * (r + 1), n)
    bench.barrier(n)
    rate = bench.sim_years_per_hour(slowest) * n  # the whole-job value of N replicas
    seeds = [s.member_seed for s in member_specs(seed=2024 + r)[:4]]
    out.put((r, n, local, slowest, rate, seeds))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, n0, l0, t0, v0, s0), (r1, n1, l1, t1, v1, s1) = got
    assert (r0, r1, n0, n1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert t0 == t1 == 0.2  # every rank reports the slowest rank's time
    assert v0 == v1
    assert set(s0).isdisjoint(s1)  # each rank's replica ensemble draws its own members
