"""Sharding of ensemble members over ranks (host logic; gloo, world size 2, no GPU)."""
import os
import socket

import numpy as np
import torch.multiprocessing as tmp

from ufemism_gb300 import ensemble as ens
from ufemism_gb300 import workloads as wl


def test_partition_covers_every_member_once_and_balances():
    rows = 4 * wl.ensemble_sizes(256)
    costs = ens.member_cost(rows)
    for world in (1, 2, 3, 8):
        parts = ens.partition(costs, world)
        flat = sorted(m for p in parts for m in p)
        assert flat == list(range(256))
        loads = [costs[p].sum() for p in parts]
        # LPT bound: no rank exceeds the mean load by more than the largest single member
        assert max(loads) <= np.mean(loads) + costs.max() + 1e-9


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = ens.member_cost(4 * wl.ensemble_sizes(n))
    mine = ens.partition(costs, world)[rank]
    # stand-in for the solve: a result that names the rank that produced it
    local = {m: {"rank": rank, "value": float(m) * 2.0} for m in mine}
    merged = ens.gather_results(local, world, rank)
    if rank == 0:
        q.put(merged)
    dist.destroy_process_group()


def test_gather_over_two_gloo_ranks():
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    n = 40
    procs = [ctx.Process(target=_worker, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert sorted(merged) == list(range(n))
    assert all(v["value"] == 2.0 * m for m, v in merged.items())
    assert {v["rank"] for v in merged.values()} == {0, 1}
