"""Host side of the batched ensemble: building seeded members in parallel, sharding members
over ranks (one GPU per rank, no collective on the data path), and gathering per-member
results on rank 0.

Members are independent solves, so a multi-GPU run partitions them by estimated cost (rows
x expected sweeps, greedy longest-processing-time first) and each rank solves its share in
its own persistent batched launch; the only communication is the final gather of results.
"""
from __future__ import annotations

import heapq
import os

import numpy as np


def member_cost(rows) -> np.ndarray:
    """Expected relative cost: rows x sweeps, the SOR sweep count growing about like the
    square root of the rows (the mesh's linear resolution)."""
    r = np.asarray(rows, dtype=np.float64)
    return r * np.sqrt(r)


def partition(costs, world: int) -> list[list[int]]:
    """Greedy LPT: members in decreasing cost, each to the currently lightest rank. Every
    member appears on exactly one rank; each rank's list is in member order."""
    costs = np.asarray(costs, dtype=np.float64)
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for m in np.argsort(-costs, kind="stable"):
        load, r = heapq.heappop(heap)
        out[r].append(int(m))
        heapq.heappush(heap, (load + float(costs[m]), r))
    return [sorted(x) for x in out]


def _build_one(args):
    n, seed = args
    from . import workloads as wl
    return wl.ensemble_member(n, seed)


def member_seed(index: int, seed0: int = 20261210) -> int:
    return seed0 + 1 + int(index)


def build_members(sizes, seeds, processes: int | None = None):
    """Seeded ensemble members (base, mesh, ssa_fields), built in a spawn-context process
    pool (call this before the first GPU call of the process)."""
    import multiprocessing as mp
    jobs = [(int(n), int(s)) for n, s in zip(sizes, seeds)]
    procs = processes or min(16, os.cpu_count() or 1)
    if procs <= 1 or len(jobs) < 4:
        return [_build_one(j) for j in jobs]
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.map(_build_one, jobs, chunksize=1)


def gather_results(local: dict, world: int, rank: int):
    """Gather {member: result} dicts on rank 0 (torch.distributed object gather; the
    process group's backend may be gloo or nccl). Returns the merged dict on rank 0, None
    elsewhere."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    parts = [None] * world if rank == 0 else None
    dist.gather_object(local, parts, dst=0)
    if rank != 0:
        return None
    merged = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise RuntimeError("member %d solved on two ranks" % k)
            merged[k] = v
    return merged
