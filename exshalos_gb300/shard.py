"""Realisations sharded over GPUs, one process per GPU.

The batched workload is a list of independent boxes of uneven size.  It is
split across the ranks by cell-count-balanced greedy bin packing (each box,
largest first, goes to the rank with the fewest cells so far; ties to the
lower rank), every rank runs its share through the batched runner on its own
GPU, and the per-realisation results (halo counts and binned spectra) are
gathered on the host in item order.  The boxes exchange nothing, so no
collective runs on the data path; the gather moves a few hundred bytes per
realisation between processes.  A single box is never split (replicas only).
"""
import heapq

import numpy as np


def partition(nds, n_ranks):
    """Items of each rank (ascending indexes) and each rank's cell count,
    for boxes of nds[i]^3 cells."""
    if n_ranks < 1:
        raise ValueError("n_ranks must be >= 1")
    cost = np.asarray(nds, dtype=np.int64) ** 3
    order = sorted(range(cost.size), key=lambda i: (-int(cost[i]), i))
    heap = [(0, r) for r in range(n_ranks)]
    parts = [[] for _ in range(n_ranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + int(cost[i]), r))
    loads = [int(cost[p].sum()) if p else 0 for p in parts]
    return [sorted(p) for p in parts], loads


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def run_sharded(nds, seeds, run):
    """Run `run(nds_part, seeds_part) -> {key: array with one row per item}`
    on this rank's part of the item list and return, on every rank, the
    results of all items in item order (host gather over torch.distributed;
    one process alone runs everything).  Also returns this rank's item
    indexes."""
    nds = np.asarray(nds, dtype=np.int64).ravel()
    seeds = np.asarray(seeds, dtype=np.int64).ravel()
    if nds.shape != seeds.shape:
        raise ValueError("nds and seeds must have the same length")
    dist = _dist()
    ws = dist.get_world_size() if dist else 1
    rank = dist.get_rank() if dist else 0
    parts, _ = partition(nds, ws)
    mine = parts[rank]
    local = run(nds[mine], seeds[mine]) if mine else None
    if dist:
        gathered = [None] * ws
        dist.all_gather_object(gathered, (mine, local))
    else:
        gathered = [(mine, local)]
    out = {}
    for idx, res in gathered:
        if res is None:
            continue
        for key, val in res.items():
            val = np.asarray(val)
            if key not in out:
                out[key] = np.zeros((nds.size,) + val.shape[1:], dtype=val.dtype)
            out[key][np.asarray(idx, dtype=np.int64)] = val
    return out, mine


def batch_run_sharded(k, P, nds, seeds, **kw):
    """lib.exshalos.batch_run over the ranks of the current process group
    (each rank on its own GPU): the results of every item on every rank."""
    from .lib import exshalos as _ext
    return run_sharded(nds, seeds, lambda n, s: _ext.batch_run(k, P, n, s, **kw))[0]
