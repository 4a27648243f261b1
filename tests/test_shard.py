"""Realisation sharding over ranks (CPU, gloo): the cell-count-balanced
partition of the batched workload's box list, and a two-rank run whose
host-gathered results equal the one-process run, every item computed once."""
import os
import socket
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from exshalos_gb300 import shard  # noqa: E402


def _batch_sizes():
    # the batched workload's draw: 256 boxes, nd uniform in {64, 96, 128, 192, 256}
    return np.random.default_rng(2024).choice([64, 96, 128, 192, 256], size=256)


def test_partition_covers_every_item_once_and_balances():
    nds = _batch_sizes()
    cost = nds.astype(np.int64) ** 3
    for n in (1, 2, 3, 4, 8, 300):
        parts, loads = shard.partition(nds, n)
        items = np.sort(np.concatenate([np.asarray(p, dtype=np.int64) for p in parts if p]))
        assert np.array_equal(items, np.arange(nds.size))
        assert sum(loads) == int(cost.sum())
        # greedy on sorted sizes: no rank exceeds another by more than the largest box
        assert max(loads) - min(loads) <= int(cost.max())
        assert parts == shard.partition(nds, n)[0]              # deterministic
    parts, loads = shard.partition(nds, 8)
    assert max(loads) <= 1.05 * sum(loads) / 8


def _fake_run(nds, seeds, log):
    log.extend(int(s) for s in seeds)
    return {"nh": nds * 1000 + seeds, "Pk": np.outer(seeds, np.arange(4)).astype(np.float32)}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from exshalos_gb300 import shard as sh
    dist.init_process_group("gloo")
    nds = np.random.default_rng(2024).choice([64, 96, 128, 192, 256], size=40)
    seeds = np.arange(100, 140)
    ran = []
    res, mine = sh.run_sharded(nds, seeds, lambda n, s: _fake_run(n, s, ran))
    out[rank] = (res["nh"].tolist(), res["Pk"].tolist(), sorted(ran), list(mine))
    dist.destroy_process_group()


def test_two_ranks_gather_equals_one_process():
    import torch.multiprocessing as mp
    nds = np.random.default_rng(2024).choice([64, 96, 128, 192, 256], size=40)
    seeds = np.arange(100, 140)
    alone, mine = shard.run_sharded(nds, seeds, lambda n, s: _fake_run(n, s, []))
    assert mine == list(range(40))
    ws = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(ws, _free_port(), out), nprocs=ws, start_method="spawn", join=True)
    ran_all = []
    for r in range(ws):
        nh, pk, ran, part = out[r]
        assert np.array_equal(nh, alone["nh"]) and np.array_equal(pk, alone["Pk"])
        assert ran == sorted(int(seeds[i]) for i in part)          # each rank ran its own part only
        ran_all += ran
    assert sorted(ran_all) == seeds.tolist()                       # every item exactly once
