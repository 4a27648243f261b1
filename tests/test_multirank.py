"""The multi-GPU bench logic (one process per GPU, weak scaling) on CPU
ranks over gloo: barrier, max-over-ranks timing and the whole-job value."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    ws_, rk, local = bench.dist_init(backend="gloo")
    assert (ws_, rk, local) == (ws, rank, rank)
    bench.barrier(ws_)
    t = 1.0 + rank                       # rank r took 1 + r seconds
    tmax = bench.max_over_ranks(t, ws_)
    out[rank] = (tmax, bench.aggregate_value(ws_, 10, tmax))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_ranks_gloo():
    import torch.multiprocessing as mp
    ws = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(ws, port, out), nprocs=ws, start_method="spawn", join=True)
    for r in range(ws):
        tmax, value = out[r]
        assert tmax == pytest.approx(2.0)
        assert value == pytest.approx(2 * 10 / 2.0)
