"""The N>1 path of bench.py (independent replicas): barrier and max-over-ranks
timing with world_size 2 over gloo on CPU, and the rank-0-only reporting."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    os.environ.update(WORLD_SIZE=str(ws), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    d, r, w, local = bench._dist()
    assert (r, w, local) == (rank, ws, rank)
    bench._barrier(d)
    t = bench._max_over_ranks(d, 1.0 + rank)        # per-rank wall time
    out[rank] = t
    # whole-job throughput: all ranks' steps over the slowest rank's time
    out[ws + rank] = 10 * w / t
    d.destroy_process_group()


def test_replicas_max_over_ranks_gloo():
    ws = 2
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(ws, _free_port(), out), nprocs=ws, join=True)
    assert out[0] == out[1] == 2.0
    assert out[2] == out[3] == 10.0
