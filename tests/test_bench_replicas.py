"""The multi-process path of bench.py on CPU: world size 2 over gloo
(127.0.0.1).  Replicas need no exchange step; the only cross-rank step is
the max over the ranks' times, and the reported throughput counts every
rank's units over that slowest time."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        assert bench.dist_env() == (ws, rank, rank)
        local_ms = [0.5, 0.75][rank]
        ms = bench.slowest_rank_ms(local_ms, ws, "cpu")
        out[rank] = (ms, bench.replica_throughput(2.0736, ms, ws))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    ws, port = 2, _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(ws, port, out), nprocs=ws, join=True)
        res = dict(out)
    assert res[0] == res[1]
    ms, v = res[0]
    assert ms == 0.75
    assert abs(v - 2 * 2.0736 / 0.75e-3) < 1e-6
