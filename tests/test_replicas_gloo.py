"""Host-side test of bench.py's replica path (world size 2, gloo on CPU): ranks set up
from the torchrun environment, meet at barriers, and the timed region is the max over
ranks; the whole-job value counts every rank's frames.  The IK path itself is not
sharded, so no collective touches the data."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    w, r, local = bench.dist_setup("gloo")
    bench.barrier(w)
    ms = 10.0 + 5.0 * r            # rank 1 is the slow one
    ms_max = bench.max_over_ranks(ms, w)
    frames, steps = 64, 3
    value = w * frames * steps / (ms_max * 1e-3)
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()
    q.put((r, w, local, ms_max, value))


def test_two_replicas_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    assert all(o[3] == 15.0 for o in out)                       # max over ranks
    assert all(abs(o[4] - 2 * 64 * 3 / 0.015) < 1e-6 for o in out)  # whole-job frames / s
