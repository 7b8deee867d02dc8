"""The multi-GPU path is replicas only: one process per GPU, no data-path
collective; the harness takes a barrier, the maximum of the per-rank times
and the whole-job rate.  Tested here with two `gloo` ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

from effsc_gpu.replicas import Replicas, job_rate, replica_seed  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    rep = Replicas(backend="gloo")
    assert (rep.world, rep.rank) == (world, rank)
    rep.barrier()
    t = 10.0 + 5.0 * rank                   # this rank's time in ms
    mx = rep.max(t)
    total = rep.sum(rank + 1)
    seed = replica_seed(100, rank)
    out.put((rank, mx, total, seed, job_rate(1000, 4, world, mx)))
    rep.barrier()
    rep.close()


def test_two_gloo_replicas():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, total, seed, rate in res:
        assert mx == 15.0                   # the slowest rank's time on every rank
        assert total == 3.0
        assert rate == world * 4 * 1000 / 15e-3
    assert res[0][3] != res[1][3]           # each replica proves its own inputs


def test_single_process_needs_no_group():
    os.environ.pop("WORLD_SIZE", None)
    rep = Replicas()
    assert rep.world == 1 and rep.max(3.5) == 3.5 and rep.sum(2) == 2.0
    rep.close()
