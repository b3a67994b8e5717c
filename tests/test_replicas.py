"""Multi-GPU replica logic on CPU: two gloo ranks (127.0.0.1) time different
amounts of work; the job time is the max over ranks and the throughput counts
both ranks' units."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank)})
    from nalu_gb300 import replicas
    ws, r, local, dist = replicas.init_from_env("gloo")
    replicas.barrier(dist)
    seconds = 1.0 + rank  # rank 1 is the slow one
    tmax = replicas.max_over_ranks(dist, seconds)
    out[rank] = (ws, r, local, tmax, replicas.job_throughput(1000, 10, tmax, ws))
    replicas.barrier(dist)
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    assert sorted(out.keys()) == [0, 1]
    for rank in (0, 1):
        ws, r, local, tmax, thr = out[rank]
        assert (ws, r, local) == (2, rank, rank)
        assert tmax == 2.0
        assert thr == pytest.approx(2 * 1000 * 10 / 2.0)


def test_single_rank_defaults(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    from nalu_gb300 import replicas
    assert replicas.init_from_env()[:3] == (1, 0, 0)
    assert replicas.max_over_ranks(None, 3.5) == 3.5
