"""The multi-GPU (replicas) measurement logic with two gloo ranks on the CPU:
each rank times its own volume, the job time is the maximum over ranks, the
throughput counts every rank's voxels, and ranks draw different volumes."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(WORLD_SIZE=str(world), RANK=str(rank), LOCAL_RANK=str(rank))
    from decaes_gb300 import replicas
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        w, r, lr = replicas.rank_info()
        replicas.barrier(w)
        ms = replicas.max_over_ranks(100.0 + 50.0 * r, w)     # rank 1 is the slow one
        value = replicas.aggregate_voxels_per_s(1000, ms, w, steps=2)
        q.put((r, w, lr, ms, value, replicas.replica_seed(7, r)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in res] == [0, 1] and all(r[1] == 2 for r in res) and [r[2] for r in res] == [0, 1]
    assert all(r[3] == pytest.approx(150.0) for r in res)            # max over ranks, seen by both
    assert all(r[4] == pytest.approx(2 * 1000 * 2 / 0.150) for r in res)
    assert res[0][5] != res[1][5]                                    # independent volumes


def test_single_rank_defaults(monkeypatch):
    from decaes_gb300 import replicas
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.rank_info() == (1, 0, 0)
    assert replicas.max_over_ranks(3.5, 1) == 3.5
    assert replicas.aggregate_voxels_per_s(2000, 1000.0, 1) == pytest.approx(2000.0)
