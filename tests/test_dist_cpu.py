"""The multi-rank bench plumbing on the CPU: two gloo ranks (127.0.0.1) split the batched
workload's worlds between them and reduce their timings, as `bench.py --gpus N` does under
torchrun on GPUs (no GPU work here)."""
import os

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    from auto_gb300 import configs
    d = bench.Dist()
    worlds = configs.batched(384)
    mine = bench.shard(worlds, d.rank, d.world)
    cells = sum(worlds[i].cells_per_step for i in mine)
    total = d.sum(cells)
    slowest = d.max(float(rank + 1))
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    out.put((rank, mine, cells, total, slowest, gathered))
    d.barrier()
    d.close()


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in procs])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, a, ca, tot0, max0, g0), (r1, b, cb, tot1, max1, g1) = res
    assert set(a).isdisjoint(b) and sorted(a + b) == list(range(384))
    assert g0 == g1 == [a, b]
    assert tot0 == tot1 == ca + cb
    assert abs(ca - cb) / (ca + cb) < 0.02
    assert max0 == max1 == 2.0


def test_each_rank_sees_only_its_gpu(monkeypatch):
    """bench.pin_gpu: under torchrun each rank gets CUDA_VISIBLE_DEVICES = its own GPU, picked from an
    inherited list when there is one; a single process keeps its environment."""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    monkeypatch.setenv("WORLD_SIZE", "1")
    monkeypatch.setenv("LOCAL_RANK", "0")
    assert bench.pin_gpu() == 0 and "CUDA_VISIBLE_DEVICES" not in os.environ
    monkeypatch.setenv("WORLD_SIZE", "4")
    monkeypatch.setenv("LOCAL_RANK", "2")
    assert bench.pin_gpu() == 2 and os.environ["CUDA_VISIBLE_DEVICES"] == "2"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    assert bench.pin_gpu() == 6 and os.environ["CUDA_VISIBLE_DEVICES"] == "6"
