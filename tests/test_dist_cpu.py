"""The multi-process host logic of bench.py on CPU (gloo, two ranks): the
frequency shards are disjoint and cover the sweep, the timing barrier and the
max-over-ranks reduction work across processes.  No GPU involved."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")  # gloo even where GPUs exist
    import bench
    dist, r, ws, local = bench._dist()
    try:
        assert dist is not None and dist.get_backend() == "gloo" and r == rank and ws == world
        mine = bench.shard_frequencies(r, ws, bench.N_FREQ)
        gathered = [None] * ws
        dist.all_gather_object(gathered, mine)
        bench._barrier(dist)
        top = bench._max_over_ranks(dist, float(10 * (rank + 1)), local)
        q.put((rank, gathered, top))
    finally:
        dist.destroy_process_group()


def test_two_rank_sharding_and_timing_reduction():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(world))
    import sys
    sys.path.insert(0, ROOT)
    import bench
    for rank, gathered, top in out:
        assert top == 20.0
        flat = sorted(k for shard in gathered for k in shard)
        assert flat == list(range(bench.N_FREQ))
        assert not set(gathered[0]) & set(gathered[1])
