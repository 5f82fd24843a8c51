"""Host-side logic of multi-GPU runs, on CPU: the scene partition and the max-time /
sum-of-units aggregation over two gloo ranks."""
import os
import socket

import pytest

from fluids_gb300.replicas import aggregate, partition_scenes


def test_partition_is_complete_deterministic_and_balanced():
    import numpy as np
    rng = np.random.default_rng(0)
    counts = [int(round(np.exp(rng.uniform(np.log(2048), np.log(65536))))) for _ in range(256)]
    for world in (1, 2, 4, 8):
        parts = partition_scenes(counts, world)
        assert parts == partition_scenes(counts, world)
        flat = sorted(s for p in parts for s in p)
        assert flat == list(range(256))
        loads = [sum(counts[s] for s in p) for p in parts]
        assert max(loads) - min(loads) <= max(counts)
    with pytest.raises(ValueError):
        partition_scenes(counts, 0)


def test_aggregate_without_process_group():
    assert aggregate(1.5, 10) == (1.5, 10.0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t, u = aggregate(1.0 + rank, 100 * (rank + 1))
        parts = partition_scenes([5, 4, 3, 3, 2, 1], world)
        q.put((rank, t, u, parts[rank]))
    finally:
        dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [2.0, 2.0]
    assert [r[2] for r in res] == [300.0, 300.0]
    assert sorted(res[0][3] + res[1][3]) == [0, 1, 2, 3, 4, 5]
