"""The replica path of bench.py across processes: world_size-2 gloo ranks on the CPU reduce
their timings (max) and counts (sum), and the ranks' workloads use disjoint seeds."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times, counts = bench.reduce_over_ranks([1.0 + rank, 10.0 - rank], [100 * (rank + 1), 7], "cpu")
        q.put((rank, times, counts))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_max_time_and_sum_counts():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, counts in got:
        assert times == [2.0, 10.0]
        assert counts == [300.0, 14.0]


def test_single_process_reduction_is_identity():
    import bench
    assert bench.reduce_over_ranks([3.0, 4.0], [5], "cpu") == ([3.0, 4.0], [5.0])


def test_rank_workloads_use_disjoint_seeds(built):
    import bench
    a, _, _ = bench.workload(ions_per_job=1, seed0=bench.rank_seed0(0))
    b, _, _ = bench.workload(ions_per_job=1, seed0=bench.rank_seed0(1))
    sa, sb = {j.seed for j in a}, {j.seed for j in b}
    assert len(sa) == len(a) and not (sa & sb)
