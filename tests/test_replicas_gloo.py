"""The replicas-only multi-GPU bookkeeping of bench.py on CPU ranks (gloo, world size 2): the job
time is the slowest rank's, and every rank solves its own seeded set of local-BA windows."""
import multiprocessing as mp
import os
import socket

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        import bench
        slowest = bench.max_over_ranks(10.0 * (rank + 1), world)
        q.put((rank, slowest, bench.window_seed(rank)))
    finally:
        dist.destroy_process_group()


def test_job_time_is_the_slowest_rank_and_windows_are_sharded():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [slowest for _, slowest, _ in out] == [20.0, 20.0]
    seeds = [seed for _, _, seed in out]
    assert len(set(seeds)) == 2


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
