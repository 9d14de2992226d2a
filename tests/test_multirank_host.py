"""The N > 1 path of bench.py on CPU with gloo, world size 2: each rank
builds its own scenarios (disjoint seeds: weak scaling, no exchange on the
data path) and the job's throughput is the sum of the ranks' cell-updates
over the slowest rank's time."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        import braids_hkt_gb300.scenarios as S
        seconds = [2.5, 3.0][rank]
        updates = [1000, 2345][rank]
        t, u = bench.aggregate(seconds, updates, dist, "cpu")
        params = S.config4_params(64, seed=4 + rank)
        out.put((rank, t, u, [p["cells"] for p in params]))
    finally:
        dist.destroy_process_group()


def test_two_ranks_aggregate_and_shard():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    results = dict((r, (t, u, cells)) for r, t, u, cells in (out.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        t, u, _ = results[r]
        assert t == 3.0 and u == 3345                 # slowest rank, summed work
    assert len(results[0][2]) == len(results[1][2]) == 64
    assert results[0][2] != results[1][2]             # each rank its own scenarios


def test_single_rank_passthrough():
    import bench
    assert bench.aggregate(1.5, 42) == (1.5, 42)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    """Under torchrun the reference arm's ranks other than 0 exit without work."""
    import bench
    monkeypatch.setenv("RANK", "1")
    assert bench.reference_arm(None) is None
