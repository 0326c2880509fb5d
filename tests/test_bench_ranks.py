"""The multi-rank host logic of bench.py on CPU: two gloo ranks.

Each rank owns an independent ladder (its own seed), the job time is the
slowest rank's (all-reduce MAX) and the job rate counts every rank's updates.
No data-path collective exists to test: ladders share nothing.
"""

import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seed = bench.ladder_seed(rank)
        local_ms = 100.0 + 50.0 * rank
        job_ms = bench.max_over_ranks(local_ms, dist, "cpu")
        rate = bench.aggregate_rate(world, 1000, 10, job_ms)
        seeds = [None] * world
        dist.all_gather_object(seeds, seed)
        Path(out_dir, f"rank{rank}.txt").write_text(f"{seed} {job_ms} {rate} {sorted(seeds)}")
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_time_the_slowest_and_seed_apart(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    rows = [Path(tmp_path, f"rank{r}.txt").read_text().split(" ", 3) for r in range(world)]
    seeds = [int(r[0]) for r in rows]
    assert len(set(seeds)) == world
    assert all(float(r[1]) == 150.0 for r in rows)          # the slower rank's time
    assert all(float(r[2]) == pytest.approx(2 * 1000 * 10 / 150e6) for r in rows)
    assert rows[0][3] == rows[1][3]


def test_single_rank_helpers_need_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(12.5, None, "cpu") == 12.5
    assert bench.ladder_seed(0) == 42 + bench.L
    assert bench.aggregate_rate(1, 52428800, 300, 300 * 600.0) == pytest.approx(52428800 / 600e6)
