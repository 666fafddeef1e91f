"""The multi-GPU path of bench.py on CPU: two gloo ranks (no GPU).  Each rank
sieves its own block of denominators (weak scaling, no data-path collective):
the blocks tile [1, world x per_rank] without overlap, and the step time
reported is the maximum over ranks."""

import json
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, per_rank, out_dir):
    sys.path.insert(0, str(ROOT))
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    first, last = bench.rank_block(rank, per_rank)
    blocks = [None] * world
    dist.all_gather_object(blocks, (first, last))
    slowest = bench.max_over_ranks(10.0 + rank, dist)
    dist.barrier()
    dist.destroy_process_group()
    (Path(out_dir) / f"rank{rank}.json").write_text(json.dumps({"blocks": blocks, "slowest": slowest}))


def test_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    world, per_rank = 2, 65536
    port = _free_port()
    mp.start_processes(_rank_main, args=(world, port, per_rank, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    for rank in range(world):
        seen = json.loads((tmp_path / f"rank{rank}.json").read_text())
        assert seen["blocks"] == [[1, per_rank], [per_rank + 1, 2 * per_rank]]
        assert seen["slowest"] == 10.0 + world - 1


def test_single_process_helpers():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.rank_block(0, 5_000_000) == (1, 5_000_000)
    assert bench.rank_block(3, 10) == (31, 40)
    assert bench.max_over_ranks(4.5, None) == 4.5


def test_site_counts_of_rank_blocks():
    # the whole job's reduced sites are the sum over the ranks' blocks
    import math

    import numpy as np

    sys.path.insert(0, str(ROOT))
    import bench

    limit = 100_000
    slow = np.ones(limit + 1, dtype=np.int8)
    composite = np.zeros(limit + 1, dtype=bool)
    for p in range(2, limit + 1):
        if not composite[p]:
            composite[p * p::p] = True
            slow[p::p] *= -1
            slow[p * p::p * p] = 0
    slow[0] = 0
    assert np.array_equal(bench.mobius(limit), slow)
    height, per_rank, world = 37, 30, 4
    total = 0
    for rank in range(world):
        first, last = bench.rank_block(rank, per_rank)
        brute = sum(1 for b in range(first, last + 1) for a in range(-height, height + 1)
                    if math.gcd(a, b) == 1)
        block = bench.reduced_sites(height, last, bench.mobius(last), first=first)
        assert block == brute
        total += block
    assert total == bench.reduced_sites(height, world * per_rank)
