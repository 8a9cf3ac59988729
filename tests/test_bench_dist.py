"""The multi-rank plumbing of bench.py on CPU: world size 2 over gloo.

bench.py runs replicas only (one independent peel per GPU, no collective on
the data path); the only cross-rank step is taking the maximum of the
per-rank timings before rank 0 reports.  That step is checked here with two
gloo ranks on 127.0.0.1.
"""
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        got = bench.max_over_ranks([1.0 + rank, 10.0 - rank, 3.5], w)
        dist.barrier()
        out.put((r, w, local, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    for r in res:
        assert r[3] == [2.0, 10.0, 3.5]


def test_max_over_ranks_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks([4.0, 2.0], 1) == [4.0, 2.0]
