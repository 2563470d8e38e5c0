"""Host logic of the multi-GPU bench (replicas only) on CPU with a gloo process group of two
ranks: rank variables from the environment, the max over ranks of the timed region, the
whole-job MLUPS, and the reference arm running on rank 0 only."""

import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    r, w, local = bench.dist_env()
    dist.init_process_group("gloo", rank=r, world_size=w)
    ms = bench.max_over_ranks(10.0 + 5.0 * r, dist)       # rank 1 is the slow replica
    value = bench.aggregate_mlups(6_000_000, 400, w, ms)
    ref = bench.run_reference(None, r, w) if r != 0 else "rank0"
    dist.barrier()
    dist.destroy_process_group()
    out.put((r, w, local, ms, value, ref))


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, ms, value, ref) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert ms == 15.0                                   # the slowest rank's time
        assert value == pytest.approx(6_000_000 * 400 * 2 / 0.015 / 1e6)
    assert res[1][5] is None                                # reference arm: rank 0 only


def test_single_process_helpers():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.aggregate_mlups(1_000_000, 10, 1, 10.0) == pytest.approx(1000.0)
