"""The N > 1 host logic of bench.py (replicas, no data-path collective) on
two gloo ranks on the CPU: the rank environment, the job time as the maximum
over ranks, the whole-job work as the sum, and the reference arm's other
ranks leaving without work."""
import argparse
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    cpu = torch.device("cpu")
    r, w, local = bench.dist_env()
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, cpu, w)
    sums = bench.sum_over_ranks([100 * (rank + 1), rank + 7], cpu, w)
    out = None
    if rank == 1:
        ns = argparse.Namespace(steps=1, warmup=0)
        out = bench.run_reference(ns)          # ranks other than 0 return at once
    torch.distributed.barrier()
    torch.distributed.destroy_process_group()
    q.put((rank, r, w, local, ms, sums, out))


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, (r, rr, w, local, ms, sums, out) in enumerate(res):
        assert (r, rr, w, local) == (rank, rank, 2, rank)
        assert ms == 15.0
        assert sums == [300, 15]
        assert out is None


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import torch
    import bench
    cpu = torch.device("cpu")
    assert bench.max_over_ranks(3.5, cpu, 1) == 3.5
    assert bench.sum_over_ranks([1, 2.0], cpu, 1) == [1, 2]
