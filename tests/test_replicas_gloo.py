"""The multi-process side of `bench.py --gpus N` on CPU: N independent replicas
coordinated over gloo with host scalars only (a barrier around the timed
region, the max of the per-rank times, the sum of the per-rank work); there is
no data-path collective.  World size 2, rendezvous on 127.0.0.1."""
import multiprocessing as mp
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank: int, port: int, q) -> None:
    os.environ.update(RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, REPO)
    import bench
    world, r, local, dist = bench.dist_setup(2)
    try:
        bench.barrier(dist)
        t_max = bench.allreduce_max(dist, 1.0 + r)            # per-rank time of the timed region
        work = bench.allreduce_sum(dist, 10.0 * (r + 1))      # per-rank DOF-iterations
        bench.barrier(dist)
        # the reference arm runs on rank 0 alone; the other ranks return at once
        class A:
            pass
        rc = bench.run_reference(A(), world, r, dist) if r != 0 else 0
        q.put((r, world, local, t_max, work, rc))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_host_scalars():
    pytest.importorskip("torch.distributed")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        out = sorted(q.get(timeout=120) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert out == [(0, 2, 0, 2.0, 30.0, 0), (1, 2, 1, 2.0, 30.0, 0)]
    assert all(p.exitcode == 0 for p in procs)
