"""The replica logic of bench.py over ranks, on CPU with the gloo backend
(world size 2, 127.0.0.1): the timed interval is the maximum and the work
the sum over the ranks, each rank seeds its own replica, and the reference
arm runs on rank 0 only (the other ranks return without work)."""
import os
import socket
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench

    t, c = bench.reduce_over_ranks(10.0 + rank, 100 * (rank + 1), world)
    rc = bench.run_reference(None) if rank != 0 else None
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, t, c, bench.replica_seed(rank), rc))


def test_replicas_over_two_gloo_ranks():
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
    (r0, t0, c0, s0, _), (r1, t1, c1, s1, rc1) = out
    assert (r0, r1) == (0, 1)
    assert t0 == t1 == 11.0          # the slower rank's interval
    assert c0 == c1 == 300           # walker-steps of both replicas
    assert s0 != s1                  # independent replicas
    assert rc1 == 0                  # the reference arm runs on rank 0 only


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_over_ranks(3.5, 42, 1) == (3.5, 42)
