"""The bench's multi-process path on CPU (gloo, world size 2): each replica times
its own copy of the work, the ranks meet at a barrier, the slowest rank's time
is the job's time, and a failure of one rank is seen by the launcher."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, world, port, q, fail_rank):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_setup(world, backend="gloo")
    try:
        if rank == fail_rank:
            raise RuntimeError("replica failed before its timed steps")
        ms = 10.0 + 5.0 * r  # this replica's time per step
        bench.barrier(w)
        slowest = bench.max_over_ranks(ms, w)
        q.put((r, w, local, slowest))
    finally:
        if rank != fail_rank:
            dist.destroy_process_group()


def _run(world, fail_rank=-1, timeout=120):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_replica, args=(r, world, port, q, fail_rank)) for r in range(world)]
    for p in ps:
        p.start()
    out = []
    for p in ps:
        p.join(timeout)
    for p in ps:
        if p.is_alive():
            p.kill()
            p.join()
    while not q.empty():
        out.append(q.get())
    return sorted(out), [p.exitcode for p in ps]


def test_two_replicas_take_the_slowest_time():
    out, codes = _run(2)
    assert codes == [0, 0]
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(o[3] == 15.0 for o in out)  # max over the ranks, seen by both


@pytest.mark.timeout(300)
def test_failed_replica_is_reported():
    # rank 1 raises before the barrier: it exits non-zero, and rank 0 does not report
    # a job time without it (its barrier or all-reduce fails or never completes)
    out, codes = _run(2, fail_rank=1, timeout=60)
    assert codes[1] != 0
    assert not out
