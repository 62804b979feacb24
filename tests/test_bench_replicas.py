"""bench.py's multi-replica host logic on CPU: two gloo ranks (world_size 2).

The SOL 101 path has no data-parallel exchange, so N GPUs run N independent
replicas; what has to hold is the rendezvous, the barrier around the timed
region and the max-over-ranks of the per-step time (the whole-job time is the
slowest replica's).
"""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, w = bench._dist()
    bench._barrier(dist)
    t = bench._allmax(dist, 0.010 + 0.005 * r)  # rank 1 is the slower replica
    bench._barrier(dist)
    q.put((r, w, t))
    dist.destroy_process_group()


def test_two_gloo_replicas_report_the_slowest():
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
    assert [o[0] for o in out] == [0, 1]
    assert all(o[1] == 2 for o in out)
    assert all(abs(o[2] - 0.015) < 1e-12 for o in out)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    os.environ.pop("WORLD_SIZE", None)
    dist, r, w = bench._dist()
    assert dist is None and r == 0 and w == 1
    assert bench._allmax(dist, 0.02) == 0.02
