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


def test_reference_arm_json_line():
    """`bench.py --impl reference` (the CPU port of the reference path, no GPU)
    prints one JSON line with the fields the harness reads: the headline metric
    and unit, impl, a cpu_baseline describing the run and an e2e object with no
    host-device traffic."""
    import json
    import subprocess
    # run bench.py's main in a child that reports, afterwards, whether the
    # product library was ever mapped into it (the arm must be oracle-only)
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('PRODUCT_LIB_MAPPED', 'libvsgb' in open('/proc/self/maps').read())")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "s" and d["higher_is_better"] is False
    assert d["steps"] == 1 and d["warmup"] == 1 and d["value"] > 0.0
    assert d["config"]["workload"] == "cantilever_84k"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert "PRODUCT_LIB_MAPPED False" in r.stdout
    # the reference's other CPU solver families, restated and timed beside it
    ic0 = cb["other_solvers"]["ic0_pcg"]
    assert ic0["iterations"] > 0 and ic0["value"] > 0.0 and "IC(0)" in ic0["label"]
    sd = cb["other_solvers"]["sparse_direct"]
    assert [x["dofs"] for x in sd["samples"]] == [1500, 35910]
    assert cb["rel_err_vs_direct"] < 1e-6
