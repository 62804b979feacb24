"""Benchmark: SOL 101 solve on the 84 000-element CHEXA8 cantilever (60x40x35,
0.01 m edge, n = 265 680) on one GB300.

One step = one pass of the hot path on the resident mesh: CHEXA8 EAS element
stiffness + CSR/block assembly + mixed-precision PCG (FP32 inner Jacobi PCG,
FP64 refinement on the GPU) with the library's default options, which stop on
an estimate of the relative displacement error (target 1e-6).  The plain FP64
Jacobi PCG is timed beside it on the same K with the same error target.  Every
solve's error is measured against the committed FP64 direct-solve fingerprints
(tests/golden/) and reported beside its time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU restatement of the reference path (element
stiffness, triplet build_csr, FP64 Jacobi PCG) on the host cores.
For N > 1 (torchrun) every rank solves an independent replica (the path has no
data-parallel exchange); value is whole-job seconds per solve.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("SOL101 solve sec & PCG iter/s, mixed vs FP64 PCG at ≤1e-6 rel err; HBM GB/s")
WORKLOAD = "cantilever_84k"
# Relative displacement error target of the GPU solves: the library default for
# mixed precision, set explicitly for the FP64 solves timed beside them.
ERROR_TARGET = 1e-6
# The CPU port of the reference stops, as the reference does, on the residual;
# sqrt(r.r)/||F|| < 1e-4 gives 6.9e-7 relative error on the 84k cantilever
# (measured against the direct fingerprint in every run: rel_err_vs_direct).
CPU_TOL = 1e-4
# FP64 FMA rate of a GB300 measured with an FMA-chain kernel (1.91 DFMA/clk/SM
# at 2.07 GHz): the compute floor of the FP64 SpMV.
FP64_TFLOPS = 1.20


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_per_iteration(kernel: str):
    """DRAM bytes per PCG iteration of the persistent `kernel`
    (dram__bytes_read.sum + dram__bytes_write.sum of one captured launch over
    its iterations), from the committed ncu summary in profiles/."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as fh:
            return float(json.load(fh)[kernel]["dram_bytes_per_iteration"])
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist, dist.get_rank(), ws


def _allmax(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _mixed_backend(B, device, tol=None, max_solves=None):
    """Mixed backend with the library defaults (error-controlled to 1e-6); a
    residual tolerance `tol` switches it to the reference's residual test."""
    be = B.Gb300MixedPcgSolverBackend.try_create(tol or 0.0, 50000, device)
    if max_solves:
        be.set_option(B.OPT_MAX_SOLVES, max_solves)
    return be


def _fp64_error_controlled(B, be):
    be.set_option(B.OPT_PRECISION, B.FP64)
    be.set_option(B.OPT_ERROR_TARGET, ERROR_TARGET)


def _mixed_defaults(B, be):
    be.set_option(B.OPT_PRECISION, B.MIXED)
    be.set_option(B.OPT_ERROR_TARGET, -1)
    be.set_option(B.OPT_TOLERANCE, 0)


def _fingerprint_err(name):
    """rel_err(u): relative error of u on a committed FP64 fingerprint."""
    with open(os.path.join(ROOT, "tests", "golden", name)) as fh:
        g = json.load(fh)
    eqs = np.concatenate([g["tip_eq"], g["sample_eq"]])
    ref = np.concatenate([g["tip_uz"], g["sample_u"]])
    return lambda u: float(np.linalg.norm(u[eqs] - ref) / np.linalg.norm(ref))


def extra_multi_rhs(B, C, device):
    """16 load cases on the 100x40x40 block (n = 504 300): one batched mixed
    PCG (16 right-hand sides per matrix sweep, CUDA-graph replayed; beside it
    the opt-in persistent tiled variant, VSGB_OPT_BATCH_TILES = 1) against 16
    sequential persistent mixed solves, all with the library defaults
    (error-controlled to 1e-6), each load case's error against the committed
    converged FP64 solutions (tests/golden/block_160k_16rhs_ref.json).  These
    random face loads leave their error in smooth modes that the residual
    hardly shows (a residual tolerance of 1e-6 gave 2-4e-5 error), which is
    what the error-controlled stop is for."""
    m = C.block_160k_16rhs()
    eq6, n = B.build_dof_map(m)
    F = np.stack([B.apply_forces(m, eq6, n, k) for k in range(16)], axis=1)
    with open(os.path.join(ROOT, "tests", "golden", "block_160k_16rhs_ref.json")) as fh:
        g = json.load(fh)
    samp = np.array(g["sample_eq"])
    refs = [np.array(c["sample_u"]) for c in g["cases"]]
    be = _mixed_backend(B, device)
    asm = B.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    asm.upload_rhs(F)
    out = {"workload": "block_160k_16rhs", "elements": m.n_elem, "dofs": n, "rhs": 16,
           "seed": m.seed, "error_target": ERROR_TARGET,
           "reference": "converged FP64 PCG fingerprints (tests/golden/block_160k_16rhs_ref.json)"}
    for mode, flag, tiles in (("batched", 2, 0), ("batched_tiled", 2, 1), ("sequential", 0, 0)):
        be.set_option(B.OPT_BATCHED, flag)
        be.set_option(B.OPT_BATCH_TILES, tiles)
        asm.solve_resident()  # warm-up (graph capture, buffers, tile size)
        B.timer_start(be)
        st = asm.solve_resident()
        ms = B.timer_stop(be)
        its = [be.rhs_stats(k)["iterations"] for k in range(16)]
        U = asm.download()
        errs = [float(np.linalg.norm(U[samp, k] - refs[k]) / np.linalg.norm(refs[k]))
                for k in range(16)]
        out[mode] = {"solve_s": ms / 1e3, "iterations_max": max(its),
                     "iterations_sum": int(sum(its)), "rel_residual_max": st.rel_residual,
                     "est_rel_error_max": st.est_rel_error, "max_rel_err": max(errs)}
        if flag == 2:
            out[mode]["tile_rows"] = st.batch_tile_rows
    be.set_option(B.OPT_BATCH_TILES, 0)
    out["speedup_batched_vs_sequential"] = out["sequential"]["solve_s"] / out["batched"]["solve_s"]
    # FP64 batched at the same error target
    _fp64_error_controlled(B, be)
    be.set_option(B.OPT_BATCHED, 2)
    asm.solve_resident()
    B.timer_start(be)
    st = asm.solve_resident()
    ms = B.timer_stop(be)
    U = asm.download()
    out["fp64_batched"] = {
        "solve_s": ms / 1e3, "iterations_max": st.iterations,
        "max_rel_err": max(float(np.linalg.norm(U[samp, k] - refs[k]) / np.linalg.norm(refs[k]))
                           for k in range(16))}
    be.close()
    return out


def extra_adjoint(B, C, device, n_fd=32):
    """Gradients of compliance and of the mean -z tip displacement w.r.t. all
    250 000 element moduli (100x50x50, n = 780 300, log-uniform E): one call
    (solves of K [u, lam] = [F, c] + one element pass), checked against the
    FP64 CPU gradient on 1024 seeded elements and central differences
    (relative step 1e-4, difference form, GPU re-assembly) on n_fd elements."""
    import copy
    from oracle import oracle as O
    m = C.block_250k_adjoint()
    eq6, n = B.build_dof_map(m)
    F = B.apply_forces(m, eq6, n)
    c = C.tip_mean_uz_functional(m, eq6, n)
    be = _mixed_backend(B, device, tol=1e-10, max_solves=8)
    asm = B.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    asm.adjoint_gradients(F, c)  # warm-up
    t0 = time.perf_counter()
    u, dC, dJ, lam = asm.adjoint_gradients(F, c, with_adjoint=True)
    wall = time.perf_counter() - t0
    st = be.last_stats
    sub = np.sort(np.random.default_rng(5).choice(m.n_elem, 1024, replace=False))
    gC = O.element_gradient(m, eq6, u, u, elems=sub)
    gJ = O.element_gradient(m, eq6, u, lam, elems=sub)
    h, fd_err = 1e-4, 0.0
    be.set_option(B.OPT_TOLERANCE, 1e-11)
    idx = O.element_dofs(m, eq6)
    for e in np.sort(np.random.default_rng(2026).choice(m.n_elem, n_fd, replace=False)):
        Ke = O.chexa8_ke(m.xyz[m.conn[e]], m.E[e], m.nu[e], m.form[e])
        sel = idx[e] >= 0
        g = idx[e][sel]
        d = []
        for s in (1.0, -1.0):
            m2 = copy.copy(m)
            m2.E = m.E.copy()
            m2.E[e] *= 1.0 + s * h
            asm.assemble(m2, eq6, n)
            rhs = np.zeros(n)
            rhs[g] = -(s * h * Ke[np.ix_(sel, sel)]) @ u[g]
            du = asm.solve(rhs)
            d.append((F @ du, c @ du))
        for k, ref in ((0, dC[e]), (1, dJ[e])):
            fd = (d[0][k] - d[1][k]) / (2.0 * h * m.E[e])
            fd_err = max(fd_err, abs(fd - ref) / abs(ref))
    be.close()
    return {"workload": "block_250k_adjoint", "elements": m.n_elem, "dofs": n, "seed": m.seed,
            "functionals": ["compliance F.u", "mean -u_z over the tip face"],
            "gradient_s": wall, "solve_s": st.solve_ms / 1e3, "iterations": st.iterations,
            "inner_solves": st.inner_solves, "tolerance": 1e-10,
            "cpu_fp64_gradient_max_rel_err": float(max(
                np.abs(gC - dC[sub]).max() / np.abs(dC).max(),
                np.abs(gJ - dJ[sub]).max() / np.abs(dJ).max())),
            "central_fd_max_rel_err": fd_err, "fd_elements": n_fd}


def extra_stress(B, C, device):
    """CHEXA8 stress recovery (centroid + 8 corners, von Mises) of the 84k
    cantilever's mixed solution on the GPU, from the device-resident
    displacements, against the oracle's recovery of the same displacements
    (vectorised numpy over the elements, one host thread)."""
    from oracle import oracle as O
    m = C.cantilever_84k()
    eq6, n = B.build_dof_map(m)
    F = B.apply_forces(m, eq6, n)
    be = _mixed_backend(B, device)
    asm = B.ChexaAssembler(be)
    asm.upload(m, eq6, n)
    asm.assemble_resident()
    asm.upload_rhs(F)
    asm.solve_resident()
    u = asm.download()
    asm.solid_stress()  # warm-up
    kern, call = [], []
    for _ in range(5):
        t0 = time.perf_counter()
        cen, nodal, ms = asm.solid_stress()
        call.append(time.perf_counter() - t0)
        kern.append(ms)
    be.close()
    t0 = time.perf_counter()
    oc, on = O.solid_stress(m, eq6, u)
    t_oracle = time.perf_counter() - t0
    err = max(float(np.abs(cen - oc).max() / np.abs(oc).max()),
              float(np.abs(nodal - on).max() / np.abs(on).max()))
    return {"workload": "cantilever_84k", "elements": m.n_elem, "points_per_element": 9,
            "kernel_ms": float(np.median(kern)),
            "call_ms_with_d2h": 1e3 * float(np.median(call)),
            "d2h_bytes": int(cen.nbytes + nodal.nbytes),
            "oracle_s": t_oracle, "max_rel_err_vs_oracle": err,
            "max_von_mises_pa": float(cen[:, 6].max())}


def extra_bdf(B, C):
    """BDF ingestion of the 250 000-element adjoint deck (one MAT1 / PSOLID
    pair per element, as the heterogeneous configs are written): the native
    reader with every host thread and with one, the deck written by
    cantilever.write_bdf into a temporary directory."""
    import tempfile
    m = C.block_250k_adjoint()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "block_250k_adjoint.bdf")
        C.write_bdf(m, path)
        size = os.path.getsize(path)
        out = {"workload": "block_250k_adjoint deck", "bytes": size}
        for label, th in (("all_threads", 0), ("one_thread", 1)):
            runs = []
            for _ in range(3):
                t0 = time.perf_counter()
                d = B.read_bdf(path=path, threads=th)
                mm = d.model()
                runs.append((time.perf_counter() - t0, d.stats))
            wall, st = min(runs, key=lambda r: r[0])
            out[label] = {"threads": st["threads"], "wall_s": wall,
                          "read_ms": st["read_ms"], "parse_ms": st["parse_ms"],
                          "lines_ms": st["lines_ms"], "cards_ms": st["cards_ms"],
                          "mesh_ms": st["mesh_ms"], "mb_per_s": size / 1e6 / wall}
        out["lines"] = st["lines"]
        out["cards"] = st["cards"]
        out["model_equal"] = bool(np.array_equal(mm.E, m.E) and
                                  np.array_equal(mm.node_ids[mm.conn], m.conn_ids()))
    return out


def extra_same_operator(B, C, device):
    """Repeated single-RHS solves with one operator (the second and later
    solves of a load-case sequence): the coarse correction alone
    (VSGB_OPT_COARSE 1, the default) against the first inner solve deflated
    by the recorded Ritz basis (2), on the uniform and the jittered
    heterogeneous 84k cantilevers, each solve's error against the FP64
    sparse-direct fingerprint."""
    out = {}
    for name in ("cantilever_84k", "cantilever_84k_jitter"):
        m = getattr(C, name)()
        eq6, n = B.build_dof_map(m)
        F = B.apply_forces(m, eq6, n)
        rel_err = _fingerprint_err(name + "_direct.json")
        for mode in (1, 2):
            be = _mixed_backend(B, device)
            be.set_option(B.OPT_COARSE, mode)
            asm = B.ChexaAssembler(be)
            asm.assemble(m, eq6, n)
            asm.upload_rhs(F)
            first = asm.solve_resident()
            runs = [asm.solve_resident() for _ in range(3)]
            err = rel_err(asm.download())
            be.close()
            out[f"{name}_coarse{mode}"] = {
                "first_solve_s": first.solve_ms / 1e3, "first_iterations": first.iterations,
                "repeat_solve_s": statistics.median(r.solve_ms for r in runs) / 1e3,
                "repeat_iterations": runs[-1].iterations, "repeat_rel_err": err}
    return out


def extra_jitter(B, C, device, uniform):
    """Jittered (U(+-0.2 h) interior nodes) heterogeneous (log-uniform E)
    84 000-element cantilever: FP64 and mixed iteration counts against the
    uniform mesh's, and every solve's error against the FP64 sparse-direct
    fingerprint, all with the same error target as the headline (library
    defaults for mixed); then the same two solves with 3x3 block Jacobi."""
    m = C.cantilever_84k_jitter()
    eq6, n = B.build_dof_map(m)
    F = B.apply_forces(m, eq6, n)
    rel_err = _fingerprint_err("cantilever_84k_jitter_direct.json")
    be = _mixed_backend(B, device)
    asm = B.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    asm.upload_rhs(F)

    def run():
        asm.solve_resident()
        st = asm.solve_resident()
        return st, rel_err(asm.download())

    st_m, e_m = run()
    _fp64_error_controlled(B, be)
    st_d, e_d = run()
    be.set_option(B.OPT_PRECOND, B.PRECOND_BLOCK_JACOBI)
    st_bd, e_bd = run()
    _mixed_defaults(B, be)
    st_bm, e_bm = run()
    be.close()
    return {"workload": "cantilever_84k_jitter", "dofs": n, "seed": m.seed,
            "error_target": ERROR_TARGET,
            "fp64": {"iterations": st_d.iterations, "solve_s": st_d.solve_ms / 1e3,
                     "rel_err_vs_direct": e_d, "est_rel_error": st_d.est_rel_error},
            "mixed": {"iterations_fp32": st_m.iterations, "inner_solves": st_m.inner_solves,
                      "solve_s": st_m.solve_ms / 1e3, "rel_err_vs_direct": e_m,
                      "est_rel_error": st_m.est_rel_error},
            "speedup_mixed_vs_fp64_solve": st_d.solve_ms / st_m.solve_ms,
            "iteration_growth_vs_uniform": {
                "fp64": st_d.iterations / uniform["fp64"],
                "fp32_inner": st_m.iterations / uniform["mixed"]},
            "block_jacobi": {
                "fp64": {"iterations": st_bd.iterations, "solve_s": st_bd.solve_ms / 1e3,
                         "rel_err_vs_direct": e_bd},
                "mixed": {"iterations_fp32": st_bm.iterations,
                          "inner_solves": st_bm.inner_solves,
                          "solve_s": st_bm.solve_ms / 1e3, "rel_err_vs_direct": e_bm}}}


def profile_case(which):
    """Small, self-contained runs of the hot kernels for ncu captures."""
    from vibestran_gb300 import backend as B
    from vibestran_gb300 import cantilever as C
    B.load_library(build_if_missing=True)
    if which == "multi":
        m = C.block_160k_16rhs()
        eq6, n = B.build_dof_map(m)
        F = np.stack([B.apply_forces(m, eq6, n, k) for k in range(16)], axis=1)
        be = _mixed_backend(B, 0)
        be.set_option(B.OPT_BATCHED, 2)
        be.set_option(B.OPT_MAX_ITERS, 48)
        asm = B.ChexaAssembler(be)
        asm.assemble(m, eq6, n)
        try:
            asm.solve(F)
        except B.SolverError as e:  # stops at 48 iterations by design
            print("stopped:", str(e)[:60])
        return
    m = C.cantilever_84k()
    eq6, n = B.build_dof_map(m)
    F = B.apply_forces(m, eq6, n)
    be = _mixed_backend(B, 0, max_solves=1 if which == "solve" else None)
    asm = B.ChexaAssembler(be)
    asm.upload(m, eq6, n)
    reps = 3 if which == "assemble" else 1
    for _ in range(reps):
        B.timer_start(be)
        asm.assemble_resident()
        print(f"assemble {B.timer_stop(be):.3f} ms")
    if which == "solve":
        asm.upload_rhs(F)
        st = asm.solve_resident()
        print(f"inner solve: {st.kernel_iterations:.0f} iterations, {st.kernel_ms:.3f} ms")
    if which == "solve64":
        _fp64_error_controlled(B, be)
        asm.upload_rhs(F)
        st = asm.solve_resident()
        print(f"FP64 solve: {st.kernel_iterations:.0f} iterations, {st.kernel_ms:.3f} ms")


def cpu_reference(model, eq6, n, F, steps, warmup, threads):
    """CPU restatement of the reference path on the host cores (oracle port):
    element stiffness + build_csr + FP64 Jacobi PCG (cuda-pcg arithmetic).
    Returns (median seconds, threads, iterations, last K, last u)."""
    from oracle import oracle as O
    used = O.set_threads(threads)
    times, iters, K, u = [], 0, None, None
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        K = O.assemble_chexa8(model, eq6, n)
        u, iters, rel = O.pcg_jacobi(K, F, CPU_TOL, 10000)
        dt = time.perf_counter() - t0
        if k >= warmup:
            times.append(dt)
    return statistics.median(times), used, iters, K, u


def _direct_fingerprint_err(u, name):
    """Relative error of u on the committed FP64 sparse-direct fingerprint."""
    path = os.path.join(ROOT, "tests", "golden", name)
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        g = json.load(fh)
    eqs = np.concatenate([g["tip_eq"], g["sample_eq"]])
    ref = np.concatenate([g["tip_uz"], g["sample_u"]])
    return float(np.linalg.norm(u[eqs] - ref) / np.linalg.norm(ref))


def cpu_other_solvers(K, F, threads):
    """The two other CPU solver families of the reference, restated and timed
    on the same K and F (one warm-up, median of 3 for IC(0); one run each for
    the direct solves):
      - IC(0)-PCG, beside --backend=cpu-pcg (Eigen ConjugateGradient +
        IncompleteCholesky, src/solver/solver_backend.cpp:349-462): zero-fill
        IC of the scaled K, not Eigen's threshold factorisation;
      - sparse direct (SuperLU through scipy), the stand-in for --backend=cpu
        (CHOLMOD, src/solver/solver_backend.cpp:106-345).  At n = 265 680 it
        needs more than 10 minutes on one core, so it is timed on bounded
        samples of the same mesh family: the 20x4x4 cantilever (n = 1 500) and
        a 30x20x18 block (n = 35 910)."""
    from oracle import oracle as O
    from vibestran_gb300 import cantilever as C
    used = O.set_threads(threads)
    O.pcg_ic0(K, F, CPU_TOL, 10000)
    runs = []
    for _ in range(3):
        t0 = time.perf_counter()
        u_ic, it_ic, rel_ic, shift = O.pcg_ic0(K, F, CPU_TOL, 10000)
        runs.append(time.perf_counter() - t0)
    out = {"ic0_pcg": {"value": statistics.median(runs), "unit": "s", "cores": used,
                       "kind": "port", "iterations": it_ic, "tolerance": CPU_TOL,
                       "shift": shift,
                       "rel_err_vs_direct": _direct_fingerprint_err(u_ic,
                                                                    "cantilever_84k_direct.json"),
                       "label": "IC(0), not Eigen's IncompleteCholesky (cpu-pcg)",
                       "sample": "full workload (solve only, K assembled)"}}
    direct = []
    for shape in ((20, 4, 4), (30, 20, 18)):
        m = C.block(*shape, 0.05 if shape == (20, 4, 4) else 0.01)
        m.loads = [C.tip_load(m)]
        eq6, n = O.dof_map(m)
        Fs = O.apply_forces(m, eq6, n)
        Ks = O.assemble_chexa8(m, eq6, n)
        t0 = time.perf_counter()
        O.sparse_direct_solve(Ks, Fs)
        direct.append({"mesh": "x".join(map(str, shape)), "dofs": n,
                       "solve_s": time.perf_counter() - t0})
    out["sparse_direct"] = {"unit": "s", "cores": 1, "kind": "port",
                            "label": "SuperLU (scipy), stand-in for --backend=cpu CHOLMOD",
                            "samples": direct,
                            "sample": "bounded samples of the mesh family (full size > 10 min)"}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the 16-load-case, adjoint and jittered-mesh measurements")
    ap.add_argument("--profile", choices=["assemble", "solve", "solve64", "multi"], default=None,
                    help="run one small case of a hot kernel for a profiler and exit "
                         "(no JSON line): assemble = 3 x element stiffness + block assembly "
                         "of cantilever_84k; solve = one FP32 inner solve (persistent "
                         "kernel) of cantilever_84k; solve64 = one FP64 persistent solve of "
                         "cantilever_84k (error target 1e-6); multi = 48 batched iterations "
                         "of the 16-load-case block")
    ap.add_argument("--extra", choices=["multi_rhs", "adjoint", "stress", "bdf", "same_operator"],
                    default=None,
                    help="run one of the additional workloads alone, print its JSON and exit")
    a = ap.parse_args()
    if a.profile:
        profile_case(a.profile)
        return
    if a.extra:
        from vibestran_gb300 import backend as B
        from vibestran_gb300 import cantilever as C
        B.load_library(build_if_missing=True)
        fn = {"multi_rhs": lambda: extra_multi_rhs(B, C, 0),
              "adjoint": lambda: extra_adjoint(B, C, 0),
              "stress": lambda: extra_stress(B, C, 0),
              "bdf": lambda: extra_bdf(B, C),
              "same_operator": lambda: extra_same_operator(B, C, 0)}[a.extra]
        print(json.dumps(fn()))
        return

    from vibestran_gb300 import cantilever as C
    dist, rank, world = _dist()
    model = C.cantilever_84k()

    if a.impl == "reference":
        if rank != 0:
            return
        # The oracle alone: DOF map, loads, element stiffness, build_csr and
        # the solvers are all its CPU restatement (no product code loaded).
        from oracle import oracle as O
        eq6, n = O.dof_map(model)
        F = O.apply_forces(model, eq6, n)
        nproc = os.cpu_count() or 1
        t, used, iters, K, u = cpu_reference(model, eq6, n, F, a.steps, a.warmup, nproc)
        others = cpu_other_solvers(K, F, nproc)
        line = {
            "impl": "reference", "metric": METRIC, "value": t, "unit": "s", "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * t,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded cantilever generator, reference mesh conventions)",
            "config": {"workload": WORKLOAD, "elements": model.n_elem, "dofs": n,
                       "path": "element stiffness + build_csr + FP64 Jacobi PCG (tol 1e-4)",
                       "l2": "working set > L2"},
            "cpu_baseline": {"value": t, "unit": "s", "cores": used, "kind": "port",
                             "sample": f"full workload, {a.steps} steps after {a.warmup} "
                                       f"warm-up, {iters} PCG iterations",
                             "rel_err_vs_direct": _direct_fingerprint_err(
                                 u, "cantilever_84k_direct.json"),
                             "other_solvers": others},
            "e2e": {"value": t, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return

    from vibestran_gb300 import backend as B
    B.load_library(build_if_missing=True)
    device = int(os.environ.get("LOCAL_RANK", "0"))
    eq6, n = B.build_dof_map(model)
    F = B.apply_forces(model, eq6, n)

    # Library defaults: mixed precision, error-controlled to 1e-6.
    be = _mixed_backend(B, device)
    if be is None:
        raise SystemExit("no sm_103 GPU visible")
    asm = B.ChexaAssembler(be)
    asm.upload(model, eq6, n)
    asm.assemble_resident()
    asm.upload_rhs(F)
    # every solve's error against the FP64 sparse-direct fingerprint
    rel_err = _fingerprint_err("cantilever_84k_direct.json")

    def step():
        asm.assemble_resident()
        return asm.solve_resident()

    for _ in range(a.warmup):
        step()
    launches0 = be.kernel_launches()
    _barrier(dist)
    with ClockSampler(device) as clk:
        B.timer_start(be)
        stats = [step() for _ in range(a.steps)]
        ms = B.timer_stop(be)
    launches = be.kernel_launches() - launches0
    u_mixed = asm.download()
    err_mixed = rel_err(u_mixed)
    t_step = _allmax(dist, ms / 1e3 / a.steps)
    # Dominant kernel of the timed region: the persistent FP32 inner solve
    # (one launch per inner solve), timed by events around each launch.
    res_ms = sum(s.kernel_ms for s in stats)
    res_it = sum(s.kernel_iterations for s in stats)
    res_launches = sum(s.inner_solves for s in stats)
    res_bytes_it = stats[-1].spmv_bytes

    # Phase split: assembly alone and solve alone (device events inside the library).
    B.timer_start(be)
    for _ in range(a.steps):
        asm.assemble_resident()
    t_asm = B.timer_stop(be) / 1e3 / a.steps
    mixed_solve = [asm.solve_resident().solve_ms for _ in range(a.steps)]
    st_mixed = be.last_stats
    _fp64_error_controlled(B, be)
    fp64_runs = [asm.solve_resident() for _ in range(a.steps)]
    fp64_solve = [r.solve_ms for r in fp64_runs]
    st_fp64 = be.last_stats
    u_fp64 = asm.download()
    err_fp64 = rel_err(u_fp64)
    fp64_us_it = (1e3 * sum(r.kernel_ms for r in fp64_runs) /
                  max(sum(r.kernel_iterations for r in fp64_runs), 1))
    # The same mixed solve with the 3x3 block Jacobi preconditioner (option).
    _mixed_defaults(B, be)
    be.set_option(B.OPT_PRECOND, B.PRECOND_BLOCK_JACOBI)
    bj_solve = [asm.solve_resident().solve_ms for _ in range(a.steps + 1)][1:]
    st_bj = be.last_stats
    u_bj = asm.download()
    err_bj = rel_err(u_bj)
    be.set_option(B.OPT_PRECOND, B.PRECOND_JACOBI)
    _fp64_error_controlled(B, be)

    # Phase split of the persistent iterations (global-timer marks by thread 0
    # of every CTA, outside the timed region): FP32 inner solves of the mixed
    # solve, then the FP64 solve.
    be.set_option(B.OPT_PHASE_TRACE, 1)
    _mixed_defaults(B, be)
    asm.solve_resident()
    split32 = B.phase_times(be)
    _fp64_error_controlled(B, be)
    asm.solve_resident()
    split64 = B.phase_times(be)
    be.set_option(B.OPT_PHASE_TRACE, 0)

    # Launch-path block SpMVs (not in the step) for comparison.
    spmv_ms, spmv_bytes = B.time_spmv(be, B.MIXED, 200)
    spmv64_ms, spmv64_bytes = B.time_spmv(be, B.FP64, 200)
    peak, peak_kind = _peaks()
    achieved = res_it * res_bytes_it / (res_ms * 1e-3) / 1e9 if res_ms > 0 else None
    fp64_floor_us = 2.0 * (2 * asm.nnz_lower - n) / FP64_TFLOPS / 1e6
    _mixed_defaults(B, be)

    # End to end through the C ABI with host buffers (mesh + F in, u out),
    # the host arrays in page-locked memory.
    be_e2e = _mixed_backend(B, device)
    pin = be_e2e.pinned_copy
    model_h = dataclasses.replace(model, xyz=pin(model.xyz), conn=pin(model.conn),
                                  E=pin(model.E), nu=pin(model.nu),
                                  form=pin(model.form.astype(np.int32)))
    eq3_h = pin(np.ascontiguousarray(eq6[:, :3], np.int32))
    F_h = pin(F)
    u_e = be_e2e.pinned_empty(n)
    asm_e = B.ChexaAssembler(be_e2e)
    for _ in range(1):
        asm_e.assemble(model_h, eq3_h, n)
        asm_e.solve(F_h, out=u_e)
    _barrier(dist)
    t0 = time.perf_counter()
    for _ in range(a.steps):
        asm_e.assemble(model_h, eq3_h, n)
        asm_e.solve(F_h, out=u_e)
    t_e2e = _allmax(dist, (time.perf_counter() - t0) / a.steps)
    h2d = (model_h.xyz.nbytes + eq3_h.nbytes + model_h.conn.nbytes + model_h.E.nbytes
           + model_h.nu.nbytes + model_h.form.nbytes + F_h.nbytes)
    d2h = u_e.nbytes
    err_e2e = rel_err(u_e)

    if rank != 0:
        return
    cpu_t, cpu_used, cpu_iters, cpu_K, cpu_u = cpu_reference(model, eq6, n, F, a.cpu_steps, 1,
                                                             os.cpu_count() or 1)
    cpu_others = cpu_other_solvers(cpu_K, F, os.cpu_count() or 1)
    it_mixed = st_mixed.iterations
    extras = None
    if not a.no_extras:
        be_e2e.close()
        extras = {"multi_rhs_16": extra_multi_rhs(B, C, device),
                  "adjoint_250k": extra_adjoint(B, C, device),
                  "stress_84k": extra_stress(B, C, device),
                  "bdf_250k": extra_bdf(B, C),
                  "same_operator_84k": extra_same_operator(B, C, device),
                  "jitter_84k": extra_jitter(B, C, device,
                                             {"fp64": st_fp64.iterations, "mixed": it_mixed})}
    line = {
        "metric": METRIC,
        "value": t_step / 1.0,  # seconds per SOL 101 step (whole job: max over ranks)
        "unit": "s",
        "n_gpus": world,
        "steps": a.steps,
        "warmup": a.warmup,
        "ms_per_step": 1e3 * t_step,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 inner / f64 refinement (mixed)",
        "data": "synthetic (seeded cantilever generator, reference mesh conventions)",
        "config": {"workload": WORKLOAD, "elements": model.n_elem, "dofs": n,
                   "nnz_lower": asm.nnz_lower, "formulation": "CHEXA8 EAS",
                   "step": "element stiffness + assembly + mixed PCG (device-resident mesh)",
                   "l2": "inputs larger than L2 (element buffer 387 MB, operator > 129 MB)",
                   "parallelism": f"replicas x{world}"},
        "error_target": ERROR_TARGET,
        "rel_err": {"mixed": err_mixed, "fp64": err_fp64,
                    "est_mixed": st_mixed.est_rel_error, "est_fp64": st_fp64.est_rel_error,
                    "reference": "FP64 sparse direct fingerprint "
                                 "(tests/golden/cantilever_84k_direct.json)"},
        "phases_s": {"assembly": t_asm, "mixed_solve": statistics.median(mixed_solve) / 1e3,
                     "fp64_solve": statistics.median(fp64_solve) / 1e3},
        "mixed_block_jacobi": {"solve_s": statistics.median(bj_solve) / 1e3,
                               "iterations": st_bj.iterations, "rel_err": err_bj},
        "mixed": {"solve_s": statistics.median(mixed_solve) / 1e3, "iterations": it_mixed,
                  "inner_solves": st_mixed.inner_solves,
                  "pcg_iter_per_s": it_mixed / (statistics.median(mixed_solve) / 1e3)},
        "fp64": {"solve_s": statistics.median(fp64_solve) / 1e3, "iterations": st_fp64.iterations,
                 "pcg_iter_per_s": st_fp64.iterations / (statistics.median(fp64_solve) / 1e3),
                 # the FP64 persistent solve against its compute floor: the
                 # SpMV's 2 nnz_full FLOPs per iteration at GB300's FP64 rate
                 "us_per_iteration": fp64_us_it,
                 "fp64_pipe_floor_us": fp64_floor_us,
                 "fp64_pipe_frac": fp64_floor_us / fp64_us_it if fp64_us_it > 0 else None,
                 # bound: FP64 pipe (73 % active in ncu), the 178 MB operator
                 # streamed from DRAM at a fraction of the HBM rate
                 "bound": "fp64-pipe",
                 "dram_bytes_per_iteration": _traffic_per_iteration("k_resident_pcg_f64"),
                 "phase_split_us": split64},
        "speedup_mixed_vs_fp64_solve": statistics.median(fp64_solve) / statistics.median(mixed_solve),
        # The FP32 block operator (94 MB) stays in the 126 MB L2 across the
        # iterations of one launch, so DRAM carries ~1 % of the algorithmic
        # bytes (ncu); the kernel is bound by the operator loads a warp keeps
        # in flight from L2 (ncu's L2 throughput stays under half its peak in
        # the SpMV phase) and the per-iteration critical path of two grid
        # reductions, not by HBM.  frac is the algorithmic rate against HBM
        # (an effective rate).
        "roofline": {"kernel": "k_resident_pcg<float> (persistent FP32 inner solve)",
                     "bound": "l2-latency+grid-sync", "achieved": achieved, "peak": peak,
                     "unit": "GB/s",
                     "frac": achieved / peak if achieved else None, "peak_source": peak_kind,
                     "frac_meaning": "algorithmic bytes per second against the HBM copy rate",
                     "traffic": (_traffic_per_iteration("k_resident_pcg_f32") * res_it
                                 / max(res_launches, 1)
                                 if _traffic_per_iteration("k_resident_pcg_f32") else None),
                     "dram_over_algorithmic": (
                         _traffic_per_iteration("k_resident_pcg_f32") / res_bytes_it
                         if _traffic_per_iteration("k_resident_pcg_f32") else None),
                     "phase_split_us": split32,
                     "reduction_share": ((split32["reduction1_us"] + split32["reduction2_us"]) /
                                         max(sum(split32[k] for k in ("gather_us", "spmv_us",
                                             "reduction1_us", "update_us", "reduction2_us")),
                                             1e-12)),
                     "algorithmic_bytes": res_it * res_bytes_it / max(res_launches, 1),
                     "avg_launch_us": 1e3 * res_ms / max(res_launches, 1),
                     "iterations_per_launch": res_it / max(res_launches, 1),
                     "bytes_per_iteration": res_bytes_it,
                     "us_per_iteration": 1e3 * res_ms / res_it if res_it else None,
                     "launch_path_spmv32": {"avg_launch_us": spmv_ms * 1e3, "bytes": spmv_bytes,
                                            "achieved_gbs": spmv_bytes / (spmv_ms * 1e-3) / 1e9},
                     "launch_path_spmv64": {"avg_launch_us": spmv64_ms * 1e3, "bytes": spmv64_bytes,
                                            "achieved_gbs": spmv64_bytes / (spmv64_ms * 1e-3) / 1e9,
                                            "fp64_fma_floor_us":
                                                2.0 * (2 * asm.nnz_lower - n) / FP64_TFLOPS / 1e6}},
        "cpu_baseline": {"value": cpu_t, "unit": "s", "cores": cpu_used, "kind": "port",
                         "sample": f"full workload x{a.cpu_steps}: element stiffness + build_csr "
                                   f"+ FP64 Jacobi PCG ({cpu_iters} it, tol {CPU_TOL:g})",
                         "rel_err_vs_direct": _direct_fingerprint_err(
                             cpu_u, "cantilever_84k_direct.json"),
                         "other_solvers": cpu_others},
        "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "host_buffers": "page-locked",
                "rel_err": err_e2e},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
    }
    if extras is not None:
        line["extra_workloads"] = extras
    print(json.dumps(line))


if __name__ == "__main__":
    main()
