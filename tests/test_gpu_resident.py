"""Persistent (one launch per solve) PCG parity and full-size checks.

The resident kernels need at least one slice of 8 block rows per SM, so these
tests use models of >= 5 000 equations; smaller models run the
launch-per-kernel path, covered by the other GPU tests.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mid_model(vsgb):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(24, 8, 8, 0.05, seed=21, jitter=0.15, hetero=True)
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    return m, eq6, n, F


def _solve(vsgb, m, eq6, n, F, precision, resident, tol, inner=0.0, fmt=0):
    cls = vsgb.Gb300MixedPcgSolverBackend if precision == vsgb.MIXED else vsgb.Gb300PcgSolverBackend
    be = cls.try_create(tol, 20000)
    assert be is not None
    be.set_option(vsgb.OPT_RESIDENT, resident)
    be.set_option(vsgb.OPT_FORMAT, fmt)
    if inner:
        be.set_option(vsgb.OPT_INNER_TOL, inner)
        be.set_option(vsgb.OPT_MAX_SOLVES, 6)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(F)
    st = be.last_stats
    be.close()
    return u, st


def test_resident_fp64_matches_launch_path_and_oracle(vsgb, oracle, mid_model):
    m, eq6, n, F = mid_model
    assert n >= 5000
    eq_o, n_o = oracle.dof_map(m)
    K = oracle.assemble_chexa8(m, eq_o, n_o)
    uo, it_o, _ = oracle.pcg_jacobi(K, F, 1e-12, 100000)
    u_res, st_res = _solve(vsgb, m, eq6, n, F, vsgb.FP64, 1, 1e-10)
    u_lp, st_lp = _solve(vsgb, m, eq6, n, F, vsgb.FP64, 0, 1e-10)
    assert st_res.format == 2
    for u in (u_res, u_lp):
        assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-8
    # same recurrence, different (deterministic) reduction order
    assert abs(st_res.iterations - st_lp.iterations) <= 2
    # deterministic: a second run is bitwise identical
    u_res2, _ = _solve(vsgb, m, eq6, n, F, vsgb.FP64, 1, 1e-10)
    assert np.array_equal(u_res, u_res2)


def test_resident_mixed(vsgb, oracle, mid_model):
    m, eq6, n, F = mid_model
    eq_o, n_o = oracle.dof_map(m)
    K = oracle.assemble_chexa8(m, eq_o, n_o)
    uo, _, _ = oracle.pcg_jacobi(K, F, 1e-12, 100000)
    u, st = _solve(vsgb, m, eq6, n, F, vsgb.MIXED, 1, 1e-8, inner=1e-3)
    assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= 1e-6
    assert st.converged and st.rel_residual <= 1e-8 and st.inner_solves >= 2


def test_resident_zero_rhs(vsgb, mid_model):
    m, eq6, n, F = mid_model
    for prec in (vsgb.FP64, vsgb.MIXED):
        u, st = _solve(vsgb, m, eq6, n, np.zeros_like(F), prec, 1, 1e-8)
        assert np.abs(u).max() == 0.0 and st.iterations == 0


def test_cantilever_84k_full_size(vsgb, oracle):
    """Full-size workload: DOF map / pattern bit-exact against the oracle,
    values to 1e-12, and displacements against the FP64 sparse-direct
    fingerprint (FP64 PCG <= 1e-8, mixed <= 1e-6)."""
    from vibestran_gb300 import cantilever as C
    with open(os.path.join(GOLDEN, "cantilever_84k_direct.json")) as fh:
        g = json.load(fh)
    m = C.cantilever_84k()
    eq6, n = vsgb.build_dof_map(m)
    eq_o, n_o = oracle.dof_map(m)
    assert n == n_o == g["n"] == 265680 and np.array_equal(eq6, eq_o)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-10, 20000)
    asm = vsgb.ChexaAssembler(be)
    assert asm.assemble(m, eq6, n) == 10406466
    K = asm.csr_lower()
    Ko = oracle.assemble_chexa8(m, eq_o, n_o)
    assert np.array_equal(K.row_ptr, Ko.row_ptr) and np.array_equal(K.col_ind, Ko.col_ind)
    assert np.abs(K.values - Ko.values).max() <= 1e-12 * np.abs(Ko.values).max()
    del K, Ko
    tip = np.array(g["tip_eq"])
    samp = np.array(g["sample_eq"])
    ref = np.concatenate([g["tip_uz"], g["sample_u"]])

    def rel_err(u):
        got = np.concatenate([u[tip], u[samp]])
        return np.linalg.norm(got - ref) / np.linalg.norm(ref)

    u = asm.solve(F)
    assert be.last_stats.format == 2
    assert rel_err(u) <= 1e-8
    assert abs(np.linalg.norm(u) - g["u_norm"]) <= 1e-8 * g["u_norm"]
    assert abs(F @ u - g["F_dot_u"]) <= 1e-8 * abs(g["F_dot_u"])
    be.set_option(vsgb.OPT_PRECISION, vsgb.MIXED)
    be.set_option(vsgb.OPT_TOLERANCE, 1e-4)
    be.set_option(vsgb.OPT_INNER_TOL, 1e-3)
    be.set_option(vsgb.OPT_MAX_SOLVES, 4)
    um = asm.solve(F)
    assert rel_err(um) <= 1e-6
    # FP32 operator in difference form: 345 FP32 iterations over two inner
    # solves (495 with the plainly rounded operator, FP64 PCG takes 326)
    assert be.last_stats.iterations <= 400
    be.close()


def test_cantilever_84k_jitter_full_size(vsgb, oracle):
    """Jittered heterogeneous 84 000-element cantilever (interior nodes moved by
    seeded U(+-0.2 h), log-uniform E per element): DOF map and pattern against
    the oracle, displacements against the FP64 sparse-direct fingerprint
    (FP64 PCG <= 1e-8, mixed <= 1e-6), with and without the L2 window."""
    from vibestran_gb300 import cantilever as C
    with open(os.path.join(GOLDEN, "cantilever_84k_jitter_direct.json")) as fh:
        g = json.load(fh)
    m = C.cantilever_84k_jitter()
    assert m.seed == g["seed"]
    eq6, n = vsgb.build_dof_map(m)
    eq_o, n_o = oracle.dof_map(m)
    assert n == n_o == g["n"] and np.array_equal(eq6, eq_o)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-10, 50000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    K = asm.csr_lower()
    Ko = oracle.assemble_chexa8(m, eq_o, n_o)
    assert np.array_equal(K.row_ptr, Ko.row_ptr) and np.array_equal(K.col_ind, Ko.col_ind)
    assert np.abs(K.values - Ko.values).max() <= 1e-12 * np.abs(Ko.values).max()
    del K, Ko
    eqs = np.concatenate([g["tip_eq"], g["sample_eq"]])
    ref = np.concatenate([g["tip_uz"], g["sample_u"]])

    def rel_err(u):
        return np.linalg.norm(u[eqs] - ref) / np.linalg.norm(ref)

    u = asm.solve(F)
    assert be.last_stats.format == 2 and rel_err(u) <= 1e-8
    be.set_option(vsgb.OPT_PRECISION, vsgb.MIXED)
    be.set_option(vsgb.OPT_TOLERANCE, 1e-6)
    be.set_option(vsgb.OPT_INNER_TOL, 1e-3)
    be.set_option(vsgb.OPT_MAX_SOLVES, 6)
    for l2 in (1, 0):
        be.set_option(vsgb.OPT_L2_PERSIST, l2)
        um = asm.solve(F)
        assert rel_err(um) <= 1e-6, l2
    be.close()


def test_resident_scrambled_node_numbering(vsgb, oracle):
    """Randomly numbered nodes: the equations follow the sorted node ids, so a
    CTA's slices reference columns all over the mesh and its window is nearly
    every node.  The window gather then takes the whole window (more
    referenced runs than it keeps) instead of the plane bands of a structured
    numbering; FP64 and mixed answers as the oracle's."""
    from vibestran_gb300 import cantilever as C
    m = C.small_block(24, 8, 8, 0.05, seed=21, jitter=0.15, hetero=True)
    rng = np.random.default_rng(9)
    new_ids = (rng.permutation(m.n_nodes) * 3 + 5).astype(np.int32)
    id_map = dict(zip(m.node_ids.tolist(), new_ids.tolist()))
    m.node_ids = new_ids
    m.spc_nodes = np.array([id_map[i] for i in m.spc_nodes.tolist()], np.int32)
    m.loads = [(np.array([id_map[i] for i in nodes.tolist()], np.int32), s, d)
               for nodes, s, d in m.loads]
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    eq_o, n_o = oracle.dof_map(m)
    K = oracle.assemble_chexa8(m, eq_o, n_o)
    uo, _, _ = oracle.pcg_jacobi(K, F, 1e-12, 100000)
    u64, st64 = _solve(vsgb, m, eq6, n, F, vsgb.FP64, 1, 1e-10)
    assert st64.kernel_iterations > 0  # the persistent solve ran
    assert np.linalg.norm(u64 - uo) / np.linalg.norm(uo) <= 1e-8
    um, stm = _solve(vsgb, m, eq6, n, F, vsgb.MIXED, 1, 1e-8, inner=1e-3)
    assert stm.kernel_iterations > 0
    assert np.linalg.norm(um - uo) / np.linalg.norm(uo) <= 1e-6
