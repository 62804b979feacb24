"""GPU PCG parity: the reference's conformance cases and solver error
semantics, through the C ABI, checked against the CPU oracle."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, banded500, tridiagonal

pytestmark = pytest.mark.gpu


def _csr(vsgb, K):
    return vsgb.CsrData(K.row_ptr, K.col_ind, K.values, K.n, K.nnz, K.lower)


@pytest.fixture(scope="module")
def be(vsgb):
    b = vsgb.Gb300PcgSolverBackend.try_create()
    assert b is not None, "no sm_103 GPU visible"
    yield b
    b.close()


@pytest.fixture(scope="module")
def be_mixed(vsgb):
    b = vsgb.Gb300MixedPcgSolverBackend.try_create()
    assert b is not None
    yield b
    b.close()


@pytest.mark.parametrize("graph", [1, 0])
def test_conformance_cases(vsgb, oracle, be, graph):
    be.set_option(vsgb.OPT_USE_GRAPH, graph)
    K = oracle.build_from_triplets(2, [0, 1], [0, 1], [4.0, 9.0])
    u = be.solve(_csr(vsgb, K), [8.0, 27.0])
    assert np.allclose(u, [2.0, 3.0], atol=1e-7) and be.last_iteration_count() <= 1
    for n, d, off, lower, tol in [(5, 3.0, -1.0, False, 1e-6), (8, 3.0, -1.0, True, 1e-6),
                                  (200, 2.0, -1.0, False, 1e-5)]:
        K = tridiagonal(n, d, off, lower)
        assert K.lower == lower
        F = np.ones(n)
        u = be.solve(_csr(vsgb, K), F)
        assert np.abs(u - oracle.direct_solve(K, F)).max() < tol
    assert be.last_relative_residual() < 1e-7
    K = oracle.build_from_triplets(100, list(range(100)), list(range(100)), [1.3e9] * 100)
    u = be.solve(_csr(vsgb, K), np.full(100, 333.0))
    assert np.allclose(u, 333.0 / 1.3e9, rtol=1e-5, atol=0)
    u = be.solve(_csr(vsgb, tridiagonal(10, 3.0, -1.0)), np.zeros(10))
    assert np.abs(u).max() == 0.0 and be.last_iteration_count() == 0
    K, F = banded500()
    u = be.solve(_csr(vsgb, K), F)
    assert np.abs(u - oracle.direct_solve(K, F)).max() < 1e-5
    assert be.name() and "CUDA" in be.name() and be.device_name()
    be.set_option(vsgb.OPT_USE_GRAPH, 1)


def test_iterations_match_oracle(vsgb, oracle, be):
    # Same Jacobi PCG recurrence => same iteration count (+-1 for rounding).
    K, F = banded500()
    be.set_option(vsgb.OPT_TOLERANCE, 1e-10)
    u = be.solve(_csr(vsgb, K), F)
    uo, it_o, rel_o = oracle.pcg_jacobi(K, F, 1e-10)
    assert abs(be.last_iteration_count() - it_o) <= 1
    assert np.abs(u - uo).max() <= 1e-9 * np.abs(uo).max()
    be.set_option(vsgb.OPT_TOLERANCE, 0)


def test_mixed_conformance(vsgb, oracle, be_mixed):
    K = tridiagonal(200, 2.0, -1.0)
    F = np.ones(200)
    u = be_mixed.solve(_csr(vsgb, K), F)
    ud = oracle.direct_solve(K, F)
    assert np.abs(u[::20] - ud[::20]).max() < 5e-3
    assert be_mixed.last_estimated_error() < 1e-4


def test_error_semantics(vsgb, oracle, be):
    K = oracle.build_from_triplets(3, [0, 1, 2], [0, 1, 2], [1.0, 0.0, 1.0])
    with pytest.raises(vsgb.SolverError, match="zero diagonal at row 1"):
        be.solve(_csr(vsgb, K), np.ones(3))
    K = oracle.build_from_triplets(3, [0, 2, 1], [0, 2, 0], [1.0, 1.0, 0.5])
    with pytest.raises(vsgb.SolverError, match="missing diagonal at row 1"):
        be.solve(_csr(vsgb, K), np.ones(3))
    with pytest.raises(vsgb.SolverError, match="force vector size 2 != matrix size 3"):
        be.solve(_csr(vsgb, K), np.ones(2))
    K = tridiagonal(200, 2.0, -1.0)
    be.set_option(vsgb.OPT_MAX_ITERS, 3)
    with pytest.raises(vsgb.SolverError, match="did not converge after 3 iterations"):
        be.solve(_csr(vsgb, K), np.ones(200))
    be.set_option(vsgb.OPT_MAX_ITERS, 0)
    # indefinite matrix -> breakdown -> non-convergence error (cuda_pcg :1934-1943)
    K = oracle.build_from_triplets(2, [0, 1, 1, 0], [0, 1, 0, 1], [1.0, 1.0, 2.0, 2.0])
    with pytest.raises(vsgb.SolverError, match="did not converge"):
        be.solve(_csr(vsgb, K), np.array([1.0, -1.0]))
    # the context stays usable after errors
    u = be.solve(_csr(vsgb, tridiagonal(5, 3.0, -1.0)), np.ones(5))
    assert np.isfinite(u).all()


def test_full_storage_and_unsorted_rows(vsgb, oracle, be):
    K, F = banded500()
    full = K  # banded500 is built with both triangles
    assert not full.lower
    u_full = be.solve(_csr(vsgb, full), F)
    low = full.lower_triangle()
    u_low = be.solve(_csr(vsgb, low), F)
    assert np.abs(u_full - u_low).max() <= 1e-12 * np.abs(u_full).max()
    # reverse each row's entries: same matrix, unsorted storage
    rp, ci, v = low.row_ptr, low.col_ind.copy(), low.values.copy()
    for r in range(low.n):
        ci[rp[r]:rp[r + 1]] = ci[rp[r]:rp[r + 1]][::-1]
        v[rp[r]:rp[r + 1]] = v[rp[r]:rp[r + 1]][::-1]
    u_rev = be.solve(vsgb.CsrData(rp, ci, v, low.n, low.nnz, True), F)
    assert np.abs(u_rev - u_low).max() <= 1e-12 * np.abs(u_low).max()


def test_dense_row_expansion(vsgb, oracle, be):
    # An arrow matrix: one row couples to every DOF (exercises the long-row
    # sort path of the lower->full expansion).
    n = 1500
    rows = list(range(n)) + [n - 1] * (n - 1)
    cols = list(range(n)) + list(range(n - 1))
    vals = [float(n)] * n + [0.5] * (n - 1)
    K = oracle.build_from_triplets(n, rows, cols, vals)
    assert K.lower
    F = np.linspace(1.0, 2.0, n)
    u = be.solve(_csr(vsgb, K), F)
    uo = oracle.direct_solve(K, F)
    assert np.abs(u - uo).max() <= 1e-8 * np.abs(uo).max()


def test_multiple_rhs(vsgb, oracle, be):
    K, F = banded500()
    F2 = np.stack([F, 2 * F, np.zeros_like(F)], axis=1)
    u = be.solve(_csr(vsgb, K), F2)
    ud = oracle.direct_solve(K, F)
    assert np.abs(u[:, 0] - ud).max() < 1e-5
    assert np.abs(u[:, 1] - 2 * ud).max() < 2e-5
    assert np.abs(u[:, 2]).max() == 0.0


def test_cpp_conformance_driver(vsgb):
    exe = os.path.join(ROOT, "vibestran_gb300", "_lib", "conformance")
    src = os.path.join(ROOT, "vibestran_gb300", "cpp", "conformance.cpp")
    libdir = os.path.dirname(vsgb.library_path())
    subprocess.check_call(["g++", "-std=c++20", "-O1", "-I", os.path.join(ROOT, "include"), src,
                           "-L", libdir, "-lvsgb", f"-Wl,-rpath,{libdir}", "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout


def test_page_locked_host_arrays(vsgb):
    """Mesh, equation table, loads and solution in page-locked host memory
    (vsgb_host_alloc) give the same solution, bit for bit, as pageable
    arrays; the blocks are freed with the context."""
    import dataclasses
    from vibestran_gb300 import cantilever as C
    m = C.small_block(6, 3, 3, 0.1, seed=3, jitter=0.1)
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300MixedPcgSolverBackend.try_create(1e-8, 20000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u_ref = asm.solve(F)
    pin = be.pinned_copy
    mh = dataclasses.replace(m, xyz=pin(m.xyz), conn=pin(m.conn), E=pin(m.E), nu=pin(m.nu),
                             form=pin(m.form))
    eq3 = pin(np.ascontiguousarray(eq6[:, :3], np.int32))
    assert eq3.shape == (m.n_nodes, 3) and np.array_equal(mh.xyz, m.xyz)
    u = be.pinned_empty(n)
    asm.assemble(mh, eq3, n)
    assert asm.solve(pin(F), out=u) is u
    assert np.array_equal(u, u_ref)
    with pytest.raises(ValueError):
        asm.solve(F, out=np.zeros(n + 1))
    assert len(be.context.pinned) == 8
    be.close()
