"""The oracle's 3x3 block Jacobi PCG (the checker of the GPU block Jacobi
solve): its block inverses, its solution against the direct solve, and the
recurrence's zero-RHS and non-SPD outcomes of run_pcg_prepared
(src/solver/cuda_pcg_backend_impl.hpp:1820-1830, :1859-1862)."""
import numpy as np
import pytest

from conftest import tridiagonal


@pytest.fixture(scope="module")
def hetero(oracle):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(8, 4, 3, 0.05, seed=11, jitter=0.2, hetero=True)
    eq6, n = oracle.dof_map(m)
    K = oracle.assemble_chexa8(m, eq6, n)
    F = oracle.apply_forces(m, eq6, n)
    return K, F


def test_block_inverses(oracle, hetero):
    K, _ = hetero
    B = oracle.block_jacobi_inverse(K)
    A = K.to_dense()
    nb = K.n // 3
    assert B.shape == (nb, 3, 3)
    for i in range(nb):
        D = A[3 * i:3 * i + 3, 3 * i:3 * i + 3]
        assert np.abs(B[i] @ D - np.eye(3)).max() < 1e-10
        assert np.abs(B[i] - B[i].T).max() <= 1e-12 * np.abs(B[i]).max()


def test_block_jacobi_solution_and_iterations(oracle, hetero):
    K, F = hetero
    u_d = oracle.direct_solve(K, F)
    u, it, rel = oracle.pcg_block_jacobi(K, F, 1e-12, 100000)
    assert rel < 1e-12
    assert np.linalg.norm(u - u_d) <= 1e-9 * np.linalg.norm(u_d)
    # the block-diagonal of K is a stronger preconditioner than its diagonal
    # on this jittered, two-material block
    _, it_j, _ = oracle.pcg_jacobi(K, F, 1e-12, 100000)
    assert it < it_j


def test_block_jacobi_zero_rhs(oracle, hetero):
    K, F = hetero
    u, it, rel = oracle.pcg_block_jacobi(K, np.zeros_like(F), 1e-8, 1000)
    assert it == 0 and rel == 0.0 and not u.any()


def test_block_jacobi_not_spd(oracle):
    # a negative-definite tridiagonal matrix: r.z < 0 at the start
    K = tridiagonal(9, -4.0, 1.0)
    with pytest.raises(oracle.OracleError, match="non-positive initial r\\*z"):
        oracle.pcg_block_jacobi(K, np.ones(9), 1e-8, 100)


def test_block_jacobi_not_converged(oracle, hetero):
    K, F = hetero
    with pytest.raises(oracle.OracleError, match="did not converge after 5 iterations"):
        oracle.pcg_block_jacobi(K, F, 1e-12, 5)
