"""GPU adjoint gradients with respect to every element's Young's modulus.

Compliance C = F^T u and the mean -z tip displacement J = c^T u on a
jittered block with log-uniform per-element E: the GPU gradients (one solve of
K [u, lam] = [F, c], one pass over the stored element matrices) against the
oracle's FP64 gradient from sparse-direct u and lam, and against central
differences (relative step 1e-4) on 32 seeded elements.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adj_case(vsgb, oracle):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(14, 5, 5, 0.02, seed=55, jitter=0.15, hetero=True)
    eq6, n, K, F, u = oracle.solve_model(m)
    c = C.tip_mean_uz_functional(m, eq6, n)
    # plus a seeded random part: with the uniform tip load the tip functional
    # alone is compliance / 1000 and lam would be a multiple of u
    c = c + np.abs(c).max() * np.random.default_rng(77).normal(size=n)
    lam = oracle.sparse_direct_solve(K, c)
    kes = oracle.chexa8_ke_batch(m)
    gC = oracle.element_gradient(m, eq6, u, u, kes)
    gJ = oracle.element_gradient(m, eq6, u, lam, kes)
    elems = np.sort(np.random.default_rng(2026).choice(m.n_elem, 32, replace=False))
    fd = oracle.fd_gradient(m, eq6, K, u, np.stack([F, c], axis=1), elems, 1e-4, kes)
    return m, eq6, n, F, c, u, gC, gJ, elems, fd


def _gpu(vsgb, m, eq6, n, mixed):
    cls = vsgb.Gb300MixedPcgSolverBackend if mixed else vsgb.Gb300PcgSolverBackend
    be = cls.try_create(1e-10 if mixed else 1e-12, 50000)
    if mixed:
        be.set_option(vsgb.OPT_INNER_TOL, 1e-3)
        be.set_option(vsgb.OPT_MAX_SOLVES, 8)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    return be, asm


@pytest.mark.parametrize("mixed", [False, True])
def test_adjoint_gradients(vsgb, adj_case, mixed):
    m, eq6, n, F, c, u_ref, gC, gJ, elems, fd = adj_case
    be, asm = _gpu(vsgb, m, eq6, n, mixed)
    u, dC, dJ = asm.adjoint_gradients(F, c)
    tol = 1e-8 if not mixed else 1e-7
    assert np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref) <= tol
    assert np.abs(dC - gC).max() <= tol * np.abs(gC).max()
    assert np.abs(dJ - gJ).max() <= tol * np.abs(gJ).max()
    # central differences on 32 seeded elements
    assert np.abs(dC[elems] - fd[:, 0]).max() <= 1e-6 * np.abs(gC).max()
    assert np.abs(dJ[elems] - fd[:, 1]).max() <= 1e-6 * np.abs(gJ).max()
    # homogeneity: sum_e E_e dJ/dE_e = -J
    assert abs(np.sum(m.E * dC) + F @ u) <= 1e-8 * (F @ u)
    assert abs(np.sum(m.E * dJ) + c @ u) <= 1e-7 * np.abs(m.E * dJ).sum()
    # compliance only (no adjoint right-hand side)
    u2, dC2, dJ2 = asm.adjoint_gradients(F)
    assert dJ2 is None and np.abs(dC2 - gC).max() <= tol * np.abs(gC).max()
    be.close()


def test_adjoint_full_size_250k(vsgb, oracle):
    """100 x 50 x 50 hexes (n = 780 300), log-uniform E: compliance and mean
    tip displacement gradients for all 250 000 moduli in one call; the FP64
    CPU gradient (oracle element matrices, GPU u and lam) on 4096 seeded
    elements, and central differences (relative step 1e-4, difference form
    with GPU re-assembly and solves) on 32 seeded elements."""
    import copy
    from vibestran_gb300 import cantilever as C
    m = C.block_250k_adjoint()
    eq6, n = vsgb.build_dof_map(m)
    assert n == 780300 and m.n_elem == 250000
    F = vsgb.apply_forces(m, eq6, n)
    c = C.tip_mean_uz_functional(m, eq6, n)
    be = vsgb.Gb300MixedPcgSolverBackend.try_create(1e-10, 50000)
    be.set_option(vsgb.OPT_INNER_TOL, 1e-3)
    be.set_option(vsgb.OPT_MAX_SOLVES, 8)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u, dC, dJ, lam = asm.adjoint_gradients(F, c, with_adjoint=True)
    assert abs(np.sum(m.E * dC) + F @ u) <= 1e-9 * (F @ u)
    sub = np.sort(np.random.default_rng(5).choice(m.n_elem, 4096, replace=False))
    gC = oracle.element_gradient(m, eq6, u, u, elems=sub)
    gJ = oracle.element_gradient(m, eq6, u, lam, elems=sub)
    assert np.abs(gC - dC[sub]).max() <= 1e-10 * np.abs(dC).max()
    assert np.abs(gJ - dJ[sub]).max() <= 1e-10 * np.abs(dJ).max()
    h = 1e-4
    be.set_option(vsgb.OPT_TOLERANCE, 1e-11)
    idx = oracle.element_dofs(m, eq6)
    for e in np.sort(np.random.default_rng(2026).choice(m.n_elem, 32, replace=False)):
        Ke = oracle.chexa8_ke(m.xyz[m.conn[e]], m.E[e], m.nu[e], m.form[e])
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
        fdC = (d[0][0] - d[1][0]) / (2.0 * h * m.E[e])
        fdJ = (d[0][1] - d[1][1]) / (2.0 * h * m.E[e])
        assert abs(fdC - dC[e]) <= 1e-6 * abs(dC[e]), e
        assert abs(fdJ - dJ[e]) <= 1e-6 * abs(dJ[e]), e
    be.close()


def test_adjoint_requires_assembly(vsgb):
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-8, 100)
    asm = vsgb.ChexaAssembler(be)
    asm.n, asm.n_elem = 3, 1
    with pytest.raises(vsgb.SolverError, match="nothing assembled"):
        asm.adjoint_gradients(np.ones(3))
    be.close()
