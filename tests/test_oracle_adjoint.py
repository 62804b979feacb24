"""The oracle's adjoint gradient against central finite differences (CPU).

Pins the formula the GPU gradients are checked with: for compliance C = F^T u
and the mean -z tip displacement J = c^T u, dJ/dE_e = -lam_e^T (K_e/E_e) u_e,
against central differences with relative step 1e-4 in the difference form,
plus the degree -1 homogeneity of u in E: sum_e E_e dJ/dE_e = -J.
"""
import numpy as np


def random_functional(n, seed, scale):
    """A seeded linear functional not proportional to F (so lam is not a
    multiple of u); with a uniform tip load the mean tip displacement is
    exactly compliance / total load."""
    return scale * np.random.default_rng(seed).normal(size=n)


def test_adjoint_matches_central_differences(oracle):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(6, 3, 3, 0.05, seed=12, jitter=0.15, hetero=True)
    eq6, n, K, F, u = oracle.solve_model(m)
    c = C.tip_mean_uz_functional(m, eq6, n)
    assert abs(c @ u - (F @ u) / 1000.0) <= 1e-12 * (F @ u)  # uniform 1000 N tip load
    c = c + random_functional(n, 9, np.abs(c).max())
    lam = oracle.sparse_direct_solve(K, c)
    kes = oracle.chexa8_ke_batch(m)
    gC = oracle.element_gradient(m, eq6, u, u, kes)
    gJ = oracle.element_gradient(m, eq6, u, lam, kes)
    J, Cmp = c @ u, F @ u
    assert Cmp > 0
    assert abs(np.sum(m.E * gC) + Cmp) <= 1e-10 * Cmp
    assert abs(np.sum(m.E * gJ) + J) <= 1e-10 * abs(J)
    # the two gradients are not proportional
    ratio = gJ / gC
    assert ratio.max() - ratio.min() > 0.1 * np.abs(ratio).max()
    elems = np.random.default_rng(3).choice(m.n_elem, 8, replace=False)
    fd = oracle.fd_gradient(m, eq6, K, u, np.stack([F, c], axis=1), elems, 1e-4, kes)
    assert np.abs(fd[:, 0] - gC[elems]).max() <= 1e-6 * np.abs(gC).max()
    assert np.abs(fd[:, 1] - gJ[elems]).max() <= 1e-6 * np.abs(gJ).max()
    # a wrong sign or a missing 1/E would be caught
    assert np.abs(fd[:, 0] + gC[elems]).max() > 1e-3 * np.abs(gC).max()
