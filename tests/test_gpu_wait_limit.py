"""The bounded waits of the persistent solve: with VSGB_OPT_SPIN_LIMIT set to
one poll, a CTA that reaches a grid reduction before the others gives up at
once; the solve must return VSGB_ERR_CUDA with the timeout text (no hang, no
fault, no partial result reported as converged), and the same context must
solve correctly once the limit is back at its default.  The wait runs out by
the limit alone: nothing is left unset or broken on the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_grid_wait_limit_fails_cleanly_and_context_recovers(vsgb, oracle, precision):
    from vibestran_gb300 import cantilever as C
    # >= 152 slices of 8 nodes: the persistent solve runs
    m = C.small_block(24, 8, 8, 0.05, seed=31, jitter=0.1, hetero=True)
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    cls = vsgb.Gb300MixedPcgSolverBackend if precision == "mixed" else vsgb.Gb300PcgSolverBackend
    be = cls.try_create(1e-10, 20000)
    assert be is not None
    try:
        asm = vsgb.ChexaAssembler(be)
        asm.assemble(m, eq6, n)
        be.set_option(vsgb.OPT_SPIN_LIMIT, 1)
        with pytest.raises(vsgb.SolverError) as e:
            asm.solve(F)
        assert e.value.code == vsgb.VSGB_ERR_CUDA
        assert "grid barrier of the persistent solve timed out" in str(e.value)
        be.set_option(vsgb.OPT_SPIN_LIMIT, 0)
        u = asm.solve(F)
        assert be.last_stats.kernel_ms > 0.0  # the persistent solve ran
        eq_o, n_o, Ko, Fo, uo = oracle.solve_model(m, tol=1e-12, direct=False)
        tol = 1e-6 if precision == "mixed" else 1e-8
        assert np.linalg.norm(u - uo) / np.linalg.norm(uo) <= tol
    finally:
        be.close()
