"""Error-controlled stopping (VSGB_OPT_ERROR_TARGET, errest.cuh) at full size.

With default options the mixed solver aims at 1e-6 relative displacement
error; these tests hold it to half of that, 5e-7, against committed FP64
fingerprints of the uniform and the jittered heterogeneous 84 000-element
cantilevers and of all 16 random face-load cases of the 100x40x40 block
(solved as one batched PCG), with no per-workload tolerance.  The FP64 solver
meets the same bound with the target set, and setting the target to 0 brings
back the reference's residual test.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

BOUND = 5e-7


def _fingerprint(name):
    with open(os.path.join(GOLDEN, name)) as fh:
        g = json.load(fh)
    eqs = np.concatenate([g["tip_eq"], g["sample_eq"]])
    ref = np.concatenate([g["tip_uz"], g["sample_u"]])
    return g, lambda u: float(np.linalg.norm(u[eqs] - ref) / np.linalg.norm(ref))


@pytest.mark.parametrize("model", ["cantilever_84k", "cantilever_84k_jitter"])
def test_defaults_meet_the_error_bound(vsgb, model):
    from vibestran_gb300 import cantilever as C
    g, rel_err = _fingerprint(model + "_direct.json")
    m = getattr(C, model)()
    eq6, n = vsgb.build_dof_map(m)
    assert n == g["n"]
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300MixedPcgSolverBackend.try_create()  # every option at its default
    assert be is not None
    try:
        asm = vsgb.ChexaAssembler(be)
        asm.assemble(m, eq6, n)
        u = asm.solve(F)
        st = be.last_stats
        assert st.format == 2 and st.converged == 1
        err = rel_err(u)
        assert err <= BOUND, (model, err, st.iterations, st.inner_solves)
        # the solve reports the estimate it stopped on: the inner solve's
        # (target 1e-6 / 3) plus the bound on the FP32 operator's share
        assert 0.0 <= st.est_rel_error <= 6.7e-7
        # FP64 with the same target: one estimate-stopped persistent solve
        be.set_option(vsgb.OPT_PRECISION, vsgb.FP64)
        be.set_option(vsgb.OPT_ERROR_TARGET, 1e-6)
        u64 = asm.solve(F)
        assert rel_err(u64) <= BOUND, (model, rel_err(u64))
        assert 0.0 <= be.last_stats.est_rel_error <= 3.4e-7
        # target 0: the reference's residual test at the chosen tolerance
        be.set_option(vsgb.OPT_ERROR_TARGET, 0)
        be.set_option(vsgb.OPT_TOLERANCE, 1e-10)
        u_res = asm.solve(F)
        assert rel_err(u_res) <= 1e-8
        assert be.last_stats.est_rel_error == -1.0
    finally:
        be.close()


def test_defaults_meet_the_error_bound_on_16_face_load_cases(vsgb):
    """All 16 random face-load cases of the 100x40x40 block in one batched
    mixed PCG with default options, each within 5e-7 of its converged FP64
    solution (tests/golden/make_direct_160k.py)."""
    from vibestran_gb300 import cantilever as C
    with open(os.path.join(GOLDEN, "block_160k_16rhs_ref.json")) as fh:
        g = json.load(fh)
    m = C.block_160k_16rhs()
    assert m.seed == g["seed"]
    eq6, n = vsgb.build_dof_map(m)
    assert n == g["n"]
    F = np.stack([vsgb.apply_forces(m, eq6, n, k) for k in range(16)], axis=1)
    be = vsgb.Gb300MixedPcgSolverBackend.try_create()
    try:
        asm = vsgb.ChexaAssembler(be)
        asm.assemble(m, eq6, n)
        U = asm.solve(F)
        samp = np.array(g["sample_eq"])
        errs = []
        for k, case in enumerate(g["cases"]):
            ref = np.array(case["sample_u"])
            errs.append(float(np.linalg.norm(U[samp, k] - ref) / np.linalg.norm(ref)))
            assert abs(np.linalg.norm(U[:, k]) - case["u_norm"]) <= BOUND * case["u_norm"]
            st = be.rhs_stats(k)
            assert st["batched"] == 1 and st["converged"] == 1
        assert max(errs) <= BOUND, errs
        # FP64 batched with the same target
        be.set_option(vsgb.OPT_PRECISION, vsgb.FP64)
        be.set_option(vsgb.OPT_ERROR_TARGET, 1e-6)
        be.set_option(vsgb.OPT_BATCHED, 2)
        U64 = asm.solve(F)
        for k, case in enumerate(g["cases"]):
            ref = np.array(case["sample_u"])
            assert np.linalg.norm(U64[samp, k] - ref) / np.linalg.norm(ref) <= BOUND, k
    finally:
        be.close()


def test_fp32_operator_share_of_the_error(vsgb, oracle):
    """A refinement step's inner estimate covers its own FP32 solve only; the
    step also leaves K^-1 (K32 - K) d, the FP32 operator's share
    (refine_bound2 in errest.cuh).  On this jittered block with a 20x
    modulus contrast and random face loads that share reached 3.4e-6 in a
    step whose inner estimate had met the target; with the bound every case
    of the one-at-a-time and the batched solve stays within 1e-6 of the
    sparse-direct answer."""
    from vibestran_gb300 import cantilever as C
    m = C.small_block(40, 16, 16, 0.05, seed=11, jitter=0.1, hetero=True)
    m.loads = C.face_random_loads(m, 20, np.random.default_rng(3))
    eq6, n = vsgb.build_dof_map(m)
    F = np.stack([vsgb.apply_forces(m, eq6, n, k) for k in range(20)], axis=1)
    eq_o, n_o = oracle.dof_map(m)
    U = oracle.sparse_direct_solve(oracle.assemble_chexa8(m, eq_o, n_o), F)
    for batched in (0, 2):
        be = vsgb.Gb300MixedPcgSolverBackend.try_create()
        try:
            be.set_option(vsgb.OPT_BATCHED, batched)
            asm = vsgb.ChexaAssembler(be)
            asm.assemble(m, eq6, n)
            Ug = asm.solve(F)
            for k in range(20):
                assert be.rhs_stats(k)["converged"], (batched, k)
                err = np.linalg.norm(Ug[:, k] - U[:, k]) / np.linalg.norm(U[:, k])
                assert err <= 1e-6, (batched, k, err)
        finally:
            be.close()
