"""GPU element stiffness + assembly parity with the oracle (pattern and DOF
map bit-exact, values to 1e-12 of the matrix scale) and end-to-end SOL 101
solves of small models against the oracle's direct solve."""
import numpy as np
import pytest

from conftest import model_from_spec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be(vsgb):
    b = vsgb.Gb300PcgSolverBackend.try_create(1e-10, 20000)
    assert b is not None, "no sm_103 GPU visible"
    yield b
    b.close()


def _models(known):
    from vibestran_gb300 import cantilever as C
    out = {
        "hex1_eas": model_from_spec(known["hexa_bar_axial_extension"], 0),
        "hex1_sri": model_from_spec(known["hexa_bar_axial_extension"], 1),
        "cantilever_1500": C.cantilever_1500(),
        "jitter_hetero": C.small_block(8, 4, 3, 0.05, seed=11, jitter=0.2, hetero=True),
        "sri_block": C.small_block(5, 3, 3, 0.1, form=C.SRI),
        "incompressible": C.small_block(4, 3, 2, 0.1),
    }
    m = out["incompressible"]
    m.nu[:] = 0.4999
    mixed = C.small_block(6, 3, 3, 0.1, seed=2, jitter=0.1)
    mixed.form[::2] = C.SRI
    out["mixed_forms"] = mixed
    # an element entered twice: its nodes carry up to 9 elements, beyond the
    # compact (structured-mesh) fill, so the general block fill runs
    dup = C.small_block(4, 3, 3, 0.1, seed=5, jitter=0.1)
    k = dup.n_elem // 2
    dup.conn = np.concatenate([dup.conn, dup.conn[k:k + 1]])
    dup.elem_ids = np.concatenate([dup.elem_ids, [dup.elem_ids.max() + 1]]).astype(np.int32)
    for f in ("E", "nu", "form"):
        setattr(dup, f, np.concatenate([getattr(dup, f), getattr(dup, f)[k:k + 1]]))
    out["duplicate_element"] = dup
    return out


MODEL_NAMES = ["hex1_eas", "hex1_sri", "cantilever_1500", "jitter_hetero", "sri_block",
               "incompressible", "mixed_forms", "duplicate_element"]


@pytest.mark.parametrize("name", MODEL_NAMES)
def test_assembly_parity(vsgb, oracle, known, be, name):
    m = _models(known)[name]
    eq6, n = vsgb.build_dof_map(m)
    eq_o, n_o = oracle.dof_map(m)
    assert n == n_o and np.array_equal(eq6, eq_o)
    asm = vsgb.ChexaAssembler(be)
    nnz = asm.assemble(m, eq6, n)
    K = asm.csr_lower()
    Ko = oracle.assemble_chexa8(m, eq_o, n_o)
    assert nnz == Ko.nnz
    assert np.array_equal(K.row_ptr, Ko.row_ptr)
    assert np.array_equal(K.col_ind, Ko.col_ind)
    scale = np.abs(Ko.values).max()
    assert np.abs(K.values - Ko.values).max() <= 1e-12 * scale


@pytest.mark.parametrize("name", MODEL_NAMES)
def test_sol101_parity(vsgb, oracle, known, be, name):
    m = _models(known)[name]
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(F)
    eq_o, n_o, Ko, Fo, uo = oracle.solve_model(m)
    assert np.array_equal(F, Fo)
    err = np.linalg.norm(u - uo) / np.linalg.norm(uo)
    assert err <= 1e-8, err


def test_hexa_bar_axial_known_answer_on_gpu(vsgb, known, be):
    spec = known["hexa_bar_axial_extension"]
    m = model_from_spec(spec)
    eq6, n = vsgb.build_dof_map(m)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(vsgb.apply_forces(m, eq6, n))
    ex = spec["expect"]
    for nid in ex["uz_top_nodes"]:
        assert abs(u[eq6[nid - 1, 2]] - ex["uz"]) < ex["abs_tol"]
    assert abs(u[eq6[5, 0]] - ex["ux_node6"]) < ex["abs_tol"]


def test_eas_vs_sri_bending_on_gpu(vsgb, known, be):
    spec = known["hexa_eas_vs_sri_bending_nearly_incompressible"]
    u5 = {}
    for isop in (0, 1):
        m = model_from_spec(spec, isop)
        eq6, n = vsgb.build_dof_map(m)
        asm = vsgb.ChexaAssembler(be)
        asm.assemble(m, eq6, n)
        u = asm.solve(vsgb.apply_forces(m, eq6, n))
        u5[isop] = u[eq6[4, 0]]
    G = spec["E"] / (2.0 * (1.0 + spec["nu"]))
    assert u5[1] > 0 and u5[0] > u5[1] and u5[0] > 0.1 * 250.0 / G


def test_element_errors(vsgb, be):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(3, 2, 2, 0.1)
    # invert element 4 (swap top and bottom faces)
    m.conn[4] = m.conn[4][[4, 5, 6, 7, 0, 1, 2, 3]]
    eq6, n = vsgb.build_dof_map(m)
    asm = vsgb.ChexaAssembler(be)
    with pytest.raises(vsgb.SolverError, match="element index 4: non-positive Jacobian"):
        asm.assemble(m, eq6, n)
    # the context stays usable
    m = C.small_block(3, 2, 2, 0.1)
    eq6, n = vsgb.build_dof_map(m)
    asm.assemble(m, eq6, n)
    assert np.isfinite(asm.solve(vsgb.apply_forces(m, eq6, n))).all()


def test_mesh_index_errors(vsgb, be):
    """Out-of-range connectivity and equation indices are rejected by the
    upload's range check before any mesh kernel runs; the context stays
    usable and holds no mesh after a rejected upload."""
    from vibestran_gb300 import cantilever as C
    asm = vsgb.ChexaAssembler(be)
    for bad in (-1, None):
        m = C.small_block(3, 2, 2, 0.1)
        m.conn[3, 5] = m.n_nodes if bad is None else bad
        eq6, n = vsgb.build_dof_map(C.small_block(3, 2, 2, 0.1))
        with pytest.raises(vsgb.SolverError,
                           match="element index 3 references a node index out of range"):
            asm.assemble(m, eq6, n)
        with pytest.raises(vsgb.SolverError, match="no mesh uploaded"):
            asm.assemble_resident()
    m = C.small_block(3, 2, 2, 0.1)
    eq6, n = vsgb.build_dof_map(m)
    for v in (n, -2):
        e = eq6.copy()
        e[5, 1] = v
        with pytest.raises(vsgb.SolverError, match="equation index out of range at node index 5"):
            asm.assemble(m, e, n)
    asm.assemble(m, eq6, n)
    assert np.isfinite(asm.solve(vsgb.apply_forces(m, eq6, n))).all()


def test_unconstrained_model_is_reported(vsgb, be):
    # no SPC: K is singular, PCG must not report convergence silently
    from vibestran_gb300 import cantilever as C
    m = C.small_block(2, 1, 1, 0.1)
    m.spc_nodes = m.spc_nodes[:0]
    m.spc_mask = m.spc_mask[:0]
    eq6, n = vsgb.build_dof_map(m)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    F = vsgb.apply_forces(m, eq6, n)
    be.set_option(vsgb.OPT_MAX_ITERS, 200)
    try:
        with pytest.raises(vsgb.SolverError, match="did not converge"):
            asm.solve(F)
    finally:
        be.set_option(vsgb.OPT_MAX_ITERS, 20000)


def test_adjoint_sensitivity_small(vsgb, oracle, be):
    """dC/dE_e = -u_e^T K_e^0 u_e against the oracle's element matrices."""
    from vibestran_gb300 import cantilever as C
    m = C.small_block(5, 2, 2, 0.1, seed=4, jitter=0.15, hetero=True)
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(F)
    g = asm.sensitivity(u, u)
    kes = oracle.chexa8_ke_batch(m)
    ref = np.zeros(m.n_elem)
    for e in range(m.n_elem):
        idx = eq6[m.conn[e]][:, :3].reshape(-1)
        ue = np.where(idx >= 0, u[np.maximum(idx, 0)], 0.0)
        ref[e] = -ue @ kes[e] @ ue / m.E[e]
    assert np.abs(g - ref).max() <= 1e-10 * np.abs(ref).max()
    # compliance identity: sum_e E_e dC/dE_e = -F^T u
    assert abs(np.sum(m.E * g) + F @ u) <= 1e-9 * abs(F @ u)


def test_distorted_eas_hexes_match_numpy_restatement(vsgb, be):
    """The GPU element kernel on the two distorted hexes of
    tests/golden/eas_distorted_hex.json (independent numpy restatement of the
    reference's EAS element with its row-of-J0^-1 enhancement mapping)."""
    import json
    import os

    from conftest import GOLDEN
    from vibestran_gb300 import cantilever as C
    with open(os.path.join(GOLDEN, "eas_distorted_hex.json")) as fh:
        cases = json.load(fh)["cases"]
    for c in cases:
        m = C.SolidModel(node_ids=np.arange(1, 9, dtype=np.int32), xyz=np.array(c["xyz"]),
                         conn=np.arange(8, dtype=np.int32).reshape(1, 8),
                         elem_ids=np.array([1], np.int32), E=np.array([c["E"]]),
                         nu=np.array([c["nu"]]), form=np.array([0], np.int32),
                         spc_nodes=np.zeros(0, np.int32), spc_mask=np.zeros(0, np.int32),
                         loads=[], name=c["name"], shape=(1, 1, 1))
        eq6, n = vsgb.build_dof_map(m)
        assert n == 24 and np.array_equal(eq6[:, :3].reshape(-1), np.arange(24))
        asm = vsgb.ChexaAssembler(be)
        asm.assemble(m, eq6, n)
        K = asm.csr_lower()
        dense = np.zeros((24, 24))
        for r in range(24):
            for k in range(K.row_ptr[r], K.row_ptr[r + 1]):
                dense[r, K.col_ind[k]] = K.values[k]
        ref = np.tril(np.array(c["ke"]))
        assert np.abs(dense - ref).max() <= 1e-12 * np.abs(ref).max(), c["name"]
