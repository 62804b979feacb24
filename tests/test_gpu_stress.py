"""GPU CHEXA8 stress recovery (centroid + corner nodes, von Mises) against the
oracle's restatement of linear_static.cpp:1059-1195 and the reference's
single-hex axial expectations."""
import numpy as np
import pytest

from conftest import model_from_spec

pytestmark = pytest.mark.gpu

# FP64 throughout; the GPU and the oracle differ only in summation order.
REL = 1e-10


def _close(a, b, rel=REL):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(np.asarray(a) - np.asarray(b)).max() <= rel * scale


@pytest.mark.parametrize("isop", [0, 1])
def test_axial_single_hex(vsgb, oracle, known, isop):
    spec = known["hexa_bar_axial_extension"]
    st = spec["expect"]["stress"]
    m = model_from_spec(spec, isop)
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-12, 1000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(F)
    cen, nodal, _ = asm.solid_stress()  # load case 0 of the last solve
    for s in [cen[0]] + list(nodal[0]):
        assert abs(s[2] - st["sz"]) <= st["sz_rel_tol"] * st["sz"]
        assert abs(s[0] - st["sx"]) <= st["sx_sy_abs_tol"]
        assert abs(s[1] - st["sy"]) <= st["sx_sy_abs_tol"]
        assert abs(s[6] - st["sz"]) <= st["sz_rel_tol"] * st["sz"]
    oc, on = oracle.solid_stress(m, eq6, u)
    assert _close(cen, oc) and _close(nodal, on)
    be.close()


@pytest.mark.parametrize("case", ["jitter_hetero", "mixed_forms", "cantilever_1500"])
def test_stress_matches_oracle(vsgb, oracle, case):
    from vibestran_gb300 import cantilever as C
    if case == "jitter_hetero":
        m = C.small_block(8, 4, 3, 0.05, seed=11, jitter=0.2, hetero=True)
    elif case == "mixed_forms":
        m = C.small_block(6, 3, 3, 0.1, seed=2, jitter=0.1)
        m.form[::2] = C.SRI
    else:
        m = C.cantilever_1500()
    eq6, n = vsgb.build_dof_map(m)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-10, 20000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    # host displacements (any field: recovery is linear in u)
    u = np.random.default_rng(7).normal(0.0, 1e-4, n)
    cen, nodal, ms = asm.solid_stress(u)
    oc, on = oracle.solid_stress(m, eq6, u)
    assert _close(cen, oc) and _close(nodal, on)
    assert ms > 0.0
    # the centroid-only call returns the same centroid values
    cen2, none, _ = asm.solid_stress(u, nodal=False)
    assert none is None and np.array_equal(cen, cen2)
    be.close()


def test_stress_needs_a_solution(vsgb):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(3, 2, 2, 0.1)
    eq6, n = vsgb.build_dof_map(m)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-10, 1000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    with pytest.raises(vsgb.SolverError):
        asm.solid_stress()
    be.close()


def test_stress_full_size_84k(vsgb, oracle):
    """84 000-element cantilever: stresses of the mixed solution recovered on
    the GPU from the device-resident displacements, against the oracle's
    recovery from the same displacements."""
    from vibestran_gb300 import cantilever as C
    m = C.cantilever_84k()
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300MixedPcgSolverBackend.try_create(1e-4, 20000)
    be.set_option(vsgb.OPT_INNER_TOL, 1e-3)
    asm = vsgb.ChexaAssembler(be)
    asm.upload(m, eq6, n)
    asm.assemble_resident()
    asm.upload_rhs(F)
    asm.solve_resident()
    u = asm.download()
    cen, nodal, ms = asm.solid_stress()
    oc, on = oracle.solid_stress(m, eq6, u)
    assert _close(cen, oc) and _close(nodal, on)
    # bending: the clamped end carries the largest von Mises stress
    i_max = int(np.argmax(cen[:, 6]))
    x_el = m.xyz[m.conn[i_max]][:, 0].mean()
    assert x_el < 0.1 * m.xyz[:, 0].max()
    be.close()


def test_deck_to_stresses_on_gpu(vsgb, oracle):
    """The reference generator's 320-element bending deck through the whole
    path: native BDF reader -> GPU DOF map, assembly, FP64 PCG -> GPU stress
    recovery, against the oracle's direct solve and recovery, and the bending
    stress against beam theory."""
    import os
    from conftest import GOLDEN
    deck = vsgb.read_bdf(path=os.path.join(GOLDEN, "ref_generator_bending_320.bdf"))
    m = deck.model()
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-12, 20000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(F)
    eq_o, n_o, K, F_o, u_o = oracle.solve_model(m)
    assert np.array_equal(eq6, eq_o)
    assert np.linalg.norm(u - u_o) <= 1e-8 * np.linalg.norm(u_o)
    cen, nodal, _ = asm.solid_stress()
    oc, on = oracle.solid_stress(m, eq6, u_o)
    assert _close(cen, oc, 1e-7) and _close(nodal, on, 1e-7)
    # away from the clamp the outer-layer centroid sigma_xx is the beam
    # stress -F (L - x)(z - H/2) / I (0.1 % on this mesh)
    cx = m.xyz[m.conn].mean(axis=1)
    beam = -1000.0 * (1.0 - cx[:, 0]) * (cx[:, 2] - 0.1) / (0.2 * 0.2 ** 3 / 12)
    sel = (cx[:, 0] > 0.2) & (cx[:, 0] < 0.8) & (np.abs(cx[:, 2] - 0.1) > 0.07)
    assert sel.sum() == 96
    assert np.all(np.abs(cen[sel, 0] / beam[sel] - 1.0) < 5e-3)
    be.close()


@pytest.mark.parametrize("isop", [0, 1])
def test_node_displacements_axial_single_hex(vsgb, known, isop, tmp_path):
    """recover_results' displacement part (linear_static.cpp:574-587) on the
    reference's axial deck: the top-face nodes rise 1e-3 m, node 6 contracts
    -3e-4 m in x, node 1 stays at 0 in z, and every rotation is 0 (the
    expectations of chexa8_axial_force.expected.json); the node CSV lists
    them as CsvWriter does."""
    spec = known["hexa_bar_axial_extension"]
    ex = spec["expect"]
    m = model_from_spec(spec, isop)
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-12, 1000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    u = asm.solve(F)
    d = asm.node_displacements()  # load case 0 of the last solve
    assert np.array_equal(d, asm.node_displacements(u))
    row = {int(nid): i for i, nid in enumerate(m.node_ids)}
    for nid in ex["uz_top_nodes"]:
        assert abs(d[row[nid], 2] - ex["uz"]) <= ex["e2e_rel_tol"] * ex["uz"]
    assert abs(d[row[6], 0] - ex["ux_node6"]) <= ex["e2e_rel_tol"] * abs(ex["ux_node6"])
    assert d[row[1], 2] == 0.0 and np.all(d[:, 3:] == 0.0)
    # the free DOFs are the solution itself
    eq = np.asarray(eq6)[:, :3]
    assert np.array_equal(d[:, :3][eq >= 0], u[eq[eq >= 0]])
    path = tmp_path / "axial.node.csv"
    vsgb.write_node_csv(str(path), m.node_ids, d, [1])
    lines = path.read_text().splitlines()
    assert lines[0] == "# node_id, subcase_id, T1, T2, T3, R1, R2, R3" and len(lines) == 9
    top = [ln for ln in lines[1:] if ln.startswith("5, 1, ")][0]
    assert abs(float(top.split(", ")[4]) - ex["uz"]) <= 1e-6 * ex["uz"]
    be.close()


def test_node_displacements_match_the_solution_84k(vsgb):
    """Full-size: every free DOF of the 84 000-element cantilever's nodal
    output equals its equation's entry of the resident solution, bit for bit,
    and the constrained ones are 0."""
    from vibestran_gb300 import cantilever as C
    m = C.cantilever_84k()
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300MixedPcgSolverBackend.try_create()
    asm = vsgb.ChexaAssembler(be)
    asm.upload(m, eq6, n)
    asm.assemble_resident()
    asm.upload_rhs(F)
    asm.solve_resident()
    u = asm.download()
    d = asm.node_displacements()
    eq = np.asarray(eq6)[:, :3]
    assert np.array_equal(d[:, :3][eq >= 0], u[eq[eq >= 0]])
    assert np.all(d[:, :3][eq < 0] == 0.0) and np.all(d[:, 3:] == 0.0)
    be.close()


def test_deck_to_node_csv_end_to_end(vsgb, oracle, tmp_path):
    """The SOL 101 path from a deck to the nodal CSV: the reference
    generator's 320-hex bending deck read by the host reader, assembled and
    solved on the GPU (FP64), recovered per node and written as CsvWriter's
    nodal CSV; every value in the file within 1e-8 of the oracle's direct
    solve (relative to the largest displacement)."""
    import os
    from conftest import GOLDEN
    d = vsgb.read_bdf(path=os.path.join(GOLDEN, "ref_generator_bending_320.bdf"))
    m = d.model()
    eq6, n = vsgb.build_dof_map(m)
    F = vsgb.apply_forces(m, eq6, n)
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-12, 20000)
    asm = vsgb.ChexaAssembler(be)
    asm.assemble(m, eq6, n)
    asm.solve(F)
    disp = asm.node_displacements()
    path = tmp_path / "bending.node.csv"
    vsgb.write_node_csv(str(path), m.node_ids, disp, [d.subcases[0][0]])
    rows = np.array([[float(x) for x in ln.split(", ")] for ln in
                     path.read_text().splitlines()[1:]])
    order = np.argsort(m.node_ids, kind="stable")
    assert np.array_equal(rows[:, 0], m.node_ids[order])
    _, _, _, _, uo = oracle.solve_model(m)
    eq = np.asarray(eq6)[:, :3]
    ref = np.zeros((m.n_nodes, 6))
    ref[:, :3][eq >= 0] = uo[eq[eq >= 0]]
    scale = np.abs(ref).max()
    assert np.abs(rows[:, 2:] - ref[order]).max() <= 1e-8 * scale
    be.close()
