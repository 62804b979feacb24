"""Native BDF reader (vsgb_bdf_*, host only): card assembly and number rules
of the reference's BdfParser (src/io/bdf_parser.cpp) on the SOL 101 CHEXA8
deck subset, checked against decks written in every field format, the
reference generator's deck, the reference's own CHEXA8 e2e decks (copied into
tests/golden/ref_e2e by tests/golden/make_ref_decks.py) and the oracle."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, model_from_spec

REF_CASES = os.path.join(GOLDEN, "ref_e2e")


@pytest.fixture(scope="module")
def B(vsgb):
    return vsgb


def _same_model(a, b):
    """a: read from a deck (nodes ascending); b: the SolidModel written."""
    order = np.argsort(b.node_ids, kind="stable")
    assert np.array_equal(a.node_ids, b.node_ids[order])
    assert np.array_equal(a.xyz, b.xyz[order])
    assert np.array_equal(a.node_ids[a.conn], b.conn_ids())
    assert np.array_equal(a.elem_ids, b.elem_ids)
    assert np.array_equal(a.E, b.E) and np.array_equal(a.nu, b.nu)
    assert np.array_equal(a.form, b.form)


@pytest.mark.parametrize("which", ["cantilever_1500", "mixed_hetero"])
def test_round_trip_of_written_decks(B, tmp_path, which):
    from vibestran_gb300 import cantilever as C
    if which == "cantilever_1500":
        m = C.cantilever_1500()
    else:
        m = C.small_block(6, 3, 3, 0.1, seed=2, jitter=0.1, hetero=True)
        m.form[::2] = C.SRI
    path = tmp_path / "deck.bdf"
    C.write_bdf(m, str(path))
    d = B.read_bdf(path=str(path))
    assert d.stats["sol"] == 101 and d.stats["mesh_ok"] == 1 and d.subcases == [(1, 1, 1)]
    assert d.warnings == ""
    r = d.model()
    _same_model(r, m)
    assert np.array_equal(r.spc_nodes, m.spc_nodes) and np.array_equal(r.spc_mask, m.spc_mask)
    for x, y in zip(r.loads[0], m.loads[0]):
        assert np.array_equal(x, y)


def test_threads_give_identical_models(B, tmp_path):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(60, 12, 12, 0.01, seed=3, jitter=0.1, hetero=True)
    path = tmp_path / "big.bdf"
    C.write_bdf(m, str(path))
    one = B.read_bdf(path=str(path), threads=1)
    many = B.read_bdf(path=str(path), threads=6)
    assert one.stats["threads"] == 1 and many.stats["threads"] > 1
    for x, y in zip(one.mesh(), many.mesh()):
        assert np.array_equal(x, y)
    for s in (one, many):
        _same_model(s.model(), m)


# ── the single-hex axial case in every field format ─────────────────────────

def _f8(v):
    return f"{v:<8}"


def _axial_decks(spec):
    nodes = spec["nodes"]
    E, nu = spec["E"], spec["nu"]
    decks = {}
    # free field, '+' continuation, comments, lower case, CRLF
    lines = ["$ free field", "sol 101", "cend", "subcase 1", "  load = 1", "  spc = 1",
             "begin bulk"]
    for n in nodes:
        lines.append(f"grid,{n[0]},,{n[1]!r},{n[2]!r},{n[3]!r}  $ a node")
    lines += [f"MAT1,1,{E!r},,{nu!r}", "PSOLID,1,1", "CHEXA,1,1,1,2,3,4,5,6,+C1", "+C1,7,8"]
    for nid, comps in spec["spc1"]:
        lines.append(f"SPC1,1,{comps},{nid}")
    for nid, sc, d in spec["force"]:
        lines.append(f"FORCE,1,{nid},0,{sc!r},{d[0]},{d[1]},{d[2]}")
    lines.append("ENDDATA")
    decks["free"] = "\r\n".join(lines) + "\r\n"
    # small field (8 columns), Nastran number forms, blank-label continuation
    lines = ["SOL 101", "CEND", "SUBCASE 1", "  LOAD = 1", "  SPC = 1", "BEGIN BULK"]
    forms = {0.0: "0.", 1.0: "1.0+0"}
    for n in nodes:
        lines.append(_f8("GRID") + _f8(n[0]) + _f8("") +
                     "".join(_f8(forms[float(v)]) for v in n[1:]))
    lines.append(_f8("MAT1") + _f8(1) + _f8("1.0D6") + _f8("") + _f8(".3"))
    lines.append(_f8("PSOLID") + _f8(1) + _f8(1))
    lines.append(_f8("CHEXA") + _f8(1) + _f8(1) + "".join(_f8(g) for g in range(1, 7)))
    lines.append(_f8("") + _f8(7) + _f8(8))
    lines.append(_f8("SPC1") + _f8(1) + _f8(3) + _f8(1) + _f8("THRU") + _f8(4))
    lines.append(_f8("SPC1") + _f8(1) + _f8(12) + _f8(1))
    lines.append(_f8("SPC1") + _f8(1) + _f8(2) + _f8(2))
    for nid, sc, d in spec["force"]:
        lines.append(_f8("FORCE") + _f8(1) + _f8(nid) + _f8(0) + _f8("2.5+2") +
                     "".join(_f8(float(x)) for x in d))
    lines.append("ENDDATA")
    decks["small"] = "\n".join(lines) + "\n"
    # large field GRID* with '*' continuations
    lines = ["SOL 101", "CEND", "BEGIN BULK"]
    for n in nodes:
        lines.append(f"{'GRID*':<8}{n[0]:<16}{'':<16}{n[1]!r:<16}{n[2]!r:<16}")
        lines.append(f"{'*':<8}{n[3]!r:<16}")
    lines += [f"MAT1,1,{E!r},,{nu!r}", "PSOLID,1,1,,,,EAS", "CHEXA,1,1,1,2,3,4,5,6",
              "+,7,8", "SPC1,1,3,1,2,3,4", "SPC1,1,12,1", "SPC1,1,2,2"]
    for nid, sc, d in spec["force"]:
        lines.append(f"FORCE,1,{nid},,{sc!r},{d[0]},{d[1]},{d[2]}")
    lines.append("ENDDATA")
    decks["large"] = "\n".join(lines) + "\n"  # no case control: LOAD = SPC = 1
    return decks


@pytest.mark.parametrize("fmt", ["free", "small", "large"])
def test_field_formats(B, known, oracle, fmt):
    spec = known["hexa_bar_axial_extension"]
    d = B.read_bdf(text=_axial_decks(spec)[fmt])
    assert d.subcases == [(1, 1, 1)]
    m = d.model()
    ref = model_from_spec(spec)
    _same_model(m, ref)
    # constraints as masks per grid, loads as written
    got, want = {}, {}
    for nid, msk in zip(m.spc_nodes, m.spc_mask):
        got[int(nid)] = got.get(int(nid), 0) | int(msk)
    for nid, msk in zip(ref.spc_nodes, ref.spc_mask):
        want[int(nid)] = want.get(int(nid), 0) | int(msk)
    assert got == want
    n, s, dirs = m.loads[0]
    assert np.array_equal(n, ref.loads[0][0]) and np.allclose(s, 250.0)
    assert np.array_equal(dirs, ref.loads[0][2])
    # and the deck solves to the reference's known answer
    eq6, ndof, K, F, u = oracle.solve_model(m)
    i5 = int(np.where(m.node_ids == 5)[0][0])
    assert abs(u[eq6[i5, 2]] - spec["expect"]["uz"]) < spec["expect"]["abs_tol"]


# ── the reference generator's deck (tests/golden/make_bdf_fixture.py) ───────

def test_reference_generator_deck(B, oracle):
    """tools/generate_chexa_mesh.py 320 --load-case bending: 20x4x4 hexes of
    0.05 m; node id = i (ny+1)(nz+1) + j (nz+1) + k + 1; clamp 123 on the
    x = 0 face by SPC1 THRU; 1000 N in +z over the 25 tip nodes; coordinates
    written as %.6E."""
    d = B.read_bdf(path=os.path.join(GOLDEN, "ref_generator_bending_320.bdf"))
    assert d.stats["sol"] == 101 and d.subcases == [(1, 1, 1)]
    m = d.model()
    nx, ny, nz, h = 20, 4, 4, 0.05
    assert m.n_elem == nx * ny * nz and len(m.node_ids) == (nx + 1) * (ny + 1) * (nz + 1)
    ids = m.node_ids - 1
    i, j, k = ids // ((ny + 1) * (nz + 1)), (ids // (nz + 1)) % (ny + 1), ids % (nz + 1)
    assert np.allclose(m.xyz, np.stack([i * h, j * h, k * h], 1), rtol=1e-6, atol=1e-12)
    assert np.all(m.E == 2e11) and np.all(m.nu == 0.3) and np.all(m.form == 0)
    # CHEXA node order: (0,0,0) (1,0,0) (1,1,0) (0,1,0) then the same at k+1
    g = m.node_ids[m.conn] - 1
    gi, gj, gk = g // ((ny + 1) * (nz + 1)), (g // (nz + 1)) % (ny + 1), g % (nz + 1)
    d_ijk = np.stack([gi - gi[:, :1], gj - gj[:, :1], gk - gk[:, :1]], 2)
    want = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                     [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    assert np.all(d_ijk == want)
    assert set(m.spc_nodes.tolist()) == set(range(1, 26)) and np.all(m.spc_mask == 7)
    n, s, dirs = m.loads[0]
    assert len(n) == 25 and np.allclose(s.sum(), 1000.0) and np.all(dirs == [0, 0, 1])
    # Euler-Bernoulli tip deflection F L^3 / (3 E I) = 1.25e-5 m, within the
    # shear and end-effect corrections of a 5:1 bar
    eq6, ndof, K, F, u = oracle.solve_model(m)
    tip = [eq6[np.where(m.node_ids == t)[0][0], 2] for t in n]
    assert 1.0 < np.mean(u[tip]) / 1.25e-5 < 1.15


# ── the reference's own CHEXA8 e2e decks (fixtures copied from its tests) ─────

def test_reference_axial_deck(B, known):
    d = B.read_bdf(path=os.path.join(REF_CASES, "chexa8_axial_force.bdf"))
    m = d.model()
    _same_model(m, model_from_spec(known["hexa_bar_axial_extension"]))
    assert "PARAM" not in d.warnings


@pytest.mark.parametrize("name", ["chexa8_constrained_thermal", "chexa8_free_thermal"])
def test_reference_thermal_decks_are_refused(B, name):
    d = B.read_bdf(path=os.path.join(REF_CASES, name + ".bdf"))
    with pytest.raises(B.SolverError, match="temperature"):
        d.model()


# ── errors, ignored cards, subcases ─────────────────────────────────────────

HEAD = "SOL 101\nCEND\nBEGIN BULK\n"
BODY = ("GRID,1,,0.,0.,0.\nGRID,2,,1.,0.,0.\nGRID,3,,1.,1.,0.\nGRID,4,,0.,1.,0.\n"
        "GRID,5,,0.,0.,1.\nGRID,6,,1.,0.,1.\nGRID,7,,1.,1.,1.\nGRID,8,,0.,1.,1.\n"
        "MAT1,1,1.+6,,.3\nPSOLID,1,1\n")
HEXA = "CHEXA,1,1,1,2,3,4,5,6\n+,7,8\n"


def test_parse_errors_carry_the_line(B):
    with pytest.raises(B.SolverError, match=r"Line 4: cannot parse double: 'abc'"):
        B.read_bdf(text=HEAD + "GRID,1,,abc,0.,0.\n")
    with pytest.raises(B.SolverError, match=r"CHEXA has 7 nodes; expected 8"):
        B.read_bdf(text=HEAD + BODY + "CHEXA,1,1,1,2,3,4,5,6\n+,7\n")
    with pytest.raises(B.SolverError, match=r"cannot parse int: 'x'"):
        B.read_bdf(text=HEAD + BODY + "CHEXA,x,1,1,2,3,4,5,6\n+,7,8\n")


def test_cards_outside_the_path(B):
    # unknown to the reference: ignored and listed
    d = B.read_bdf(text=HEAD + BODY + HEXA + "FOOBAR,1,2\nENDDATA\n")
    assert d.stats["mesh_ok"] == 1 and "FOOBAR" in d.warnings
    # another element type: no mesh
    d = B.read_bdf(text=HEAD + BODY + HEXA + "CQUAD4,2,1,1,2,3,4\n")
    assert d.stats["mesh_ok"] == 0 and "CQUAD4" in d.mesh_error
    with pytest.raises(B.SolverError, match="CQUAD4"):
        d.mesh()
    # a coordinate system in use
    d = B.read_bdf(text=HEAD + BODY.replace("GRID,8,,", "GRID,8,2,") + HEXA)
    with pytest.raises(B.SolverError, match="coordinate systems"):
        d.mesh()
    # undefined references
    with pytest.raises(B.SolverError, match="PSOLID 9 is not defined"):
        B.read_bdf(text=HEAD + BODY + HEXA.replace("CHEXA,1,1,", "CHEXA,1,9,")).mesh()
    with pytest.raises(B.SolverError, match="GRID 99 is not defined"):
        B.read_bdf(text=HEAD + BODY + HEXA.replace("+,7,8", "+,7,99")).mesh()
    # a MOMENT of the selected load set, a FORCE in a local system
    d = B.read_bdf(text=HEAD + BODY + HEXA + "MOMENT,1,5,0,1.,0.,0.,1.\n")
    with pytest.raises(B.SolverError, match="MOMENT"):
        d.forces(0)
    d = B.read_bdf(text=HEAD + BODY + HEXA + "FORCE,1,5,3,1.,0.,0.,1.\n")
    with pytest.raises(B.SolverError, match="coordinate system 3"):
        d.forces(0)
    # ... but a MOMENT of another set is never applied
    d = B.read_bdf(text=HEAD + BODY + HEXA + "MOMENT,7,5,0,1.,0.,0.,1.\nFORCE,1,5,,1.,0.,0.,1.\n")
    assert d.forces(0)[0].tolist() == [5]


def test_subcases_and_defaults(B):
    cc = ("SOL 101\nCEND\nSPC = 1\nSUBCASE 1\n  LOAD = 1\nSUBCASE 2\n  LOAD = 2\n"
          "SUBCASE=5\n  LOAD = 2\n  SPC = 3\nBEGIN BULK\n")
    loads = "FORCE,1,5,,10.,0.,0.,1.\nFORCE,2,6,,20.,1.,0.,0.\nFORCE,2,7,,30.,1.,0.,0.\n"
    spcs = "SPC1,1,123,1,THRU,4\nSPC1,3,123,1,2\n"
    d = B.read_bdf(text=cc + BODY + HEXA + loads + spcs + "ENDDATA\n")
    assert d.subcases == [(1, 1, 1), (2, 2, 1), (5, 2, 3)]
    m = d.model(subcases=[0, 1])
    assert len(m.loads) == 2 and m.loads[1][0].tolist() == [6, 7]
    assert m.spc_nodes.tolist() == [1, 2, 3, 4]
    with pytest.raises(B.SolverError, match="different SPC sets"):
        d.model()
    assert d.constraints(2)[0].tolist() == [1, 2]
    # cards after ENDDATA are not read
    d = B.read_bdf(text=cc + BODY + HEXA + "ENDDATA\nCQUAD4,2,1,1,2,3,4\n")
    assert d.stats["mesh_ok"] == 1
