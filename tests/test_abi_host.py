"""C ABI surface and host-side logic of libvsgb.so (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, model_from_spec


def _declared_symbols():
    with open(os.path.join(ROOT, "include", "vsgb.h")) as fh:
        txt = fh.read()
    return sorted(set(re.findall(r"^\s*(?:int|void|long long)\s+\**(vsgb_\w+)\s*\(", txt, re.M)))


def test_library_exports_every_declared_symbol(vsgb):
    syms = _declared_symbols()
    assert len(syms) >= 20
    lib = ctypes.CDLL(vsgb.library_path())
    for s in syms:
        assert hasattr(lib, s), s
    assert set(syms) == set(vsgb.EXPORTS)
    out = subprocess.run(["nm", "-D", "--defined-only", vsgb.library_path()],
                         capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (vsgb_\w+)", out))
    assert set(syms) <= exported


def test_create_without_gpu_reports_no_device(vsgb):
    import ctypes as ct
    L = vsgb.load_library()
    p = ct.c_void_p()
    rc = L.vsgb_create(0, 0.0, 0, vsgb.FP64, ct.byref(p))
    if rc == vsgb.VSGB_OK:  # running on a GPU machine
        L.vsgb_destroy(p)
        pytest.skip("a GPU is present")
    assert rc == vsgb.VSGB_ERR_NO_DEVICE and not p.value
    assert vsgb.Gb300PcgSolverBackend.try_create() is None


@pytest.mark.parametrize("which", ["hex1", "cantilever_1500", "jitter_block", "partial_spc"])
def test_dof_map_bit_exact_vs_oracle(vsgb, oracle, known, which):
    from vibestran_gb300 import cantilever as C
    if which == "hex1":
        m = model_from_spec(known["hexa_bar_axial_extension"])
    elif which == "cantilever_1500":
        m = C.cantilever_1500()
    elif which == "jitter_block":
        m = C.small_block(5, 4, 3, 0.1, seed=3, jitter=0.2, hetero=True)
        # shuffle node order and ids so the sorted-rank logic is exercised
        rng = np.random.default_rng(5)
        perm = rng.permutation(m.n_nodes)
        new_ids = (rng.permutation(m.n_nodes) * 7 + 11).astype(np.int32)
        old_ids = m.node_ids.copy()
        id_map = dict(zip(old_ids.tolist(), new_ids.tolist()))
        inv = np.empty_like(perm)
        inv[perm] = np.arange(m.n_nodes)
        m.node_ids = new_ids[perm]
        m.xyz = m.xyz[perm]
        m.conn = inv[m.conn].astype(np.int32)
        m.spc_nodes = np.array([id_map[i] for i in m.spc_nodes.tolist()], np.int32)
        m.loads = [(np.array([id_map[i] for i in nodes.tolist()], np.int32), s, d)
                   for nodes, s, d in m.loads]
    else:
        m = C.small_block(4, 2, 2, 0.1)
        m.spc_nodes = np.concatenate([m.spc_nodes, m.node_ids[[20, 33]]]).astype(np.int32)
        m.spc_mask = np.concatenate([m.spc_mask, [0b101, 0b010]]).astype(np.int32)
    eq_p, n_p = vsgb.build_dof_map(m)
    eq_o, n_o = oracle.dof_map(m)
    assert n_p == n_o
    assert np.array_equal(eq_p, eq_o)
    Fp = vsgb.apply_forces(m, eq_p, n_p)
    Fo = oracle.apply_forces(m, eq_o, n_o)
    assert np.array_equal(Fp, Fo)


def test_dof_map_errors(vsgb):
    from vibestran_gb300 import cantilever as C
    m = C.small_block(2, 1, 1, 0.1)
    m.spc_nodes = np.array([999], np.int32)
    m.spc_mask = np.array([1], np.int32)
    with pytest.raises(vsgb.SolverError, match="node 999 not in DofMap"):
        vsgb.build_dof_map(m)
    m = C.small_block(2, 1, 1, 0.1)
    eq, n = vsgb.build_dof_map(m)
    m.loads = [(np.array([12345], np.int32), np.ones(1), np.ones((1, 3)))]
    with pytest.raises(vsgb.SolverError, match="node 12345 not found"):
        vsgb.apply_forces(m, eq, n)


def test_cpp_backend_header_compiles(vsgb):
    # The C++20 SolverBackend wrapper and the conformance driver compile
    # against the standalone interface declarations.
    src = os.path.join(ROOT, "vibestran_gb300", "cpp", "conformance.cpp")
    r = subprocess.run(["g++", "-std=c++20", "-fsyntax-only", "-Wall", "-Wextra",
                        "-I", os.path.join(ROOT, "include"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
