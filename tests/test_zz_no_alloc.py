"""vsgb_pcg_solve_noalloc: the allocation-free FP64 PCG entry point.

It exists for callers that may not allocate GPU memory (code inside another
framework's memory pool, or a latency-critical loop where cudaMalloc is not
allowed); its scratch is a static device array of fixed size shared by all
calls.  This file is collected last so that a failure here leaves every other
test already run.  Device buffers come from torch (plumbing only); the solve
goes through the C ABI.
"""
import ctypes

import numpy as np
import pytest

from conftest import banded500

pytestmark = pytest.mark.gpu


def _call_noalloc(vsgb, torch, K, F, tol=1e-10, max_iters=10000):
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(np.ascontiguousarray(K.row_ptr, np.int32)).to(dev)
    ci = torch.from_numpy(np.ascontiguousarray(K.col_ind, np.int32)).to(dev)
    v = torch.from_numpy(np.ascontiguousarray(K.values, np.float64)).to(dev)
    f = torch.from_numpy(np.ascontiguousarray(F, np.float64)).to(dev)
    u = torch.full((K.n,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    it = ctypes.c_int()
    rel = ctypes.c_double()
    err = ctypes.create_string_buffer(512)
    rc = vsgb.load_library().vsgb_pcg_solve_noalloc(
        K.n, K.nnz, rp.data_ptr(), ci.data_ptr(), v.data_ptr(), f.data_ptr(), u.data_ptr(),
        tol, max_iters, ctypes.c_void_p(stream.cuda_stream), ctypes.byref(it), ctypes.byref(rel),
        err, 512)
    torch.cuda.synchronize()
    return rc, u.cpu().numpy(), it.value, rel.value, err.value.decode()


def _full(K):
    return K.expanded_symmetric() if K.lower else K


def test_noalloc_matches_existing_entry_point_twice(vsgb, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vibestran_gb300 import cantilever as C
    m = C.cantilever_1500()
    eq6, n = vsgb.build_dof_map(m)
    F1 = vsgb.apply_forces(m, eq6, n)
    K1 = _full(oracle.assemble_chexa8(m, eq6, n))
    K2, F2 = banded500()
    be = vsgb.Gb300PcgSolverBackend.try_create(1e-10, 10000)
    assert be is not None
    try:
        # two different systems back to back (the static scratch keeps the
        # previous call's contents), then the first one again
        for K, F in ((K1, F1), (K2, F2), (K1, F1)):
            rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, F)
            assert rc == vsgb.VSGB_OK, msg
            u_ref = be.solve(vsgb.CsrData(K.row_ptr, K.col_ind, K.values, K.n, K.nnz, False), F)
            err = np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)
            assert err <= 1e-8, err
            assert rel < 1e-10 and it > 0
    finally:
        be.close()


def test_noalloc_limits_and_errors(vsgb, oracle):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    K, F = banded500()
    # beyond the static scratch: rejected before any device access
    rc = vsgb.load_library().vsgb_pcg_solve_noalloc(
        vsgb.NOALLOC_MAX_N + 1, 1, 1, 1, 1, 1, 1, 1e-8, 100, None, None, None, None, 0)
    assert rc == vsgb.VSGB_ERR_LIMIT
    err = ctypes.create_string_buffer(256)
    rc = vsgb.load_library().vsgb_pcg_solve_noalloc(
        vsgb.NOALLOC_MAX_N + 1, 1, 1, 1, 1, 1, 1, 1e-8, 100, None, None, None, err, 256)
    assert rc == vsgb.VSGB_ERR_LIMIT and b"65536" in err.value
    # zero RHS -> zeros, 0 iterations; zero diagonal -> the reference's error text
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, np.zeros(K.n))
    assert rc == vsgb.VSGB_OK and it == 0 and np.abs(u).max() == 0.0
    Kz = oracle.build_from_triplets(3, [0, 1, 2], [0, 1, 2], [1.0, 0.0, 1.0])
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, Kz, np.ones(3))
    assert rc == vsgb.VSGB_ERR_SINGULAR and "zero diagonal at row 1" in msg
    # and a normal solve still works afterwards
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, F)
    assert rc == vsgb.VSGB_OK, msg
    assert np.abs(u - oracle.direct_solve(K, F)).max() < 1e-8
