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


def _call_noalloc(vsgb, torch, K, F, tol=1e-10, max_iters=10000, row_ptr=None):
    dev = torch.device("cuda:0")
    rp = torch.from_numpy(np.ascontiguousarray(K.row_ptr if row_ptr is None else row_ptr,
                                               np.int32)).to(dev)
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
            # and against the oracle's direct solve of the same system
            u_dir = oracle.direct_solve(K, F)
            assert np.linalg.norm(u - u_dir) / np.linalg.norm(u_dir) <= 1e-8
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


def test_noalloc_rejects_bad_csr_and_reports_non_convergence(vsgb, oracle):
    """Every error branch of the entry point on inputs whose reads stay inside
    the caller's buffers: the row pointer and column indices are checked on
    the device before anything is read through them."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    K, F = banded500()
    # a decreasing row pointer, and one whose last entry is not nnz
    rp = np.array(K.row_ptr, np.int32)
    rp[100] = rp[101] + 1
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, F, row_ptr=rp)
    assert rc == vsgb.VSGB_ERR_INVALID and "row_ptr" in msg and "row 100" in msg, msg
    rp = np.array(K.row_ptr, np.int32)
    rp[-1] = K.nnz + 5
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, F, row_ptr=rp)
    assert rc == vsgb.VSGB_ERR_INVALID and "row_ptr" in msg, msg
    # a column index equal to n
    ci = np.array(K.col_ind, np.int32)
    ci[K.row_ptr[7]] = K.n
    Kc = vsgb.CsrData(K.row_ptr, ci, K.values, K.n, K.nnz, False)
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, Kc, F)
    assert rc == vsgb.VSGB_ERR_INVALID and "column index out of range in row 7" in msg, msg
    # a row without its diagonal entry
    Km = oracle.build_from_triplets(3, [0, 1, 2, 1, 2], [0, 2, 2, 0, 1],
                                    [2.0, -1.0, 2.0, -1.0, -1.0])
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, Km, np.ones(3))
    assert rc == vsgb.VSGB_ERR_SINGULAR and "missing diagonal at row 1" in msg, msg
    # too few iterations
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, F, max_iters=3)
    assert rc == vsgb.VSGB_ERR_NOT_CONVERGED and "did not converge after 3" in msg, msg
    assert it == 3
    # an indefinite matrix (positive diagonal): p*Ap < 0 at the first step
    Ki = oracle.build_from_triplets(2, [0, 0, 1, 1], [0, 1, 0, 1], [1.0, 2.0, 2.0, 1.0])
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, Ki, np.array([1.0, -1.0]), max_iters=50)
    assert rc == vsgb.VSGB_ERR_NOT_CONVERGED and "non-positive p*Ap" in msg, msg
    assert it == 50
    # the shared scratch is usable again afterwards
    rc, u, it, rel, msg = _call_noalloc(vsgb, torch, K, F)
    assert rc == vsgb.VSGB_OK, msg
    u_dir = oracle.direct_solve(K, F)
    assert np.linalg.norm(u - u_dir) / np.linalg.norm(u_dir) <= 1e-8
