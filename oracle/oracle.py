"""ctypes front end of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.  Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline / reference arm import
this module, as the checker or as the timed CPU reference.  The product
(vibestran_gb300) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle restatement into oracle/_build/liboracle.so."""
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src)):
        return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-fopenmp", "-shared", "-fPIC",
                           src, "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        cp = ctypes.c_char_p
        ci = ctypes.c_int
        L.orc_num_threads.argtypes = [ci]
        L.orc_num_threads.restype = ci
        L.orc_chexa8_ke.argtypes = [_f64p, ctypes.c_double, ctypes.c_double, ci, _f64p, cp, ci]
        L.orc_chexa8_ke_batch.argtypes = [ci, _f64p, _i32p, _f64p, _f64p, _i32p, _f64p, cp, ci]
        L.orc_dof_map.argtypes = [ci, _i32p, ci, _i32p, ci, _i32p, _i32p, _i32p,
                                  ctypes.POINTER(ci), cp, ci]
        L.orc_dof_constrain.argtypes = [ci, _i32p, ci, _i32p, _i32p, ci, _i32p,
                                        ctypes.POINTER(ci), cp, ci]
        L.orc_apply_forces.argtypes = [ci, _i32p, _i32p, ci, _i32p, _f64p, _f64p, ci, _f64p,
                                       cp, ci]
        L.orc_assemble_dense_elements.argtypes = [ci, ci, ci, _i32p, _f64p]
        L.orc_assemble_dense_elements.restype = _vp
        L.orc_build_from_triplets.argtypes = [ci, ci, _i32p, _i32p, _f64p]
        L.orc_build_from_triplets.restype = _vp
        L.orc_assemble_chexa8.argtypes = [ci, _f64p, _i32p, ci, _i32p, _f64p, _f64p, _i32p,
                                          ci, cp, ci]
        L.orc_assemble_chexa8.restype = _vp
        L.orc_csr_from_arrays.argtypes = [ci, ci, _i32p, _i32p, _f64p, ci]
        L.orc_csr_from_arrays.restype = _vp
        L.orc_csr_info.argtypes = [_vp, ctypes.POINTER(ci), ctypes.POINTER(ci),
                                   ctypes.POINTER(ci)]
        L.orc_csr_copy.argtypes = [_vp, _i32p, _i32p, _f64p]
        L.orc_csr_free.argtypes = [_vp]
        L.orc_csr_expand.argtypes = [_vp]
        L.orc_csr_expand.restype = _vp
        L.orc_csr_lower.argtypes = [_vp]
        L.orc_csr_lower.restype = _vp
        L.orc_csr_multiply.argtypes = [_vp, _f64p, _f64p]
        L.orc_pcg_jacobi.argtypes = [_vp, _f64p, ctypes.c_double, ci, ci, _f64p,
                                     ctypes.POINTER(ci), ctypes.POINTER(ctypes.c_double), cp, ci]
        L.orc_pcg_mixed.argtypes = [_vp, _f64p, ctypes.c_double, ci, _f64p, ctypes.POINTER(ci),
                                    ctypes.POINTER(ci), ctypes.POINTER(ctypes.c_double), cp, ci]
        L.orc_dense_cholesky_solve.argtypes = [_vp, _f64p, _f64p, cp, ci]
        L.orc_pcg_ic0.argtypes = [_vp, _f64p, ctypes.c_double, ci, _f64p, ctypes.POINTER(ci),
                                  ctypes.POINTER(ctypes.c_double),
                                  ctypes.POINTER(ctypes.c_double), cp, ci]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _err():
    return ctypes.create_string_buffer(512)


def set_threads(n: int) -> int:
    return lib().orc_num_threads(int(n))


@dataclass
class Csr:
    """CSR in the reference's CsrData layout (include/core/sparse_matrix.hpp:63-87)."""
    row_ptr: np.ndarray
    col_ind: np.ndarray
    values: np.ndarray
    n: int
    nnz: int
    lower: bool

    def handle(self):
        return _CsrHandle(lib().orc_csr_from_arrays(
            self.n, self.nnz, np.ascontiguousarray(self.row_ptr, np.int32),
            np.ascontiguousarray(self.col_ind, np.int32),
            np.ascontiguousarray(self.values, np.float64), int(self.lower)))

    def multiply(self, x):
        with self.handle() as h:
            y = np.zeros(self.n)
            lib().orc_csr_multiply(h.ptr, np.ascontiguousarray(x, np.float64), y)
            return y

    def expanded_symmetric(self) -> "Csr":
        with self.handle() as h:
            return _take(lib().orc_csr_expand(h.ptr))

    def lower_triangle(self) -> "Csr":
        with self.handle() as h:
            return _take(lib().orc_csr_lower(h.ptr))

    def to_dense(self) -> np.ndarray:
        A = np.zeros((self.n, self.n))
        rows = np.repeat(np.arange(self.n), np.diff(self.row_ptr))
        np.add.at(A, (rows, self.col_ind), self.values)
        if self.lower:
            A = A + np.tril(A, -1).T
        return A


class _CsrHandle:
    def __init__(self, ptr):
        self.ptr = ptr

    def __enter__(self):
        return self

    def __exit__(self, *a):
        lib().orc_csr_free(self.ptr)


def _take(ptr) -> Csr:
    if not ptr:
        raise OracleError("null CSR handle")
    L = lib()
    n, nnz, lower = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    L.orc_csr_info(ptr, ctypes.byref(n), ctypes.byref(nnz), ctypes.byref(lower))
    rp = np.empty(n.value + 1, np.int32)
    ci = np.empty(nnz.value, np.int32)
    v = np.empty(nnz.value, np.float64)
    L.orc_csr_copy(ptr, rp, ci, v)
    L.orc_csr_free(ptr)
    return Csr(rp, ci, v, n.value, nnz.value, bool(lower.value))


def chexa8_ke(xyz24, E, nu, formulation=0) -> np.ndarray:
    ke = np.zeros(576)
    err = _err()
    if lib().orc_chexa8_ke(np.ascontiguousarray(xyz24, np.float64).reshape(-1), float(E),
                           float(nu), int(formulation), ke, err, 512) != 0:
        raise OracleError(err.value.decode())
    return ke.reshape(24, 24)


def chexa8_ke_batch(model) -> np.ndarray:
    out = np.zeros((model.n_elem, 576))
    err = _err()
    if lib().orc_chexa8_ke_batch(model.n_elem, np.ascontiguousarray(model.xyz),
                                 np.ascontiguousarray(model.conn, np.int32), model.E, model.nu,
                                 np.ascontiguousarray(model.form, np.int32), out, err, 512) != 0:
        raise OracleError(err.value.decode())
    return out.reshape(model.n_elem, 24, 24)


def dof_map(model):
    """(eq6 (N,6) int32 in model node order, n_free)."""
    eq = np.empty(model.n_nodes * 6, np.int32)
    nf = ctypes.c_int()
    err = _err()
    rc = lib().orc_dof_map(model.n_nodes, np.ascontiguousarray(model.node_ids, np.int32),
                           model.n_elem, np.ascontiguousarray(model.conn_ids(), np.int32),
                           int(model.spc_nodes.shape[0]),
                           np.ascontiguousarray(model.spc_nodes, np.int32),
                           np.ascontiguousarray(model.spc_mask, np.int32), eq,
                           ctypes.byref(nf), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    return eq.reshape(-1, 6), nf.value


def dof_constrain(node_ids, pairs, batch: bool):
    ids = np.ascontiguousarray(node_ids, np.int32)
    cn = np.ascontiguousarray([p[0] for p in pairs], np.int32)
    cd = np.ascontiguousarray([p[1] for p in pairs], np.int32)
    eq = np.empty(ids.shape[0] * 6, np.int32)
    nf = ctypes.c_int()
    err = _err()
    if lib().orc_dof_constrain(ids.shape[0], ids, cn.shape[0], cn, cd, 1 if batch else 0, eq,
                               ctypes.byref(nf), err, 512) != 0:
        raise OracleError(err.value.decode())
    return eq.reshape(-1, 6), nf.value


def apply_forces(model, eq6, n, load_index=0):
    nodes, scale, dirs = model.loads[load_index]
    F = np.zeros(n)
    err = _err()
    if lib().orc_apply_forces(model.n_nodes, np.ascontiguousarray(model.node_ids, np.int32),
                              np.ascontiguousarray(eq6, np.int32).reshape(-1),
                              int(len(nodes)), np.ascontiguousarray(nodes, np.int32),
                              np.ascontiguousarray(scale, np.float64),
                              np.ascontiguousarray(dirs, np.float64).reshape(-1), n, F,
                              err, 512) != 0:
        raise OracleError(err.value.decode())
    return F


def assemble_chexa8(model, eq6, n) -> Csr:
    err = _err()
    ptr = lib().orc_assemble_chexa8(model.n_nodes, np.ascontiguousarray(model.xyz),
                                    np.ascontiguousarray(eq6, np.int32).reshape(-1),
                                    model.n_elem, np.ascontiguousarray(model.conn, np.int32),
                                    model.E, model.nu, np.ascontiguousarray(model.form, np.int32),
                                    n, err, 512)
    if not ptr:
        raise OracleError(err.value.decode())
    return _take(ptr)


def assemble_dense_elements(n, gdofs, kes) -> Csr:
    gdofs = np.ascontiguousarray(gdofs, np.int32)
    kes = np.ascontiguousarray(kes, np.float64)
    ne, nd = gdofs.shape
    return _take(lib().orc_assemble_dense_elements(n, ne, nd, gdofs.reshape(-1),
                                                    kes.reshape(-1)))


def build_from_triplets(n, rows, cols, vals) -> Csr:
    r = np.ascontiguousarray(rows, np.int32)
    return _take(lib().orc_build_from_triplets(n, r.shape[0], r,
                                               np.ascontiguousarray(cols, np.int32),
                                               np.ascontiguousarray(vals, np.float64)))


def pcg_jacobi(K: Csr, F, tol=1e-8, max_iters=10000, precision=64):
    u = np.zeros(K.n)
    it = ctypes.c_int()
    rel = ctypes.c_double()
    err = _err()
    with K.handle() as h:
        rc = lib().orc_pcg_jacobi(h.ptr, np.ascontiguousarray(F, np.float64), float(tol),
                                  int(max_iters), int(precision), u, ctypes.byref(it),
                                  ctypes.byref(rel), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    return u, it.value, rel.value


def pcg_mixed(K: Csr, F, tol=1e-6, max_iters=10000):
    u = np.zeros(K.n)
    it = ctypes.c_int()
    ns = ctypes.c_int()
    rel = ctypes.c_double()
    err = _err()
    with K.handle() as h:
        rc = lib().orc_pcg_mixed(h.ptr, np.ascontiguousarray(F, np.float64), float(tol),
                                 int(max_iters), u, ctypes.byref(it), ctypes.byref(ns),
                                 ctypes.byref(rel), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    return u, it.value, ns.value, rel.value


def pcg_ic0(K: Csr, F, tol=1e-8, max_iters=10000):
    """IC(0)-preconditioned CG (zero-fill incomplete Cholesky of the unit-diagonal
    scaled K, Manteuffel shift), the CPU baseline beside the reference's cpu-pcg
    (Eigen CG + IncompleteCholesky, src/solver/solver_backend.cpp:349-462) — not
    Eigen's factorisation.  Returns (u, iterations, relative residual, shift)."""
    u = np.zeros(K.n)
    it = ctypes.c_int()
    rel = ctypes.c_double()
    shift = ctypes.c_double()
    err = _err()
    with K.handle() as h:
        rc = lib().orc_pcg_ic0(h.ptr, np.ascontiguousarray(F, np.float64), float(tol),
                               int(max_iters), u, ctypes.byref(it), ctypes.byref(rel),
                               ctypes.byref(shift), err, 512)
    if rc != 0:
        raise OracleError(err.value.decode())
    return u, it.value, rel.value, shift.value


def direct_solve(K: Csr, F):
    """FP64 direct solve: dense LLT up to n = 20000 (the --backend=cpu stand-in)."""
    u = np.zeros(K.n)
    err = _err()
    with K.handle() as h:
        if lib().orc_dense_cholesky_solve(h.ptr, np.ascontiguousarray(F, np.float64), u, err,
                                          512) != 0:
            raise OracleError(err.value.decode())
    return u


def sparse_direct_solve(K: Csr, F):
    """FP64 sparse direct solve (SuperLU via scipy) for sizes a dense factor cannot take."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    full = K.expanded_symmetric() if K.lower else K
    A = sp.csc_matrix(sp.csr_matrix((full.values, full.col_ind, full.row_ptr),
                                    shape=(K.n, K.n)))
    return spla.spsolve(A, np.asarray(F, np.float64), permc_spec="MMD_AT_PLUS_A")


def solve_model(model, tol=None, load_index=0, direct=True):
    """Whole oracle pipeline for a model: DOF map, assembly, forces, solve."""
    eq6, n = dof_map(model)
    K = assemble_chexa8(model, eq6, n)
    F = apply_forces(model, eq6, n, load_index)
    if direct:
        u = direct_solve(K, F) if n <= 6000 else sparse_direct_solve(K, F)
    else:
        u, _, _ = pcg_jacobi(K, F, tol or 1e-10, 100000)
    return eq6, n, K, F, u


# ── gradients with respect to element moduli ──────────────────────────────
# The reference has no sensitivity analysis; these restate the adjoint of the
# linear-static equations K(E) u = F for the GPU gradients to be checked
# against: for J = c^T u, dJ/dE_e = -lam_e^T (dK_e/dE_e) u_e with K lam = c,
# and dK_e/dE_e = K_e / E_e because the CHEXA8 stiffness is linear in E for a
# fixed Poisson ratio (isotropic_D, src/elements/solid_elements.cpp:17-27).

def element_dofs(model, eq6) -> np.ndarray:
    """(M, 24) equation numbers of each element's T1-T3 DOFs, -1 when
    constrained (solid_global_dof_indices, src/elements/solid_elements.cpp:29-42)."""
    return np.asarray(eq6)[model.conn][:, :, :3].reshape(model.n_elem, 24)


def element_gradient(model, eq6, u, lam, kes=None, elems=None) -> np.ndarray:
    """FP64 dJ/dE_e = -lam_e^T (K_e / E_e) u_e for every element, or for the
    listed elements only (their K_e formed one by one)."""
    idx = element_dofs(model, eq6)
    E = np.asarray(model.E)
    if elems is not None:
        elems = np.asarray(elems)
        idx, E = idx[elems], E[elems]
        kes = np.stack([chexa8_ke(model.xyz[model.conn[e]], model.E[e], model.nu[e],
                                  model.form[e]) for e in elems])
    elif kes is None:
        kes = chexa8_ke_batch(model)

    def take(v):
        return np.where(idx >= 0, np.asarray(v, np.float64)[np.maximum(idx, 0)], 0.0)

    return -np.einsum("ei,eij,ej->e", take(lam), kes, take(u)) / E


def fd_gradient(model, eq6, K: Csr, u, C, elems, h=1e-4, kes=None) -> np.ndarray:
    """Central differences of J_k = C[:, k]^T u for E_e -> E_e (1 +- h).

    Difference form: with dK = +-h K_e (the element's stiffness scales with
    E_e), (K + dK) du = -dK u gives J(E_e (1 +- h)) - J = C^T du exactly, so
    nothing is lost to subtracting two nearly equal solutions.  Sparse direct
    solves in FP64.  Returns (len(elems), C.shape[1])."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    kes = chexa8_ke_batch(model) if kes is None else kes
    C = np.asarray(C, np.float64).reshape(K.n, -1)
    full = K.expanded_symmetric() if K.lower else K
    A = sp.csr_matrix((full.values, full.col_ind, full.row_ptr), shape=(K.n, K.n))
    idx = element_dofs(model, eq6)
    out = np.zeros((len(elems), C.shape[1]))
    for t, e in enumerate(elems):
        sel = idx[e] >= 0
        g = idx[e][sel]
        Ke = kes[e][np.ix_(sel, sel)]
        rows = np.repeat(g, g.shape[0])
        cols = np.tile(g, g.shape[0])
        dJ = []
        for s in (1.0, -1.0):
            dK = s * h * Ke
            Ap = (A + sp.csr_matrix((dK.reshape(-1), (rows, cols)), shape=A.shape)).tocsc()
            rhs = np.zeros(K.n)
            rhs[g] = -(dK @ np.asarray(u)[g])
            du = spla.spsolve(Ap, rhs, permc_spec="MMD_AT_PLUS_A")
            dJ.append(C.T @ du)
        out[t] = (dJ[0] - dJ[1]) / (2.0 * h * model.E[e])
    return out


# ── CHEXA8 stress recovery ────────────────────────────────────────────────
# LinearStaticSolver::recover_results, solid branch (src/solver/linear_static.cpp):
# u_e from the element's global DOFs with constrained DOFs zero (:661-672);
# sigma = D (B u_e - eps_th) at the centroid and at the 8 corner nodes
# (eval_chexa8 at :1059-1118, points at :1164-1185), D = solid_constitutive_matrix
# (:119-138), B rows xx, yy, zz, xy, yz, zx with engineering shears (:1088-1113),
# von Mises as solid_von_mises (:140-150).  No TEMP loads are on this path, so
# the point temperature equals the reference temperature and eps_th = 0
# (solid_sigma_from_B, :186-196).

# Corner coordinates in CHEXA8 node order (kHexCoords at :1165-1174).
HEX_CORNERS = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                        [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], np.float64)


def _hex_dN(xi):
    """dN/d(xi, eta, zeta) (3, 8) of CHexa8::shape_functions
    (src/elements/solid_elements.cpp:76-93) at one point."""
    s = HEX_CORNERS
    f = 1.0 + s * np.asarray(xi, np.float64)  # (8, 3)
    return 0.125 * np.stack([s[:, 0] * f[:, 1] * f[:, 2],
                             s[:, 1] * f[:, 0] * f[:, 2],
                             s[:, 2] * f[:, 0] * f[:, 1]])


def solid_stress(model, eq6, u):
    """Centroid and corner-node stresses of every CHEXA8 element.

    Returns (centroid (M, 7), nodal (M, 8, 7)), each row
    (sx, sy, sz, sxy, syz, szx, von_mises)."""
    idx = element_dofs(model, eq6)
    u = np.asarray(u, np.float64)
    ue = np.where(idx >= 0, u[np.maximum(idx, 0)], 0.0).reshape(-1, 8, 3)
    X = np.asarray(model.xyz, np.float64)[model.conn]            # (M, 8, 3)
    E = np.asarray(model.E, np.float64)
    nu = np.asarray(model.nu, np.float64)
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))

    def at(xi):
        dN = _hex_dN(xi)                                          # (3, 8)
        J = np.einsum("in,enc->eic", dN, X)                       # rows d/dxi_i, cols x,y,z
        g = np.einsum("eij,jn->ein", np.linalg.inv(J), dN)        # (M, 3, 8): dN/dx, dy, dz
        du = np.einsum("ein,enc->eci", g, ue)                     # du_c / dx_i
        exx, eyy, ezz = du[:, 0, 0], du[:, 1, 1], du[:, 2, 2]
        gxy = du[:, 0, 1] + du[:, 1, 0]
        gyz = du[:, 1, 2] + du[:, 2, 1]
        gzx = du[:, 2, 0] + du[:, 0, 2]
        tr = exx + eyy + ezz
        s = np.stack([lam * tr + 2.0 * mu * exx, lam * tr + 2.0 * mu * eyy,
                      lam * tr + 2.0 * mu * ezz, mu * gxy, mu * gyz, mu * gzx], axis=1)
        vm = np.sqrt(0.5 * ((s[:, 0] - s[:, 1]) ** 2 + (s[:, 1] - s[:, 2]) ** 2 +
                            (s[:, 2] - s[:, 0]) ** 2 +
                            6.0 * (s[:, 3] ** 2 + s[:, 4] ** 2 + s[:, 5] ** 2)))
        return np.concatenate([s, vm[:, None]], axis=1)

    centroid = at(np.zeros(3))
    nodal = np.stack([at(HEX_CORNERS[k]) for k in range(8)], axis=1)
    return centroid, nodal


def block_jacobi_inverse(K: Csr) -> np.ndarray:
    """Inverse 3x3 diagonal block of every node (equations 3i..3i+2), from the
    blocks' upper triangles mirrored (the symmetric part), (n/3, 3, 3).

    No reference counterpart: the reference's cuda-pcg preconditions with IC0
    and falls back to scalar Jacobi (src/solver/cuda_pcg_backend_impl.hpp:
    1041-1252); the 3x3 block form is the block-diagonal of the same K."""
    if K.n % 3:
        raise OracleError("block Jacobi needs node-aligned equation triples")
    full = K if not K.lower else K.expanded_symmetric()
    nb = K.n // 3
    D = np.zeros((nb, 3, 3))
    rows = np.repeat(np.arange(full.n), np.diff(full.row_ptr))
    cols = np.asarray(full.col_ind)
    sel = (rows // 3 == cols // 3) & (rows % 3 <= cols % 3)
    r, c, v = rows[sel], cols[sel], np.asarray(full.values)[sel]
    D[r // 3, r % 3, c % 3] = v
    D[r // 3, c % 3, r % 3] = v
    return np.linalg.inv(D)


def pcg_block_jacobi(K: Csr, F, tol=1e-8, max_iters=10000):
    """FP64 PCG with the 3x3 block Jacobi preconditioner z_I = B_I r_I: the
    recurrence, stopping test (sqrt(r.r)/||b|| < tol) and zero-RHS / rz <= 0 /
    pAp <= 0 handling of the oracle's scalar Jacobi PCG (run_pcg_prepared,
    src/solver/cuda_pcg_backend_impl.hpp:1688-1999).  Returns (u, iters, rel)."""
    import scipy.sparse as sp
    full = K if not K.lower else K.expanded_symmetric()
    A = sp.csr_matrix((full.values, full.col_ind, full.row_ptr), shape=(full.n, full.n))
    B = block_jacobi_inverse(K)
    nb = K.n // 3

    def prec(r):
        return np.einsum("ijk,ik->ij", B, r.reshape(nb, 3)).reshape(-1)

    b = np.asarray(F, np.float64)
    u = np.zeros(K.n)
    norm_b = np.sqrt(abs(b @ b))
    if norm_b < 1e-300:
        return u, 0, 0.0
    r = b.copy()
    z = prec(r)
    p = z.copy()
    rz = r @ z
    if not rz > 0.0:
        raise OracleError("non-positive initial r*z -- preconditioner is not SPD or matrix "
                          "is singular")
    rel = 1.0
    for it in range(max_iters):
        Ap = A @ p
        pAp = p @ Ap
        if not pAp > 0.0:
            break
        alpha = rz / pAp
        u += alpha * p
        r -= alpha * Ap
        z = prec(r)
        rz_new = r @ z
        rel = np.sqrt(abs(r @ r)) / norm_b
        if rel < tol:
            return u, it + 1, rel
        p = z + (rz_new / rz) * p
        rz = rz_new
    raise OracleError(f"did not converge after {max_iters} iterations (relative residual "
                      f"{rel:g} > tolerance {tol:g})")
