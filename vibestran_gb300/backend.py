"""Host-side mirror of vibestran's SolverBackend over the libvsgb C ABI.

The classes follow the reference's interface for this path:

* :class:`CsrData` — ``SparseMatrixBuilder::CsrData``
  (include/core/sparse_matrix.hpp:63-87): row_ptr / col_ind / values, n, nnz
  and the symmetry tag (lower-triangle or full storage).
* :class:`Gb300PcgSolverBackend` — a drop-in for ``CudaPCGSolverBackend``
  (include/solver/cuda_pcg_solver_backend.hpp:33-75): ``try_create`` returns
  ``None`` when no usable GPU exists, ``solve`` raises :class:`SolverError`
  with the reference's messages, and the diagnostics accessors match.
* :class:`Gb300MixedPcgSolverBackend` — ``CudaMixedPCGSolverBackend``
  (include/solver/cuda_mixed_pcg_solver_backend.hpp), with the refinement
  residual, update and norms kept in FP64 on the GPU.
* :class:`ChexaAssembler` — GPU element stiffness + assembly for a CHEXA8
  model (the layers above ``SolverBackend::solve`` in
  src/solver/linear_static.cpp:233-260).

Every numeric call goes through ``libvsgb.so``; there is no CPU fallback —
importing on a machine without the built library raises immediately.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

VSGB_OK = 0
VSGB_ERR_INVALID = -1
VSGB_ERR_SINGULAR = -2
VSGB_ERR_NOT_CONVERGED = -3
VSGB_ERR_CUDA = -4
VSGB_ERR_ELEMENT = -5
VSGB_ERR_NO_DEVICE = -6
VSGB_ERR_STATE = -7
VSGB_ERR_LIMIT = -8

FP64 = 64
MIXED = 32
EAS = 0
SRI = 1

OPT_TOLERANCE = 1
OPT_MAX_ITERS = 2
OPT_PRECISION = 3
OPT_INNER_TOL = 4
OPT_MAX_SOLVES = 5
OPT_CHECK_EVERY = 6
OPT_USE_GRAPH = 7
OPT_FORMAT = 8
OPT_RESIDENT = 9
OPT_BATCHED = 10
OPT_L2_PERSIST = 11
OPT_ADAPTIVE_INNER = 12
OPT_PRECOND = 13
OPT_ERROR_TARGET = 14
OPT_SPIN_LIMIT = 15
OPT_PHASE_TRACE = 16
OPT_BATCH_TILES = 17
OPT_COARSE = 18

PRECOND_JACOBI = 0
PRECOND_BLOCK_JACOBI = 1

# The symbols include/vsgb.h declares (checked by tests against the .so).
EXPORTS = (
    "vsgb_rhs_stats", "vsgb_adjoint_gradients", "vsgb_solid_stress",
    "vsgb_bdf_read", "vsgb_bdf_parse", "vsgb_bdf_free", "vsgb_bdf_info", "vsgb_bdf_message",
    "vsgb_bdf_subcase", "vsgb_bdf_mesh", "vsgb_bdf_constraints", "vsgb_bdf_forces",
    "vsgb_create", "vsgb_destroy", "vsgb_set_option", "vsgb_last_error", "vsgb_device_name",
    "vsgb_backend_name", "vsgb_solve_csr", "vsgb_build_dof_map", "vsgb_apply_forces",
    "vsgb_assemble_chexa8", "vsgb_copy_csr_lower", "vsgb_solve_assembled", "vsgb_mesh_upload",
    "vsgb_assemble_resident", "vsgb_rhs_upload", "vsgb_solve_resident",
    "vsgb_host_alloc", "vsgb_host_free",
    "vsgb_solution_download", "vsgb_element_sensitivity", "vsgb_timer_start",
    "vsgb_timer_stop", "vsgb_time_spmv", "vsgb_kernel_launches", "vsgb_phase_times",
    "vsgb_pcg_solve_noalloc", "vsgb_node_displacements", "vsgb_write_node_csv",
)
NOALLOC_MAX_N = 65536  # VSGB_NOALLOC_MAX_N


class SolverError(RuntimeError):
    """vibestran::SolverError (include/core/exceptions.hpp:14)."""

    def __init__(self, msg: str, code: int = VSGB_ERR_INVALID):
        super().__init__(msg)
        self.code = code


class BdfStats(ctypes.Structure):
    """vsgb_bdf_stats."""
    _fields_ = [("n_nodes", ctypes.c_int), ("n_elem", ctypes.c_int),
                ("n_subcases", ctypes.c_int), ("sol", ctypes.c_int),
                ("lines", ctypes.c_longlong), ("cards", ctypes.c_longlong),
                ("threads", ctypes.c_int), ("read_ms", ctypes.c_double),
                ("parse_ms", ctypes.c_double), ("mesh_ok", ctypes.c_int),
                ("lines_ms", ctypes.c_double), ("cards_ms", ctypes.c_double),
                ("mesh_ms", ctypes.c_double)]


class VsgbStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("inner_solves", ctypes.c_int),
                ("converged", ctypes.c_int), ("format", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("solve_ms", ctypes.c_double),
                ("setup_ms", ctypes.c_double), ("spmv_bytes", ctypes.c_double),
                ("kernel_ms", ctypes.c_double), ("kernel_iterations", ctypes.c_double),
                ("est_rel_error", ctypes.c_double), ("batch_tile_rows", ctypes.c_int)]


_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_lib = None


def library_path() -> str:
    return _build.LIB


def load_library(build_if_missing: bool = False):
    """Load libvsgb.so (raises if it was not built — no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(f"libvsgb.so is not built ({path}); run __graft_entry__.build()")
    L = ctypes.CDLL(path)
    c_int, c_dbl, c_ll = ctypes.c_int, ctypes.c_double, ctypes.c_longlong
    vp, cp, sz = ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t
    L.vsgb_create.argtypes = [c_int, c_dbl, c_int, c_int, ctypes.POINTER(vp)]
    L.vsgb_destroy.argtypes = [vp]
    L.vsgb_destroy.restype = None
    L.vsgb_set_option.argtypes = [vp, c_int, c_dbl]
    L.vsgb_last_error.argtypes = [vp, cp, sz]
    L.vsgb_device_name.argtypes = [vp, cp, sz]
    L.vsgb_backend_name.argtypes = [vp, cp, sz]
    L.vsgb_solve_csr.argtypes = [vp, c_int, c_int, _i32p, _i32p, _f64p, c_int, _f64p, c_int,
                                 _f64p, ctypes.POINTER(VsgbStats)]
    L.vsgb_build_dof_map.argtypes = [c_int, _i32p, c_int, _i32p, c_int, _i32p, _i32p, _i32p,
                                     ctypes.POINTER(c_int), cp, sz]
    L.vsgb_apply_forces.argtypes = [c_int, _i32p, _i32p, c_int, _i32p, _f64p, _f64p, c_int,
                                    _f64p, cp, sz]
    L.vsgb_assemble_chexa8.argtypes = [vp, c_int, _f64p, _i32p, c_int, _i32p, _f64p, _f64p, vp,
                                       c_int, ctypes.POINTER(c_ll)]
    L.vsgb_mesh_upload.argtypes = [vp, c_int, _f64p, _i32p, c_int, _i32p, _f64p, _f64p, vp, c_int]
    L.vsgb_assemble_resident.argtypes = [vp, ctypes.POINTER(c_ll)]
    L.vsgb_copy_csr_lower.argtypes = [vp, _i32p, _i32p, _f64p]
    L.vsgb_solve_assembled.argtypes = [vp, _f64p, c_int, _f64p, ctypes.POINTER(VsgbStats)]
    L.vsgb_rhs_upload.argtypes = [vp, _f64p, c_int]
    L.vsgb_solve_resident.argtypes = [vp, ctypes.POINTER(VsgbStats)]
    L.vsgb_solution_download.argtypes = [vp, _f64p]
    L.vsgb_host_alloc.argtypes = [vp, sz, ctypes.POINTER(vp)]
    L.vsgb_host_free.argtypes = [vp, vp]
    L.vsgb_element_sensitivity.argtypes = [vp, _f64p, _f64p, _f64p]
    L.vsgb_timer_start.argtypes = [vp]
    L.vsgb_timer_stop.argtypes = [vp, ctypes.POINTER(c_dbl)]
    L.vsgb_time_spmv.argtypes = [vp, c_int, c_int, ctypes.POINTER(c_dbl), ctypes.POINTER(c_dbl)]
    L.vsgb_kernel_launches.argtypes = [vp]
    L.vsgb_kernel_launches.restype = c_ll
    L.vsgb_phase_times.argtypes = [vp, _f64p]
    L.vsgb_adjoint_gradients.argtypes = [vp, _f64p, vp, vp, vp, vp, vp, ctypes.POINTER(VsgbStats)]
    L.vsgb_solid_stress.argtypes = [vp, vp, c_int, _f64p, vp, ctypes.POINTER(c_dbl)]
    L.vsgb_node_displacements.argtypes = [vp, vp, c_int, _f64p]
    L.vsgb_write_node_csv.argtypes = [cp, c_int, _i32p, c_int, _i32p, _f64p, cp, sz]
    L.vsgb_bdf_read.argtypes = [cp, c_int, ctypes.POINTER(vp), cp, sz]
    L.vsgb_bdf_parse.argtypes = [cp, sz, c_int, ctypes.POINTER(vp), cp, sz]
    L.vsgb_bdf_free.argtypes = [vp]
    L.vsgb_bdf_free.restype = None
    L.vsgb_bdf_info.argtypes = [vp, ctypes.POINTER(BdfStats)]
    L.vsgb_bdf_message.argtypes = [vp, c_int, cp, sz]
    L.vsgb_bdf_subcase.argtypes = [vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                                   ctypes.POINTER(c_int)]
    L.vsgb_bdf_mesh.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp]
    L.vsgb_bdf_constraints.argtypes = [vp, c_int, ctypes.POINTER(c_int), vp, vp]
    L.vsgb_bdf_forces.argtypes = [vp, c_int, ctypes.POINTER(c_int), vp, vp, vp]
    L.vsgb_rhs_stats.argtypes = [vp, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_dbl),
                                 ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.vsgb_pcg_solve_noalloc.argtypes = [c_int, c_int, vp, vp, vp, vp, vp, c_dbl, c_int, vp,
                                         ctypes.POINTER(c_int), ctypes.POINTER(c_dbl), cp, sz]
    _lib = L
    return L


@dataclass
class CsrData:
    """SparseMatrixBuilder::CsrData: lower-triangle (``lower=True``) or full storage."""
    row_ptr: np.ndarray
    col_ind: np.ndarray
    values: np.ndarray
    n: int
    nnz: int
    lower: bool = True

    def stores_lower_triangle_only(self) -> bool:
        return self.lower


class _Context:
    def __init__(self, ptr):
        self.ptr = ptr
        self.pinned = []  # page-locked host blocks, freed with the context

    def check(self, rc: int):
        if rc != VSGB_OK:
            raise SolverError(self.last_error(), rc)

    def last_error(self) -> str:
        buf = ctypes.create_string_buffer(1024)
        load_library().vsgb_last_error(self.ptr, buf, 1024)
        return buf.value.decode(errors="replace")

    def close(self):
        if self.ptr:
            L = load_library()
            for p in self.pinned:
                L.vsgb_host_free(self.ptr, p)
            self.pinned = []
            L.vsgb_destroy(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _create(device: int, tol: float, max_iters: int, precision: int):
    L = load_library()
    p = ctypes.c_void_p()
    rc = L.vsgb_create(device, float(tol), int(max_iters), precision, ctypes.byref(p))
    if rc == VSGB_ERR_NO_DEVICE:
        return None
    if rc != VSGB_OK:
        raise SolverError(f"vsgb_create failed with status {rc}", rc)
    return _Context(p)


class Gb300PcgSolverBackend:
    """Drop-in for CudaPCGSolverBackend (FP64 Jacobi PCG on sm_103a)."""

    precision = FP64

    def __init__(self, ctx: _Context):
        self._ctx = ctx
        self._iters = 0
        self._rel = 0.0
        self.last_stats = VsgbStats()

    @classmethod
    def try_create(cls, tolerance: float = 0.0, max_iters: int = 0, device: int = 0):
        """None when no CUDA device (cuda_pcg_solver_backend.cu:19-25)."""
        ctx = _create(device, tolerance, max_iters, cls.precision)
        return None if ctx is None else cls(ctx)

    def set_option(self, option: int, value: float):
        self._ctx.check(load_library().vsgb_set_option(self._ctx.ptr, option, float(value)))

    def pinned_empty(self, shape, dtype=np.float64) -> np.ndarray:
        """Uninitialised page-locked host array (vsgb_host_alloc) for the
        host arrays handed to the library; valid until close()."""
        dt = np.dtype(dtype)
        shape = (int(shape),) if np.isscalar(shape) else tuple(int(x) for x in shape)
        count = int(np.prod(shape))
        nbytes = max(count * dt.itemsize, 1)
        p = ctypes.c_void_p()
        self._ctx.check(load_library().vsgb_host_alloc(self._ctx.ptr, nbytes, ctypes.byref(p)))
        self._ctx.pinned.append(p.value)
        buf = (ctypes.c_char * nbytes).from_address(p.value)
        return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)

    def pinned_copy(self, a) -> np.ndarray:
        """Page-locked copy of a host array (same shape and dtype)."""
        a = np.asarray(a)
        out = self.pinned_empty(a.shape, a.dtype)
        out[...] = a
        return out

    def solve(self, K: CsrData, F, factor_ratio_policy=None) -> np.ndarray:
        """SolverBackend::solve: K as CsrData, F (n,) or (n, nrhs) -> u."""
        F = np.asarray(F, dtype=np.float64)
        if K.n == 0:
            raise SolverError("CUDA PCG: stiffness matrix is empty -- no free DOFs")
        if F.shape[0] != K.n:
            raise SolverError(f"CUDA PCG: force vector size {F.shape[0]} != matrix size {K.n}")
        nrhs = 1 if F.ndim == 1 else F.shape[1]
        Fc = np.ascontiguousarray(F.T if F.ndim == 2 else F).reshape(-1)
        u = np.zeros(K.n * nrhs)
        st = VsgbStats()
        rc = load_library().vsgb_solve_csr(
            self._ctx.ptr, int(K.n), int(K.nnz), np.ascontiguousarray(K.row_ptr, np.int32),
            np.ascontiguousarray(K.col_ind, np.int32), np.ascontiguousarray(K.values, np.float64),
            1 if K.lower else 0, Fc, nrhs, u, ctypes.byref(st))
        self._ctx.check(rc)
        self._record(st)
        return u if nrhs == 1 else u.reshape(nrhs, K.n).T.copy()

    def _record(self, st: VsgbStats):
        self.last_stats = st
        self._iters = st.iterations
        self._rel = st.rel_residual

    def name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        load_library().vsgb_backend_name(self._ctx.ptr, buf, 256)
        return buf.value.decode()

    def device_name(self) -> str:
        buf = ctypes.create_string_buffer(256)
        load_library().vsgb_device_name(self._ctx.ptr, buf, 256)
        return buf.value.decode()

    def last_iteration_count(self) -> int:
        return self._iters

    def last_relative_residual(self) -> float:
        return self._rel

    def last_estimated_error(self) -> float:
        return self._rel

    def requires_full_symmetric_csr(self) -> bool:
        return False

    def kernel_launches(self) -> int:
        return int(load_library().vsgb_kernel_launches(self._ctx.ptr))

    def rhs_stats(self, k: int) -> dict:
        """Outcome of load case k in the last solve (iterations, relative
        residual, converged, whether the cases ran as one batched PCG)."""
        it, conv, bat = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
        rel = ctypes.c_double(0.0)
        self._ctx.check(load_library().vsgb_rhs_stats(
            self._ctx.ptr, k, ctypes.byref(it), ctypes.byref(rel), ctypes.byref(conv),
            ctypes.byref(bat)))
        return {"iterations": it.value, "rel_residual": rel.value,
                "converged": bool(conv.value), "batched": bool(bat.value)}

    @property
    def context(self) -> _Context:
        return self._ctx

    def close(self):
        self._ctx.close()


class Gb300MixedPcgSolverBackend(Gb300PcgSolverBackend):
    """Drop-in for CudaMixedPCGSolverBackend (default tolerance 1e-6)."""

    precision = MIXED


def build_dof_map(model):
    """Analysis DOF map through the library (host C++): (eq6 (N,6), n_free)."""
    L = load_library()
    eq = np.empty(model.n_nodes * 6, np.int32)
    nf = ctypes.c_int()
    err = ctypes.create_string_buffer(512)
    rc = L.vsgb_build_dof_map(model.n_nodes, np.ascontiguousarray(model.node_ids, np.int32),
                              model.n_elem, np.ascontiguousarray(model.conn_ids(), np.int32).reshape(-1),
                              int(model.spc_nodes.shape[0]),
                              np.ascontiguousarray(model.spc_nodes, np.int32),
                              np.ascontiguousarray(model.spc_mask, np.int32), eq,
                              ctypes.byref(nf), err, 512)
    if rc != VSGB_OK:
        raise SolverError(err.value.decode(), rc)
    return eq.reshape(-1, 6), nf.value


def apply_forces(model, eq6, n, load_index=0):
    nodes, scale, dirs = model.loads[load_index]
    F = np.zeros(n)
    err = ctypes.create_string_buffer(512)
    rc = load_library().vsgb_apply_forces(
        model.n_nodes, np.ascontiguousarray(model.node_ids, np.int32),
        np.ascontiguousarray(eq6, np.int32).reshape(-1), int(len(nodes)),
        np.ascontiguousarray(nodes, np.int32), np.ascontiguousarray(scale, np.float64),
        np.ascontiguousarray(dirs, np.float64).reshape(-1), int(n), F, err, 512)
    if rc != VSGB_OK:
        raise SolverError(err.value.decode(), rc)
    return F


class ChexaAssembler:
    """GPU CHEXA8 element stiffness + assembly bound to a backend context.

    ``assemble(model, eq6, n)`` uploads the mesh and assembles K on the GPU;
    ``csr_lower()`` returns the reference's lower-triangle CsrData;
    ``solve(F)`` solves with the resident K (F may hold several load cases).
    """

    def __init__(self, backend: Gb300PcgSolverBackend):
        self.backend = backend
        self.n = 0
        self.nnz_lower = 0
        self.n_elem = 0
        self.n_nodes = 0

    def upload(self, model, eq6, n):
        L = load_library()
        eq6 = np.asarray(eq6)
        # an (N, 3) int32 table is passed as is (no copy); (N, 6) is sliced
        eq3 = np.ascontiguousarray(eq6 if eq6.shape[1] == 3 else eq6[:, :3], np.int32).reshape(-1)
        form = np.ascontiguousarray(model.form, np.int32)
        rc = L.vsgb_mesh_upload(self.backend.context.ptr, model.n_nodes,
                                np.ascontiguousarray(model.xyz, np.float64).reshape(-1), eq3,
                                model.n_elem, np.ascontiguousarray(model.conn, np.int32).reshape(-1),
                                np.ascontiguousarray(model.E, np.float64),
                                np.ascontiguousarray(model.nu, np.float64),
                                form.ctypes.data_as(ctypes.c_void_p), int(n))
        self.backend.context.check(rc)
        self.n = int(n)
        self.n_elem = model.n_elem
        self.n_nodes = model.n_nodes

    def assemble_resident(self) -> int:
        nnz = ctypes.c_longlong()
        self.backend.context.check(
            load_library().vsgb_assemble_resident(self.backend.context.ptr, ctypes.byref(nnz)))
        self.nnz_lower = int(nnz.value)
        return self.nnz_lower

    def assemble(self, model, eq6, n) -> int:
        self.upload(model, eq6, n)
        return self.assemble_resident()

    def csr_lower(self) -> CsrData:
        rp = np.empty(self.n + 1, np.int32)
        ci = np.empty(self.nnz_lower, np.int32)
        v = np.empty(self.nnz_lower, np.float64)
        self.backend.context.check(
            load_library().vsgb_copy_csr_lower(self.backend.context.ptr, rp, ci, v))
        return CsrData(rp, ci, v, self.n, self.nnz_lower, True)

    def solve(self, F, out=None) -> np.ndarray:
        """u for F (n,) or (n, nrhs); out: optional (n,) float64 array that
        receives u (single load case, e.g. a page-locked one)."""
        F = np.asarray(F, dtype=np.float64)
        nrhs = 1 if F.ndim == 1 else F.shape[1]
        Fc = np.ascontiguousarray(F.T if F.ndim == 2 else F).reshape(-1)
        if out is not None:
            if nrhs != 1 or out.dtype != np.float64 or out.shape != (self.n,) or \
                    not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous (n,) float64 array, one load case")
            u = out
        else:
            u = np.zeros(self.n * nrhs)
        st = VsgbStats()
        self.backend.context.check(load_library().vsgb_solve_assembled(
            self.backend.context.ptr, Fc, nrhs, u, ctypes.byref(st)))
        self.backend._record(st)
        return u if nrhs == 1 else u.reshape(nrhs, self.n).T.copy()

    def upload_rhs(self, F):
        F = np.asarray(F, dtype=np.float64)
        nrhs = 1 if F.ndim == 1 else F.shape[1]
        Fc = np.ascontiguousarray(F.T if F.ndim == 2 else F).reshape(-1)
        self.backend.context.check(
            load_library().vsgb_rhs_upload(self.backend.context.ptr, Fc, nrhs))
        self._nrhs = nrhs

    def solve_resident(self) -> VsgbStats:
        st = VsgbStats()
        self.backend.context.check(
            load_library().vsgb_solve_resident(self.backend.context.ptr, ctypes.byref(st)))
        self.backend._record(st)
        return st

    def download(self) -> np.ndarray:
        nrhs = getattr(self, "_nrhs", 1)
        u = np.zeros(self.n * nrhs)
        self.backend.context.check(
            load_library().vsgb_solution_download(self.backend.context.ptr, u))
        return u if nrhs == 1 else u.reshape(nrhs, self.n).T.copy()

    def solid_stress(self, u=None, k=0, nodal=True):
        """CHEXA8 stresses (linear_static.cpp:1059-1195): returns (centroid
        (n_elem, 7), nodal (n_elem, 8, 7) or None, kernel ms), columns sx, sy,
        sz, sxy, syz, szx, von Mises.  u: host displacements, or None for load
        case k of the last solve."""
        cen = np.zeros((self.n_elem, 7))
        nod = np.zeros((self.n_elem, 8, 7)) if nodal else None
        u_in = None if u is None else np.ascontiguousarray(u, np.float64)
        ms = ctypes.c_double(0.0)
        self.backend.context.check(load_library().vsgb_solid_stress(
            self.backend.context.ptr,
            None if u_in is None else u_in.ctypes.data_as(ctypes.c_void_p), k, cen,
            None if nod is None else nod.ctypes.data_as(ctypes.c_void_p), ctypes.byref(ms)))
        return cen, nod, ms.value

    def node_displacements(self, u=None, k=0) -> np.ndarray:
        """Nodal displacements (recover_results, linear_static.cpp:574-587):
        (n_nodes, 6) T1 T2 T3 R1 R2 R3 in the uploaded node order, 0 for
        constrained DOFs.  u: host displacements, or None for load case k of
        the last solve."""
        out = np.zeros((self.n_nodes, 6))
        u_in = None if u is None else np.ascontiguousarray(u, np.float64)
        self.backend.context.check(load_library().vsgb_node_displacements(
            self.backend.context.ptr,
            None if u_in is None else u_in.ctypes.data_as(ctypes.c_void_p), k, out.reshape(-1)))
        return out

    def adjoint_gradients(self, F, dJdu=None, with_adjoint=False):
        """Compliance and linear-response gradients w.r.t. every element's E
        from one solve of K [u, lam] = [F, dJdu]: returns (u, dC/dE, dJ/dE or
        None), plus lam when with_adjoint."""
        F = np.ascontiguousarray(F, np.float64)
        u = np.zeros(self.n)
        dC = np.zeros(self.n_elem)
        has_j = dJdu is not None
        dJ = np.zeros(self.n_elem) if has_j else None
        lam = np.zeros(self.n) if (has_j and with_adjoint) else None
        dj_in = np.ascontiguousarray(dJdu, np.float64) if has_j else None

        def ptr(a):
            return None if a is None else a.ctypes.data_as(ctypes.c_void_p)

        st = VsgbStats()
        self.backend.context.check(load_library().vsgb_adjoint_gradients(
            self.backend.context.ptr, F, ptr(dj_in), ptr(u), ptr(lam), ptr(dC), ptr(dJ),
            ctypes.byref(st)))
        self.backend._record(st)
        return (u, dC, dJ, lam) if with_adjoint else (u, dC, dJ)

    def sensitivity(self, u, lam) -> np.ndarray:
        out = np.zeros(self.n_elem)
        self.backend.context.check(load_library().vsgb_element_sensitivity(
            self.backend.context.ptr, np.ascontiguousarray(u, np.float64),
            np.ascontiguousarray(lam, np.float64), out))
        return out


def timer_start(backend):
    backend.context.check(load_library().vsgb_timer_start(backend.context.ptr))


def timer_stop(backend) -> float:
    ms = ctypes.c_double()
    backend.context.check(load_library().vsgb_timer_stop(backend.context.ptr, ctypes.byref(ms)))
    return ms.value


def phase_times(backend) -> dict:
    """Per-iteration phase split of the last persistent solve (us, mean over
    CTAs) when OPT_PHASE_TRACE is on."""
    t = np.zeros(11)
    backend.context.check(load_library().vsgb_phase_times(backend.context.ptr, t))
    return {"gather_us": t[0], "spmv_us": t[1],
            "reduction1_us": t[2] + t[3] + t[4], "reduction1_cta_us": t[2],
            "reduction1_wait_us": t[3], "reduction1_total_us": t[4], "update_us": t[5],
            "reduction2_us": t[6] + t[7] + t[8], "reduction2_cta_us": t[6],
            "reduction2_wait_us": t[7], "reduction2_total_us": t[8],
            "spmv_slowest_cta_us": t[9], "iterations": int(t[10])}


def time_spmv(backend, precision: int, reps: int = 50):
    ms = ctypes.c_double()
    by = ctypes.c_double()
    backend.context.check(load_library().vsgb_time_spmv(backend.context.ptr, precision, reps,
                                                        ctypes.byref(ms), ctypes.byref(by)))
    return ms.value, by.value


# ── BDF decks ──────────────────────────────────────────────────────────────

class BdfDeck:
    """A deck read by the native reader (vsgb_bdf_*): ``stats``, ``subcases``
    [(id, load set, spc set)], ``warnings`` (ignored cards) and ``model()``,
    the SolidModel of the CHEXA8 path.  Parse errors raise SolverError with
    the reference's "Line N: ..." text."""

    def __init__(self, path=None, text=None, threads=0):
        L = load_library()
        self._L = L
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(1024)
        if path is not None:
            rc = L.vsgb_bdf_read(os.fsencode(path), threads, ctypes.byref(h), err, 1024)
        else:
            data = text.encode() if isinstance(text, str) else bytes(text)
            rc = L.vsgb_bdf_parse(data, len(data), threads, ctypes.byref(h), err, 1024)
        if rc != VSGB_OK:
            raise SolverError(err.value.decode(errors="replace"), rc)
        self._h = h
        st = BdfStats()
        L.vsgb_bdf_info(h, ctypes.byref(st))
        self.stats = {k: getattr(st, k) for k, _ in BdfStats._fields_}
        self.subcases = []
        for s_ in range(st.n_subcases):
            a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            L.vsgb_bdf_subcase(h, s_, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
            self.subcases.append((a.value, b.value, c.value))
        self.warnings = self._message(1)
        self.mesh_error = self._message(0)

    def _message(self, which):
        buf = ctypes.create_string_buffer(4096)
        self._L.vsgb_bdf_message(self._h, which, buf, 4096)
        return buf.value.decode(errors="replace")

    def _check(self, rc):
        if rc != VSGB_OK:
            raise SolverError(self._message(2), rc)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.vsgb_bdf_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def mesh(self):
        """(node_ids, xyz, elem_ids, conn, E, nu, form)."""
        st = self.stats
        N, M = st["n_nodes"], st["n_elem"]
        ids = np.zeros(N, np.int32)
        xyz = np.zeros((N, 3))
        eids = np.zeros(M, np.int32)
        conn = np.zeros((M, 8), np.int32)
        E = np.zeros(M)
        nu = np.zeros(M)
        form = np.zeros(M, np.int32)

        def p(a):
            return a.ctypes.data_as(ctypes.c_void_p)

        self._check(self._L.vsgb_bdf_mesh(self._h, p(ids), p(xyz), p(eids), p(conn), p(E), p(nu),
                                          p(form)))
        return ids, xyz, eids, conn, E, nu, form

    def constraints(self, s=0):
        n = ctypes.c_int()
        self._check(self._L.vsgb_bdf_constraints(self._h, s, ctypes.byref(n), None, None))
        nodes = np.zeros(n.value, np.int32)
        masks = np.zeros(n.value, np.int32)
        self._check(self._L.vsgb_bdf_constraints(self._h, s, ctypes.byref(n),
                                                 nodes.ctypes.data_as(ctypes.c_void_p),
                                                 masks.ctypes.data_as(ctypes.c_void_p)))
        return nodes, masks

    def forces(self, s=0):
        n = ctypes.c_int()
        self._check(self._L.vsgb_bdf_forces(self._h, s, ctypes.byref(n), None, None, None))
        nodes = np.zeros(n.value, np.int32)
        scale = np.zeros(n.value)
        dirs = np.zeros((n.value, 3))
        self._check(self._L.vsgb_bdf_forces(self._h, s, ctypes.byref(n),
                                            nodes.ctypes.data_as(ctypes.c_void_p),
                                            scale.ctypes.data_as(ctypes.c_void_p),
                                            dirs.ctypes.data_as(ctypes.c_void_p)))
        return nodes, scale, dirs

    def model(self, subcases=None, name="bdf"):
        """SolidModel with the SPC set of the first chosen subcase and one load
        case per chosen subcase (all must share that SPC set)."""
        from . import cantilever as C
        chosen = list(range(len(self.subcases))) if subcases is None else list(subcases)
        spc_sets = {self.subcases[s][2] for s in chosen}
        if len(spc_sets) != 1:
            raise SolverError("the chosen subcases use different SPC sets; take one at a time")
        ids, xyz, eids, conn, E, nu, form = self.mesh()
        spc_nodes, spc_mask = self.constraints(chosen[0])
        loads = [self.forces(s) for s in chosen]
        return C.SolidModel(node_ids=ids, xyz=xyz, conn=conn, elem_ids=eids, E=E, nu=nu,
                            form=form, spc_nodes=spc_nodes, spc_mask=spc_mask, loads=loads,
                            name=name)


def write_node_csv(path, node_ids, disp, subcase_ids=(1,)):
    """CsvWriter's nodal CSV (csv_writer.cpp:34-57) of disp ((n_subcases,)
    n_nodes, 6) in the node order of node_ids, listed in ascending id order."""
    ids = np.ascontiguousarray(node_ids, np.int32)
    d = np.ascontiguousarray(disp, np.float64).reshape(-1, ids.size, 6)
    sc = np.ascontiguousarray(subcase_ids, np.int32)
    if sc.size != d.shape[0]:
        raise SolverError("one subcase id per displacement block")
    err = ctypes.create_string_buffer(512)
    rc = load_library().vsgb_write_node_csv(os.fsencode(path), ids.size, ids, sc.size, sc,
                                            d.reshape(-1), err, 512)
    if rc != VSGB_OK:
        raise SolverError(err.value.decode(), rc)


def read_bdf(path=None, text=None, threads=0) -> BdfDeck:
    """Read a BDF deck (a file path, or the deck text) with the native reader."""
    if (path is None) == (text is None):
        raise ValueError("give exactly one of path / text")
    return BdfDeck(path=path, text=text, threads=threads)
