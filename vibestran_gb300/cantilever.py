"""Synthetic CHEXA8 block models with the conventions of vibestran's mesh generator.

The reference generator (tools/generate_chexa_mesh.py:93-125, 249, 257-273,
313, 347-348) numbers nodes ``id = i*(ny+1)*(nz+1) + j*(nz+1) + k + 1`` (i along
x, j along y, k along z), writes CHEXA8 connectivity bottom face first
(z-min, counter-clockwise) then top face, uses ``PSOLID,1,1,,2`` (ISOP blank,
so the default EAS formulation), clamps T1-T3 on every x=0 node with SPC1 and
applies FORCE cards on the x=L face.  The models here follow those
conventions; coordinates and moduli are kept as exact doubles (a BDF written by
:func:`write_bdf` uses round-trip ``%.17g`` formatting, not the generator's
``%.6E``), so every path sees identical inputs.

Standard workloads (all edges in metres, E in Pa):

* ``cantilever_1500``: 20x4x4 elements, 0.05 m edge, 525 grids, n = 1 500,
  1000 N in -z over the x=L face.
* ``cantilever_84k``: 60x40x35 elements, 0.01 m edge, 90 036 grids,
  n = 265 680, same material, clamp and load.
* ``cantilever_84k_jitter``: the same block with interior nodes jittered by a
  seeded uniform +-0.2*edge and per-element E log-uniform in [20e9, 400e9].
* ``block_160k_16rhs``: 100x40x40, n = 504 300, 16 load cases of seeded
  N(0, 100 N) nodal forces in x/y/z on the z-max face.
* ``block_250k_adjoint``: 100x50x50, n = 780 300, per-element log-uniform E,
  1000 N -z tip load.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

EAS = 0
SRI = 1


@dataclass
class SolidModel:
    """A CHEXA8-only SOL 101 model in flat arrays.

    node_ids:  (N,) int32 grid ids (any order, unique, positive)
    xyz:       (N, 3) float64 coordinates
    conn:      (M, 8) int32 element connectivity as 0-based indices into the
               node arrays (CHEXA8 node order G1..G8)
    elem_ids:  (M,) int32 element ids
    E, nu:     (M,) float64 per-element MAT1 modulus and Poisson ratio
    form:      (M,) int32 per-element formulation (EAS=0, SRI=1)
    spc_nodes: (S,) int32 grid ids with an SPC1
    spc_mask:  (S,) int32 constrained components, bit d = DOF d+1
    force_nodes / force_scale / force_dir: FORCE cards (CID 0); force_dir is
               (F, 3); several load cases are given as a list of such triples
    """

    node_ids: np.ndarray
    xyz: np.ndarray
    conn: np.ndarray
    elem_ids: np.ndarray
    E: np.ndarray
    nu: np.ndarray
    form: np.ndarray
    spc_nodes: np.ndarray
    spc_mask: np.ndarray
    loads: list = field(default_factory=list)  # list of (nodes, scale, dir)
    name: str = ""
    shape: tuple = ()
    seed: int | None = None

    @property
    def n_nodes(self) -> int:
        return int(self.node_ids.shape[0])

    @property
    def n_elem(self) -> int:
        return int(self.conn.shape[0])

    def conn_ids(self) -> np.ndarray:
        """Connectivity as grid ids (what a CHEXA card holds)."""
        return self.node_ids[self.conn]


def node_id(i, j, k, ny, nz):
    """1-based grid id of mesh index (i, j, k) (generate_chexa_mesh.py:93-95)."""
    return i * (ny + 1) * (nz + 1) + j * (nz + 1) + k + 1


def block(nx: int, ny: int, nz: int, edge: float, E: float = 200e9, nu: float = 0.3,
          form: int = EAS, name: str = "") -> SolidModel:
    """Clamped-at-x=0 CHEXA8 block of nx*ny*nz cubes of the given edge."""
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1),
                          indexing="ij")
    ids = node_id(i, j, k, ny, nz).reshape(-1).astype(np.int32)
    xyz = np.stack([i * edge, j * edge, k * edge], axis=-1).reshape(-1, 3).astype(np.float64)
    # Node index == id - 1 because ids are generated in index order.
    ie, je, ke = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ie, je, ke = ie.reshape(-1), je.reshape(-1), ke.reshape(-1)

    def nidx(di, dj, dk):
        return node_id(ie + di, je + dj, ke + dk, ny, nz) - 1

    # generate_chexa_mesh.py:98-125 element node order
    conn = np.stack([nidx(0, 0, 0), nidx(1, 0, 0), nidx(1, 1, 0), nidx(0, 1, 0),
                     nidx(0, 0, 1), nidx(1, 0, 1), nidx(1, 1, 1), nidx(0, 1, 1)],
                    axis=1).astype(np.int32)
    m = conn.shape[0]
    clamp = ids[(i == 0).reshape(-1)]
    return SolidModel(
        node_ids=ids, xyz=xyz, conn=conn,
        elem_ids=np.arange(1, m + 1, dtype=np.int32),
        E=np.full(m, E, dtype=np.float64), nu=np.full(m, nu, dtype=np.float64),
        form=np.full(m, form, dtype=np.int32),
        spc_nodes=clamp.astype(np.int32), spc_mask=np.full(clamp.shape[0], 0b111, np.int32),
        name=name, shape=(nx, ny, nz))


def tip_load(model: SolidModel, total: float = 1000.0, direction=(0.0, 0.0, -1.0)):
    """FORCE cards splitting `total` equally over the x=L face nodes."""
    nx, ny, nz = model.shape
    i = (model.node_ids - 1) // ((ny + 1) * (nz + 1))
    nodes = model.node_ids[i == nx].astype(np.int32)
    scale = np.full(nodes.shape[0], total / nodes.shape[0])
    dirs = np.tile(np.asarray(direction, dtype=np.float64), (nodes.shape[0], 1))
    return nodes, scale, dirs


def jitter_interior(model: SolidModel, edge: float, frac: float, rng: np.random.Generator):
    nx, ny, nz = model.shape
    ids0 = model.node_ids - 1
    k = ids0 % (nz + 1)
    j = (ids0 // (nz + 1)) % (ny + 1)
    i = ids0 // ((ny + 1) * (nz + 1))
    interior = (i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)
    d = rng.uniform(-frac * edge, frac * edge, size=(int(interior.sum()), 3))
    model.xyz[interior] += d


def log_uniform_E(model: SolidModel, lo: float, hi: float, rng: np.random.Generator):
    model.E = np.exp(rng.uniform(np.log(lo), np.log(hi), size=model.n_elem))


def cantilever_1500() -> SolidModel:
    m = block(20, 4, 4, 0.05, name="cantilever_1500")
    m.loads = [tip_load(m)]
    return m


def cantilever_84k() -> SolidModel:
    m = block(60, 40, 35, 0.01, name="cantilever_84k")
    m.loads = [tip_load(m)]
    return m


def cantilever_84k_jitter(seed: int = 20260301) -> SolidModel:
    rng = np.random.default_rng(seed)
    m = block(60, 40, 35, 0.01, name="cantilever_84k_jitter")
    jitter_interior(m, 0.01, 0.2, rng)
    log_uniform_E(m, 20e9, 400e9, rng)
    m.loads = [tip_load(m)]
    m.seed = seed
    return m


def face_random_loads(m: SolidModel, nrhs: int, rng: np.random.Generator,
                      sigma: float = 100.0) -> list:
    """nrhs load cases of i.i.d. N(0, sigma) x/y/z FORCEs on the free z-max
    face nodes (the clamped i = 0 column excluded)."""
    nx, ny, nz = m.shape
    ids0 = m.node_ids - 1
    k = ids0 % (nz + 1)
    i = ids0 // ((ny + 1) * (nz + 1))
    face = m.node_ids[(k == nz) & (i > 0)].astype(np.int32)
    loads = []
    for _ in range(nrhs):
        f = rng.normal(0.0, sigma, size=(face.shape[0], 3))
        loads.append((face, np.ones(face.shape[0]), f))
    return loads


def tip_mean_uz_functional(m: SolidModel, eq6: np.ndarray, n: int) -> np.ndarray:
    """dJ/du of J = mean of -u_z over the free x = L (i = nx) face nodes."""
    nx, ny, nz = m.shape
    i = (m.node_ids - 1) // ((ny + 1) * (nz + 1))
    eqz = np.asarray(eq6)[np.nonzero(i == nx)[0], 2]
    eqz = eqz[eqz >= 0]
    c = np.zeros(n)
    c[eqz] = -1.0 / eqz.shape[0]
    return c


def block_160k_16rhs(seed: int = 20260304, nrhs: int = 16) -> SolidModel:
    rng = np.random.default_rng(seed)
    m = block(100, 40, 40, 0.01, name="block_160k_16rhs")
    m.loads = face_random_loads(m, nrhs, rng)
    m.seed = seed
    return m


def block_250k_adjoint(seed: int = 20260305) -> SolidModel:
    rng = np.random.default_rng(seed)
    m = block(100, 50, 50, 0.01, name="block_250k_adjoint")
    log_uniform_E(m, 20e9, 400e9, rng)
    m.loads = [tip_load(m)]
    m.seed = seed
    return m


def small_block(nx=6, ny=3, nz=3, edge=0.1, seed=None, jitter=0.0, hetero=False,
                form=EAS) -> SolidModel:
    """Small test block (optionally jittered / heterogeneous) with a -z tip load."""
    m = block(nx, ny, nz, edge, form=form, name=f"block_{nx}x{ny}x{nz}")
    rng = np.random.default_rng(seed if seed is not None else 0)
    if jitter > 0:
        jitter_interior(m, edge, jitter, rng)
    if hetero:
        log_uniform_E(m, 20e9, 400e9, rng)
    m.loads = [tip_load(m)]
    return m


def write_bdf(model: SolidModel, path: str, load_index: int = 0) -> None:
    """Write the model as a free-field BDF with round-trip float formatting."""
    with open(path, "w") as out:
        out.write("SOL 101\nCEND\nSUBCASE 1\n  LOAD = 1\n  SPC = 1\n"
                  "  DISPLACEMENT = ALL\nBEGIN BULK\n")
        uniq = {}
        for e in range(model.n_elem):
            key = (float(model.E[e]), float(model.nu[e]), int(model.form[e]))
            uniq.setdefault(key, len(uniq) + 1)
        for (E, nu, form), pid in uniq.items():
            out.write(f"MAT1,{pid},{E:.17g},,{nu:.17g}\n")
            isop = "SRI" if form == SRI else ""
            out.write(f"PSOLID,{pid},{pid},,2,,{isop}\n" if isop else f"PSOLID,{pid},{pid},,2\n")
        for nid, (x, y, z) in zip(model.node_ids, model.xyz):
            out.write(f"GRID,{nid},,{x:.17g},{y:.17g},{z:.17g}\n")
        ids = model.conn_ids()
        for e in range(model.n_elem):
            pid = uniq[(float(model.E[e]), float(model.nu[e]), int(model.form[e]))]
            n = ids[e]
            out.write(f"CHEXA,{model.elem_ids[e]},{pid},{n[0]},{n[1]},{n[2]},{n[3]},{n[4]},{n[5]}\n")
            out.write(f"+,{n[6]},{n[7]}\n")
        for nid, mask in zip(model.spc_nodes, model.spc_mask):
            comps = "".join(str(d + 1) for d in range(6) if mask & (1 << d))
            out.write(f"SPC1,1,{comps},{nid}\n")
        nodes, scale, dirs = model.loads[load_index]
        for nid, s, d in zip(nodes, scale, dirs):
            out.write(f"FORCE,1,{nid},0,{s:.17g},{d[0]:.17g},{d[1]:.17g},{d[2]:.17g}\n")
        out.write("ENDDATA\n")


WORKLOADS = {
    "cantilever_1500": cantilever_1500,
    "cantilever_84k": cantilever_84k,
    "cantilever_84k_jitter": cantilever_84k_jitter,
    "block_160k_16rhs": block_160k_16rhs,
    "block_250k_adjoint": block_250k_adjoint,
}
