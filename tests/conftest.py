import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the built libvsgb.so")
    config.addinivalue_line("markers", "slow: full-size workloads (minutes)")


@pytest.fixture(scope="session")
def known():
    with open(os.path.join(GOLDEN, "reference_known_answers.json")) as fh:
        return json.load(fh)


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build()
    return O


@pytest.fixture(scope="session")
def vsgb():
    from vibestran_gb300 import backend as B
    from vibestran_gb300 import build as b
    b.build()
    B.load_library()
    return B


def model_from_spec(spec, isop=0):
    """SolidModel for the single-hex reference cases."""
    from vibestran_gb300 import cantilever as C
    nodes = spec.get("nodes") or [[1, 0, 0, 0], [2, 1, 0, 0], [3, 1, 1, 0], [4, 0, 1, 0],
                                  [5, 0, 0, 1], [6, 1, 0, 1], [7, 1, 1, 1], [8, 0, 1, 1]]
    ids = np.array([n[0] for n in nodes], np.int32)
    xyz = np.array([n[1:] for n in nodes], np.float64)
    spc_nodes, spc_mask = [], []
    for nid, comps in spec["spc1"]:
        m = 0
        for ch in comps:
            m |= 1 << (int(ch) - 1)
        spc_nodes.append(nid)
        spc_mask.append(m)
    f = spec["force"]
    loads = [(np.array([x[0] for x in f], np.int32), np.array([x[1] for x in f], np.float64),
              np.array([x[2] for x in f], np.float64))]
    return C.SolidModel(node_ids=ids, xyz=xyz, conn=np.arange(8, dtype=np.int32).reshape(1, 8),
                        elem_ids=np.array([1], np.int32), E=np.array([spec["E"]], np.float64),
                        nu=np.array([spec["nu"]], np.float64),
                        form=np.array([isop], np.int32),
                        spc_nodes=np.array(spc_nodes, np.int32),
                        spc_mask=np.array(spc_mask, np.int32), loads=loads, name="hex1",
                        shape=(1, 1, 1))


def tridiagonal(n, d, off, lower_only=False):
    from oracle import oracle as O
    rows, cols, vals = [], [], []
    for i in range(n):
        rows.append(i); cols.append(i); vals.append(d)
        if i > 0:
            rows.append(i); cols.append(i - 1); vals.append(off)
            if not lower_only:
                rows.append(i - 1); cols.append(i); vals.append(off)
    return O.build_from_triplets(n, rows, cols, vals)


def banded500():
    from oracle import oracle as O
    n = 500
    rows, cols, vals = [], [], []
    for i in range(n):
        rows.append(i); cols.append(i); vals.append(float(n + 1))
        if i > 0:
            rows += [i, i - 1]; cols += [i - 1, i]; vals += [-1.0, -1.0]
        if i > 1:
            rows += [i, i - 2]; cols += [i - 2, i]; vals += [-0.5, -0.5]
    K = O.build_from_triplets(n, rows, cols, vals)
    F = np.array([(i % 7) + 1 for i in range(n)], np.float64)
    return K, F
