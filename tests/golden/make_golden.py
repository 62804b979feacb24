"""Generate tests/golden/oracle_fixtures.json from the CPU oracle.

The fixture pins the oracle's element stiffness (unit cube EAS/SRI and a
seeded distorted hex) and its config-1 cantilever assembly + direct solve, so
that the x86 and Arm builds of the oracle, and later changes to it, are held
to the same numbers.  Run:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vibestran_gb300 import cantilever as C  # noqa: E402


def main():
    cube = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                     [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    rng = np.random.default_rng(1234)
    dist = cube * np.array([0.3, 0.2, 0.25]) + rng.uniform(-0.04, 0.04, size=(8, 3))
    elements = {}
    for name, xyz, E, nu, form in [("cube_eas", cube, 1e6, 0.3, 0), ("cube_sri", cube, 1e6, 0.3, 1),
                                   ("distorted_eas", dist, 2e11, 0.3, 0),
                                   ("distorted_sri", dist, 2e11, 0.3, 1),
                                   ("cube_eas_incompressible", cube, 1e6, 0.4999, 0)]:
        ke = O.chexa8_ke(xyz, E, nu, form)
        elements[name] = {"xyz": xyz.tolist(), "E": E, "nu": nu, "form": form,
                          "ke": [float(v) for v in ke.reshape(-1)]}
    m = C.cantilever_1500()
    eq6, n, K, F, u = O.solve_model(m)
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(K.row_ptr, np.int32).tobytes())
    h.update(np.ascontiguousarray(K.col_ind, np.int32).tobytes())
    out = {
        "_about": "oracle outputs; regenerate with tests/golden/make_golden.py",
        "elements": elements,
        "cantilever_1500": {"n": n, "nnz_lower": int(K.nnz), "pattern_sha256": h.hexdigest(),
                            "u_head": [float(v) for v in u[:32]],
                            "u_norm": float(np.linalg.norm(u))},
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_fixtures.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
