"""Generate tests/golden/cantilever_84k_direct.json (uniform mesh) or
cantilever_84k_jitter_direct.json (--model jitter: interior nodes jittered by
seeded U(+-0.2 h), per-element log-uniform E in [20, 400] GPa): a
fingerprint of the FP64 sparse DIRECT solution of the 84 000-element
cantilever (60x40x35 CHEXA8, n = 265 680), the stand-in for the reference's
--backend=cpu (CHOLMOD) solve.

The oracle assembles K (restated element stiffness + build_csr) and scipy's
SuperLU factors it (about 13 minutes on 8 cores).  Stored: ||u||_2, the
u_z of every loaded tip node (1 476 values) and u at a seeded sample of 4 096
equations — enough to measure the relative displacement error of a GPU
solution at full size without the 2 MB vector.

    python tests/golden/make_direct_84k.py [--model uniform|jitter] [--solution u.npy]

--solution reuses a direct solution computed earlier by this same procedure.
"""
import argparse
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vibestran_gb300 import cantilever as C  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--solution", default=None)
    ap.add_argument("--model", choices=("uniform", "jitter"), default="uniform")
    a = ap.parse_args()
    jitter = a.model == "jitter"
    m = C.cantilever_84k_jitter() if jitter else C.cantilever_84k()
    eq6, n = O.dof_map(m)
    F = O.apply_forces(m, eq6, n)
    if a.solution:
        u = np.load(a.solution)
    else:
        K = O.assemble_chexa8(m, eq6, n)
        u = O.sparse_direct_solve(K, F)
    assert u.shape == (n,)
    nodes = m.loads[0][0]
    tip_eq = eq6[nodes - 1, 2]
    rng = np.random.default_rng(84000)
    sample = np.sort(rng.choice(n, size=4096, replace=False))
    name = "cantilever_84k_jitter" if jitter else "cantilever_84k"
    out = {
        "_about": f"FP64 sparse direct (SuperLU) solution of {name}; see make_direct_84k.py",
        "seed": m.seed,
        "n": int(n),
        "u_norm": float(np.linalg.norm(u)),
        "F_dot_u": float(F @ u),
        "tip_eq": tip_eq.tolist(),
        "tip_uz": [float(v) for v in u[tip_eq]],
        "sample_eq": sample.tolist(),
        "sample_u": [float(v) for v in u[sample]],
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), f"{name}_direct.json")
    with open(path, "w") as fh:
        json.dump(out, fh)
    print("wrote", path, "||u|| =", out["u_norm"])


if __name__ == "__main__":
    main()
