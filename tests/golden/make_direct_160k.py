"""Generate tests/golden/block_160k_16rhs_ref.json: a fingerprint of converged
FP64 solutions of the 16 random face-load cases on the 100x40x40 CHEXA8 block
(160 000 elements, n = 504 300), the reference the batched GPU solves are
measured against.

A sparse direct factorisation of this system takes hours in scipy's SuperLU
here (it already needs ~13 minutes at n = 265 680), so each case is solved by
the oracle's FP64 Jacobi PCG (the cuda-pcg recurrence restated on the CPU) to
relative residual 1e-13; on this block the relative error of an iterate stays
within about 10x its relative residual, so the stored solutions are exact to
~1e-12 for the 5e-7 checks they serve.  Stored per case: ||u||_2, F.u and u at
a seeded sample of 2 048 equations.

    python tests/golden/make_direct_160k.py
"""
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vibestran_gb300 import cantilever as C  # noqa: E402


def main():
    m = C.block_160k_16rhs()
    eq6, n = O.dof_map(m)
    K = O.assemble_chexa8(m, eq6, n)
    rng = np.random.default_rng(160000)
    sample = np.sort(rng.choice(n, size=2048, replace=False))
    cases = []
    for k in range(len(m.loads)):
        F = O.apply_forces(m, eq6, n, k)
        t0 = time.time()
        u, it, rel = O.pcg_jacobi(K, F, 1e-13, 100000)
        print(f"case {k}: {it} iterations, residual {rel:.2e}, {time.time() - t0:.1f} s",
              flush=True)
        cases.append({"u_norm": float(np.linalg.norm(u)), "F_dot_u": float(F @ u),
                      "sample_u": [float(v) for v in u[sample]], "iterations": int(it),
                      "rel_residual": float(rel)})
    out = {"_about": "converged FP64 PCG (oracle, residual 1e-13) solutions of "
                     "block_160k_16rhs; see make_direct_160k.py",
           "seed": m.seed, "n": int(n), "sample_eq": sample.tolist(), "cases": cases}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "block_160k_16rhs_ref.json")
    with open(path, "w") as fh:
        json.dump(out, fh)
    print("wrote", path)


if __name__ == "__main__":
    main()
