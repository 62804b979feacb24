"""Element stiffness of distorted CHEXA8 EAS hexes by an independent numpy
restatement of CHexa8Eas::stiffness_matrix (vibestran
src/elements/solid_elements.cpp:1054-1206), written to
tests/golden/eas_distorted_hex.json.

The restatement works with whole matrices (numpy inverse, determinant and a
Cholesky solve) where the oracle works entry by entry, so the two agree only
through the mathematics.  It keeps the reference's enhancement gradient: the
ROW k of J0^-1 scaled by the parametric coordinate k and by detJ0/detJ
(solid_elements.cpp:1132-1134), which differs from the textbook column of
J0^-T only when J0 is not symmetric, i.e. on a distorted element.  The
fixture therefore also records the textbook variant, so a test can check that
the elements chosen really tell the two apart.

    python tests/golden/make_eas_distorted.py
"""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "eas_distorted_hex.json")

# parametric node coordinates, solid_elements.cpp:76-93
XI = np.array([-1, 1, 1, -1, -1, 1, 1, -1], float)
ETA = np.array([-1, -1, 1, 1, -1, -1, 1, 1], float)
ZETA = np.array([-1, -1, -1, -1, 1, 1, 1, 1], float)


def dshape(xi, eta, zeta):
    """3 x 8: rows d/dxi, d/deta, d/dzeta of the trilinear shape functions."""
    return 0.125 * np.stack([XI * (1 + ETA * eta) * (1 + ZETA * zeta),
                             ETA * (1 + XI * xi) * (1 + ZETA * zeta),
                             ZETA * (1 + XI * xi) * (1 + ETA * eta)])


def isotropic_d(E, nu):
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = lam
    D[np.arange(3), np.arange(3)] = lam + 2 * mu
    D[np.arange(3, 6), np.arange(3, 6)] = mu
    return D


def sym_grad(g, alpha):
    """Voigt (xx, yy, zz, xy, yz, zx) strain of the field g-gradient times e_alpha."""
    col = np.zeros(6)
    gx, gy, gz = g
    if alpha == 0:
        col[[0, 3, 5]] = gx, gy, gz
    elif alpha == 1:
        col[[3, 1, 4]] = gx, gy, gz
    else:
        col[[5, 4, 2]] = gx, gy, gz
    return col


def eas_ke(xyz, E, nu, textbook=False):
    """24 x 24 condensed EAS stiffness; textbook=True maps the modes with the
    columns of J0^-1 (rows of J0^-T) instead of the reference's rows."""
    D = isotropic_d(E, nu)
    J0 = dshape(0.0, 0.0, 0.0) @ xyz
    det0 = np.linalg.det(J0)
    J0i = np.linalg.inv(J0)
    g0 = J0i.T if textbook else J0i
    Kuu = np.zeros((24, 24))
    Kua = np.zeros((24, 9))
    Kaa = np.zeros((9, 9))
    gp = 1.0 / np.sqrt(3.0)
    for xi in (-gp, gp):
        for eta in (-gp, gp):
            for zeta in (-gp, gp):
                dN = dshape(xi, eta, zeta)
                J = dN @ xyz
                det = np.linalg.det(J)
                dX = np.linalg.inv(J) @ dN  # 3 x 8 physical derivatives
                B = np.zeros((6, 24))
                for a in range(3):
                    B[:, a::3] = np.array([sym_grad(dX[:, n], a) for n in range(8)]).T
                par = (xi, eta, zeta)
                G = np.zeros((6, 9))
                for k in range(3):
                    for a in range(3):
                        G[:, 3 * k + a] = sym_grad(g0[k] * par[k], a)
                G *= det0 / det
                Kuu += B.T @ D @ B * det
                Kua += B.T @ D @ G * det
                Kaa += G.T @ D @ G * det
    L = np.linalg.cholesky(Kaa)
    Y = np.linalg.solve(L, Kua.T)
    return Kuu - Y.T @ Y


def cases():
    rng = np.random.default_rng(20261204)
    cube = np.stack([(XI + 1) / 2, (ETA + 1) / 2, (ZETA + 1) / 2], axis=1) * 0.01
    out = []
    # 1: every node jittered by U(+-0.2 edge)
    out.append(("jittered", cube + rng.uniform(-0.2, 0.2, (8, 3)) * 0.01, 200e9, 0.3))
    # 2: a sheared and tapered brick (J0 far from symmetric), nearly incompressible
    x = cube.copy()
    x[:, 0] += 0.4 * x[:, 1] + 0.2 * x[:, 2]
    x[4:, :2] *= 0.8
    out.append(("sheared_tapered", x, 70e9, 0.45))
    return out


def main():
    res = []
    for name, xyz, E, nu in cases():
        K = eas_ke(xyz, E, nu)
        Kt = eas_ke(xyz, E, nu, textbook=True)
        res.append({"name": name, "xyz": xyz.tolist(), "E": E, "nu": nu, "ke": K.tolist(),
                    "textbook_rel_diff": float(np.abs(K - Kt).max() / np.abs(K).max())})
    with open(OUT, "w") as fh:
        json.dump({"source": "tests/golden/make_eas_distorted.py", "cases": res}, fh)
    for r in res:
        print(r["name"], "textbook form differs by", r["textbook_rel_diff"])


if __name__ == "__main__":
    main()
