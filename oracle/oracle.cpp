// oracle/oracle.cpp
//
// TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
// CPU restatement of the vibestran SOL 101 CHEXA8 path (element stiffness ->
// DOF map -> lower-triangle CSR assembly -> Jacobi PCG).  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may load
// this library, and only as the checker or as the timed CPU reference.  The
// product library (vibestran_gb300/csrc) never calls it.
//
// Every function cites the reference file:line it restates.  The reference
// itself cannot be built here (Eigen 3.4, spdlog, gtest, meson, CHOLMOD and
// cuDSS are absent), so the dense 3x3 / 6x6 / 9x9 algebra Eigen performs is
// restated with plain loops.  Parity of this restatement is pinned against the
// known answers the reference's own tests hold (tests/golden/).
//
// Build: g++ -std=c++20 -O2 -fopenmp -shared -fPIC oracle.cpp -o _build/liboracle.so

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

constexpr int kConstrained = -1;  // include/core/dof_map.hpp:20 CONSTRAINED_DOF

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

static void set_err(char* buf, int len, const char* msg) {
  if (buf && len > 0) {
    std::snprintf(buf, static_cast<size_t>(len), "%s", msg);
  }
}

// ── Element algebra ────────────────────────────────────────────────────────

// src/elements/solid_elements.cpp:17-27 (isotropic_D)
static void isotropic_D(double E, double nu, double D[6][6]) {
  const double lam = E * nu / ((1 + nu) * (1 - 2 * nu));
  const double mu = E / (2 * (1 + nu));
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) D[i][j] = 0.0;
  D[0][0] = lam + 2 * mu; D[0][1] = lam;          D[0][2] = lam;
  D[1][0] = lam;          D[1][1] = lam + 2 * mu; D[1][2] = lam;
  D[2][0] = lam;          D[2][1] = lam;          D[2][2] = lam + 2 * mu;
  D[3][3] = mu; D[4][4] = mu; D[5][5] = mu;
}

struct Shape {
  double N[8], dxi[8], deta[8], dzeta[8];
};

// src/elements/solid_elements.cpp:76-93 (CHexa8::shape_functions)
static Shape shape_functions(double xi, double eta, double zeta) {
  static const double xn[8] = {-1, +1, +1, -1, -1, +1, +1, -1};
  static const double en[8] = {-1, -1, +1, +1, -1, -1, +1, +1};
  static const double zn[8] = {-1, -1, -1, -1, +1, +1, +1, +1};
  Shape s;
  for (int i = 0; i < 8; ++i) {
    s.N[i] = 0.125 * (1 + xn[i] * xi) * (1 + en[i] * eta) * (1 + zn[i] * zeta);
    s.dxi[i] = 0.125 * xn[i] * (1 + en[i] * eta) * (1 + zn[i] * zeta);
    s.deta[i] = 0.125 * en[i] * (1 + xn[i] * xi) * (1 + zn[i] * zeta);
    s.dzeta[i] = 0.125 * zn[i] * (1 + xn[i] * xi) * (1 + en[i] * eta);
  }
  return s;
}

// J(r, c) = d x_c / d xi_r  (solid_elements.cpp:1177-1182: rows are the
// parametric derivatives, columns are x, y, z).
static void jacobian(const double X[8][3], const Shape& s, double J[3][3]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) J[r][c] = 0.0;
  for (int n = 0; n < 8; ++n) {
    for (int c = 0; c < 3; ++c) {
      J[0][c] += s.dxi[n] * X[n][c];
      J[1][c] += s.deta[n] * X[n][c];
      J[2][c] += s.dzeta[n] * X[n][c];
    }
  }
}

static double det3(const double m[3][3]) {
  return m[0][0] * (m[1][1] * m[2][2] - m[2][1] * m[1][2]) -
         m[1][0] * (m[0][1] * m[2][2] - m[2][1] * m[0][2]) +
         m[2][0] * (m[0][1] * m[1][2] - m[1][1] * m[0][2]);
}

// Cofactor inverse (what Eigen::Matrix3d::inverse computes).
static void inv3(const double m[3][3], double o[3][3]) {
  const double d = det3(m);
  o[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / d;
  o[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / d;
  o[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / d;
  o[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / d;
  o[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / d;
  o[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / d;
  o[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / d;
  o[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / d;
  o[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / d;
}

// src/elements/solid_elements.cpp:1080-1093 (build_B; same as :121-135)
static void build_B(const Shape& s, const double Ji[3][3], double B[6][24]) {
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 24; ++j) B[i][j] = 0.0;
  for (int n = 0; n < 8; ++n) {
    const double dnx = Ji[0][0] * s.dxi[n] + Ji[0][1] * s.deta[n] + Ji[0][2] * s.dzeta[n];
    const double dny = Ji[1][0] * s.dxi[n] + Ji[1][1] * s.deta[n] + Ji[1][2] * s.dzeta[n];
    const double dnz = Ji[2][0] * s.dxi[n] + Ji[2][1] * s.deta[n] + Ji[2][2] * s.dzeta[n];
    const int c0 = 3 * n;
    B[0][c0 + 0] = dnx;
    B[1][c0 + 1] = dny;
    B[2][c0 + 2] = dnz;
    B[3][c0 + 0] = dny; B[3][c0 + 1] = dnx;
    B[4][c0 + 1] = dnz; B[4][c0 + 2] = dny;
    B[5][c0 + 0] = dnz; B[5][c0 + 2] = dnx;
  }
}

// out(a x b) += scale * L^T * D * R, with L: 6 x a, R: 6 x b (row-major).
template <int A, int Bc>
static void add_ltdr(const double (&L)[6][A], const double D[6][6],
                     const double (&R)[6][Bc], double scale, double (&out)[A][Bc]) {
  double DR[6][Bc];
  for (int k = 0; k < 6; ++k)
    for (int j = 0; j < Bc; ++j) {
      double acc = 0.0;
      for (int m = 0; m < 6; ++m) acc += D[k][m] * R[m][j];
      DR[k][j] = acc;
    }
  for (int i = 0; i < A; ++i)
    for (int j = 0; j < Bc; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) acc += L[k][i] * DR[k][j];
      out[i][j] += acc * scale;
    }
}

static void read_coords(const double* xyz24, double X[8][3]) {
  for (int n = 0; n < 8; ++n)
    for (int c = 0; c < 3; ++c) X[n][c] = xyz24[3 * n + c];
}

// src/elements/solid_elements.cpp:95-180 (CHexa8::stiffness_matrix, SRI).
static void chexa8_sri_ke(const double* xyz24, double E, double nu, double* ke) {
  double X[8][3];
  read_coords(xyz24, X);
  double D[6][6];
  isotropic_D(E, nu, D);
  const double lam = D[0][1];
  double Dvol[6][6] = {};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Dvol[i][j] = lam;
  double Ddev[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) Ddev[i][j] = D[i][j] - Dvol[i][j];

  double K[24][24] = {};
  const double gp = 1.0 / std::sqrt(3.0);
  const double g[2] = {-gp, gp};
  for (int gi = 0; gi < 2; ++gi)
    for (int gj = 0; gj < 2; ++gj)
      for (int gk = 0; gk < 2; ++gk) {
        const Shape s = shape_functions(g[gi], g[gj], g[gk]);
        double J[3][3], Ji[3][3];
        jacobian(X, s, J);
        const double detJ = det3(J);
        if (detJ <= 0) throw Error("CHEXA8: non-positive Jacobian");
        inv3(J, Ji);
        double B[6][24];
        build_B(s, Ji, B);
        add_ltdr<24, 24>(B, Ddev, B, detJ, K);
      }
  {
    const Shape s0 = shape_functions(0.0, 0.0, 0.0);
    double J0[3][3], J0i[3][3];
    jacobian(X, s0, J0);
    const double detJ0 = det3(J0);
    if (detJ0 <= 0) throw Error("CHEXA8: non-positive centroidal Jacobian");
    inv3(J0, J0i);
    double B0[6][24];
    build_B(s0, J0i, B0);
    add_ltdr<24, 24>(B0, Dvol, B0, detJ0 * 8.0, K);
  }
  for (int i = 0; i < 24; ++i)
    for (int j = 0; j < 24; ++j) ke[i * 24 + j] = K[i][j];
}

// src/elements/solid_elements.cpp:1054-1206 (CHexa8Eas::stiffness_matrix).
// The enhancement gradients use ROWS of the centroidal inverse Jacobian,
// J0^{-1}.row(k) * xi_k, scaled by detJ0/detJ (:1109, :1131-1133, :1163).
static void chexa8_eas_ke(const double* xyz24, double E, double nu, double* ke) {
  double X[8][3];
  read_coords(xyz24, X);
  double D[6][6];
  isotropic_D(E, nu, D);

  const Shape s0 = shape_functions(0.0, 0.0, 0.0);
  double J0[3][3], J0i[3][3];
  jacobian(X, s0, J0);
  const double detJ0 = det3(J0);
  if (detJ0 <= 0) throw Error("CHEXA8EAS: non-positive centroidal Jacobian");
  inv3(J0, J0i);

  double Kuu[24][24] = {};
  double Kua[24][9] = {};
  double Kaa[9][9] = {};

  const double gp = 1.0 / std::sqrt(3.0);
  const double g[2] = {-gp, gp};
  for (int gi = 0; gi < 2; ++gi)
    for (int gj = 0; gj < 2; ++gj)
      for (int gk = 0; gk < 2; ++gk) {
        const double xi = g[gi], eta = g[gj], zeta = g[gk];
        const Shape s = shape_functions(xi, eta, zeta);
        double J[3][3], Ji[3][3];
        jacobian(X, s, J);
        const double detJ = det3(J);
        if (detJ <= 0) throw Error("CHEXA8EAS: non-positive Jacobian");
        inv3(J, Ji);
        double B[6][24];
        build_B(s, Ji, B);

        // G (6 x 9): columns (xi, eta, zeta) x (x, y, z) modes.
        double G[6][9] = {};
        const double par[3] = {xi, eta, zeta};
        const double scale = detJ0 / detJ;
        for (int p = 0; p < 3; ++p) {
          const double gx = J0i[p][0] * par[p];
          const double gy = J0i[p][1] * par[p];
          const double gz = J0i[p][2] * par[p];
          const int c = 3 * p;
          G[0][c + 0] = gx; G[3][c + 0] = gy; G[5][c + 0] = gz;  // alpha = x
          G[3][c + 1] = gx; G[1][c + 1] = gy; G[4][c + 1] = gz;  // alpha = y
          G[5][c + 2] = gx; G[4][c + 2] = gy; G[2][c + 2] = gz;  // alpha = z
        }
        for (int r = 0; r < 6; ++r)
          for (int c = 0; c < 9; ++c) G[r][c] *= scale;

        const double w = detJ;
        add_ltdr<24, 24>(B, D, B, w, Kuu);
        add_ltdr<24, 9>(B, D, G, w, Kua);
        add_ltdr<9, 9>(G, D, G, w, Kaa);
      }

  // Eigen::LLT of Kaa (:1201-1203): Cholesky, fails on a non-positive pivot.
  double L[9][9] = {};
  for (int j = 0; j < 9; ++j) {
    double d = Kaa[j][j];
    for (int k = 0; k < j; ++k) d -= L[j][k] * L[j][k];
    if (!(d > 0.0)) throw Error("CHEXA8EAS: Kaa factorization failed");
    L[j][j] = std::sqrt(d);
    for (int i = j + 1; i < 9; ++i) {
      double v = Kaa[i][j];
      for (int k = 0; k < j; ++k) v -= L[i][k] * L[j][k];
      L[i][j] = v / L[j][j];
    }
  }
  // Xs = Kaa^{-1} Kua^T  (9 x 24)
  double Xs[9][24];
  for (int c = 0; c < 24; ++c) {
    double y[9];
    for (int i = 0; i < 9; ++i) {
      double v = Kua[c][i];
      for (int k = 0; k < i; ++k) v -= L[i][k] * y[k];
      y[i] = v / L[i][i];
    }
    for (int i = 8; i >= 0; --i) {
      double v = y[i];
      for (int k = i + 1; k < 9; ++k) v -= L[k][i] * Xs[k][c];
      Xs[i][c] = v / L[i][i];
    }
  }
  for (int i = 0; i < 24; ++i)
    for (int j = 0; j < 24; ++j) {
      double acc = 0.0;
      for (int k = 0; k < 9; ++k) acc += Kua[i][k] * Xs[k][j];
      ke[i * 24 + j] = Kuu[i][j] - acc;
    }
}

// src/elements/element_factory.cpp:31-43: EAS unless PSOLID ISOP = SRI.
enum Formulation { kEAS = 0, kSRI = 1 };

static void chexa8_ke(const double* xyz24, double E, double nu, int form, double* ke) {
  if (form == kSRI)
    chexa8_sri_ke(xyz24, E, nu, ke);
  else
    chexa8_eas_ke(xyz24, E, nu, ke);
}

// ── DOF map ────────────────────────────────────────────────────────────────

struct DofMap {
  // node id -> 6 equation indices
  std::unordered_map<int, std::array<int, 6>> blocks;
  int num_free = 0;

  // src/core/dof_map.cpp:10-33 (DofMap::build): sorted node ids, 6 slots.
  void build(const std::vector<int>& node_ids) {
    std::vector<int> ids(node_ids);
    std::sort(ids.begin(), ids.end());
    blocks.clear();
    num_free = 0;
    for (int id : ids) {
      auto& b = blocks[id];
      for (int d = 0; d < 6; ++d) b[d] = num_free++;
    }
  }

  // src/core/dof_map.cpp:55-97 (DofMap::constrain_batch)
  void constrain_batch(const std::vector<std::pair<int, int>>& dofs) {
    std::vector<int> removed;
    removed.reserve(dofs.size());
    for (const auto& [nid, d] : dofs) {
      auto it = blocks.find(nid);
      if (it == blocks.end())
        throw Error("constrain_batch: node " + std::to_string(nid) + " not in DofMap");
      if (it->second[d] != kConstrained) removed.push_back(it->second[d]);
    }
    if (removed.empty()) return;
    std::sort(removed.begin(), removed.end());
    removed.erase(std::unique(removed.begin(), removed.end()), removed.end());
    for (auto& [_, b] : blocks)
      for (auto& e : b) {
        if (e == kConstrained) continue;
        e -= static_cast<int>(std::lower_bound(removed.begin(), removed.end(), e) -
                              removed.begin());
      }
    for (const auto& [nid, d] : dofs) blocks.at(nid)[d] = kConstrained;
    num_free -= static_cast<int>(removed.size());
  }

  // src/core/dof_map.cpp:55-76 (DofMap::constrain): serial form used by the
  // reference's batch-equals-serial test (tests/unit/test_dof_map.cpp:160-191).
  void constrain(int nid, int d) {
    auto it = blocks.find(nid);
    if (it == blocks.end())
      throw Error("constrain: node " + std::to_string(nid) + " not in DofMap");
    int& eq = it->second[d];
    if (eq == kConstrained) return;
    const int removed = eq;
    eq = kConstrained;
    for (auto& [_, b] : blocks)
      for (auto& e : b)
        if (e > removed) --e;
    --num_free;
  }
};

// ── Sparse builder ─────────────────────────────────────────────────────────

struct Triplet {
  int32_t row, col;
  double value;
};

struct Csr {
  std::vector<int> row_ptr, col_ind;
  std::vector<double> values;
  int n = 0;
  int nnz = 0;
  bool lower = false;
};

// src/core/sparse_matrix.cpp:16-35 (add_element_stiffness): keep gi >= gj,
// both free, value exactly != 0.0.
static void add_element_stiffness(const int* gdofs, int ndof, const double* ke,
                                  std::vector<Triplet>& out) {
  for (int i = 0; i < ndof; ++i) {
    if (gdofs[i] == kConstrained) continue;
    for (int j = 0; j < ndof; ++j) {
      if (gdofs[j] == kConstrained) continue;
      if (gdofs[i] < gdofs[j]) continue;
      const double v = ke[i * ndof + j];
      if (v != 0.0) out.push_back({gdofs[i], gdofs[j], v});
    }
  }
}

// src/core/sparse_matrix.cpp:62-150 (build_csr): histogram, scatter, per-row
// sort by column, duplicate sum.  stable_sort keeps the (arbitrary) triplet
// order fixed; the reference's std::sort only changes the order duplicates
// are summed in.
static Csr build_csr(std::vector<Triplet>& trips, int n) {
  bool lower_only = true;
  for (const auto& t : trips)
    if (t.row < t.col) {
      lower_only = false;
      break;
    }
  std::vector<int> bucket(static_cast<size_t>(n) + 1, 0);
  for (const auto& t : trips) ++bucket[static_cast<size_t>(t.row) + 1];
  std::partial_sum(bucket.begin(), bucket.end(), bucket.begin());
  std::vector<int> cursor(bucket.begin(), bucket.begin() + n);
  std::vector<Triplet> staged(trips.size());
  for (const auto& t : trips) staged[static_cast<size_t>(cursor[t.row]++)] = t;
  trips.clear();
  trips.shrink_to_fit();
#pragma omp parallel for schedule(dynamic, 256)
  for (int row = 0; row < n; ++row)
    std::stable_sort(staged.begin() + bucket[row], staged.begin() + bucket[row + 1],
                     [](const Triplet& a, const Triplet& b) { return a.col < b.col; });
  Csr c;
  c.n = n;
  c.row_ptr.assign(static_cast<size_t>(n) + 1, 0);
  c.col_ind.resize(staged.size());
  c.values.resize(staged.size());
  int out = 0;
  for (int row = 0; row < n; ++row) {
    const int b = bucket[row], e = bucket[row + 1];
    for (int i = b; i < e; ++i) {
      if (i > b && staged[i].col == staged[i - 1].col) {
        c.values[out - 1] += staged[i].value;
      } else {
        c.col_ind[out] = staged[i].col;
        c.values[out] = staged[i].value;
        ++out;
      }
    }
    c.row_ptr[row + 1] = out;
  }
  c.nnz = out;
  c.col_ind.resize(out);
  c.values.resize(out);
  c.lower = lower_only;
  return c;
}

// src/core/sparse_matrix.cpp:153-181 (CsrData::multiply)
static void csr_multiply(int n, const int* rp, const int* ci, const double* v, bool lower,
                         const double* x, double* y) {
  for (int i = 0; i < n; ++i) y[i] = 0.0;
  if (lower) {
    for (int row = 0; row < n; ++row)
      for (int k = rp[row]; k < rp[row + 1]; ++k) {
        const int col = ci[k];
        y[row] += v[k] * x[col];
        if (col != row) y[col] += v[k] * x[row];
      }
    return;
  }
#pragma omp parallel for schedule(static)
  for (int row = 0; row < n; ++row) {
    double acc = 0.0;
    for (int k = rp[row]; k < rp[row + 1]; ++k) acc += v[k] * x[ci[k]];
    y[row] = acc;
  }
}

// src/core/sparse_matrix.cpp:183-235 (CsrData::expanded_symmetric)
static Csr expanded_symmetric(const Csr& L) {
  if (!L.lower) return L;
  Csr f;
  f.n = L.n;
  f.lower = false;
  f.row_ptr.assign(static_cast<size_t>(L.n) + 1, 0);
  for (int row = 0; row < L.n; ++row)
    for (int k = L.row_ptr[row]; k < L.row_ptr[row + 1]; ++k) {
      const int col = L.col_ind[k];
      ++f.row_ptr[row + 1];
      if (col != row) ++f.row_ptr[col + 1];
    }
  std::partial_sum(f.row_ptr.begin(), f.row_ptr.end(), f.row_ptr.begin());
  f.nnz = f.row_ptr[L.n];
  f.col_ind.resize(f.nnz);
  f.values.resize(f.nnz);
  std::vector<int> cur(f.row_ptr.begin(), f.row_ptr.begin() + L.n);
  for (int row = 0; row < L.n; ++row)
    for (int k = L.row_ptr[row]; k < L.row_ptr[row + 1]; ++k) {
      const int col = L.col_ind[k];
      int o = cur[row]++;
      f.col_ind[o] = col;
      f.values[o] = L.values[k];
      if (col != row) {
        o = cur[col]++;
        f.col_ind[o] = row;
        f.values[o] = L.values[k];
      }
    }
  return f;
}

// src/core/sparse_matrix.cpp:237-279 (CsrData::lower_triangle)
static Csr lower_triangle(const Csr& F) {
  if (F.lower) return F;
  Csr l;
  l.n = F.n;
  l.lower = true;
  l.row_ptr.assign(static_cast<size_t>(F.n) + 1, 0);
  for (int row = 0; row < F.n; ++row) {
    for (int k = F.row_ptr[row]; k < F.row_ptr[row + 1]; ++k)
      if (F.col_ind[k] <= row) {
        l.col_ind.push_back(F.col_ind[k]);
        l.values.push_back(F.values[k]);
      }
    l.row_ptr[row + 1] = static_cast<int>(l.col_ind.size());
  }
  l.nnz = static_cast<int>(l.col_ind.size());
  return l;
}

// ── PCG ────────────────────────────────────────────────────────────────────

// src/solver/cuda_pcg_backend_impl.hpp:2076-2101 (build_jacobi_diagonal)
static std::vector<double> jacobi_diagonal(const Csr& K) {
  std::vector<double> d(static_cast<size_t>(K.n), 0.0);
  for (int i = 0; i < K.n; ++i) {
    bool found = false;
    for (int k = K.row_ptr[i]; k < K.row_ptr[i + 1]; ++k)
      if (K.col_ind[k] == i) {
        if (K.values[k] == 0.0)
          throw Error("zero diagonal at row " + std::to_string(i) +
                      " -- matrix is singular. Check boundary conditions.");
        d[i] = K.values[k];
        found = true;
        break;
      }
    if (!found)
      throw Error("missing diagonal at row " + std::to_string(i) +
                  " -- matrix is singular. Check boundary conditions.");
  }
  return d;
}

// src/solver/cuda_pcg_backend_impl.hpp:2103-2114 (validate_pcg_inputs)
static void validate(const Csr& K, size_t f_size) {
  if (K.n == 0) throw Error("stiffness matrix is empty -- no free DOFs");
  if (static_cast<int>(f_size) != K.n)
    throw Error("force vector size " + std::to_string(f_size) + " != matrix size " +
                std::to_string(K.n));
}

template <typename T>
static double dot(const std::vector<T>& a, const std::vector<T>& b) {
  double s = 0.0;
  const long n = static_cast<long>(a.size());
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (long i = 0; i < n; ++i) s += static_cast<double>(a[i]) * static_cast<double>(b[i]);
  return s;
}

// Full-storage matvec used inside the PCG loop (the lower-storage operator
// L + L^T - diag of cuda_pcg_backend_impl.hpp:1741-1768 applied through its
// expanded form).
template <typename T>
static void spmv_full(const Csr& F, const std::vector<T>& vals, const std::vector<T>& x,
                      std::vector<T>& y) {
#pragma omp parallel for schedule(static)
  for (int row = 0; row < F.n; ++row) {
    T acc = 0;
    for (int k = F.row_ptr[row]; k < F.row_ptr[row + 1]; ++k) acc += vals[k] * x[F.col_ind[k]];
    y[row] = acc;
  }
}

struct PcgResult {
  int iters = 0;
  double rel = 0.0;
};

// src/solver/cuda_pcg_backend_impl.hpp:1688-1999 (run_pcg_prepared) with the
// Jacobi preconditioner (:629-639).  Convergence is the UNPRECONDITIONED
// relative residual sqrt(r.r)/||b|| < tol (:723-729); zero RHS returns zeros
// with 0 iterations (:1820-1830); rz0 <= 0 throws (:1859-1862); pAp <= 0 is a
// breakdown that ends in the non-convergence error (:1934-1943, :1964-1970).
template <typename T>
static PcgResult pcg_jacobi(const Csr& full, const std::vector<T>& vals,
                            const std::vector<T>& diag, const std::vector<T>& b, double tol,
                            int max_iters, std::vector<T>& u) {
  const int n = full.n;
  u.assign(static_cast<size_t>(n), T(0));
  std::vector<T> r(b), z(n), p(n), Ap(n);
  PcgResult res;
  const double norm_b = std::sqrt(std::abs(dot(r, r)));
  if (norm_b < 1e-300) {
    res.iters = 0;
    res.rel = 0.0;
    return res;
  }
  for (int i = 0; i < n; ++i) z[i] = r[i] / diag[i];
  p = z;
  double rz = dot(r, z);
  if (rz <= 0.0)
    throw Error("non-positive initial r*z -- preconditioner is not SPD or matrix is singular");
  int iter = 0;
  double rel = 1.0;
  bool converged = false;
  for (; iter < max_iters; ++iter) {
    spmv_full(full, vals, p, Ap);
    const double pAp = dot(p, Ap);
    if (!(pAp > 0.0)) {
      iter = max_iters;
      break;
    }
    const T alpha = static_cast<T>(rz / pAp);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      u[i] += alpha * p[i];
      r[i] -= alpha * Ap[i];
      z[i] = r[i] / diag[i];
    }
    const double rz_new = dot(r, z);
    const double rr = dot(r, r);
    rel = std::sqrt(std::abs(rr)) / norm_b;
    if (rel < tol) {
      ++iter;
      converged = true;
      break;
    }
    const T beta = static_cast<T>(rz_new / rz);
    rz = rz_new;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
  }
  res.iters = iter;
  res.rel = rel;
  if (!converged)
    throw Error("did not converge after " + std::to_string(max_iters) +
                " iterations (relative residual " + std::to_string(rel) + " > tolerance " +
                std::to_string(tol) + ")");
  return res;
}

}  // namespace orc

// ═══════════════════════════════════════════════════════════════════════════
// C ABI for ctypes (tests / bench CPU arm only)
// ═══════════════════════════════════════════════════════════════════════════

using namespace orc;

extern "C" {

int orc_num_threads(int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
  return omp_get_max_threads();
#else
  (void)threads;
  return 1;
#endif
}

// One element stiffness (24x24 row-major).  Returns 0 or -1 (message in err).
int orc_chexa8_ke(const double* xyz24, double E, double nu, int formulation, double* ke576,
                  char* err, int errlen) {
  try {
    chexa8_ke(xyz24, E, nu, formulation, ke576);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// Batched element stiffness over a node-indexed mesh.
int orc_chexa8_ke_batch(int n_elem, const double* node_xyz, const int* conn, const double* E,
                        const double* nu, const int* form, double* ke_out, char* err,
                        int errlen) {
  int bad = -1;
  std::string msg;
#pragma omp parallel for schedule(dynamic, 64)
  for (int e = 0; e < n_elem; ++e) {
    double xyz[24];
    for (int a = 0; a < 8; ++a)
      for (int c = 0; c < 3; ++c) xyz[3 * a + c] = node_xyz[3 * conn[8 * e + a] + c];
    try {
      chexa8_ke(xyz, E[e], nu[e], form ? form[e] : kEAS, ke_out + static_cast<size_t>(e) * 576);
    } catch (const std::exception& ex) {
#pragma omp critical
      {
        if (bad < 0 || e < bad) {
          bad = e;
          msg = ex.what();
        }
      }
    }
  }
  if (bad >= 0) {
    set_err(err, errlen, (msg + " (element index " + std::to_string(bad) + ")").c_str());
    return -1;
  }
  return 0;
}

// Analysis DOF map for a CHEXA8-only model:
// src/solver/analysis_support.cpp:176-214 (build_analysis_dof_map) with the
// solid active mask (:39-57): T1-T3 of element nodes active, everything else
// constrained; then SPC components (bit d set = DOF d+1 constrained).
// eq_out is n_nodes*6 in the caller's node order.
int orc_dof_map(int n_nodes, const int* node_ids, int n_elem, const int* conn_ids, int n_spc,
                const int* spc_node_ids, const int* spc_masks, int* eq_out, int* n_free,
                char* err, int errlen) {
  try {
    DofMap dm;
    std::vector<int> ids(node_ids, node_ids + n_nodes);
    dm.build(ids);
    std::unordered_map<int, std::array<bool, 6>> mask;
    for (int i = 0; i < n_nodes; ++i) mask[node_ids[i]] = {false, false, false, false, false, false};
    for (int e = 0; e < n_elem; ++e)
      for (int a = 0; a < 8; ++a) {
        auto& m = mask[conn_ids[8 * e + a]];
        m[0] = m[1] = m[2] = true;
      }
    std::vector<std::pair<int, int>> inactive;
    for (const auto& [nid, m] : mask)
      for (int d = 0; d < 6; ++d)
        if (!m[d]) inactive.emplace_back(nid, d);
    dm.constrain_batch(inactive);
    std::vector<std::pair<int, int>> spc;
    for (int s = 0; s < n_spc; ++s)
      for (int d = 0; d < 6; ++d)
        if (spc_masks[s] & (1 << d)) spc.emplace_back(spc_node_ids[s], d);
    dm.constrain_batch(spc);
    for (int i = 0; i < n_nodes; ++i) {
      const auto& b = dm.blocks.at(node_ids[i]);
      for (int d = 0; d < 6; ++d) eq_out[6 * i + d] = b[d];
    }
    *n_free = dm.num_free;
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// Serial-vs-batch DOF constraint (tests/unit/test_dof_map.cpp:160-208).
// mode 0: build + constrain() each entry; mode 1: build + constrain_batch().
int orc_dof_constrain(int n_nodes, const int* node_ids, int n_c, const int* c_nodes,
                      const int* c_dofs, int mode, int* eq_out, int* n_free, char* err,
                      int errlen) {
  try {
    DofMap dm;
    dm.build(std::vector<int>(node_ids, node_ids + n_nodes));
    if (mode == 0) {
      for (int i = 0; i < n_c; ++i) dm.constrain(c_nodes[i], c_dofs[i]);
    } else {
      std::vector<std::pair<int, int>> v;
      for (int i = 0; i < n_c; ++i) v.emplace_back(c_nodes[i], c_dofs[i]);
      dm.constrain_batch(v);
    }
    for (int i = 0; i < n_nodes; ++i)
      for (int d = 0; d < 6; ++d) eq_out[6 * i + d] = dm.blocks.at(node_ids[i])[d];
    *n_free = dm.num_free;
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// src/solver/linear_static.cpp:344-374 (apply_point_loads, FORCE with CID 0).
int orc_apply_forces(int n_nodes, const int* node_ids, const int* eq6, int n_force,
                     const int* f_nodes, const double* scale, const double* dir, int n,
                     double* F, char* err, int errlen) {
  std::unordered_map<int, int> idx;
  for (int i = 0; i < n_nodes; ++i) idx[node_ids[i]] = i;
  for (int f = 0; f < n_force; ++f) {
    auto it = idx.find(f_nodes[f]);
    if (it == idx.end()) {
      set_err(err, errlen, ("DofMap: node " + std::to_string(f_nodes[f]) + " not found").c_str());
      return -1;
    }
    for (int d = 0; d < 3; ++d) {
      const int eq = eq6[6 * it->second + d];
      if (eq == kConstrained) continue;
      if (eq >= n) {
        set_err(err, errlen, "Force vector index out of range");
        return -1;
      }
      F[eq] += scale[f] * dir[3 * f + d];
    }
  }
  return 0;
}

// Triplet-level assembly from user-supplied element matrices (used for the
// SparseMatrixBuilder fixtures): elements are ndof x ndof row-major.
void* orc_assemble_dense_elements(int n, int n_elem, int ndof, const int* gdofs,
                                  const double* kes) {
  std::vector<Triplet> trips;
  for (int e = 0; e < n_elem; ++e)
    add_element_stiffness(gdofs + static_cast<size_t>(e) * ndof, ndof,
                          kes + static_cast<size_t>(e) * ndof * ndof, trips);
  return new Csr(build_csr(trips, n));
}

// SparseMatrixBuilder::add() + build_csr() (tests/unit/test_sparse_matrix.cpp).
void* orc_build_from_triplets(int n, int nt, const int* rows, const int* cols,
                              const double* vals) {
  std::vector<Triplet> trips(static_cast<size_t>(nt));
  for (int i = 0; i < nt; ++i) trips[i] = {rows[i], cols[i], vals[i]};
  return new Csr(build_csr(trips, n));
}

// Full path: element stiffness for every CHEXA8 (src/solver/assembly_parallel.hpp:69-110:
// thread-local triplet lists merged in thread order), then build_csr.
void* orc_assemble_chexa8(int n_nodes, const double* node_xyz, const int* node_eq6, int n_elem,
                          const int* conn, const double* E, const double* nu, const int* form,
                          int n_dof, char* err, int errlen) {
  (void)n_nodes;
  int nthreads = 1;
#ifdef _OPENMP
  nthreads = omp_get_max_threads();
#endif
  std::vector<std::vector<Triplet>> local(static_cast<size_t>(nthreads));
  int bad = -1;
  std::string msg;
#pragma omp parallel
  {
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    auto& out = local[t];
    out.reserve(static_cast<size_t>(n_elem / nthreads + 1) * 300);
    double ke[576];
    double xyz[24];
    int gd[24];
#pragma omp for schedule(static)
    for (int e = 0; e < n_elem; ++e) {
      for (int a = 0; a < 8; ++a) {
        const int nd = conn[8 * e + a];
        for (int c = 0; c < 3; ++c) {
          xyz[3 * a + c] = node_xyz[3 * nd + c];
          gd[3 * a + c] = node_eq6[6 * nd + c];
        }
      }
      try {
        chexa8_ke(xyz, E[e], nu[e], form ? form[e] : kEAS, ke);
        add_element_stiffness(gd, 24, ke, out);
      } catch (const std::exception& ex) {
#pragma omp critical
        {
          if (bad < 0 || e < bad) {
            bad = e;
            msg = ex.what();
          }
        }
      }
    }
  }
  if (bad >= 0) {
    set_err(err, errlen, (msg + " (element index " + std::to_string(bad) + ")").c_str());
    return nullptr;
  }
  size_t total = 0;
  for (auto& v : local) total += v.size();
  std::vector<Triplet> trips;
  trips.reserve(total);
  for (auto& v : local) {
    trips.insert(trips.end(), v.begin(), v.end());
    std::vector<Triplet>().swap(v);
  }
  return new Csr(build_csr(trips, n_dof));
}

void* orc_csr_from_arrays(int n, int nnz, const int* rp, const int* ci, const double* v,
                          int lower) {
  auto* c = new Csr();
  c->n = n;
  c->nnz = nnz;
  c->row_ptr.assign(rp, rp + n + 1);
  c->col_ind.assign(ci, ci + nnz);
  c->values.assign(v, v + nnz);
  c->lower = lower != 0;
  return c;
}

void orc_csr_info(void* h, int* n, int* nnz, int* lower) {
  const auto* c = static_cast<Csr*>(h);
  *n = c->n;
  *nnz = c->nnz;
  *lower = c->lower ? 1 : 0;
}

void orc_csr_copy(void* h, int* rp, int* ci, double* v) {
  const auto* c = static_cast<Csr*>(h);
  std::copy(c->row_ptr.begin(), c->row_ptr.end(), rp);
  std::copy(c->col_ind.begin(), c->col_ind.end(), ci);
  std::copy(c->values.begin(), c->values.end(), v);
}

void orc_csr_free(void* h) { delete static_cast<Csr*>(h); }

void* orc_csr_expand(void* h) { return new Csr(expanded_symmetric(*static_cast<Csr*>(h))); }

void* orc_csr_lower(void* h) { return new Csr(lower_triangle(*static_cast<Csr*>(h))); }

void orc_csr_multiply(void* h, const double* x, double* y) {
  const auto* c = static_cast<Csr*>(h);
  csr_multiply(c->n, c->row_ptr.data(), c->col_ind.data(), c->values.data(), c->lower, x, y);
}

// FP64 (precision 64) or FP32 (precision 32) Jacobi PCG on the CSR handle
// (lower or full storage), restating run_pcg_prepared.  Returns 0 on
// convergence, -1 on an error (message in err).  iters / rel are always set.
int orc_pcg_jacobi(void* h, const double* F, double tol, int max_iters, int precision,
                   double* u_out, int* iters, double* rel, char* err, int errlen) {
  const Csr& K = *static_cast<Csr*>(h);
  *iters = 0;
  *rel = 0.0;
  try {
    validate(K, static_cast<size_t>(K.n));
    const std::vector<double> d = jacobi_diagonal(K);
    const Csr full = expanded_symmetric(K);
    std::vector<double> b(F, F + K.n);
    PcgResult res;
    if (precision == 32) {
      std::vector<float> vf(full.values.begin(), full.values.end());
      std::vector<float> df(d.begin(), d.end());
      std::vector<float> bf(b.begin(), b.end());
      std::vector<float> uf;
      try {
        res = pcg_jacobi<float>(full, vf, df, bf, tol, max_iters, uf);
      } catch (...) {
        *iters = max_iters;
        throw;
      }
      for (int i = 0; i < K.n; ++i) u_out[i] = uf[i];
    } else {
      std::vector<double> u;
      try {
        res = pcg_jacobi<double>(full, full.values, d, b, tol, max_iters, u);
      } catch (...) {
        *iters = max_iters;
        throw;
      }
      std::copy(u.begin(), u.end(), u_out);
    }
    *iters = res.iters;
    *rel = res.rel;
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// src/solver/cuda_pcg_backend_impl.hpp:2134-2262 (solve_cuda_pcg_mixed):
// FP32 inner Jacobi PCG with inner tolerance clamp(100*tol, 1e-4, 1e-2), at
// most 2 corrections after the first solve, true FP64 residual after each,
// stop on stall (res >= 0.9 * previous).
int orc_pcg_mixed(void* h, const double* F, double tol, int max_iters, double* u_out,
                  int* total_inner, int* n_solves, double* true_rel, char* err, int errlen) {
  const Csr& K = *static_cast<Csr*>(h);
  try {
    validate(K, static_cast<size_t>(K.n));
    const int n = K.n;
    const std::vector<double> d = jacobi_diagonal(K);
    const Csr full = expanded_symmetric(K);
    std::vector<float> vf(full.values.begin(), full.values.end());
    std::vector<float> df(d.begin(), d.end());
    double inner_tol = tol * 100.0;
    inner_tol = std::min(std::max(inner_tol, 1e-4), 1e-2);
    std::vector<double> x(static_cast<size_t>(n), 0.0), rhs(F, F + n), res(n), Ax(n);
    double bnorm2 = 0.0;
    for (int i = 0; i < n; ++i) bnorm2 += F[i] * F[i];
    int total = 0, solves = 0;
    double tr = 0.0, prev = 0.0;
    bool have_prev = false;
    for (int step = 0; step <= 2; ++step) {
      std::vector<float> rf(rhs.begin(), rhs.end()), df_out;
      const PcgResult pr = pcg_jacobi<float>(full, vf, df, rf, inner_tol, max_iters, df_out);
      total += pr.iters;
      ++solves;
      for (int i = 0; i < n; ++i) x[i] += static_cast<double>(df_out[i]);
      csr_multiply(n, K.row_ptr.data(), K.col_ind.data(), K.values.data(), K.lower, x.data(),
                   Ax.data());
      double rn = 0.0;
      for (int i = 0; i < n; ++i) {
        res[i] = F[i] - Ax[i];
        rn += res[i] * res[i];
      }
      tr = bnorm2 > 1e-300 ? std::sqrt(rn / bnorm2) : std::sqrt(rn);
      if (tr <= tol || step == 2) break;
      if (have_prev && tr >= prev * 0.9) break;
      prev = tr;
      have_prev = true;
      rhs = res;
    }
    std::copy(x.begin(), x.end(), u_out);
    *total_inner = total;
    *n_solves = solves;
    *true_rel = tr;
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// IC(0)-preconditioned CG: the CPU baseline beside the reference's cpu-pcg
// backend (src/solver/solver_backend.cpp:349-462, Eigen ConjugateGradient with
// IncompleteCholesky).  NOT Eigen's IncompleteCholesky (a threshold
// factorisation with fill, AMD ordering and its own scaling, whose iteration
// counts cannot be pinned without restating Eigen): this is the zero-fill
// incomplete Cholesky on K's own lower pattern, after the symmetric scaling
// D^-1/2 K D^-1/2 (unit diagonal), with a diagonal shift that starts at 0 and
// becomes 1e-3, 2e-3, ... while a pivot is not positive (the Manteuffel
// shift).  CG stops, as Eigen's does, on the unpreconditioned residual:
// ||b - K u|| < tol ||b|| (recurrence residual).  Triangular solves are
// serial; the matvec uses all threads.
struct Ic0 {
  int n = 0;
  std::vector<int> rp, ci;   // lower pattern, columns ascending, diagonal last
  std::vector<double> l;     // factor values
  std::vector<double> s;     // scaling D^-1/2
  double shift = 0.0;
};

static bool ic0_factor(const Csr& L, double shift, Ic0& f) {
  const int n = L.n;
  f.l.assign(L.values.size(), 0.0);
  for (int i = 0; i < n; ++i) {
    const int b = f.rp[i], e = f.rp[i + 1];
    for (int p = b; p < e; ++p) {
      const int k = f.ci[p];
      double v = L.values[p] * f.s[i] * f.s[k];
      if (k == i) {
        v += shift;
        for (int q = b; q < p; ++q) v -= f.l[q] * f.l[q];
        if (!(v > 0.0)) return false;
        f.l[p] = std::sqrt(v);
      } else {
        // sum over j < k in both row i and row k
        int q = b, r = f.rp[k];
        const int re = f.rp[k + 1] - 1;  // row k without its diagonal
        while (q < p && r < re) {
          const int cq = f.ci[q], cr = f.ci[r];
          if (cq == cr) {
            v -= f.l[q] * f.l[r];
            ++q;
            ++r;
          } else if (cq < cr) {
            ++q;
          } else {
            ++r;
          }
        }
        f.l[p] = v / f.l[f.rp[k + 1] - 1];
      }
    }
  }
  return true;
}

// z = (S L L^T S)^-1 r in the original variables: z = S L^-T L^-1 S r
static void ic0_apply(const Ic0& f, const std::vector<double>& r, std::vector<double>& z) {
  const int n = f.n;
  for (int i = 0; i < n; ++i) {
    double v = r[i] * f.s[i];
    const int e = f.rp[i + 1] - 1;
    for (int p = f.rp[i]; p < e; ++p) v -= f.l[p] * z[f.ci[p]];
    z[i] = v / f.l[e];
  }
  for (int i = n - 1; i >= 0; --i) {
    const int e = f.rp[i + 1] - 1;
    const double xi = z[i] / f.l[e];
    z[i] = xi;
    for (int p = f.rp[i]; p < e; ++p) z[f.ci[p]] -= f.l[p] * xi;
  }
  for (int i = 0; i < n; ++i) z[i] *= f.s[i];
}

int orc_pcg_ic0(void* h, const double* F, double tol, int max_iters, double* u_out, int* iters,
                double* rel, double* shift_out, char* err, int errlen) {
  const Csr& K = *static_cast<Csr*>(h);
  *iters = 0;
  *rel = 0.0;
  try {
    validate(K, static_cast<size_t>(K.n));
    const int n = K.n;
    const Csr L = K.lower ? K : lower_triangle(K);
    const Csr full = expanded_symmetric(L);
    Ic0 f;
    f.n = n;
    f.rp = L.row_ptr;
    f.ci = L.col_ind;
    f.s.resize(n);
    for (int i = 0; i < n; ++i) {
      const int e = L.row_ptr[i + 1] - 1;
      if (e < L.row_ptr[i] || L.col_ind[e] != i || !(L.values[e] > 0.0))
        throw Error("IC(0): missing or non-positive diagonal at row " + std::to_string(i));
      f.s[i] = 1.0 / std::sqrt(L.values[e]);
    }
    double shift = 0.0;
    while (!ic0_factor(L, shift, f)) {
      shift = shift == 0.0 ? 1e-3 : 2.0 * shift;
      if (shift > 1e3) throw Error("IC(0): no positive shift found");
    }
    *shift_out = shift;
    std::vector<double> u(n, 0.0), r(F, F + n), z(n), p(n), Ap(n);
    const double norm_b = std::sqrt(dot(r, r));
    if (norm_b < 1e-300) {
      std::fill(u_out, u_out + n, 0.0);
      return 0;
    }
    ic0_apply(f, r, z);
    p = z;
    double rz = dot(r, z);
    int it = 0;
    double rr_rel = 1.0;
    bool conv = false;
    for (; it < max_iters; ++it) {
      spmv_full(full, full.values, p, Ap);
      const double pAp = dot(p, Ap);
      if (!(pAp > 0.0)) break;
      const double alpha = rz / pAp;
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) {
        u[i] += alpha * p[i];
        r[i] -= alpha * Ap[i];
      }
      rr_rel = std::sqrt(dot(r, r)) / norm_b;
      if (rr_rel < tol) {
        ++it;
        conv = true;
        break;
      }
      ic0_apply(f, r, z);
      const double rz_new = dot(r, z);
      const double beta = rz_new / rz;
      rz = rz_new;
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    }
    *iters = it;
    *rel = rr_rel;
    std::copy(u.begin(), u.end(), u_out);
    if (!conv)
      throw Error("IC(0) PCG did not converge after " + std::to_string(max_iters) +
                  " iterations (relative residual " + std::to_string(rr_rel) + ")");
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

// Dense LLT solve of the symmetric system (lower or full storage) — the
// direct-solve stand-in for --backend=cpu at sizes a dense factor affords.
int orc_dense_cholesky_solve(void* h, const double* F, double* u_out, char* err, int errlen) {
  const Csr& K = *static_cast<Csr*>(h);
  const int n = K.n;
  try {
    if (n == 0) throw Error("stiffness matrix is empty -- no free DOFs");
    if (n > 20000) throw Error("dense solve limited to n <= 20000");
    std::vector<double> A(static_cast<size_t>(n) * n, 0.0);
    const Csr full = expanded_symmetric(K);
    for (int r = 0; r < n; ++r)
      for (int k = full.row_ptr[r]; k < full.row_ptr[r + 1]; ++k)
        A[static_cast<size_t>(r) * n + full.col_ind[k]] += full.values[k];
    // Right-looking Cholesky on the lower triangle.
    for (int j = 0; j < n; ++j) {
      double* rowj = &A[static_cast<size_t>(j) * n];
      double dj = rowj[j];
      for (int k = 0; k < j; ++k) dj -= rowj[k] * rowj[k];
      if (!(dj > 0.0)) throw Error("matrix is not positive definite");
      const double ljj = std::sqrt(dj);
      rowj[j] = ljj;
#pragma omp parallel for schedule(static)
      for (int i = j + 1; i < n; ++i) {
        double* rowi = &A[static_cast<size_t>(i) * n];
        double v = rowi[j];
        for (int k = 0; k < j; ++k) v -= rowi[k] * rowj[k];
        rowi[j] = v / ljj;
      }
    }
    std::vector<double> y(F, F + n);
    for (int i = 0; i < n; ++i) {
      const double* rowi = &A[static_cast<size_t>(i) * n];
      double v = y[i];
      for (int k = 0; k < i; ++k) v -= rowi[k] * y[k];
      y[i] = v / rowi[i];
    }
    for (int i = n - 1; i >= 0; --i) {
      double v = y[i];
      for (int k = i + 1; k < n; ++k) v -= A[static_cast<size_t>(k) * n + i] * y[k];
      y[i] = v / A[static_cast<size_t>(i) * n + i];
    }
    std::copy(y.begin(), y.end(), u_out);
    return 0;
  } catch (const std::exception& e) {
    set_err(err, errlen, e.what());
    return -1;
  }
}

}  // extern "C"
