// vibestran_gb300/csrc/element.cu — CHEXA8 element stiffness on the GPU (FP64).
//
// One warp per element.  The reference forms K = sum_gp B^T D B detJ with
// dense 6x24 B and 6x6 D matrices (src/elements/solid_elements.cpp:95-180 SRI,
// :1054-1206 EAS).  For an isotropic D the 3x3 block that couples a "gradient
// vector" g in direction i with a gradient vector h in direction j is
//     lambda*g_i*h_j + mu*g_j*h_i + mu*delta_ij*(g.h)
// so every block of Kuu, Kua and Kaa follows from the 3x3 moment matrices
//     M_AB = sum_gp w_gp * g_A (x) g_B
// over 11 virtual nodes: the 8 element nodes (g = J^-1 dN/dxi) and the three
// EAS enhancement gradients h_p = J0^-1.row(p) * xi_p * detJ0/detJ (the
// reference's row-of-inverse form, solid_elements.cpp:1131-1133, :1109).
// The 66 M_AB (594 FP64 values) replace the 24x24 / 24x9 / 9x9 B^T D B
// products.  h_p is a fixed vector times a per-point scalar, so with
// c_p = detJ0 J0^-1.row(p) the enhancement moments factor as
//     M_{A,8+p}   = (sum_gp xi_p g_A) (x) c_p
//     M_{8+p,8+q} = (sum_gp xi_p xi_q / detJ) c_p (x) c_q
// (78 eight-term sums instead of 270).  Ke = Kuu - Kua Kaa^-1 Kau is then
// condensed with a 9x9 Cholesky (Eigen::LLT at :1201-1204), as Kuu - Y^T Y
// with Y = L^-1 Kau.
// Ke is written exactly symmetric (entry (c,r) is a copy of (r,c)).
//
// Roofline: FP64-pipe bound (ncu: FP64 pipe ~90% busy; GB300 issues one FP64
// warp instruction per ~17 cycles per SM whatever its active lanes, so the
// work is spread over the warp wherever it can be).  Inputs 8 node
// coordinates + E, nu (~220 B), output 576 doubles (4.6 kB) per element.

#include <cstddef>

#include "common.cuh"
#include "kernels.cuh"

namespace vsgb {

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr int kVN = 11;        // virtual nodes: 8 element nodes + 3 enhancement gradients
constexpr int kPairs = 66;     // A <= B over 11 virtual nodes


// 16-byte aligned size: warp w's area starts at w * sizeof(WarpSmem), and the
// staged Ke is copied out with 16-byte loads.
struct alignas(16) WarpSmem {
  // Phases A-C; Ke is staged over these in phase D (all dead by then).
  double g[9][8][3];      // node gradients at the 8 Gauss points + centroid (index 8)
  double wg[9][8][3];     // weighted gradients (w = detJ; centroid: 8*detJ0 for SRI)
  double V[8][3][3];      // EAS: sum_gp xi_p(gp) g_A,i(gp)  [A][p][i]
  double C[6];            // EAS: sum_gp xi_p xi_q / detJ  (p <= q: 00 01 02 11 12 22)
  double idet[8];         // 1 / detJ at the Gauss points
  double c0[9];           // detJ0 * J0^-1
  double L[9][9];         // unit lower factor of Kaa = L D L^T (strictly lower part)
  double Dinv[9];         // 1 / D[i]
  double col[9];          // unscaled pivot column of the current elimination step
  union {
    double Kua[24][9];
    double X[9][24];      // L^-1 Kau, written over Kua once every lane has read its row
  };
  // Phase D inputs.
  double M[kPairs][9];    // moment matrices M_AB (row i, col j)
  double tr[kPairs];      // their traces
  double XD[9][24];       // D^-1 L^-1 Kau
  double j0[12];          // J0^-1 (9), detJ0
};
static_assert(offsetof(WarpSmem, M) >= sizeof(double) * 576, "Ke staging over g..Kua");
static_assert(sizeof(WarpSmem) % 16 == 0, "per-warp areas and the Ke copy need 16-byte alignment");

// (p, q), p <= q, of the six enhancement pairs u = 0..5.
__device__ __forceinline__ int pp_first(int u) { return u < 3 ? 0 : (u < 5 ? 1 : 2); }
__device__ __forceinline__ int pp_second(int u) { return u < 3 ? u : (u < 5 ? u - 2 : 2); }

// 1/d in FP64 from the correctly rounded FP32 reciprocal and one
// Newton-Raphson step y <- y + y (1 - d y): quadratic convergence takes the
// <= 2^-24 relative error of the seed (plus the 2^-24 of rounding d to FP32)
// to ~2^-46, far inside the 1e-12 agreement the element matrices are held
// to.  Outside the FP32 range the FP64 division is used.
__device__ __forceinline__ double rcp_nr(double d) {
  if (!(d > 1e-30 && d < 1e30)) return 1.0 / d;
  const double y = static_cast<double>(__frcp_rn(static_cast<float>(d)));
  return fma(y, fma(-d, y, 1.0), y);
}

__device__ __forceinline__ int pair_index(int A, int B) {  // A <= B < 11
  return A * kVN - (A * (A - 1)) / 2 + (B - A);
}

// Second virtual node B of each pair index (pairs (A, B), A <= B, A-major).
__constant__ unsigned char kPairB[kPairs] = {
    0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 2, 3, 4, 5, 6, 7, 8, 9,
    10, 3, 4, 5, 6, 7, 8, 9, 10, 4, 5, 6, 7, 8, 9, 10, 5, 6, 7, 8, 9, 10, 6, 7, 8, 9, 10, 7,
    8, 9, 10, 8, 9, 10, 9, 10, 10};

// Stiffness coupling of virtual nodes (A,i) and (B,j) for the EAS element
// (full isotropic D), from the canonical (A <= B) moment matrix.
__device__ __forceinline__ double kval(const WarpSmem& s, double lam, double mu, int A, int i,
                                       int B, int j) {
  if (A > B) {
    int t = A; A = B; B = t;
    t = i; i = j; j = t;
  }
  const int pr = pair_index(A, B);
  const double* m = s.M[pr];
  double v = lam * m[i * 3 + j] + mu * m[j * 3 + i];
  if (i == j) v += mu * s.tr[pr];
  return v;
}

// SRI: deviatoric part from the Gauss-point moments (lambda removed) plus the
// centroidal volumetric term lambda * 8*detJ0 * g0_A,i * g0_B,j.
__device__ __forceinline__ double kval_sri(const WarpSmem& s, double lam, double mu, int A,
                                           int i, int B, int j) {
  int a = A, b = B, ii = i, jj = j;
  if (a > b) {
    int t = a; a = b; b = t;
    t = ii; ii = jj; jj = t;
  }
  const int pr = pair_index(a, b);
  const double* m = s.M[pr];
  double v = mu * m[jj * 3 + ii];
  if (ii == jj) v += mu * s.tr[pr];
  // volumetric: symmetric product, use canonical order for exact symmetry
  v += lam * (s.wg[8][a][ii] * s.g[8][b][jj]);
  return v;
}

// Lame constants of isotropic_D (solid_elements.cpp:17-27), one element per
// thread: the two FP64 divisions take one warp instruction per 32 elements
// here instead of one per element inside the warp-per-element kernel.
__global__ void k_lame(int n_elem, const double* __restrict__ E, const double* __restrict__ nu,
                       double2* __restrict__ lame) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n_elem; e += gridDim.x * blockDim.x) {
    const double Ee = E[e], ne = nu[e];
    lame[e] = make_double2(Ee * ne / ((1 + ne) * (1 - 2 * ne)), Ee / (2 * (1 + ne)));
  }
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
k_chexa8_stiffness(int n_elem, const double* __restrict__ xyz, const int* __restrict__ conn,
                   const double2* __restrict__ lame, const int* __restrict__ form,
                   double* __restrict__ kbuf, ElementError* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem& s = reinterpret_cast<WarpSmem*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * kWarpsPerBlock;
  const double gpt = 0.57735026918962576451;  // 1/sqrt(3)
  // Gauss point coordinates xi_p(gp) (gp = 4 i_xi + 2 i_eta + i_zeta) and the
  // products xi_p xi_q of the six enhancement pairs.
  __shared__ double s_par[3][8], s_pp[6][8];
  // |dN_n/dxi_r| at a Gauss point is 0.125 (1 +- g)(1 +- g), g = 1/sqrt(3):
  // s_mag[k] with k factors (1 + g), each formed as (0.125 fa) fb with the
  // factors fa = fma(+-1, g, 1) of the direct evaluation (so bit for bit the
  // same value); s_mag[3] = 0.125 at the centroid.
  __shared__ double s_mag[4];
  if (threadIdx.x < 4) {
    const double fm = fma(-1.0, gpt, 1.0), fp = fma(1.0, gpt, 1.0);
    const int k = threadIdx.x;
    s_mag[k] = k == 3 ? 0.125 : (0.125 * (k == 2 ? fp : fm)) * (k == 0 ? fm : fp);
  }
  if (threadIdx.x < 24) {
    const int p = threadIdx.x >> 3, q = threadIdx.x & 7;
    s_par[p][q] = ((q >> (2 - p)) & 1) ? gpt : -gpt;
  }
  if (threadIdx.x < 48) {
    const int u = threadIdx.x >> 3, q = threadIdx.x & 7;
    const double a = ((q >> (2 - pp_first(u))) & 1) ? gpt : -gpt;
    const double b = ((q >> (2 - pp_second(u))) & 1) ? gpt : -gpt;
    s_pp[u][q] = a * b;
  }
  __syncthreads();

  for (int e = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); e < n_elem; e += warps_total) {
    const bool sri = form != nullptr && form[e] == VSGB_SRI;
    const double2 lm = __ldg(&lame[e]);
    const double lam = lm.x, mu = lm.y;

    // ── Phase A: Jacobians and gradients at the 8 Gauss points + centroid ──
    double X[8][3];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int nd = __ldg(&conn[8 * e + n]);
#pragma unroll
      for (int c = 0; c < 3; ++c) X[n][c] = __ldg(&xyz[3 * nd + c]);
    }
    // Three lanes per point (lane = 3*gp + r; gp 8 = centroid, lanes 27-31
    // mirror it and store nothing): lane r forms row r of dN/dxi and of J,
    // gets the other rows from its two partner lanes by shuffles, and forms
    // component r of every gradient.  Every lane runs the same FP64
    // instructions (row / axis choices are operand selects, not branches),
    // each value with the operation order of the one-lane-per-point form.
    const bool act = lane < 27;
    const int gp = act ? lane / 3 : 8, rr = act ? lane - 3 * (lane / 3) : lane - 27 < 3 ? lane - 27 : 0;
    const int l0 = 3 * gp;  // lane holding row 0 of this point
    // dN_n/dxi_r = (0.125 s_r(n)) (1 + s_a(n) xi_a) (1 + s_b(n) xi_b), (a, b)
    // the other two axes in increasing order, xi_k = +-g at the Gauss points
    // (gp bit 2 - k set for +g: xi slowest, zeta fastest, the reference's loop
    // order) and 0 at the centroid.  Node signs s_k(n) of the CHEXA8 node
    // order (src/elements/solid_elements.cpp:76-93) as bit masks, bit n set
    // for +1: xi {-,+,+,-,-,+,+,-}, eta {-,-,+,+,-,-,+,+}, zeta {-,-,-,-,+,+,+,+}.
    // A factor is 1 + g where the node sign and the point coordinate agree, so
    // the value is a signed entry of s_mag: selects and a sign bit, no FP64
    // arithmetic.
    constexpr unsigned kPos[3] = {0x66u, 0xCCu, 0xF0u};
    const int ax1 = rr == 0 ? 1 : 0, ax2 = rr == 2 ? 1 : 2;
    const unsigned m0 = kPos[0], m1 = kPos[1], m2 = kPos[2];
    const unsigned ms = rr == 0 ? m0 : (rr == 1 ? m1 : m2);
    const unsigned ma = ax1 == 0 ? m0 : m1;
    const unsigned mb = ax2 == 1 ? m1 : m2;
    const unsigned ga = (gp >> (2 - ax1)) & 1u, gb = (gp >> (2 - ax2)) & 1u;
    double dNr[8];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int k = gp == 8 ? 3 : static_cast<int>((((ma >> n) & 1u) == ga) + (((mb >> n) & 1u) == gb));
      const unsigned long long neg = ((ms >> n) & 1u) ? 0ull : 0x8000000000000000ull;
      dNr[n] = __longlong_as_double(__double_as_longlong(s_mag[k]) ^ neg);
    }
    double Jr[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int n = 0; n < 8; ++n) acc = fma(dNr[n], X[n][c], acc);
      Jr[c] = acc;
    }
    double J[3][3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) J[k][c] = __shfl_sync(0xffffffffu, Jr[c], l0 + k);
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    const double c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    const double detJ = J[0][0] * c00 + J[1][0] * c01 + J[2][0] * c02;
    const int bad = act && !(detJ > 0.0);
    const double id = rcp_nr(detJ);
    // row rr of J^-1: (J[c+1][rr+1] J[c+2][rr+2] - J[c+1][rr+2] J[c+2][rr+1]) / det
    const int q1 = rr == 2 ? 0 : rr + 1, q2 = rr == 0 ? 2 : rr - 1;
    double Jir[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const int i1 = (c + 1) % 3, i2 = (c + 2) % 3;
      const double a1 = q1 == 0 ? J[i1][0] : (q1 == 1 ? J[i1][1] : J[i1][2]);
      const double b2 = q2 == 0 ? J[i2][0] : (q2 == 1 ? J[i2][1] : J[i2][2]);
      const double a2 = q2 == 0 ? J[i1][0] : (q2 == 1 ? J[i1][1] : J[i1][2]);
      const double b1 = q1 == 0 ? J[i2][0] : (q1 == 1 ? J[i2][1] : J[i2][2]);
      Jir[c] = (a1 * b2 - a2 * b1) * id;
    }
    if (gp == 8 && act) {
#pragma unroll
      for (int c = 0; c < 3; ++c) s.j0[3 * rr + c] = Jir[c];
      if (rr == 0) s.j0[9] = detJ;
    }
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) record_element_error(err, e, 1);
      continue;
    }
    // dN rows of the partner lanes
    double dN[3][8];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int n = 0; n < 8; ++n) dN[k][n] = __shfl_sync(0xffffffffu, dNr[n], l0 + k);
    __syncwarp();
    const double w = (gp == 8) ? 8.0 * detJ : detJ;
    if (act) {
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const double gv = Jir[0] * dN[0][n] + Jir[1] * dN[1][n] + Jir[2] * dN[2][n];
        s.g[gp][n][rr] = gv;
        s.wg[gp][n][rr] = w * gv;
      }
      if (gp < 8 && rr == 0) s.idet[gp] = id;
    }
    __syncwarp();
    if (!sri && lane < 9) s.c0[lane] = s.j0[9] * s.j0[lane];

    // ── Phase B: moment matrices M_AB = sum_gp w g_A (x) g_B ──
    // Work items with the same eight-FMA body: the 8 symmetric M_AA (x 6),
    // the 28 node pairs A < B (x 9), and for EAS the enhancement sums V (72)
    // and C (6).
    const int n_items = sri ? 300 : 378;
    for (int t = lane; t < n_items; t += 32) {
      const double* pa;
      const double* pb;
      int sa, sb;
      double* dst;
      double* dst2 = nullptr;  // mirrored entry of a symmetric M_AA
      if (t < 48) {
        const int A = t / 6, u = t - 6 * A, i = pp_first(u), j = pp_second(u);
        pa = &s.wg[0][A][i];
        pb = &s.g[0][A][j];
        sa = sb = 24;
        dst = &s.M[pair_index(A, A)][3 * i + j];
        if (i != j) dst2 = &s.M[pair_index(A, A)][3 * j + i];
      } else if (t < 300) {
        const int pr = (t - 48) / 9, ij = (t - 48) - 9 * pr, i = ij / 3, j = ij - 3 * i;
        int rem = pr, A = 0;  // pairs of the strict 8x8 upper triangle in row order
        while (rem >= 7 - A) {
          rem -= 7 - A;
          ++A;
        }
        const int B = A + 1 + rem;
        pa = &s.wg[0][A][i];
        pb = &s.g[0][B][j];
        sa = sb = 24;
        dst = &s.M[pair_index(A, B)][ij];
      } else if (t < 372) {
        const int u = t - 300, A = u / 9, rem = u - 9 * A, p = rem / 3, i = rem - 3 * p;
        pa = &s.g[0][A][i];
        sa = 24;
        pb = &s_par[p][0];
        sb = 1;
        dst = &s.V[A][p][i];
      } else {
        const int u = t - 372;
        pa = &s_pp[u][0];
        pb = &s.idet[0];
        sa = sb = 1;
        dst = &s.C[u];
      }
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q) acc = fma(pa[q * sa], pb[q * sb], acc);
      *dst = acc;
      if (dst2) *dst2 = acc;
    }
    __syncwarp();
    if (!sri) {
      // enhancement moments from V, C and c0 (the same two products per item)
      for (int t = lane; t < 270; t += 32) {
        double x, y, z;
        double* dst;
        if (t < 216) {
          const int A = t / 27, rem = t - 27 * A, p = rem / 9, ij = rem - 9 * p;
          const int i = ij / 3, j = ij - 3 * i;
          x = s.V[A][p][i];
          y = s.c0[3 * p + j];
          z = 1.0;
          dst = &s.M[pair_index(A, 8 + p)][ij];
        } else {
          const int u = (t - 216) / 9, ij = (t - 216) - 9 * u, i = ij / 3, j = ij - 3 * i;
          const int p = pp_first(u), q = pp_second(u);
          x = s.c0[3 * p + i];
          y = s.c0[3 * q + j];
          z = s.C[u];
          dst = &s.M[pair_index(8 + p, 8 + q)][ij];
        }
        *dst = x * y * z;
      }
      __syncwarp();
    }
    // traces, once per pair (SRI: only the pairs of the 8 element nodes hold
    // moments)
    for (int t = lane; t < kPairs; t += 32)
      if (!sri || kPairB[t] < 8) s.tr[t] = s.M[t][0] + s.M[t][4] + s.M[t][8];
    __syncwarp();

    double* ke_s = &s.g[0][0][0];  // Ke staging over g..Kua (EAS only; SRI writes global)
    if (!sri) {
      // ── Phase C: Kaa = L D L^T and Kua ──
      for (int t = lane; t < 24 * 9; t += 32) {
        const int r = t / 9, k = t - 9 * r;
        s.Kua[r][k] = kval(s, lam, mu, r / 3, r % 3, 8 + k / 3, k % 3);
      }
      // Right-looking L D L^T factorisation of Kaa spread over the warp (the
      // condensation needs Kua Kaa^-1 Kau only, which Eigen's LLT at
      // :1201-1204 gives as well): per column one lane forms the pivot
      // reciprocal, the lanes below scale the column and the trailing triangle
      // (<= 36 entries) is updated by all lanes.  Every FP64 warp instruction
      // occupies GB300's FP64 pipe regardless of active lanes, so the serial
      // (one-lane) form costs ~5x more, and the pivot needs no square root.
      for (int t = lane; t < 45; t += 32) {
        const int i = static_cast<int>((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f + 1e-4f);
        const int k = t - i * (i + 1) / 2;
        s.L[i][k] = kval(s, lam, mu, 8 + i / 3, i % 3, 8 + k / 3, k % 3);
      }
      __syncwarp();
      int fail = 0;
      for (int jc = 0; jc < 9; ++jc) {
        if (lane == 0) {
          double d = s.L[jc][jc];
          if (!(d > 0.0)) {
            fail = 1;
            d = 1.0;
          }
          s.Dinv[jc] = rcp_nr(d);
        }
        __syncwarp();
        const double inv = s.Dinv[jc];
        if (lane > jc && lane < 9) {
          const double a = s.L[lane][jc];
          s.col[lane] = a;
          s.L[lane][jc] = a * inv;
        }
        __syncwarp();
        const int m = 8 - jc;  // trailing size
        for (int t = lane; t < m * (m + 1) / 2; t += 32) {
          const int ii = static_cast<int>((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f + 1e-4f);
          const int kk = t - ii * (ii + 1) / 2;
          const int i = jc + 1 + ii, k = jc + 1 + kk;
          s.L[i][k] -= s.col[i] * s.L[k][jc];
        }
        __syncwarp();
      }
      if (lane == 0 && fail) record_element_error(err, e, 2);
      __syncwarp();
      // Kua Kaa^-1 Kau = (L^-1 Kau)^T D^-1 (L^-1 Kau) with Kaa = L D L^T, so
      // only the forward substitution is needed: X[:, c] = L^-1 Kau[:, c] for
      // the 24 columns (one lane each, unit diagonal), and XD = D^-1 X.
      double y[9];
      if (lane < 24) {
#pragma unroll
        for (int i = 0; i < 9; ++i) y[i] = s.Kua[lane][i];
#pragma unroll
        for (int i = 1; i < 9; ++i)
#pragma unroll
          for (int k = 0; k < i; ++k) y[i] -= s.L[i][k] * y[k];
      }
      __syncwarp();  // every row of Kua read before X overwrites it
      if (lane < 24) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          s.X[i][lane] = y[i];
          s.XD[i][lane] = y[i] * s.Dinv[i];
        }
      }
      __syncwarp();
      // ── Phase D: Ke = Kuu - X^T X (lower triangle, mirrored) ──
      for (int t = lane; t < 300; t += 32) {
        // t -> (r, c) with c <= r in row order
        int r = static_cast<int>((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
        while ((r + 1) * (r + 2) / 2 <= t) ++r;
        while (r * (r + 1) / 2 > t) --r;
        const int c = t - r * (r + 1) / 2;
        double v = kval(s, lam, mu, r / 3, r % 3, c / 3, c % 3);
        double corr = 0.0;
#pragma unroll
        for (int k = 0; k < 9; ++k) corr = fma(s.XD[k][r], s.X[k][c], corr);
        v -= corr;
        ke_s[r * 24 + c] = v;
        ke_s[c * 24 + r] = v;
      }
    } else {
      // SRI: write Kuu directly; the centroid gradients (g[8], wg[8]) are
      // still needed, so stage Ke in the Kua/X area (432 doubles) + L (81) + M tail.
      double* out = kbuf + static_cast<size_t>(e) * 576;
      for (int t = lane; t < 300; t += 32) {
        int r = static_cast<int>((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
        while ((r + 1) * (r + 2) / 2 <= t) ++r;
        while (r * (r + 1) / 2 > t) --r;
        const int c = t - r * (r + 1) / 2;
        const double v = kval_sri(s, lam, mu, c / 3, c % 3, r / 3, r % 3);
        out[r * 24 + c] = v;
        out[c * 24 + r] = v;
      }
      __syncwarp();
      continue;
    }
    __syncwarp();
    // Coalesced copy of the staged Ke (576 doubles) to global memory.
    double2* dst = reinterpret_cast<double2*>(kbuf + static_cast<size_t>(e) * 576);
    const double2* src = reinterpret_cast<const double2*>(ke_s);
    for (int t = lane; t < 288; t += 32) dst[t] = src[t];
    __syncwarp();
  }
}

// Adjoint sensitivity: dJ/dE_e = -lam_e^T (Ke / E_e) u_e (Ke is linear in E
// for fixed nu, so dK_e/dE_e = Ke / E_e).  One warp per element; lane r < 24
// forms row r of Ke u_e from the stored element matrix (the 24 row reads of
// one element share their sectors through L1), then the lam and lam2 dot
// products are warp sums.  FP64-pipe bound: 24 warp FMAs per element.
__global__ void k_element_sensitivity(int n_elem, const int* __restrict__ conn,
                                      const int* __restrict__ eq3, const double* __restrict__ E,
                                      const double* __restrict__ kbuf,
                                      const double* __restrict__ u,
                                      const double* __restrict__ lam,
                                      double* __restrict__ out,
                                      const double* __restrict__ lam2,
                                      double* __restrict__ out2) {
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * (blockDim.x >> 5);
  for (int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); e < n_elem;
       e += warps_total) {
    double ue = 0.0, le = 0.0, le2 = 0.0;
    if (lane < 24) {
      const int eq = eq3[3 * conn[8 * e + lane / 3] + lane % 3];
      if (eq >= 0) {
        ue = u[eq];
        le = lam[eq];
        if (lam2) le2 = lam2[eq];
      }
    }
    // (Ke u_e)_r for r = lane
    const double* ke = kbuf + static_cast<size_t>(e) * 576;
    double acc = 0.0;
    for (int c = 0; c < 24; ++c) {
      const double uc = __shfl_sync(0xffffffffu, ue, c);
      if (lane < 24) acc = fma(__ldg(&ke[lane * 24 + c]), uc, acc);
    }
    const double inv_e = 1.0 / E[e];
    const double v = warp_sum((lane < 24) ? le * acc : 0.0);
    if (lane == 0) out[e] = -v * inv_e;
    if (out2) {
      const double v2 = warp_sum((lane < 24) ? le2 * acc : 0.0);
      if (lane == 0) out2[e] = -v2 * inv_e;
    }
  }
}

}  // namespace

size_t element_smem_bytes() { return sizeof(WarpSmem) * kWarpsPerBlock; }

void launch_lame(int n_elem, const double* E, const double* nu, double* lame, int num_sms,
                 cudaStream_t s) {
  if (n_elem <= 0) return;
  k_lame<<<grid_for(n_elem, kThreads, num_sms * 8), kThreads, 0, s>>>(
      n_elem, E, nu, reinterpret_cast<double2*>(lame));
  VSGB_LAUNCH_CHECK();
}

void launch_chexa8_stiffness(int n_elem, const double* xyz, const int* conn, const double* E,
                             const double* nu, const int* form, double* kbuf, ElementError* err,
                             double* lame, int num_sms, cudaStream_t s) {
  if (n_elem <= 0) return;
  launch_lame(n_elem, E, nu, lame, num_sms, s);
  const double2* lm = reinterpret_cast<const double2*>(lame);
  const size_t smem = element_smem_bytes();
  VSGB_CUDA(cudaFuncSetAttribute(k_chexa8_stiffness, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
  const int blocks_needed = (n_elem + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const int grid = blocks_needed < num_sms * 8 ? blocks_needed : num_sms * 8;
  k_chexa8_stiffness<<<grid, kWarpsPerBlock * 32, smem, s>>>(n_elem, xyz, conn, lm, form, kbuf,
                                                             err);
  VSGB_LAUNCH_CHECK();
}

void launch_element_sensitivity(int n_elem, const int* conn, const int* eq3, const double* E,
                                const double* kbuf, const double* u, const double* lam,
                                double* out, const double* lam2, double* out2, int num_sms,
                                cudaStream_t s) {
  if (n_elem <= 0) return;
  const int grid = grid_for(static_cast<long long>(n_elem) * 32, kThreads, num_sms * 16);
  k_element_sensitivity<<<grid, kThreads, 0, s>>>(n_elem, conn, eq3, E, kbuf, u, lam, out, lam2,
                                                  out2);
  VSGB_LAUNCH_CHECK();
}

}  // namespace vsgb
