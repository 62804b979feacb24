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
// Accumulating the 66 M_AB (594 FP64 values) replaces the 24x24 / 24x9 / 9x9
// B^T D B products, then Ke = Kuu - Kua Kaa^-1 Kau is condensed with a 9x9
// Cholesky (Eigen::LLT at :1201-1204).  Ke is written exactly symmetric
// (entry (c,r) is a copy of (r,c)).
//
// Roofline: FP64-compute bound (~10k DFMA per EAS element); inputs 8 node
// coordinates + E, nu (≈ 220 B), output 576 doubles (4.6 kB) per element.

#include "common.cuh"
#include "kernels.cuh"

namespace vsgb {

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr int kVN = 11;        // virtual nodes: 8 element nodes + 3 enhancement gradients
constexpr int kPairs = 66;     // A <= B over 11 virtual nodes
constexpr int kPairsSri = 36;  // A <= B over the 8 element nodes

__constant__ signed char c_xn[8] = {-1, +1, +1, -1, -1, +1, +1, -1};
__constant__ signed char c_en[8] = {-1, -1, +1, +1, -1, -1, +1, +1};
__constant__ signed char c_zn[8] = {-1, -1, -1, -1, +1, +1, +1, +1};

struct WarpSmem {
  double g[9][kVN][3];    // gradients at the 8 Gauss points + centroid (index 8)
  double wg[9][kVN][3];   // weighted gradients (w = detJ; centroid: 8*detJ0 for SRI)
  double M[kPairs][9];    // moment matrices M_AB (row i, col j)
  double L[9][9];         // Cholesky factor of Kaa
  double Linv[9];         // 1 / L[i][i]
  double Kua[24][9];
  double X[9][24];        // Kaa^-1 Kau
  double j0[12];          // J0^-1 (9), detJ0
};
// Ke staging aliases g/wg (dead after the moment accumulation): 594 >= 576.
static_assert(sizeof(double) * 2 * 9 * kVN * 3 >= sizeof(double) * 576, "Ke alias");

// 1/sqrt(d) in FP64 from an FP32 seed and two Newton-Raphson steps
// y <- y * (1.5 - 0.5 d y^2): quadratic convergence takes the ~2^-22 seed error
// below FP64 rounding.  Outside the FP32 range the library square root is used.
__device__ __forceinline__ double rsqrt_nr(double d) {
  if (!(d > 1e-30 && d < 1e30)) return 1.0 / sqrt(d);
  double y = static_cast<double>(rsqrtf(static_cast<float>(d)));
  const double h = 0.5 * d;
  y = y * fma(-h * y, y, 1.5);
  y = y * fma(-h * y, y, 1.5);
  return y;
}

__device__ __forceinline__ int pair_index(int A, int B) {  // A <= B < 11
  return A * kVN - (A * (A - 1)) / 2 + (B - A);
}

// Stiffness coupling of virtual nodes (A,i) and (B,j) for the EAS element
// (full isotropic D), from the canonical (A <= B) moment matrix.
__device__ __forceinline__ double kval(const WarpSmem& s, double lam, double mu, int A, int i,
                                       int B, int j) {
  if (A > B) {
    int t = A; A = B; B = t;
    t = i; i = j; j = t;
  }
  const double* m = s.M[pair_index(A, B)];
  const double tr = m[0] + m[4] + m[8];
  double v = lam * m[i * 3 + j] + mu * m[j * 3 + i];
  if (i == j) v += mu * tr;
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
  const double* m = s.M[pair_index(a, b)];
  const double tr = m[0] + m[4] + m[8];
  double v = mu * m[jj * 3 + ii];
  if (ii == jj) v += mu * tr;
  // volumetric: symmetric product, use canonical order for exact symmetry
  v += lam * (s.wg[8][a][ii] * s.g[8][b][jj]);
  return v;
}

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
k_chexa8_stiffness(int n_elem, const double* __restrict__ xyz, const int* __restrict__ conn,
                   const double* __restrict__ E, const double* __restrict__ nu,
                   const int* __restrict__ form, double* __restrict__ kbuf,
                   ElementError* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpSmem& s = reinterpret_cast<WarpSmem*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * kWarpsPerBlock;
  const double gpt = 0.57735026918962576451;  // 1/sqrt(3)

  for (int e = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); e < n_elem; e += warps_total) {
    const bool sri = form != nullptr && form[e] == VSGB_SRI;
    const double Ee = E[e], ne = nu[e];
    const double lam = Ee * ne / ((1 + ne) * (1 - 2 * ne));
    const double mu = Ee / (2 * (1 + ne));

    // ── Phase A: Jacobians and gradients at the 8 Gauss points + centroid ──
    double X[8][3];
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int nd = __ldg(&conn[8 * e + n]);
#pragma unroll
      for (int c = 0; c < 3; ++c) X[n][c] = __ldg(&xyz[3 * nd + c]);
    }
    int bad = 0;
    double detJ = 1.0;
    double Ji[3][3];
    double dN[3][8];
    double par[3] = {0.0, 0.0, 0.0};
    if (lane < 9) {
      if (lane < 8) {
        // Gauss point order of the reference loops: xi slowest, zeta fastest.
        par[0] = (lane & 4) ? gpt : -gpt;
        par[1] = (lane & 2) ? gpt : -gpt;
        par[2] = (lane & 1) ? gpt : -gpt;
      }
#pragma unroll
      for (int n = 0; n < 8; ++n) {
        const double xn = c_xn[n], en = c_en[n], zn = c_zn[n];
        const double a = 1 + xn * par[0], b = 1 + en * par[1], c = 1 + zn * par[2];
        dN[0][n] = 0.125 * xn * b * c;
        dN[1][n] = 0.125 * en * a * c;
        dN[2][n] = 0.125 * zn * a * b;
      }
      double J[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          double acc = 0.0;
#pragma unroll
          for (int n = 0; n < 8; ++n) acc = fma(dN[r][n], X[n][c], acc);
          J[r][c] = acc;
        }
      const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
      const double c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
      const double c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
      detJ = J[0][0] * c00 + J[1][0] * c01 + J[2][0] * c02;
      if (!(detJ > 0.0)) bad = 1;
      const double id = 1.0 / detJ;
      Ji[0][0] = c00 * id;
      Ji[0][1] = c01 * id;
      Ji[0][2] = c02 * id;
      Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
      Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
      Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
      Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
      Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
      Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
      if (lane == 8) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
          for (int c = 0; c < 3; ++c) s.j0[3 * r + c] = Ji[r][c];
        s.j0[9] = detJ;
      }
    }
    if (__any_sync(0xffffffffu, bad)) {
      if (lane == 0) record_element_error(err, e, 1);
      continue;
    }
    __syncwarp();
    if (lane < 9) {
      const double w = (lane == 8) ? 8.0 * detJ : detJ;
#pragma unroll
      for (int n = 0; n < 8; ++n)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const double gv = Ji[c][0] * dN[0][n] + Ji[c][1] * dN[1][n] + Ji[c][2] * dN[2][n];
          s.g[lane][n][c] = gv;
          s.wg[lane][n][c] = w * gv;
        }
      if (lane < 8) {
        // Enhancement gradients: J0^-1.row(p) * xi_p * detJ0/detJ.
        const double scale = s.j0[9] / detJ;
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const double hv = s.j0[3 * p + c] * par[p] * scale;
            s.g[lane][8 + p][c] = hv;
            s.wg[lane][8 + p][c] = w * hv;
          }
      }
    }
    __syncwarp();

    // ── Phase B: moment matrices M_AB = sum_gp w g_A (x) g_B ──
    const int n_entries = (sri ? kPairsSri : kPairs) * 9;
    for (int t = lane; t < n_entries; t += 32) {
      const int pr = t / 9, ij = t - 9 * pr;
      const int i = ij / 3, j = ij - 3 * i;
      // decode pair index -> (A, B) over 11 virtual nodes (SRI uses the
      // first 36 pairs of the 8-node triangle, remapped below)
      int A, B;
      if (sri) {
        // pairs of the 8x8 upper triangle in row order
        int rem = pr;
        A = 0;
        while (rem >= 8 - A) {
          rem -= 8 - A;
          ++A;
        }
        B = A + rem;
      } else {
        int rem = pr;
        A = 0;
        while (rem >= kVN - A) {
          rem -= kVN - A;
          ++A;
        }
        B = A + rem;
      }
      double acc = 0.0;
#pragma unroll
      for (int q = 0; q < 8; ++q) acc = fma(s.wg[q][A][i], s.g[q][B][j], acc);
      s.M[pair_index(A, B)][ij] = acc;
    }
    __syncwarp();

    double* ke_s = &s.g[0][0][0];  // alias (g/wg dead after this point except SRI centroid)
    if (!sri) {
      // ── Phase C: Kaa Cholesky (lane 0) and Kua ──
      for (int t = lane; t < 24 * 9; t += 32) {
        const int r = t / 9, k = t - 9 * r;
        s.Kua[r][k] = kval(s, lam, mu, r / 3, r % 3, 8 + k / 3, k % 3);
      }
      // Right-looking Cholesky of Kaa spread over the warp: per column one lane
      // forms the pivot, the lanes below scale the column and the trailing
      // triangle (<= 36 entries) is updated by all lanes.  Every FP64 warp
      // instruction occupies GB300's FP64 pipe regardless of active lanes, so
      // the serial (one-lane) form costs ~5x more.
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
          const double inv = rsqrt_nr(d);
          s.L[jc][jc] = d * inv;
          s.Linv[jc] = inv;
        }
        __syncwarp();
        const double inv = s.Linv[jc];
        if (lane > jc && lane < 9) s.L[lane][jc] *= inv;
        __syncwarp();
        const int m = 8 - jc;  // trailing size
        for (int t = lane; t < m * (m + 1) / 2; t += 32) {
          const int ii = static_cast<int>((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f + 1e-4f);
          const int kk = t - ii * (ii + 1) / 2;
          const int i = jc + 1 + ii, k = jc + 1 + kk;
          s.L[i][k] -= s.L[i][jc] * s.L[k][jc];
        }
        __syncwarp();
      }
      if (lane == 0 && fail) record_element_error(err, e, 2);
      __syncwarp();
      // X[:, c] = Kaa^-1 Kau[:, c] for the 24 columns (one lane each).
      if (lane < 24) {
        double y[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
          double v = s.Kua[lane][i];
#pragma unroll
          for (int k = 0; k < i; ++k) v -= s.L[i][k] * y[k];
          y[i] = v * s.Linv[i];
        }
#pragma unroll
        for (int i = 8; i >= 0; --i) {
          double v = y[i];
#pragma unroll
          for (int k = i + 1; k < 9; ++k) v -= s.L[k][i] * y[k];
          y[i] = v * s.Linv[i];
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) s.X[i][lane] = y[i];
      }
      __syncwarp();
      // ── Phase D: Ke = Kuu - Kua X (lower triangle, mirrored) ──
      for (int t = lane; t < 300; t += 32) {
        // t -> (r, c) with c <= r in row order
        int r = static_cast<int>((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
        while ((r + 1) * (r + 2) / 2 <= t) ++r;
        while (r * (r + 1) / 2 > t) --r;
        const int c = t - r * (r + 1) / 2;
        double v = kval(s, lam, mu, r / 3, r % 3, c / 3, c % 3);
        double corr = 0.0;
#pragma unroll
        for (int k = 0; k < 9; ++k) corr = fma(s.Kua[r][k], s.X[k][c], corr);
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

void launch_chexa8_stiffness(int n_elem, const double* xyz, const int* conn, const double* E,
                             const double* nu, const int* form, double* kbuf, ElementError* err,
                             int num_sms, cudaStream_t s) {
  if (n_elem <= 0) return;
  const size_t smem = element_smem_bytes();
  VSGB_CUDA(cudaFuncSetAttribute(k_chexa8_stiffness, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
  const int blocks_needed = (n_elem + kWarpsPerBlock - 1) / kWarpsPerBlock;
  const int grid = blocks_needed < num_sms * 8 ? blocks_needed : num_sms * 8;
  k_chexa8_stiffness<<<grid, kWarpsPerBlock * 32, smem, s>>>(n_elem, xyz, conn, E, nu, form,
                                                             kbuf, err);
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
