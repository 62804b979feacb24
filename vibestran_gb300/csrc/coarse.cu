// vibestran_gb300/csrc/coarse.cu — coarse (Ritz) correction of the mixed
// refinement: basis from the first inner solve's Lanczos record, Galerkin
// correction after every FP64 residual (see coarse.cuh).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "coarse.cuh"

namespace vsgb {

namespace {

constexpr int kCT = 256;  // threads per block of the coarse kernels

// Number of eigenvalues of the tridiagonal (d, e) below sigma (Sturm count of
// the LDL^T pivots of T - sigma I).
int sturm_count(const std::vector<double>& d, const std::vector<double>& e, double sigma) {
  const size_t k = d.size();
  int cnt = 0;
  double q = d[0] - sigma;
  for (size_t j = 0;; ++j) {
    if (q < 0.0) ++cnt;
    if (j + 1 == k) break;
    if (q == 0.0) q = 1e-300;
    q = d[j + 1] - sigma - e[j] * e[j] / q;
  }
  return cnt;
}

// The same count for ns shifts at once (e2 = e^2): the recurrences of kSturmW
// shifts advance together, so their divisions overlap instead of forming one
// serial chain per count (a count is latency-bound: K dependent divisions).
// Each count equals sturm_count's for the same shift.
constexpr int kSturmW = 8;
void sturm_counts(const std::vector<double>& d, const std::vector<double>& e2,
                  const double* sig, int ns, int* cnt) {
  const size_t k = d.size();
  for (int g = 0; g < ns; g += kSturmW) {
    double s[kSturmW], q[kSturmW];
    int c[kSturmW];
    for (int u = 0; u < kSturmW; ++u) {
      s[u] = sig[g + (g + u < ns ? u : 0)];
      q[u] = d[0] - s[u];
      c[u] = 0;
    }
    for (size_t j = 0;; ++j) {
      for (int u = 0; u < kSturmW; ++u) c[u] += q[u] < 0.0 ? 1 : 0;
      if (j + 1 == k) break;
      const double dj = d[j + 1], ej = e2[j];
      for (int u = 0; u < kSturmW; ++u) {
        const double qq = q[u] == 0.0 ? 1e-300 : q[u];
        q[u] = dj - s[u] - ej / qq;
      }
    }
    for (int u = 0; u < kSturmW && g + u < ns; ++u) cnt[g + u] = c[u];
  }
}

// Solves (T - sigma I) x = b for a tridiagonal T by Gaussian elimination
// with partial pivoting (x overwrites b); zero pivots are replaced by a tiny
// value, as inverse iteration wants.
void tridiag_shifted_solve(const std::vector<double>& d, const std::vector<double>& e,
                           double sigma, std::vector<double>& b) {
  const int k = static_cast<int>(d.size());
  if (k == 1) {
    const double p = d[0] - sigma;
    b[0] /= (p != 0.0 ? p : 1e-300);
    return;
  }
  // row i after elimination: a0[i] x_i + a1[i] x_{i+1} + a2[i] x_{i+2} = b_i;
  // (diag, sup, sup2) is the row being reduced, at columns i, i+1, i+2
  std::vector<double> a0(k), a1(k, 0.0), a2(k, 0.0);
  double diag = d[0] - sigma, sup = e[0], sup2 = 0.0;
  double scale = 0.0;
  for (int i = 0; i < k; ++i) scale = std::max(scale, std::fabs(d[i] - sigma));
  const double tiny = 1e-300 + 1e-15 * scale;
  for (int i = 0; i < k - 1; ++i) {
    // rows: current (diag, sup, sup2 | b_i), next (e[i], d[i+1]-sigma, e[i+1] | b_{i+1})
    const double nl = e[i], nd = d[i + 1] - sigma, nu = (i + 1 < k - 1) ? e[i + 1] : 0.0;
    if (std::fabs(nl) > std::fabs(diag)) {
      // swap the two rows
      const double f = diag / nl;
      a0[i] = nl;
      a1[i] = nd;
      a2[i] = nu;
      const double bi = b[i];
      b[i] = b[i + 1];
      // new next row = old current - f * new current
      diag = sup - f * nd;
      sup = sup2 - f * nu;
      sup2 = 0.0;
      b[i + 1] = bi - f * b[i];
    } else {
      const double piv = diag != 0.0 ? diag : tiny;
      const double f = nl / piv;
      a0[i] = piv;
      a1[i] = sup;
      a2[i] = sup2;
      diag = nd - f * sup;
      sup = nu - f * sup2;
      sup2 = 0.0;
      b[i + 1] -= f * b[i];
    }
  }
  a0[k - 1] = diag != 0.0 ? diag : tiny;
  for (int i = k - 1; i >= 0; --i) {
    double v = b[i];
    if (i + 1 < k) v -= a1[i] * b[i + 1];
    if (i + 2 < k) v -= a2[i] * b[i + 2];
    b[i] = v / (a0[i] != 0.0 ? a0[i] : tiny);
  }
}

// tridiag_shifted_solve for ns shifts at once (vectors b[s], shifts sig[s]):
// the same operations for each shift, in the same order, with the shifts'
// elimination chains interleaved row by row so that their divisions overlap.
void tridiag_shifted_solve_multi(const std::vector<double>& d, const std::vector<double>& e,
                                 const double* sig, std::vector<double>* const* b, int ns) {
  const int k = static_cast<int>(d.size());
  if (k == 1) {
    for (int t = 0; t < ns; ++t) tridiag_shifted_solve(d, e, sig[t], *b[t]);
    return;
  }
  std::vector<double> a0(static_cast<size_t>(ns) * k), a1(static_cast<size_t>(ns) * k, 0.0),
      a2(static_cast<size_t>(ns) * k, 0.0);
  std::vector<double> diag(ns), sup(ns), sup2(ns), tiny(ns);
  for (int t = 0; t < ns; ++t) {
    diag[t] = d[0] - sig[t];
    sup[t] = e[0];
    sup2[t] = 0.0;
    double scale = 0.0;
    for (int i = 0; i < k; ++i) scale = std::max(scale, std::fabs(d[i] - sig[t]));
    tiny[t] = 1e-300 + 1e-15 * scale;
  }
  for (int i = 0; i < k - 1; ++i) {
    for (int t = 0; t < ns; ++t) {
      std::vector<double>& bb = *b[t];
      double* A0 = a0.data() + static_cast<size_t>(t) * k;
      double* A1 = a1.data() + static_cast<size_t>(t) * k;
      double* A2 = a2.data() + static_cast<size_t>(t) * k;
      const double nl = e[i], nd = d[i + 1] - sig[t], nu = (i + 1 < k - 1) ? e[i + 1] : 0.0;
      if (std::fabs(nl) > std::fabs(diag[t])) {
        const double f = diag[t] / nl;
        A0[i] = nl;
        A1[i] = nd;
        A2[i] = nu;
        const double bi = bb[i];
        bb[i] = bb[i + 1];
        diag[t] = sup[t] - f * nd;
        sup[t] = sup2[t] - f * nu;
        sup2[t] = 0.0;
        bb[i + 1] = bi - f * bb[i];
      } else {
        const double piv = diag[t] != 0.0 ? diag[t] : tiny[t];
        const double f = nl / piv;
        A0[i] = piv;
        A1[i] = sup[t];
        A2[i] = sup2[t];
        diag[t] = nd - f * sup[t];
        sup[t] = nu - f * sup2[t];
        sup2[t] = 0.0;
        bb[i + 1] -= f * bb[i];
      }
    }
  }
  for (int t = 0; t < ns; ++t)
    a0[static_cast<size_t>(t) * k + k - 1] = diag[t] != 0.0 ? diag[t] : tiny[t];
  for (int i = k - 1; i >= 0; --i) {
    for (int t = 0; t < ns; ++t) {
      std::vector<double>& bb = *b[t];
      const double* A0 = a0.data() + static_cast<size_t>(t) * k;
      const double* A1 = a1.data() + static_cast<size_t>(t) * k;
      const double* A2 = a2.data() + static_cast<size_t>(t) * k;
      double v = bb[i];
      if (i + 1 < k) v -= A1[i] * bb[i + 1];
      if (i + 2 < k) v -= A2[i] * bb[i + 2];
      bb[i] = v / (A0[i] != 0.0 ? A0[i] : tiny[t]);
    }
  }
}

// ── device kernels ────────────────────────────────────────────────────────

// Z[i][g] = sum_k W[k][i] hist[k][g'] (g' = 4 R + q for g = 3 R + q when
// the record is node-padded, else g), i < m.
// FP32 sums: Z only has to span the low modes to the Ritz vectors' accuracy
// (~1e-2); the Galerkin correction is exact for whatever Z holds, as K Z is
// formed from it in FP64.  GB300's FP64 rate would make this pass (K x m FMAs
// per DOF) the most expensive part of the basis.
// The pass streams the whole record (K x 16 bytes per node: 0.4 GB for 285
// iterations at 88 560 nodes), so it is HBM-bound: the node-padded form reads
// one 16-byte record entry per node and iteration (a thread per node, kRitzAhead
// entries in flight) with the weights in shared memory.
constexpr int kRitzAhead = 8;
__global__ void __launch_bounds__(kCT)
k_ritz_combine4(int nb, int K, int m, const float4* __restrict__ hist,
                const float* __restrict__ W, double* __restrict__ Z) {
  __shared__ float sw[kCoarseHistMax * kCoarseMax];
  for (int t = threadIdx.x; t < K * m; t += kCT) sw[t] = W[t];
  __syncthreads();
  const size_t n = 3 * static_cast<size_t>(nb);
  for (int R = blockIdx.x * kCT + threadIdx.x; R < nb; R += gridDim.x * kCT) {
    float acc[kCoarseMax][3];
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i) acc[i][0] = acc[i][1] = acc[i][2] = 0.f;
    const float4* h = hist + R;
    for (int k0 = 0; k0 < K; k0 += kRitzAhead) {
      float4 v[kRitzAhead];
#pragma unroll
      for (int u = 0; u < kRitzAhead; ++u)
        v[u] = k0 + u < K ? __ldcs(h + static_cast<size_t>(k0 + u) * nb)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int u = 0; u < kRitzAhead; ++u) {
        if (k0 + u >= K) break;
        const float* wk = sw + (k0 + u) * m;
#pragma unroll
        for (int i = 0; i < kCoarseMax; ++i)
          if (i < m) {
            const float w = wk[i];
            acc[i][0] = fmaf(w, v[u].x, acc[i][0]);
            acc[i][1] = fmaf(w, v[u].y, acc[i][1]);
            acc[i][2] = fmaf(w, v[u].z, acc[i][2]);
          }
      }
    }
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i)
      if (i < m)
#pragma unroll
        for (int q = 0; q < 3; ++q)
          Z[static_cast<size_t>(i) * n + 3 * static_cast<size_t>(R) + q] =
              static_cast<double>(acc[i][q]);
  }
}

// The same for a record of n floats per iteration (the batched solve's):
// a thread per DOF.
__global__ void __launch_bounds__(kCT)
k_ritz_combine(int n, int K, int m, const float* __restrict__ hist, const float* __restrict__ W,
               double* __restrict__ Z) {
  __shared__ float sw[kCoarseHistMax * kCoarseMax];
  for (int t = threadIdx.x; t < K * m; t += kCT) sw[t] = W[t];
  __syncthreads();
  for (int g = blockIdx.x * kCT + threadIdx.x; g < n; g += gridDim.x * kCT) {
    float acc[kCoarseMax];
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i) acc[i] = 0.f;
    const float* h = hist + g;
    for (int k0 = 0; k0 < K; k0 += kRitzAhead) {
      float v[kRitzAhead];
#pragma unroll
      for (int u = 0; u < kRitzAhead; ++u)
        v[u] = k0 + u < K ? __ldcs(h + static_cast<size_t>(k0 + u) * n) : 0.f;
#pragma unroll
      for (int u = 0; u < kRitzAhead; ++u) {
        if (k0 + u >= K) break;
        const float* wk = sw + (k0 + u) * m;
#pragma unroll
        for (int i = 0; i < kCoarseMax; ++i)
          if (i < m) acc[i] = fmaf(wk[i], v[u], acc[i]);
      }
    }
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i)
      if (i < m) Z[static_cast<size_t>(i) * n + g] = static_cast<double>(acc[i]);
  }
}

// Block sum of kCT doubles per value, fixed order; result in thread 0.
template <int NV>
__device__ __forceinline__ void block_sums(double (&v)[NV], double* sm /* NV * kCT/32 */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) sm[k * (kCT / 32) + w] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int j = 0; j < kCT / 32; ++j) s += sm[k * (kCT / 32) + j];
      v[k] = s;
    }
}

// In the last block: tot[v] = sum over blocks of part[v * nblk + b] for v <
// nv, one warp per value (lane l adds blocks l, l+32, ... in order, then a
// fixed butterfly): the partials load 32 at a time instead of one by one.
__device__ __forceinline__ void last_block_sums(const double* part, int nv, unsigned nblk,
                                                double* tot /* shared, nv */) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int v = w; v < nv; v += kCT / 32) {
    double s = 0.0;
    for (unsigned b = lane; b < nblk; b += 32) s += __ldcg(&part[static_cast<size_t>(v) * nblk + b]);
    s = warp_sum(s);
    if (lane == 0) tot[v] = s;
  }
  __syncthreads();
}

// Last-block detection: true in the block that finished last (its partials
// and every other block's are then visible).
__device__ __forceinline__ bool last_block(unsigned* counter) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// Pair dots of the Gram matrix: part[p * nblk + b], p over the lower
// triangle (i >= j) in row order.
__global__ void __launch_bounds__(kCT)
k_gram(int n, int m, const double* __restrict__ Z, const double* __restrict__ KZ,
       double* __restrict__ part) {
  __shared__ double sm[kCT / 32];
  int p = blockIdx.y, i = 0;
  while (p > i) {
    p -= i + 1;
    ++i;
  }
  const int j = p;
  const double* zi = Z + static_cast<size_t>(i) * n;
  const double* kj = KZ + static_cast<size_t>(j) * n;
  double v[1] = {0.0};
  for (int g = blockIdx.x * kCT + threadIdx.x; g < n; g += gridDim.x * kCT)
    v[0] = fma(zi[g], kj[g], v[0]);
  block_sums<1>(v, sm);
  if (threadIdx.x == 0) part[static_cast<size_t>(blockIdx.y) * gridDim.x + blockIdx.x] = v[0];
}

// Cholesky solve with the lower factor L (m x m, row stride kCoarseMax).
__device__ __forceinline__ void chol_solve(const double* L, int m, double* x) {
  for (int i = 0; i < m; ++i) {
    double v = x[i];
    for (int j = 0; j < i; ++j) v -= L[i * kCoarseMax + j] * x[j];
    x[i] = v / L[i * kCoarseMax + i];
  }
  for (int i = m - 1; i >= 0; --i) {
    double v = x[i];
    for (int j = i + 1; j < m; ++j) v -= L[j * kCoarseMax + i] * x[j];
    x[i] = v / L[i * kCoarseMax + i];
  }
}

// The coarse matrix G = Z^T K Z from the pair partials (fixed order) and its
// Cholesky factor; a pivot that is not clearly positive ends the basis there
// (the later Ritz vectors are the less accurate ones): meff vectors are used.
__global__ void __launch_bounds__(kCT) k_coarse_chol(int m, int nblk, const double* __restrict__ part,
                                                      double* __restrict__ L,
                                                      int* __restrict__ meff) {
  __shared__ double tot[kCoarseMax * (kCoarseMax + 1) / 2];
  last_block_sums(part, m * (m + 1) / 2, nblk, tot);
  if (threadIdx.x != 0) return;
  double G[kCoarseMax][kCoarseMax];
  for (int p = 0, i = 0; i < m; ++i)
    for (int j = 0; j <= i; ++j, ++p) G[i][j] = G[j][i] = tot[p];
  int keep = 0;
  for (int i = 0; i < m; ++i) {
    bool ok = true;
    for (int j = 0; j <= i && ok; ++j) {
      double v = G[i][j];
      for (int k = 0; k < j; ++k) v -= L[i * kCoarseMax + k] * L[j * kCoarseMax + k];
      if (i == j) {
        if (!(v > 1e-10 * G[i][i]))
          ok = false;
        else
          L[i * kCoarseMax + i] = sqrt(v);
      } else {
        L[i * kCoarseMax + j] = v / L[j * kCoarseMax + j];
      }
    }
    if (!ok) break;
    keep = i + 1;
  }
  *meff = keep;
}

// c = (Z^T K Z)^-1 Z^T r.
__global__ void __launch_bounds__(kCT)
k_coarse_dots(int n, const int* __restrict__ meff, const double* __restrict__ Z,
              const double* __restrict__ r, const double* __restrict__ L,
              double* __restrict__ part, unsigned* counter, double* __restrict__ c) {
  __shared__ double sm[kCoarseMax * (kCT / 32)];
  const int m = *meff;
  double v[kCoarseMax];
#pragma unroll
  for (int i = 0; i < kCoarseMax; ++i) v[i] = 0.0;
  for (int g = blockIdx.x * kCT + threadIdx.x; g < n; g += gridDim.x * kCT) {
    const double rv = r[g];
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i)
      if (i < m) v[i] = fma(Z[static_cast<size_t>(i) * n + g], rv, v[i]);
  }
  block_sums<kCoarseMax>(v, sm);
  if (threadIdx.x == 0)
    for (int i = 0; i < m; ++i) part[static_cast<size_t>(i) * gridDim.x + blockIdx.x] = v[i];
  if (!last_block(counter)) return;
  __shared__ double tot[kCoarseMax];
  last_block_sums(part, m, gridDim.x, tot);
  if (threadIdx.x == 0) {
    double b[kCoarseMax];
    for (int i = 0; i < m; ++i) b[i] = tot[i];
    chol_solve(L, m, b);
    for (int i = 0; i < m; ++i) c[i] = b[i];
    *counter = 0u;
  }
}

// u += Z c, r -= K Z c; ||r||^2 and ||u||_D^2 refresh the outer record.
__global__ void __launch_bounds__(kCT)
k_coarse_update(int n, const int* __restrict__ meff, const double* __restrict__ Z,
                const double* __restrict__ KZ, const double* __restrict__ c,
                double* __restrict__ u, double* __restrict__ r, const double* __restrict__ dinv,
                PcgScalars* O, double* __restrict__ part, unsigned* counter) {
  __shared__ double sm[2 * (kCT / 32)];
  const int m = *meff;
  double cc[kCoarseMax];
#pragma unroll
  for (int i = 0; i < kCoarseMax; ++i) cc[i] = i < m ? c[i] : 0.0;
  double v[2] = {0.0, 0.0};
  for (int g = blockIdx.x * kCT + threadIdx.x; g < n; g += gridDim.x * kCT) {
    double uv = u[g], rv = r[g];
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i)
      if (i < m) {
        uv = fma(cc[i], Z[static_cast<size_t>(i) * n + g], uv);
        rv = fma(-cc[i], KZ[static_cast<size_t>(i) * n + g], rv);
      }
    u[g] = uv;
    r[g] = rv;
    v[0] = fma(rv, rv, v[0]);
    v[1] = fma(uv * uv, 1.0 / dinv[g], v[1]);
  }
  block_sums<2>(v, sm);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = v[0];
    part[gridDim.x + blockIdx.x] = v[1];
  }
  if (!last_block(counter)) return;
  __shared__ double tot[2];
  last_block_sums(part, 2, gridDim.x, tot);
  if (threadIdx.x == 0) {
    const double rr = tot[0], ud = tot[1];
    const double rn = sqrt(rr);
    O->rr = rr;
    O->rel = O->norm_b > 1e-300 ? rn / O->norm_b : rn;
    O->scale = rn > 0.0 ? 1.0 / rn : 1.0;
    O->uD2 = ud;
    *counter = 0u;
  }
}

// Panels [n][16]: thread = DOF g x 4 columns (cb = 4 * (lane & 3)).
// b[i][col] = Z_i . R[:, col]; C = (Z^T K Z)^-1 b per active column.
__global__ void __launch_bounds__(kCT)
k_coarse_dots_panel(int n, const int* __restrict__ meff, const double* __restrict__ Z,
                    const double* __restrict__ R, const double* __restrict__ L,
                    const int* __restrict__ active, double* __restrict__ part, unsigned* counter,
                    double* __restrict__ C) {
  __shared__ double sm[kCoarseMax * 16 * (kCT / 32)];
  const int m = *meff;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, cb = 4 * (lane & 3);
  double v[kCoarseMax][4];
#pragma unroll
  for (int i = 0; i < kCoarseMax; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) v[i][j] = 0.0;
  const long long nc = static_cast<long long>(n) * 4;
  for (long long t = static_cast<long long>(blockIdx.x) * kCT + threadIdx.x; t < nc;
       t += static_cast<long long>(gridDim.x) * kCT) {
    const long long g = t >> 2;
    const double* rp = R + static_cast<size_t>(g) * 16 + cb;
    const double r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3];
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i)
      if (i < m) {
        const double z = Z[static_cast<size_t>(i) * n + g];
        v[i][0] = fma(z, r0, v[i][0]);
        v[i][1] = fma(z, r1, v[i][1]);
        v[i][2] = fma(z, r2, v[i][2]);
        v[i][3] = fma(z, r3, v[i][3]);
      }
  }
  // lanes with the same lane & 3 hold the same columns
#pragma unroll
  for (int i = 0; i < kCoarseMax; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double x = v[i][j];
      x += __shfl_xor_sync(0xffffffffu, x, 4);
      x += __shfl_xor_sync(0xffffffffu, x, 8);
      x += __shfl_xor_sync(0xffffffffu, x, 16);
      v[i][j] = x;
    }
  if (lane < 4)
    for (int i = 0; i < m; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) sm[((i * 16) + cb + j) * (kCT / 32) + w] = v[i][j];
  __syncthreads();
  for (int q = threadIdx.x; q < m * 16; q += kCT) {
    double s = 0.0;
    for (int j = 0; j < kCT / 32; ++j) s += sm[q * (kCT / 32) + j];
    part[static_cast<size_t>(q) * gridDim.x + blockIdx.x] = s;
  }
  if (!last_block(counter)) return;
  __shared__ double tot[kCoarseMax * 16];
  last_block_sums(part, m * 16, gridDim.x, tot);
  if (threadIdx.x < 16) {
    const int col = threadIdx.x;
    double b[kCoarseMax];
    for (int i = 0; i < m; ++i) b[i] = tot[i * 16 + col];
    if (active[col]) {
      chol_solve(L, m, b);
    } else {
      for (int i = 0; i < m; ++i) b[i] = 0.0;
    }
    for (int i = 0; i < m; ++i) C[i * 16 + col] = b[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) *counter = 0u;
}

// U += Z C, R -= K Z C (active columns); per-column ||R||^2, ||U||_D^2.
__global__ void __launch_bounds__(kCT)
k_coarse_update_panel(int n, const int* __restrict__ meff, const double* __restrict__ Z,
                      const double* __restrict__ KZ, const double* __restrict__ C,
                      double* __restrict__ U, double* __restrict__ R,
                      const double* __restrict__ dinv, const int* __restrict__ active,
                      const double* __restrict__ norm_f, double* rel, double* scale, double* uD2,
                      double* __restrict__ part, unsigned* counter) {
  __shared__ double sm[2 * 16 * (kCT / 32)];
  const int m = *meff;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, cb = 4 * (lane & 3);
  double cc[kCoarseMax][4];
#pragma unroll
  for (int i = 0; i < kCoarseMax; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) cc[i][j] = i < m ? C[i * 16 + cb + j] : 0.0;
  double v[2][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
  const long long nc = static_cast<long long>(n) * 4;
  for (long long t = static_cast<long long>(blockIdx.x) * kCT + threadIdx.x; t < nc;
       t += static_cast<long long>(gridDim.x) * kCT) {
    const long long g = t >> 2;
    double* up = U + static_cast<size_t>(g) * 16 + cb;
    double* rp = R + static_cast<size_t>(g) * 16 + cb;
    double uv[4], rv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uv[j] = up[j];
      rv[j] = rp[j];
    }
#pragma unroll
    for (int i = 0; i < kCoarseMax; ++i)
      if (i < m) {
        const double z = Z[static_cast<size_t>(i) * n + g], kz = KZ[static_cast<size_t>(i) * n + g];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          uv[j] = fma(cc[i][j], z, uv[j]);
          rv[j] = fma(-cc[i][j], kz, rv[j]);
        }
      }
    const double dg = 1.0 / dinv[g];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      up[j] = uv[j];
      rp[j] = rv[j];
      v[0][j] = fma(rv[j], rv[j], v[0][j]);
      v[1][j] = fma(uv[j] * uv[j], dg, v[1][j]);
    }
  }
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      double x = v[a][j];
      x += __shfl_xor_sync(0xffffffffu, x, 4);
      x += __shfl_xor_sync(0xffffffffu, x, 8);
      x += __shfl_xor_sync(0xffffffffu, x, 16);
      v[a][j] = x;
    }
  if (lane < 4)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int j = 0; j < 4; ++j) sm[(a * 16 + cb + j) * (kCT / 32) + w] = v[a][j];
  __syncthreads();
  for (int q = threadIdx.x; q < 32; q += kCT) {
    double s = 0.0;
    for (int j = 0; j < kCT / 32; ++j) s += sm[q * (kCT / 32) + j];
    part[static_cast<size_t>(q) * gridDim.x + blockIdx.x] = s;
  }
  if (!last_block(counter)) return;
  __shared__ double tot[32];
  last_block_sums(part, 32, gridDim.x, tot);
  if (threadIdx.x < 16) {
    const int col = threadIdx.x;
    if (active[col]) {
      const double rr = tot[col], ud = tot[16 + col];
      const double rn = sqrt(rr);
      rel[col] = norm_f[col] > 1e-300 ? rn / norm_f[col] : rn;
      scale[col] = rn > 0.0 ? 1.0 / rn : 1.0;
      uD2[col] = ud;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *counter = 0u;
}

// FP32 deflation arrays: W (node-padded, 4 x 4 nb, pad slot zero), A W
// (4 x n), vectors past meff zero; per-block partials of sum (A w_i)^2 dinv.
__global__ void __launch_bounds__(kCT)
k_defl_convert(int n, int nb, const int* __restrict__ meff, const double* __restrict__ Z,
               const double* __restrict__ KZ, const double* __restrict__ dinv,
               float* __restrict__ w32, float* __restrict__ aw32, double* __restrict__ part) {
  __shared__ double sm[4 * (kCT / 32)];
  const int m = *meff;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int g = blockIdx.x * kCT + threadIdx.x; g < n; g += gridDim.x * kCT) {
    const int R = g / 3, q = g - 3 * R;
    const double di = dinv[g];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const double z = i < m ? Z[static_cast<size_t>(i) * n + g] : 0.0;
      const double kz = i < m ? KZ[static_cast<size_t>(i) * n + g] : 0.0;
      w32[(static_cast<size_t>(i) * nb + R) * 4 + q] = static_cast<float>(z);
      if (q == 0) w32[(static_cast<size_t>(i) * nb + R) * 4 + 3] = 0.f;
      aw32[static_cast<size_t>(i) * n + g] = static_cast<float>(kz);
      v[i] = fma(kz * kz, di, v[i]);
    }
  }
  block_sums<4>(v, sm);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < 4; ++i) part[static_cast<size_t>(i) * gridDim.x + blockIdx.x] = v[i];
  }
}

// (W^T A W)^-1 from the Cholesky factor (zero past meff) and the bounds c_i.
__global__ void __launch_bounds__(kCT)
k_defl_finish(int nblk, const int* __restrict__ meff, const double* __restrict__ L,
              const double* __restrict__ part, float* __restrict__ ginv32,
              double* __restrict__ cbound) {
  __shared__ double tot[4];
  last_block_sums(part, 4, nblk, tot);
  if (threadIdx.x != 0) return;
  const int m = min(*meff, 4);
  for (int i = 0; i < 4; ++i) {
    // a zero vector gets bound 1: any positive scale (its dots are zero)
    cbound[i] = (i < m && tot[i] > 0.0) ? sqrt(tot[i]) : 1.0;
    for (int j = 0; j < 4; ++j) ginv32[i * 4 + j] = 0.f;
  }
  for (int j = 0; j < m; ++j) {
    double x[kCoarseMax] = {};
    x[j] = 1.0;
    chol_solve(L, m, x);
    for (int i = 0; i < m; ++i) ginv32[i * 4 + j] = static_cast<float>(x[i]);
  }
}

int coarse_grid(int num_sms) { return num_sms; }

}  // namespace

int tridiag_lowest(const std::vector<double>& d, const std::vector<double>& e, int m,
                   std::vector<double>& w, std::vector<double>& Y) {
  const int k = static_cast<int>(d.size());
  w.clear();
  Y.clear();
  if (k == 0 || m <= 0) return 0;
  double lo = d[0], hi = d[0];
  for (int i = 0; i < k; ++i) {
    const double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i + 1 < k ? std::fabs(e[i]) : 0.0);
    lo = std::min(lo, d[i] - r);
    hi = std::max(hi, d[i] + r);
  }
  const double span = std::max(std::fabs(lo), std::fabs(hi));
  auto open = [span](double a, double b) {
    return b - a > 1e-4 * std::max(std::fabs(a), std::fabs(b)) && b - a > 1e-16 * span;
  };
  // Each value: bisection on Sturm counts to 1e-4 of the value, then inverse
  // iteration with Rayleigh-quotient shifts, cubically convergent from there;
  // the copies of a converged value (finite-precision Lanczos) are skipped
  // with one count.
  // The brackets of the L = 2m lowest eigenvalues (by index) are bisected
  // together: a round counts at every open bracket's midpoint with the
  // recurrences interleaved (sturm_counts), and every count narrows every
  // bracket (count > j: eigenvalue j lies below the shift).  A serial
  // bisection per value spent ~0.5 ms of host time here for m = 4 at K = 285.
  const int L = std::min(k, 2 * m);
  std::vector<double> e2(e.size());
  for (size_t j = 0; j < e.size(); ++j) e2[j] = e[j] * e[j];
  std::vector<double> ba(static_cast<size_t>(L), lo), bb(static_cast<size_t>(L), hi), mids;
  std::vector<int> cnts;
  for (int round = 0; round < 200; ++round) {
    // the distinct open brackets (indices j share one until a count splits
    // them), each cut at p interior points so that a round counts at about
    // kSturmW shifts
    mids.clear();
    int nopen = 0;
    for (int j = 0; j < L; ++j)
      if (open(ba[j], bb[j]) && (j == 0 || ba[j] != ba[j - 1] || bb[j] != bb[j - 1])) ++nopen;
    if (nopen == 0) break;
    const int p = std::max(1, kSturmW / nopen);
    for (int j = 0; j < L; ++j)
      if (open(ba[j], bb[j]) && (j == 0 || ba[j] != ba[j - 1] || bb[j] != bb[j - 1]))
        for (int i = 1; i <= p; ++i) mids.push_back(ba[j] + (bb[j] - ba[j]) * i / (p + 1));
    cnts.resize(mids.size());
    sturm_counts(d, e2, mids.data(), static_cast<int>(mids.size()), cnts.data());
    for (size_t t = 0; t < mids.size(); ++t)
      for (int j = 0; j < L; ++j) {
        if (cnts[t] > j)
          bb[j] = std::min(bb[j], mids[t]);
        else
          ba[j] = std::max(ba[j], mids[t]);
      }
  }
  std::vector<double> vals;
  int idx = 0;
  while (idx < L && static_cast<int>(vals.size()) < m) {
    vals.push_back(0.5 * (ba[idx] + bb[idx]));
    idx = std::max(idx + 1, sturm_count(d, e, bb[idx] + 1e-6 * std::fabs(bb[idx])));
  }
  // (more copies than the L brackets held: the rest one value at a time)
  while (idx < k && static_cast<int>(vals.size()) < m) {
    double a = vals.empty() ? lo : vals.back(), b = hi;
    if (sturm_count(d, e, a) > idx) a = lo;
    for (int it = 0; it < 200 && b - a > 1e-4 * std::max(std::fabs(a), std::fabs(b)) &&
                     b - a > 1e-16 * span;
         ++it) {
      const double mid = 0.5 * (a + b);
      if (sturm_count(d, e, mid) > idx)
        b = mid;
      else
        a = mid;
    }
    vals.push_back(0.5 * (a + b));
    // skip the copies of this value (within 1e-6 past the bracket)
    idx = std::max(idx + 1, sturm_count(d, e, b + 1e-6 * std::fabs(b)));
  }
  // Inverse iteration with Rayleigh-quotient shifts, the values' solves
  // interleaved (tridiag_shifted_solve_multi); each value follows the same
  // sequence of operations it would alone.
  const int nv = static_cast<int>(vals.size());
  std::vector<std::vector<double>> ys(static_cast<size_t>(nv), std::vector<double>(static_cast<size_t>(k)));
  std::vector<double> ths(vals);
  std::vector<char> live(static_cast<size_t>(nv), 1);
  for (auto& y : ys)
    for (int i = 0; i < k; ++i) y[i] = 1.0 + 0.001 * ((i * 7919) % 101);  // deterministic start
  for (int rep = 0; rep < 4; ++rep) {
    std::vector<int> act;
    for (int v = 0; v < nv; ++v)
      if (live[v]) act.push_back(v);
    if (act.empty()) break;
    std::vector<double> sh(act.size());
    std::vector<std::vector<double>*> yp(act.size());
    for (size_t t = 0; t < act.size(); ++t) {
      sh[t] = ths[act[t]];
      yp[t] = &ys[act[t]];
    }
    tridiag_shifted_solve_multi(d, e, sh.data(), yp.data(), static_cast<int>(act.size()));
    for (int v : act) {
      std::vector<double>& y = ys[v];
      double nrm = 0.0;
      for (double x : y) nrm += x * x;
      nrm = std::sqrt(nrm);
      if (!(nrm > 0.0) || !std::isfinite(nrm)) {
        live[v] = 0;
        continue;
      }
      for (double& x : y) x /= nrm;
      double rq = 0.0;  // Rayleigh quotient y^T T y: the next shift
      for (int i = 0; i < k; ++i) {
        double t = d[i] * y[i];
        if (i > 0) t += e[i - 1] * y[i - 1];
        if (i + 1 < k) t += e[i] * y[i + 1];
        rq += y[i] * t;
      }
      // cubic convergence: once the shift stands still, more solves only
      // polish y below what the FP32 record resolves
      const bool settled = rep > 0 && std::fabs(rq - ths[v]) <= 1e-12 * std::fabs(ths[v]);
      ths[v] = rq;
      if (settled) live[v] = 0;
    }
  }
  for (int v = 0; v < nv; ++v) {
    std::vector<double>& y = ys[v];
    const double th = ths[v];
    // orthogonalise against the vectors kept (a near-duplicate pair)
    const size_t cols = w.size();
    for (size_t c = 0; c < cols; ++c) {
      double dot = 0.0;
      for (int i = 0; i < k; ++i) dot += y[i] * Y[c * k + i];
      for (int i = 0; i < k; ++i) y[i] -= dot * Y[c * k + i];
    }
    double nrm = 0.0;
    for (double x : y) nrm += x * x;
    nrm = std::sqrt(nrm);
    if (!(nrm > 1e-3) || !std::isfinite(nrm)) continue;
    for (double& x : y) x /= nrm;
    w.push_back(th);
    Y.insert(Y.end(), y.begin(), y.end());
  }
  return static_cast<int>(w.size());
}

int coarse_host_basis(CoarseSpace& cs, const std::vector<double>& coef, int K, int m) {
  if (K < 8 || m <= 0) return 0;
  m = std::min(m, kCoarseMax);
  // Lanczos tridiagonal of the preconditioned CG (Saad, Iterative Methods,
  // sec. 6.7.3): diagonal 1/alpha_k + beta_{k-1}/alpha_{k-1}, off-diagonal
  // sqrt(beta_k)/alpha_k
  std::vector<double> d(static_cast<size_t>(K)), e(static_cast<size_t>(K - 1));
  for (int k = 0; k < K; ++k) {
    const double al = coef[3 * k], rz = coef[3 * k + 2];
    if (!(al > 0.0) || !(rz > 0.0)) return 0;
    d[k] = 1.0 / al;
    if (k > 0) {
      const double alp = coef[3 * (k - 1)], bep = coef[3 * (k - 1) + 1];
      if (!(bep > 0.0)) return 0;
      d[k] += bep / alp;
      e[k - 1] = std::sqrt(bep) / alp;
    }
  }
  std::vector<double> w, Y;
  const int found = tridiag_lowest(d, e, m, w, Y);
  if (found == 0) return 0;
  // weights of the Lanczos vectors v_k = (-1)^k z_k / sqrt(r_k.z_k), each
  // column scaled to unit largest weight (Z's scale is free)
  std::vector<double> Wd(static_cast<size_t>(K) * found);
  for (int k = 0; k < K; ++k) {
    const double f = ((k & 1) ? -1.0 : 1.0) / std::sqrt(coef[3 * k + 2]);
    for (int i = 0; i < found; ++i)
      Wd[static_cast<size_t>(k) * found + i] = Y[static_cast<size_t>(i) * K + k] * f;
  }
  cs.Wh.assign(Wd.size(), 0.f);
  for (int i = 0; i < found; ++i) {
    double mx = 0.0;
    for (int k = 0; k < K; ++k) mx = std::max(mx, std::fabs(Wd[static_cast<size_t>(k) * found + i]));
    const double sc = mx > 0.0 ? 1.0 / mx : 1.0;
    for (int k = 0; k < K; ++k)
      cs.Wh[static_cast<size_t>(k) * found + i] = static_cast<float>(Wd[static_cast<size_t>(k) * found + i] * sc);
  }
  cs.ritz = w;
  return found;
}

bool coarse_basis(CoarseSpace& cs, const float* hist, bool padded,
                  const std::vector<double>& coef, int K, int nb, int m, int num_sms,
                  cudaStream_t s) {
  cs.valid = false;
  cs.defl_ready = false;
  cs.m = 0;
  if (K < 8 || m <= 0) return false;
  // the host part, unless it was computed ahead for this record
  int found = 0;
  if (cs.pre_found >= 0 && cs.pre_K == K && cs.pre_gen == cs.gen)
    found = cs.pre_found;
  else
    found = coarse_host_basis(cs, coef, K, m);
  cs.pre_found = -1;
  if (found == 0) return false;
  const int n = 3 * nb;
  cs.n = n;
  cs.m = found;
  cs.Z.reserve(static_cast<size_t>(kCoarseMax) * n);
  cs.KZ.reserve(static_cast<size_t>(kCoarseMax) * n);
  cs.W.reserve(static_cast<size_t>(kCoarseHistMax) * kCoarseMax);
  VSGB_CUDA(cudaMemcpyAsync(cs.W.ptr, cs.Wh.data(), sizeof(float) * cs.Wh.size(),
                            cudaMemcpyHostToDevice, s));
  if (padded)
    k_ritz_combine4<<<(nb + kCT - 1) / kCT, kCT, 0, s>>>(nb, K, found,
                                                       reinterpret_cast<const float4*>(hist),
                                                       cs.W.ptr, cs.Z.ptr);
  else
    k_ritz_combine<<<(n + kCT - 1) / kCT, kCT, 0, s>>>(n, K, found, hist, cs.W.ptr, cs.Z.ptr);
  VSGB_LAUNCH_CHECK();
  return true;
}

bool coarse_finish(CoarseSpace& cs, int num_sms, cudaStream_t s) {
  const int m = cs.m, n = cs.n;
  const int grid = coarse_grid(num_sms);
  const int pairs = m * (m + 1) / 2;
  cs.part.reserve(static_cast<size_t>(2 * kCoarseMax * 16) * grid * 2);
  cs.counter.reserve(2);
  cs.c.reserve(kCoarseMax * 16);
  cs.L.reserve(static_cast<size_t>(kCoarseMax) * kCoarseMax);
  cs.meff.reserve(1);
  VSGB_CUDA(cudaMemsetAsync(cs.counter.ptr, 0, 2 * sizeof(unsigned), s));
  k_gram<<<dim3(grid, pairs), kCT, 0, s>>>(n, m, cs.Z.ptr, cs.KZ.ptr, cs.part.ptr);
  VSGB_LAUNCH_CHECK();
  k_coarse_chol<<<1, kCT, 0, s>>>(m, grid, cs.part.ptr, cs.L.ptr, cs.meff.ptr);
  VSGB_LAUNCH_CHECK();
  cs.valid = true;  // (meff = 0 makes the corrections no-ops)
  return true;
}

void coarse_apply(const CoarseSpace& cs, double* u, double* r, const double* dinv,
                  PcgScalars* O, int num_sms, cudaStream_t s) {
  if (!cs.valid) return;
  const int grid = coarse_grid(num_sms);
  k_coarse_dots<<<grid, kCT, 0, s>>>(cs.n, cs.meff.ptr, cs.Z.ptr, r, cs.L.ptr, cs.part.ptr,
                                      cs.counter.ptr, cs.c.ptr);
  VSGB_LAUNCH_CHECK();
  k_coarse_update<<<grid, kCT, 0, s>>>(cs.n, cs.meff.ptr, cs.Z.ptr, cs.KZ.ptr, cs.c.ptr, u, r,
                                        dinv, O, cs.part.ptr, cs.counter.ptr + 1);
  VSGB_LAUNCH_CHECK();
}

void coarse_apply_panel(const CoarseSpace& cs, double* U, double* R, const double* dinv,
                        const int* active, const double* norm_f, double* rel, double* scale,
                        double* uD2, int num_sms, cudaStream_t s) {
  if (!cs.valid) return;
  const int grid = coarse_grid(num_sms);
  k_coarse_dots_panel<<<grid, kCT, 0, s>>>(cs.n, cs.meff.ptr, cs.Z.ptr, R, cs.L.ptr, active,
                                            cs.part.ptr, cs.counter.ptr, cs.c.ptr);
  VSGB_LAUNCH_CHECK();
  k_coarse_update_panel<<<grid, kCT, 0, s>>>(cs.n, cs.meff.ptr, cs.Z.ptr, cs.KZ.ptr, cs.c.ptr, U,
                                              R, dinv, active, norm_f, rel, scale, uD2,
                                              cs.part.ptr, cs.counter.ptr + 1);
  VSGB_LAUNCH_CHECK();
}

void coarse_deflation_prep(CoarseSpace& cs, const double* dinv, int num_sms, cudaStream_t s) {
  cs.defl_ready = false;
  if (!cs.valid) return;
  const int n = cs.n, nb = n / 3, grid = coarse_grid(num_sms);
  cs.w32.reserve(static_cast<size_t>(4) * 4 * nb);
  cs.aw32.reserve(static_cast<size_t>(4) * n);
  cs.ginv32.reserve(16);
  cs.cbound.reserve(4);
  k_defl_convert<<<grid, kCT, 0, s>>>(n, nb, cs.meff.ptr, cs.Z.ptr, cs.KZ.ptr, dinv, cs.w32.ptr,
                                       cs.aw32.ptr, cs.part.ptr);
  VSGB_LAUNCH_CHECK();
  k_defl_finish<<<1, kCT, 0, s>>>(grid, cs.meff.ptr, cs.L.ptr, cs.part.ptr, cs.ginv32.ptr,
                                   cs.cbound.ptr);
  VSGB_LAUNCH_CHECK();
  cs.defl_ready = true;
}

}  // namespace vsgb
