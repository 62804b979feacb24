// vibestran_gb300/csrc/pcg.cu — Jacobi-preconditioned CG on the GPU.
//
// Replaces run_pcg_prepared (src/solver/cuda_pcg_backend_impl.hpp:1688-1999),
// which issues per iteration three cuSPARSE SpMV passes over the lower CSR, four
// cuBLAS dots, two axpys, two single-thread scalar kernels and a blocking
// device->host copy.  Here:
//   FP64:  3 kernels / iteration
//     p  = z + beta p                       (k_search64)
//     Ap = K p, pAp, alpha                  (k_spmv64, last-block reduction)
//     u += alpha p, r -= alpha Ap, z = r/d, r.z, r.r, beta, convergence
//                                           (k_update64, last-block reduction)
//   FP32 inner (mixed):  2 kernels / iteration — the search-direction update is
//     fused into the SpMV gather (x_j = z_j + beta p_j recomputed per nonzero,
//     with an explicit fma so every consumer rounds identically), p ping-pongs
//     between two buffers.
// Scalars live on the device (PcgScalars); the host reads them every
// `check_every` iterations (iterations after convergence early-exit), and the
// iteration batch is replayed as a CUDA graph.
// The operator is full-storage CSR (both triangles), one SpMV pass.
// Roofline: HBM (12 B/nnz FP64, 8 B/nnz FP32 + vectors) and, on GB300, the
// FP64 FMA rate for the FP64 path.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <string>

#include "common.cuh"
#include "kernels.cuh"
#include "bsr.cuh"
#include "pcg.cuh"

namespace vsgb {

namespace {

constexpr int kSpmvThreads = 256;
constexpr int kLpr = 8;  // lanes per CSR row

// Lanes of the 8-lane group that shares one CSR row.  Row loops may end at
// different trip counts for different groups of a warp (n % 4 != 0), so the
// row reduction must only name its own group.
__device__ __forceinline__ unsigned group_mask() {
  return 0xffu << ((threadIdx.x & 31) & ~(kLpr - 1));
}

// ── FP64 kernels ───────────────────────────────────────────────────────────

__global__ void __launch_bounds__(kThreads)
k_init64(int n, const double* __restrict__ f, const double* __restrict__ dinv,
         double* __restrict__ r, double* __restrict__ u, double* __restrict__ z,
         double* __restrict__ p, PcgScalars* S, double* partials, unsigned* counter) {
  __shared__ double sm[64];
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = f[i];
    const double zi = ri * dinv[i];
    r[i] = ri;
    u[i] = 0.0;
    z[i] = zi;
    p[i] = 0.0;
    acc[0] = fma(ri, ri, acc[0]);
    acc[1] = fma(ri, zi, acc[1]);
  }
  double tot[2];
  if (grid_sum_last<2>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double norm_b = sqrt(fabs(tot[0]));
    S->norm_b = norm_b;
    S->rz = tot[1];
    S->rr = tot[0];
    S->rel = 1.0;
    S->beta = 0.0;
    S->alpha = 0.0;
    S->iter = 0;
    int flags = 0;
    if (norm_b < 1e-300) {
      flags = kFlagDone | kFlagZeroRhs | kFlagConverged;
      S->rel = 0.0;
    } else if (!(tot[1] > 0.0)) {
      flags = kFlagDone | kFlagNonPosRz;
    }
    S->flags = flags;
  }
}

__global__ void __launch_bounds__(kThreads)
k_search64(int n, const double* __restrict__ z, double* __restrict__ p, const PcgScalars* S) {
  if (S->flags & kFlagDone) return;
  const double beta = S->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = fma(beta, p[i], z[i]);
}

template <typename T, typename Acc>
__device__ __forceinline__ Acc row_dot(const int* __restrict__ rp, const int* __restrict__ ci,
                                       const T* __restrict__ val, const T* __restrict__ x,
                                       int row, int sub) {
  Acc s = 0;
  const int e = rp[row + 1];
  for (int k = rp[row] + sub; k < e; k += kLpr) s = fma(static_cast<Acc>(val[k]), static_cast<Acc>(x[ci[k]]), s);
  return s;
}

__global__ void __launch_bounds__(kSpmvThreads)
k_spmv64(int n, const int* __restrict__ rp, const int* __restrict__ ci,
         const double* __restrict__ val, const double* __restrict__ p, double* __restrict__ Ap,
         PcgScalars* S, double* partials, unsigned* counter) {
  if (S->flags & kFlagDone) return;
  __shared__ double sm[32];
  const int sub = threadIdx.x & (kLpr - 1);
  const int rows_per_block = kSpmvThreads / kLpr;
  double acc[1] = {0.0};
  for (int row = blockIdx.x * rows_per_block + threadIdx.x / kLpr; row < n;
       row += gridDim.x * rows_per_block) {
    double s = row_dot<double, double>(rp, ci, val, p, row, sub);
#pragma unroll
    for (int o = kLpr / 2; o > 0; o >>= 1) s += __shfl_xor_sync(group_mask(), s, o);
    if (sub == 0) {
      Ap[row] = s;
      acc[0] = fma(p[row], s, acc[0]);
    }
  }
  double tot[1];
  if (grid_sum_last<1>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double pAp = tot[0];
    S->pAp = pAp;
    if (!(pAp > 0.0)) {
      S->alpha = 0.0;
      S->flags |= kFlagDone | kFlagBreakdown;
    } else {
      S->alpha = S->rz / pAp;
    }
  }
}

__global__ void __launch_bounds__(kThreads)
k_update64(int n, double* __restrict__ u, double* __restrict__ r, double* __restrict__ z,
           const double* __restrict__ p, const double* __restrict__ Ap,
           const double* __restrict__ dinv, PcgScalars* S, double* partials, unsigned* counter) {
  if (S->flags & kFlagDone) return;
  __shared__ double sm[64];
  const double alpha = S->alpha;
  double acc[2] = {0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    u[i] = fma(alpha, p[i], u[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    const double zi = ri * dinv[i];
    r[i] = ri;
    z[i] = zi;
    acc[0] = fma(ri, zi, acc[0]);
    acc[1] = fma(ri, ri, acc[1]);
  }
  double tot[2];
  if (grid_sum_last<2>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double rz_new = tot[0], rr = tot[1];
    const double rel = sqrt(fabs(rr)) / S->norm_b;
    const int it = S->iter + 1;
    S->iter = it;
    S->rr = rr;
    S->rel = rel;
    int flags = S->flags;
    if (rel < S->tol) {
      flags |= kFlagDone | kFlagConverged;
      S->beta = 0.0;
    } else {
      S->beta = rz_new / S->rz;
      if (it >= S->max_iters) flags |= kFlagDone | kFlagMaxIters;
    }
    S->rz = rz_new;
    S->flags = flags;
  }
}

// ── FP32 inner kernels (mixed precision) ───────────────────────────────────

// r32 = (float)(r64 * scale); u32 = 0; z = r*dinv; p_old = 0; dots.
__global__ void __launch_bounds__(kThreads)
k_init32(int n, const double* __restrict__ r64, double scale_unused, const float* __restrict__ dinv,
         float* __restrict__ r, float* __restrict__ u, float* __restrict__ z,
         float* __restrict__ p, PcgScalars* S, const PcgScalars* outer, double* partials,
         unsigned* counter) {
  __shared__ double sm[64];
  const double scale = outer->scale;
  float a0 = 0.f, a1 = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float ri = static_cast<float>(r64[i] * scale);
    const float zi = ri * dinv[i];
    r[i] = ri;
    u[i] = 0.f;
    z[i] = zi;
    p[i] = 0.f;
    a0 = fmaf(ri, ri, a0);
    a1 = fmaf(ri, zi, a1);
  }
  double acc[2] = {a0, a1};
  double tot[2];
  if (grid_sum_last<2>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double norm_b = sqrt(fabs(tot[0]));
    S->norm_b = norm_b;
    S->rz = tot[1];
    S->rr = tot[0];
    S->rel = 1.0;
    S->beta = 0.0;
    S->alpha = 0.0;
    S->iter = 0;
    int flags = 0;
    if (norm_b < 1e-300) {
      flags = kFlagDone | kFlagZeroRhs | kFlagConverged;
      S->rel = 0.0;
    } else if (!(tot[1] > 0.0)) {
      flags = kFlagDone | kFlagNonPosRz;
    }
    S->flags = flags;
  }
  (void)scale_unused;
}

__global__ void __launch_bounds__(kSpmvThreads)
k_spmv32_fused(int n, const int* __restrict__ rp, const int* __restrict__ ci,
               const float* __restrict__ val, const float* __restrict__ z,
               const float* __restrict__ p_old, float* __restrict__ p_new,
               float* __restrict__ Ap, PcgScalars* S, double* partials, unsigned* counter) {
  if (S->flags & kFlagDone) return;
  __shared__ double sm[32];
  const float beta = static_cast<float>(S->beta);
  const int sub = threadIdx.x & (kLpr - 1);
  const int rows_per_block = kSpmvThreads / kLpr;
  float accf = 0.f;
  for (int row = blockIdx.x * rows_per_block + threadIdx.x / kLpr; row < n;
       row += gridDim.x * rows_per_block) {
    float s = 0.f;
    const int e = rp[row + 1];
    for (int k = rp[row] + sub; k < e; k += kLpr) {
      const int c = ci[k];
      s = fmaf(val[k], fmaf(beta, p_old[c], z[c]), s);
    }
#pragma unroll
    for (int o = kLpr / 2; o > 0; o >>= 1) s += __shfl_xor_sync(group_mask(), s, o);
    if (sub == 0) {
      const float pn = fmaf(beta, p_old[row], z[row]);
      p_new[row] = pn;
      Ap[row] = s;
      accf = fmaf(pn, s, accf);
    }
  }
  double acc[1] = {accf};
  double tot[1];
  if (grid_sum_last<1>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double pAp = tot[0];
    S->pAp = pAp;
    if (!(pAp > 0.0)) {
      S->alpha = 0.0;
      S->flags |= kFlagDone | kFlagBreakdown;
    } else {
      S->alpha = S->rz / pAp;
    }
  }
}

__global__ void __launch_bounds__(kThreads)
k_update32(int n, float* __restrict__ u, float* __restrict__ r, float* __restrict__ z,
           const float* __restrict__ p, const float* __restrict__ Ap,
           const float* __restrict__ dinv, PcgScalars* S, double* partials, unsigned* counter) {
  if (S->flags & kFlagDone) return;
  __shared__ double sm[64];
  const float alpha = static_cast<float>(S->alpha);
  float a0 = 0.f, a1 = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    u[i] = fmaf(alpha, p[i], u[i]);
    const float ri = fmaf(-alpha, Ap[i], r[i]);
    const float zi = ri * dinv[i];
    r[i] = ri;
    z[i] = zi;
    a0 = fmaf(ri, zi, a0);
    a1 = fmaf(ri, ri, a1);
  }
  double acc[2] = {a0, a1};
  double tot[2];
  if (grid_sum_last<2>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double rz_new = tot[0], rr = tot[1];
    const double rel = sqrt(fabs(rr)) / S->norm_b;
    const int it = S->iter + 1;
    S->iter = it;
    S->rr = rr;
    S->rel = rel;
    int flags = S->flags;
    if (rel < S->tol) {
      flags |= kFlagDone | kFlagConverged;
      S->beta = 0.0;
    } else {
      S->beta = rz_new / S->rz;
      if (it >= S->max_iters) flags |= kFlagDone | kFlagMaxIters;
    }
    S->rz = rz_new;
    S->flags = flags;
  }
}

// ── FP64 refinement kernels ────────────────────────────────────────────────

// r64 = f - K u64; ||r64||^2 -> outer scalars (rel vs ||f||, scale = 1/||r||).
__global__ void __launch_bounds__(kSpmvThreads)
k_residual64(int n, const int* __restrict__ rp, const int* __restrict__ ci,
             const double* __restrict__ val, const double* __restrict__ u,
             const double* __restrict__ f, double* __restrict__ r, PcgScalars* O,
             double* partials, unsigned* counter) {
  __shared__ double sm[32];
  const int sub = threadIdx.x & (kLpr - 1);
  const int rows_per_block = kSpmvThreads / kLpr;
  double acc[1] = {0.0};
  for (int row = blockIdx.x * rows_per_block + threadIdx.x / kLpr; row < n;
       row += gridDim.x * rows_per_block) {
    double s = row_dot<double, double>(rp, ci, val, u, row, sub);
#pragma unroll
    for (int o = kLpr / 2; o > 0; o >>= 1) s += __shfl_xor_sync(group_mask(), s, o);
    if (sub == 0) {
      const double ri = f[row] - s;
      r[row] = ri;
      acc[0] = fma(ri, ri, acc[0]);
    }
  }
  double tot[1];
  if (grid_sum_last<1>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double rn = sqrt(fabs(tot[0]));
    O->rr = tot[0];
    O->rel = O->norm_b > 1e-300 ? rn / O->norm_b : rn;
    O->scale = rn > 0.0 ? 1.0 / rn : 1.0;
  }
}

// ||f||^2 and the first correction RHS (r64 = f, u64 = 0).
__global__ void __launch_bounds__(kThreads)
k_outer_init(int n, const double* __restrict__ f, double* __restrict__ r,
             double* __restrict__ u, PcgScalars* O, double* partials, unsigned* counter) {
  __shared__ double sm[32];
  double acc[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double fi = f[i];
    r[i] = fi;
    u[i] = 0.0;
    acc[0] = fma(fi, fi, acc[0]);
  }
  double tot[1];
  if (grid_sum_last<1>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double nb = sqrt(fabs(tot[0]));
    O->norm_b = nb;
    O->rr = tot[0];
    O->rel = nb > 1e-300 ? 1.0 : 0.0;
    O->scale = nb > 1e-300 ? 1.0 / nb : 1.0;
    O->uD2 = 0.0;
    O->flags = nb < 1e-300 ? (kFlagDone | kFlagZeroRhs | kFlagConverged) : 0;
    O->iter = 0;
  }
}

__global__ void __launch_bounds__(kThreads)
k_accumulate(int n, double* __restrict__ u64, const float* __restrict__ d32,
             const PcgScalars* O) {
  const double inv = 1.0 / O->scale;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    u64[i] = fma(static_cast<double>(d32[i]), inv, u64[i]);
}

__global__ void k_cast_f32(long long n, const double* __restrict__ in, float* __restrict__ out) {
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    out[i] = static_cast<float>(in[i]);
}

template <typename T>
__global__ void k_fill(long long n, T* __restrict__ out, T v) {
  for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    out[i] = v;
}

// ── 3x3 node-block (sliced-ELL) SpMV kernels ──────────────────────────────
// One warp per slice of 8 block rows; lane = 4*row + q handles block slots
// q, q+4, ...; the three row sums are reduced over the 4 lanes of a row and
// lanes q = 0..2 write component q (24 consecutive outputs per warp).

__device__ __forceinline__ double fmat(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmat(float a, float b, float c) { return fmaf(a, b, c); }

struct BsrView {
  int nb, nslices;
  const int* __restrict__ slice_ptr;
  const int* __restrict__ rowlen;
  const int* __restrict__ cols;
};

// The FP32 operator is in difference form (bsr.cuh): block columns other
// than the row itself multiply x_J - x_I, the diagonal slot (holding the row
// sum R_I) multiplies x_I.  With m = 0 on the diagonal and 1 elsewhere,
// fma(-m, x_I, x_J) is exactly that operand.
template <typename T>
__device__ __forceinline__ void diff_operand(bool on, int c, int R, T i0, T i1, T i2, T& x0,
                                             T& x1, T& x2) {
  if (on) {
    const T m = c != R ? T(1) : T(0);
    x0 = fmat(-m, i0, x0);
    x1 = fmat(-m, i1, x1);
    x2 = fmat(-m, i2, x2);
  }
}

template <typename T, typename Gather>
__device__ __forceinline__ void bsr_row_block(const BsrView& B, const T* __restrict__ vals,
                                              int sl, int lane, Gather gx, T& y0, T& y1, T& y2) {
  constexpr bool kDiff = sizeof(T) == 4;
  const int base = B.slice_ptr[sl], steps = B.slice_ptr[sl + 1] - base;
  const int R = 8 * sl + (lane >> 2);
  T i0 = T(0), i1 = T(0), i2 = T(0);
  if (kDiff && R < B.nb) gx(R, i0, i1, i2);
  y0 = y1 = y2 = T(0);
  // Branch-free over the slice's steps: padding slots hold block column 0 and
  // zero values (allocated and zero-filled), so they add nothing, and the
  // loads of several steps can be in flight at once.
  const int* cp = B.cols + static_cast<size_t>(base) * 32 + lane;
  const T* vp = vals + static_cast<size_t>(base) * 288 + lane;
  int t = 0;
  for (; t + 2 <= steps; t += 2) {
    const int c0 = __ldcg(cp + 32 * t), c1 = __ldcg(cp + 32 * (t + 1));
    T a[2][9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      a[0][k] = __ldcg(vp + 288 * t + 32 * k);
      a[1][k] = __ldcg(vp + 288 * (t + 1) + 32 * k);
    }
    T x0, x1, x2, w0, w1, w2;
    gx(c0, x0, x1, x2);
    gx(c1, w0, w1, w2);
    diff_operand(kDiff, c0, R, i0, i1, i2, x0, x1, x2);
    diff_operand(kDiff, c1, R, i0, i1, i2, w0, w1, w2);
    y0 = fmat(a[0][0], x0, fmat(a[0][1], x1, fmat(a[0][2], x2, y0)));
    y1 = fmat(a[0][3], x0, fmat(a[0][4], x1, fmat(a[0][5], x2, y1)));
    y2 = fmat(a[0][6], x0, fmat(a[0][7], x1, fmat(a[0][8], x2, y2)));
    y0 = fmat(a[1][0], w0, fmat(a[1][1], w1, fmat(a[1][2], w2, y0)));
    y1 = fmat(a[1][3], w0, fmat(a[1][4], w1, fmat(a[1][5], w2, y1)));
    y2 = fmat(a[1][6], w0, fmat(a[1][7], w1, fmat(a[1][8], w2, y2)));
  }
  if (t < steps) {
    const int c0 = __ldcg(cp + 32 * t);
    T a[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) a[k] = __ldcg(vp + 288 * t + 32 * k);
    T x0, x1, x2;
    gx(c0, x0, x1, x2);
    diff_operand(kDiff, c0, R, i0, i1, i2, x0, x1, x2);
    y0 = fmat(a[0], x0, fmat(a[1], x1, fmat(a[2], x2, y0)));
    y1 = fmat(a[3], x0, fmat(a[4], x1, fmat(a[5], x2, y1)));
    y2 = fmat(a[6], x0, fmat(a[7], x1, fmat(a[8], x2, y2)));
  }
#pragma unroll
  for (int o = 1; o <= 2; o <<= 1) {
    y0 += __shfl_xor_sync(0xffffffffu, y0, o);
    y1 += __shfl_xor_sync(0xffffffffu, y1, o);
    y2 += __shfl_xor_sync(0xffffffffu, y2, o);
  }
}

__global__ void __launch_bounds__(kSpmvThreads)
k_bsr_spmv64(BsrView B, const double* __restrict__ vals, const double* __restrict__ p,
             double* __restrict__ Ap, PcgScalars* S, double* partials, unsigned* counter) {
  if (S->flags & kFlagDone) return;
  __shared__ double sm[32];
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  double acc[1] = {0.0};
  for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < B.nslices; sl += gridDim.x * wpb) {
    double y0, y1, y2;
    bsr_row_block<double>(B, vals, sl, lane,
                          [&](int c, double& a, double& b, double& d) {
                            a = p[3 * c];
                            b = p[3 * c + 1];
                            d = p[3 * c + 2];
                          },
                          y0, y1, y2);
    const int R = sl * 8 + (lane >> 2), q = lane & 3;
    if (R < B.nb && q < 3) {
      const double yq = q == 0 ? y0 : (q == 1 ? y1 : y2);
      Ap[3 * R + q] = yq;
      acc[0] = fma(p[3 * R + q], yq, acc[0]);
    }
  }
  double tot[1];
  if (grid_sum_last<1>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double pAp = tot[0];
    S->pAp = pAp;
    if (!(pAp > 0.0)) {
      S->alpha = 0.0;
      S->flags |= kFlagDone | kFlagBreakdown;
    } else {
      S->alpha = S->rz / pAp;
    }
  }
}

// K X for M vectors at once (vector v at X + v n, result at Y + v n): the
// coarse basis products K Z.  The FP64 operator is read once for all M
// vectors; per vector the arithmetic and its order are those of
// bsr_row_block, so each column equals a k_bsr_spmv64 product bit for bit.
template <int M>
__global__ void __launch_bounds__(kSpmvThreads)
k_bsr_spmm64_cols(BsrView B, const double* __restrict__ vals, const double* __restrict__ X,
                  double* __restrict__ Y, int n) {
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < B.nslices; sl += gridDim.x * wpb) {
    const int base = B.slice_ptr[sl], steps = B.slice_ptr[sl + 1] - base;
    const int* cp = B.cols + static_cast<size_t>(base) * 32 + lane;
    const double* vp = vals + static_cast<size_t>(base) * 288 + lane;
    double y[M][3];
#pragma unroll
    for (int v = 0; v < M; ++v) y[v][0] = y[v][1] = y[v][2] = 0.0;
    for (int t = 0; t < steps; ++t) {
      const int c = __ldcg(cp + 32 * t);
      double a[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) a[k] = __ldcg(vp + 288 * t + 32 * k);
#pragma unroll
      for (int v = 0; v < M; ++v) {
        const double* x = X + static_cast<size_t>(v) * n + 3 * static_cast<size_t>(c);
        const double x0 = __ldg(x), x1 = __ldg(x + 1), x2 = __ldg(x + 2);
        y[v][0] = fma(a[0], x0, fma(a[1], x1, fma(a[2], x2, y[v][0])));
        y[v][1] = fma(a[3], x0, fma(a[4], x1, fma(a[5], x2, y[v][1])));
        y[v][2] = fma(a[6], x0, fma(a[7], x1, fma(a[8], x2, y[v][2])));
      }
    }
    const int R = sl * 8 + (lane >> 2), q = lane & 3;
#pragma unroll
    for (int v = 0; v < M; ++v) {
#pragma unroll
      for (int o = 1; o <= 2; o <<= 1) {
        y[v][0] += __shfl_xor_sync(0xffffffffu, y[v][0], o);
        y[v][1] += __shfl_xor_sync(0xffffffffu, y[v][1], o);
        y[v][2] += __shfl_xor_sync(0xffffffffu, y[v][2], o);
      }
      if (R < B.nb && q < 3)
        Y[static_cast<size_t>(v) * n + 3 * static_cast<size_t>(R) + q] =
            q == 0 ? y[v][0] : (q == 1 ? y[v][1] : y[v][2]);
    }
  }
}

__global__ void __launch_bounds__(kSpmvThreads)
k_bsr_spmv32_fused(BsrView B, const float* __restrict__ vals, const float* __restrict__ z,
                   const float* __restrict__ p_old, float* __restrict__ p_new,
                   float* __restrict__ Ap, PcgScalars* S, double* partials, unsigned* counter) {
  if (S->flags & kFlagDone) return;
  __shared__ double sm[32];
  const float beta = static_cast<float>(S->beta);
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  float accf = 0.f;
  for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < B.nslices; sl += gridDim.x * wpb) {
    float y0, y1, y2;
    bsr_row_block<float>(B, vals, sl, lane,
                         [&](int c, float& a, float& b, float& d) {
                           a = fmaf(beta, p_old[3 * c], z[3 * c]);
                           b = fmaf(beta, p_old[3 * c + 1], z[3 * c + 1]);
                           d = fmaf(beta, p_old[3 * c + 2], z[3 * c + 2]);
                         },
                         y0, y1, y2);
    const int R = sl * 8 + (lane >> 2), q = lane & 3;
    if (R < B.nb && q < 3) {
      const int i = 3 * R + q;
      const float yq = q == 0 ? y0 : (q == 1 ? y1 : y2);
      const float pn = fmaf(beta, p_old[i], z[i]);
      p_new[i] = pn;
      Ap[i] = yq;
      accf = fmaf(pn, yq, accf);
    }
  }
  double acc[1] = {accf};
  double tot[1];
  if (grid_sum_last<1>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double pAp = tot[0];
    S->pAp = pAp;
    if (!(pAp > 0.0)) {
      S->alpha = 0.0;
      S->flags |= kFlagDone | kFlagBreakdown;
    } else {
      S->alpha = S->rz / pAp;
    }
  }
}

// r = f - K u (FP64), ||r||^2 and ||u||_D^2 (D = 1 / dinv, the Jacobi
// diagonal: the scale of an error-controlled refinement step's target).
__global__ void __launch_bounds__(kSpmvThreads)
k_bsr_residual64(BsrView B, const double* __restrict__ vals, const double* __restrict__ u,
                 const double* __restrict__ f, const double* __restrict__ dinv,
                 double* __restrict__ r, PcgScalars* O, double* partials, unsigned* counter) {
  __shared__ double sm[64];
  const int lane = threadIdx.x & 31;
  const int wpb = blockDim.x >> 5;
  double acc[2] = {0.0, 0.0};
  for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < B.nslices; sl += gridDim.x * wpb) {
    double y0, y1, y2;
    bsr_row_block<double>(B, vals, sl, lane,
                          [&](int c, double& a, double& b, double& d) {
                            a = u[3 * c];
                            b = u[3 * c + 1];
                            d = u[3 * c + 2];
                          },
                          y0, y1, y2);
    const int R = sl * 8 + (lane >> 2), q = lane & 3;
    if (R < B.nb && q < 3) {
      const int i = 3 * R + q;
      const double ri = f[i] - (q == 0 ? y0 : (q == 1 ? y1 : y2));
      r[i] = ri;
      acc[0] = fma(ri, ri, acc[0]);
      const double ui = u[i];
      acc[1] += ui * ui / dinv[i];
    }
  }
  double tot[2];
  if (grid_sum_last<2>(acc, partials, counter, sm, tot) && threadIdx.x == 0) {
    const double rn = sqrt(fabs(tot[0]));
    O->rr = tot[0];
    O->rel = O->norm_b > 1e-300 ? rn / O->norm_b : rn;
    O->scale = rn > 0.0 ? 1.0 / rn : 1.0;
    O->uD2 = tot[1];
  }
}

}  // namespace

// ── host orchestration ─────────────────────────────────────────────────────

void PcgEngine::prepare(const AssembledCsr& op, bool need32, cudaStream_t s, bool prebuilt) {
  op_ = &op;
  n_ = op.n;
  const size_t n = static_cast<size_t>(n_ > 0 ? n_ : 1);
  const int vgrid = grid_for(n_, kThreads, num_sms_ * 4);
  vec_grid_ = vgrid;
  spmv_grid_ = grid_for(static_cast<long long>(n_) * kLpr, kSpmvThreads, num_sms_ * 8);
  use_bsr_ = false;
  if (prebuilt) {
    // blocks assembled directly (assemble_blocks); add the FP32 copy if asked
    if (!bsr_.valid) throw Error(VSGB_ERR_STATE, "no block operator was assembled");
    use_bsr_ = true;
    if (need32 && !bsr_.has32) {
      bsr_make_f32(bsr_, num_sms_, s);
      launches_ += 1;
    }
  } else if (format_ != 1) {
    use_bsr_ = build_bsr(op, bsr_, true, need32, num_sms_, s);
    if (!use_bsr_ && format_ == 2)
      throw Error(VSGB_ERR_INVALID, "3x3 block format requested but the equations are not "
                                    "node-aligned triples with filled blocks");
  }
  bsr_grid_ = use_bsr_ ? grid_for(static_cast<long long>(bsr_.nslices) * 32, kSpmvThreads,
                                  1 << 30)
                       : 1;
  res_.ok32 = res_.ok64 = false;
  if (use_bsr_ && resident_) {
    int dev = 0;
    VSGB_CUDA(cudaGetDevice(&dev));
    resident_prepare(bsr_, need32, dev, num_sms_, res_, s);
    launches_ += 2;
  }
  int pmax = (vec_grid_ > spmv_grid_ ? vec_grid_ : spmv_grid_);
  if (bsr_grid_ > pmax) pmax = bsr_grid_;
  partials_.reserve(static_cast<size_t>(pmax) * 2);
  counters_.reserve(8);
  scal_.reserve(2);
  VSGB_CUDA(cudaMemsetAsync(counters_.ptr, 0, sizeof(unsigned) * 8, s));
  if (need32 && use_bsr_) {
    dinv32_.reserve(n);
    k_cast_f32<<<num_sms_ * 4, kThreads, 0, s>>>(n_, op.dinv.ptr, dinv32_.ptr);
    VSGB_LAUNCH_CHECK();
    launches_ += 1;
    has32_ = true;
  } else if (need32) {
    val32_.reserve(static_cast<size_t>(op.nnz > 0 ? op.nnz : 1));
    dinv32_.reserve(n);
    k_cast_f32<<<num_sms_ * 8, kThreads, 0, s>>>(op.nnz, op.values.ptr, val32_.ptr);
    VSGB_LAUNCH_CHECK();
    k_cast_f32<<<num_sms_ * 4, kThreads, 0, s>>>(n_, op.dinv.ptr, dinv32_.ptr);
    VSGB_LAUNCH_CHECK();
    launches_ += 2;
    has32_ = true;
  } else {
    has32_ = false;
  }
  ++generation_;
}

void PcgEngine::ensure_vectors(bool mixed) {
  const size_t n = static_cast<size_t>(n_ > 0 ? n_ : 1);
  r_.reserve(n);
  z_.reserve(n);
  p_.reserve(n);
  Ap_.reserve(n);
  u_.reserve(n);
  if (mixed) {
    r32_.reserve(n);
    z32_.reserve(n);
    p32a_.reserve(n);
    p32b_.reserve(n);
    Ap32_.reserve(n);
    u32_.reserve(n);
  }
}

void PcgEngine::read_scalars(cudaStream_t s, PcgScalars* host, int which) {
  VSGB_CUDA(cudaMemcpyAsync(host, scal_.ptr + which, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
}

void PcgEngine::set_limits(cudaStream_t s, int which, double tol, int max_iters) {
  // tol / max_iters are written into the record by a tiny H2D copy before init.
  PcgScalars h{};
  h.tol = tol;
  h.max_iters = max_iters;
  VSGB_CUDA(cudaMemcpyAsync(&scal_.ptr[which].tol, &h.tol, sizeof(double), cudaMemcpyHostToDevice, s));
  VSGB_CUDA(cudaMemcpyAsync(&scal_.ptr[which].max_iters, &h.max_iters, sizeof(int),
                            cudaMemcpyHostToDevice, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
}

namespace {
BsrView view_of(const BsrSell& b) {
  return BsrView{b.nb, b.nslices, b.slice_ptr.ptr, b.rowlen.ptr, b.cols.ptr};
}
}  // namespace

void PcgEngine::launch_spmv64(cudaStream_t s, const double* x, double* y) {
  const AssembledCsr& op = *op_;
  if (use_bsr_)
    k_bsr_spmv64<<<bsr_grid_, kSpmvThreads, 0, s>>>(view_of(bsr_), bsr_.val64.ptr, x, y,
                                                    scal_.ptr, partials_.ptr, counters_.ptr + 1);
  else
    k_spmv64<<<spmv_grid_, kSpmvThreads, 0, s>>>(n_, op.row_ptr.ptr, op.col_ind.ptr,
                                                 op.values.ptr, x, y, scal_.ptr, partials_.ptr,
                                                 counters_.ptr + 1);
}

void PcgEngine::launch_spmv32(cudaStream_t s, const float* pin, float* pout) {
  const AssembledCsr& op = *op_;
  if (use_bsr_)
    k_bsr_spmv32_fused<<<bsr_grid_, kSpmvThreads, 0, s>>>(view_of(bsr_), bsr_.val32.ptr,
                                                          z32_.ptr, pin, pout, Ap32_.ptr,
                                                          scal_.ptr, partials_.ptr,
                                                          counters_.ptr + 1);
  else
    k_spmv32_fused<<<spmv_grid_, kSpmvThreads, 0, s>>>(n_, op.row_ptr.ptr, op.col_ind.ptr,
                                                       val32_.ptr, z32_.ptr, pin, pout,
                                                       Ap32_.ptr, scal_.ptr, partials_.ptr,
                                                       counters_.ptr + 1);
}

void PcgEngine::launch_residual64(cudaStream_t s, const double* d_f) {
  const AssembledCsr& op = *op_;
  if (use_bsr_)
    k_bsr_residual64<<<bsr_grid_, kSpmvThreads, 0, s>>>(view_of(bsr_), bsr_.val64.ptr, u_.ptr,
                                                        d_f, op.dinv.ptr, r_.ptr, scal_.ptr + 1,
                                                        partials_.ptr, counters_.ptr + 3);
  else
    k_residual64<<<spmv_grid_, kSpmvThreads, 0, s>>>(n_, op.row_ptr.ptr, op.col_ind.ptr,
                                                     op.values.ptr, u_.ptr, d_f, r_.ptr,
                                                     scal_.ptr + 1, partials_.ptr,
                                                     counters_.ptr + 3);
}

void PcgEngine::launch_batch64(cudaStream_t s) {
  const AssembledCsr& op = *op_;
  for (int k = 0; k < check_every_; ++k) {
    k_search64<<<vec_grid_, kThreads, 0, s>>>(n_, z_.ptr, p_.ptr, scal_.ptr);
    launch_spmv64(s, p_.ptr, Ap_.ptr);
    k_update64<<<vec_grid_, kThreads, 0, s>>>(n_, u_.ptr, r_.ptr, z_.ptr, p_.ptr, Ap_.ptr,
                                              op.dinv.ptr, scal_.ptr, partials_.ptr,
                                              counters_.ptr + 2);
  }
  VSGB_LAUNCH_CHECK();
}

void PcgEngine::launch_batch32(cudaStream_t s) {
  for (int k = 0; k < check_every_; ++k) {
    float* pin = (k & 1) ? p32b_.ptr : p32a_.ptr;
    float* pout = (k & 1) ? p32a_.ptr : p32b_.ptr;
    launch_spmv32(s, pin, pout);
    k_update32<<<vec_grid_, kThreads, 0, s>>>(n_, u32_.ptr, r32_.ptr, z32_.ptr, pout, Ap32_.ptr,
                                              dinv32_.ptr, scal_.ptr, partials_.ptr,
                                              counters_.ptr + 2);
  }
  VSGB_LAUNCH_CHECK();
}

// Runs batches until the device flags say done.  Uses a cached CUDA graph of
// one batch when enabled.
void PcgEngine::iterate(cudaStream_t s, bool fp32, PcgScalars* host) {
  const int key = fp32 ? 1 : 0;
  cudaGraphExec_t* exec = &graph_exec_[key];
  if (use_graph_ && (graph_gen_[key] != generation_ || graph_batch_[key] != check_every_ ||
                     *exec == nullptr)) {
    if (*exec) {
      cudaGraphExecDestroy(*exec);
      *exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    VSGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      if (fp32)
        launch_batch32(s);
      else
        launch_batch64(s);
      VSGB_CUDA(cudaMemcpyAsync(host, scal_.ptr, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    } catch (...) {
      cudaStreamEndCapture(s, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    VSGB_CUDA(cudaStreamEndCapture(s, &g));
    VSGB_CUDA(cudaGraphInstantiate(exec, g, 0));
    cudaGraphDestroy(g);
    graph_gen_[key] = generation_;
    graph_batch_[key] = check_every_;
    graph_host_[key] = host;
  }
  const int per_iter = fp32 ? 2 : 3;
  // The device stops at max_iters; the host bound below only guards against
  // a device that never reports completion.
  const long long max_batches = (host->max_iters + check_every_ - 1) / check_every_ + 4;
  for (long long batch = 0;; ++batch) {
    if (batch > max_batches)
      throw Error(VSGB_ERR_CUDA, "PCG device state did not report completion (flags=" +
                                     std::to_string(host->flags) + ", iter=" +
                                     std::to_string(host->iter) + ")");
    if (use_graph_ && graph_host_[key] == host) {
      VSGB_CUDA(cudaGraphLaunch(*exec, s));
    } else {
      if (fp32)
        launch_batch32(s);
      else
        launch_batch64(s);
      VSGB_CUDA(cudaMemcpyAsync(host, scal_.ptr, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
    }
    launches_ += static_cast<long long>(per_iter) * check_every_;
    VSGB_CUDA(cudaStreamSynchronize(s));
    if (host->flags & kFlagDone) break;
  }
}

// The persistent solve sweeps the same operator values every iteration; an
// access-policy window marks them persisting in L2 for the launch (the
// context's set-aside is raised to the device maximum for the launch and
// restored, and persisting lines are released, right after it).
void PcgEngine::resident_begin(cudaStream_t s, const void* hot, size_t hot_bytes) {
  if (!rev_[0]) {
    VSGB_CUDA(cudaEventCreate(&rev_[0]));
    VSGB_CUDA(cudaEventCreate(&rev_[1]));
    int dev = 0, pmax = 0, wmax = 0;
    VSGB_CUDA(cudaGetDevice(&dev));
    if (cudaDeviceGetAttribute(&pmax, cudaDevAttrMaxPersistingL2CacheSize, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&wmax, cudaDevAttrMaxAccessPolicyWindowSize, dev) != cudaSuccess) {
      cudaGetLastError();
      pmax = wmax = 0;
    }
    l2_persist_max_ = pmax > 0 ? static_cast<size_t>(pmax) : 0;
    l2_window_max_ = wmax > 0 ? static_cast<size_t>(wmax) : 0;
  }
  if (l2_persist_ && l2_persist_max_ > 0 && l2_window_max_ > 0 && hot && hot_bytes > 0) {
    VSGB_CUDA(cudaDeviceGetLimit(&l2_prev_limit_, cudaLimitPersistingL2CacheSize));
    VSGB_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, l2_persist_max_));
    const size_t bytes = hot_bytes < l2_window_max_ ? hot_bytes : l2_window_max_;
    cudaStreamAttrValue v{};
    v.accessPolicyWindow.base_ptr = const_cast<void*>(hot);
    v.accessPolicyWindow.num_bytes = bytes;
    const double ratio = static_cast<double>(l2_persist_max_) / static_cast<double>(bytes);
    v.accessPolicyWindow.hitRatio = ratio < 1.0 ? static_cast<float>(ratio) : 1.0f;
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    VSGB_CUDA(cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &v));
    l2_window_set_ = true;
  }
  VSGB_CUDA(cudaEventRecord(rev_[0], s));
}

void PcgEngine::resident_end(cudaStream_t s) {
  VSGB_CUDA(cudaEventRecord(rev_[1], s));
  VSGB_CUDA(cudaEventSynchronize(rev_[1]));
  resident_finish(s);
}

void PcgEngine::resident_finish(cudaStream_t s) {
  float ms = 0.f;
  VSGB_CUDA(cudaEventElapsedTime(&ms, rev_[0], rev_[1]));
  resident_ms_ += ms;
  if (l2_window_set_) {
    cudaStreamAttrValue v{};
    v.accessPolicyWindow.num_bytes = 0;
    VSGB_CUDA(cudaStreamSetAttribute(s, cudaStreamAttributeAccessPolicyWindow, &v));
    VSGB_CUDA(cudaCtxResetPersistingL2Cache());
    VSGB_CUDA(cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, l2_prev_limit_));
    l2_window_set_ = false;
  }
}

bool PcgEngine::block_jacobi(bool mixed, cudaStream_t s) {
  if (precond_ == 0) return false;
  if (!resident_used(mixed))
    throw Error(VSGB_ERR_INVALID,
                "3x3 block Jacobi needs the persistent solve on the 3x3 block operator");
  if (bj_gen_ != generation_) {
    const int bad = resident_block_jacobi(bsr_, res_, has32_, s);
    ++launches_;
    if (bad >= 0)
      throw Error(VSGB_ERR_SINGULAR, "GB300 PCG: the diagonal block of equations " +
                                         std::to_string(3 * bad) + ".." +
                                         std::to_string(3 * bad + 2) +
                                         " is not positive definite");
    bj_gen_ = generation_;
  }
  return true;
}

void PcgEngine::trace_reset() {
  for (double& v : phase_ns_) v = 0.0;
  for (double& v : phase_us_) v = 0.0;
  phase_its_ = 0;
}

void PcgEngine::trace_add(cudaStream_t s) {
  if (!trace_) return;
  double sums[kTracePhases], mx = 0.0;
  long long its = 0;
  resident_trace(res_, s, sums, &mx, &its);
  for (int k = 0; k < kTracePhases; ++k) phase_ns_[k] += sums[k];
  phase_ns_[kTracePhases] += mx;
  phase_its_ += its;
  const double d = phase_its_ > 0 ? 1e3 * static_cast<double>(phase_its_) : 1.0;
  for (int k = 0; k <= kTracePhases; ++k) phase_us_[k] = phase_ns_[k] / d;
  phase_us_[kTracePhases + 1] = static_cast<double>(phase_its_);
}

void PcgEngine::coarse_from_record(int count, cudaStream_t s, bool padded) {
  coarse_.gen = generation_;  // built (or found unusable) once per operator
  coarse_.valid = false;
  if (count < 8) {
    coarse_.pre_found = -1;
    return;
  }
  // the host part may have been computed from this record already (while
  // the residual ran); otherwise read the record now
  if (!(coarse_.pre_found >= 0 && coarse_.pre_K == count && coarse_.pre_gen == generation_)) {
    coarse_.pre_found = -1;
    coef_h_.resize(static_cast<size_t>(3) * count);
    VSGB_CUDA(cudaMemcpyAsync(coef_h_.data(), coef_.ptr, sizeof(double) * coef_h_.size(),
                              cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  }
  coarse_build(coarse_, hist_.ptr, padded, coef_h_, count, n_ / 3, 4,
               [&](const double* X, double* Y, int m) {
                 // the basis has at most 4 vectors here (m requested above)
                 auto fn = m <= 2 ? (m <= 1 ? k_bsr_spmm64_cols<1> : k_bsr_spmm64_cols<2>)
                                  : (m <= 3 ? k_bsr_spmm64_cols<3> : k_bsr_spmm64_cols<4>);
                 fn<<<bsr_grid_, kSpmvThreads, 0, s>>>(view_of(bsr_), bsr_.val64.ptr, X, Y, n_);
                 VSGB_LAUNCH_CHECK();
                 ++launches_;
               },
               num_sms_, s);
  launches_ += 3;  // k_ritz_combine*, k_gram, k_coarse_chol
}

void PcgEngine::ensure_diag32(cudaStream_t s) {
  if (diag_gen_ == generation_) return;
  resident_diag(res_, op_->dinv.ptr, n_, num_sms_, s);
  ++launches_;
  diag_gen_ = generation_;
}

void PcgEngine::solve_fp64(const double* d_f, double tol, int max_iters, cudaStream_t s,
                           PcgScalars* host, SolveResult& res) {
  ensure_vectors(false);
  resident_ms_ = 0.0;
  resident_iters_ = 0;
  const bool bj = block_jacobi(false, s);
  if (resident_used(false)) {
    ResidentCtl ctl;
    ctl.tol = tol;
    ctl.max_iters = max_iters;
    ctl.block_jacobi = bj;
    ctl.spin_limit = spin_limit_;
    ctl.trace = trace_;
    trace_reset();
    if (err_target_ > 0.0) {
      // error-controlled: ||e||_M <= (target / safety) ||u||_M
      ensure_diag32(s);
      ctl.err_mode = kErrRelative;
      ctl.err_rel = err_target_ / kErrSafety;
    }
    resident_begin(s, bsr_.val64.ptr, static_cast<size_t>(bsr_.steps) * 288 * sizeof(double));
    resident_solve64(bsr_, res_, d_f, u_.ptr, scal_.ptr, ctl, s, op_->dinv.ptr);
    resident_end(s);
    ++launches_;
    read_scalars(s, host, 0);
    resident_iters_ += host->iter;
    trace_add(s);
    if ((host->flags & kFlagResidentAbort) || host->abort)
      throw Error(VSGB_ERR_CUDA, "GB300 PCG: a grid barrier of the persistent solve timed out");
    if (host->flags & kFlagNonPosRz)
      throw Error(VSGB_ERR_SINGULAR,
                  "GB300 PCG: non-positive initial r*z=" + std::to_string(host->rz) +
                      " -- preconditioner is not SPD or matrix is singular");
    res.iterations = host->iter;
    res.rel = host->rel;
    res.converged = (host->flags & kFlagConverged) != 0;
    res.breakdown = (host->flags & kFlagBreakdown) != 0;
    if (err_target_ > 0.0) {
      res.err_est = (host->err2 >= 0.0 && host->total2 > 0.0)
                        ? std::sqrt(host->err2 / host->total2)
                        : (host->flags & kFlagZeroRhs ? 0.0 : -1.0);
      res.err_met = (host->flags & kFlagErrTarget) != 0;
    }
    return;
  }
  set_limits(s, 0, tol, max_iters);
  k_init64<<<vec_grid_, kThreads, 0, s>>>(n_, d_f, op_->dinv.ptr, r_.ptr, u_.ptr, z_.ptr, p_.ptr,
                                          scal_.ptr, partials_.ptr, counters_.ptr);
  VSGB_LAUNCH_CHECK();
  ++launches_;
  read_scalars(s, host, 0);
  res.iterations = 0;
  res.converged = false;
  res.rel = host->rel;
  if (host->flags & kFlagZeroRhs) {
    VSGB_CUDA(cudaMemsetAsync(u_.ptr, 0, sizeof(double) * n_, s));
    res.converged = true;
    res.rel = 0.0;
    return;
  }
  if (host->flags & kFlagNonPosRz)
    throw Error(VSGB_ERR_SINGULAR,
                "GB300 PCG: non-positive initial r*z=" + std::to_string(host->rz) +
                    " -- preconditioner is not SPD or matrix is singular");
  iterate(s, false, host);
  res.iterations = host->iter;
  res.rel = host->rel;
  res.converged = (host->flags & kFlagConverged) != 0;
  res.breakdown = (host->flags & kFlagBreakdown) != 0;
}

void PcgEngine::solve_mixed(const double* d_f, double tol, double inner_tol, int max_iters,
                            int max_solves, cudaStream_t s, PcgScalars* host, SolveResult& res) {
  ensure_vectors(true);
  resident_ms_ = 0.0;
  resident_iters_ = 0;
  const bool bj = block_jacobi(true, s);
  // Outer record (index 1) holds ||f||, the true residual and the RHS scale.
  k_outer_init<<<vec_grid_, kThreads, 0, s>>>(n_, d_f, r_.ptr, u_.ptr, scal_.ptr + 1,
                                              partials_.ptr, counters_.ptr + 3);
  VSGB_LAUNCH_CHECK();
  ++launches_;
  PcgScalars outer{};
  res.iterations = 0;
  res.inner_solves = 0;
  res.converged = false;
  const bool resident = resident_used(true);
  if (resident) {
    // u starts at 0, so the true residual starts at 1 (0 for a zero right-hand
    // side, which the first inner solve reports): no read-back needed here.
    outer.rel = 1.0;
  } else {
    read_scalars(s, &outer, 1);
    if (outer.flags & kFlagZeroRhs) {
      res.converged = true;
      res.rel = 0.0;
      return;
    }
  }
  res.rel = outer.rel;
  double prev = 0.0;
  bool have_prev = false;
  // Error-controlled refinement (persistent solve only): the first inner
  // solve stops on its residual (inner_tol), every later one on the error
  // estimate of errest.cuh; the loop ends when a step met the error target.
  const bool err_control = err_target_ > 0.0 && resident;
  if (err_control) ensure_diag32(s);
  // Coarse correction (coarse.cuh): the first inner solve on this operator
  // records its Lanczos vectors for the basis.
  const bool coarse = err_control && coarse_mode_ > 0 && use_bsr_;
  const bool record = coarse && coarse_.gen != generation_;
  if (record) coarse_.valid = false;  // a basis of an earlier operator
  // Deflated first inner solve (coarse_mode_ 2, scalar Jacobi) when an
  // earlier solve built the basis of this operator: it starts from a residual
  // the correction made orthogonal to the basis, so u = 0 is corrected first.
  // Only the first, residual-stopped solve is deflated (deflating the later
  // steps as well saved no iterations on the 265k-equation cantilever, and a
  // deflated iteration costs ~10 % more).  Not the default: a basis recorded
  // from one load can miss a low mode (one of the two near-degenerate bending
  // modes of a square section, which that load barely excited), and after a
  // deflated first step the error can sit in that mode, where the estimate
  // of the next step does not see it: 2 of 19 load cases of the 40x16x16
  // heterogeneous block ended at 1e-6 and 3e-6 for a 1e-6 target.
  const bool deflate =
      coarse && coarse_mode_ == 2 && !bj && res_.win32 && res_.defl32 && coarse_.valid;
  if (deflate) {
    if (!coarse_.defl_ready) {
      coarse_deflation_prep(coarse_, op_->dinv.ptr, num_sms_, s);
      launches_ += 2;
    }
    coarse_apply(coarse_, u_.ptr, r_.ptr, op_->dinv.ptr, scal_.ptr + 1, num_sms_, s);
    launches_ += 2;
  }
  const int hist_max = std::min(kCoarseHistMax, max_iters + 1);
  if (record) {
    hist_.reserve(static_cast<size_t>(hist_max) * 4 * (n_ / 3));
    coef_.reserve(static_cast<size_t>(3) * hist_max);
  }
  trace_reset();
  double prev_uD2 = 0.0, prev_scale = 1.0, prev_d2 = 0.0;
  for (int step = 0; step < max_solves; ++step) {
    // Inexact refinement: the correction only has to bring the true residual
    // (outer.rel, relative to ||f||) below tol, so its inner solve may stop
    // at 0.5 * tol / outer.rel instead of inner_tol when that is looser.
    double itol = inner_tol;
    if (adaptive_inner_ && outer.rel > 0.0) {
      const double want = 0.5 * tol / outer.rel;
      itol = std::max(inner_tol, std::min(0.5, want));
    }
    if (resident_used(true)) {
      // One launch: FP32 inner solve of the scaled correction and the FP64
      // accumulation u += delta / scale.
      // The true residual is launched right behind it, and both records come
      // back after one synchronisation (the residual is not used when the
      // inner solve failed).
      ResidentCtl ctl;
      ctl.tol = itol;
      ctl.max_iters = max_iters;
      ctl.block_jacobi = bj;
      ctl.spin_limit = spin_limit_;
      ctl.trace = trace_;
      if (record && step == 0) {
        ctl.hist = hist_.ptr;
        ctl.coef = coef_.ptr;
        ctl.hist_max = hist_max;
      }
      if (deflate && step == 0) {
        ctl.defl_w = coarse_.w32.ptr;
        ctl.defl_aw = coarse_.aw32.ptr;
        ctl.defl_ginv = coarse_.ginv32.ptr;
        ctl.defl_c = coarse_.cbound.ptr;
      }
      if (err_control && step > 0) {
        // refinement step: the correction's error must fall below
        // (target / safety) ||u||_D of the current iterate; the relative
        // floor keeps an FP32 solve from chasing more than it can deliver
        // (another refinement step follows instead)
        ctl.err_mode = kErrAbsolute;
        ctl.err_target = err_target_ / kErrSafety;
        ctl.err_rel = kErrRelFloor;
      }
      resident_begin(s, bsr_.val32.ptr, static_cast<size_t>(bsr_.steps) * 288 * sizeof(float));
      resident_solve32(bsr_, res_, r_.ptr, u_.ptr, scal_.ptr, scal_.ptr + 1, ctl, s,
                       op_->dinv.ptr);
      VSGB_CUDA(cudaEventRecord(rev_[1], s));
      ++launches_;
      launch_residual64(s, d_f);
      VSGB_LAUNCH_CHECK();
      ++launches_;
      // The coarse basis' host part (the Ritz pairs of the recorded
      // tridiagonal, ~0.1 ms) runs while the FP64 residual does: the record
      // is read on a copy stream that waits for the inner solve only.
      if (coarse && record && step == 0 && !coarse_.valid) {
        if (!copy_s_) VSGB_CUDA(cudaStreamCreateWithFlags(&copy_s_, cudaStreamNonBlocking));
        VSGB_CUDA(cudaStreamWaitEvent(copy_s_, rev_[1], 0));
        coef_h_.resize(static_cast<size_t>(3) * hist_max);
        VSGB_CUDA(cudaMemcpyAsync(host, scal_.ptr, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                  copy_s_));
        VSGB_CUDA(cudaMemcpyAsync(coef_h_.data(), coef_.ptr, sizeof(double) * coef_h_.size(),
                                  cudaMemcpyDeviceToHost, copy_s_));
        VSGB_CUDA(cudaStreamSynchronize(copy_s_));
        const int K = std::min(host->iter, hist_max);
        coarse_.pre_found = -1;
        if ((host->flags & kFlagConverged) && K >= 8) {
          coarse_.pre_found = coarse_host_basis(coarse_, coef_h_, K, 4);
          coarse_.pre_K = K;
          coarse_.pre_gen = generation_;
        }
      }
      // Galerkin correction in the coarse space right behind the residual
      // (the next inner solve reads the refreshed outer record on the device;
      // after a failed inner solve the iterate is not used)
      const bool corrected = coarse && coarse_.valid;
      if (corrected) {
        coarse_apply(coarse_, u_.ptr, r_.ptr, op_->dinv.ptr, scal_.ptr + 1, num_sms_, s);
        launches_ += 2;
      }
      VSGB_CUDA(cudaMemcpyAsync(host, scal_.ptr, 2 * sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                s));
      VSGB_CUDA(cudaStreamSynchronize(s));
      resident_finish(s);
      outer = host[1];
      resident_iters_ += host->iter;
      trace_add(s);
      if (step == 0 && (host->flags & kFlagZeroRhs)) {  // f = 0: u stays 0
        res.converged = true;
        res.rel = 0.0;
        return;
      }
      if ((host->flags & kFlagResidentAbort) || host->abort)
        throw Error(VSGB_ERR_CUDA, "GB300 PCG: a grid barrier of the persistent solve timed out");
      if (host->flags & kFlagNonPosRz)
        throw Error(VSGB_ERR_SINGULAR,
                    "GB300 PCG: non-positive initial r*z=" + std::to_string(host->rz) +
                        " -- preconditioner is not SPD or matrix is singular");
      ++res.inner_solves;
      res.iterations += host->iter;
      if (!(host->flags & kFlagConverged)) {
        res.breakdown = (host->flags & kFlagBreakdown) != 0;
        res.rel = host->rel;
        res.inner_failed = true;
        return;
      }
      if (coarse && !corrected && record && step == 0) {
        // the basis of this operator, from the solve just recorded
        coarse_from_record(std::min(host->iter, hist_max), s);
        if (coarse_.valid) {
          coarse_apply(coarse_, u_.ptr, r_.ptr, op_->dinv.ptr, scal_.ptr + 1, num_sms_, s);
          launches_ += 2;
          VSGB_CUDA(cudaMemcpyAsync(host + 1, scal_.ptr + 1, sizeof(PcgScalars),
                                    cudaMemcpyDeviceToHost, s));
          VSGB_CUDA(cudaStreamSynchronize(s));
          outer = host[1];
        }
      }
      res.rel = outer.rel;
      if (err_control) {
        // the step's estimate of its own error, relative to ||u||_D of the
        // iterate it corrected
        if (step > 0 && host->err2 >= 0.0 && prev_uD2 > 0.0)
          res.err_est = std::sqrt(host->err2 / prev_uD2) / prev_scale;
        // ||d||^2 of this step's correction (the first one is u itself) and
        // the bound on the error the FP32 operator left (refine_bound2)
        const double dn2 = step == 0 ? outer.uD2 : host->total2 / (prev_scale * prev_scale);
        bool done = false;
        if (step > 0) {
          const double pb2 = refine_bound2(dn2, prev_d2);
          if (res.err_est >= 0.0 && outer.uD2 > 0.0) res.err_est += std::sqrt(pb2 / outer.uD2);
          const double goal = err_target_ / kErrSafety;
          done = (host->flags & kFlagErrTarget) && pb2 <= goal * goal * outer.uD2;
        }
        prev_d2 = dn2;
        prev_uD2 = outer.uD2;
        prev_scale = outer.scale;
        if (done) {
          res.converged = true;
          res.err_met = true;
          break;
        }
        continue;  // first solve, the relative floor only, or the FP32 operator's share
      }
      if (outer.rel <= tol) {
        res.converged = true;
        break;
      }
      if (have_prev && outer.rel >= prev * 0.9) {
        res.stalled = true;
        break;
      }
      prev = outer.rel;
      have_prev = true;
      continue;
    }
    set_limits(s, 0, itol, max_iters);
    k_init32<<<vec_grid_, kThreads, 0, s>>>(n_, r_.ptr, 0.0, dinv32_.ptr, r32_.ptr, u32_.ptr,
                                            z32_.ptr, p32a_.ptr, scal_.ptr, scal_.ptr + 1,
                                            partials_.ptr, counters_.ptr);
    VSGB_LAUNCH_CHECK();
    ++launches_;
    read_scalars(s, host, 0);
    if (host->flags & kFlagNonPosRz)
      throw Error(VSGB_ERR_SINGULAR,
                  "GB300 PCG: non-positive initial r*z=" + std::to_string(host->rz) +
                      " -- preconditioner is not SPD or matrix is singular");
    if (!(host->flags & kFlagDone)) iterate(s, true, host);
    ++res.inner_solves;
    res.iterations += host->iter;
    if (!(host->flags & kFlagConverged)) {
      res.breakdown = (host->flags & kFlagBreakdown) != 0;
      res.rel = host->rel;
      res.inner_failed = true;
      return;
    }
    k_accumulate<<<vec_grid_, kThreads, 0, s>>>(n_, u_.ptr, u32_.ptr, scal_.ptr + 1);
    launch_residual64(s, d_f);
    VSGB_LAUNCH_CHECK();
    launches_ += 2;
    read_scalars(s, &outer, 1);
    res.rel = outer.rel;
    if (outer.rel <= tol) {
      res.converged = true;
      break;
    }
    if (have_prev && outer.rel >= prev * 0.9) {
      res.stalled = true;
      break;
    }
    prev = outer.rel;
    have_prev = true;
  }
}

void PcgEngine::time_spmv(int precision, int reps, cudaStream_t s, double* avg_ms) {
  ensure_vectors(precision == VSGB_MIXED);
  const AssembledCsr& op = *op_;
  // Done flag cleared so the kernel does full work; scalars are scratch.
  PcgScalars h{};
  h.rz = 1.0;
  h.beta = 0.5;
  h.tol = 0.0;
  h.max_iters = 1 << 30;
  VSGB_CUDA(cudaMemcpyAsync(scal_.ptr, &h, sizeof(PcgScalars), cudaMemcpyHostToDevice, s));
  // Nonzero inputs: p = 1 gives p.Ap = 1^T K 1 > 0 for an SPD K, so the
  // breakdown flag never stops the timed launches.
  k_fill<double><<<num_sms_ * 4, kThreads, 0, s>>>(n_, p_.ptr, 1.0);
  if (precision == VSGB_MIXED) {
    k_fill<float><<<num_sms_ * 4, kThreads, 0, s>>>(n_, z32_.ptr, 1.0f);
    k_fill<float><<<num_sms_ * 4, kThreads, 0, s>>>(n_, p32a_.ptr, 0.0f);
  }
  VSGB_LAUNCH_CHECK();
  (void)op;
  cudaEvent_t e0, e1;
  VSGB_CUDA(cudaEventCreate(&e0));
  VSGB_CUDA(cudaEventCreate(&e1));
  auto one = [&]() {
    if (precision == VSGB_MIXED)
      launch_spmv32(s, p32a_.ptr, p32b_.ptr);
    else
      launch_spmv64(s, p_.ptr, Ap_.ptr);
  };
  for (int w = 0; w < 3; ++w) one();
  VSGB_CUDA(cudaStreamSynchronize(s));
  VSGB_CUDA(cudaEventRecord(e0, s));
  for (int k = 0; k < reps; ++k) one();
  VSGB_CUDA(cudaEventRecord(e1, s));
  VSGB_LAUNCH_CHECK();
  VSGB_CUDA(cudaEventSynchronize(e1));
  float ms = 0.f;
  VSGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  launches_ += reps + 3;
  *avg_ms = static_cast<double>(ms) / reps;
}

double PcgEngine::spmv_bytes(int precision) const {
  if (use_bsr_) return bsr_bytes(bsr_, precision);
  // Algorithmic bytes of one full-storage CSR SpMV: values + column indices +
  // row pointers + x read once + y written once.
  const double nnz = static_cast<double>(op_->nnz), n = static_cast<double>(n_);
  if (precision == VSGB_MIXED) return 8.0 * nnz + 4.0 * (n + 1) + 8.0 * n;
  return 12.0 * nnz + 4.0 * (n + 1) + 16.0 * n;
}

PcgEngine::~PcgEngine() {
  for (auto& g : graph_exec_)
    if (g) cudaGraphExecDestroy(g);
  for (auto& e : rev_)
    if (e) cudaEventDestroy(e);
  if (copy_s_) cudaStreamDestroy(copy_s_);
  destroy_multi(multi_);
}

// ── Allocation-free FP64 PCG (vsgb_pcg_solve_noalloc) ─────────────────────
//
// For callers that must not allocate GPU memory: code that runs inside
// another framework's memory pool, or a latency-critical loop where a
// cudaMalloc (which can synchronise the device and can fail under memory
// pressure) is not allowed.  The solver's scratch — Jacobi inverse diagonal,
// r, z, p, Ap, the per-block reduction partials, the grid-reduction counters
// and the PCG scalar record — lives in one file-scope __device__ array of
// kNoAllocScratchBytes, held by every GPU that loads the library until the
// process exits.  Systems are limited to VSGB_NOALLOC_MAX_N equations.

namespace {

constexpr int kNoAllocMaxGrid = 4096;  // blocks of any launch below
constexpr size_t kNoAllocVecBytes = sizeof(double) * VSGB_NOALLOC_MAX_N;
constexpr size_t kNoAllocPartialsBytes = sizeof(double) * 2 * kNoAllocMaxGrid;
constexpr size_t kNoAllocCounterBytes = 256;
constexpr size_t kNoAllocScalarsBytes = 256;
constexpr size_t kNoAllocErrorBytes = 256;
constexpr size_t kNoAllocScratchBytes = 5 * kNoAllocVecBytes + kNoAllocPartialsBytes +
                                        kNoAllocCounterBytes + kNoAllocScalarsBytes +
                                        kNoAllocErrorBytes;
static_assert(sizeof(PcgScalars) <= kNoAllocScalarsBytes, "scalar record");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch per device (a host-side copy of the
// symbol is only a stand-in, never a device address).  The address belongs to
// the device's primary context as it was when the first call resolved it: a
// cudaDeviceReset (or anything else that destroys that context) leaves the
// cached address stale, so after one the library has to be loaded anew
// (a new process) before this entry point is called again on that device.
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

struct NoAllocError {
  int code;  // 0 ok, 2 column out of range, 4 zero diagonal, 5 missing diagonal, 6 bad row_ptr
  int index;
};

// Row pointer, column range check and Jacobi inverse diagonal of a
// full-storage CSR (first entry with col == row, as build_jacobi_diagonal).
// Row r reads only rp[r], rp[r+1] (inside the caller's n+1 entries) until its
// extent is known to lie in [0, nnz): a bad row pointer is reported before any
// column or value is read through it.
__global__ void k_noalloc_diag(int n, int nnz, const int* __restrict__ rp,
                               const int* __restrict__ ci, const double* __restrict__ v,
                               double* __restrict__ dinv, NoAllocError* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int b = rp[r], e = rp[r + 1];
  if (b < 0 || b > e || e > nnz || (r == 0 && b != 0) || (r == n - 1 && e != nnz)) {
    if (atomicCAS(&err->code, 0, 6) == 0) err->index = r;
    dinv[r] = 0.0;
    return;
  }
  bool found = false;
  for (int k = b; k < e; ++k) {
    const int c = ci[k];
    if (c < 0 || c >= n) {
      if (atomicCAS(&err->code, 0, 2) == 0) err->index = r;
      dinv[r] = 0.0;
      return;
    }
    if (!found && c == r) {
      found = true;
      if (v[k] == 0.0) {
        if (atomicCAS(&err->code, 0, 4) == 0) err->index = r;
        dinv[r] = 0.0;
      } else {
        dinv[r] = 1.0 / v[k];
      }
    }
  }
  if (!found) {
    if (atomicCAS(&err->code, 0, 5) == 0) err->index = r;
    dinv[r] = 0.0;
  }
}

void noalloc_err(char* err, size_t len, const std::string& m) {
  if (err && len > 0) std::snprintf(err, len, "%s", m.c_str());
}

}  // namespace

}  // namespace vsgb

extern "C" int vsgb_pcg_solve_noalloc(int n, int nnz, const int* d_row_ptr, const int* d_col_ind,
                                      const double* d_values, const double* d_F, double* d_u,
                                      double tol, int max_iters, void* stream,
                                      int* iterations_out, double* rel_residual_out, char* err,
                                      size_t errlen) {
  using namespace vsgb;
  if (iterations_out) *iterations_out = 0;
  if (rel_residual_out) *rel_residual_out = 0.0;
  if (n <= 0) {
    noalloc_err(err, errlen, "CUDA PCG: stiffness matrix is empty -- no free DOFs");
    return VSGB_ERR_INVALID;
  }
  if (n > VSGB_NOALLOC_MAX_N) {
    noalloc_err(err, errlen, "vsgb_pcg_solve_noalloc: n = " + std::to_string(n) +
                                 " exceeds the allocation-free limit of " +
                                 std::to_string(VSGB_NOALLOC_MAX_N) + " equations");
    return VSGB_ERR_LIMIT;
  }
  if (nnz < 0 || !d_row_ptr || (nnz > 0 && (!d_col_ind || !d_values)) || !d_F || !d_u) {
    noalloc_err(err, errlen, "vsgb_pcg_solve_noalloc: invalid argument");
    return VSGB_ERR_INVALID;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0;
  int num_sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices ||
      cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    noalloc_err(err, errlen, "vsgb_pcg_solve_noalloc: no usable current device");
    return VSGB_ERR_NO_DEVICE;
  }
  unsigned char* base = nullptr;
  {
    // First call on a device resolves the scratch address (do it before any
    // stream capture on that device).
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) {
        noalloc_err(err, errlen, std::string("cudaGetSymbolAddress failed: ") +
                                     cudaGetErrorString(e));
        return VSGB_ERR_CUDA;
      }
      g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    base = g_noalloc_ptr[dev];
  }
  double* dinv = reinterpret_cast<double*>(base);
  double* r = reinterpret_cast<double*>(base + kNoAllocVecBytes);
  double* z = reinterpret_cast<double*>(base + 2 * kNoAllocVecBytes);
  double* p = reinterpret_cast<double*>(base + 3 * kNoAllocVecBytes);
  double* Ap = reinterpret_cast<double*>(base + 4 * kNoAllocVecBytes);
  unsigned char* tail = base + 5 * kNoAllocVecBytes;
  double* partials = reinterpret_cast<double*>(tail);
  unsigned* counters = reinterpret_cast<unsigned*>(tail + kNoAllocPartialsBytes);
  PcgScalars* S = reinterpret_cast<PcgScalars*>(tail + kNoAllocPartialsBytes + kNoAllocCounterBytes);
  NoAllocError* derr = reinterpret_cast<NoAllocError*>(tail + kNoAllocPartialsBytes +
                                                        kNoAllocCounterBytes + kNoAllocScalarsBytes);
  const int vec_grid = grid_for(n, kThreads, num_sms * 4);
  const int spmv_grid = grid_for(static_cast<long long>(n) * kLpr, kSpmvThreads, num_sms * 8);
  if (vec_grid > kNoAllocMaxGrid || spmv_grid > kNoAllocMaxGrid) {
    noalloc_err(err, errlen, "vsgb_pcg_solve_noalloc: launch grid exceeds the scratch layout");
    return VSGB_ERR_LIMIT;
  }
  auto cuda_fail = [&](cudaError_t e, const char* what) {
    noalloc_err(err, errlen, std::string("CUDA error in ") + what + ": " + cudaGetErrorString(e));
    return VSGB_ERR_CUDA;
  };
  cudaError_t e;
  // The array keeps the previous call's contents: counters, error record and
  // the scalar limits are reset here; vectors are fully rewritten by k_init64.
  if ((e = cudaMemsetAsync(counters, 0, kNoAllocCounterBytes, s)) != cudaSuccess)
    return cuda_fail(e, "reset counters");
  if ((e = cudaMemsetAsync(derr, 0, sizeof(NoAllocError), s)) != cudaSuccess)
    return cuda_fail(e, "reset error record");
  PcgScalars h{};
  h.tol = tol > 0.0 ? tol : 1e-8;
  h.max_iters = max_iters > 0 ? max_iters : 10000;
  if ((e = cudaMemcpyAsync(S, &h, sizeof(PcgScalars), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    return cuda_fail(e, "write limits");
  k_noalloc_diag<<<grid_for(n, kThreads, 1 << 30), kThreads, 0, s>>>(n, nnz, d_row_ptr,
                                                                      d_col_ind, d_values, dinv,
                                                                      derr);
  NoAllocError herr{};
  if ((e = cudaMemcpyAsync(&herr, derr, sizeof(herr), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(e, "diagonal check");
  if (herr.code == 2) {
    noalloc_err(err, errlen, "column index out of range in row " + std::to_string(herr.index));
    return VSGB_ERR_INVALID;
  }
  if (herr.code == 6) {
    noalloc_err(err, errlen, "row_ptr is not a valid CSR row pointer (0 = row_ptr[0] <= ... <= "
                             "row_ptr[n] = nnz) at row " + std::to_string(herr.index));
    return VSGB_ERR_INVALID;
  }
  if (herr.code == 4 || herr.code == 5) {
    noalloc_err(err, errlen, std::string("CUDA PCG: ") + (herr.code == 4 ? "zero" : "missing") +
                                 " diagonal at row " + std::to_string(herr.index) +
                                 " -- matrix is singular. Check boundary conditions.");
    return VSGB_ERR_SINGULAR;
  }
  k_init64<<<vec_grid, kThreads, 0, s>>>(n, d_F, dinv, r, d_u, z, p, S, partials, counters);
  if ((e = cudaMemcpyAsync(&h, S, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(e, "PCG init");
  if (h.flags & kFlagZeroRhs) return VSGB_OK;  // u = 0, 0 iterations
  if (h.flags & kFlagNonPosRz) {
    noalloc_err(err, errlen, "CUDA PCG: non-positive initial r*z=" + std::to_string(h.rz) +
                                 " -- preconditioner is not SPD or matrix is singular");
    return VSGB_ERR_SINGULAR;
  }
  const int check_every = 16;
  const long long max_batches = (h.max_iters + check_every - 1) / check_every + 4;
  for (long long batch = 0; batch <= max_batches; ++batch) {
    for (int k = 0; k < check_every; ++k) {
      k_search64<<<vec_grid, kThreads, 0, s>>>(n, z, p, S);
      k_spmv64<<<spmv_grid, kSpmvThreads, 0, s>>>(n, d_row_ptr, d_col_ind, d_values, p, Ap, S,
                                                  partials, counters + 1);
      k_update64<<<vec_grid, kThreads, 0, s>>>(n, d_u, r, z, p, Ap, dinv, S, partials,
                                               counters + 2);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "PCG launch");
    if ((e = cudaMemcpyAsync(&h, S, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return cuda_fail(e, "PCG iteration");
    if (h.flags & kFlagDone) break;
  }
  // A non-positive p*Ap stops the solve as the reference does
  // (cuda_pcg_backend_impl.hpp:1932-1939): the iteration count reported is
  // max_iters and the did-not-converge error follows, here with the p*Ap
  // value and the iteration it was met at appended.
  const bool breakdown = (h.flags & kFlagBreakdown) != 0;
  if (iterations_out) *iterations_out = breakdown ? h.max_iters : h.iter;
  if (rel_residual_out) *rel_residual_out = h.rel;
  if (breakdown || !(h.flags & kFlagConverged) || h.iter >= h.max_iters) {
    std::string m = "CUDA PCG: did not converge after " + std::to_string(h.max_iters) +
                    " iterations (relative residual " + std::to_string(h.rel) + " > tolerance " +
                    std::to_string(h.tol) +
                    "). Consider increasing max iterations or using a direct solver.";
    if (breakdown)
      m += " (non-positive p*Ap=" + std::to_string(h.pAp) + " at iteration " +
           std::to_string(h.iter) + ")";
    noalloc_err(err, errlen, m);
    return VSGB_ERR_NOT_CONVERGED;
  }
  return VSGB_OK;
}
