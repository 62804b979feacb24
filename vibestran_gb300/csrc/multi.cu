// vibestran_gb300/csrc/multi.cu — batched Jacobi-PCG over up to 16 load cases.
//
// The reference solves subcases one after another, each with its own
// cuda-pcg call (linear_static.cpp:212-275; cuda_pcg_backend_impl.hpp:1688-1999).
// Here the right-hand sides of one model share each sweep of the matrix:
// vectors are stored as panels [n][16] (the 16 load cases of a DOF are
// contiguous), so one 3x3 block of K meets 3 x 16 values of the panel and the
// SpMM does 144 FMAs per 9 matrix values — the matrix stream, which bounds a
// single-RHS iteration, is amortised 16 ways.  Each column keeps its own PCG
// scalars (alpha, beta, rz, stopping test on the unpreconditioned residual
// sqrt(r.r)/||b|| < tol), so every column follows the reference recurrence;
// a finished column gets alpha = 0 and no longer moves.  Mixed precision runs
// FP32 inner solves of the scaled residual and refines each column in FP64
// on the GPU (cuda_pcg_backend_impl.hpp:2134-2262 refines on the host).
//
// Rooflines (config of 504 300 equations, 4.36 M stored 3x3 blocks):
//   FP32 SpMM  — matrix 4.36M x (36 + 4) B streamed once, the panel gathered
//                through L1/L2: HBM-bound, ~1.26 GFLOP at ~2.7 flop/B.
//   FP64 SpMM  — 628 M DFMA per sweep: FP64-pipe bound on GB300.
//   vector kernels — HBM streams of 16-wide panels.
// All reductions are fixed-order (per-lane -> warp -> block -> block-ordered
// grid sum), so a batched solve is bitwise reproducible.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "coarse.cuh"
#include "errest.cuh"
#include "multi.cuh"
#include "pcg.cuh"

namespace vsgb {

namespace {

constexpr int kMT = 256;   // threads per block of the SpMM / transpose kernels
constexpr int kVT = 1024;  // threads per block of the panel vector kernels (one block per SM)

struct MView {
  int nb, nslices;
  const int* __restrict__ slice_ptr;
  const int* __restrict__ cols;
};

// Lanczos record of one column of the FP32 batched solve (coarse.cuh): z_k
// of column col for k < max (n floats each) and alpha_k, beta_k, r_k.z_k.
struct MultiRecord {
  float* hist = nullptr;
  double* coef = nullptr;
  int col = -1, max = 0;
};

// Fixed-order grid reduction of per-column sums.  acc[Q][R] holds this
// thread's sums of quantity q for columns cb..cb+R-1, where cb is the same
// for every lane with the same (lane & 3) in a warp.  Returns true in the
// block that finished last, with the Q x 16 totals in s_tot[q * 16 + k].
// BT is the block size; s_red holds BT doubles.
template <int Q, int R, int BT>
__device__ __forceinline__ bool mcol_sum_last(double (&acc)[Q][R], int cb, double* partials,
                                              unsigned* counter, double* s_red /* BT */,
                                              double* s_tot /* Q * kP */) {
  constexpr int QM = Q * kP;
  constexpr int NW = BT / 32;
  static_assert(QM <= BT && NW * QM <= BT, "reduction shape");
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      double v = acc[q][r];
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 8);
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      acc[q][r] = v;
    }
  for (int t = threadIdx.x; t < NW * QM; t += BT) s_red[t] = 0.0;
  __syncthreads();
  if (lane < 4)
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int r = 0; r < R; ++r) s_red[(wid * Q + q) * kP + cb + r] = acc[q][r];
  __syncthreads();
  const int nblk = gridDim.x * gridDim.y;
  const int b = blockIdx.y * gridDim.x + blockIdx.x;
  // partials are column-major (column t at partials + t * nblk) so that the
  // last block reads each column with coalesced loads
  if (threadIdx.x < QM) {
    double s = 0.0;
    for (int w = 0; w < NW; ++w) s += s_red[w * QM + threadIdx.x];
    partials[static_cast<size_t>(threadIdx.x) * nblk + b] = s;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == static_cast<unsigned>(nblk - 1));
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  // one warp per column: lane l takes blocks l, l+32, ...; each round issues
  // 8 independent loads before adding them in block order, then a butterfly
  for (int col = wid; col < QM; col += NW) {
    const double* pc = partials + static_cast<size_t>(col) * nblk;
    double s = 0.0;
    for (int b0 = lane; b0 < nblk; b0 += 256) {
      double v[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) v[m] = (b0 + 32 * m < nblk) ? __ldcg(pc + b0 + 32 * m) : 0.0;
#pragma unroll
      for (int m = 0; m < 8; ++m) s += v[m];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) s_tot[col] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// The FP32 solve's form of mcol_sum_last: acc holds FP32 sums, the warp and
// block sums stay in FP32 and the block partials are stored as FP32; the last
// block adds each column's partials as a double-float pair (Knuth's TwoSum,
// ~48 significant bits) and converts once per column.  On GB300 a warp-wide
// FP64 instruction costs the SM ~16 cycles whatever its active lanes, so the
// FP64 form spent ~260 FP64 warp instructions per block on its shuffle sums
// and conversions and ~1 400 in the last block (32 columns of one partial per
// block, 1 216 blocks at 8 per SM), all at the end of the kernel, where the
// blocks finish together.
// Same fixed order everywhere: reproducible bit for bit.
__device__ __forceinline__ void two_sum_acc(float& s, float& e, float x) {
  const float t = __fadd_rn(s, x);
  const float bp = __fsub_rn(t, s);
  const float er = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
  s = t;
  e = __fadd_rn(e, er);
}

template <int Q, int R, int BT>
__device__ __forceinline__ bool mcol_sum_last32(float (&acc)[Q][R], int cb, double* partials,
                                                unsigned* counter, float* s_red /* BT */,
                                                double* s_tot /* Q * kP */) {
  constexpr int QM = Q * kP;
  constexpr int NW = BT / 32;
  static_assert(2 * QM <= BT && NW * QM <= BT, "reduction shape");
  __shared__ bool s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < Q; ++q)
#pragma unroll
    for (int r = 0; r < R; ++r) {
      float v = acc[q][r];
      v += __shfl_xor_sync(0xffffffffu, v, 4);
      v += __shfl_xor_sync(0xffffffffu, v, 8);
      v += __shfl_xor_sync(0xffffffffu, v, 16);
      acc[q][r] = v;
    }
  for (int t = threadIdx.x; t < NW * QM; t += BT) s_red[t] = 0.f;
  __syncthreads();
  if (lane < 4)
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
      for (int r = 0; r < R; ++r) s_red[(wid * Q + q) * kP + cb + r] = acc[q][r];
  __syncthreads();
  const int nblk = gridDim.x * gridDim.y;
  const int b = blockIdx.y * gridDim.x + blockIdx.x;
  float* pf = reinterpret_cast<float*>(partials);  // column t at pf + t * nblk
  if (threadIdx.x < QM) {
    float sum = 0.f;
    for (int w = 0; w < NW; ++w) sum += s_red[w * QM + threadIdx.x];
    pf[static_cast<size_t>(threadIdx.x) * nblk + b] = sum;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(counter, 1u) == static_cast<unsigned>(nblk - 1));
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  for (int col = wid; col < QM; col += NW) {
    const float* pc = pf + static_cast<size_t>(col) * nblk;
    float sum = 0.f, err = 0.f;
    for (int b0 = lane; b0 < nblk; b0 += 256) {
      float v[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) v[m] = (b0 + 32 * m < nblk) ? __ldcg(pc + b0 + 32 * m) : 0.f;
#pragma unroll
      for (int m = 0; m < 8; ++m) two_sum_acc(sum, err, v[m]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float so = __shfl_xor_sync(0xffffffffu, sum, o);
      const float eo = __shfl_xor_sync(0xffffffffu, err, o);
      two_sum_acc(sum, err, so);
      err = __fadd_rn(err, eo);
    }
    if (lane == 0) {
      s_red[col] = sum;
      s_red[QM + col] = err;
    }
  }
  __syncthreads();
  if (threadIdx.x < QM)
    s_tot[threadIdx.x] = static_cast<double>(s_red[threadIdx.x]) +
                         static_cast<double>(s_red[QM + threadIdx.x]);
  __syncthreads();
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// mcol_sum_last in the accumulators' precision
template <int Q, int R, int BT, typename A>
__device__ __forceinline__ bool mcol_sum(A (&acc)[Q][R], int cb, double* partials,
                                         unsigned* counter, double* s_red /* BT */,
                                         double* s_tot /* Q * kP */) {
  if constexpr (sizeof(A) == 4) {
    return mcol_sum_last32<Q, R, BT>(acc, cb, partials, counter, reinterpret_cast<float*>(s_red),
                                     s_tot);
  } else {
    return mcol_sum_last<Q, R, BT>(acc, cb, partials, counter, s_red, s_tot);
  }
}

__device__ __forceinline__ void all_done(MultiState* S) {
  int all = 1;
  for (int k = 0; k < kP; ++k) all &= (S->flags[k] & kFlagDone) ? 1 : 0;
  S->done = all;
}

// ── panel <-> column-major transposes (32 DOFs per block) ─────────────────

__global__ void __launch_bounds__(kMT)
k_pack(int n, int ncols, const double* __restrict__ F, double* __restrict__ panel) {
  __shared__ double tile[kP][33];
  const int i0 = blockIdx.x * 32;
  for (int t = threadIdx.x; t < kP * 32; t += kMT) {
    const int k = t >> 5, i = t & 31;
    tile[k][i] = (k < ncols && i0 + i < n) ? F[static_cast<size_t>(k) * n + i0 + i] : 0.0;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kP * 32; t += kMT) {
    const int i = t >> 4, k = t & 15;
    if (i0 + i < n) panel[static_cast<size_t>(i0 + i) * kP + k] = tile[k][i];
  }
}

__global__ void __launch_bounds__(kMT)
k_unpack(int n, int ncols, const double* __restrict__ panel, double* __restrict__ U) {
  __shared__ double tile[kP][33];
  const int i0 = blockIdx.x * 32;
  for (int t = threadIdx.x; t < kP * 32; t += kMT) {
    const int i = t >> 4, k = t & 15;
    tile[k][i] = (i0 + i < n) ? panel[static_cast<size_t>(i0 + i) * kP + k] : 0.0;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kP * 32; t += kMT) {
    const int k = t >> 5, i = t & 31;
    if (k < ncols && i0 + i < n) U[static_cast<size_t>(k) * n + i0 + i] = tile[k][i];
  }
}

// ── 4-wide panel chunk access ─────────────────────────────────────────────

__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 a = *reinterpret_cast<const float4*>(p);
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }

// RN consecutive panel values (RN = 2 or 4, 8/16-byte aligned).
template <int RN, typename T>
__device__ __forceinline__ void ldn(const T* p, T (&v)[RN]) {
  if constexpr (RN == 4) {
    ld4(p, v);
  } else if constexpr (sizeof(T) == 8) {
    const double2 a = *reinterpret_cast<const double2*>(p);
    v[0] = a.x; v[1] = a.y;
  } else {
    const float2 a = *reinterpret_cast<const float2*>(p);
    v[0] = a.x; v[1] = a.y;
  }
}
template <int RN, typename T>
__device__ __forceinline__ void stn(T* p, const T (&v)[RN]) {
  if constexpr (RN == 4) {
    st4(p, v);
  } else if constexpr (sizeof(T) == 8) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  } else {
    *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
  }
}

// ── SpMM on the 3x3 sliced-ELL operator ───────────────────────────────────
// One warp per slice of 8 block rows; the 4 lanes of block row r = lane/4
// share every block of that row, and lane q = lane%4 owns columns
// g0 + q*G/4 .. +G/4-1 of the 3 output rows.  Per step the warp loads the
// step's 32 blocks coalesced (lane = slot, L1-bypassing), then in 4 sub-steps
// broadcasts block u of each row over its quad and every lane gathers its
// G/4 panel columns of the block column: the quad reads one contiguous
// 64-byte run per block row of x, so a gather touches 8 cache lines for 8
// blocks instead of one line per 16 bytes.  Sums run in slot order, so the
// result is reproducible.  The next step's blocks are loaded before the
// current step is consumed.
template <typename T, int G>
__device__ __forceinline__ void mspmm_slice(const MView& B, const T* __restrict__ vals,
                                            const T* __restrict__ x, int sl, int lane, int g0,
                                            T (&out)[3][G / 4]) {
  constexpr int RN = G / 4;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int r = 0; r < RN; ++r) out[i][r] = T(0);
  const int base = B.slice_ptr[sl], steps = B.slice_ptr[sl + 1] - base;
  const int* cp = B.cols + static_cast<size_t>(base) * 32 + lane;
  const T* vp = vals + static_cast<size_t>(base) * 288 + lane;
  const T* xq = x + g0 + RN * (lane & 3);
  const int quad = lane & ~3;
  // FP32: difference form (the diagonal slot holds the block-row sum), so
  // non-diagonal blocks multiply x_J - x_I; xi holds the row's own panel rows.
  constexpr bool kDiff = sizeof(T) == 4;
  const int Rrow = 8 * sl + (lane >> 2);
  T xi[3][RN];
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int r = 0; r < RN; ++r) xi[j][r] = T(0);
  if (kDiff && Rrow < B.nb) {
#pragma unroll
    for (int j = 0; j < 3; ++j) ldn<RN>(xq + static_cast<size_t>(Rrow) * (3 * kP) + j * kP, xi[j]);
  }
  int cn = 0;
  T an[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) an[k] = T(0);
  if (steps > 0) {
    cn = __ldcg(cp);
#pragma unroll
    for (int k = 0; k < 9; ++k) an[k] = __ldcg(vp + 32 * k);
  }
  for (int t = 0; t < steps; ++t) {
    const int cown = cn;
    T aown[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) aown[k] = an[k];
    if (t + 1 < steps) {
      cn = __ldcg(cp + 32 * (t + 1));
#pragma unroll
      for (int k = 0; k < 9; ++k) an[k] = __ldcg(vp + 288 * (t + 1) + 32 * k);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int src = quad | u;
      const int c = __shfl_sync(0xffffffffu, cown, src);
      T a[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) a[k] = __shfl_sync(0xffffffffu, aown[k], src);
      const T* xc = xq + static_cast<size_t>(c) * (3 * kP);
      const T m = kDiff && c != Rrow ? T(1) : T(0);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T xv[RN];
        ldn<RN>(xc + j * kP, xv);
        if (kDiff) {
#pragma unroll
          for (int r = 0; r < RN; ++r) xv[r] = fmaT(-m, xi[j][r], xv[r]);
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int r = 0; r < RN; ++r) out[i][r] = fmaT(a[3 * i + j], xv[r], out[i][r]);
      }
    }
  }
}

// Ap = K p for the columns of block row group blockIdx.y; p.Ap per column,
// then alpha = rz / p.Ap (breakdown when p.Ap <= 0, as cuda_pcg_backend_impl.hpp:688-694).
template <typename T, int G>
__global__ void __launch_bounds__(kMT, sizeof(T) == 4 ? 3 : 1)
k_mspmm(MView B, const T* __restrict__ vals, const T* __restrict__ p, T* __restrict__ Ap,
        const float* __restrict__ diag32, MultiState* S, ErrEst* est, double* partials,
        unsigned* counter) {
  if (S->done) return;
  __shared__ double s_red[kMT];
  __shared__ double s_tot[2 * kP];
  constexpr int RN = G / 4;
  const int lane = threadIdx.x & 31;
  const int g0 = blockIdx.y * G, cb = g0 + (lane & 3) * RN;
  constexpr int wpb = kMT / 32;
  const bool err_on = S->err_mode != kErrOff;
  T pap[RN];
  float pmp[RN];
#pragma unroll
  for (int r = 0; r < RN; ++r) {
    pap[r] = T(0);
    pmp[r] = 0.f;
  }
  // odd iterations walk the slices from the end: the operator lines read last
  // (the ones still in L2) are read first
  const bool rev = (S->iter & 1) != 0;
  for (int sq = blockIdx.x * wpb + (threadIdx.x >> 5); sq < B.nslices; sq += gridDim.x * wpb) {
    const int sl = rev ? B.nslices - 1 - sq : sq;
    T out[3][RN];
    mspmm_slice<T, G>(B, vals, p, sl, lane, g0, out);
    const int R = sl * 8 + (lane >> 2);
    if (R < B.nb) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const size_t o = static_cast<size_t>(3 * R + i) * kP + cb;
        T pv[RN];
        ldn<RN>(p + o, pv);
        stn<RN>(Ap + o, out[i]);
#pragma unroll
        for (int r = 0; r < RN; ++r) pap[r] = fmaT(pv[r], out[i][r], pap[r]);
        if (err_on) {
          // p.Dp per column for the error estimate (FP32 suffices)
          const float d = __ldg(diag32 + 3 * R + i);
#pragma unroll
          for (int r = 0; r < RN; ++r) {
            const float pf = static_cast<float>(pv[r]);
            pmp[r] = fmaf(pf * pf, d, pmp[r]);
          }
        }
      }
    }
  }
  T a[2][RN];
#pragma unroll
  for (int r = 0; r < RN; ++r) {
    a[0][r] = pap[r];
    a[1][r] = static_cast<T>(pmp[r]);
  }
  if (mcol_sum<2, RN, kMT>(a, cb, partials, counter, s_red, s_tot)) {
    if (threadIdx.x < kP) {
      const int k = threadIdx.x;
      int f = S->flags[k];
      if (!(f & kFlagDone)) {
        const double pAp = s_tot[k];
        S->pAp[k] = pAp;
        if (!(pAp > 0.0)) {
          S->alpha[k] = 0.0;
          f |= kFlagDone | kFlagBreakdown;
          S->iters[k] = S->iter;
        } else {
          S->alpha[k] = S->rz[k] / pAp;
          if (err_on) err_record(est[k], S->rz[k] * S->alpha[k], s_tot[kP + k] / pAp);
        }
        S->flags[k] = f;
      } else {
        S->alpha[k] = 0.0;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) all_done(S);
  }
}

// r = f - K u (FP64) and ||r|| per column; updates the refinement record:
// convergence (rel <= tol), stagnation (rel >= 0.9 * previous) and the scale
// 1/||r|| of the next inner right-hand side.
// err_stop replaces the residual test by the error control of the
// refinement (err_goal = target / safety, relative): 2 after the first inner
// solve (records ||d_0||_D = ||u||_D), 1 after a refinement step, when a
// column is done if its inner solve met the error target and the
// FP32-operator part of the error is below the goal too (refine_bound).
template <int G>
__global__ void __launch_bounds__(kMT)
k_mresidual(MView B, const double* __restrict__ vals, const double* __restrict__ u,
            const double* __restrict__ f, const double* __restrict__ dinv,
            double* __restrict__ r, MultiOuter* O, const MultiState* S, const ErrEst* est,
            int err_stop, double err_goal, double tol, double* partials, unsigned* counter) {
  __shared__ double s_red[kMT];
  __shared__ double s_tot[2 * kP];
  constexpr int RN = G / 4;
  const int lane = threadIdx.x & 31;
  const int g0 = blockIdx.y * G, cb = g0 + (lane & 3) * RN;
  constexpr int wpb = kMT / 32;
  double a[2][RN];
#pragma unroll
  for (int q = 0; q < RN; ++q) a[0][q] = a[1][q] = 0.0;
  for (int sl = blockIdx.x * wpb + (threadIdx.x >> 5); sl < B.nslices; sl += gridDim.x * wpb) {
    double out[3][RN];
    mspmm_slice<double, G>(B, vals, u, sl, lane, g0, out);
    const int R = sl * 8 + (lane >> 2);
    if (R < B.nb) {
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const size_t o = static_cast<size_t>(3 * R + i) * kP + cb;
        double fv[RN], rv[RN], uv[RN];
        ldn<RN>(f + o, fv);
        ldn<RN>(u + o, uv);
        const double dg = 1.0 / dinv[3 * R + i];
#pragma unroll
        for (int q = 0; q < RN; ++q) {
          rv[q] = fv[q] - out[i][q];
          a[0][q] = fma(rv[q], rv[q], a[0][q]);
          a[1][q] = fma(uv[q] * uv[q], dg, a[1][q]);
        }
        stn<RN>(r + o, rv);
      }
    }
  }
  if (mcol_sum_last<2, RN, kMT>(a, cb, partials, counter, s_red, s_tot)) {
    if (threadIdx.x < kP) {
      const int k = threadIdx.x;
      if (O->active[k]) {
        const double rn = sqrt(fabs(s_tot[k]));
        const double rel = O->norm_f[k] > 1e-300 ? rn / O->norm_f[k] : rn;
        const double uD2 = s_tot[kP + k];
        int fl = O->flags[k];
        if (err_stop == 1) {
          // the step's correction d = x / scale (||x||_M^2 from the estimate)
          const double sc = O->scale[k];
          const double dn2 = est[k].total2 / (sc * sc);
          const double pb2 = refine_bound2(dn2, O->dD2[k]);
          O->pert[k] = uD2 > 0.0 ? sqrt(pb2 / uD2) : -1.0;
          if ((S->flags[k] & kFlagErrTarget) && pb2 <= err_goal * err_goal * uD2)
            fl |= kFlagDone | kFlagConverged;
          O->dD2[k] = dn2;
        } else if (err_stop == 2) {
          O->dD2[k] = uD2;
          O->pert[k] = -1.0;
        }
        O->rel[k] = rel;
        O->scale[k] = rn > 0.0 ? 1.0 / rn : 1.0;
        O->uD2[k] = uD2;
        if (err_stop) {
        } else if (rel <= tol) {
          fl |= kFlagDone | kFlagConverged;
        } else if (O->prev[k] > 0.0 && rel >= O->prev[k] * 0.9) {
          fl |= kFlagDone | kFlagStalled;
        }
        O->prev[k] = rel;
        O->flags[k] = fl;
        O->active[k] = (fl & kFlagDone) ? 0 : 1;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int all = 1;
      for (int k = 0; k < kP; ++k) all &= (O->flags[k] & kFlagDone) ? 1 : 0;
      O->done = all;
    }
  }
}

// ── panel vector kernels: thread = one DOF x 4 columns (cb = 4*(lane&3)) ─

// r = f, u = 0 (FP64 panels) and ||f|| per column for the refinement record.
__global__ void __launch_bounds__(kVT, 1)
k_mouter_init(int n, int ncols, const double* __restrict__ f, double* __restrict__ r,
              double* __restrict__ u, MultiOuter* O, double* partials, unsigned* counter) {
  __shared__ double s_red[kVT];
  __shared__ double s_tot[kP];
  const int cb = 4 * (threadIdx.x & 3);
  double a[1][4] = {{0.0, 0.0, 0.0, 0.0}};
  const double zero[4] = {0.0, 0.0, 0.0, 0.0};
  const long long nc = static_cast<long long>(n) * 4;
  for (long long c = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x; c < nc;
       c += static_cast<long long>(gridDim.x) * kVT) {
    const size_t o = static_cast<size_t>(c >> 2) * kP + cb;
    double fv[4];
    ld4(f + o, fv);
#pragma unroll
    for (int j = 0; j < 4; ++j) a[0][j] = fma(fv[j], fv[j], a[0][j]);
    st4(r + o, fv);
    st4(u + o, zero);
  }
  if (mcol_sum_last<1, 4, kVT>(a, cb, partials, counter, s_red, s_tot)) {
    if (threadIdx.x < kP) {
      const int k = threadIdx.x;
      const double nb = sqrt(fabs(s_tot[k]));
      int fl = 0;
      if (k >= ncols)
        fl = kFlagDone | kFlagInactive;
      else if (nb < 1e-300)  // zero load case: u = 0 (cuda_pcg_backend_impl.hpp:1820-1830)
        fl = kFlagDone | kFlagZeroRhs | kFlagConverged;
      O->norm_f[k] = nb;
      O->rel[k] = (fl & kFlagDone) ? 0.0 : 1.0;
      O->prev[k] = 0.0;
      O->scale[k] = nb > 1e-300 ? 1.0 / nb : 1.0;
      O->uD2[k] = 0.0;
      O->dD2[k] = 0.0;
      O->pert[k] = -1.0;
      O->flags[k] = fl;
      O->active[k] = (fl & kFlagDone) ? 0 : 1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int all = 1;
      for (int k = 0; k < kP; ++k) all &= (O->flags[k] & kFlagDone) ? 1 : 0;
      O->done = all;
    }
  }
}

// PCG start: r = src * scale (src = f, or the FP64 residual of the
// refinement), u = 0, z = D^-1 r, p = z; r.z and r.r per column.
// err_mode != kErrOff makes the columns error-controlled (errest.cuh):
// kErrRelative with err_rel the relative target (FP64 solve), kErrAbsolute
// with the target err_target * scale * ||u||_D of the column's outer record
// and err_rel the relative floor (refinement steps of the mixed solve).
template <typename T>
__global__ void __launch_bounds__(kVT, 1)
k_minit(int n, int ncols, const double* __restrict__ src, const MultiOuter* O,
        const T* __restrict__ dinv, T* __restrict__ r, T* __restrict__ u, T* __restrict__ p,
        MultiState* S, ErrEst* est, int err_mode, double err_target, double err_rel,
        double tol, double outer_tol, int max_iters, double* partials, unsigned* counter,
        const MultiRecord rec = MultiRecord{}) {
  __shared__ double s_red[kVT];
  __shared__ double s_tot[2 * kP];
  const int cb = 4 * (threadIdx.x & 3);
  double sc[4];
  bool act[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    act[j] = O ? (O->active[cb + j] != 0) : (cb + j < ncols);
    sc[j] = O ? O->scale[cb + j] : 1.0;
  }
  T rz[4] = {T(0), T(0), T(0), T(0)}, rr[4] = {T(0), T(0), T(0), T(0)};
  const T zero[4] = {T(0), T(0), T(0), T(0)};
  const long long nc = static_cast<long long>(n) * 4;
  for (long long c = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x; c < nc;
       c += static_cast<long long>(gridDim.x) * kVT) {
    const long long i = c >> 2;
    const size_t o = static_cast<size_t>(i) * kP + cb;
    double sv[4];
    ld4(src + o, sv);
    const T d = dinv[i];
    T rv[4], zv[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      rv[j] = act[j] ? static_cast<T>(sv[j] * sc[j]) : T(0);
      zv[j] = rv[j] * d;
      rz[j] = fmaT(rv[j], zv[j], rz[j]);
      rr[j] = fmaT(rv[j], rv[j], rr[j]);
    }
    if (rec.hist && rec.col >= cb && rec.col < cb + 4)
      rec.hist[i] = static_cast<float>(zv[rec.col - cb]);
    st4(r + o, rv);
    st4(u + o, zero);
    st4(p + o, zv);
  }
  T a[2][4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    a[0][j] = rz[j];
    a[1][j] = rr[j];
  }
  if (mcol_sum<2, 4, kVT>(a, cb, partials, counter, s_red, s_tot)) {
    if (threadIdx.x < kP) {
      const int k = threadIdx.x;
      const double rzk = s_tot[k], rrk = s_tot[kP + k], nb = sqrt(fabs(rrk));
      const bool active = O ? (O->active[k] != 0) : (k < ncols);
      int fl = 0;
      if (!active)
        fl = kFlagDone | kFlagInactive;
      else if (nb < 1e-300)
        fl = kFlagDone | kFlagZeroRhs | kFlagConverged;
      else if (!(rzk > 0.0))  // cuda_pcg_backend_impl.hpp:1859-1862
        fl = kFlagDone | kFlagNonPosRz;
      // Inexact refinement per load case (as the single-case solve): with
      // outer_tol > 0 a correction stops at 0.5 * outer_tol / (its case's
      // true residual) when that is looser than tol.
      double tk = tol;
      if (O && outer_tol > 0.0 && O->rel[k] > 0.0) {
        const double want = 0.5 * outer_tol / O->rel[k];
        tk = fmax(tol, fmin(0.5, want));
      }
      S->tolk[k] = tk;
      err_reset(est[k]);
      const double sk = O ? O->scale[k] : 1.0;
      const double un2 = (O && err_mode == kErrAbsolute) ? sk * sk * O->uD2[k] : 0.0;
      S->err_t2[k] = err_target * err_target * un2;
      S->err_norm2[k] = un2;
      S->rz[k] = rzk;
      S->rr[k] = rrk;
      if (rec.coef && k == rec.col) rec.coef[2] = rzk;
      S->norm_b[k] = nb;
      S->rel[k] = (fl & kFlagDone) ? 0.0 : 1.0;
      S->alpha[k] = S->beta[k] = S->pAp[k] = 0.0;
      S->flags[k] = fl;
      S->iters[k] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      S->iter = 0;
      S->tol = tol;
      S->max_iters = max_iters;
      S->ncols = ncols;
      S->err_mode = err_mode;
      S->err_rel2 = err_rel * err_rel;
      all_done(S);
    }
  }
}

// u += alpha p, r -= alpha Ap, z = D^-1 r (not stored); r.z, r.r per column,
// then the per-column stopping test rel = sqrt(r.r)/||b|| < tol
// (cuda_pcg_backend_impl.hpp:723-729) and beta = rz_new / rz.
template <typename T>
__global__ void __launch_bounds__(kVT, 1)
k_mupdate(int n, T* __restrict__ u, T* __restrict__ r, const T* __restrict__ p,
          const T* __restrict__ Ap, const T* __restrict__ dinv, MultiState* S, ErrEst* est,
          double* partials, unsigned* counter, const MultiRecord rec = MultiRecord{}) {
  if (S->done) return;
  // iteration of this update (the last block advances S->iter when every
  // block has read it)
  const int it0 = S->iter;
  const bool keep = rec.hist && it0 + 1 < rec.max;
  __shared__ double s_red[kVT];
  __shared__ double s_tot[2 * kP];
  const int cb = 4 * (threadIdx.x & 3);
  T al[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) al[j] = static_cast<T>(S->alpha[cb + j]);
  T rz[4] = {T(0), T(0), T(0), T(0)}, rr[4] = {T(0), T(0), T(0), T(0)};
  const long long nc = static_cast<long long>(n) * 4;
  for (long long c = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x; c < nc;
       c += static_cast<long long>(gridDim.x) * kVT) {
    const long long i = c >> 2;
    const size_t o = static_cast<size_t>(i) * kP + cb;
    T uv[4], rv[4], pv[4], av[4];
    ld4(u + o, uv);
    ld4(r + o, rv);
    ld4(p + o, pv);
    ld4(Ap + o, av);
    const T d = dinv[i];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      uv[j] = fmaT(al[j], pv[j], uv[j]);
      rv[j] = fmaT(-al[j], av[j], rv[j]);
      const T z = rv[j] * d;
      rz[j] = fmaT(rv[j], z, rz[j]);
      rr[j] = fmaT(rv[j], rv[j], rr[j]);
      if (keep && cb + j == rec.col)
        rec.hist[static_cast<size_t>(it0 + 1) * n + i] = static_cast<float>(z);
    }
    st4(u + o, uv);
    st4(r + o, rv);
  }
  T a[2][4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    a[0][j] = rz[j];
    a[1][j] = rr[j];
  }
  if (mcol_sum<2, 4, kVT>(a, cb, partials, counter, s_red, s_tot)) {
    if (threadIdx.x < kP) {
      const int k = threadIdx.x;
      int fl = S->flags[k];
      if (!(fl & kFlagDone)) {
        const double rzn = s_tot[k], rrk = s_tot[kP + k];
        const double rel = sqrt(fabs(rrk)) / S->norm_b[k];
        const int it = S->iter + 1;
        S->rr[k] = rrk;
        S->rel[k] = rel;
        bool conv;
        if (S->err_mode != kErrOff) {
          conv = err_block_end(est[k], S->err_t2[k], S->err_rel2);
          bool met = conv && (S->err_mode == kErrRelative ||
                              (est[k].est2 <= S->err_t2[k] && est[k].lag2 <= S->err_t2[k]));
          if (!(fabs(rrk) > (sizeof(T) == 4 ? 1e-20 : 1e-28) * S->norm_b[k] * S->norm_b[k])) {
            conv = true;
            met = met || sizeof(T) == 8;
          }
          if (met) fl |= kFlagErrTarget;
        } else {
          conv = rel < S->tolk[k];
        }
        if (conv) {
          fl |= kFlagDone | kFlagConverged;
          S->beta[k] = 0.0;
          S->iters[k] = it;
        } else {
          S->beta[k] = rzn / S->rz[k];
          if (it >= S->max_iters) {
            fl |= kFlagDone | kFlagMaxIters;
            S->iters[k] = it;
          }
        }
        if (rec.coef && k == rec.col && it0 < rec.max) {
          rec.coef[3 * it0] = S->alpha[k];
          rec.coef[3 * it0 + 1] = S->beta[k];
          if (it0 + 1 < rec.max) rec.coef[3 * (it0 + 1) + 2] = rzn;
        }
        S->rz[k] = rzn;
        S->flags[k] = fl;
      } else {
        S->beta[k] = 0.0;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      S->iter += 1;
      all_done(S);
    }
  }
}

// p = D^-1 r + beta p.
template <typename T>
__global__ void __launch_bounds__(kVT, 1)
k_mdirection(int n, const T* __restrict__ r, const T* __restrict__ dinv, T* __restrict__ p,
             const MultiState* S) {
  if (S->done) return;
  const int cb = 4 * (threadIdx.x & 3);
  T be[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) be[j] = static_cast<T>(S->beta[cb + j]);
  const long long nc = static_cast<long long>(n) * 4;
  for (long long c = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x; c < nc;
       c += static_cast<long long>(gridDim.x) * kVT) {
    const long long i = c >> 2;
    const size_t o = static_cast<size_t>(i) * kP + cb;
    T rv[4], pv[4];
    ld4(r + o, rv);
    ld4(p + o, pv);
    const T d = dinv[i];
#pragma unroll
    for (int j = 0; j < 4; ++j) pv[j] = fmaT(be[j], pv[j], rv[j] * d);
    st4(p + o, pv);
  }
}

// u64 += d32 / scale for the columns refined in this step.
__global__ void __launch_bounds__(kVT, 1)
k_maccumulate(int n, double* __restrict__ u64, const float* __restrict__ d32,
              const MultiOuter* O) {
  const int k = threadIdx.x & 15;
  const bool act = O->active[k] != 0;
  const double inv = 1.0 / O->scale[k];
  if (!act) return;
  const long long tot = static_cast<long long>(n) * kP;
  for (long long i = static_cast<long long>(blockIdx.x) * kVT + threadIdx.x; i < tot;
       i += static_cast<long long>(gridDim.x) * kVT)
    u64[i] = fma(static_cast<double>(d32[i]), inv, u64[i]);
}

// Loop control of the single-launch batched inner solve: the kernel that
// closes each body (check_every iterations) of the solve graph's WHILE node.
// The body runs again while a column is active (S->done, set by k_mupdate at
// max_iters at the latest), and never more than max_rounds times: the round
// count, zeroed by the graph before the loop, bounds the loop by itself.
__global__ void k_mloop(MultiState* S, unsigned max_rounds, cudaGraphConditionalHandle h) {
  const unsigned r = S->loop_rounds + 1u;
  S->loop_rounds = r;
  cudaGraphSetConditional(h, (S->done == 0 && r < max_rounds) ? 1u : 0u);
}

}  // namespace

}  // namespace vsgb

namespace vsgb {

struct MultiWork {
  DevBuf<double> f, r64, u64, p64, Ap64;  // FP64 panels
  DevBuf<float> r32, u32, p32, Ap32;      // FP32 panels (mixed inner solves)
  DevBuf<float> p32b;                     // second direction panel (tiled solve)
  DevBuf<unsigned long long> trace;       // tiled solve phase timer (ctas x 8)
  DevBuf<int> cmask;                      // columns of a step (coarse correction)
  std::vector<unsigned long long> htrace;
  DevBuf<double> mpart;                   // tiled solve: 2 x ctas x 32 partials
  MultiTiles tiles[2];                    // tiled solve: chosen + candidate
  int tbest = -1;                         // tiles[tbest] in use (-1: none fit)
  unsigned long long tile_key = 0;        // sparsity pattern the tiles belong to
  int tile_mode = -1, tile_nb = -1;
  long long tile_steps = -1;
  DevBuf<MultiState> S;
  DevBuf<MultiOuter> O;
  DevBuf<ErrEst> est;  // per-column error estimate (kP)
  DevBuf<double> partials;
  DevBuf<unsigned> counters;
  MultiState* hS = nullptr;  // pinned
  MultiOuter* hO = nullptr;  // pinned
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  unsigned exec_epoch[2] = {0, 0};
  int exec_batch[2] = {0, 0};
  // single-launch inner solves: graph of a WHILE node around check_every
  // iterations (FP64 / FP32), its key, and whether the driver refused one
  cudaGraphExec_t lexec[2] = {nullptr, nullptr};
  unsigned lexec_epoch[2] = {0, 0};
  int lexec_batch[2] = {0, 0};
  long long lexec_rounds[2] = {0, 0};
  bool loop_off = false;
  unsigned epoch = 1;     // bumped whenever a buffer moves or the operator changes
  unsigned op_gen = 0;    // operator generation the buffers were sized for

  ~MultiWork() {
    for (auto& g : exec)
      if (g) cudaGraphExecDestroy(g);
    for (auto& g : lexec)
      if (g) cudaGraphExecDestroy(g);
    if (hS) cudaFreeHost(hS);
    if (hO) cudaFreeHost(hO);
  }
};

void destroy_multi(MultiWork* w) { delete w; }

namespace {

int occupancy_grid(const void* fn, int num_sms) {
  int per_sm = 0;
  VSGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kMT, 0));
  return num_sms * (per_sm > 0 ? per_sm : 1);
}

// One iteration for T: SpMM (+alpha), update (+beta, stopping test), direction.
template <typename T, int G>
void launch_multi_iter(const MView& B, const T* vals, const T* dinv, const float* diag32, T* r,
                       T* u, T* p, T* Ap, MultiWork& W, int n, dim3 sgrid, int vgrid,
                       cudaStream_t s, const MultiRecord& rec = MultiRecord{}) {
  k_mspmm<T, G><<<sgrid, kMT, 0, s>>>(B, vals, p, Ap, diag32, W.S.ptr, W.est.ptr,
                                      W.partials.ptr, W.counters.ptr + 1);
  k_mupdate<T><<<vgrid, kVT, 0, s>>>(n, u, r, p, Ap, dinv, W.S.ptr, W.est.ptr, W.partials.ptr,
                                     W.counters.ptr + 2, rec);
  k_mdirection<T><<<vgrid, kVT, 0, s>>>(n, r, dinv, p, W.S.ptr);
}

}  // namespace

bool PcgEngine::ensure_tiles(MultiWork& W, int ncols, cudaStream_t s) {
  tile_rows_used_ = 0;
  const int nb = bsr_.nb;
  if (batch_tiles_ == 0 || !coords_ || coords_->size() != static_cast<size_t>(nb) * 3 ||
      nb <= 0)
    return false;
  const size_t np = static_cast<size_t>(n_) * kP;
  const size_t npart = static_cast<size_t>(num_sms_) * 2 * 2 * kP;
  if (W.p32b.cap < np || W.mpart.cap < npart) {
    W.p32b.reserve(np);
    W.mpart.reserve(npart);
    ++W.epoch;
  }
  if (W.tile_key == pattern_key_ && W.tile_mode == batch_tiles_ && W.tile_nb == nb &&
      W.tile_steps == bsr_.steps) {
    if (W.tbest < 0) return false;  // no tile size fits this pattern
    MultiTiles& T = W.tiles[W.tbest];
    if (T.gen != generation_) {
      mres_gather_values(bsr_, dinv32_.ptr, T, s);
      launches_ += 1;
      T.gen = generation_;
    }
    tile_rows_used_ = T.tn;
    return true;
  }
  // New sparsity pattern: build the candidate tile sizes (rows per tile for
  // 2..8 tiles per CTA, or the fixed size asked for) and keep the fastest
  // over a fixed number of iterations of the current load cases.
  W.tile_key = 0;
  W.tile_mode = -1;
  W.tbest = -1;
  W.tiles[0].release();
  W.tiles[1].release();
  int dev = 0;
  VSGB_CUDA(cudaGetDevice(&dev));
  const size_t cap = mres_smem_cap(dev);
  const int ctas = num_sms_;
  auto up8 = [](long long v) { return static_cast<int>(std::max(8LL, (v + 7) / 8 * 8)); };
  std::vector<int> cands;
  if (batch_tiles_ >= 8) {
    cands.push_back(up8(batch_tiles_));
  } else {
    for (int m : {4, 6, 8, 10, 12, 16}) {
      const int tn = up8((static_cast<long long>(nb) + static_cast<long long>(ctas) * m - 1) /
                         (static_cast<long long>(ctas) * m));
      if (std::find(cands.begin(), cands.end(), tn) == cands.end()) cands.push_back(tn);
    }
  }
  cudaEvent_t ev[2] = {nullptr, nullptr};
  VSGB_CUDA(cudaEventCreate(&ev[0]));
  VSGB_CUDA(cudaEventCreate(&ev[1]));
  float best_ms = 0.f;
  try {
    for (int tn : cands) {
      const int slot = W.tbest == 0 ? 1 : 0;
      MultiTiles& T = W.tiles[slot];
      T.release();
      if (!mres_build_tiles(bsr_, dinv32_.ptr, *coords_, tn, ctas, cap, T, s)) continue;
      if (mres_ctas(num_sms_, T.smem) < 1) {
        T.release();
        continue;
      }
      T.gen = generation_;
      launches_ += 1;
      if (cands.size() == 1) {
        W.tbest = slot;
        break;
      }
      MresSolve q{};
      q.r64 = W.r64.ptr;
      q.u64 = W.u64.ptr;
      q.r = W.r32.ptr;
      q.u = W.u32.ptr;
      q.pa = W.p32.ptr;
      q.pb = W.p32b.ptr;
      q.Ap = W.Ap32.ptr;
      q.dinv32 = dinv32_.ptr;
      q.diag32 = nullptr;
      q.S = W.S.ptr;
      q.O = W.O.ptr;
      q.est = W.est.ptr;
      q.partials = W.mpart.ptr;
      q.count = W.counters.ptr + 6;
      q.tol = 0.0;
      q.outer_tol = 0.0;
      q.max_iters = 24;
      q.ncols = ncols;
      q.err_mode = kErrOff;
      q.spin_limit = spin_limit_;
      q.accumulate = 0;
      mres_solve(T, n_, q, s);  // warm-up
      VSGB_CUDA(cudaEventRecord(ev[0], s));
      mres_solve(T, n_, q, s);
      VSGB_CUDA(cudaEventRecord(ev[1], s));
      launches_ += 2;
      VSGB_CUDA(cudaEventSynchronize(ev[1]));
      VSGB_CUDA(cudaMemcpyAsync(W.hS, W.S.ptr, sizeof(MultiState), cudaMemcpyDeviceToHost, s));
      VSGB_CUDA(cudaStreamSynchronize(s));
      for (int k = 0; k < kP; ++k)
        if (W.hS->flags[k] & kFlagResidentAbort)
          throw Error(VSGB_ERR_CUDA,
                      "GB300 PCG: a grid barrier of the persistent solve timed out (tiled batched solve)");
      float ms = 0.f;
      VSGB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      if (W.tbest < 0 || ms < best_ms) {
        if (W.tbest >= 0) W.tiles[W.tbest].release();
        W.tbest = slot;
        best_ms = ms;
      } else {
        T.release();
      }
    }
  } catch (...) {
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    W.tiles[0].release();
    W.tiles[1].release();
    W.tbest = -1;  // the next solve builds them again
    throw;
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  W.tile_key = pattern_key_;
  W.tile_mode = batch_tiles_;
  W.tile_nb = nb;
  W.tile_steps = bsr_.steps;
  if (W.tbest < 0) return false;
  tile_rows_used_ = W.tiles[W.tbest].tn;
  return true;
}

void PcgEngine::solve_multi(const double* d_F, int nrhs, double* d_U, bool mixed, double tol,
                            double inner_tol, int max_iters, int max_solves, cudaStream_t s,
                            std::vector<SolveResult>& res) {
  tile_rows_used_ = 0;
  if (!use_bsr_) throw Error(VSGB_ERR_STATE, "batched PCG needs the 3x3 block operator");
  if (precond_ != 0)
    throw Error(VSGB_ERR_INVALID, "the batched PCG runs the scalar Jacobi preconditioner only");
  if (mixed && !(bsr_.has32 && has32_))
    throw Error(VSGB_ERR_STATE, "batched mixed PCG needs the FP32 operator copy");
  if (!multi_) multi_ = new MultiWork();
  MultiWork& W = *multi_;
  if (W.op_gen != generation_) {
    W.op_gen = generation_;
    ++W.epoch;
  }
  const size_t n = static_cast<size_t>(n_);
  const size_t np = n * kP;
  auto grow = [&W](auto& buf, size_t cnt) {
    if (cnt > buf.cap) {
      buf.reserve(cnt);
      ++W.epoch;
    }
  };
  grow(W.f, np);
  grow(W.u64, np);
  grow(W.r64, np);
  if (mixed) {
    grow(W.r32, np);
    grow(W.u32, np);
    grow(W.p32, np);
    grow(W.Ap32, np);
  } else {
    grow(W.p64, np);
    grow(W.Ap64, np);
  }
  grow(W.S, 1);
  grow(W.O, 1);
  grow(W.est, kP);
  grow(W.counters, 8);
  // Error control (errest.cuh): FP64 columns stop on their own estimate
  // relative to ||u||; mixed columns refine until a refinement step met the
  // absolute target err_target * ||u||_D (first inner solve: inner_tol).
  const bool err_control = err_target_ > 0.0;
  const double err_goal = err_target_ / kErrSafety;
  if (err_control) ensure_diag32(s);
  const float* diag32 = res_.diag32.ptr;
  if (!W.hS) VSGB_CUDA(cudaMallocHost(&W.hS, sizeof(MultiState)));
  if (!W.hO) VSGB_CUDA(cudaMallocHost(&W.hO, sizeof(MultiOuter)));

  const MView B{bsr_.nb, bsr_.nslices, bsr_.slice_ptr.ptr, bsr_.cols.ptr};
  const int vgrid = grid_for(static_cast<long long>(n) * 4, kVT, num_sms_);
  const int slice_blocks = (bsr_.nslices + kMT / 32 - 1) / (kMT / 32);
  auto cap = [slice_blocks](int g) { return g < slice_blocks ? g : (slice_blocks > 0 ? slice_blocks : 1); };
  const dim3 g32(cap(occupancy_grid(reinterpret_cast<const void*>(&k_mspmm<float, 16>), num_sms_)), 1);
  const dim3 g64(cap(occupancy_grid(reinterpret_cast<const void*>(&k_mspmm<double, 8>), num_sms_)), 2);
  const dim3 gres(cap(occupancy_grid(reinterpret_cast<const void*>(&k_mresidual<8>), num_sms_)), 2);
  size_t pmax = static_cast<size_t>(vgrid);
  for (const dim3& g : {g32, g64, gres})
    if (static_cast<size_t>(g.x) * g.y > pmax) pmax = static_cast<size_t>(g.x) * g.y;
  grow(W.partials, pmax * 2 * kP);
  VSGB_CUDA(cudaMemsetAsync(W.counters.ptr, 0, sizeof(unsigned) * 8, s));

  auto read_state = [&]() {
    VSGB_CUDA(cudaMemcpyAsync(W.hS, W.S.ptr, sizeof(MultiState), cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  };
  auto read_outer = [&]() {
    VSGB_CUDA(cudaMemcpyAsync(W.hO, W.O.ptr, sizeof(MultiOuter), cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  };
  auto iters = [&](bool fp32, const MultiRecord& rec) {
    for (int k = 0; k < check_every_; ++k) {
      if (fp32)
        launch_multi_iter<float, 16>(B, bsr_.val32.ptr, dinv32_.ptr, diag32, W.r32.ptr,
                                     W.u32.ptr, W.p32.ptr, W.Ap32.ptr, W, n_, g32, vgrid, s,
                                     rec);
      else
        launch_multi_iter<double, 8>(B, bsr_.val64.ptr, op_->dinv.ptr, diag32, W.r64.ptr,
                                     W.u64.ptr, W.p64.ptr, W.Ap64.ptr, W, n_, g64, vgrid, s);
    }
    VSGB_LAUNCH_CHECK();
  };
  auto batch = [&](bool fp32, const MultiRecord& rec) {
    iters(fp32, rec);
    VSGB_CUDA(cudaMemcpyAsync(W.hS, W.S.ptr, sizeof(MultiState), cudaMemcpyDeviceToHost, s));
  };
  // The whole inner solve as one graph launch: a memset of the round count,
  // then a WHILE node whose body is check_every iterations and k_mloop, which
  // keeps the body running on the device while a column is active (no host
  // round trip inside a solve).  Cached per key, buffers, batch size and round
  // bound; false (and the batch loop below from then on) when the driver
  // refuses any part of it.
  auto ensure_loop_graph = [&](int key, bool fp32, long long max_rounds) -> bool {
    if (W.lexec[key] && W.lexec_epoch[key] == W.epoch && W.lexec_batch[key] == check_every_ &&
        W.lexec_rounds[key] == max_rounds)
      return true;
    if (W.lexec[key]) {
      cudaGraphExecDestroy(W.lexec[key]);
      W.lexec[key] = nullptr;
    }
    cudaGraph_t g = nullptr;
    bool ok = false, capturing = false;
    try {
      do {
        if (cudaGraphCreate(&g, 0) != cudaSuccess) break;
        cudaGraphConditionalHandle h;
        if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess)
          break;
        cudaMemsetParams mp = {};
        mp.dst = &W.S.ptr->loop_rounds;
        mp.value = 0;
        mp.elementSize = sizeof(unsigned);
        mp.width = 1;
        mp.height = 1;
        mp.pitch = sizeof(unsigned);
        cudaGraphNode_t n0 = nullptr, n1 = nullptr;
        if (cudaGraphAddMemsetNode(&n0, g, nullptr, 0, &mp) != cudaSuccess) break;
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        if (cudaGraphAddNode(&n1, g, &n0, nullptr, 1, &cp) != cudaSuccess) break;
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        if (cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) != cudaSuccess)
          break;
        capturing = true;
        iters(fp32, MultiRecord{});
        k_mloop<<<1, 1, 0, s>>>(W.S.ptr, static_cast<unsigned>(max_rounds), h);
        cudaGraph_t done_body = nullptr;
        capturing = false;
        if (cudaStreamEndCapture(s, &done_body) != cudaSuccess) break;
        if (cudaGraphInstantiate(&W.lexec[key], g, 0) != cudaSuccess) {
          W.lexec[key] = nullptr;
          break;
        }
        ok = true;
      } while (false);
    } catch (...) {
      if (capturing) {
        cudaGraph_t t = nullptr;
        cudaStreamEndCapture(s, &t);
      }
      if (g) cudaGraphDestroy(g);
      throw;
    }
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      cudaGetLastError();  // the refusal is not sticky: fall back
      W.loop_off = true;
      return false;
    }
    W.lexec_epoch[key] = W.epoch;
    W.lexec_batch[key] = check_every_;
    W.lexec_rounds[key] = max_rounds;
    return true;
  };
  // Batches of check_every iterations (a cached CUDA graph) until every
  // column reports done; the device stops itself at max_iters.
  // (a recorded solve launches directly: the record is not part of the graph)
  auto iterate_all = [&](bool fp32, const MultiRecord& rec = MultiRecord{}) {
    const int key = fp32 ? 1 : 0;
    const bool graph = use_graph_ && rec.hist == nullptr;
    const long long max_rounds = (static_cast<long long>(max_iters) + check_every_ - 1) /
                                     check_every_ + 4;
    if (graph && !W.loop_off && ensure_loop_graph(key, fp32, max_rounds)) {
      VSGB_CUDA(cudaGraphLaunch(W.lexec[key], s));
      read_state();
      launches_ += (3LL * check_every_ + 1) * W.hS->loop_rounds;
      if (!W.hS->done)
        throw Error(VSGB_ERR_CUDA, "batched PCG device state did not report completion");
      return;
    }
    if (graph && (W.exec[key] == nullptr || W.exec_epoch[key] != W.epoch ||
                       W.exec_batch[key] != check_every_)) {
      if (W.exec[key]) {
        cudaGraphExecDestroy(W.exec[key]);
        W.exec[key] = nullptr;
      }
      cudaGraph_t g = nullptr;
      VSGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      try {
        batch(fp32, MultiRecord{});
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      VSGB_CUDA(cudaStreamEndCapture(s, &g));
      VSGB_CUDA(cudaGraphInstantiate(&W.exec[key], g, 0));
      cudaGraphDestroy(g);
      W.exec_epoch[key] = W.epoch;
      W.exec_batch[key] = check_every_;
    }
    const long long max_batches = (static_cast<long long>(max_iters) + check_every_ - 1) /
                                      check_every_ + 4;
    for (long long b = 0;; ++b) {
      if (b > max_batches)
        throw Error(VSGB_ERR_CUDA, "batched PCG device state did not report completion");
      if (graph)
        VSGB_CUDA(cudaGraphLaunch(W.exec[key], s));
      else
        batch(fp32, rec);
      launches_ += 3LL * check_every_;
      VSGB_CUDA(cudaStreamSynchronize(s));
      if (W.hS->done) break;
    }
  };
  auto check_start = [&]() {
    for (int k = 0; k < kP; ++k)
      if (W.hS->flags[k] & kFlagNonPosRz)
        throw Error(VSGB_ERR_SINGULAR,
                    "GB300 PCG: non-positive initial r*z=" + std::to_string(W.hS->rz[k]) +
                        " -- preconditioner is not SPD or matrix is singular");
  };

  std::vector<ErrEst> hest(kP);
  auto read_est = [&]() {
    VSGB_CUDA(cudaMemcpyAsync(hest.data(), W.est.ptr, sizeof(ErrEst) * kP, cudaMemcpyDeviceToHost,
                              s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  };
  res.assign(static_cast<size_t>(nrhs), SolveResult{});
  const int pack_grid = static_cast<int>((n + 31) / 32);
  for (int k0 = 0; k0 < nrhs; k0 += kP) {
    const int nc = nrhs - k0 < kP ? nrhs - k0 : kP;
    k_pack<<<pack_grid, kMT, 0, s>>>(n_, nc, d_F + static_cast<size_t>(k0) * n, W.f.ptr);
    VSGB_LAUNCH_CHECK();
    ++launches_;
    if (!mixed) {
      k_minit<double><<<vgrid, kVT, 0, s>>>(
          n_, nc, W.f.ptr, nullptr, op_->dinv.ptr, W.r64.ptr, W.u64.ptr, W.p64.ptr, W.S.ptr,
          W.est.ptr, err_control ? kErrRelative : kErrOff, 0.0, err_goal, tol, 0.0, max_iters,
          W.partials.ptr, W.counters.ptr);
      VSGB_LAUNCH_CHECK();
      ++launches_;
      if (!use_graph_ || W.loop_off) {
        read_state();
        check_start();
        if (!W.hS->done) iterate_all(false);
      } else {
        iterate_all(false);  // one launch, also when init finished every column
      }
      read_state();
      check_start();
      if (err_control) read_est();
      for (int k = 0; k < nc; ++k) {
        SolveResult& R = res[static_cast<size_t>(k0 + k)];
        const int fl = W.hS->flags[k];
        R.iterations = W.hS->iters[k];
        R.rel = W.hS->rel[k];
        R.converged = (fl & kFlagConverged) != 0;
        R.breakdown = (fl & kFlagBreakdown) != 0;
        if (err_control) {
          R.err_met = (fl & kFlagErrTarget) != 0;
          const ErrEst& e = hest[static_cast<size_t>(k)];
          const double e2 = std::max(e.est2, e.lag2);
          R.err_est = (e.est2 >= 0.0 && e.lag2 >= 0.0 && e.total2 > 0.0)
                          ? std::sqrt(e2 / e.total2)
                          : ((fl & kFlagZeroRhs) ? 0.0 : -1.0);
        }
      }
    } else {
      k_mouter_init<<<vgrid, kVT, 0, s>>>(n_, nc, W.f.ptr, W.r64.ptr, W.u64.ptr, W.O.ptr,
                                          W.partials.ptr, W.counters.ptr + 3);
      VSGB_LAUNCH_CHECK();
      ++launches_;
      read_outer();
      for (int k = 0; k < nc; ++k) res[static_cast<size_t>(k0 + k)].inner_solves = 0;
      // the persistent tiled kernel runs each inner solve in one launch
      const bool tiled = !W.hO->done && ensure_tiles(W, nc, s);
      // Coarse correction (coarse.cuh) after every FP64 residual; without a
      // basis for this operator the first active column's first inner solve
      // (launch-per-kernel path) records its Lanczos vectors for one.
      const bool coarse = err_control && coarse_mode_ > 0;
      if (coarse && coarse_.gen != generation_) coarse_.valid = false;
      MultiRecord rec;
      if (coarse && coarse_.gen != generation_ && !tiled)
        for (int k = 0; k < nc; ++k)
          if (W.hO->active[k]) {
            rec.col = k;
            rec.max = std::min(kCoarseHistMax, max_iters + 1);
            hist_.reserve(static_cast<size_t>(rec.max) * n);
            coef_.reserve(static_cast<size_t>(3) * rec.max);
            rec.hist = hist_.ptr;
            rec.coef = coef_.ptr;
            break;
          }
      if (coarse) W.cmask.reserve(kP);
      if (tiled && trace_ && k0 == 0) {
        for (double& v : tile_ns_) v = 0.0;
        tile_its_ = 0;
      }
      for (int step = 0; step < max_solves && !W.hO->done; ++step) {
        const bool err_step = err_control && step > 0;
        const double outer = (adaptive_inner_ && !err_control) ? tol : 0.0;
        if (tiled) {
          MresSolve q{};
          q.r64 = W.r64.ptr;
          q.u64 = W.u64.ptr;
          q.r = W.r32.ptr;
          q.u = W.u32.ptr;
          q.pa = W.p32.ptr;
          q.pb = W.p32b.ptr;
          q.Ap = W.Ap32.ptr;
          q.dinv32 = dinv32_.ptr;
          q.diag32 = err_control ? diag32 : nullptr;
          q.S = W.S.ptr;
          q.O = W.O.ptr;
          q.est = W.est.ptr;
          q.partials = W.mpart.ptr;
          q.count = W.counters.ptr + 6;
          q.tol = inner_tol;
          q.outer_tol = outer;
          q.max_iters = max_iters;
          q.ncols = nc;
          q.err_mode = err_step ? kErrAbsolute : kErrOff;
          q.err_target = err_goal;
          q.err_rel = kErrRelFloor;
          q.spin_limit = spin_limit_;
          q.accumulate = 1;
          const size_t ntr = static_cast<size_t>(W.tiles[W.tbest].ctas) * 8;
          if (trace_) {
            W.trace.reserve(ntr);
            q.trace = W.trace.ptr;
          }
          mres_solve(W.tiles[W.tbest], n_, q, s);
          ++launches_;
          read_state();
          if (trace_) {
            // per-iteration means over CTAs (us): staging, multiply, first
            // reduction, update, second reduction; slowest CTA's multiply
            W.htrace.resize(ntr);
            VSGB_CUDA(cudaMemcpy(W.htrace.data(), W.trace.ptr, ntr * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost));
            const int ct = W.tiles[W.tbest].ctas;
            double sum[5] = {}, mx = 0.0;
            long long its = 0;
            for (int c = 0; c < ct; ++c) {
              for (int k = 0; k < 5; ++k) sum[k] += static_cast<double>(W.htrace[8 * c + k]);
              mx = std::max(mx, static_cast<double>(W.htrace[8 * c + 1]));
              its = std::max(its, static_cast<long long>(W.htrace[8 * c + 5]));
            }
            tile_ns_[0] += sum[0] / ct;
            tile_ns_[1] += sum[1] / ct;
            tile_ns_[2] += sum[2] / ct;
            tile_ns_[3] += sum[3] / ct;
            tile_ns_[4] += sum[4] / ct;
            tile_ns_[5] += mx;
            tile_its_ += its;
            const double d = tile_its_ > 0 ? 1e3 * static_cast<double>(tile_its_) : 1.0;
            for (double& v : phase_us_) v = 0.0;
            phase_us_[0] = tile_ns_[0] / d;
            phase_us_[1] = tile_ns_[1] / d;
            phase_us_[4] = tile_ns_[2] / d;
            phase_us_[5] = tile_ns_[3] / d;
            phase_us_[8] = tile_ns_[4] / d;
            phase_us_[kTracePhases] = tile_ns_[5] / d;
            phase_us_[kTracePhases + 1] = static_cast<double>(tile_its_);
          }
          for (int k = 0; k < kP; ++k)
            if (W.hS->flags[k] & kFlagResidentAbort)
              throw Error(VSGB_ERR_CUDA,
                      "GB300 PCG: a grid barrier of the persistent solve timed out (tiled batched solve)");
          check_start();
        } else {
          const MultiRecord r0 = step == 0 ? rec : MultiRecord{};
          k_minit<float><<<vgrid, kVT, 0, s>>>(
              n_, nc, W.r64.ptr, W.O.ptr, dinv32_.ptr, W.r32.ptr, W.u32.ptr, W.p32.ptr,
              W.S.ptr, W.est.ptr, err_step ? kErrAbsolute : kErrOff, err_goal, kErrRelFloor,
              inner_tol, outer, max_iters, W.partials.ptr, W.counters.ptr, r0);
          VSGB_LAUNCH_CHECK();
          ++launches_;
          if (!use_graph_ || W.loop_off || r0.hist) {
            read_state();
            check_start();
            if (!W.hS->done) iterate_all(true, r0);
          } else {
            iterate_all(true, r0);  // one launch, also when init finished every column
          }
          read_state();
          check_start();
          if (r0.hist && (W.hS->flags[r0.col] & kFlagConverged))
            coarse_from_record(std::min(W.hS->iters[r0.col], r0.max), s, false);
        }
        if (err_step) read_est();
        bool failed = false;
        int stepped[kP] = {};
        for (int k = 0; k < nc; ++k) {
          if (!W.hO->active[k]) continue;
          stepped[k] = 1;
          SolveResult& R = res[static_cast<size_t>(k0 + k)];
          ++R.inner_solves;
          R.iterations += W.hS->iters[k];
          if (err_step) {
            const ErrEst& e = hest[static_cast<size_t>(k)];
            if (e.est2 >= 0.0 && e.lag2 >= 0.0 && W.hS->err_norm2[k] > 0.0)
              R.err_est = std::sqrt(std::max(e.est2, e.lag2) / W.hS->err_norm2[k]);
            R.err_met = (W.hS->flags[k] & kFlagErrTarget) != 0;
          }
          if (!(W.hS->flags[k] & kFlagConverged)) {
            R.inner_failed = true;
            R.breakdown = (W.hS->flags[k] & kFlagBreakdown) != 0;
            R.rel = W.hS->rel[k];
            failed = true;
          }
        }
        if (failed) return;
        if (!tiled) {
          k_maccumulate<<<num_sms_, kVT, 0, s>>>(n_, W.u64.ptr, W.u32.ptr, W.O.ptr);
          ++launches_;
        }
        const bool corrected = coarse && coarse_.valid;
        if (corrected)  // the columns of this step, before the residual retires some
          VSGB_CUDA(cudaMemcpyAsync(W.cmask.ptr, W.O.ptr->active, sizeof(int) * kP,
                                    cudaMemcpyDeviceToDevice, s));
        k_mresidual<8><<<gres, kMT, 0, s>>>(B, bsr_.val64.ptr, W.u64.ptr, W.f.ptr,
                                            op_->dinv.ptr, W.r64.ptr, W.O.ptr, W.S.ptr,
                                            W.est.ptr, err_control ? (err_step ? 1 : 2) : 0,
                                            err_goal, err_control ? 0.0 : tol,
                                            W.partials.ptr, W.counters.ptr + 4);
        VSGB_LAUNCH_CHECK();
        ++launches_;
        if (corrected) {
          MultiOuter* O = W.O.ptr;
          coarse_apply_panel(coarse_, W.u64.ptr, W.r64.ptr, op_->dinv.ptr, W.cmask.ptr,
                             O->norm_f, O->rel, O->scale, O->uD2, num_sms_, s);
          launches_ += 2;
        }
        read_outer();
        // reported error: the inner estimate plus the FP32-operator bound
        if (err_step)
          for (int k = 0; k < nc; ++k) {
            SolveResult& R = res[static_cast<size_t>(k0 + k)];
            if (stepped[k] && W.hO->pert[k] >= 0.0 && R.err_est >= 0.0)
              R.err_est += W.hO->pert[k];
          }
      }
      for (int k = 0; k < nc; ++k) {
        SolveResult& R = res[static_cast<size_t>(k0 + k)];
        const int fl = W.hO->flags[k];
        R.rel = W.hO->rel[k];
        R.converged = (fl & kFlagConverged) != 0;
        R.stalled = (fl & kFlagStalled) != 0;
      }
    }
    k_unpack<<<pack_grid, kMT, 0, s>>>(n_, nc, W.u64.ptr, d_U + static_cast<size_t>(k0) * n);
    VSGB_LAUNCH_CHECK();
    ++launches_;
  }
}

}  // namespace vsgb
