// vibestran_gb300/csrc/resident.cu — persistent Jacobi PCG (one launch per solve).
//
// Why: per PCG iteration the launch-per-kernel form pays two or three kernel
// boundaries (~2 us each on GB300) plus per-kernel reduction tails, while the
// FP32 block operator of the 84k-element cantilever (94 MB) fits in the 126 MB
// L2, where it streams at ~18-22 TB/s (vs ~7 TB/s from HBM).  Here one
// cooperative launch keeps one CTA per SM for the whole solve:
//   * each CTA owns a step-balanced, contiguous range of block-row slices, so
//     its rows are the contiguous equations [24*s0, 24*s1);
//   * the CTA's own vectors (r, z, u, p, Ap, diag^-1) live in shared memory;
//   * each iteration first stages x = z + beta*p over the CTA's column window
//     into shared memory (one L2 read per needed node instead of one per
//     block), then streams its slices of the operator from L2;
//   * the two dot-product reductions per iteration are grid-wide: per-CTA
//     partials, a bounded-spin grid barrier, and a fixed-order sum that every
//     CTA computes identically (so all CTAs take the same branch).
// The recurrence, convergence test and breakdown / zero-RHS handling are those
// of run_pcg_prepared (src/solver/cuda_pcg_backend_impl.hpp:1688-1999).

#include <algorithm>
#include <climits>

#include "errest.cuh"
#include "gridsync.cuh"
#include "kernels.cuh"
#include "resident.cuh"

namespace vsgb {

namespace {

constexpr int kResThreads = 512;
constexpr int kResWarps = kResThreads / 32;
constexpr int kFlagAbort = 64;

template <typename T>
struct ResArgs {
  int nb, n;
  const int* __restrict__ slice_ptr;
  const int* __restrict__ cols;
  const T* __restrict__ vals;
  const int* __restrict__ cta_slice;
  const int* __restrict__ cta_win;
  const int* __restrict__ cta_runs;  // kRunStride per CTA: referenced runs of the window
  const double* __restrict__ dinv;
  const T* __restrict__ bj;  // 3x3 block Jacobi: inverse diagonal blocks, 6 per node
  const double* __restrict__ rhs;
  double* __restrict__ u_out;
  T* z4;
  T* p4a;
  T* p4b;
  double* partials;
  unsigned* count;
  unsigned long long* fx;  // FP32: fused reduction words (kFxSlots x 2), null: counter barrier
  int* abort_flag;
  PcgScalars* S;
  const PcgScalars* O;
  double tol;
  int max_iters;
  int rows_max;  // own-row stride of the shared-memory vectors
  T* u_glob;     // solution accumulator in global memory (null: in shared memory)
  long long spin_limit;  // polls of a grid wait before it gives up
  // error-controlled stop (errest.cuh): p.Mp per iteration with M = the Jacobi
  // diagonal (diag32) or the 3x3 node blocks (bjd32, upper triangles)
  int err_mode;          // ErrMode
  double err_target;     // kErrAbsolute: target relative to ||u||_D of the outer record O
  double err_rel;        // relative floor (kErrAbsolute) or relative target (kErrRelative)
  const float* __restrict__ diag32;
  const float* __restrict__ bjd32;
  // phase timer (null: off): per CTA, nanoseconds summed over the iterations
  // of gather, SpMV, first reduction (CTA sums, wait for the other CTAs,
  // total and recurrence), update, second reduction (same three parts), then
  // the iteration count (kTraceWords per CTA)
  unsigned long long* trace;
  // Lanczos record of the FP32 solve (null: off): z_k of every row for
  // k < hist_max (node-padded, 4 * nb floats per k) and, CTA 0, the
  // recurrence scalars alpha_k, beta_k, r_k.z_k (3 doubles per k)
  float* hist;
  double* coef;
  int hist_max;
  // deflated FP32 solve (kDM > 0): W (node-padded, kDM x 4 nb), A W (kDM x
  // n), (W^T A W)^-1 (kDM x kDM) and bounds c_i with |(A w_i).z| <= c_i
  // sqrt(r.z) (the fixed-point scales of those dots)
  const float* __restrict__ defl_w;
  const float* __restrict__ defl_aw;  // staged for the own rows in shared memory behind the window
  int win_words;                      // 4 x the largest window: start of that copy
  const float* __restrict__ defl_ginv;
  const double* __restrict__ defl_c;
};

// Cost of a slice beyond its steps, in steps, when slice ranges are split
// across CTAs: starting a slice costs dependent loads (its extent, then its
// first blocks) and ending it a reduction, so CTAs at the mesh ends, whose
// rows have fewer blocks and whose slices are therefore more numerous, ran
// slower with a weight of 1.  Measured per iteration on GB300 (FP32 / FP64,
// 265k and 504k equations), cyclic slice order: weight 1: 25.5 / 75.5 and
// 50.3 / 156 us; 3: 24.1 / 72.5 and 46.8 / 146 us; 5: 23.8 / 72.9 and 46.4 /
// 144 us.  Snake order (kSnake): 4: 17.31 / 66.75 and 33.64 / 144.1 us; 8:
// 17.09 / 65.94 and 33.64 / 143.8 us; 12: 17.09 / 65.75 and 33.57 / 144.0 us;
// 16: 17.06 / 66.15 us (265k).  The partition also fixes the reduction order,
// and with it the rounding of the FP32 inner solves: the 265k cantilever's
// mixed-solve error (tolerance 1e-4) is 8.2e-7 / 6.0e-7 / 9.8e-7 at weights
// 4 / 8 / 12.
constexpr int kSliceWeight = 8;

// Window kernels keep p (the deflated solve: q) over the window in shared
// memory between iterations.
constexpr bool kKeepWindowP = true;

// Window gather over the referenced runs of the window (k_window_runs): at
// most kWinRuns runs per CTA, gaps under kRunGap nodes merged.
constexpr int kWinRuns = 16;
constexpr int kRunGap = 32;
constexpr int kRunStride = 1 + 2 * kWinRuns;

// Deflated solves (coarse.cuh): kDeflVecs coarse vectors, FP32 mixed
// solves with the window only.
constexpr int kDeflVecs = 4;
constexpr int kDeflThread = 32;  // lane 0 of warp 1 forms the deflation scalars
template <typename T, bool kWindow, bool kMixed>
constexpr bool kDeflatable = sizeof(T) == 4 && kWindow && kMixed && kKeepWindowP;
// Shared memory the deflated solve takes beyond the plan's: A W and W of the
// own rows.
inline size_t defl_smem(int rows_max) {
  return 2 * static_cast<size_t>(kDeflVecs) * rows_max * sizeof(float);
}

// FP32 solve: alpha and beta divided in FP32 (they are applied as floats), the
// stopping test as r.r < (tol |b|)^2 with the relative residual formed once
// at the exit; the FP64 solve keeps the FP64 scalar arithmetic.  The FP64
// square root and divisions sat on every iteration's critical path (thread 0,
// GB300's FP64 pipe): 18.4 -> 17.5 us per FP32 iteration at 84k.
constexpr bool kFastScalars32 = true;

// Direction of the SpMV slice walk alternates between iterations.  The
// operator is read once per iteration and does not fit the L2 as a whole; in
// a cyclic walk the lines read last are the ones the next walk reaches last,
// when they are gone, while a reversed walk starts on them.  Measured per
// FP32 iteration: 84k 21.7 -> 18.6 us, 504k 41.0 -> 35.0 us, 780k 69.1 ->
// 63.1 us.
constexpr bool kSnake = true;

// Grid-wide sum of NV doubles: CTA sums -> partial slot -> barrier -> fixed
// order sum by warp 0 of every CTA (bitwise identical in all CTAs), after which
// thread 0 runs fin(totals, ok) — the scalar recurrence, which writes its
// results to shared memory — and one CTA barrier publishes them.
// Per-thread partials are summed over the warp in their own precision A (FP32
// in the FP32 solve: GB300 runs FP64 at 1/58 of the FP32 rate), then the
// kResWarps warp sums (a fixed shuffle tree in warp 0) and the CTA partials
// are added in FP64.
// kW: the warps 0..kW-1 hold per-thread partials (the others hold none and
// skip the warp sums: on GB300 every warp-wide FP64 add costs the SM's FP64
// pipe ~17 cycles whatever the lanes); kW = 0: thread 0 already holds the
// CTA totals, so there is neither a CTA tree nor a CTA barrier before the
// arrival (the caller's last CTA barrier orders the CTA's writes).
template <typename A, int NV, int kW = kResWarps, typename Fin>
__device__ bool grid_allreduce(A (&v)[NV], double* partials, int slot, unsigned* count,
                               unsigned& target, int* abort_flag, double* sm, int* s_ok,
                               long long spin_limit, Fin&& fin) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (kW > 0) {
    if (wid < kW) {
#pragma unroll
      for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
      if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) sm[wid * NV + k] = static_cast<double>(v[k]);
    }
    __syncthreads();
  }
  double* part = partials + static_cast<size_t>(slot) * gridDim.x * NV;
  if (wid == 0) {
    double w[NV];
    if (kW > 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) w[k] = lane < kW ? sm[lane * NV + k] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        if (o < kW)
#pragma unroll
          for (int k = 0; k < NV; ++k) w[k] += __shfl_xor_sync(0xffffffffu, w[k], o);
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) w[k] = static_cast<double>(v[k]);
    }
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) part[blockIdx.x * NV + k] = w[k];
  }
  const bool ok = grid_sync(count, target, abort_flag, s_ok, spin_limit, kW > 0);
  if (threadIdx.x < 32) {
    // Lane l adds the partials of CTAs l, l+32, ... in that order; the loads
    // of a round are all issued before the first add (one L2 round trip per
    // round of 8 instead of one per CTA).
    constexpr int kRound = 8;
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (unsigned c0 = threadIdx.x; c0 < gridDim.x; c0 += 32 * kRound) {
      double u[kRound][NV];
#pragma unroll
      for (int r = 0; r < kRound; ++r) {
        const unsigned c = c0 + 32u * r;
#pragma unroll
        for (int k = 0; k < NV; ++k) u[r][k] = c < gridDim.x ? __ldcg(&part[c * NV + k]) : 0.0;
      }
#pragma unroll
      for (int r = 0; r < kRound; ++r)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += u[r][k];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = warp_sum(acc[k]);
    if (threadIdx.x == 0) fin(acc, ok);
  }
  __syncthreads();
  return ok;
}

// ── Fused fixed-point reductions (FP32 solve) ──
// One 64-bit word per summed value carries the arrivals (bits 0-7), overflow
// reports (bits 8-15) and the sum of the CTA partials as 48-bit signed fixed
// point (bits 16-63) at a scale 2^s chosen from the previous total of the same
// quantity (|previous| 2^s ~ 2^36).  A CTA arrives with one release add of
// (q << 16) + 1, q = rint(partial 2^s), so a waiter that sees every arrival
// holds the total in the same load: one L2 round trip fewer than reading the
// partials after a counter barrier.  Integer addition is exact and
// associative, so the total is the same bits in every CTA and every run.  The
// FP64 partials are stored as before; the reduction falls back to them when
// there is no previous total, when a partial would leave the 48-bit range
// (|q| >= 2^39, reported in bits 8-15) or when the total came out below 2^30
// (a drop of more than 64x, where the fixed point has too few digits).
constexpr bool kFusedReductions = true;
constexpr int kFxSlots = 4;          // reductions in flight before a word is reused
constexpr int kFxWords = 8;          // words per slot (6 values in the deflated FP32 solve)
constexpr int kFxScaleBits = 36;
constexpr double kFxPartMax = 549755813888.0;   // 2^39
constexpr long long kFxTotalMin = 1LL << 30;
constexpr int kFxPartSlot = 96;      // sm[96..103]: the CTA's FP64 partials (sm holds 112)

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_relaxed_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_acq_rel_gpu() {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");
}
// 2^e for e in [-1022, 1023], from the exponent bits
__device__ __forceinline__ double pow2i(int e) {
  return __longlong_as_double(static_cast<long long>(e + 1023) << 52);
}
// round(v 2^sc) for an FP32 v by integer operations (the FP32 solve's CTA
// totals: no FP64 instruction on the reduction's critical path); ok = false
// when the result would reach 2^39 (or v is not finite).  Ties round up in
// magnitude; every CTA and run rounds alike.
__device__ __forceinline__ long long f32_fixed(float v, int sc, bool& ok) {
  const unsigned b = __float_as_uint(v);
  const int e = static_cast<int>((b >> 23) & 0xFFu);
  if (e == 0) return 0;  // zero or subnormal: far below the total's resolution
  const int sh = e - 150 + sc;  // |v| 2^sc = m 2^sh, m < 2^24
  if (e == 0xFF || sh > 15) {
    ok = false;
    return 0;
  }
  const long long m = static_cast<long long>((b & 0x7FFFFFu) | 0x800000u);
  long long r = 0;
  if (sh >= 0)
    r = m << sh;
  else if (sh > -26)
    r = (m + (1LL << (-sh - 1))) >> (-sh);
  return (b >> 31) ? -r : r;
}

// Scale exponent for a total near `prev` (0: none usable)
__device__ __forceinline__ int fx_scale(double prev, bool& usable) {
  const long long bits = __double_as_longlong(prev);
  const int ex = static_cast<int>((bits >> 52) & 0x7FF);
  usable = prev > 0.0 && ex > 64 && ex < 2046 - 64;
  return usable ? kFxScaleBits - (ex - 1023) : 0;
}

// Warp totals of NV <= 8 values with 9 shuffles instead of 5 NV: a butterfly
// that halves the values each lane carries (8 -> 4 -> 2 -> 1 at offsets 16,
// 8, 4), then two plain steps.  Lane L ends with the total of value
// 4 b4 + 2 b3 + b2 (bits of L); the lanes with L % 4 == 0 store it to out.
// The order of the additions is fixed, so the totals are reproducible.
template <int NV, typename TV>
__device__ __forceinline__ void warp_sums_to(const TV (&v)[NV], TV* out) {
  static_assert(NV <= 8, "at most 8 values");
  const int lane = threadIdx.x & 31;
  TV a8[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a8[k] = k < NV ? v[k] : TV(0);
  const bool h4 = (lane & 16) != 0, h3 = (lane & 8) != 0, h2 = (lane & 4) != 0;
  TV a4[4], a2[2];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    a4[k] = (h4 ? a8[k + 4] : a8[k]) + __shfl_xor_sync(0xffffffffu, h4 ? a8[k] : a8[k + 4], 16);
#pragma unroll
  for (int k = 0; k < 2; ++k)
    a2[k] = (h3 ? a4[k + 2] : a4[k]) + __shfl_xor_sync(0xffffffffu, h3 ? a4[k] : a4[k + 2], 8);
  TV a1 = (h2 ? a2[1] : a2[0]) + __shfl_xor_sync(0xffffffffu, h2 ? a2[0] : a2[1], 4);
  a1 += __shfl_xor_sync(0xffffffffu, a1, 2);
  a1 += __shfl_xor_sync(0xffffffffu, a1, 1);
  const int k = (h4 ? 4 : 0) + (h3 ? 2 : 0) + (h2 ? 1 : 0);
  if ((lane & 3) == 0 && k < NV) out[k] = a1;
}

// grid_allreduce for the FP32 solve over the fused words of reduction `red`
// (ring slot red % kFxSlots of kFxWords words, NV of them used): prev[k] > 0 is the previous total
// of value k (<= 0: none, fall back).  CTA 0 clears the slot two reductions
// ahead (its last readers all arrived at the reduction before this one).
// kW as in grid_allreduce.
// kRelease false: the arrival is a relaxed reduction and the wait has no
// acquire fence — for a reduction that publishes nothing but its sums (the
// fixed-point words carry them; GB300 spends ~0.8 us in a release fence
// whose store has yet to reach L2).  The FP64 partials of the fallback sum
// are written only when it is needed (every CTA sees the same words) and
// ordered by a counter barrier (count, target).
// The fx slot cleared two reductions ahead is ordered by the release of the
// reduction in between, so two relaxed reductions must not follow each other.
// FP64 solve (TV = double): each value takes two words, the integer part of
// the scaled CTA partial and its next 32 fraction bits (the low words' sum of
// at most 255 CTAs stays below 2^40), so the total carries ~68 bits below
// the previous total's leading bit and no FP64 partial sum is needed after
// the barrier.
// Values from kMinChk on may fall far below their scale (the deflation dots,
// scaled by a bound): they skip the "total fell more than 64x" fallback.
template <int NV, int kW = kResWarps, bool kRelease = true, int kMinChk = NV, typename TV,
          typename Fin>
__device__ bool grid_allreduce_fx(TV (&v)[NV], const double (&prev)[NV], double* partials,
                                  int slot, unsigned long long* fx, int red, int* abort_flag,
                                  double* sm, int* s_ok, int* s_fb, double* s_tot,
                                  long long spin_limit, unsigned* count, unsigned& target,
                                  Fin&& fin) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // CTA totals in the input type (FP32 solve: FP32 throughout, as its
  // per-thread and per-warp sums are)
  TV* smv = reinterpret_cast<TV*>(sm);
  if (kW > 0) {
    if (wid < kW) {
      if constexpr (NV > 2 && sizeof(TV) == 4) {
        warp_sums_to(v, smv + wid * NV);  // the deflated solve's 6 values
      } else if constexpr (NV == 2 && sizeof(TV) == 8) {
        // FP64 pair: lanes 16-31 carry value 1 and lanes 0-15 value 0 after
        // the first step, so the warp adds 5 times instead of 10 (each
        // warp-wide FP64 add costs the SM ~16 cycles); lane 0 ends with the
        // total of value 0, lane 16 with that of value 1
        const bool hi = (lane & 16) != 0;
        TV keep = hi ? v[1] : v[0];
        keep += __shfl_xor_sync(0xffffffffu, hi ? v[0] : v[1], 16);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) keep += __shfl_xor_sync(0xffffffffu, keep, o);
        if ((lane & 15) == 0) smv[wid * NV + (hi ? 1 : 0)] = keep;
      } else {
#pragma unroll
        for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
        if (lane == 0)
#pragma unroll
          for (int k = 0; k < NV; ++k) smv[wid * NV + k] = v[k];
      }
    }
    __syncthreads();
  }
  double* part = partials + static_cast<size_t>(slot) * gridDim.x * NV;
  constexpr bool kSplit = sizeof(TV) == 8;
  constexpr int kWpv = kSplit ? 2 : 1;  // words per value
  static_assert(NV * kWpv <= kFxWords, "a fused reduction sums at most kFxWords words");
  static_assert(kW * NV <= kFxPartSlot, "warp sums overlap the partial slots");
  unsigned long long* words = fx + static_cast<size_t>(red % kFxSlots) * kFxWords;
  if (wid == 0) {
    TV w[NV];
    if (kW > 0) {
#pragma unroll
      for (int k = 0; k < NV; ++k) w[k] = lane < kW ? smv[lane * NV + k] : TV(0);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
        if (o < kW)
#pragma unroll
          for (int k = 0; k < NV; ++k) w[k] += __shfl_xor_sync(0xffffffffu, w[k], o);
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) w[k] = v[k];
    }
    if (lane == 0) {
      if (blockIdx.x == 0) {
        unsigned long long* ahead = fx + static_cast<size_t>((red + 2) % kFxSlots) * kFxWords;
#pragma unroll
        for (int k = 0; k < kFxWords; ++k) ahead[k] = 0ull;
      }
      int sc[NV];
      bool fx_ok = true;
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        bool u;
        sc[k] = fx_scale(prev[k], u);
        fx_ok = fx_ok && u;
      }
      unsigned long long adds[NV * kWpv];
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        unsigned long long add = 1ull, add_lo = 1ull;
        if (fx_ok) {
          if constexpr (kSplit) {
            const double y = w[k] * pow2i(sc[k]);
            if (fabs(y) < kFxPartMax) {
              const double hi = floor(y);
              add += static_cast<unsigned long long>(static_cast<long long>(hi)) << 16;
              add_lo += static_cast<unsigned long long>(__double2ll_rn((y - hi) * 4294967296.0))
                        << 16;
            } else {
              add += 1ull << 8;
            }
          } else {
            bool in_range = true;
            const long long q = f32_fixed(w[k], sc[k], in_range);
            add += in_range ? static_cast<unsigned long long>(q) << 16 : 1ull << 8;
          }
        }
        adds[kWpv * k] = add;
        if (kSplit) adds[kWpv * k + 1] = add_lo;
      }
      // one fence orders the CTA's writes before all the words' adds (a
      // release per word would wait once per word)
      if (kRelease) fence_acq_rel_gpu();
#pragma unroll
      for (int k = 0; k < NV * kWpv; ++k) red_relaxed_add_u64(words + k, adds[k]);
#pragma unroll
      for (int k = 0; k < NV; ++k) sm[kFxPartSlot + k] = static_cast<double>(w[k]);  // fallback
      // wait for every arrival on every word
      unsigned long long* tm = tmarks();
      if (tm[2]) tm[0] = gtime();
      int ok = 1;
      long long spins = 0;
      unsigned long long got[NV * kWpv];
      for (;;) {
        bool all = true;
#pragma unroll
        for (int k = 0; k < NV * kWpv; ++k) {
          got[k] = ld_relaxed_u64(words + k);
          all = all && (got[k] & 0xFFull) >= gridDim.x;
        }
        if (all) break;
        ++spins;
        if ((spins & 63) == 0 && *reinterpret_cast<volatile int*>(abort_flag)) {
          ok = 0;
          break;
        }
        if (spins > spin_limit) {
          atomicExch(abort_flag, 1);
          ok = 0;
          break;
        }
        if (spins > 4096) __nanosleep(64);
      }
      if (kRelease) fence_acq_rel_gpu();
      if (tm[2]) tm[1] = gtime();
      int fb = fx_ok ? 0 : 1;
#pragma unroll
      for (int k = 0; k < NV; ++k) {
        const unsigned long long g = got[kWpv * k];
        const long long q = static_cast<long long>(g) >> 16;
        if (((g >> 8) & 0xFFull) != 0ull || (k < kMinChk && q < kFxTotalMin && q > -kFxTotalMin))
          fb = 1;
        double t = static_cast<double>(q);
        if (kSplit)
          t += static_cast<double>(got[kWpv * k + 1] >> 16) * (1.0 / 4294967296.0);
        s_tot[k] = t * pow2i(-sc[k]);
      }
      *s_ok = ok;
      *s_fb = fb;
    }
  }
  __syncthreads();
  bool ok = *s_ok != 0;
  const bool fb = *s_fb != 0;
  if (fb && ok) {
    // every CTA takes this branch (the same words): publish the FP64
    // partials behind a counter barrier (no store sits before the fast
    // path's arrival, whose release would wait for it)
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; ++k) part[blockIdx.x * NV + k] = sm[kFxPartSlot + k];
    ok = grid_sync(count, target, abort_flag, s_ok, spin_limit);
  }
  if (threadIdx.x < 32) {
    double acc[NV];
    if (fb) {
      // fixed-order sum of the FP64 partials, as grid_allreduce
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = 0.0;
      for (unsigned c = threadIdx.x; c < gridDim.x; c += 32)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&part[c * NV + k]);
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = warp_sum(acc[k]);
    } else {
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = s_tot[k];
    }
    if (threadIdx.x == 0) fin(acc, ok);
  }
  __syncthreads();
  return ok;
}

// Per-slice sum slots between the own-row vectors and the window: two per
// slice of the largest CTA range (rows_max = 24 * max_slices) — p.Ap and, for
// an error-controlled solve, p.Mp (stored as T) — padded so the window stays
// 16/32-byte aligned.
__host__ __device__ __forceinline__ int slot_half(int rows_max) {
  const int s = ((rows_max / 24) + 3) & ~3;
  return s > kResWarps ? s : kResWarps;  // per-warp sums of the FP64 solve
}
__host__ __device__ __forceinline__ int slot_count(int rows_max) { return 2 * slot_half(rows_max); }

__device__ __forceinline__ float rfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return fma(a, b, c); }

// Three components of a node-padded vector (4 per node, 16/32-byte aligned),
// read through L2 (other CTAs wrote them before the last grid barrier).
__device__ __forceinline__ void ld3(const float* p, float& a, float& b, float& c) {
  const float4 v = __ldcg(reinterpret_cast<const float4*>(p));
  a = v.x;
  b = v.y;
  c = v.z;
}
__device__ __forceinline__ void ld3(const double* p, double& a, double& b, double& c) {
  const double2 v = __ldcg(reinterpret_cast<const double2*>(p));
  a = v.x;
  b = v.y;
  c = __ldcg(p + 2);
}
// Three components of a node of the shared-memory window (one 16-byte load
// for FP32).
__device__ __forceinline__ void lds3(const float* p, float& a, float& b, float& c) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = v.x;
  b = v.y;
  c = v.z;
}
__device__ __forceinline__ void lds3(const double* p, double& a, double& b, double& c) {
  const double2 v = *reinterpret_cast<const double2*>(p);
  a = v.x;
  b = v.y;
  c = p[2];
}
__device__ __forceinline__ void st3(float* p, float a, float b, float c) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, 0.f);
}
__device__ __forceinline__ void st3(double* p, double a, double b, double c) {
  *reinterpret_cast<double2*>(p) = make_double2(a, b);
  p[2] = c;
}

// z = B r for one node, B the symmetric inverse of its diagonal block stored
// as its upper triangle (xx, xy, xz, yy, yz, zz).
template <typename T>
__device__ __forceinline__ void bj_apply(const T* __restrict__ b, const T (&r)[3], T (&z)[3]) {
  const T b0 = __ldg(b), b1 = __ldg(b + 1), b2 = __ldg(b + 2);
  const T b3 = __ldg(b + 3), b4 = __ldg(b + 4), b5 = __ldg(b + 5);
  z[0] = rfma(b0, r[0], rfma(b1, r[1], b2 * r[2]));
  z[1] = rfma(b1, r[0], rfma(b3, r[1], b4 * r[2]));
  z[2] = rfma(b2, r[0], rfma(b4, r[1], b5 * r[2]));
}

// kBJ: 3x3 block Jacobi (z = B_I r_I per node) instead of the scalar one; the
// fourth own-row vector then holds z itself instead of diag^-1, and the row
// loops of the init and of phase 2 run over nodes.
// kDM > 0 (FP32 mixed, scalar Jacobi, window): deflated PCG (Saad, Yeung,
// Erhel & Guyomarc'h 2000) with kDM coarse vectors W: the start residual is
// W-orthogonal (the coarse correction before the solve) and every direction
// is made A-orthogonal to W, p = z + beta p - W mu, mu = (W^T A W)^-1 (A W)^T z.
// The window carries the undeflated recurrence q = z + beta q instead, so
// that no CTA needs W beyond its own rows: p = q - W nu with nu = mu + beta nu
// (kDM scalars), and A p = A q - (A W) nu on the own rows, whose W and A W
// sit in shared memory.  The dots (A W)^T z ride on the second reduction.
template <typename T, bool kWindow, bool kMixed, bool kBJ, int kDM>
__global__ void __launch_bounds__(kResThreads, 1) k_resident_pcg(ResArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[112];
  __shared__ int s_ok;
  __shared__ int s_fb;         // fused reduction fell back to the partials
  __shared__ double s_tot[6];  // totals of a fused reduction
  __shared__ float s_nu[kDM > 0 ? kDM : 1];  // deflation coefficients of the direction
  __shared__ int s_next;  // next slice handed to a warp in phase 1
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = blockIdx.x;
  const int s0 = a.cta_slice[c], s1 = a.cta_slice[c + 1], ns = s1 - s0;
  const int g0 = 24 * s0;
  const int nrows = max(0, min(24 * s1, a.n) - g0);
  // Own-row vectors r, p, Ap, diag^-1 (and the solution accumulator u unless
  // it lives in global memory; z = r diag^-1 is recomputed where needed).
  // With kBJ the diag^-1 slot holds z.
  T* RR = reinterpret_cast<T*>(smem);
  T* P = RR + a.rows_max;
  T* AP = P + a.rows_max;
  T* D = AP + a.rows_max;
  T* U = a.u_glob ? a.u_glob + g0 : D + a.rows_max;
  T* SL = D + (a.u_glob ? 1 : 2) * a.rows_max;  // per-slice p.Ap sums (slices are handed out dynamically)
  T* SLm = SL + slot_half(a.rows_max);           // per-slice p.Mp sums (error-controlled solve)
  T* win = SL + slot_count(a.rows_max);  // 4 per node when kWindow
  // deflated solve: A W and W of the own rows (kDM x rows_max each)
  float* AWs = reinterpret_cast<float*>(win + a.win_words);
  float* WOs = AWs + kDM * a.rows_max;
  const bool err_on = a.err_mode != kErrOff;
  // Phase 2 (u, r, z and the r.z, r.r partials): all warps in the FP32
  // solve; in the FP64 solve kP2Warps of them, which keep the FP64 pipe as
  // busy (the phase is bound by it) and leave a quarter of the warp sums for
  // the reduction.
  constexpr int kP2Warps = sizeof(T) == 8 ? 8 : kResWarps;
  constexpr int kP2Threads = 32 * kP2Warps;
  const int wb = a.cta_win[2 * c], we = a.cta_win[2 * c + 1];
  // referenced runs of the window: starts and cumulative lengths
  __shared__ int s_rs[kWinRuns], s_rc[kWinRuns + 1], s_nrun;
  if (kWindow && tid == 0) {
    const int* rr = a.cta_runs + static_cast<size_t>(c) * kRunStride;
    const int nr = min(max(rr[0], 0), kWinRuns);
    int acc = 0;
    s_rc[0] = 0;
    for (int i = 0; i < nr; ++i) {
      s_rs[i] = rr[1 + 2 * i];
      acc += rr[2 + 2 * i] - rr[1 + 2 * i];
      s_rc[i + 1] = acc;
    }
    s_nrun = nr;
  }
  unsigned target = 0;
  int slot = 0;
  bool ok = true;
  const double scale = kMixed ? a.O->scale : 1.0;

  // ── init: r = rhs, u = 0, z = r / diag, p = 0 ──
  T acc2[2 + kDM] = {};
  if (kBJ) {
    for (int ln = tid; 3 * ln < nrows; ln += kResThreads) {
      const int lr = 3 * ln, R = 8 * s0 + ln;
      T rv[3], zv[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double f = a.rhs[g0 + lr + q];
        rv[q] = kMixed ? static_cast<T>(f * scale) : static_cast<T>(f);
      }
      bj_apply(a.bj + 6 * static_cast<size_t>(R), rv, zv);
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        RR[lr + q] = rv[q];
        U[lr + q] = T(0);
        P[lr + q] = T(0);
        AP[lr + q] = T(0);
        D[lr + q] = zv[q];
        acc2[0] = rfma(rv[q], rv[q], acc2[0]);
        acc2[1] = rfma(rv[q], zv[q], acc2[1]);
      }
      st3(a.z4 + 4 * static_cast<size_t>(R), zv[0], zv[1], zv[2]);
      if (kMixed && a.hist)
#pragma unroll
        for (int q = 0; q < 3; ++q) a.hist[4 * static_cast<size_t>(R) + q] = static_cast<float>(zv[q]);
      st3(a.p4a + 4 * static_cast<size_t>(R), T(0), T(0), T(0));
      st3(a.p4b + 4 * static_cast<size_t>(R), T(0), T(0), T(0));
    }
  }
  for (int lr = tid; !kBJ && lr < nrows; lr += kResThreads) {
    const int g = g0 + lr;
    const int R = g / 3, q = g - 3 * R;
    const double d = a.dinv[g];
    const T rv = kMixed ? static_cast<T>(a.rhs[g] * scale) : static_cast<T>(a.rhs[g]);
    const T dv = static_cast<T>(d);
    const T zv = rv * dv;
    RR[lr] = rv;
    U[lr] = T(0);
    P[lr] = T(0);
    AP[lr] = T(0);
    D[lr] = dv;
    a.z4[4 * R + q] = zv;
    if (kMixed && a.hist) a.hist[4 * R + q] = static_cast<float>(zv);
    if constexpr (kDM > 0) {
#pragma unroll
      for (int i = 0; i < kDM; ++i) {
        const float w = __ldg(a.defl_aw + static_cast<size_t>(i) * a.n + g);
        AWs[i * a.rows_max + lr] = w;
        WOs[i * a.rows_max + lr] = __ldg(a.defl_w + (static_cast<size_t>(i) * a.nb + R) * 4 + q);
        acc2[2 + i] = rfma(w, zv, acc2[2 + i]);
      }
    }
    a.p4a[4 * R + q] = T(0);
    a.p4b[4 * R + q] = T(0);
    acc2[0] = rfma(rv, rv, acc2[0]);
    acc2[1] = rfma(rv, zv, acc2[1]);
  }
  if (kWindow && kKeepWindowP)  // p_{-1} = 0 over the window
    for (int j = tid; j <= we - wb; j += kResThreads) st3(win + 4 * j, T(0), T(0), T(0));
  // The scalar recurrence runs on thread 0 only (FP64 sqrt / division are long
  // instruction sequences on GB300's FP64 pipe), inside the reductions, and is
  // broadcast through shared memory: s_sc = {alpha, beta}.
  __shared__ double s_sc[2];
  __shared__ int s_flags;
  // Recurrence scalars: thread 0 only, in shared memory so that they hold no
  // registers of the other threads across the SpMV.
  __shared__ double norm_b, rz, rel, pAp, rr, beta, alpha, rr_stop, pMp;
  // Error-controlled stop: the Hestenes-Stiefel estimate (errest.cuh) and its
  // targets, thread 0 only (every CTA computes the same values).
  __shared__ ErrEst s_err;
  __shared__ double s_err_t2, s_err_rel2;
  // Deflation: (W^T A W)^-1, the bounds c_i and the dots (A W)^T z of the
  // last reduction, which thread 0 leaves for kDeflThread
  __shared__ float s_ginv[kDM > 0 ? kDM * kDM : 1];
  __shared__ float s_dc[kDM > 0 ? kDM : 1];
  __shared__ double s_dt[kDM > 0 ? kDM : 1];
  __shared__ double s_dsc[kDM > 0 ? kDM : 1];  // c_i sqrt(r.z): scales of the next dots
  if constexpr (kDM > 0) {
    if (tid == kDeflThread) {
      for (int i = 0; i < kDM * kDM; ++i) s_ginv[i] = a.defl_ginv[i];
      for (int i = 0; i < kDM; ++i) {
        s_dc[i] = static_cast<float>(a.defl_c[i]);
        s_nu[i] = 0.f;
      }
    }
  }
  // kDeflThread, in phase 1 (off thread 0's scalar path; the SpMV that needs
  // nu follows the phase's barrier): mu = (W^T A W)^-1 (A W)^T z,
  // nu = mu + beta nu (the direction is p = q - W nu) and the scales of the
  // next dots from r.z
  auto defl_next = [&]() {
    if constexpr (kDM > 0) {
      float tf[kDM];
#pragma unroll
      for (int j = 0; j < kDM; ++j) tf[j] = static_cast<float>(s_dt[j]);
      const float sr = sqrtf(fabsf(static_cast<float>(rz)));
      const float tbn = static_cast<float>(s_sc[1]);
#pragma unroll
      for (int i = 0; i < kDM; ++i) {
        float mu = 0.f;
#pragma unroll
        for (int j = 0; j < kDM; ++j) mu = fmaf(s_ginv[i * kDM + j], tf[j], mu);
        s_nu[i] = fmaf(tbn, s_nu[i], mu);
        s_dsc[i] = static_cast<double>(s_dc[i] * sr);
      }
    }
  };
  if (tid == 0) {
    norm_b = rz = pAp = rr = beta = alpha = rr_stop = pMp = 0.0;
    rel = 1.0;
    tmarks()[2] = a.trace != nullptr ? 1ull : 0ull;
    err_reset(s_err);
    s_err_t2 = 0.0;
    s_err_rel2 = a.err_rel * a.err_rel;
    if (a.err_mode == kErrAbsolute) {
      // the inner solve's unknown is scale * (correction of u): its error
      // target is scale * err_target * ||u||_D of the outer iterate
      const double t = a.err_target * scale;
      s_err_t2 = t * t * (kMixed ? a.O->uD2 : 0.0);
    }
  }
  int flags = 0, it = 0;
  int fx_red = 0;  // fused reductions done (FP32)
  T* p_old = a.p4a;
  T* p_new = a.p4b;
  ok = grid_allreduce<T, 2 + kDM>(acc2, a.partials, slot, a.count, target, a.abort_flag, red,
                                  &s_ok, a.spin_limit, [&](const double (&t)[2 + kDM], bool good) {
                              if constexpr (kDM > 0) {
                                for (int j = 0; j < kDM; ++j) s_dt[j] = t[2 + j];
                              }
                              norm_b = sqrt(fabs(t[0]));
                              rz = t[1];
                              rr = t[0];
                              if (kMixed && a.coef && blockIdx.x == 0) a.coef[2] = rz;
                              rr_stop = (a.tol * norm_b) * (a.tol * norm_b);
                              if (!good) {
                                flags = kFlagDone | kFlagAbort;
                              } else if (norm_b < 1e-300) {
                                flags = kFlagDone | kFlagZeroRhs | kFlagConverged;
                                rel = 0.0;
                              } else if (!(rz > 0.0)) {
                                flags = kFlagDone | kFlagNonPosRz;
                              }
                              s_flags = flags;
                              s_sc[1] = 0.0;
                            });
  slot ^= 1;
  flags = s_flags;

  // phase timer, thread 0 only: tick(k) closes phase k; a reduction's time
  // is split at its arrival and release marks
  const bool tr = a.trace != nullptr && tid == 0;
  __shared__ unsigned long long tsum[kTracePhases];  // thread 0's sums (no registers held)
  __shared__ unsigned long long tmark;
  if (tid == 0) {
    tmarks()[2] = tr ? 1ull : 0ull;
    for (int k = 0; k < kTracePhases; ++k) tsum[k] = 0ull;
    tmark = 0ull;
  }
  auto tick = [&](int k) {
    if (tr) {
      const unsigned long long t = gtime();
      if (k >= 0) tsum[k] += t - tmark;
      tmark = t;
    }
  };
  auto tick_red = [&](int k) {  // closes a reduction: phases k, k+1, k+2
    if (tr) {
      const unsigned long long t = gtime(), *m = tmarks();
      tsum[k] += m[0] - tmark;
      tsum[k + 1] += m[1] - m[0];
      tsum[k + 2] += t - m[1];
      tmark = t;
    }
  };
  while (!(flags & kFlagDone)) {
    // ── phase 1: x = z + beta p over the window, Ap = K x, own p update ──
    tick(-1);
    const T tb = static_cast<T>(s_sc[1]);
    if (tid == 0) s_next = kResWarps;
    if (kDM > 0 && tid == kDeflThread) defl_next();
    if (!kWindow) __syncthreads();
    if (kWindow) {
      // kFill nodes per thread per round: all their loads are in flight
      // together (one L2 round trip per round instead of one per node).
      // With kKeepWindowP the window already holds p_k of every window node
      // (each CTA forms p = z + beta p for them with the operands and order of
      // the owner, so the copies are bitwise the owner's): only z is read.
      // Only the runs of the window that the CTA's columns reference
      // (k_window_runs): entry t of their concatenation is node
      // s_rs[i] + t - s_rc[i] of run i.
      constexpr int kFill = 4;
      const int total = s_rc[s_nrun];
      for (int t0 = tid; t0 < total; t0 += kFill * kResThreads) {
        T z[kFill][3], q[kFill][3];
        int jj[kFill];
#pragma unroll
        for (int u = 0; u < kFill; ++u) {
          const int t = t0 + u * kResThreads;
          int j = -1;
          if (t < total) {
            int i = 0;
            while (t >= s_rc[i + 1]) ++i;
            j = s_rs[i] + (t - s_rc[i]);
          }
          jj[u] = j;
          if (j >= 0) {
            ld3(a.z4 + 4 * static_cast<size_t>(j), z[u][0], z[u][1], z[u][2]);
            if (kKeepWindowP)
              lds3(win + 4 * (j - wb), q[u][0], q[u][1], q[u][2]);
            else
              ld3(p_old + 4 * static_cast<size_t>(j), q[u][0], q[u][1], q[u][2]);
          }
        }
#pragma unroll
        for (int u = 0; u < kFill; ++u) {
          const int j = jj[u];
          if (j >= 0)
            st3(win + 4 * (j - wb), rfma(tb, q[u][0], z[u][0]), rfma(tb, q[u][1], z[u][1]),
                rfma(tb, q[u][2], z[u][2]));
        }
      }
      __syncthreads();
    }
    tick(0);
    T accp[1] = {T(0)};
    // FP32: slices are handed out dynamically (first one per warp
    // statically), so warps that drew short slices take more and the phase
    // ends together; the p.Ap of each slice is then stored by slice, so the
    // CTA sum is in slice order whichever warp computed it.  FP64: the SpMV
    // is bound by the FP64 pipe, where the per-slice warp sum (5 FP64 adds of
    // the whole warp) is a tenth of the slice's work; the slices go to the
    // warps round-robin instead and each lane accumulates its p.Ap across
    // them, one warp sum per warp at the end (fixed order either way).
    constexpr bool kStatic = sizeof(T) == 8;
    T part_acc = T(0);
    float partm_acc = 0.f;
    for (int lq = warp; lq < ns;) {
      // kSnake: odd iterations walk the CTA's slices backwards, so the lines
      // touched last (most likely still in L2) are read first
      const int ls = (kSnake && (it & 1)) ? ns - 1 - lq : lq;
      const int sl = s0 + ls;
      const int base = a.slice_ptr[sl], steps = a.slice_ptr[sl + 1] - base;
      const int* cp = a.cols + static_cast<size_t>(base) * 32 + lane;
      const T* vp = a.vals + static_cast<size_t>(base) * 288 + lane;
      T y0 = T(0), y1 = T(0), y2 = T(0);
      // FP32: the operator is in difference form (the diagonal slot holds the
      // block-row sum): non-diagonal blocks multiply x_J - x_I.
      constexpr bool kDiff = sizeof(T) == 4;
      const int Rrow = 8 * sl + (lane >> 2);
      T i0 = T(0), i1 = T(0), i2 = T(0);
      if (kDiff && Rrow < a.nb) {
        if (kWindow) {
          // the diagonal block column is one of the slice's columns, so it
          // lies in the window; the test only guards the shared-memory read
          if (Rrow >= wb && Rrow <= we) lds3(win + 4 * (Rrow - wb), i0, i1, i2);
        } else {
          T z0, z1, z2, q0, q1, q2;
          ld3(a.z4 + 4 * static_cast<size_t>(Rrow), z0, z1, z2);
          ld3(p_old + 4 * static_cast<size_t>(Rrow), q0, q1, q2);
          i0 = rfma(tb, q0, z0);
          i1 = rfma(tb, q1, z1);
          i2 = rfma(tb, q2, z2);
        }
      }
      // Up to kAhead steps of operator loads are issued before any of them is
      // consumed, so each warp keeps ~kAhead*40 B (FP32) per lane in flight.
      constexpr int kAhead = sizeof(T) == 4 ? 4 : 2;
      for (int t0 = 0; t0 < steps; t0 += kAhead) {
        int col[kAhead];
        T v[kAhead][9];
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
          if (t0 + u < steps) {
            col[u] = __ldcg(cp + 32 * (t0 + u));
#pragma unroll
            for (int k = 0; k < 9; ++k) v[u][k] = __ldcg(vp + 288 * (t0 + u) + 32 * k);
          }
        }
#pragma unroll
        for (int u = 0; u < kAhead; ++u) {
          if (t0 + u < steps) {
            T x0, x1, x2;
            if (kWindow) {
              lds3(win + 4 * (col[u] - wb), x0, x1, x2);
            } else {
              T z0, z1, z2, q0, q1, q2;
              ld3(a.z4 + 4 * static_cast<size_t>(col[u]), z0, z1, z2);
              ld3(p_old + 4 * static_cast<size_t>(col[u]), q0, q1, q2);
              x0 = rfma(tb, q0, z0);
              x1 = rfma(tb, q1, z1);
              x2 = rfma(tb, q2, z2);
            }
            if (kDiff) {
              const T m = col[u] != Rrow ? T(1) : T(0);
              x0 = rfma(-m, i0, x0);
              x1 = rfma(-m, i1, x1);
              x2 = rfma(-m, i2, x2);
            }
            y0 = rfma(v[u][0], x0, rfma(v[u][1], x1, rfma(v[u][2], x2, y0)));
            y1 = rfma(v[u][3], x0, rfma(v[u][4], x1, rfma(v[u][5], x2, y1)));
            y2 = rfma(v[u][6], x0, rfma(v[u][7], x1, rfma(v[u][8], x2, y2)));
          }
        }
      }
      const int r = lane >> 2, q = lane & 3;
      T yq;
      if constexpr (sizeof(T) == 8) {
        // The row's 4 lanes hold partials of its 3 components.  A butterfly
        // that halves the values each lane carries leaves lane q with the
        // total of component q in 3 FP64 adds instead of the 6 of a
        // reduction of all three (every FP64 warp instruction costs the SM
        // ~16 cycles whatever its active lanes): over lanes xor 2, lanes 0-1
        // keep components 0-1 and lanes 2-3 component 2 (and a zero), then
        // over lanes xor 1 each lane keeps one.
        const bool h = (lane & 2) != 0, b = (lane & 1) != 0;
        T k0 = h ? y2 : y0, k1 = h ? T(0) : y1;
        const T s0 = h ? y0 : y2, s1 = h ? y1 : T(0);
        k0 += __shfl_xor_sync(0xffffffffu, s0, 2);
        k1 += __shfl_xor_sync(0xffffffffu, s1, 2);
        yq = b ? k1 : k0;
        yq += __shfl_xor_sync(0xffffffffu, b ? k0 : k1, 1);
      } else {
#pragma unroll
        for (int o = 1; o <= 2; o <<= 1) {
          y0 += __shfl_xor_sync(0xffffffffu, y0, o);
          y1 += __shfl_xor_sync(0xffffffffu, y1, o);
          y2 += __shfl_xor_sync(0xffffffffu, y2, o);
        }
        yq = q == 0 ? y0 : (q == 1 ? y1 : y2);
      }
      const int R = 8 * sl + r;
      T part = T(0);
      float pf = 0.f;
      if (q < 3 && R < a.nb) {
        const int lr = 24 * ls + 3 * r + q;
        // z = r diag^-1 (or the stored block Jacobi z), as in z4
        T pn, apn = yq;
        if constexpr (kDM > 0) {
          // the window holds q (own rows lie in it): p = q - W nu, Ap = Aq - (A W) nu
          pn = win[4 * (R - wb) + q];
#pragma unroll
          for (int i = 0; i < kDM; ++i) {
            const float nu = s_nu[i];
            pn = fmaf(-nu, WOs[i * a.rows_max + lr], pn);
            apn = fmaf(-nu, AWs[i * a.rows_max + lr], apn);
          }
        } else {
          pn = rfma(tb, P[lr], kBJ ? D[lr] : RR[lr] * D[lr]);
        }
        P[lr] = pn;
        AP[lr] = apn;
        if (!(kWindow && kKeepWindowP)) p_new[4 * R + q] = pn;
        part = pn * apn;
        pf = static_cast<float>(pn);
      }
      // p.Mp for the error estimate, in FP32 (an estimate needs no more):
      // M = the Jacobi diagonal, or the node's 3x3 diagonal block, whose
      // three rows sit on lanes 4r..4r+2
      float partm = 0.f;
      if (err_on) {
        if (kBJ) {
          const int g4 = lane & ~3;
          const float p0 = __shfl_sync(0xffffffffu, pf, g4);
          const float p1 = __shfl_sync(0xffffffffu, pf, g4 + 1);
          const float p2 = __shfl_sync(0xffffffffu, pf, g4 + 2);
          if (q < 3 && R < a.nb) {
            const float* bd = a.bjd32 + 6 * static_cast<size_t>(R);
            const float k0 = __ldg(bd + (q == 0 ? 0 : (q == 1 ? 1 : 2)));
            const float k1 = __ldg(bd + (q == 0 ? 1 : (q == 1 ? 3 : 4)));
            const float k2 = __ldg(bd + (q == 0 ? 2 : (q == 1 ? 4 : 5)));
            partm = pf * fmaf(k0, p0, fmaf(k1, p1, k2 * p2));
          }
        } else if (q < 3 && R < a.nb) {
          partm = pf * pf * __ldg(a.diag32 + 24 * static_cast<size_t>(sl) + 3 * r + q);
        }
        if (!kStatic) partm = warp_sum(partm);
      }
      if (kStatic) {
        part_acc += part;
        partm_acc += partm;
        lq += kResWarps;
        continue;
      }
      part = warp_sum(part);
      int nxt = 0;
      if (lane == 0) {
        SL[ls] = part;
        if (err_on) SLm[ls] = static_cast<T>(partm);
        nxt = atomicAdd(&s_next, 1);
      }
      lq = __shfl_sync(0xffffffffu, nxt, 0);
    }
    if (kStatic) {
      part_acc = warp_sum(part_acc);
      if (err_on) partm_acc = warp_sum(partm_acc);
      if (lane == 0) {
        SL[warp] = part_acc;
        if (err_on) SLm[warp] = static_cast<T>(partm_acc);
      }
    }
    // p.Ap (and p.Mp) of the CTA in slice order (FP64: in warp order),
    // whichever warp computed each slice.
    __syncthreads();
    tick(1);
    T accm = T(0);
    if (warp == 0) {
      T s = T(0), sm = T(0);
      const int nsum = kStatic ? kResWarps : ns;
      for (int k = lane; k < nsum; k += 32) {
        s += SL[k];
        if (err_on) sm += SLm[k];
      }
      s = warp_sum(s);
      if (err_on) sm = warp_sum(sm);
      if (lane == 0) {
        accp[0] = s;
        accm = sm;
      }
    }
    auto fin1 = [&](double pApv, double pMpv, bool good) {
      pAp = pApv;
      if (!good) {
        flags |= kFlagDone | kFlagAbort;
      } else if (!(pAp > 0.0)) {
        flags |= kFlagDone | kFlagBreakdown;
      } else {
        double rp;  // 1 / pAp
        if (kFastScalars32 && sizeof(T) == 4) {
          alpha = static_cast<double>(static_cast<float>(rz) / static_cast<float>(pAp));
          rp = static_cast<double>(__frcp_rn(static_cast<float>(pAp)));
        } else {
          rp = rcp_nr2(pAp);
          alpha = div_nr(rz, pAp, rp);
        }
        if (err_on) {
          pMp = pMpv;
          err_record(s_err, rz * alpha, pMp * rp);
        }
        if (kMixed && a.coef && blockIdx.x == 0 && it < a.hist_max) a.coef[3 * it] = alpha;
      }
      s_flags = flags;
      s_sc[0] = alpha;
    };
    auto fin1a = [&](const double (&t)[1], bool good) { fin1(t[0], 0.0, good); };
    auto fin1b = [&](const double (&t)[2], bool good) { fin1(t[0], t[1], good); };
    // The first reduction publishes nothing but its sums (relaxed arrival,
    // grid_allreduce_fx); without the fused words, the counter barrier.
    if (err_on) {
      T accb[2] = {accp[0], accm};
      if (a.fx) {
        const double prev[2] = {pAp, pMp};
        ok = grid_allreduce_fx<2, 0, false>(accb, prev, a.partials, slot, a.fx, fx_red++,
                                            a.abort_flag, red, &s_ok, &s_fb, s_tot,
                                            a.spin_limit, a.count, target, fin1b);
      } else {
        ok = grid_allreduce<T, 2, 0>(accb, a.partials, slot, a.count, target, a.abort_flag, red,
                                     &s_ok, a.spin_limit, fin1b);
      }
    } else if (a.fx) {
      const double prev[1] = {pAp};
      ok = grid_allreduce_fx<1, 0, false>(accp, prev, a.partials, slot, a.fx, fx_red++,
                                          a.abort_flag, red, &s_ok, &s_fb, s_tot, a.spin_limit,
                                          a.count, target, fin1a);
    } else {
      ok = grid_allreduce<T, 1, 0>(accp, a.partials, slot, a.count, target, a.abort_flag, red,
                                   &s_ok, a.spin_limit, fin1a);
    }
    slot ^= 1;
    flags = s_flags;
    tick_red(2);
    if (flags & kFlagDone) break;
    const T ta = static_cast<T>(s_sc[0]);
    // ── phase 2: u, r, z updates on the own rows ──
#pragma unroll
    for (int k = 0; k < 2 + kDM; ++k) acc2[k] = T(0);
    if (kBJ) {
      for (int ln = tid; tid < kP2Threads && 3 * ln < nrows; ln += kP2Threads) {
        const int lr = 3 * ln, R = 8 * s0 + ln;
        T rv[3], zv[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          U[lr + q] = rfma(ta, P[lr + q], U[lr + q]);
          rv[q] = rfma(-ta, AP[lr + q], RR[lr + q]);
        }
        bj_apply(a.bj + 6 * static_cast<size_t>(R), rv, zv);
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          RR[lr + q] = rv[q];
          D[lr + q] = zv[q];
          acc2[0] = rfma(rv[q], zv[q], acc2[0]);
          acc2[1] = rfma(rv[q], rv[q], acc2[1]);
        }
        st3(a.z4 + 4 * static_cast<size_t>(R), zv[0], zv[1], zv[2]);
        if (kMixed && a.hist && it + 1 < a.hist_max) {
          float* h = a.hist + static_cast<size_t>(it + 1) * 4 * a.nb + 4 * static_cast<size_t>(R);
#pragma unroll
          for (int q = 0; q < 3; ++q) h[q] = static_cast<float>(zv[q]);
        }
      }
    }
    auto p2row = [&](int lr) {
      const int g = g0 + lr;
      const int R = g / 3, q = g - 3 * R;
      U[lr] = rfma(ta, P[lr], U[lr]);
      const T rv = rfma(-ta, AP[lr], RR[lr]);
      const T zv = rv * D[lr];
      RR[lr] = rv;
      a.z4[4 * R + q] = zv;
      if (kMixed && a.hist && it + 1 < a.hist_max)
        a.hist[static_cast<size_t>(it + 1) * 4 * a.nb + 4 * R + q] = static_cast<float>(zv);
      if constexpr (kDM > 0) {
#pragma unroll
        for (int i = 0; i < kDM; ++i) acc2[2 + i] = rfma(AWs[i * a.rows_max + lr], zv, acc2[2 + i]);
      }
      acc2[0] = rfma(rv, zv, acc2[0]);
      acc2[1] = rfma(rv, rv, acc2[1]);
    };
    // (the deflated form is kept rolled: unrolled, its extra dots spill)
    if constexpr (kDM > 0) {
#pragma unroll 1
      for (int lr = tid; lr < nrows; lr += kP2Threads) p2row(lr);
    } else {
      for (int lr = tid; !kBJ && tid < kP2Threads && lr < nrows; lr += kP2Threads) p2row(lr);
    }
    ++it;
    tick(5);
    auto fin2 = [&](const double (&t)[2 + kDM], bool good) {
      if (!good) {
        flags |= kFlagDone | kFlagAbort;
      } else {
        rr = t[1];
        bool conv;
        if (err_on) {
          // Error-controlled: the residual test is not used; the solve stops
          // when two consecutive blocks' estimates meet the target, or when
          // the residual is zero to working precision.
          conv = err_block_end(s_err, s_err_t2, s_err_rel2);
          bool met = conv && (a.err_mode == kErrRelative ||
                              (s_err.est2 <= s_err_t2 && s_err.lag2 <= s_err_t2));
          // residual at working-precision zero: converged (an FP32 refinement
          // step then leaves the decision to the next step's estimate)
          if (!(fabs(rr) > (sizeof(T) == 4 ? 1e-20 : 1e-28) * norm_b * norm_b)) {
            conv = true;
            met = met || sizeof(T) == 8;
          }
          if (met) flags |= kFlagErrTarget;
        } else {
          // rel < tol as rr < (tol |b|)^2 (no square root or division on the
          // critical path); rel itself at the exit
          conv = fabs(rr) < rr_stop;
        }
        if (conv) {
          flags |= kFlagDone | kFlagConverged;
          beta = 0.0;
        } else {
          beta = kFastScalars32 && sizeof(T) == 4
                     ? static_cast<double>(static_cast<float>(t[0]) / static_cast<float>(rz))
                     : div_nr(t[0], rz, rcp_nr2(rz));
          if (it >= a.max_iters) flags |= kFlagDone | kFlagMaxIters;
        }
        if (kMixed && a.coef && blockIdx.x == 0 && it < a.hist_max) {
          a.coef[3 * (it - 1) + 1] = beta;  // it was incremented before the reduction
          a.coef[3 * it + 2] = t[0];
        }
        rz = t[0];
        if constexpr (kDM > 0) {
          for (int j = 0; j < kDM; ++j) s_dt[j] = t[2 + j];
        }
      }
      s_flags = flags;
      s_sc[1] = beta;
    };
    constexpr int kW2 = sizeof(T) == 4 ? kResWarps : kP2Warps;  // warps holding partials
    if (a.fx) {
      double prev[2 + kDM];
      prev[0] = rz;
      prev[1] = rr;
      // the deflation dots: |(A w_i).z| <= c_i sqrt(r.z) sets their scale
#pragma unroll
      for (int i = 0; i < kDM; ++i) prev[2 + i] = s_dsc[i];
      ok = grid_allreduce_fx<2 + kDM, kW2, true, 2>(acc2, prev, a.partials, slot, a.fx, fx_red++,
                                                    a.abort_flag, red, &s_ok, &s_fb, s_tot,
                                                    a.spin_limit, a.count, target, fin2);
    } else {
      ok = grid_allreduce<T, 2 + kDM, kW2>(acc2, a.partials, slot, a.count, target, a.abort_flag,
                                           red, &s_ok, a.spin_limit, fin2);
    }
    slot ^= 1;
    flags = s_flags;
    tick_red(6);
    if (flags & kFlagAbort) break;
    T* t = p_old;
    p_old = p_new;
    p_new = t;
  }

  if (tr) {
    for (int k = 0; k < kTracePhases; ++k) a.trace[kTraceWords * c + k] = tsum[k];
    a.trace[kTraceWords * c + kTracePhases] = static_cast<unsigned long long>(it);
  }
  // ── results ──
  if (!(flags & kFlagAbort)) {
    const double inv_scale = kMixed ? 1.0 / scale : 1.0;
    for (int lr = tid; lr < nrows; lr += kResThreads) {
      const int g = g0 + lr;
      if (kMixed)
        a.u_out[g] = fma(static_cast<double>(U[lr]), inv_scale, a.u_out[g]);
      else
        a.u_out[g] = static_cast<double>(U[lr]);
    }
  }
  if (c == 0 && tid == 0) {
    if (norm_b > 1e-300) rel = sqrt(fabs(rr)) / norm_b;
    a.S->err2 = s_err.est2 >= 0.0 && s_err.lag2 >= 0.0 ? fmax(s_err.est2, s_err.lag2) : -1.0;
    a.S->total2 = s_err.total2;
    a.S->iter = it;
    a.S->rel = rel;
    a.S->rr = rr;
    a.S->rz = rz;
    a.S->pAp = pAp;
    a.S->norm_b = norm_b;
    a.S->beta = beta;
    a.S->flags = flags;
  }
}

// Padding slots point at a column inside the slice's own range (values are
// zero), so every column read stays inside the CTA window.
__global__ void k_fix_padding(int nb, int nslices, const int* __restrict__ slice_ptr,
                              const int* __restrict__ rowlen, int* __restrict__ cols) {
  const int sl = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (sl >= nslices) return;
  const int lane = threadIdx.x & 31, r = lane >> 2, q = lane & 3;
  const int R = 8 * sl + r;
  const int len = R < nb ? rowlen[R] : 0;
  for (int t = 0; t < slice_ptr[sl + 1] - slice_ptr[sl]; ++t)
    if (4 * t + q >= len) cols[(static_cast<size_t>(slice_ptr[sl]) + t) * 32 + lane] = 8 * sl;
}

__global__ void k_slice_minmax(int nslices, const int* __restrict__ slice_ptr,
                               const int* __restrict__ cols, int* __restrict__ mm) {
  const int sl = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (sl >= nslices) return;
  const int lane = threadIdx.x & 31;
  int lo = INT_MAX, hi = -1;
  for (int t = 0; t < slice_ptr[sl + 1] - slice_ptr[sl]; ++t) {
    const int c = cols[(static_cast<size_t>(slice_ptr[sl]) + t) * 32 + lane];
    lo = min(lo, c);
    hi = max(hi, c);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (lane == 0) {
    mm[2 * sl] = lo;
    mm[2 * sl + 1] = hi;
  }
}

// The runs of a CTA's window that its columns reference: one block per CTA
// marks every column of its slices (padding included: it points at the
// slice's own rows) in a shared-memory bitmap over [wb, we], then thread 0
// turns the bitmap into at most kWinRuns runs, merging runs less than kRunGap
// nodes apart.  On a structured mesh a CTA's rows are a contiguous node range
// that reaches one node plane up and down, so the runs are the three plane
// bands (~2 150 of a 5 700-node window at 84k); the window gather then loads
// only those.  More runs than kWinRuns: the whole window as one run.
// runs[c * kRunStride]: count, then (start, end) node pairs, end exclusive.
__global__ void __launch_bounds__(512)
k_window_runs(const int* __restrict__ slice_ptr, const int* __restrict__ cols,
              const int* __restrict__ cta_slice, const int* __restrict__ cta_win,
              int* __restrict__ runs) {
  extern __shared__ unsigned bm[];
  const int c = blockIdx.x;
  const int wb = cta_win[2 * c], we = cta_win[2 * c + 1];
  const int nw = (we - wb + 1 + 31) >> 5;
  for (int w = threadIdx.x; w < nw; w += blockDim.x) bm[w] = 0u;
  __syncthreads();
  const long long t0 = static_cast<long long>(slice_ptr[cta_slice[c]]) * 32;
  const long long t1 = static_cast<long long>(slice_ptr[cta_slice[c + 1]]) * 32;
  for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x) {
    const int o = cols[t] - wb;
    if (o >= 0 && o <= we - wb) atomicOr(&bm[o >> 5], 1u << (o & 31));
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  int* out = runs + static_cast<size_t>(c) * kRunStride;
  int nr = 0, cs = -1, ce = -1;
  bool over = false;
  for (int w = 0; w < nw && !over; ++w) {
    unsigned b = bm[w];
    while (b) {
      const int lo = __ffs(static_cast<int>(b)) - 1;
      const unsigned above = b | ((1u << lo) - 1u);  // ones through the run
      const int hi = ~above ? __ffs(static_cast<int>(~above)) - 1 : 32;
      const int rs = wb + 32 * w + lo, re = wb + 32 * w + hi;
      if (ce >= 0 && rs - ce <= kRunGap) {
        ce = re;
      } else {
        if (ce >= 0) {
          if (nr == kWinRuns) {
            over = true;
            break;
          }
          out[1 + 2 * nr] = cs;
          out[2 + 2 * nr] = ce;
          ++nr;
        }
        cs = rs;
        ce = re;
      }
      b = hi == 32 ? 0u : (b & ~((1u << hi) - 1u));
    }
  }
  if (!over && ce >= 0) {
    if (nr == kWinRuns) {
      over = true;
    } else {
      out[1 + 2 * nr] = cs;
      out[2 + 2 * nr] = ce;
      ++nr;
    }
  }
  if (over || nr == 0) {
    nr = 1;
    out[1] = wb;
    out[2] = we + 1;
  }
  out[0] = nr;
}

// Thread per node: finds the diagonal block among the node's stored blocks
// (entries 4t+q < rowlen of its slice row; padding comes after them), and
// inverts its symmetric part (upper triangle) by cofactors in FP64.  A block
// is accepted when its leading minors are positive (SPD, Sylvester).
__global__ void k_block_jacobi_inverse(int nb, const int* __restrict__ slice_ptr,
                                       const int* __restrict__ rowlen,
                                       const int* __restrict__ cols,
                                       const double* __restrict__ v64, double* __restrict__ bj64,
                                       float* __restrict__ bj32, float* __restrict__ bjd32,
                                       int* __restrict__ bad) {
  const int R = blockIdx.x * blockDim.x + threadIdx.x;
  if (R >= nb) return;
  const int sl = R >> 3, ln0 = (R & 7) * 4, len = rowlen[R];
  const long long sp = slice_ptr[sl];
  long long at = -1;
  for (int j = 0; j < len && at < 0; ++j) {
    const long long o = (sp + (j >> 2)) * 32 + ln0 + (j & 3);
    if (cols[o] == R) at = (sp + (j >> 2)) * 288 + ln0 + (j & 3);
  }
  if (at < 0) {
    atomicMin(bad, R);
    return;
  }
  const double a00 = v64[at], a01 = v64[at + 32], a02 = v64[at + 64];
  const double a11 = v64[at + 128], a12 = v64[at + 160], a22 = v64[at + 256];
  // the block itself (upper triangle): the preconditioner's norm of the error estimate
  const double blk[6] = {a00, a01, a02, a11, a12, a22};
#pragma unroll
  for (int k = 0; k < 6; ++k) bjd32[6 * static_cast<size_t>(R) + k] = static_cast<float>(blk[k]);
  const double c00 = a11 * a22 - a12 * a12;
  const double c01 = a02 * a12 - a01 * a22;
  const double c02 = a01 * a12 - a02 * a11;
  const double c11 = a00 * a22 - a02 * a02;
  const double c12 = a01 * a02 - a00 * a12;
  const double c22 = a00 * a11 - a01 * a01;
  const double det = a00 * c00 + a01 * c01 + a02 * c02;
  if (!(a00 > 0.0) || !(c22 > 0.0) || !(det > 0.0)) {
    atomicMin(bad, R);
    return;
  }
  const double id = 1.0 / det;
  const double b[6] = {c00 * id, c01 * id, c02 * id, c11 * id, c12 * id, c22 * id};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    bj64[6 * static_cast<size_t>(R) + k] = b[k];
    if (bj32) bj32[6 * static_cast<size_t>(R) + k] = static_cast<float>(b[k]);
  }
}

template <typename T, bool kWindow, bool kMixed>
void launch_resident(const BsrSell& B, ResidentPlan& P, const T* vals, const double* rhs,
                     double* u, PcgScalars* S, const PcgScalars* O, const ResidentCtl& ctl,
                     T* z4, T* p4a, T* p4b, const double* dinv, const T* bj, size_t smem,
                     T* u_glob, cudaStream_t s) {
  ResArgs<T> a;
  a.nb = B.nb;
  a.n = 3 * B.nb;
  a.slice_ptr = B.slice_ptr.ptr;
  a.cols = B.cols.ptr;
  a.vals = vals;
  a.cta_slice = P.cta_slice.ptr;
  a.cta_win = P.cta_win.ptr;
  a.cta_runs = P.cta_runs.ptr;
  a.dinv = dinv;
  a.bj = bj;
  a.rhs = rhs;
  a.u_out = u;
  a.z4 = z4;
  a.p4a = p4a;
  a.p4b = p4b;
  a.partials = P.partials.ptr;
  a.count = P.barrier.ptr;
  // fused reductions: FP32 solve, arrivals counted in 8 bits
  a.fx = (kFusedReductions && P.ctas <= 255) ? P.fx.ptr : nullptr;
  if (a.fx)
    VSGB_CUDA(cudaMemsetAsync(P.fx.ptr, 0, sizeof(unsigned long long) * kFxSlots * kFxWords, s));
  // The abort word lives in the solve's scalar record, which the host reads
  // back after the launch: a CTA that gave up waiting is seen even when CTA 0
  // finished normally.
  a.abort_flag = &S->abort;
  a.S = S;
  a.O = O;
  a.tol = ctl.tol;
  a.max_iters = ctl.max_iters;
  a.rows_max = 24 * P.max_slices;
  a.u_glob = u_glob;
  a.spin_limit = ctl.spin_limit > 0 ? ctl.spin_limit : kDefaultSpinLimit;
  a.err_mode = ctl.err_mode;
  a.err_target = ctl.err_target;
  a.err_rel = ctl.err_rel;
  a.diag32 = P.diag32.ptr;
  a.bjd32 = P.bjd32.ptr;
  a.hist = ctl.hist;
  a.coef = ctl.coef;
  a.hist_max = ctl.hist ? ctl.hist_max : 0;
  a.trace = nullptr;
  if (ctl.trace) {
    P.trace.reserve(static_cast<size_t>(kTraceWords) * P.ctas);
    a.trace = P.trace.ptr;
  }
  if (ctl.err_mode != kErrOff && (bj ? !P.bjd32.ptr : !P.diag32.ptr))
    throw Error(VSGB_ERR_STATE, "error-controlled solve without the preconditioner's diagonal");
  VSGB_CUDA(cudaMemsetAsync(P.barrier.ptr, 0, sizeof(unsigned), s));
  VSGB_CUDA(cudaMemsetAsync(&S->abort, 0, sizeof(int), s));
  void* args[] = {&a};
  a.defl_w = ctl.defl_w;
  a.defl_aw = ctl.defl_aw;
  a.win_words = 4 * P.max_win;
  a.defl_ginv = ctl.defl_ginv;
  a.defl_c = ctl.defl_c;
  const void* fn = bj ? reinterpret_cast<const void*>(k_resident_pcg<T, kWindow, kMixed, true, 0>)
                      : reinterpret_cast<const void*>(k_resident_pcg<T, kWindow, kMixed, false, 0>);
  if (ctl.defl_w && (bj || !P.defl32))
    throw Error(VSGB_ERR_STATE, "deflated solve: needs the FP32 windowed plan, scalar Jacobi");
  if constexpr (kDeflatable<T, kWindow, kMixed>) {
    if (ctl.defl_w) {
      fn = reinterpret_cast<const void*>(k_resident_pcg<T, kWindow, kMixed, false, kDeflVecs>);
      smem += defl_smem(a.rows_max);
    }
  } else {
    if (ctl.defl_w) throw Error(VSGB_ERR_STATE, "deflated solve: needs the FP32 windowed plan");
  }
  VSGB_CUDA(cudaLaunchCooperativeKernel(fn, dim3(P.ctas), dim3(kResThreads), args, smem, s));
}

// Both preconditioner forms of a kernel take the same shared memory; the plan
// holds when both fit one CTA per SM.  The deflated form (more shared memory)
// is optional: *defl says whether it fits too.
template <typename T, bool kWindow, bool kMixed>
bool configure(size_t smem, int rows, int* blocks, bool* defl) {
  const void* fns[2] = {reinterpret_cast<const void*>(k_resident_pcg<T, kWindow, kMixed, false, 0>),
                        reinterpret_cast<const void*>(k_resident_pcg<T, kWindow, kMixed, true, 0>)};
  for (const void* fn : fns) {
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem)) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, fn, kResThreads, smem) !=
            cudaSuccess ||
        *blocks < 1) {
      cudaGetLastError();
      return false;
    }
  }
  *defl = false;
  if constexpr (kDeflatable<T, kWindow, kMixed>) {
    const void* fn =
        reinterpret_cast<const void*>(k_resident_pcg<T, kWindow, kMixed, false, kDeflVecs>);
    int b = 0;
    const size_t sd = smem + defl_smem(rows);
    *defl = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(sd)) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, kResThreads, sd) ==
                cudaSuccess &&
            b >= 1;
    if (!*defl) cudaGetLastError();
  }
  return true;
}

}  // namespace

void resident_prepare(const BsrSell& B, bool need32, int device, int num_sms, ResidentPlan& P,
                      cudaStream_t s) {
  P.ok32 = P.ok64 = false;
  P.defl32 = false;
  if (!B.valid || B.nslices < num_sms) return;
  int coop = 0;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device) != cudaSuccess ||
      !coop) {
    cudaGetLastError();
    return;
  }
  int smem_optin = 0;
  VSGB_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  const int ns = B.nslices, nb = B.nb;
  // Steps per slice (host copy of the block-row lengths from build_bsr).
  std::vector<long long> pre(static_cast<size_t>(ns) + 1, 0);
  for (int sl = 0; sl < ns; ++sl) {
    int mx = 0;
    for (int r = 0; r < 8; ++r) {
      const int R = 8 * sl + r;
      if (R < nb) mx = std::max(mx, B.h_blen[R]);
    }
    pre[sl + 1] = pre[sl] + (mx + 3) / 4 + kSliceWeight;
  }
  const int G = num_sms;
  std::vector<int> cs(static_cast<size_t>(G) + 1, 0);
  for (int g = 1; g < G; ++g) {
    const long long goal = pre[ns] * g / G;
    cs[g] = static_cast<int>(std::lower_bound(pre.begin(), pre.end(), goal) - pre.begin());
    cs[g] = std::max(cs[g], cs[g - 1]);
  }
  cs[G] = ns;
  int max_slices = 0;
  for (int g = 0; g < G; ++g) max_slices = std::max(max_slices, cs[g + 1] - cs[g]);
  // Padding slots -> in-range columns; per-slice column ranges -> CTA windows.
  const int wgrid = (ns + 7) / 8;
  k_fix_padding<<<wgrid, 256, 0, s>>>(nb, ns, B.slice_ptr.ptr, B.rowlen.ptr, B.cols.ptr);
  VSGB_LAUNCH_CHECK();
  P.slice_mm.reserve(2 * static_cast<size_t>(ns));
  k_slice_minmax<<<wgrid, 256, 0, s>>>(ns, B.slice_ptr.ptr, B.cols.ptr, P.slice_mm.ptr);
  VSGB_LAUNCH_CHECK();
  std::vector<int> hmm(2 * static_cast<size_t>(ns));
  VSGB_CUDA(cudaMemcpyAsync(hmm.data(), P.slice_mm.ptr, sizeof(int) * 2 * ns,
                            cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  std::vector<int> win(2 * static_cast<size_t>(G));
  int max_win = 0;
  for (int g = 0; g < G; ++g) {
    int lo = INT_MAX, hi = -1;
    for (int sl = cs[g]; sl < cs[g + 1]; ++sl) {
      lo = std::min(lo, hmm[2 * sl]);
      hi = std::max(hi, hmm[2 * sl + 1]);
    }
    if (hi < lo) lo = hi = 0;
    win[2 * g] = lo;
    win[2 * g + 1] = hi;
    max_win = std::max(max_win, hi - lo + 1);
  }
  P.ctas = G;
  P.threads = kResThreads;
  P.max_slices = max_slices;
  P.max_win = max_win;
  P.cta_slice.reserve(static_cast<size_t>(G) + 1);
  P.cta_win.reserve(2 * static_cast<size_t>(G));
  VSGB_CUDA(cudaMemcpyAsync(P.cta_slice.ptr, cs.data(), sizeof(int) * (G + 1),
                            cudaMemcpyHostToDevice, s));
  VSGB_CUDA(cudaMemcpyAsync(P.cta_win.ptr, win.data(), sizeof(int) * 2 * G,
                            cudaMemcpyHostToDevice, s));
  P.cta_runs.reserve(static_cast<size_t>(kRunStride) * G);
  {
    const size_t bm_bytes = sizeof(unsigned) * ((static_cast<size_t>(max_win) + 31) / 32);
    if (bm_bytes <= 48 * 1024) {
      k_window_runs<<<G, 512, bm_bytes, s>>>(B.slice_ptr.ptr, B.cols.ptr, P.cta_slice.ptr,
                                            P.cta_win.ptr, P.cta_runs.ptr);
      VSGB_LAUNCH_CHECK();
    } else {
      // (a window of more than 393 216 nodes: gather it whole)
      std::vector<int> whole(static_cast<size_t>(kRunStride) * G, 0);
      for (int g = 0; g < G; ++g) {
        whole[static_cast<size_t>(kRunStride) * g] = 1;
        whole[static_cast<size_t>(kRunStride) * g + 1] = win[2 * g];
        whole[static_cast<size_t>(kRunStride) * g + 2] = win[2 * g + 1] + 1;
      }
      VSGB_CUDA(cudaMemcpyAsync(P.cta_runs.ptr, whole.data(), sizeof(int) * whole.size(),
                                cudaMemcpyHostToDevice, s));
      VSGB_CUDA(cudaStreamSynchronize(s));
    }
  }
  P.partials.reserve(2 * static_cast<size_t>(G) * (2 + kDeflVecs));  // 2 slots x CTAs x values
  P.fx.reserve(kFxSlots * kFxWords);
  P.barrier.reserve(1);
  const size_t rows = 24 * static_cast<size_t>(max_slices);
  const size_t nodes4 = 4 * static_cast<size_t>(nb);
  auto fit = [&](size_t bytes) { return bytes <= static_cast<size_t>(smem_optin); };
  // Shared memory per CTA: own-row vectors r, p, Ap, diag^-1 (+ the solution
  // accumulator when it fits), the per-slice sums and the x window.  Tried in
  // order: window with u in shared memory, window with u in global memory,
  // then the same two without the window.
  auto plan = [&](size_t elem, auto cfg_win, auto cfg_nowin, bool& ok, bool& win, bool& ug,
                  bool& defl, size_t& smem) {
    const size_t slots = slot_count(static_cast<int>(rows));
    const size_t w = 4 * static_cast<size_t>(max_win) * elem;
    int blocks = 0;
    for (int mode = 0; mode < 4 && !ok; ++mode) {
      const bool want_win = mode < 2, u_global = (mode & 1) != 0;
      const size_t bytes = ((u_global ? 4 : 5) * rows + slots) * elem + (want_win ? w : 0);
      if (!fit(bytes)) continue;
      const int r = static_cast<int>(rows);
      if (!(want_win ? cfg_win(bytes, r, &blocks, &defl) : cfg_nowin(bytes, r, &blocks, &defl)))
        continue;
      ok = true;
      win = want_win;
      ug = u_global;
      smem = bytes;
    }
  };
  bool defl64 = false, defl32 = false;
  plan(sizeof(double), configure<double, true, false>, configure<double, false, false>, P.ok64,
       P.win64, P.ug64, defl64, P.smem64);
  if (P.ok64) {
    P.z4d.reserve(nodes4);
    P.p4da.reserve(nodes4);
    P.p4db.reserve(nodes4);
    VSGB_CUDA(cudaMemsetAsync(P.z4d.ptr, 0, sizeof(double) * nodes4, s));
    VSGB_CUDA(cudaMemsetAsync(P.p4da.ptr, 0, sizeof(double) * nodes4, s));
    VSGB_CUDA(cudaMemsetAsync(P.p4db.ptr, 0, sizeof(double) * nodes4, s));
  }
  if (need32 && B.has32) {
    plan(sizeof(float), configure<float, true, true>, configure<float, false, true>, P.ok32,
         P.win32, P.ug32, defl32, P.smem32);
    P.defl32 = P.win32 && defl32;
    if (P.ok32) {
      P.z4f.reserve(nodes4);
      P.p4fa.reserve(nodes4);
      P.p4fb.reserve(nodes4);
      VSGB_CUDA(cudaMemsetAsync(P.z4f.ptr, 0, sizeof(float) * nodes4, s));
      VSGB_CUDA(cudaMemsetAsync(P.p4fa.ptr, 0, sizeof(float) * nodes4, s));
      VSGB_CUDA(cudaMemsetAsync(P.p4fb.ptr, 0, sizeof(float) * nodes4, s));
      if (P.ug32) P.u32g.reserve(3 * static_cast<size_t>(nb));
    }
  }
  VSGB_CUDA(cudaStreamSynchronize(s));
}

int resident_block_jacobi(const BsrSell& B, ResidentPlan& P, bool need32, cudaStream_t s) {
  const size_t m = 6 * static_cast<size_t>(B.nb > 0 ? B.nb : 1);
  P.bj64.reserve(m);
  if (need32) P.bj32.reserve(m);
  P.bjd32.reserve(m);
  P.bj_bad.reserve(1);
  const int big = INT_MAX;
  VSGB_CUDA(cudaMemcpyAsync(P.bj_bad.ptr, &big, sizeof(int), cudaMemcpyHostToDevice, s));
  k_block_jacobi_inverse<<<(B.nb + 255) / 256, 256, 0, s>>>(
      B.nb, B.slice_ptr.ptr, B.rowlen.ptr, B.cols.ptr, B.val64.ptr, P.bj64.ptr,
      need32 ? P.bj32.ptr : nullptr, P.bjd32.ptr, P.bj_bad.ptr);
  VSGB_LAUNCH_CHECK();
  int bad = big;
  VSGB_CUDA(cudaMemcpyAsync(&bad, P.bj_bad.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  return bad == big ? -1 : bad;
}

void resident_solve32(const BsrSell& B, ResidentPlan& P, const double* r64, double* u64,
                      PcgScalars* S, const PcgScalars* O, const ResidentCtl& ctl, cudaStream_t s,
                      const double* dinv) {
  float* ug = P.ug32 ? P.u32g.ptr : nullptr;
  const float* bj = ctl.block_jacobi ? P.bj32.ptr : nullptr;
  if (P.win32)
    launch_resident<float, true, true>(B, P, B.val32.ptr, r64, u64, S, O, ctl, P.z4f.ptr,
                                       P.p4fa.ptr, P.p4fb.ptr, dinv, bj, P.smem32, ug, s);
  else
    launch_resident<float, false, true>(B, P, B.val32.ptr, r64, u64, S, O, ctl, P.z4f.ptr,
                                        P.p4fa.ptr, P.p4fb.ptr, dinv, bj, P.smem32, ug, s);
}

void resident_solve64(const BsrSell& B, ResidentPlan& P, const double* f, double* u,
                      PcgScalars* S, const ResidentCtl& ctl, cudaStream_t s,
                      const double* dinv) {
  // the FP64 solve accumulates straight into its output when u is global
  double* ug = P.ug64 ? u : nullptr;
  const double* bj = ctl.block_jacobi ? P.bj64.ptr : nullptr;
  if (P.win64)
    launch_resident<double, true, false>(B, P, B.val64.ptr, f, u, S, nullptr, ctl, P.z4d.ptr,
                                         P.p4da.ptr, P.p4db.ptr, dinv, bj, P.smem64, ug, s);
  else
    launch_resident<double, false, false>(B, P, B.val64.ptr, f, u, S, nullptr, ctl, P.z4d.ptr,
                                          P.p4da.ptr, P.p4db.ptr, dinv, bj, P.smem64, ug, s);
}

// diag32 = 1 / dinv (the Jacobi diagonal, FP32) for the error estimate.
__global__ void k_recip_f32(int n, const double* __restrict__ dinv, float* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    d[i] = static_cast<float>(1.0 / dinv[i]);
}

void resident_trace(const ResidentPlan& P, cudaStream_t s, double* sums_ns, double* max_spmv_ns,
                    long long* iterations) {
  std::vector<unsigned long long> h(static_cast<size_t>(kTraceWords) * P.ctas);
  VSGB_CUDA(cudaMemcpyAsync(h.data(), P.trace.ptr, sizeof(unsigned long long) * h.size(),
                            cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < kTracePhases; ++k) sums_ns[k] = 0.0;
  *max_spmv_ns = 0.0;
  *iterations = 0;
  for (int c = 0; c < P.ctas; ++c) {
    const unsigned long long* t = h.data() + static_cast<size_t>(kTraceWords) * c;
    for (int k = 0; k < kTracePhases; ++k) sums_ns[k] += static_cast<double>(t[k]) / P.ctas;
    *max_spmv_ns = std::max(*max_spmv_ns, static_cast<double>(t[1]));
    *iterations = static_cast<long long>(t[kTracePhases]);
  }
}

void resident_diag(ResidentPlan& P, const double* dinv, int n, int num_sms, cudaStream_t s) {
  P.diag32.reserve(static_cast<size_t>(n > 0 ? n : 1));
  k_recip_f32<<<num_sms * 4, 256, 0, s>>>(n, dinv, P.diag32.ptr);
  VSGB_LAUNCH_CHECK();
}

}  // namespace vsgb
