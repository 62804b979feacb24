// vibestran_gb300/csrc/mres.cu — persistent tiled batched PCG: every FP32
// inner solve of up to 16 load cases is one cooperative launch.
//
// The reference solves load cases one after another (linear_static.cpp:
// 212-275, one cuda-pcg solve each, cuda_pcg_backend_impl.hpp:1688-1999);
// the batched form shares each matrix sweep among the cases (panels [n][16]).
// The launch-per-kernel batched SpMM (multi.cu) gathers the 192-byte panel
// row of every block column straight from L1/L2, 27 times per node and in
// 64-byte runs per quad: it is bound by L1 wavefronts, not by HBM.  Here:
//   * block rows are grouped into tiles of ~tn rows by recursive coordinate
//     bisection of the node coordinates (boxes of aspect ~1), so a tile's
//     window — the distinct nodes its rows touch — is 2.2-3x its own rows;
//   * once per iteration and tile the window's r and p rows (192 B each) and
//     Jacobi inverses arrive in shared memory by asynchronous 16-byte copies
//     and are combined in place into x = z + beta p, the direction update of
//     the cases fused into the gather; the owning CTA writes p for its rows;
//   * the tile's rows, in 8-row slices of the sliced-ELL layout with
//     window-local 16-bit column indices, multiply the staged window (FP32
//     difference form, as every FP32 product of this library), the matrix
//     arriving through a per-warp ring of asynchronous copies that runs
//     ahead across slices, tiles and iterations;
//   * two grid reductions per iteration carry the 16 cases' sums (p.Ap and
//     p.Dp; r.z and r.r), each case's recurrence runs on its own lane of warp
//     0 (the same recurrence and stopping tests as the launch-per-kernel
//     path, error control included), and a case that stopped gets
//     alpha = beta = 0.
// All sums are in fixed order (per lane, warp shuffles, warps, CTAs), so a
// solve is bitwise reproducible for a given tile size.
//
// Measured on the 16 face-load cases of the 100x40x40 block (GB300, phase
// timer): 48 us staging (2.9x window volume at 112 rows per tile), 92 us
// multiply (shared-memory reads of x, 2-way bank conflicts between the two
// nodes of a quarter-warp), 44 us update, 29 us in the two reductions per
// iteration: 0.37 s against 0.31 s for the launch-per-kernel path, which
// stays the default (VSGB_OPT_BATCH_TILES).

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <numeric>
#include <vector>

#include "errest.cuh"
#include "gridsync.cuh"
#include "multi.cuh"

namespace vsgb {

namespace {

constexpr int kMresThreads = 512;
constexpr int kMresWarps = kMresThreads / 32;
constexpr int kNV = 2 * kP;  // values per grid reduction
constexpr int kWinFloats = 3 * kP;  // staged floats per window node

__device__ __forceinline__ float4 ld4f(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4f(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 ld4g(const float* p) {
  return __ldcg(reinterpret_cast<const float4*>(p));
}
__device__ __forceinline__ float comp(const float4& v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

struct MresArgs {
  int nb, n, ncols;
  const int* __restrict__ tile_slice;
  const int* __restrict__ tile_win;
  const int* __restrict__ win_row;
  const int* __restrict__ slice_step;
  const int* __restrict__ slice_row;
  const unsigned short* __restrict__ slice_own;
  const unsigned short* __restrict__ col16;
  const float* __restrict__ val;
  const int* __restrict__ cta_tile;
  const float* __restrict__ dinv32;
  const float* __restrict__ diag32;
  const double* __restrict__ r64;
  double* u64;
  float *r, *u, *pa, *pb, *Ap;
  MultiState* S;
  const MultiOuter* O;
  ErrEst* est;
  double* partials;
  unsigned* count;
  int* abort_flag;
  double tol, outer_tol;
  int max_iters;
  int err_mode;
  double err_target, err_rel;
  long long spin_limit;
  int accumulate;
  const float4* __restrict__ dinv4;  // per block row: the 3 Jacobi inverses (+ pad)
  // byte offsets in dynamic shared memory: p_old staging, the diagonal
  // staging, the window's block rows and the matrix-stream rings (the window
  // x itself starts at 0)
  int wp_off, wd_off, wrow_off, ring_off;
  unsigned long long* trace;  // null, or 8 per CTA: phase times (ns), iterations
};

// Per-lane column partials (4 cases per lane, lane % 4 selects which) summed
// over the warp: after the shuffles lanes 0..3 hold the warp's sums of cases
// 4q..4q+3; written to wsum[warp][case] (FP64).
__device__ __forceinline__ void warp_cols(const float (&v)[4], double* wsum_row, int lane) {
  float w[4] = {v[0], v[1], v[2], v[3]};
#pragma unroll
  for (int o = 4; o < 32; o <<= 1)
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k] += __shfl_xor_sync(0xffffffffu, w[k], o);
  if (lane < 4)
#pragma unroll
    for (int k = 0; k < 4; ++k) wsum_row[4 * lane + k] = static_cast<double>(w[k]);
}

// Grid sum of the kNV values of every CTA (wsum[warp][value], kMresWarps rows,
// rows that hold nothing are zero): CTA totals in warp order, a bounded grid
// barrier, then the CTA partials in CTA order by 8 lanes per value; the
// totals land in tot[] (shared).  Returns false when the barrier gave up.
__device__ bool mres_grid_sum(const double* wsum, double* partials, int slot, unsigned* count,
                              unsigned& target, int* abort_flag, long long spin_limit,
                              double* tot, int* s_ok) {
  const int tid = threadIdx.x;
  __syncthreads();
  double* part = partials + static_cast<size_t>(slot) * gridDim.x * kNV;
  if (tid < kNV) {
    double s = 0.0;
    for (int w = 0; w < kMresWarps; ++w) s += wsum[w * kNV + tid];
    part[blockIdx.x * kNV + tid] = s;
  }
  const bool ok = grid_sync(count, target, abort_flag, s_ok, spin_limit);
  if (tid < 8 * kNV) {
    const int v = tid >> 3, p = tid & 7;
    double s = 0.0;
    for (unsigned c = p; c < gridDim.x; c += 8) s += __ldcg(&part[c * kNV + v]);
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (p == 0) tot[v] = s;
  }
  __syncthreads();
  return ok;
}

// ── matrix stream: a per-warp ring of kRing steps in shared memory, filled
// with asynchronous 16-byte copies (cp.async) kRing - 1 steps ahead of the
// multiply.  The warp's steps form one sequence over its slices of every
// tile of the CTA and wrap round to the first tile (the next iteration), so
// the stream never drains at a slice, tile or iteration boundary.
constexpr int kRing = 3;
constexpr int kStepBytes = 288 * 4 + 64;  // 9 x 32 values + 32 window indices
constexpr int kRingBytes = kMresWarps * kRing * kStepBytes;

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
// The same with an L2 evict-first hint (the matrix: streamed once per
// iteration, larger than L2; the panels it would displace are reused).
__device__ __forceinline__ void cp_async16_stream(void* dst, const void* src,
                                                  unsigned long long policy) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(d), "l"(src),
               "l"(policy)
               : "memory");
}
__device__ __forceinline__ unsigned long long evict_first_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;" ::: "memory");
}

struct StepCursor {
  int tile, sl, g, gend;  // tile, slice, global step and end of the slice's steps
};
// (kept in shared memory, one per warp: the values are warp-uniform and the
// multiply needs every register)

// First step of the warp's sequence; false when the warp has no slice.
__device__ inline bool cursor_first(StepCursor& c, const MresArgs& a, int t0, int t1, int warp) {
  for (int t = t0; t < t1; ++t) {
    const int sl = a.tile_slice[t] + warp;
    if (sl < a.tile_slice[t + 1]) {
      c.tile = t;
      c.sl = sl;
      c.g = a.slice_step[sl];
      c.gend = a.slice_step[sl + 1];
      return true;
    }
  }
  return false;
}

// Next step (every slice has at least one step; some tile holds a slice of
// this warp, so the search ends).
__device__ inline void cursor_next(StepCursor& c, const MresArgs& a, int t0, int t1, int warp) {
  if (++c.g < c.gend) return;
  c.sl += kMresWarps;
  while (c.sl >= a.tile_slice[c.tile + 1]) {
    if (++c.tile == t1) c.tile = t0;
    c.sl = a.tile_slice[c.tile] + warp;
  }
  c.g = a.slice_step[c.sl];
  c.gend = a.slice_step[c.sl + 1];
}

// Copies step g (values, then window indices) into ring slot seq % kRing and
// commits the group (every lane commits, with or without a copy).
__device__ __forceinline__ void ring_issue(unsigned char* ring_w, unsigned seq, int g,
                                           const MresArgs& a, int lane) {
  unsigned char* dst = ring_w + (seq % kRing) * kStepBytes;
  const unsigned char* vsrc = reinterpret_cast<const unsigned char*>(a.val + static_cast<size_t>(g) * 288);
  const unsigned char* csrc = reinterpret_cast<const unsigned char*>(a.col16 + static_cast<size_t>(g) * 32);
  const unsigned long long pol = evict_first_policy();
  cp_async16_stream(dst + 16 * lane, vsrc + 16 * lane, pol);
  cp_async16_stream(dst + 512 + 16 * lane, vsrc + 512 + 16 * lane, pol);
  if (lane < 8)
    cp_async16_stream(dst + 1024 + 16 * lane, vsrc + 1024 + 16 * lane, pol);
  else if (lane < 12)
    cp_async16_stream(dst + 1152 + 16 * (lane - 8), csrc + 16 * (lane - 8), pol);
  cp_async_commit();
}

// Phase timer (thread 0): adds the time since the last mark to phase k.
__device__ __forceinline__ void tr_mark(unsigned long long* tr, int k) {
  if (threadIdx.x == 0) {
    const unsigned long long t = gtime();
    tr[k] += t - tr[7];
    tr[7] = t;
  }
}

__global__ void __launch_bounds__(kMresThreads, 1) k_mres(MresArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  float* win = reinterpret_cast<float*>(smem);
  float* wpo = reinterpret_cast<float*>(smem + a.wp_off);
  float4* wd = reinterpret_cast<float4*>(smem + a.wd_off);
  int* wrow = reinterpret_cast<int*>(smem + a.wrow_off);
  __shared__ unsigned long long tr[8];  // phase sums (thread 0), last mark at [7]
  const bool trace = a.trace != nullptr;
  __shared__ double wsum[kMresWarps * kNV];
  __shared__ double tot[kNV];
  __shared__ __align__(16) float s_alpha[kP];
  __shared__ __align__(16) float s_beta[kP];
  __shared__ double c_rz[kP], c_rr[kP], c_nb[kP], c_tol[kP], c_t2[kP];
  __shared__ int c_flags[kP], c_iters[kP];
  __shared__ ErrEst c_est[kP];
  __shared__ int s_ok, s_done;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int c = blockIdx.x;
  const int t0 = a.cta_tile[c], t1 = a.cta_tile[c + 1];
  const int sl0 = a.tile_slice[t0], sl1 = a.tile_slice[t1];  // the CTA's slices
  const int nown = 8 * (sl1 - sl0) * 12;                     // own-row elements
  const bool err_on = a.err_mode != kErrOff;
  unsigned char* ring_w = smem + a.ring_off + warp * (kRing * kStepBytes);
  unsigned target = 0;
  int slot = 0;
  if (tid == 0) tmarks()[2] = 0;  // no phase trace in this kernel
  for (int k = tid; k < kMresWarps * kNV; k += kMresThreads) wsum[k] = 0.0;

  // start the matrix stream (seq: steps issued; the multiply consumes step
  // seq - kRing after issuing one more)
  __shared__ StepCursor s_cur[kMresWarps];
  StepCursor& cur = s_cur[warp];
  unsigned seq = 0;
  {
    StepCursor c0;
    const bool streams = cursor_first(c0, a, t0, t1, warp);
    if (streams)
      for (int k = 0; k < kRing - 1; ++k) {
        ring_issue(ring_w, seq++, c0.g, a, lane);
        cursor_next(c0, a, t0, t1, warp);
      }
    __syncwarp();
    if (lane == 0) cur = c0;
    __syncwarp();
  }

  // ── init: r = scale * r64 (active cases), u = 0, p_old = 0; r.z, r.r ──
  // Own-row loops: element e is DOF 3 R + (e / 4) % 3 of the row in slot
  // e / 12, cases 4 c4..4 c4+3 with c4 = e % 4 = lane % 4 (the stride is a
  // multiple of 4), the lane grouping of warp_cols.
  {
    float4 sc4;
    {
      float scv[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int col = 4 * (tid & 3) + k;
        const bool act = col < a.ncols && a.O->active[col] != 0;
        scv[k] = act ? static_cast<float>(a.O->scale[col]) : 0.f;
      }
      sc4 = make_float4(scv[0], scv[1], scv[2], scv[3]);
    }
    float rzp[4] = {0.f, 0.f, 0.f, 0.f}, rrp[4] = {0.f, 0.f, 0.f, 0.f};
    for (int e = tid; e < nown; e += kMresThreads) {
      const int R = a.slice_row[8 * sl0 + (e >> 2) / 3];
      if (R < 0) continue;
      const int j = (e >> 2) % 3, c4 = e & 3;
      const size_t o = static_cast<size_t>(3 * R + j) * kP + 4 * c4;
      const double2 fa = __ldcg(reinterpret_cast<const double2*>(a.r64 + o));
      const double2 fb = __ldcg(reinterpret_cast<const double2*>(a.r64 + o + 2));
      const float4 rv = make_float4(static_cast<float>(fa.x * sc4.x), static_cast<float>(fa.y * sc4.y),
                                    static_cast<float>(fb.x * sc4.z), static_cast<float>(fb.y * sc4.w));
      const float d = a.dinv32[3 * R + j];
      st4f(a.r + o, rv);
      st4f(a.u + o, make_float4(0.f, 0.f, 0.f, 0.f));
      st4f(a.pa + o, make_float4(0.f, 0.f, 0.f, 0.f));
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float x = comp(rv, k);
        rzp[k] = fmaf(x, x * d, rzp[k]);
        rrp[k] = fmaf(x, x, rrp[k]);
      }
    }
    warp_cols(rzp, wsum + warp * kNV, lane);
    warp_cols(rrp, wsum + warp * kNV + kP, lane);
  }
  bool ok = mres_grid_sum(wsum, a.partials, slot, a.count, target, a.abort_flag, a.spin_limit,
                          tot, &s_ok);
  slot ^= 1;
  if (warp == 0 && lane < kP) {
    const int k = lane;
    const double rz0 = tot[k], rr0 = tot[kP + k], nb = sqrt(fabs(rr0));
    const bool active = k < a.ncols && a.O->active[k] != 0;
    int fl = 0;
    if (!ok)
      fl = kFlagDone | 64;
    else if (!active)
      fl = kFlagDone | kFlagInactive;
    else if (nb < 1e-300)
      fl = kFlagDone | kFlagZeroRhs | kFlagConverged;
    else if (!(rz0 > 0.0))
      fl = kFlagDone | kFlagNonPosRz;
    double tk = a.tol;
    if (a.outer_tol > 0.0 && a.O->rel[k] > 0.0)
      tk = fmax(a.tol, fmin(0.5, 0.5 * a.outer_tol / a.O->rel[k]));
    c_tol[k] = tk;
    c_rz[k] = rz0;
    c_rr[k] = rr0;
    c_nb[k] = nb;
    c_flags[k] = fl;
    c_iters[k] = 0;
    err_reset(c_est[k]);
    const double sk = a.O->scale[k];
    c_t2[k] = a.err_mode == kErrAbsolute ? a.err_target * a.err_target * sk * sk * a.O->uD2[k]
                                          : 0.0;
    s_alpha[k] = 0.f;
    s_beta[k] = 0.f;
  }
  __syncthreads();
  if (tid == 0) {
    int all = 1;
    for (int k = 0; k < kP; ++k) all &= (c_flags[k] & kFlagDone) ? 1 : 0;
    s_done = all;
  }
  __syncthreads();

  const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
  float* p_old = a.pa;
  float* p_new = a.pb;
  int it = 0;
  if (trace && tid == 0) {
    for (int k = 0; k < 7; ++k) tr[k] = 0;
    tr[7] = gtime();
  }
  while (!s_done) {
    // ── phase 1: per tile, stage x = z + beta p_old over the window, write
    // the own rows' p, multiply the tile's rows; p.Ap (and p.Dp) per case ──
    float pap[4] = {0.f, 0.f, 0.f, 0.f}, pdp[4] = {0.f, 0.f, 0.f, 0.f};
    for (int tl = t0; tl < t1; ++tl) {
      const int w0 = a.tile_win[tl], nw = a.tile_win[tl + 1] - w0;
      // the window's rows, then asynchronous copies of r and p_old (192 B
      // per row each) and of the row's diagonal (16 B): 25 copies per row
      // in flight at once, no registers held
      for (int w = tid; w < nw; w += kMresThreads) wrow[w] = a.win_row[w0 + w];
      __syncthreads();
      for (int e = tid; e < nw * 25; e += kMresThreads) {
        const int w = e / 25, ch = e % 25, R = wrow[w];
        if (ch < 12)
          cp_async16(win + w * kWinFloats + 4 * ch, a.r + static_cast<size_t>(R) * kWinFloats + 4 * ch);
        else if (ch < 24)
          cp_async16(wpo + w * kWinFloats + 4 * (ch - 12),
                     p_old + static_cast<size_t>(R) * kWinFloats + 4 * (ch - 12));
        else
          cp_async16(wd + w, a.dinv4 + R);
      }
      cp_async_commit();
      cp_async_wait<0>();
      __syncthreads();
      // x = D^-1 r + beta p_old, in place of r
      for (int e = tid; e < nw * 12; e += kMresThreads) {
        const int w = e / 12, ch = e % 12, j = ch >> 2, c4 = ch & 3;
        const int o = w * kWinFloats + j * kP + 4 * c4;
        const float4 rv = ld4f(win + o), pv = ld4f(wpo + o);
        const float d = comp(wd[w], j);
        const float4 b = *reinterpret_cast<const float4*>(s_beta + 4 * c4);
        st4f(win + o, make_float4(fmaf(b.x, pv.x, rv.x * d), fmaf(b.y, pv.y, rv.y * d),
                                  fmaf(b.z, pv.z, rv.z * d), fmaf(b.w, pv.w, rv.w * d)));
      }
      if (trace) tr_mark(tr, 0);
      __syncthreads();
      const int ts0 = a.tile_slice[tl], ts1 = a.tile_slice[tl + 1];
      for (int e = tid; e < 8 * (ts1 - ts0) * 12; e += kMresThreads) {
        const int rs = 8 * ts0 + e / 12, R = a.slice_row[rs];
        if (R < 0) continue;
        const int ch = e % 12, j = ch >> 2, c4 = ch & 3;
        st4f(p_new + static_cast<size_t>(3 * R + j) * kP + 4 * c4,
             ld4f(win + a.slice_own[rs] * kWinFloats + j * kP + 4 * c4));
      }
      // 8-row slices, one warp each; lane 4r+q: row r, cases 4q..4q+3
      const int r8 = lane >> 2, q = lane & 3;
      for (int sl = ts0 + warp; sl < ts1; sl += kMresWarps) {
        const int R = a.slice_row[8 * sl + r8];
        const int own = a.slice_own[8 * sl + r8];
        const float* xo = win + own * kWinFloats + 4 * q;
        float4 xi[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) xi[j] = ld4f(xo + j * kP);
        float4 y[3] = {zero4, zero4, zero4};
        const int steps = a.slice_step[sl + 1] - a.slice_step[sl];
        for (int t = 0; t < steps; ++t) {
          // keep kRing - 1 steps in flight, then wait for this one
          {
            StepCursor cw = cur;
            ring_issue(ring_w, seq++, cw.g, a, lane);
            cursor_next(cw, a, t0, t1, warp);
            __syncwarp();
            if (lane == 0) cur = cw;
          }
          cp_async_wait<kRing - 1>();
          __syncwarp();
          const unsigned char* st = ring_w + (seq % kRing) * kStepBytes;
          // value k of the quad's 4 blocks: 4 consecutive floats; their
          // window indices: 4 consecutive u16
          const float4* v4 = reinterpret_cast<const float4*>(st) + r8;
          float4 av4[9];
#pragma unroll
          for (int k = 0; k < 9; ++k) av4[k] = v4[8 * k];
          const uint2 c4w = *reinterpret_cast<const uint2*>(st + 1152 + 8 * r8);
          __syncwarp();  // the slot is refilled by the next issue
#pragma unroll
          for (int uu = 0; uu < 4; ++uu) {
            const unsigned w2 = uu < 2 ? c4w.x : c4w.y;
            const int cc = (uu & 1) ? static_cast<int>(w2 >> 16) : static_cast<int>(w2 & 0xFFFFu);
            // difference form: off-diagonal blocks multiply x_J - x_I
            const float m = cc != own ? 1.f : 0.f;
            const float* xc = win + cc * kWinFloats + 4 * q;
            float4 xv[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const float4 v = ld4f(xc + j * kP);
              xv[j] = make_float4(fmaf(-m, xi[j].x, v.x), fmaf(-m, xi[j].y, v.y),
                                  fmaf(-m, xi[j].z, v.z), fmaf(-m, xi[j].w, v.w));
            }
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              float4& o = y[i];
#pragma unroll
              for (int j = 0; j < 3; ++j) {
                const float aij = comp(av4[3 * i + j], uu);
                o.x = fmaf(aij, xv[j].x, o.x);
                o.y = fmaf(aij, xv[j].y, o.y);
                o.z = fmaf(aij, xv[j].z, o.z);
                o.w = fmaf(aij, xv[j].w, o.w);
              }
            }
          }
        }
        if (R >= 0) {
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            st4f(a.Ap + static_cast<size_t>(3 * R + j) * kP + 4 * q, y[j]);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const float pk = comp(xi[j], k);
              pap[k] = fmaf(pk, comp(y[j], k), pap[k]);
            }
          }
          if (err_on)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const float dg = __ldg(a.diag32 + 3 * R + j);
#pragma unroll
              for (int k = 0; k < 4; ++k) {
                const float pk = comp(xi[j], k);
                pdp[k] = fmaf(pk * pk, dg, pdp[k]);
              }
            }
        }
      }
      __syncthreads();  // the window is restaged for the next tile
      if (trace) tr_mark(tr, 1);
    }
    warp_cols(pap, wsum + warp * kNV, lane);
    warp_cols(pdp, wsum + warp * kNV + kP, lane);
    ok = mres_grid_sum(wsum, a.partials, slot, a.count, target, a.abort_flag, a.spin_limit, tot,
                       &s_ok);
    slot ^= 1;
    if (warp == 0 && lane < kP) {
      const int k = lane;
      int fl = c_flags[k];
      float al = 0.f;
      if (!ok) {
        fl |= kFlagDone | 64;
      } else if (!(fl & kFlagDone)) {
        const double pAp = tot[k];
        if (!(pAp > 0.0)) {
          fl |= kFlagDone | kFlagBreakdown;
          c_iters[k] = it;
        } else {
          const double y = rcp_nr2(pAp);
          const double alpha = div_nr(c_rz[k], pAp, y);
          al = static_cast<float>(alpha);
          if (err_on) err_record(c_est[k], c_rz[k] * alpha, tot[kP + k] * y);
        }
      }
      c_flags[k] = fl;
      s_alpha[k] = al;
    }
    __syncthreads();
    if (trace) tr_mark(tr, 2);
    if (!ok) break;

    // ── phase 2: u += alpha p, r -= alpha Ap, z = D^-1 r on the own rows;
    // r.z, r.r per case ──
    {
      float rzp[4] = {0.f, 0.f, 0.f, 0.f}, rrp[4] = {0.f, 0.f, 0.f, 0.f};
      const float4 al = *reinterpret_cast<const float4*>(s_alpha + 4 * (tid & 3));
      for (int e = tid; e < nown; e += kMresThreads) {
        const int R = a.slice_row[8 * sl0 + (e >> 2) / 3];
        if (R < 0) continue;
        const int j = (e >> 2) % 3, c4 = e & 3;
        const size_t o = static_cast<size_t>(3 * R + j) * kP + 4 * c4;
        const float4 uv = ld4g(a.u + o), rv = ld4g(a.r + o);
        const float4 pv = ld4g(p_new + o), av = ld4g(a.Ap + o);
        const float d = __ldg(a.dinv32 + 3 * R + j);
        const float4 un = make_float4(fmaf(al.x, pv.x, uv.x), fmaf(al.y, pv.y, uv.y),
                                      fmaf(al.z, pv.z, uv.z), fmaf(al.w, pv.w, uv.w));
        const float4 rn = make_float4(fmaf(-al.x, av.x, rv.x), fmaf(-al.y, av.y, rv.y),
                                      fmaf(-al.z, av.z, rv.z), fmaf(-al.w, av.w, rv.w));
        st4f(a.u + o, un);
        st4f(a.r + o, rn);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float x = comp(rn, k);
          rzp[k] = fmaf(x, x * d, rzp[k]);
          rrp[k] = fmaf(x, x, rrp[k]);
        }
      }
      warp_cols(rzp, wsum + warp * kNV, lane);
      warp_cols(rrp, wsum + warp * kNV + kP, lane);
    }
    if (trace) tr_mark(tr, 3);
    ++it;
    ok = mres_grid_sum(wsum, a.partials, slot, a.count, target, a.abort_flag, a.spin_limit, tot,
                       &s_ok);
    slot ^= 1;
    if (warp == 0 && lane < kP) {
      const int k = lane;
      int fl = c_flags[k];
      float be = 0.f;
      if (!ok) {
        fl |= kFlagDone | 64;
      } else if (!(fl & kFlagDone)) {
        const double rzn = tot[k], rrk = tot[kP + k];
        c_rr[k] = rrk;
        bool conv;
        if (err_on) {
          conv = err_block_end(c_est[k], c_t2[k], a.err_rel * a.err_rel);
          bool met = conv && (a.err_mode == kErrRelative ||
                              (c_est[k].est2 <= c_t2[k] && c_est[k].lag2 <= c_t2[k]));
          if (!(fabs(rrk) > 1e-20 * c_nb[k] * c_nb[k])) conv = true;
          if (met) fl |= kFlagErrTarget;
        } else {
          conv = fabs(rrk) < (c_tol[k] * c_nb[k]) * (c_tol[k] * c_nb[k]);
        }
        if (conv) {
          fl |= kFlagDone | kFlagConverged;
          c_iters[k] = it;
        } else {
          be = static_cast<float>(div_nr(rzn, c_rz[k], rcp_nr2(c_rz[k])));
          if (it >= a.max_iters) {
            fl |= kFlagDone | kFlagMaxIters;
            c_iters[k] = it;
          }
        }
        c_rz[k] = rzn;
      }
      c_flags[k] = fl;
      s_beta[k] = (fl & kFlagDone) ? 0.f : be;
    }
    __syncthreads();
    if (tid == 0) {
      int all = 1;
      for (int k = 0; k < kP; ++k) all &= (c_flags[k] & kFlagDone) ? 1 : 0;
      s_done = all || !ok;
    }
    __syncthreads();
    if (trace) tr_mark(tr, 4);
    float* t = p_old;
    p_old = p_new;
    p_new = t;
  }
  cp_async_wait_all();  // the stream's copies in flight land before the CTA exits

  // ── results: u64 += u / scale for the active cases (own rows) ──
  if (ok && a.accumulate) {
    for (int e = tid; e < nown; e += kMresThreads) {
      const int R = a.slice_row[8 * sl0 + (e >> 2) / 3];
      if (R < 0) continue;
      const int j = (e >> 2) % 3, c4 = e & 3;
      const size_t o = static_cast<size_t>(3 * R + j) * kP + 4 * c4;
      const float4 uv = ld4g(a.u + o);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int col = 4 * c4 + k;
        if (col < a.ncols && a.O->active[col] != 0)
          a.u64[o + k] = fma(static_cast<double>(comp(uv, k)), 1.0 / a.O->scale[col], a.u64[o + k]);
      }
    }
  }
  if (trace && tid == 0) {
    for (int k = 0; k < 5; ++k) a.trace[8 * c + k] = tr[k];
    a.trace[8 * c + 5] = static_cast<unsigned long long>(it);
  }
  if (c == 0 && warp == 0 && lane < kP) {
    const int k = lane;
    MultiState* S = a.S;
    S->flags[k] = c_flags[k];
    S->iters[k] = (c_flags[k] & kFlagDone) ? c_iters[k] : it;
    S->rz[k] = c_rz[k];
    S->rr[k] = c_rr[k];
    S->norm_b[k] = c_nb[k];
    S->rel[k] = c_nb[k] > 1e-300 ? sqrt(fabs(c_rr[k])) / c_nb[k] : 0.0;
    S->tolk[k] = c_tol[k];
    S->err_t2[k] = c_t2[k];
    const double sk = a.O->scale[k];
    S->err_norm2[k] = a.err_mode == kErrAbsolute ? sk * sk * a.O->uD2[k] : 0.0;
    a.est[k] = c_est[k];
    if (k == 0) {
      S->iter = it;
      S->done = 1;
      S->err_mode = a.err_mode;
      S->err_rel2 = a.err_rel * a.err_rel;
    }
  }
}

// New slot s of the tiled layout <- old slot slot_map[s] (-1: padding, zero
// values) of the block operator's FP32 values.
__global__ void k_tile_values(long long nslots, const int* __restrict__ slot_map,
                              const float* __restrict__ v32, float* __restrict__ out) {
  for (long long s = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; s < nslots;
       s += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int o = slot_map[s];
    const long long ns = (s / 32) * 288 + (s % 32);
    const long long os = o >= 0 ? (static_cast<long long>(o) / 32) * 288 + (o % 32) : 0;
#pragma unroll
    for (int k = 0; k < 9; ++k) out[ns + 32 * k] = o >= 0 ? v32[os + 32 * k] : 0.f;
  }
}

// The Jacobi inverses of each block row as one 16-byte record.
__global__ void k_dinv4(int nb, const float* __restrict__ dinv32, float4* __restrict__ out) {
  for (int R = blockIdx.x * blockDim.x + threadIdx.x; R < nb; R += gridDim.x * blockDim.x)
    out[R] = make_float4(dinv32[3 * R], dinv32[3 * R + 1], dinv32[3 * R + 2], 0.f);
}


}  // namespace

bool mres_build_tiles(const BsrSell& B, const float* dinv32, const std::vector<float>& coords,
                      int tn, int ctas, size_t smem_cap, MultiTiles& T, cudaStream_t s) {
  T.valid = false;
  const int nb = B.nb;
  if (!B.valid || !B.has32 || nb <= 0 || static_cast<int>(coords.size()) != 3 * nb || tn < 8)
    return false;
  // host copy of the block structure
  std::vector<int> sp(static_cast<size_t>(B.nslices) + 1);
  VSGB_CUDA(cudaMemcpyAsync(sp.data(), B.slice_ptr.ptr, sizeof(int) * sp.size(),
                            cudaMemcpyDeviceToHost, s));
  std::vector<int> cols(static_cast<size_t>(B.steps) * 32);
  VSGB_CUDA(cudaMemcpyAsync(cols.data(), B.cols.ptr, sizeof(int) * cols.size(),
                            cudaMemcpyDeviceToHost, s));
  std::vector<int> rowlen(static_cast<size_t>(nb));
  VSGB_CUDA(cudaMemcpyAsync(rowlen.data(), B.rowlen.ptr, sizeof(int) * nb, cudaMemcpyDeviceToHost,
                            s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  auto old_slot = [&](int R, int j) {  // slot of block j of row R in the block layout
    return (sp[R >> 3] + (j >> 2)) * 32 + (R & 7) * 4 + (j & 3);
  };
  // Tiles by recursive coordinate bisection: a set of rows is cut at the
  // median of its longest extent, the two halves sized for ceil(size / tn)
  // tiles between them, until a set fits one tile; the tiles are boxes of
  // aspect ~1 and come out in a spatially coherent order.
  std::vector<int> order(static_cast<size_t>(nb));
  std::iota(order.begin(), order.end(), 0);
  std::vector<int> tile_start(1, 0);
  struct Range {
    int b, e;
  };
  std::vector<Range> stack{{0, nb}};
  while (!stack.empty()) {
    const Range r = stack.back();
    stack.pop_back();
    const int size = r.e - r.b, leaves = (size + tn - 1) / tn;
    if (leaves <= 1) {
      tile_start.push_back(r.e);
      continue;
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = r.b; k < r.e; ++k)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], coords[3 * order[k] + d]);
        hi[d] = std::max(hi[d], coords[3 * order[k] + d]);
      }
    int ax = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    const int mid = r.b + static_cast<int>(static_cast<long long>(size) * (leaves / 2) / leaves);
    std::nth_element(order.begin() + r.b, order.begin() + mid, order.begin() + r.e,
                     [&](int x, int y) {
                       const float cx = coords[3 * x + ax], cy = coords[3 * y + ax];
                       return cx < cy || (cx == cy && x < y);
                     });
    stack.push_back({mid, r.e});  // the left half is tiled first
    stack.push_back({r.b, mid});
  }
  const int ntiles = static_cast<int>(tile_start.size()) - 1;
  std::vector<int> tile_slice(static_cast<size_t>(ntiles) + 1, 0), tile_win(ntiles + 1, 0);
  std::vector<int> win_row, slice_step(1, 0), slice_row;
  std::vector<unsigned short> slice_own, col16;
  std::vector<int> slot_map;
  std::vector<int> tile_steps(static_cast<size_t>(ntiles), 0);
  int max_win = 0;
  for (int t = 0; t < ntiles; ++t) {
    const std::vector<int> rows(order.begin() + tile_start[t], order.begin() + tile_start[t + 1]);
    std::vector<int> w;
    for (int R : rows) {
      w.push_back(R);
      for (int j = 0; j < rowlen[R]; ++j) w.push_back(cols[old_slot(R, j)]);
    }
    std::sort(w.begin(), w.end());
    w.erase(std::unique(w.begin(), w.end()), w.end());
    if (w.size() > 65535) return false;
    max_win = std::max(max_win, static_cast<int>(w.size()));
    auto widx = [&](int col) {
      return static_cast<unsigned short>(std::lower_bound(w.begin(), w.end(), col) - w.begin());
    };
    for (size_t i0 = 0; i0 < rows.size(); i0 += 8) {
      int mx = 0;
      for (size_t i = i0; i < std::min(rows.size(), i0 + 8); ++i) mx = std::max(mx, rowlen[rows[i]]);
      const int steps = (mx + 3) / 4;
      for (int r = 0; r < 8; ++r) {
        const bool has = i0 + r < rows.size();
        slice_row.push_back(has ? rows[i0 + r] : -1);
        slice_own.push_back(has ? widx(rows[i0 + r]) : 0);
      }
      for (int st = 0; st < steps; ++st)
        for (int lane = 0; lane < 32; ++lane) {
          const int r = lane >> 2, qq = lane & 3, j = 4 * st + qq;
          const bool has = i0 + r < rows.size();
          const int R = has ? rows[i0 + r] : -1;
          if (has && j < rowlen[R]) {
            const int os = old_slot(R, j);
            slot_map.push_back(os);
            col16.push_back(widx(cols[os]));
          } else {
            slot_map.push_back(-1);
            col16.push_back(has ? widx(R) : 0);  // zero values; any in-window index
          }
        }
      slice_step.push_back(slice_step.back() + steps);
      tile_steps[t] += steps + 2;  // + slice start cost
    }
    tile_slice[t + 1] = static_cast<int>(slice_step.size()) - 1;
    win_row.insert(win_row.end(), w.begin(), w.end());
    tile_win[t + 1] = static_cast<int>(win_row.size());
  }
  // the window x (= r on arrival), p_old, the diagonals and block rows of
  // the window, then the matrix-stream rings of the warps
  const size_t mw = static_cast<size_t>(max_win);
  const size_t smem = (2 * mw * kWinFloats * sizeof(float) + mw * 16 + mw * 4 + 15) / 16 * 16 +
                      kRingBytes;
  if (smem > smem_cap) return false;
  // contiguous tile ranges per CTA, balanced by steps (+ window staging)
  std::vector<long long> pre(static_cast<size_t>(ntiles) + 1, 0);
  for (int t = 0; t < ntiles; ++t)
    pre[t + 1] = pre[t] + tile_steps[t] + (tile_win[t + 1] - tile_win[t]) / 8;
  std::vector<int> ct(static_cast<size_t>(ctas) + 1, 0);
  for (int g = 1; g < ctas; ++g) {
    const long long goal = pre[ntiles] * g / ctas;
    ct[g] = static_cast<int>(std::lower_bound(pre.begin(), pre.end(), goal) - pre.begin());
    ct[g] = std::max(ct[g], ct[g - 1]);
  }
  ct[ctas] = ntiles;
  const long long nsl = static_cast<long long>(slice_step.size()) - 1;
  const long long steps = slice_step.back();
  T.tn = tn;
  T.ntiles = ntiles;
  T.nslices = static_cast<int>(nsl);
  T.ctas = ctas;
  T.max_win = max_win;
  T.steps = steps;
  T.smem = smem;
  auto up = [&](auto& buf, const auto& h) {
    buf.reserve(h.size() > 0 ? h.size() : 1);
    VSGB_CUDA(cudaMemcpyAsync(buf.ptr, h.data(), sizeof(h[0]) * h.size(), cudaMemcpyHostToDevice,
                              s));
  };
  up(T.tile_slice, tile_slice);
  up(T.tile_win, tile_win);
  up(T.win_row, win_row);
  up(T.slice_step, slice_step);
  up(T.slice_row, slice_row);
  up(T.slice_own, slice_own);
  up(T.col16, col16);
  up(T.slot_map, slot_map);
  up(T.cta_tile, ct);
  T.nb = nb;
  mres_gather_values(B, dinv32, T, s);
  VSGB_CUDA(cudaStreamSynchronize(s));
  T.valid = true;
  return true;
}

void mres_gather_values(const BsrSell& B, const float* dinv32, MultiTiles& T, cudaStream_t s) {
  T.val.reserve(T.steps * 288 > 0 ? static_cast<size_t>(T.steps) * 288 : 1);
  k_tile_values<<<1024, 256, 0, s>>>(T.steps * 32, T.slot_map.ptr, B.val32.ptr, T.val.ptr);
  VSGB_LAUNCH_CHECK();
  T.dinv4.reserve(static_cast<size_t>(T.nb) * 4);
  k_dinv4<<<grid_for(T.nb, 256, 1024), 256, 0, s>>>(T.nb, dinv32,
                                                   reinterpret_cast<float4*>(T.dinv4.ptr));
  VSGB_LAUNCH_CHECK();
}

size_t mres_smem_cap(int device) {
  int optin = 0;
  VSGB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
  cudaFuncAttributes fa{};
  VSGB_CUDA(cudaFuncGetAttributes(&fa, reinterpret_cast<const void*>(k_mres)));
  const size_t stat = fa.sharedSizeBytes;
  return static_cast<size_t>(optin) > stat ? static_cast<size_t>(optin) - stat : 0;
}

int mres_ctas(int num_sms, size_t smem) {
  VSGB_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(k_mres),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
  int per_sm = 0;
  VSGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, reinterpret_cast<const void*>(k_mres), kMresThreads, smem));
  return per_sm >= 1 ? num_sms : 0;
}

void mres_solve(const MultiTiles& T, int n, const MresSolve& q, cudaStream_t s) {
  MresArgs a;
  a.nb = n / 3;
  a.n = n;
  a.ncols = q.ncols;
  a.tile_slice = T.tile_slice.ptr;
  a.tile_win = T.tile_win.ptr;
  a.win_row = T.win_row.ptr;
  a.slice_step = T.slice_step.ptr;
  a.slice_row = T.slice_row.ptr;
  a.slice_own = T.slice_own.ptr;
  a.col16 = T.col16.ptr;
  a.val = T.val.ptr;
  a.cta_tile = T.cta_tile.ptr;
  a.dinv32 = q.dinv32;
  a.diag32 = q.diag32;
  a.r64 = q.r64;
  a.u64 = q.u64;
  a.r = q.r;
  a.u = q.u;
  a.pa = q.pa;
  a.pb = q.pb;
  a.Ap = q.Ap;
  a.S = q.S;
  a.O = q.O;
  a.est = q.est;
  a.partials = q.partials;
  a.count = q.count;
  a.abort_flag = reinterpret_cast<int*>(q.count + 1);
  a.tol = q.tol;
  a.outer_tol = q.outer_tol;
  a.max_iters = q.max_iters;
  a.err_mode = q.err_mode;
  a.err_target = q.err_target;
  a.err_rel = q.err_rel;
  a.spin_limit = q.spin_limit > 0 ? q.spin_limit : (1LL << 22);
  a.accumulate = q.accumulate;
  a.dinv4 = reinterpret_cast<const float4*>(T.dinv4.ptr);
  const int mw = T.max_win;
  a.wp_off = mw * kWinFloats * static_cast<int>(sizeof(float));
  a.wd_off = 2 * a.wp_off;
  a.wrow_off = a.wd_off + 16 * mw;
  a.ring_off = (a.wrow_off + 4 * mw + 15) / 16 * 16;
  a.trace = q.trace;
  if (q.err_mode != kErrOff && !q.diag32)
    throw Error(VSGB_ERR_STATE, "error-controlled batched solve without the Jacobi diagonal");
  VSGB_CUDA(cudaFuncSetAttribute(reinterpret_cast<const void*>(k_mres),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(T.smem)));
  VSGB_CUDA(cudaMemsetAsync(q.count, 0, 2 * sizeof(unsigned), s));
  void* args[] = {&a};
  VSGB_CUDA(cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(k_mres), dim3(T.ctas),
                                        dim3(kMresThreads), args, T.smem, s));
}

}  // namespace vsgb
