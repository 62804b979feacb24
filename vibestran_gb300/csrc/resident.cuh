// vibestran_gb300/csrc/resident.cuh — persistent (SM-resident) Jacobi or 3x3
// block Jacobi PCG on the 3x3 block operator: one cooperative launch runs
// every iteration of a solve.
#pragma once

#include <vector>

#include "bsr.cuh"
#include "common.cuh"
#include "errest.cuh"

namespace vsgb {

struct ResidentPlan {
  bool ok32 = false, ok64 = false;  // usable for FP32 inner / FP64 solves
  bool win32 = false, win64 = false;  // x window staged in shared memory
  bool ug32 = false, ug64 = false;    // solution accumulator in global memory
  bool defl32 = false;                // the deflated FP32 solve fits the plan too
  int ctas = 0, threads = 0;
  size_t smem32 = 0, smem64 = 0;
  int max_slices = 0;               // slices of the largest CTA range
  int max_win = 0;                  // nodes of the largest x window
  DevBuf<int> cta_slice;            // ctas + 1: slice range of each CTA
  DevBuf<int> cta_win;              // 2 * ctas: [first, last] block column per CTA
  DevBuf<int> cta_runs;             // per CTA: the runs of its window its columns reference
  DevBuf<int> slice_mm;             // 2 * nslices: column range per slice (planning scratch)
  DevBuf<double> partials;          // 2 barrier slots x ctas x up to 6 values
  DevBuf<unsigned> barrier;         // monotonic arrival counter
  DevBuf<unsigned long long> fx;    // FP32 solve: fused reduction words
  DevBuf<float> u32g;                       // FP32 solution accumulator when ug32
  DevBuf<float> z4f, p4fa, p4fb;    // node-padded FP32 vectors (4 per node)
  DevBuf<double> z4d, p4da, p4db;   // node-padded FP64 vectors
  // 3x3 block Jacobi: inverse diagonal block of every node, upper triangle
  // (xx, xy, xz, yy, yz, zz), FP64 and its FP32 copy for the inner solve
  DevBuf<double> bj64;
  DevBuf<float> bj32;
  DevBuf<float> bjd32;              // the diagonal blocks themselves (upper triangle, FP32)
  DevBuf<int> bj_bad;               // smallest node whose block is not SPD
  DevBuf<float> diag32;             // Jacobi diagonal (FP32) for the error estimate
  DevBuf<unsigned long long> trace; // phase timer, kTraceWords per CTA
};

constexpr int kTracePhases = 9;  // gather, SpMV, 3 x reduction 1, update, 3 x reduction 2
constexpr int kTraceWords = 10;  // the phases and the iteration count

// Polls of a grid wait of the persistent solve before it gives up (~1 s).
constexpr long long kDefaultSpinLimit = 1LL << 22;

// Stopping and wait controls of one persistent solve.
struct ResidentCtl {
  double tol = 0.0;          // residual tolerance (err_mode == kErrOff)
  int max_iters = 0;
  int err_mode = 0;          // ErrMode (errest.cuh)
  double err_target = 0.0;   // kErrAbsolute: target relative to ||u||_D of the outer record
  double err_rel = 0.0;      // relative floor (kErrAbsolute) or relative target (kErrRelative)
  long long spin_limit = kDefaultSpinLimit;
  bool block_jacobi = false; // 3x3 block Jacobi instead of the scalar one
  bool trace = false;        // time the phases of every iteration (P.trace)
  // FP32 solve: Lanczos record (z_k of the first hist_max iterations, node
  // padded, and alpha_k, beta_k, r_k.z_k); null: off
  float* hist = nullptr;
  double* coef = nullptr;
  int hist_max = 0;
  // FP32 solve deflated by 4 coarse vectors (null: off; coarse.cuh): W
  // node-padded (4 x 4 nb), A W (4 x n), (W^T A W)^-1 (4 x 4) and bounds c_i
  // with |(A w_i).z| <= c_i sqrt(r.z)
  const float* defl_w = nullptr;
  const float* defl_aw = nullptr;
  const float* defl_ginv = nullptr;
  const double* defl_c = nullptr;
};

// Plans CTA ranges / windows and allocates the padded vectors; leaves both
// ok flags false when the device or the operator does not allow it.
void resident_prepare(const BsrSell& B, bool need32, int device, int num_sms, ResidentPlan& P,
                      cudaStream_t s);

// Inverts the 3x3 diagonal block of every node of the FP64 operator into
// P.bj64 (and P.bj32 when need32).  Returns -1, or the smallest node whose
// block is not symmetric positive definite (nothing is usable then).
int resident_block_jacobi(const BsrSell& B, ResidentPlan& P, bool need32, cudaStream_t s);

// One FP32 inner solve: rhs = (float)(r64 * O->scale); on convergence
// u64 += delta / O->scale.  Final counts/flags land in *S (S->abort set when
// any CTA's grid wait gave up).  ctl.block_jacobi selects the 3x3 block
// preconditioner in P.bj32 instead of dinv.
void resident_solve32(const BsrSell& B, ResidentPlan& P, const double* r64, double* u64,
                      PcgScalars* S, const PcgScalars* O, const ResidentCtl& ctl, cudaStream_t s,
                      const double* dinv);

// One FP64 solve of K u = f; u written (zeros on a zero RHS).
void resident_solve64(const BsrSell& B, ResidentPlan& P, const double* f, double* u,
                      PcgScalars* S, const ResidentCtl& ctl, cudaStream_t s,
                      const double* dinv);

// Phase times of the last traced launch: sums over its iterations, averaged
// over the CTAs (kTracePhases values in ns: gather, SpMV, first reduction as
// CTA sums / wait for the other CTAs / total and recurrence, update, second
// reduction likewise), the largest CTA's SpMV sum and the iteration count.
void resident_trace(const ResidentPlan& P, cudaStream_t s, double* sums_ns, double* max_spmv_ns,
                    long long* iterations);

// P.diag32 = 1 / dinv (needed by error-controlled solves with scalar Jacobi).
void resident_diag(ResidentPlan& P, const double* dinv, int n, int num_sms, cudaStream_t s);

// Flag set in PcgScalars::flags when a grid barrier gave up waiting.
constexpr int kFlagResidentAbort = 64;

}  // namespace vsgb
