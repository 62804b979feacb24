// vibestran_gb300/csrc/pcg.cuh — PCG engine over a resident full-storage CSR.
#pragma once

#include <vector>

#include "bsr.cuh"
#include "coarse.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "resident.cuh"

namespace vsgb {

struct MultiWork;
void destroy_multi(MultiWork* w);

struct SolveResult {
  int iterations = 0;
  int inner_solves = 1;
  bool converged = false;
  bool breakdown = false;
  bool stalled = false;
  bool inner_failed = false;
  double rel = 0.0;
  double err_est = -1.0;  // error-controlled solve: estimated relative error (< 0: none)
  bool err_met = false;   // error-controlled solve: the error target was met
};

// Error-controlled stopping (errest.cuh): a solve aims at target / kErrSafety
// so that an estimate low by up to that factor still meets the target; a
// refinement step stops at the relative floor kErrRelFloor of its own
// correction at the latest (FP32 cannot deliver much more) and the next step
// continues from the FP64 residual.
constexpr double kErrSafety = 3.0;
constexpr double kErrRelFloor = 1e-4;

class PcgEngine {
 public:
  explicit PcgEngine(int num_sms) : num_sms_(num_sms) {}
  ~PcgEngine();
  PcgEngine(const PcgEngine&) = delete;
  PcgEngine& operator=(const PcgEngine&) = delete;

  // Binds the operator; builds the FP32 copy when need32.  With prebuilt the
  // block operator in blocks() was assembled directly and op holds n, dinv
  // and the nnz counts only (no scalar CSR).
  void prepare(const AssembledCsr& op, bool need32, cudaStream_t s, bool prebuilt = false);
  BsrSell& blocks() { return bsr_; }
  bool has32() const { return has32_; }

  // FP64 PCG on d_f; the solution is left in solution().
  void solve_fp64(const double* d_f, double tol, int max_iters, cudaStream_t s,
                  PcgScalars* host_pinned, SolveResult& res);
  // FP32 inner PCG + FP64 refinement on the GPU; solution in solution().
  // host_pinned holds two records (inner solve, outer residual).
  void solve_mixed(const double* d_f, double tol, double inner_tol, int max_iters,
                   int max_solves, cudaStream_t s, PcgScalars* host_pinned, SolveResult& res);

  const double* solution() const { return u_.ptr; }
  void time_spmv(int precision, int reps, cudaStream_t s, double* avg_ms);
  double spmv_bytes(int precision) const;

  void set_check_every(int k) { check_every_ = k < 2 ? 2 : (k + (k & 1)); }
  void set_use_graph(bool g) { use_graph_ = g; }
  // 0 auto (3x3 blocks when node-aligned), 1 scalar CSR, 2 blocks required.
  void set_format(int f) { format_ = f; }
  int format_used() const { return use_bsr_ ? 2 : 1; }
  // Persistent one-launch-per-solve kernels on the block operator (default on).
  void set_resident(bool r) { resident_ = r; }
  // Mark the operator values as persisting in L2 around each persistent
  // launch (CUDA access-policy window, reset after the launch).
  void set_l2_persist(bool on) { l2_persist_ = on; }
  // Mixed refinement: loosen later inner tolerances to what the outer
  // tolerance still needs (never tighter than the inner tolerance).
  void set_adaptive_inner(bool on) { adaptive_inner_ = on; }
  // 0: scalar Jacobi; 1: 3x3 block Jacobi (persistent solve on the block
  // operator only).
  void set_precond(int p) { precond_ = p; }
  // Relative displacement error target of error-controlled solves (<= 0:
  // the reference's residual test).  Persistent solves only.
  void set_error_target(double e) { err_target_ = e; }
  double error_target() const { return err_target_; }
  // Polls of a grid wait of the persistent solve before it gives up and the
  // solve fails with VSGB_ERR_CUDA (<= 0: the default, ~1 s).
  void set_spin_limit(long long k) { spin_limit_ = k > 0 ? k : kDefaultSpinLimit; }
  // Time the phases of every persistent-solve iteration (globaltimer, thread
  // 0 of each CTA); phase_times() then holds the last solve's per-iteration
  // means over CTAs (us): gather, SpMV, first reduction (CTA sums, wait for
  // the other CTAs, total and recurrence), update, second reduction (same
  // parts), then the slowest CTA's SpMV (us) and the iterations.  For the
  // tiled batched solve: [0] window staging, [1] multiply, [4] first
  // reduction, [5] update, [8] second reduction, [9] slowest multiply.
  void set_phase_trace(bool on) { trace_ = on; }
  const double* phase_times() const { return phase_us_; }
  int precond() const { return precond_; }
  bool resident_used(bool mixed) const {
    return resident_ && use_bsr_ && (mixed ? res_.ok32 : res_.ok64);
  }
  // Device time and iterations of the persistent launches of the last solve.
  double resident_ms() const { return resident_ms_; }
  long long resident_iterations() const { return resident_iters_; }
  long long launches() const { return launches_; }
  void add_launches(long long k) { launches_ += k; }
  int num_sms() const { return num_sms_; }

  // Batched PCG over several load cases (3x3 block operator only): every
  // iteration sweeps the matrix once for up to 16 right-hand sides, each
  // with its own alpha/beta and convergence test.  d_F and d_U are
  // column-major n x nrhs device arrays (load case k at F + k*n).  Mixed
  // precision runs FP32 inner solves with per-case FP64 refinement.
  bool multi_supported() const { return use_bsr_; }
  // Coordinates of the block rows (3 floats each) for the tiled batched
  // solve, and a key of the sparsity pattern they belong to (tiles are
  // rebuilt when it changes, their values re-gathered when the operator
  // does).  The vector must outlive the solves; null: no tiles.
  void set_block_coords(const std::vector<float>* xyz, unsigned long long pattern_key) {
    coords_ = xyz;
    pattern_key_ = pattern_key;
  }
  // Coarse (Ritz) space of error-controlled mixed solves (coarse.cuh): 0
  // off, 1 (default) the Galerkin correction after every FP64 residual, 2
  // that and, in later solves with the same operator, a first FP32 inner
  // solve deflated by the basis (single right-hand sides, scalar Jacobi; the
  // batched solve takes the correction only).
  void set_coarse(int mode) { coarse_mode_ = mode; }
  int coarse_size() const { return coarse_.valid ? coarse_.m : 0; }
  // Tiled batched FP32 solve: 0 off (default: the launch-per-kernel path
  // measured faster), 1 automatic (tile size timed on first use of a
  // sparsity pattern), >= 8 fixed rows per tile.
  void set_batch_tiles(int mode) { batch_tiles_ = mode; }
  // Rows per tile of the last batched solve (0: the launch-per-kernel path).
  int batch_tile_rows() const { return tile_rows_used_; }
  void solve_multi(const double* d_F, int nrhs, double* d_U, bool mixed, double tol,
                   double inner_tol, int max_iters, int max_solves, cudaStream_t s,
                   std::vector<SolveResult>& res);

 private:
  void ensure_vectors(bool mixed);
  void read_scalars(cudaStream_t s, PcgScalars* host, int which);
  void set_limits(cudaStream_t s, int which, double tol, int max_iters);
  void launch_spmv64(cudaStream_t s, const double* x, double* y);
  void launch_spmv32(cudaStream_t s, const float* pin, float* pout);
  void launch_residual64(cudaStream_t s, const double* d_f);
  void launch_batch64(cudaStream_t s);
  void launch_batch32(cudaStream_t s);
  void iterate(cudaStream_t s, bool fp32, PcgScalars* host);
  bool block_jacobi(bool mixed, cudaStream_t s);  // builds the blocks on first use
  void ensure_diag32(cudaStream_t s);             // FP32 Jacobi diagonal for the estimate

  int num_sms_;
  const AssembledCsr* op_ = nullptr;
  int n_ = 0;
  int vec_grid_ = 1, spmv_grid_ = 1;
  int check_every_ = 16;
  bool use_graph_ = true;
  bool has32_ = false;
  long long launches_ = 0;
  unsigned generation_ = 0;

  BsrSell bsr_;
  ResidentPlan res_;
  bool resident_ = true;
  bool use_bsr_ = false;
  int format_ = 0;
  int bsr_grid_ = 1;
  DevBuf<float> val32_, dinv32_;
  DevBuf<double> r_, z_, p_, Ap_, u_;
  DevBuf<float> r32_, z32_, p32a_, p32b_, Ap32_, u32_;
  DevBuf<PcgScalars> scal_;
  DevBuf<double> partials_;
  DevBuf<unsigned> counters_;

  cudaGraphExec_t graph_exec_[2] = {nullptr, nullptr};
  unsigned graph_gen_[2] = {0, 0};
  int graph_batch_[2] = {0, 0};
  PcgScalars* graph_host_[2] = {nullptr, nullptr};

  MultiWork* multi_ = nullptr;  // batched-solve buffers (multi.cu)
  // coarse correction: the basis, and the Lanczos record it is built from
  CoarseSpace coarse_;
  int coarse_mode_ = 1;
  DevBuf<float> hist_;
  DevBuf<double> coef_;
  std::vector<double> coef_h_;
  // the first inner solve of an operator records its Lanczos vectors; this
  // builds the basis from them (count = iterations recorded)
  void coarse_from_record(int count, cudaStream_t s, bool padded = true);
  const std::vector<float>* coords_ = nullptr;
  unsigned long long pattern_key_ = 0;
  int batch_tiles_ = 0;
  int tile_rows_used_ = 0;
  // the tiles of the batched FP32 solve for the current operator (false:
  // none fit, or no coordinates); autotunes on first use of a pattern
  bool ensure_tiles(MultiWork& W, int ncols, cudaStream_t s);
  double tile_ns_[6] = {};  // tiled-solve phase sums (ns, means over CTAs) + slowest multiply
  long long tile_its_ = 0;

  // Events around each persistent launch; the host syncs after every launch
  // anyway to read the scalar record.
  cudaEvent_t rev_[2] = {nullptr, nullptr};
  cudaStream_t copy_s_ = nullptr;  // reads a finished solve's record while later kernels run
  double resident_ms_ = 0.0;
  long long resident_iters_ = 0;
  void resident_begin(cudaStream_t s, const void* hot, size_t hot_bytes);  // before the launch
  void resident_end(cudaStream_t s);    // right after it (waits for it)
  void resident_finish(cudaStream_t s); // once rev_[1] (the launch's end) has completed
  bool l2_persist_ = false;
  bool adaptive_inner_ = true;
  int precond_ = 0;
  unsigned bj_gen_ = ~0u;  // operator generation the block inverses belong to
  unsigned diag_gen_ = ~0u;  // operator generation of res_.diag32
  double err_target_ = 0.0;
  long long spin_limit_ = kDefaultSpinLimit;
  bool trace_ = false;
  double phase_ns_[kTracePhases + 1] = {};  // sums over the traced launches (+ slowest SpMV)
  long long phase_its_ = 0;
  double phase_us_[kTracePhases + 2] = {};
  void trace_reset();
  void trace_add(cudaStream_t s);  // after a traced persistent launch completed
  bool l2_window_set_ = false;
  size_t l2_persist_max_ = 0;   // device limit (0: not supported)
  size_t l2_window_max_ = 0;
  size_t l2_prev_limit_ = 0;
};

}  // namespace vsgb
