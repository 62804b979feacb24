// include/vsgb/gb300_pcg_solver_backend.hpp
//
// C++20 SolverBackend for vibestran over the libvsgb C ABI: a drop-in for
// CudaPCGSolverBackend / CudaMixedPCGSolverBackend
// (include/solver/cuda_pcg_solver_backend.hpp:33-75,
//  include/solver/cuda_mixed_pcg_solver_backend.hpp) on a GB300 (sm_103a).
//
//   auto be = vibestran::Gb300PcgSolverBackend::try_create();   // nullopt: no GPU
//   LinearStaticSolver solver(std::make_unique<vibestran::Gb300PcgSolverBackend>(std::move(*be)));
//
// Header-only; link with -lvsgb.  Errors from the library are rethrown as
// vibestran::SolverError with the reference backend's messages.
#pragma once

#if defined(VSGB_IN_VIBESTRAN_TREE)
#include "core/exceptions.hpp"
#include "solver/solver_backend.hpp"
#else
#include "vsgb/vibestran_interface.hpp"
#endif

#include <optional>
#include <string>
#include <string_view>
#include <utility>
#include <vector>

#include "vsgb.h"

namespace vibestran {

class Gb300PcgSolverBackend : public SolverBackend {
 public:
  ~Gb300PcgSolverBackend() override { vsgb_destroy(ctx_); }
  Gb300PcgSolverBackend(Gb300PcgSolverBackend&& o) noexcept
      : ctx_(std::exchange(o.ctx_, nullptr)),
        precision_(o.precision_),
        name_(std::move(o.name_)),
        device_(std::move(o.device_)),
        stats_(o.stats_) {}
  Gb300PcgSolverBackend& operator=(Gb300PcgSolverBackend&& o) noexcept {
    if (this != &o) {
      vsgb_destroy(ctx_);
      ctx_ = std::exchange(o.ctx_, nullptr);
      precision_ = o.precision_;
      name_ = std::move(o.name_);
      device_ = std::move(o.device_);
      stats_ = o.stats_;
    }
    return *this;
  }
  Gb300PcgSolverBackend(const Gb300PcgSolverBackend&) = delete;
  Gb300PcgSolverBackend& operator=(const Gb300PcgSolverBackend&) = delete;

  /// nullopt when no sm_103 device is present (cuda_pcg_solver_backend.cu:19-25).
  /// tolerance <= 0 selects 1e-8; max_iters <= 0 selects 10000.
  [[nodiscard]] static std::optional<Gb300PcgSolverBackend> try_create(
      double tolerance = 0.0, int max_iters = 0, int device = 0) noexcept {
    return create(tolerance, max_iters, device, VSGB_FP64);
  }

  [[nodiscard]] std::vector<double> solve(
      const SparseMatrixBuilder::CsrData& K, const std::vector<double>& F,
      const FactorRatioCheckPolicy* = nullptr) override {
    if (K.n == 0) throw SolverError("CUDA PCG: stiffness matrix is empty -- no free DOFs");
    if (static_cast<int>(F.size()) != K.n)
      throw SolverError("CUDA PCG: force vector size " + std::to_string(F.size()) +
                        " != matrix size " + std::to_string(K.n));
    std::vector<double> u(static_cast<size_t>(K.n), 0.0);
    const int rc = vsgb_solve_csr(ctx_, K.n, K.nnz, K.row_ptr.data(), K.col_ind.data(),
                                  K.values.data(), K.stores_lower_triangle_only() ? 1 : 0,
                                  F.data(), 1, u.data(), &stats_);
    if (rc != VSGB_OK) throw SolverError(last_error());
    return u;
  }

  [[nodiscard]] std::string_view name() const noexcept override { return name_; }
  [[nodiscard]] int last_iteration_count() const noexcept override { return stats_.iterations; }
  [[nodiscard]] double last_relative_residual() const noexcept { return stats_.rel_residual; }
  [[nodiscard]] double last_estimated_error() const noexcept override {
    return stats_.rel_residual;
  }
  [[nodiscard]] std::string_view device_name() const noexcept { return device_; }
  [[nodiscard]] const vsgb_stats& last_stats() const noexcept { return stats_; }
  [[nodiscard]] vsgb_ctx* context() const noexcept { return ctx_; }

  /// vsgb_set_option (VSGB_OPT_*); the display name follows the
  /// preconditioner (VSGB_OPT_PRECOND).
  void set_option(int option, double value) {
    if (vsgb_set_option(ctx_, option, value) != VSGB_OK) throw SolverError(last_error());
    char buf[256];
    if (vsgb_backend_name(ctx_, buf, sizeof buf) == VSGB_OK) name_ = buf;
  }

 protected:
  static std::optional<Gb300PcgSolverBackend> create(double tol, int max_iters, int device,
                                                     int precision) noexcept {
    vsgb_ctx* c = nullptr;
    if (vsgb_create(device, tol, max_iters, precision, &c) != VSGB_OK || !c) return std::nullopt;
    return Gb300PcgSolverBackend(c, precision);
  }
  Gb300PcgSolverBackend(vsgb_ctx* c, int precision) noexcept : ctx_(c), precision_(precision) {
    char buf[256];
    if (vsgb_backend_name(c, buf, sizeof buf) == VSGB_OK) name_ = buf;
    if (vsgb_device_name(c, buf, sizeof buf) == VSGB_OK) device_ = buf;
  }
  std::string last_error() const {
    char buf[1024] = {0};
    vsgb_last_error(ctx_, buf, sizeof buf);
    return buf;
  }

  vsgb_ctx* ctx_ = nullptr;
  int precision_ = VSGB_FP64;
  std::string name_;
  std::string device_;
  vsgb_stats stats_{};
};

/// CudaMixedPCGSolverBackend counterpart: FP32 inner PCG, FP64 refinement on
/// the GPU; tolerance <= 0 selects 1e-6 (cuda_mixed_pcg_solver_backend.cu:25-33).
class Gb300MixedPcgSolverBackend final : public Gb300PcgSolverBackend {
 public:
  Gb300MixedPcgSolverBackend(Gb300MixedPcgSolverBackend&&) noexcept = default;
  Gb300MixedPcgSolverBackend& operator=(Gb300MixedPcgSolverBackend&&) noexcept = default;

  [[nodiscard]] static std::optional<Gb300MixedPcgSolverBackend> try_create(
      double tolerance = 0.0, int max_iters = 0, int device = 0) noexcept {
    vsgb_ctx* c = nullptr;
    if (vsgb_create(device, tolerance, max_iters, VSGB_MIXED, &c) != VSGB_OK || !c)
      return std::nullopt;
    return Gb300MixedPcgSolverBackend(c);
  }

 private:
  explicit Gb300MixedPcgSolverBackend(vsgb_ctx* c) noexcept : Gb300PcgSolverBackend(c, VSGB_MIXED) {}
};

}  // namespace vibestran
