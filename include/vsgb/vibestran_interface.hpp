// include/vsgb/vibestran_interface.hpp
//
// Stand-alone declarations of the vibestran types the GB300 backend plugs
// into, for builds outside the vibestran source tree (the conformance driver
// and the tests here).  Inside vibestran, gb300_pcg_solver_backend.hpp
// includes the real headers instead.  The declarations keep the reference's
// names, members and virtual signatures so the backend class compiles
// unchanged against either:
//   - SparseMatrixBuilder::CsrData / SymmetryStorage
//     (include/core/sparse_matrix.hpp:28-31, 63-87)
//   - SolverBackend (include/solver/solver_backend.hpp:20-51)
//   - SolverError (include/core/exceptions.hpp:14-17)
#pragma once

#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

namespace vibestran {

class SolverError : public std::runtime_error {
 public:
  explicit SolverError(const std::string& msg) : std::runtime_error(msg) {}
};

enum class SymmetryStorage { Full, Lower };

struct FactorRatioCheckPolicy;

class SparseMatrixBuilder {
 public:
  struct CsrData {
    std::vector<int> row_ptr;    // n + 1
    std::vector<int> col_ind;    // nnz
    std::vector<double> values;  // nnz
    int n = 0;
    int nnz = 0;
    SymmetryStorage symmetry{SymmetryStorage::Full};

    [[nodiscard]] bool stores_lower_triangle_only() const noexcept {
      return symmetry == SymmetryStorage::Lower;
    }
  };
};

class SolverBackend {
 public:
  virtual ~SolverBackend() = default;
  [[nodiscard]] virtual std::vector<double> solve(
      const SparseMatrixBuilder::CsrData& K, const std::vector<double>& F,
      const FactorRatioCheckPolicy* factor_ratio_policy = nullptr) = 0;
  [[nodiscard]] virtual std::string_view name() const noexcept = 0;
  [[nodiscard]] virtual int last_iteration_count() const noexcept { return -1; }
  [[nodiscard]] virtual double last_estimated_error() const noexcept { return -1.0; }
  [[nodiscard]] virtual bool requires_full_symmetric_csr() const noexcept { return false; }
};

}  // namespace vibestran
