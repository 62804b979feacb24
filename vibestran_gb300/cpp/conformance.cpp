// vibestran_gb300/cpp/conformance.cpp — the reference's CUDA PCG conformance
// cases (tests/unit/test_pcg_solver.cpp:243-425, CudaPCGTest and
// CudaMixedPCGTest) run against Gb300PcgSolverBackend /
// Gb300MixedPcgSolverBackend through the C++20 SolverBackend interface.
// Exit status 0 = all cases pass; 77 = no GPU (the GTEST_SKIP path).
//
// Build: g++ -std=c++20 -Iinclude conformance.cpp -Lvibestran_gb300/_lib -lvsgb

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <memory>
#include <tuple>
#include <vector>

#include "vsgb/gb300_pcg_solver_backend.hpp"

using vibestran::Gb300MixedPcgSolverBackend;
using vibestran::Gb300PcgSolverBackend;
using vibestran::SolverBackend;
using vibestran::SolverError;
using Csr = vibestran::SparseMatrixBuilder::CsrData;

namespace {

int g_fail = 0;

void check(bool ok, const char* what, int line) {
  if (!ok) {
    std::printf("  FAIL line %d: %s\n", line, what);
    ++g_fail;
  }
}
#define CHECK(x) check((x), #x, __LINE__)

// SparseMatrixBuilder::add + build_csr semantics: rows sorted by column,
// duplicates summed; lower_only tag when no entry lies above the diagonal.
Csr build(int n, std::vector<std::tuple<int, int, double>> t) {
  std::stable_sort(t.begin(), t.end(), [](auto& a, auto& b) {
    return std::get<0>(a) != std::get<0>(b) ? std::get<0>(a) < std::get<0>(b)
                                            : std::get<1>(a) < std::get<1>(b);
  });
  Csr c;
  c.n = n;
  c.row_ptr.assign(n + 1, 0);
  bool lower = true;
  for (size_t i = 0; i < t.size(); ++i) {
    auto [r, col, v] = t[i];
    if (r < col) lower = false;
    if (i > 0 && std::get<0>(t[i - 1]) == r && std::get<1>(t[i - 1]) == col) {
      c.values.back() += v;
      continue;
    }
    c.col_ind.push_back(col);
    c.values.push_back(v);
    c.row_ptr[r + 1]++;
  }
  for (int i = 0; i < n; ++i) c.row_ptr[i + 1] += c.row_ptr[i];
  c.nnz = static_cast<int>(c.values.size());
  c.symmetry = lower ? vibestran::SymmetryStorage::Lower : vibestran::SymmetryStorage::Full;
  return c;
}

Csr tridiagonal(int n, double d, double off, bool lower_only = false) {
  std::vector<std::tuple<int, int, double>> t;
  for (int i = 0; i < n; ++i) {
    t.emplace_back(i, i, d);
    if (i > 0) {
      t.emplace_back(i, i - 1, off);
      if (!lower_only) t.emplace_back(i - 1, i, off);
    }
  }
  return build(n, t);
}

// Dense LLT reference solve (the EigenSolverBackend role in the reference tests).
std::vector<double> direct(const Csr& K, const std::vector<double>& F) {
  const int n = K.n;
  std::vector<double> A(static_cast<size_t>(n) * n, 0.0);
  for (int r = 0; r < n; ++r)
    for (int k = K.row_ptr[r]; k < K.row_ptr[r + 1]; ++k) {
      const int c = K.col_ind[k];
      A[static_cast<size_t>(r) * n + c] += K.values[k];
      if (K.stores_lower_triangle_only() && c != r) A[static_cast<size_t>(c) * n + r] += K.values[k];
    }
  for (int j = 0; j < n; ++j) {
    double d = A[static_cast<size_t>(j) * n + j];
    for (int k = 0; k < j; ++k) d -= A[static_cast<size_t>(j) * n + k] * A[static_cast<size_t>(j) * n + k];
    const double l = std::sqrt(d);
    A[static_cast<size_t>(j) * n + j] = l;
    for (int i = j + 1; i < n; ++i) {
      double v = A[static_cast<size_t>(i) * n + j];
      for (int k = 0; k < j; ++k) v -= A[static_cast<size_t>(i) * n + k] * A[static_cast<size_t>(j) * n + k];
      A[static_cast<size_t>(i) * n + j] = v / l;
    }
  }
  std::vector<double> y(F);
  for (int i = 0; i < n; ++i) {
    for (int k = 0; k < i; ++k) y[i] -= A[static_cast<size_t>(i) * n + k] * y[k];
    y[i] /= A[static_cast<size_t>(i) * n + i];
  }
  for (int i = n - 1; i >= 0; --i) {
    for (int k = i + 1; k < n; ++k) y[i] -= A[static_cast<size_t>(k) * n + i] * y[k];
    y[i] /= A[static_cast<size_t>(i) * n + i];
  }
  return y;
}

void run_fp64(Gb300PcgSolverBackend& be) {
  std::printf("CudaPCGTest cases on %s / %s\n", std::string(be.name()).c_str(),
              std::string(be.device_name()).c_str());
  {  // DiagonalSystemExactSolution (:269-283)
    auto K = build(2, {{0, 0, 4.0}, {1, 1, 9.0}});
    auto u = be.solve(K, {8.0, 27.0});
    CHECK(u.size() == 2);
    CHECK(std::abs(u[0] - 2.0) < 1e-7 && std::abs(u[1] - 3.0) < 1e-7);
    CHECK(be.last_iteration_count() <= 1);
  }
  {  // TridiagonalAgreesWithEigen (:287-301) and lower-triangular variant (:303-319)
    for (int lower = 0; lower < 2; ++lower) {
      const int n = lower ? 8 : 5;
      auto K = tridiagonal(n, 3.0, -1.0, lower != 0);
      CHECK(K.stores_lower_triangle_only() == (lower != 0));
      std::vector<double> F(n, 1.0);
      auto u = be.solve(K, F);
      auto ud = direct(K, F);
      for (int i = 0; i < n; ++i) CHECK(std::abs(u[i] - ud[i]) < 1e-6);
    }
  }
  {  // LargerTridiagonalConverges (:323-339)
    auto K = tridiagonal(200, 2.0, -1.0);
    std::vector<double> F(200, 1.0);
    auto u = be.solve(K, F);
    auto ud = direct(K, F);
    for (int i = 0; i < 200; i += 20) CHECK(std::abs(u[i] - ud[i]) < 1e-5);
    CHECK(be.last_relative_residual() < 1e-7);
  }
  {  // StiffDiagonalDoesNotConvergeFalsely (:343-357)
    std::vector<std::tuple<int, int, double>> t;
    for (int i = 0; i < 100; ++i) t.emplace_back(i, i, 1.3e9);
    auto u = be.solve(build(100, t), std::vector<double>(100, 333.0));
    const double ex = 333.0 / 1.3e9;
    for (double v : u) CHECK(std::abs(v - ex) < ex * 1e-5);
  }
  {  // ZeroRhsReturnZeroDisplacement (:361-371)
    auto u = be.solve(tridiagonal(10, 3.0, -1.0), std::vector<double>(10, 0.0));
    for (double v : u) CHECK(std::abs(v) < 1e-15);
    CHECK(be.last_iteration_count() == 0);
  }
  {  // LargeBandedSpdAgreesWithEigen (:375-396)
    const int n = 500;
    std::vector<std::tuple<int, int, double>> t;
    for (int i = 0; i < n; ++i) {
      t.emplace_back(i, i, static_cast<double>(n + 1));
      if (i > 0) {
        t.emplace_back(i, i - 1, -1.0);
        t.emplace_back(i - 1, i, -1.0);
      }
      if (i > 1) {
        t.emplace_back(i, i - 2, -0.5);
        t.emplace_back(i - 2, i, -0.5);
      }
    }
    auto K = build(n, t);
    std::vector<double> F(n);
    for (int i = 0; i < n; ++i) F[i] = (i % 7) + 1;
    auto u = be.solve(K, F);
    auto ud = direct(K, F);
    for (int i = 0; i < n; i += 50) CHECK(std::abs(u[i] - ud[i]) < 1e-5);
  }
  {  // NameAndDeviceNameAreNonEmpty (:400-406)
    CHECK(!be.name().empty());
    CHECK(be.name().find("CUDA") != std::string_view::npos);
    CHECK(!be.device_name().empty());
  }
  {  // error semantics: size mismatch, empty K, zero diagonal, non-convergence
    bool threw = false;
    try {
      (void)be.solve(tridiagonal(4, 3.0, -1.0), std::vector<double>(3, 1.0));
    } catch (const SolverError&) {
      threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
      (void)be.solve(build(3, {{0, 0, 1.0}, {1, 1, 0.0}, {2, 2, 1.0}}), {1.0, 1.0, 1.0});
    } catch (const SolverError& e) {
      threw = std::string(e.what()).find("zero diagonal at row 1") != std::string::npos;
    }
    CHECK(threw);
  }
}

void run_mixed(Gb300MixedPcgSolverBackend& be) {
  std::printf("CudaMixedPCGTest cases on %s\n", std::string(be.name()).c_str());
  auto K = tridiagonal(200, 2.0, -1.0);  // (:408-425)
  std::vector<double> F(200, 1.0);
  auto u = be.solve(K, F);
  auto ud = direct(K, F);
  for (int i = 0; i < 200; i += 20) CHECK(std::abs(u[i] - ud[i]) < 5e-3);
  CHECK(be.last_estimated_error() < 1e-4);
  // options through the backend: the name follows the preconditioner, and a
  // bad value is reported as a SolverError
  be.set_option(VSGB_OPT_PRECOND, VSGB_PRECOND_BLOCK_JACOBI);
  CHECK(be.name().find("3x3 block Jacobi") != std::string_view::npos);
  be.set_option(VSGB_OPT_PRECOND, VSGB_PRECOND_JACOBI);
  CHECK(be.name().find("block") == std::string_view::npos);
  bool threw = false;
  try {
    be.set_option(VSGB_OPT_PRECOND, 7);
  } catch (const SolverError& e) {
    threw = std::string(e.what()).find("preconditioner must be") != std::string::npos;
  }
  CHECK(threw);
}

}  // namespace

int main() {
  auto be = Gb300PcgSolverBackend::try_create();
  if (!be) {
    std::printf("SKIP: no sm_103 CUDA device\n");
    return 77;
  }
  // Polymorphic use through the reference interface.
  std::unique_ptr<SolverBackend> as_base =
      std::make_unique<Gb300PcgSolverBackend>(std::move(*be));
  run_fp64(static_cast<Gb300PcgSolverBackend&>(*as_base));
  auto mixed = Gb300MixedPcgSolverBackend::try_create();
  CHECK(mixed.has_value());
  if (mixed) run_mixed(*mixed);
  std::printf(g_fail ? "FAILED (%d)\n" : "ALL PASS\n", g_fail);
  return g_fail ? 1 : 0;
}
