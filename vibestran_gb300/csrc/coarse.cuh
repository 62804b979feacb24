// vibestran_gb300/csrc/coarse.cuh — coarse (Ritz) correction of the mixed
// refinement.
//
// The FP32 inner solves converge slowest on the smooth, small-eigenvalue
// modes, and their error there is the one no estimate from the recurrence
// sees: a refinement step's CG can run 100-300 iterations before its Krylov
// space finds the lowest mode again, while the error it left there (measured:
// 1.2e-6 of ||u|| on the 84k cantilever) sits unchanged and the estimate of
// the step falls.  The first inner solve on an operator records its Lanczos
// vectors (z_k / sqrt(r_k.z_k), alternating signs) and scalars; the lowest
// Ritz pairs of its tridiagonal (bisection on Sturm counts, inverse iteration)
// give m vectors Z = V Y that approximate the lowest modes.  After every FP64
// residual of the refinement the iterate gets the Galerkin correction in
// span(Z) with the FP64 operator (Rayleigh-Ritz, two-level deflation in the
// sense of Nicolaides 1987 / Frank & Vuik 2001, applied between steps):
//   c = (Z^T K Z)^-1 Z^T r,   u += Z c,   r -= (K Z) c,
// which removes the error in those modes to the Ritz vectors' accuracy.
// The basis depends on the operator only; it is kept per operator generation.
#pragma once

#include <vector>

#include "common.cuh"

namespace vsgb {

constexpr int kCoarseMax = 8;        // basis vectors at most
constexpr int kCoarseHistMax = 512;  // Lanczos vectors recorded at most

struct CoarseSpace {
  bool valid = false;
  unsigned gen = ~0u;   // operator generation of the basis
  int m = 0, n = 0;
  DevBuf<double> Z, KZ;  // m x n each (vector i at i * n)
  DevBuf<double> L;      // Cholesky factor of Z^T K Z (lower, row stride kCoarseMax)
  DevBuf<int> meff;      // vectors the factor covers (device; 0: no correction)
  DevBuf<double> part;   // reduction partials
  DevBuf<double> c;      // coefficients of the last correction (m x 16)
  DevBuf<unsigned> counter;
  DevBuf<float> W;           // K x m combination weights of the Lanczos vectors
  std::vector<float> Wh;     // their host copy (pinned by the next copy only)
  std::vector<double> ritz;  // the Ritz values used (smallest first)
  // host part of a basis computed ahead (coarse_host_basis): the Ritz pairs
  // of a record of pre_K iterations for operator generation pre_gen, found
  // vectors (Wh, ritz); pre_found < 0: none
  int pre_found = -1, pre_K = 0;
  unsigned pre_gen = ~0u;
  // deflated FP32 inner solves (resident.cu, 4 vectors, the unused ones
  // zero): W node-padded, A W, (W^T A W)^-1 and the bounds c_i
  bool defl_ready = false;
  DevBuf<float> w32, aw32, ginv32;
  DevBuf<double> cbound;
};

// Prepares the FP32 deflation arrays of a built basis (dinv: the Jacobi
// inverse diagonal, for the bounds c_i^2 = sum_g (A w_i)_g^2 dinv_g).
void coarse_deflation_prep(CoarseSpace& cs, const double* dinv, int num_sms, cudaStream_t s);

// Lowest m eigenpairs of the symmetric tridiagonal (diag d, off-diagonal e,
// size k): values ascending in w, vectors column-major in Y (k x m).  Ritz
// values closer than 1e-6 (relative) to the previous one are ghosts of
// finite-precision Lanczos and are skipped.  Returns the pairs found.
int tridiag_lowest(const std::vector<double>& d, const std::vector<double>& e, int m,
                   std::vector<double>& w, std::vector<double>& Y);

// Builds the basis from a Lanczos record: hist (K slots of 4 * nb floats,
// node-padded, or of n = 3 nb floats), coef (alpha_k, beta_k, r_k.z_k for
// k < K).  spmm64(Z, KZ, m) applies the FP64 operator to the m basis
// vectors (vector i at i * n, m <= 4).  False (and cs.valid
// false) when fewer than 8 iterations were recorded, the recurrence is not
// that of an SPD solve, or no positive-definite coarse matrix resulted.
template <typename SpMM>
bool coarse_build(CoarseSpace& cs, const float* hist, bool padded,
                  const std::vector<double>& coef, int K, int nb, int m, SpMM&& spmm64,
                  int num_sms, cudaStream_t s);

// Galerkin correction of one FP64 iterate: u += Z c, r -= K Z c with
// c = (Z^T K Z)^-1 Z^T r; refreshes the outer record O (rr, rel, scale and
// ||u||_D^2 with D = 1 / dinv) on the device.  Two launches, no host wait.
void coarse_apply(const CoarseSpace& cs, double* u, double* r, const double* dinv,
                  PcgScalars* O, int num_sms, cudaStream_t s);

// The same for the columns of FP64 panels [n][16] (columns with active[k]
// == 0 unchanged): refreshes rel, scale and uD2 of the batched outer record
// through the given pointers (16 doubles each; norm_f the columns' ||f||).
void coarse_apply_panel(const CoarseSpace& cs, double* U, double* R, const double* dinv,
                        const int* active, const double* norm_f, double* rel, double* scale,
                        double* uD2, int num_sms, cudaStream_t s);

// The host part of coarse_basis alone (the Ritz pairs of the record's
// tridiagonal and the weights Wh): returns the vectors found (0: no basis),
// without any CUDA call, so that it can run while the GPU works.
int coarse_host_basis(CoarseSpace& cs, const std::vector<double>& coef, int K, int m);

// Host part of coarse_build (the template forwards to it after K Z).
bool coarse_finish(CoarseSpace& cs, int num_sms, cudaStream_t s);
bool coarse_basis(CoarseSpace& cs, const float* hist, bool padded,
                  const std::vector<double>& coef, int K, int nb, int m, int num_sms,
                  cudaStream_t s);

template <typename SpMM>
bool coarse_build(CoarseSpace& cs, const float* hist, bool padded,
                  const std::vector<double>& coef, int K, int nb, int m, SpMM&& spmm64,
                  int num_sms, cudaStream_t s) {
  if (!coarse_basis(cs, hist, padded, coef, K, nb, m, num_sms, s)) return false;
  spmm64(cs.Z.ptr, cs.KZ.ptr, cs.m);
  return coarse_finish(cs, num_sms, s);
}

}  // namespace vsgb
