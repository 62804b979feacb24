// vibestran_gb300/csrc/errest.cuh — error-controlled stopping for PCG.
//
// The stopping test of the reference (cuda_pcg_backend_impl.hpp:723-729) is on
// the residual, sqrt(r.r)/||b|| < tol.  On these operators the error left at a
// given residual varies by orders of magnitude with the load: it sits in the
// smooth, small-eigenvalue modes, whose residual is tiny (84k cantilever tip
// load: error/residual ~ 4e-3; 16 random face-load cases: ~0.3 after a
// refinement step, ~4 after the first solve).  This file estimates the error
// itself, in the norm of the preconditioner M (the Jacobi diagonal D, or the
// 3x3 node blocks), which weights every DOF by its stiffness and follows the
// relative 2-norm error of the displacements closely (within a few percent
// on the meshes of this path).
//
// Published method: Hestenes and Stiefel's identity for CG (1952, Thm. 6:3),
// in its preconditioned form (Strakos and Tichy, BIT 45 (2005) 789-817):
//   ||e_k||_M^2 - ||e_{k+1}||_M^2 = c_k (||e_k||_A^2 + ||e_{k+1}||_A^2),
//   ||e_k||_A^2 - ||e_{k+1}||_A^2 = a_k,
//   a_k = alpha_k gamma_k,  c_k = (p_k^T M p_k) / (p_k^T A p_k),  gamma_k = r_k.z_k.
// Summed over a block of kErrBlock iterations with the A-norm tails taken at
// the block end m, S_b = sum_i c_i (A_i + A_{i+1}) = ||e_{m-16}||_M^2 -
// ||e_m||_M^2 (in exact arithmetic, up to the A-norm error left at m).  Two
// estimates are formed at every block end and both must meet the target:
//   * the error of the current iterate by a geometric tail,
//       ||e_m||_M^2 ~ S_b q / (1 - q),  q = the larger (slower) of the last two
//       block ratios S_b / S_{b-1}, S_{b-1} / S_{b-2} (no estimate if either >= 1);
//   * the delayed lower bound of the error 32 iterations back,
//       ||e_{m-32}||_M^2 >= S_b + S_{b-1} + 2 C_{b-1} A_b
//       (C = sum of c over a block, A = sum of a over a block),
//     which a slowly decreasing plateau cannot drive below its level;
// and the solve stops when two consecutive blocks pass.  CG on these
// operators alternates fast phases with plateaus in which a smooth mode not
// yet resolved keeps the error while the block sums drop; one block's tail
// estimate can then be low by 20x.  Measured on recorded FP32 solves (the
// uniform and the jittered heterogeneous 84k cantilevers, 16 random face-load
// cases of the 100x40x40 block, 20 cases of a small jittered block), this rule
// with target / 3 kept every true error below 3.4e-7 for a 1e-6 target.
// Summed over all blocks with the tails taken at the current iteration, the
// same identity gives ||x_m||_M^2 (x_0 = 0), the scale of a relative target.
#pragma once

namespace vsgb {

constexpr int kErrBlock = 16;

// Stopping mode of an error-controlled solve.
enum ErrMode : int {
  kErrOff = 0,       // residual test of the reference
  kErrAbsolute = 1,  // ||e||_M <= target (refinement step: target from ||u||_D of the outer iterate)
  kErrRelative = 2,  // ||e||_M <= rel ||x||_M
};

// Flag set when a solve stopped because the error target was met (as opposed
// to the relative floor of a refinement step, which asks for another step).
constexpr int kFlagErrTarget = 512;

struct ErrEst {
  double a[kErrBlock];  // alpha_i gamma_i of the current block
  double c[kErrBlock];  // p_i.M p_i / p_i.A p_i of the current block
  double s_hist[3];     // S of the last three blocks (newest first; < 0: none)
  double c_prev;        // C of the previous block
  double s_sum, c_sum, cp_sum, p_cum;  // running sums for ||x_m||_M^2
  double est2;          // last tail estimate of ||e_m||_M^2 (< 0: none)
  double lag2;          // last delayed estimate of ||e_{m-32}||_M^2 (< 0: none)
  double total2;        // ||x_m||_M^2 at the last block end
  int n;                // entries of the current block
  int pass_prev;        // the previous block met its target
};

__host__ __device__ inline void err_reset(ErrEst& e) {
  e.s_hist[0] = e.s_hist[1] = e.s_hist[2] = -1.0;
  e.c_prev = 0.0;
  e.s_sum = e.c_sum = e.cp_sum = e.p_cum = 0.0;
  e.est2 = e.lag2 = -1.0;
  e.total2 = 0.0;
  e.n = 0;
  e.pass_prev = 0;
}

// One iteration's coefficients a = alpha gamma and c = p.Mp / p.Ap (the
// caller forms them from the recurrence it already has, without a division
// of its own on the critical path).
__device__ inline void err_record(ErrEst& e, double a, double c) {
  if (e.n < kErrBlock) {
    e.a[e.n] = a;
    e.c[e.n] = c;
    ++e.n;
  }
}

// Called after every iteration; at a block end it folds the block in and
// returns true when this block and the one before met the target
// max(target2_abs, rel2 * ||x||_M^2).  Otherwise returns false.
__device__ inline bool err_block_end(ErrEst& e, double target2_abs, double rel2) {
  if (e.n < kErrBlock) return false;
  double A = 0.0, s = 0.0, csum = 0.0;
  for (int i = kErrBlock - 1; i >= 0; --i) {
    const double An = A;
    A += e.a[i];
    s += e.c[i] * (A + An);
    csum += e.c[i];
  }
  const double asum = A;
  e.n = 0;
  e.p_cum += asum;
  e.s_sum += s;
  e.c_sum += csum;
  e.cp_sum += csum * e.p_cum;
  e.total2 = e.s_sum + 2.0 * (e.p_cum * e.c_sum - e.cp_sum);
  const double s1 = e.s_hist[0], s2 = e.s_hist[1];
  double est2 = -1.0;
  if (s <= 0.0) {
    est2 = 0.0;  // no change over a whole block: converged to working precision
  } else if (s1 > 0.0 && s < s1) {
    double q = s / s1;
    if (s2 > 0.0) q = s1 < s2 ? fmax(q, s1 / s2) : 1.0;
    if (q < 1.0) est2 = s * q / (1.0 - q);
  }
  const double lag2 = s1 >= 0.0 ? s + s1 + 2.0 * e.c_prev * asum : -1.0;
  e.s_hist[2] = e.s_hist[1];
  e.s_hist[1] = e.s_hist[0];
  e.s_hist[0] = s;
  e.c_prev = csum;
  e.est2 = est2;
  e.lag2 = lag2;
  const double goal = fmax(target2_abs, rel2 * e.total2);
  const int pass = (est2 >= 0.0 && est2 <= goal && lag2 >= 0.0 && lag2 <= goal) ? 1 : 0;
  const bool stop = pass && e.pass_prev;
  e.pass_prev = pass;
  return stop;
}

// Refinement with an FP32 operator K32 = K + dK (mixed precision): a step's
// correction d_j solves K32 d = r, so besides the inner solve's error the
// step leaves (K^-1 - K32^-1) r ~ K^-1 dK d_j, which no estimate of the inner
// solve sees.  Its contraction rho = ||K^-1 dK d|| / ||d|| is a property of
// the operator (largest on the smooth modes, ~1e-4 to 1e-3 measured on these
// meshes); the ratio of successive corrections estimates it from above
// (the correction of a step is the error the step before left, the
// FP32-operator part plus that step's inner error): rho <= ||d_j|| /
// ||d_{j-1}||.  Squared bound on the FP32-operator part of the error after
// step j: (rho ||d_j||)^2 <= ||d_j||^4 / ||d_{j-1}||^2.
__host__ __device__ inline double refine_bound2(double dn2, double dprev2) {
  if (!(dn2 > 0.0)) return 0.0;
  return dprev2 > 0.0 ? dn2 * (dn2 / dprev2) : dn2;
}

}  // namespace vsgb
