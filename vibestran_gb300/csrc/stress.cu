// vibestran_gb300/csrc/stress.cu — CHEXA8 stress recovery on the GPU (FP64).
//
// LinearStaticSolver::recover_results, solid branch
// (src/solver/linear_static.cpp:1059-1195): for each element the stress
// sigma = D (B u_e) at the centroid and at the 8 corner nodes (xi = +-1), with
// u_e the element's displacements (constrained DOFs zero, :661-672), B the
// 6x24 strain-displacement matrix of the plain trilinear element (no EAS
// modes in recovery; rows xx, yy, zz, xy, yz, zx, engineering shears,
// :1088-1113), D = solid_constitutive_matrix (:119-138) and von Mises as
// solid_von_mises (:140-150).  The thermal strain of solid_sigma_from_B
// (:186-196) is zero: no TEMP loads are on this path.
//
// One thread per (element, point), nine per element: every FP64 instruction
// runs on a full warp (GB300 issues one FP64 warp instruction per ~17 cycles
// per SM whatever its active lanes).  A thread keeps only J^-1 and the nine
// displacement gradients in registers; dN is recomputed per node for the
// second pass.  ~250 FP64 operations per point; the element's coordinates
// and displacements are read by its nine threads through L1.

#include "common.cuh"
#include "kernels.cuh"

namespace vsgb {

namespace {

// Node signs of the CHEXA8 node order (src/elements/solid_elements.cpp:76-93)
// as bit masks, bit n set for +1: xi, eta, zeta.
constexpr unsigned kPosXi = 0x66u, kPosEta = 0xCCu, kPosZeta = 0xF0u;

__device__ __forceinline__ double sgn(unsigned mask, int n) {
  return ((mask >> n) & 1u) ? 1.0 : -1.0;
}

// dN_n / d(xi, eta, zeta) at (a, b, c).
__device__ __forceinline__ void hex_dn(int n, double a, double b, double c, double& d0,
                                       double& d1, double& d2) {
  const double sa = sgn(kPosXi, n), sb = sgn(kPosEta, n), sc = sgn(kPosZeta, n);
  const double fa = fma(sa, a, 1.0), fb = fma(sb, b, 1.0), fc = fma(sc, c, 1.0);
  d0 = 0.125 * sa * fb * fc;
  d1 = 0.125 * sb * fa * fc;
  d2 = 0.125 * sc * fa * fb;
}

__global__ void k_solid_stress(int n_elem, const double* __restrict__ xyz,
                               const int* __restrict__ conn, const int* __restrict__ eq3,
                               const double2* __restrict__ lame, const double* __restrict__ u,
                               int n_dof, double* __restrict__ centroid,
                               double* __restrict__ nodal) {
  const long long total = 9LL * n_elem;
  for (long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
       t += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int e = static_cast<int>(t / 9), pt = static_cast<int>(t - 9LL * e);
    // point 0: centroid; point k >= 1: corner node k-1 (kHexCoords, :1165-1174)
    const double a = pt == 0 ? 0.0 : sgn(kPosXi, pt - 1);
    const double b = pt == 0 ? 0.0 : sgn(kPosEta, pt - 1);
    const double c = pt == 0 ? 0.0 : sgn(kPosZeta, pt - 1);
    const int* cn = conn + 8 * static_cast<size_t>(e);
    // J rows d/dxi_i, columns x, y, z
    double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int nd = __ldg(cn + n);
      double d[3];
      hex_dn(n, a, b, c, d[0], d[1], d[2]);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double x = __ldg(xyz + 3 * static_cast<size_t>(nd) + k);
#pragma unroll
        for (int i = 0; i < 3; ++i) J[i][k] = fma(d[i], x, J[i][k]);
      }
    }
    const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const double c01 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    const double c02 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    const double det = J[0][0] * c00 + J[1][0] * c01 + J[2][0] * c02;
    const double id = 1.0 / det;
    double Ji[3][3];
    Ji[0][0] = c00 * id;
    Ji[0][1] = c01 * id;
    Ji[0][2] = c02 * id;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) * id;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) * id;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
    // du[c][i] = d u_c / d x_i
    double du[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
#pragma unroll
    for (int n = 0; n < 8; ++n) {
      const int nd = __ldg(cn + n);
      double d[3];
      hex_dn(n, a, b, c, d[0], d[1], d[2]);
      double g[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) g[i] = Ji[i][0] * d[0] + Ji[i][1] * d[1] + Ji[i][2] * d[2];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int eq = __ldg(eq3 + 3 * static_cast<size_t>(nd) + k);
        const double uv = (eq >= 0 && eq < n_dof) ? __ldg(u + eq) : 0.0;
#pragma unroll
        for (int i = 0; i < 3; ++i) du[k][i] = fma(g[i], uv, du[k][i]);
      }
    }
    const double2 lm = __ldg(&lame[e]);
    const double lam = lm.x, mu = lm.y;
    const double exx = du[0][0], eyy = du[1][1], ezz = du[2][2];
    const double tr = exx + eyy + ezz;
    double s[7];
    s[0] = lam * tr + 2.0 * mu * exx;
    s[1] = lam * tr + 2.0 * mu * eyy;
    s[2] = lam * tr + 2.0 * mu * ezz;
    s[3] = mu * (du[0][1] + du[1][0]);
    s[4] = mu * (du[1][2] + du[2][1]);
    s[5] = mu * (du[2][0] + du[0][2]);
    const double d01 = s[0] - s[1], d12 = s[1] - s[2], d20 = s[2] - s[0];
    s[6] = sqrt(0.5 * (d01 * d01 + d12 * d12 + d20 * d20 +
                       6.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5])));
    double* out = pt == 0 ? centroid + 7 * static_cast<size_t>(e)
                          : (nodal ? nodal + 7 * (8 * static_cast<size_t>(e) + (pt - 1)) : nullptr);
    if (out)
#pragma unroll
      for (int k = 0; k < 7; ++k) out[k] = s[k];
  }
}

}  // namespace

// Nodal displacements (recover_results, src/solver/linear_static.cpp:581-587):
// thread per node, out[6 i + d] = u[eq] of its translational DOF d when free,
// else 0; R1-R3 are 0 (solid elements activate T1-T3 only, so the DOF map
// constrains the rotations of every node of this path).
__global__ void k_node_displacements(int n_nodes, const int* __restrict__ eq3,
                                     const double* __restrict__ u, int n_dof,
                                     double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += gridDim.x * blockDim.x) {
    double d[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const int eq = eq3[3 * i + q];
      if (eq >= 0 && eq < n_dof) d[q] = u[eq];
    }
    double2* o = reinterpret_cast<double2*>(out + 6 * static_cast<size_t>(i));
    o[0] = make_double2(d[0], d[1]);
    o[1] = make_double2(d[2], d[3]);
    o[2] = make_double2(d[4], d[5]);
  }
}

void launch_node_displacements(int n_nodes, const int* eq3, const double* u, int n_dof,
                               double* out, int num_sms, cudaStream_t s) {
  if (n_nodes <= 0) return;
  const int grid = grid_for(n_nodes, kThreads, num_sms * 8);
  k_node_displacements<<<grid, kThreads, 0, s>>>(n_nodes, eq3, u, n_dof, out);
  VSGB_LAUNCH_CHECK();
}

void launch_solid_stress(int n_elem, const double* xyz, const int* conn, const int* eq3,
                         const double* E, const double* nu, const double* u, int n_dof,
                         double* lame, double* centroid, double* nodal, int num_sms,
                         cudaStream_t s) {
  if (n_elem <= 0) return;
  launch_lame(n_elem, E, nu, lame, num_sms, s);
  const int grid = grid_for(9LL * n_elem, kThreads, num_sms * 16);
  k_solid_stress<<<grid, kThreads, 0, s>>>(n_elem, xyz, conn, eq3,
                                           reinterpret_cast<const double2*>(lame), u, n_dof,
                                           centroid, nodal);
  VSGB_LAUNCH_CHECK();
}

}  // namespace vsgb
