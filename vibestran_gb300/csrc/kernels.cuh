// vibestran_gb300/csrc/kernels.cuh — host-side launch interfaces of the device kernels.
#pragma once

#include "common.cuh"

namespace vsgb {

// ── element.cu ─────────────────────────────────────────────────────────────

struct ElementError {
  int index;  // smallest failing element index (INT_MAX when none)
  int code;   // 1 non-positive Jacobian, 2 EAS Kaa not SPD
};

__device__ __forceinline__ void record_element_error(ElementError* err, int e, int code) {
  const int old = atomicMin(&err->index, e);
  if (e <= old) atomicExch(&err->code, code);
}

size_t element_smem_bytes();
// Per-element Lame constants (lambda, mu) of isotropic_D into lame[2 * n_elem].
void launch_lame(int n_elem, const double* E, const double* nu, double* lame, int num_sms,
                 cudaStream_t s);
// CHEXA8 centroid (n_elem x 7) and corner (n_elem x 8 x 7, may be null)
// stresses from the displacements u[n_dof] (stress.cu); lame: 2 * n_elem scratch.
void launch_node_displacements(int n_nodes, const int* eq3, const double* u, int n_dof,
                               double* out, int num_sms, cudaStream_t s);
void launch_solid_stress(int n_elem, const double* xyz, const int* conn, const int* eq3,
                         const double* E, const double* nu, const double* u, int n_dof,
                         double* lame, double* centroid, double* nodal, int num_sms,
                         cudaStream_t s);
// lame: scratch of 2 * n_elem doubles (per-element lambda, mu).
void launch_chexa8_stiffness(int n_elem, const double* xyz, const int* conn, const double* E,
                             const double* nu, const int* form, double* kbuf, ElementError* err,
                             double* lame, int num_sms, cudaStream_t s);
// out[e] = -lam_e^T (K_e / E_e) u_e; with lam2/out2 non-null the same pass
// also gives out2[e] = -lam2_e^T (K_e / E_e) u_e (K_e u_e is formed once).
void launch_element_sensitivity(int n_elem, const int* conn, const int* eq3, const double* E,
                                const double* kbuf, const double* u, const double* lam,
                                double* out, const double* lam2, double* out2, int num_sms,
                                cudaStream_t s);

// ── assembly.cu ────────────────────────────────────────────────────────────

struct AssemblyError {
  int code;   // 1 duplicate equation, 2 equation/column out of range, 3 valence limit,
              // 4 zero diagonal, 5 missing diagonal, 6 node index out of range
  int index;
};

// Device scratch for the pattern build, sized from the mesh.
struct AssemblyScratch {
  DevBuf<int> node_cnt, node_ptr, node_elem, dof_node, row_cnt, lower_rp, scan_tmp, flag;
  DevBuf<long long> total;
  DevBuf<unsigned long long> counts;  // block assembly: scalar nnz full / lower, blocks
  DevBuf<int> max_valence;            // block assembly: most elements at one node
  DevBuf<AssemblyError> err;
};

// Builds the full (both triangles) CSR of K from the element stiffness buffer.
// Outputs: row_ptr[n+1], col_ind/values sized by the returned nnz; dinv[n].
struct AssembledCsr {
  DevBuf<int> row_ptr, col_ind;
  DevBuf<double> values;
  DevBuf<double> dinv;
  int n = 0;
  long long nnz = 0;
  long long nnz_lower = 0;
};

void assemble_csr(int n_nodes, int n_elem, const int* conn, const int* eq3, int n_dof,
                  const double* kbuf, AssemblyScratch& scr, AssembledCsr& out, int num_sms,
                  cudaStream_t s);

// Lower-triangle extraction (the reference's CsrData storage).
void extract_lower(const AssembledCsr& full, int* d_row_ptr, int* d_col_ind, double* d_values,
                   AssemblyScratch& scr, int num_sms, cudaStream_t s);

// Expand a lower-storage CSR on the device into full storage (both triangles,
// rows sorted by column) and compute the inverse diagonal.  Full-storage
// input is copied.  Errors (zero/missing diagonal, bad index) are reported
// through scr.err.
void prepare_full_csr(int n, long long nnz, const int* rp, const int* ci, const double* v,
                      bool lower, AssemblyScratch& scr, AssembledCsr& out, int num_sms,
                      cudaStream_t s);

// ── pcg.cu ─────────────────────────────────────────────────────────────────

}  // namespace vsgb
