// vibestran_gb300/csrc/bsr.cuh — 3x3 node-block sliced-ELL operator.
#pragma once

#include <vector>

#include "common.cuh"
#include "kernels.cuh"

namespace vsgb {

struct BsrSell {
  int nb = 0;              // block rows (n / 3)
  int nslices = 0;         // ceil(nb / 8)
  long long steps = 0;     // 32-lane steps over all slices
  long long nblocks = 0;   // stored (non-padding) blocks
  bool valid = false, has64 = false, has32 = false;
  DevBuf<int> slice_ptr;   // nslices + 1, in steps
  DevBuf<int> rowlen;      // blocks per block row
  DevBuf<int> cols;        // steps * 32
  DevBuf<double> val64;    // steps * 32 * 9
  // FP32 copy in difference form: the diagonal block of block row I holds
  // R_I = sum_J K_IJ (summed in FP64), the other blocks K_IJ rounded, and
  // every FP32 block product computes y_I = sum_{J != I} K_IJ (x_J - x_I) +
  // R_I x_I.  K annihilates rigid translations, so R_I is ~0 away from the
  // constraints and the differences are small for smooth x: the rounding of
  // K to FP32 then perturbs the smooth, small-eigenvalue modes far less than
  // in the plain product (fewer FP32 iterations after each refinement).
  DevBuf<float> val32;     // steps * 32 * 9
  DevBuf<int> tmp;
  DevBuf<int> slice_steps;  // scratch of bsr_layout (kept: a free would synchronise the device)
  DevBuf<long long> total;
  std::vector<int> h_blen;
};

// Converts the full-storage CSR into the block layout; returns false (and
// leaves B.valid false) when the equations are not node-aligned triples or the
// blocks are less than 90% filled.
bool build_bsr(const AssembledCsr& K, BsrSell& B, bool need64, bool need32, int num_sms,
               cudaStream_t s);

// Slice steps from the block-row lengths in B.rowlen (nb rows), scanned into
// B.slice_ptr, the total into B.total (device); sets nb and nslices.  Only
// enqueues work on s: the caller reads the total back.
void bsr_layout(BsrSell& B, int nb, cudaStream_t s);

// Block operator straight from the element stiffness buffer when the
// equations are node-aligned triples (no scalar CSR is built); returns false,
// with B left invalid, when they are not or the blocks are < 90% filled.
// out receives n, dinv and the scalar nnz (full and lower).  The topology
// passes (incidence, block counts, layout) run on topo, concurrently with
// whatever s is still running (the element kernel); s waits for them (through
// the event joined) before the fill, on every return path.
bool assemble_blocks(int n_nodes, int n_elem, const int* conn, const int* eq3, int n_dof,
                     const double* kbuf, AssemblyScratch& scr, AssembledCsr& out, BsrSell& B,
                     bool need32, int num_sms, cudaStream_t s, cudaStream_t topo,
                     cudaEvent_t joined);

// FP32 copy of the block operator (difference form) from val64.
void bsr_make_f32(BsrSell& B, int num_sms, cudaStream_t s);

// Algorithmic bytes of one block SpMV (values + block indices + x + y).
double bsr_bytes(const BsrSell& B, int precision);

}  // namespace vsgb
