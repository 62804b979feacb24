// vibestran_gb300/csrc/bsr.cu — 3x3 node-block operator in a sliced-ELL layout.
//
// CHEXA8 stiffness couples the three translations of node pairs, so K is a
// matrix of dense 3x3 blocks.  Storing one column index per block (instead of
// per scalar) cuts index bytes 9x; in FP32 the operator of the 84k-element
// cantilever drops from 167.6 MB (scalar CSR) to ~92 MB.
//
// Layout ("slice" = 8 consecutive block rows, one warp; 4 lanes per block row;
// lane = 4*row_in_slice + q; block slot = 4*t + q at step t):
//   cols[(slice_ptr[s] + t)*32 + lane]                 block column
//   vals[((slice_ptr[s] + t)*9 + k)*32 + lane]          k = 3*a + b (row a, col b)
// so every load instruction of a warp reads 32 consecutive words.
// Block rows are equation triples (3R, 3R+1, 3R+2); the format is used when
// the equations are node-aligned and the blocks are >= 90% filled
// (otherwise the scalar CSR path runs).

#include <climits>

#include "bsr.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace vsgb {

namespace {

constexpr int kBsrWarps = 4;
constexpr int kMaxBlockRowEntries = 768;

struct BsrSmem {
  int key[kMaxBlockRowEntries];
  int first[kMaxBlockRowEntries];
};

// Per block row: number of distinct block columns (or -1 when the block row
// is too long for the on-chip dedupe).
__global__ void __launch_bounds__(kBsrWarps * 32)
k_bsr_count(int nb, const int* __restrict__ rp, const int* __restrict__ ci,
            int* __restrict__ blen) {
  __shared__ BsrSmem sm_all[kBsrWarps];
  BsrSmem& s = sm_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  for (int R = blockIdx.x * kBsrWarps + (threadIdx.x >> 5); R < nb; R += gridDim.x * kBsrWarps) {
    const int b = rp[3 * R], E = rp[3 * R + 3] - b;
    if (E > kMaxBlockRowEntries) {
      if (lane == 0) blen[R] = -1;
      continue;
    }
    for (int e = lane; e < E; e += 32) s.key[e] = ci[b + e] / 3;
    __syncwarp();
    int U = 0;
    for (int e = lane; e < E; e += 32) {
      const int k = s.key[e];
      int f = 1;
      for (int m = 0; m < e && f; ++m)
        if (s.key[m] == k) f = 0;
      U += f;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) U += __shfl_xor_sync(0xffffffffu, U, o);
    if (lane == 0) blen[R] = U;
    __syncwarp();
  }
}

// Steps (groups of 4 slots) per slice of 8 block rows.
__global__ void k_slice_steps(int nb, int nslices, const int* __restrict__ blen,
                              int* __restrict__ steps) {
  const int sl = blockIdx.x * blockDim.x + threadIdx.x;
  if (sl >= nslices) return;
  int mx = 0;
  for (int r = 0; r < 8; ++r) {
    const int R = sl * 8 + r;
    if (R < nb) mx = max(mx, blen[R]);
  }
  steps[sl] = (mx + 3) / 4;
}

template <typename T>
__global__ void __launch_bounds__(kBsrWarps * 32)
k_bsr_fill(int nb, const int* __restrict__ rp, const int* __restrict__ ci,
           const double* __restrict__ v, const int* __restrict__ slice_ptr,
           int* __restrict__ cols, T* __restrict__ vals) {
  __shared__ BsrSmem sm_all[kBsrWarps];
  BsrSmem& s = sm_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  for (int R = blockIdx.x * kBsrWarps + (threadIdx.x >> 5); R < nb; R += gridDim.x * kBsrWarps) {
    const int b = rp[3 * R], E = rp[3 * R + 3] - b;
    for (int e = lane; e < E; e += 32) s.key[e] = ci[b + e] / 3;
    __syncwarp();
    for (int e = lane; e < E; e += 32) {
      const int k = s.key[e];
      int f = 1;
      for (int m = 0; m < e && f; ++m)
        if (s.key[m] == k) f = 0;
      s.first[e] = f;
    }
    __syncwarp();
    const int sl = R >> 3, rr = R & 7;
    const long long base = slice_ptr[sl];
    for (int e = lane; e < E; e += 32) {
      const int k = s.key[e];
      // slot = rank of this block column among the distinct block columns
      int slot = 0;
      for (int m = 0; m < E; ++m) slot += (s.first[m] && s.key[m] < k);
      const int t = slot >> 2, q = slot & 3;
      const long long st = base + t;
      const int ln = rr * 4 + q;
      if (s.first[e]) cols[st * 32 + ln] = k;
      // scalar row of entry e
      int row = 3 * R;
      while (row < 3 * R + 2 && b + e >= rp[row + 1]) ++row;
      const int a = row - 3 * R, bb = ci[b + e] - 3 * k;
      vals[(st * 9 + 3 * a + bb) * 32 + ln] = static_cast<T>(v[b + e]);
    }
    __syncwarp();
  }
}

// FP32 copy in difference form: every stored block is rounded from val64,
// except the diagonal block of each block row, which holds the FP64 sum of
// all blocks of that row (R_I = sum_J K_IJ).  One warp per slice; lane
// 4r+q accumulates its slots of row r over the steps, the quad adds its four
// sums (the same value in all four lanes), and the slot whose column is the
// row itself (a stored slot, not padding) receives the sum.
__global__ void __launch_bounds__(kBsrWarps * 32)
k_bsr_diff32(int nb, int nslices, const int* __restrict__ slice_ptr,
             const int* __restrict__ rowlen, const int* __restrict__ cols,
             const double* __restrict__ v64, float* __restrict__ v32) {
  const int lane = threadIdx.x & 31;
  for (int sl = blockIdx.x * kBsrWarps + (threadIdx.x >> 5); sl < nslices;
       sl += gridDim.x * kBsrWarps) {
    const long long base = slice_ptr[sl];
    const int steps = static_cast<int>(slice_ptr[sl + 1] - base);
    const int R = 8 * sl + (lane >> 2), q = lane & 3;
    const int len = R < nb ? rowlen[R] : 0;
    double rs[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) rs[k] = 0.0;
    for (int t = 0; t < steps; ++t)
#pragma unroll
      for (int k = 0; k < 9; ++k) rs[k] += v64[((base + t) * 9 + k) * 32 + lane];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      rs[k] += __shfl_xor_sync(0xffffffffu, rs[k], 1);
      rs[k] += __shfl_xor_sync(0xffffffffu, rs[k], 2);
    }
    for (int t = 0; t < steps; ++t) {
      const long long st = base + t;
      const bool diag = 4 * t + q < len && cols[st * 32 + lane] == R;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const long long o = (st * 9 + k) * 32 + lane;
        v32[o] = static_cast<float>(diag ? rs[k] : v64[o]);
      }
    }
  }
}

}  // namespace

void bsr_make_f32(BsrSell& B, int num_sms, cudaStream_t s) {
  if (!B.has64) throw Error(VSGB_ERR_STATE, "the FP32 block operator is made from the FP64 one");
  const size_t nstep = static_cast<size_t>(B.steps > 0 ? B.steps : 1);
  B.val32.reserve(nstep * 288);
  if (B.nslices > 0) {
    const int grid = grid_for(static_cast<long long>(B.nslices) * 32, kBsrWarps * 32,
                              num_sms * 16);
    k_bsr_diff32<<<grid, kBsrWarps * 32, 0, s>>>(B.nb, B.nslices, B.slice_ptr.ptr,
                                                 B.rowlen.ptr, B.cols.ptr, B.val64.ptr,
                                                 B.val32.ptr);
    VSGB_LAUNCH_CHECK();
  }
  B.has32 = true;
}

void bsr_layout(BsrSell& B, int nb, cudaStream_t s) {
  const int nslices = (nb + 7) / 8;
  B.nb = nb;
  B.nslices = nslices;
  B.slice_ptr.reserve(static_cast<size_t>(nslices) + 1);
  B.tmp.reserve(scan_tmp_size(nslices + 1));
  B.total.reserve(1);
  B.slice_steps.reserve(static_cast<size_t>(nslices) + 1);
  k_slice_steps<<<grid_for(nslices, kThreads, 1 << 30), kThreads, 0, s>>>(
      nb, nslices, B.rowlen.ptr, B.slice_steps.ptr);
  VSGB_LAUNCH_CHECK();
  exclusive_scan_checked(B.slice_steps.ptr, B.slice_ptr.ptr, nslices, B.tmp.ptr, B.total.ptr, s);
}

bool build_bsr(const AssembledCsr& K, BsrSell& B, bool need64, bool need32, int num_sms,
               cudaStream_t s) {
  B.valid = false;
  if (K.n <= 0 || K.n % 3 != 0) return false;
  const int nb = K.n / 3;
  const int nslices = (nb + 7) / 8;
  B.nb = nb;
  B.nslices = nslices;
  B.rowlen.reserve(static_cast<size_t>(nb));
  B.slice_ptr.reserve(static_cast<size_t>(nslices) + 1);
  B.tmp.reserve(scan_tmp_size(nslices + 1));
  B.total.reserve(1);
  const int wgrid = grid_for(static_cast<long long>(nb) * 32, kBsrWarps * 32, num_sms * 16);
  k_bsr_count<<<wgrid, kBsrWarps * 32, 0, s>>>(nb, K.row_ptr.ptr, K.col_ind.ptr, B.rowlen.ptr);
  VSGB_LAUNCH_CHECK();
  // blocks total and eligibility, computed on the host from blen (nb ints).
  B.h_blen.resize(static_cast<size_t>(nb));
  VSGB_CUDA(cudaMemcpyAsync(B.h_blen.data(), B.rowlen.ptr, sizeof(int) * nb,
                            cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  long long blocks = 0;
  for (int R = 0; R < nb; ++R) {
    if (B.h_blen[R] < 0) return false;
    blocks += B.h_blen[R];
  }
  if (blocks == 0 || static_cast<double>(K.nnz) < 0.9 * 9.0 * static_cast<double>(blocks))
    return false;
  B.nblocks = blocks;
  DevBuf<int> steps;
  steps.reserve(static_cast<size_t>(nslices) + 1);
  k_slice_steps<<<grid_for(nslices, kThreads, 1 << 30), kThreads, 0, s>>>(nb, nslices,
                                                                          B.rowlen.ptr, steps.ptr);
  VSGB_LAUNCH_CHECK();
  exclusive_scan_checked(steps.ptr, B.slice_ptr.ptr, nslices, B.tmp.ptr, B.total.ptr, s);
  long long total_steps = 0;
  VSGB_CUDA(cudaMemcpyAsync(&total_steps, B.total.ptr, sizeof(long long), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  B.steps = total_steps;
  const size_t nstep = static_cast<size_t>(total_steps > 0 ? total_steps : 1);
  B.cols.reserve(nstep * 32);
  VSGB_CUDA(cudaMemsetAsync(B.cols.ptr, 0, sizeof(int) * nstep * 32, s));
  if (need64 || need32) {
    B.val64.reserve(nstep * 32 * 9);
    VSGB_CUDA(cudaMemsetAsync(B.val64.ptr, 0, sizeof(double) * nstep * 32 * 9, s));
    k_bsr_fill<double><<<wgrid, kBsrWarps * 32, 0, s>>>(nb, K.row_ptr.ptr, K.col_ind.ptr,
                                                        K.values.ptr, B.slice_ptr.ptr,
                                                        B.cols.ptr, B.val64.ptr);
    VSGB_LAUNCH_CHECK();
  }
  B.has64 = true;  // the FP32 copy is made from it
  B.has32 = false;
  if (need32) bsr_make_f32(B, num_sms, s);
  B.valid = true;
  return true;
}

double bsr_bytes(const BsrSell& B, int precision) {
  // Stored blocks (padding slots are never read): values + one index per
  // block, plus x read once and y written once (scalar vectors).
  const double n = 3.0 * B.nb, blocks = static_cast<double>(B.nblocks);
  if (precision == VSGB_MIXED) return blocks * (36.0 + 4.0) + 4.0 * B.nb + 8.0 * n;
  return blocks * (72.0 + 4.0) + 4.0 * B.nb + 16.0 * n;
}

}  // namespace vsgb
