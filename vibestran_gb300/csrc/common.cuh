// vibestran_gb300/csrc/common.cuh — shared device/host utilities for libvsgb.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/vsgb.h"

namespace vsgb {

// Error carrying a vsgb status code; converted to a return value at the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    char buf[512];
    std::snprintf(buf, sizeof(buf), "CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e),
                  cudaGetErrorString(e), what, file, line);
    throw Error(VSGB_ERR_CUDA, buf);
  }
}
#define VSGB_CUDA(call) ::vsgb::cuda_check((call), #call, __FILE__, __LINE__)
#define VSGB_LAUNCH_CHECK() ::vsgb::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__)

// Owning device buffer (cudaMalloc'd, grown on demand, never shrunk).
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  T* reserve(size_t n) {
    if (n > cap) {
      release();
      if (n > 0) VSGB_CUDA(cudaMalloc(&ptr, n * sizeof(T)));
      cap = n;
    }
    return ptr;
  }
  operator T*() const { return ptr; }
};

// Device launch geometry for GB300: 152 SMs.
constexpr int kThreads = 256;

inline int grid_for(long long work, int threads, int max_blocks) {
  long long b = (work + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > max_blocks) b = max_blocks;
  return static_cast<int>(b);
}

// ── Device-side PCG scalars (one record per right-hand side) ──────────────
// Convergence and recurrence scalars stay on the device; the host only reads
// `flags`/`iter` every few iterations.
enum PcgFlags : int {
  kFlagDone = 1,
  kFlagConverged = 2,
  kFlagBreakdown = 4,   // p.Ap <= 0 (cuda_pcg_backend_impl.hpp:688-694)
  kFlagZeroRhs = 8,     // ||b|| < 1e-300 (cuda_pcg_backend_impl.hpp:1820-1830)
  kFlagNonPosRz = 16,   // r.z <= 0 at start (cuda_pcg_backend_impl.hpp:1859-1862)
  kFlagMaxIters = 32,
};

struct PcgScalars {
  double rz;      // r.z of the current iterate
  double pAp;
  double alpha;
  double beta;
  double rr;      // r.r after the last update
  double rel;     // sqrt(rr)/norm_b
  double norm_b;
  double tol;
  double scale;   // mixed: scale applied to the correction RHS
  double uD2;     // mixed outer record: ||u||_D^2 of the outer iterate (D = Jacobi diagonal)
  double err2;    // error-controlled solve: last estimate of ||e||_M^2 (< 0: none)
  double total2;  // error-controlled solve: ||x||_M^2 of the iterate
  int iter;
  int max_iters;
  int flags;
  int abort;      // persistent solve: set by any CTA whose grid wait gave up
};

// ── Reductions ────────────────────────────────────────────────────────────

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum of NV doubles (fixed tree => deterministic).  All threads of
// the block must call it; the result is valid in thread 0.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* smem /* >= 32*NV */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; ++k) smem[wid * NV + k] = v[k];
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double x = lane < nw ? smem[lane * NV + k] : 0.0;
      v[k] = warp_sum(x);
    }
  }
  __syncthreads();
}

// Last-block-done grid reduction.  Each block writes NV partials; the block
// that arrives last at `counter` sums all partials in block order (fixed
// order => deterministic) and returns true in all of its threads with the
// totals in `tot` (valid in thread 0).  The counter is reset for reuse.
template <int NV>
__device__ __forceinline__ bool grid_sum_last(double (&v)[NV], double* partials,
                                              unsigned int* counter, double* smem,
                                              double (&tot)[NV]) {
  __shared__ bool s_last;
  block_sum<NV>(v, smem);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) partials[blockIdx.x * NV + k] = v[k];
    __threadfence();
    const unsigned prev = atomicAdd(counter, 1u);
    s_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  double acc[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) acc[k] = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] += __ldcg(&partials[b * NV + k]);
  block_sum<NV>(acc, smem);
#pragma unroll
  for (int k = 0; k < NV; ++k) tot[k] = acc[k];
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// ── Exclusive scan of int counts (three-phase, deterministic) ─────────────
// Host entry: scans `count[0..n)` into `out[0..n]` (out[n] = total) using
// `tmp` (>= scan_tmp_size(n) ints).  Returns nothing; total read separately.
size_t scan_tmp_size(long long n);
void exclusive_scan(const int* count, int* out, long long n, int* tmp, cudaStream_t s);
// Same for 64-bit totals guard: throws VSGB_ERR_LIMIT when the total exceeds int32.
void exclusive_scan_checked(const int* count, int* out, long long n, int* tmp,
                            long long* tmp_total, cudaStream_t s);

}  // namespace vsgb
