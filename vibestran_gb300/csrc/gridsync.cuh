// vibestran_gb300/csrc/gridsync.cuh — device primitives of the persistent
// (one cooperative launch per solve) kernels: the bounded grid barrier, the
// phase-timer marks and an FP64 quotient without the division sequence.
#pragma once

namespace vsgb {

__device__ __forceinline__ unsigned long long gtime() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Phase-timer marks of thread 0 inside a grid reduction: [0] its arrival
// (partial published), [1] the release (all CTAs arrived); [2] != 0 while the
// kernel's trace is on.  Thread 0 writes and reads them.
__device__ __forceinline__ unsigned long long* tmarks() {
  __shared__ unsigned long long m[3];
  return m;
}

// 1/b and a/b in FP64 without the division instruction sequence, whose long
// dependent chain sits on the critical path of every grid reduction (thread
// 0, GB300's FP64 pipe).  Newton-Raphson from the correctly rounded FP32
// reciprocal: y <- y + y (1 - b y) twice takes the seed's ~2^-24 relative
// error below FP64 rounding; the quotient gets Markstein's residual
// correction q <- q + y (a - b q), which leaves it within an ulp of the
// correctly rounded a / b.  Outside the FP32 exponent range of b the division
// is used.
__device__ __forceinline__ double rcp_nr2(double b) {
  const double ab = fabs(b);
  if (!(ab > 1e-30 && ab < 1e30)) return 1.0 / b;
  double y = static_cast<double>(__frcp_rn(static_cast<float>(b)));
  y = fma(y, fma(-b, y, 1.0), y);
  return fma(y, fma(-b, y, 1.0), y);
}
__device__ __forceinline__ double div_nr(double a, double b, double y /* rcp_nr2(b) */) {
  const double ab = fabs(b);
  if (!(ab > 1e-30 && ab < 1e30)) return a / b;
  const double q = a * y;
  return fma(y, fma(-b, q, a), q);
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier over a monotonic counter; false when it gave up (the abort flag
// is then set for every CTA).  Arrival is a release reduction by thread 0
// after the CTA barrier (it orders every write the CTA made before it), the
// wait an acquire load; the CTA barrier after the wait hands the acquired
// writes to the other threads.  The abort flag is polled every 64 spins and
// the loop backs off only after the first 4096.
__device__ inline bool grid_sync(unsigned* count, unsigned& target, int* abort_flag, int* s_ok,
                          long long spin_limit, bool sync_first = true) {
  target += gridDim.x;
  if (sync_first) __syncthreads();
  if (threadIdx.x == 0) {
    red_release_add_u32(count, 1u);
    unsigned long long* tm = tmarks();
    if (tm[2]) tm[0] = gtime();
    int ok = 1;
    long long spins = 0;
    while (ld_acquire_u32(count) < target) {
      ++spins;
      if ((spins & 63) == 0 && *reinterpret_cast<volatile int*>(abort_flag)) {
        ok = 0;
        break;
      }
      if (spins > spin_limit) {
        atomicExch(abort_flag, 1);
        ok = 0;
        break;
      }
      if (spins > 4096) __nanosleep(64);
    }
    if (tm[2]) tm[1] = gtime();
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

}  // namespace vsgb
