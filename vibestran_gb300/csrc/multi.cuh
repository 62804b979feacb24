// vibestran_gb300/csrc/multi.cuh — records of the batched (several load
// cases per matrix sweep) PCG shared by its launch-per-kernel path
// (multi.cu) and its persistent tiled path (mres.cu).
#pragma once

#include <vector>

#include "bsr.cuh"
#include "common.cuh"
#include "errest.cuh"

namespace vsgb {

constexpr int kP = 16;     // panel width (load cases per batch)
constexpr int kFlagStalled = 128;   // refinement stopped improving (outer record)
constexpr int kFlagInactive = 256;  // column not part of this solve

struct MultiState {
  int done;       // every column finished
  int iter;       // iterations run in this solve
  int max_iters;
  int ncols;
  double tol;
  double rz[kP], pAp[kP], alpha[kP], beta[kP], rr[kP], rel[kP], norm_b[kP];
  double tolk[kP];  // per-column stopping tolerance of this solve
  int flags[kP];
  int iters[kP];  // iteration count at which the column finished
  // error-controlled stop (errest.cuh): mode, per-column absolute target^2,
  // relative target^2 (or floor), and the scale^2 ||u||_D^2 the absolute
  // target refers to (for reporting the estimate relative to ||u||)
  int err_mode;
  double err_t2[kP];
  double err_rel2;
  double err_norm2[kP];
  // bodies run by the device-side loop of the single-launch inner solve
  unsigned loop_rounds;
};

struct MultiOuter {
  double norm_f[kP], rel[kP], prev[kP], scale[kP];
  double uD2[kP];  // ||u||_D^2 of each column's outer iterate
  // error-controlled refinement: ||d||_M^2 of the column's last correction
  // and the bound on the FP32-operator part of the error it left (relative
  // to ||u||_D; < 0: none)
  double dD2[kP], pert[kP];
  int flags[kP];
  int active[kP];  // column takes part in the current inner solve
  int done;
  int pad;
};


// ── persistent tiled batched solve (mres.cu) ──────────────────────────────
// The block rows are grouped into spatially compact tiles (recursive
// coordinate bisection of the node coordinates); each tile's window — the
// distinct block columns of its rows — is staged in shared memory once per
// iteration, and the tile's rows are stored as 8-row slices of the
// sliced-ELL layout with window-local column indices.
struct MultiTiles {
  bool valid = false;
  int tn = 0;                      // target rows per tile
  int ntiles = 0, nslices = 0, ctas = 0;
  int max_win = 0;                 // largest window (block rows)
  long long steps = 0;
  size_t smem = 0;                 // dynamic shared memory of the kernel
  unsigned gen = ~0u;              // operator generation the tiles belong to
  DevBuf<int> tile_slice;          // ntiles + 1: slice range of each tile
  DevBuf<int> tile_win;            // ntiles + 1: window range of each tile
  DevBuf<int> win_row;             // window block rows, each tile's sorted
  DevBuf<int> slice_step;          // nslices + 1: step range of each slice
  DevBuf<int> slice_row;           // 8 per slice: block row (-1: none)
  DevBuf<unsigned short> slice_own;  // 8 per slice: the row's window index
  DevBuf<unsigned short> col16;    // steps * 32: window index of each slot
  DevBuf<float> val;               // steps * 288: FP32 difference-form values
  DevBuf<int> cta_tile;            // ctas + 1: tile range of each CTA
  DevBuf<int> slot_map;            // old slot of each new slot (value gather)
  DevBuf<float> dinv4;             // nb x 4: Jacobi inverses of each block row (+ pad)
  int nb = 0;
  void release() {
    valid = false;
    tile_slice.release();
    tile_win.release();
    win_row.release();
    slice_step.release();
    slice_row.release();
    slice_own.release();
    col16.release();
    val.release();
    cta_tile.release();
    slot_map.release();
    dinv4.release();
  }
};

// Builds the tile structure of rows-per-tile `tn` from the block operator and
// one coordinate triple per block row and gathers the FP32 values; false
// (T.valid false) when a window does not fit `smem_cap` bytes of shared
// memory.  The structure depends on the sparsity pattern only.
bool mres_build_tiles(const BsrSell& B, const float* dinv32, const std::vector<float>& coords,
                      int tn, int ctas, size_t smem_cap, MultiTiles& T, cudaStream_t s);
// Re-gathers the FP32 values (and the Jacobi inverses) into built tiles
// (same sparsity pattern, new values).
void mres_gather_values(const BsrSell& B, const float* dinv32, MultiTiles& T, cudaStream_t s);
// Dynamic shared memory a window may use (the device's opt-in maximum less
// the kernel's static shared memory).
size_t mres_smem_cap(int device);
// CTAs of the cooperative launch with `smem` bytes of window: one per SM
// (0 when one CTA does not fit).
int mres_ctas(int num_sms, size_t smem);

struct MresSolve {
  const double* r64;   // FP64 residual panel [n][kP] of the outer iterate
  double* u64;         // FP64 solution panel: u64 += u / scale on exit
  float *r, *u, *pa, *pb, *Ap;  // FP32 panels [n][kP]
  const float* dinv32;
  const float* diag32; // Jacobi diagonal (error estimate); may be null without it
  MultiState* S;
  MultiOuter* O;
  ErrEst* est;         // kP records
  double* partials;    // 2 x ctas x 32
  unsigned* count;     // 2 words: barrier counter, abort flag
  double tol, outer_tol;
  int max_iters, ncols;
  int err_mode;
  double err_target, err_rel;
  long long spin_limit;
  int accumulate;      // 0: leave u64 alone (timing runs of the tile autotuner)
  unsigned long long* trace;  // null, or ctas x 8: per-CTA phase times (ns) and iterations
};

// One FP32 inner solve of every active column as one cooperative launch.
void mres_solve(const MultiTiles& T, int n, const MresSolve& a, cudaStream_t s);

}  // namespace vsgb
