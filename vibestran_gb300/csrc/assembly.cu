// vibestran_gb300/csrc/assembly.cu — deterministic CSR assembly on the GPU.
//
// Replaces the reference's triplet path (add_element_stiffness + build_csr,
// src/core/sparse_matrix.cpp:16-150; assembly_parallel.hpp:69-110):
//   * node -> element incidence (count, scan, fill, per-node ascending sort);
//   * one warp per node gathers the neighbour nodes of all incident elements,
//     orders them by their first equation index, and for every (row DOF,
//     neighbour DOF) pair sums the element contributions in ascending element
//     order.  A pair enters the pattern only if some element contributes a
//     value != 0.0 — the add_element_stiffness filter (:31) — so the pattern is
//     bit-identical to the reference's, and no atomics touch matrix values.
//   * Both triangles are produced (the symmetric SpMV wants full storage); the
//     reference's lower-triangle CsrData is extracted on request.
// Memory-bound: each pass reads the element stiffness buffer once
// (576 doubles per element) and writes 12 B per stored nonzero.

#include <climits>

#include "bsr.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace vsgb {

namespace {

constexpr int kMaxValence = 32;                 // elements per node in the pattern kernel
constexpr int kMaxNbr = 128;                    // unique neighbour nodes per node
constexpr int kPatWarps = 4;

__device__ __forceinline__ void set_error(AssemblyError* err, int code, int index) {
  if (atomicCAS(&err->code, 0, code) == 0) err->index = index;
}

// ── scan ───────────────────────────────────────────────────────────────────

constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out, long long n,
                             long long* __restrict__ tile_sum) {
  __shared__ long long s[kScanThreads];
  const long long base = static_cast<long long>(blockIdx.x) * kScanTile;
  long long v[kScanItems];
  long long local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long long i = base + threadIdx.x * kScanItems + k;
    v[k] = (i < n) ? in[i] : 0;
    local += v[k];
  }
  s[threadIdx.x] = local;
  __syncthreads();
  for (int off = 1; off < kScanThreads; off <<= 1) {
    long long t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  long long run = s[threadIdx.x] - local;  // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    const long long i = base + threadIdx.x * kScanItems + k;
    if (i < n) out[i] = static_cast<int>(run);  // tile-local; fixed up below
    run += v[k];
  }
  if (threadIdx.x == kScanThreads - 1) tile_sum[blockIdx.x] = s[threadIdx.x];
}

__global__ void k_scan_tile_sums(long long* __restrict__ tile_sum, int ntiles,
                                 long long* __restrict__ total) {
  // single block: exclusive scan of tile sums in place
  __shared__ long long s[1024];
  long long carry = 0;
  for (int base = 0; base < ntiles; base += 1024) {
    const int i = base + threadIdx.x;
    const long long v = (i < ntiles) ? tile_sum[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
      long long t = (threadIdx.x >= off) ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < ntiles) tile_sum[i] = carry + s[threadIdx.x] - v;
    const long long blk = s[1023];
    __syncthreads();
    carry += blk;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* __restrict__ out, long long n,
                           const long long* __restrict__ tile_sum,
                           const long long* __restrict__ total) {
  const long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n) out[i] = static_cast<int>(out[i] + tile_sum[i / kScanTile]);
  if (i == 0) out[n] = static_cast<int>(*total);
}

}  // namespace

size_t scan_tmp_size(long long n) { return static_cast<size_t>((n + kScanTile - 1) / kScanTile + 1) * 2; }

// tmp is reinterpreted as long long storage (scan_tmp_size counts ints).
void exclusive_scan_checked(const int* count, int* out, long long n, int* tmp,
                            long long* d_total, cudaStream_t s) {
  const long long ntiles = (n + kScanTile - 1) / kScanTile;
  long long* tile_sum = reinterpret_cast<long long*>(tmp);
  if (n > 0) {
    k_scan_tiles<<<static_cast<unsigned>(ntiles), kScanThreads, 0, s>>>(count, out, n, tile_sum);
    VSGB_LAUNCH_CHECK();
  }
  k_scan_tile_sums<<<1, 1024, 0, s>>>(tile_sum, static_cast<int>(ntiles), d_total);
  VSGB_LAUNCH_CHECK();
  const long long blocks = (n + 1 + 255) / 256;
  k_scan_add<<<static_cast<unsigned>(blocks), 256, 0, s>>>(out, n, tile_sum, d_total);
  VSGB_LAUNCH_CHECK();
}

namespace {

// ── DOF / incidence ────────────────────────────────────────────────────────

__global__ void k_dof_node(int n_nodes, const int* __restrict__ eq3, int n_dof,
                           int* __restrict__ dof_node, AssemblyError* err) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * n_nodes) return;
  const int eq = eq3[i];
  if (eq < 0) return;
  if (eq >= n_dof) {
    set_error(err, 2, i / 3);
    return;
  }
  if (atomicExch(&dof_node[eq], i) != -1) set_error(err, 1, eq);
}

__global__ void k_dof_check(int n_dof, const int* __restrict__ dof_node, AssemblyError* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n_dof && dof_node[r] < 0) set_error(err, 5, r);
}

__global__ void k_node_count(long long n_slots, const int* __restrict__ conn, int n_nodes,
                             int* __restrict__ cnt, AssemblyError* err) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n_slots) return;
  const int nd = conn[t];
  if (nd < 0 || nd >= n_nodes) {
    set_error(err, 6, static_cast<int>(t / 8));
    return;
  }
  atomicAdd(&cnt[nd], 1);
}

__global__ void k_node_fill(long long n_slots, const int* __restrict__ conn, int n_nodes,
                            const int* __restrict__ ptr, int* __restrict__ cursor,
                            int* __restrict__ node_elem) {
  const long long t = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n_slots) return;
  const int nd = conn[t];
  if (nd < 0 || nd >= n_nodes) return;
  node_elem[ptr[nd] + atomicAdd(&cursor[nd], 1)] = static_cast<int>(t);
}

__global__ void k_node_sort(int n_nodes, const int* __restrict__ ptr, int* __restrict__ node_elem) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n_nodes) return;
  const int b = ptr[a], e = ptr[a + 1];
  for (int i = b + 1; i < e; ++i) {  // insertion sort: slot = 8*element + local node
    const int v = node_elem[i];
    int j = i - 1;
    while (j >= b && node_elem[j] > v) {
      node_elem[j + 1] = node_elem[j];
      --j;
    }
    node_elem[j + 1] = v;
  }
}

// ── pattern + values ───────────────────────────────────────────────────────

// Neighbour gathering scratch for nodes of up to kVal incident elements and
// kNbr distinct neighbours.
template <int kVal, int kNbr>
struct PatSmemT {
  static constexpr int kValence = kVal, kCand = 8 * kVal, kNeighbours = kNbr;
  int cand[kCand];
  int key[kCand];
  int first[kCand];
  int nbr[kNbr];
  int nkey[kNbr];  // first free equation of nbr[r] (ascending)
};
using PatSmem = PatSmemT<kMaxValence, kMaxNbr>;
// Structured hexahedral meshes: 8 elements, 27 neighbours per node.
using PatSmemSmall = PatSmemT<8, 32>;

__device__ __forceinline__ int first_free_eq(const int* eq3, int b) {
  int k = INT_MAX;
#pragma unroll
  for (int d = 2; d >= 0; --d) {
    const int q = eq3[3 * b + d];
    if (q >= 0) k = q < k ? q : k;
  }
  return k;
}

// Warp-inclusive scan of ints across lanes.
__device__ __forceinline__ int warp_incl_scan(int v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Ascending warp-wide bitonic sort of 64 keys, element i held by lane i & 31
// in v[i >> 5]: the compare-exchange network over i (partner i ^ j, direction
// from bit k of i); j = 32 pairs the two registers of a lane, smaller j pair
// lanes through shuffles.
__device__ __forceinline__ void warp_sort64(unsigned long long (&v)[2]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 2; k <= 64; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      if (j == 32) {
        // i = lane (register 0) against i ^ 32 = lane + 32; k = 64: ascending
        const unsigned long long lo = v[0] < v[1] ? v[0] : v[1];
        const unsigned long long hi = v[0] < v[1] ? v[1] : v[0];
        v[0] = lo;
        v[1] = hi;
      } else {
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          const int i = lane + 32 * r;
          const unsigned long long o = __shfl_xor_sync(0xffffffffu, v[r], j);
          const bool up = (i & k) == 0;          // this block sorts ascending
          const bool low = (i & j) == 0;         // this element is the pair's lower index
          const bool take_min = up == low;
          v[r] = take_min ? (o < v[r] ? o : v[r]) : (o < v[r] ? v[r] : o);
        }
      }
    }
  }
}

// Distinct neighbour nodes of node a (itself included) over its incident
// elements, those with a free DOF only, ordered by their first free equation
// into s.nbr.  Returns their number, or -1 (error 3 recorded) when node a
// exceeds the valence / neighbour limits.  Warp-collective.  Nodes of up to 8
// elements (64 candidates) sort (first free equation, node) pairs in
// registers and keep the first of each run; larger ones compare every
// candidate with the earlier ones in shared memory.
template <typename Pat>
__device__ int gather_neighbors(int a, int pb, int L, const int* __restrict__ conn,
                                const int* __restrict__ eq3, const int* __restrict__ node_elem,
                                Pat& s, AssemblyError* err) {
  const int lane = threadIdx.x & 31;
  if (L > Pat::kValence) {
    if (lane == 0) set_error(err, 3, a);
    return -1;
  }
  const int C = 8 * L;
  if (C <= 64) {
    unsigned long long v[2];
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int c = lane + 32 * r;
      v[r] = ~0ull;
      if (c < C) {
        const int slot = node_elem[pb + (c >> 3)];
        const int b = conn[(slot & ~7) + (c & 7)];
        const int k = first_free_eq(eq3, b);
        s.cand[c] = b;
        s.key[c] = k;
        // constrained nodes (k = INT_MAX) sort after every free one
        v[r] = (static_cast<unsigned long long>(static_cast<unsigned>(k)) << 32) |
               static_cast<unsigned>(b);
      }
    }
    warp_sort64(v);
    // first of each run of equal (key, node) among the free nodes
    const unsigned long long prev0 = __shfl_up_sync(0xffffffffu, v[0], 1);
    const unsigned long long last0 = __shfl_sync(0xffffffffu, v[0], 31);
    const unsigned long long prev1 = __shfl_up_sync(0xffffffffu, v[1], 1);
    bool f[2];
    f[0] = (lane == 0 || prev0 != v[0]) && (v[0] >> 32) < static_cast<unsigned>(INT_MAX);
    f[1] = (lane == 0 ? last0 != v[1] : prev1 != v[1]) &&
           (v[1] >> 32) < static_cast<unsigned>(INT_MAX);
    const unsigned m0 = __ballot_sync(0xffffffffu, f[0]);
    const unsigned m1 = __ballot_sync(0xffffffffu, f[1]);
    const unsigned below = (1u << lane) - 1u;
    const int U = __popc(m0) + __popc(m1);
    if (U > Pat::kNeighbours) {
      if (lane == 0) set_error(err, 3, a);
      return -1;
    }
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      if (f[r]) {
        const int rank = (r ? __popc(m0) : 0) + __popc((r ? m1 : m0) & below);
        s.nbr[rank] = static_cast<int>(static_cast<unsigned>(v[r]));
        s.nkey[rank] = static_cast<int>(v[r] >> 32);
      }
    }
    __syncwarp();
    return U;
  }
  for (int c = lane; c < C; c += 32) {
    const int slot = node_elem[pb + (c >> 3)];
    const int b = conn[(slot & ~7) + (c & 7)];
    s.cand[c] = b;
    s.key[c] = first_free_eq(eq3, b);
  }
  __syncwarp();
  for (int c = lane; c < C; c += 32) {
    const int b = s.cand[c];
    int f = s.key[c] != INT_MAX;
    for (int m = 0; m < c && f; ++m)
      if (s.cand[m] == b) f = 0;
    s.first[c] = f;
  }
  __syncwarp();
  int U = 0;
  for (int c = lane; c < C; c += 32) {
    if (s.first[c]) {
      const int k = s.key[c];
      int r = 0;
      for (int m = 0; m < C; ++m) r += (s.first[m] && s.key[m] < k);
      if (r < Pat::kNeighbours) {
        s.nbr[r] = s.cand[c];
        s.nkey[r] = k;
      }
    }
  }
  for (int c = lane; c < C; c += 32) U += s.first[c];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) U += __shfl_xor_sync(0xffffffffu, U, o);
  if (U > Pat::kNeighbours) {
    if (lane == 0) set_error(err, 3, a);
    return -1;
  }
  __syncwarp();
  return U;
}

// The 3x3 block coupling node a (rows) with node b (columns), summed over the
// incident elements of a in ascending element order; nz marks entries that
// received a value != 0.0 (add_element_stiffness, src/core/sparse_matrix.cpp:31).
__device__ __forceinline__ void node_block(int b, int pb, int L, const int* __restrict__ conn,
                                           const int* __restrict__ node_elem,
                                           const double* __restrict__ kbuf, double (&sum)[3][3],
                                           bool (&nz)[3][3]) {
#pragma unroll
  for (int d = 0; d < 3; ++d)
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      sum[d][q] = 0.0;
      nz[d][q] = false;
    }
  for (int k = 0; k < L; ++k) {
    const int slot = node_elem[pb + k];
    const int e = slot >> 3, la = slot & 7;
    int lb = -1;
#pragma unroll
    for (int m = 0; m < 8; ++m)
      if (conn[8 * e + m] == b) lb = m;
    if (lb < 0) continue;
    const double* ke = kbuf + static_cast<size_t>(e) * 576 + (3 * la) * 24 + 3 * lb;
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double v = ke[d * 24 + q];
        sum[d][q] += v;
        nz[d][q] = nz[d][q] || (v != 0.0);
      }
  }
}

template <bool kFill>
__global__ void __launch_bounds__(kPatWarps * 32)
k_pattern(int n_nodes, const int* __restrict__ conn, const int* __restrict__ eq3,
          const int* __restrict__ node_ptr, const int* __restrict__ node_elem,
          const double* __restrict__ kbuf, int* __restrict__ row_cnt,
          const int* __restrict__ row_ptr, int* __restrict__ col_ind,
          double* __restrict__ values, double* __restrict__ dinv, AssemblyError* err) {
  __shared__ PatSmem smem_all[kPatWarps];
  PatSmem& s = smem_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * kPatWarps;
  for (int a = blockIdx.x * kPatWarps + (threadIdx.x >> 5); a < n_nodes; a += warps_total) {
    int row[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) row[d] = eq3[3 * a + d];
    if (row[0] < 0 && row[1] < 0 && row[2] < 0) continue;
    const int pb = node_ptr[a], L = node_ptr[a + 1] - pb;
    const int U = gather_neighbors(a, pb, L, conn, eq3, node_elem, s, err);
    if (U < 0) continue;

    int carry[3] = {0, 0, 0};
    int base[3] = {0, 0, 0};
    if (kFill) {
#pragma unroll
      for (int d = 0; d < 3; ++d) base[d] = row[d] >= 0 ? row_ptr[row[d]] : 0;
    }
    bool diag_seen[3] = {false, false, false};
    for (int u0 = 0; u0 < U; u0 += 32) {
      const int u = u0 + lane;
      const bool act = u < U;
      const int b = act ? s.nbr[u] : -1;
      int colq[3] = {-1, -1, -1};
      double sum[3][3];
      bool nz[3][3];
      if (act) {
#pragma unroll
        for (int q = 0; q < 3; ++q) colq[q] = eq3[3 * b + q];
        node_block(b, pb, L, conn, node_elem, kbuf, sum, nz);
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int q = 0; q < 3; ++q) {
            sum[d][q] = 0.0;
            nz[d][q] = false;
          }
      }
      int cnt[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        cnt[d] = 0;
        if (row[d] >= 0)
#pragma unroll
          for (int q = 0; q < 3; ++q) cnt[d] += (colq[q] >= 0 && nz[d][q]);
      }
      if (!kFill) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          int t = cnt[d];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
          carry[d] += t;
        }
      } else {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int incl = warp_incl_scan(cnt[d]);
          int pos = base[d] + carry[d] + incl - cnt[d];
          carry[d] += __shfl_sync(0xffffffffu, incl, 31);
          if (act && row[d] >= 0) {
#pragma unroll
            for (int q = 0; q < 3; ++q) {
              if (colq[q] >= 0 && nz[d][q]) {
                col_ind[pos] = colq[q];
                values[pos] = sum[d][q];
                ++pos;
              }
            }
            if (b == a) {
              if (nz[d][d]) {
                diag_seen[d] = true;
                if (sum[d][d] == 0.0)
                  set_error(err, 4, row[d]);
                else
                  dinv[row[d]] = 1.0 / sum[d][d];
              }
            }
          }
        }
      }
    }
    if (!kFill) {
      if (lane == 0)
#pragma unroll
        for (int d = 0; d < 3; ++d)
          if (row[d] >= 0) row_cnt[row[d]] = carry[d];
    } else {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const bool seen = __any_sync(0xffffffffu, diag_seen[d]);
        if (lane == 0 && row[d] >= 0 && !seen) set_error(err, 5, row[d]);
      }
    }
    __syncwarp();
  }
}

// ── direct 3x3 node-block assembly (node-aligned equations) ───────────────
//
// When every node with a free DOF owns the equation triple (3R, 3R+1, 3R+2)
// (the reference's DofMap with whole-node constraints), block row R is node
// a's row and block column C is neighbour b's, and the neighbour blocks that
// k_pattern forms are written straight into the sliced-ELL operator (no
// scalar CSR, no CSR-to-block conversion).  A block is stored when any of its
// entries received a value != 0.0, so the block pattern is the one the
// reference's scalar pattern induces; the scalar counts (full and lower
// triangle) are totalled for reporting.

__global__ void k_node_aligned(int n_nodes, const int* __restrict__ eq3, int* __restrict__ flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  const int e0 = eq3[3 * i], e1 = eq3[3 * i + 1], e2 = eq3[3 * i + 2];
  if (e0 < 0 && e1 < 0 && e2 < 0) return;
  if (!(e0 >= 0 && e0 % 3 == 0 && e1 == e0 + 1 && e2 == e0 + 2)) atomicOr(flag, 1);
}

// Block-row lengths: the structural neighbour count of every free node (a
// block is stored for every neighbour; entries that received no value != 0.0
// are zeros in the block and are not counted as scalar nonzeros).
__global__ void __launch_bounds__(kPatWarps * 32)
k_block_count(int n_nodes, const int* __restrict__ conn, const int* __restrict__ eq3,
              const int* __restrict__ node_ptr, const int* __restrict__ node_elem,
              int* __restrict__ blen, int* __restrict__ max_valence, AssemblyError* err) {
  __shared__ PatSmem smem_all[kPatWarps];
  PatSmem& s = smem_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * kPatWarps;
  for (int a = blockIdx.x * kPatWarps + (threadIdx.x >> 5); a < n_nodes; a += warps_total) {
    const int r0 = eq3[3 * a];
    if (r0 < 0) continue;  // aligned: all three constrained
    const int pb = node_ptr[a], L = node_ptr[a + 1] - pb;
    const int U = gather_neighbors(a, pb, L, conn, eq3, node_elem, s, err);
    if (U >= 0 && lane == 0) {
      blen[r0 / 3] = U;
      atomicMax(max_valence, L);
    }
    __syncwarp();
  }
}

template <typename Pat>
struct FillSmemT {
  Pat p;
  double acc[Pat::kNeighbours][9];         // block sums per neighbour slot
  unsigned char nz[Pat::kNeighbours][9];   // entry received a value != 0.0
  short slot[Pat::kCand];                  // neighbour slot of candidate c (-1: constrained)
  double rsum[9];                          // FP64 sum of the row's blocks (FP32 diagonal slot)
  int diag;                                // neighbour slot of the node itself
};
// Warps per CTA of the general fill (15 KB of shared memory per warp) and of
// the structured-mesh fill (4 KB per warp).
template <typename Pat>
__host__ __device__ constexpr int fill_warps() { return Pat::kNeighbours > 32 ? 2 : 4; }

// Block row of node a: for each incident element (ascending, the reference's
// summation order), its three rows of K_e (576 contiguous bytes, one
// coalesced read) are added into the neighbour blocks in shared memory, then
// the row is written to the sliced-ELL operator (FP64, and FP32 in difference
// form) with its padding, the inverse diagonal and the scalar nonzero counts
// (full and lower triangle).
template <typename Pat>
__global__ void __launch_bounds__(fill_warps<Pat>() * 32)
k_block_fill(int n_nodes, const int* __restrict__ conn, const int* __restrict__ eq3,
             const int* __restrict__ node_ptr, const int* __restrict__ node_elem,
             const double* __restrict__ kbuf, unsigned long long* __restrict__ counts,
             const int* __restrict__ slice_ptr, int* __restrict__ cols,
             double* __restrict__ v64, float* __restrict__ v32, double* __restrict__ dinv,
             AssemblyError* err) {
  constexpr int kFillWarps = fill_warps<Pat>();
  __shared__ FillSmemT<Pat> smem_all[kFillWarps];
  FillSmemT<Pat>& s = smem_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int warps_total = gridDim.x * kFillWarps;
  for (int a = blockIdx.x * kFillWarps + (threadIdx.x >> 5); a < n_nodes; a += warps_total) {
    const int r0 = eq3[3 * a];
    if (r0 < 0) continue;
    const int R = r0 / 3;
    const int pb = node_ptr[a], L = node_ptr[a + 1] - pb;
    const int U = gather_neighbors(a, pb, L, conn, eq3, node_elem, s.p, err);
    if (U < 0) continue;
    const int C = 8 * L;
    for (int c = lane; c < C; c += 32) {
      const int key = s.p.key[c];
      int slot = -1;
      if (key != INT_MAX) {
        int lo = 0, hi = U - 1;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (s.p.nkey[mid] < key) lo = mid + 1; else hi = mid;
        }
        slot = lo;
      }
      s.slot[c] = static_cast<short>(slot);
    }
    for (int t = lane; t < 9 * U; t += 32) {
      (&s.acc[0][0])[t] = 0.0;
      (&s.nz[0][0])[t] = 0;
    }
    __syncwarp();
    // Incident elements in one load (L <= 32), then their rows of K_e four
    // elements at a time: 12 loads per lane in flight before any is added,
    // the adds in ascending element order.
    const int ek_lane = lane < L ? node_elem[pb + lane] : 0;
    for (int k0 = 0; k0 < L; k0 += 4) {
      double v[4][3];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int ek = __shfl_sync(0xffffffffu, ek_lane, (k0 + j) & 31);
        const double* rows = kbuf + static_cast<size_t>(ek >> 3) * 576 + 3 * (ek & 7) * 24;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
          const int idx = lane + 32 * r;
          v[j][r] = (k0 + j < L && idx < 72) ? __ldg(rows + idx) : 0.0;
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int k = k0 + j;
        if (k < L) {
#pragma unroll
          for (int r = 0; r < 3; ++r) {
            const int idx = lane + 32 * r;
            if (idx < 72) {
              const int d = idx / 24, col = idx - 24 * d, m = col / 3, q = col - 3 * m;
              const int slot = s.slot[8 * k + m];
              if (slot >= 0) {
                s.acc[slot][3 * d + q] += v[j][r];
                if (v[j][r] != 0.0) s.nz[slot][3 * d + q] = 1;
              }
            }
          }
        }
        __syncwarp();
      }
    }
    // FP32 difference form: the diagonal slot holds the sum of the row's
    // blocks.  Lane 3k+h (k < 9) adds blocks h, h+3, ... of entry k, then the
    // three partial sums are added in fixed order (every FP64 warp
    // instruction costs the same pipe time whatever its active lanes, so the
    // sum is spread over 27 lanes).
    if (v32) {
      const int k = lane / 3, h = lane - 3 * k;
      double t = 0.0;
      if (lane < 27)
        for (int u = h; u < U; u += 3) t += s.acc[u][k];
      const double t1 = __shfl_down_sync(0xffffffffu, t, 1);
      const double t2 = __shfl_down_sync(0xffffffffu, t, 2);
      if (lane < 27 && h == 0) s.rsum[k] = (t + t1) + t2;
    }
    __syncwarp();
    const int sl = R >> 3, ln0 = (R & 7) * 4;
    const long long sp = slice_ptr[sl];
    unsigned long long full = 0, lower = 0;
    if (lane == 0) s.diag = -1;
    __syncwarp();
    for (int u = lane; u < U; u += 32) {
      const int b = s.p.nbr[u], Cb = s.p.nkey[u] / 3;
      if (b == a) s.diag = u;
      const long long st = sp + (u >> 2);
      const int ln = ln0 + (u & 3);
      cols[st * 32 + ln] = Cb;
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const double v = s.acc[u][3 * d + q];
          const size_t o = static_cast<size_t>((st * 9 + 3 * d + q) * 32 + ln);
          v64[o] = v;
          if (v32) v32[o] = static_cast<float>(b == a ? s.rsum[3 * d + q] : v);
          const bool z = s.nz[u][3 * d + q] != 0;
          full += z;
          lower += z && (3 * Cb + q <= 3 * R + d);
        }
    }
    // Inverse diagonal: one equation per lane (an FP64 division is a long
    // instruction sequence on the FP64 pipe, whatever its active lanes);
    // missing or zero pivots are reported in equation order by lane 0.
    __syncwarp();
    {
      const int ud = s.diag;
      if (lane < 3 && ud >= 0 && s.nz[ud][4 * lane] && s.acc[ud][4 * lane] != 0.0)
        dinv[3 * R + lane] = 1.0 / s.acc[ud][4 * lane];
      if (lane == 0)
        for (int d = 0; d < 3; ++d) {
          if (ud < 0 || !s.nz[ud][4 * d])
            set_error(err, 5, 3 * R + d);
          else if (s.acc[ud][4 * d] == 0.0)
            set_error(err, 4, 3 * R + d);
        }
    }
    // padding slots: a valid block column (the slice's first row), zeros
    const int slots = 4 * (slice_ptr[sl + 1] - slice_ptr[sl]);
    for (int j = U + lane; j < slots; j += 32) {
      const long long st = sp + (j >> 2);
      const int ln = ln0 + (j & 3);
      cols[st * 32 + ln] = 8 * sl;
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        const size_t o = static_cast<size_t>((st * 9 + k) * 32 + ln);
        v64[o] = 0.0;
        if (v32) v32[o] = 0.f;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      full += __shfl_xor_sync(0xffffffffu, full, o);
      lower += __shfl_xor_sync(0xffffffffu, lower, o);
    }
    if (lane == 0) {
      atomicAdd(&counts[0], full);
      atomicAdd(&counts[1], lower);
    }
    __syncwarp();
  }
}

// Sort each row by column (stable rank sort; rows already sorted are left
// untouched).  Rows up to kRowSmem entries are ranked in shared memory,
// longer rows in global memory.
constexpr int kRowSmem = 512;
constexpr int kSortWarps = 4;

__global__ void __launch_bounds__(kSortWarps * 32)
k_sort_rows(int n, const int* __restrict__ rp, int* __restrict__ ci, double* __restrict__ v,
            int* __restrict__ tmp_ci, double* __restrict__ tmp_v, int* __restrict__ need_tmp) {
  __shared__ int s_c[kSortWarps][kRowSmem];
  __shared__ double s_v[kSortWarps][kRowSmem];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int r = blockIdx.x * kSortWarps + w; r < n; r += gridDim.x * kSortWarps) {
    const int b = rp[r], len = rp[r + 1] - b;
    int unsorted = 0;
    for (int k = lane + 1; k < len; k += 32) unsorted |= (ci[b + k - 1] > ci[b + k]);
    if (!__any_sync(0xffffffffu, unsorted)) continue;
    if (len <= kRowSmem) {
      for (int k = lane; k < len; k += 32) {
        s_c[w][k] = ci[b + k];
        s_v[w][k] = v[b + k];
      }
      __syncwarp();
      for (int k = lane; k < len; k += 32) {
        const int c = s_c[w][k];
        int rank = 0;
        for (int m = 0; m < len; ++m) {
          const int cm = s_c[w][m];
          rank += (cm < c) || (cm == c && m < k);
        }
        ci[b + rank] = c;
        v[b + rank] = s_v[w][k];
      }
      __syncwarp();
    } else if (tmp_ci == nullptr) {
      if (lane == 0) *need_tmp = 1;  // host reruns with scratch buffers
    } else {
      for (int k = lane; k < len; k += 32) {
        tmp_ci[b + k] = ci[b + k];
        tmp_v[b + k] = v[b + k];
      }
      __syncwarp();
      for (int k = lane; k < len; k += 32) {
        const int c = tmp_ci[b + k];
        int rank = 0;
        for (int m = 0; m < len; ++m) {
          const int cm = tmp_ci[b + m];
          rank += (cm < c) || (cm == c && m < k);
        }
        ci[b + rank] = c;
        v[b + rank] = tmp_v[b + k];
      }
      __syncwarp();
    }
  }
}

// ── lower-triangle extraction ──────────────────────────────────────────────

__global__ void k_lower_count(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                              int* __restrict__ cnt) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  int lo = rp[r], hi = rp[r + 1];  // rows are sorted: first index with col > r
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ci[mid] <= r)
      lo = mid + 1;
    else
      hi = mid;
  }
  cnt[r] = lo - rp[r];
}

__global__ void k_lower_fill(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                             const double* __restrict__ v, const int* __restrict__ lrp,
                             int* __restrict__ lci, double* __restrict__ lv) {
  const int lane = threadIdx.x & 31;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += (gridDim.x * blockDim.x) >> 5) {
    const int b = rp[r], lb = lrp[r], len = lrp[r + 1] - lb;
    for (int k = lane; k < len; k += 32) {
      lci[lb + k] = ci[b + k];
      lv[lb + k] = v[b + k];
    }
  }
}

// ── lower -> full expansion of an uploaded CSR ─────────────────────────────

__global__ void k_check_cols(long long nnz, const int* __restrict__ ci, int n,
                             AssemblyError* err) {
  const long long k = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k < nnz && (ci[k] < 0 || ci[k] >= n)) set_error(err, 2, static_cast<int>(k));
}

__global__ void k_expand_count(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                               int* __restrict__ cnt /* zeroed, gets transposed counts */) {
  const int lane = threadIdx.x & 31;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += (gridDim.x * blockDim.x) >> 5) {
    for (int k = rp[r] + lane; k < rp[r + 1]; k += 32) {
      const int c = ci[k];
      if (c != r && c >= 0 && c < n) atomicAdd(&cnt[c], 1);
    }
  }
}

__global__ void k_add_rowlen(int n, const int* __restrict__ rp, int* __restrict__ cnt) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) cnt[r] += rp[r + 1] - rp[r];
}

__global__ void k_expand_fill(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                              const double* __restrict__ v, const int* __restrict__ frp,
                              int* __restrict__ cursor, int* __restrict__ fci,
                              double* __restrict__ fv) {
  const int lane = threadIdx.x & 31;
  for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n;
       r += (gridDim.x * blockDim.x) >> 5) {
    const int b = rp[r], len = rp[r + 1] - b, fb = frp[r];
    for (int k = lane; k < len; k += 32) {
      const int c = ci[b + k];
      const double x = v[b + k];
      fci[fb + k] = c;
      fv[fb + k] = x;
      if (c != r && c >= 0 && c < n) {
        const int pos = frp[c] + (rp[c + 1] - rp[c]) + atomicAdd(&cursor[c], 1);
        fci[pos] = r;
        fv[pos] = x;
      }
    }
  }
}

// Inverse Jacobi diagonal from full storage: first entry with col == row
// (build_jacobi_diagonal, cuda_pcg_backend_impl.hpp:2076-2101).
__global__ void k_diag_inverse(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                               const double* __restrict__ v, double* __restrict__ dinv,
                               AssemblyError* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  for (int k = rp[r]; k < rp[r + 1]; ++k) {
    if (ci[k] == r) {
      if (v[k] == 0.0) {
        set_error(err, 4, r);
        dinv[r] = 0.0;
      } else {
        dinv[r] = 1.0 / v[k];
      }
      return;
    }
  }
  set_error(err, 5, r);
  dinv[r] = 0.0;
}

}  // namespace

namespace {

// DOF table validation and the node -> element incidence (ascending element
// order per node), shared by the scalar and the block assembly.
void build_incidence(int n_nodes, int n_elem, const int* conn, const int* eq3, int n_dof,
                     AssemblyScratch& scr, cudaStream_t s) {
  const long long slots = 8LL * n_elem;
  scr.node_cnt.reserve(static_cast<size_t>(n_nodes) + 1);
  scr.node_ptr.reserve(static_cast<size_t>(n_nodes) + 1);
  scr.node_elem.reserve(static_cast<size_t>(slots > 0 ? slots : 1));
  scr.dof_node.reserve(static_cast<size_t>(n_dof > 0 ? n_dof : 1));
  scr.row_cnt.reserve(static_cast<size_t>(n_dof) + 1);
  const long long scan_n = n_nodes > n_dof ? n_nodes : n_dof;
  scr.scan_tmp.reserve(scan_tmp_size(scan_n + 1));
  scr.total.reserve(1);

  // DOF -> node map and validation of the equation table.
  VSGB_CUDA(cudaMemsetAsync(scr.dof_node.ptr, 0xFF, sizeof(int) * (n_dof > 0 ? n_dof : 1), s));
  k_dof_node<<<grid_for(3LL * n_nodes, kThreads, 1 << 30), kThreads, 0, s>>>(
      n_nodes, eq3, n_dof, scr.dof_node.ptr, scr.err.ptr);
  VSGB_LAUNCH_CHECK();
  k_dof_check<<<grid_for(n_dof, kThreads, 1 << 30), kThreads, 0, s>>>(n_dof, scr.dof_node.ptr,
                                                                      scr.err.ptr);
  VSGB_LAUNCH_CHECK();

  // Node -> element incidence.
  VSGB_CUDA(cudaMemsetAsync(scr.node_cnt.ptr, 0, sizeof(int) * (n_nodes + 1), s));
  k_node_count<<<grid_for(slots, kThreads, 1 << 30), kThreads, 0, s>>>(slots, conn, n_nodes,
                                                                      scr.node_cnt.ptr, scr.err.ptr);
  VSGB_LAUNCH_CHECK();
  exclusive_scan_checked(scr.node_cnt.ptr, scr.node_ptr.ptr, n_nodes, scr.scan_tmp.ptr,
                         scr.total.ptr, s);
  VSGB_CUDA(cudaMemsetAsync(scr.node_cnt.ptr, 0, sizeof(int) * (n_nodes + 1), s));
  k_node_fill<<<grid_for(slots, kThreads, 1 << 30), kThreads, 0, s>>>(
      slots, conn, n_nodes, scr.node_ptr.ptr, scr.node_cnt.ptr, scr.node_elem.ptr);
  VSGB_LAUNCH_CHECK();
  k_node_sort<<<grid_for(n_nodes, 128, 1 << 30), 128, 0, s>>>(n_nodes, scr.node_ptr.ptr,
                                                              scr.node_elem.ptr);
  VSGB_LAUNCH_CHECK();
}

}  // namespace

void assemble_csr(int n_nodes, int n_elem, const int* conn, const int* eq3, int n_dof,
                  const double* kbuf, AssemblyScratch& scr, AssembledCsr& out, int num_sms,
                  cudaStream_t s) {
  out.n = n_dof;
  out.row_ptr.reserve(static_cast<size_t>(n_dof) + 1);
  out.dinv.reserve(static_cast<size_t>(n_dof > 0 ? n_dof : 1));
  build_incidence(n_nodes, n_elem, conn, eq3, n_dof, scr, s);

  // Pattern count -> row_ptr.
  VSGB_CUDA(cudaMemsetAsync(scr.row_cnt.ptr, 0, sizeof(int) * (n_dof + 1), s));
  const int pgrid = grid_for(static_cast<long long>(n_nodes) * 32, kPatWarps * 32, num_sms * 16);
  k_pattern<false><<<pgrid, kPatWarps * 32, 0, s>>>(n_nodes, conn, eq3, scr.node_ptr.ptr,
                                                    scr.node_elem.ptr, kbuf, scr.row_cnt.ptr,
                                                    nullptr, nullptr, nullptr, nullptr,
                                                    scr.err.ptr);
  VSGB_LAUNCH_CHECK();
  exclusive_scan_checked(scr.row_cnt.ptr, out.row_ptr.ptr, n_dof, scr.scan_tmp.ptr,
                         scr.total.ptr, s);
  long long nnz = 0;
  VSGB_CUDA(cudaMemcpyAsync(&nnz, scr.total.ptr, sizeof(long long), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  if (nnz >= INT_MAX) throw Error(VSGB_ERR_LIMIT, "assembled nnz exceeds the int32 CSR limit");
  out.nnz = nnz;
  out.col_ind.reserve(static_cast<size_t>(nnz > 0 ? nnz : 1));
  out.values.reserve(static_cast<size_t>(nnz > 0 ? nnz : 1));
  k_pattern<true><<<pgrid, kPatWarps * 32, 0, s>>>(n_nodes, conn, eq3, scr.node_ptr.ptr,
                                                   scr.node_elem.ptr, kbuf, nullptr,
                                                   out.row_ptr.ptr, out.col_ind.ptr,
                                                   out.values.ptr, out.dinv.ptr, scr.err.ptr);
  VSGB_LAUNCH_CHECK();
  // Columns come out sorted for node-major equation numbering (the
  // reference's DofMap); any other numbering is sorted here.
  k_sort_rows<<<grid_for(static_cast<long long>(n_dof) * 32, kSortWarps * 32, num_sms * 16),
                kSortWarps * 32, 0, s>>>(n_dof, out.row_ptr.ptr, out.col_ind.ptr,
                                         out.values.ptr, nullptr, nullptr, scr.flag.ptr);
  VSGB_LAUNCH_CHECK();
  // Lower-triangle nnz for reporting.
  k_lower_count<<<grid_for(n_dof, kThreads, 1 << 30), kThreads, 0, s>>>(
      n_dof, out.row_ptr.ptr, out.col_ind.ptr, scr.row_cnt.ptr);
  VSGB_LAUNCH_CHECK();
  scr.lower_rp.reserve(static_cast<size_t>(n_dof) + 1);
  exclusive_scan_checked(scr.row_cnt.ptr, scr.lower_rp.ptr, n_dof, scr.scan_tmp.ptr,
                         scr.total.ptr, s);
  long long nl = 0;
  VSGB_CUDA(cudaMemcpyAsync(&nl, scr.total.ptr, sizeof(long long), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  out.nnz_lower = nl;
}

bool assemble_blocks(int n_nodes, int n_elem, const int* conn, const int* eq3, int n_dof,
                     const double* kbuf, AssemblyScratch& scr, AssembledCsr& out, BsrSell& B,
                     bool need32, int num_sms, cudaStream_t s, cudaStream_t topo,
                     cudaEvent_t joined) {
  if (n_dof <= 0 || n_dof % 3 != 0) return false;
  // Everything up to the fill depends on the mesh topology only: it runs on
  // `topo` (its host round trips wait for topology work alone, not for the
  // element kernel already queued on s), and s waits for it before the fill.
  auto join = [&] {
    VSGB_CUDA(cudaEventRecord(joined, topo));
    VSGB_CUDA(cudaStreamWaitEvent(s, joined, 0));
  };
  // The topology passes are enqueued back to back and read back after one
  // synchronisation (they run in the element kernel's tail, where every
  // host round trip shows): whether the equations are node-aligned, the
  // layout's total steps, the block-row lengths and the largest valence.
  // On misaligned equations the passes below are harmless (every index they
  // form stays below n_dof) and their results are discarded.
  scr.flag.reserve(1);
  VSGB_CUDA(cudaMemsetAsync(scr.flag.ptr, 0, sizeof(int), topo));
  k_node_aligned<<<grid_for(n_nodes, kThreads, 1 << 30), kThreads, 0, topo>>>(n_nodes, eq3,
                                                                            scr.flag.ptr);
  VSGB_LAUNCH_CHECK();

  build_incidence(n_nodes, n_elem, conn, eq3, n_dof, scr, topo);
  const int nb = n_dof / 3;
  B.valid = false;
  B.rowlen.reserve(static_cast<size_t>(nb));
  VSGB_CUDA(cudaMemsetAsync(B.rowlen.ptr, 0, sizeof(int) * nb, topo));
  scr.counts.reserve(2);
  VSGB_CUDA(cudaMemsetAsync(scr.counts.ptr, 0, sizeof(unsigned long long) * 2, topo));
  scr.max_valence.reserve(1);
  VSGB_CUDA(cudaMemsetAsync(scr.max_valence.ptr, 0, sizeof(int), topo));
  const int pgrid = grid_for(static_cast<long long>(n_nodes) * 32, kPatWarps * 32, num_sms * 16);
  k_block_count<<<pgrid, kPatWarps * 32, 0, topo>>>(n_nodes, conn, eq3, scr.node_ptr.ptr,
                                                    scr.node_elem.ptr, B.rowlen.ptr,
                                                    scr.max_valence.ptr, scr.err.ptr);
  VSGB_LAUNCH_CHECK();
  bsr_layout(B, nb, topo);
  // stored blocks (the sum of the row lengths)
  B.h_blen.resize(static_cast<size_t>(nb));
  VSGB_CUDA(cudaMemcpyAsync(B.h_blen.data(), B.rowlen.ptr, sizeof(int) * nb,
                            cudaMemcpyDeviceToHost, topo));
  long long total_steps = 0;
  VSGB_CUDA(cudaMemcpyAsync(&total_steps, B.total.ptr, sizeof(long long), cudaMemcpyDeviceToHost,
                            topo));
  int last = 0;  // first step of the last slice
  VSGB_CUDA(cudaMemcpyAsync(&last, B.slice_ptr.ptr + B.nslices - 1, sizeof(int),
                            cudaMemcpyDeviceToHost, topo));
  int max_valence = 0;
  VSGB_CUDA(cudaMemcpyAsync(&max_valence, scr.max_valence.ptr, sizeof(int),
                            cudaMemcpyDeviceToHost, topo));
  int misaligned = 0;
  VSGB_CUDA(cudaMemcpyAsync(&misaligned, scr.flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, topo));
  VSGB_CUDA(cudaStreamSynchronize(topo));
  if (misaligned) {
    join();
    return false;
  }
  B.steps = total_steps;
  long long blocks = 0;
  int max_blen = 0;
  for (int R = 0; R < nb; ++R) {
    blocks += B.h_blen[R];
    max_blen = B.h_blen[R] > max_blen ? B.h_blen[R] : max_blen;
  }
  if (blocks == 0) {
    join();
    return false;
  }

  const size_t nstep = static_cast<size_t>(total_steps > 0 ? total_steps : 1);
  B.cols.reserve(nstep * 32);
  B.val64.reserve(nstep * 288);
  if (need32) B.val32.reserve(nstep * 288);
  if (nb % 8 != 0) {
    // lanes of the last slice beyond nb belong to no node: block column 0,
    // zero values (read, never stored)
    const size_t tail = nstep - static_cast<size_t>(last);
    VSGB_CUDA(cudaMemsetAsync(B.cols.ptr + static_cast<size_t>(last) * 32, 0,
                              sizeof(int) * tail * 32, topo));
    VSGB_CUDA(cudaMemsetAsync(B.val64.ptr + static_cast<size_t>(last) * 288, 0,
                              sizeof(double) * tail * 288, topo));
    if (need32)
      VSGB_CUDA(cudaMemsetAsync(B.val32.ptr + static_cast<size_t>(last) * 288, 0,
                                sizeof(float) * tail * 288, topo));
  }
  join();
  out.n = n_dof;
  out.dinv.reserve(static_cast<size_t>(n_dof));
  // The compact fill serves meshes whose nodes have at most 8 elements and 32
  // neighbours (every structured hexahedral mesh): 4 KB of shared memory per
  // warp instead of 15 KB, so more warps hide the element-matrix loads.
  auto fill = [&](auto pat) {
    using Pat = decltype(pat);
    constexpr int warps = fill_warps<Pat>();
    const int fgrid = grid_for(static_cast<long long>(n_nodes) * 32, warps * 32, num_sms * 32);
    k_block_fill<Pat><<<fgrid, warps * 32, 0, s>>>(
        n_nodes, conn, eq3, scr.node_ptr.ptr, scr.node_elem.ptr, kbuf, scr.counts.ptr,
        B.slice_ptr.ptr, B.cols.ptr, B.val64.ptr, need32 ? B.val32.ptr : nullptr, out.dinv.ptr,
        scr.err.ptr);
    VSGB_LAUNCH_CHECK();
  };
  if (max_valence <= PatSmemSmall::kValence && max_blen <= PatSmemSmall::kNeighbours)
    fill(PatSmemSmall{});
  else
    fill(PatSmem{});
  unsigned long long cnt[2] = {0, 0};
  VSGB_CUDA(cudaMemcpyAsync(cnt, scr.counts.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  if (cnt[0] >= static_cast<unsigned long long>(INT_MAX))
    throw Error(VSGB_ERR_LIMIT, "assembled nnz exceeds the int32 CSR limit");
  // blocks much emptier than 3x3 (< 90% of the entries nonzero): scalar CSR
  if (static_cast<double>(cnt[0]) < 0.9 * 9.0 * static_cast<double>(blocks)) return false;
  out.nnz = static_cast<long long>(cnt[0]);
  out.nnz_lower = static_cast<long long>(cnt[1]);
  B.nblocks = blocks;
  B.has64 = true;
  B.has32 = need32;
  B.valid = true;
  return true;
}

void extract_lower(const AssembledCsr& full, int* d_row_ptr, int* d_col_ind, double* d_values,
                   AssemblyScratch& scr, int num_sms, cudaStream_t s) {
  const int n = full.n;
  scr.row_cnt.reserve(static_cast<size_t>(n) + 1);
  scr.scan_tmp.reserve(scan_tmp_size(n + 1));
  scr.total.reserve(1);
  k_lower_count<<<grid_for(n, kThreads, 1 << 30), kThreads, 0, s>>>(n, full.row_ptr.ptr,
                                                                    full.col_ind.ptr,
                                                                    scr.row_cnt.ptr);
  VSGB_LAUNCH_CHECK();
  exclusive_scan_checked(scr.row_cnt.ptr, d_row_ptr, n, scr.scan_tmp.ptr, scr.total.ptr, s);
  k_lower_fill<<<grid_for(static_cast<long long>(n) * 32, kThreads, num_sms * 16), kThreads, 0,
                 s>>>(n, full.row_ptr.ptr, full.col_ind.ptr, full.values.ptr, d_row_ptr,
                      d_col_ind, d_values);
  VSGB_LAUNCH_CHECK();
}

void prepare_full_csr(int n, long long nnz, const int* rp, const int* ci, const double* v,
                      bool lower, AssemblyScratch& scr, AssembledCsr& out, int num_sms,
                      cudaStream_t s) {
  out.n = n;
  out.row_ptr.reserve(static_cast<size_t>(n) + 1);
  out.dinv.reserve(static_cast<size_t>(n));
  if (nnz > 0) {
    k_check_cols<<<grid_for(nnz, kThreads, 1 << 30), kThreads, 0, s>>>(nnz, ci, n, scr.err.ptr);
    VSGB_LAUNCH_CHECK();
  }
  if (!lower) {
    out.nnz = nnz;
    out.col_ind.reserve(static_cast<size_t>(nnz > 0 ? nnz : 1));
    out.values.reserve(static_cast<size_t>(nnz > 0 ? nnz : 1));
    VSGB_CUDA(cudaMemcpyAsync(out.row_ptr.ptr, rp, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice, s));
    if (nnz > 0) {
      VSGB_CUDA(cudaMemcpyAsync(out.col_ind.ptr, ci, sizeof(int) * nnz, cudaMemcpyDeviceToDevice, s));
      VSGB_CUDA(cudaMemcpyAsync(out.values.ptr, v, sizeof(double) * nnz, cudaMemcpyDeviceToDevice, s));
    }
  } else {
    scr.row_cnt.reserve(static_cast<size_t>(n) + 1);
    scr.node_cnt.reserve(static_cast<size_t>(n) + 1);
    scr.scan_tmp.reserve(scan_tmp_size(n + 1));
    scr.total.reserve(1);
    VSGB_CUDA(cudaMemsetAsync(scr.row_cnt.ptr, 0, sizeof(int) * (n + 1), s));
    const int wgrid = grid_for(static_cast<long long>(n) * 32, kThreads, num_sms * 16);
    k_expand_count<<<wgrid, kThreads, 0, s>>>(n, rp, ci, scr.row_cnt.ptr);
    VSGB_LAUNCH_CHECK();
    k_add_rowlen<<<grid_for(n, kThreads, 1 << 30), kThreads, 0, s>>>(n, rp, scr.row_cnt.ptr);
    VSGB_LAUNCH_CHECK();
    exclusive_scan_checked(scr.row_cnt.ptr, out.row_ptr.ptr, n, scr.scan_tmp.ptr, scr.total.ptr, s);
    long long fnnz = 0;
    VSGB_CUDA(cudaMemcpyAsync(&fnnz, scr.total.ptr, sizeof(long long), cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
    if (fnnz >= INT_MAX) throw Error(VSGB_ERR_LIMIT, "expanded nnz exceeds the int32 CSR limit");
    out.nnz = fnnz;
    out.col_ind.reserve(static_cast<size_t>(fnnz > 0 ? fnnz : 1));
    out.values.reserve(static_cast<size_t>(fnnz > 0 ? fnnz : 1));
    VSGB_CUDA(cudaMemsetAsync(scr.node_cnt.ptr, 0, sizeof(int) * (n + 1), s));
    k_expand_fill<<<wgrid, kThreads, 0, s>>>(n, rp, ci, v, out.row_ptr.ptr, scr.node_cnt.ptr,
                                              out.col_ind.ptr, out.values.ptr);
    VSGB_LAUNCH_CHECK();
  }
  // Sort rows (mirrored entries arrive unordered).  Rows longer than the
  // shared-memory tile are sorted in a second pass with global scratch.
  const int sgrid = grid_for(static_cast<long long>(n) * 32, kSortWarps * 32, num_sms * 16);
  VSGB_CUDA(cudaMemsetAsync(scr.flag.ptr, 0, sizeof(int), s));
  k_sort_rows<<<sgrid, kSortWarps * 32, 0, s>>>(n, out.row_ptr.ptr, out.col_ind.ptr,
                                                out.values.ptr, nullptr, nullptr, scr.flag.ptr);
  VSGB_LAUNCH_CHECK();
  int need_tmp = 0;
  VSGB_CUDA(cudaMemcpyAsync(&need_tmp, scr.flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
  VSGB_CUDA(cudaStreamSynchronize(s));
  if (need_tmp) {
    DevBuf<int> tci;
    DevBuf<double> tv;
    tci.reserve(static_cast<size_t>(out.nnz));
    tv.reserve(static_cast<size_t>(out.nnz));
    k_sort_rows<<<sgrid, kSortWarps * 32, 0, s>>>(n, out.row_ptr.ptr, out.col_ind.ptr,
                                                  out.values.ptr, tci.ptr, tv.ptr, scr.flag.ptr);
    VSGB_LAUNCH_CHECK();
    VSGB_CUDA(cudaStreamSynchronize(s));
  }
  k_diag_inverse<<<grid_for(n, kThreads, 1 << 30), kThreads, 0, s>>>(
      n, out.row_ptr.ptr, out.col_ind.ptr, out.values.ptr, out.dinv.ptr, scr.err.ptr);
  VSGB_LAUNCH_CHECK();
}

}  // namespace vsgb
