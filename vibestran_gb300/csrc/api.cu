// vibestran_gb300/csrc/api.cu — C ABI (include/vsgb.h): context, solve, assembly.
//
// The context mirrors CudaPCGContext (src/solver/cuda_pcg_backend_impl.hpp:2031-2065):
// device, tolerance, max iterations, last iteration count / residual, device
// name — plus the resident mesh, the assembled operator and the PCG engine.
// Error texts follow the reference's SolverError messages so a C++ wrapper can
// rethrow them unchanged.

#include <climits>
#include <cstring>
#include <memory>
#include <string>

#include "common.cuh"
#include "kernels.cuh"
#include "pcg.cuh"

using vsgb::DevBuf;
using vsgb::Error;

struct vsgb_ctx {
  int device = 0;
  int num_sms = 152;
  cudaStream_t stream = nullptr;
  // Topology passes beside the element kernel, at the lowest priority: their
  // blocks then fill the element kernel's tail instead of displacing its
  // second wave (84k: assembly 4.1-4.4 ms with a high-priority stream, 3.84 ms
  // serial, 3.72 ms low priority).
  cudaStream_t topo = nullptr;
  cudaEvent_t topo_done = nullptr;  // joins topo into stream
  cudaEvent_t topo_start = nullptr; // orders topo after earlier work on stream
  std::string device_name;
  std::string last_error;
  double tol = 1e-8;
  int max_iters = 10000;
  int precision = VSGB_FP64;
  double inner_tol = 0.0;
  int max_solves = 0;  // 0: 3, or 5 for an error-controlled mixed solve
  double err_target = -1.0;  // < 0: automatic (mixed 1e-6 unless tol was set, FP64 off)
  bool tol_explicit = false; // the caller chose the residual tolerance
  int format = 0;

  // resident mesh
  int n_nodes = 0, n_elem = 0, n_dof = 0;
  bool mesh_ok = false, assembled = false, has_form = false;
  DevBuf<double> xyz, E, nu, kbuf, lame;
  DevBuf<int> eq3, conn, form;
  DevBuf<vsgb::ElementError> elem_err;
  vsgb::AssemblyScratch scr;
  vsgb::AssembledCsr K;
  std::unique_ptr<vsgb::PcgEngine> eng;

  // right-hand sides / solutions
  int nrhs = 0;
  int u_cases = 0;                     // load cases held in u by the last solve
  DevBuf<double> f, u;
  DevBuf<double> u_in, stress_c, stress_n;  // stress recovery staging
  DevBuf<double> node_disp;                  // nodal displacement recovery
  // staging of an uploaded CSR (solve_csr)
  DevBuf<int> in_rp, in_ci;
  DevBuf<double> in_v;

  vsgb::PcgScalars* h_scal = nullptr;  // pinned
  int* h_bad = nullptr;                // pinned: first bad conn / eq3 index of an upload
  DevBuf<int> mesh_bad;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  long long launches = 0;
  int last_iters = 0;
  double last_rel = 0.0;
  DevBuf<double> grad;                 // adjoint gradients (2 x n_elem)
  int batched = 1;                     // 0 never, 1 auto, 2 always batch load cases
  bool csr_ready = false;              // K holds the scalar full CSR
  bool blocks_prebuilt = false;        // the engine's block operator came from assemble_blocks
  bool last_batched = false;
  std::vector<vsgb::SolveResult> rhs;  // per-load-case results of the last solve
  // tiled batched solve: coordinates of the block rows of the uploaded mesh
  // (3 per row; empty when the equations are not node-aligned triples) and a
  // key of its sparsity pattern (node count, element count, equations, conn)
  std::vector<float> block_xyz;
  unsigned long long pattern_key = 0;
  bool coords_ready = false;  // block_xyz / pattern_key belong to the uploaded mesh
  int batch_tiles = 0;        // VSGB_OPT_BATCH_TILES
};

namespace {

void set_device(vsgb_ctx* c) { VSGB_CUDA(cudaSetDevice(c->device)); }

template <typename F>
int guarded(vsgb_ctx* c, F&& fn) {
  if (!c) return VSGB_ERR_INVALID;
  try {
    set_device(c);
    fn();
    c->last_error.clear();
    return VSGB_OK;
  } catch (const Error& e) {
    c->last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    c->last_error = "host allocation failed";
    return VSGB_ERR_LIMIT;
  } catch (const std::exception& e) {
    c->last_error = e.what();
    return VSGB_ERR_INVALID;
  }
}

double default_tol(int precision) { return precision == VSGB_MIXED ? 1e-6 : 1e-8; }

// Relative displacement error target of the next solve (0: the reference's
// residual test).  Mixed precision controls the error by default (1e-6, the
// accuracy the mixed form is quoted at) unless the caller chose a residual
// tolerance; FP64 keeps cuda-pcg's residual test unless a target is set.
double error_target(const vsgb_ctx* c) {
  if (c->err_target >= 0.0) return c->err_target;
  return (c->precision == VSGB_MIXED && !c->tol_explicit) ? 1e-6 : 0.0;
}

// Inner solves of a mixed solve: the option, else 3 (the reference's 1 + 2
// corrections) or, error-controlled, 5 (a refinement step may be repeated
// when the FP32 operator's share of the error is not yet below the target).
int max_solves(const vsgb_ctx* c) {
  if (c->max_solves > 0) return c->max_solves;
  return (c->precision == VSGB_MIXED && error_target(c) > 0.0) ? 5 : 3;
}

double inner_tolerance(const vsgb_ctx* c, bool batched) {
  if (c->inner_tol > 0.0) return c->inner_tol;
  // error-controlled refinement (batched, or persistent single solves): the
  // first inner solve only has to bring the error to where the next,
  // error-controlled step takes over
  if (c->precision == VSGB_MIXED && error_target(c) > 0.0 &&
      (batched || c->eng->resident_used(true)))
    return 1e-3;
  // cuda_pcg_backend_impl.hpp:2166-2171: clamp(100 * tol, 1e-4, 1e-2)
  double t = c->tol * 100.0;
  if (t < 1e-4) t = 1e-4;
  if (t > 1e-2) t = 1e-2;
  return t;
}

void check_assembly_error(vsgb_ctx* c) {
  vsgb::AssemblyError h{};
  VSGB_CUDA(cudaMemcpyAsync(&h, c->scr.err.ptr, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  VSGB_CUDA(cudaStreamSynchronize(c->stream));
  if (h.code == 0) return;
  const std::string i = std::to_string(h.index);
  switch (h.code) {
    case 1:
      throw Error(VSGB_ERR_INVALID, "equation index " + i + " is assigned to two DOFs");
    case 2:
      throw Error(VSGB_ERR_INVALID, "index out of range at position " + i);
    case 3:
      throw Error(VSGB_ERR_LIMIT, "node index " + i +
                                      " exceeds the device assembly limits (32 elements or 128 "
                                      "neighbour nodes per node)");
    case 4:
      throw Error(VSGB_ERR_SINGULAR, "CUDA PCG: zero diagonal at row " + i +
                                         " -- matrix is singular. Check boundary conditions.");
    case 5:
      throw Error(VSGB_ERR_SINGULAR, "CUDA PCG: missing diagonal at row " + i +
                                         " -- matrix is singular. Check boundary conditions.");
    case 6:
      throw Error(VSGB_ERR_INVALID, "element index " + i + " references a node index out of range");
    default:
      throw Error(VSGB_ERR_INVALID, "assembly error code " + std::to_string(h.code));
  }
}

void reset_assembly_error(vsgb_ctx* c, cudaStream_t s) {
  c->scr.err.reserve(1);
  VSGB_CUDA(cudaMemsetAsync(c->scr.err.ptr, 0, sizeof(vsgb::AssemblyError), s));
  c->scr.flag.reserve(1);
}

// Scalar full CSR of the resident mesh from the stored element matrices
// (after a block assembly it is built on first request).
void ensure_csr(vsgb_ctx* c) {
  if (c->csr_ready) return;
  if (!c->mesh_ok) throw Error(VSGB_ERR_STATE, "no mesh uploaded");
  reset_assembly_error(c, c->stream);
  vsgb::assemble_csr(c->n_nodes, c->n_elem, c->conn.ptr, c->eq3.ptr, c->n_dof, c->kbuf.ptr,
                     c->scr, c->K, c->num_sms, c->stream);
  c->eng->add_launches(18);
  check_assembly_error(c);
  c->csr_ready = true;
}

// (Re)binds the operator to the engine for the current precision and format.
void prepare_operator(vsgb_ctx* c) {
  const bool mixed = c->precision == VSGB_MIXED;
  if (c->blocks_prebuilt && c->format != 1) {
    c->eng->prepare(c->K, mixed, c->stream, true);
    return;
  }
  ensure_csr(c);
  c->blocks_prebuilt = false;  // a scalar prepare may rebuild the blocks from the CSR
  c->eng->prepare(c->K, mixed, c->stream);
}

std::string not_converged_text(const vsgb_ctx* c, double rel) {
  // cuda_pcg_backend_impl.hpp:1964-1970
  return "CUDA PCG: did not converge after " + std::to_string(c->max_iters) +
         " iterations (relative residual " + std::to_string(rel) + " > tolerance " +
         std::to_string(c->tol) + "). Consider increasing max iterations or using a direct solver.";
}

// nrhs > 1 on the block operator: one batched PCG for all load cases.
// Block-row coordinates (3 floats per block row, node-aligned equation
// triples only) and a key of the sparsity pattern (FNV-1a over the node
// count, element count, equations and connectivity) for the tiled batched
// solve, from host copies of the mesh arrays.
void block_coords(vsgb_ctx* c, const double* xyz, const int* eq3, const int* conn) {
  const int n_nodes = c->n_nodes, n_dof = c->n_dof;
  unsigned long long key = 1469598103934665603ULL;
  auto mix = [&key](unsigned v) { key = (key ^ v) * 1099511628211ULL; };
  mix(static_cast<unsigned>(n_nodes));
  mix(static_cast<unsigned>(c->n_elem));
  mix(static_cast<unsigned>(n_dof));
  for (long long k = 0; k < 3LL * n_nodes; ++k) mix(static_cast<unsigned>(eq3[k]));
  for (long long k = 0; k < 8LL * c->n_elem; ++k) mix(static_cast<unsigned>(conn[k]));
  c->pattern_key = key;
  c->block_xyz.clear();
  if (n_dof % 3 == 0) {
    c->block_xyz.assign(static_cast<size_t>(n_dof), 0.f);
    for (int i = 0; i < n_nodes; ++i) {
      const int e0 = eq3[3 * i];
      if (e0 >= 0 && e0 % 3 == 0 && e0 + 2 < n_dof && eq3[3 * i + 1] == e0 + 1 &&
          eq3[3 * i + 2] == e0 + 2)
        for (int d = 0; d < 3; ++d)
          c->block_xyz[static_cast<size_t>(e0) + d] = static_cast<float>(xyz[3 * i + d]);
    }
  }
  c->coords_ready = true;
}

// The same from the device copies of the uploaded mesh (the option was off
// at upload time).
void block_coords_from_device(vsgb_ctx* c) {
  std::vector<double> xyz(3 * static_cast<size_t>(c->n_nodes));
  std::vector<int> eq3(3 * static_cast<size_t>(c->n_nodes)), conn(8 * static_cast<size_t>(c->n_elem));
  VSGB_CUDA(cudaMemcpyAsync(xyz.data(), c->xyz.ptr, sizeof(double) * xyz.size(),
                            cudaMemcpyDeviceToHost, c->stream));
  VSGB_CUDA(cudaMemcpyAsync(eq3.data(), c->eq3.ptr, sizeof(int) * eq3.size(),
                            cudaMemcpyDeviceToHost, c->stream));
  VSGB_CUDA(cudaMemcpyAsync(conn.data(), c->conn.ptr, sizeof(int) * conn.size(),
                            cudaMemcpyDeviceToHost, c->stream));
  VSGB_CUDA(cudaStreamSynchronize(c->stream));
  block_coords(c, xyz.data(), eq3.data(), conn.data());
}

void run_batched(vsgb_ctx* c, int nrhs, vsgb_stats* stats) {
  const int n = c->K.n;
  c->u.reserve(static_cast<size_t>(n) * nrhs);
  const bool mixed = c->precision == VSGB_MIXED;
  c->eng->set_error_target(error_target(c));
  // the tiled batched solve needs the mesh the operator was assembled from
  if (c->batch_tiles != 0 && mixed && c->assembled && c->mesh_ok && !c->coords_ready)
    block_coords_from_device(c);
  c->eng->set_block_coords(
      c->assembled && c->coords_ready && !c->block_xyz.empty() ? &c->block_xyz : nullptr,
      c->pattern_key);
  VSGB_CUDA(cudaEventRecord(c->ev[0], c->stream));
  c->eng->solve_multi(c->f.ptr, nrhs, c->u.ptr, mixed, c->tol, inner_tolerance(c, true), c->max_iters,
                      max_solves(c), c->stream, c->rhs);
  VSGB_CUDA(cudaEventRecord(c->ev[1], c->stream));
  VSGB_CUDA(cudaEventSynchronize(c->ev[1]));
  float ms = 0.f;
  VSGB_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
  c->last_batched = true;
  vsgb_stats st{};
  st.batch_tile_rows = c->eng->batch_tile_rows();
  st.format = c->eng->format_used();
  st.converged = 1;
  st.est_rel_error = -1.0;
  for (const vsgb::SolveResult& r : c->rhs) {
    st.iterations = r.iterations > st.iterations ? r.iterations : st.iterations;
    st.inner_solves += r.inner_solves;
    st.rel_residual = r.rel > st.rel_residual ? r.rel : st.rel_residual;
    if (r.err_est > st.est_rel_error) st.est_rel_error = r.err_est;
    if (!r.converged) st.converged = 0;
  }
  c->last_iters = st.iterations;
  c->last_rel = st.rel_residual;
  for (const vsgb::SolveResult& r : c->rhs) {
    // Same outcomes as one solve per load case: FP64 throws on a case that
    // did not converge, mixed throws only when an inner solve failed.
    if (mixed ? r.inner_failed : !r.converged)
      throw Error(VSGB_ERR_NOT_CONVERGED, not_converged_text(c, r.rel));
  }
  if (stats) {
    st.solve_ms = ms;
    st.spmv_bytes = c->eng->spmv_bytes(c->precision);
    *stats = st;
  }
  c->u_cases = nrhs;
}

// Auto mode batches from the load-case count where one 16-wide sweep beats
// that many single-case iterations of the persistent solver: about 3 (mixed,
// the FP32 sweep is bound by gathering the 16-wide panel) and about 9 (FP64,
// both forms are bound by the FP64 pipe).
bool use_batched(const vsgb_ctx* c, int nrhs) {
  if (nrhs < 2 || c->batched == 0 || !c->eng->multi_supported()) return false;
  if (c->eng->precond() != 0 && c->batched == 1) return false;  // scalar Jacobi only
  if (c->batched == 2) return true;
  return nrhs >= (c->precision == VSGB_MIXED ? 4 : 10);
}

void run_solves(vsgb_ctx* c, int nrhs, vsgb_stats* stats) {
  if (use_batched(c, nrhs)) {
    run_batched(c, nrhs, stats);
    return;
  }
  c->last_batched = false;
  c->rhs.assign(static_cast<size_t>(nrhs), vsgb::SolveResult{});
  const int n = c->K.n;
  c->u.reserve(static_cast<size_t>(n) * nrhs);
  vsgb_stats st{};
  st.format = c->eng->format_used();
  st.inner_solves = 0;
  st.converged = 1;
  st.est_rel_error = -1.0;
  c->eng->set_error_target(error_target(c));
  float ms_total = 0.f;
  for (int k = 0; k < nrhs; ++k) {
    const double* fk = c->f.ptr + static_cast<size_t>(k) * n;
    vsgb::SolveResult res;
    VSGB_CUDA(cudaEventRecord(c->ev[0], c->stream));
    if (c->precision == VSGB_MIXED) {
      c->eng->solve_mixed(fk, c->tol, inner_tolerance(c, false), c->max_iters, max_solves(c),
                          c->stream,
                          c->h_scal, res);
    } else {
      c->eng->solve_fp64(fk, c->tol, c->max_iters, c->stream, c->h_scal, res);
    }
    VSGB_CUDA(cudaMemcpyAsync(c->u.ptr + static_cast<size_t>(k) * n, c->eng->solution(),
                              sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
    VSGB_CUDA(cudaEventRecord(c->ev[1], c->stream));
    VSGB_CUDA(cudaEventSynchronize(c->ev[1]));
    float ms = 0.f;
    VSGB_CUDA(cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]));
    ms_total += ms;
    st.iterations = res.iterations > st.iterations ? res.iterations : st.iterations;
    st.inner_solves += res.inner_solves;
    st.kernel_ms += c->eng->resident_ms();
    st.kernel_iterations += static_cast<double>(c->eng->resident_iterations());
    st.rel_residual = res.rel > st.rel_residual ? res.rel : st.rel_residual;
    if (res.err_est > st.est_rel_error) st.est_rel_error = res.err_est;
    c->last_iters = res.iterations;
    c->last_rel = res.rel;
    c->rhs[static_cast<size_t>(k)] = res;
    const std::string tail = " (relative residual " + std::to_string(res.rel) + " > tolerance " +
                             std::to_string(c->tol) +
                             "). Consider increasing max iterations or using a direct solver.";
    if (c->precision == VSGB_MIXED) {
      if (res.inner_failed)
        throw Error(VSGB_ERR_NOT_CONVERGED, "CUDA PCG: did not converge after " +
                                                std::to_string(c->max_iters) + " iterations" + tail);
      if (!res.converged) st.converged = 0;  // mixed returns the refined solution (warns)
    } else if (!res.converged || res.iterations >= c->max_iters) {
      // cuda_pcg_backend_impl.hpp:1964-1970 (also reached on breakdown)
      throw Error(VSGB_ERR_NOT_CONVERGED, "CUDA PCG: did not converge after " +
                                              std::to_string(c->max_iters) + " iterations" + tail);
    }
  }
  if (stats) {
    st.solve_ms = ms_total;
    st.spmv_bytes = c->eng->spmv_bytes(c->precision);
    *stats = st;
  }
  c->u_cases = nrhs;
}

void upload(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes) VSGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s));
}

// Range check of every index the mesh kernels dereference: bad[0] = first
// connectivity entry outside [0, n_nodes), bad[1] = first equation entry
// outside [-1, n_dof) (INT_MAX when none).
__global__ void k_check_mesh(long long n_conn, const int* __restrict__ conn, int n_nodes,
                             long long n_eq, const int* __restrict__ eq3, int n_dof,
                             int* __restrict__ bad) {
  const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
       k < n_conn + n_eq; k += stride) {
    if (k < n_conn) {
      const int v = conn[k];
      if (v < 0 || v >= n_nodes) atomicMin(&bad[0], static_cast<int>(k));
    } else {
      const int v = eq3[k - n_conn];
      if (v < -1 || v >= n_dof) atomicMin(&bad[1], static_cast<int>(k - n_conn));
    }
  }
}

}  // namespace

extern "C" {

int vsgb_create(int device, double tol, int max_iters, int precision, vsgb_ctx** out) {
  if (!out) return VSGB_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0 || device < 0 || device >= count) {
    cudaGetLastError();
    return VSGB_ERR_NO_DEVICE;
  }
  if (precision != VSGB_FP64 && precision != VSGB_MIXED) return VSGB_ERR_INVALID;
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return VSGB_ERR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return VSGB_ERR_NO_DEVICE;  // built for sm_103a only
  if (cudaSetDevice(device) != cudaSuccess) return VSGB_ERR_NO_DEVICE;
  auto* c = new (std::nothrow) vsgb_ctx();
  if (!c) return VSGB_ERR_LIMIT;
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  c->device_name = prop.name;
  c->precision = precision;
  c->tol = tol > 0.0 ? tol : default_tol(precision);
  c->tol_explicit = tol > 0.0;
  c->max_iters = max_iters > 0 ? max_iters : 10000;
  int prio_low = 0, prio_high = 0;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) != cudaSuccess ||
      cudaStreamCreateWithPriority(&c->topo, cudaStreamNonBlocking, prio_low) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->topo_done, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->topo_start, cudaEventDisableTiming) != cudaSuccess ||
      cudaMallocHost(&c->h_scal, sizeof(vsgb::PcgScalars) * 2) != cudaSuccess ||
      cudaMallocHost(&c->h_bad, sizeof(int) * 2) != cudaSuccess) {
    vsgb_destroy(c);
    return VSGB_ERR_CUDA;
  }
  for (auto& e : c->ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      vsgb_destroy(c);
      return VSGB_ERR_CUDA;
    }
  c->eng = std::make_unique<vsgb::PcgEngine>(c->num_sms);
  *out = c;
  return VSGB_OK;
}

void vsgb_destroy(vsgb_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->topo) cudaStreamSynchronize(c->topo);
  c->eng.reset();
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->h_scal) cudaFreeHost(c->h_scal);
  if (c->h_bad) cudaFreeHost(c->h_bad);
  if (c->topo_done) cudaEventDestroy(c->topo_done);
  if (c->topo_start) cudaEventDestroy(c->topo_start);
  if (c->topo) cudaStreamDestroy(c->topo);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int vsgb_set_option(vsgb_ctx* c, int option, double value) {
  return guarded(c, [&] {
    switch (option) {
      case VSGB_OPT_TOLERANCE:
        c->tol = value > 0.0 ? value : default_tol(c->precision);
        c->tol_explicit = value > 0.0;
        break;
      case VSGB_OPT_MAX_ITERS:
        c->max_iters = value > 0 ? static_cast<int>(value) : 10000;
        break;
      case VSGB_OPT_PRECISION: {
        const int p = static_cast<int>(value);
        if (p != VSGB_FP64 && p != VSGB_MIXED) throw Error(VSGB_ERR_INVALID, "bad precision");
        const bool changed = p != c->precision;
        c->precision = p;
        if (changed && c->assembled) prepare_operator(c);
        break;
      }
      case VSGB_OPT_INNER_TOL:
        c->inner_tol = value;
        break;
      case VSGB_OPT_MAX_SOLVES:
        c->max_solves = value >= 1 ? static_cast<int>(value) : 0;
        break;
      case VSGB_OPT_CHECK_EVERY:
        c->eng->set_check_every(static_cast<int>(value));
        break;
      case VSGB_OPT_USE_GRAPH:
        c->eng->set_use_graph(value != 0.0);
        break;
      case VSGB_OPT_FORMAT:
        c->format = static_cast<int>(value);
        c->eng->set_format(c->format);
        if (c->assembled) prepare_operator(c);
        break;
      case VSGB_OPT_RESIDENT:
        c->eng->set_resident(value != 0.0);
        if (c->assembled) prepare_operator(c);
        break;
      case VSGB_OPT_L2_PERSIST:
        c->eng->set_l2_persist(value != 0.0);
        break;
      case VSGB_OPT_ADAPTIVE_INNER:
        c->eng->set_adaptive_inner(value != 0.0);
        break;
      case VSGB_OPT_PRECOND: {
        const int p = static_cast<int>(value);
        if (p != VSGB_PRECOND_JACOBI && p != VSGB_PRECOND_BLOCK_JACOBI)
          throw Error(VSGB_ERR_INVALID, "preconditioner must be 0 (Jacobi) or 1 (3x3 block Jacobi)");
        c->eng->set_precond(p);
        break;
      }
      case VSGB_OPT_BATCHED: {
        const int b = static_cast<int>(value);
        if (b < 0 || b > 2) throw Error(VSGB_ERR_INVALID, "batched mode must be 0, 1 or 2");
        c->batched = b;
        break;
      }
      case VSGB_OPT_ERROR_TARGET:
        c->err_target = value;
        break;
      case VSGB_OPT_SPIN_LIMIT:
        c->eng->set_spin_limit(static_cast<long long>(value));
        break;
      case VSGB_OPT_BATCH_TILES:
        if (!(value == 0.0 || value == 1.0 || (value >= 8.0 && value <= 65536.0)))
          throw Error(VSGB_ERR_INVALID, "VSGB_OPT_BATCH_TILES: 0, 1 or 8..65536 rows per tile");
        c->batch_tiles = static_cast<int>(value);
        c->eng->set_batch_tiles(c->batch_tiles);
        break;
      case VSGB_OPT_COARSE:
        if (!(value == 0.0 || value == 1.0 || value == 2.0))
          throw Error(VSGB_ERR_INVALID, "VSGB_OPT_COARSE: 0, 1 or 2");
        c->eng->set_coarse(static_cast<int>(value));
        break;
      case VSGB_OPT_PHASE_TRACE:
        c->eng->set_phase_trace(value != 0.0);
        break;
      default:
        throw Error(VSGB_ERR_INVALID, "unknown option " + std::to_string(option));
    }
  });
}

int vsgb_last_error(vsgb_ctx* c, char* buf, size_t len) {
  if (!c || !buf || len == 0) return VSGB_ERR_INVALID;
  std::snprintf(buf, len, "%s", c->last_error.c_str());
  return VSGB_OK;
}

int vsgb_device_name(vsgb_ctx* c, char* buf, size_t len) {
  if (!c || !buf || len == 0) return VSGB_ERR_INVALID;
  std::snprintf(buf, len, "%s", c->device_name.c_str());
  return VSGB_OK;
}

int vsgb_backend_name(vsgb_ctx* c, char* buf, size_t len) {
  if (!c || !buf || len == 0) return VSGB_ERR_INVALID;
  const char* pre = c->eng && c->eng->precond() != 0 ? "3x3 block Jacobi" : "Jacobi";
  if (c->precision == VSGB_MIXED)
    std::snprintf(buf, len, "CUDA GB300 mixed-precision PCG + %s, FP64 refinement on GPU (GPU)",
                  pre);
  else
    std::snprintf(buf, len, "CUDA GB300 PCG + %s float64 (GPU)", pre);
  return VSGB_OK;
}

int vsgb_solve_csr(vsgb_ctx* c, int n, int nnz, const int* row_ptr, const int* col_ind,
                   const double* values, int lower_only, const double* F, int nrhs,
                   double* u_out, vsgb_stats* stats) {
  return guarded(c, [&] {
    if (n <= 0) throw Error(VSGB_ERR_INVALID, "CUDA PCG: stiffness matrix is empty -- no free DOFs");
    if (nnz < 0 || !row_ptr || (nnz > 0 && (!col_ind || !values)) || !F || !u_out || nrhs < 1)
      throw Error(VSGB_ERR_INVALID, "vsgb_solve_csr: invalid argument");
    if (row_ptr[0] != 0 || row_ptr[n] != nnz)
      throw Error(VSGB_ERR_INVALID, "vsgb_solve_csr: row_ptr does not span nnz");
    for (int r = 0; r < n; ++r)
      if (row_ptr[r + 1] < row_ptr[r])
        throw Error(VSGB_ERR_INVALID, "vsgb_solve_csr: row_ptr decreases at row " + std::to_string(r));
    cudaStream_t s = c->stream;
    VSGB_CUDA(cudaEventRecord(c->ev[2], s));
    c->in_rp.reserve(static_cast<size_t>(n) + 1);
    c->in_ci.reserve(static_cast<size_t>(nnz > 0 ? nnz : 1));
    c->in_v.reserve(static_cast<size_t>(nnz > 0 ? nnz : 1));
    upload(c->in_rp.ptr, row_ptr, sizeof(int) * (n + 1), s);
    upload(c->in_ci.ptr, col_ind, sizeof(int) * nnz, s);
    upload(c->in_v.ptr, values, sizeof(double) * nnz, s);
    reset_assembly_error(c, s);
    c->assembled = false;
    vsgb::prepare_full_csr(n, nnz, c->in_rp.ptr, c->in_ci.ptr, c->in_v.ptr, lower_only != 0,
                           c->scr, c->K, c->num_sms, s);
    check_assembly_error(c);
    c->csr_ready = true;
    c->blocks_prebuilt = false;
    c->eng->prepare(c->K, c->precision == VSGB_MIXED, s);
    VSGB_CUDA(cudaEventRecord(c->ev[3], s));
    c->f.reserve(static_cast<size_t>(n) * nrhs);
    upload(c->f.ptr, F, sizeof(double) * n * nrhs, s);
    c->nrhs = nrhs;
    run_solves(c, nrhs, stats);
    VSGB_CUDA(cudaMemcpyAsync(u_out, c->u.ptr, sizeof(double) * n * nrhs, cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
    if (stats) {
      float ms = 0.f;
      VSGB_CUDA(cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
      stats->setup_ms = ms;
    }
  });
}

int vsgb_mesh_upload(vsgb_ctx* c, int n_nodes, const double* node_xyz, const int* node_eq3,
                     int n_elem, const int* conn, const double* E, const double* nu,
                     const int* formulation, int n_dof) {
  return guarded(c, [&] {
    if (n_nodes < 0 || n_elem < 0 || n_dof < 0 || (n_nodes > 0 && (!node_xyz || !node_eq3)) ||
        (n_elem > 0 && (!conn || !E || !nu)))
      throw Error(VSGB_ERR_INVALID, "vsgb_mesh_upload: invalid argument");
    if (n_elem > INT_MAX / 8 || n_nodes > INT_MAX / 3)
      throw Error(VSGB_ERR_LIMIT, "too many elements or nodes");
    c->u_cases = 0;
    c->mesh_ok = false;
    c->assembled = false;
    cudaStream_t s = c->stream;
    c->n_nodes = n_nodes;
    c->n_elem = n_elem;
    c->n_dof = n_dof;
    c->xyz.reserve(static_cast<size_t>(n_nodes) * 3 + 1);
    c->eq3.reserve(static_cast<size_t>(n_nodes) * 3 + 1);
    c->conn.reserve(static_cast<size_t>(n_elem) * 8 + 1);
    c->E.reserve(static_cast<size_t>(n_elem) + 1);
    c->nu.reserve(static_cast<size_t>(n_elem) + 1);
    upload(c->xyz.ptr, node_xyz, sizeof(double) * 3 * n_nodes, s);
    upload(c->eq3.ptr, node_eq3, sizeof(int) * 3 * n_nodes, s);
    upload(c->conn.ptr, conn, sizeof(int) * 8 * n_elem, s);
    upload(c->E.ptr, E, sizeof(double) * n_elem, s);
    upload(c->nu.ptr, nu, sizeof(double) * n_elem, s);
    c->has_form = formulation != nullptr;
    if (c->has_form) {
      c->form.reserve(static_cast<size_t>(n_elem) + 1);
      upload(c->form.ptr, formulation, sizeof(int) * n_elem, s);
    }
    // Every index a kernel will dereference is range-checked here, on the
    // device, before any kernel reads the mesh.
    c->mesh_bad.reserve(2);
    c->h_bad[0] = c->h_bad[1] = INT_MAX;
    upload(c->mesh_bad.ptr, c->h_bad, sizeof(int) * 2, s);
    const long long n_conn = 8LL * n_elem, n_eq = 3LL * n_nodes;
    if (n_conn + n_eq > 0) {
      k_check_mesh<<<4 * c->num_sms, 256, 0, s>>>(n_conn, c->conn.ptr, n_nodes, n_eq,
                                                 c->eq3.ptr, n_dof, c->mesh_bad.ptr);
      VSGB_LAUNCH_CHECK();
      c->eng->add_launches(1);
    }
    VSGB_CUDA(cudaMemcpyAsync(c->h_bad, c->mesh_bad.ptr, sizeof(int) * 2, cudaMemcpyDeviceToHost,
                              s));
    VSGB_CUDA(cudaStreamSynchronize(s));
    if (c->h_bad[0] != INT_MAX)
      throw Error(VSGB_ERR_INVALID, "element index " + std::to_string(c->h_bad[0] / 8) +
                                        " references a node index out of range");
    if (c->h_bad[1] != INT_MAX)
      throw Error(VSGB_ERR_INVALID, "equation index out of range at node index " +
                                        std::to_string(c->h_bad[1] / 3));
    // the tiled batched solve's coordinates: now from the caller's arrays
    // when it is on, else from the device copies on its first use
    c->coords_ready = false;
    if (c->batch_tiles != 0) block_coords(c, node_xyz, node_eq3, conn);
    c->mesh_ok = true;
  });
}

int vsgb_assemble_resident(vsgb_ctx* c, long long* nnz_lower_out) {
  return guarded(c, [&] {
    if (!c->mesh_ok) throw Error(VSGB_ERR_STATE, "no mesh uploaded");
    if (c->n_dof <= 0) throw Error(VSGB_ERR_INVALID, "CUDA PCG: stiffness matrix is empty -- no free DOFs");
    cudaStream_t s = c->stream;
    c->assembled = false;
    c->kbuf.reserve(static_cast<size_t>(c->n_elem) * 576 + 1);
    c->elem_err.reserve(1);
    const vsgb::ElementError init{INT_MAX, 0};
    VSGB_CUDA(cudaMemcpyAsync(c->elem_err.ptr, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    c->lame.reserve(2 * static_cast<size_t>(c->n_elem));
    // the topology passes (side stream) rewrite the block layout: they follow
    // everything queued on the stream before the element kernel
    VSGB_CUDA(cudaEventRecord(c->topo_start, s));
    VSGB_CUDA(cudaStreamWaitEvent(c->topo, c->topo_start, 0));
    vsgb::launch_chexa8_stiffness(c->n_elem, c->xyz.ptr, c->conn.ptr, c->E.ptr, c->nu.ptr,
                                  c->has_form ? c->form.ptr : nullptr, c->kbuf.ptr,
                                  c->elem_err.ptr, c->lame.ptr, c->num_sms, s);
    c->eng->add_launches(2);
    c->csr_ready = false;
    c->blocks_prebuilt = false;
    // Node-aligned equations: assemble the 3x3 block operator directly; the
    // scalar CSR is built only when asked for (vsgb_copy_csr_lower, or the
    // scalar format).  Its topology passes run on the side stream while the
    // element kernel runs.
    if (c->format != 1) {
      reset_assembly_error(c, c->topo);
      c->blocks_prebuilt = vsgb::assemble_blocks(
          c->n_nodes, c->n_elem, c->conn.ptr, c->eq3.ptr, c->n_dof, c->kbuf.ptr, c->scr, c->K,
          c->eng->blocks(), c->precision == VSGB_MIXED, c->num_sms, s, c->topo, c->topo_done);
    } else {
      reset_assembly_error(c, s);
    }
    if (c->blocks_prebuilt) {
      c->eng->add_launches(12);
    } else {
      vsgb::assemble_csr(c->n_nodes, c->n_elem, c->conn.ptr, c->eq3.ptr, c->n_dof, c->kbuf.ptr,
                         c->scr, c->K, c->num_sms, s);
      c->csr_ready = true;
      c->eng->add_launches(18);
    }
    vsgb::ElementError he{};
    VSGB_CUDA(cudaMemcpyAsync(&he, c->elem_err.ptr, sizeof(he), cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
    if (he.index != INT_MAX) {
      throw Error(VSGB_ERR_ELEMENT,
                  std::string("CHEXA8") + (he.code == 2 ? "EAS element index " : " element index ") +
                      std::to_string(he.index) +
                      (he.code == 2 ? ": Kaa factorization failed" : ": non-positive Jacobian"));
    }
    check_assembly_error(c);
    prepare_operator(c);
    c->assembled = true;
    if (nnz_lower_out) *nnz_lower_out = c->K.nnz_lower;
  });
}

int vsgb_assemble_chexa8(vsgb_ctx* c, int n_nodes, const double* node_xyz, const int* node_eq3,
                         int n_elem, const int* conn, const double* E, const double* nu,
                         const int* formulation, int n_dof, long long* nnz_lower_out) {
  int rc = vsgb_mesh_upload(c, n_nodes, node_xyz, node_eq3, n_elem, conn, E, nu, formulation,
                            n_dof);
  if (rc != VSGB_OK) return rc;
  return vsgb_assemble_resident(c, nnz_lower_out);
}

int vsgb_copy_csr_lower(vsgb_ctx* c, int* row_ptr, int* col_ind, double* values) {
  return guarded(c, [&] {
    if (!c->assembled) throw Error(VSGB_ERR_STATE, "nothing assembled");
    cudaStream_t s = c->stream;
    ensure_csr(c);
    DevBuf<int> lrp, lci;
    DevBuf<double> lv;
    lrp.reserve(static_cast<size_t>(c->K.n) + 1);
    lci.reserve(static_cast<size_t>(c->K.nnz_lower > 0 ? c->K.nnz_lower : 1));
    lv.reserve(static_cast<size_t>(c->K.nnz_lower > 0 ? c->K.nnz_lower : 1));
    vsgb::extract_lower(c->K, lrp.ptr, lci.ptr, lv.ptr, c->scr, c->num_sms, s);
    VSGB_CUDA(cudaMemcpyAsync(row_ptr, lrp.ptr, sizeof(int) * (c->K.n + 1), cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaMemcpyAsync(col_ind, lci.ptr, sizeof(int) * c->K.nnz_lower, cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaMemcpyAsync(values, lv.ptr, sizeof(double) * c->K.nnz_lower, cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  });
}

int vsgb_rhs_upload(vsgb_ctx* c, const double* F, int nrhs) {
  return guarded(c, [&] {
    if (!c->assembled) throw Error(VSGB_ERR_STATE, "nothing assembled");
    if (!F || nrhs < 1) throw Error(VSGB_ERR_INVALID, "vsgb_rhs_upload: invalid argument");
    c->f.reserve(static_cast<size_t>(c->K.n) * nrhs);
    upload(c->f.ptr, F, sizeof(double) * c->K.n * nrhs, c->stream);
    VSGB_CUDA(cudaStreamSynchronize(c->stream));
    c->nrhs = nrhs;
  });
}

int vsgb_solve_resident(vsgb_ctx* c, vsgb_stats* stats) {
  return guarded(c, [&] {
    if (!c->assembled || c->nrhs < 1) throw Error(VSGB_ERR_STATE, "assemble and upload RHS first");
    run_solves(c, c->nrhs, stats);
  });
}

int vsgb_solution_download(vsgb_ctx* c, double* u_out) {
  return guarded(c, [&] {
    if (!u_out) throw Error(VSGB_ERR_INVALID, "null output");
    VSGB_CUDA(cudaMemcpyAsync(u_out, c->u.ptr, sizeof(double) * c->K.n * c->nrhs,
                              cudaMemcpyDeviceToHost, c->stream));
    VSGB_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int vsgb_host_alloc(vsgb_ctx* c, size_t bytes, void** out) {
  return guarded(c, [&] {
    if (!out) throw Error(VSGB_ERR_INVALID, "vsgb_host_alloc: null output");
    *out = nullptr;
    if (cudaMallocHost(out, bytes ? bytes : 1) != cudaSuccess) {
      cudaGetLastError();
      *out = nullptr;
      throw Error(VSGB_ERR_CUDA, "cudaMallocHost of " + std::to_string(bytes) + " bytes failed");
    }
  });
}

int vsgb_host_free(vsgb_ctx* c, void* p) {
  return guarded(c, [&] {
    if (p) VSGB_CUDA(cudaFreeHost(p));
  });
}

int vsgb_solve_assembled(vsgb_ctx* c, const double* F, int nrhs, double* u_out,
                         vsgb_stats* stats) {
  int rc = vsgb_rhs_upload(c, F, nrhs);
  if (rc != VSGB_OK) return rc;
  rc = vsgb_solve_resident(c, stats);
  if (rc != VSGB_OK) return rc;
  return vsgb_solution_download(c, u_out);
}

int vsgb_node_displacements(vsgb_ctx* c, const double* u, int k, double* disp_out) {
  return guarded(c, [&] {
    if (!c->mesh_ok) throw Error(VSGB_ERR_STATE, "no mesh uploaded");
    if (!disp_out) throw Error(VSGB_ERR_INVALID, "null output");
    cudaStream_t s = c->stream;
    const int n = c->n_dof;
    const double* du = nullptr;
    if (u) {
      c->u_in.reserve(static_cast<size_t>(n > 0 ? n : 1));
      upload(c->u_in.ptr, u, sizeof(double) * n, s);
      du = c->u_in.ptr;
    } else {
      if (k < 0 || k >= c->u_cases || c->K.n != n)
        throw Error(VSGB_ERR_STATE, "no solution of load case " + std::to_string(k) +
                                        " on this context");
      du = c->u.ptr + static_cast<size_t>(k) * n;
    }
    const size_t nn = static_cast<size_t>(c->n_nodes);
    c->node_disp.reserve(6 * nn + 1);
    vsgb::launch_node_displacements(c->n_nodes, c->eq3.ptr, du, n, c->node_disp.ptr, c->num_sms,
                                    s);
    c->eng->add_launches(1);
    VSGB_CUDA(cudaMemcpyAsync(disp_out, c->node_disp.ptr, sizeof(double) * 6 * nn,
                              cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  });
}

int vsgb_solid_stress(vsgb_ctx* c, const double* u, int k, double* centroid_out,
                      double* nodal_out, double* kernel_ms) {
  return guarded(c, [&] {
    if (!c->mesh_ok) throw Error(VSGB_ERR_STATE, "no mesh uploaded");
    if (!centroid_out) throw Error(VSGB_ERR_INVALID, "null output");
    cudaStream_t s = c->stream;
    const int n = c->n_dof;
    const double* du = nullptr;
    if (u) {
      c->u_in.reserve(static_cast<size_t>(n > 0 ? n : 1));
      upload(c->u_in.ptr, u, sizeof(double) * n, s);
      du = c->u_in.ptr;
    } else {
      if (k < 0 || k >= c->u_cases || c->K.n != n)
        throw Error(VSGB_ERR_STATE, "no solution of load case " + std::to_string(k) +
                                        " on this context");
      du = c->u.ptr + static_cast<size_t>(k) * n;
    }
    const size_t ne = static_cast<size_t>(c->n_elem);
    c->stress_c.reserve(7 * ne + 1);
    if (nodal_out) c->stress_n.reserve(56 * ne + 1);
    c->lame.reserve(2 * ne + 1);
    VSGB_CUDA(cudaEventRecord(c->ev[2], s));
    vsgb::launch_solid_stress(c->n_elem, c->xyz.ptr, c->conn.ptr, c->eq3.ptr, c->E.ptr, c->nu.ptr,
                              du, n, c->lame.ptr, c->stress_c.ptr,
                              nodal_out ? c->stress_n.ptr : nullptr, c->num_sms, s);
    VSGB_CUDA(cudaEventRecord(c->ev[3], s));
    c->eng->add_launches(2);
    VSGB_CUDA(cudaMemcpyAsync(centroid_out, c->stress_c.ptr, sizeof(double) * 7 * ne,
                              cudaMemcpyDeviceToHost, s));
    if (nodal_out)
      VSGB_CUDA(cudaMemcpyAsync(nodal_out, c->stress_n.ptr, sizeof(double) * 56 * ne,
                                cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
    if (kernel_ms) {
      float ms = 0.f;
      VSGB_CUDA(cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]));
      *kernel_ms = ms;
    }
  });
}

int vsgb_element_sensitivity(vsgb_ctx* c, const double* u, const double* lambda,
                             double* dJdE_out) {
  return guarded(c, [&] {
    if (!c->assembled) throw Error(VSGB_ERR_STATE, "nothing assembled");
    if (!u || !lambda || !dJdE_out) throw Error(VSGB_ERR_INVALID, "null argument");
    cudaStream_t s = c->stream;
    DevBuf<double> du, dl, out;
    du.reserve(static_cast<size_t>(c->n_dof) + 1);
    dl.reserve(static_cast<size_t>(c->n_dof) + 1);
    out.reserve(static_cast<size_t>(c->n_elem) + 1);
    upload(du.ptr, u, sizeof(double) * c->n_dof, s);
    upload(dl.ptr, lambda, sizeof(double) * c->n_dof, s);
    vsgb::launch_element_sensitivity(c->n_elem, c->conn.ptr, c->eq3.ptr, c->E.ptr, c->kbuf.ptr,
                                     du.ptr, dl.ptr, out.ptr, nullptr, nullptr, c->num_sms, s);
    c->eng->add_launches(1);
    VSGB_CUDA(cudaMemcpyAsync(dJdE_out, out.ptr, sizeof(double) * c->n_elem,
                              cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  });
}

int vsgb_adjoint_gradients(vsgb_ctx* c, const double* F, const double* dJdu, double* u_out,
                           double* lambda_out, double* dCdE_out, double* dJdE_out,
                           vsgb_stats* stats) {
  return guarded(c, [&] {
    if (!c->assembled) throw Error(VSGB_ERR_STATE, "nothing assembled");
    if (!F) throw Error(VSGB_ERR_INVALID, "vsgb_adjoint_gradients: F is null");
    if ((dJdE_out || lambda_out) && !dJdu)
      throw Error(VSGB_ERR_INVALID, "vsgb_adjoint_gradients: dJ/du is needed for lambda / dJdE");
    cudaStream_t s = c->stream;
    const size_t n = static_cast<size_t>(c->K.n);
    const int nrhs = dJdu ? 2 : 1;
    c->f.reserve(n * nrhs);
    upload(c->f.ptr, F, sizeof(double) * n, s);
    if (dJdu) upload(c->f.ptr + n, dJdu, sizeof(double) * n, s);
    c->nrhs = nrhs;
    run_solves(c, nrhs, stats);  // u and lambda from one batched solve
    c->grad.reserve(2 * static_cast<size_t>(c->n_elem) + 2);
    double* dC = c->grad.ptr;
    double* dJ = c->grad.ptr + c->n_elem + 1;
    // compliance: lambda = u; J: lambda solves K lambda = dJ/du
    vsgb::launch_element_sensitivity(c->n_elem, c->conn.ptr, c->eq3.ptr, c->E.ptr, c->kbuf.ptr,
                                     c->u.ptr, c->u.ptr, dC, dJdu ? c->u.ptr + n : nullptr,
                                     dJdu ? dJ : nullptr, c->num_sms, s);
    c->eng->add_launches(1);
    if (u_out) VSGB_CUDA(cudaMemcpyAsync(u_out, c->u.ptr, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (lambda_out)
      VSGB_CUDA(cudaMemcpyAsync(lambda_out, c->u.ptr + n, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (dCdE_out)
      VSGB_CUDA(cudaMemcpyAsync(dCdE_out, dC, sizeof(double) * c->n_elem, cudaMemcpyDeviceToHost, s));
    if (dJdE_out)
      VSGB_CUDA(cudaMemcpyAsync(dJdE_out, dJ, sizeof(double) * c->n_elem, cudaMemcpyDeviceToHost, s));
    VSGB_CUDA(cudaStreamSynchronize(s));
  });
}

int vsgb_timer_start(vsgb_ctx* c) {
  return guarded(c, [&] {
    VSGB_CUDA(cudaStreamSynchronize(c->stream));
    VSGB_CUDA(cudaEventRecord(c->ev[2], c->stream));
  });
}

int vsgb_timer_stop(vsgb_ctx* c, double* ms) {
  return guarded(c, [&] {
    VSGB_CUDA(cudaEventRecord(c->ev[3], c->stream));
    VSGB_CUDA(cudaEventSynchronize(c->ev[3]));
    VSGB_CUDA(cudaStreamSynchronize(c->stream));
    float m = 0.f;
    VSGB_CUDA(cudaEventElapsedTime(&m, c->ev[2], c->ev[3]));
    if (ms) *ms = m;
  });
}

int vsgb_time_spmv(vsgb_ctx* c, int precision, int reps, double* avg_ms, double* bytes) {
  return guarded(c, [&] {
    if (!c->assembled && c->K.n == 0) throw Error(VSGB_ERR_STATE, "no operator");
    if (precision == VSGB_MIXED && !c->eng->has32())
      c->eng->prepare(c->K, true, c->stream, c->blocks_prebuilt && c->format != 1);
    c->eng->time_spmv(precision, reps > 0 ? reps : 20, c->stream, avg_ms);
    if (bytes) *bytes = c->eng->spmv_bytes(precision);
  });
}

long long vsgb_kernel_launches(vsgb_ctx* c) { return c ? c->eng->launches() : -1; }

int vsgb_phase_times(vsgb_ctx* c, double* out11) {
  if (!c || !out11) return VSGB_ERR_INVALID;
  const double* t = c->eng->phase_times();
  for (int k = 0; k < vsgb::kTracePhases + 2; ++k) out11[k] = t[k];
  return VSGB_OK;
}

int vsgb_rhs_stats(vsgb_ctx* c, int k, int* iterations, double* rel_residual, int* converged,
                   int* batched) {
  return guarded(c, [&] {
    if (k < 0 || static_cast<size_t>(k) >= c->rhs.size())
      throw Error(VSGB_ERR_INVALID, "vsgb_rhs_stats: load case " + std::to_string(k) +
                                        " not in the last solve");
    const vsgb::SolveResult& r = c->rhs[static_cast<size_t>(k)];
    if (iterations) *iterations = r.iterations;
    if (rel_residual) *rel_residual = r.rel;
    if (converged) *converged = r.converged ? 1 : 0;
    if (batched) *batched = c->last_batched ? 1 : 0;
  });
}

}  // extern "C"
