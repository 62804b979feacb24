/* include/vsgb.h — C ABI of the GB300 (sm_103a) SOL 101 CHEXA8 backend.
 *
 * One shared library (libvsgb.so) replaces three layers of vibestran's
 * SOL 101 solid path on one GPU:
 *   - the CHEXA8 element stiffness (src/elements/solid_elements.cpp:95-180 SRI,
 *     :1054-1206 EAS) and the lower-triangle CSR assembly
 *     (src/solver/assembly_parallel.hpp:69-110, src/core/sparse_matrix.cpp:16-150),
 *   - the analysis DOF map (src/core/dof_map.cpp:10-97,
 *     src/solver/analysis_support.cpp:176-214) and FORCE loads
 *     (src/solver/linear_static.cpp:344-374),
 *   - the SolverBackend::solve of --backend=cuda-pcg / cuda-pcg-mixed
 *     (include/solver/solver_backend.hpp:20-51,
 *     src/solver/cuda_pcg_backend_impl.hpp:1688-2262).
 *
 * Conventions: plain C types, host pointers unless a name says "device",
 * 0-based equation indices, -1 marks a constrained DOF (CONSTRAINED_DOF,
 * include/core/dof_map.hpp:20).  Every function returns VSGB_OK (0) or a
 * negative status; the message of the last failure on a context is returned
 * by vsgb_last_error().  A context is single-threaded: one host thread at a
 * time (the reference backend has the same contract).
 */
#ifndef VSGB_H
#define VSGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ── status codes ───────────────────────────────────────────────────────── */
#define VSGB_OK 0
#define VSGB_ERR_INVALID (-1)       /* bad argument: size mismatch, empty K, bad index */
#define VSGB_ERR_SINGULAR (-2)      /* zero / missing diagonal, r.z <= 0 at start */
#define VSGB_ERR_NOT_CONVERGED (-3) /* max iterations reached, or p.Ap <= 0 breakdown */
#define VSGB_ERR_CUDA (-4)          /* CUDA runtime error (message has the CUDA text) */
#define VSGB_ERR_ELEMENT (-5)       /* non-positive Jacobian / EAS Kaa not SPD */
#define VSGB_ERR_NO_DEVICE (-6)     /* no CUDA device, or not an sm_103 device */
#define VSGB_ERR_STATE (-7)         /* call order: e.g. solve before assemble */
#define VSGB_ERR_LIMIT (-8)         /* a documented device limit was exceeded */

/* ── precision / formulation selectors ──────────────────────────────────── */
#define VSGB_FP64 64  /* FP64 Jacobi PCG (cuda-pcg semantics) */
#define VSGB_MIXED 32 /* FP32 inner PCG + FP64 refinement on the GPU (cuda-pcg-mixed) */

#define VSGB_EAS 0 /* CHexa8Eas (default, PSOLID ISOP blank or EAS) */
#define VSGB_SRI 1 /* CHexa8 selective reduced integration (ISOP = SRI) */

/* ── options for vsgb_set_option ────────────────────────────────────────── */
#define VSGB_OPT_TOLERANCE 1      /* relative residual target (default 1e-8 FP64, 1e-6 mixed);
                                     the stopping test of a solve that is not
                                     error-controlled (VSGB_OPT_ERROR_TARGET) */
#define VSGB_OPT_MAX_ITERS 2      /* max PCG iterations per solve (default 10000) */
#define VSGB_OPT_PRECISION 3      /* VSGB_FP64 or VSGB_MIXED */
#define VSGB_OPT_INNER_TOL 4      /* mixed: inner FP32 tolerance (<=0: 1e-3 when error-controlled,
                                     otherwise clamp(100*tol,1e-4,1e-2) as cuda-pcg-mixed).
                                     Error-controlled solves should keep the default: below
                                     1e-3 the bound on the FP32 operator's share of the
                                     error can miss the target. */
#define VSGB_OPT_MAX_SOLVES 5     /* mixed: max inner solves (<= 0: default, 3 = 1 + 2
                                     corrections; 5 when error-controlled) */
#define VSGB_OPT_CHECK_EVERY 6    /* iterations launched between convergence checks (the
                                     batched solve: per body of its device-side loop) */
#define VSGB_OPT_USE_GRAPH 7      /* 1: replay iteration batches as CUDA graphs, the batched
                                     inner solve as one graph launch (default 1) */
#define VSGB_OPT_FORMAT 8         /* 0 auto, 1 scalar CSR, 2 3x3 node blocks */
#define VSGB_OPT_RESIDENT 9       /* 1: one persistent launch per PCG solve (default 1) */
#define VSGB_OPT_BATCHED 10       /* load cases (nrhs > 1) on the 3x3 block operator:
                                     0 one solve per case, as the reference's subcase
                                     loop; 1 (default) one batched PCG from 4 cases
                                     (mixed) or 10 cases (FP64) up, where it is faster;
                                     2 always batched */
#define VSGB_OPT_ADAPTIVE_INNER 12 /* mixed: 1 (default) lets a refinement step's inner
                                     solve stop at 0.5*tol/(current true residual) when
                                     that is looser than the inner tolerance; 0: every
                                     inner solve runs to the inner tolerance, as
                                     cuda-pcg-mixed */
#define VSGB_OPT_L2_PERSIST 11    /* 1: mark the operator values persisting in L2 during
                                     each persistent PCG launch (default 0: measured no
                                     gain, the solve is not bound by L2 misses) */
#define VSGB_OPT_PRECOND 13       /* VSGB_PRECOND_JACOBI (default, the reference's Jacobi
                                     fallback, cuda_pcg_backend_impl.hpp:1041-1252) or
                                     VSGB_PRECOND_BLOCK_JACOBI: the inverse 3x3 diagonal
                                     block of every node (the persistent solve on the
                                     block operator, FP64 and mixed; one solve per load
                                     case); a solve it cannot run returns
                                     VSGB_ERR_INVALID, a block that is not positive
                                     definite VSGB_ERR_SINGULAR */

#define VSGB_OPT_ERROR_TARGET 14  /* relative displacement error target of an
                                     error-controlled solve; < 0 (default): 1e-6 for
                                     mixed precision unless a residual tolerance was
                                     chosen (vsgb_create tol > 0 or VSGB_OPT_TOLERANCE
                                     > 0), off for FP64; 0: off (the reference's
                                     residual test, VSGB_OPT_TOLERANCE).
                                     The solve estimates its error in the
                                     preconditioner's norm from its own recurrence
                                     (Hestenes-Stiefel identity over blocks of 16
                                     iterations: a geometric tail of the current error
                                     and a 32-iteration delayed bound, both within
                                     target/3 in two blocks in a row) and ignores the
                                     residual tolerance.  Mixed: the first inner solve stops on
                                     VSGB_OPT_INNER_TOL, every later one on the error
                                     estimate; FP64: one estimate-stopped solve.
                                     Persistent solves and the batched solve only (the
                                     launch-per-kernel path keeps the residual test).
                                     No reference counterpart. */
#define VSGB_OPT_SPIN_LIMIT 15    /* polls of a grid wait of the persistent solve before
                                     it gives up and the solve returns VSGB_ERR_CUDA
                                     ("a grid barrier ... timed out"); <= 0: the default
                                     (2^22, about a second).  For tests of that path. */
#define VSGB_OPT_PHASE_TRACE 16   /* 1: time the phases of every iteration of the
                                     persistent solve (thread 0 of each CTA reads the
                                     global timer at the phase boundaries; a few
                                     instructions per iteration); read with
                                     vsgb_phase_times.  Default 0. */
#define VSGB_OPT_BATCH_TILES 17   /* batched mixed solve on the uploaded mesh: each FP32
                                     inner solve of up to 16 load cases as one persistent
                                     launch over spatially compact tiles of block rows
                                     (recursive coordinate bisection of the node
                                     coordinates) whose neighbour nodes are staged in
                                     shared memory.  0 (default): off, one launch per
                                     kernel (measured faster on GB300); 1: tile size timed
                                     on the first solve of a sparsity pattern; 8..65536:
                                     fixed rows per tile. */
#define VSGB_OPT_COARSE 18        /* error-controlled mixed solves: 1 (default) adds the
                                     Galerkin correction in the span of the lowest Ritz
                                     vectors of the operator's first inner solve after
                                     every FP64 residual (the smooth modes the FP32 inner
                                     solves resolve last); 2 also deflates the first FP32
                                     inner solve of later single-RHS solves with the same
                                     operator by that basis (scalar Jacobi; faster, but
                                     the error target can be missed when the basis lacks
                                     a low mode the load excites); 0: off. */

#define VSGB_PRECOND_JACOBI 0
#define VSGB_PRECOND_BLOCK_JACOBI 1

typedef struct vsgb_ctx vsgb_ctx;

/* Per-solve diagnostics (SolverBackend::last_iteration_count /
 * last_estimated_error, include/solver/solver_backend.hpp:39-43, plus timing). */
typedef struct vsgb_stats {
  int iterations;        /* PCG iterations (mixed: summed over inner solves; nrhs>1: max) */
  int inner_solves;      /* mixed: FP32 solves run (1 for FP64) */
  int converged;         /* 1 when the tolerance was met */
  int format;            /* operator format used: 1 scalar CSR, 2 3x3 node blocks */
  double rel_residual;   /* FP64: sqrt(r.r)/||F|| of the recursion; mixed: true FP64 residual */
  double solve_ms;       /* device time of the iteration phase (CUDA events) */
  double setup_ms;       /* device time of operator preparation (upload/expand/convert) */
  double spmv_bytes;     /* algorithmic bytes of one SpMV of the operator used */
  double kernel_ms;      /* device time of the persistent (one launch per solve) PCG
                            kernels of this solve, CUDA events around each launch;
                            0 when the launch-per-kernel path ran */
  double kernel_iterations; /* PCG iterations those launches ran */
  double est_rel_error;  /* error-controlled solve: estimated relative displacement
                            error (max over load cases); -1 when not estimated */
  int batch_tile_rows;   /* batched solve: rows per tile of the persistent tiled
                            FP32 solve (0: one launch per kernel, or not batched) */
} vsgb_stats;

/* Create a context on `device` (cuda-pcg uses device 0,
 * src/solver/cuda_pcg_backend_impl.hpp:2040-2065).  tol <= 0 selects the
 * default (1e-8 FP64, 1e-6 mixed, as CudaPCGSolverBackend::try_create and
 * CudaMixedPCGSolverBackend::try_create); max_iters <= 0 selects 10000.
 * Returns VSGB_ERR_NO_DEVICE (and *out = NULL) when no usable GPU exists —
 * the try_create() -> nullopt contract. */
int vsgb_create(int device, double tol, int max_iters, int precision, vsgb_ctx** out);
void vsgb_destroy(vsgb_ctx* ctx);
int vsgb_set_option(vsgb_ctx* ctx, int option, double value);
/* Copies the last error message (NUL-terminated, truncated to len). */
int vsgb_last_error(vsgb_ctx* ctx, char* buf, size_t len);
int vsgb_device_name(vsgb_ctx* ctx, char* buf, size_t len);
/* Backend display name, e.g. "GB300 PCG + Jacobi float64 (GPU)". */
int vsgb_backend_name(vsgb_ctx* ctx, char* buf, size_t len);

/* Drop-in SolverBackend::solve (include/solver/solver_backend.hpp:27-30):
 * K as CsrData (row_ptr[n+1], col_ind[nnz], values[nnz]; lower_only != 0 for
 * SymmetryStorage::Lower), F[n*nrhs] (column-major: rhs k at F + k*n) ->
 * u_out[n*nrhs].  Errors follow cuda-pcg: empty K, |F| != n, zero or missing
 * diagonal, r.z <= 0, non-convergence or breakdown.  A zero RHS returns zeros
 * with 0 iterations. */
int vsgb_solve_csr(vsgb_ctx* ctx, int n, int nnz, const int* row_ptr, const int* col_ind,
                   const double* values, int lower_only, const double* F, int nrhs,
                   double* u_out, vsgb_stats* stats);

/* ── DOF map and loads (host) ───────────────────────────────────────────── */

/* Analysis DOF map of a CHEXA8-only model (DofMap::build + constrain_batch,
 * src/core/dof_map.cpp:10-97; build_analysis_dof_map,
 * src/solver/analysis_support.cpp:176-214): node ids are ranked ascending,
 * each node owns 6 slots, T1-T3 of element nodes are active, SPC components
 * (bit d set = DOF d+1) are removed, remaining slots are numbered densely.
 * conn_ids holds grid ids (8 per element).  eq6_out[6*i+d] is the equation of
 * DOF d of node_ids[i], or -1. */
int vsgb_build_dof_map(int n_nodes, const int* node_ids, int n_elem, const int* conn_ids,
                       int n_spc, const int* spc_node_ids, const int* spc_masks, int* eq6_out,
                       int* n_free, char* err, size_t errlen);

/* FORCE cards with CID 0 (LinearStaticSolver::apply_point_loads,
 * src/solver/linear_static.cpp:344-374): F[eq(node, d)] += scale * dir[d]. */
int vsgb_apply_forces(int n_nodes, const int* node_ids, const int* eq6, int n_force,
                      const int* force_node_ids, const double* scale, const double* dir,
                      int n, double* F, char* err, size_t errlen);

/* ── GPU element stiffness + assembly ───────────────────────────────────── */

/* Upload a node-indexed CHEXA8 mesh and assemble K on the GPU (element
 * stiffness, lower-triangle pattern with the value != 0.0 filter of
 * add_element_stiffness, duplicate sums in ascending element order).
 * node_xyz[3*n_nodes]; node_eq3[3*n_nodes] = equations of T1-T3 (-1 =
 * constrained); conn[8*n_elem] = 0-based node indices; E, nu per element;
 * formulation per element (NULL = all EAS).  The assembled K stays resident
 * in the context for vsgb_solve_assembled; *nnz_lower_out receives the nnz of
 * the reference's lower-triangle CsrData. */
int vsgb_assemble_chexa8(vsgb_ctx* ctx, int n_nodes, const double* node_xyz,
                         const int* node_eq3, int n_elem, const int* conn, const double* E,
                         const double* nu, const int* formulation, int n_dof,
                         long long* nnz_lower_out);

/* Copy the resident K out as the reference's lower-triangle CsrData. */
int vsgb_copy_csr_lower(vsgb_ctx* ctx, int* row_ptr, int* col_ind, double* values);

/* Solve with the resident K: F[n*nrhs] host -> u_out[n*nrhs] host.
 * Several load cases on the 3x3 block operator run as one batched PCG (16
 * right-hand sides per matrix sweep, each with its own recurrence and
 * stopping test) as VSGB_OPT_BATCHED selects; otherwise, and on the
 * scalar-CSR operator, they are solved one after another. */
int vsgb_solve_assembled(vsgb_ctx* ctx, const double* F, int nrhs, double* u_out,
                         vsgb_stats* stats);

/* ── device-resident staging (inputs already in HBM) ────────────────────── */

/* Upload the mesh only (no assembly). */
int vsgb_mesh_upload(vsgb_ctx* ctx, int n_nodes, const double* node_xyz, const int* node_eq3,
                     int n_elem, const int* conn, const double* E, const double* nu,
                     const int* formulation, int n_dof);
/* Element stiffness + assembly from the resident mesh (no host traffic). */
int vsgb_assemble_resident(vsgb_ctx* ctx, long long* nnz_lower_out);
/* Upload right-hand sides into the context (n*nrhs doubles). */
int vsgb_rhs_upload(vsgb_ctx* ctx, const double* F, int nrhs);
/* Solve resident K against the resident RHS; the solution stays on the GPU. */
int vsgb_solve_resident(vsgb_ctx* ctx, vsgb_stats* stats);
/* Download the resident solution (n*nrhs doubles). */
int vsgb_solution_download(vsgb_ctx* ctx, double* u_out);

/* Page-locked host memory on the context's device, for the host arrays the
 * calls above copy from or into (mesh, loads, solutions): those copies then
 * run at the host link's rate instead of through a pageable staging copy.
 * No reference counterpart (the reference's host arrays are std::vector). */
int vsgb_host_alloc(vsgb_ctx* ctx, size_t bytes, void** out);
int vsgb_host_free(vsgb_ctx* ctx, void* p);

/* ── adjoint sensitivities ──────────────────────────────────────────────── */

/* dJ/dE_e = -lambda_e^T (K_e / E_e) u_e for every element of the resident
 * mesh, given host vectors u[n] and lambda[n] (lambda solves K lambda = dJ/du;
 * for compliance F^T u, lambda = u). */
int vsgb_element_sensitivity(vsgb_ctx* ctx, const double* u, const double* lambda,
                             double* dJdE_out);

/* Adjoint gradients of the resident model with respect to every element's
 * Young's modulus.  No counterpart in the reference (it has no sensitivity
 * analysis); the functionals are compliance C = F^T u and a linear response
 * J = dJdu^T u.  Solves K [u, lambda] = [F, dJdu] (one load case when dJdu
 * is NULL) with the context's precision and tolerance, then in one pass over
 * the stored element matrices
 *   dC/dE_e = -u_e^T K_e^0 u_e,   dJ/dE_e = -lambda_e^T K_e^0 u_e,
 * K_e^0 = K_e / E_e.  u_out[n], lambda_out[n], dCdE_out[n_elem] and
 * dJdE_out[n_elem] may each be NULL; lambda_out and dJdE_out need dJdu. */
int vsgb_adjoint_gradients(vsgb_ctx* ctx, const double* F, const double* dJdu, double* u_out,
                           double* lambda_out, double* dCdE_out, double* dJdE_out,
                           vsgb_stats* stats);

/* CHEXA8 stresses of the resident mesh (LinearStaticSolver::recover_results,
 * solid branch, src/solver/linear_static.cpp:1059-1195): for every element the
 * stress at the centroid and at its 8 corner nodes, each as (sx, sy, sz, sxy,
 * syz, szx, von_mises), sigma = D B u_e of the plain trilinear element.  u:
 * n_dof host displacements, or NULL for load case k of the last solve on this
 * context.  centroid_out: n_elem*7 doubles; nodal_out: n_elem*8*7 doubles
 * (corner j of element e at (8e+j)*7) or NULL; kernel_ms (may be NULL): device
 * time of the recovery kernels.  No TEMP loads are on this path, so the thermal
 * strain of solid_sigma_from_B (:186-196) is zero. */
int vsgb_solid_stress(vsgb_ctx* ctx, const double* u, int k, double* centroid_out,
                      double* nodal_out, double* kernel_ms);

/* Nodal displacements of the resident mesh (LinearStaticSolver::recover_results,
 * displacement part, src/solver/linear_static.cpp:574-587): disp_out[6 i + d]
 * = T1 T2 T3 R1 R2 R3 of node i in the uploaded node order, u[eq] where the
 * DOF is free and 0 where it is constrained (the rotations always are: solid
 * elements activate T1-T3 only).  u: n_dof host displacements, or NULL for
 * load case k of the last solve on this context; disp_out: n_nodes*6 doubles.
 * The deck subset of this path has no CD frames, so the values stay in the
 * basic frame (the reference rotates only nodes that name one, :589-612);
 * vsgb_write_node_csv lists them in ascending node-id order as the reference
 * does. */
int vsgb_node_displacements(vsgb_ctx* ctx, const double* u, int k, double* disp_out);

/* The nodal CSV of CsvWriter (src/io/csv_writer.cpp:34-57): the header
 * "# node_id, subcase_id, T1, T2, T3, R1, R2, R3", then for each subcase s in
 * the order given and each node in ascending id order the line
 * "id, subcase, d0, ..., d5" with the values in scientific notation with 8
 * digits after the point.  disp: n_subcases blocks of n_nodes*6 doubles in
 * the node order of node_ids (vsgb_node_displacements' output).  Host only.
 * Returns VSGB_ERR_INVALID with the reference's "Cannot write CSV: <path>"
 * when the file cannot be opened. */
int vsgb_write_node_csv(const char* path, int n_nodes, const int* node_ids, int n_subcases,
                        const int* subcase_ids, const double* disp, char* err, size_t errlen);

/* ── BDF decks (host only, no GPU needed) ────────────────────────────────── */

/* Reader of the deck subset of the SOL 101 CHEXA8 path, in place of
 * BdfParser::parse_file / parse_string (src/io/bdf_parser.cpp:83-95) for it:
 * GRID, CHEXA, PSOLID, MAT1, SPC1, FORCE, PARAM bulk cards (free, small and
 * large field, continuations, Nastran number forms) and SOL / SUBCASE / LOAD /
 * SPC case control, with the reference's card assembly rules.  Cards the
 * reference does not know are ignored and listed (vsgb_bdf_message 1); cards
 * it knows that change the model outside this path (other elements, rigid
 * elements, coordinate systems in use, other loads / SPCs or temperatures of
 * a selected set, MPC sets) make vsgb_bdf_mesh or the per-subcase calls
 * fail with the reason.  The bulk data is parsed by `threads` host threads
 * (<= 0: all).  Parse errors return VSGB_ERR_INVALID with the reference's
 * "Line N: ..." text in err. */
typedef struct vsgb_bdf vsgb_bdf;

typedef struct {
  int n_nodes;       /* distinct GRIDs */
  int n_elem;        /* CHEXA cards */
  int n_subcases;
  int sol;           /* 101, 103, or 0 when the deck has no SOL line */
  long long lines;   /* physical lines */
  long long cards;   /* logical bulk cards */
  int threads;       /* host threads used for the bulk data */
  double read_ms;    /* file read (vsgb_bdf_read) */
  double parse_ms;   /* line split, cards, mesh arrays */
  int mesh_ok;       /* 1 when vsgb_bdf_mesh succeeds */
  double lines_ms;   /* of parse_ms: line index, markers, case control */
  double cards_ms;   /* of parse_ms: bulk cards (the threaded part) */
  double mesh_ms;    /* of parse_ms: mesh arrays and checks */
} vsgb_bdf_stats;

int vsgb_bdf_read(const char* path, int threads, vsgb_bdf** out, char* err, size_t err_len);
int vsgb_bdf_parse(const char* text, size_t len, int threads, vsgb_bdf** out, char* err,
                   size_t err_len);
void vsgb_bdf_free(vsgb_bdf* deck);
int vsgb_bdf_info(vsgb_bdf* deck, vsgb_bdf_stats* info);
/* which: 0 why the mesh cannot be formed ("" when it can), 1 ignored-card
 * warnings, 2 the last error of a call on this deck. */
int vsgb_bdf_message(vsgb_bdf* deck, int which, char* buf, size_t len);
/* Subcase s (file order): its id and LOAD / SPC set ids. */
int vsgb_bdf_subcase(vsgb_bdf* deck, int s, int* id, int* load_set, int* spc_set);
/* Mesh arrays, each optional: node_ids[n_nodes] ascending, xyz[3 n_nodes];
 * elem_ids[n_elem], conn[8 n_elem] (0-based indices into node_ids, CHEXA G1-G8
 * order), E / nu[n_elem] (MAT1 of the element's PSOLID), form[n_elem]
 * (VSGB_EAS / VSGB_SRI from PSOLID ISOP).  Elements in card order. */
int vsgb_bdf_mesh(vsgb_bdf* deck, int* node_ids, double* xyz, int* elem_ids, int* conn,
                  double* E, double* nu, int* form);
/* SPC1 entries (grid id, component mask bit d = DOF d+1) and FORCE cards
 * (grid id, scale, direction[3]) of subcase s's sets, in card order; call
 * with null arrays for *count first. */
int vsgb_bdf_constraints(vsgb_bdf* deck, int s, int* count, int* nodes, int* masks);
int vsgb_bdf_forces(vsgb_bdf* deck, int s, int* count, int* nodes, double* scale,
                    double* dir);

/* ── measurement helpers ────────────────────────────────────────────────── */

/* Events on the context stream, synchronised on both sides. */
int vsgb_timer_start(vsgb_ctx* ctx);
int vsgb_timer_stop(vsgb_ctx* ctx, double* ms);
/* Average device time of `reps` back-to-back launches of the resident
 * operator's SpMV (precision VSGB_FP64 or VSGB_MIXED). */
int vsgb_time_spmv(vsgb_ctx* ctx, int precision, int reps, double* avg_ms, double* bytes);
/* Number of kernels this context launched since creation. */
long long vsgb_kernel_launches(vsgb_ctx* ctx);
/* With VSGB_OPT_PHASE_TRACE on: the last solve's persistent launches split
 * into phases, per iteration and averaged over the CTAs (us): out11[0] gather
 * of the x window, [1] block SpMV (+ the own-row p update and p.Ap); the
 * first grid reduction (p.Ap) as [2] the CTA's own sums up to its arrival,
 * [3] the wait for the other CTAs, [4] the grid total and the recurrence;
 * [5] the u / r / z update; the second grid reduction (r.z, r.r) as [6], [7],
 * [8]; [9] the slowest CTA's SpMV; [10] iterations timed.  No reference
 * counterpart (a measurement helper). */
int vsgb_phase_times(vsgb_ctx* ctx, double* out11);

/* Per-load-case outcome of the last solve (k < nrhs): PCG iterations
 * (mixed: summed over inner solves), relative residual, converged flag and
 * whether the load cases ran as one batched PCG.  The reference reports one
 * subcase per solve() call (SolverBackend::last_iteration_count /
 * last_estimated_error, include/solver/solver_backend.hpp:39-43). */
int vsgb_rhs_stats(vsgb_ctx* ctx, int k, int* iterations, double* rel_residual, int* converged,
                   int* batched);

/* ── allocation-free solve ──────────────────────────────────────────────── */

/* Largest system (equations) vsgb_pcg_solve_noalloc accepts. */
#define VSGB_NOALLOC_MAX_N 65536

/* FP64 Jacobi PCG that allocates no GPU or pinned memory, for callers that
 * cannot call cudaMalloc: code running inside another framework's memory pool,
 * or a latency-critical loop where an allocation (which may synchronise the
 * device or fail under memory pressure) is not allowed.  This entry point has
 * no counterpart in the reference; it is the cuda-pcg FP64 Jacobi iteration
 * (same recurrence, convergence test and error texts as vsgb_solve_csr) on
 * caller-owned DEVICE buffers:
 *   d_row_ptr[n+1], d_col_ind[nnz], d_values[nnz] — FULL-storage symmetric CSR
 *   (both triangles), d_F[n] in, d_u[n] out; `stream` is a cudaStream_t (NULL =
 *   legacy default stream) of the current device.
 * Its scratch (inverse diagonal, r, z, p, Ap, reduction partials, scalars;
 * about 2.7 MB) is one static __device__ array that every GPU loading the
 * library holds until exit, so n is limited to VSGB_NOALLOC_MAX_N (larger n
 * returns VSGB_ERR_LIMIT).  The first call on a device resolves the array's
 * device address — make it before any stream capture on that device.  That
 * address is kept for the device's primary context of that moment: after a
 * cudaDeviceReset the library must be loaded again (a new process) before
 * this entry point is used on that device.  All calls share the array: calls
 * that overlap on the GPU (other streams or host threads) race and must be
 * serialised by the caller.  The row pointer is checked on the device before
 * anything is read through it (VSGB_ERR_INVALID); column indices outside
 * [0, n) are VSGB_ERR_INVALID, a zero or missing diagonal VSGB_ERR_SINGULAR.
 * A non-positive p*Ap stops the solve as in cuda-pcg: iterations_out is then
 * max_iters and VSGB_ERR_NOT_CONVERGED is returned.  err receives the message
 * of a failure (may be NULL). */
int vsgb_pcg_solve_noalloc(int n, int nnz, const int* d_row_ptr, const int* d_col_ind,
                           const double* d_values, const double* d_F, double* d_u, double tol,
                           int max_iters, void* stream, int* iterations_out,
                           double* rel_residual_out, char* err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* VSGB_H */
