/*
 * lss.h -- C ABI of the GB300-native locally-stiff linear solver.
 *
 * One solver object = one polysolve `GPUHybrid` linear solver
 * (src/polysolve/linear/GPUHybrid.hpp:27-192 in the reference), re-built for
 * a single GB300: l1 row-norm scoring and 1D-GMM stiff-DOF selection, a
 * multilevel additive Schwarz (MAS) preconditioner composed with a dense FP64
 * factor of the stiff block, and FP64 PCG.  Hand-written sm_103a kernels.
 *
 * Conventions
 *  - Matrices are Eigen-style compressed storage (`StiffnessMatrix`,
 *    src/polysolve/Types.hpp:11-15): int32 outer[n+1], int32 inner[nnz],
 *    double values[nnz].  As in the reference (GPUHybrid.cu:203-209, the CSC
 *    arrays are handed to hypre as CSR) the outer index is the row; the matrix
 *    must be symmetric positive definite, so CSC and CSR coincide.
 *  - Host pointers in, host pointers out, unless a name ends in `_device`.
 *  - Every entry point returns an lss_status and never exits the process
 *    (the reference calls exit() on CUDA errors, GPUHybrid.cu:34-63).
 *  - A solver is not thread-safe (the reference's objects are not copyable or
 *    movable, Solver.hpp:8-12); use one solver per host thread.
 *  - The device is selected by the "device" key of the "gb300" parameter
 *    object (the reference hard-codes device 0, GPUHybrid.cu:96).
 */
#ifndef LSS_H
#define LSS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum lss_status {
    LSS_OK = 0,
    LSS_ERR_INVALID_ARGUMENT = 1,
    LSS_ERR_CUDA = 2,
    LSS_ERR_OOM = 3,
    LSS_ERR_NOT_FACTORIZED = 4,
    LSS_ERR_NOT_SPD = 5,          /* a MAS or stiff block has a zero / non-finite pivot */
    LSS_ERR_NONFINITE = 6,        /* NaN or Inf in the matrix or right-hand side */
    LSS_ERR_INTERNAL = 7,
    LSS_ERR_BUFFER_TOO_SMALL = 8,
    LSS_ERR_NO_DEVICE = 9,
    LSS_ERR_UNSUPPORTED = 10
} lss_status;

typedef struct lss_solver lss_solver;

/* Human-readable name of a status code. */
const char *lss_status_string(lss_status s);

/* Last error message of `s`; with s == NULL, of the last failed lss_create on
 * this thread.  Valid until the next call on the same solver / thread. */
const char *lss_last_error(const lss_solver *s);

/* Solver::create(json) + GPUHybrid::GPUHybrid + set_parameters
 * (Solver.cpp:143-173, GPUHybrid.cu:79-179).  params_json: the polysolve
 * parameter object, e.g. {"solver": "GPUHybrid", "GPUHybrid": {...}} (the
 * alias "GPUHybridSolver" is accepted; keys of linear-solver-spec.json:646-747,
 * with that file's defaults), plus an optional "gb300" object for the
 * extensions (precision, composition, ...).  NULL or "" = all defaults. */
lss_status lss_create(const char *params_json, lss_solver **out);

/* GPUHybrid::~GPUHybrid (GPUHybrid.cu:1514-1533). */
lss_status lss_destroy(lss_solver *s);

/* GPUHybrid::set_parameters (GPUHybrid.cu:106-179). */
lss_status lss_set_parameters(lss_solver *s, const char *params_json);

/* GPUHybrid::get_info (GPUHybrid.cu:181-185): writes a JSON object with
 * "num_iterations" and "final_res_norm" (absolute ||b - A x||) plus extras.
 * *len receives the full length (excluding the NUL); returns
 * LSS_ERR_BUFFER_TOO_SMALL when cap <= *len. */
lss_status lss_get_info(const lss_solver *s, char *buf, size_t cap, size_t *len);

/* GPUHybrid::name (GPUHybrid.hpp:57-67): "GPUHybrid" / "GPUAMGF" / "GPUAMG". */
lss_status lss_name(const lss_solver *s, char *buf, size_t cap);

/* Solver::analyze_pattern (Solver.hpp:97; a no-op in GPUHybrid).  Here it
 * partitions the block graph, builds the permuted BSR layout and the MAS
 * coarse space once; factorize() with the same pattern reuses them. */
lss_status lss_analyze_pattern(lss_solver *s, int32_t n, int64_t nnz, const int32_t *outer,
                               const int32_t *inner);

/* GPUHybrid::factorize (GPUHybrid.cu:195-282): stiff-DOF selection,
 * subdomain post-processing, stiff-block factor, MAS setup.  Calls
 * analyze_pattern itself when the pattern is new. */
lss_status lss_factorize(lss_solver *s, int32_t n, int64_t nnz, const int32_t *outer,
                         const int32_t *inner, const double *values);

/* factorize with the values already in device memory (d_values[nnz] in the
 * storage order of the analysed pattern), ordered on `stream` (a cudaStream_t;
 * NULL = the solver's own stream).  Requires a previous analyze_pattern or
 * factorize with the same pattern.  For callers that assemble on the GPU. */
lss_status lss_factorize_device(lss_solver *s, const double *d_values, void *stream);

/* GPUHybrid::set_problematic_dofs (GPUHybrid.hpp:69): the DOF set used
 * when select_bad_dofs_from_l1_norm is false.  idx need not be sorted. */
lss_status lss_set_problematic_dofs(lss_solver *s, const int32_t *idx, int32_t count);

/* GPUHybrid::solve (GPUHybrid.cu:342-399): x is the initial guess on entry
 * (GPUHybrid.cu:347) and the solution on exit.  nrhs right-hand sides are
 * stored column by column with leading dimension ld (>= n); they are solved
 * one after the other.  Returns LSS_OK whether or not the tolerance was met
 * (as the reference); lss_get_info reports the stop reason. */
lss_status lss_solve(lss_solver *s, const double *b, double *x, int32_t nrhs, int64_t ld);

/* Same as lss_solve with device pointers (one right-hand side), ordered on
 * `stream` (a cudaStream_t; NULL = the solver's own stream, synchronised
 * before returning).  Used by the PyTorch extension. */
lss_status lss_solve_device(lss_solver *s, const double *d_b, double *d_x, void *stream);

/* Backward of x = A^-1 b (no counterpart in the reference): solves
 * A^T lambda = g with the same factorized hybrid preconditioner and PCG
 * (A is SPD so A^T = A), writing lambda; lambda is the initial guess. */
lss_status lss_solve_transpose(lss_solver *s, const double *g, double *lambda);

/* dL/dA on A's pattern (no counterpart in the reference):
 * dA_values[k] = -lambda[row(k)] * x[col(k)] for every stored entry k, with
 * row = outer index and col = inner index, in the input's storage order. */
lss_status lss_grad_A_pattern(lss_solver *s, const double *lambda, const double *x,
                              double *dA_values);
lss_status lss_grad_A_pattern_device(lss_solver *s, const double *d_lambda, const double *d_x,
                                     double *d_dA_values, void *stream);

/* Fused adjoint scatter to element parameters (no counterpart in the
 * reference): for a linear parameterisation A.values = M theta + c, with M^T
 * given in CSR (n_params rows; column indices are stored-entry indices of A in
 * the input storage order; values are d(A.values[v]) / d(theta[e])), writes
 * dtheta[e] = sum_v M[v][e] * (-lambda[row(v)] * x[col(v)]) -- the chain rule
 * of dL/dA_ij = -lambda_i x_j without forming dL/dA.  Device pointers. */
lss_status lss_grad_params_device(lss_solver *s, const double *d_lambda, const double *d_x, int32_t n_params,
                                  const int64_t *d_mt_rowptr, const int32_t *d_mt_cols,
                                  const double *d_mt_vals, double *d_dtheta, void *stream);

/* Forward of the same linear parameterisation (no counterpart in the
 * reference): d_values[v] = sum_e M[v][e] theta[e] + c[v] for the n_values
 * stored entries of A, with M in CSR (d_m_rowptr[n_values + 1], column = the
 * parameter e); d_c may be NULL.  Device pointers, ordered on `stream`. */
lss_status lss_assemble_values_device(int64_t n_values, const int64_t *d_m_rowptr, const int32_t *d_m_cols,
                                      const double *d_m_vals, const double *d_theta, const double *d_c,
                                      double *d_values, void *stream);

/* The selected stiff DOF set after post-processing (the union of the stiff
 * subdomains, ascending; GPUHybrid.cu:240-262 d_all_bad_dofs).  With
 * out == NULL only *count is written. */
lss_status lss_selected_dofs(const lss_solver *s, int32_t *out, int32_t cap, int32_t *count);

/* The GMM stage's raw selection {i : gamma0_i < gamma1_i} before filter /
 * expand / decompose (GPUHybrid.cu:859-879). */
lss_status lss_gmm_selection(const lss_solver *s, int32_t *out, int32_t cap, int32_t *count);

/* Stiff subdomains (GPUHybrid.cu:691-735 bad_indices_arrays): offsets[nsub+1]
 * into dofs[]; each subdomain ascending, subdomains ordered by first DOF. */
lss_status lss_subdomains(const lss_solver *s, int32_t *offsets, int32_t cap_offsets,
                          int32_t *dofs, int32_t cap_dofs, int32_t *nsub, int32_t *ndofs);

/* The partition behind the MAS preconditioner (MASSolver.cu:292-311):
 * perm[old block row] = new block row (size n / block_size) and
 * part_offsets[nparts+1] in the new numbering. */
lss_status lss_partition(const lss_solver *s, int32_t *perm, int32_t cap_perm,
                         int32_t *part_offsets, int32_t cap_offsets, int32_t *nparts);

/* The same partition computed from a pattern alone, on the host (no device
 * needed): the graph_partition step of MASSolverImpl::factorize
 * (MASSolver.cu:389-406 calling GraphPartition.cpp:176-289, KaMinPar with
 * k = ceil(n / 30) parts of at most 32 block rows) as this library does it.
 * threads <= 0: all host cores (the result does not depend on it).  With
 * perm == NULL or part_offsets == NULL only *nparts is written. */
lss_status lss_partition_pattern(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                 int32_t block_size, int32_t threads, int32_t *perm, int32_t cap_perm,
                                 int32_t *part_offsets, int32_t cap_offsets, int32_t *nparts);

/* The elimination tree of the multifrontal stiff-block factor for one stiff
 * subdomain, computed on the host (no device needed): the nested dissection
 * and front plan the solver builds for a subdomain above the dense size (the
 * reference's sparse LDL^T via cuDSS, GPUHybrid.cu:1075-1196 / 1248-1249).
 * dofs: ndofs ascending scalar DOF ids of the pattern (outer index = row).
 * out[0..3] = fronts, tree levels, largest front (variables), FMAs of the
 * numeric factorization. */
lss_status lss_stiff_elimination_tree(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                      int32_t block_size, const int32_t *dofs, int32_t ndofs, double *out);

/* The post-processing of a stiff-DOF selection as the solver runs it, on the
 * host (no device needed): filter_subdomains (GPUHybrid.cu:885-970; the
 * Gershgorin sums over the selected submatrix come from `values` here, the
 * solver forms them on the device), one-ring expansion (:972-991) and the
 * decomposition into connected components (:691-735), switched and sized by
 * the "GPUHybrid" parameters of params_json.  sel: nsel ascending scalar
 * ids (the GMM selection).  Output: the subdomains, each ascending, ordered by
 * their first DOF: sub_off[nsub + 1] into sub_dofs. */
lss_status lss_postprocess_selection(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                     const double *values, const char *params_json, const int32_t *sel,
                                     int32_t nsel, int32_t *sub_off, int32_t cap_off, int32_t *sub_dofs,
                                     int32_t cap_dofs, int32_t *nsub);

/* The MAS coarse space the solver builds for a pattern, on the host (no
 * device needed): MASPreconditioner.cu:376-481 semantics on the partition
 * of lss_partition_pattern.  *levels = matrix levels including level 0;
 * items[l] (cap_items >= *levels) = nodes (l = 0) or coarse items of level l;
 * cmap[(l - 1) * nb + i] (cap_cmap >= (*levels - 1) * nb) = the level-l item
 * of permuted block row i.  With items == NULL or cmap == NULL only *levels
 * is written. */
lss_status lss_coarse_space(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner, int32_t block_size,
                            int32_t max_coarse_levels, int32_t *levels, int32_t *items, int32_t cap_items,
                            int32_t *cmap, int64_t cap_cmap);

/* The full plan behind lss_stiff_elimination_tree, for checking it: call
 * with the arrays NULL to get counts[0..3] = fronts, positions, boundary
 * entries, child entries; then with arrays of those sizes.  Fronts in
 * postorder (children first): front f owns positions front_p0[f] ..
 * + front_s[f] - 1 and couples to the later positions bnd_pos[bnd_off[f] ..
 * bnd_off[f+1]) (ascending, front_u[f] of them); its children are
 * child[child_off[f] .. child_off[f+1]); pos2j[p] = the index into dofs of
 * position p. */
lss_status lss_stiff_elimination_plan(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                      int32_t block_size, const int32_t *dofs, int32_t ndofs, int64_t *counts,
                                      int32_t *front_p0, int32_t *front_s, int32_t *front_u, int32_t *bnd_off,
                                      int32_t *bnd_pos, int32_t *child_off, int32_t *child, int32_t *pos2j);

/* ---- operator-level entry points (parity tests and benchmarks) ---------- */

/* rn[i] = sum |values| of outer slice i, on the GPU (GPUHybrid.cu:753-765). */
lss_status lss_op_row_l1_norms(int32_t n, int64_t nnz, const int32_t *outer,
                               const double *values, double *rn);

/* y = A x with the factorized FP64 operator (original ordering). */
lss_status lss_op_spmv(lss_solver *s, const double *x, double *y);

/* Per scalar row of the permuted operator (partition order): |diagonal|,
 * max |off-diagonal| and the l1 norm -- the scores of MASSolver's bad-DOF
 * selections (BadDOFPreconditioner.cu:110-145, BadDofKMeanPreconditioner.cu:
 * 187-226, BadDofGMMPreconditioner.cu:285-310).  Arrays of n. */
lss_status lss_op_row_scores(lss_solver *s, double *diag_abs, double *offdiag_max, double *l1);

/* MASSolver's bad-DOF selection on host scores (the solver applies it with
 * "gb300": {"bad_dof_strategy": ...}): strategy 1 elbow on |diagonal|
 * (BadDOFPreconditioner.cu:61-100); 2 k-means with p1 = search fraction,
 * p2 = jump threshold, i1 = max iterations, i2 = expand neighbours
 * (BadDofKMeanPreconditioner.cu:63-172); 3 GMM with p1 = jump threshold,
 * p2 = tol, i1 = max iterations, i2 = expand neighbours
 * (BadDofGMMPreconditioner.cu:73-255).  Writes the selected positions in the
 * reference's output order to out (capacity n; may be NULL) and their number
 * to count. */
lss_status lss_op_select_bad_dofs(int32_t strategy, int32_t n, const double *score, double p1, double p2,
                                  int32_t i1, int32_t i2, int32_t *out, int32_t *count);

/* y = A x with the PCG's own operator product (the A p of pcg_solve,
 * GPUHybrid.cu:1458): FP64, or double-float on the FP32 pipe when
 * gb300.outer_spmv resolves to "df32". */
lss_status lss_op_spmv_outer(lss_solver *s, const double *x, double *y);

/* z = MAS^-1 r alone (MASPreconditioner::apply, MASPreconditioner.cu:1099). */
lss_status lss_op_mas_apply(lss_solver *s, const double *r, double *z);

/* z = M^-1 r, the full hybrid preconditioner (GPUHybrid.cu:521-542 with
 * MAS in place of BoomerAMG). */
lss_status lss_op_precond(lss_solver *s, const double *r, double *z);

/* Time `reps` launches of one kernel family on device-resident operands:
 * kind 0 = FP64 SpMV, 1 = MAS apply, 2 = full preconditioner, 3 = one PCG
 * iteration, 4 = the level-0 bank SYMV kernel of MAS alone, 5 = the residual
 * SpMV inside the preconditioner (FP32 operator in mixed precision), 6 = the
 * PCG's own A p with p.Ap (FP64, or double-float on the FP32 pipe when
 * gb300.outer_spmv resolves to "df32").  Writes the mean milliseconds per
 * launch (CUDA events on the solver's stream) and the algorithmic bytes of
 * one launch. */
lss_status lss_op_time(lss_solver *s, int32_t kind, int32_t reps, double *ms_per_launch,
                       double *bytes_per_launch);

/* Cap device allocations of solvers created afterwards (bytes, 0 = none):
 * exercises the out-of-memory path without exhausting the GPU. */
lss_status lss_set_memory_cap(size_t bytes);

/* ---- batched solves -------------------------------------------------------- */

/* Solve many independent systems, each with nrhs right-hand sides, at once
 * (no single counterpart in the reference, which solves one system per call:
 * this is its GPUHybrid::solve, GPUHybrid.cu:342-399, for every system and
 * right-hand side).  solvers[s] is a factorized solver of system s (distinct
 * objects); d_b[s] and d_x[s] are device arrays of n_s x nrhs (column-major,
 * leading dimension n_s); x is the initial guess on entry, as in lss_solve.
 * Host threads (threads <= 0: one per system) each drive one system's PCG on
 * that solver's own stream, so the GPU overlaps the systems; every system and
 * right-hand side converges on its own scalars and stop flag.
 * iterations (optional, count x nrhs): iterations per solve.  Returns the
 * first failing system's status (lss_last_error(NULL) names it); the other
 * systems still run. */
lss_status lss_solve_batched_device(lss_solver *const *solvers, int32_t count, const double *const *d_b,
                                    double *const *d_x, int32_t nrhs, int32_t threads, int32_t *iterations);

/* lss_factorize_device for every system s (values d_values[s], the layout of
 * that solver's analysed pattern), from the same host-thread pool. */
lss_status lss_factorize_batched_device(lss_solver *const *solvers, int32_t count, const double *const *d_values,
                                        int32_t threads);

/* ---- batched PCG: one launch per step over all systems and right-hand sides */

/* Number of right-hand sides per system of a batch (pad with zero columns:
 * a zero right-hand side gives x = 0 after 0 iterations, GPUHybrid.cu:1428-1439). */
#define LSS_BATCH_RHS 16

typedef struct lss_batch lss_batch;

/* No single counterpart in the reference, which solves one system per call
 * (GPUHybrid::solve, GPUHybrid.cu:342-399).  A batch groups `count` solvers
 * (distinct objects on one device; block size 3, "gb300": {"precision":
 * "mixed"}, the GPUHybrid selection and the multiplicative composition).
 * Each batched step runs the reference's PCG (GPUHybrid.cu:1413-1512) for
 * every (system, right-hand side) lane -- own alpha, beta, gamma and stopping
 * test -- with every kernel launch covering all systems and LSS_BATCH_RHS
 * right-hand sides: each matrix, MAS inverse and stiff factor is read once per
 * iteration for all of them.  The PCG vectors are double-float (FP32 pairs,
 * about 2^-48 relative), the lane scalars and the final residual FP64.  The
 * solvers stay owned by the caller and must outlive the batch. */
lss_status lss_batch_create(lss_solver *const *solvers, int32_t count, lss_batch **out);
lss_status lss_batch_destroy(lss_batch *b);
/* Last error of `b` (NULL: of the last failed lss_batch_create on this thread). */
const char *lss_batch_last_error(const lss_batch *b);

/* GPUHybrid::factorize (GPUHybrid.cu:195-282) of every system from device
 * values (d_values[s]: the storage order of solver s's analysed pattern), on a
 * pool of host threads (threads <= 0: one per system), then the merge into the
 * batch's device image. */
lss_status lss_batch_factorize_device(lss_batch *b, const double *const *d_values, int32_t threads);

/* Solve: d_b[s] and d_x[s] are device arrays of n_s x LSS_BATCH_RHS,
 * column-major (leading dimension n_s); x is the initial guess on entry.
 * iterations (optional, count x LSS_BATCH_RHS): PCG iterations per lane. */
lss_status lss_batch_solve_device(lss_batch *b, const double *const *d_b, double *const *d_x,
                                  int32_t *iterations);

/* JSON: lanes' iteration statistics, timings, kernels per graph chunk. */
lss_status lss_batch_get_info(const lss_batch *b, char *buf, size_t cap, size_t *len);

/* ---- allocation-free entry point ----------------------------------------- */

/* Largest n accepted by lss_gmm_select_device_noalloc. */
#define LSS_NOALLOC_MAX_ROWS (1 << 20)

/* No counterpart in the reference: an allocation-free form of the selection
 * that lss_gmm_selection reports (l1 row norms GPUHybrid.cu:753-765, GMM
 * GPUHybrid.cu:767-879), for callers that cannot allocate (pre-reserved
 * memory, allocator-free contexts).  Same kernels, same result: the selected
 * rows, ascending, bit-identical to lss_gmm_selection of a solver factorized
 * with the same matrix and GMM parameters.
 *   - n <= LSS_NOALLOC_MAX_ROWS, else LSS_ERR_INVALID_ARGUMENT before any
 *     device work;
 *   - d_outer[n+1], d_values[nnz]: device arrays of the matrix (CSC, or CSR:
 *     the matrix is symmetric); d_selected[n] receives the rows, d_count[1]
 *     their number; all on the current device;
 *   - stream: a cudaStream_t of the current device (NULL = legacy default).
 * Allocates nothing: every intermediate lives in one static device scratch
 * area of 8,716,800 bytes inside liblss.so.  Every call looks the scratch
 * address up in the current context (cudaGetSymbolAddress, which allocates
 * nothing, so the address stays valid across cudaDeviceReset); the first call
 * on a device, or the first after a reset, can load the module: make it
 * before any stream capture.  Calls share the scratch, so
 * calls that can overlap (other streams or threads) race and must be
 * serialised by the caller.  Only the scratch's grid-reduction arrival counter
 * must start at zero: it is zero at module load and every reduction leaves it
 * at zero.  Stream-ordered; no host synchronisation. */
lss_status lss_gmm_select_device_noalloc(int32_t n, int64_t nnz, const int32_t *d_outer,
                                         const double *d_values, double gmm_jump_threshold,
                                         double gmm_tol, int32_t max_gmm_iterations,
                                         int32_t *d_selected, int32_t *d_count, void *stream);

#ifdef __cplusplus
}
#endif
#endif
