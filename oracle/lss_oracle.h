/*
 * lss_oracle.h -- CPU restatement of the reference's GPU hybrid solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is what the GPU path is compared
 * against: tests, the smoke entry point and the CPU-baseline leg of the
 * benchmark may call it; the product (the CUDA library) never links or calls
 * it.
 *
 * Parity status: UNPINNED.  The reference (geometryprocessing/local-stiff-solver)
 * ships no golden vectors or known-answer tests for this path, and its code
 * cannot be compiled here (hypre, cuDSS, Eigen, MPI, KaMinPar are absent).
 * Every function below restates the cited reference code; a second, independent
 * numpy restatement (oracle/oracle.py) cross-checks the selection pipeline.
 *
 * Conventions: the input matrix is Eigen-style compressed column storage
 * (StiffnessMatrix, src/polysolve/Types.hpp:11-15) with int32 indices.  Like the
 * reference (GPUHybrid.cu:203-209, "outer/inner" handed to hypre as CSR), the
 * outer index is treated as the row: "row i" means the entries stored in
 * outer slice i.  For a symmetric matrix this is the same thing.
 */
#ifndef LSS_ORACLE_H
#define LSS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- selection: GPUHybrid.cu:737-883 ---------------------------------- */

typedef struct {
    double global_mean, global_var;
    double mean0, mean1, var0, var1, w0, w1;
    double min_log_margin; /* min_i |log g0_i - log g1_i| of the final E-step */
    int32_t gmm_iters;     /* value of the loop counter at exit (reference log) */
    int32_t estep_count;   /* number of E-steps executed */
    int32_t jump_passed;   /* |mean1|/|mean0| > threshold */
    int32_t num_selected;
} lsso_gmm_stats;

/* rn[i] = sum_{k in outer slice i} |values[k]|   (GPUHybrid.cu:753-765) */
void lsso_row_l1_norms(int32_t n, const int32_t *outer, const double *values, double *rn);

/* Two-component 1D GMM by EM on rn and the jump test; writes the ascending
 * index set {i : gamma0_i < gamma1_i} to sel (capacity n), returns its size.
 * (GPUHybrid.cu:767-879; formulas identical to Hybrid.cpp:850-949.) */
int32_t lsso_gmm_select(int32_t n, const double *rn, double jump_threshold, double tol,
                        int32_t max_iterations, int32_t *sel, lsso_gmm_stats *stats);

/* filter_subdomains (GPUHybrid.cu:885-970): connected components of the
 * selected set in A's pattern; drop components outside [min_size, max_size];
 * keep a component only if its Gershgorin bounds give lmin*lmax < 0 or
 * lmax/lmin > cond_threshold.  sel must be ascending; out (capacity nsel) gets
 * the kept set, ascending.  counters[3] = {too_small, too_large, not_poorly_conditioned}. */
int32_t lsso_filter_subdomains(int32_t n, const int32_t *outer, const int32_t *inner,
                               const double *values, const int32_t *sel, int32_t nsel,
                               int32_t min_size, int32_t max_size, double cond_threshold,
                               int32_t *out, int32_t *counters);

/* expand_subdomains_to_strongly_connected (GPUHybrid.cu:972-991): every index
 * stored in the outer slices of the selected set.  out capacity n, ascending. */
int32_t lsso_expand_subdomains(int32_t n, const int32_t *outer, const int32_t *inner,
                               const int32_t *sel, int32_t nsel, int32_t *out);

/* decompose_subdomains_to_disjoint_subsets (GPUHybrid.cu:691-735): connected
 * components of the selected set, dropping those larger than max_size.
 * The reference's component order is unspecified (unordered_map); here the
 * components are ordered by their smallest index, each one ascending.
 * offsets has capacity nsel+1, dofs capacity nsel.  Returns #components. */
int32_t lsso_decompose_subdomains(int32_t n, const int32_t *outer, const int32_t *inner,
                                  const int32_t *sel, int32_t nsel, int32_t max_size,
                                  int32_t *offsets, int32_t *dofs);

/* ---- MAS preconditioner: MASPreconditioner.cu:376-1164 -------------------- */

/* Block CSR in partition order: nb block rows, bd x bd row-major blocks,
 * part_offsets[nparts+1] (each part <= 32 block rows).  Matches the input of
 * MASPreconditioner::factorize (MASPreconditioner.hpp:79). */
typedef struct lsso_mas lsso_mas;
lsso_mas *lsso_mas_create(int32_t nb, int32_t bd, const int32_t *rows, const int32_t *cols,
                          const double *vals, int32_t nparts, const int32_t *part_offsets,
                          int32_t max_coarse_levels, int32_t *status);
void lsso_mas_apply(const lsso_mas *m, const double *r, double *z);
int32_t lsso_mas_level_count(const lsso_mas *m);            /* matrix levels incl. level 0 */
int32_t lsso_mas_level_items(const lsso_mas *m, int32_t l);  /* nodes (l=0) or CCOs */
/* coarse map of level l (1..level_count-1): coarse id of every block row, size nb */
void lsso_mas_coarse_map(const lsso_mas *m, int32_t l, int32_t *out);
void lsso_mas_destroy(lsso_mas *m);

/* ---- the full CPU method ---------------------------------------------------- */

typedef struct {
    int32_t max_iter;
    double rel_tol, abs_tol;
    int32_t block_size;
    int32_t do_hybrid;           /* do_hybrid_precond */
    int32_t select_from_l1;      /* select_bad_dofs_from_l1_norm */
    double jump_threshold, gmm_tol;
    int32_t max_gmm_iterations;
    double cond_threshold;
    int32_t decompose, min_sub, max_sub, expand;
    int32_t max_coarse_levels;
    int32_t threads;             /* OpenMP threads, <=0: default */
    int32_t additive;            /* 1: z = M r + S^T A_SS^-1 S r (MASSolver.cu:583-615) */
    double mas_omega;            /* damping of MAS in the multiplicative form; <= 0: auto */
    int32_t omega_iters;         /* PCG-Lanczos steps of the automatic estimate */
    double omega_factor;         /* omega = omega_factor / lambda_max(M A) */
    int32_t greedy_partition;    /* 1: the oracle's greedy partition; 0: the library's bisection */
} lsso_params;

void lsso_default_params(lsso_params *p);
size_t lsso_params_size(void); /* sizeof(lsso_params), checked by the Python binding */

typedef struct lsso_solver lsso_solver;
/* Sets up selection + post-processing + partition + MAS + stiff factors.
 * perm (block old->new) and part_offsets are optional: when NULL the oracle
 * partitions the block graph itself (greedy BFS region growing). */
lsso_solver *lsso_solver_create(int32_t n, const int32_t *outer, const int32_t *inner,
                                const double *values, const lsso_params *p,
                                const int32_t *perm, int32_t nparts,
                                const int32_t *part_offsets, int32_t *status);
/* PCG (GPUHybrid.cu:1413-1512); x is the initial guess on entry. */
int32_t lsso_solver_solve(lsso_solver *s, const double *b, double *x, int32_t *iterations,
                          double *final_res_norm);
int32_t lsso_solver_num_stiff(const lsso_solver *s);
double lsso_solver_omega(const lsso_solver *s);
void lsso_solver_set_max_iter(lsso_solver *s, int32_t max_iter);
double lsso_solver_lambda_max(const lsso_solver *s);

/* Largest eigenvalue of the symmetric tridiagonal with diagonal d[0..k) and
 * off-diagonal e[0..k-1) (bisection on Sturm counts). */
double lsso_tridiag_max_eig(int32_t k, const double *d, const double *e);

/* The deterministic probe vector of the lambda_max estimate:
 * v_i = ((i * 2654435761) mod 2^32) / 2^32 - 0.5, i in the original ordering. */
void lsso_probe_vector(int32_t n, double *v);
int32_t lsso_solver_num_subdomains(const lsso_solver *s);
/* Apply the hybrid preconditioner once (z = M^-1 r, original ordering). */
void lsso_solver_precond(lsso_solver *s, const double *r, double *z);
void lsso_solver_destroy(lsso_solver *s);

/* the library's partition restated (recursive breadth-first bisection,
 * k = ceil(m / 30) parts of <= 32 block rows, uncoupled rows last):
 * perm[old] = new, part_offsets[nparts + 1] (capacity nb + 1); returns nparts */
int32_t lsso_bisect_partition(int32_t nb, const int32_t *rows, const int32_t *cols, int32_t *perm,
                              int32_t *part_offsets);

/* the oracle's own partition: part id per block row of a CSR block graph */
int32_t lsso_greedy_partition(int32_t nb, const int32_t *rows, const int32_t *cols,
                              int32_t max_part, int32_t *part_of);

/* ---- MAS-side bad-DOF selections (MASSolver use_bad_dof_precond) ----------
 * Scores are per scalar row in the partition order of the permuted operator;
 * the results are positions in that order (not sorted: the reference's own
 * output order).  Sorting ties break by position. */

/* Elbow of the ascending log|diag| curve against its chord: the positions from
 * the largest deviation on (BadDOFPreconditioner.cu:61-100). */
int32_t lsso_mas_select_elbow(int32_t n, const double *diag_abs, int32_t *out);

/* 2-means (Lloyd) on the search_fraction largest max|off-diagonal| scores, the
 * centroid ratio test, positions above the midpoint, each widened by
 * +-expand_neighbors positions (BadDofKMeanPreconditioner.cu:63-172). */
int32_t lsso_mas_select_kmean(int32_t n, const double *offdiag_max, double search_fraction,
                              double jump_threshold, int32_t max_iterations, int32_t expand_neighbors,
                              int32_t *out);

/* Two-component GMM by EM on l1 row norms, the high/low mean ratio test,
 * positions of the high component, each widened by +-expand_neighbors
 * (BadDofGMMPreconditioner.cu:73-255). */
int32_t lsso_mas_select_gmm(int32_t n, const double *l1, double jump_threshold, double tol,
                            int32_t max_iterations, int32_t expand_neighbors, int32_t *out);

#ifdef __cplusplus
}
#endif
#endif
