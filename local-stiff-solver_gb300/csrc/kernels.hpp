// Device data views and kernel launchers of the GB300 hybrid solver.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lss_common.hpp"

namespace lss {

constexpr int RED_MAX_VALUES = 8;  // values per grid reduction
constexpr int GRID_MAX = 4096;     // CTAs of any reducing kernel at most (size of the reduction partials)

// CTAs for `per_sm` resident CTAs on every SM of the current device (the SM
// count is queried once per device), capped at GRID_MAX.
int sm_grid(int per_sm);

// Raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes` (never lowers it): solvers driven from several host threads
// set different sizes for the same kernel, and a lower value set by one
// would make another's launch invalid.
void raise_smem_limit(const void *kernel, size_t bytes);

// Scratch of the deterministic grid reductions (device memory, counter zeroed once).
struct GridReduce {
    double *partials = nullptr;  // GRID_MAX * RED_MAX_VALUES
    unsigned *counter = nullptr; // one arrival counter
};

inline int grid_for(long long work_items, int items_per_cta, int max_ctas)
{
    long long g = (work_items + items_per_cta - 1) / items_per_cta;
    if (g < 1) g = 1;
    if (g > max_ctas) g = max_ctas;
    return (int)g;
}

// ---------------------------------------------------------------- selection
struct GmmState {
    double sum, mean, var, mn, mx;
    double m0, m1, v0, v1, w0, w1;        // current parameters
    double em0, em1, ev0, ev1, ew0, ew1;  // parameters of the last E-step
    double s0, s1;                        // responsibilities' sums of the last E-step
    int esteps, converged, pad0, pad1;
};

void launch_row_l1_norms(int32_t n, int64_t nnz, const int32_t *outer, const double *vals, double *rn,
                         cudaStream_t s);
void launch_gmm(int32_t n, const double *rn, GmmState *st, int max_iterations, double tol, GridReduce gr,
                cudaStream_t s);
void launch_gmm_mark(int32_t n, const double *rn, const GmmState *st, double threshold, int32_t *block_count,
                     double *block_margin, cudaStream_t s);
void launch_gmm_scatter(int32_t n, const double *rn, const GmmState *st, double threshold,
                        const int32_t *block_offset, int32_t *out, cudaStream_t s);

// Gershgorin data of the selected rows (filter_subdomains, GPUHybrid.cu:936-958):
// for every selected original row k, diag = A_kk and off = sum of |A_kj| over
// selected j != k, read from the permuted operator.  sel: original scalar ids.
void launch_gershgorin(int nb, int bd, const int32_t *rows, const int32_t *cols, const double *vals,
                       const int32_t *perm, const int32_t *sel, int32_t nsel, uint8_t *mask, double *diag,
                       double *off, cudaStream_t s);

// ---------------------------------------------------------------- operator
struct BsrDev {
    int32_t nb = 0, bd = 1;
    int lanes = 4;                 // threads per block row of the FP64 SpMV (autotuned)
    int lanes32 = 4;               // threads per block row of the FP32 residual SpMV (autotuned)
    const int32_t *rows = nullptr;
    const int32_t *cols = nullptr;
    const double *vals = nullptr;  // row-sliced layout (spmv.cuh)
    const float *vals32 = nullptr; // FP32 copy (mixed precision preconditioner)
    const float2 *vals_df = nullptr; // df32 pairs (hi, lo): vals = hi + lo to 2^-48 relative
};

// per scalar row of the permuted operator: |diagonal|, max |off-diagonal|, l1 norm
void launch_row_scores(const BsrDev &A, double *diag, double *offmax, double *l1, cudaStream_t s);

// vals[j] = src >= 0 ? csc[src] : 0  (BSR slot gather)
void launch_gather_values(int64_t count, const int64_t *src, const double *csc, double *vals, float *vals32,
                          cudaStream_t s, float2 *vals_df = nullptr);
// y = A x  (FP64)
void launch_spmv(const BsrDev &A, const double *x, double *y, const int *done, cudaStream_t s);
// y = r - A x in FP64
void launch_residual_spmv(const BsrDev &A, const double *r, const double *x, double *y, const int *done,
                          cudaStream_t s);
// y32 = r32 - A x32 in FP32 with the FP32 operator copy (the mixed
// preconditioner's residual); block rows flagged in `precise` (optional) are
// evaluated in double-float from r64, the df32 values and x32 + x_lo.
void launch_residual32(const BsrDev &A, const float *r32, const float *x32, float *y32, const int *done,
                       cudaStream_t s, const uint8_t *precise = nullptr, const double *r64 = nullptr,
                       const float *x_lo = nullptr);

// ---------------------------------------------------------------- PCG
enum StopReason : int {
    STOP_RUNNING = 0,
    STOP_CONVERGED_REL = 1,
    STOP_CONVERGED_ABS = 2,
    STOP_ZERO_PAP = 3,
    STOP_NEGATIVE_ALPHA = 4,
    STOP_SUBNORMAL_ALPHA = 5,
    STOP_MAX_ITER = 6,
    STOP_NONFINITE = 7,
};

constexpr int PCG_HIST = 64;  // alpha / beta history kept for the Lanczos estimate

struct PcgState {
    double bb, gamma, alpha, beta, pAp, rr, rel_eps, abs_eps;
    int iter, done, max_iter, pad;
    double hist_alpha[PCG_HIST], hist_beta[PCG_HIST];
};

void launch_dot(int64_t n, const double *a, const double *b, double *out, GridReduce gr, cudaStream_t s);
// Ap = A p; pAp = p.Ap; alpha = gamma / pAp with the reference's breakdown tests
void launch_pcg_spmv_alpha(const BsrDev &A, const double *p, double *Ap, PcgState *st, GridReduce gr,
                           cudaStream_t s);
// x += alpha p; r -= alpha Ap; rr = r.r; convergence tests
// r32 (optional): also r rounded to FP32
void launch_pcg_update_xr(int64_t n, double *x, double *r, const double *p, const double *Ap, PcgState *st,
                          GridReduce gr, cudaStream_t s, float *r32 = nullptr);
// the same with A p as df32 (hi, lo) pairs
void launch_pcg_update_xr_df(int64_t n, double *x, double *r, const double *p, const float2 *Ap_df, PcgState *st,
                             GridReduce gr, cudaStream_t s, float *r32 = nullptr);
void launch_df_to_double(int64_t n, const float2 *src, double *dst, cudaStream_t s);
// the damping estimate's probe, v_i = ((i * 2654435761) mod 2^32) / 2^32 - 0.5 over
// original indices i, written in the permuted order
void launch_probe(int64_t nb, int bd, const int32_t *perm, double *dst, cudaStream_t s);
// p = z + beta p
// p_df (optional): the df32 split of the new p, the x operand of the df32 SpMV
void launch_pcg_update_p(int64_t n, double *p, const double *z, const PcgState *st, cudaStream_t s,
                         float2 *p_df = nullptr);
// dst = (fl32(src), fl32(src - fl32(src)))
void launch_split(int64_t n, const double *src, float2 *dst, cudaStream_t s);
// Ap = A p, p.Ap and alpha like launch_pcg_spmv_alpha, with the products and
// row sums in double-float arithmetic on the FP32 pipe: A and p as (hi, lo)
// FP32 pairs (both to 2^-48 relative), error-free products and sums
// (TwoProd / TwoSum), the result rounded to FP64 once per row component.
void launch_pcg_spmv_alpha_df(const BsrDev &A, const float2 *p_df, float2 *Ap_df, PcgState *st, GridReduce gr,
                              cudaStream_t s);
void launch_copy(int64_t n, const double *src, double *dst, const int *done, cudaStream_t s);
void launch_permute(int64_t nb, int bd, const int32_t *perm, const double *src, double *dst, bool to_new,
                    cudaStream_t s);
void launch_grad_pattern(int32_t n, const int32_t *outer, const int32_t *inner, const double *lambda,
                         const double *x, double *dA, cudaStream_t s);
// dtheta[e] = sum_k Mt_vals[k] * (-lambda[row(v)] * x[inner[v]]), v = Mt_cols[k], over the CSR row e of Mt
void launch_grad_params(int32_t nparams, const int64_t *mt_rowptr, const int32_t *mt_cols, const double *mt_vals,
                        const int32_t *row_of, const int32_t *inner, const double *lambda, const double *x,
                        double *dtheta, cudaStream_t s);
void launch_row_of(int32_t n, const int32_t *outer, int32_t *row_of, cudaStream_t s);
// out[v] = sum_k mvals[k] theta[mcols[k]] over CSR row v (+ c[v], c optional)
void launch_assemble_values(int64_t nvals, const int64_t *rowptr, const int32_t *mcols, const double *mvals,
                            const double *theta, const double *c, double *out, cudaStream_t s);

// ---------------------------------------------------------------- MAS
constexpr int MAS_MAXL = 7;

struct MasDev {
    int L = 1, bd = 1;
    int32_t nb = 0, nparts = 0;
    const int32_t *part_off = nullptr;  // nparts+1
    const uint8_t *key0 = nullptr;      // per node: local level-1 aggregate id inside its part
    const int32_t *cbase0 = nullptr;    // per part: first level-1 item
    const uint8_t *ccnt0 = nullptr;     // per part: number of level-1 items
    int32_t nitems[MAS_MAXL] = {};      // level l >= 1 items
    int32_t nbanks[MAS_MAXL] = {};      // level l banks (level 0: nparts)
    int64_t voff[MAS_MAXL] = {};        // l >= 1: element offset of level-l vectors
    int32_t boff[MAS_MAXL] = {};        // l >= 1: first coarse bank of level l
    const uint8_t *key[MAS_MAXL] = {};  // l >= 1: per item local aggregate id at level l+1
    const int32_t *cbase[MAS_MAXL] = {};
    const uint8_t *ccnt[MAS_MAXL] = {};
    int32_t ncoarse = 0;                // total coarse banks
    int64_t tile_elems = 0;             // inverse elements per bank
    int64_t bank_bytes0 = 0;            // > 0: level-0 banks hold FP32 diagonal and BF16 off-diagonal tiles, this stride
    int64_t level_elems = 0;            // elements of the level-vector buffers
};

int64_t mas_tile_elems(int bd);

// Galerkin assembly into per-bank dense N x N FP64 staging (N = 32 bd)
void launch_mas_assemble0(const BsrDev &A, const int32_t *part_of, const int32_t *part_off, double *stage,
                          cudaStream_t s);
// members of the coarse items in chunks (CoarseSpace::memb_rows,
// item_chunk, chunk_r0), device copies; items are numbered flat over levels
// 1..L-1
struct CoarseMembers {
    const int32_t *rows = nullptr;
    const int32_t *item_chunk = nullptr;  // nitem + 1
    const int32_t *chunk_r0 = nullptr;    // nchunk + 1
    int64_t nitem = 0, nchunk = 0;
};
// partial: nchunk * bd * bd * 32 doubles of scratch
void launch_mas_assemble_coarse(const BsrDev &A, const MasDev &m, const int32_t *cmap /* nb*(L-1) */,
                                const CoarseMembers &mb, double *partial, double *stage, cudaStream_t s);
// pad zero diagonals, invert (symmetric sweep), write bank tiles (FP32 or FP64)
void launch_mas_invert(int bd, int64_t nbanks, const double *stage, void *out, bool fp32, int *bad,
                       cudaStream_t s, bool bf16_offdiag = false);
// bytes of one bank with FP32 diagonal and BF16 off-diagonal tiles
int64_t mas_bank_bytes_bf16(int bd);
// z = MAS^-1 xin (acc: z += MAS^-1 xin).  dot_mode 1: st->gamma = rdot.z;
// dot_mode 2: st->beta = rdot.z / st->gamma, st->gamma = rdot.z.
// z = scale * MAS^-1 xin, or z += scale * MAS^-1 xin with acc.
// z32 (optional): also store z rounded to FP32 (the input of the FP32 residual)
// and, with z_lo, the remainder z - z32 rounded to FP32.
// xin32 (optional, FP32 MAS only): an FP32 input used in place of xin.
void launch_mas_apply(const MasDev &m, const void *inv0, const void *invc, void *v, void *u, bool fp32,
                      const double *xin, double *z, bool acc, double scale, const double *rdot, PcgState *st,
                      int dot_mode, GridReduce gr, const int *done, cudaStream_t s, float *z32 = nullptr,
                      const float *xin32 = nullptr, float *z_lo = nullptr);

// level-0 bank SYMV alone (z = Inv_0 xin + coarse correction already in u), for timing
void launch_mas_level0(const MasDev &m, const void *inv0, const void *u, bool fp32, const double *xin, double *z,
                       cudaStream_t s);

// ---------------------------------------------------------------- stiff blocks
struct StiffDev {
    int32_t nsub = 0, ndof = 0;
    int32_t ndof_dense = 0;            // DOFs j < ndof_dense belong to subdomains with a dense inverse
                                       // (the rest to the multifrontal factor, multifrontal.hpp)
    const int32_t *dofs = nullptr;     // ndof permuted scalar ids, grouped by subdomain
    const int32_t *sub_of = nullptr;   // ndof
    const int32_t *off = nullptr;      // nsub+1 (into dofs)
    const int64_t *inv_off = nullptr;  // nsub (into inverse storage)
    const double *inv = nullptr;       // row-major m x m per subdomain
    const float *inv32 = nullptr;
    double *t = nullptr;               // ndof scratch
};

void launch_stiff_extract(const BsrDev &A, const StiffDev &S, double *stage, cudaStream_t s);
// dense inverses of the subdomains 0 .. nsub-1 (each at most STIFF_DENSE_MAX DOFs)
constexpr int STIFF_DENSE_MAX = 160;
void launch_stiff_invert(const StiffDev &S, const int32_t *h_off, int32_t nsub, double *inv, int *bad,
                         cudaStream_t s);
void launch_stiff_to_fp32(int64_t count, const double *src, float *dst, cudaStream_t s);
// t = r_S - (A z)_S   (residual = true) or t = r_S
void launch_stiff_gather(const BsrDev &A, const StiffDev &S, const double *r, const double *z, bool residual,
                         const int *done, cudaStream_t s);
// z_S += Inv t over the subdomains with a dense inverse
// z32, z_lo (optional): FP32 shadow of z and its remainder, updated at the
// DOFs the correction changes
void launch_stiff_apply(const StiffDev &S, bool fp32, double *z, const int *done, cudaStream_t s,
                        float *z32 = nullptr, float *z_lo = nullptr);

}  // namespace lss
