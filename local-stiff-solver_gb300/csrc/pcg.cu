// Operator and PCG kernels (sm_103a): FP64 BSR/CSR SpMV with fused epilogues,
// PCG vector updates with deterministic fused reductions, permutation and
// the pattern-restricted gradient of the adjoint.
//
// PCG follows GPUHybrid::pcg_solve (GPUHybrid.cu:1413-1512): recurrence
// residual, relative test rr / bb < rel_tol^2 and absolute test rr < abs_tol^2
// every iteration, breakdown stops on p.Ap == 0, alpha <= 0 and subnormal
// alpha.  The scalars live on the device; every kernel of an iteration
// returns immediately once st->done is set, so the host only polls the flag
// every few iterations (the reference synchronises on every dot product).
#include <cfloat>

#include "device_common.cuh"
#include "kernels.hpp"
#include "spmv.cuh"

namespace lss {
namespace {

__global__ void gather_values_kernel(int64_t count, const int64_t *__restrict__ src, const double *__restrict__ csc,
                                     double *__restrict__ vals, float *__restrict__ vals32,
                                     float2 *__restrict__ vals_df)
{
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < count;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = src[j];
        const double v = k >= 0 ? csc[k] : 0.0;
        vals[j] = v;
        if (vals32) vals32[j] = (float)v;
        if (vals_df) {
            const float h = (float)v;
            vals_df[j] = make_float2(h, (float)(v - (double)h));
        }
    }
}

// y = A x
template <int BD, int LANES>
__global__ void __launch_bounds__(256) spmv_kernel(BsrDev A, const double *__restrict__ x, double *__restrict__ y,
                                                   const int *done)
{
    if (done && *done) return;
    const int lane = threadIdx.x % LANES;
    constexpr int RPW = 32 / LANES;  // block rows per warp and sweep
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // warp-uniform trip count: every lane reaches the group shuffles together
    for (int64_t wr = w0 * RPW; wr < A.nb; wr += nw * RPW) {
        const int64_t i = wr + (threadIdx.x & 31) / LANES;
        const bool valid = i < A.nb;
        double acc[BD];
        bsr_block_row<BD, LANES, double, double, double>(A.rows, A.cols, A.vals, (int32_t)i, valid, x, lane, acc);
        // lane l of the group stores the components k with k % LANES == l
        // (all BD of them when LANES == 1)
        if (valid) {
#pragma unroll
            for (int k = 0; k < BD; ++k)
                if (k % LANES == lane) y[i * BD + k] = acc[k];
        }
    }
}

// y = r - A x, operator in VT precision, accumulation in ACC
template <int BD, int LANES, typename VT, typename ACC, typename XT>
__global__ void __launch_bounds__(256) residual_kernel(BsrDev A, const VT *__restrict__ vals,
                                                       const double *__restrict__ r, const XT *__restrict__ x,
                                                       double *__restrict__ y, const int *done)
{
    if (done && *done) return;
    const int lane = threadIdx.x % LANES;
    constexpr int RPW = 32 / LANES;  // block rows per warp and sweep
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // warp-uniform trip count: every lane reaches the group shuffles together
    for (int64_t wr = w0 * RPW; wr < A.nb; wr += nw * RPW) {
        const int64_t i = wr + (threadIdx.x & 31) / LANES;
        const bool valid = i < A.nb;
        ACC acc[BD];
        bsr_block_row<BD, LANES, VT, XT, ACC>(A.rows, A.cols, vals, (int32_t)i, valid, x, lane, acc);
        if (valid) {
#pragma unroll
            for (int k = 0; k < BD; ++k)
                if (k % LANES == lane) y[i * BD + k] = r[i * BD + k] - (double)acc[k];
        }
    }
}

// y32 = r - A x for the mixed preconditioner, rounded to FP32 (its result
// feeds the FP32 MAS).  Rows flagged in `precise` (the stiff rows: there r - A
// z cancels terms many orders larger than the result -- entries of 1e7 times a
// nearly rigid z -- which FP32 would turn into noise of the result's size) are
// evaluated in double-float (values as (hi, lo) pairs, x = x32 + x_lo, r in
// FP64); all other rows entirely in FP32.  A warp takes the double-float branch
// for all of its rows when any of them is flagged, so the group shuffles stay
// warp-uniform.
template <int BD, int LANES>
__global__ void __launch_bounds__(256) residual32_kernel(BsrDev A, const float *__restrict__ r32,
                                                         const float *__restrict__ x32, float *__restrict__ y32,
                                                         const uint8_t *__restrict__ precise,
                                                         const double *__restrict__ r64,
                                                         const float *__restrict__ x_lo, const int *done)
{
    if (done && *done) return;
    const int lane = threadIdx.x % LANES;
    constexpr int RPW = 32 / LANES;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t wr = w0 * RPW; wr < A.nb; wr += nw * RPW) {
        const int64_t i = wr + (threadIdx.x & 31) / LANES;
        const bool valid = i < A.nb;
        const bool mine = precise && valid && precise[i];
        if (__any_sync(0xffffffffu, mine)) {
            float sh[BD], sl[BD];
            bsr_block_row_df_split<BD, LANES>(A.rows, A.cols, A.vals_df, (int32_t)i, valid, x32, x_lo, lane, sh, sl);
            if (valid) {
#pragma unroll
                for (int k = 0; k < BD; ++k)
                    if (k % LANES == lane)
                        y32[i * BD + k] = (float)(r64[i * BD + k] - ((double)sh[k] + (double)sl[k]));
            }
        } else {
            float acc[BD];
            bsr_block_row<BD, LANES, float, float, float>(A.rows, A.cols, A.vals32, (int32_t)i, valid, x32, lane,
                                                          acc);
            if (valid) {
#pragma unroll
                for (int k = 0; k < BD; ++k)
                    if (k % LANES == lane) y32[i * BD + k] = r32[i * BD + k] - acc[k];
            }
        }
    }
}

// Ap = A p, p.Ap, then alpha with the breakdown tests (GPUHybrid.cu:1458-1480)
template <int BD, int LANES>
__global__ void __launch_bounds__(256) spmv_alpha_kernel(BsrDev A, const double *__restrict__ p,
                                                         double *__restrict__ Ap, PcgState *st, GridReduce gr)
{
    if (st->done) return;
    const int lane = threadIdx.x % LANES;
    constexpr int RPW = 32 / LANES;  // block rows per warp and sweep
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double dot[1] = {0.0};
    // warp-uniform trip count: every lane reaches the group shuffles together
    for (int64_t wr = w0 * RPW; wr < A.nb; wr += nw * RPW) {
        const int64_t i = wr + (threadIdx.x & 31) / LANES;
        const bool valid = i < A.nb;
        double acc[BD];
        bsr_block_row<BD, LANES, double, double, double>(A.rows, A.cols, A.vals, (int32_t)i, valid, p, lane, acc);
        if (valid) {
#pragma unroll
            for (int k = 0; k < BD; ++k)
                if (k % LANES == lane) {
                    Ap[i * BD + k] = acc[k];
                    dot[0] += p[i * BD + k] * acc[k];
                }
        }
    }
    double tot[1];
    if (grid_sum<1>(dot, gr, tot)) {
        st->iter += 1;
        const double pAp = tot[0];
        st->pAp = pAp;
        if (pAp == 0.0) { st->done = STOP_ZERO_PAP; return; }
        const double alpha = st->gamma / pAp;
        if (!(alpha == alpha) || isinf(alpha)) { st->done = STOP_NONFINITE; return; }
        if (alpha <= 0.0) { st->done = STOP_NEGATIVE_ALPHA; return; }
        if (alpha < DBL_MIN) { st->done = STOP_SUBNORMAL_ALPHA; return; }
        st->alpha = alpha;
        if (st->iter <= PCG_HIST) st->hist_alpha[st->iter - 1] = alpha;
    }
}

// x += alpha p; r -= alpha Ap; rr; convergence (GPUHybrid.cu:1482-1496)
__device__ __forceinline__ double as_double(double v) { return v; }
__device__ __forceinline__ double as_double(float2 v) { return (double)v.x + (double)v.y; }

// AT: double, or float2 for the (hi, lo) product of the df32 SpMV.  r32
// (optional): r rounded to FP32, the input of the mixed preconditioner's
// FP32 residual -- converted here, where every lane of a warp converts one
// entry (a partly predicated FP64 instruction costs the pipe a full warp).
template <typename AT>
__global__ void __launch_bounds__(256) update_xr_kernel(int64_t n, double *__restrict__ x, double *__restrict__ r,
                                                        const double *__restrict__ p, const AT *__restrict__ Ap,
                                                        PcgState *st, GridReduce gr, float *__restrict__ r32)
{
    if (st->done) return;
    const double alpha = st->alpha;
    double s[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * as_double(Ap[i]);
        r[i] = ri;
        if (r32) r32[i] = (float)ri;
        s[0] += ri * ri;
    }
    double tot[1];
    if (grid_sum<1>(s, gr, tot)) {
        const double rr = tot[0];
        st->rr = rr;
        if (!(rr == rr) || isinf(rr)) { st->done = STOP_NONFINITE; return; }
        if (st->rel_eps > 0 && rr / st->bb < st->rel_eps) { st->done = STOP_CONVERGED_REL; return; }
        if (st->abs_eps > 0 && rr < st->abs_eps) { st->done = STOP_CONVERGED_ABS; return; }
        if (st->iter >= st->max_iter) { st->done = STOP_MAX_ITER; return; }
    }
}

// p = z + beta p (GPUHybrid.cu:1506-1507); optionally also its df32 split
__global__ void __launch_bounds__(256) update_p_kernel(int64_t n, double *__restrict__ p, const double *__restrict__ z,
                                                       const PcgState *st, float2 *__restrict__ p_df)
{
    if (st->done) return;
    const double beta = st->beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = z[i] + beta * p[i];
        p[i] = v;
        if (p_df) {
            const float h = (float)v;
            p_df[i] = make_float2(h, (float)(v - (double)h));
        }
    }
}

__global__ void split_kernel(int64_t n, const double *__restrict__ src, float2 *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = src[i];
        const float h = (float)v;
        dst[i] = make_float2(h, (float)(v - (double)h));
    }
}

// spmv_alpha_kernel with the SpMV in double-float on the FP32 pipe.  A p
// leaves as (hi, lo) pairs and p.Ap accumulates in double-float, so the loop
// issues no FP64 instruction: the storing lanes (k % LANES == lane) would
// run them as partly predicated warps, each costing the FP64 pipe a full warp.
template <int BD, int LANES>
__global__ void __launch_bounds__(256) spmv_alpha_df_kernel(BsrDev A, const float2 *__restrict__ p_df,
                                                            float2 *__restrict__ Ap, PcgState *st, GridReduce gr)
{
    if (st->done) return;
    const int lane = threadIdx.x % LANES;
    constexpr int RPW = 32 / LANES;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    float dh = 0.f, dl = 0.f;
    for (int64_t wr = w0 * RPW; wr < A.nb; wr += nw * RPW) {
        const int64_t i = wr + (threadIdx.x & 31) / LANES;
        const bool valid = i < A.nb;
        float sh[BD], sl[BD];
        bsr_block_row_df<BD, LANES>(A.rows, A.cols, A.vals_df, (int32_t)i, valid, p_df, lane, sh, sl);
        if (valid) {
#pragma unroll
            for (int k = 0; k < BD; ++k)
                if (k % LANES == lane) {
                    Ap[i * BD + k] = make_float2(sh[k], sl[k]);
                    const float2 pk = p_df[i * BD + k];
                    df_fma(dh, dl, pk.x, pk.y, sh[k], sl[k]);
                }
        }
    }
    double dot[1] = {(double)dh + (double)dl};
    double tot[1];
    if (grid_sum<1>(dot, gr, tot)) {
        st->iter += 1;
        const double pAp = tot[0];
        st->pAp = pAp;
        if (pAp == 0.0) { st->done = STOP_ZERO_PAP; return; }
        const double alpha = st->gamma / pAp;
        if (!(alpha == alpha) || isinf(alpha)) { st->done = STOP_NONFINITE; return; }
        if (alpha <= 0.0) { st->done = STOP_NEGATIVE_ALPHA; return; }
        if (alpha < DBL_MIN) { st->done = STOP_SUBNORMAL_ALPHA; return; }
        st->alpha = alpha;
        if (st->iter <= PCG_HIST) st->hist_alpha[st->iter - 1] = alpha;
    }
}

__global__ void __launch_bounds__(256) dot_kernel(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                                                  double *out, GridReduce gr)
{
    double s[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s[0] += a[i] * b[i];
    double tot[1];
    if (grid_sum<1>(s, gr, tot)) *out = tot[0];
}

__global__ void copy_kernel(int64_t n, const double *__restrict__ src, double *__restrict__ dst, const int *done)
{
    if (done && *done) return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

__global__ void permute_kernel(int64_t nb, int bd, const int32_t *__restrict__ perm, const double *__restrict__ src,
                               double *__restrict__ dst, bool to_new)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb * bd;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t blk = i / bd, c = i % bd;
        const int64_t q = (int64_t)perm[blk] * bd + c;
        if (to_new) dst[q] = src[i];
        else dst[i] = src[q];
    }
}

// dA[k] = -lambda[row] * x[col] over the stored pattern (outer = row)
__global__ void grad_pattern_kernel(int32_t n, const int32_t *__restrict__ outer, const int32_t *__restrict__ inner,
                                    const double *__restrict__ lambda, const double *__restrict__ x,
                                    double *__restrict__ dA)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw) {
        const double li = lambda[i];
        for (int32_t k = outer[i] + lane; k < outer[i + 1]; k += 32) dA[k] = -li * x[inner[k]];
    }
}

// gamma bookkeeping from r.z: mode 1 initial gamma, mode 2 beta and new gamma
__global__ void __launch_bounds__(256) rz_kernel(int64_t n, const double *__restrict__ r, const double *__restrict__ z,
                                                 PcgState *st, int mode, GridReduce gr)
{
    if (st->done) return;
    double s[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s[0] += r[i] * z[i];
    double tot[1];
    if (grid_sum<1>(s, gr, tot)) {
        if (mode == 2) {
            st->beta = tot[0] / st->gamma;
            if (st->iter >= 1 && st->iter <= PCG_HIST) st->hist_beta[st->iter - 1] = st->beta;
        }
        st->gamma = tot[0];
    }
}

__global__ void check_finite_kernel(int64_t n, const double *__restrict__ v, int *flag)
{
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        bad |= !isfinite(v[i]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Fused adjoint scatter: the pattern gradient -lambda_i x_j is formed on the
// fly for the stored entries an element touches and reduced into its
// parameter (one warp per parameter row of the element -> entry map).
__global__ void __launch_bounds__(256) grad_params_kernel(int32_t nparams, const int64_t *__restrict__ rp,
                                                          const int32_t *__restrict__ cols,
                                                          const double *__restrict__ vals,
                                                          const int32_t *__restrict__ row_of,
                                                          const int32_t *__restrict__ inner,
                                                          const double *__restrict__ lambda,
                                                          const double *__restrict__ x, double *__restrict__ dtheta)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t e = w0; e < nparams; e += nw) {
        double acc = 0.0;
        for (int64_t k = rp[e] + lane; k < rp[e + 1]; k += 32) {
            const int32_t v = cols[k];
            acc -= vals[k] * lambda[row_of[v]] * x[inner[v]];
        }
        acc = warp_sum(acc);
        if (lane == 0) dtheta[e] = acc;
    }
}

// values[v] = sum_k mvals[k] theta[mcols[k]] over the CSR row v of M, + c[v]:
// one thread per stored entry of A (rows of a few dozen parameters)
__global__ void __launch_bounds__(256) assemble_values_kernel(int64_t nvals, const int64_t *__restrict__ rowptr,
                                                              const int32_t *__restrict__ mcols,
                                                              const double *__restrict__ mvals,
                                                              const double *__restrict__ theta,
                                                              const double *__restrict__ c, double *__restrict__ out)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvals; v += (int64_t)gridDim.x * blockDim.x) {
        double acc = c ? c[v] : 0.0;
        for (int64_t k = rowptr[v]; k < rowptr[v + 1]; ++k) acc += mvals[k] * theta[mcols[k]];
        out[v] = acc;
    }
}

__global__ void row_of_kernel(int32_t n, const int32_t *__restrict__ outer, int32_t *__restrict__ row_of)
{
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t i = w0; i < n; i += nw)
        for (int32_t k = outer[i] + lane; k < outer[i + 1]; k += 32) row_of[k] = (int32_t)i;
}

template <int BD>
void spmv_dispatch(const BsrDev &A, const double *x, double *y, const int *done, cudaStream_t s)
{
    const int grid = grid_for((int64_t)A.nb * A.lanes, 256, sm_grid(16));
    switch (A.lanes) {
    case 1: spmv_kernel<BD, 1><<<grid, 256, 0, s>>>(A, x, y, done); break;
    case 2: spmv_kernel<BD, 2><<<grid, 256, 0, s>>>(A, x, y, done); break;
    case 4: spmv_kernel<BD, 4><<<grid, 256, 0, s>>>(A, x, y, done); break;
    case 8: spmv_kernel<BD, 8><<<grid, 256, 0, s>>>(A, x, y, done); break;
    case 16: spmv_kernel<BD, 16><<<grid, 256, 0, s>>>(A, x, y, done); break;
    default: spmv_kernel<BD, 32><<<grid, 256, 0, s>>>(A, x, y, done); break;
    }
}

template <int BD, typename VT, typename ACC, typename XT>
void residual_dispatch(const BsrDev &A, const VT *vals, const double *r, const XT *x, double *y,
                       const int *done, cudaStream_t s)
{
    const int lanes = sizeof(VT) == 4 ? A.lanes32 : A.lanes;
    const int grid = grid_for((int64_t)A.nb * lanes, 256, sm_grid(16));
    switch (lanes) {
    case 1: residual_kernel<BD, 1, VT, ACC, XT><<<grid, 256, 0, s>>>(A, vals, r, x, y, done); break;
    case 2: residual_kernel<BD, 2, VT, ACC, XT><<<grid, 256, 0, s>>>(A, vals, r, x, y, done); break;
    case 4: residual_kernel<BD, 4, VT, ACC, XT><<<grid, 256, 0, s>>>(A, vals, r, x, y, done); break;
    case 8: residual_kernel<BD, 8, VT, ACC, XT><<<grid, 256, 0, s>>>(A, vals, r, x, y, done); break;
    case 16: residual_kernel<BD, 16, VT, ACC, XT><<<grid, 256, 0, s>>>(A, vals, r, x, y, done); break;
    default: residual_kernel<BD, 32, VT, ACC, XT><<<grid, 256, 0, s>>>(A, vals, r, x, y, done); break;
    }
}

template <int BD>
void spmv_alpha_dispatch(const BsrDev &A, const double *p, double *Ap, PcgState *st, GridReduce gr, cudaStream_t s)
{
    const int grid = grid_for((int64_t)A.nb * A.lanes, 256, sm_grid(16));
    switch (A.lanes) {
    case 1: spmv_alpha_kernel<BD, 1><<<grid, 256, 0, s>>>(A, p, Ap, st, gr); break;
    case 2: spmv_alpha_kernel<BD, 2><<<grid, 256, 0, s>>>(A, p, Ap, st, gr); break;
    case 4: spmv_alpha_kernel<BD, 4><<<grid, 256, 0, s>>>(A, p, Ap, st, gr); break;
    case 8: spmv_alpha_kernel<BD, 8><<<grid, 256, 0, s>>>(A, p, Ap, st, gr); break;
    case 16: spmv_alpha_kernel<BD, 16><<<grid, 256, 0, s>>>(A, p, Ap, st, gr); break;
    default: spmv_alpha_kernel<BD, 32><<<grid, 256, 0, s>>>(A, p, Ap, st, gr); break;
    }
}

}  // namespace

void launch_gather_values(int64_t count, const int64_t *src, const double *csc, double *vals, float *vals32,
                          cudaStream_t s, float2 *vals_df)
{
    if (count == 0) return;
    gather_values_kernel<<<grid_for(count, 256, sm_grid(16)), 256, 0, s>>>(count, src, csc, vals, vals32, vals_df);
    LSS_LAUNCH_CHECK();
}

void launch_spmv(const BsrDev &A, const double *x, double *y, const int *done, cudaStream_t s)
{
    if (A.bd == 1) spmv_dispatch<1>(A, x, y, done, s);
    else if (A.bd == 2) spmv_dispatch<2>(A, x, y, done, s);
    else spmv_dispatch<3>(A, x, y, done, s);
    LSS_LAUNCH_CHECK();
}

void launch_residual_spmv(const BsrDev &A, const double *r, const double *x, double *y, const int *done,
                          cudaStream_t s)
{
    if (A.bd == 1) residual_dispatch<1, double, double, double>(A, A.vals, r, x, y, done, s);
    else if (A.bd == 2) residual_dispatch<2, double, double, double>(A, A.vals, r, x, y, done, s);
    else residual_dispatch<3, double, double, double>(A, A.vals, r, x, y, done, s);
    LSS_LAUNCH_CHECK();
}

template <int BD>
void residual32_dispatch(const BsrDev &A, const float *r32, const float *x32, float *y32, const uint8_t *precise,
                         const double *r64, const float *x_lo, const int *done, cudaStream_t s)
{
    const int grid = grid_for((int64_t)A.nb * A.lanes32, 256, sm_grid(16));
#define LSS_R32(L_) residual32_kernel<BD, L_><<<grid, 256, 0, s>>>(A, r32, x32, y32, precise, r64, x_lo, done)
    switch (A.lanes32) {
    case 1: LSS_R32(1); break;
    case 2: LSS_R32(2); break;
    case 4: LSS_R32(4); break;
    case 8: LSS_R32(8); break;
    case 16: LSS_R32(16); break;
    default: LSS_R32(32); break;
    }
#undef LSS_R32
}

void launch_residual32(const BsrDev &A, const float *r32, const float *x32, float *y32, const int *done,
                       cudaStream_t s, const uint8_t *precise, const double *r64, const float *x_lo)
{
    if (A.nb > 0 && (!A.vals32 || !r32 || !x32 || !y32))
        fail(LSS_ERR_INTERNAL, "FP32 residual SpMV launched without its operand arrays");
    if (precise && (!A.vals_df || !r64 || !x_lo))
        fail(LSS_ERR_INTERNAL, "double-float rows of the FP32 residual need their operand arrays");
    if (A.bd == 1) residual32_dispatch<1>(A, r32, x32, y32, precise, r64, x_lo, done, s);
    else if (A.bd == 2) residual32_dispatch<2>(A, r32, x32, y32, precise, r64, x_lo, done, s);
    else residual32_dispatch<3>(A, r32, x32, y32, precise, r64, x_lo, done, s);
    LSS_LAUNCH_CHECK();
}

void launch_dot(int64_t n, const double *a, const double *b, double *out, GridReduce gr, cudaStream_t s)
{
    dot_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, a, b, out, gr);
    LSS_LAUNCH_CHECK();
}

void launch_pcg_spmv_alpha(const BsrDev &A, const double *p, double *Ap, PcgState *st, GridReduce gr, cudaStream_t s)
{
    if (A.bd == 1) spmv_alpha_dispatch<1>(A, p, Ap, st, gr, s);
    else if (A.bd == 2) spmv_alpha_dispatch<2>(A, p, Ap, st, gr, s);
    else spmv_alpha_dispatch<3>(A, p, Ap, st, gr, s);
    LSS_LAUNCH_CHECK();
}

template <int BD>
void spmv_alpha_df_dispatch(const BsrDev &A, const float2 *pd, float2 *Ap, PcgState *st, GridReduce gr,
                            cudaStream_t s)
{
    const int grid = grid_for((int64_t)A.nb * A.lanes, 256, sm_grid(16));
    switch (A.lanes) {
    case 1: spmv_alpha_df_kernel<BD, 1><<<grid, 256, 0, s>>>(A, pd, Ap, st, gr); break;
    case 2: spmv_alpha_df_kernel<BD, 2><<<grid, 256, 0, s>>>(A, pd, Ap, st, gr); break;
    case 4: spmv_alpha_df_kernel<BD, 4><<<grid, 256, 0, s>>>(A, pd, Ap, st, gr); break;
    case 8: spmv_alpha_df_kernel<BD, 8><<<grid, 256, 0, s>>>(A, pd, Ap, st, gr); break;
    case 16: spmv_alpha_df_kernel<BD, 16><<<grid, 256, 0, s>>>(A, pd, Ap, st, gr); break;
    default: spmv_alpha_df_kernel<BD, 32><<<grid, 256, 0, s>>>(A, pd, Ap, st, gr); break;
    }
}

void launch_pcg_spmv_alpha_df(const BsrDev &A, const float2 *p_df, float2 *Ap_df, PcgState *st, GridReduce gr,
                              cudaStream_t s)
{
    if (A.nb > 0 && (!A.vals_df || !p_df || !Ap_df))
        fail(LSS_ERR_INTERNAL, "df32 SpMV launched without its operand arrays");
    if (A.bd == 1) spmv_alpha_df_dispatch<1>(A, p_df, Ap_df, st, gr, s);
    else if (A.bd == 2) spmv_alpha_df_dispatch<2>(A, p_df, Ap_df, st, gr, s);
    else spmv_alpha_df_dispatch<3>(A, p_df, Ap_df, st, gr, s);
    LSS_LAUNCH_CHECK();
}

// dst[perm-ordered] = v_i = ((i * 2654435761) mod 2^32) / 2^32 - 0.5 of the
// original index i (the damping estimate's probe vector)
__global__ void probe_kernel(int64_t nb, int bd, const int32_t *__restrict__ perm, double *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nb * bd;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t h = (uint32_t)((uint64_t)(uint32_t)i * 2654435761u);
        dst[(int64_t)perm[i / bd] * bd + i % bd] = (double)h / 4294967296.0 - 0.5;
    }
}

void launch_probe(int64_t nb, int bd, const int32_t *perm, double *dst, cudaStream_t s)
{
    if (nb == 0) return;
    probe_kernel<<<grid_for(nb * bd, 1024, sm_grid(16)), 256, 0, s>>>(nb, bd, perm, dst);
    LSS_LAUNCH_CHECK();
}

__global__ void df_to_double_kernel(int64_t n, const float2 *__restrict__ src, double *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = as_double(src[i]);
}

void launch_df_to_double(int64_t n, const float2 *src, double *dst, cudaStream_t s)
{
    if (n == 0) return;
    df_to_double_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, src, dst);
    LSS_LAUNCH_CHECK();
}

void launch_split(int64_t n, const double *src, float2 *dst, cudaStream_t s)
{
    if (n == 0) return;
    if (!src || !dst) fail(LSS_ERR_INTERNAL, "split launched without its arrays");
    split_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, src, dst);
    LSS_LAUNCH_CHECK();
}

void launch_pcg_update_xr(int64_t n, double *x, double *r, const double *p, const double *Ap, PcgState *st,
                          GridReduce gr, cudaStream_t s, float *r32)
{
    update_xr_kernel<double><<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, x, r, p, Ap, st, gr, r32);
    LSS_LAUNCH_CHECK();
}

void launch_pcg_update_xr_df(int64_t n, double *x, double *r, const double *p, const float2 *Ap_df, PcgState *st,
                             GridReduce gr, cudaStream_t s, float *r32)
{
    update_xr_kernel<float2><<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, x, r, p, Ap_df, st, gr, r32);
    LSS_LAUNCH_CHECK();
}

void launch_pcg_update_p(int64_t n, double *p, const double *z, const PcgState *st, cudaStream_t s, float2 *p_df)
{
    update_p_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, p, z, st, p_df);
    LSS_LAUNCH_CHECK();
}

void launch_copy(int64_t n, const double *src, double *dst, const int *done, cudaStream_t s)
{
    copy_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, src, dst, done);
    LSS_LAUNCH_CHECK();
}

void launch_permute(int64_t nb, int bd, const int32_t *perm, const double *src, double *dst, bool to_new,
                    cudaStream_t s)
{
    permute_kernel<<<grid_for(nb * bd, 1024, sm_grid(16)), 256, 0, s>>>(nb, bd, perm, src, dst, to_new);
    LSS_LAUNCH_CHECK();
}

void launch_pcg_rz(int64_t n, const double *r, const double *z, PcgState *st, int dot_mode, GridReduce gr,
                   cudaStream_t s)
{
    rz_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, r, z, st, dot_mode, gr);
    LSS_LAUNCH_CHECK();
}

void launch_check_finite(int64_t n, const double *v, int *flag, cudaStream_t s)
{
    if (n == 0) return;
    check_finite_kernel<<<grid_for(n, 1024, sm_grid(16)), 256, 0, s>>>(n, v, flag);
    LSS_LAUNCH_CHECK();
}

void launch_grad_params(int32_t nparams, const int64_t *mt_rowptr, const int32_t *mt_cols, const double *mt_vals,
                        const int32_t *row_of, const int32_t *inner, const double *lambda, const double *x,
                        double *dtheta, cudaStream_t s)
{
    if (nparams <= 0) return;
    grad_params_kernel<<<grid_for((int64_t)nparams * 32, 256, sm_grid(16)), 256, 0, s>>>(
        nparams, mt_rowptr, mt_cols, mt_vals, row_of, inner, lambda, x, dtheta);
    LSS_LAUNCH_CHECK();
}

void launch_assemble_values(int64_t nvals, const int64_t *rowptr, const int32_t *mcols, const double *mvals,
                            const double *theta, const double *c, double *out, cudaStream_t s)
{
    if (nvals <= 0) return;
    assemble_values_kernel<<<grid_for(nvals, 256, sm_grid(16)), 256, 0, s>>>(nvals, rowptr, mcols, mvals, theta, c,
                                                                            out);
    LSS_LAUNCH_CHECK();
}

void launch_row_of(int32_t n, const int32_t *outer, int32_t *row_of, cudaStream_t s)
{
    row_of_kernel<<<grid_for((int64_t)n * 32, 256, sm_grid(16)), 256, 0, s>>>(n, outer, row_of);
    LSS_LAUNCH_CHECK();
}

void launch_grad_pattern(int32_t n, const int32_t *outer, const int32_t *inner, const double *lambda,
                         const double *x, double *dA, cudaStream_t s)
{
    grad_pattern_kernel<<<grid_for((int64_t)n * 32, 256, sm_grid(16)), 256, 0, s>>>(n, outer, inner, lambda, x, dA);
    LSS_LAUNCH_CHECK();
}

}  // namespace lss
