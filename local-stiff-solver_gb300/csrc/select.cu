// Stiff-DOF scoring and selection on the GPU (sm_103a).
//
// Restates GPUHybrid::select_bad_dofs (GPUHybrid.cu:737-883):
//   * l1 row norms rn_i = sum_j |a_ij| over each outer slice (:753-765);
//   * global mean / population variance / min / max (:767-777);
//   * EM for a two-component 1D Gaussian mixture in log space, at most
//     max_gmm_iterations iterations, stopping when all four relative parameter
//     changes are below gmm_tol (:795-857);
//   * jump test |mean1| / |mean0| > threshold, selection {i : g0_i < g1_i}
//     in ascending order (:859-879).
// Differences in form, not in result: the responsibilities are recomputed
// instead of stored (the E-step is a pure function of the row norm and the
// previous parameters), every reduction is a deterministic fixed-order grid
// reduction, and the parameters stay on the device between passes (the
// reference reads every reduction back to the host).
#include "device_common.cuh"
#include "kernels.hpp"

namespace lss {
namespace {

// ---- l1 row norms: LANES threads per row, coalesced over the row's entries
template <int LANES>
__global__ void __launch_bounds__(256) l1_norm_kernel(int32_t n, const int32_t *__restrict__ outer,
                                                      const double *__restrict__ vals,
                                                      double *__restrict__ rn)
{
    const int lane = threadIdx.x % LANES;
    constexpr int RPW = 32 / LANES;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    // warp-uniform trip count so the group shuffles see the whole warp
    for (int64_t wr = w0 * RPW; wr < n; wr += nw * RPW) {
        const int64_t i = wr + (threadIdx.x & 31) / LANES;
        const bool valid = i < n;
        const int32_t b = valid ? outer[i] : 0, e = valid ? outer[i + 1] : 0;
        double s = 0.0;
        for (int32_t k = b + lane; k < e; k += LANES) s += fabs(__ldcs(vals + k));
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LANES);
        if (valid && lane == 0) rn[i] = s;
    }
}

// ---- global sum, min, max of rn (one fused pass, last CTA finishes)
__global__ void __launch_bounds__(256) stats_kernel(int32_t n, const double *__restrict__ rn,
                                                    GmmState *st, GridReduce gr)
{
    __shared__ double smin[8], smax[8];
    __shared__ bool last;
    double s[1] = {0.0};
    double mn = INFINITY, mx = -INFINITY;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double x = rn[i];
        s[0] += x;
        mn = fmin(mn, x);
        mx = fmax(mx, x);
    }
    mn = warp_min(mn);
    mx = warp_max(mx);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { smin[wid] = mn; smax[wid] = mx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { mn = fmin(mn, smin[w]); mx = fmax(mx, smax[w]); }
        gr.partials[GRID_MAX * 2 + blockIdx.x] = mn;
        gr.partials[GRID_MAX * 3 + blockIdx.x] = mx;
    }
    double tot[1];
    if (grid_sum<1>(s, gr, tot)) {
        double gmn = INFINITY, gmx = -INFINITY;
        for (int b = 0; b < (int)gridDim.x; ++b) {
            gmn = fmin(gmn, __ldcg(gr.partials + GRID_MAX * 2 + b));
            gmx = fmax(gmx, __ldcg(gr.partials + GRID_MAX * 3 + b));
        }
        st->sum = tot[0];
        st->mean = tot[0] / n;
        st->mn = gmn;
        st->mx = gmx;
    }
    (void)last;
}

__global__ void __launch_bounds__(256) var_kernel(int32_t n, const double *__restrict__ rn, GmmState *st,
                                                  GridReduce gr)
{
    const double mean = st->mean;
    double s[1] = {0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double d = __dsub_rn(rn[i], mean);
        s[0] += __dmul_rn(d, d);
    }
    double tot[1];
    if (grid_sum<1>(s, gr, tot)) {
        st->var = tot[0] / n;
        // initial parameters, GPUHybrid.cu:778-785
        st->m0 = st->mn;
        st->m1 = st->mx;
        st->v0 = st->var;
        st->v1 = st->var;
        st->w0 = 0.5;
        st->w1 = 0.5;
        st->esteps = 0;
        st->converged = 0;
    }
}

// E-step of one row (GPUHybrid.cu:800-818), evaluated without contraction so
// that it rounds like the reference expression tree.
struct Resp {
    double g0, g1, lg0, lg1;
};
__device__ __noinline__ Resp estep(double x, double w0, double w1, double m0, double m1, double v0, double v1)
{
    const double two_pi = 2.0 * 3.14159265358979323846;
    const double log_w0 = log(w0), log_w1 = log(w1);
    const double d0 = __dsub_rn(x, m0), d1 = __dsub_rn(x, m1);
    const double logN0 = __dsub_rn(__dmul_rn(-0.5, log(__dmul_rn(two_pi, v0))),
                                   __ddiv_rn(__dmul_rn(__dmul_rn(0.5, d0), d0), v0));
    const double logN1 = __dsub_rn(__dmul_rn(-0.5, log(__dmul_rn(two_pi, v1))),
                                   __ddiv_rn(__dmul_rn(__dmul_rn(0.5, d1), d1), v1));
    const double lg0 = __dadd_rn(log_w0, logN0), lg1 = __dadd_rn(log_w1, logN1);
    const double mx = fmax(lg0, lg1);
    const double lt = __dadd_rn(mx, log(__dadd_rn(exp(__dsub_rn(lg0, mx)), exp(__dsub_rn(lg1, mx)))));
    Resp r;
    r.g0 = exp(__dsub_rn(lg0, lt));
    r.g1 = exp(__dsub_rn(lg1, lt));
    r.lg0 = lg0;
    r.lg1 = lg1;
    return r;
}

// pass A: responsibilities with the current parameters; sums of g and g*x;
// the last CTA performs the weight and mean updates (GPUHybrid.cu:823-833).
__global__ void __launch_bounds__(256) em_pass_a(int32_t n, const double *__restrict__ rn, GmmState *st,
                                                 GridReduce gr)
{
    if (st->converged) return;
    const double w0 = st->w0, w1 = st->w1, m0 = st->m0, m1 = st->m1, v0 = st->v0, v1 = st->v1;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double x = rn[i];
        const Resp r = estep(x, w0, w1, m0, m1, v0, v1);
        s[0] += r.g0;
        s[1] += r.g1;
        s[2] += __dmul_rn(r.g0, x);
        s[3] += __dmul_rn(r.g1, x);
    }
    double t[4];
    if (grid_sum<4>(s, gr, t)) {
        st->ew0 = w0; st->ew1 = w1; st->em0 = m0; st->em1 = m1; st->ev0 = v0; st->ev1 = v1;
        st->s0 = t[0];
        st->s1 = t[1];
        st->w0 = t[0] / n;
        st->w1 = t[1] / n;
        st->m0 = t[2] / t[0];
        st->m1 = t[3] / t[1];
        st->esteps += 1;
    }
}

// pass B: weighted variances around the new means with the same
// responsibilities; the last CTA applies var_reg and the stopping test
// (GPUHybrid.cu:835-856).
__global__ void __launch_bounds__(256) em_pass_b(int32_t n, const double *__restrict__ rn, GmmState *st,
                                                 GridReduce gr, double tol)
{
    if (st->converged) return;
    const double w0 = st->ew0, w1 = st->ew1, m0 = st->em0, m1 = st->em1, v0 = st->ev0, v1 = st->ev1;
    const double nm0 = st->m0, nm1 = st->m1;
    double s[2] = {0.0, 0.0};
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double x = rn[i];
        const Resp r = estep(x, w0, w1, m0, m1, v0, v1);
        const double d0 = __dsub_rn(x, nm0), d1 = __dsub_rn(x, nm1);
        s[0] += __dmul_rn(__dmul_rn(r.g0, d0), d0);
        s[1] += __dmul_rn(__dmul_rn(r.g1, d1), d1);
    }
    double t[2];
    if (grid_sum<2>(s, gr, t)) {
        const double var_reg = 1e-6;
        const double nv0 = t[0] / st->s0 + var_reg, nv1 = t[1] / st->s1 + var_reg;
        st->v0 = nv0;
        st->v1 = nv1;
        if (fabs(nm0 - m0) / fabs(m0) < tol && fabs(nm1 - m1) / fabs(m1) < tol &&
            fabs(nv0 - v0) / fabs(v0) < tol && fabs(nv1 - v1) / fabs(v1) < tol)
            st->converged = 1;
    }
}

// Selection flags with the parameters of the last E-step; per-CTA counts and
// per-CTA minimum decision margin |lg0 - lg1|.
__global__ void __launch_bounds__(256) mark_kernel(int32_t n, const double *__restrict__ rn,
                                                   const GmmState *st, double threshold,
                                                   int32_t *__restrict__ block_count,
                                                   double *__restrict__ block_margin)
{
    __shared__ int wcount[8];
    __shared__ double wmargin[8];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool jump = st->esteps > 0 && fabs(st->m1) / fabs(st->m0) > threshold;
    bool flag = false;
    double margin = INFINITY;
    if (i < n && st->esteps > 0) {
        const Resp r = estep(rn[i], st->ew0, st->ew1, st->em0, st->em1, st->ev0, st->ev1);
        flag = jump && (r.g0 < r.g1);
        margin = fabs(r.lg0 - r.lg1);
    }
    const unsigned b = __ballot_sync(0xffffffffu, flag);
    margin = warp_min(margin);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { wcount[wid] = __popc(b); wmargin[wid] = margin; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int c = 0;
        double m = INFINITY;
        for (int w = 0; w < 8; ++w) { c += wcount[w]; m = fmin(m, wmargin[w]); }
        block_count[blockIdx.x] = c;
        block_margin[blockIdx.x] = m;
    }
}

__global__ void __launch_bounds__(256) scatter_kernel(int32_t n, const double *__restrict__ rn,
                                                      const GmmState *st, double threshold,
                                                      const int32_t *__restrict__ block_offset,
                                                      int32_t *__restrict__ out)
{
    __shared__ int wbase[8];
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool jump = st->esteps > 0 && fabs(st->m1) / fabs(st->m0) > threshold;
    bool flag = false;
    if (i < n && jump) {
        const Resp r = estep(rn[i], st->ew0, st->ew1, st->em0, st->em1, st->ev0, st->ev1);
        flag = r.g0 < r.g1;
    }
    const unsigned b = __ballot_sync(0xffffffffu, flag);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) wbase[wid] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int acc = block_offset[blockIdx.x];
        for (int w = 0; w < 8; ++w) { int c = wbase[w]; wbase[w] = acc; acc += c; }
    }
    __syncthreads();
    if (flag) out[wbase[wid] + __popc(b & ((1u << lane) - 1u))] = (int32_t)i;
}

__global__ void mark_selected_kernel(int bd, const int32_t *__restrict__ perm, const int32_t *__restrict__ sel,
                                     int32_t nsel, uint8_t *__restrict__ mask)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nsel) return;
    const int32_t k = sel[j];
    mask[(int64_t)perm[k / bd] * bd + k % bd] = 1;
}

__global__ void __launch_bounds__(256) gershgorin_kernel(int bd, const int32_t *__restrict__ rows,
                                                         const int32_t *__restrict__ cols,
                                                         const double *__restrict__ vals,
                                                         const int32_t *__restrict__ perm,
                                                         const int32_t *__restrict__ sel, int32_t nsel,
                                                         const uint8_t *__restrict__ mask, double *__restrict__ diag,
                                                         double *__restrict__ off)
{
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= nsel) return;
    const int32_t k = sel[j];
    const int64_t pk = (int64_t)perm[k / bd] * bd + k % bd;
    const int32_t I = (int32_t)(pk / bd), comp = (int32_t)(pk % bd);
    const int32_t b = rows[I], len = rows[I + 1] - b;
    const double *v = vals + (int64_t)b * bd * bd;
    double d = 0.0, o = 0.0;
    int has_d = 0;
    for (int32_t l = lane; l < len; l += 32) {
        const int64_t J = cols[b + l];
        for (int c = 0; c < bd; ++c) {
            const int64_t col = J * bd + c;
            if (!mask[col]) continue;
            const double a = v[(int64_t)(comp * bd + c) * len + l];
            if (col == pk) { d = a; has_d = 1; }
            else o += fabs(a);
        }
    }
    o = warp_sum(o);
    const unsigned who = __ballot_sync(0xffffffffu, has_d);
    const int src = who ? __ffs(who) - 1 : 0;
    d = __shfl_sync(0xffffffffu, d, src);
    if (lane == 0) {
        diag[j] = who ? d : 0.0;
        off[j] = o;
    }
}

// Per scalar row of the permuted operator (BSR block order, then column within
// the block, as MASSolver's BSR traversal): |diagonal|, the largest |off-
// diagonal| and the l1 norm (BadDOFPreconditioner.cu:110-145,
// BadDofKMeanPreconditioner.cu:187-226, BadDofGMMPreconditioner.cu:285-310).
template <int BD>
__global__ void row_scores_kernel(BsrDev A, double *__restrict__ diag, double *__restrict__ offmax,
                                  double *__restrict__ l1)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (int64_t)A.nb * BD) return;
    const int32_t i = (int32_t)(s / BD), r = (int32_t)(s % BD);
    const int32_t b = A.rows[i], len = A.rows[i + 1] - b;
    const double *v = A.vals + (int64_t)b * BD * BD;
    double d = 0.0, mx = 0.0, sum = 0.0;
    for (int32_t l = 0; l < len; ++l) {
        const int32_t j = A.cols[b + l];
        for (int k = 0; k < BD; ++k) {
            const double a = fabs(v[(int64_t)(r * BD + k) * len + l]);
            sum += a;
            if (j == i && k == r) d = a;
            else mx = fmax(mx, a);
        }
    }
    diag[s] = d;
    offmax[s] = mx;
    l1[s] = sum;
}

}  // namespace

void launch_gershgorin(int nb, int bd, const int32_t *rows, const int32_t *cols, const double *vals,
                       const int32_t *perm, const int32_t *sel, int32_t nsel, uint8_t *mask, double *diag,
                       double *off, cudaStream_t s)
{
    (void)nb;
    if (nsel == 0) return;
    mark_selected_kernel<<<(nsel + 255) / 256, 256, 0, s>>>(bd, perm, sel, nsel, mask);
    gershgorin_kernel<<<(unsigned)(((int64_t)nsel * 32 + 255) / 256), 256, 0, s>>>(bd, rows, cols, vals, perm, sel,
                                                                                  nsel, mask, diag, off);
    LSS_LAUNCH_CHECK();
}

void launch_row_l1_norms(int32_t n, int64_t nnz, const int32_t *outer, const double *vals, double *rn,
                         cudaStream_t s)
{
    const double avg = n > 0 ? (double)nnz / n : 0.0;
    const int grid = grid_for((long long)n * 8, 256, sm_grid(16));
    if (avg <= 6) l1_norm_kernel<4><<<grid, 256, 0, s>>>(n, outer, vals, rn);
    else if (avg <= 16) l1_norm_kernel<8><<<grid, 256, 0, s>>>(n, outer, vals, rn);
    else if (avg <= 40) l1_norm_kernel<16><<<grid, 256, 0, s>>>(n, outer, vals, rn);
    else l1_norm_kernel<32><<<grid, 256, 0, s>>>(n, outer, vals, rn);
    LSS_LAUNCH_CHECK();
}

void launch_gmm(int32_t n, const double *rn, GmmState *st, int max_iterations, double tol, GridReduce gr,
                cudaStream_t s)
{
    const int grid = grid_for(n, 256, sm_grid(8));
    stats_kernel<<<grid, 256, 0, s>>>(n, rn, st, gr);
    LSS_LAUNCH_CHECK();
    var_kernel<<<grid, 256, 0, s>>>(n, rn, st, gr);
    LSS_LAUNCH_CHECK();
    for (int it = 0; it < max_iterations; ++it) {
        em_pass_a<<<grid, 256, 0, s>>>(n, rn, st, gr);
        em_pass_b<<<grid, 256, 0, s>>>(n, rn, st, gr, tol);
    }
    LSS_LAUNCH_CHECK();
}

void launch_gmm_mark(int32_t n, const double *rn, const GmmState *st, double threshold, int32_t *block_count,
                     double *block_margin, cudaStream_t s)
{
    const int grid = (int)((n + 255) / 256);
    if (grid > 0) mark_kernel<<<grid, 256, 0, s>>>(n, rn, st, threshold, block_count, block_margin);
    LSS_LAUNCH_CHECK();
}

void launch_gmm_scatter(int32_t n, const double *rn, const GmmState *st, double threshold,
                        const int32_t *block_offset, int32_t *out, cudaStream_t s)
{
    const int grid = (int)((n + 255) / 256);
    if (grid > 0) scatter_kernel<<<grid, 256, 0, s>>>(n, rn, st, threshold, block_offset, out);
    LSS_LAUNCH_CHECK();
}

void launch_row_scores(const BsrDev &A, double *diag, double *offmax, double *l1, cudaStream_t s)
{
    const int64_t n = (int64_t)A.nb * A.bd;
    if (n == 0) return;
    const unsigned grid = (unsigned)((n + 255) / 256);
    if (A.bd == 1) row_scores_kernel<1><<<grid, 256, 0, s>>>(A, diag, offmax, l1);
    else if (A.bd == 2) row_scores_kernel<2><<<grid, 256, 0, s>>>(A, diag, offmax, l1);
    else row_scores_kernel<3><<<grid, 256, 0, s>>>(A, diag, offmax, l1);
    LSS_LAUNCH_CHECK();
}

}  // namespace lss
