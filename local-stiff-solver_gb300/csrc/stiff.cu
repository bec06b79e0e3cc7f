// Stiff-block direct solve (sm_103a).
//
// The reference factors each stiff subdomain with cuDSS (batched sparse
// LDL^T) or, up to max_dense_size, with cuBLAS getrf/getri explicit inverses
// (GPUHybrid.cu:993-1411), and applies next_z = z + S^T A_SS^-1 S (r - A z)
// (dss_precond_iter, GPUHybrid.cu:544-675).  Here every subdomain is gathered
// into a dense FP64 block, inverted in FP64 by the symmetric sweep (one CTA in
// shared memory up to 128 DOFs, a per-pivot grid-wide update beyond), and
// applied as a warp-per-row GEMV fused with the scatter.  The residual rows
// r - A z are only computed on the stiff rows (the reference forms the full
// product and gathers it).
#include <algorithm>

#include "device_common.cuh"
#include "kernels.hpp"
#include "spmv.cuh"

namespace lss {
namespace {

template <int BD>
__global__ void __launch_bounds__(256) extract_kernel(BsrDev A, StiffDev S, double *__restrict__ stage)
{
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= S.ndof) return;
    const int32_t d = S.dofs[j], I = d / BD, comp = d % BD;
    const int32_t s = S.sub_of[j], o = S.off[s], m = S.off[s + 1] - o;
    const int32_t *list = S.dofs + o;
    double *row = stage + S.inv_off[s] + (int64_t)(j - o) * m;
    const int32_t b = A.rows[I], len = A.rows[I + 1] - b;
    const double *v = A.vals + (int64_t)b * BD * BD;
    for (int32_t l = lane; l < len; l += 32) {
        const int32_t J = A.cols[b + l];
#pragma unroll
        for (int k = 0; k < BD; ++k) {
            const int32_t col = J * BD + k;
            int32_t lo = 0, hi = m;
            while (lo < hi) {
                const int32_t mid = (lo + hi) >> 1;
                if (list[mid] < col) lo = mid + 1;
                else hi = mid;
            }
            if (lo < m && list[lo] == col) row[lo] = v[(int64_t)(comp * BD + k) * len + l];
        }
    }
}

__device__ void sweep_invert_small(double *S, int ld, int N, double *col, double *scol, int *bad)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    for (int p = 0; p < N; ++p) {
        const double piv = S[p * ld + p];
        for (int t = tid; t < N; t += nt) {
            const double cv = (t == p) ? 0.0 : S[t * ld + p];
            col[t] = cv;
            scol[t] = cv / piv;
        }
        if (tid == 0 && (!isfinite(piv) || piv == 0.0)) atomicOr(bad, 4);
        __syncthreads();
        for (int t = wid; t < N; t += nw) {
            if (t == p) continue;
            const double st = scol[t];
            for (int c = lane; c < N; c += 32)
                if (c != p) S[t * ld + c] -= st * col[c];
        }
        __syncthreads();
        for (int t = tid; t < N; t += nt) {
            if (t == p) S[p * ld + p] = -1.0 / piv;
            else {
                S[t * ld + p] = scol[t];
                S[p * ld + t] = scol[t];
            }
        }
        __syncthreads();
    }
}

// one CTA per small subdomain (m <= 128), in place in global storage
__global__ void __launch_bounds__(256) invert_small_kernel(const int32_t *__restrict__ sub_ids,
                                                           const int32_t *__restrict__ off,
                                                           const int64_t *__restrict__ inv_off,
                                                           double *__restrict__ inv, int *bad)
{
    extern __shared__ double sm[];
    const int32_t s = sub_ids[blockIdx.x];
    const int m = off[s + 1] - off[s], ld = m + 1;
    double *S = sm, *col = sm + m * ld, *scol = col + m;
    double *g = inv + inv_off[s];
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int r = idx / m, c = idx % m;
        S[r * ld + c] = (r <= c) ? g[(int64_t)r * m + c] : g[(int64_t)c * m + r];
    }
    __syncthreads();
    sweep_invert_small(S, ld, m, col, scol, bad);
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int r = idx / m, c = idx % m;
        const double val = -S[r * ld + c];
        if (!isfinite(val)) atomicOr(bad, 8);
        g[(int64_t)r * m + c] = val;
    }
}

// large subdomains: grid-wide sweep, two launches per pivot
__global__ void symmetrize_kernel(double *__restrict__ S, int m)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)m * m) return;
    const int r = (int)(idx / m), c = (int)(idx % m);
    if (r > c) S[idx] = S[(int64_t)c * m + r];
}

__global__ void sweep_update_kernel(double *__restrict__ S, int m, int p, int *bad)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)m * m) return;
    const int t = (int)(idx / m), c = (int)(idx % m);
    const double piv = S[(int64_t)p * m + p];
    if (idx == 0 && (!isfinite(piv) || piv == 0.0)) atomicOr(bad, 4);
    if (t == p || c == p) return;
    S[idx] -= (S[(int64_t)t * m + p] / piv) * S[(int64_t)p * m + c];
}

__global__ void sweep_pivot_kernel(double *__restrict__ S, int m, int p)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m) return;
    const double piv = S[(int64_t)p * m + p];
    if (t == p) return;
    const double v = S[(int64_t)t * m + p] / piv;
    S[(int64_t)t * m + p] = v;
    S[(int64_t)p * m + t] = v;
}

__global__ void sweep_finish_kernel(double *__restrict__ S, int m, int p_last_done, int *bad)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)m * m) return;
    (void)p_last_done;
    const double v = -S[idx];
    if (!isfinite(v)) atomicOr(bad, 8);
    S[idx] = v;
}

__global__ void set_pivot_kernel(double *__restrict__ S, int m, int p)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double piv = S[(int64_t)p * m + p];
        S[(int64_t)p * m + p] = -1.0 / piv;
    }
}

template <int BD>
__global__ void __launch_bounds__(256) gather_kernel(BsrDev A, StiffDev S, const double *__restrict__ r,
                                                     const double *__restrict__ z, bool residual, const int *done)
{
    if (done && *done) return;
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= S.ndof) return;
    const int32_t d = S.dofs[j];
    double t = r[d];
    if (residual) t -= bsr_scalar_row<BD, double, double>(A.rows, A.cols, A.vals, d / BD, d % BD, z, lane);
    if (lane == 0) S.t[j] = t;
}

template <typename VT>
__global__ void __launch_bounds__(256) apply_kernel(StiffDev S, const VT *__restrict__ inv, double *__restrict__ z,
                                                    const int *done)
{
    if (done && *done) return;
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= S.ndof) return;
    const int32_t s = S.sub_of[j], o = S.off[s], m = S.off[s + 1] - o;
    const VT *row = inv + S.inv_off[s] + (int64_t)(j - o) * m;
    const double *t = S.t + o;
    double acc = 0.0;
    for (int32_t k = lane; k < m; k += 32) acc += (double)row[k] * t[k];
    acc = warp_sum(acc);
    if (lane == 0) z[S.dofs[j]] += acc;
}

__global__ void to_fp32_kernel(int64_t count, const double *__restrict__ src, float *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

}  // namespace

void launch_stiff_extract(const BsrDev &A, const StiffDev &S, double *stage, cudaStream_t s)
{
    if (S.ndof == 0) return;
    const int grid = (int)(((int64_t)S.ndof * 32 + 255) / 256);
    switch (A.bd) {
    case 1: extract_kernel<1><<<grid, 256, 0, s>>>(A, S, stage); break;
    case 2: extract_kernel<2><<<grid, 256, 0, s>>>(A, S, stage); break;
    default: extract_kernel<3><<<grid, 256, 0, s>>>(A, S, stage); break;
    }
    LSS_LAUNCH_CHECK();
}

void launch_stiff_invert(const StiffDev &S, const int32_t *h_off, int32_t nsub, const int64_t *h_inv_off,
                         double *inv, int *bad, cudaStream_t s)
{
    (void)h_inv_off;
    constexpr int SMALL = 128;
    std::vector<int32_t> small;
    for (int32_t q = 0; q < nsub; ++q)
        if (h_off[q + 1] - h_off[q] <= SMALL) small.push_back(q);
    if (!small.empty()) {
        int maxm = 0;
        for (int32_t q : small) maxm = std::max(maxm, h_off[q + 1] - h_off[q]);
        const size_t smem = (size_t)(maxm * (maxm + 1) + 2 * maxm) * sizeof(double);
        LSS_CUDA(cudaFuncSetAttribute(invert_small_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        DBuf<int32_t> ids;
        ids.upload(small, s);
        invert_small_kernel<<<(unsigned)small.size(), 256, smem, s>>>(ids.data(), S.off, S.inv_off, inv, bad);
        LSS_LAUNCH_CHECK();
        LSS_CUDA(cudaStreamSynchronize(s));  // ids is freed at scope exit
    }
    std::vector<int64_t> hoff(nsub);
    // inverse offsets are the running sum of m*m
    int64_t acc = 0;
    for (int32_t q = 0; q < nsub; ++q) {
        hoff[q] = acc;
        acc += (int64_t)(h_off[q + 1] - h_off[q]) * (h_off[q + 1] - h_off[q]);
    }
    for (int32_t q = 0; q < nsub; ++q) {
        const int m = h_off[q + 1] - h_off[q];
        if (m <= SMALL) continue;
        double *Sq = inv + hoff[q];
        const int64_t mm = (int64_t)m * m;
        const unsigned g = (unsigned)((mm + 255) / 256);
        symmetrize_kernel<<<g, 256, 0, s>>>(Sq, m);
        for (int p = 0; p < m; ++p) {
            sweep_update_kernel<<<g, 256, 0, s>>>(Sq, m, p, bad);
            sweep_pivot_kernel<<<(m + 255) / 256, 256, 0, s>>>(Sq, m, p);
            set_pivot_kernel<<<1, 32, 0, s>>>(Sq, m, p);
        }
        sweep_finish_kernel<<<g, 256, 0, s>>>(Sq, m, m, bad);
        LSS_LAUNCH_CHECK();
    }
}

void launch_stiff_to_fp32(int64_t count, const double *src, float *dst, cudaStream_t s)
{
    if (count == 0) return;
    to_fp32_kernel<<<grid_for(count, 256, 152 * 8), 256, 0, s>>>(count, src, dst);
    LSS_LAUNCH_CHECK();
}

void launch_stiff_gather(const BsrDev &A, const StiffDev &S, const double *r, const double *z, bool residual,
                         const int *done, cudaStream_t s)
{
    if (S.ndof == 0) return;
    const int grid = (int)(((int64_t)S.ndof * 32 + 255) / 256);
    switch (A.bd) {
    case 1: gather_kernel<1><<<grid, 256, 0, s>>>(A, S, r, z, residual, done); break;
    case 2: gather_kernel<2><<<grid, 256, 0, s>>>(A, S, r, z, residual, done); break;
    default: gather_kernel<3><<<grid, 256, 0, s>>>(A, S, r, z, residual, done); break;
    }
    LSS_LAUNCH_CHECK();
}

void launch_stiff_apply(const StiffDev &S, bool fp32, double *z, const int *done, cudaStream_t s)
{
    if (S.ndof == 0) return;
    const int grid = (int)(((int64_t)S.ndof * 32 + 255) / 256);
    if (fp32) apply_kernel<float><<<grid, 256, 0, s>>>(S, S.inv32, z, done);
    else apply_kernel<double><<<grid, 256, 0, s>>>(S, S.inv, z, done);
    LSS_LAUNCH_CHECK();
}

}  // namespace lss
