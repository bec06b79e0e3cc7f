// Stiff-block direct solve (sm_103a), dense part.
//
// The reference factors each stiff subdomain with cuDSS (batched sparse
// LDL^T) or, up to max_dense_size, with cuBLAS getrf/getri explicit inverses
// (GPUHybrid.cu:993-1411), and applies next_z = z + S^T A_SS^-1 S (r - A z)
// (dss_precond_iter, GPUHybrid.cu:544-675).  Here a subdomain of up to
// STIFF_DENSE_MAX DOFs is gathered into a dense FP64 block, inverted in FP64
// by the symmetric sweep (one CTA in shared memory) and applied as a
// warp-per-row GEMV fused with the scatter; larger subdomains get the FP64
// multifrontal factor (multifrontal.cu).  The residual rows r - A z are only
// computed on the stiff rows (the reference forms the full product and
// gathers it).
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
    if (j >= S.ndof_dense) return;
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

// one CTA per small subdomain (m <= 160), in place in global storage
__global__ void __launch_bounds__(256) invert_small_kernel(const int32_t *__restrict__ off,
                                                           const int64_t *__restrict__ inv_off,
                                                           double *__restrict__ inv, int *bad)
{
    extern __shared__ double sm[];
    const int32_t s = blockIdx.x;  // the dense subdomains come first
    const int m = off[s + 1] - off[s], ld = m + 1;
    double *S = sm, *col = sm + m * ld, *scol = col + m;
    double *g = inv + inv_off[s];
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int r = idx / m, c = idx % m;
        S[r * ld + c] = (r <= c) ? g[(int64_t)r * m + c] : g[(int64_t)c * m + r];
    }
    __syncthreads();
    sweep_invert_small(S, ld, m, col, scol, bad);
    // stored transposed (column-major): thread j of the apply reads row j as a column
    for (int idx = threadIdx.x; idx < m * m; idx += blockDim.x) {
        const int r = idx / m, c = idx % m;
        const double val = -S[r * ld + c];
        if (!isfinite(val)) atomicOr(bad, 8);
        g[(int64_t)c * m + r] = val;
    }
}

// t_j = r_d (- (A z)_d) for the stiff DOFs d = dofs[j]: one thread per DOF
// walking its row (a few to a few dozen terms), so no warp reduction -- an FP64
// shuffle sum would cost the FP64 pipe five full warps per DOF
template <int BD>
__global__ void __launch_bounds__(256) gather_kernel(BsrDev A, StiffDev S, const double *__restrict__ r,
                                                     const double *__restrict__ z, bool residual, const int *done)
{
    if (done && *done) return;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= S.ndof) return;
    const int32_t d = S.dofs[j];
    double t = r[d];
    if (residual) {
        const int32_t i = d / BD, comp = d % BD;
        const int32_t b = A.rows[i], len = A.rows[i + 1] - b;
        const double *v = A.vals + (int64_t)b * BD * BD;
        double acc = 0.0;
        for (int32_t l = 0; l < len; ++l) {
            const int32_t c = A.cols[b + l];
#pragma unroll
            for (int k = 0; k < BD; ++k) acc += v[(int64_t)(comp * BD + k) * len + l] * z[(int64_t)c * BD + k];
        }
        t -= acc;
    }
    S.t[j] = t;
}

// z_S += Inv t over the dense subdomains: one thread per stiff DOF row j,
// the row read as column j of the transposed storage (consecutive threads,
// consecutive addresses), the sum in column order -- no FP64 shuffles
template <typename VT>
__global__ void __launch_bounds__(256) apply_kernel(StiffDev S, const VT *__restrict__ inv, double *__restrict__ z,
                                                    float *__restrict__ z32, float *__restrict__ z_lo, const int *done)
{
    if (done && *done) return;
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= S.ndof_dense) return;
    const int32_t s = S.sub_of[j], o = S.off[s], m = S.off[s + 1] - o;
    const VT *__restrict__ col = inv + S.inv_off[s] + (j - o);
    const double *__restrict__ t = S.t + o;
    double acc = 0.0;
#pragma unroll 4
    for (int32_t q = 0; q < m; ++q) acc += (double)col[(int64_t)q * m] * t[q];
    const int32_t d = S.dofs[j];
    const double nz = z[d] + acc;
    z[d] = nz;
    if (z32) {
        const float h = (float)nz;
        z32[d] = h;
        if (z_lo) z_lo[d] = (float)(nz - (double)h);
    }
}

__global__ void to_fp32_kernel(int64_t count, const double *__restrict__ src, float *__restrict__ dst)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

}  // namespace

void launch_stiff_extract(const BsrDev &A, const StiffDev &S, double *stage, cudaStream_t s)
{
    if (S.ndof_dense == 0) return;
    const int grid = (int)(((int64_t)S.ndof_dense * 32 + 255) / 256);
    switch (A.bd) {
    case 1: extract_kernel<1><<<grid, 256, 0, s>>>(A, S, stage); break;
    case 2: extract_kernel<2><<<grid, 256, 0, s>>>(A, S, stage); break;
    default: extract_kernel<3><<<grid, 256, 0, s>>>(A, S, stage); break;
    }
    LSS_LAUNCH_CHECK();
}

void launch_stiff_invert(const StiffDev &S, const int32_t *h_off, int32_t nsub, double *inv, int *bad,
                         cudaStream_t s)
{
    if (nsub == 0) return;
    int maxm = 0;
    for (int32_t q = 0; q < nsub; ++q) {
        const int m = h_off[q + 1] - h_off[q];
        if (m > STIFF_DENSE_MAX) fail(LSS_ERR_INTERNAL, "a dense stiff block above the shared-memory size");
        maxm = std::max(maxm, m);
    }
    // (160 * 161 + 320) doubles = 204 KB of shared memory at most
    const size_t smem = (size_t)(maxm * (maxm + 1) + 2 * maxm) * sizeof(double);
    raise_smem_limit((const void *)invert_small_kernel, smem);
    invert_small_kernel<<<(unsigned)nsub, 256, smem, s>>>(S.off, S.inv_off, inv, bad);
    LSS_LAUNCH_CHECK();
}

void launch_stiff_to_fp32(int64_t count, const double *src, float *dst, cudaStream_t s)
{
    if (count > 0 && (!src || !dst)) fail(LSS_ERR_INTERNAL, "FP32 conversion launched without its arrays");
    if (count == 0) return;
    to_fp32_kernel<<<grid_for(count, 256, sm_grid(8)), 256, 0, s>>>(count, src, dst);
    LSS_LAUNCH_CHECK();
}

void launch_stiff_gather(const BsrDev &A, const StiffDev &S, const double *r, const double *z, bool residual,
                         const int *done, cudaStream_t s)
{
    if (S.ndof == 0) return;
    const int grid = (int)(((int64_t)S.ndof + 255) / 256);
    switch (A.bd) {
    case 1: gather_kernel<1><<<grid, 256, 0, s>>>(A, S, r, z, residual, done); break;
    case 2: gather_kernel<2><<<grid, 256, 0, s>>>(A, S, r, z, residual, done); break;
    default: gather_kernel<3><<<grid, 256, 0, s>>>(A, S, r, z, residual, done); break;
    }
    LSS_LAUNCH_CHECK();
}

void launch_stiff_apply(const StiffDev &S, bool fp32, double *z, const int *done, cudaStream_t s, float *z32,
                        float *z_lo)
{
    if (S.ndof_dense == 0) return;
    const int grid = (int)(((int64_t)S.ndof_dense + 255) / 256);
    if (fp32) apply_kernel<float><<<grid, 256, 0, s>>>(S, S.inv32, z, z32, z_lo, done);
    else apply_kernel<double><<<grid, 256, 0, s>>>(S, S.inv, z, z32, z_lo, done);
    LSS_LAUNCH_CHECK();
}

}  // namespace lss
