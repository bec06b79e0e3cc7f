// Stiff-block direct solve (sm_103a).
//
// The reference factors each stiff subdomain with cuDSS (batched sparse
// LDL^T) or, up to max_dense_size, with cuBLAS getrf/getri explicit inverses
// (GPUHybrid.cu:993-1411), and applies next_z = z + S^T A_SS^-1 S (r - A z)
// (dss_precond_iter, GPUHybrid.cu:544-675).  Here every subdomain is gathered
// into a dense FP64 block, inverted in FP64 by the symmetric sweep (one CTA in
// shared memory up to 160 DOFs, a blocked multi-CTA sweep beyond), and
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

// one CTA per small subdomain (m <= 160), in place in global storage
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

// Large subdomains: blocked symmetric sweep.  Sweeping the pivots of a block
// K at once is the same operator as sweeping them one by one:
//   P = S[:,K] D^-1 (D = S[K,K]);  S[I,J] -= P[I] S[K,J]  (I, J outside K);
//   S[I,K] = P[I];  S[K,J] = P[J]^T;  S[K,K] = -D^-1.
// After every block has been swept S holds -A^-1.  Four launches per block of
// SW_T pivots; the trailing update is a tiled rank-SW_T product.
constexpr int SW_T = 32;

// ---- large subdomains in double-float: the working matrix W holds (hi, lo)
// FP32 pairs in place of the FP64 entries (same 8 bytes), only its upper
// triangle is kept (the sweep preserves symmetry), and the m^3 / 2 trailing
// updates run error-free products and compensated sums on the FP32 pipe (GB300
// issues 2 DFMA/clk/SM against 128 FP32 FMA).  The pivot blocks (32 x 32) and
// the panels (32 m^2 in total) stay in FP64.

__device__ __forceinline__ float2 df_split(double v)
{
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double df_value(float2 w) { return (double)w.x + (double)w.y; }

// in place, elementwise: the FP64 entry becomes its (hi, lo) pair
__global__ void to_df_kernel(double *__restrict__ S, int64_t count)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        reinterpret_cast<float2 *>(S)[i] = df_split(S[i]);
}

// D^-1 of the pivot block (upper triangle of W[K][K]) by the FP64 scalar sweep
__global__ void __launch_bounds__(256) blk_diag_df_kernel(const float2 *__restrict__ W, int m, int k0, int t,
                                                          double *__restrict__ Dinv, int *bad)
{
    __shared__ double D[SW_T * (SW_T + 1)], col[SW_T], scol[SW_T];
    const int ld = SW_T + 1;
    for (int e = threadIdx.x; e < t * t; e += blockDim.x) {
        const int r = e / t, c = e % t;
        const int a = min(r, c), b = max(r, c);
        D[r * ld + c] = df_value(W[(int64_t)(k0 + a) * m + k0 + b]);
    }
    __syncthreads();
    sweep_invert_small(D, ld, t, col, scol, bad);
    for (int e = threadIdx.x; e < t * t; e += blockDim.x) {
        const int r = e / t, c = e % t;
        Dinv[r * SW_T + c] = -D[r * ld + c];  // the sweep leaves -D^-1
    }
}

// P[i][:] = S[i][K] Dinv for every row i (one thread per row, FP64), stored as pairs
__global__ void __launch_bounds__(128) blk_panel_df_kernel(const float2 *__restrict__ W, int m, int k0, int t,
                                                           const double *__restrict__ Dinv, float2 *__restrict__ P)
{
    __shared__ double Ds[SW_T * SW_T];
    for (int e = threadIdx.x; e < SW_T * SW_T; e += blockDim.x) Ds[e] = Dinv[e];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m || (i >= k0 && i < k0 + t)) return;
    double acc[SW_T];
#pragma unroll
    for (int c = 0; c < SW_T; ++c) acc[c] = 0.0;
    for (int q = 0; q < t; ++q) {
        const int kq = k0 + q;
        const double s = df_value(i < kq ? W[(int64_t)i * m + kq] : W[(int64_t)kq * m + i]);
#pragma unroll
        for (int c = 0; c < SW_T; ++c) acc[c] += s * Ds[q * SW_T + c];
    }
#pragma unroll
    for (int c = 0; c < SW_T; ++c) P[(int64_t)i * SW_T + c] = df_split(c < t ? acc[c] : 0.0);
}

// W[i][j] -= sum_q P[i][q] S[k0+q][j] for the upper-triangle tiles outside K,
// in double-float; 32 x 32 output tiles, four rows per thread
__global__ void __launch_bounds__(256) blk_update_df_kernel(float2 *__restrict__ W, int m, int k0, int t,
                                                            const float2 *__restrict__ P)
{
    const int bi = blockIdx.y, bj = blockIdx.x, bk = k0 / 32;
    if (bj < bi || bi == bk || bj == bk) return;
    __shared__ float2 Pt[32][SW_T + 1], Kt[SW_T][33];
    const int i0 = bi * 32, j0 = bj * 32;
    for (int e = threadIdx.x; e < 32 * SW_T; e += blockDim.x) {
        const int r = e / SW_T, q = e % SW_T;
        const int i = i0 + r;
        Pt[r][q] = (i < m && q < t) ? P[(int64_t)i * SW_T + q] : make_float2(0.f, 0.f);
    }
    if (j0 < k0) {  // S[k0+q][j] = W[j][k0+q] (upper storage): read rows j, contiguous in q
        for (int e = threadIdx.x; e < 32 * SW_T; e += blockDim.x) {
            const int cc = e / SW_T, q = e % SW_T;
            const int j = j0 + cc;
            Kt[q][cc] = (j < m && q < t) ? W[(int64_t)j * m + k0 + q] : make_float2(0.f, 0.f);
        }
    } else {        // S[k0+q][j] = W[k0+q][j]: contiguous in j
        for (int e = threadIdx.x; e < 32 * SW_T; e += blockDim.x) {
            const int q = e / 32, cc = e % 32;
            const int j = j0 + cc;
            Kt[q][cc] = (j < m && q < t) ? W[(int64_t)(k0 + q) * m + j] : make_float2(0.f, 0.f);
        }
    }
    __syncthreads();
    const int cc = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int j = j0 + cc;
    float sh[4], sl[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) sh[s] = sl[s] = 0.f;
#pragma unroll 4
    for (int q = 0; q < SW_T; ++q) {
        const float2 k = Kt[q][cc];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
            const float2 a = Pt[wid + 8 * s][q];
            df_fma(sh[s], sl[s], a.x, a.y, k.x, k.y);
        }
    }
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        const int i = i0 + wid + 8 * s;
        if (i >= m || j >= m || j < i) continue;
        float2 w = W[(int64_t)i * m + j];
        df_add(w.x, w.y, -sh[s], -sl[s]);
        const float hsum = __fadd_rn(w.x, w.y);  // renormalise the pair
        w.y = __fsub_rn(w.y, __fsub_rn(hsum, w.x));
        w.x = hsum;
        W[(int64_t)i * m + j] = w;
    }
}

// the swept pivot rows (upper storage): S[i][K] = P[i] for i < k0, S[K][i] = P[i]
// for i past K, S[K][K] = -Dinv
__global__ void __launch_bounds__(256) blk_write_df_kernel(float2 *__restrict__ W, int m, int k0, int t,
                                                           const float2 *__restrict__ P,
                                                           const double *__restrict__ Dinv)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)m * SW_T) return;
    const int i = (int)(idx / SW_T), c = (int)(idx % SW_T);
    if (c >= t) return;
    if (i >= k0 && i < k0 + t) W[(int64_t)i * m + k0 + c] = df_split(-Dinv[(i - k0) * SW_T + c]);
    else if (i < k0) W[(int64_t)i * m + k0 + c] = P[(int64_t)i * SW_T + c];
    else W[(int64_t)(k0 + c) * m + i] = P[(int64_t)i * SW_T + c];
}

// lower triangle := upper triangle (pairs)
__global__ void mirror_df_kernel(float2 *__restrict__ W, int m)
{
    const int64_t mm = (int64_t)m * m;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < mm;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(idx / m), c = (int)(idx % m);
        if (r > c) W[idx] = W[(int64_t)c * m + r];
    }
}

// in place, elementwise: the pair becomes the FP64 entry of A^-1 (the sweep leaves -A^-1)
__global__ void finish_df_kernel(double *__restrict__ S, int64_t count, int *bad)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double v = -df_value(reinterpret_cast<const float2 *>(S)[i]);
        if (!isfinite(v)) atomicOr(bad, 8);
        S[i] = v;
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

template <typename VT>
__global__ void __launch_bounds__(256) apply_kernel(StiffDev S, const VT *__restrict__ inv, double *__restrict__ z,
                                                    float *__restrict__ z32, float *__restrict__ z_lo, const int *done)
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
    if (lane == 0) {
        const int32_t d = S.dofs[j];
        const double nz = z[d] + acc;
        z[d] = nz;
        if (z32) {
            const float h = (float)nz;
            z32[d] = h;
            if (z_lo) z_lo[d] = (float)(nz - (double)h);
        }
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
    constexpr int SMALL = 160;  // (160 * 161 + 320) doubles = 204 KB of shared memory
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
    int maxm = 0;
    for (int32_t q = 0; q < nsub; ++q) maxm = std::max(maxm, h_off[q + 1] - h_off[q]);
    if (maxm > SMALL) {
        // The blocked sweeps of different subdomains are independent chains of
        // small launches; they run on up to STREAMS_MAX side streams, each with its
        // own pivot-block and panel scratch, joined back to s by events.  The
        // largest subdomain goes first to the stream with the least work (m^3).
        constexpr int STREAMS_MAX = 16;
        std::vector<int32_t> large;
        for (int32_t q = 0; q < nsub; ++q)
            if (h_off[q + 1] - h_off[q] > SMALL) large.push_back(q);
        std::stable_sort(large.begin(), large.end(), [&](int32_t a, int32_t b) {
            return h_off[a + 1] - h_off[a] > h_off[b + 1] - h_off[b];
        });
        const int ns = std::min<int>(STREAMS_MAX, (int)large.size());
        std::vector<cudaStream_t> side(ns, nullptr);
        std::vector<cudaEvent_t> joined(ns, nullptr);
        cudaEvent_t ready = nullptr;
        std::vector<DBuf<double>> Dinv;
        std::vector<DBuf<float2>> P;
        std::vector<double> load(ns, 0.0);
        auto release = [&]() {
            for (cudaEvent_t e : joined)
                if (e) cudaEventDestroy(e);
            if (ready) cudaEventDestroy(ready);
            for (cudaStream_t t : side)
                if (t) cudaStreamDestroy(t);
        };
        try {
            LSS_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
            LSS_CUDA(cudaEventRecord(ready, s));
            for (int i = 0; i < ns; ++i) {
                LSS_CUDA(cudaStreamCreateWithFlags(&side[i], cudaStreamNonBlocking));
                LSS_CUDA(cudaEventCreateWithFlags(&joined[i], cudaEventDisableTiming));
                LSS_CUDA(cudaStreamWaitEvent(side[i], ready, 0));
                Dinv.emplace_back((size_t)SW_T * SW_T);
                P.emplace_back((size_t)maxm * SW_T);
            }
            for (int32_t q : large) {
                const int m = h_off[q + 1] - h_off[q];
                const int i = (int)(std::min_element(load.begin(), load.end()) - load.begin());
                load[i] += (double)m * m * m;
                const cudaStream_t t = side[i];
                double *Sq = inv + hoff[q];
                float2 *Wq = reinterpret_cast<float2 *>(Sq);
                const int64_t mm = (int64_t)m * m;
                to_df_kernel<<<grid_for(mm, 1024, sm_grid(8)), 256, 0, t>>>(Sq, mm);
                const unsigned gp = (unsigned)(((int64_t)m * SW_T + 255) / 256);
                const unsigned gr = (unsigned)((m + 127) / 128);
                const dim3 gu((m + 31) / 32, (m + 31) / 32);
                for (int k0 = 0; k0 < m; k0 += SW_T) {
                    const int w = std::min(SW_T, m - k0);
                    blk_diag_df_kernel<<<1, 256, 0, t>>>(Wq, m, k0, w, Dinv[i].data(), bad);
                    blk_panel_df_kernel<<<gr, 128, 0, t>>>(Wq, m, k0, w, Dinv[i].data(), P[i].data());
                    blk_update_df_kernel<<<gu, 256, 0, t>>>(Wq, m, k0, w, P[i].data());
                    blk_write_df_kernel<<<gp, 256, 0, t>>>(Wq, m, k0, w, P[i].data(), Dinv[i].data());
                }
                mirror_df_kernel<<<grid_for(mm, 1024, sm_grid(8)), 256, 0, t>>>(Wq, m);
                finish_df_kernel<<<grid_for(mm, 1024, sm_grid(8)), 256, 0, t>>>(Sq, mm, bad);
                LSS_LAUNCH_CHECK();
            }
            for (int i = 0; i < ns; ++i) {
                LSS_CUDA(cudaEventRecord(joined[i], side[i]));
                LSS_CUDA(cudaStreamWaitEvent(s, joined[i], 0));
            }
            LSS_CUDA(cudaStreamSynchronize(s));  // scratch is freed at scope exit
        } catch (...) {
            for (cudaStream_t t : side)
                if (t) cudaStreamSynchronize(t);
            release();
            throw;
        }
        release();
    }
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
    if (S.ndof == 0) return;
    const int grid = (int)(((int64_t)S.ndof * 32 + 255) / 256);
    if (fp32) apply_kernel<float><<<grid, 256, 0, s>>>(S, S.inv32, z, z32, z_lo, done);
    else apply_kernel<double><<<grid, 256, 0, s>>>(S, S.inv, z, z32, z_lo, done);
    LSS_LAUNCH_CHECK();
}

}  // namespace lss
