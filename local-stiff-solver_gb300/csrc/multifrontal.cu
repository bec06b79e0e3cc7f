// Numeric factorization and solve of the multifrontal stiff-block factor
// (sm_103a, FP64).  The symbolic structure comes from mf_symbolic.cpp.
//
// Factorization, per tree level (leaves first):
//   extend-add      one CTA per front, children summed in ascending order
//   small fronts    f <= MF_SMEM_F: one CTA sweeps the own pivots in shared memory
//   large fronts    blocked sweep over 32-pivot panels, batched over the
//                   level's fronts: pivot-block inverse, panel P = S[:,K] D^-1,
//                   rank-32 update of the upper-triangle tiles, panel write-back;
//                   then the swept rows are mirrored into the lower triangle
// (the original entries are assembled into every front once, before level 0).
// Solve, per level: a gather extend-add of every front's vector and a forward
// GEMV launch (leaves first), then one backward GEMV launch per level (root
// first) and one scatter.  GEMV CTAs take 32 output columns and at most 256
// of a front's rows; larger fronts split their rows over several CTAs whose
// partial sums the last CTA of the group adds in a fixed order.  The
// per-level launches use programmatic dependent launch.  The solve with one
// right-hand side is FP64; the batched solve with 16 reads the fronts as
// double-float pairs (below).
#include <algorithm>
#include <utility>

#include "device_common.cuh"
#include "multifrontal.hpp"
#include "spmv.cuh"

namespace lss {
namespace {

constexpr int PW = 32;  // panel width / outputs per CTA

struct MfView {
    const int32_t *p0, *s, *u, *woff, *bnd_off, *bnd_pos, *child_off, *child, *ea_map, *front_of_pos, *pos2j,
        *j2pos, *poff;
    const int64_t *foff;
    int32_t j_base, npos;
};

__device__ __forceinline__ int find_front(const MfWork &w, int64_t cta)
{
    if (w.cta_item) return w.cta_item[cta];
    int lo = 0, hi = w.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (w.prefix[mid] <= cta) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// original entries: warp per position, upper triangle of its front row
template <int BD>
__global__ void __launch_bounds__(256) mf_assemble_kernel(BsrDev A, StiffDev S, MfView v, double *__restrict__ F)
{
    const int lane = threadIdx.x & 31;
    const int64_t p = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (p >= v.npos) return;
    const int32_t N = v.front_of_pos[p], p0 = v.p0[N], s = v.s[N], u = v.u[N], f = s + u;
    const int32_t fi = (int32_t)p - p0;
    const int32_t j = v.pos2j[p], d = S.dofs[j], sub = S.sub_of[j], lo = S.off[sub], m = S.off[sub + 1] - lo;
    const int32_t *list = S.dofs + lo;
    const int32_t *bp = v.bnd_pos + v.bnd_off[N];
    double *row = F + v.foff[N] + (int64_t)fi * f;
    const int32_t I = d / BD, comp = d % BD;
    const int32_t b = A.rows[I], len = A.rows[I + 1] - b;
    const double *vals = A.vals + (int64_t)b * BD * BD;
    for (int32_t l = lane; l < len; l += 32) {
        const int32_t J = A.cols[b + l];
#pragma unroll
        for (int k = 0; k < BD; ++k) {
            const int32_t col = J * BD + k;
            int32_t a = 0, e = m;
            while (a < e) {
                const int32_t mid = (a + e) >> 1;
                if (list[mid] < col) a = mid + 1;
                else e = mid;
            }
            if (a >= m || list[a] != col) continue;
            const int32_t q = v.j2pos[lo + a - v.j_base];
            if (q < p0) continue;  // an earlier front assembled this entry
            int32_t fj;
            if (q < p0 + s) {
                fj = q - p0;
                if (fj < fi) continue;  // upper triangle
            } else {
                int32_t x = 0, y = u;
                while (x < y) {
                    const int32_t mid = (x + y) >> 1;
                    if (bp[mid] < q) x = mid + 1;
                    else y = mid;
                }
                if (x >= u || bp[x] != q) continue;
                fj = s + x;
            }
            row[fj] = vals[(int64_t)(comp * BD + k) * len + l];
        }
    }
}

// children's Schur complements into the parent (upper triangle), in child order
__global__ void __launch_bounds__(256) mf_extend_add_kernel(MfView v, MfWork w, double *__restrict__ F)
{
    const int32_t N = w.front[blockIdx.x];
    const int32_t fN = v.s[N] + v.u[N];
    double *Fn = F + v.foff[N];
    for (int32_t ci = v.child_off[N]; ci < v.child_off[N + 1]; ++ci) {
        const int32_t c = v.child[ci], sc = v.s[c], uc = v.u[c], fc = sc + uc;
        const double *Fc = F + v.foff[c];
        const int32_t *map = v.ea_map + v.bnd_off[c];
        const int64_t total = (int64_t)uc * uc;
        for (int64_t e = threadIdx.x; e < total; e += blockDim.x) {
            const int32_t a = (int32_t)(e / uc), bb = (int32_t)(e % uc);
            if (a > bb) continue;
            Fn[(int64_t)map[a] * fN + map[bb]] += Fc[(int64_t)(sc + a) * fc + sc + bb];
        }
        __syncthreads();
    }
}

// sweep of the leading `np` pivots of the n x n matrix S (ld, shared memory,
// full square): S[t][c] -= S[t][p] S[p][c] / S[p][p] off the pivot row and
// column, the pivot row and column scaled, the pivot replaced by -1 / piv
__device__ void sweep_leading(double *S, int ld, int n, int np, double *col, double *scol, int *bad)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
    for (int p = 0; p < np; ++p) {
        const double piv = S[p * ld + p];
        const double rpiv = 1.0 / piv;
        for (int t = tid; t < n; t += nt) {
            const double cv = (t == p) ? 0.0 : S[t * ld + p];
            col[t] = cv;
            scol[t] = cv * rpiv;
        }
        if (tid == 0 && (!isfinite(piv) || piv == 0.0)) atomicOr(bad, 16);
        __syncthreads();
        for (int t = wid; t < n; t += nw) {
            if (t == p) continue;
            const double st = scol[t];
            for (int c = lane; c < n; c += 32)
                if (c != p) S[t * ld + c] -= st * col[c];
        }
        __syncthreads();
        for (int t = tid; t < n; t += nt) {
            if (t == p) S[p * ld + p] = -rpiv;
            else {
                S[t * ld + p] = scol[t];
                S[p * ld + t] = scol[t];
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) mf_sweep_small_kernel(MfView v, MfWork w, double *__restrict__ F, int *bad)
{
    extern __shared__ double sm[];
    const int32_t N = w.front[blockIdx.x];
    const int s = v.s[N], f = s + v.u[N], ld = f + 1;
    double *S = sm, *col = sm + f * ld, *scol = col + f;
    double *g = F + v.foff[N];
    for (int idx = threadIdx.x; idx < f * f; idx += blockDim.x) {
        const int r = idx / f, c = idx % f;
        S[r * ld + c] = (r <= c) ? g[(int64_t)r * f + c] : g[(int64_t)c * f + r];
    }
    __syncthreads();
    sweep_leading(S, ld, f, s, col, scol, bad);
    for (int idx = threadIdx.x; idx < f * f; idx += blockDim.x) {
        const int r = idx / f, c = idx % f;
        const double val = S[r * ld + c];
        if (!isfinite(val)) atomicOr(bad, 32);
        g[(int64_t)r * f + c] = val;
    }
}

// ---- blocked sweep of the large fronts of a level (upper-triangle storage)

__device__ __forceinline__ double up(const double *Fn, int f, int r, int c)
{
    return r <= c ? Fn[(int64_t)r * f + c] : Fn[(int64_t)c * f + r];
}

// Dinv = (S[K][K])^-1 for the panel K = [k0, k0 + t)
__global__ void __launch_bounds__(256) mf_blk_diag_kernel(MfView v, MfWork w, const double *__restrict__ F, int k0,
                                                          double *__restrict__ Dinv, int *bad)
{
    __shared__ double D[PW * (PW + 1)], col[PW], scol[PW];
    const int i = blockIdx.x;
    const int32_t N = w.front[i];
    const int s = v.s[N], f = s + v.u[N];
    if (s <= k0) return;
    const int t = min(PW, s - k0), ld = PW + 1;
    const double *Fn = F + v.foff[N];
    for (int e = threadIdx.x; e < t * t; e += blockDim.x) {
        const int r = e / t, c = e % t;
        D[r * ld + c] = up(Fn, f, k0 + r, k0 + c);
    }
    __syncthreads();
    sweep_leading(D, ld, t, t, col, scol, bad);
    for (int e = threadIdx.x; e < PW * PW; e += blockDim.x) {
        const int r = e / PW, c = e % PW;
        Dinv[(int64_t)i * PW * PW + e] = (r < t && c < t) ? -D[r * ld + c] : 0.0;
    }
}

// P[r][:] = S[r][K] Dinv for every row r outside K (one thread per row)
__global__ void __launch_bounds__(128) mf_blk_panel_kernel(MfView v, MfWork w, const double *__restrict__ F, int k0,
                                                           const double *__restrict__ Dinv, double *__restrict__ P)
{
    __shared__ double Ds[PW * PW];
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], f = s + v.u[N];
    if (s <= k0) return;
    const int t = min(PW, s - k0);
    for (int e = threadIdx.x; e < PW * PW; e += blockDim.x) Ds[e] = Dinv[(int64_t)i * PW * PW + e];
    __syncthreads();
    const int r = (int)(blockIdx.x - w.prefix[i]) * blockDim.x + threadIdx.x;
    if (r >= f || (r >= k0 && r < k0 + t)) return;
    const double *Fn = F + v.foff[N];
    double acc[PW];
#pragma unroll
    for (int c = 0; c < PW; ++c) acc[c] = 0.0;
    for (int q = 0; q < t; ++q) {
        const double a = up(Fn, f, r, k0 + q);
#pragma unroll
        for (int c = 0; c < PW; ++c) acc[c] += a * Ds[q * PW + c];
    }
    double *Pr = P + v.poff[N] + (int64_t)r * PW;
#pragma unroll
    for (int c = 0; c < PW; ++c) Pr[c] = c < t ? acc[c] : 0.0;
}

// S[a][b] -= sum_q P[a][q] S[k0+q][b] on the upper-triangle 32 x 32 tiles,
// every entry with a and b outside the panel K = [k0, k0 + t) (the last panel
// can end inside its tile, whose remaining rows are boundary rows that still
// take the update); four rows per thread
__global__ void __launch_bounds__(256) mf_blk_update_kernel(MfView v, MfWork w, double *__restrict__ F, int k0,
                                                            const double *__restrict__ P)
{
    __shared__ double Pt[32][PW + 1], Kt[PW][33];
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], f = s + v.u[N];
    if (s <= k0) return;
    const int t = min(PW, s - k0);
    const int T = (f + 31) / 32, bk = k0 / 32;
    int tile = (int)(blockIdx.x - w.prefix[i]), bi = 0;
    while (tile >= T - bi) {
        tile -= T - bi;
        ++bi;
    }
    const int bj = bi + tile;
    if ((bi == bk || bj == bk) && t == PW) return;  // a full panel covers its whole tile
    double *Fn = F + v.foff[N];
    const double *Pn = P + v.poff[N];
    const int i0 = bi * 32, j0 = bj * 32;
    for (int e = threadIdx.x; e < 32 * PW; e += blockDim.x) {
        const int r = e / PW, q = e % PW;
        const int a = i0 + r;
        Pt[r][q] = (a < f && q < t) ? Pn[(int64_t)a * PW + q] : 0.0;
    }
    if (j0 < k0) {  // S[k0+q][b] = Fn[b][k0+q]
        for (int e = threadIdx.x; e < 32 * PW; e += blockDim.x) {
            const int cc = e / PW, q = e % PW;
            const int b = j0 + cc;
            Kt[q][cc] = (b < f && q < t) ? Fn[(int64_t)b * f + k0 + q] : 0.0;
        }
    } else {
        for (int e = threadIdx.x; e < 32 * PW; e += blockDim.x) {
            const int q = e / 32, cc = e % 32;
            const int b = j0 + cc;
            Kt[q][cc] = (b < f && q < t) ? Fn[(int64_t)(k0 + q) * f + b] : 0.0;
        }
    }
    __syncthreads();
    const int cc = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int b = j0 + cc;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll 8
    for (int q = 0; q < PW; ++q) {
        const double kq = Kt[q][cc];
#pragma unroll
        for (int r = 0; r < 4; ++r) acc[r] += Pt[wid + 8 * r][q] * kq;
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int a = i0 + wid + 8 * r;
        if (a >= f || b >= f || b < a) continue;
        if ((a >= k0 && a < k0 + t) || (b >= k0 && b < k0 + t)) continue;  // the panel itself
        Fn[(int64_t)a * f + b] -= acc[r];
    }
}

// swept panel rows: S[r][K] = P[r] (r before K), S[K][r] = P[r] (after), S[K][K] = -Dinv
__global__ void __launch_bounds__(256) mf_blk_write_kernel(MfView v, MfWork w, double *__restrict__ F, int k0,
                                                           const double *__restrict__ P,
                                                           const double *__restrict__ Dinv)
{
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], f = s + v.u[N];
    if (s <= k0) return;
    const int t = min(PW, s - k0);
    const int64_t idx = (int64_t)(blockIdx.x - w.prefix[i]) * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)f * PW) return;
    const int r = (int)(idx / PW), c = (int)(idx % PW);
    if (c >= t) return;
    double *Fn = F + v.foff[N];
    const double *Pn = P + v.poff[N];
    if (r >= k0 && r < k0 + t) {
        if (r - k0 <= c) Fn[(int64_t)r * f + k0 + c] = -Dinv[(int64_t)i * PW * PW + (r - k0) * PW + c];
    } else if (r < k0) {
        Fn[(int64_t)r * f + k0 + c] = Pn[(int64_t)r * PW + c];
    } else {
        Fn[(int64_t)(k0 + c) * f + r] = Pn[(int64_t)r * PW + c];
    }
}

// lower triangle of the swept columns: Fn[r][c] = Fn[c][r] for c < min(r, s)
__global__ void __launch_bounds__(256) mf_mirror_kernel(MfView v, MfWork w, double *__restrict__ F, int *bad)
{
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], f = s + v.u[N];
    const int64_t idx = (int64_t)(blockIdx.x - w.prefix[i]) * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)f * s) return;
    const int r = (int)(idx / s), c = (int)(idx % s);
    double *Fn = F + v.foff[N];
    if (c < r) Fn[(int64_t)r * f + c] = Fn[(int64_t)c * f + r];
    else if (!isfinite(Fn[(int64_t)r * f + c])) atomicOr(bad, 32);
}

// ---- solve

// Programmatic dependent launch across the solve's per-level kernels: each
// lets the next launch be dispatched at once and waits for the previous
// grid's completion (and memory) before it reads anything -- the launches'
// latency overlaps the previous level's tail instead of adding to it.
__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

template <typename... KArgs, typename... Args>
void launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                Args &&...args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    LSS_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

constexpr int NR_COLS = 32;    // output columns per GEMV CTA of the solves
constexpr int NR_KROWS = 256;  // front rows per GEMV CTA of the solves

__host__ __device__ __forceinline__ int nr_kchunks(int rows) { return (rows + NR_KROWS - 1) / NR_KROWS; }

// ---- solve with one right-hand side (FP64).  The same decomposition as the
// batched solve below: per level, CTAs of 256 entries gather each front's
// vector (right-hand side + the children's contributions, children in
// order), then GEMV CTAs of 32 columns x at most 256 front rows (8 warps =
// 8 row slices, lane = column), fronts with more rows split over several
// CTAs whose partial sums the last CTA of the group adds in row-chunk order.

constexpr int NR_COLS1 = 32;

struct NrScratch1 {
    double *part;   // per CTA of a launch: NR_COLS1 partial sums
    unsigned *cnt;  // per group: arrivals
};

// res[c] = sum over the CTA's rows of Fn[q][col0 + c] xs[q - q0]; slices in order
__device__ __forceinline__ void gemv1(const double *__restrict__ Fn, int f, int col0, int ncol, int q0, int nrow,
                                      const double *__restrict__ xs, double *__restrict__ red,
                                      double *__restrict__ res)
{
    const int cl = threadIdx.x & 31, ks = threadIdx.x >> 5;
    double acc = 0.0;
    if (cl < ncol) {
        const double *Fc = Fn + (int64_t)q0 * f + col0 + cl;
#pragma unroll 8
        for (int q = ks; q < nrow; q += 8) acc += __ldg(Fc + (int64_t)q * f) * xs[q];
    }
    red[ks * 32 + cl] = acc;
    __syncthreads();
    if (threadIdx.x < ncol) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < 8; ++q) sum += red[q * 32 + threadIdx.x];
        res[threadIdx.x] = sum;
    }
    __syncthreads();
}

__device__ __forceinline__ bool combine1(NrScratch1 sc, int kc, int nkc, double *__restrict__ res, int ncol)
{
    if (nkc == 1) return true;
    __shared__ bool last;
    if (threadIdx.x < ncol) sc.part[(int64_t)blockIdx.x * NR_COLS1 + threadIdx.x] = res[threadIdx.x];
    __threadfence();
    __syncthreads();
    const int64_t g = (int64_t)blockIdx.x - kc;
    if (threadIdx.x == 0) last = atomicAdd(sc.cnt + g, 1u) == (unsigned)(nkc - 1);
    __syncthreads();
    if (!last) return false;
    __threadfence();
    if (threadIdx.x < ncol) {
        double sum = 0.0;
        for (int j = 0; j < nkc; ++j) sum += __ldcg(sc.part + (g + j) * NR_COLS1 + threadIdx.x);
        res[threadIdx.x] = sum;
    }
    if (threadIdx.x == 0) sc.cnt[g] = 0u;
    __syncthreads();
    return true;
}

// forward, step 1: W_N = [t_own ; 0] + the children's contributions (gathered)
__global__ void __launch_bounds__(256) mf_fassemble1_kernel(MfView v, MfWork w, const int32_t *__restrict__ gptr,
                                                            const int32_t *__restrict__ gsrc, const StiffDev S,
                                                            double *__restrict__ W, const int *done)
{
    pdl_enter();
    if (done && *done) return;
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], f = s + v.u[N];
    const int q = (int)(blockIdx.x - w.prefix[i]) * 256 + (int)threadIdx.x;
    if (q >= f) return;
    const int64_t e = (int64_t)v.woff[N] + q;
    double acc = q < s ? S.t[v.pos2j[v.p0[N] + q]] : 0.0;
    for (int32_t g = gptr[e]; g < gptr[e + 1]; ++g) acc += W[gsrc[g]];
    W[e] = acc;
}

// forward, step 2: W_N[bnd] -= P W_N[own] over the CTA's boundary columns
__global__ void __launch_bounds__(256) mf_forward_kernel(MfView v, MfWork w, const double *__restrict__ F,
                                                         double *__restrict__ W, NrScratch1 sc, const int *done)
{
    pdl_enter();
    if (done && *done) return;
    __shared__ double xs[NR_KROWS], red[256], res[NR_COLS1];
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], u = v.u[N], f = s + u;
    const int nkc = nr_kchunks(s), local = (int)(blockIdx.x - w.prefix[i]);
    const int kc = local % nkc, col0 = s + (local / nkc) * NR_COLS1, ncol = min(NR_COLS1, f - col0);
    const int q0 = kc * NR_KROWS, nrow = min(NR_KROWS, s - q0);
    double *Wn = W + v.woff[N];
    for (int r = threadIdx.x; r < nrow; r += blockDim.x) xs[r] = Wn[q0 + r];
    __syncthreads();
    gemv1(F + v.foff[N], f, col0, ncol, q0, nrow, xs, red, res);
    if (!combine1(sc, kc, nkc, res, ncol)) return;
    if (threadIdx.x < ncol) Wn[col0 + threadIdx.x] -= res[threadIdx.x];
}

// backward: x_own = F11^-1 (w_own - F12 x_bnd) = -(columns of the swept front) . [w_own; x_bnd]
__global__ void __launch_bounds__(256) mf_backward_kernel(MfView v, MfWork w, const double *__restrict__ F,
                                                          const double *__restrict__ W, double *__restrict__ X,
                                                          NrScratch1 sc, const int *done)
{
    pdl_enter();
    if (done && *done) return;
    __shared__ double vec[NR_KROWS], red[256], res[NR_COLS1];
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    const int s = v.s[N], u = v.u[N], f = s + u;
    const int nkc = nr_kchunks(f), local = (int)(blockIdx.x - w.prefix[i]);
    const int kc = local % nkc, c0 = (local / nkc) * NR_COLS1, ncol = min(NR_COLS1, s - c0);
    const int q0 = kc * NR_KROWS, nrow = min(NR_KROWS, f - q0);
    const double *Wn = W + v.woff[N];
    const int32_t *bp = v.bnd_pos + v.bnd_off[N];
    for (int r = threadIdx.x; r < nrow; r += blockDim.x) {
        const int q = q0 + r;
        vec[r] = q < s ? Wn[q] : X[bp[q - s]];
    }
    __syncthreads();
    gemv1(F + v.foff[N], f, c0, ncol, q0, nrow, vec, red, res);
    if (!combine1(sc, kc, nkc, res, ncol)) return;
    if (threadIdx.x < ncol) X[v.p0[N] + c0 + threadIdx.x] = -res[threadIdx.x];
}

__global__ void mf_scatter_kernel(MfView v, const StiffDev S, const double *__restrict__ X, double *__restrict__ z,
                                  float *__restrict__ z32, float *__restrict__ z_lo, const int *done)
{
    pdl_enter();
    if (done && *done) return;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= v.npos) return;
    const int32_t d = S.dofs[v.pos2j[p]];
    const double nz = z[d] + X[p];
    z[d] = nz;
    if (z32) {
        const float h = (float)nz;
        z32[d] = h;
        if (z_lo) z_lo[d] = (float)(nz - (double)h);
    }
}

// ---- solve with NR right-hand sides at once (the batched PCG): t, w and x
// hold NR values per entry, [entry][NR]; z is a double-float pair vector.
// The fronts are read as double-float pairs (Fp: the FP64 factor split into
// FP32 (hi, lo), 8 bytes per entry like FP64) and every product runs on the
// FP32 pipe with error-free products and compensated sums (about 2^-48
// relative per term): GB300 issues 64 FP32 FMAs per FP64 FMA, and the NR
// right-hand sides make the solve arithmetic-bound.
//
// Forward, per level: CTAs of 16 entries sum the right-hand side and the
// children's contributions into each front's vector (extend-add as a gather,
// children in order), then GEMV CTAs apply c = w_bnd - P w_own.  Backward,
// per level: GEMV CTAs apply x_own = F11^-1 (w_own - F12 x_bnd).  A GEMV CTA
// takes 32 output columns and at most 256 of the front's rows: its 256
// threads are 32 columns x 8 row slices (thread t: column t % 32, rows
// t / 32 + 8 j), each keeping all NR sums of its column; the slices meet in
// shared memory in slice order.  A front with more rows splits them over
// several CTAs, whose partial sums meet in global memory: the last CTA of the
// group to arrive adds them in row-chunk order (fixed-order, deterministic).
// The solve vector in shared memory is pairs, the 16-byte slots of row q
// XOR-swizzled by q % 8 so that the rows a warp reads at once fall into
// different banks.

__device__ __forceinline__ float2 split_pair(double d)
{
    const float h = (float)d;
    return make_float2(h, (float)(d - (double)h));
}

// pair index of right-hand side k in row q (swizzled 16-byte slots)
template <int NR>
__device__ __forceinline__ int swz(int q, int k)
{
    return q * NR + ((((k >> 1) ^ (q & 7))) << 1) + (k & 1);
}

struct NrScratch {
    float2 *part;   // per CTA of a launch: NR_COLS x NR partial sums
    unsigned *cnt;  // per group (first CTA of the group): arrivals
};

// res[c][k] = sum over the CTA's rows q0 .. q0 + nrow - 1 of Fn[q][col0 + c] xs[q - q0][k]
// (c < ncol); res in shared memory, NR_COLS x NR pairs
template <int NR>
__device__ __forceinline__ void nr_gemv(const float2 *__restrict__ Fn, int f, int col0, int ncol, int q0, int nrow,
                                        const float2 *__restrict__ xs, float2 *__restrict__ red,
                                        float2 *__restrict__ res)
{
    constexpr int COLS = NR_COLS, SL = 256 / NR_COLS;
    const int cl = threadIdx.x % COLS, ks = threadIdx.x / COLS;
    float ah[NR], al[NR];
#pragma unroll
    for (int k = 0; k < NR; ++k) ah[k] = al[k] = 0.f;
    if (cl < ncol) {
        const float2 *Fc = Fn + (int64_t)q0 * f + col0 + cl;
        auto step = [&](const float2 a, int q) {
            const float4 *xv = reinterpret_cast<const float4 *>(xs + q * NR);
            const int sw = q & 7;
#pragma unroll
            for (int kk = 0; kk < NR / 2; ++kk) {
                const float4 x2 = xv[kk ^ sw];
                df_fma(ah[2 * kk], al[2 * kk], a.x, a.y, x2.x, x2.y);
                df_fma(ah[2 * kk + 1], al[2 * kk + 1], a.x, a.y, x2.z, x2.w);
            }
        };
        // eight rows' loads in flight before their products
        int q = ks;
        for (; q + 7 * SL < nrow; q += 8 * SL) {
            float2 a[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) a[u] = __ldg(Fc + (int64_t)(q + u * SL) * f);
#pragma unroll
            for (int u = 0; u < 8; ++u) step(a[u], q + u * SL);
        }
        for (; q < nrow; q += SL) step(__ldg(Fc + (int64_t)q * f), q);
    }
    // partials of (slice, column), slots swizzled by the column
    float4 *dst = reinterpret_cast<float4 *>(red + (ks * COLS + cl) * NR);
#pragma unroll
    for (int kk = 0; kk < NR / 2; ++kk)
        dst[kk ^ (cl & 7)] = make_float4(ah[2 * kk], al[2 * kk], ah[2 * kk + 1], al[2 * kk + 1]);
    __syncthreads();
    for (int o = threadIdx.x; o < ncol * NR; o += blockDim.x) {
        const int c = o / NR, k = o % NR;
        const int slot = (((k >> 1) ^ (c & 7)) << 1) | (k & 1);
        float h = 0.f, l = 0.f;
#pragma unroll
        for (int q = 0; q < SL; ++q) {
            const float2 v = red[(q * COLS + c) * NR + slot];
            df_add(h, l, v.x, v.y);
        }
        res[o] = make_float2(h, l);
    }
    __syncthreads();
}

// Row-chunk kc of nkc: true in the CTA whose res then holds the group's total
// (every CTA when nkc == 1, else the last of the group to arrive).
template <int NR>
__device__ __forceinline__ bool nr_combine(NrScratch sc, int kc, int nkc, float2 *__restrict__ res, int ncol)
{
    if (nkc == 1) return true;
    __shared__ bool last;
    float2 *mine = sc.part + (int64_t)blockIdx.x * NR_COLS * NR;
    for (int o = threadIdx.x; o < ncol * NR; o += blockDim.x) mine[o] = res[o];
    __threadfence();
    __syncthreads();
    const int64_t g = (int64_t)blockIdx.x - kc;  // the group's first CTA
    if (threadIdx.x == 0) last = atomicAdd(sc.cnt + g, 1u) == (unsigned)(nkc - 1);
    __syncthreads();
    if (!last) return false;
    __threadfence();
    for (int o = threadIdx.x; o < ncol * NR; o += blockDim.x) {
        float h = 0.f, l = 0.f;
        for (int j = 0; j < nkc; ++j) {
            const float2 v = __ldcg(sc.part + (g + j) * NR_COLS * NR + o);
            df_add(h, l, v.x, v.y);
        }
        res[o] = make_float2(h, l);
    }
    if (threadIdx.x == 0) sc.cnt[g] = 0u;
    __syncthreads();
    return true;
}

constexpr size_t NR_SMEM = (size_t)(NR_KROWS * 16 + 256 * 16 + NR_COLS * 16) * sizeof(float2);  // NR = 16

// forward, step 1: W_N = [t_own ; 0] + the children's contributions, every
// entry gathered from its contributors (gptr/gsrc: per entry of W, the child
// entries that extend-add into it, children in ascending order); CTAs of 16
// entries x NR right-hand sides
template <int NR>
__global__ void __launch_bounds__(256) mf_fassemble_nr_kernel(MfView v, MfWork w, const int32_t *__restrict__ gptr,
                                                              const int32_t *__restrict__ gsrc,
                                                              const double *__restrict__ T, float2 *__restrict__ W,
                                                              const int *sys_done, const int32_t *front_sys)
{
    pdl_enter();
    static_assert(NR == 16, "16 entries x 16 right-hand sides per CTA");
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    if (sys_done && sys_done[front_sys[N]]) return;
    const int s = v.s[N], f = s + v.u[N];
    const int q = (int)(blockIdx.x - w.prefix[i]) * 16 + (int)(threadIdx.x >> 4), k = threadIdx.x & 15;
    if (q >= f) return;
    const int64_t e = (int64_t)v.woff[N] + q;
    float2 acc = q < s ? split_pair(T[(int64_t)v.pos2j[v.p0[N] + q] * NR + k]) : make_float2(0.f, 0.f);
    for (int32_t g = gptr[e]; g < gptr[e + 1]; ++g) {
        const float2 c = W[(int64_t)gsrc[g] * NR + k];
        df_add(acc.x, acc.y, c.x, c.y);
    }
    W[e * NR + k] = acc;
}

// forward, step 2: W_N[bnd] -= P W_N[own] over the CTA's boundary columns
template <int NR>
__global__ void __launch_bounds__(256) mf_forward_nr_kernel(MfView v, MfWork w, const float2 *__restrict__ Fp,
                                                            float2 *__restrict__ W, NrScratch sc, const int *sys_done,
                                                            const int32_t *front_sys)
{
    pdl_enter();
    extern __shared__ double sm[];
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    if (sys_done && sys_done[front_sys[N]]) return;
    const int s = v.s[N], u = v.u[N], f = s + u;
    const int nkc = nr_kchunks(s), local = (int)(blockIdx.x - w.prefix[i]);
    const int kc = local % nkc, col0 = s + (local / nkc) * NR_COLS, ncol = min(NR_COLS, f - col0);
    const int q0 = kc * NR_KROWS, nrow = min(NR_KROWS, s - q0);
    float2 *xs = reinterpret_cast<float2 *>(sm), *red = xs + NR_KROWS * NR, *res = red + 256 * NR;
    float2 *Wn = W + (int64_t)v.woff[N] * NR;
    for (int e = threadIdx.x; e < nrow * NR; e += blockDim.x) xs[swz<NR>(e / NR, e % NR)] = Wn[(int64_t)q0 * NR + e];
    __syncthreads();
    nr_gemv<NR>(Fp + v.foff[N], f, col0, ncol, q0, nrow, xs, red, res);
    if (!nr_combine<NR>(sc, kc, nkc, res, ncol)) return;
    for (int o = threadIdx.x; o < ncol * NR; o += blockDim.x) {
        float2 &t = Wn[(int64_t)col0 * NR + o];
        float th = t.x, tl = t.y;
        df_add(th, tl, -res[o].x, -res[o].y);
        t = make_float2(th, tl);
    }
}

template <int NR>
__global__ void __launch_bounds__(256) mf_backward_nr_kernel(MfView v, MfWork w, const float2 *__restrict__ Fp,
                                                             const float2 *__restrict__ W, float2 *__restrict__ X,
                                                             NrScratch sc, const int *sys_done,
                                                             const int32_t *front_sys)
{
    pdl_enter();
    extern __shared__ double sm[];
    const int i = find_front(w, blockIdx.x);
    const int32_t N = w.front[i];
    if (sys_done && sys_done[front_sys[N]]) return;
    const int s = v.s[N], u = v.u[N], f = s + u;
    const int nkc = nr_kchunks(f), local = (int)(blockIdx.x - w.prefix[i]);
    const int kc = local % nkc, c0 = (local / nkc) * NR_COLS, ncol = min(NR_COLS, s - c0);
    const int q0 = kc * NR_KROWS, nrow = min(NR_KROWS, f - q0);
    float2 *vec = reinterpret_cast<float2 *>(sm), *red = vec + NR_KROWS * NR, *res = red + 256 * NR;
    const float2 *Wn = W + (int64_t)v.woff[N] * NR;
    const int32_t *bp = v.bnd_pos + v.bnd_off[N];
#pragma unroll 8
    for (int e = threadIdx.x; e < nrow * NR; e += blockDim.x) {
        const int r = e / NR, k = e % NR, q = q0 + r;
        vec[swz<NR>(r, k)] = q < s ? Wn[(int64_t)q * NR + k] : X[(int64_t)bp[q - s] * NR + k];
    }
    __syncthreads();
    // x_own = F11^-1 (w_own - F12 x_bnd) = -(column c of the swept front) . vec
    nr_gemv<NR>(Fp + v.foff[N], f, c0, ncol, q0, nrow, vec, red, res);
    if (!nr_combine<NR>(sc, kc, nkc, res, ncol)) return;
    float2 *xo = X + ((int64_t)v.p0[N] + c0) * NR;
    for (int o = threadIdx.x; o < ncol * NR; o += blockDim.x) xo[o] = make_float2(-res[o].x, -res[o].y);
}

__global__ void split_pairs_kernel(int64_t n, const double *__restrict__ src, float2 *__restrict__ dst)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) dst[t] = split_pair(src[t]);
}

template <int NR>
__global__ void mf_scatter_nr_kernel(MfView v, const StiffDev S, const float2 *__restrict__ X,
                                     float2 *__restrict__ z)
{
    pdl_enter();
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)v.npos * NR) return;
    const int64_t p = t / NR;
    const int k = (int)(t % NR);
    const int64_t e = (int64_t)S.dofs[v.pos2j[p]] * NR + k;
    float h = z[e].x, l = z[e].y;
    const float2 xv = X[t];
    df_add(h, l, xv.x, xv.y);
    const float r = __fadd_rn(h, l);
    z[e] = make_float2(r, __fsub_rn(l, __fsub_rn(r, h)));
}

}  // namespace

int64_t MfFactor::bytes() const
{
    return (int64_t)(d_F_.bytes() + d_w_.bytes() + d_x_.bytes() + d_P_.bytes() + d_D_.bytes() + d_i32_.bytes() +
                     d_i64_.bytes());
}

void MfFactor::setup(const MfSymbolic &sym, cudaStream_t st)
{
    sym_ = sym;
    levels_.clear();
    if (sym_.nfront == 0) {
        d_F_.release();
        return;
    }
    const MfSymbolic &M = sym_;
    const int32_t nf = M.nfront;
    // per-level work lists; P scratch offsets per large front within its level
    std::vector<int32_t> poff(nf, 0);
    std::vector<std::vector<int32_t>> lv_all(M.levels), lv_small(M.levels), lv_large(M.levels), lv_ea(M.levels);
    for (int32_t id = 0; id < nf; ++id) {
        const int h = M.height[id];
        lv_all[h].push_back(id);
        if (M.child_off[id + 1] > M.child_off[id]) lv_ea[h].push_back(id);
        (M.s[id] + M.u[id] <= MF_SMEM_F ? lv_small : lv_large)[h].push_back(id);
    }
    int64_t pmax = 0;
    size_t dmax = 0;
    for (int h = 0; h < M.levels; ++h) {
        int64_t acc = 0;
        for (int32_t id : lv_large[h]) {
            poff[id] = (int32_t)acc;
            acc += (int64_t)(M.s[id] + M.u[id]) * PW;
        }
        pmax = std::max(pmax, acc);
        dmax = std::max(dmax, lv_large[h].size());
    }
    std::vector<int32_t> i32;
    std::vector<int64_t> i64;
    auto put32 = [&](const std::vector<int32_t> &a) {
        const size_t at = i32.size();
        i32.insert(i32.end(), a.begin(), a.end());
        return at;
    };
    const size_t a_p0 = put32(M.p0), a_s = put32(M.s), a_u = put32(M.u), a_woff = put32(M.woff),
                 a_bo = put32(M.bnd_off), a_bp = put32(M.bnd_pos), a_co = put32(M.child_off), a_ch = put32(M.child),
                 a_ea = put32(M.ea_map), a_fp = put32(M.front_of_pos), a_pj = put32(M.pos2j),
                 a_jp = put32(M.j2pos), a_po = put32(poff);
    const size_t a_fo = i64.size();
    i64.insert(i64.end(), M.foff.begin(), M.foff.end());
    struct Pending {
        MfWork *w;
        size_t fat, pat, cat;
    };
    std::vector<Pending> pend;
    levels_.resize(M.levels);
    auto make = [&](MfWork &w, const std::vector<int32_t> &fronts, auto ctas_of, bool table = false) {
        w.count = (int32_t)fronts.size();
        const size_t fat = put32(fronts);
        const size_t pat = i64.size();
        int64_t acc = 0;
        i64.push_back(0);
        std::vector<int32_t> item;
        for (int32_t k = 0; k < (int32_t)fronts.size(); ++k) {
            const int64_t c = ctas_of(fronts[k]);
            acc += c;
            i64.push_back(acc);
            if (table) item.insert(item.end(), (size_t)c, k);
        }
        w.ctas = acc;
        pend.push_back({&w, fat, pat, table ? put32(item) : SIZE_MAX});
    };
    auto F_of = [&](int32_t id) { return (int64_t)M.s[id] + M.u[id]; };
    for (int h = 0; h < M.levels; ++h) {
        Level &L = levels_[h];
        make(L.ea, lv_ea[h], [](int32_t) { return (int64_t)1; });
        make(L.small, lv_small[h], [](int32_t) { return (int64_t)1; });
        make(L.diag, lv_large[h], [](int32_t) { return (int64_t)1; });
        make(L.panel, lv_large[h], [&](int32_t id) { return (F_of(id) + 127) / 128; });
        make(L.update, lv_large[h], [&](int32_t id) {
            const int64_t T = (F_of(id) + 31) / 32;
            return T * (T + 1) / 2;
        });
        make(L.write, lv_large[h], [&](int32_t id) { return (F_of(id) * PW + 255) / 256; });
        make(L.mirror, lv_large[h], [&](int32_t id) { return (F_of(id) * M.s[id] + 255) / 256; });
        make(L.fasm_nr, lv_all[h], [&](int32_t id) { return (F_of(id) + 15) / 16; }, true);
        make(L.fasm1, lv_all[h], [&](int32_t id) { return (F_of(id) + 255) / 256; }, true);
        make(L.fwd_nr, lv_all[h], [&](int32_t id) {
            return (int64_t)((M.u[id] + NR_COLS - 1) / NR_COLS) * nr_kchunks(M.s[id]);
        }, true);
        make(L.bwd_nr, lv_all[h], [&](int32_t id) {
            return (int64_t)((M.s[id] + NR_COLS - 1) / NR_COLS) * nr_kchunks(M.s[id] + M.u[id]);
        }, true);
        for (int32_t id : lv_large[h]) L.max_s_large = std::max(L.max_s_large, M.s[id]);
    }
    // extend-add as a gather: per entry of W, the child entries that add into it
    std::vector<int32_t> gptr((size_t)M.welems + 1, 0), gsrc;
    {
        for (int32_t id = 0; id < nf; ++id)
            for (int32_t ci = M.child_off[id]; ci < M.child_off[id + 1]; ++ci) {
                const int32_t c = M.child[ci];
                for (int32_t j = 0; j < M.u[c]; ++j) ++gptr[(size_t)M.woff[id] + M.ea_map[M.bnd_off[c] + j] + 1];
            }
        for (size_t e = 0; e < (size_t)M.welems; ++e) gptr[e + 1] += gptr[e];
        gsrc.resize(gptr.back());
        std::vector<int32_t> fill(gptr.begin(), gptr.end() - 1);
        for (int32_t id = 0; id < nf; ++id)
            for (int32_t ci = M.child_off[id]; ci < M.child_off[id + 1]; ++ci) {
                const int32_t c = M.child[ci];
                for (int32_t j = 0; j < M.u[c]; ++j)
                    gsrc[fill[(size_t)M.woff[id] + M.ea_map[M.bnd_off[c] + j]]++] = M.woff[c] + M.s[c] + j;
            }
    }
    const size_t a_gp = put32(gptr), a_gs = put32(gsrc);
    d_i32_.upload(i32, st);
    d_i64_.upload(i64, st);
    const int32_t *b32 = d_i32_.data();
    gptr_ = b32 + a_gp;
    gsrc_ = b32 + a_gs;
    const int64_t *b64 = d_i64_.data();
    for (const Pending &q : pend) {
        q.w->front = b32 + q.fat;
        q.w->prefix = b64 + q.pat;
        q.w->cta_item = q.cat == SIZE_MAX ? nullptr : b32 + q.cat;
    }
    p0_ = b32 + a_p0;
    s_ = b32 + a_s;
    u_ = b32 + a_u;
    woff_ = b32 + a_woff;
    bnd_off_ = b32 + a_bo;
    bnd_pos_ = b32 + a_bp;
    child_off_ = b32 + a_co;
    child_ = b32 + a_ch;
    ea_map_ = b32 + a_ea;
    front_of_pos_ = b32 + a_fp;
    pos2j_ = b32 + a_pj;
    j2pos_ = b32 + a_jp;
    poff_ = b32 + a_po;
    foff_ = b64 + a_fo;
    // shared memory of the solve kernels, set here: solve() runs inside graph captures
    d_F_.resize(M.elems);
    d_w_.resize(std::max<int64_t>(M.welems, 1));
    // scratch of the split fronts' partial sums (both solves), zeroed counters
    int64_t maxctas = 1;
    for (const Level &L : levels_) maxctas = std::max({maxctas, L.fwd_nr.ctas, L.bwd_nr.ctas});
    d_part1_.resize((size_t)maxctas * NR_COLS1);
    d_nrcnt_.resize((size_t)maxctas);
    d_nrcnt_.zero(st);
    d_x_.resize(std::max<int32_t>(M.npos, 1));
    d_P_.resize(std::max<int64_t>(pmax, 1));
    d_D_.resize(std::max<size_t>(dmax, 1) * PW * PW);
}

namespace {
MfView make_view(const int32_t *p0, const int32_t *s, const int32_t *u, const int32_t *woff, const int32_t *bo,
                 const int32_t *bp, const int32_t *co, const int32_t *ch, const int32_t *ea, const int32_t *fp,
                 const int32_t *pj, const int32_t *jp, const int32_t *po, const int64_t *fo, int32_t j_base,
                 int32_t npos)
{
    MfView v;
    v.p0 = p0; v.s = s; v.u = u; v.woff = woff; v.bnd_off = bo; v.bnd_pos = bp; v.child_off = co; v.child = ch;
    v.ea_map = ea; v.front_of_pos = fp; v.pos2j = pj; v.j2pos = jp; v.poff = po; v.foff = fo;
    v.j_base = j_base; v.npos = npos;
    return v;
}
}  // namespace

void MfFactor::factorize(const BsrDev &A, const StiffDev &S, int *bad, cudaStream_t st)
{
    if (sym_.nfront == 0) return;
    const MfView v = make_view(p0_, s_, u_, woff_, bnd_off_, bnd_pos_, child_off_, child_, ea_map_, front_of_pos_,
                               pos2j_, j2pos_, poff_, foff_, sym_.j_base, sym_.npos);
    double *F = d_F_.data();
    d_F_.zero(st);
    const unsigned ga = (unsigned)(((int64_t)sym_.npos * 32 + 255) / 256);
    switch (A.bd) {
    case 1: mf_assemble_kernel<1><<<ga, 256, 0, st>>>(A, S, v, F); break;
    case 2: mf_assemble_kernel<2><<<ga, 256, 0, st>>>(A, S, v, F); break;
    default: mf_assemble_kernel<3><<<ga, 256, 0, st>>>(A, S, v, F); break;
    }
    LSS_LAUNCH_CHECK();
    const size_t small_smem = (size_t)(MF_SMEM_F * (MF_SMEM_F + 1) + 2 * MF_SMEM_F) * sizeof(double);
    raise_smem_limit((const void *)mf_sweep_small_kernel, small_smem);
    for (const Level &L : levels_) {
        if (L.ea.count) {
            mf_extend_add_kernel<<<L.ea.count, 256, 0, st>>>(v, L.ea, F);
            LSS_LAUNCH_CHECK();
        }
        if (L.small.count) {
            mf_sweep_small_kernel<<<L.small.count, 256, small_smem, st>>>(v, L.small, F, bad);
            LSS_LAUNCH_CHECK();
        }
        if (L.diag.count) {
            for (int k0 = 0; k0 < L.max_s_large; k0 += PW) {
                mf_blk_diag_kernel<<<L.diag.count, 256, 0, st>>>(v, L.diag, F, k0, d_D_.data(), bad);
                mf_blk_panel_kernel<<<(unsigned)L.panel.ctas, 128, 0, st>>>(v, L.panel, F, k0, d_D_.data(),
                                                                            d_P_.data());
                mf_blk_update_kernel<<<(unsigned)L.update.ctas, 256, 0, st>>>(v, L.update, F, k0, d_P_.data());
                mf_blk_write_kernel<<<(unsigned)L.write.ctas, 256, 0, st>>>(v, L.write, F, k0, d_P_.data(),
                                                                            d_D_.data());
                LSS_LAUNCH_CHECK();
            }
            mf_mirror_kernel<<<(unsigned)L.mirror.ctas, 256, 0, st>>>(v, L.mirror, F, bad);
            LSS_LAUNCH_CHECK();
        }
    }
}

void MfFactor::solve(const StiffDev &S, double *z, float *z32, float *z_lo, const int *done, cudaStream_t st)
{
    if (sym_.nfront == 0) return;
    const MfView v = make_view(p0_, s_, u_, woff_, bnd_off_, bnd_pos_, child_off_, child_, ea_map_, front_of_pos_,
                               pos2j_, j2pos_, poff_, foff_, sym_.j_base, sym_.npos);
    const NrScratch1 sc{d_part1_.data(), d_nrcnt_.data()};
    for (const Level &L : levels_) {
        launch_pdl(mf_fassemble1_kernel, (unsigned)L.fasm1.ctas, 256, 0, st, v, L.fasm1, gptr_, gsrc_, S,
                   d_w_.data(), done);
        if (L.fwd_nr.ctas > 0)
            launch_pdl(mf_forward_kernel, (unsigned)L.fwd_nr.ctas, 256, 0, st, v, L.fwd_nr,
                       (const double *)d_F_.data(), d_w_.data(), sc, done);
        LSS_LAUNCH_CHECK();
    }
    for (int h = (int)levels_.size() - 1; h >= 0; --h) {
        const Level &L = levels_[h];
        launch_pdl(mf_backward_kernel, (unsigned)L.bwd_nr.ctas, 256, 0, st, v, L.bwd_nr, (const double *)d_F_.data(),
                   (const double *)d_w_.data(), d_x_.data(), sc, done);
        LSS_LAUNCH_CHECK();
    }
    launch_pdl(mf_scatter_kernel, (unsigned)((sym_.npos + 255) / 256), 256, 0, st, v, S, (const double *)d_x_.data(),
               z, z32, z_lo, done);
    LSS_LAUNCH_CHECK();
}

void MfFactor::make_pairs(cudaStream_t st)
{
    int64_t maxctas = 1;
    for (const Level &L : levels_) maxctas = std::max({maxctas, L.fwd_nr.ctas, L.bwd_nr.ctas});
    d_nrpart_.resize((size_t)maxctas * NR_COLS * 16);
    d_Fp_.resize(std::max<int64_t>(sym_.elems, 1));
    if (sym_.elems > 0) {
        split_pairs_kernel<<<(unsigned)((sym_.elems + 255) / 256), 256, 0, st>>>(sym_.elems, d_F_.data(), d_Fp_.data());
        LSS_LAUNCH_CHECK();
    }
}

void MfFactor::solve_batch(const StiffDev &S, const double *t, float2 *z, const int *sys_done,
                           const int32_t *front_sys, cudaStream_t st)
{
    if (sym_.nfront == 0) return;
    if (d_Fp_.size() < (size_t)sym_.elems) fail(LSS_ERR_INTERNAL, "batched multifrontal solve before make_pairs");
    constexpr int NR = 16;
    const MfView v = make_view(p0_, s_, u_, woff_, bnd_off_, bnd_pos_, child_off_, child_, ea_map_, front_of_pos_,
                               pos2j_, j2pos_, poff_, foff_, sym_.j_base, sym_.npos);
    const size_t smem = NR_SMEM;
    raise_smem_limit((const void *)mf_forward_nr_kernel<NR>, smem);
    raise_smem_limit((const void *)mf_backward_nr_kernel<NR>, smem);
    if (d_wb_.size() < (size_t)std::max<int64_t>(sym_.welems, 1) * NR) d_wb_.resize(std::max<int64_t>(sym_.welems, 1) * NR);
    if (d_xb_.size() < (size_t)std::max<int32_t>(sym_.npos, 1) * NR) d_xb_.resize(std::max<int32_t>(sym_.npos, 1) * NR);
    int64_t maxctas = 1;
    for (const Level &L : levels_) maxctas = std::max({maxctas, L.fwd_nr.ctas, L.bwd_nr.ctas});
    if (d_nrpart_.size() < (size_t)maxctas * NR_COLS * NR)
        fail(LSS_ERR_INTERNAL, "batched multifrontal solve before make_pairs");
    const NrScratch sc{d_nrpart_.data(), d_nrcnt_.data()};
    for (const Level &L : levels_) {
        launch_pdl(mf_fassemble_nr_kernel<NR>, (unsigned)L.fasm_nr.ctas, 256, 0, st, v, L.fasm_nr, gptr_, gsrc_, t,
                   d_wb_.data(), sys_done, front_sys);
        if (L.fwd_nr.ctas > 0)
            launch_pdl(mf_forward_nr_kernel<NR>, (unsigned)L.fwd_nr.ctas, 256, smem, st, v, L.fwd_nr,
                       (const float2 *)d_Fp_.data(), d_wb_.data(), sc, sys_done, front_sys);
        LSS_LAUNCH_CHECK();
    }
    for (int h = (int)levels_.size() - 1; h >= 0; --h) {
        const Level &L = levels_[h];
        launch_pdl(mf_backward_nr_kernel<NR>, (unsigned)L.bwd_nr.ctas, 256, smem, st, v, L.bwd_nr,
                   (const float2 *)d_Fp_.data(), (const float2 *)d_wb_.data(), d_xb_.data(), sc, sys_done, front_sys);
        LSS_LAUNCH_CHECK();
    }
    launch_pdl(mf_scatter_nr_kernel<NR>, (unsigned)(((int64_t)sym_.npos * NR + 255) / 256), 256, 0, st, v, S,
               (const float2 *)d_xb_.data(), z);
    LSS_LAUNCH_CHECK();
}

}  // namespace lss
