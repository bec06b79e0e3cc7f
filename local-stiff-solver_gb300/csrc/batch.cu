// Kernels of the batched PCG (sm_103a): every launch covers all systems and
// all BK right-hand sides of a batch (batch.hpp).  Block size 3.
//
// Precision.  GB300 issues 2 FP64 FMAs per clock and SM against 128 FP32
// FMAs, and a batch multiplies the vector work by BK, so the PCG vectors x,
// r, p and z are double-float pairs (hi, lo) of FP32 (the FP64 entry's 8
// bytes, about 2^-48 relative) and every vector operation, dot product and the
// operator product A p run on the FP32 pipe with error-free products and
// compensated sums; the per-lane scalars alpha, beta, gamma and the stopping
// tests are FP64, and the final residual b - A x is checked in FP64.  The
// MAS apply is FP32, as in the single-system mixed mode; the preconditioner's
// residual r - A z is FP32 except on the rows of stiff DOFs (double-float).
//
// Work decomposition.  A chunk is up to BATCH_CHUNK consecutive MAS
// partitions of one system (<= 32 block rows each); row kernels run one CTA
// per chunk, and a system whose lanes have all stopped skips its chunks.
// Per-lane sums are reduced per CTA, written to a partials slot of the chunk,
// and summed in chunk order by the last CTA of the system to arrive.
#include <cfloat>

#include "batch.hpp"
#include "bulk.cuh"
#include "device_common.cuh"
#include "spmv.cuh"

namespace lss {
namespace bk {

constexpr int BD = 3;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float2 df_from(double v)
{
    const float h = (float)v;
    return make_float2(h, (float)(v - (double)h));
}
__device__ __forceinline__ double df_val(float2 a) { return (double)a.x + (double)a.y; }

// (ah, al) * b for an FP32 pair and a double-float scalar (bh, bl)
__device__ __forceinline__ float2 df_mul(float2 a, float bh, float bl)
{
    const float p = __fmul_rn(a.x, bh);
    const float e = __fmaf_rn(a.x, bh, -p);
    const float lo = __fadd_rn(e, __fmaf_rn(a.x, bl, __fmul_rn(a.y, bh)));
    const float s = __fadd_rn(p, lo);
    return make_float2(s, __fsub_rn(lo, __fsub_rn(s, p)));
}
// a + b for pairs, renormalised
__device__ __forceinline__ float2 df_sum(float2 a, float2 b)
{
    float h = a.x, l = a.y;
    df_add(h, l, b.x, b.y);
    const float s = __fadd_rn(h, l);
    return make_float2(s, __fsub_rn(l, __fsub_rn(s, h)));
}

struct Chunk {
    int sys;
    int32_t r0, r1;  // block rows
    int32_t p0, p1;  // MAS partitions
};

__device__ __forceinline__ Chunk chunk_of(const BatchDev &B, int c)
{
    Chunk k;
    k.sys = B.chunk_sys[c];
    k.p0 = B.chunk_p0[c];
    k.p1 = B.chunk_p0[c + 1];
    k.r0 = B.part_off[k.p0];
    k.r1 = B.part_off[k.p1];
    return k;
}

// Per-lane totals of NV values over the chunks of one system.  part[v] holds
// the CTA's sum of value v for right-hand side threadIdx.x (threads < BK).
// Returns true in the threads < BK of the last CTA of the system to arrive,
// where tot[v] is the system's sum in chunk order; the counter is reset.
template <int NV>
__device__ bool sys_finish(const BatchDev &B, int c, int sys, const double (&part)[NV], double (&tot)[NV])
{
    __shared__ bool last;
    const int t = threadIdx.x;
    if (t < BK)
#pragma unroll
        for (int v = 0; v < NV; ++v) B.partials[((int64_t)c * BK + t) * NV + v] = part[v];
    __threadfence();
    __syncthreads();
    if (t == 0) {
        const unsigned arrived = atomicAdd(B.counters + sys, 1u);
        last = arrived == (unsigned)(B.sys_chunk0[sys + 1] - B.sys_chunk0[sys] - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    if (t < BK) {
#pragma unroll
        for (int v = 0; v < NV; ++v) tot[v] = 0.0;
        for (int q = B.sys_chunk0[sys]; q < B.sys_chunk0[sys + 1]; ++q)
#pragma unroll
            for (int v = 0; v < NV; ++v) tot[v] += __ldcg(B.partials + ((int64_t)q * BK + t) * NV + v);
    }
    if (t == 0) B.counters[sys] = 0u;
    return t < BK;
}

// lanes of system s all stopped -> sys_done[s] (called by the finishing CTA)
__device__ void mark_system(const BatchDev &B, int sys)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        int all = 1;
        for (int k = 0; k < BK; ++k) all &= B.lane[sys * BK + k].done != 0;
        const_cast<int *>(B.sys_done)[sys] = all;
    }
}

// ---------------------------------------------------------------- A p, p.Ap, alpha

// One warp per block row: half-warp h takes the row's blocks l = h, h + 2, ...,
// lane k of the half the right-hand side k; the 9 values of a block are
// broadcast to the half-warp, p and A p move as 128-byte lines of 16 pairs.
// The row's column indices are loaded once (lane l: block l) and handed out
// by shuffles, U blocks per half-warp at a time, so that their loads are in
// flight together.
template <int U, typename Blk>
__device__ __forceinline__ void row_blocks(const BatchDev &B, int32_t b, int32_t len, int lane, Blk blk)
{
    const int h = lane >> 4;
    for (int32_t l0 = 0; l0 < len; l0 += 32) {
        const int n = min(32, len - l0);
        const int32_t cj = lane < n ? B.cols[b + l0 + lane] : 0;
        for (int j0 = 0; j0 < n; j0 += 2 * U) {
            int32_t J[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int l = j0 + 2 * u + h;
                ok[u] = l < n;
                J[u] = __shfl_sync(FULL, cj, l & 31);
            }
            blk(l0 + j0 + h, J, ok);
        }
    }
}

__global__ void __launch_bounds__(256) spmm_alpha_kernel(BatchDev B, const float2 *__restrict__ p,
                                                         float2 *__restrict__ ap)
{
    constexpr int U = 2;
    const Chunk ch = chunk_of(B, blockIdx.x);
    if (B.sys_done[ch.sys]) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = lane >> 4, k = lane & 15;
    float dh = 0.f, dl = 0.f;
    for (int32_t I = ch.r0 + w; I < ch.r1; I += 8) {
        const int32_t b = B.rows[I], len = B.rows[I + 1] - b;
        const float2 *__restrict__ v = B.vals_df + (int64_t)b * 9;
        // one double-float accumulator per (block slot u, row r): 3 U independent chains
        float uh[U][BD], ul[U][BD];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int r = 0; r < BD; ++r) uh[u][r] = ul[u][r] = 0.f;
        row_blocks<U>(B, b, len, lane, [&](int l, const int32_t (&J)[U], const bool (&ok)[U]) {
            float2 x[U][BD], a[U][BD * BD];
#pragma unroll
            for (int u = 0; u < U; ++u) {
#pragma unroll
                for (int c = 0; c < BD; ++c)
                    x[u][c] = ok[u] ? p[((int64_t)J[u] * BD + c) * BK + k] : make_float2(0.f, 0.f);
#pragma unroll
                for (int e = 0; e < BD * BD; ++e)
                    a[u][e] = ok[u] ? __ldg(v + (int64_t)e * len + l + 2 * u) : make_float2(0.f, 0.f);
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
#pragma unroll
                for (int r = 0; r < BD; ++r)
#pragma unroll
                    for (int c = 0; c < BD; ++c)
                        df_fma(uh[u][r], ul[u][r], a[u][r * BD + c].x, a[u][r * BD + c].y, x[u][c].x, x[u][c].y);
        });
        float sh[BD], sl[BD];
#pragma unroll
        for (int r = 0; r < BD; ++r) {
            sh[r] = uh[0][r];
            sl[r] = ul[0][r];
#pragma unroll
            for (int u = 1; u < U; ++u) df_add(sh[r], sl[r], uh[u][r], ul[u][r]);
        }
#pragma unroll
        for (int r = 0; r < BD; ++r) {
            const float bh = __shfl_xor_sync(FULL, sh[r], 16), bl = __shfl_xor_sync(FULL, sl[r], 16);
            df_add(sh[r], sl[r], bh, bl);
        }
        if (h == 0) {
#pragma unroll
            for (int r = 0; r < BD; ++r) {
                const int64_t e = ((int64_t)I * BD + r) * BK + k;
                const float s = __fadd_rn(sh[r], sl[r]);
                ap[e] = make_float2(s, __fsub_rn(sl[r], __fsub_rn(s, sh[r])));
                const float2 pk = p[e];
                df_fma(dh, dl, pk.x, pk.y, sh[r], sl[r]);
            }
        }
    }
    __shared__ double red[8][BK];
    if (h == 0) red[w][k] = (double)dh + (double)dl;
    __syncthreads();
    double part[1] = {0.0}, tot[1];
    if (threadIdx.x < BK)
        for (int q = 0; q < 8; ++q) part[0] += red[q][threadIdx.x];
    if (sys_finish<1>(B, blockIdx.x, ch.sys, part, tot)) {
        BatchLane &L = B.lane[ch.sys * BK + threadIdx.x];
        if (!L.done) {
            // GPUHybrid.cu:1458-1480 per lane
            L.iter += 1;
            const double pAp = tot[0];
            L.pAp = pAp;
            const double alpha = L.gamma / pAp;
            if (pAp == 0.0) L.done = STOP_ZERO_PAP;
            else if (!(alpha == alpha) || isinf(alpha)) L.done = STOP_NONFINITE;
            else if (alpha <= 0.0) L.done = STOP_NEGATIVE_ALPHA;
            else if (alpha < DBL_MIN) L.done = STOP_SUBNORMAL_ALPHA;
            else L.alpha = alpha;
        }
    }
}

// ---------------------------------------------------------------- x, r, rr, stopping tests

__global__ void __launch_bounds__(256) update_xr_kernel(BatchDev B, float2 *__restrict__ x, float2 *__restrict__ r,
                                                        const float2 *__restrict__ p, const float2 *__restrict__ ap)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    if (B.sys_done[ch.sys]) return;
    const int k = threadIdx.x & (BK - 1);
    const BatchLane &L = B.lane[ch.sys * BK + k];
    const bool live = !L.done;
    const double alpha = L.alpha;
    const float ah = (float)alpha, al = (float)(alpha - (double)ah);
    float rh = 0.f, rl = 0.f;
    const int64_t e1 = (int64_t)ch.r1 * BD * BK;
#pragma unroll 4
    for (int64_t e = (int64_t)ch.r0 * BD * BK + threadIdx.x; e < e1; e += blockDim.x) {
        if (!live) continue;
        x[e] = df_sum(x[e], df_mul(p[e], ah, al));
        const float2 d = df_mul(ap[e], ah, al);
        const float2 ri = df_sum(r[e], make_float2(-d.x, -d.y));
        r[e] = ri;
        df_fma(rh, rl, ri.x, ri.y, ri.x, ri.y);
    }
    __shared__ double red[16][BK];
    red[threadIdx.x >> 4][k] = (double)rh + (double)rl;
    __syncthreads();
    double part[1] = {0.0}, tot[1];
    if (threadIdx.x < BK)
        for (int q = 0; q < 16; ++q) part[0] += red[q][threadIdx.x];
    const bool fin = sys_finish<1>(B, blockIdx.x, ch.sys, part, tot);
    if (fin) {
        BatchLane &M = B.lane[ch.sys * BK + threadIdx.x];
        if (!M.done) {
            // GPUHybrid.cu:1482-1496 per lane
            const double rr = tot[0];
            M.rr = rr;
            if (!(rr == rr) || isinf(rr)) M.done = STOP_NONFINITE;
            else if (M.rel_eps > 0 && rr / M.bb < M.rel_eps) M.done = STOP_CONVERGED_REL;
            else if (M.abs_eps > 0 && rr < M.abs_eps) M.done = STOP_CONVERGED_ABS;
            else if (M.iter >= M.max_iter) M.done = STOP_MAX_ITER;
        }
    }
    // the finishing CTA (threads < BK returned true there) marks the system
    __shared__ int fin_cta;
    if (threadIdx.x == 0) fin_cta = 0;
    __syncthreads();
    if (fin && threadIdx.x == 0) fin_cta = 1;
    __syncthreads();
    if (fin_cta) mark_system(B, ch.sys);
}

// p = z + beta p
__global__ void __launch_bounds__(256) update_p_kernel(BatchDev B, float2 *__restrict__ p, const float2 *__restrict__ z)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    if (B.sys_done[ch.sys]) return;
    const int k = threadIdx.x & (BK - 1);
    const BatchLane &L = B.lane[ch.sys * BK + k];
    if (L.done) return;  // uniform per thread (k fixed): no barrier below
    const double beta = L.beta;
    const float bh = (float)beta, bl = (float)(beta - (double)bh);
    const int64_t e1 = (int64_t)ch.r1 * BD * BK;
#pragma unroll 4
    for (int64_t e = (int64_t)ch.r0 * BD * BK + threadIdx.x; e < e1; e += blockDim.x)
        p[e] = df_sum(z[e], df_mul(p[e], bh, bl));
}

// p = z (the first direction)
__global__ void __launch_bounds__(256) copy_pairs_kernel(BatchDev B, float2 *__restrict__ dst,
                                                         const float2 *__restrict__ src)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    const int64_t e1 = (int64_t)ch.r1 * BD * BK;
    for (int64_t e = (int64_t)ch.r0 * BD * BK + threadIdx.x; e < e1; e += blockDim.x) dst[e] = src[e];
}

// ---------------------------------------------------------------- true residual (FP64)

// r = b - A x in FP64 (values and x FP64), rr per lane; mode 0: the start of
// a solve or a restart (r also replaces the recurrence residual), mode 1: the
// final check (rr only)
__global__ void __launch_bounds__(256) residual64_kernel(BatchDev B, const double *__restrict__ bvec,
                                                         const double *__restrict__ x, float2 *__restrict__ r,
                                                         int mode, double *__restrict__ out_rr)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = lane >> 4, k = lane & 15;
    double acc_rr = 0.0;
    for (int32_t I = ch.r0 + w; I < ch.r1; I += 8) {
        const int32_t b = B.rows[I], len = B.rows[I + 1] - b;
        const double *__restrict__ v = B.vals + (int64_t)b * 9;
        double y[BD] = {0.0, 0.0, 0.0};
        row_blocks<2>(B, b, len, lane, [&](int l, const int32_t (&J)[2], const bool (&ok)[2]) {
            double xv[2][BD], a[2][BD * BD];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
#pragma unroll
                for (int c = 0; c < BD; ++c) xv[u][c] = ok[u] ? x[((int64_t)J[u] * BD + c) * BK + k] : 0.0;
#pragma unroll
                for (int e = 0; e < BD * BD; ++e) a[u][e] = ok[u] ? __ldg(v + (int64_t)e * len + l + 2 * u) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int rr = 0; rr < BD; ++rr)
#pragma unroll
                    for (int c = 0; c < BD; ++c) y[rr] += a[u][rr * BD + c] * xv[u][c];
        });
#pragma unroll
        for (int rr = 0; rr < BD; ++rr) y[rr] += __shfl_xor_sync(FULL, y[rr], 16);
        if (h == 0) {
#pragma unroll
            for (int rr = 0; rr < BD; ++rr) {
                const int64_t e = ((int64_t)I * BD + rr) * BK + k;
                const double ri = bvec[e] - y[rr];
                if (mode == 0) r[e] = df_from(ri);
                acc_rr += ri * ri;
            }
        }
    }
    __shared__ double red[8][BK];
    if (h == 0) red[w][k] = acc_rr;
    __syncthreads();
    double part[1] = {0.0}, tot[1];
    if (threadIdx.x < BK)
        for (int q = 0; q < 8; ++q) part[0] += red[q][threadIdx.x];
    if (sys_finish<1>(B, blockIdx.x, ch.sys, part, tot)) out_rr[ch.sys * BK + threadIdx.x] = tot[0];
}

// ---------------------------------------------------------------- MAS (FP32), BK right-hand sides

// Level vectors: item-major, [(item * BD + c) * BK + k].

// Segment sums of one bank (cnt <= 32 items of BD x BK values each, item j
// contributing to aggregate key[j] < ncc) into out[a * BD * BK ...], one warp:
// lane e owns the values e and e + 32 of the BD * BK = 48 of an item; the
// per-aggregate sums collect in the warp's shared rows acc[a][48].
template <typename XT>
__device__ __forceinline__ void bank_restrict(const XT *__restrict__ x, const uint8_t *__restrict__ key, int cnt,
                                              int ncc, float *__restrict__ out, float *__restrict__ acc, int lane)
{
    constexpr int W = BD * BK;  // 48
    for (int q = lane; q < ncc * W; q += 32) acc[q] = 0.f;
    __syncwarp();
    for (int j = 0; j < cnt; ++j) {
        const int a = key[j];
        const XT *xj = x + (int64_t)j * W;
        float v0, v1 = 0.f;
        if constexpr (sizeof(XT) == 8) {
            v0 = reinterpret_cast<const float2 *>(xj)[lane].x;
            if (lane < W - 32) v1 = reinterpret_cast<const float2 *>(xj)[lane + 32].x;
        } else {
            v0 = (float)xj[lane];
            if (lane < W - 32) v1 = (float)xj[lane + 32];
        }
        acc[a * W + lane] += v0;
        if (lane < W - 32) acc[a * W + lane + 32] += v1;
    }
    __syncwarp();
    for (int q = lane; q < ncc * W; q += 32) out[q] = acc[q];
    __syncwarp();
}

// level 0 -> 1: per part, the sums of its nodes' entries per level-1 aggregate
// (warp per part, eight warps per CTA = the chunk's parts)
template <typename XT>
__global__ void __launch_bounds__(256) restrict0_kernel(BatchDev B, MasDev m, const XT *__restrict__ xin,
                                                        float *__restrict__ v)
{
    __shared__ float acc_all[8][32 * BD * BK];
    const Chunk ch = chunk_of(B, blockIdx.x);
    if (B.sys_done[ch.sys]) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float *v1 = v + m.voff[1] * BK;
    const int32_t p = ch.p0 + w;
    if (p >= ch.p1) return;
    const int ncc = m.ccnt0[p];
    if (ncc == 0) return;
    const int32_t lo = m.part_off[p], cnt = m.part_off[p + 1] - lo;
    bank_restrict<XT>(xin + (int64_t)lo * BD * BK, m.key0 + lo, cnt, ncc, v1 + (int64_t)m.cbase0[p] * BD * BK,
                      acc_all[w], lane);
}

// level l -> l + 1 (warp per level-l bank)
__global__ void __launch_bounds__(256) restrict_kernel(MasDev m, int l, float *__restrict__ v)
{
    __shared__ float acc_all[8][32 * BD * BK];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t g = (int64_t)blockIdx.x * 8 + w;
    if (g >= m.nbanks[l]) return;
    const int ncc = m.ccnt[l][g];
    if (ncc == 0) return;
    bank_restrict<float>(v + (m.voff[l] + g * 32 * BD) * BK, m.key[l] + g * 32, 32, ncc,
                         v + (m.voff[l + 1] + (int64_t)m.cbase[l][g] * BD) * BK, acc_all[w], lane);
}

// Y (96 x BK) = Inv (96 x 96) X (96 x BK) for a sequence of banks, one CTA of
// eight warps per sequence.  Per bank, the copy engine brings the inverse's
// 147 stored diagonals (the tiles (c, c2 >= c) of mas_tile_elems, 18,816
// bytes) and the bank's X block into a shared-memory stage (cp.async.bulk,
// two stages: bank i + 1 arrives while bank i computes); the CTA expands the
// diagonals into the full 96 x 96 matrix S (column-major, rows and columns in
// node-major order q = 3 node + component, the order of X) and multiplies:
// warp w takes the right-hand sides 8 (w & 1) .. + 7 and the columns
// 24 (w >> 1) .. + 23, lane (g, h) the rows 12 g .. 12 g + 11 and the
// right-hand sides 8 (w & 1) + 2 h, + 1 -- per column three float4 of S, one
// vector load of X, 24 FMAs.  The four column quarters meet in shared memory
// (in the stage just consumed), summed in quarter order.
constexpr int BANK_THREADS = 256;
constexpr int NB = 32 * BD;                             // 96
constexpr int TILE_FLOATS = 3 * 17 * 32 + 3 * 32 * 32;  // 4704 (mas_tile_elems(3))
constexpr int TILE_BYTES = TILE_FLOATS * 4;             // 18,816
constexpr int XBUF_BYTES = 32 * BD * BK * 8;            // 32 nodes of pairs: 12,288
constexpr int STAGE_BYTES = TILE_BYTES + XBUF_BYTES + 512;  // + pad: the partial sums need 25,600
constexpr int RSTRIDE = NB * BK + 64;                   // partial sums of one column quarter (+ skew)
constexpr int BANK_SMEM = NB * NB * 4 + 2 * STAGE_BYTES + 16;
// pre-expanded banks (level 0): a stage holds the full 96 x 96 matrix, then X
constexpr int FULL_BYTES = NB * NB * 4;                  // 36,864
constexpr int STAGE_FULL_BYTES = FULL_BYTES + XBUF_BYTES;  // 49,152
constexpr int BANK_SMEM_FULL = 2 * STAGE_FULL_BYTES + 16;
static_assert(4 * RSTRIDE * 4 <= STAGE_FULL_BYTES && STAGE_FULL_BYTES % 16 == 0, "full-bank stages");
static_assert(4 * RSTRIDE * 4 <= STAGE_BYTES, "the partial sums fit in a stage");
static_assert(STAGE_BYTES % 16 == 0 && TILE_BYTES % 16 == 0, "bulk copies need 16-byte alignment");

struct BankSmem {
    float *S;            // 96 x 96 (stored diagonals expanded here; unused with pre-expanded banks)
    unsigned char *st;   // 2 stages: the bank's inverse (tiles or the full matrix), then X
    uint64_t *bar;
};

template <bool FULL>
__device__ __forceinline__ BankSmem bank_smem(unsigned char *raw)
{
    BankSmem b;
    b.S = reinterpret_cast<float *>(raw);
    b.st = FULL ? raw : raw + NB * NB * 4;
    b.bar = reinterpret_cast<uint64_t *>(b.st + 2 * (FULL ? STAGE_FULL_BYTES : STAGE_BYTES));
    return b;
}

// stored diagonal D (0..146) -> tile (c, c2) and diagonal d
__device__ __forceinline__ void diag_of(int D, int &c, int &c2, int &d)
{
    if (D < 81) {
        c = 0;
        if (D < 17) { c2 = 0; d = D; }
        else { c2 = 1 + (D - 17) / 32; d = (D - 17) % 32; }
    } else if (D < 130) {
        c = 1;
        if (D < 98) { c2 = 1; d = D - 81; }
        else { c2 = 2; d = D - 98; }
    } else {
        c = 2; c2 = 2; d = D - 130;
    }
}

// tile diagonals (shared) -> S[col * 96 + row]; warp w takes diagonals w, w + 8, ...
// Diagonal tile, d = 16: entry [r][r + 16] belongs to row r only (row r + 16
// has its own stored value), as in the single-system MAS.
__device__ __forceinline__ void expand_tile(const float *__restrict__ T, float *__restrict__ S, int w, int lane)
{
    for (int D = w; D < 147; D += BANK_THREADS / 32) {
        int c, c2, d;
        diag_of(D, c, c2, d);
        const float a = T[D * 32 + lane];
        const int qi = 3 * lane + c, qj = 3 * ((lane + d) & 31) + c2;
        S[qj * NB + qi] = a;
        if (c != c2 || (d != 0 && d != 16)) S[qi * NB + qj] = a;
    }
}

// stored diagonals -> full column-major matrices, once per factorization
// (one CTA per bank)
__global__ void __launch_bounds__(BANK_THREADS) expand_banks_kernel(const float *__restrict__ tiles,
                                                                    float *__restrict__ full)
{
    const int64_t b = blockIdx.x;
    expand_tile(tiles + b * TILE_FLOATS, full + b * NB * NB, threadIdx.x >> 5, threadIdx.x & 31);
}

template <typename XT>
__device__ __forceinline__ void bank_mma(const float *__restrict__ S, const float *__restrict__ X, int ncol, int w,
                                         int lane, float (&acc)[12][2])
{
    const int rh = w & 1, kq = w >> 1, g = lane >> 2, h = lane & 3;
#pragma unroll
    for (int j = 0; j < 12; ++j) acc[j][0] = acc[j][1] = 0.f;
    const int q0 = 24 * kq, q1 = min(q0 + 24, ncol);
    const int xo = 8 * rh + 2 * h;
#pragma unroll 4
    for (int q = q0; q < q1; ++q) {
        const float4 *col = reinterpret_cast<const float4 *>(S + q * NB + 12 * g);
        const float4 a0 = col[0], a1 = col[1], a2 = col[2];
        float x0, x1;
        if constexpr (sizeof(XT) == 8) {
            const float4 xv = *reinterpret_cast<const float4 *>(X + 2 * (q * BK + xo));
            x0 = xv.x;
            x1 = xv.z;
        } else {
            const float2 xv = *reinterpret_cast<const float2 *>(X + q * BK + xo);
            x0 = xv.x;
            x1 = xv.y;
        }
        const float a[12] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w, a2.x, a2.y, a2.z, a2.w};
#pragma unroll
        for (int j = 0; j < 12; ++j) {
            acc[j][0] = fmaf(a[j], x0, acc[j][0]);
            acc[j][1] = fmaf(a[j], x1, acc[j][1]);
        }
    }
}

// partial sums -> R[kq][row][k] (skewed by 8 per row group of 12)
__device__ __forceinline__ void bank_store_partials(float *__restrict__ R, int w, int lane, const float (&acc)[12][2])
{
    const int rh = w & 1, kq = w >> 1, g = lane >> 2, h = lane & 3;
#pragma unroll
    for (int j = 0; j < 12; ++j) {
        const int row = 12 * g + j;
        *reinterpret_cast<float2 *>(R + kq * RSTRIDE + row * BK + 8 * g + 8 * rh + 2 * h) =
            make_float2(acc[j][0], acc[j][1]);
    }
}

__device__ __forceinline__ float bank_result(const float *__restrict__ R, int row, int k)
{
    const int o = row * BK + 8 * (row / 12) + k;
    return ((R[o] + R[RSTRIDE + o]) + R[2 * RSTRIDE + o]) + R[3 * RSTRIDE + o];
}

// The bank pipeline of one CTA (BANK_THREADS threads): jobs 0 .. nj - 1,
// job(i, tile, x, cnt) names the bank's inverse, its X block and item count,
// epi(i, R, cnt) consumes the result rows 0 .. 3 cnt - 1 (R as bank_result
// reads it; thread t takes rows t / 16 + 16 j, right-hand side t % 16).
// Returns false, with *err set, when a copy did not arrive within the poll
// limit.
// FULL: the banks were expanded once into full column-major matrices (the
// layout expand_tile writes), which the copy engine brings instead of the
// stored diagonals -- twice the bytes, no expansion per apply.
template <typename XT, bool FULL, typename Job, typename Epi>
__device__ bool bank_pipeline(unsigned char *raw, int nj, Job job, Epi epi, int *err)
{
    constexpr int STG = FULL ? STAGE_FULL_BYTES : STAGE_BYTES;
    constexpr int MATB = FULL ? FULL_BYTES : TILE_BYTES;
    const BankSmem sm = bank_smem<FULL>(raw);
    __shared__ int s_fail;
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    auto issue = [&](int i, int b) {
        const float *tile;
        const XT *x;
        int cnt;
        job(i, tile, x, cnt);
        const uint32_t xbytes = (uint32_t)cnt * BD * BK * sizeof(XT);
        unsigned char *stage = sm.st + b * STG;
        mbar_arrive_expect_tx(sm.bar + b, MATB + xbytes);
        bulk_load(stage, tile, MATB, sm.bar + b);
        bulk_load(stage + MATB, x, xbytes, sm.bar + b);
    };
    if (t == 0) {
        mbar_init(sm.bar, 1);
        mbar_init(sm.bar + 1, 1);
        mbar_init_fence();
        s_fail = 0;
    }
    __syncthreads();
    if (t == 0) {
        issue(0, 0);
        if (nj > 1) issue(1, 1);
    }
    for (int i = 0; i < nj; ++i) {
        const int b = i & 1;
        if (t == 0 && !mbar_wait_bounded(sm.bar + b, (i >> 1) & 1)) s_fail = 1;
        __syncthreads();
        if (s_fail) {
            if (t == 0) {
                atomicExch(err, 1);
                // let the copies in flight land before the CTA's shared memory goes
                mbar_wait_bounded(sm.bar + b, (i >> 1) & 1);
                if (i + 1 < nj) mbar_wait_bounded(sm.bar + (b ^ 1), ((i + 1) >> 1) & 1);
            }
            return false;
        }
        if (t != 0) (void)mbar_test(sm.bar + b, (i >> 1) & 1);  // acquire the completed phase in every thread
        const float *tile;
        const XT *xsrc;
        int cnt;
        job(i, tile, xsrc, cnt);
        unsigned char *stage = sm.st + b * STG;
        const float *S = reinterpret_cast<const float *>(stage);
        if (!FULL) {
            expand_tile(reinterpret_cast<const float *>(stage), sm.S, w, lane);
            __syncthreads();
            S = sm.S;
        }
        float acc[12][2];
        bank_mma<XT>(S, reinterpret_cast<const float *>(stage + MATB), 3 * cnt, w, lane, acc);
        __syncthreads();
        float *R = reinterpret_cast<float *>(stage);  // the stage is consumed: partial sums
        bank_store_partials(R, w, lane, acc);
        __syncthreads();
        epi(i, R, cnt);
        __syncthreads();
        if (t == 0 && i + 2 < nj) {
            proxy_async_fence();
            issue(i + 2, b);
        }
    }
    return true;
}

// u_1 += P (u_2 + P (u_3 + ...)) for every level-1 item, stopping where a
// system has no coarser level (ccnt == 0)
__global__ void __launch_bounds__(256) prolong_kernel(MasDev m, float *__restrict__ u)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)m.nitems[1] * BD * BK;
    if (t >= total) return;
    const int64_t item1 = t / (BD * BK);
    const int rest = (int)(t % (BD * BK));
    int64_t item[MAS_MAXL];
    item[1] = item1;
    int top = 1;
    for (int l = 1; l + 1 < m.L; ++l) {
        const int64_t bank = item[l] >> 5;
        if (m.ccnt[l][bank] == 0) break;
        item[l + 1] = m.cbase[l][bank] + m.key[l][item[l]];
        top = l + 1;
    }
    float acc = u[(m.voff[top] + item[top] * BD) * BK + rest];
    for (int l = top - 1; l >= 1; --l) acc = u[(m.voff[l] + item[l] * BD) * BK + rest] + acc;
    u[(m.voff[1] + item1 * BD) * BK + rest] = acc;
}

// coarse banks: u = Inv_l v, all levels in one launch (banks grid-strided)
__global__ void __launch_bounds__(BANK_THREADS) symv_coarse_kernel(MasDev m, const float *__restrict__ invc,
                                                          const float *__restrict__ v, float *__restrict__ u,
                                                          int *err)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int nj = (int)((m.ncoarse - blockIdx.x + gridDim.x - 1) / gridDim.x);
    if (nj <= 0) return;
    auto locate = [&](int i, int64_t &gb, int64_t &at) {
        gb = blockIdx.x + (int64_t)i * gridDim.x;
        int l = 1;
        while (l + 1 < m.L && gb >= m.boff[l + 1]) ++l;
        at = (m.voff[l] + (gb - m.boff[l]) * 32 * BD) * BK;
    };
    auto job = [&](int i, const float *&tile, const float *&x, int &cnt) {
        int64_t gb, at;
        locate(i, gb, at);
        tile = invc + gb * TILE_FLOATS;
        x = v + at;
        cnt = 32;
    };
    auto epi = [&](int i, const float *R, int) {
        int64_t gb, at;
        locate(i, gb, at);
        const int k = threadIdx.x & (BK - 1);
#pragma unroll 4
        for (int row = threadIdx.x >> 4; row < NB; row += BANK_THREADS / BK) u[at + row * BK + k] = bank_result(R, row, k);
    };
    bank_pipeline<float, false>(smem_raw, nj, job, epi, err);
}

// level 0: z = omega (Inv_0 x + u_1) (+ z with acc), as pairs; optional
// gamma = r.z per lane (dot 1: initial gamma; dot 2: beta and the new gamma).
// One CTA per chunk, its parts in sequence through the bank pipeline.
template <typename XT, bool ACC, int DOT>
__global__ void __launch_bounds__(BANK_THREADS) symv0_kernel(BatchDev B, MasDev m, const float *__restrict__ inv0,
                                                    const float *__restrict__ u, const XT *__restrict__ xin,
                                                    float2 *__restrict__ z, const float2 *__restrict__ rdot)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const Chunk ch = chunk_of(B, blockIdx.x);
    if (B.sys_done[ch.sys]) return;
    const double om = B.omega[ch.sys];
    const float oh = (float)om, ol = (float)(om - (double)oh);
    const float *u1 = u + m.voff[1] * BK;
    const int k = threadIdx.x & (BK - 1);
    float dh = 0.f, dl = 0.f;
    auto job = [&](int i, const float *&tile, const XT *&x, int &cnt) {
        const int32_t p = ch.p0 + i, lo = m.part_off[p];
        tile = inv0 + (int64_t)p * NB * NB;  // pre-expanded
        x = xin + (int64_t)lo * BD * BK;
        cnt = m.part_off[p + 1] - lo;
    };
    auto epi = [&](int i, const float *R, int cnt) {
        constexpr int RPT = NB / (BANK_THREADS / BK);  // rows per thread: 6
        const int32_t p = ch.p0 + i, lo = m.part_off[p];
        const bool coarse = m.L > 1 && m.ccnt0[p] > 0;
        const int32_t cb = coarse ? m.cbase0[p] : 0;
        const int r0 = threadIdx.x >> 4, nrow = 3 * cnt;
        // every gather of the thread's rows first, then the arithmetic
        float cu[RPT];
        float2 zo[RPT], rv[RPT];
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const int row = r0 + j * (BANK_THREADS / BK);
            cu[j] = 0.f;
            zo[j] = rv[j] = make_float2(0.f, 0.f);
            if (row >= nrow) continue;
            const int node = row / 3, c = row - 3 * node;
            const int64_t e = ((int64_t)lo * BD + row) * BK + k;
            if (coarse) cu[j] = u1[((int64_t)(cb + m.key0[lo + node]) * BD + c) * BK + k];
            if (ACC) zo[j] = z[e];
            if (DOT) rv[j] = rdot[e];
        }
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const int row = r0 + j * (BANK_THREADS / BK);
            if (row >= nrow) continue;
            const int64_t e = ((int64_t)lo * BD + row) * BK + k;
            float2 val = df_mul(make_float2(bank_result(R, row, k) + cu[j], 0.f), oh, ol);
            if (ACC) val = df_sum(zo[j], val);
            z[e] = val;
            if (DOT) df_fma(dh, dl, rv[j].x, rv[j].y, val.x, val.y);
        }
    };
    if (!bank_pipeline<XT, true>(smem_raw, ch.p1 - ch.p0, job, epi, B.err)) return;
    if (DOT) {
        __shared__ double red[BANK_THREADS / BK][BK];
        red[threadIdx.x >> 4][k] = (double)dh + (double)dl;
        __syncthreads();
        double part[1] = {0.0}, tot[1];
        if (threadIdx.x < BK)
            for (int q = 0; q < BANK_THREADS / BK; ++q) part[0] += red[q][threadIdx.x];
        if (sys_finish<1>(B, blockIdx.x, ch.sys, part, tot)) {
            BatchLane &L = B.lane[ch.sys * BK + threadIdx.x];
            if (!L.done) {
                if (DOT == 2) L.beta = tot[0] / L.gamma;  // GPUHybrid.cu:1501-1504
                L.gamma = tot[0];
            }
        }
    }
}

// ---------------------------------------------------------------- preconditioner residual

// w = r - A z in FP32 (values FP32, r and z by their high words), except block
// rows flagged precise: double-float (values as pairs, r and z as pairs)
__global__ void __launch_bounds__(256) residual32_kernel(BatchDev B, const float2 *__restrict__ r,
                                                         const float2 *__restrict__ z, float *__restrict__ wout)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    if (B.sys_done[ch.sys]) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = lane >> 4, k = lane & 15;
    for (int32_t I = ch.r0 + w; I < ch.r1; I += 8) {
        const int32_t b = B.rows[I], len = B.rows[I + 1] - b;
        const bool precise = B.precise && B.precise[I];
        if (!precise) {
            constexpr int U = 4;
            const float *__restrict__ v = B.vals32 + (int64_t)b * 9;
            float y[BD] = {0.f, 0.f, 0.f};
            row_blocks<U>(B, b, len, lane, [&](int l, const int32_t (&J)[U], const bool (&ok)[U]) {
                float xv[U][BD], a[U][BD * BD];
#pragma unroll
                for (int u = 0; u < U; ++u) {
#pragma unroll
                    for (int c = 0; c < BD; ++c) xv[u][c] = ok[u] ? z[((int64_t)J[u] * BD + c) * BK + k].x : 0.f;
#pragma unroll
                    for (int e = 0; e < BD * BD; ++e) a[u][e] = ok[u] ? __ldg(v + (int64_t)e * len + l + 2 * u) : 0.f;
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int rr = 0; rr < BD; ++rr)
#pragma unroll
                        for (int c = 0; c < BD; ++c) y[rr] += a[u][rr * BD + c] * xv[u][c];
            });
#pragma unroll
            for (int rr = 0; rr < BD; ++rr) y[rr] += __shfl_xor_sync(FULL, y[rr], 16);
            if (h == 0)
#pragma unroll
                for (int rr = 0; rr < BD; ++rr) {
                    const int64_t e = ((int64_t)I * BD + rr) * BK + k;
                    wout[e] = r[e].x - y[rr];
                }
        } else {
            constexpr int U = 2;
            const float2 *__restrict__ v = B.vals_df + (int64_t)b * 9;
            float sh[BD] = {0.f, 0.f, 0.f}, sl[BD] = {0.f, 0.f, 0.f};
            row_blocks<U>(B, b, len, lane, [&](int l, const int32_t (&J)[U], const bool (&ok)[U]) {
                float2 xv[U][BD], a[U][BD * BD];
#pragma unroll
                for (int u = 0; u < U; ++u) {
#pragma unroll
                    for (int c = 0; c < BD; ++c)
                        xv[u][c] = ok[u] ? z[((int64_t)J[u] * BD + c) * BK + k] : make_float2(0.f, 0.f);
#pragma unroll
                    for (int e = 0; e < BD * BD; ++e)
                        a[u][e] = ok[u] ? __ldg(v + (int64_t)e * len + l + 2 * u) : make_float2(0.f, 0.f);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int rr = 0; rr < BD; ++rr)
#pragma unroll
                        for (int c = 0; c < BD; ++c)
                            df_fma(sh[rr], sl[rr], a[u][rr * BD + c].x, a[u][rr * BD + c].y, xv[u][c].x, xv[u][c].y);
            });
#pragma unroll
            for (int rr = 0; rr < BD; ++rr) {
                const float bh = __shfl_xor_sync(FULL, sh[rr], 16), bl = __shfl_xor_sync(FULL, sl[rr], 16);
                df_add(sh[rr], sl[rr], bh, bl);
            }
            if (h == 0)
#pragma unroll
                for (int rr = 0; rr < BD; ++rr) {
                    const int64_t e = ((int64_t)I * BD + rr) * BK + k;
                    float th = r[e].x, tl = r[e].y;
                    df_add(th, tl, -sh[rr], -sl[rr]);
                    wout[e] = __fadd_rn(th, tl);
                }
        }
    }
}

// ---------------------------------------------------------------- stiff blocks

// t[j][k] = r_d - (A z)_d for the stiff DOFs d = dofs[j]: one warp per DOF,
// lane k of half h over the row's blocks, double-float
__global__ void __launch_bounds__(256) stiff_gather_kernel(BatchDev B, StiffDev S, const float2 *__restrict__ r,
                                                           const float2 *__restrict__ z, double *__restrict__ t)
{
    const int lane = threadIdx.x & 31, h = lane >> 4, k = lane & 15;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= S.ndof) return;
    const int32_t d = S.dofs[j], I = d / BD, comp = d % BD;
    const int32_t b = B.rows[I], len = B.rows[I + 1] - b;
    const float2 *__restrict__ v = B.vals_df + (int64_t)b * 9;
    float sh = 0.f, sl = 0.f;
    for (int32_t l = h; l < len; l += 2) {
        const int32_t J = B.cols[b + l];
#pragma unroll
        for (int c = 0; c < BD; ++c) {
            const float2 a = __ldg(v + (int64_t)(comp * BD + c) * len + l);
            const float2 xv = z[((int64_t)J * BD + c) * BK + k];
            df_fma(sh, sl, a.x, a.y, xv.x, xv.y);
        }
    }
    const float bh = __shfl_xor_sync(FULL, sh, 16), bl = __shfl_xor_sync(FULL, sl, 16);
    df_add(sh, sl, bh, bl);
    if (h == 0) t[j * BK + k] = df_val(r[(int64_t)d * BK + k]) - ((double)sh + (double)sl);
}

// z_S += Inv t over the dense subdomains: one warp per stiff DOF row, lane k
// of half h over the columns of its subdomain; FP64 products
__global__ void __launch_bounds__(256) stiff_apply_kernel(StiffDev S, const double *__restrict__ t,
                                                          float2 *__restrict__ z)
{
    const int lane = threadIdx.x & 31, h = lane >> 4, k = lane & 15;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= S.ndof_dense) return;
    const int32_t s = S.sub_of[j], o = S.off[s], m = S.off[s + 1] - o;
    const double *col = S.inv + S.inv_off[s] + (j - o);  // row j of the inverse (stored transposed)
    double acc = 0.0;
    for (int32_t q = h; q < m; q += 2) acc += col[(int64_t)q * m] * t[(int64_t)(o + q) * BK + k];
    acc += __shfl_xor_sync(FULL, acc, 16);
    if (h == 0) {
        const int64_t e = (int64_t)S.dofs[j] * BK + k;
        z[e] = df_from(df_val(z[e]) + acc);
    }
}

// ---------------------------------------------------------------- layout changes

// dst[(perm[i] * BD + c) * BK + k] = src_s[k * n_s + i * BD + c] for every system

__global__ void to_batch_kernel(const ScatterSys *__restrict__ sys, int nsys, const int64_t *__restrict__ prefix,
                                double *__restrict__ bvec)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= prefix[nsys]) return;
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const ScatterSys &S = sys[lo];
    const int64_t e = t - prefix[lo];  // e = k * n_s + q
    const int64_t n = (int64_t)S.nb * BD;
    const int k = (int)(e / n);
    const int64_t q = e % n;
    const int64_t blk = q / BD, c = q % BD;
    const int64_t dst = (((int64_t)S.row0 + S.perm[blk]) * BD + c) * BK + k;
    bvec[dst] = S.src[e];
}

__global__ void from_batch_kernel(const ScatterSys *__restrict__ sys, int nsys, const int64_t *__restrict__ prefix,
                                  const double *__restrict__ xv)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= prefix[nsys]) return;
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    const ScatterSys &S = sys[lo];
    const int64_t e = t - prefix[lo];
    const int64_t n = (int64_t)S.nb * BD;
    const int k = (int)(e / n);
    const int64_t q = e % n;
    const int64_t blk = q / BD, c = q % BD;
    S.dst[e] = xv[(((int64_t)S.row0 + S.perm[blk]) * BD + c) * BK + k];
}

// bb per lane
__global__ void __launch_bounds__(256) lane_norms_kernel(BatchDev B, const double *__restrict__ b,
                                                         double *__restrict__ out)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    const int k = threadIdx.x & (BK - 1);
    double s2 = 0.0;
    const int64_t e1 = (int64_t)ch.r1 * BD * BK;
    for (int64_t e = (int64_t)ch.r0 * BD * BK + threadIdx.x; e < e1; e += blockDim.x) s2 += b[e] * b[e];
    __shared__ double red[16][BK];
    red[threadIdx.x >> 4][k] = s2;
    __syncthreads();
    double part[1] = {0.0}, tot[1];
    if (threadIdx.x < BK)
        for (int q = 0; q < 16; ++q) part[0] += red[q][threadIdx.x];
    if (sys_finish<1>(B, blockIdx.x, ch.sys, part, tot)) out[ch.sys * BK + threadIdx.x] = tot[0];
}

__global__ void __launch_bounds__(256) zero_done_lanes_kernel(BatchDev B, double *__restrict__ x)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    const int k = threadIdx.x & (BK - 1);
    const BatchLane &L = B.lane[ch.sys * BK + k];
    if (L.bb > 0.0) return;
    const int64_t e1 = (int64_t)ch.r1 * BD * BK;
    for (int64_t e = (int64_t)ch.r0 * BD * BK + threadIdx.x; e < e1; e += blockDim.x) x[e] = 0.0;
}

// xt += x (the pair correction of the attempt, in FP64); x = 0
__global__ void __launch_bounds__(256) fold_kernel(BatchDev B, double *__restrict__ xt, float2 *__restrict__ x)
{
    const Chunk ch = chunk_of(B, blockIdx.x);
    const int64_t e1 = (int64_t)ch.r1 * BD * BK;
    for (int64_t e = (int64_t)ch.r0 * BD * BK + threadIdx.x; e < e1; e += blockDim.x) {
        xt[e] += df_val(x[e]);
        x[e] = make_float2(0.f, 0.f);
    }
}

}  // namespace bk

namespace bk {

void launch_spmm_alpha(const BatchDev &B, const float2 *p, float2 *ap, cudaStream_t s)
{
    spmm_alpha_kernel<<<B.nchunk, 256, 0, s>>>(B, p, ap);
    LSS_LAUNCH_CHECK();
}

void launch_update_xr(const BatchDev &B, float2 *x, float2 *r, const float2 *p, const float2 *ap, cudaStream_t s)
{
    update_xr_kernel<<<B.nchunk, 256, 0, s>>>(B, x, r, p, ap);
    LSS_LAUNCH_CHECK();
}

void launch_update_p(const BatchDev &B, float2 *p, const float2 *z, cudaStream_t s)
{
    update_p_kernel<<<B.nchunk, 256, 0, s>>>(B, p, z);
    LSS_LAUNCH_CHECK();
}

void launch_copy_pairs(const BatchDev &B, float2 *dst, const float2 *src, cudaStream_t s)
{
    copy_pairs_kernel<<<B.nchunk, 256, 0, s>>>(B, dst, src);
    LSS_LAUNCH_CHECK();
}

void launch_residual64(const BatchDev &B, const double *b, const double *x, float2 *r, int mode, double *rr,
                       cudaStream_t s)
{
    residual64_kernel<<<B.nchunk, 256, 0, s>>>(B, b, x, r, mode, rr);
    LSS_LAUNCH_CHECK();
}

void launch_lane_norms(const BatchDev &B, const double *b, double *bb, cudaStream_t s)
{
    lane_norms_kernel<<<B.nchunk, 256, 0, s>>>(B, b, bb);
    LSS_LAUNCH_CHECK();
}

void launch_mas(const BatchDev &B, const BatchMas &M, const float2 *xin_pair, const float *xin32, float2 *z, bool acc,
                int dot, const float2 *rdot, cudaStream_t s)
{
    const MasDev &m = M.m;
    if (m.tile_elems != TILE_FLOATS) fail(LSS_ERR_INTERNAL, "batched MAS: unexpected bank tile size");
    const size_t smem = (size_t)BANK_SMEM;
    if (m.L > 1) {
        if (xin_pair) restrict0_kernel<float2><<<B.nchunk, 256, 0, s>>>(B, m, xin_pair, M.v);
        else restrict0_kernel<float><<<B.nchunk, 256, 0, s>>>(B, m, xin32, M.v);
        for (int l = 1; l + 1 < m.L; ++l)
            if (m.nbanks[l] > 0) restrict_kernel<<<(unsigned)((m.nbanks[l] + 7) / 8), 256, 0, s>>>(m, l, M.v);
        raise_smem_limit((const void *)symv_coarse_kernel, smem);
        if (m.ncoarse > 0)
            symv_coarse_kernel<<<(unsigned)std::min<int64_t>(m.ncoarse, sm_grid(2)), BANK_THREADS, smem, s>>>(m, M.invc, M.v,
                                                                                                    M.u, B.err);
        if (m.L > 2 && m.nitems[1] > 0)
            prolong_kernel<<<(unsigned)(((int64_t)m.nitems[1] * BD * BK + 255) / 256), 256, 0, s>>>(m, M.u);
    }
    const size_t smem0 = (size_t)BANK_SMEM_FULL;
#define LSS_B0(XT_, X_, A_, D_)                                                                           \
    do {                                                                                                  \
        raise_smem_limit((const void *)symv0_kernel<XT_, A_, D_>, smem0);                                 \
        symv0_kernel<XT_, A_, D_><<<B.nchunk, BANK_THREADS, smem0, s>>>(B, m, M.inv0, M.u, X_, z, rdot);  \
    } while (0)
    if (xin_pair) {
        if (acc) {
            if (dot == 1) LSS_B0(float2, xin_pair, true, 1);
            else if (dot == 2) LSS_B0(float2, xin_pair, true, 2);
            else LSS_B0(float2, xin_pair, true, 0);
        } else {
            if (dot == 1) LSS_B0(float2, xin_pair, false, 1);
            else if (dot == 2) LSS_B0(float2, xin_pair, false, 2);
            else LSS_B0(float2, xin_pair, false, 0);
        }
    } else {
        if (acc) {
            if (dot == 1) LSS_B0(float, xin32, true, 1);
            else if (dot == 2) LSS_B0(float, xin32, true, 2);
            else LSS_B0(float, xin32, true, 0);
        } else {
            if (dot == 1) LSS_B0(float, xin32, false, 1);
            else if (dot == 2) LSS_B0(float, xin32, false, 2);
            else LSS_B0(float, xin32, false, 0);
        }
    }
#undef LSS_B0
    LSS_LAUNCH_CHECK();
}

void launch_expand_banks(const float *tiles, float *full, int64_t nbank, cudaStream_t s)
{
    if (nbank == 0) return;
    expand_banks_kernel<<<(unsigned)nbank, BANK_THREADS, 0, s>>>(tiles, full);
    LSS_LAUNCH_CHECK();
}

void launch_residual32(const BatchDev &B, const float2 *r, const float2 *z, float *w, cudaStream_t s)
{
    residual32_kernel<<<B.nchunk, 256, 0, s>>>(B, r, z, w);
    LSS_LAUNCH_CHECK();
}

void launch_stiff(const BatchDev &B, const StiffDev &S, const float2 *r, const float2 *z_in, double *t, float2 *z,
                  cudaStream_t s)
{
    if (S.ndof == 0) return;
    stiff_gather_kernel<<<(unsigned)(((int64_t)S.ndof * 32 + 255) / 256), 256, 0, s>>>(B, S, r, z_in, t);
    if (S.ndof_dense > 0)
        stiff_apply_kernel<<<(unsigned)(((int64_t)S.ndof_dense * 32 + 255) / 256), 256, 0, s>>>(S, t, z);
    LSS_LAUNCH_CHECK();
}

void launch_to_batch(const ScatterSys *sys, int nsys, const int64_t *prefix, int64_t total, double *dst,
                     cudaStream_t s)
{
    if (total == 0) return;
    to_batch_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(sys, nsys, prefix, dst);
    LSS_LAUNCH_CHECK();
}

void launch_from_batch(const ScatterSys *sys, int nsys, const int64_t *prefix, int64_t total, const double *src,
                       cudaStream_t s)
{
    if (total == 0) return;
    from_batch_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(sys, nsys, prefix, src);
    LSS_LAUNCH_CHECK();
}

void launch_zero_done_lanes(const BatchDev &B, double *x, cudaStream_t s)
{
    zero_done_lanes_kernel<<<B.nchunk, 256, 0, s>>>(B, x);
    LSS_LAUNCH_CHECK();
}

void launch_fold(const BatchDev &B, double *xt, float2 *x, cudaStream_t s)
{
    fold_kernel<<<B.nchunk, 256, 0, s>>>(B, xt, x);
    LSS_LAUNCH_CHECK();
}

}  // namespace bk
}  // namespace lss
