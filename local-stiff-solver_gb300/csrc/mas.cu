// Multilevel additive Schwarz (MAS) preconditioner kernels (sm_103a).
//
// Semantics follow MASPreconditioner (MASPreconditioner.cu:376-1164 in the
// reference): level 0 = one 32*bd x 32*bd block per partition ("bank"), coarse
// level l = banks of 32 consecutive components of level l-1; each bank's
// Galerkin block is inverted exactly; apply = restrict (sum) -> per-bank
// symmetric matrix-vector product -> prolong (inject and add).
//
// GB300 layout of the inverses ("circulant tiles").  Inside a bank the scalar
// index is component-major (comp * 32 + lane).  The N x N inverse is cut into
// 32 x 32 tiles (c, c2), c <= c2; tile element [d][r] holds
// Inv[c*32 + r][c2*32 + (r+d) % 32], d = 0..16 for diagonal tiles (d = 16 kept
// twice, so 17*32 entries = the packed-triangle size plus 16) and d = 0..31 for
// off-diagonal tiles.  A warp owns a bank, lane r owns row r of every tile:
// every tile load is one 128-byte (FP32) / 256-byte (FP64) coalesced line,
// and the symmetric partner term travels by warp shuffle instead of being
// stored twice.  The inverse streams from HBM once per apply with evict-first
// loads; residual and coarse vectors stay in L2.
#include <cuda_bf16.h>

#include <type_traits>

#include "device_common.cuh"
#include "kernels.hpp"

namespace lss {

int64_t mas_tile_elems(int bd) { return (int64_t)bd * 17 * 32 + (int64_t)bd * (bd - 1) / 2 * 1024; }
int64_t mas_bank_bytes_bf16(int bd) { return (int64_t)bd * 17 * 32 * 4 + (int64_t)bd * (bd - 1) / 2 * 1024 * 2; }

namespace {

constexpr unsigned FULL = 0xffffffffu;

template <int BD>
__host__ __device__ constexpr int64_t tile_elems() { return (int64_t)BD * 17 * 32 + (int64_t)BD * (BD - 1) / 2 * 1024; }

template <typename T>
__device__ __forceinline__ T ld_stream(const T *p) { return __ldcs(p); }

// y = Inv x for one bank; lane r holds x[c] = x_{c*32+r}.
template <int BD, typename T>
__device__ __forceinline__ void tile_symv(const T *__restrict__ tile, const T (&x)[BD], T (&y)[BD], int lane)
{
#pragma unroll
    for (int c = 0; c < BD; ++c) y[c] = T(0);
    const T *__restrict__ t = tile;
#pragma unroll
    for (int c = 0; c < BD; ++c) {
        {
            T a = ld_stream(t + lane);
            y[c] += a * x[c];
#pragma unroll
            for (int d = 1; d < 16; ++d) {
                a = ld_stream(t + d * 32 + lane);
                const T xs = __shfl_sync(FULL, x[c], (lane + d) & 31);
                y[c] += a * xs;
                const T tr = a * x[c];
                y[c] += __shfl_sync(FULL, tr, (lane - d) & 31);
            }
            a = ld_stream(t + 16 * 32 + lane);
            y[c] += a * __shfl_xor_sync(FULL, x[c], 16);
            t += 17 * 32;
        }
#pragma unroll
        for (int c2 = c + 1; c2 < BD; ++c2) {
#pragma unroll 8
            for (int d = 0; d < 32; ++d) {
                const T a = ld_stream(t + d * 32 + lane);
                const T xs = __shfl_sync(FULL, x[c2], (lane + d) & 31);
                y[c] += a * xs;
                const T tr = a * x[c];
                y[c2] += __shfl_sync(FULL, tr, (lane - d) & 31);
            }
            t += 32 * 32;
        }
    }
}

// tile_symv for a bank whose diagonal tiles are FP32 and whose off-diagonal
// tiles (c < c2) are BF16 (the same order: for each c, tile (c, c) then the
// tiles (c, c2 > c)).  In a BF16 tile, 32-bit word k * 32 + r holds the
// entries [2k][r] (low half) and [2k + 1][r] (high half), so every warp load
// is still one 128-byte line; a BF16 value widens to FP32 exactly by a shift.
template <int BD>
__device__ __forceinline__ void tile_symv_bf(const unsigned char *__restrict__ bank, const float (&x)[BD],
                                             float (&y)[BD], int lane)
{
#pragma unroll
    for (int c = 0; c < BD; ++c) y[c] = 0.f;
    const unsigned char *t = bank;
#pragma unroll
    for (int c = 0; c < BD; ++c) {
        {
            const float *__restrict__ dt = reinterpret_cast<const float *>(t);
            float a = ld_stream(dt + lane);
            y[c] += a * x[c];
#pragma unroll
            for (int d = 1; d < 16; ++d) {
                a = ld_stream(dt + d * 32 + lane);
                const float xs = __shfl_sync(FULL, x[c], (lane + d) & 31);
                y[c] += a * xs;
                const float tr = a * x[c];
                y[c] += __shfl_sync(FULL, tr, (lane - d) & 31);
            }
            a = ld_stream(dt + 16 * 32 + lane);
            y[c] += a * __shfl_xor_sync(FULL, x[c], 16);
            t += 17 * 32 * sizeof(float);
        }
#pragma unroll
        for (int c2 = c + 1; c2 < BD; ++c2) {
            const unsigned int *__restrict__ ot = reinterpret_cast<const unsigned int *>(t);
#pragma unroll 4
            for (int k = 0; k < 16; ++k) {
                const unsigned int w = __ldcs(ot + k * 32 + lane);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int d = 2 * k + h;
                    const float a = __uint_as_float(h ? (w & 0xffff0000u) : (w << 16));
                    const float xs = __shfl_sync(FULL, x[c2], (lane + d) & 31);
                    y[c] += a * xs;
                    const float tr = a * x[c];
                    y[c2] += __shfl_sync(FULL, tr, (lane - d) & 31);
                }
            }
            t += 32 * 32 * sizeof(unsigned short);
        }
    }
}

// ------------------------------------------------------------------ setup

template <int BD>
__global__ void __launch_bounds__(256) assemble0_kernel(BsrDev A, const int32_t *__restrict__ part_of,
                                                        const int32_t *__restrict__ part_off,
                                                        double *__restrict__ stage)
{
    constexpr int N = 32 * BD;
    const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.nb) return;
    const int32_t p = part_of[i], lo = part_off[p], hi = part_off[p + 1], li = i - lo;
    double *base = stage + (int64_t)p * N * N;
    const int32_t b = A.rows[i], len = A.rows[i + 1] - b;
    const double *v = A.vals + (int64_t)b * BD * BD;
    for (int32_t l = 0; l < len; ++l) {
        const int32_t j = A.cols[b + l];
        if (j < lo || j >= hi) continue;
        const int32_t lj = j - lo;
#pragma unroll
        for (int bi = 0; bi < BD; ++bi)
#pragma unroll
            for (int bj = 0; bj < BD; ++bj)
                base[(int64_t)(bi * 32 + li) * N + bj * 32 + lj] = v[(int64_t)(bi * BD + bj) * len + l];
    }
}

// Galerkin blocks of every coarse level, deterministically, in two passes.
// Pass 1: one warp per chunk of at most MEMB_CHUNK member rows of a coarse
// item ci (its row strip of the bank matrix), lane c accumulating the BD x BD
// block of the column items cj with cj % 32 == c.  The chunk's rows come in
// ascending order and each row's blocks in column order; the blocks of a
// 32-wide piece whose column item falls into the same bank are handed to
// their owner lanes one at a time by shuffles.  Pass 2: one warp per item sums
// its chunks' partial strips in chunk order and writes the upper triangle
// (each entry belongs to exactly one item, so the stores never collide).
// Every sum runs in one fixed order (no atomics): two factorizations of the
// same matrix give bit-identical coarse inverses.
__device__ __forceinline__ void flat_item(const MasDev &m, int64_t w, int &l, int32_t &ci)
{
    l = 1;
    while (l < m.L && w >= m.nitems[l]) w -= m.nitems[l++];
    ci = (int32_t)w;
}

template <int BD>
__global__ void __launch_bounds__(256) assemble_coarse_chunk_kernel(BsrDev A, MasDev m, const int32_t *__restrict__ cmap,
                                                                    CoarseMembers mb, double *__restrict__ partial)
{
    __shared__ int8_t slot_all[8][32];  // per warp: column slot -> lane holding its group sum
    const int lane = threadIdx.x & 31;
    int8_t *slot = slot_all[threadIdx.x >> 5];
    slot[lane] = -1;
    __syncwarp();
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (c >= mb.nchunk) return;
    // the chunk's item: last i with item_chunk[i] <= c
    int32_t lo = 0, hi = mb.nitem - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi + 1) >> 1;
        if (mb.item_chunk[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    int l;
    int32_t ci;
    flat_item(m, lo, l, ci);
    const int32_t *map = cmap + (int64_t)(l - 1) * A.nb;
    double acc[BD * BD];
#pragma unroll
    for (int k = 0; k < BD * BD; ++k) acc[k] = 0.0;
    for (int32_t r = mb.chunk_r0[c]; r < mb.chunk_r0[c + 1]; ++r) {
        const int32_t i = mb.rows[r];
        const int32_t b = A.rows[i], len = A.rows[i + 1] - b;
        const double *v = A.vals + (int64_t)b * BD * BD;
        for (int32_t q0 = 0; q0 < len; q0 += 32) {
            const int32_t q = q0 + lane;
            int32_t cj = -1;
            double val[BD * BD];
            if (q < len) {
                cj = map[A.cols[b + q]];
#pragma unroll
                for (int k = 0; k < BD * BD; ++k) val[k] = v[(int64_t)k * len + q];
            } else {
#pragma unroll
                for (int k = 0; k < BD * BD; ++k) val[k] = 0.0;
            }
            const bool mine = cj >= 0 && (cj >> 5) == (ci >> 5);
            if (!__any_sync(0xffffffffu, mine)) continue;
            // lanes holding the same column item form a group; its leader (lowest
            // lane) sums the group in lane order, then hands the sum to the lane
            // that owns the item's slot -- groups proceed in parallel
            const unsigned grp = __match_any_sync(0xffffffffu, mine ? cj : (int32_t)(0x80000000u | (unsigned)lane));
            const bool leader = mine && __ffs(grp) - 1 == lane;
            unsigned rest = mine ? grp & (grp - 1) : 0u;
            const int rounds = __reduce_max_sync(0xffffffffu, __popc(rest));
            double gs[BD * BD];
#pragma unroll
            for (int k = 0; k < BD * BD; ++k) gs[k] = val[k];
            for (int it = 0; it < rounds; ++it) {
                const bool have = rest != 0u;
                const int src = have ? __ffs(rest) - 1 : lane;
                rest &= rest - 1u;
#pragma unroll
                for (int k = 0; k < BD * BD; ++k) {
                    const double x = __shfl_sync(0xffffffffu, val[k], src);
                    if (have) gs[k] += x;
                }
            }
            if (leader) slot[cj & 31] = (int8_t)lane;
            __syncwarp();
            const int from = slot[lane];
            __syncwarp();
            if (leader) slot[cj & 31] = -1;
#pragma unroll
            for (int k = 0; k < BD * BD; ++k) {
                const double x = __shfl_sync(0xffffffffu, gs[k], from >= 0 ? from : lane);
                if (from >= 0) acc[k] += x;
            }
            __syncwarp();
        }
    }
    double *out = partial + c * (BD * BD * 32);
#pragma unroll
    for (int k = 0; k < BD * BD; ++k) out[k * 32 + lane] = acc[k];
}

template <int BD>
__global__ void __launch_bounds__(256) assemble_coarse_sum_kernel(MasDev m, CoarseMembers mb,
                                                                  const double *__restrict__ partial,
                                                                  double *__restrict__ stage)
{
    constexpr int N = 32 * BD;
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= mb.nitem) return;
    int l;
    int32_t ci;
    flat_item(m, w, l, ci);
    const int32_t g = m.boff[l] + (ci >> 5);
    double acc[BD * BD];
#pragma unroll
    for (int k = 0; k < BD * BD; ++k) acc[k] = 0.0;
    for (int32_t c = mb.item_chunk[w]; c < mb.item_chunk[w + 1]; ++c) {
        const double *p = partial + (int64_t)c * (BD * BD * 32);
#pragma unroll
        for (int k = 0; k < BD * BD; ++k) acc[k] += p[k * 32 + lane];
    }
    double *base = stage + (int64_t)g * N * N;
#pragma unroll
    for (int bi = 0; bi < BD; ++bi)
#pragma unroll
        for (int bj = 0; bj < BD; ++bj) {
            const int row = bi * 32 + (ci & 31), col = bj * 32 + lane;
            if (row <= col) base[(int64_t)row * N + col] = acc[bi * BD + bj];
        }
}

// Symmetric sweep inversion of S (N x N, leading dimension ld, in shared
// memory): the Gauss-Jordan variant of MASPreconditioner.cu:799-900, which
// leaves -A^-1 in S.  Only the upper triangle (t <= c) is read and kept:
// the sweep preserves symmetry, so half the FP64 updates suffice.  The
// triangle's entries are dealt to the CTA's threads in linear order, so
// every update instruction runs on full warps (a partly predicated FP64
// instruction costs the pipe a whole warp).  Flags zero / non-finite pivots.
// Needs blockDim.x == 256.
template <int N>
__device__ void sweep_invert(double *S, int ld, double *col, double *scol, int *bad)
{
    constexpr int NE = N * (N + 1) / 2;
    constexpr int PER = (NE + 255) / 256;
    const int tid = threadIdx.x;
    uint32_t tc[PER];  // (t << 16) | c of this thread's entries; ~0u past the end
#pragma unroll
    for (int k = 0; k < PER; ++k) {
        const int e = tid + k * 256;
        tc[k] = ~0u;
        if (e < NE) {
            int t = 0, off = 0;
            while (off + (N - t) <= e) {
                off += N - t;
                ++t;
            }
            tc[k] = ((uint32_t)t << 16) | (uint32_t)(t + (e - off));
        }
    }
    for (int p = 0; p < N; ++p) {
        const double piv = S[p * ld + p];
        const double rpiv = 1.0 / piv;  // one division per pivot; the column is scaled by multiplication
        for (int t = tid; t < N; t += 256) {
            const double cv = (t == p) ? 0.0 : (t < p ? S[t * ld + p] : S[p * ld + t]);
            col[t] = cv;
            scol[t] = cv * rpiv;
        }
        if (tid == 0 && (!isfinite(piv) || piv == 0.0)) atomicOr(bad, 1);
        __syncthreads();
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            if (tc[k] == ~0u) continue;
            const int t = (int)(tc[k] >> 16), c = (int)(tc[k] & 0xffffu);
            if (t != p && c != p) S[t * ld + c] -= scol[t] * col[c];
        }
        __syncthreads();
        for (int t = tid; t < N; t += 256) {
            if (t == p) S[p * ld + p] = -rpiv;
            else if (t < p) S[t * ld + p] = scol[t];
            else S[p * ld + t] = scol[t];
        }
        __syncthreads();
    }
}

template <int BD, typename T, bool BF>
__global__ void __launch_bounds__(256, 2) mas_invert_kernel(const double *__restrict__ stage, T *__restrict__ out,
                                                         int *bad)
{
    constexpr int N = 32 * BD, LD = N + 1;
    extern __shared__ double sm[];
    double *S = sm, *col = sm + N * LD, *scol = col + N;
    const int64_t bank = blockIdx.x;
    const double *src = stage + bank * N * N;
    for (int idx = threadIdx.x; idx < N * N; idx += blockDim.x) {
        const int r = idx / N, c = idx % N;
        if (r > c) continue;  // the upper triangle is all the sweep uses
        double v = src[(int64_t)r * N + c];
        if (r == c && v == 0.0) v = 1.0;  // padding (MASPreconditioner.cu:779-796)
        S[r * LD + c] = v;
    }
    __syncthreads();
    sweep_invert<N>(S, LD, col, scol, bad);
    // the swept entry (i, j), i <= j
    auto entry = [&](int i, int j) -> double { return S[i * LD + j]; };
    // tiles
    if (BF) {  // FP32 diagonal tiles, BF16 off-diagonal tiles (round to nearest even)
        unsigned char *dst = reinterpret_cast<unsigned char *>(out) + bank * (int64_t)(BD * 17 * 32 * 4 + BD * (BD - 1) / 2 * 2048);
        for (int c = 0; c < BD; ++c)
            for (int c2 = c; c2 < BD; ++c2) {
                const int nd = (c == c2) ? 17 : 32;
                for (int e = threadIdx.x; e < nd * 32; e += blockDim.x) {
                    const int d = e >> 5, r = e & 31;
                    const int gi = c * 32 + r, gj = c2 * 32 + ((r + d) & 31);
                    const double val = -entry(min(gi, gj), max(gi, gj));
                    if (!isfinite(val)) atomicOr(bad, 2);
                    if (c == c2) reinterpret_cast<float *>(dst)[e] = (float)val;
                    else reinterpret_cast<__nv_bfloat16 *>(dst)[(d >> 1) * 64 + 2 * r + (d & 1)] =
                        __float2bfloat16_rn((float)val);
                }
                dst += (c == c2) ? 17 * 32 * 4 : 32 * 32 * 2;
            }
        return;
    }
    T *dst = out + bank * tile_elems<BD>();
    int64_t off = 0;
    for (int c = 0; c < BD; ++c)
        for (int c2 = c; c2 < BD; ++c2) {
            const int nd = (c == c2) ? 17 : 32;
            for (int e = threadIdx.x; e < nd * 32; e += blockDim.x) {
                const int d = e >> 5, r = e & 31;
                const int gi = c * 32 + r, gj = c2 * 32 + ((r + d) & 31);
                const double val = -entry(min(gi, gj), max(gi, gj));
                if (!isfinite(val)) atomicOr(bad, 2);
                dst[off + e] = (T)val;
            }
            off += nd * 32;
        }
}

// ------------------------------------------------------------------ apply

// Segmented sums of one bank: 32 items (values staged item-major in xs, the
// target aggregate of each item in ks) into ncc aggregates.  Output slot
// s = k * BD + c (aggregate k, component c) belongs to lane s % 32, which adds
// the items of aggregate k in item order: no FP64 shuffles (each costs 16
// cycles of the SM's FP64 pipe on this part), a fixed summation order, and in
// FP32 mode no FP64 instruction at all.
template <int BD, typename T>
__device__ __forceinline__ void bank_segment_sums(const T *xs, const uint8_t *ks, int ncc, T *__restrict__ out,
                                                  int lane)
{
    for (int sl = lane; sl < ncc * BD; sl += 32) {
        const int k = sl / BD, c = sl - k * BD;
        T acc = T(0);
#pragma unroll 8
        for (int j = 0; j < 32; ++j)
            if (ks[j] == k) acc += xs[j * BD + c];
        out[(int64_t)k * BD + c] = acc;
    }
}

// level 0 -> level 1: per-part component sums of r
template <int BD, typename T, typename XT>
__global__ void __launch_bounds__(256) restrict0_kernel(MasDev m, const XT *__restrict__ r, T *__restrict__ v,
                                                        const int *done)
{
    if (done && *done) return;
    __shared__ T xs_all[8][32 * BD];
    __shared__ uint8_t ks_all[8][32];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    T *xs = xs_all[wl];
    uint8_t *ks = ks_all[wl];
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    T *v1 = v + m.voff[1];
    for (int64_t p = w0; p < m.nparts; p += nw) {
        const int32_t lo = m.part_off[p], cnt = m.part_off[p + 1] - lo;
        // the part's values are one contiguous run: coalesced loads
#pragma unroll
        for (int q = 0; q < BD; ++q) {
            const int e = q * 32 + lane;
            xs[e] = e < cnt * BD ? (T)r[(int64_t)lo * BD + e] : T(0);
        }
        ks[lane] = lane < cnt ? m.key0[lo + lane] : (uint8_t)0xff;
        __syncwarp();
        bank_segment_sums<BD, T>(xs, ks, m.ccnt0[p], v1 + (int64_t)m.cbase0[p] * BD, lane);
        __syncwarp();
    }
}

// level l -> level l+1 (l >= 1)
template <int BD, typename T>
__global__ void __launch_bounds__(256) restrict_kernel(MasDev m, int l, T *__restrict__ v, const int *done)
{
    if (done && *done) return;
    __shared__ T xs_all[8][32 * BD];
    __shared__ uint8_t ks_all[8][32];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    T *xs = xs_all[wl];
    uint8_t *ks = ks_all[wl];
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const T *vl = v + m.voff[l];
    T *vn = v + m.voff[l + 1];
    const uint8_t *key_l = m.key[l];
    const uint8_t *ccnt_l = m.ccnt[l];
    const int32_t *cbase_l = m.cbase[l];
    const int32_t nitems = m.nitems[l];
    for (int64_t b = w0; b < m.nbanks[l]; b += nw) {
        const int64_t i0 = b * 32;
        const int cnt = nitems - i0 < 32 ? (int)(nitems - i0) : 32;
#pragma unroll
        for (int q = 0; q < BD; ++q) {
            const int e = q * 32 + lane;
            xs[e] = e < cnt * BD ? vl[i0 * BD + e] : T(0);
        }
        ks[lane] = lane < cnt ? key_l[i0 + lane] : (uint8_t)0xff;
        __syncwarp();
        bank_segment_sums<BD, T>(xs, ks, ccnt_l[b], vn + (int64_t)cbase_l[b] * BD, lane);
        __syncwarp();
    }
}

// all coarse banks: u_l = Inv_l v_l
template <int BD, typename T>
__global__ void __launch_bounds__(256) symv_coarse_kernel(MasDev m, const T *__restrict__ invc,
                                                          const T *__restrict__ v, T *__restrict__ u,
                                                          const int *done)
{
    if (done && *done) return;
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t g = w0; g < m.ncoarse; g += nw) {
        int l = 1;
        while (l + 1 < m.L && g >= m.boff[l + 1]) ++l;
        const int64_t b = g - m.boff[l];
        const int64_t e0 = m.voff[l] + (b * 32 + lane) * BD;
        T x[BD], y[BD];
#pragma unroll
        for (int c = 0; c < BD; ++c) x[c] = v[e0 + c];
        tile_symv<BD, T>(invc + g * m.tile_elems, x, y, lane);
#pragma unroll
        for (int c = 0; c < BD; ++c) u[e0 + c] = y[c];
    }
}

// u_1 += P (u_2 + P (u_3 + ...)): every level-1 item gathers its ancestors'
// corrections and sums them from the top level down, as level-by-level
// prolongation would, in one launch.
template <int BD, typename T>
__global__ void __launch_bounds__(256) prolong_all_kernel(MasDev m, T *__restrict__ u, const int *done)
{
    if (done && *done) return;
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m.nitems[1]) return;
    int64_t item[MAS_MAXL];
    item[1] = k;
    for (int l = 1; l + 1 < m.L; ++l) item[l + 1] = m.cbase[l][item[l] >> 5] + m.key[l][item[l]];
#pragma unroll
    for (int c = 0; c < BD; ++c) {
        T acc = u[m.voff[m.L - 1] + item[m.L - 1] * BD + c];
        for (int l = m.L - 2; l >= 1; --l) acc = u[m.voff[l] + item[l] * BD + c] + acc;
        u[m.voff[1] + k * BD + c] = acc;
    }
}

// level 0: z = Inv_0 x (+ coarse correction u_1), optional accumulate and r.z;
// x in FP64, or in FP32 (XT = float) when it comes from the FP32 residual
template <int BD, typename T, bool ACC, int DOT, typename XT, bool BF = false>
__global__ void __launch_bounds__(256) symv0_kernel(MasDev m, const T *__restrict__ inv0, const T *__restrict__ u,
                                                    const XT *__restrict__ xin, double *__restrict__ z,
                                                    double scale, const double *__restrict__ rdot, PcgState *st,
                                                    GridReduce gr, const int *done, float *__restrict__ z32,
                                                    float *__restrict__ z_lo)
{
    if (done && *done) return;
    const int lane = threadIdx.x & 31;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double dot[1] = {0.0};
    const T *u1 = u + m.voff[1];
    for (int64_t p = w0; p < m.nparts; p += nw) {
        const int32_t lo = m.part_off[p], node = lo + lane;
        const bool valid = node < m.part_off[p + 1];
        T x[BD], y[BD];
#pragma unroll
        for (int c = 0; c < BD; ++c) x[c] = valid ? (T)xin[(int64_t)node * BD + c] : T(0);
        if constexpr (BF && std::is_same<T, float>::value)
            tile_symv_bf<BD>(reinterpret_cast<const unsigned char *>(inv0) + p * m.bank_bytes0, x, y, lane);
        else
            tile_symv<BD, T>(inv0 + p * m.tile_elems, x, y, lane);
        if (valid) {
            int64_t cidx = -1;
            if (m.L > 1) cidx = (int64_t)(m.cbase0[p] + m.key0[node]) * BD;
#pragma unroll
            for (int c = 0; c < BD; ++c) {
                double val = (double)y[c];
                if (cidx >= 0) val += (double)u1[cidx + c];
                val *= scale;
                const int64_t e = (int64_t)node * BD + c;
                if (ACC) val += z[e];
                z[e] = val;
                if (z32) {
                    const float h = (float)val;
                    z32[e] = h;
                    if (z_lo) z_lo[e] = (float)(val - (double)h);
                }
                if (DOT) dot[0] += rdot[e] * val;
            }
        }
    }
    if (DOT) {
        double tot[1];
        if (grid_sum<1>(dot, gr, tot)) {
            // DOT == 1: initial gamma (GPUHybrid.cu:1450-1451); DOT == 2: new gamma and
            // beta = gamma_new / gamma_old (GPUHybrid.cu:1501-1504)
            if (DOT == 2) {
                st->beta = tot[0] / st->gamma;
                if (st->iter >= 1 && st->iter <= PCG_HIST) st->hist_beta[st->iter - 1] = st->beta;
            }
            st->gamma = tot[0];
        }
    }
}

template <int BD, typename T, typename XT>
void mas_apply_dot_t(const MasDev &m, const T *inv0, const T *invc, T *v, T *u, const XT *xin, double *z,
                     bool acc, double scale, const double *rdot, PcgState *st, int dot_mode, GridReduce gr,
                     const int *done, cudaStream_t s, float *z32, float *z_lo)
{
    if (m.L > 1) {
        restrict0_kernel<BD, T, XT><<<grid_for((int64_t)m.nparts * 32, 256, sm_grid(16)), 256, 0, s>>>(m, xin, v, done);
        for (int l = 1; l + 1 < m.L; ++l)
            restrict_kernel<BD, T><<<grid_for((int64_t)m.nbanks[l] * 32, 256, sm_grid(16)), 256, 0, s>>>(m, l, v, done);
        symv_coarse_kernel<BD, T><<<grid_for((int64_t)m.ncoarse * 32, 256, sm_grid(16)), 256, 0, s>>>(m, invc, v, u,
                                                                                                   done);
        if (m.L > 2)
            prolong_all_kernel<BD, T><<<grid_for(m.nitems[1], 256, 1 << 30), 256, 0, s>>>(m, u, done);
    }
    const int grid = grid_for((int64_t)m.nparts * 32, 256, sm_grid(16));
#define LSS_S0(A_, D_)                                                                                          \
    do {                                                                                                        \
        if (std::is_same<T, float>::value && m.bank_bytes0 > 0)                                                 \
            symv0_kernel<BD, T, A_, D_, XT, true><<<grid, 256, 0, s>>>(m, inv0, u, xin, z, scale, rdot, st, gr,   \
                                                                       done, z32, z_lo);                        \
        else                                                                                                    \
            symv0_kernel<BD, T, A_, D_, XT, false><<<grid, 256, 0, s>>>(m, inv0, u, xin, z, scale, rdot, st, gr,  \
                                                                        done, z32, z_lo);                       \
    } while (0)
    if (dot_mode == 0) {
        if (acc) LSS_S0(true, 0);
        else LSS_S0(false, 0);
    } else if (dot_mode == 1) {
        if (acc) LSS_S0(true, 1);
        else LSS_S0(false, 1);
    } else {
        if (acc) LSS_S0(true, 2);
        else LSS_S0(false, 2);
    }
#undef LSS_S0
    LSS_LAUNCH_CHECK();
}

}  // namespace

void launch_mas_assemble0(const BsrDev &A, const int32_t *part_of, const int32_t *part_off, double *stage,
                          cudaStream_t s)
{
    const int grid = (int)((A.nb + 255) / 256);
    if (grid == 0) return;
    switch (A.bd) {
    case 1: assemble0_kernel<1><<<grid, 256, 0, s>>>(A, part_of, part_off, stage); break;
    case 2: assemble0_kernel<2><<<grid, 256, 0, s>>>(A, part_of, part_off, stage); break;
    default: assemble0_kernel<3><<<grid, 256, 0, s>>>(A, part_of, part_off, stage); break;
    }
    LSS_LAUNCH_CHECK();
}

void launch_mas_assemble_coarse(const BsrDev &A, const MasDev &m, const int32_t *cmap, const CoarseMembers &mb,
                                double *partial, double *stage, cudaStream_t s)
{
    if (mb.nitem == 0 || m.L < 2) return;
    const int g1 = (int)((mb.nchunk * 32 + 255) / 256), g2 = (int)((mb.nitem * 32 + 255) / 256);
    switch (A.bd) {
    case 1:
        assemble_coarse_chunk_kernel<1><<<g1, 256, 0, s>>>(A, m, cmap, mb, partial);
        assemble_coarse_sum_kernel<1><<<g2, 256, 0, s>>>(m, mb, partial, stage);
        break;
    case 2:
        assemble_coarse_chunk_kernel<2><<<g1, 256, 0, s>>>(A, m, cmap, mb, partial);
        assemble_coarse_sum_kernel<2><<<g2, 256, 0, s>>>(m, mb, partial, stage);
        break;
    default:
        assemble_coarse_chunk_kernel<3><<<g1, 256, 0, s>>>(A, m, cmap, mb, partial);
        assemble_coarse_sum_kernel<3><<<g2, 256, 0, s>>>(m, mb, partial, stage);
        break;
    }
    LSS_LAUNCH_CHECK();
}

template <int BD, typename T, bool BF = false>
static void invert_t(int64_t nbanks, const double *stage, T *out, int *bad, cudaStream_t s)
{
    constexpr int N = 32 * BD;
    const size_t smem = (size_t)(N * (N + 1) + 2 * N) * sizeof(double);
    LSS_CUDA(cudaFuncSetAttribute(mas_invert_kernel<BD, T, BF>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem));
    for (int64_t b0 = 0; b0 < nbanks; b0 += 1 << 30) {
        const int64_t cnt = std::min<int64_t>(nbanks - b0, 1 << 30);
        T *o = BF ? reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(out) + b0 * mas_bank_bytes_bf16(BD))
                  : out + b0 * mas_tile_elems(BD);
        mas_invert_kernel<BD, T, BF><<<(unsigned)cnt, 256, smem, s>>>(stage + b0 * N * N, o, bad);
    }
    LSS_LAUNCH_CHECK();
}

void launch_mas_invert(int bd, int64_t nbanks, const double *stage, void *out, bool fp32, int *bad, cudaStream_t s,
                       bool bf16_offdiag)
{
    if (nbanks == 0) return;
    if (bf16_offdiag) {
        if (!fp32) fail(LSS_ERR_INTERNAL, "BF16 off-diagonal tiles need the FP32 MAS");
        if (bd == 1) invert_t<1, float, true>(nbanks, stage, (float *)out, bad, s);
        else if (bd == 2) invert_t<2, float, true>(nbanks, stage, (float *)out, bad, s);
        else invert_t<3, float, true>(nbanks, stage, (float *)out, bad, s);
        return;
    }
    if (fp32) {
        if (bd == 1) invert_t<1, float>(nbanks, stage, (float *)out, bad, s);
        else if (bd == 2) invert_t<2, float>(nbanks, stage, (float *)out, bad, s);
        else invert_t<3, float>(nbanks, stage, (float *)out, bad, s);
    } else {
        if (bd == 1) invert_t<1, double>(nbanks, stage, (double *)out, bad, s);
        else if (bd == 2) invert_t<2, double>(nbanks, stage, (double *)out, bad, s);
        else invert_t<3, double>(nbanks, stage, (double *)out, bad, s);
    }
}

void launch_mas_level0(const MasDev &m, const void *inv0, const void *u, bool fp32, const double *xin, double *z,
                       cudaStream_t s)
{
    const int grid = grid_for((int64_t)m.nparts * 32, 256, sm_grid(16));
    GridReduce gr{};
#define LSS_L0(BD_, T_)                                                                                        \
    symv0_kernel<BD_, T_, false, 0, double><<<grid, 256, 0, s>>>(m, (const T_ *)inv0, (const T_ *)u, xin, z, 1.0,   \
                                                                 nullptr, nullptr, gr, nullptr, nullptr, nullptr)
#define LSS_L0BF(BD_)                                                                                          \
    symv0_kernel<BD_, float, false, 0, double, true><<<grid, 256, 0, s>>>(                                     \
        m, (const float *)inv0, (const float *)u, xin, z, 1.0, nullptr, nullptr, gr, nullptr, nullptr, nullptr)
    if (fp32 && m.bank_bytes0 > 0) {
        if (m.bd == 2) LSS_L0BF(2);
        else LSS_L0BF(3);
    } else if (fp32) {
        if (m.bd == 1) LSS_L0(1, float);
        else if (m.bd == 2) LSS_L0(2, float);
        else LSS_L0(3, float);
    } else {
        if (m.bd == 1) LSS_L0(1, double);
        else if (m.bd == 2) LSS_L0(2, double);
        else LSS_L0(3, double);
    }
#undef LSS_L0
#undef LSS_L0BF
    LSS_LAUNCH_CHECK();
}

void launch_mas_apply(const MasDev &m, const void *inv0, const void *invc, void *v, void *u, bool fp32,
                      const double *xin, double *z, bool acc, double scale, const double *rdot, PcgState *st,
                      int dot_mode, GridReduce gr, const int *done, cudaStream_t s, float *z32, const float *xin32,
                      float *z_lo)
{
#define LSS_MAS(BD_, T_)                                                                                          \
    mas_apply_dot_t<BD_, T_, double>(m, (const T_ *)inv0, (const T_ *)invc, (T_ *)v, (T_ *)u, xin, z, acc, scale, \
                                     rdot, st, dot_mode, gr, done, s, z32, z_lo)
#define LSS_MAS32(BD_)                                                                                            \
    mas_apply_dot_t<BD_, float, float>(m, (const float *)inv0, (const float *)invc, (float *)v, (float *)u, xin32, \
                                       z, acc, scale, rdot, st, dot_mode, gr, done, s, z32, z_lo)
    if (xin32) {
        if (!fp32) fail(LSS_ERR_INTERNAL, "an FP32 input needs the FP32 MAS");
        if (m.bd == 1) LSS_MAS32(1);
        else if (m.bd == 2) LSS_MAS32(2);
        else LSS_MAS32(3);
        return;
    }
    if (fp32) {
        if (m.bd == 1) LSS_MAS(1, float);
        else if (m.bd == 2) LSS_MAS(2, float);
        else LSS_MAS(3, float);
    } else {
        if (m.bd == 1) LSS_MAS(1, double);
        else if (m.bd == 2) LSS_MAS(2, double);
        else LSS_MAS(3, double);
    }
#undef LSS_MAS
#undef LSS_MAS32
}

}  // namespace lss
