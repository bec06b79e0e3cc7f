// Block-row SpMV building blocks (sm_103a).
//
// Operator layout in HBM ("row-sliced BSR"): block rows in partition order,
// rows[nb+1], cols[nnzb]; the bd*bd values of the len blocks of block row i
// are stored as bd*bd contiguous arrays of length len:
//     vals[rows[i]*bd*bd + k*len + l] = entry k (row major in the block) of
// the l-th block of row i.  A group of LANES threads handles one block row;
// lane l reads block l, l+LANES, ...: every value load of the group is one
// contiguous, fully used segment, and the column index load is too.  For
// bd == 1 this is plain CSR.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace lss {

template <int LANES, typename T>
__device__ __forceinline__ T group_sum(T v)
{
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, LANES);
    return v;
}

// y[0..BD) = (A x)[block row i], reduced over the LANES-wide group (valid in
// every lane of the group).  VT: stored value type; XT: x type; ACC: accumulator.
// Every lane of the warp must call it (the group reduction is a full-warp
// shuffle); a group without a row passes valid = false and gets zeros.
template <int BD, int LANES, typename VT, typename XT, typename ACC>
__device__ __forceinline__ void bsr_block_row(const int32_t *__restrict__ rows, const int32_t *__restrict__ cols,
                                              const VT *__restrict__ vals, int32_t i, bool valid,
                                              const XT *__restrict__ x, int lane, ACC (&y)[BD])
{
    const int32_t b = valid ? rows[i] : 0, e = valid ? rows[i + 1] : 0, len = e - b;
    const VT *__restrict__ v = vals + (int64_t)b * (BD * BD);
#pragma unroll
    for (int r = 0; r < BD; ++r) y[r] = ACC(0);
#pragma unroll 2
    for (int32_t l = lane; l < len; l += LANES) {
        const int32_t c = __ldcs(cols + b + l);
        ACC xv[BD];
#pragma unroll
        for (int k = 0; k < BD; ++k) xv[k] = (ACC)x[(int64_t)c * BD + k];
#pragma unroll
        for (int r = 0; r < BD; ++r)
#pragma unroll
            for (int k = 0; k < BD; ++k) y[r] += (ACC)__ldcs(v + (int64_t)(r * BD + k) * len + l) * xv[k];
    }
#pragma unroll
    for (int r = 0; r < BD; ++r) y[r] = group_sum<LANES>(y[r]);
}

// One scalar row (component comp of block row i) of A x, warp-wide (valid in all lanes).
template <int BD, typename VT, typename XT>
__device__ __forceinline__ double bsr_scalar_row(const int32_t *__restrict__ rows, const int32_t *__restrict__ cols,
                                                 const VT *__restrict__ vals, int32_t i, int comp,
                                                 const XT *__restrict__ x, int lane)
{
    const int32_t b = rows[i], e = rows[i + 1], len = e - b;
    const VT *__restrict__ v = vals + (int64_t)b * (BD * BD);
    double acc = 0.0;
    for (int32_t l = lane; l < len; l += 32) {
        const int32_t c = cols[b + l];
#pragma unroll
        for (int k = 0; k < BD; ++k) acc += (double)v[(int64_t)(comp * BD + k) * len + l] * (double)x[(int64_t)c * BD + k];
    }
    return group_sum<32>(acc);
}

// ---- double-float (an FP32 pair hi + lo) arithmetic on the FP32 pipe.  The
// intrinsics keep the compiler from contracting the error-free transforms.

// (sh, sl) += (ah + al) * (xh + xl): TwoProd of the high words (exact product
// and its rounding error by FMA), TwoSum into sh, the error terms and the two
// cross products into sl; al * xl (2^-48 relative) is dropped.
__device__ __forceinline__ void df_fma(float &sh, float &sl, float ah, float al, float xh, float xl)
{
    const float p = __fmul_rn(ah, xh);
    const float e = __fmaf_rn(ah, xh, -p);
    const float t = __fadd_rn(sh, p);
    const float z = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, z)), __fsub_rn(p, z));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, __fadd_rn(e, __fmaf_rn(ah, xl, __fmul_rn(al, xh)))));
}

// (ah, al) += (bh, bl)
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl)
{
    const float t = __fadd_rn(ah, bh);
    const float z = __fsub_rn(t, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(t, z)), __fsub_rn(bh, z));
    ah = t;
    al = __fadd_rn(__fadd_rn(al, bl), err);
}

// Block row i of A x in double-float: values and x as (hi, lo) pairs, one
// 8-byte load each.  The group reduction runs on the pairs with FP32
// shuffles; the sums are valid in every lane of the group.
template <int BD, int LANES>
__device__ __forceinline__ void bsr_block_row_df(const int32_t *__restrict__ rows, const int32_t *__restrict__ cols,
                                                 const float2 *__restrict__ vals, int32_t i, bool valid,
                                                 const float2 *__restrict__ x, int lane, float (&sh)[BD],
                                                 float (&sl)[BD])
{
    const int32_t b = valid ? rows[i] : 0, e = valid ? rows[i + 1] : 0, len = e - b;
    const float2 *__restrict__ v = vals + (int64_t)b * (BD * BD);
#pragma unroll
    for (int r = 0; r < BD; ++r) sh[r] = sl[r] = 0.f;
#pragma unroll 2
    for (int32_t l = lane; l < len; l += LANES) {
        const int32_t c = __ldcs(cols + b + l);
        float2 xv[BD];
#pragma unroll
        for (int k = 0; k < BD; ++k) xv[k] = x[(int64_t)c * BD + k];
#pragma unroll
        for (int r = 0; r < BD; ++r)
#pragma unroll
            for (int k = 0; k < BD; ++k) {
                const float2 a = __ldcs(v + (int64_t)(r * BD + k) * len + l);
                df_fma(sh[r], sl[r], a.x, a.y, xv[k].x, xv[k].y);
            }
    }
#pragma unroll
    for (int r = 0; r < BD; ++r)
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) {
            const float bh = __shfl_xor_sync(0xffffffffu, sh[r], o, LANES);
            const float bl = __shfl_xor_sync(0xffffffffu, sl[r], o, LANES);
            df_add(sh[r], sl[r], bh, bl);
        }
}

// bsr_block_row_df with x given as separate high and low FP32 arrays
template <int BD, int LANES>
__device__ __forceinline__ void bsr_block_row_df_split(const int32_t *__restrict__ rows,
                                                       const int32_t *__restrict__ cols,
                                                       const float2 *__restrict__ vals, int32_t i, bool valid,
                                                       const float *__restrict__ xh, const float *__restrict__ xl,
                                                       int lane, float (&sh)[BD], float (&sl)[BD])
{
    const int32_t b = valid ? rows[i] : 0, e = valid ? rows[i + 1] : 0, len = e - b;
    const float2 *__restrict__ v = vals + (int64_t)b * (BD * BD);
#pragma unroll
    for (int r = 0; r < BD; ++r) sh[r] = sl[r] = 0.f;
    for (int32_t l = lane; l < len; l += LANES) {
        const int32_t c = __ldcs(cols + b + l);
        float x1[BD], x2[BD];
#pragma unroll
        for (int k = 0; k < BD; ++k) {
            x1[k] = xh[(int64_t)c * BD + k];
            x2[k] = xl[(int64_t)c * BD + k];
        }
#pragma unroll
        for (int r = 0; r < BD; ++r)
#pragma unroll
            for (int k = 0; k < BD; ++k) {
                const float2 a = __ldcs(v + (int64_t)(r * BD + k) * len + l);
                df_fma(sh[r], sl[r], a.x, a.y, x1[k], x2[k]);
            }
    }
#pragma unroll
    for (int r = 0; r < BD; ++r)
#pragma unroll
        for (int o = LANES / 2; o > 0; o >>= 1) {
            const float bh = __shfl_xor_sync(0xffffffffu, sh[r], o, LANES);
            const float bl = __shfl_xor_sync(0xffffffffu, sl[r], o, LANES);
            df_add(sh[r], sl[r], bh, bl);
        }
}

}  // namespace lss
