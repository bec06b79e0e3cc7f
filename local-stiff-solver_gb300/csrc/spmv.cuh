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

}  // namespace lss
