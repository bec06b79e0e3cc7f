// Device helpers shared by the sm_103a kernels: warp/block reductions and the
// deterministic grid reduction ("last CTA finishes": every CTA writes its
// partial, the last one to arrive sums all partials in a fixed order, so the
// result depends only on the grid size, never on scheduling).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"

namespace lss {

constexpr int WARP = 32;
constexpr int BANK = 32;  // MAS bank width (MASPreconditioner.cu:33)

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the CTA; the result is valid in thread 0.  smem: >= 32 * NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *smem)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NV; ++k) smem[wid * NV + k] = v[k];
    __syncthreads();
    if (wid == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? smem[lane * NV + k] : 0.0;
            v[k] = warp_sum(t);
        }
    }
}

// Grid-wide deterministic sum.  Every thread of every CTA must call it.
// Returns true in exactly one thread (thread 0 of the last CTA), where
// total[] holds the sums; the arrival counter is reset for the next use.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], GridReduce gr, double (&total)[NV])
{
    __shared__ double smem[32 * RED_MAX_VALUES];
    __shared__ bool last;
    block_sum<NV>(v, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) gr.partials[blockIdx.x * NV + k] = v[k];
        __threadfence();
        unsigned t = atomicAdd(gr.counter, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] += __ldcg(gr.partials + b * NV + k);
    block_sum<NV>(acc, smem);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) total[k] = acc[k];
        *gr.counter = 0u;
        return true;
    }
    return false;
}

// Grid-wide min/max (deterministic, order independent).
__device__ __forceinline__ double warp_min(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ double warp_max(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}


}  // namespace lss
