// Allocation-free stiff-DOF selection: l1 row norms -> two-component GMM ->
// rows of the stiff component, on caller-owned device arrays.
//
// The stages are the launchers the solver's own selection uses (select.cu);
// what differs is where their intermediates live.  The solver allocates the
// norms, the GMM state, the per-CTA counts and the selection per call and
// prefix-sums the counts on the host; this variant keeps every intermediate
// in one file-scope static device array and prefix-sums on the device, so a
// call allocates nothing (no cudaMalloc / cudaFree, no allocating library)
// and never synchronises with the host.
//
// Scratch layout (256-byte aligned sections of g_noalloc_scratch):
//   rn            NOALLOC_MAX_ROWS doubles          row l1 norms
//   partials      GRID_MAX * RED_MAX_VALUES doubles grid-reduction partials
//   block_margin  NOALLOC_MAX_BLOCKS doubles        per-CTA decision margins
//   block_count   NOALLOC_MAX_BLOCKS int32          per-CTA selected counts
//   block_offset  NOALLOC_MAX_BLOCKS int32          their exclusive prefix sum
//   gmm           one GmmState                      fully written by the stats
//                                                   and variance kernels
//   counter       one unsigned                      grid-reduction arrivals
// Only `counter` must start at zero: static device memory is zero when the
// module loads, and every grid reduction resets it to zero on completion.
#include "device_common.cuh"
#include "kernels.hpp"
#include "lss_common.hpp"
#include "noalloc.hpp"

namespace lss {
namespace {

constexpr int32_t NOALLOC_MAX_BLOCKS = NOALLOC_MAX_ROWS / 256;  // mark / scatter CTAs of 256 rows

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }

constexpr size_t OFF_RN = 0;
constexpr size_t OFF_PARTIALS = OFF_RN + align256(sizeof(double) * NOALLOC_MAX_ROWS);
constexpr size_t OFF_MARGIN = OFF_PARTIALS + align256(sizeof(double) * GRID_MAX * RED_MAX_VALUES);
constexpr size_t OFF_COUNT = OFF_MARGIN + align256(sizeof(double) * NOALLOC_MAX_BLOCKS);
constexpr size_t OFF_OFFSET = OFF_COUNT + align256(sizeof(int32_t) * NOALLOC_MAX_BLOCKS);
constexpr size_t OFF_GMM = OFF_OFFSET + align256(sizeof(int32_t) * NOALLOC_MAX_BLOCKS);
constexpr size_t OFF_COUNTER = OFF_GMM + align256(sizeof(GmmState));
constexpr size_t SCRATCH_BYTES = OFF_COUNTER + 256;
static_assert(SCRATCH_BYTES == NOALLOC_SCRATCH_BYTES, "scratch size out of sync with noalloc.hpp");

static __device__ __align__(256) unsigned char g_noalloc_scratch[SCRATCH_BYTES];

// Device address of the scratch in the current context.  Looked up on every
// call rather than cached: after cudaDeviceReset, or in another context on the
// same device, the module is loaded again and the array can move, and a cached
// address would then point at unmapped memory.  cudaGetSymbolAddress
// allocates nothing; the lookup that first loads the module on a device (the
// first call there, or the first after a reset) must not happen inside a
// stream capture.
unsigned char *scratch_base()
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cudaGetLastError();
        fail(e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? LSS_ERR_NO_DEVICE : LSS_ERR_CUDA,
             std::string("cudaGetSymbolAddress of the selection scratch failed: ") + cudaGetErrorString(e));
    }
    return (unsigned char *)p;
}

// Exclusive prefix sum of the per-CTA counts (one CTA of 1024 threads, each
// owning a contiguous run of counts) and the total.
__global__ void __launch_bounds__(1024) block_offsets_kernel(int32_t nblk, const int32_t *__restrict__ count,
                                                             int32_t *__restrict__ offset, int32_t *__restrict__ total)
{
    __shared__ int32_t wsum[32];
    const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    const int32_t per = (nblk + blockDim.x - 1) / blockDim.x;
    const int32_t lo = min(nblk, t * per), hi = min(nblk, lo + per);
    int32_t s = 0;
    for (int32_t b = lo; b < hi; ++b) s += count[b];
    // inclusive scan of s over the CTA
    int32_t v = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) wsum[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int32_t w = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += u;
        }
        wsum[lane] = w;
    }
    __syncthreads();
    int32_t run = v - s + (wid > 0 ? wsum[wid - 1] : 0);
    for (int32_t b = lo; b < hi; ++b) {
        offset[b] = run;
        run += count[b];
    }
    if (t == blockDim.x - 1) *total = wsum[(blockDim.x >> 5) - 1];
}

}  // namespace

void noalloc_gmm_select(int32_t n, int64_t nnz, const int32_t *d_outer, const double *d_values, double threshold,
                        double tol, int32_t max_iterations, int32_t *d_selected, int32_t *d_count, cudaStream_t s)
{
    if (n < 0 || nnz < 0 || max_iterations < 0) fail(LSS_ERR_INVALID_ARGUMENT, "negative size or iteration count");
    if (n > NOALLOC_MAX_ROWS)
        fail(LSS_ERR_INVALID_ARGUMENT, "n = " + std::to_string(n) + " exceeds the allocation-free limit of " +
                                           std::to_string(NOALLOC_MAX_ROWS) + " rows");
    if (!d_count || (n > 0 && (!d_outer || !d_values || !d_selected)))
        fail(LSS_ERR_INVALID_ARGUMENT, "null device pointer");
    unsigned char *base = scratch_base();
    double *rn = (double *)(base + OFF_RN);
    GridReduce gr{(double *)(base + OFF_PARTIALS), (unsigned *)(base + OFF_COUNTER)};
    double *margin = (double *)(base + OFF_MARGIN);
    int32_t *count = (int32_t *)(base + OFF_COUNT);
    int32_t *offset = (int32_t *)(base + OFF_OFFSET);
    GmmState *gmm = (GmmState *)(base + OFF_GMM);
    const int32_t nblk = (n + 255) / 256;
    if (n > 0) {
        launch_row_l1_norms(n, nnz, d_outer, d_values, rn, s);
        launch_gmm(n, rn, gmm, max_iterations, tol, gr, s);
        launch_gmm_mark(n, rn, gmm, threshold, count, margin, s);
    }
    block_offsets_kernel<<<1, 1024, 0, s>>>(nblk, count, offset, d_count);
    LSS_LAUNCH_CHECK();
    if (n > 0) launch_gmm_scatter(n, rn, gmm, threshold, offset, d_selected, s);
}

}  // namespace lss
