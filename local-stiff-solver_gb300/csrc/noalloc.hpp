// Allocation-free stiff-DOF selection on caller-owned device arrays
// (lss_gmm_select_device_noalloc in include/lss.h).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "lss_common.hpp"

namespace lss {

// Largest system the static scratch holds, and the scratch's size in bytes:
// 8 MiB of row norms plus the reduction partials, per-CTA counts and offsets,
// the GMM state and the arrival counter.
constexpr int32_t NOALLOC_MAX_ROWS = LSS_NOALLOC_MAX_ROWS;
constexpr size_t NOALLOC_SCRATCH_BYTES = 8716800;

// Throws lss::Error (LSS_ERR_INVALID_ARGUMENT for n > NOALLOC_MAX_ROWS, before
// any device work).  Stream-ordered on s; no host synchronisation.
void noalloc_gmm_select(int32_t n, int64_t nnz, const int32_t *d_outer, const double *d_values, double threshold,
                        double tol, int32_t max_iterations, int32_t *d_selected, int32_t *d_count, cudaStream_t s);

}  // namespace lss
