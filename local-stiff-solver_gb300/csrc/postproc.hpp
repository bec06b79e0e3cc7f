// Host post-processing of the stiff-DOF selection (GPUHybrid.cu:691-991).
#pragma once

#include <cstdint>
#include <vector>

namespace lss {

// Non-owning view of the caller's compressed matrix (outer index = row).
struct CscView {
    int32_t n = 0;
    int64_t nnz = 0;
    const int32_t *outer = nullptr;
    const int32_t *inner = nullptr;
    const double *values = nullptr;
};

struct FilterCounters {
    int32_t too_small = 0, too_large = 0, not_poorly_conditioned = 0;
};

// Keep the connected components of `sel` (ascending) whose size lies in
// [min_size, max_size] and whose Gershgorin bounds flag them as poorly
// conditioned.  Result ascending.
// diag[a], off[a]: A_kk and sum_{j in sel, j != k} |A_kj| of k = sel[a]
// (computed on the device, launch_gershgorin).
std::vector<int32_t> filter_subdomains(const CscView &A, const std::vector<int32_t> &sel,
                                       const std::vector<double> &diag, const std::vector<double> &off,
                                       int32_t min_size, int32_t max_size, double cond_threshold,
                                       FilterCounters *cnt);

// One-ring expansion: every row index stored in the selected outer slices.
std::vector<int32_t> expand_subdomains(const CscView &A, const std::vector<int32_t> &sel);

// Connected components of `sel`, those larger than max_size dropped; each
// component ascending, components ordered by their smallest member.
std::vector<std::vector<int32_t>> decompose_subdomains(const CscView &A, const std::vector<int32_t> &sel,
                                                       int64_t max_size);

}  // namespace lss
