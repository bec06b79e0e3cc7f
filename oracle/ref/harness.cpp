// Harness around the reference's OWN stiff-DOF selection code -- TEST
// INFRASTRUCTURE ONLY (never linked by the product).
//
// oracle/build_ref.py extracts, unmodified, from the reference sources:
//   src/polysolve/linear/Hybrid.hpp     struct disjointSet
//   src/polysolve/linear/GPUHybrid.cu   GPUHybrid::select_bad_dofs (l1 row
//       norms + GMM EM + jump test, thrust), filter_subdomains,
//       expand_subdomains_to_strongly_connected,
//       decompose_subdomains_to_disjoint_subsets
// into oracle/_ref/gpuhybrid_selection.inc, and compiles this file with g++
// against CCCL's thrust on its sequential host backend
// (THRUST_DEVICE_SYSTEM_CPP: thrust::device_vector lives in host memory and
// thrust::device runs on the calling thread) and the Eigen stand-in in
// oracle/stubs.  This file supplies what the extracted code needs from its
// class and its translation unit -- the data members it reads and writes
// (declared as in GPUHybrid.hpp:69-126), name(), the phase clock, and
// SPDLOG_INFO -- and restates the four-line orchestration of
// GPUHybrid::factorize (GPUHybrid.cu:215-238).  SPDLOG_INFO records the
// arguments of the "[bad_dof_selection]" log line (GPUHybrid.cu:881-882),
// which carry the GMM statistics, so they can be compared too.
//
// Differences from the reference build that can matter: the device lambdas
// run on the host (glibc log/exp instead of CUDA's), and thrust's reductions
// run sequentially instead of as device tree reductions, so the GMM
// statistics may differ from a GPU run in the last bits; the unqualified abs()
// of the host code resolves to the floating-point overload.
#include <thrust/binary_search.h>
#include <thrust/copy.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/distance.h>
#include <thrust/execution_policy.h>
#include <thrust/extrema.h>
#include <thrust/for_each.h>
#include <thrust/gather.h>
#include <thrust/host_vector.h>
#include <thrust/inner_product.h>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/scatter.h>
#include <thrust/sequence.h>
#include <thrust/sort.h>
#include <thrust/transform.h>
#include <thrust/transform_reduce.h>

#include <Eigen/Sparse>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <iostream>
#include <limits>
#include <set>
#include <string>
#include <tuple>
#include <type_traits>
#include <unordered_map>
#include <vector>

namespace lssref {
// arguments of the last "[bad_dof_selection]" log line: global mean, global
// variance, mean_0, mean_1, var_0, var_1, gmm_iter, num_bad_dofs
thread_local double g_stats[8];
thread_local bool g_have_stats = false;

template <typename T>
double as_double(const T &v)
{
    if constexpr (std::is_arithmetic_v<std::decay_t<T>>) return (double)v;
    else return std::numeric_limits<double>::quiet_NaN();
}

template <typename... Args>
void log_line(const char *fmt, Args &&...args)
{
    if (!std::strstr(fmt, "[bad_dof_selection]")) return;
    if constexpr (sizeof...(Args) == 10) {
        const double v[10] = {as_double(args)...};
        for (int k = 0; k < 8; ++k) g_stats[k] = v[2 + k];
        g_have_stats = true;
    }
}
}  // namespace lssref

#define SPDLOG_INFO(...) ::lssref::log_line(__VA_ARGS__)

namespace polysolve::linear {

using std::abs;
using std::max;
using std::min;

namespace {
using clock = std::chrono::steady_clock;
double elapsed_seconds(const std::chrono::time_point<clock> &begin)
{
    return std::chrono::duration<double>(clock::now() - begin).count();
}
}  // namespace

#include "gpuhybrid_disjoint_set.inc"

class GPUHybrid {
public:
    std::string name() const { return "GPUHybrid"; }

    // GPUHybrid.hpp:76-98 (defaults overwritten by every call)
    bool select_bad_dofs_from_l1_row_norm = true;
    bool decompose_subdomains = false;
    int min_subdomain_size = 1;
    int max_subdomain_size = 1e9;
    double gmm_jump_threshold = 100.0;
    double gmm_tol = 1e-3;
    int max_gmm_iterations = 20;
    bool expand_subdomains = true;
    double conditioning_threshold = 100.0;

    // GPUHybrid.hpp:108-116
    std::set<int> h_all_bad_dofs;
    thrust::device_vector<int> d_all_bad_dofs;
    std::vector<std::vector<int>> bad_indices_arrays;
    thrust::device_vector<int> d_outer_indices;
    thrust::device_vector<double> d_values;

    void decompose_subdomains_to_disjoint_subsets(const Eigen::SparseMatrix<double> &sparse_A);
    void filter_subdomains(const Eigen::SparseMatrix<double> &sparse_A);
    void expand_subdomains_to_strongly_connected(const Eigen::SparseMatrix<double> &sparse_A);
    void select_bad_dofs();
};

#include "gpuhybrid_selection.inc"

}  // namespace polysolve::linear

extern "C" {

// The reference's selection pipeline on one matrix (outer index = row, as in
// GPUHybrid::factorize).  raw[n]: the GMM selection (ascending); sub_off[n+1],
// sub_dofs[n]: the final subdomains in the reference's own order (each
// ascending); stats[8]: the "[bad_dof_selection]" log arguments.  Returns 0,
// or -1 on an exception (message in err, capacity errcap).
int lssref_select(int32_t n, const int32_t *outer, const int32_t *inner, const double *vals,
                  double gmm_jump_threshold, double gmm_tol, int32_t max_gmm_iterations,
                  double conditioning_threshold, int32_t decompose, int32_t min_sub, int32_t max_sub, int32_t expand,
                  int32_t *raw, int32_t *nraw, int32_t *sub_off, int32_t *sub_dofs, int32_t *nsub, double *stats,
                  char *err, int32_t errcap)
{
    try {
        polysolve::linear::GPUHybrid g;
        g.gmm_jump_threshold = gmm_jump_threshold;
        g.gmm_tol = gmm_tol;
        g.max_gmm_iterations = max_gmm_iterations;
        g.conditioning_threshold = conditioning_threshold;
        g.decompose_subdomains = decompose != 0;
        g.min_subdomain_size = min_sub;
        g.max_subdomain_size = max_sub;
        g.expand_subdomains = expand != 0;
        const int64_t nnz = outer[n];
        g.d_outer_indices.assign(outer, outer + n + 1);
        g.d_values.assign(vals, vals + nnz);
        Eigen::SparseMatrix<double> A;
        A.assign_compressed(n, n, outer, inner, vals);
        lssref::g_have_stats = false;

        // GPUHybrid.cu:215-238
        g.bad_indices_arrays.clear();
        g.select_bad_dofs();
        *nraw = (int32_t)g.h_all_bad_dofs.size();
        std::copy(g.h_all_bad_dofs.begin(), g.h_all_bad_dofs.end(), raw);
        if (g.decompose_subdomains) g.filter_subdomains(A);
        if (g.expand_subdomains) g.expand_subdomains_to_strongly_connected(A);
        if (g.decompose_subdomains) g.decompose_subdomains_to_disjoint_subsets(A);
        else g.bad_indices_arrays.emplace_back(g.h_all_bad_dofs.begin(), g.h_all_bad_dofs.end());

        int32_t k = 0;
        sub_off[0] = 0;
        for (size_t s = 0; s < g.bad_indices_arrays.size(); ++s) {
            for (int v : g.bad_indices_arrays[s]) sub_dofs[k++] = v;
            sub_off[s + 1] = k;
        }
        *nsub = (int32_t)g.bad_indices_arrays.size();
        for (int q = 0; q < 8; ++q)
            stats[q] = lssref::g_have_stats ? lssref::g_stats[q] : std::numeric_limits<double>::quiet_NaN();
        return 0;
    } catch (const std::exception &e) {
        if (err && errcap > 0) {
            std::strncpy(err, e.what(), (size_t)errcap - 1);
            err[errcap - 1] = '\0';
        }
        return -1;
    }
}

}  // extern "C"
