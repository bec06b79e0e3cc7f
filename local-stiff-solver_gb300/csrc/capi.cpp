// extern "C" entry points (include/lss.h).  Every call converts exceptions
// into status codes and records the message; nothing here exits the process.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "baddof.hpp"
#include "batch.hpp"
#include "multifrontal.hpp"
#include "noalloc.hpp"
#include "postproc.hpp"
#include "solver.hpp"

namespace lss {
std::atomic<size_t> &alloc_cap_bytes()
{
    static std::atomic<size_t> cap{0};
    return cap;
}
std::atomic<size_t> &alloc_cap_base()
{
    static std::atomic<size_t> base{0};
    return base;
}
std::atomic<unsigned long long> &launch_count()
{
    static std::atomic<unsigned long long> c{0};
    return c;
}
std::atomic<size_t> &alloc_live_bytes()
{
    static std::atomic<size_t> live{0};
    return live;
}
void raise_smem_limit(const void *kernel, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> set;
    int dev = 0;
    LSS_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = set[{dev, kernel}];
    if (bytes <= cur) return;
    LSS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    // the largest shared-memory carveout, so that as many CTAs as fit are resident
    LSS_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
    cur = bytes;
}
int sm_grid(int per_sm)
{
    constexpr int MAX_DEVICES = 64;
    static std::atomic<int> sms[MAX_DEVICES] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
        cudaGetLastError();
        dev = -1;
    }
    int n = dev >= 0 && dev < MAX_DEVICES ? sms[dev].load() : 0;
    if (n <= 0) {
        if (dev < 0 || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
            cudaGetLastError();
            n = 1;
        }
        if (dev >= 0 && dev < MAX_DEVICES) sms[dev] = n;
    }
    const long long g = (long long)n * (per_sm > 0 ? per_sm : 1);
    return (int)std::min<long long>(g, GRID_MAX);
}
}  // namespace lss

struct lss_solver {
    lss::HybridSolver *impl = nullptr;
};

struct lss_batch {
    lss::BatchSolver *impl = nullptr;
    std::string last_error;
};

namespace {
thread_local std::string g_create_error;

template <typename F>
lss_status guarded(lss_solver *s, F f)
{
    try {
        f();
        if (s) s->impl->last_error.clear();
        return LSS_OK;
    } catch (const lss::Error &e) {
        if (s) s->impl->last_error = e.what();
        else g_create_error = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        if (s) s->impl->last_error = "host allocation failed";
        else g_create_error = "host allocation failed";
        return LSS_ERR_OOM;
    } catch (const std::exception &e) {
        if (s) s->impl->last_error = e.what();
        else g_create_error = e.what();
        return LSS_ERR_INTERNAL;
    }
}

bool valid(const lss_solver *s) { return s && s->impl; }

lss_status copy_out(const std::string &src, char *buf, size_t cap, size_t *len)
{
    if (len) *len = src.size();
    if (!buf || cap <= src.size()) {
        if (buf && cap) buf[0] = '\0';
        return LSS_ERR_BUFFER_TOO_SMALL;
    }
    std::memcpy(buf, src.c_str(), src.size() + 1);
    return LSS_OK;
}
}  // namespace

extern "C" {

const char *lss_status_string(lss_status s)
{
    switch (s) {
    case LSS_OK: return "ok";
    case LSS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case LSS_ERR_CUDA: return "CUDA error";
    case LSS_ERR_OOM: return "out of memory";
    case LSS_ERR_NOT_FACTORIZED: return "not factorized";
    case LSS_ERR_NOT_SPD: return "matrix block not positive definite";
    case LSS_ERR_NONFINITE: return "non-finite input";
    case LSS_ERR_INTERNAL: return "internal error";
    case LSS_ERR_BUFFER_TOO_SMALL: return "buffer too small";
    case LSS_ERR_NO_DEVICE: return "no CUDA device";
    case LSS_ERR_UNSUPPORTED: return "unsupported";
    }
    return "unknown status";
}

const char *lss_last_error(const lss_solver *s)
{
    if (!s) return g_create_error.c_str();
    if (!s->impl) return "invalid solver";
    return s->impl->last_error.c_str();
}

lss_status lss_create(const char *params_json, lss_solver **out)
{
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    lss::HybridSolver *impl = nullptr;
    lss_status st = guarded(nullptr, [&]() {
        lss::Params p = lss::parse_params(params_json, lss::Params());
        if (p.memory_cap_bytes) {
            lss::alloc_cap_bytes() = 0;
            lss::alloc_cap_base() = lss::alloc_live_bytes().load();
            lss::alloc_cap_bytes() = p.memory_cap_bytes;
        }
        impl = new lss::HybridSolver(p);
    });
    if (st != LSS_OK) return st;
    *out = new lss_solver{impl};
    return LSS_OK;
}

lss_status lss_destroy(lss_solver *s)
{
    if (!s) return LSS_OK;
    delete s->impl;
    delete s;
    return LSS_OK;
}

lss_status lss_set_parameters(lss_solver *s, const char *params_json)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->set_parameters(params_json); });
}

lss_status lss_get_info(const lss_solver *s, char *buf, size_t cap, size_t *len)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return copy_out(s->impl->info_json(), buf, cap, len);
}

lss_status lss_name(const lss_solver *s, char *buf, size_t cap)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return copy_out(s->impl->name(), buf, cap, nullptr);
}

lss_status lss_analyze_pattern(lss_solver *s, int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->analyze(n, nnz, outer, inner); });
}

lss_status lss_factorize(lss_solver *s, int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                         const double *values)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->factorize(n, nnz, outer, inner, values); });
}

lss_status lss_factorize_device(lss_solver *s, const double *d_values, void *stream)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->factorize_device(d_values, (cudaStream_t)stream); });
}

lss_status lss_set_problematic_dofs(lss_solver *s, const int32_t *idx, int32_t count)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->set_problematic_dofs(idx, count); });
}

lss_status lss_solve(lss_solver *s, const double *b, double *x, int32_t nrhs, int64_t ld)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() {
        if (nrhs < 0 || (nrhs > 1 && ld < s->impl->n())) lss::fail(LSS_ERR_INVALID_ARGUMENT, "invalid nrhs / ld");
        for (int32_t k = 0; k < nrhs; ++k) s->impl->solve_host(b + (int64_t)k * ld, x + (int64_t)k * ld);
    });
}

lss_status lss_solve_device(lss_solver *s, const double *d_b, double *d_x, void *stream)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->solve_device(d_b, d_x, (cudaStream_t)stream); });
}

lss_status lss_solve_transpose(lss_solver *s, const double *g, double *lambda)
{
    // A is symmetric positive definite: A^T lambda = g is the same system
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->solve_host(g, lambda); });
}

lss_status lss_grad_A_pattern(lss_solver *s, const double *lambda, const double *x, double *dA_values)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->grad_pattern_host(lambda, x, dA_values); });
}

lss_status lss_grad_A_pattern_device(lss_solver *s, const double *d_lambda, const double *d_x, double *d_dA_values,
                                     void *stream)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->grad_pattern_device(d_lambda, d_x, d_dA_values, (cudaStream_t)stream); });
}

lss_status lss_grad_params_device(lss_solver *s, const double *d_lambda, const double *d_x, int32_t n_params,
                                  const int64_t *d_mt_rowptr, const int32_t *d_mt_cols, const double *d_mt_vals,
                                  double *d_dtheta, void *stream)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() {
        s->impl->grad_params_device(d_lambda, d_x, n_params, d_mt_rowptr, d_mt_cols, d_mt_vals, d_dtheta,
                                    (cudaStream_t)stream);
    });
}

lss_status lss_assemble_values_device(int64_t n_values, const int64_t *d_m_rowptr, const int32_t *d_m_cols,
                                      const double *d_m_vals, const double *d_theta, const double *d_c,
                                      double *d_values, void *stream)
{
    if (n_values < 0 || (n_values > 0 && (!d_m_rowptr || !d_m_cols || !d_m_vals || !d_theta || !d_values))) {
        g_create_error = "invalid parameter-map arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        lss::launch_assemble_values(n_values, d_m_rowptr, d_m_cols, d_m_vals, d_theta, d_c, d_values,
                                    (cudaStream_t)stream);
    });
}

lss_status lss_selected_dofs(const lss_solver *s, int32_t *out, int32_t cap, int32_t *count)
{
    if (!valid(s) || !count) return LSS_ERR_INVALID_ARGUMENT;
    const std::vector<int32_t> sel = s->impl->selected();
    *count = (int32_t)sel.size();
    if (!out) return LSS_OK;
    if (cap < (int32_t)sel.size()) return LSS_ERR_BUFFER_TOO_SMALL;
    std::memcpy(out, sel.data(), sel.size() * sizeof(int32_t));
    return LSS_OK;
}

lss_status lss_gmm_selection(const lss_solver *s, int32_t *out, int32_t cap, int32_t *count)
{
    if (!valid(s) || !count) return LSS_ERR_INVALID_ARGUMENT;
    const std::vector<int32_t> &sel = s->impl->gmm_selection();
    *count = (int32_t)sel.size();
    if (!out) return LSS_OK;
    if (cap < (int32_t)sel.size()) return LSS_ERR_BUFFER_TOO_SMALL;
    std::memcpy(out, sel.data(), sel.size() * sizeof(int32_t));
    return LSS_OK;
}

lss_status lss_subdomains(const lss_solver *s, int32_t *offsets, int32_t cap_offsets, int32_t *dofs, int32_t cap_dofs,
                          int32_t *nsub, int32_t *ndofs)
{
    if (!valid(s) || !nsub || !ndofs) return LSS_ERR_INVALID_ARGUMENT;
    const auto &subs = s->impl->subdomains();
    int64_t total = 0;
    for (const auto &v : subs) total += (int64_t)v.size();
    *nsub = (int32_t)subs.size();
    *ndofs = (int32_t)total;
    if (!offsets || !dofs) return LSS_OK;
    if (cap_offsets < (int32_t)subs.size() + 1 || cap_dofs < total) return LSS_ERR_BUFFER_TOO_SMALL;
    int32_t pos = 0;
    offsets[0] = 0;
    for (size_t k = 0; k < subs.size(); ++k) {
        std::memcpy(dofs + pos, subs[k].data(), subs[k].size() * sizeof(int32_t));
        pos += (int32_t)subs[k].size();
        offsets[k + 1] = pos;
    }
    return LSS_OK;
}

lss_status lss_partition(const lss_solver *s, int32_t *perm, int32_t cap_perm, int32_t *part_offsets,
                         int32_t cap_offsets, int32_t *nparts)
{
    if (!valid(s) || !nparts) return LSS_ERR_INVALID_ARGUMENT;
    const auto &P = s->impl->pattern();
    *nparts = P.part.part_offsets.empty() ? 0 : (int32_t)P.part.part_offsets.size() - 1;
    if (!perm || !part_offsets) return LSS_OK;
    if (cap_perm < (int32_t)P.part.perm.size() || cap_offsets < (int32_t)P.part.part_offsets.size())
        return LSS_ERR_BUFFER_TOO_SMALL;
    std::memcpy(perm, P.part.perm.data(), P.part.perm.size() * sizeof(int32_t));
    std::memcpy(part_offsets, P.part.part_offsets.data(), P.part.part_offsets.size() * sizeof(int32_t));
    return LSS_OK;
}

lss_status lss_partition_pattern(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                 int32_t block_size, int32_t threads, int32_t *perm, int32_t cap_perm,
                                 int32_t *part_offsets, int32_t cap_offsets, int32_t *nparts)
{
    if (n <= 0 || nnz < 0 || !outer || !inner || block_size < 1 || !nparts) {
        g_create_error = "invalid partition arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        const lss::Pattern P = lss::analyze_pattern(n, nnz, outer, inner, block_size, threads);
        *nparts = (int32_t)P.part.part_offsets.size() - 1;
        if (!perm || !part_offsets) return;
        if (cap_perm < (int32_t)P.part.perm.size() || cap_offsets < (int32_t)P.part.part_offsets.size())
            lss::fail(LSS_ERR_BUFFER_TOO_SMALL, "partition output buffers too small");
        std::memcpy(perm, P.part.perm.data(), P.part.perm.size() * sizeof(int32_t));
        std::memcpy(part_offsets, P.part.part_offsets.data(), P.part.part_offsets.size() * sizeof(int32_t));
    });
}

namespace {
// the multifrontal plan of one stiff subdomain (dofs ascending) of a pattern
lss::MfSymbolic elimination_plan(int32_t n, const int32_t *outer, const int32_t *inner, int32_t block_size,
                                 const int32_t *dofs, int32_t ndofs)
{
    const int32_t bd = block_size, nb = n / bd;
    for (int32_t k = 0; k < ndofs; ++k)
        if (dofs[k] < 0 || dofs[k] >= n || (k > 0 && dofs[k] <= dofs[k - 1]))
            lss::fail(LSS_ERR_INVALID_ARGUMENT, "dofs must be ascending ids below n");
    // block pattern (outer index = row, as the solver reads it)
    std::vector<int32_t> rows{0}, cols, mark(nb, -1);
    for (int32_t I = 0; I < nb; ++I) {
        for (int32_t i = I * bd; i < (I + 1) * bd; ++i)
            for (int64_t e = outer[i]; e < outer[i + 1]; ++e) {
                const int32_t J = inner[e] / bd;
                if (J < 0 || J >= nb) lss::fail(LSS_ERR_INVALID_ARGUMENT, "inner index out of range");
                if (mark[J] != I) {
                    mark[J] = I;
                    cols.push_back(J);
                }
            }
        std::sort(cols.begin() + rows.back(), cols.end());
        rows.push_back((int32_t)cols.size());
    }
    const std::vector<int32_t> d(dofs, dofs + ndofs), off{0, ndofs};
    return lss::mf_symbolic(d, off, 0, rows, cols, bd);
}
}  // namespace

lss_status lss_stiff_elimination_plan(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                      int32_t block_size, const int32_t *dofs, int32_t ndofs, int64_t *counts,
                                      int32_t *front_p0, int32_t *front_s, int32_t *front_u, int32_t *bnd_off,
                                      int32_t *bnd_pos, int32_t *child_off, int32_t *child, int32_t *pos2j)
{
    if (n <= 0 || nnz < 0 || !outer || !inner || block_size < 1 || n % block_size || !dofs || ndofs <= 0 ||
        !counts) {
        g_create_error = "invalid elimination-plan arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        const lss::MfSymbolic M = elimination_plan(n, outer, inner, block_size, dofs, ndofs);
        counts[0] = M.nfront;
        counts[1] = M.npos;
        counts[2] = (int64_t)M.bnd_pos.size();
        counts[3] = (int64_t)M.child.size();
        if (!front_p0 || !front_s || !front_u || !bnd_off || !bnd_pos || !child_off || !child || !pos2j) return;
        std::copy(M.p0.begin(), M.p0.end(), front_p0);
        std::copy(M.s.begin(), M.s.end(), front_s);
        std::copy(M.u.begin(), M.u.end(), front_u);
        std::copy(M.bnd_off.begin(), M.bnd_off.end(), bnd_off);
        std::copy(M.bnd_pos.begin(), M.bnd_pos.end(), bnd_pos);
        std::copy(M.child_off.begin(), M.child_off.end(), child_off);
        std::copy(M.child.begin(), M.child.end(), child);
        std::copy(M.pos2j.begin(), M.pos2j.end(), pos2j);
    });
}

lss_status lss_stiff_elimination_tree(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                      int32_t block_size, const int32_t *dofs, int32_t ndofs, double *out)
{
    if (n <= 0 || nnz < 0 || !outer || !inner || block_size < 1 || n % block_size || !dofs || ndofs <= 0 || !out) {
        g_create_error = "invalid elimination-tree arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        const lss::MfSymbolic M = elimination_plan(n, outer, inner, block_size, dofs, ndofs);
        out[0] = M.nfront;
        out[1] = M.levels;
        out[2] = M.max_f;
        out[3] = M.fmas;
    });
}

lss_status lss_postprocess_selection(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner,
                                     const double *values, const char *params_json, const int32_t *sel,
                                     int32_t nsel, int32_t *sub_off, int32_t cap_off, int32_t *sub_dofs,
                                     int32_t cap_dofs, int32_t *nsub)
{
    if (n <= 0 || nnz < 0 || !outer || !inner || !values || nsel < 0 || (nsel > 0 && !sel) || !nsub) {
        g_create_error = "invalid post-processing arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        const lss::Params p = lss::parse_params(params_json, lss::Params());
        std::vector<int32_t> s(sel, sel + nsel);
        for (int32_t k = 0; k < nsel; ++k)
            if (s[k] < 0 || s[k] >= n || (k > 0 && s[k] <= s[k - 1]))
                lss::fail(LSS_ERR_INVALID_ARGUMENT, "sel must be ascending ids below n");
        const lss::CscView A{n, nnz, outer, inner, nullptr};
        // the solver's steps after the GMM selection (HybridSolver::select_stiff)
        if (p.decompose) {
            // Gershgorin data of the selected submatrix: diagonal entry and the
            // sum of |a| over the other selected columns of the row
            std::vector<uint8_t> mask((size_t)n, 0);
            for (int32_t k : s) mask[k] = 1;
            std::vector<double> diag(s.size(), 0.0), off(s.size(), 0.0);
            for (size_t a = 0; a < s.size(); ++a) {
                const int32_t k = s[a];
                for (int64_t e = outer[k]; e < outer[k + 1]; ++e) {
                    const int32_t j = inner[e];
                    if (j < 0 || j >= n) lss::fail(LSS_ERR_INVALID_ARGUMENT, "inner index out of range");
                    if (!mask[j]) continue;
                    if (j == k) diag[a] = values[e];
                    else off[a] += std::fabs(values[e]);
                }
            }
            s = lss::filter_subdomains(A, s, diag, off, p.min_sub, p.max_sub, p.cond_threshold, nullptr);
        }
        if (p.expand && !s.empty()) s = lss::expand_subdomains(A, s);
        std::vector<std::vector<int32_t>> subs;
        if (!s.empty()) subs = lss::decompose_subdomains(A, s, p.decompose ? (int64_t)p.max_sub : INT64_MAX);
        *nsub = (int32_t)subs.size();
        if (!sub_off || !sub_dofs) return;
        int64_t total = 0;
        for (const auto &c : subs) total += (int64_t)c.size();
        if (cap_off < *nsub + 1 || cap_dofs < total)
            lss::fail(LSS_ERR_BUFFER_TOO_SMALL, "post-processing output buffers too small");
        int32_t at = 0;
        sub_off[0] = 0;
        for (int32_t q = 0; q < *nsub; ++q) {
            std::copy(subs[q].begin(), subs[q].end(), sub_dofs + at);
            at += (int32_t)subs[q].size();
            sub_off[q + 1] = at;
        }
    });
}

lss_status lss_coarse_space(int32_t n, int64_t nnz, const int32_t *outer, const int32_t *inner, int32_t block_size,
                            int32_t max_coarse_levels, int32_t *levels, int32_t *items, int32_t cap_items,
                            int32_t *cmap, int64_t cap_cmap)
{
    if (n <= 0 || nnz < 0 || !outer || !inner || block_size < 1 || !levels || max_coarse_levels < 0) {
        g_create_error = "invalid coarse-space arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        const lss::Pattern P = lss::analyze_pattern(n, nnz, outer, inner, block_size, 0);
        const lss::CoarseSpace cs = lss::build_coarse_space(P, max_coarse_levels);
        *levels = cs.L;
        if (!items || !cmap) return;
        if (cap_items < cs.L || cap_cmap < (int64_t)cs.cmap.size())
            lss::fail(LSS_ERR_BUFFER_TOO_SMALL, "coarse-space output buffers too small");
        for (int l = 0; l < cs.L; ++l) items[l] = l == 0 ? P.nb : cs.nitems[l];
        std::copy(cs.cmap.begin(), cs.cmap.end(), cmap);
    });
}

lss_status lss_op_row_l1_norms(int32_t n, int64_t nnz, const int32_t *outer, const double *values, double *rn)
{
    if (n <= 0 || nnz < 0 || !outer || !values || !rn) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(nullptr, [&]() {
        if (outer[0] != 0 || (int64_t)outer[n] != nnz)
            lss::fail(LSS_ERR_INVALID_ARGUMENT, "outer index must start at 0 and end at nnz");
        for (int32_t i = 0; i < n; ++i)
            if (outer[i + 1] < outer[i]) lss::fail(LSS_ERR_INVALID_ARGUMENT, "outer index is not monotone");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            lss::fail(LSS_ERR_NO_DEVICE, "no CUDA device available");
        }
        cudaStream_t st;
        LSS_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        {
            lss::DBuf<int32_t> d_outer;
            lss::DBuf<double> d_vals, d_rn(n);
            d_outer.upload(outer, (size_t)n + 1, st);
            d_vals.upload(values, (size_t)nnz, st);
            lss::launch_row_l1_norms(n, nnz, d_outer.data(), d_vals.data(), d_rn.data(), st);
            LSS_CUDA(cudaMemcpyAsync(rn, d_rn.data(), (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, st));
            LSS_CUDA(cudaStreamSynchronize(st));
        }
        cudaStreamDestroy(st);
    });
}

lss_status lss_op_spmv(lss_solver *s, const double *x, double *y)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->op_spmv(x, y); });
}

lss_status lss_op_spmv_outer(lss_solver *s, const double *x, double *y)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->op_spmv_outer(x, y); });
}

lss_status lss_op_mas_apply(lss_solver *s, const double *r, double *z)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->op_mas(r, z); });
}

lss_status lss_op_precond(lss_solver *s, const double *r, double *z)
{
    if (!valid(s)) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->op_precond(r, z); });
}

lss_status lss_op_time(lss_solver *s, int32_t kind, int32_t reps, double *ms_per_launch, double *bytes_per_launch)
{
    if (!valid(s) || !ms_per_launch || !bytes_per_launch) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->op_time(kind, reps, ms_per_launch, bytes_per_launch); });
}

lss_status lss_set_memory_cap(size_t bytes)
{
    lss::alloc_cap_bytes() = 0;  // no reservation sees the new base with the old cap
    lss::alloc_cap_base() = lss::alloc_live_bytes().load();
    lss::alloc_cap_bytes() = bytes;
    return LSS_OK;
}

}  // extern "C"

lss_status lss_gmm_select_device_noalloc(int32_t n, int64_t nnz, const int32_t *d_outer, const double *d_values,
                                         double gmm_jump_threshold, double gmm_tol, int32_t max_gmm_iterations,
                                         int32_t *d_selected, int32_t *d_count, void *stream)
{
    return guarded(nullptr, [&]() {
        lss::noalloc_gmm_select(n, nnz, d_outer, d_values, gmm_jump_threshold, gmm_tol, max_gmm_iterations,
                                d_selected, d_count, (cudaStream_t)stream);
    });
}

namespace {
// Runs work(s) for every system from a pool of host threads (threads <= 0:
// one per system); returns the first failing system's status.
template <typename F>
lss_status for_each_system(lss_solver *const *solvers, int32_t count, int32_t threads, F work)
{
    for (int32_t s = 0; s < count; ++s)
        if (!valid(solvers[s])) {
            g_create_error = "invalid solver of system " + std::to_string(s);
            return LSS_ERR_INVALID_ARGUMENT;
        }
    // one host thread drives each solver: the systems must be distinct objects
    for (int32_t s = 0; s < count; ++s)
        for (int32_t t = s + 1; t < count; ++t)
            if (solvers[s] == solvers[t]) {
                g_create_error = "batched systems must be distinct solver objects";
                return LSS_ERR_INVALID_ARGUMENT;
            }
    if (count == 0) return LSS_OK;
    // the calling thread runs a worker, which selects each solver's device:
    // the caller's current device is restored on every exit path
    struct DeviceRestore {
        int dev = -1;
        DeviceRestore()
        {
            if (cudaGetDevice(&dev) != cudaSuccess) {
                cudaGetLastError();
                dev = -1;
            }
        }
        ~DeviceRestore()
        {
            if (dev >= 0) cudaSetDevice(dev);
        }
    } restore;
    const int nthreads = threads > 0 ? std::min<int>(threads, count) : count;
    std::atomic<int32_t> next{0};
    std::mutex mu;
    lss_status first = LSS_OK;
    std::string first_msg;
    auto worker = [&]() {
        for (;;) {
            const int32_t s = next.fetch_add(1);
            if (s >= count) return;
            lss_solver *sv = solvers[s];
            const lss_status st = guarded(sv, [&]() {
                LSS_CUDA(cudaSetDevice(sv->impl->device()));
                work(s, sv);
            });
            if (st != LSS_OK) {
                std::lock_guard<std::mutex> lock(mu);
                if (first == LSS_OK) {
                    first = st;
                    first_msg = "system " + std::to_string(s) + ": " + sv->impl->last_error;
                }
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto &th : pool) th.join();
    if (first != LSS_OK) g_create_error = first_msg;
    return first;
}
}  // namespace

lss_status lss_factorize_batched_device(lss_solver *const *solvers, int32_t count, const double *const *d_values,
                                        int32_t threads)
{
    if (count < 0 || (count > 0 && (!solvers || !d_values))) {
        g_create_error = "invalid batched-factorize arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    for (int32_t s = 0; s < count; ++s)
        if (!d_values[s]) {
            g_create_error = "null values of system " + std::to_string(s);
            return LSS_ERR_INVALID_ARGUMENT;
        }
    return for_each_system(solvers, count, threads,
                           [&](int32_t s, lss_solver *sv) { sv->impl->factorize_device(d_values[s], nullptr); });
}

lss_status lss_solve_batched_device(lss_solver *const *solvers, int32_t count, const double *const *d_b,
                                    double *const *d_x, int32_t nrhs, int32_t threads, int32_t *iterations)
{
    if (count < 0 || nrhs < 0 || (count > 0 && (!solvers || !d_b || !d_x))) {
        g_create_error = "invalid batched-solve arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    for (int32_t s = 0; s < count && nrhs > 0; ++s)
        if (!d_b[s] || !d_x[s]) {
            g_create_error = "null vector of system " + std::to_string(s);
            return LSS_ERR_INVALID_ARGUMENT;
        }
    if (nrhs == 0) return for_each_system(solvers, count, threads, [](int32_t, lss_solver *) {});
    return for_each_system(solvers, count, threads, [&](int32_t s, lss_solver *sv) {
        const int64_t n = sv->impl->n();
        for (int32_t k = 0; k < nrhs; ++k) {
            sv->impl->solve_device(d_b[s] + k * n, d_x[s] + k * n, nullptr);
            if (iterations) iterations[(int64_t)s * nrhs + k] = sv->impl->iterations();
        }
    });
}

lss_status lss_op_row_scores(lss_solver *s, double *diag_abs, double *offdiag_max, double *l1)
{
    if (!valid(s) || !diag_abs || !offdiag_max || !l1) return LSS_ERR_INVALID_ARGUMENT;
    return guarded(s, [&]() { s->impl->op_row_scores(diag_abs, offdiag_max, l1); });
}

lss_status lss_op_select_bad_dofs(int32_t strategy, int32_t n, const double *score, double p1, double p2, int32_t i1,
                                  int32_t i2, int32_t *out, int32_t *count)
{
    if (n < 0 || (n > 0 && !score) || !count || strategy < 1 || strategy > 3) {
        g_create_error = "invalid bad-DOF selection arguments";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    return guarded(nullptr, [&]() {
        const std::vector<double> v(score, score + n);
        std::vector<int32_t> sel;
        if (strategy == lss::BADDOF_ELBOW) sel = lss::mas_select_elbow(v);
        else if (strategy == lss::BADDOF_KMEAN) sel = lss::mas_select_kmean(v, p1, p2, i1, i2);
        else sel = lss::mas_select_gmm(v, p1, p2, i1, i2);
        *count = (int32_t)sel.size();
        if (out) std::copy(sel.begin(), sel.end(), out);
    });
}

// ---- batched PCG (batch.hpp)

namespace {
template <typename F>
lss_status batch_guarded(lss_batch *b, F f)
{
    try {
        f();
        b->last_error.clear();
        return LSS_OK;
    } catch (const lss::Error &e) {
        b->last_error = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        b->last_error = "host allocation failed";
        return LSS_ERR_OOM;
    } catch (const std::exception &e) {
        b->last_error = e.what();
        return LSS_ERR_INTERNAL;
    }
}
}  // namespace

lss_status lss_batch_create(lss_solver *const *solvers, int32_t count, lss_batch **out)
{
    if (!out) return LSS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (count <= 0 || !solvers) {
        g_create_error = "a batch needs at least one solver";
        return LSS_ERR_INVALID_ARGUMENT;
    }
    std::vector<lss::HybridSolver *> sys(count);
    for (int32_t s = 0; s < count; ++s) {
        if (!valid(solvers[s])) {
            g_create_error = "invalid solver of system " + std::to_string(s);
            return LSS_ERR_INVALID_ARGUMENT;
        }
        sys[s] = solvers[s]->impl;
    }
    lss::BatchSolver *impl = nullptr;
    const lss_status st = guarded(nullptr, [&]() { impl = new lss::BatchSolver(sys, sys[0]->device()); });
    if (st != LSS_OK) return st;
    *out = new lss_batch{impl, std::string()};
    return LSS_OK;
}

lss_status lss_batch_destroy(lss_batch *b)
{
    if (!b) return LSS_OK;
    delete b->impl;
    delete b;
    return LSS_OK;
}

const char *lss_batch_last_error(const lss_batch *b)
{
    if (!b) return g_create_error.c_str();
    return b->last_error.c_str();
}

lss_status lss_batch_factorize_device(lss_batch *b, const double *const *d_values, int32_t threads)
{
    if (!b || !b->impl || !d_values) return LSS_ERR_INVALID_ARGUMENT;
    return batch_guarded(b, [&]() {
        lss::CudaDeviceGuard guard(b->impl->device());
        b->impl->factorize_device(d_values, threads);
    });
}

lss_status lss_batch_solve_device(lss_batch *b, const double *const *d_b, double *const *d_x, int32_t *iterations)
{
    if (!b || !b->impl || !d_b || !d_x) return LSS_ERR_INVALID_ARGUMENT;
    return batch_guarded(b, [&]() {
        lss::CudaDeviceGuard guard(b->impl->device());
        b->impl->solve_device(d_b, d_x, iterations);
    });
}

lss_status lss_batch_get_info(const lss_batch *b, char *buf, size_t cap, size_t *len)
{
    if (!b || !b->impl) return LSS_ERR_INVALID_ARGUMENT;
    return copy_out(b->impl->info_json(), buf, cap, len);
}
