// Host post-processing of the stiff-DOF selection, as in the reference:
//   filter_subdomains                       GPUHybrid.cu:885-970
//   expand_subdomains_to_strongly_connected GPUHybrid.cu:972-991
//   decompose_subdomains_to_disjoint_subsets GPUHybrid.cu:691-735
// The work is proportional to the entries of the selected rows, so it stays on
// the host next to the caller's pattern arrays.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <numeric>

#include "postproc.hpp"

namespace lss {
namespace {

// union-find with path halving and union by rank
struct UnionFind {
    std::vector<int32_t> parent, rank;
    explicit UnionFind(int32_t n) : parent(n), rank(n, 0) { std::iota(parent.begin(), parent.end(), 0); }
    int32_t find(int32_t v)
    {
        while (parent[v] != v) {
            parent[v] = parent[parent[v]];
            v = parent[v];
        }
        return v;
    }
    void unite(int32_t a, int32_t b)
    {
        a = find(a);
        b = find(b);
        if (a == b) return;
        if (rank[a] < rank[b]) std::swap(a, b);
        parent[b] = a;
        if (rank[a] == rank[b]) ++rank[a];
    }
};

// Component label (0..nc-1, numbered by smallest member) of every entry of the
// ascending set `sel`, connectivity through A's stored entries.
int32_t label_components(const CscView &A, const std::vector<int32_t> &sel,
                         std::vector<int32_t> &g2l, std::vector<int32_t> &label)
{
    const int32_t m = (int32_t)sel.size();
    for (int32_t a = 0; a < m; ++a) g2l[sel[a]] = a;
    UnionFind uf(m);
    for (int32_t a = 0; a < m; ++a) {
        const int32_t k = sel[a];
        for (int64_t e = A.outer[k]; e < A.outer[k + 1]; ++e) {
            const int32_t r = A.inner[e];
            if (g2l[r] >= 0) uf.unite(g2l[r], a);
        }
    }
    label.assign(m, -1);
    std::vector<int32_t> root_label(m, -1);
    int32_t nc = 0;
    for (int32_t a = 0; a < m; ++a) {
        const int32_t r = uf.find(a);
        if (root_label[r] < 0) root_label[r] = nc++;
        label[a] = root_label[r];
    }
    return nc;
}

void clear_g2l(std::vector<int32_t> &g2l, const std::vector<int32_t> &sel)
{
    for (int32_t v : sel) g2l[v] = -1;
}

}  // namespace

std::vector<int32_t> filter_subdomains(const CscView &A, const std::vector<int32_t> &sel,
                                       const std::vector<double> &diag, const std::vector<double> &offsum,
                                       int32_t min_size, int32_t max_size, double cond_threshold,
                                       FilterCounters *cnt)
{
    std::vector<int32_t> g2l(A.n, -1), label;
    const int32_t nc = label_components(A, sel, g2l, label);
    std::vector<int64_t> size(nc, 0);
    std::vector<double> lmin(nc, DBL_MAX), lmax(nc, 0.0);
    for (size_t a = 0; a < sel.size(); ++a) {
        const int32_t c = label[a];
        ++size[c];
        lmin[c] = std::min(lmin[c], diag[a] - offsum[a]);
        lmax[c] = std::max(lmax[c], diag[a] + offsum[a]);
    }
    std::vector<char> keep(nc, 0);
    FilterCounters fc;
    for (int32_t c = 0; c < nc; ++c) {
        if (size[c] < min_size) { ++fc.too_small; continue; }
        if (size[c] > max_size) { ++fc.too_large; continue; }
        // Gershgorin test, GPUHybrid.cu:960
        if (lmin[c] * lmax[c] < 0.0 || lmax[c] / lmin[c] > cond_threshold) { keep[c] = 1; continue; }
        ++fc.not_poorly_conditioned;
    }
    std::vector<int32_t> out;
    out.reserve(sel.size());
    for (size_t a = 0; a < sel.size(); ++a)
        if (keep[label[a]]) out.push_back(sel[a]);
    if (cnt) *cnt = fc;
    return out;
}

std::vector<int32_t> expand_subdomains(const CscView &A, const std::vector<int32_t> &sel)
{
    std::vector<char> mark(A.n, 0);
    for (int32_t k : sel)
        for (int64_t e = A.outer[k]; e < A.outer[k + 1]; ++e) mark[A.inner[e]] = 1;
    std::vector<int32_t> out;
    for (int32_t i = 0; i < A.n; ++i)
        if (mark[i]) out.push_back(i);
    return out;
}

std::vector<std::vector<int32_t>> decompose_subdomains(const CscView &A, const std::vector<int32_t> &sel,
                                                       int64_t max_size)
{
    std::vector<int32_t> g2l(A.n, -1), label;
    const int32_t nc = label_components(A, sel, g2l, label);
    std::vector<std::vector<int32_t>> comps(nc);
    for (size_t a = 0; a < sel.size(); ++a) comps[label[a]].push_back(sel[a]);
    std::vector<std::vector<int32_t>> out;
    for (auto &c : comps)
        if ((int64_t)c.size() <= max_size) out.push_back(std::move(c));
    return out;
}

}  // namespace lss
