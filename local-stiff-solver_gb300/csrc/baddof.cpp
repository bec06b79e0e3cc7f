// MASSolver's bad-DOF selections, on the host as in the reference (the scores
// come from the device, select.cu launch_row_scores).  Built with
// -ffp-contract=off so that every platform rounds these expression trees alike.
#include "baddof.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <numeric>

namespace lss {
namespace {

// positions sorted by score (ties by position: a total order)
std::vector<int32_t> by_score(const std::vector<double> &key, bool descending)
{
    std::vector<int32_t> order(key.size());
    std::iota(order.begin(), order.end(), 0);
    std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        if (key[a] != key[b]) return descending ? key[a] > key[b] : key[a] < key[b];
        return a < b;
    });
    return order;
}

// the hit positions of `visit`, each widened to [pos - w, pos + w]; first-seen order
std::vector<int32_t> widen_hits(int32_t n, const std::vector<int32_t> &visit, const std::vector<char> &hit, int w)
{
    std::vector<int32_t> out;
    if (w <= 0) {
        for (size_t t = 0; t < visit.size(); ++t)
            if (hit[t]) out.push_back(visit[t]);
        return out;
    }
    std::vector<char> taken(n, 0);
    for (size_t t = 0; t < visit.size(); ++t) {
        if (!hit[t]) continue;
        const int32_t pos = visit[t];
        for (int32_t j = std::max(0, pos - w); j <= std::min(n - 1, pos + w); ++j)
            if (!taken[j]) {
                taken[j] = 1;
                out.push_back(j);
            }
    }
    return out;
}

double relative_change(double now, double before)
{
    return std::fabs(now - before) / std::max(std::fabs(before), 1e-300);
}

double log_density(double x, double mean, double var)
{
    const double two_pi = 2.0 * 3.141592653589793238462643383279502884;
    return -0.5 * std::log(two_pi * var) - 0.5 * (x - mean) * (x - mean) / var;
}

}  // namespace

std::vector<int32_t> mas_select_elbow(const std::vector<double> &d)
{
    const int32_t n = (int32_t)d.size();
    if (n == 0) return {};
    const std::vector<int32_t> order = by_score(d, false);
    int32_t cut = 0;
    if (n > 1) {
        const double lo = std::log(d[order.front()]), hi = std::log(d[order.back()]);
        double best = -1.0;
        for (int32_t i = 0; i < n; ++i) {
            const double chord = (hi - lo) / (n - 1.0) * i + lo;
            const double dev = std::fabs(chord - std::log(d[order[i]]));
            if (dev > best) {
                best = dev;
                cut = i;
            }
        }
    }
    return std::vector<int32_t>(order.begin() + cut, order.end());
}

std::vector<int32_t> mas_select_kmean(const std::vector<double> &v, double search_fraction, double jump_threshold,
                                      int max_iterations, int expand_neighbors)
{
    const int32_t n = (int32_t)v.size();
    if (n < 2) return {};
    std::vector<int32_t> order = by_score(v, true);
    const int32_t m = std::clamp((int32_t)(n * search_fraction), 2, n);
    order.resize(m);
    // centres start at the subset's extremes; a value counts toward the
    // cluster of the other centre and the second centre moves only with two or
    // more members, as in the reference
    double c0 = v[order.front()], c1 = v[order.back()];
    for (int it = 0; it < max_iterations; ++it) {
        double sum[2] = {0.0, 0.0};
        int32_t cnt[2] = {0, 0};
        for (int32_t p : order) {
            const int cid = std::fabs(v[p] - c0) < std::fabs(v[p] - c1) ? 1 : 0;
            ++cnt[cid];
            sum[cid] += v[p];
        }
        const double n0 = cnt[0] > 0 ? sum[0] / cnt[0] : c0;
        const double n1 = cnt[1] > 1 ? sum[1] / cnt[1] : c1;
        if (n0 == c0 && n1 == c1) break;
        c0 = n0;
        c1 = n1;
    }
    if (c0 < c1) std::swap(c0, c1);
    const double ratio = c0 / c1;
    if (std::isnan(ratio) || ratio < jump_threshold) return {};
    const double sep = 0.5 * (c0 + c1);
    std::vector<char> hit(m);
    for (int32_t t = 0; t < m; ++t) hit[t] = v[order[t]] > sep;
    return widen_hits(n, order, hit, expand_neighbors);
}

std::vector<int32_t> mas_select_gmm(const std::vector<double> &x, double jump_threshold, double tol,
                                    int max_iterations, int expand_neighbors)
{
    const int32_t n = (int32_t)x.size();
    if (n < 2) return {};
    double sum = 0.0;
    for (double a : x) sum += a;
    const double gmean = sum / n;
    double vsum = 0.0;
    for (double a : x) {
        const double d = a - gmean;
        vsum += d * d;
    }
    const double gvar = vsum / n;
    const auto mm = std::minmax_element(x.begin(), x.end());
    double m0 = *mm.first, m1 = *mm.second;
    constexpr double var_reg = 1e-6;
    double v0 = std::max(gvar, var_reg), v1 = v0, w0 = 0.5, w1 = 0.5;
    if (m0 == m1 || !std::isfinite(gvar)) return {};
    std::vector<double> g0(n, 0.0), g1(n, 0.0);
    const int iters = std::max(1, max_iterations);
    for (int it = 0; it < iters; ++it) {
        const double lw0 = std::log(std::max(w0, DBL_MIN)), lw1 = std::log(std::max(w1, DBL_MIN));
        for (int32_t i = 0; i < n; ++i) {
            const double a = lw0 + log_density(x[i], m0, v0);
            const double b = lw1 + log_density(x[i], m1, v1);
            const double top = std::max(a, b);
            const double total = top + std::log(std::exp(a - top) + std::exp(b - top));
            g0[i] = std::exp(a - total);
            g1[i] = std::exp(b - total);
        }
        double s0 = 0.0, s1 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            s0 += g0[i];
            s1 += g1[i];
        }
        if (s0 <= 0.0 || s1 <= 0.0) break;
        w0 = s0 / n;
        w1 = s1 / n;
        const double pm0 = m0, pm1 = m1, pv0 = v0, pv1 = v1;
        m0 = 0.0;
        m1 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            m0 += g0[i] * x[i];
            m1 += g1[i] * x[i];
        }
        m0 /= s0;
        m1 /= s1;
        v0 = 0.0;
        v1 = 0.0;
        for (int32_t i = 0; i < n; ++i) {
            const double d0 = x[i] - m0, d1 = x[i] - m1;
            v0 += g0[i] * d0 * d0;
            v1 += g1[i] * d1 * d1;
        }
        v0 = v0 / s0 + var_reg;
        v1 = v1 / s1 + var_reg;
        if (relative_change(m0, pm0) < tol && relative_change(m1, pm1) < tol && relative_change(v0, pv0) < tol &&
            relative_change(v1, pv1) < tol)
            break;
    }
    const bool high0 = std::fabs(m0) > std::fabs(m1);
    const double ratio = high0 ? std::fabs(m0) / std::fabs(m1) : std::fabs(m1) / std::fabs(m0);
    if (std::isnan(ratio) || ratio < jump_threshold) return {};
    std::vector<int32_t> visit(n);
    std::iota(visit.begin(), visit.end(), 0);
    std::vector<char> hit(n);
    for (int32_t i = 0; i < n; ++i) hit[i] = high0 ? g0[i] > g1[i] : g1[i] > g0[i];
    return widen_hits(n, visit, hit, expand_neighbors);
}

}  // namespace lss
