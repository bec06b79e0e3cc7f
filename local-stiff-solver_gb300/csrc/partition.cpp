// Graph partition of the block graph into parts of <= 32 block rows for MAS.
//
// The reference calls KaMinPar (GraphPartition.cpp:176-289) with
// k = ceil(n / 30) parts and a maximum block weight of 32.  KaMinPar is not
// available, so this is a from-scratch recursive bisection designed around
// what MAS needs from a partition:
//   * the same k = ceil(n / 30), so leaves hold about 30 nodes (<= 32);
//   * connected parts: each half is a breadth-first prefix from a
//     pseudo-peripheral node (connected by construction); when the remainder
//     falls apart, its small pieces are swapped with the last-visited nodes of
//     the prefix until it is connected again;
//   * bank alignment: a subtree with k parts is split at a multiple of the
//     largest power of 32 below k, so every aligned run of 32^l consecutive
//     parts is one subtree -- one compact, connected region.  MAS's coarse
//     level l groups 32 consecutive components of level l-1, so with connected,
//     aligned parts every coarse level shrinks by about 32x;
//   * nodes without couplings (e.g. Dirichlet rows kept as identity rows) are
//     packed into parts of their own after all others, so they cannot break
//     that alignment.
// Subtrees run on host threads; the result does not depend on the thread count.
#include <algorithm>
#include <atomic>
#include <thread>

#include "partition.hpp"

namespace lss {
namespace {

constexpr int32_t PART = 32;
constexpr int32_t TARGET = 30;

struct Ctx {
    const int32_t *rows;
    const int32_t *cols;
    std::vector<int32_t> owner;  // task id currently owning each node
    std::vector<int32_t> seen;   // visit stamp per node
    std::atomic<int32_t> next_task{1};
    std::atomic<int32_t> next_stamp{1};
    std::vector<std::vector<int32_t>> parts;  // parts[p] = node list
};

// Breadth-first order of `nodes` (all owned by `task`) from `start`, restarting
// at the next unvisited node of `nodes` for disconnected pieces.
void bfs_order(Ctx &c, int32_t task, const std::vector<int32_t> &nodes, int32_t start, std::vector<int32_t> &order)
{
    const int32_t stamp = c.next_stamp.fetch_add(1);
    order.clear();
    order.reserve(nodes.size());
    size_t head = 0, scan = 0;
    int32_t s = start;
    for (;;) {
        if (c.seen[s] != stamp) {
            c.seen[s] = stamp;
            order.push_back(s);
            while (head < order.size()) {
                const int32_t u = order[head++];
                for (int32_t k = c.rows[u]; k < c.rows[u + 1]; ++k) {
                    const int32_t v = c.cols[k];
                    if (c.owner[v] == task && c.seen[v] != stamp) {
                        c.seen[v] = stamp;
                        order.push_back(v);
                    }
                }
            }
        }
        while (scan < nodes.size() && c.seen[nodes[scan]] == stamp) ++scan;
        if (scan == nodes.size()) break;
        s = nodes[scan];
    }
}

// Connected components of `nodes` (owned by `task`): comp[i] for nodes[i]
// aligned with the returned list order; returns the component lists.
std::vector<std::vector<int32_t>> components(Ctx &c, int32_t task, const std::vector<int32_t> &nodes)
{
    std::vector<std::vector<int32_t>> comps;
    const int32_t stamp = c.next_stamp.fetch_add(1);
    std::vector<int32_t> q;
    for (int32_t s : nodes) {
        if (c.seen[s] == stamp) continue;
        q.clear();
        q.push_back(s);
        c.seen[s] = stamp;
        for (size_t h = 0; h < q.size(); ++h) {
            const int32_t u = q[h];
            for (int32_t k = c.rows[u]; k < c.rows[u + 1]; ++k) {
                const int32_t v = c.cols[k];
                if (c.owner[v] == task && c.seen[v] != stamp) {
                    c.seen[v] = stamp;
                    q.push_back(v);
                }
            }
        }
        comps.push_back(q);
    }
    return comps;
}

// Parts of a subtree with k leaves in the left child: a multiple of the
// largest power of 32 below k (bank alignment of MAS's coarse levels).
int32_t left_parts(int32_t k)
{
    int64_t B = 1;
    while (B * PART < k) B *= PART;
    const int64_t g = (k + B - 1) / B;
    int64_t k1 = (g / 2) * B;
    if (k1 <= 0 || k1 >= k) k1 = k / 2;
    return (int32_t)k1;
}

void split(Ctx &c, int32_t task, std::vector<int32_t> nodes, int32_t part0, int32_t k, int32_t depth,
           int32_t spawn_depth)
{
    const int32_t m = (int32_t)nodes.size();
    if (k <= 1 || m <= 1) {
        std::vector<int32_t> o;
        if (m > 1) {
            bfs_order(c, task, nodes, nodes[0], o);
            bfs_order(c, task, nodes, o.back(), o);
        } else {
            o = nodes;
        }
        c.parts[part0] = std::move(o);
        return;
    }
    const int32_t k1 = left_parts(k), k2 = k - k1;
    int64_t m1 = ((int64_t)m * k1 + k / 2) / k;
    m1 = std::max<int64_t>(m1, m - (int64_t)PART * k2);
    m1 = std::min<int64_t>(m1, (int64_t)PART * k1);
    m1 = std::max<int64_t>(1, std::min<int64_t>(m1, m - 1));
    std::vector<int32_t> order;
    bfs_order(c, task, nodes, nodes[0], order);
    bfs_order(c, task, nodes, order.back(), order);
    // left = BFS prefix (connected); right = the rest
    const int32_t tl = c.next_task.fetch_add(1), tr = c.next_task.fetch_add(1);
    std::vector<int32_t> left(order.begin(), order.begin() + m1), right(order.begin() + m1, order.end());
    for (int32_t v : left) c.owner[v] = tl;
    for (int32_t v : right) c.owner[v] = tr;
    // reconnect the right side: swap its small pieces with the prefix's tail
    for (int round = 0; round < 4; ++round) {
        auto comps = components(c, tr, right);
        if (comps.size() <= 1) break;
        size_t big = 0;
        for (size_t q = 1; q < comps.size(); ++q)
            if (comps[q].size() > comps[big].size()) big = q;
        std::vector<int32_t> pieces;
        for (size_t q = 0; q < comps.size(); ++q)
            if (q != big) pieces.insert(pieces.end(), comps[q].begin(), comps[q].end());
        if (pieces.size() >= left.size()) break;
        // the last nodes of the prefix go right, the pieces go left
        std::vector<int32_t> moved(left.end() - pieces.size(), left.end());
        left.resize(left.size() - pieces.size());
        for (int32_t v : pieces) c.owner[v] = tl;
        for (int32_t v : moved) c.owner[v] = tr;
        left.insert(left.end(), pieces.begin(), pieces.end());
        right = comps[big];
        right.insert(right.end(), moved.begin(), moved.end());
    }
    if (depth < spawn_depth) {
        std::thread th([&c, tl, l = std::move(left), part0, k1, depth, spawn_depth]() mutable {
            split(c, tl, std::move(l), part0, k1, depth + 1, spawn_depth);
        });
        split(c, tr, std::move(right), part0 + k1, k2, depth + 1, spawn_depth);
        th.join();
    } else {
        split(c, tl, std::move(left), part0, k1, depth + 1, spawn_depth);
        split(c, tr, std::move(right), part0 + k1, k2, depth + 1, spawn_depth);
    }
}

}  // namespace

Partition partition_graph(int32_t nb, const int32_t *rows, const int32_t *cols, int threads)
{
    Partition out;
    if (nb <= 0) {
        out.part_offsets = {0};
        return out;
    }
    Ctx c;
    c.rows = rows;
    c.cols = cols;
    c.owner.assign(nb, 0);
    c.seen.assign(nb, 0);
    std::vector<int32_t> coupled, isolated;
    for (int32_t i = 0; i < nb; ++i) {
        bool any = false;
        for (int32_t q = rows[i]; q < rows[i + 1] && !any; ++q) any = cols[q] != i;
        (any ? coupled : isolated).push_back(i);
    }
    for (int32_t v : isolated) c.owner[v] = -1;
    const int32_t m = (int32_t)coupled.size();
    const int32_t k = m == 0 ? 0 : (m <= PART ? 1 : (m + TARGET - 1) / TARGET);
    c.parts.resize(k);
    if (threads <= 0) threads = (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    int spawn_depth = 0;
    while ((1 << spawn_depth) < threads) ++spawn_depth;
    if (k > 0) split(c, 0, std::move(coupled), 0, k, 0, spawn_depth);
    for (size_t s = 0; s < isolated.size(); s += PART)
        c.parts.emplace_back(isolated.begin() + s, isolated.begin() + std::min(isolated.size(), s + PART));

    out.perm.assign(nb, -1);
    out.part_offsets.assign(1, 0);
    int32_t next = 0;
    for (const auto &p : c.parts) {
        if (p.empty()) continue;
        // a leaf larger than a bank (possible only after the reconnect swaps) is cut in BFS order
        for (size_t s = 0; s < p.size(); s += PART) {
            const size_t e = std::min(p.size(), s + PART);
            for (size_t q = s; q < e; ++q) out.perm[p[q]] = next++;
            out.part_offsets.push_back(next);
        }
    }
    return out;
}

}  // namespace lss
