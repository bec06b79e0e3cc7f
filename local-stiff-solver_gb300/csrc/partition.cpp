// Graph partition of the block graph into parts of <= 32 block rows for MAS.
//
// The reference calls KaMinPar (GraphPartition.cpp:176-289, k = ceil(n/30),
// max block weight 32).  KaMinPar is not available, so this is a from-scratch
// recursive bisection: each subgraph of m nodes is split into
// ceil(m/32)-proportional halves along a breadth-first level structure rooted
// at a pseudo-peripheral node, until parts hold <= 32 nodes.  The in-order
// sequence of leaves is the part order, so consecutive parts are graph
// neighbours at every scale -- which is what MAS's coarse levels (banks of 32
// consecutive components) rely on.  Subtrees run on a pool of host threads;
// the result does not depend on the thread count.
#include <algorithm>
#include <atomic>
#include <thread>

#include "partition.hpp"

namespace lss {
namespace {

constexpr int32_t PART = 32;

struct Ctx {
    const int32_t *rows;
    const int32_t *cols;
    std::vector<int32_t> owner;  // task id currently owning each node
    std::vector<int32_t> seen;   // BFS stamp per node
    std::atomic<int32_t> next_task{1};
    std::atomic<int32_t> next_stamp{1};
    std::vector<std::vector<int32_t>> parts;  // parts[p] = node list
};

// Breadth-first order of `nodes` (all owned by `task`) starting at `start`,
// restarting at the next unvisited node of `nodes` for disconnected pieces.
void bfs_order(Ctx &c, int32_t task, const std::vector<int32_t> &nodes, int32_t start,
               std::vector<int32_t> &order)
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

void split(Ctx &c, int32_t task, std::vector<int32_t> nodes, int32_t part0, int32_t depth,
           int32_t spawn_depth)
{
    const int32_t m = (int32_t)nodes.size();
    if (m <= PART) {
        // order inside the part: BFS from a pseudo-peripheral node keeps lanes local
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
    const int32_t k = (m + PART - 1) / PART;
    const int32_t k1 = k / 2, k2 = k - k1;
    int64_t m1 = ((int64_t)m * k1 + k / 2) / k;
    m1 = std::max<int64_t>(m1, m - (int64_t)PART * k2);
    m1 = std::min<int64_t>(m1, (int64_t)PART * k1);
    std::vector<int32_t> order;
    bfs_order(c, task, nodes, nodes[0], order);
    const int32_t far = order.back();
    bfs_order(c, task, nodes, far, order);
    std::vector<int32_t> left(order.begin(), order.begin() + m1);
    std::vector<int32_t> right(order.begin() + m1, order.end());
    const int32_t tl = c.next_task.fetch_add(1), tr = c.next_task.fetch_add(1);
    for (int32_t v : left) c.owner[v] = tl;
    for (int32_t v : right) c.owner[v] = tr;
    if (depth < spawn_depth) {
        std::thread th([&c, tl, l = std::move(left), part0, k1, depth, spawn_depth]() mutable {
            split(c, tl, std::move(l), part0, depth + 1, spawn_depth);
        });
        split(c, tr, std::move(right), part0 + k1, depth + 1, spawn_depth);
        th.join();
    } else {
        split(c, tl, std::move(left), part0, depth + 1, spawn_depth);
        split(c, tr, std::move(right), part0 + k1, depth + 1, spawn_depth);
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
    const int32_t k = (nb + PART - 1) / PART;
    c.parts.resize(k);
    if (threads <= 0) threads = (int)std::min(16u, std::max(1u, std::thread::hardware_concurrency()));
    int spawn_depth = 0;
    while ((1 << spawn_depth) < threads) ++spawn_depth;
    std::vector<int32_t> all(nb);
    for (int32_t i = 0; i < nb; ++i) all[i] = i;
    split(c, 0, std::move(all), 0, 0, spawn_depth);

    out.perm.assign(nb, -1);
    out.part_offsets.assign(1, 0);
    int32_t next = 0;
    for (const auto &p : c.parts) {
        if (p.empty()) continue;
        for (int32_t v : p) out.perm[v] = next++;
        out.part_offsets.push_back(next);
    }
    return out;
}

}  // namespace lss
