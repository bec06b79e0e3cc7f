// Symbolic phase of the multifrontal stiff-block factor (host): nested
// dissection of every large subdomain's node graph, the elimination order,
// and the fronts with their boundaries and extend-add maps.
//
// Nested dissection: a connected node set above the leaf size is split by a
// level set of a breadth-first search from a pseudo-peripheral node (the
// smallest level near the median), thinned by moving separator nodes with no
// neighbour on the far side back; disconnected sets become sibling subtrees.
// Fronts are numbered in postorder (children first), and positions are
// handed out front by front, so a subtree's variables are contiguous and a
// front's own variables come last in it.  A front's boundary is the set of
// later variables coupled to its subtree: the later neighbours of its own
// variables plus the children's boundaries, minus its own variables.
#include <algorithm>
#include <numeric>

#include "multifrontal.hpp"

namespace lss {
namespace {

constexpr int32_t LEAF_DOFS = 48;

struct Nd {
    const std::vector<int32_t> &aoff, &adj;  // local node graph (no self loops)
    int32_t leaf_nodes;
    std::vector<int32_t> stamp, lvl;
    int32_t cur = 0;
    std::vector<std::vector<int32_t>> own;       // fronts: own nodes
    std::vector<std::vector<int32_t>> children;  // fronts: child fronts (local ids)

    Nd(const std::vector<int32_t> &o, const std::vector<int32_t> &a, int32_t nn, int32_t leaf)
        : aoff(o), adj(a), leaf_nodes(leaf), stamp(nn, 0), lvl(nn, -1)
    {
    }

    int32_t make(std::vector<int32_t> nodes, std::vector<int32_t> kids)
    {
        std::sort(nodes.begin(), nodes.end());
        own.push_back(std::move(nodes));
        children.push_back(std::move(kids));
        return (int32_t)own.size() - 1;
    }

    // members of `nodes` get stamp `st`
    void mark(const std::vector<int32_t> &nodes, int32_t st)
    {
        for (int32_t v : nodes) stamp[v] = st;
    }

    // breadth-first levels from `src` over the stamped set; returns the order
    std::vector<int32_t> bfs(int32_t src, int32_t st)
    {
        std::vector<int32_t> q{src};
        lvl[src] = 0;
        const int32_t seen = -st;  // visited marker, distinct from every membership stamp
        stamp[src] = seen;
        for (size_t h = 0; h < q.size(); ++h) {
            const int32_t v = q[h];
            for (int32_t k = aoff[v]; k < aoff[v + 1]; ++k) {
                const int32_t w = adj[k];
                if (stamp[w] == st) {
                    stamp[w] = seen;
                    lvl[w] = lvl[v] + 1;
                    q.push_back(w);
                }
            }
        }
        for (int32_t v : q) stamp[v] = st;  // restore membership
        return q;
    }

    std::vector<int32_t> dissect(std::vector<int32_t> nodes)
    {
        if ((int32_t)nodes.size() <= leaf_nodes) return {make(std::move(nodes), {})};
        const int32_t st = ++cur;
        mark(nodes, st);
        // connected components
        std::vector<int32_t> order = bfs(nodes[0], st);
        if (order.size() < nodes.size()) {
            std::vector<std::vector<int32_t>> comps;
            const int32_t cs = ++cur;
            for (int32_t v : nodes) {
                if (stamp[v] != st) continue;
                std::vector<int32_t> c = bfs(v, st);
                mark(c, cs);  // claimed
                comps.push_back(std::move(c));
            }
            std::vector<int32_t> roots;
            for (auto &c : comps) {
                std::vector<int32_t> r = dissect(std::move(c));
                roots.insert(roots.end(), r.begin(), r.end());
            }
            return roots;
        }
        // pseudo-peripheral start: the last node of a BFS, twice
        order = bfs(order.back(), st);
        order = bfs(order.back(), st);
        const int32_t depth = lvl[order.back()];
        if (depth < 2) return {make(std::move(nodes), {})};
        std::vector<int32_t> count(depth + 1, 0);
        for (int32_t v : order) ++count[lvl[v]];
        // the separator level: the smallest level among those that leave at
        // least 30% of the nodes on either side (balanced subtrees keep the
        // tree shallow); the median level when no level does
        const int64_t nn = (int64_t)nodes.size();
        int32_t med = 0, acc = 0;
        while (med < depth && 2 * (acc + count[med]) < (int32_t)nn) acc += count[med++];
        int32_t best = std::clamp(med, 1, depth - 1);
        int64_t below = 0;
        int32_t best_cnt = -1;
        for (int32_t l = 0; l <= depth; ++l) {
            const int64_t above = nn - below - count[l];
            if (l >= 1 && l <= depth - 1 && 10 * std::min(below, above) >= 3 * nn &&
                (best_cnt < 0 || count[l] < best_cnt)) {
                best = l;
                best_cnt = count[l];
            }
            below += count[l];
        }
        std::vector<int32_t> A, B, S;
        for (int32_t v : order) (lvl[v] < best ? A : (lvl[v] > best ? B : S)).push_back(v);
        // thin: a separator node without a neighbour in B joins A
        std::vector<int32_t> S2;
        for (int32_t v : S) {
            bool touches_b = false;
            for (int32_t k = aoff[v]; k < aoff[v + 1] && !touches_b; ++k)
                touches_b = stamp[adj[k]] == st && lvl[adj[k]] > best;
            (touches_b ? S2 : A).push_back(v);
        }
        if (A.empty() || B.empty() || S2.empty()) return {make(std::move(nodes), {})};
        std::vector<int32_t> kids = dissect(std::move(A));
        std::vector<int32_t> kb = dissect(std::move(B));
        kids.insert(kids.end(), kb.begin(), kb.end());
        return {make(std::move(S2), std::move(kids))};
    }
};

}  // namespace

MfSymbolic mf_symbolic(const std::vector<int32_t> &dofs, const std::vector<int32_t> &off, int32_t first_large,
                       const std::vector<int32_t> &rows, const std::vector<int32_t> &cols, int bd)
{
    MfSymbolic M;
    const int32_t nsub = (int32_t)off.size() - 1;
    if (first_large >= nsub) return M;
    M.j_base = off[first_large];
    const int32_t nj = off[nsub] - M.j_base;
    M.j2pos.assign(nj, -1);
    M.pos2j.assign(nj, -1);
    M.front_of_pos.assign(nj, -1);
    const int32_t nb = (int32_t)rows.size() - 1;
    std::vector<int32_t> node_local(nb, -1);
    std::vector<int32_t> pos_stamp(nj, -1);
    std::vector<int32_t> parent;
    int32_t pos = 0;
    M.bnd_off.push_back(0);
    M.child_off.push_back(0);
    for (int32_t k = first_large; k < nsub; ++k) {
        const int32_t J0 = off[k], m = off[k + 1] - J0;
        // nodes of the subdomain and their DOF ranges (dofs ascending => grouped by node)
        std::vector<int32_t> node_g, node_l0{0};
        for (int32_t l = 0; l < m; ++l) {
            const int32_t I = dofs[J0 + l] / bd;
            if (node_g.empty() || node_g.back() != I) {
                if (!node_g.empty()) node_l0.push_back(l);
                node_g.push_back(I);
            }
        }
        node_l0.push_back(m);
        const int32_t nn = (int32_t)node_g.size();
        for (int32_t a = 0; a < nn; ++a) node_local[node_g[a]] = a;
        std::vector<int32_t> aoff{0}, adj;
        for (int32_t a = 0; a < nn; ++a) {
            const int32_t I = node_g[a];
            for (int32_t q = rows[I]; q < rows[I + 1]; ++q) {
                const int32_t b = node_local[cols[q]];
                if (b >= 0 && b != a) adj.push_back(b);
            }
            aoff.push_back((int32_t)adj.size());
        }
        Nd nd(aoff, adj, nn, std::max(1, LEAF_DOFS / bd));
        std::vector<int32_t> all(nn);
        std::iota(all.begin(), all.end(), 0);
        nd.dissect(std::move(all));
        // positions, front by front (postorder)
        const int32_t fbase = M.nfront;
        std::vector<int32_t> node_pos0(nn, -1);
        for (size_t f = 0; f < nd.own.size(); ++f) {
            const int32_t id = fbase + (int32_t)f;
            M.p0.push_back(pos);
            for (int32_t a : nd.own[f]) {
                node_pos0[a] = pos;
                for (int32_t l = node_l0[a]; l < node_l0[a + 1]; ++l) {
                    M.pos2j[pos] = J0 + l;
                    M.j2pos[J0 + l - M.j_base] = pos;
                    M.front_of_pos[pos] = id;
                    ++pos;
                }
            }
            M.s.push_back(pos - M.p0.back());
            parent.push_back(-1);
            std::vector<int32_t> kids;
            for (int32_t c : nd.children[f]) kids.push_back(fbase + c);
            std::sort(kids.begin(), kids.end());
            int32_t h = 0;
            for (int32_t c : kids) {
                parent[c] = id;
                h = std::max(h, M.height[c] + 1);
            }
            M.height.push_back(h);
            M.child.insert(M.child.end(), kids.begin(), kids.end());
            M.child_off.push_back((int32_t)M.child.size());
            M.bnd_off.push_back(0);  // set below, once every position of the subdomain is known
        }
        M.nfront += (int32_t)nd.own.size();
        // boundaries (all positions of the subdomain are known now)
        std::vector<std::vector<int32_t>> bnd_lists(nd.own.size());
        for (size_t f = 0; f < nd.own.size(); ++f) {
            const int32_t id = fbase + (int32_t)f;
            const int32_t last = M.p0[id] + M.s[id] - 1;
            std::vector<int32_t> &bnd = bnd_lists[f];
            auto add = [&](int32_t q) {
                if (q > last && pos_stamp[q] != id) {
                    pos_stamp[q] = id;
                    bnd.push_back(q);
                }
            };
            for (int32_t a : nd.own[f]) {
                const int32_t I = node_g[a];
                for (int32_t q = rows[I]; q < rows[I + 1]; ++q) {
                    const int32_t b = node_local[cols[q]];
                    if (b < 0) continue;
                    const int32_t nd_dofs = node_l0[b + 1] - node_l0[b];
                    for (int32_t c = 0; c < nd_dofs; ++c) add(node_pos0[b] + c);
                }
            }
            for (int32_t c = M.child_off[id]; c < M.child_off[id + 1]; ++c) {
                const int32_t ch = M.child[c] - fbase;
                for (int32_t q : bnd_lists[ch]) add(q);
            }
            std::sort(bnd.begin(), bnd.end());
        }
        for (size_t f = 0; f < nd.own.size(); ++f) {
            const int32_t id = fbase + (int32_t)f;
            M.bnd_off[id + 1] = M.bnd_off[id] + (int32_t)bnd_lists[f].size();
            M.bnd_pos.insert(M.bnd_pos.end(), bnd_lists[f].begin(), bnd_lists[f].end());
            M.u.push_back((int32_t)bnd_lists[f].size());
        }
        for (int32_t a = 0; a < nn; ++a) node_local[node_g[a]] = -1;
    }
    M.npos = pos;
    // extend-add maps, storage offsets, levels
    M.ea_map.assign(M.bnd_pos.size(), -1);
    M.foff.assign(M.nfront + 1, 0);
    M.woff.assign(M.nfront + 1, 0);
    for (int32_t id = 0; id < M.nfront; ++id) {
        const int64_t f = (int64_t)M.s[id] + M.u[id];
        M.foff[id + 1] = M.foff[id] + f * f;
        M.woff[id + 1] = M.woff[id] + (int32_t)f;
        M.max_f = std::max<int32_t>(M.max_f, (int32_t)f);
        M.max_s = std::max(M.max_s, M.s[id]);
        M.fmas += 0.5 * (double)M.s[id] * (double)f * (double)f;
        M.levels = std::max(M.levels, M.height[id] + 1);
        const int32_t p = parent[id];
        if (p < 0) {
            if (M.u[id] != 0) fail(LSS_ERR_INTERNAL, "multifrontal: a root front has a boundary");
            continue;
        }
        const int32_t *pb = M.bnd_pos.data() + M.bnd_off[p];
        const int32_t pu = M.u[p];
        for (int32_t e = M.bnd_off[id]; e < M.bnd_off[id + 1]; ++e) {
            const int32_t q = M.bnd_pos[e];
            if (q >= M.p0[p] && q < M.p0[p] + M.s[p]) {
                M.ea_map[e] = q - M.p0[p];
            } else {
                const int32_t *it = std::lower_bound(pb, pb + pu, q);
                if (it == pb + pu || *it != q) fail(LSS_ERR_INTERNAL, "multifrontal: boundary not in the parent front");
                M.ea_map[e] = M.s[p] + (int32_t)(it - pb);
            }
        }
    }
    M.elems = M.foff[M.nfront];
    M.welems = M.woff[M.nfront];
    return M;
}

}  // namespace lss
