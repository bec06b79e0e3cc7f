"""The multifrontal stiff factor's elimination tree (host only, through
lss_stiff_elimination_tree): nested dissection of a stiff subdomain's node
graph with the separator level chosen among those that leave at least 30% of
the nodes on either side.  Its height sets the number of level-by-level
launches of the factorization and of every solve, so it must stay
logarithmic: a stiff ball of n DOFs gives a tree of height close to
log2(n / 48) (the leaf size), not the near-linear chains of a separator choice
that ignores balance.  Also: deterministic, and every variable in one front."""
import numpy as np
import pytest

import lss
from lss import gen


def _ball(nodes, radius):
    m = nodes
    E = np.ones(6 * (m - 1) ** 3)
    A = gen.elasticity_cube(m, m, m, E).tocsc()
    A.sum_duplicates()
    c = (m - 1) / 2.0
    idx = np.arange(m ** 3)
    x, y, z = idx // (m * m), (idx // m) % m, idx % m
    inside = np.sqrt((x - c) ** 2 + (y - c) ** 2 + (z - c) ** 2) <= radius * (m - 1)
    nodes_in = idx[inside]
    dofs = (3 * nodes_in[:, None] + np.arange(3)[None, :]).ravel()
    return A, np.sort(dofs)


@pytest.mark.parametrize("nodes,radius", [(14, 0.45), (18, 0.45), (22, 0.4)])
def test_tree_is_shallow(nodes, radius, built):
    A, dofs = _ball(nodes, radius)
    t = lss.stiff_elimination_tree(A, 3, dofs)
    n = len(dofs)
    assert t["fronts"] > 1
    # a balanced nested dissection: height ~ log2(n / leaf) + a small constant
    bound = int(np.ceil(np.log2(n / 48.0))) + 5
    assert t["levels"] <= bound, (n, t)
    assert t["max_front"] <= n
    assert t["fmas"] > 0


def test_tree_is_deterministic(built):
    A, dofs = _ball(16, 0.45)
    assert lss.stiff_elimination_tree(A, 3, dofs) == lss.stiff_elimination_tree(A, 3, dofs)


def test_tree_rejects_bad_input(built):
    A, dofs = _ball(10, 0.45)
    with pytest.raises(lss.LssError):
        lss.stiff_elimination_tree(A, 3, dofs[::-1].copy() * 0 - 1)


def _multifrontal_solve(App, plan, b):
    """Dense numpy multifrontal factor + solve following the plan: every front
    sums its original entries (own rows x own and boundary columns) and its
    children's update matrices, eliminates its own variables, and passes the
    Schur complement on; then forward and backward sweeps."""
    p0, s_, u_ = plan["p0"], plan["s"], plan["u"]
    bo, bp, co, ch = plan["bnd_off"], plan["bnd_pos"], plan["child_off"], plan["child"]
    nf = len(p0)
    idx, upd, fac = [], [None] * nf, [None] * nf
    for f in range(nf):
        own = np.arange(p0[f], p0[f] + s_[f])
        bnd = bp[bo[f]:bo[f + 1]]
        assert len(bnd) == u_[f] and np.all(np.diff(bnd) > 0) and (len(bnd) == 0 or bnd[0] > own[-1])
        ix = np.concatenate([own, bnd])
        idx.append(ix)
        F = np.zeros((len(ix), len(ix)))
        F[:len(own), :] = App[np.ix_(own, ix)]
        F[:, :len(own)] = App[np.ix_(ix, own)]
        where = {q: k for k, q in enumerate(ix)}
        for c in ch[co[f]:co[f + 1]]:
            cb = idx[c][s_[c]:]
            m = np.array([where[q] for q in cb], dtype=np.int64)  # the child's boundary lies in this front
            F[np.ix_(m, m)] += upd[c]
        s = len(own)
        Foo, Fob = F[:s, :s], F[:s, s:]
        X = np.linalg.solve(Foo, Fob)
        upd[f] = F[s:, s:] - Fob.T @ X
        fac[f] = (Foo, Fob)
    # forward: w of each front = its right-hand side + the children's contributions
    w = [None] * nf
    for f in range(nf):
        ix = idx[f]
        wf = np.zeros(len(ix))
        wf[:s_[f]] = b[ix[:s_[f]]]
        where = {q: k for k, q in enumerate(ix)}
        for c in ch[co[f]:co[f + 1]]:
            for k, q in enumerate(idx[c][s_[c]:]):
                wf[where[q]] += w[c][s_[c] + k]
        Foo, Fob = fac[f]
        wf[s_[f]:] -= Fob.T @ np.linalg.solve(Foo, wf[:s_[f]])
        w[f] = wf
    x = np.zeros(len(b))
    for f in reversed(range(nf)):
        ix = idx[f]
        Foo, Fob = fac[f]
        x[ix[:s_[f]]] = np.linalg.solve(Foo, w[f][:s_[f]] - Fob @ x[ix[s_[f]:]])
    return x


@pytest.mark.parametrize("nodes,radius", [(10, 0.45), (13, 0.45)])
def test_plan_factorizes_the_block(nodes, radius, built):
    """The plan is a valid multifrontal factorization of the subdomain's block:
    positions are a permutation of the DOFs, every front's boundary lies in
    its parent, and the numpy multifrontal solve along it reproduces a dense
    solve of the block to rounding."""
    A, dofs = _ball(nodes, radius)
    plan = lss.stiff_elimination_plan(A, 3, dofs)
    n = len(dofs)
    assert sorted(plan["pos2j"].tolist()) == list(range(n))
    assert plan["bnd_off"][-1] == len(plan["bnd_pos"])
    Ar = A.tocsr()
    Ass = Ar[dofs][:, dofs].toarray()
    App = Ass[np.ix_(plan["pos2j"], plan["pos2j"])]
    b = np.random.default_rng(0).standard_normal(n)
    x = _multifrontal_solve(App, plan, b)
    xd = np.linalg.solve(App, b)
    assert np.linalg.norm(x - xd) <= 1e-9 * np.linalg.norm(xd)
