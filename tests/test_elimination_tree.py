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
