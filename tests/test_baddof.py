"""MASSolver's bad-DOF selections (elbow, k-means, GMM with an expansion
window): the library's host code (lss_op_select_bad_dofs) against the C
oracle's restatement of the reference (identical positions in the same
order), and the selections' expected behaviour on constructed scores."""
import numpy as np
import pytest

CASES = [
    # (strategy, p1, p2, i1, i2): the spec defaults and variants
    ("elbow", 0.0, 0.0, 0, 0),
    ("kmean", 0.2, 10.0, 32, 128),
    ("kmean", 0.02, 10.0, 32, 0),
    ("kmean", 0.5, 3.0, 1, 4),
    ("gmm", 10.0, 1e-3, 20, 16),
    ("gmm", 10.0, 1e-3, 5, 0),
    ("gmm", 2.0, 1e-6, 50, 3),
]


def _scores(seed, n, frac_hi, jump):
    rng = np.random.default_rng(seed)
    v = np.exp(rng.standard_normal(n))
    hi = rng.random(n) < frac_hi
    v[hi] *= jump
    return v


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_library_matches_oracle(case, seed, built):
    import lss
    from oracle import oracle as O
    strategy, p1, p2, i1, i2 = case
    for n, frac, jump in [(5000, 0.02, 1e4), (20000, 0.1, 1e2), (3000, 0.0, 1.0), (777, 0.3, 1e6)]:
        v = _scores(seed, n, frac, jump)
        if seed == 2:
            v = np.round(v, 1) + 0.1  # ties
        a = lss.select_bad_dofs(strategy, v, p1, p2, i1, i2)
        b = O.c_mas_select(strategy, v, p1, p2, i1, i2)
        np.testing.assert_array_equal(a, b, err_msg=f"{strategy} n={n} frac={frac}")


def test_edge_sizes(built):
    import lss
    from oracle import oracle as O
    for v in [np.zeros(0), np.ones(1), np.array([1.0, 1e6])]:
        for strategy, p1, p2, i1, i2 in CASES:
            np.testing.assert_array_equal(lss.select_bad_dofs(strategy, v, p1, p2, i1, i2),
                                          O.c_mas_select(strategy, v, p1, p2, i1, i2))


def test_selections_find_the_stiff_cluster(built):
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    n = 4000
    v = np.exp(0.1 * rng.standard_normal(n))
    stiff = np.sort(rng.choice(n, 40, replace=False))
    v[stiff] *= 1e6
    # elbow: the positions from the elbow of the ascending log curve on
    assert set(stiff) <= set(O.c_mas_select("elbow", v))
    # k-means on the top 2%: exactly the stiff positions; with a window of 2
    # every stiff position's neighbourhood
    assert np.array_equal(np.sort(O.c_mas_select("kmean", v, 0.02, 10.0, 32, 0)), stiff)
    widened = set(O.c_mas_select("kmean", v, 0.02, 10.0, 32, 2))
    assert widened == {j for s in stiff for j in range(max(0, s - 2), min(n, s + 3))}
    # GMM on the same scores: the stiff positions
    assert np.array_equal(np.sort(O.c_mas_select("gmm", v, 10.0, 1e-3, 20, 0)), stiff)
    # no jump: nothing
    assert len(O.c_mas_select("kmean", np.exp(0.1 * rng.standard_normal(n)), 0.2, 10.0, 32, 0)) == 0
