"""Levels above 16 (the runtime-level kernel) against the oracle, in every precision.

The data follow H -> C_1..C_17 -> Z: the edge H - Z is separated only by all seventeen
C's together, so the skeleton run until exhausted removes it at level 17 exactly, after
levels 2-16 have tested every smaller subset of H's and Z's neighbours (875,160 tests at
level 8). Edge sets, per-level edge counts and potential tests must equal the oracle's,
and the level-17 separation set must be the seventeen C's."""
import numpy as np
import pytest

import heterogpc as hg
from helpers import edge_set
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

K, N, ALPHA = 17, 20000, 0.01


def fan_data(k, n, a, b, seed):
    rng = np.random.default_rng(seed)
    H = rng.standard_normal(n)
    Cs = [a * H + rng.standard_normal(n) for _ in range(k)]
    Z = b * sum(Cs) + rng.standard_normal(n)
    return np.ascontiguousarray(np.vstack([H] + Cs + [Z]))  # p x n, each variable's samples contiguous


@pytest.fixture(scope="module")
def fan():
    X = fan_data(K, N, 0.6, 0.35, 7)
    Cm = orc.correlation(X)
    ref = orc.run(Cm, N, ALPHA, -1)
    assert len(ref.levels) == K + 1 and ref.levels[-1]["edges_after"] == ref.levels[-2]["edges_after"] - 1
    return X, Cm, ref


@pytest.mark.parametrize("precision", [hg.PREC_FP64, hg.PREC_MIXED, hg.PREC_MIXED_TC])
def test_level_17_removal_matches_oracle(fan, precision):
    X, Cm, ref = fan
    p = K + 2
    sk = hg.SkeletonCalculator(p, N, alpha=ALPHA, max_level=-1, precision=precision)
    if precision == hg.PREC_MIXED_TC:
        sk.add_observations(X)
    else:
        sk.add_correlation_matrix(Cm)
    st = sk.run()
    assert edge_set(sk.adjacency()) == edge_set(ref.adj)
    ran = [s for s in st if s["level"] == 0 or s["potential_tests"] > 0]
    assert [s["edges_after"] for s in ran] == [lv["edges_after"] for lv in ref.levels]
    assert [s["potential_tests"] for s in ran[1:]] == [lv["potential_tests"] for lv in ref.levels[1:]]
    recs = {(i, j): (lev, ids) for i, j, lev, ids, pmax in sk.sepset_records()}
    assert recs[(0, K + 1)] == (K, tuple(range(1, K + 1)))
    for (i, j), (lev, ids) in recs.items():
        assert orc.verify_sepset(Cm, N, ALPHA, i, j, ids), (i, j, ids)
    sk.close()
