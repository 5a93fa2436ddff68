"""Dense problems whose edges survive to high levels: the level kernels of levels 9-16
(their own instantiations) against the oracle, level by level, in every precision,
with every stored separation set re-verified in FP64.

The correlation matrices are an equicorrelation matrix plus a bounded symmetric
perturbation (positive definite): partial correlations given up to ten other variables
stay significant for most pairs, so the skeleton runs to level 10 or 11 with removals
at most levels."""
import numpy as np
import pytest

import heterogpc as hg
from helpers import edge_set
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

CASES = [dict(p=18, rho=0.35, eps=0.08, seed=1, n=4000, alpha=0.01),
         dict(p=20, rho=0.30, eps=0.12, seed=3, n=3000, alpha=0.05)]


def dense_matrix(p, rho, eps, seed):
    rng = np.random.default_rng(seed)
    E = rng.uniform(-eps, eps, (p, p))
    R = np.full((p, p), rho) + (E + E.T) / 2
    np.fill_diagonal(R, 1.0)
    assert np.linalg.eigvalsh(R).min() > 0.2
    return R


@pytest.mark.parametrize("case", CASES, ids=lambda c: "p%d_seed%d" % (c["p"], c["seed"]))
@pytest.mark.parametrize("precision", [hg.PREC_FP64, hg.PREC_MIXED, hg.PREC_MIXED_TC])
def test_high_levels_match_oracle(case, precision):
    Cm = dense_matrix(case["p"], case["rho"], case["eps"], case["seed"])
    p, n, alpha = case["p"], case["n"], case["alpha"]
    ref = orc.run(Cm, n, alpha, -1)
    assert len(ref.levels) >= 11, "the case does not reach level 10"
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=-1, precision=precision)
    sk.add_correlation_matrix(Cm)
    st = sk.run()
    assert edge_set(sk.adjacency()) == edge_set(ref.adj)
    ran = [s for s in st if s["level"] == 0 or s["potential_tests"] > 0]  # the oracle omits the empty last level
    assert [s["edges_after"] for s in ran] == [lv["edges_after"] for lv in ref.levels]
    assert [s["potential_tests"] for s in ran[1:]] == [lv["potential_tests"] for lv in ref.levels[1:]]
    assert len(ran) >= 11
    for i, j, lev, ids, pmax in sk.sepset_records():
        assert orc.verify_sepset(Cm, n, alpha, i, j, ids), (i, j, ids)
    sk.close()
