"""Split-BF16 tcgen05 Gram (HPC_PREC_MIXED_TC) against the FP64 oracle correlation."""
import numpy as np
import pytest

import heterogpc as hg
from helpers import gen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

def tc_tol(n):
    """|error| bound of the split-BF16 Gram (hi.hi + hi.lo + lo.hi + lo.lo, FP32
    accumulation), the same model the library's FP32 decision bands use."""
    return 4.0 * (1.6e-5 / np.sqrt(n) + 1e-7)


@pytest.mark.parametrize("p,n,dtype", [(130, 70, np.float64), (300, 1000, np.float64), (777, 2049, np.float32),
                                       (2000, 5000, np.float32)])
def test_tensorcore_gram_accuracy(p, n, dtype):
    X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=p + n, dtype=dtype)
    want = orc.correlation(X.astype(np.float64))
    sk = hg.SkeletonCalculator(p, n, precision=hg.PREC_MIXED_TC)
    sk.add_observations(X)
    C32 = sk.correlation_f32()
    assert np.array_equal(C32, C32.T)  # written from the upper triangle only
    err = np.abs(C32.astype(np.float64) - want)
    off = err[~np.eye(p, dtype=bool)]
    print("p=%d n=%d max |err| off-diagonal %.3g, diagonal %.3g" % (p, n, off.max(), np.diag(err).max()))
    assert off.max() < tc_tol(n), off.max()
    assert np.diag(err).max() < tc_tol(n)


def test_tensorcore_skeleton_matches_oracle():
    X = gen(dict(p=400, n=2000, graph=hg.GRAPH_PA, pa_parents=2, w_lo=0.2, seed=91))
    Cm = orc.correlation(X)
    want = orc.run(Cm, 2000, 0.05, 6)
    sk = hg.SkeletonCalculator(400, 2000, alpha=0.05, max_level=6, precision=hg.PREC_MIXED_TC)
    sk.add_observations(X)
    sk.run()
    assert np.array_equal(sk.adjacency(), want.adj)


@pytest.mark.parametrize("graph,p,n,alpha,ml,seed", [
    (hg.GRAPH_ER, 2000, 5000, 0.01, 6, 2),    # the p=2000 workload of the benchmark
    (hg.GRAPH_PA, 1500, 1200, 0.05, 4, 93),
    (hg.GRAPH_ER, 600, 300, 0.05, -1, 94),
])
def test_tensorcore_mode_without_fp64_matrix(graph, p, n, alpha, ml, seed):
    """Tensor-core mode keeps no FP64 matrix: FP64 re-tests (level 0 band and every
    undecided test) take their entries from dot products of the standardised data,
    and the skeleton still equals the oracle's."""
    X = hg.sem_generate(p, n, graph, 4.0, 2, 0.2 if graph == hg.GRAPH_PA else 0.1, 1.0, seed, dtype=np.float32)
    Cm = orc.correlation(X.astype(np.float64))
    want = orc.run(Cm, n, alpha, ml)
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=ml, precision=hg.PREC_MIXED_TC)
    sk.add_observations(X)
    for _ in range(2):  # eager run, then the graph replay
        sk.reset()
        st = sk.run()
        assert np.array_equal(sk.adjacency(), want.adj)
        ran = [s_ for s_ in st if s_["level"] == 0 or s_["potential_tests"] > 0]  # the oracle omits the empty last level
        assert [s_["edges_after"] for s_ in ran] == [l["edges_after"] for l in want.levels]
    recs = sk.sepset_records()
    assert len(recs) == len(want.records)
    for i, j, lev, ids, pmax in recs[:2000]:
        assert orc.verify_sepset(Cm, n, alpha, i, j, ids)
