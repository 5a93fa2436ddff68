"""Queued skeleton runs (hpc_run_skeleton_async / hpc_wait): the same skeleton as a
synchronous run and as the oracle, several runs queued behind each other, results
read without an explicit wait, and the first run of a context (which sizes the
neighbour lists synchronously)."""
import numpy as np
import pytest

import heterogpc as hg
from helpers import edge_set, gen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [hg.PREC_FP64, hg.PREC_MIXED, hg.PREC_MIXED_TC])
def test_async_matches_sync_and_oracle(precision):
    X = gen(dict(p=120, n=1500, graph=hg.GRAPH_ER, degree=3.0, seed=41))
    p, n = X.shape[0], X.shape[1]
    Cm = orc.correlation(X)
    alpha, max_level = 0.01, 4
    ref = orc.run(Cm, n, alpha, max_level)
    sync = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=max_level, precision=precision)
    sync.add_correlation_matrix(Cm)
    sync_stats = sync.run()
    want = edge_set(sync.adjacency())
    assert want == edge_set(ref.adj)

    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=max_level, precision=precision)
    sk.add_correlation_matrix(Cm)
    sk.run_async()  # first run of the context: sized and run synchronously inside
    st = sk.wait()
    assert edge_set(sk.adjacency()) == want
    for _ in range(3):  # queued behind each other, collected once
        sk.run_async()
    st = sk.wait()
    assert [s["edges_after"] for s in st] == [s["edges_after"] for s in sync_stats]
    assert edge_set(sk.adjacency()) == want
    sk.run_async()  # results read without an explicit wait
    assert edge_set(sk.adjacency()) == want
    assert sk.edge_count() == len(want)
    recs = sk.sepset_records()
    assert len(recs) == sum(s["edges_before"] - s["edges_after"] for s in st if s["level"] >= 1)
    for i, j, lev, ids, pmax in recs:
        assert orc.verify_sepset(Cm, n, alpha, i, j, ids), (i, j, ids)
    sync.close()
    sk.close()


def test_async_until_exhausted_after_a_first_run():
    """max_level -1: the first run_async runs synchronously (it finds the extent of the
    levels), later ones are queued; results equal the oracle's."""
    X = gen(dict(p=30, n=400, graph=hg.GRAPH_ER, degree=2.0, seed=7))
    Cm = orc.correlation(X)
    want = orc.run(Cm, X.shape[1], 0.05, -1)
    sk = hg.SkeletonCalculator(X.shape[0], X.shape[1], alpha=0.05, max_level=-1, precision=hg.PREC_MIXED)
    sk.add_observations(X)
    for _ in range(3):
        sk.run_async()
    st = sk.wait()
    assert np.array_equal(sk.adjacency(), want.adj)
    # the device's list ends with the first level without tests, the oracle's before it
    assert [s["edges_after"] for s in st][:len(want.levels)] == [l["edges_after"] for l in want.levels]
    sk.close()
