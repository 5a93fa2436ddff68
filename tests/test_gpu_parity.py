"""GPU skeletons through the C ABI against the reference's golden fixtures and the
oracle. Accept/reject decisions are compared exactly (edge sets bit-identical);
every stored separation set is re-verified as independent by the FP64 oracle."""
import numpy as np
import pytest

import heterogpc as hg
from helpers import case_inputs, edge_set, gen, golden_edges
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

PRECISIONS = [hg.PREC_FP64, hg.PREC_MIXED]


def run_gpu(Cm, n, alpha, max_level, precision, X=None):
    p = Cm.shape[0] if Cm is not None else X.shape[0]
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=max_level, precision=precision)
    if X is not None:
        sk.add_observations(X)
    else:
        sk.add_correlation_matrix(Cm)
    sk.run()
    return sk


def check_sepsets(sk, Cm, n, alpha):
    recs = sk.sepset_records()
    seen = set()
    for i, j, lev, ids, pmax in recs:
        assert i < j and (i, j) not in seen
        seen.add((i, j))
        assert len(ids) == lev and list(ids) == sorted(ids) and i not in ids and j not in ids
        assert orc.verify_sepset(Cm, n, alpha, i, j, ids), (i, j, ids)
        assert pmax >= alpha
    return recs


@pytest.mark.parametrize("precision", PRECISIONS)
def test_golden_correlation_input(golden, precision):
    for case in golden["cases"]:
        _, Cm = case_inputs(case)
        sk = run_gpu(Cm, case["n_obs"], case["alpha"], case["max_level"], precision)
        assert edge_set(sk.adjacency()) == golden_edges(case), case["name"]
        assert sk.edge_count() == case["n_edges"]
        check_sepsets(sk, Cm, case["n_obs"], case["alpha"])
        # level-0 markers in the reference's dense layout (cpuUtil.cpp:3-21)
        mc = max(case["max_level"], 1)
        dense = sk.sepsets(mc)
        ref_l0 = {(i, j) for i, j, lev, ids in case["ref_sepsets"] if lev == 0}
        got_l0 = set(zip(*np.nonzero(dense[:, :, 0] == -2)))
        assert {(int(a), int(b)) for a, b in got_l0} == ref_l0, case["name"]
        sk.close()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_golden_observation_input(golden, precision):
    for case in golden["cases"]:
        if case["source"] != "sem":
            continue
        X, Cm = case_inputs(case)
        sk = run_gpu(None, case["n_obs"], case["alpha"], case["max_level"], precision, X=X)
        err = np.abs(sk.correlation() - Cm).max()
        assert err < 1e-12, (case["name"], err)
        assert edge_set(sk.adjacency()) == golden_edges(case), case["name"]
        sk.close()


def test_levels_match_oracle_level_by_level():
    X = gen(dict(p=120, n=800, graph=hg.GRAPH_ER, degree=4.0, seed=44))
    Cm = orc.correlation(X)
    want = orc.run(Cm, 800, 0.05, 6)
    sk = hg.SkeletonCalculator(120, 800, alpha=0.05, max_level=6)
    sk.add_correlation_matrix(Cm)
    for lv in want.levels:
        st = sk.calc_level(lv["level"])
        assert st["edges_after"] == lv["edges_after"], lv
        if lv["level"] >= 1:
            assert st["potential_tests"] == lv["potential_tests"]
    assert np.array_equal(sk.adjacency(), want.adj)


@pytest.mark.parametrize("seed,graph,p,n,alpha", [
    (101, hg.GRAPH_ER, 300, 1500, 0.01),
    (102, hg.GRAPH_PA, 400, 1000, 0.05),
    (103, hg.GRAPH_ER, 250, 300, 0.05),
    (104, hg.GRAPH_PA, 200, 5000, 0.01),
])
@pytest.mark.parametrize("precision", PRECISIONS)
def test_seeded_against_oracle(seed, graph, p, n, alpha, precision):
    X = gen(dict(p=p, n=n, graph=graph, degree=3.0, w_lo=0.2 if graph == hg.GRAPH_PA else 0.1, seed=seed))
    Cm = orc.correlation(X)
    want = orc.run(Cm, n, alpha, -1)
    sk = run_gpu(Cm, n, alpha, -1, precision)
    assert np.array_equal(sk.adjacency(), want.adj)
    check_sepsets(sk, Cm, n, alpha)
    for got, exp in zip(sk.level_stats, want.levels):
        assert got["edges_after"] == exp["edges_after"]


def test_config2_full_size_mixed():
    """p=2000, n=5000, FP32 data, ER degree 4, alpha 0.01, max level 6."""
    X = hg.sem_generate(2000, 5000, hg.GRAPH_ER, 4.0, 2, 0.1, 1.0, 2, dtype=np.float32)
    Cm = orc.correlation(X.astype(np.float64))
    want = orc.run(Cm, 5000, 0.01, 6)
    sk = hg.SkeletonCalculator(2000, 5000, alpha=0.01, max_level=6, precision=hg.PREC_MIXED)
    sk.add_observations(X)
    sk.run()
    assert np.abs(sk.correlation() - Cm).max() < 1e-12
    assert np.array_equal(sk.adjacency(), want.adj)
    recs = check_sepsets(sk, Cm, 5000, 0.01)
    assert len(recs) == len(want.records)


def test_reset_and_rerun_identical():
    X = gen(dict(p=80, n=600, graph=hg.GRAPH_ER, degree=3.0, seed=55))
    Cm = orc.correlation(X)
    sk = run_gpu(Cm, 600, 0.05, -1, hg.PREC_MIXED)
    a1 = sk.adjacency()
    sk.reset()
    sk.run()
    assert np.array_equal(a1, sk.adjacency())


def test_call_order_errors():
    sk = hg.SkeletonCalculator(10, 100)
    with pytest.raises(hg.HpcError) as e:
        sk.calc_level(0)
    assert e.value.status == 6  # HPC_ERR_STATE: no correlation yet
    sk.add_correlation_matrix(np.eye(10))
    with pytest.raises(hg.HpcError) as e:
        sk.calc_level(1)
    assert e.value.status == 6  # levels run in order
    sk.calc_level(0)
    assert sk.edge_count() == 0  # identity: every pair independent
    # levels above the context's max_level are refused (its records hold that many ids)
    X = gen(dict(p=30, n=500, graph=hg.GRAPH_ER, degree=3.0, seed=45))
    sk = hg.SkeletonCalculator(30, 500, alpha=0.05, max_level=1)
    sk.add_correlation_matrix(orc.correlation(X))
    sk.calc_level(0)
    sk.calc_level(1)
    with pytest.raises(hg.HpcError) as e:
        sk.calc_level(2)
    assert e.value.status == 1  # HPC_ERR_INVALID_ARG


@pytest.mark.parametrize("alpha,max_level", [(1.0, 3), (0.999, 2), (1e-300, 0), (1e-12, 3)])
def test_extreme_alpha(alpha, max_level):
    """alpha = 1 removes only pairs with p == 1 exactly (r == 0 or NaN, cpuInd.cpp:10-13);
    tiny alpha removes almost nothing."""
    X = gen(dict(p=30, n=200, graph=hg.GRAPH_ER, degree=3.0, seed=66))
    Cm = orc.correlation(X)
    Cm[3, 1] = Cm[1, 3] = 0.0  # p == 1 exactly at level 0
    want = orc.run(Cm, 200, alpha, max_level)
    for precision in PRECISIONS:
        sk = run_gpu(Cm, 200, alpha, max_level, precision)
        assert np.array_equal(sk.adjacency(), want.adj)


def test_graph_replays_and_changing_data():
    """Repeated runs replay the captured level sequence; loading denser data afterwards
    outgrows the neighbour-list buffer, which is detected on the device, resized and rerun."""
    p, n = 150, 1000
    Xa = gen(dict(p=p, n=n, graph=hg.GRAPH_ER, degree=1.5, seed=71))
    Xb = gen(dict(p=p, n=n, graph=hg.GRAPH_ER, degree=8.0, seed=72))
    sk = hg.SkeletonCalculator(p, n, alpha=0.05, max_level=5, precision=hg.PREC_MIXED)
    for X in (Xa, Xa, Xa, Xb, Xb, Xa):
        Cm = orc.correlation(X)
        want = orc.run(Cm, n, 0.05, 5)
        sk.add_correlation_matrix(Cm)
        sk.run()
        assert np.array_equal(sk.adjacency(), want.adj)
        assert len(sk.sepset_records()) == len(want.records)
        for got, exp in zip(sk.level_stats, want.levels):
            assert got["edges_after"] == exp["edges_after"]
