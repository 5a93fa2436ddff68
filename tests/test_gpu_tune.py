"""Tile policies and the autotuner on the GPU: the CI tests' tiling (subset chunk per
lane, tiles per lane, level 1's lane mapping) changes only the schedule, so every
policy -- forced, or picked by hpc_autotune -- gives the oracle's skeleton, and every
separation set still re-tests as independent in FP64. The hub-heavy case (preferential
attachment, p = 500, level 2 starting with ~60 neighbours per row) runs the bisection
unranking and skips the tiles of removed edges."""
import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

POLICIES = [
    None,                                                                        # table / defaults
    {"tile_cap": 1, "tiles_per_lane": 1, "edge_lanes": 32, "l1_prefetch": 0},      # one test per lane per tile
    {"tile_cap": 1024, "tiles_per_lane": 8, "edge_lanes": 1, "l1_prefetch": 0},    # long chunks, chunked level 1
    {"tile_cap": 16, "tiles_per_lane": 64, "edge_lanes": 1, "l1_prefetch": 0},
    {"tile_cap": 65536, "tiles_per_lane": 1, "edge_lanes": 32, "l1_prefetch": 0},  # a few huge tiles
    {"tile_cap": 256, "tiles_per_lane": 4, "edge_lanes": 32, "l1_prefetch": 1},    # level 1 loads a step ahead
    {"tile_cap": 2, "tiles_per_lane": 2, "edge_lanes": 32, "l1_prefetch": 1},
]


@pytest.fixture(scope="module")
def hub_case():
    p, n, alpha, ml = 500, 2000, 0.05, 3
    X = hg.sem_generate(p, n, hg.GRAPH_PA, 4.0, 2, 0.2, 1.0, seed=11)
    Cm = orc.correlation(X)
    want = orc.run(Cm, n, alpha, ml)
    return p, n, alpha, ml, X, Cm, want


@pytest.mark.parametrize("precision", [hg.PREC_FP64, hg.PREC_MIXED, hg.PREC_MIXED_TC])
def test_forced_policies_give_the_oracle_skeleton(hub_case, precision):
    p, n, alpha, ml, X, Cm, want = hub_case
    hg.tune_clear()
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=ml, precision=precision)
    if precision == hg.PREC_MIXED_TC:
        sk.add_observations(X.astype(np.float32))
    else:
        sk.add_correlation_matrix(Cm)
    for pol in POLICIES:
        sk.set_tune(pol)
        for _ in range(2):  # eager run, then the graph replay
            sk.reset()
            st = sk.run()
            assert np.array_equal(sk.adjacency(), want.adj), pol
            for s, lv in zip(st, want.levels):  # level by level
                assert s["edges_after"] == lv["edges_after"], (pol, s["level"])
        for i, j, lev, ids, pmax in sk.sepset_records():
            assert orc.verify_sepset(Cm, n, alpha, i, j, ids), (pol, i, j, ids)
    sk.close()


def test_autotune_stores_per_level_choices(hub_case, tmp_path):
    p, n, alpha, ml, X, Cm, want = hub_case
    hg.tune_clear()
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=ml, precision=hg.PREC_MIXED)
    sk.add_correlation_matrix(Cm)
    st0 = sk.run()
    cands = [{"tile_cap": 16, "tiles_per_lane": 4, "edge_lanes": 32, "l1_prefetch": 0},
             {"tile_cap": 256, "tiles_per_lane": 2, "edge_lanes": 1, "l1_prefetch": 0},
             {"tile_cap": 64, "tiles_per_lane": 8, "edge_lanes": 32, "l1_prefetch": 1}]
    chosen, entries = sk.autotune(cands, reps=2)
    assert entries == len([s for s in st0 if s["level"] >= 1 and s["potential_tests"] > 0]) > 0
    for s in st0:
        if s["level"] >= 1 and s["potential_tests"] > 0:
            pol, found = hg.tune_lookup(p, s["level"], s["max_degree"])
            assert found and pol == chosen[s["level"]] and pol in cands
    # the tuned table steers the next runs (eager, then captured) without changing results
    for _ in range(2):
        sk.reset()
        sk.run()
        assert np.array_equal(sk.adjacency(), want.adj)
    path = str(tmp_path / "policy.txt")
    hg.tune_save(path)
    hg.tune_clear()
    hg.tune_load(path)
    for s in st0:
        if s["level"] >= 1 and s["potential_tests"] > 0:
            assert hg.tune_lookup(p, s["level"], s["max_degree"]) == (chosen[s["level"]], True)
    sk.close()
    hg.tune_clear()


def test_autotune_on_a_batch():
    rng = np.random.default_rng(8)
    k = 24
    ps = rng.integers(20, 300, k)
    ns = rng.integers(200, 3000, k)
    alphas = np.array([0.01, 0.05] * (k // 2))
    Xs = [hg.sem_generate(int(ps[b]), int(ns[b]), hg.GRAPH_ER, float(rng.uniform(1, 5)), 2, 0.1, 1.0, 400 + b,
                          dtype=np.float32) for b in range(k)]
    hg.tune_clear()
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=-1, precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack(Xs))
    bt.run()
    before = [bt.adjacency(b) for b in range(k)]
    chosen, entries = bt.autotune(None, reps=1)  # the built-in candidate grid
    assert entries > 0 and 1 in chosen
    bt.run()
    for b in range(k):
        assert np.array_equal(bt.adjacency(b), before[b]), b
        want = orc.run(orc.correlation(Xs[b].astype(np.float64)), int(ns[b]), float(alphas[b]), -1)
        assert np.array_equal(before[b], want.adj), b
    bt.close()
    hg.tune_clear()
