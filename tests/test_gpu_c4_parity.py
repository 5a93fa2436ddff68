"""The full batched workload (512 instances, p ~ U[20, 800], n ~ U[200, 8000], ER degree
~ U[1, 5], alpha 0.01 / 0.05, FP32 data, levels until exhausted) in one context against
the committed oracle results (tests/golden/c4_golden.json, made on the CPU by
tests/golden/make_c4_golden.py): every instance's skeleton -- in tensor-core mixed
precision, eager and graph-replayed -- has the oracle's adjacency (hash of the upper
triangle), its edge count after every level and its number of separation-set records,
and every stored separation set re-tests as independent in FP64 (a sample of 64
instances, whose FP64 correlations the oracle computes here). The plain FP64 path
equals the oracle on 64 of the instances. The level logic checked is the reference's
(src/executor/testing/cpuRowTests.cpp:58-136, src/independence/skeleton.cpp:152-190)."""
import os

import numpy as np
import pytest

import bench
import heterogpc as hg
from helpers import sha
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

GOLD = bench.c4_golden()
needs_gold = pytest.mark.skipif(GOLD is None, reason="tests/golden/c4_golden.json not generated")


def _data():
    wl = bench.WORKLOADS["c4"]
    ps, ns, degs, alphas = bench.c4_instances(wl)
    Xs = [bench.c4_instance_data(wl, b) for b in range(len(ps))]
    return wl, ps, ns, alphas, Xs


@needs_gold
def test_c4_every_instance_equals_oracle():
    wl, ps, ns, alphas, Xs = _data()
    assert len(GOLD["instances"]) == len(ps)
    for b, g in enumerate(GOLD["instances"]):
        assert sha(Xs[b]) == g["data_sha256"], "generator output differs from the fixture (instance %d)" % b
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=wl["max_level"], precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack(Xs))
    for rep in range(2):  # the first run sizes the buffers, the second replays the captured graph
        bt.reset()
        bt.run()
        bits, off = bt.adjacency_bits()
        pre = bt.record_prefix()
        bad = []
        for b, g in enumerate(GOLD["instances"]):
            p = int(ps[b])
            adj = bench.bits_to_matrix(bits[off[b]:off[b + 1]], p)
            lv = [s["edges_after"] for s in bt.instance_levels(b)]
            n_rec = int(pre[b + 1] - pre[b])
            if (bench.c4_adj_sha(adj) != g["adj_sha256"] or lv[:len(g["edges_per_level"])] != g["edges_per_level"]
                    or n_rec != g["records"]):
                bad.append(b)
        assert not bad, "rep %d: instances differing from the oracle: %s" % (rep, bad[:20])
    # every stored separation set of a sample of instances re-tests as independent in FP64
    rng = np.random.default_rng(4)
    for b in sorted(rng.choice(len(ps), 64, replace=False)):
        Cm = orc.correlation(Xs[b].astype(np.float64))
        rs = bt.sepset_records(int(b))
        ok = orc.verify_sepsets(Cm, int(ns[b]), float(alphas[b]), [(i, j, lev, ids) for i, j, lev, ids, _ in rs])
        assert ok.all(), (b, [rs[t] for t in np.nonzero(~ok)[0][:5]])
        assert all(pm >= alphas[b] for *_, pm in rs)
    bt.close()


@needs_gold
def test_c4_plain_fp64_path_on_64_instances():
    wl, ps, ns, alphas, Xs = _data()
    rng = np.random.default_rng(40)
    for b in sorted(rng.choice(len(ps), 64, replace=False)):
        sk = hg.SkeletonCalculator(int(ps[b]), int(ns[b]), alpha=float(alphas[b]), max_level=wl["max_level"],
                                   precision=hg.PREC_FP64)
        sk.add_observations(Xs[b])
        st = sk.run()
        g = GOLD["instances"][b]
        assert bench.c4_adj_sha(sk.adjacency()) == g["adj_sha256"], b
        assert [s["edges_after"] for s in st][:len(g["edges_per_level"])] == g["edges_per_level"], b
        assert len(sk.sepset_records()) == g["records"], b
        sk.close()


@needs_gold
@pytest.mark.parametrize("set_from", [0, 2])
def test_c4_both_test_orders_equal_oracle(set_from):
    """The CI tests in the edge order at every level (set_from 0) and in the set order
    from level 2 on (one Cholesky factor per conditioning set shared by the neighbours
    outside it; level 2 has rows wider than the 64-bit masks): every instance equals the
    oracle, and every stored separation set of a sample re-tests as independent."""
    wl, ps, ns, alphas, Xs = _data()
    hg.set_order_from(set_from)
    try:
        bt = hg.SkeletonBatch(ps, ns, alphas, max_level=wl["max_level"], precision=hg.PREC_MIXED_TC)
        bt.add_observations(bt.pack(Xs))
        st = bt.run()
        if set_from == 2:
            assert max(s["max_degree"] for s in st if s["level"] == 2) > 64
        bits, off = bt.adjacency_bits()
        pre = bt.record_prefix()
        bad = []
        for b, g in enumerate(GOLD["instances"]):
            adj = bench.bits_to_matrix(bits[off[b]:off[b + 1]], int(ps[b]))
            lv = [s["edges_after"] for s in bt.instance_levels(b)]
            if (bench.c4_adj_sha(adj) != g["adj_sha256"] or lv[:len(g["edges_per_level"])] != g["edges_per_level"]
                    or int(pre[b + 1] - pre[b]) != g["records"]):
                bad.append(b)
        assert not bad, "instances differing from the oracle: %s" % bad[:20]
        rng = np.random.default_rng(5)
        for b in sorted(rng.choice(len(ps), 16, replace=False)):
            Cm = orc.correlation(Xs[b].astype(np.float64))
            rs = bt.sepset_records(int(b))
            ok = orc.verify_sepsets(Cm, int(ns[b]), float(alphas[b]), [(i, j, lev, ids) for i, j, lev, ids, _ in rs])
            assert ok.all(), (b, [rs[t] for t in np.nonzero(~ok)[0][:5]])
        bt.close()
    finally:
        hg.set_order_from(hg.SET_ORDER_DEFAULT)


@needs_gold
def test_c4_retest_queue_overflow_reruns_in_the_edge_order():
    """A set-order level that finds the FP64 re-test queue full flags it; the host repeats
    the run from level 0 in the edge order (whose tests re-test inline when the queue is
    full) and the skeleton is still the oracle's."""
    wl, ps, ns, alphas, Xs = _data()
    idx = list(range(0, len(ps), 16))
    bt = hg.SkeletonBatch(ps[idx], ns[idx], alphas[idx], max_level=wl["max_level"], precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack([Xs[b] for b in idx]))
    bt.set_retest_queue(4)
    assert bt.set_order_active()
    st = bt.run()
    assert sum(s["retests"] for s in st if s["level"] >= hg.SET_ORDER_DEFAULT) > 4
    assert not bt.set_order_active()
    bits, off = bt.adjacency_bits()
    pre = bt.record_prefix()
    for q, b in enumerate(idx):
        g = GOLD["instances"][b]
        adj = bench.bits_to_matrix(bits[off[q]:off[q + 1]], int(ps[b]))
        assert bench.c4_adj_sha(adj) == g["adj_sha256"], b
        assert int(pre[q + 1] - pre[q]) == g["records"], b
    bt.close()


@needs_gold
def test_c4_queued_runs_continue_past_the_previous_extent():
    """A run until exhausted queues the levels the previous run needed as one sequence;
    when the new data reach further, hpc_wait continues level by level. Here the first
    run sees exactly uncorrelated variables (centred orthonormal columns: level 0 removes
    every edge) of the deep instances' shapes, then the real observations are queued: the
    result is still the oracle's skeleton."""
    wl, ps, ns, alphas, Xs = _data()
    deep = sorted(range(len(ps)), key=lambda b: -len(GOLD["instances"][b]["edges_per_level"]))
    idx = [b for b in deep if ns[b] > ps[b] + 8][:8]
    bt = hg.SkeletonBatch(ps[idx], ns[idx], alphas[idx], max_level=-1, precision=hg.PREC_MIXED_TC)
    rng = np.random.default_rng(900)
    shallow = []
    for b in idx:
        n, p = int(ns[b]), int(ps[b])
        a = np.concatenate([np.ones((n, 1)), rng.standard_normal((n, p))], axis=1)
        q, _ = np.linalg.qr(a)
        shallow.append(np.ascontiguousarray((q[:, 1:] * np.sqrt(n)).T, dtype=np.float32))
    bt.add_observations(bt.pack(shallow))
    first = bt.run()
    assert first[0]["edges_after"] == 0
    bt.add_observations(bt.pack([Xs[b] for b in idx]))
    bt.run_async()
    st = bt.wait()
    assert len(st) > len(first)
    bits, off = bt.adjacency_bits()
    for q, b in enumerate(idx):
        adj = bench.bits_to_matrix(bits[off[q]:off[q + 1]], int(ps[b]))
        assert bench.c4_adj_sha(adj) == GOLD["instances"][b]["adj_sha256"], b
    # and queued again on the same data: one replay per run
    for _ in range(3):
        bt.add_observations(bt.pack([Xs[b] for b in idx]))
        bt.run_async()
    bt.wait()
    bits, off = bt.adjacency_bits()
    for q, b in enumerate(idx):
        adj = bench.bits_to_matrix(bits[off[q]:off[q + 1]], int(ps[b]))
        assert bench.c4_adj_sha(adj) == GOLD["instances"][b]["adj_sha256"], b
    bt.close()


def test_c4_fixture_consistent_with_workload():
    if GOLD is None:
        pytest.skip("no fixture")
    wl = bench.WORKLOADS["c4"]
    ps, ns, degs, alphas = bench.c4_instances(wl)
    for b, g in enumerate(GOLD["instances"]):
        assert (g["p"], g["n"]) == (int(ps[b]), int(ns[b]))
        assert abs(g["alpha"] - float(alphas[b])) < 1e-15
    assert os.path.basename(GOLD["generator"]) == "make_c4_golden.py"
