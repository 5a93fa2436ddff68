"""Batches: many independent skeleton problems of uneven p, n and alpha in one
context, every level kernel launched once for all of them. Each instance's skeleton
must equal the oracle's for that instance alone."""
import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def make_batch(count, seed, p_range=(20, 160), n_range=(200, 2000)):
    rng = np.random.default_rng(seed)
    ps = rng.integers(p_range[0], p_range[1] + 1, count)
    ns = rng.integers(n_range[0], n_range[1] + 1, count)
    alphas = np.where(np.arange(count) % 2 == 0, 0.01, 0.05)
    degs = rng.uniform(1, 5, count)
    Xs = [hg.sem_generate(int(p), int(n), hg.GRAPH_ER, float(d), 2, 0.1, 1.0, 1000 + seed * 100 + b,
                          dtype=np.float32)
          for b, (p, n, d) in enumerate(zip(ps, ns, degs))]
    return ps, ns, alphas, Xs


@pytest.mark.parametrize("precision", [hg.PREC_MIXED_TC, hg.PREC_MIXED, hg.PREC_FP64])
def test_batch_matches_oracle_per_instance(precision):
    ps, ns, alphas, Xs = make_batch(24, seed=1)
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=5, precision=precision)
    bt.add_observations(bt.pack(Xs))
    for rep in range(2):  # eager, then the graph replay
        bt.reset()
        bt.run()
        for b in range(bt.count):
            Cm = orc.correlation(Xs[b].astype(np.float64))
            want = orc.run(Cm, int(ns[b]), float(alphas[b]), 5)
            assert np.array_equal(bt.adjacency(b), want.adj), (rep, b)
            assert bt.edge_count(b) == want.edges()
            if rep == 1:
                recs = bt.sepset_records(b)
                assert len(recs) == len(want.records)
                for i, j, lev, ids, pmax in recs:
                    assert orc.verify_sepset(Cm, int(ns[b]), float(alphas[b]), i, j, ids)


def test_batch_result_same_alone_and_in_the_mix():
    ps, ns, alphas, Xs = make_batch(10, seed=2)
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=-1, precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack(Xs))
    bt.run()
    for b in (0, 3, 9):
        alone = hg.SkeletonBatch(ps[b:b + 1], ns[b:b + 1], alphas[b:b + 1], max_level=-1,
                                 precision=hg.PREC_MIXED_TC)
        alone.add_observations(alone.pack([Xs[b]]))
        alone.run()
        assert np.array_equal(alone.adjacency(0), bt.adjacency(b))
        assert alone.instance_levels(0)[-1]["edges_after"] == bt.instance_levels(b)[-1]["edges_after"]


def test_batch_correlation_input():
    ps, ns, alphas, Xs = make_batch(8, seed=3)
    mats = [orc.correlation(X.astype(np.float64)) for X in Xs]
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=4, precision=hg.PREC_MIXED)
    bt.add_correlation_matrices(mats)
    bt.run()
    for b in range(bt.count):
        want = orc.run(mats[b], int(ns[b]), float(alphas[b]), 4)
        assert np.array_equal(bt.adjacency(b), want.adj)


def test_whole_batch_result_copies():
    """Adjacency bitmasks and records of every instance in one copy each (plain, packed
    and per instance agree)."""
    ps, ns, alphas, Xs = make_batch(12, seed=4)
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=-1, precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack(Xs))
    bt.run()
    bits, off = bt.adjacency_bits()
    allrec = bt.all_sepset_records()
    packed = bt.records_packed()
    for b in range(bt.count):
        p = int(ps[b])
        W = (p + 31) // 32
        m = np.unpackbits(bits[off[b]:off[b + 1]].view(np.uint8), bitorder="little").reshape(p, W * 32)[:, :p]
        assert np.array_equal(m, bt.adjacency(b))
        one = bt.sepset_records(b)
        assert allrec[b] == one
        assert [(i, j, lev, ids) for i, j, lev, ids, _ in packed[b]] == [(i, j, lev, ids) for i, j, lev, ids, _
                                                                          in one]
        assert [pm for *_, pm in packed[b]] == [pm for *_, pm in one]
        assert [lev for _, _, lev, _, _ in packed[b]] == sorted(lev for _, _, lev, _, _ in packed[b])


def test_batch_new_data_on_the_same_context_matches_oracle():
    """The neighbour lists a context keeps between levels (rows are extracted again only
    where an edge was removed) belong to one skeleton: new observations of the same
    shapes, and then the first ones again, must each give the oracle's skeletons, run
    whole and level by level."""
    ps, ns, alphas, Xs = make_batch(12, seed=5)
    rng = np.random.default_rng(55)
    degs = rng.uniform(1, 5, len(ps))
    Ys = [hg.sem_generate(int(p), int(n), hg.GRAPH_ER, float(d), 2, 0.1, 1.0, 9000 + b, dtype=np.float32)
          for b, (p, n, d) in enumerate(zip(ps, ns, degs))]
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=8, precision=hg.PREC_MIXED_TC)
    for data in (Xs, Ys, Xs):
        bt.add_observations(bt.pack(data))
        wants = [orc.run(orc.correlation(data[b].astype(np.float64)), int(ns[b]), float(alphas[b]), 8)
                 for b in range(bt.count)]
        bt.run()
        for b in range(bt.count):
            assert np.array_equal(bt.adjacency(b), wants[b].adj), b
        bt.reset()
        for level in range(9):
            bt.calc_level(level)
        for b in range(bt.count):
            assert np.array_equal(bt.adjacency(b), wants[b].adj), ("level by level", b)


def test_batch_level_phase_times():
    """Kernel-by-kernel runs report the level kernels' rebuild and scan phases (device
    timer), within the kernel's own time."""
    ps, ns, alphas, Xs = make_batch(16, seed=7)
    bt = hg.SkeletonBatch(ps, ns, alphas, max_level=4, precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack(Xs))
    bt.set_graphs(False)
    st = bt.run()
    t = bt.timings()
    ran = [s["level"] for s in st if s["level"] >= 1]
    assert ran
    for level in ran:
        assert t["rebuild_ms"][level] > 0.0, level
        assert t["scan_ms"][level] >= 0.0, level
        assert t["rebuild_ms"][level] + t["scan_ms"][level] <= t["test_ms"][level] + 5e-3, level
