"""Continuous-batching server: requests arriving while others run are admitted as
batches; every result equals the oracle's and the same request served alone."""
import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def requests(k, seed):
    rng = np.random.default_rng(seed)
    out = []
    for r in range(k):
        p = int(np.exp(rng.uniform(np.log(20), np.log(300))))
        n = int(np.exp(rng.uniform(np.log(200), np.log(3000))))
        graph = hg.GRAPH_ER if r % 2 == 0 else hg.GRAPH_PA
        X = hg.sem_generate(p, n, graph, 3.0, 2, 0.1, 1.0, 500 + seed * 1000 + r, dtype=np.float32)
        out.append(X)
    return out


def test_served_results_equal_oracle_and_alone():
    reqs = requests(24, seed=1)
    alpha, ml = 0.01, 4
    # one batch in flight: requests arriving while it runs wait and are admitted
    # together as the next batch
    sv = hg.SkeletonServer(max_level=ml, max_batch=8, max_inflight=1)
    ids = []
    for X in reqs:
        ids.append(sv.submit(X, alpha, want_adjacency=True))
    sv.drain()
    done = {d["id"]: d for d in sv.poll()}
    assert sorted(done) == sorted(ids)
    assert max(d["batch_size"] for d in done.values()) > 1
    for rid, X in zip(ids, reqs):
        d = done[rid]
        assert d["status"] == 0
        Cm = orc.correlation(X.astype(np.float64))
        want = orc.run(Cm, X.shape[1], alpha, ml)
        assert np.array_equal(d["adjacency"], want.adj)
        assert d["edges"] == want.edges()
        assert d["latency_ms"] >= d["run_ms"] > 0
    # the same requests served alone (batch of one) give the same skeletons
    alone = hg.SkeletonServer(max_level=ml, max_batch=1, max_inflight=1)
    for rid, X in list(zip(ids, reqs))[:6]:
        aid = alone.submit(X, alpha, want_adjacency=True)
        alone.drain()
        (d,) = alone.poll()
        assert d["id"] == aid and d["batch_size"] == 1
        assert np.array_equal(d["adjacency"], done[rid]["adjacency"])
    alone.close()
    sv.close()


def test_budget_admits_one_at_a_time_when_tight():
    reqs = requests(6, seed=2)
    sv = hg.SkeletonServer(max_level=3, budget_bytes=1, max_batch=64, max_inflight=4)
    for X in reqs:
        sv.submit(X, 0.05)
    sv.drain()
    done = sv.poll()
    assert len(done) == 6 and all(d["status"] == 0 for d in done)
    assert all(d["batch_size"] == 1 for d in done)  # nothing fits beside another request
    sv.close()
