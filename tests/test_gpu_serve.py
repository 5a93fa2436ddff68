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
    # at most 8 requests on the device, admitted while the others run
    sv = hg.SkeletonServer(max_level=ml, max_batch=8, max_inflight=2)
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


def test_request_joins_a_running_batch_at_the_next_level():
    """A long request runs level after level; requests submitted while it runs are
    admitted between its steps (joined > 0), share its level launches, and give the
    oracle's skeleton, as they do alone."""
    big = hg.sem_generate(900, 3000, hg.GRAPH_PA, 3.0, 2, 0.2, 1.0, 4242, dtype=np.float32)
    small = requests(10, seed=3)
    alpha, ml = 0.01, 4
    # at most two admissions between steps: the later requests are admitted while the
    # first ones run their levels
    sv = hg.SkeletonServer(max_level=ml, max_batch=16, max_inflight=2)
    bid = sv.submit(big, alpha, want_adjacency=True)
    ids = [sv.submit(X, alpha, want_adjacency=True) for X in small]
    sv.drain()
    done = {d["id"]: d for d in sv.poll()}
    assert done[bid]["status"] == 0
    assert any(done[r]["joined"] > 0 for r in ids)
    assert max(d["batch_size"] for d in done.values()) > 1
    for rid, X in [(bid, big)] + list(zip(ids, small)):
        d = done[rid]
        assert d["status"] == 0
        Cm = orc.correlation(X.astype(np.float64))
        want = orc.run(Cm, X.shape[1], alpha, ml)
        assert np.array_equal(d["adjacency"], want.adj), (rid, d["joined"])
        assert d["edges"] == want.edges()
    sv.close()


def _c5_fixture():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "c5_golden.json")
    if not os.path.exists(path):
        return None
    with open(path) as f:
        return json.load(f)


C5 = _c5_fixture()


@pytest.mark.skipif(C5 is None, reason="tests/golden/c5_golden.json not generated")
def test_full_range_requests_equal_the_oracle():
    """Requests spanning the served workload's range (p up to 5000, n up to 20000,
    hub-heavy preferential-attachment graphs), served together to the served workload's
    level cap, against the committed oracle results (tests/golden/make_c5_golden.py)."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import make_c5_golden as g5
    from helpers import sha
    import bench
    sv = hg.SkeletonServer(max_level=C5["max_level"])
    ids, data = [], []
    for row in C5["requests"]:
        X = g5.request_data(row["q"])
        assert sha(X) == row["data_sha256"], row["q"]
        data.append(X)
        ids.append(sv.submit(X, C5["alpha"], want_adjacency=True))
    sv.drain()
    done = {d["id"]: d for d in sv.poll()}
    for rid, row in zip(ids, C5["requests"]):
        d = done[rid]
        assert d["status"] == 0, row
        assert bench.c4_adj_sha(d["adjacency"]) == row["adj_sha256"], row
        assert d["edges"] == row["edges"]
    sv.close()
