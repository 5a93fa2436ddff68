"""Oracle against the reference's own CPU code on fresh seeds (only where the
reference-pinning library oracle/_ref was built, i.e. beside the reference tree)."""
import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.skipif(not orc.ref_available(), reason="oracle/_ref not built on this host")


@pytest.mark.parametrize("seed", range(30, 42))
def test_oracle_equals_reference_code(seed):
    rng = np.random.default_rng(seed)
    p = int(rng.integers(10, 70))
    n = int(rng.integers(60, 1500))
    graph = hg.GRAPH_PA if seed % 2 else hg.GRAPH_ER
    X = hg.sem_generate(p, n, graph, float(rng.uniform(1, 5)), 2, 0.1, 1.0, seed)
    Cm = orc.correlation(X)
    alpha = [0.01, 0.05, 0.2][seed % 3]
    ml = int(rng.integers(0, 6))
    adj_ref, _, _ = orc.ref_run(Cm, n, alpha, ml)
    res = orc.run(Cm, n, alpha, ml, threads=4)
    assert np.array_equal(res.adj, adj_ref)
