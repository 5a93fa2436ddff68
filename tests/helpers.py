"""Shared helpers of the test suite: golden-case inputs and comparisons."""
import hashlib

import numpy as np

import heterogpc as hg
from oracle import oracle as orc


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def gen(params):
    kw = dict(degree=2.0, pa_parents=2, w_lo=0.1, w_hi=1.0)
    kw.update(params)
    return hg.sem_generate(kw["p"], kw["n"], kw["graph"], kw["degree"], kw["pa_parents"], kw["w_lo"], kw["w_hi"],
                           kw["seed"])


def case_inputs(case):
    """(X or None, correlation matrix) of a golden case; checks the stored hashes."""
    if case["source"] == "sem":
        X = gen(case["params"])
        assert sha(X) == case["data_sha256"], "generator output differs on this host"
        Cm = orc.correlation(X)
    else:
        X = None
        Cm = np.array([[np.nan if v is None else v for v in row] for row in case["cor"]], dtype=np.float64)
    assert sha(Cm) == case["cor_sha256"], "correlation differs from the fixture on this host"
    return X, Cm


def edge_set(adj):
    i, j = np.nonzero(np.triu(adj, 1))
    return set(zip(i.tolist(), j.tolist()))


def golden_edges(case):
    return set(tuple(e) for e in case["edges"])
