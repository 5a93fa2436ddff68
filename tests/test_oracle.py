"""The oracle against the reference's golden fixtures, numpy/scipy and itself."""
import itertools
import math

import numpy as np
import pytest

from helpers import case_inputs, edge_set, golden_edges
from oracle import oracle as orc


def test_golden_cases_reproduced(golden):
    """Oracle edge sets equal the reference CPU code's on every fixture."""
    for case in golden["cases"]:
        _, Cm = case_inputs(case)
        res = orc.run(Cm, case["n_obs"], case["alpha"], case["max_level"])
        assert edge_set(res.adj) == golden_edges(case), case["name"]


def test_golden_sepsets_separate(golden):
    """Every separation set of the oracle re-tests as independent in FP64, and the
    level-0 removals agree with the reference's -2 markers."""
    for case in golden["cases"]:
        _, Cm = case_inputs(case)
        n, a = case["n_obs"], case["alpha"]
        res = orc.run(Cm, n, a, case["max_level"])
        for (i, j), (lev, ids, pmax) in res.records.items():
            assert len(ids) == lev
            assert orc.verify_sepset(Cm, n, a, i, j, ids), (case["name"], i, j, ids)
            assert pmax >= a
        ref_l0 = {(i, j) for i, j, lev, ids in case["ref_sepsets"] if lev == 0}
        ora_l0 = {(i, j) for i, j in zip(*np.nonzero(res.l0_deleted))}
        assert ref_l0 == ora_l0, case["name"]


def test_golden_sepsets_serial_equal_for_levels_2_3(golden):
    """Single-threaded, the oracle visits tests in the reference's order, so the
    stored sets for levels 2 and 3 are identical (level 1 differs by the reference's
    adj_compact[col*p + subIndex] indexing, cpuRowTests.cpp:47; levels >= 4 use the
    reference's descending workstealing order)."""
    for case in golden["cases"]:
        _, Cm = case_inputs(case)
        res = orc.run(Cm, case["n_obs"], case["alpha"], case["max_level"], threads=1)
        for i, j, lev, ids in case["ref_sepsets"]:
            if lev in (2, 3):
                assert res.records[(i, j)][1] == tuple(ids), (case["name"], i, j)


def test_pvalue_known_answers():
    scipy_special = pytest.importorskip("scipy.special")
    for r, n in [(0.0, 10), (0.1, 100), (-0.3, 1000), (0.05, 5000), (0.9, 50), (0.99999999, 1000)]:
        rr = min(0.9999999, abs(r))
        z = math.sqrt(n - 3) * math.atanh(rr)
        want = scipy_special.erfc(z / math.sqrt(2))
        assert orc.calc_pvalue(r, n) == pytest.approx(want, rel=1e-12, abs=1e-300)
    assert orc.calc_pvalue(float("nan"), 100) == 1.0  # NaN r counts as 0 (cpuInd.cpp:10)


def test_pval_l1_closed_form_and_nan():
    x1, x2, x3, n = 0.3, 0.2, 0.4, 500
    r = (x1 - x2 * x3) / math.sqrt((1 - x3 * x3) * (1 - x2 * x2))
    assert orc.pval_l1(x1, x2, x3, n) == orc.calc_pvalue(r, n)
    assert math.isnan(orc.pval_l1(float("nan"), 0.1, 0.1, n))


def test_pinv_matches_numpy():
    rng = np.random.default_rng(3)
    for k in range(2, 9):
        A = rng.standard_normal((k, 2 * k))
        M = np.corrcoef(A)
        np.testing.assert_allclose(orc.pinv(M), np.linalg.pinv(M, rcond=k * np.finfo(float).eps), rtol=1e-9,
                                   atol=1e-10)
        # rank-deficient: duplicated variable
        A[1] = A[0]
        M = np.corrcoef(A)
        np.testing.assert_allclose(orc.pinv(M), np.linalg.pinv(M, rcond=k * np.finfo(float).eps, hermitian=True),
                                   rtol=1e-7, atol=1e-8)


def test_pval_ln_equals_partial_correlation():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((6, 40))
    M = np.corrcoef(A)
    P = np.linalg.inv(M)
    r = -P[0, 1] / math.sqrt(P[0, 0] * P[1, 1])
    assert orc.pval_ln(M, 40) == pytest.approx(orc.calc_pvalue(r, 40), rel=1e-10)


def test_unranking_matches_combinations():
    """ithCombination (cuda_util.cu:34-50) enumerates 1-based lexicographic subsets."""
    for m in range(1, 9):
        for l in range(1, m + 1):
            combos = list(itertools.combinations(range(1, m + 1), l))
            assert orc.binom(m, l) == len(combos)
            for rank, c in enumerate(combos):
                assert tuple(orc.ith_combination(rank, l, m)) == c


def test_correlation_matches_numpy():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((7, 300)) * np.arange(1, 8)[:, None] + 3.0
    np.testing.assert_allclose(orc.correlation(X), np.corrcoef(X), rtol=0, atol=1e-13)
