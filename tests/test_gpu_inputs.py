"""Correlation inputs the other parity tests do not reach, against the oracle:

  * observations with missing samples (NaN) through hpc_correlation_f64/_f32 in every
    precision: the pairwise skip of src/correlation/corHelper.cu:22-28,98-106 (mean and
    SD over each variable's present samples, products with a missing sample left out,
    the n - 1 denominator);
  * the reference-compatible standard deviation (ref_compat_sd: sqrtf of the variance,
    corHelper.cu:75) against orc.correlation(X, ref_compat=True);
  * the full p=2000, n=5000 workload (ER degree 4, alpha 0.01, max level 6) on the plain
    FP64 path.
"""
import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12


def with_missing(X, seed, frac=0.03, columns=(1, 4, 7, 11)):
    rng = np.random.default_rng(seed)
    Y = X.copy()
    for v in columns:
        Y[v, rng.random(Y.shape[1]) < frac] = np.nan
    return Y


@pytest.mark.parametrize("precision", [hg.PREC_FP64, hg.PREC_MIXED, hg.PREC_MIXED_TC])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_nan_observations(precision, dtype):
    p, n, alpha = 60, 900, 0.05
    X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=31, dtype=dtype)
    Xn = with_missing(X, 5)
    Cm = orc.correlation(Xn.astype(np.float64))
    assert np.isfinite(Cm).all()
    want = orc.run(Cm, n, alpha, -1)
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=-1, precision=precision)
    sk.add_observations(Xn)
    sk.run()
    assert np.abs(sk.correlation() - Cm).max() <= TOL
    assert np.array_equal(sk.adjacency(), want.adj)
    for i, j, lev, ids, pmax in sk.sepset_records():
        assert orc.verify_sepset(Cm, n, alpha, i, j, ids)
    sk.close()


def test_nan_observations_in_a_batch():
    ps, ns = np.array([30, 45, 60]), np.array([500, 700, 900])
    Xs = [with_missing(hg.sem_generate(int(p), int(n), hg.GRAPH_ER, 2.5, seed=40 + b, dtype=np.float32), b)
          for b, (p, n) in enumerate(zip(ps, ns))]
    bt = hg.SkeletonBatch(ps, ns, np.array([0.05, 0.01, 0.05]), max_level=-1, precision=hg.PREC_MIXED_TC)
    bt.add_observations(bt.pack(Xs))
    bt.run()
    for b in range(3):
        Cm = orc.correlation(Xs[b].astype(np.float64))
        want = orc.run(Cm, int(ns[b]), [0.05, 0.01, 0.05][b], -1)
        assert np.array_equal(bt.adjacency(b), want.adj)


@pytest.mark.parametrize("precision", [hg.PREC_FP64, hg.PREC_MIXED, hg.PREC_MIXED_TC])
def test_reference_compatible_sd(precision):
    p, n, alpha = 80, 1200, 0.01
    X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=32)
    Cr = orc.correlation(X, ref_compat=True)
    C64 = orc.correlation(X)
    assert np.abs(Cr - C64).max() > 1e-10  # the float SD changes the entries
    want = orc.run(Cr, n, alpha, -1)
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=-1, precision=precision, ref_compat_sd=True)
    sk.add_observations(X)
    sk.run()
    assert np.abs(sk.correlation() - Cr).max() <= TOL
    assert np.array_equal(sk.adjacency(), want.adj)
    sk.close()


def test_config2_full_size_plain_fp64():
    """p=2000, n=5000, FP32 data, ER degree 4, alpha 0.01, max level 6 on the plain path."""
    X = hg.sem_generate(2000, 5000, hg.GRAPH_ER, 4.0, 2, 0.1, 1.0, 2, dtype=np.float32)
    Cm = orc.correlation(X.astype(np.float64))
    want = orc.run(Cm, 5000, 0.01, 6)
    sk = hg.SkeletonCalculator(2000, 5000, alpha=0.01, max_level=6, precision=hg.PREC_FP64)
    sk.add_observations(X)
    st = sk.run()
    assert np.abs(sk.correlation() - Cm).max() < TOL
    assert np.array_equal(sk.adjacency(), want.adj)
    assert [s["edges_after"] for s in st] == [l["edges_after"] for l in want.levels]
    recs = sk.sepset_records()
    assert len(recs) == len(want.records)
    ok = orc.verify_sepsets(Cm, 5000, 0.01, [(i, j, lev, ids) for i, j, lev, ids, _ in recs])
    assert ok.all()
    assert all(pm >= 0.01 for *_, pm in recs)
    sk.close()
