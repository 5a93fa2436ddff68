"""Split-BF16 tcgen05 Gram (HPC_PREC_MIXED_TC) against the FP64 oracle correlation."""
import numpy as np
import pytest

import heterogpc as hg
from helpers import gen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

# |error| bound of the split-BF16 Gram with FP32 accumulation (hi.hi + hi.lo + lo.hi):
# each product term carries about 2^-16 relative error, the FP32 sums about 2^-24
TC_TOL = 2e-6


@pytest.mark.parametrize("p,n,dtype", [(130, 70, np.float64), (300, 1000, np.float64), (777, 2049, np.float32),
                                       (2000, 5000, np.float32)])
def test_tensorcore_gram_accuracy(p, n, dtype):
    X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=p + n, dtype=dtype)
    want = orc.correlation(X.astype(np.float64))
    sk = hg.SkeletonCalculator(p, n, precision=hg.PREC_MIXED_TC)
    sk.add_observations(X)
    C32 = sk.correlation_f32()
    assert np.array_equal(C32, C32.T)  # written from the upper triangle only
    err = np.abs(C32.astype(np.float64) - want)
    off = err[~np.eye(p, dtype=bool)]
    print("p=%d n=%d max |err| off-diagonal %.3g, diagonal %.3g" % (p, n, off.max(), np.diag(err).max()))
    assert off.max() < TC_TOL, off.max()
    assert np.diag(err).max() < 5 * TC_TOL


def test_tensorcore_skeleton_matches_oracle():
    X = gen(dict(p=400, n=2000, graph=hg.GRAPH_PA, pa_parents=2, w_lo=0.2, seed=91))
    Cm = orc.correlation(X)
    want = orc.run(Cm, 2000, 0.05, 6)
    sk = hg.SkeletonCalculator(400, 2000, alpha=0.05, max_level=6, precision=hg.PREC_MIXED_TC)
    sk.add_observations(X)
    sk.run()
    assert np.array_equal(sk.adjacency(), want.adj)
