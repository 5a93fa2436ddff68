"""The FP64-accurate tensor-core Gram (exact BF16 digits, csrc/gram_emu.cu), which
computes the correlation of HPC_PREC_MIXED contexts of one instance with p >= 256,
against the oracle's FP64 correlation (src/correlation/corHelper.cu:8-116): within
1e-12 everywhere, its FP32 copy the rounding of the FP64 entries, and the skeleton the
oracle's."""
import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.mark.parametrize("p,n,dtype", [(256, 500, np.float64), (300, 1100, np.float64), (777, 2049, np.float32),
                                       (2000, 5000, np.float32), (1024, 20000, np.float32), (400, 32768, np.float32)])
def test_emulated_gram_accuracy(p, n, dtype):
    X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=p + n, dtype=dtype)
    want = orc.correlation(X.astype(np.float64))
    sk = hg.SkeletonCalculator(p, n, precision=hg.PREC_MIXED, max_level=0)
    sk.add_observations(X)
    got = sk.correlation()
    err = np.abs(got - want).max()
    print("p=%d n=%d max |err| %.3g" % (p, n, err))
    assert err <= TOL
    assert np.array_equal(got, got.T)
    assert np.array_equal(sk.correlation_f32(), got.astype(np.float32))
    sk.close()


@pytest.mark.parametrize("ref_compat", [False, True])
def test_emulated_gram_nan_and_reference_sd(ref_compat):
    p, n = 320, 3000
    X = hg.sem_generate(p, n, hg.GRAPH_PA, 3.0, 2, 0.2, 1.0, 71)
    X[5, ::11] = np.nan
    X[200, 3::29] = np.nan
    want = orc.correlation(X, ref_compat=ref_compat)
    sk = hg.SkeletonCalculator(p, n, alpha=0.05, max_level=-1, precision=hg.PREC_MIXED, ref_compat_sd=ref_compat)
    sk.add_observations(X)
    assert np.abs(sk.correlation() - want).max() <= TOL
    sk.run()
    assert np.array_equal(sk.adjacency(), orc.run(want, n, 0.05, -1).adj)
    sk.close()
