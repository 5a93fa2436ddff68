"""Failure detection without a GPU fault (the reference exits the process on any CUDA
error, src/util/cuda_util.cuh:28-50; here every failure is a status code):

  * a grid-barrier wait of the level kernels that cannot complete (its arrival target
    raised by one through the test hook) runs out after its bound, the kernel returns,
    the run reports HPC_ERR_TIMEOUT, and the same context then gives the oracle's
    skeleton again after the hook is cleared and the context reset;
  * the k-th device allocation failing, for every k a context's life reaches, gives
    HPC_ERR_OOM from whichever call made it and leaves no device allocation behind.
"""
import numpy as np
import pytest

import heterogpc as hg
from helpers import gen
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_barrier_wait_runs_out_and_context_recovers():
    p, n, alpha = 150, 1000, 0.05
    X = gen(dict(p=p, n=n, graph=hg.GRAPH_ER, degree=3.0, seed=81))
    Cm = orc.correlation(X)
    want = orc.run(Cm, n, alpha, 4)
    sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=4, precision=hg.PREC_MIXED)
    sk.add_correlation_matrix(Cm)
    sk.run()
    assert np.array_equal(sk.adjacency(), want.adj)
    sk.set_barrier(50_000_000, 1)  # 50 ms, one arrival more than the grid makes
    sk.reset()
    with pytest.raises(hg.HpcError) as e:
        sk.run()
    assert e.value.status == 4  # HPC_ERR_TIMEOUT
    assert b"timed out" in hg.lib().hpc_last_error_string()
    sk.set_barrier(2_000_000_000, 0)
    sk.reset()
    sk.run()
    assert np.array_equal(sk.adjacency(), want.adj)
    # a level run by itself reports the same way
    sk.set_barrier(20_000_000, 1)
    sk.reset()
    sk.calc_level(0)
    with pytest.raises(hg.HpcError) as e:
        sk.calc_level(1)
    assert e.value.status == 4
    sk.set_barrier(2_000_000_000, 0)
    sk.reset()
    sk.run()
    assert np.array_equal(sk.adjacency(), want.adj)
    sk.close()


def test_every_allocation_failure_reported_without_leak():
    p, n, alpha = 60, 500, 0.05
    X = gen(dict(p=p, n=n, graph=hg.GRAPH_ER, degree=3.0, seed=82))
    L = hg.lib()
    base = L.hpc_debug_live_allocations()
    failures = 0
    for k in range(1, 200):
        L.hpc_debug_fail_allocation(k)
        failed = False
        sk = None
        try:
            sk = hg.SkeletonCalculator(p, n, alpha=alpha, max_level=3, precision=hg.PREC_MIXED_TC)
            sk.add_observations(X.astype(np.float32))
            sk.run()
            sk.sepset_records()
            sk.adjacency()
        except hg.HpcError as e:
            assert e.status == 2, e  # HPC_ERR_OOM
            assert b"injected" in L.hpc_last_error_string()
            failed = True
        finally:
            L.hpc_debug_fail_allocation(0)
            if sk is not None:
                sk.close()
        assert L.hpc_debug_live_allocations() == base, k
        if not failed:
            break  # k beyond the allocations a context makes: all have been tried
        failures += 1
    assert failures >= 10
