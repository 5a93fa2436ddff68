"""The allocation-free correlation entry point, through the C ABI.

hpc_correlation_noalloc_f64 is for callers that cannot allocate device memory when
they need a correlation matrix (a plugin whose host application owns all GPU memory
through its own pool, or a latency-critical caller that cannot afford the
device-wide synchronisation of cudaMalloc/cudaFree). It keeps its scratch in one
library-wide __device__ array shared by every call, so this test checks two calls
in a row, of different shapes, against the allocating entry point
(hpc_correlation_device_f64 read back with hpc_get_correlation), and the size limit.

This file is collected last so that a run stopping at the first failure has already
run every other test; it also passes when run alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import heterogpc as hg

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the correlation tolerance used by the other GPU tests


def _reference_correlation(Xd, p, n, ref_compat=False):
    sk = hg.SkeletonCalculator(p, n, precision=hg.PREC_FP64, ref_compat_sd=ref_compat)
    sk.add_observations_device(Xd.data_ptr(), np.float64)
    out = sk.correlation()
    sk.close()
    return out


def _noalloc(Xd, p, n, Cd, stream, ref_compat=0):
    return hg.lib().hpc_correlation_noalloc_f64(C.c_void_p(Xd.data_ptr()), n, p, int(ref_compat),
                                                C.c_void_p(Cd.data_ptr()), C.c_void_p(stream) if stream else None)


def test_noalloc_matches_allocating_entry_point_twice():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    shapes = [(48, 700, 3), (96, 1500, 4)]  # (p, n, seed): the second call reuses the scratch
    for p, n, seed in shapes:
        X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=seed)  # (p, n): column-major n x p
        Xd = torch.from_numpy(X).to(dev)
        Cd = torch.full((p, p), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = _noalloc(Xd, p, n, Cd, stream.cuda_stream)
        assert st == 0, hg.lib().hpc_last_error_string()
        stream.synchronize()
        got = Cd.cpu().numpy()
        want = _reference_correlation(Xd, p, n)
        assert np.isfinite(got).all()
        assert np.abs(got - want).max() <= TOL


@pytest.mark.parametrize("ref_compat,missing,default_stream", [(1, False, False), (0, True, False),
                                                              (1, True, True)])
def test_noalloc_variants_twice(ref_compat, missing, default_stream):
    """The float-rounded standard deviation (ref_compat_sd = 1), observations with
    missing samples and the default stream (NULL), each on two calls in a row."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = None if default_stream else torch.cuda.Stream(device=dev)
    for p, n, seed in [(40, 600, 5), (72, 1100, 6)]:
        X = hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=seed)
        if missing:
            X[2, ::13] = np.nan
            X[p - 1, 5::17] = np.nan
        Xd = torch.from_numpy(X).to(dev)
        Cd = torch.full((p, p), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        st = _noalloc(Xd, p, n, Cd, stream.cuda_stream if stream else None, ref_compat)
        assert st == 0, hg.lib().hpc_last_error_string()
        torch.cuda.synchronize()
        got = Cd.cpu().numpy()
        want = _reference_correlation(Xd, p, n, bool(ref_compat))
        assert np.isfinite(got).all()
        assert np.abs(got - want).max() <= TOL


def test_noalloc_rejects_oversize_inputs():
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    limit = 4 * 1024 * 1024
    p, n = 1024, limit // 1024 + 1
    Xd = torch.zeros(8, dtype=torch.float64, device=dev)  # never read: the call is refused first
    Cd = torch.zeros(8, dtype=torch.float64, device=dev)
    st = hg.lib().hpc_correlation_noalloc_f64(C.c_void_p(Xd.data_ptr()), n, p, 0, C.c_void_p(Cd.data_ptr()), None)
    assert st == 7  # HPC_ERR_CAPACITY
    assert b"allocation-free limit" in hg.lib().hpc_last_error_string()


def test_noalloc_captured_into_a_graph_and_replayed():
    """The call only enqueues kernels on the caller's stream (its shapes are written by a
    one-thread kernel, nothing is copied from host memory), so after a first call outside
    any capture it can be captured into a CUDA graph; each replay computes the
    correlation of the observations then in the input buffer."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    p, n = 64, 900
    Xd = torch.from_numpy(hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=7)).to(dev)
    Cd = torch.full((p, p), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()
    assert _noalloc(Xd, p, n, Cd, stream.cuda_stream) == 0, hg.lib().hpc_last_error_string()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        st = _noalloc(Xd, p, n, Cd, stream.cuda_stream)
    assert st == 0, hg.lib().hpc_last_error_string()
    for seed in (8, 9):
        Xd.copy_(torch.from_numpy(hg.sem_generate(p, n, hg.GRAPH_ER, 3.0, seed=seed)).to(dev))
        Cd.fill_(float("nan"))
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        got = Cd.cpu().numpy()
        want = _reference_correlation(Xd, p, n)
        assert np.isfinite(got).all()
        assert np.abs(got - want).max() <= TOL
