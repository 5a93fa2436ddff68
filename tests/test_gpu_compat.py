"""The reference-named entry points (include/heterogpc_compat.h: gpuPMCC, callCompact,
MMState; include/heterogpc_gpu_ind.cuh: GPU::calcPValue, GPU::pValL1) through a C++
program written as a caller of the reference would be (tests/compat_check.cu), built
with nvcc and linked against libheterogpc.so; its outputs are checked against the
oracle: the correlation of src/correlation/corOwn.cu:10-48 (float-rounded SD, pairwise
NaN skip), the compaction of src/independence/compact.cu:4-99 and the statistics of
src/executor/independence/gpuInd.cu:4-19."""
import os
import subprocess

import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.dirname(hg.LIB_PATH)


@pytest.fixture(scope="module")
def out(tmp_path_factory):
    d = tmp_path_factory.mktemp("compat")
    exe = str(d / "compat_check")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                    os.path.join(ROOT, "tests", "compat_check.cu"), "-o", exe, "-L", LIBDIR, "-lheterogpc",
                    "-Xlinker", "-rpath," + LIBDIR], check=True, capture_output=True)
    r = subprocess.run([exe, str(d)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return d


def load(d, name, dtype):
    return np.fromfile(os.path.join(d, name), dtype=dtype)


def test_gpuPMCC_matches_the_reference_arithmetic(out):
    p, dim = 40, 500
    X = load(out, "X.f64", np.float64).reshape(p, dim)
    got = load(out, "cors.f64", np.float64).reshape(p, p)
    want = orc.correlation(X, ref_compat=True)
    assert np.isnan(X).sum() == 2
    assert np.abs(got - want).max() <= 1e-12


def test_callCompact_lists_and_counts(out):
    q = 70
    adj = load(out, "adj.i32", np.int32).reshape(q, q)
    for name, rows, mx in (("compact_all.i32", range(q), "max_all.i32"), ("compact_blk.i32", range(24, 48),
                                                                          "max_blk.i32")):
        comp = load(out, name, np.int32).reshape(q, q)
        counts = []
        for i in range(q):
            if i not in rows:
                assert np.all(comp[i] == -7)  # rows of other blocks untouched
                continue
            ids = np.nonzero(adj[i])[0]
            d = len(ids)
            counts.append(d)
            assert np.array_equal(comp[i, :d], ids)
            assert np.all(comp[i, d:q - 1] == 0)
            assert comp[i, q - 1] == d
        assert load(out, mx, np.int32)[0] == max(counts)


def test_gpu_statistics(out):
    r = load(out, "r.f64", np.float64)
    x = load(out, "x.f64", np.float64).reshape(-1, 3)
    for kind in ("dev", "host"):
        p0 = load(out, kind + "_p0.f64", np.float64)
        p1 = load(out, kind + "_p1.f64", np.float64)
        for t in range(len(r)):
            # 2 (1 - Phi(z)) as the reference's device code: absolute agreement with the
            # oracle's complement form
            assert abs(p0[t] - orc.calc_pvalue(r[t], 900)) <= 1e-14, (kind, t)
            assert abs(p1[t] - orc.pval_l1(*x[t], 900)) <= 1e-14, (kind, t)
