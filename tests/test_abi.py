"""The C ABI library without a GPU: it loads, exports every declared entry point,
and its host-side pieces (statistics, generator, argument checks) behave."""
import os
import re

import numpy as np
import pytest

import heterogpc as hg
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^(?:const\s+)?[a-z_0-9]+\s*\**\s*(hpc_[a-z0-9_]+)\s*\(", src, re.M))
    return names


def test_library_exports_every_declared_symbol():
    L = hg.lib()
    names = declared_symbols()
    assert "hpc_ctx_create" in names and "hpc_run_level" in names
    for name in sorted(names):
        assert hasattr(L, name), name


def test_reference_named_entry_points_exported():
    """gpuPMCC and callCompact with the reference's C++ signatures (heterogpc_compat.h)."""
    import ctypes
    L = ctypes.CDLL(hg.LIB_PATH)
    for mangled in ("_Z7gpuPMCCPKdmiPdib", "_Z11callCompactP7MMStateiiii"):
        assert hasattr(L, mangled), mangled


def test_compat_header_layout():
    """MMState has the reference's member order (src/util/state.cuh:29-56)."""
    src = open(os.path.join(ROOT, "include", "heterogpc_compat.h")).read()
    body = src[src.index("struct MMState {"):src.index("};", src.index("struct MMState {"))]
    members = re.findall(r"\b(\w+);", body)
    assert members == ["ats", "pMax", "adj", "adj_compact", "cor", "sepSets", "p", "observations", "alpha",
                       "maxCondSize", "max_adj", "lock", "maxLevel", "node_status", "gpu_done"]


def test_binding_covers_header():
    assert declared_symbols() <= set(hg.exported_symbols()) | {"hpc_ctx_footprint"}


def test_host_statistics_match_oracle():
    rng = np.random.default_rng(0)
    for _ in range(200):
        r = float(rng.uniform(-1, 1))
        n = int(rng.integers(4, 10000))
        assert hg.calcPValue(r, n) == orc.calc_pvalue(r, n)
        x = rng.uniform(-0.9, 0.9, 3)
        assert hg.pValL1(*x, n) == orc.pval_l1(*x, n)
    for k in range(3, 9):
        A = rng.standard_normal((k, 3 * k))
        M = np.corrcoef(A)
        assert hg.pValLN(M, 500) == pytest.approx(orc.pval_ln(M, 500), rel=1e-9)


def test_z_crit():
    assert hg.z_crit(0.05) == pytest.approx(1.959963984540054, rel=1e-12)
    assert hg.z_crit(0.01) == pytest.approx(2.5758293035489004, rel=1e-12)


def test_generator_deterministic_and_shaped():
    X1, dag = hg.sem_generate(30, 200, hg.GRAPH_ER, 3.0, seed=5, want_dag=True)
    X2 = hg.sem_generate(30, 200, hg.GRAPH_ER, 3.0, seed=5)
    assert X1.shape == (30, 200) and np.array_equal(X1, X2)
    assert dag.sum() > 0 and np.all(np.diag(dag) == 0)
    assert not np.any(dag & dag.T)  # acyclic pairs
    X3 = hg.sem_generate(30, 200, hg.GRAPH_ER, 3.0, seed=6)
    assert not np.array_equal(X1, X3)
    Xf = hg.sem_generate(30, 200, hg.GRAPH_ER, 3.0, seed=5, dtype=np.float32)
    assert Xf.dtype == np.float32 and np.array_equal(Xf, X1.astype(np.float32))
    _, dpa = hg.sem_generate(200, 10, hg.GRAPH_PA, pa_parents=2, seed=1, want_dag=True)
    assert dpa.sum() == 2 * 200 - 3  # node 1 has one parent, later nodes two
    deg = dpa.sum(0) + dpa.sum(1)
    assert deg.max() >= 8  # hubs


def test_no_device_fails_loudly():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(hg.HpcError) as e:
        hg.SkeletonCalculator(10, 100)
    assert e.value.status == 8  # HPC_ERR_NO_DEVICE


def test_invalid_arguments_rejected():
    with pytest.raises(hg.HpcError) as e:
        hg.SkeletonCalculator(1, 100)
    assert e.value.status == 1
    with pytest.raises(hg.HpcError):
        hg.SkeletonCalculator(10, 100, alpha=0.0)
    with pytest.raises(hg.HpcError):
        hg.SkeletonCalculator(10, 100, max_level=hg.HPC_MAX_LEVEL + 1)


def _footprint(p, n, precision=hg.PREC_MIXED, max_level=4):
    import ctypes as C
    o = hg.Opts()
    hg.lib().hpc_opts_default(C.byref(o))
    o.precision, o.max_level = precision, max_level
    b = C.c_int64(0)
    st = hg.lib().hpc_ctx_footprint(p, n, C.byref(o), C.byref(b))
    return st, b.value


def test_footprint_follows_the_layout():
    """The device bytes the server admits a request by (hpc_ctx_footprint): they grow with
    p and n, tensor-core mode holds the split operands and the re-test queue instead of
    the FP64 matrix, and records grow with the max level (one id slot per level)."""
    st, small = _footprint(100, 1000)
    assert st == 0 and small > 0
    assert _footprint(2000, 1000)[1] > small and _footprint(100, 5000)[1] > small
    p, n = 2000, 5000
    fp64 = _footprint(p, n, hg.PREC_FP64)[1]
    mixed = _footprint(p, n, hg.PREC_MIXED)[1]
    tc = _footprint(p, n, hg.PREC_MIXED_TC)[1]
    assert mixed - fp64 == p * p * 4                       # the FP32 copy
    assert tc > mixed - p * p * 8                          # split operands + re-test queue replace cor64
    assert _footprint(p, n, hg.PREC_MIXED, -1)[1] > _footprint(p, n, hg.PREC_MIXED, 4)[1]
    assert _footprint(1, n)[0] == 1 and _footprint(p, 3)[0] == 1  # HPC_ERR_INVALID_ARG
