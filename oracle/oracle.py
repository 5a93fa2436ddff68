"""ORACLE -- test infrastructure only.

ctypes wrapper of liboracle.so (the FP64 OpenMP restatement of the reference's CPU
skeleton path, oracle/oracle.cpp) and, where it was built, of oracle/_ref/libref_cpu.so
(the reference's own CPU test sources compiled against restated Armadillo/Boost
headers). Only the tests, the smoke check and the CPU-baseline legs of bench.py use
this module; the product never imports it.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_cpu.so")

_orc = None
_ref = None


def _p(a):
    return C.c_void_p(a.ctypes.data)


def lib():
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_SO):
            raise ImportError("oracle not built: %s" % ORACLE_SO)
        L = C.CDLL(ORACLE_SO)
        L.orc_calc_pvalue.restype = C.c_double
        L.orc_calc_pvalue.argtypes = [C.c_double, C.c_int]
        L.orc_pval_l1.restype = C.c_double
        L.orc_pval_l1.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int]
        L.orc_pval_ln.restype = C.c_double
        L.orc_pval_ln.argtypes = [C.c_void_p, C.c_int, C.c_int]
        L.orc_pinv.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.orc_binom.restype = C.c_uint64
        L.orc_binom.argtypes = [C.c_int, C.c_int]
        L.orc_ith_combination.argtypes = [C.c_void_p, C.c_uint64, C.c_int, C.c_int]
        L.orc_correlation.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_void_p]
        L.orc_run.restype = C.c_void_p
        L.orc_run.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_int, C.c_int]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_levels_run.argtypes = [C.c_void_p]
        for f in ("orc_tests", "orc_potential", "orc_edges_after"):
            getattr(L, f).restype = C.c_int64
            getattr(L, f).argtypes = [C.c_void_p, C.c_int]
        L.orc_ms.restype = C.c_double
        L.orc_ms.argtypes = [C.c_void_p, C.c_int]
        L.orc_adjacency.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_num_records.restype = C.c_int64
        L.orc_num_records.argtypes = [C.c_void_p]
        L.orc_records.restype = C.c_int64
        L.orc_records.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int64]
        L.orc_l0_deleted.argtypes = [C.c_void_p, C.c_int64, C.c_int64]
        _orc = L
    return _orc


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.ref_run.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                              C.c_void_p]
        _ref = L
    return _ref


def calc_pvalue(r, n):
    return lib().orc_calc_pvalue(float(r), int(n))


def pval_l1(x1, x2, x3, n):
    return lib().orc_pval_l1(float(x1), float(x2), float(x3), int(n))


def pval_ln(M, n):
    M = np.ascontiguousarray(M, np.float64)
    return lib().orc_pval_ln(_p(M), M.shape[0], int(n))


def pinv(M):
    M = np.ascontiguousarray(M, np.float64)
    P = np.empty_like(M)
    lib().orc_pinv(_p(M), M.shape[0], _p(P))
    return P


def binom(n, k):
    return lib().orc_binom(n, k)


def ith_combination(rank, level, neighbours):
    out = np.zeros(level, np.int32)
    lib().orc_ith_combination(_p(out), rank, level, neighbours)
    return out


def correlation(X, ref_compat=False):
    """X shape (p, n): each variable's samples contiguous. Returns the p x p matrix."""
    X = np.ascontiguousarray(X, np.float64)
    p, n = X.shape
    Cm = np.empty((p, p), np.float64)
    rc = lib().orc_correlation(_p(X), n, p, int(ref_compat), _p(Cm))
    assert rc == 0
    return Cm


class Result:
    def __init__(self, adj, levels, records, l0_deleted):
        self.adj = adj
        self.levels = levels  # list of dicts
        self.records = records  # {(i, j): (level, ids tuple, pmax)}
        self.l0_deleted = l0_deleted

    def edges(self):
        p = self.adj.shape[0]
        iu = np.triu_indices(p, 1)
        return int(self.adj[iu].sum())

    def edge_set(self):
        i, j = np.nonzero(np.triu(self.adj, 1))
        return set(zip(i.tolist(), j.tolist()))


def run(Cm, n_obs, alpha, max_level, threads=0):
    """Skeleton of the reference CPU path on correlation matrix Cm."""
    Cm = np.ascontiguousarray(Cm, np.float64)
    p = Cm.shape[0]
    L = lib()
    h = L.orc_run(_p(Cm), p, int(n_obs), float(alpha), int(max_level), int(threads))
    if not h:
        raise ValueError("oracle rejected the arguments")
    try:
        adj = np.empty((p, p), np.uint8)
        L.orc_adjacency(h, _p(adj))
        levels = []
        for l in range(L.orc_levels_run(h)):
            levels.append({"level": l, "potential_tests": L.orc_potential(h, l), "executed_tests": L.orc_tests(h, l),
                           "edges_after": L.orc_edges_after(h, l), "ms": L.orc_ms(h, l)})
        n = L.orc_num_records(h)
        recs = {}
        if n:
            mi = 64
            ijl = np.empty((n, 3), np.int32)
            ids = np.empty((n, mi), np.int32)
            pm = np.empty(n, np.float64)
            L.orc_records(h, _p(ijl), _p(ids), mi, _p(pm), n)
            for t in range(n):
                i, j, lev = ijl[t].tolist()
                recs[(i, j)] = (lev, tuple(ids[t, :lev].tolist()), float(pm[t]))
        l0 = np.zeros((p, p), np.uint8)
        if p <= 4096:
            for i in range(p):
                for j in range(i + 1, p):
                    if not adj[i, j] and (i, j) not in recs:
                        l0[i, j] = 1
        return Result(adj, levels, recs, l0)
    finally:
        L.orc_free(h)


def ref_run(Cm, n_obs, alpha, max_level, threads=1):
    """Run the reference's own CPU test code (only where oracle/_ref was built)."""
    Cm = np.ascontiguousarray(Cm, np.float64)
    p = Cm.shape[0]
    mc = max(max_level, 1)
    adj = np.empty((p, p), np.uint8)
    sep = np.empty((p, p, mc), np.int32)
    pmax = np.empty((p, p), np.float64)
    ref_lib().ref_run(_p(Cm), p, int(n_obs), C.c_double(alpha), int(max_level), int(threads), _p(adj), _p(sep),
                      _p(pmax))
    return adj, sep, pmax


def verify_sepset(Cm, n_obs, alpha, i, j, ids):
    """FP64 re-test of a stored separation set: True iff p >= alpha given ids."""
    ids = list(ids)
    if len(ids) == 0:
        return calc_pvalue(Cm[max(i, j), min(i, j)], n_obs) >= alpha
    if len(ids) == 1:
        k = ids[0]
        return pval_l1(Cm[i, j], Cm[i, k], Cm[j, k], n_obs) >= alpha
    idx = [i, j] + sorted(ids)
    k = len(idx)
    M = np.eye(k)
    for a in range(k):
        for b in range(a + 1, k):
            M[a, b] = M[b, a] = Cm[idx[a], idx[b]]
    return pval_ln(M, n_obs) >= alpha
