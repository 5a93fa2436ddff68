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
        L.orc_verify_sepsets.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_int64, C.c_void_p,
                                         C.c_void_p, C.c_int, C.c_void_p]
        L.orc_check_retained.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_int, C.c_void_p,
                                         C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
        L.hpc_sem_generate.restype = C.c_int
        L.hpc_sem_generate.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
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


class _SemParams(C.Structure):
    _fields_ = [("p", C.c_int64), ("n", C.c_int64), ("graph", C.c_int), ("degree", C.c_double),
                ("pa_parents", C.c_int), ("w_lo", C.c_double), ("w_hi", C.c_double), ("seed", C.c_uint64)]


def sem_generate(p, n, graph=0, degree=2.0, pa_parents=2, w_lo=0.1, w_hi=1.0, seed=1, dtype=np.float64):
    """The seeded SEM generator (masterthesis-heterogeneous-pc_gb300/host/semgen.cpp, host
    code compiled into this library): the same bytes as the product's hpc_sem_generate,
    for CPU-only legs that must not load the product library."""
    prm = _SemParams(p, n, graph, degree, pa_parents, w_lo, w_hi, seed)
    X = np.empty((p, n), dtype)
    x64 = _p(X) if dtype == np.float64 else None
    x32 = _p(X) if dtype == np.float32 else None
    rc = lib().hpc_sem_generate(C.byref(prm), x64, x32, None, None)
    if rc != 0:
        raise ValueError("sem_generate rejected the parameters (%d)" % rc)
    return X


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


def verify_sepsets(Cm, n_obs, alpha, records):
    """FP64 re-test of many stored separation sets at once: records is a list of
    (i, j, level, ids); returns a bool array, True where p >= alpha given ids."""
    Cm = np.ascontiguousarray(Cm, np.float64)
    k = len(records)
    if k == 0:
        return np.zeros(0, bool)
    mi = max(1, max(r[2] for r in records))
    ijl = np.empty((k, 3), np.int32)
    ids = np.full((k, mi), -1, np.int32)
    for t, r in enumerate(records):
        ijl[t] = (r[0], r[1], r[2])
        ids[t, :r[2]] = r[3][:r[2]]
    ok = np.zeros(k, np.uint8)
    lib().orc_verify_sepsets(_p(Cm), Cm.shape[0], int(n_obs), float(alpha), k, _p(ijl), _p(ids), mi, _p(ok))
    return ok.astype(bool)


def check_retained(Cm, n_obs, alpha, level, adj_before, edges, max_subsets):
    """Exhaustive FP64 check of kept edges (k x 2 array, i < j) at `level`: every subset of
    either endpoint's snapshot neighbours (adj_before, the adjacency at the level start)
    is tested. Returns per edge 0 = no subset separates, 1 = a subset separates,
    2 = not checked (more than max_subsets subsets on a side)."""
    Cm = np.ascontiguousarray(Cm, np.float64)
    A = np.ascontiguousarray(adj_before, np.uint8)
    E = np.ascontiguousarray(edges, np.int32).reshape(-1, 2)
    st = np.zeros(len(E), np.int8)
    lib().orc_check_retained(_p(Cm), Cm.shape[0], int(n_obs), float(alpha), int(level), _p(A), len(E), _p(E),
                             int(max_subsets), _p(st))
    return st


def verify_record_array(Cm, n_obs, alpha, recs):
    """verify_sepsets for a numpy structured array of records with fields i, j, level and
    ids (one row per record, ids padded): True where p >= alpha given the stored set."""
    Cm = np.ascontiguousarray(Cm, np.float64)
    k = len(recs)
    if k == 0:
        return np.zeros(0, bool)
    ijl = np.ascontiguousarray(np.stack([recs["i"], recs["j"], recs["level"]], axis=1), np.int32)
    ids = np.ascontiguousarray(recs["ids"], np.int32)
    ok = np.zeros(k, np.uint8)
    lib().orc_verify_sepsets(_p(Cm), Cm.shape[0], int(n_obs), float(alpha), k, _p(ijl), _p(ids), ids.shape[1],
                             _p(ok))
    return ok.astype(bool)
