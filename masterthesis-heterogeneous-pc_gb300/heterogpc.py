"""Python binding of libheterogpc (ctypes over the C ABI in include/heterogpc.h).

Mirrors the reference's skeleton interface (src/independence/skeleton.hpp:10-73):
``SkeletonCalculator(max_level, alpha, ...)`` with ``add_observations`` /
``add_correlation_matrix`` / ``calc_level`` / ``run``, backed by one GPU context.
There is no CPU fallback: importing works without a GPU, but every compute call
goes to the CUDA library and raises ``HpcError`` when no device is usable.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libheterogpc.so")

HPC_MAX_LEVEL = 32
PREC_FP64, PREC_MIXED, PREC_MIXED_TC = 0, 1, 2
GRAPH_ER, GRAPH_PA = 0, 1

STATUS = {0: "HPC_OK", 1: "HPC_ERR_INVALID_ARG", 2: "HPC_ERR_OOM", 3: "HPC_ERR_CUDA", 4: "HPC_ERR_TIMEOUT",
          5: "HPC_ERR_NUMERIC", 6: "HPC_ERR_STATE", 7: "HPC_ERR_CAPACITY", 8: "HPC_ERR_NO_DEVICE"}


class HpcError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))
        self.status = status


class Opts(C.Structure):
    _fields_ = [("device", C.c_int), ("alpha", C.c_double), ("max_level", C.c_int), ("precision", C.c_int),
                ("retest_margin", C.c_double), ("ref_compat_sd", C.c_int), ("verbose", C.c_int)]


class LevelStats(C.Structure):
    _fields_ = [("level", C.c_int), ("max_degree", C.c_int), ("rows", C.c_int64), ("potential_tests", C.c_int64),
                ("executed_tests", C.c_int64), ("retests", C.c_int64), ("edges_before", C.c_int64),
                ("edges_after", C.c_int64), ("ms", C.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class SepsetRecord(C.Structure):
    _fields_ = [("i", C.c_int32), ("j", C.c_int32), ("level", C.c_int32), ("pad", C.c_int32),
                ("pmax", C.c_double), ("ids", C.c_int32 * HPC_MAX_LEVEL)]


class Timings(C.Structure):
    _fields_ = [("standardise_ms", C.c_double), ("gram_ms", C.c_double), ("convert_ms", C.c_double),
                ("level_ms", C.c_double * (HPC_MAX_LEVEL + 1)), ("compact_ms", C.c_double * (HPC_MAX_LEVEL + 1)),
                ("test_ms", C.c_double * (HPC_MAX_LEVEL + 1)), ("launches", C.c_int64),
                ("skeleton_ms", C.c_double), ("retest_ms", C.c_double * (HPC_MAX_LEVEL + 1)),
                ("rebuild_ms", C.c_double * (HPC_MAX_LEVEL + 1)), ("scan_ms", C.c_double * (HPC_MAX_LEVEL + 1))]

    def as_dict(self):
        return {"standardise_ms": self.standardise_ms, "gram_ms": self.gram_ms, "convert_ms": self.convert_ms,
                "level_ms": list(self.level_ms), "compact_ms": list(self.compact_ms), "test_ms": list(self.test_ms),
                "launches": self.launches, "skeleton_ms": self.skeleton_ms, "retest_ms": list(self.retest_ms),
                "rebuild_ms": list(self.rebuild_ms), "scan_ms": list(self.scan_ms)}


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("max_level", C.c_int), ("budget_bytes", C.c_int64),
                ("max_batch", C.c_int), ("max_inflight", C.c_int)]


class Served(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("levels", C.c_int32), ("edges", C.c_int64),
                ("queue_ms", C.c_double), ("run_ms", C.c_double), ("latency_ms", C.c_double),
                ("batch_size", C.c_int32), ("joined", C.c_int32)]


class TuneParams(C.Structure):
    _fields_ = [("tile_cap", C.c_int), ("tiles_per_lane", C.c_int), ("edge_lanes", C.c_int), ("l1_prefetch", C.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class SemParams(C.Structure):
    _fields_ = [("p", C.c_int64), ("n", C.c_int64), ("graph", C.c_int), ("degree", C.c_double),
                ("pa_parents", C.c_int), ("w_lo", C.c_double), ("w_hi", C.c_double), ("seed", C.c_uint64)]


_lib = None

# symbol -> (restype, argtypes)
_SIGS = {
    "hpc_last_error_string": (C.c_char_p, []),
    "hpc_status_string": (C.c_char_p, [C.c_int]),
    "hpc_opts_default": (C.c_int, [C.POINTER(Opts)]),
    "hpc_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int64, C.c_int64, C.POINTER(Opts)]),
    "hpc_ctx_destroy": (C.c_int, [C.c_void_p]),
    "hpc_ctx_reset": (C.c_int, [C.c_void_p]),
    "hpc_ctx_footprint": (C.c_int, [C.c_int64, C.c_int64, C.POINTER(Opts), C.POINTER(C.c_int64)]),
    "hpc_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_get_timings": (C.c_int, [C.c_void_p, C.POINTER(Timings)]),
    "hpc_ctx_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "hpc_correlation_f64": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_correlation_f32": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_correlation_device_f64": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_correlation_device_f32": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_load_correlation": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_load_correlation_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_get_correlation": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_get_correlation_f32": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_correlation_noalloc_f64": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_void_p, C.c_void_p]),
    "hpc_run_level": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(LevelStats)]),
    "hpc_run_skeleton": (C.c_int, [C.c_void_p, C.POINTER(LevelStats), C.c_int, C.POINTER(C.c_int)]),
    "hpc_run_skeleton_async": (C.c_int, [C.c_void_p]),
    "hpc_wait": (C.c_int, [C.c_void_p, C.POINTER(LevelStats), C.c_int, C.POINTER(C.c_int)]),
    "hpc_get_adjacency": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_edge_count": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "hpc_get_sepsets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "hpc_get_sepset_records": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "hpc_calc_pvalue": (C.c_double, [C.c_double, C.c_int]),
    "hpc_pval_l1": (C.c_double, [C.c_double, C.c_double, C.c_double, C.c_int]),
    "hpc_pval_ln": (C.c_double, [C.c_void_p, C.c_int, C.c_int]),
    "hpc_z_crit": (C.c_double, [C.c_double]),
    "hpc_debug_fail_allocation": (C.c_int, [C.c_int64]),
    "hpc_debug_live_allocations": (C.c_int64, []),
    "hpc_debug_set_barrier": (C.c_int, [C.c_void_p, C.c_int64, C.c_int]),
    "hpc_debug_set_order_from": (C.c_int, [C.c_int]),
    "hpc_debug_set_retest_queue": (C.c_int, [C.c_void_p, C.c_int64]),
    "hpc_debug_set_order_active": (C.c_int, [C.c_void_p]),
    "hpc_sem_generate": (C.c_int, [C.POINTER(SemParams), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "hpc_server_opts_default": (C.c_int, [C.POINTER(ServerOpts)]),
    "hpc_server_create": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(ServerOpts)]),
    "hpc_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_double, C.c_void_p,
                                    C.POINTER(C.c_int64)]),
    "hpc_server_poll": (C.c_int, [C.c_void_p, C.POINTER(Served), C.c_int, C.POINTER(C.c_int)]),
    "hpc_server_drain": (C.c_int, [C.c_void_p]),
    "hpc_server_destroy": (C.c_int, [C.c_void_p]),
    "hpc_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.POINTER(Opts)]),
    "hpc_batch_size": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "hpc_batch_offsets": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hpc_batch_level_stats": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(LevelStats), C.c_int, C.POINTER(C.c_int)]),
    "hpc_batch_get_adjacency": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "hpc_batch_edge_count": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int64)]),
    "hpc_batch_get_sepset_records": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]),
    "hpc_batch_get_sepset_records_from": (C.c_int, [C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_int64,
                                                    C.POINTER(C.c_int64)]),
    "hpc_batch_adjacency_words": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hpc_batch_get_records_packed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "hpc_batch_get_adjacency_bits": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "hpc_batch_get_all_sepset_records": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "hpc_tune_set": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.POINTER(TuneParams)]),
    "hpc_tune_lookup": (C.c_int, [C.c_int64, C.c_int, C.c_int, C.POINTER(TuneParams), C.POINTER(C.c_int)]),
    "hpc_tune_clear": (C.c_int, []),
    "hpc_tune_save": (C.c_int, [C.c_char_p]),
    "hpc_tune_load": (C.c_int, [C.c_char_p]),
    "hpc_ctx_set_tune": (C.c_int, [C.c_void_p, C.POINTER(TuneParams)]),
    "hpc_autotune": (C.c_int, [C.c_void_p, C.POINTER(TuneParams), C.c_int, C.c_int, C.POINTER(TuneParams),
                               C.POINTER(C.c_int)]),
}


# ---- tile policy and autotuner (hpc_tune_* / hpc_autotune) ----------------------

def tune_set(p, level, max_degree, tile_cap=None, tiles_per_lane=4, edge_lanes=32, l1_prefetch=0):
    """Set (tile_cap given) or erase (None) the tile policy of a key's buckets."""
    prm = None if tile_cap is None else C.byref(TuneParams(tile_cap, tiles_per_lane, edge_lanes, l1_prefetch))
    _check(lib().hpc_tune_set(int(p), int(level), int(max_degree), prm))


def tune_lookup(p, level, max_degree):
    """(policy dict, found) of the key."""
    t, f = TuneParams(), C.c_int(0)
    _check(lib().hpc_tune_lookup(int(p), int(level), int(max_degree), C.byref(t), C.byref(f)))
    return t.as_dict(), bool(f.value)


def tune_clear():
    _check(lib().hpc_tune_clear())


def tune_save(path):
    _check(lib().hpc_tune_save(os.fsencode(path)))


def tune_load(path):
    _check(lib().hpc_tune_load(os.fsencode(path)))


SET_ORDER_DEFAULT = 3  # the library's default lowest set-order level (kSetOrderFrom)


def set_order_from(level):
    """The lowest level whose CI tests run in the set order, 0 for the edge order at every
    level (hpc_debug_set_order_from; process-wide). Both orders give the same skeleton."""
    _check(lib().hpc_debug_set_order_from(int(level)))


def _params(c):
    return TuneParams(c["tile_cap"], c.get("tiles_per_lane", 4), c.get("edge_lanes", 32), c.get("l1_prefetch", 0))


def _set_tune(h, policy):
    prm = None if policy is None else C.byref(_params(policy))
    _check(lib().hpc_ctx_set_tune(h, prm))


def _autotune(h, candidates, reps):
    """hpc_autotune on a context: {level: chosen policy}, entries written."""
    cap = HPC_MAX_LEVEL + 1
    chosen = (TuneParams * cap)()
    n = C.c_int(0)
    if candidates is None:
        _check(lib().hpc_autotune(h, None, 0, int(reps), chosen, C.byref(n)))
    else:
        arr = (TuneParams * len(candidates))(*[_params(c) for c in candidates])
        _check(lib().hpc_autotune(h, arr, len(candidates), int(reps), chosen, C.byref(n)))
    return {l: chosen[l].as_dict() for l in range(cap) if chosen[l].tile_cap > 0}, n.value


def lib():
    """Load libheterogpc.so (built in-tree); raise if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libheterogpc.so not built (%s); run __graft_entry__.build()" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGS)


def _check(status):
    if status != 0:
        msg = lib().hpc_last_error_string()
        raise HpcError(status, msg.decode() if msg else "")


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


# ---- independence statistics (CPU::calcPValue / pValL1 / pValLN, cpuInd.hpp:3-10)
def calcPValue(r, n):
    return lib().hpc_calc_pvalue(float(r), int(n))


def pValL1(x1, x2, x3, n):
    return lib().hpc_pval_l1(float(x1), float(x2), float(x3), int(n))


def pValLN(M, n):
    M = np.ascontiguousarray(M, dtype=np.float64)
    return lib().hpc_pval_ln(_ptr(M), int(M.shape[0]), int(n))


def z_crit(alpha):
    return lib().hpc_z_crit(float(alpha))


# ---- synthetic data
def sem_generate(p, n, graph=GRAPH_ER, degree=2.0, pa_parents=2, w_lo=0.1, w_hi=1.0, seed=1, dtype=np.float64,
                 want_dag=False):
    """Seeded linear-Gaussian SEM; returns X with shape (p, n) (each variable's samples
    contiguous, i.e. the column-major n x p layout of the C ABI) and optionally the DAG."""
    prm = SemParams(p, n, graph, degree, pa_parents, w_lo, w_hi, seed)
    X64 = np.empty((p, n), np.float64) if dtype == np.float64 else None
    X32 = np.empty((p, n), np.float32) if dtype == np.float32 else None
    dag = np.empty((p, p), np.uint8) if want_dag else None
    _check(lib().hpc_sem_generate(C.byref(prm), _ptr(X64) if X64 is not None else None,
                                  _ptr(X32) if X32 is not None else None,
                                  _ptr(dag) if dag is not None else None, None))
    X = X64 if X64 is not None else X32
    return (X, dag) if want_dag else X


RECORD_DTYPE = np.dtype([("i", np.int32), ("j", np.int32), ("level", np.int32), ("pad", np.int32),
                         ("pmax", np.float64), ("ids", np.int32, (HPC_MAX_LEVEL,))])


def record_chunks(h, idx=0, chunk=1 << 22):
    """Separation-set records of instance idx as numpy structured arrays (RECORD_DTYPE),
    chunk by chunk (hpc_batch_get_sepset_records_from)."""
    n = C.c_int64(0)
    _check(lib().hpc_batch_get_sepset_records_from(h, idx, 0, None, 0, C.byref(n)))
    total = n.value
    buf = (SepsetRecord * max(1, min(chunk, total)))()
    first = 0
    while first < total:
        k = min(chunk, total - first)
        _check(lib().hpc_batch_get_sepset_records_from(h, idx, first, buf, k, C.byref(n)))
        yield np.frombuffer(buf, dtype=RECORD_DTYPE, count=k).copy()
        first += k


class SkeletonCalculator:
    """One skeleton problem on one GPU (src/independence/skeleton.hpp:10-73).

    alpha: edges are removed iff p >= alpha; max_level: highest level (-1 = until no
    edge has enough neighbours); precision: PREC_FP64 (plain path), PREC_MIXED or
    PREC_MIXED_TC."""

    def __init__(self, p, n_obs, alpha=0.05, max_level=4, precision=PREC_MIXED, device=0, retest_margin=1e-3,
                 ref_compat_sd=False, verbose=False):
        self.p, self.n = int(p), int(n_obs)
        o = Opts()
        lib().hpc_opts_default(C.byref(o))
        o.device, o.alpha, o.max_level, o.precision = device, alpha, max_level, precision
        o.retest_margin, o.ref_compat_sd, o.verbose = retest_margin, int(ref_compat_sd), int(verbose)
        self.opts = o
        h = C.c_void_p()
        _check(lib().hpc_ctx_create(C.byref(h), self.p, self.n, C.byref(o)))
        self._h = h
        self.level_stats = []

    def close(self):
        if getattr(self, "_h", None):
            lib().hpc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    # add_observations (skeleton.cpp:53-58); X shape (p, n), FP64 or FP32
    def add_observations(self, X):
        X = np.asarray(X)
        assert X.shape == (self.p, self.n), X.shape
        if X.dtype == np.float32:
            X = np.ascontiguousarray(X)
            _check(lib().hpc_correlation_f32(self._h, _ptr(X)))
        else:
            X = np.ascontiguousarray(X, dtype=np.float64)
            _check(lib().hpc_correlation_f64(self._h, _ptr(X)))
        self.level_stats = []

    # add_correlation_matrix (skeleton.cpp:60-65)
    def add_correlation_matrix(self, Cm):
        Cm = np.ascontiguousarray(Cm, dtype=np.float64)
        assert Cm.shape == (self.p, self.p)
        _check(lib().hpc_load_correlation(self._h, _ptr(Cm)))
        self.level_stats = []

    def reset(self):
        _check(lib().hpc_ctx_reset(self._h))
        self.level_stats = []

    def calc_level(self, level):
        st = LevelStats()
        _check(lib().hpc_run_level(self._h, int(level), C.byref(st)))
        self.level_stats.append(st.as_dict())
        return st.as_dict()

    def run(self):
        cap = HPC_MAX_LEVEL + 1
        arr = (LevelStats * cap)()
        ran = C.c_int(0)
        _check(lib().hpc_run_skeleton(self._h, arr, cap, C.byref(ran)))
        self.level_stats.extend(arr[i].as_dict() for i in range(ran.value))
        return self.level_stats

    def run_async(self):
        """Queue a whole skeleton (from level 0) on the context's stream and return;
        wait() collects it (hpc_run_skeleton_async / hpc_wait)."""
        _check(lib().hpc_run_skeleton_async(self._h))

    def wait(self):
        cap = HPC_MAX_LEVEL + 1
        arr = (LevelStats * cap)()
        ran = C.c_int(0)
        _check(lib().hpc_wait(self._h, arr, cap, C.byref(ran)))
        self.level_stats = [arr[i].as_dict() for i in range(ran.value)]
        return self.level_stats

    def set_stream(self, stream_handle):
        """Run on a caller-owned cudaStream_t (an int handle, e.g. torch's cuda_stream)."""
        _check(lib().hpc_ctx_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def set_graphs(self, enable):
        _check(lib().hpc_ctx_set_graphs(self._h, int(bool(enable))))

    def set_barrier(self, wait_ns, extra_arrivals):
        """Test hook (hpc_debug_set_barrier): grid-barrier wait bound and added arrivals."""
        _check(lib().hpc_debug_set_barrier(self._h, int(wait_ns), int(extra_arrivals)))

    def set_tune(self, policy):
        """Force a tile policy ({"tile_cap", "tiles_per_lane", "edge_lanes"}) on every level; None = the table."""
        _set_tune(self._h, policy)

    def autotune(self, candidates=None, reps=1):
        """Time every candidate tile policy on this context's skeleton and store the fastest per level."""
        return _autotune(self._h, candidates, reps)

    def timings(self):
        t = Timings()
        _check(lib().hpc_get_timings(self._h, C.byref(t)))
        return t.as_dict()

    def add_observations_device(self, ptr, dtype):
        """Observations already in device memory (pointer to a column-major n x p array)."""
        fn = lib().hpc_correlation_device_f32 if dtype == np.float32 else lib().hpc_correlation_device_f64
        _check(fn(self._h, C.c_void_p(ptr)))
        self.level_stats = []

    def add_correlation_matrix_device(self, ptr):
        _check(lib().hpc_load_correlation_device(self._h, C.c_void_p(ptr)))
        self.level_stats = []

    def add_observations_ptr(self, ptr, dtype):
        """Observations in host memory at ptr (e.g. pinned), column-major n x p."""
        fn = lib().hpc_correlation_f32 if dtype == np.float32 else lib().hpc_correlation_f64
        _check(fn(self._h, C.c_void_p(ptr)))
        self.level_stats = []

    def add_correlation_matrix_ptr(self, ptr):
        """Host pointer (e.g. pinned memory) to a row-major p x p FP64 matrix."""
        _check(lib().hpc_load_correlation(self._h, C.c_void_p(ptr)))
        self.level_stats = []

    def adjacency_into(self, ptr):
        """Copy the p x p uint8 adjacency into caller memory at ptr."""
        _check(lib().hpc_get_adjacency(self._h, C.c_void_p(ptr)))

    def correlation(self):
        out = np.empty((self.p, self.p), np.float64)
        _check(lib().hpc_get_correlation(self._h, _ptr(out)))
        return out

    def correlation_f32(self):
        out = np.empty((self.p, self.p), np.float32)
        _check(lib().hpc_get_correlation_f32(self._h, _ptr(out)))
        return out

    def adjacency(self):
        out = np.empty((self.p, self.p), np.uint8)
        _check(lib().hpc_get_adjacency(self._h, _ptr(out)))
        return out

    def edge_count(self):
        e = C.c_int64(0)
        _check(lib().hpc_edge_count(self._h, C.byref(e)))
        return e.value

    def sepsets(self, max_cond):
        out = np.empty((self.p, self.p, max_cond), np.int32)
        _check(lib().hpc_get_sepsets(self._h, _ptr(out), int(max_cond)))
        return out

    def sepset_records(self):
        n = C.c_int64(0)
        _check(lib().hpc_get_sepset_records(self._h, None, 0, C.byref(n)))
        recs = (SepsetRecord * max(1, n.value))()
        _check(lib().hpc_get_sepset_records(self._h, recs, n.value, C.byref(n)))
        return [(r.i, r.j, r.level, tuple(r.ids[:r.level]), r.pmax) for r in recs[:n.value]]


def record_buffer(n):
    """A ctypes array of n hpc_sepset_record (for the *_into record calls)."""
    return (SepsetRecord * max(1, int(n)))()


class SkeletonBatch:
    """Many independent skeleton problems in one context: every level kernel runs
    once for all of them (hpc_batch_* in include/heterogpc.h)."""

    def __init__(self, ps, ns, alphas=None, max_level=4, precision=PREC_MIXED_TC, device=0, retest_margin=1e-3,
                 verbose=False):
        self.ps = np.ascontiguousarray(ps, dtype=np.int64)
        self.ns = np.ascontiguousarray(ns, dtype=np.int64)
        self.count = len(self.ps)
        o = Opts()
        lib().hpc_opts_default(C.byref(o))
        o.device, o.max_level, o.precision, o.retest_margin, o.verbose = device, max_level, precision, \
            retest_margin, int(verbose)
        self.max_level = int(max_level)
        self.alphas = None if alphas is None else np.ascontiguousarray(alphas, dtype=np.float64)
        h = C.c_void_p()
        _check(lib().hpc_batch_create(C.byref(h), self.count, _ptr(self.ps), _ptr(self.ns),
                                      _ptr(self.alphas) if self.alphas is not None else None, C.byref(o)))
        self._h = h
        self.obs_off = np.empty(self.count + 1, np.int64)
        self.cor_off = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_offsets(self._h, _ptr(self.obs_off), _ptr(self.cor_off)))
        self.level_stats = []

    def close(self):
        if getattr(self, "_h", None):
            lib().hpc_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pack(self, Xs, dtype=np.float32):
        """Packed observations from per-instance arrays of shape (p_b, n_b)."""
        out = np.empty(int(self.obs_off[-1]), dtype)
        for b, X in enumerate(Xs):
            out[self.obs_off[b]:self.obs_off[b + 1]] = np.asarray(X, dtype).reshape(-1)
        return out

    def add_observations(self, packed):
        packed = np.ascontiguousarray(packed)
        fn = lib().hpc_correlation_f32 if packed.dtype == np.float32 else lib().hpc_correlation_f64
        _check(fn(self._h, _ptr(packed)))

    def add_observations_device(self, ptr, dtype):
        fn = lib().hpc_correlation_device_f32 if dtype == np.float32 else lib().hpc_correlation_device_f64
        _check(fn(self._h, C.c_void_p(ptr)))

    def add_observations_ptr(self, ptr, dtype):
        """Packed observations in host memory at ptr (e.g. pinned), copied inside the call."""
        fn = lib().hpc_correlation_f32 if dtype == np.float32 else lib().hpc_correlation_f64
        _check(fn(self._h, C.c_void_p(ptr)))

    def calc_level(self, level):
        """One level of every instance (hpc_run_level); summed statistics."""
        st = LevelStats()
        _check(lib().hpc_run_level(self._h, int(level), C.byref(st)))
        return st.as_dict()

    def add_correlation_matrices(self, mats):
        packed = np.empty(int(self.cor_off[-1]), np.float64)
        for b, M in enumerate(mats):
            packed[self.cor_off[b]:self.cor_off[b + 1]] = np.asarray(M, np.float64).reshape(-1)
        _check(lib().hpc_load_correlation(self._h, _ptr(packed)))

    def set_stream(self, stream_handle):
        _check(lib().hpc_ctx_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None))

    def set_graphs(self, enable):
        _check(lib().hpc_ctx_set_graphs(self._h, int(bool(enable))))

    def set_tune(self, policy):
        """Force a tile policy ({"tile_cap", "tiles_per_lane", "edge_lanes"}) on every level; None = the table."""
        _set_tune(self._h, policy)

    def autotune(self, candidates=None, reps=1):
        """Time every candidate tile policy on this context's skeleton and store the fastest per level."""
        return _autotune(self._h, candidates, reps)

    def reset(self):
        _check(lib().hpc_ctx_reset(self._h))

    def run(self):
        cap = HPC_MAX_LEVEL + 1
        arr = (LevelStats * cap)()
        ran = C.c_int(0)
        _check(lib().hpc_run_skeleton(self._h, arr, cap, C.byref(ran)))
        self.level_stats = [arr[i].as_dict() for i in range(ran.value)]
        return self.level_stats

    def timings(self):
        t = Timings()
        _check(lib().hpc_get_timings(self._h, C.byref(t)))
        return t.as_dict()

    def adjacency(self, idx):
        p = int(self.ps[idx])
        out = np.empty((p, p), np.uint8)
        _check(lib().hpc_batch_get_adjacency(self._h, idx, _ptr(out)))
        return out

    def edge_count(self, idx):
        e = C.c_int64(0)
        _check(lib().hpc_batch_edge_count(self._h, idx, C.byref(e)))
        return e.value

    def instance_levels(self, idx):
        cap = HPC_MAX_LEVEL + 1
        arr = (LevelStats * cap)()
        k = C.c_int(0)
        _check(lib().hpc_batch_level_stats(self._h, idx, arr, cap, C.byref(k)))
        return [arr[i].as_dict() for i in range(k.value)]

    def set_retest_queue(self, entries):
        """Test hook (hpc_debug_set_retest_queue): a re-test queue of `entries` entries."""
        _check(lib().hpc_debug_set_retest_queue(self._h, int(entries)))

    def set_order_active(self):
        """Test hook: whether the context still runs levels in the set order."""
        return bool(lib().hpc_debug_set_order_active(self._h))

    def run_async(self):
        """Queue the whole batch's skeleton and return (hpc_run_skeleton_async)."""
        _check(lib().hpc_run_skeleton_async(self._h))

    def wait(self):
        cap = HPC_MAX_LEVEL + 1
        arr = (LevelStats * cap)()
        ran = C.c_int(0)
        _check(lib().hpc_wait(self._h, arr, cap, C.byref(ran)))
        self.level_stats = [arr[i].as_dict() for i in range(ran.value)]
        return self.level_stats

    def adjacency_words(self):
        """Word offsets (count + 1) of every instance's bitmask in adjacency_bits()."""
        off = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_adjacency_words(self._h, _ptr(off)))
        return off

    def adjacency_bits_into(self, ptr, words):
        """Every instance's adjacency bitmask into caller memory (uint32 words at ptr)."""
        _check(lib().hpc_batch_get_adjacency_bits(self._h, C.c_void_p(ptr), int(words)))

    def adjacency_bits(self):
        off = self.adjacency_words()
        out = np.empty(int(off[-1]), np.uint32)
        self.adjacency_bits_into(out.ctypes.data, out.size)
        return out, off

    def packed_words(self):
        """Word offsets (count + 1) of every instance's packed records."""
        w = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_get_records_packed(self._h, None, 0, _ptr(w)))
        return w

    def records_packed_into(self, ptr, cap_words):
        """Every instance's records in the packed form into caller memory at ptr (int32
        words); returns the instances' word offsets."""
        w = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_get_records_packed(self._h, C.c_void_p(ptr), int(cap_words), _ptr(w)))
        return w

    def records_packed(self):
        """{instance: [(i, j, level, ids, pmax), ...]} decoded from the packed copy."""
        w = self.packed_words()
        buf = np.empty(max(1, int(w[-1])), np.int32)
        w = self.records_packed_into(buf.ctypes.data, buf.size)
        out = {}
        for b in range(self.count):
            recs, q = [], int(w[b])
            while q < int(w[b + 1]):
                i, j, lev = int(buf[q]), int(buf[q + 1]), int(buf[q + 2])
                pmax = float(buf[q + 4:q + 6].view(np.float64)[0])
                recs.append((i, j, lev, tuple(int(x) for x in buf[q + 6:q + 6 + lev]), pmax))
                q += 6 + 2 * ((lev + 1) // 2)
            out[b] = recs
        return out

    def record_prefix(self):
        """Exclusive prefix (count + 1) of the instances' separation-set record counts."""
        pre = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_get_all_sepset_records(self._h, None, 0, _ptr(pre)))
        return pre

    def record_stride_bytes(self):
        """Device bytes of one packed record (head + one id slot per level up to max_level)."""
        ids = HPC_MAX_LEVEL if self.max_level < 0 else min(max(self.max_level, 1), HPC_MAX_LEVEL)
        return 4 * (6 + ((ids + 1) & ~1))

    def all_sepset_records_into(self, recs, cap):
        """Every instance's records into a ctypes SepsetRecord array; returns the prefix."""
        pre = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_get_all_sepset_records(self._h, recs, int(cap), _ptr(pre)))
        return pre

    def all_sepset_records(self):
        """{instance: [(i, j, level, ids, pmax), ...]} of every instance in one copy."""
        pre = np.empty(self.count + 1, np.int64)
        _check(lib().hpc_batch_get_all_sepset_records(self._h, None, 0, _ptr(pre)))
        total = int(pre[-1])
        recs = (SepsetRecord * max(1, total))()
        pre = self.all_sepset_records_into(recs, total)
        out = {}
        for b in range(self.count):
            out[b] = [(r.i, r.j, r.level, tuple(r.ids[:r.level]), r.pmax) for r in recs[int(pre[b]):int(pre[b + 1])]]
        return out

    def sepset_records(self, idx):
        n = C.c_int64(0)
        _check(lib().hpc_batch_get_sepset_records(self._h, idx, None, 0, C.byref(n)))
        recs = (SepsetRecord * max(1, n.value))()
        _check(lib().hpc_batch_get_sepset_records(self._h, idx, recs, n.value, C.byref(n)))
        return [(r.i, r.j, r.level, tuple(r.ids[:r.level]), r.pmax) for r in recs[:n.value]]


class SkeletonServer:
    """Continuous-batching skeleton server (hpc_server_* in include/heterogpc.h)."""

    def __init__(self, precision=PREC_MIXED_TC, max_level=4, budget_bytes=150 * 10**9, max_batch=256,
                 max_inflight=32, device=0):
        o = ServerOpts()
        lib().hpc_server_opts_default(C.byref(o))
        o.device, o.precision, o.max_level = device, precision, max_level
        o.budget_bytes, o.max_batch, o.max_inflight = budget_bytes, max_batch, max_inflight
        h = C.c_void_p()
        _check(lib().hpc_server_create(C.byref(h), C.byref(o)))
        self._h = h
        self._keep = {}

    def submit(self, X, alpha, want_adjacency=False):
        """X: float32 array (p, n), kept alive until the request completes."""
        X = np.ascontiguousarray(X, np.float32)
        p, n = X.shape
        adj = np.empty((p, p), np.uint8) if want_adjacency else None
        rid = C.c_int64(0)
        _check(lib().hpc_server_submit(self._h, _ptr(X), p, n, float(alpha), _ptr(adj) if adj is not None else None,
                                       C.byref(rid)))
        self._keep[rid.value] = (X, adj)
        return rid.value

    def poll(self, cap=1024):
        arr = (Served * cap)()
        k = C.c_int(0)
        _check(lib().hpc_server_poll(self._h, arr, cap, C.byref(k)))
        out = []
        for r in arr[:k.value]:
            X, adj = self._keep.pop(r.id)
            out.append(dict(id=r.id, status=r.status, levels=r.levels, edges=r.edges, queue_ms=r.queue_ms,
                            run_ms=r.run_ms, latency_ms=r.latency_ms, batch_size=r.batch_size, joined=r.joined,
                            adjacency=adj))
        return out

    def drain(self):
        _check(lib().hpc_server_drain(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().hpc_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
