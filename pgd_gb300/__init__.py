"""pgd_gb300 -- GB300-native exact graphlet decomposition (PGD's hot path).

Python access to the native library `lib/libpgd_gb300.so` (C ABI declared in
include/pgd_gb300.h).  All counting runs in the library's CUDA kernels; this
module only moves arrays across the ABI.  If the library has not been built,
importing works but every call raises: there is no Python or CPU fallback.

    import pgd_gb300 as pgd
    ctx = pgd.Context()
    g = ctx.graph_from_edges(src, dst, dedup=True)
    g.preprocess("deg"); g.sort_edges("kcore")
    res = g.decompose(micro=True)          # res.totals: the 17 global counts
    src1, dst1, cols = g.micro()           # per-edge rows in E_ordered order
"""
import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libpgd_gb300.so")
CLI_PATH = os.path.join(PKG, "bin", "pgd")

NSUMS, NTOTALS, NMICRO = 15, 17, 8
MICRO = 1
EDGES_DEDUP = 1

# field order of graphlet_core.h:310-329
TOTAL_NAMES = [
    "total_2_1edge", "total_2_indep", "total_3_tris", "total_2_star", "total_3_1edge",
    "total_3_indep", "total_4_clique", "total_4_chordcycle", "total_4_tailed_tris",
    "total_4_cycle", "total_3_star", "total_4_path", "total_4_2edge", "total_4_1edge",
    "total_4_2star", "total_4_tri", "total_4_indep",
]
MICRO_NAMES = ["triangle", "2-star", "4-clique", "4-chordal-cycle", "4-tailed-triangle",
               "4-cycle", "3-star", "4-path"]
STATUS = {0: "PGD_OK", 1: "PGD_EINVAL", 2: "PGD_ENOMEM", 3: "PGD_ETIMEOUT", 4: "PGD_ECUDA",
          5: "PGD_EIO", 6: "PGD_EUNSUPPORTED"}

# every symbol include/pgd_gb300.h and include/pgd_gen.h declare
EXPORTS = [
    "pgd_status_string", "pgd_context_create", "pgd_context_destroy", "pgd_last_error",
    "pgd_context_resident_bytes", "pgd_context_kernel_launches", "pgd_graph_from_file", "pgd_graph_from_edges",
    "pgd_graph_from_csr", "pgd_graph_destroy", "pgd_graph_info", "pgd_graph_resident_bytes",
    "pgd_preprocess", "pgd_compute_cores", "pgd_get_kcore", "pgd_assortativity",
    "pgd_sort_edges", "pgd_decompose", "pgd_get_micro", "pgd_get_edges", "pgd_close_counts",
    "pgd_decompose_batch", "pgd_gen_u01", "pgd_gen_rmat", "pgd_gen_er", "pgd_gen_ba",
    "pgd_gen_rgg3d", "pgd_decompose_csr_noalloc", "pgd_noalloc_scratch_bytes", "pgd_set_thresholds",
    "pgd_get_thresholds", "pgd_autotune", "pgd_decompose_pairs_batch", "pgd_server_create", "pgd_server_submit",
    "pgd_server_poll", "pgd_server_wait", "pgd_server_stats", "pgd_server_destroy", "pgd_sort_edges_sample",
    "pgd_graph_order_length", "pgd_set_tensor_min_degree", "pgd_get_tensor_min_degree",
]


class PGDError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        super().__init__("%s: %s" % (STATUS.get(status, status), msg))


class pgd_opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("reserved0", ctypes.c_int),
                ("hbm_budget", ctypes.c_uint64), ("stream", ctypes.c_void_p)]


class pgd_counts(ctypes.Structure):
    _fields_ = [("totals", ctypes.c_uint64 * NTOTALS), ("sums", ctypes.c_uint64 * NSUMS),
                ("n", ctypes.c_int64), ("m", ctypes.c_int64), ("kernel_ms", ctypes.c_float),
                ("hub_ms", ctypes.c_float), ("tri_ms", ctypes.c_float), ("reserved", ctypes.c_float)]


class pgd_server_opts(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("workers", ctypes.c_int), ("max_batch", ctypes.c_int),
                ("max_wait_ms", ctypes.c_int), ("hbm_budget", ctypes.c_uint64)]


class pgd_server_stat(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("rejected", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("inflight_bytes", ctypes.c_uint64), ("peak_bytes", ctypes.c_uint64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("graphs_per_s", ctypes.c_double), ("queue_p50_ms", ctypes.c_double),
                ("queue_p99_ms", ctypes.c_double), ("service_p50_ms", ctypes.c_double),
                ("service_p99_ms", ctypes.c_double), ("skipped_ahead", ctypes.c_uint64)]


class pgd_info(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("max_degree", ctypes.c_int32),
                ("avg_degree", ctypes.c_int32), ("self_loops", ctypes.c_int64),
                ("duplicates", ctypes.c_int64)]


_P = ctypes.c_void_p
_PP = ctypes.POINTER(ctypes.c_void_p)
_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_U64 = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")

_lib = None


def lib():
    """The loaded native library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("pgd_gb300 native library missing at %s: run "
                               "`python -m pgd_gb300.build` (there is no CPU fallback)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        sig = {
            "pgd_status_string": (ctypes.c_char_p, [ctypes.c_int]),
            "pgd_context_create": (ctypes.c_int, [ctypes.POINTER(pgd_opts), _PP]),
            "pgd_context_destroy": (ctypes.c_int, [_P]),
            "pgd_last_error": (ctypes.c_char_p, [_P]),
            "pgd_context_resident_bytes": (ctypes.c_uint64, [_P]),
            "pgd_context_kernel_launches": (ctypes.c_uint64, [_P]),
            "pgd_graph_from_file": (ctypes.c_int, [_P, ctypes.c_char_p, _PP]),
            "pgd_graph_from_edges": (ctypes.c_int, [_P, _P, _P, ctypes.c_int64, ctypes.c_int64,
                                                    ctypes.c_uint32, _PP]),
            "pgd_graph_from_csr": (ctypes.c_int, [_P, _I64, _I32, ctypes.c_int64, _PP]),
            "pgd_graph_destroy": (ctypes.c_int, [_P]),
            "pgd_graph_info": (ctypes.c_int, [_P, ctypes.POINTER(pgd_info)]),
            "pgd_graph_resident_bytes": (ctypes.c_uint64, [_P]),
            "pgd_preprocess": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int]),
            "pgd_compute_cores": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32)]),
            "pgd_get_kcore": (ctypes.c_int, [_P, _I32]),
            "pgd_assortativity": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double)]),
            "pgd_sort_edges": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int]),
            "pgd_sort_edges_sample": (ctypes.c_int, [_P, ctypes.c_char_p, ctypes.c_int, _I64, ctypes.c_int64]),
            "pgd_graph_order_length": (ctypes.c_int64, [_P]),
            "pgd_decompose": (ctypes.c_int, [_P, ctypes.c_uint32, ctypes.POINTER(pgd_counts)]),
            "pgd_get_micro": (ctypes.c_int, [_P, _P, _P, _P]),
            "pgd_get_edges": (ctypes.c_int, [_P, _P, _P, _P]),
            "pgd_close_counts": (None, [_U64, ctypes.c_int64, ctypes.c_int64, _U64]),
            "pgd_decompose_batch": (ctypes.c_int, [_P, _PP, ctypes.c_int, ctypes.c_uint32,
                                                   ctypes.POINTER(pgd_counts)]),
            "pgd_gen_u01": (ctypes.c_double, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]),
            "pgd_gen_rmat": (None, [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_uint64, _I32, _I32]),
            "pgd_gen_er": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_double, ctypes.c_uint64, _I32,
                                            _I32, ctypes.c_int64]),
            "pgd_gen_ba": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_int, ctypes.c_uint64, _I32, _I32,
                                            ctypes.c_int64]),
            "pgd_gen_rgg3d": (ctypes.c_int64, [ctypes.c_int64, ctypes.c_double, ctypes.c_uint64, _I32,
                                               _I32, ctypes.c_int64]),
            "pgd_decompose_csr_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int,
                                                         _P, ctypes.POINTER(pgd_counts), ctypes.c_char_p,
                                                         ctypes.c_size_t]),
            "pgd_noalloc_scratch_bytes": (ctypes.c_uint64, []),
            "pgd_set_thresholds": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            "pgd_set_tensor_min_degree": (ctypes.c_int, [_P, ctypes.c_int]),
            "pgd_get_tensor_min_degree": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
            "pgd_decompose_pairs_batch": (ctypes.c_int, [_P, ctypes.c_int, _I64, _I32, _I32, _P,
                                                         ctypes.POINTER(pgd_counts)]),
            "pgd_server_create": (ctypes.c_int, [ctypes.POINTER(pgd_server_opts), _PP]),
            "pgd_server_submit": (ctypes.c_int, [_P, _I32, _I32, ctypes.c_int64, ctypes.c_int64,
                                                 ctypes.POINTER(ctypes.c_uint64)]),
            "pgd_server_poll": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.POINTER(pgd_counts),
                                               ctypes.POINTER(ctypes.c_int)]),
            "pgd_server_wait": (ctypes.c_int, [_P, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(pgd_counts)]),
            "pgd_server_stats": (ctypes.c_int, [_P, ctypes.POINTER(pgd_server_stat)]),
            "pgd_server_destroy": (ctypes.c_int, [_P]),
            "pgd_get_thresholds": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                                  ctypes.POINTER(ctypes.c_int)]),
            "pgd_autotune": (ctypes.c_int, [_P, _PP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int),
                                            ctypes.POINTER(ctypes.c_float)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def close_counts(sums, n, m):
    out = np.zeros(NTOTALS, np.uint64)
    lib().pgd_close_counts(np.ascontiguousarray(sums, np.uint64), n, m, out)
    return out


class Counts:
    """Result of one decomposition."""

    def __init__(self, c):
        self.totals = np.array(list(c.totals), dtype=np.uint64)
        self.sums = np.array(list(c.sums), dtype=np.uint64)
        self.n, self.m, self.kernel_ms = c.n, c.m, c.kernel_ms
        self.hub_ms, self.tri_ms = c.hub_ms, c.tri_ms

    def as_dict(self):
        return {k: int(v) for k, v in zip(TOTAL_NAMES, self.totals)}


class Context:
    """A CUDA device + stream + HBM budget (pgd_context_create)."""

    def __init__(self, device=0, hbm_budget=0, stream=None):
        o = pgd_opts(device, 0, hbm_budget, stream)
        h = ctypes.c_void_p()
        st = lib().pgd_context_create(ctypes.byref(o), ctypes.byref(h))
        if st:
            raise PGDError(st, "pgd_context_create failed (is a CUDA device visible?)")
        self.h = h

    def _check(self, st, what):
        if st:
            msg = lib().pgd_last_error(self.h) or b""
            raise PGDError(st, "%s: %s" % (what, msg.decode()))

    def close(self):
        if getattr(self, "h", None):
            lib().pgd_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def resident_bytes(self):
        return lib().pgd_context_resident_bytes(self.h)

    @property
    def kernel_launches(self):
        return lib().pgd_context_kernel_launches(self.h)

    def graph_from_edges(self, src, dst, n_min=0, dedup=True):
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        h = ctypes.c_void_p()
        self._check(lib().pgd_graph_from_edges(self.h, _ptr(src), _ptr(dst), len(src), n_min,
                                               EDGES_DEDUP if dedup else 0, ctypes.byref(h)),
                    "pgd_graph_from_edges")
        return Graph(self, h)

    def graph_from_csr(self, off, adj):
        off = np.ascontiguousarray(off, np.int64)
        adj = np.ascontiguousarray(adj, np.int32)
        if len(adj) == 0:
            adj = np.zeros(1, np.int32)
        h = ctypes.c_void_p()
        self._check(lib().pgd_graph_from_csr(self.h, off, adj, len(off) - 1, ctypes.byref(h)),
                    "pgd_graph_from_csr")
        return Graph(self, h)

    def graph_from_file(self, path):
        h = ctypes.c_void_p()
        self._check(lib().pgd_graph_from_file(self.h, str(path).encode(), ctypes.byref(h)),
                    "pgd_graph_from_file")
        return Graph(self, h)

    def set_thresholds(self, anchor_hub, cache_hub, dense_max=2048):
        self._check(lib().pgd_set_thresholds(self.h, anchor_hub, cache_hub, dense_max), "pgd_set_thresholds")

    def thresholds(self):
        a, c, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._check(lib().pgd_get_thresholds(self.h, ctypes.byref(a), ctypes.byref(c), ctypes.byref(d)),
                    "pgd_get_thresholds")
        return a.value, c.value, d.value

    def set_tensor_min_degree(self, d):
        """Dense batch graphs: runs with q of degree in [d, 1088] count k4 on the tensor cores (0: never)."""
        self._check(lib().pgd_set_tensor_min_degree(self.h, d), "pgd_set_tensor_min_degree")

    def tensor_min_degree(self):
        d = ctypes.c_int()
        self._check(lib().pgd_get_tensor_min_degree(self.h, ctypes.byref(d)), "pgd_get_tensor_min_degree")
        return d.value

    def autotune(self, graphs, reps=1):
        """Pick the fastest thresholds for these graphs; returns (anchor_hub, cache_hub, dense_max, ms)."""
        arr = (ctypes.c_void_p * len(graphs))(*[g.h.value for g in graphs])
        a, c, d, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        self._check(lib().pgd_autotune(self.h, arr, len(graphs), reps, ctypes.byref(a), ctypes.byref(c),
                                       ctypes.byref(d), ctypes.byref(ms)), "pgd_autotune")
        return a.value, c.value, d.value, ms.value

    def decompose_pairs_batch(self, graphs, n_min=None):
        """graphs: list of (src, dst) local-id pair arrays.  One device build and one pass for all."""
        off, src, dst = concat_pairs(graphs)
        return self.decompose_pairs_batch_flat(off, src, dst, n_min)

    def decompose_pairs_batch_flat(self, pair_off, src, dst, n_min=None):
        """The batch as pgd_decompose_pairs_batch takes it: graph i's pairs are
        src/dst[pair_off[i]:pair_off[i + 1]] (int32 local ids, int64 offsets)."""
        k = len(pair_off) - 1
        off = np.ascontiguousarray(pair_off, np.int64)
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        if len(src) == 0:
            src = dst = np.zeros(1, np.int32)
        nm = None if n_min is None else np.ascontiguousarray(n_min, np.int64)
        out = (pgd_counts * k)()
        self._check(lib().pgd_decompose_pairs_batch(self.h, k, off, src, dst, _ptr(nm), out),
                    "pgd_decompose_pairs_batch")
        return [Counts(c) for c in out]

    def decompose_batch(self, graphs, micro=False):
        arr = (ctypes.c_void_p * len(graphs))(*[g.h.value for g in graphs])
        out = (pgd_counts * len(graphs))()
        self._check(lib().pgd_decompose_batch(self.h, arr, len(graphs), MICRO if micro else 0, out),
                    "pgd_decompose_batch")
        return [Counts(c) for c in out]


class Graph:
    """A graph resident on the device (pgd_graph)."""

    def __init__(self, ctx, h):
        self.ctx, self.h = ctx, h

    def destroy(self):
        if getattr(self, "h", None):
            lib().pgd_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            if self.ctx.h is not None:
                self.destroy()
        except Exception:
            pass

    def info(self):
        i = pgd_info()
        self.ctx._check(lib().pgd_graph_info(self.h, ctypes.byref(i)), "pgd_graph_info")
        return i

    @property
    def n(self):
        return self.info().n

    @property
    def m(self):
        return self.info().m

    @property
    def resident_bytes(self):
        return lib().pgd_graph_resident_bytes(self.h)

    def preprocess(self, neigh="deg", s2l=False):
        self.ctx._check(lib().pgd_preprocess(self.h, neigh.encode(), int(s2l)), "pgd_preprocess")
        return self

    def compute_cores(self):
        k = ctypes.c_int32()
        self.ctx._check(lib().pgd_compute_cores(self.h, ctypes.byref(k)), "pgd_compute_cores")
        return k.value

    def kcore(self):
        out = np.zeros(self.n + 1, np.int32)
        self.ctx._check(lib().pgd_get_kcore(self.h, out), "pgd_get_kcore")
        return out

    def assortativity(self):
        r = ctypes.c_double()
        self.ctx._check(lib().pgd_assortativity(self.h, ctypes.byref(r)), "pgd_assortativity")
        return r.value

    def sort_edges(self, order="deg", s2l=False):
        self.ctx._check(lib().pgd_sort_edges(self.h, order.encode(), int(s2l)), "pgd_sort_edges")
        return self

    def sort_edges_sample(self, edge_ids, order="deg", s2l=False):
        """Order (and later decompose) only the given edge ids (E_s)."""
        ids = np.ascontiguousarray(edge_ids, dtype=np.int64)
        self.ctx._check(lib().pgd_sort_edges_sample(self.h, order.encode(), int(s2l), ids, len(ids)),
                        "pgd_sort_edges_sample")
        return self

    @property
    def order_length(self):
        """Length of E_ordered: m, or the sample size."""
        return int(lib().pgd_graph_order_length(self.h))

    def decompose(self, micro=False):
        c = pgd_counts()
        self.ctx._check(lib().pgd_decompose(self.h, MICRO if micro else 0, ctypes.byref(c)),
                        "pgd_decompose")
        return Counts(c)

    def micro(self, ids=True, out=None):
        m = self.order_length
        cols = out if out is not None else np.empty((max(m, 1), NMICRO), np.uint64)
        src = np.empty(max(m, 1), np.int64) if ids else None
        dst = np.empty(max(m, 1), np.int64) if ids else None
        self.ctx._check(lib().pgd_get_micro(self.h, _ptr(src), _ptr(dst), _ptr(cols)), "pgd_get_micro")
        if ids:
            return src[:m], dst[:m], cols[:m]
        return cols[:m]

    def edges(self, with_order=True):
        m = self.m
        ev = np.empty(max(m, 1), np.int64)
        eu = np.empty(max(m, 1), np.int64)
        order = np.empty(max(m, 1), np.int32) if with_order else None
        self.ctx._check(lib().pgd_get_edges(self.h, _ptr(ev), _ptr(eu), _ptr(order)), "pgd_get_edges")
        return ev[:m], eu[:m], (order[:self.order_length] if with_order else None)


class Server:
    """Continuous-batching request server (pgd_server_*)."""

    def __init__(self, device=0, workers=2, max_batch=4096, hbm_budget=0, max_wait_ms=0):
        o = pgd_server_opts(device, workers, max_batch, max_wait_ms, hbm_budget)
        h = ctypes.c_void_p()
        st = lib().pgd_server_create(ctypes.byref(o), ctypes.byref(h))
        if st:
            raise PGDError(st, "pgd_server_create failed")
        self.h = h

    def submit(self, src, dst, n_min=0):
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        if len(src) == 0:
            src = dst = np.zeros(1, np.int32)
            k = 0
        else:
            k = len(src)
        t = ctypes.c_uint64()
        st = lib().pgd_server_submit(self.h, src, dst, k, n_min, ctypes.byref(t))
        if st:
            raise PGDError(st, "pgd_server_submit failed")
        return t.value

    def poll(self, ticket):
        """None while running, else (status, Counts)."""
        c = pgd_counts()
        done = ctypes.c_int()
        st = lib().pgd_server_poll(self.h, ticket, ctypes.byref(c), ctypes.byref(done))
        return (st, Counts(c)) if done.value else None

    def wait(self, ticket, timeout_ms=60000):
        """(status, Counts); status PGD_ETIMEOUT (3) leaves the request running."""
        c = pgd_counts()
        st = lib().pgd_server_wait(self.h, ticket, timeout_ms, ctypes.byref(c))
        return st, Counts(c)

    def stats(self):
        s = pgd_server_stat()
        lib().pgd_server_stats(self.h, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in pgd_server_stat._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib().pgd_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# synthetic inputs (include/pgd_gen.h)

def rmat(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1):
    k = edge_factor << scale
    src = np.empty(k, np.int32)
    dst = np.empty(k, np.int32)
    lib().pgd_gen_rmat(scale, edge_factor, a, b, c, seed, src, dst)
    return src, dst


def concat_pairs(graphs):
    """(pair_off, src, dst) of a list of (src, dst) arrays, as the batch call takes them."""
    off = np.zeros(len(graphs) + 1, np.int64)
    for i, (s, _) in enumerate(graphs):
        off[i + 1] = off[i] + len(s)
    src = np.ascontiguousarray(np.concatenate([s for s, _ in graphs]) if graphs else np.zeros(0), np.int32)
    dst = np.ascontiguousarray(np.concatenate([d for _, d in graphs]) if graphs else np.zeros(0), np.int32)
    return off, src, dst


def erdos_renyi(n, p, seed=1):
    cap = max(1, int(n * (n - 1) // 2 * min(1.0, p * 1.2 + 0.01)) + 1024)
    while True:
        src = np.empty(cap, np.int32)
        dst = np.empty(cap, np.int32)
        k = lib().pgd_gen_er(n, p, seed, src, dst, cap)
        if k <= cap:
            return src[:k], dst[:k]
        cap = k


def barabasi_albert(n, m_attach, seed=1):
    cap = max(1, n * m_attach + m_attach * m_attach + 16)
    src = np.empty(cap, np.int32)
    dst = np.empty(cap, np.int32)
    k = lib().pgd_gen_ba(n, m_attach, seed, src, dst, cap)
    return src[:k], dst[:k]


def rgg3d(n, radius, seed=1, cap=None):
    if cap is None:
        cap = int(n * (4.0 / 3.0 * np.pi * radius ** 3) * n / 2 * 1.3) + 1024
    while True:
        src = np.empty(cap, np.int32)
        dst = np.empty(cap, np.int32)
        k = lib().pgd_gen_rgg3d(n, radius, seed, src, dst, cap)
        if k <= cap:
            return src[:k], dst[:k]
        cap = k
