"""ctypes access to the test oracle (oracle/_build/libpgd_oracle.so) and, when it
was built here, the reference compiled from source (oracle/_ref/libpgd_ref.so).

Test infrastructure only: the product package never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "libpgd_oracle.so")
REF_SO = os.path.join(ORACLE_DIR, "_ref", "libpgd_ref.so")
REF_BIN = os.path.join(ORACLE_DIR, "_ref", "pgd")

# Field order of graphlet_core.h:310-329.
TOTAL_NAMES = [
    "total_2_1edge", "total_2_indep", "total_3_tris", "total_2_star", "total_3_1edge",
    "total_3_indep", "total_4_clique", "total_4_chordcycle", "total_4_tailed_tris",
    "total_4_cycle", "total_3_star", "total_4_path", "total_4_2edge", "total_4_1edge",
    "total_4_2star", "total_4_tri", "total_4_indep",
]
MICRO_NAMES = ["triangle", "2-star", "4-clique", "4-chordal-cycle", "4-tailed-triangle",
               "4-cycle", "3-star", "4-path"]

_P = ctypes.c_void_p
_I64P = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_I32P = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_U64P = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "oracle"], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = ctypes.CDLL(ORACLE_SO)
        L.po_read_file.restype = _P
        L.po_read_file.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.po_from_csr.restype = _P
        L.po_from_csr.argtypes = [ctypes.c_int64, _I64P, _I32P, ctypes.c_char_p]
        L.po_from_pairs.restype = _P
        L.po_from_pairs.argtypes = [ctypes.c_int64, _I32P, _I32P, ctypes.c_int64, ctypes.c_int,
                                    ctypes.c_char_p]
        L.po_free.argtypes = [_P]
        L.po_preprocess.argtypes = [_P, ctypes.c_char_p, ctypes.c_int]
        L.po_compute_cores.argtypes = [_P]
        L.po_assortativity.argtypes = [_P]
        L.po_assortativity.restype = ctypes.c_double
        L.po_sort_edges.argtypes = [_P, ctypes.c_char_p, ctypes.c_int]
        L.po_sort_edges_sample.argtypes = [_P, ctypes.c_char_p, ctypes.c_int, _I64P, ctypes.c_int64]
        L.po_n_ord.restype = ctypes.c_int64
        L.po_n_ord.argtypes = [_P]
        L.po_decompose.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.po_close.argtypes = [_U64P, ctypes.c_int64, ctypes.c_int64, _U64P]
        L.po_edge_sample.argtypes = [_P, ctypes.c_int64, _I64P, _I64P, _U64P, _U64P, _U64P, ctypes.c_int]
        L.po_decompose_sample.restype = ctypes.c_int64
        L.po_decompose_sample.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                                          ctypes.POINTER(ctypes.c_double)]
        for f in ("po_n", "po_m"):
            getattr(L, f).restype = ctypes.c_int64
            getattr(L, f).argtypes = [_P]
        for f in ("po_max_degree", "po_max_core"):
            getattr(L, f).restype = ctypes.c_int
            getattr(L, f).argtypes = [_P]
        L.po_get_csr.argtypes = [_P, _I64P, _I32P]
        L.po_get_edges.argtypes = [_P, _I64P, _I64P]
        L.po_get_order.argtypes = [_P, _I32P]
        L.po_get_kcore.argtypes = [_P, _I32P]
        L.po_get_sums.argtypes = [_P, _U64P]
        L.po_get_totals.argtypes = [_P, _U64P]
        L.po_get_micro.argtypes = [_P, _I64P, _I64P, _U64P]
        L.po_get_edge_tkc.argtypes = [_P, _U64P, _U64P, _U64P]
        L.po_gen_rmat.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                  ctypes.c_uint64, _I32P, _I32P]
        L.po_gen_rmat.restype = None
        L.po_micro_row.argtypes = [ctypes.c_longlong, ctypes.c_longlong, ctypes.c_uint64, ctypes.c_uint64,
                                   ctypes.c_uint64, _U64P]
        L.po_micro_row.restype = None
        _lib = L
    return _lib


class OracleGraph:
    """One graph in the oracle, run through the reference's pipeline."""

    def __init__(self, handle):
        if not handle:
            raise ValueError("oracle rejected the graph: " + self._err.value.decode())
        self.h = handle

    _err = ctypes.create_string_buffer(256)

    @classmethod
    def from_file(cls, path):
        return cls(lib().po_read_file(path.encode(), cls._err))

    @classmethod
    def from_csr(cls, off, adj):
        off = np.ascontiguousarray(off, np.int64)
        adj = np.ascontiguousarray(adj, np.int32)
        return cls(lib().po_from_csr(len(off) - 1, off, adj, cls._err))

    @classmethod
    def from_pairs(cls, src, dst, n_min=0, dedup=False):
        src = np.ascontiguousarray(src, np.int32)
        dst = np.ascontiguousarray(dst, np.int32)
        return cls(lib().po_from_pairs(len(src), src, dst, n_min, int(dedup), cls._err))

    def __del__(self):
        if getattr(self, "h", None):
            lib().po_free(self.h)
            self.h = None

    @property
    def n(self):
        return lib().po_n(self.h)

    @property
    def m(self):
        return lib().po_m(self.h)

    def run(self, neigh="deg", s2l_neigh=False, order="deg", s2l=False, micro=True, threads=0,
            cheap_side=False):
        L = lib()
        rc = L.po_preprocess(self.h, neigh.encode(), int(s2l_neigh))
        if rc:
            raise ValueError("preprocess failed: %d" % rc)
        L.po_compute_cores(self.h)
        rc = L.po_sort_edges(self.h, order.encode(), int(s2l))
        if rc:
            raise ValueError("sort_edges failed: %d" % rc)
        if L.po_decompose(self.h, int(micro), threads, int(cheap_side)):
            raise RuntimeError("decompose failed")
        return self

    def run_sample(self, ids, neigh="deg", order="deg", s2l=False, micro=True, threads=0):
        """preprocess, cores, sort_edges over the sampled edge ids, decompose"""
        L = lib()
        if L.po_preprocess(self.h, neigh.encode(), 0):
            raise ValueError("preprocess failed")
        L.po_compute_cores(self.h)
        ids = np.ascontiguousarray(ids, np.int64)
        if L.po_sort_edges_sample(self.h, order.encode(), int(s2l), ids, len(ids)):
            raise ValueError("sort_edges (sample) failed")
        if L.po_decompose(self.h, int(micro), threads, 0):
            raise RuntimeError("decompose failed")
        return self

    @property
    def n_ord(self):
        return lib().po_n_ord(self.h)

    def prepare(self, neigh="deg", s2l_neigh=False, order="deg", s2l=False):
        """preprocess + cores + sort_edges, no decomposition"""
        L = lib()
        if L.po_preprocess(self.h, neigh.encode(), int(s2l_neigh)):
            raise ValueError("preprocess failed")
        L.po_compute_cores(self.h)
        if L.po_sort_edges(self.h, order.encode(), int(s2l)):
            raise ValueError("sort_edges failed")
        return self

    def time_sample(self, stride, threads=0, cheap_side=False):
        """(edges, seconds) of the per-edge loop over every stride-th edge"""
        sec = ctypes.c_double()
        k = lib().po_decompose_sample(self.h, threads, int(cheap_side), stride, ctypes.byref(sec))
        return k, sec.value

    def edge_sample(self, vs, us, threads=0):
        """(t, k4, c4) of the edges (vs[i], us[i]) by the reference's marking procedure"""
        vs = np.ascontiguousarray(vs, np.int64)
        us = np.ascontiguousarray(us, np.int64)
        t, k, c = (np.zeros(max(1, len(vs)), np.uint64) for _ in range(3))
        if lib().po_edge_sample(self.h, len(vs), vs, us, t, k, c, threads):
            raise ValueError("vertex id out of range")
        return t[: len(vs)], k[: len(vs)], c[: len(vs)]

    def csr(self):
        off = np.zeros(self.n + 1, np.int64)
        adj = np.zeros(2 * self.m + 1, np.int32)
        lib().po_get_csr(self.h, off, adj)
        return off, adj[: off[-1]]

    def edges(self):
        ev = np.zeros(self.m + 1, np.int64)
        eu = np.zeros(self.m + 1, np.int64)
        lib().po_get_edges(self.h, ev, eu)
        return ev[: self.m], eu[: self.m]

    def order(self):
        k = self.n_ord
        o = np.zeros(k + 1, np.int32)
        lib().po_get_order(self.h, o)
        return o[:k]

    def kcore(self):
        k = np.zeros(self.n + 1, np.int32)
        lib().po_get_kcore(self.h, k)
        return k

    @property
    def max_core(self):
        return lib().po_max_core(self.h)

    def assortativity(self):
        return lib().po_assortativity(self.h)

    def sums(self):
        s = np.zeros(15, np.uint64)
        lib().po_get_sums(self.h, s)
        return s

    def totals(self):
        t = np.zeros(17, np.uint64)
        lib().po_get_totals(self.h, t)
        return t

    def micro(self):
        m = self.n_ord
        src = np.zeros(m + 1, np.int64)
        dst = np.zeros(m + 1, np.int64)
        cols = np.zeros((m + 1) * 8, np.uint64)
        lib().po_get_micro(self.h, src, dst, cols)
        return src[:m], dst[:m], cols[: 8 * m].reshape(m, 8)

    def edge_tkc(self):
        m = self.m
        t, k, c = (np.zeros(m + 1, np.uint64) for _ in range(3))
        lib().po_get_edge_tkc(self.h, t, k, c)
        return t[:m], k[:m], c[:m]


def rmat(scale, edge_factor=16, seed=1, a=0.57, b=0.19, c=0.19):
    """Seeded RMAT pairs from the oracle's own generator (same draws as the
    product's pgd_gen_rmat), for callers that must not load the product."""
    k = edge_factor << scale
    src = np.empty(k, np.int32)
    dst = np.empty(k, np.int32)
    lib().po_gen_rmat(scale, edge_factor, a, b, c, seed, src, dst)
    return src, dst


def micro_rows(dv, du, t, k4, c4):
    """The 8 per-edge columns of each edge i from its endpoint degrees and
    t, k4, c4 (the oracle's micro stores)."""
    out = np.zeros((len(t), 8), np.uint64)
    row = np.zeros(8, np.uint64)
    for i in range(len(t)):
        lib().po_micro_row(int(dv[i]), int(du[i]), int(t[i]), int(k4[i]), int(c4[i]), row)
        out[i] = row
    return out


def close(sums, n, m):
    out = np.zeros(17, np.uint64)
    lib().po_close(np.ascontiguousarray(sums, np.uint64), n, m, out)
    return out


# ---------------------------------------------------------------------------
# The reference itself (only where it was compiled, i.e. in the build container).

_ref = None


def ref_available():
    return os.path.exists(REF_SO)


def ref_lib():
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_SO)
        R.ref_open_file.restype = _P
        R.ref_open_file.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_char_p]
        R.ref_open_csr.restype = _P
        R.ref_open_csr.argtypes = [ctypes.c_int64, _I64P, _I32P, ctypes.c_char_p, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_char_p]
        R.ref_run.argtypes = [_P, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        R.ref_totals.argtypes = [_P, _U64P]
        R.ref_run_ids.argtypes = [_P, ctypes.c_char_p, ctypes.c_int, _I64P, ctypes.c_longlong, ctypes.c_int,
                                  ctypes.c_int]
        R.ref_n_ord.restype = ctypes.c_int64
        R.ref_n_ord.argtypes = [_P]
        R.ref_run_sample.restype = ctypes.c_longlong
        R.ref_run_sample.argtypes = [_P, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_longlong,
                                     ctypes.POINTER(ctypes.c_double)]
        for f in ("ref_n", "ref_m"):
            getattr(R, f).restype = ctypes.c_int64
            getattr(R, f).argtypes = [_P]
        R.ref_max_core.argtypes = [_P]
        R.ref_r.restype = ctypes.c_double
        R.ref_r.argtypes = [_P]
        R.ref_is_adj.argtypes = [_P]
        R.ref_micro.argtypes = [_P, _I64P, _I64P, _U64P]
        R.ref_csr.argtypes = [_P, _I64P, _I32P]
        R.ref_close.argtypes = [_P]
        _ref = R
    return _ref


class RefGraph:
    """The reference's graphlet_core driven through its public API."""

    def __init__(self, handle):
        self.h = handle

    @classmethod
    def from_file(cls, path, neigh="deg", s2l_neigh=False, adj_limit=10000, rep=""):
        return cls(ref_lib().ref_open_file(path.encode(), neigh.encode(), int(s2l_neigh), adj_limit,
                                           rep.encode()))

    @classmethod
    def from_csr(cls, off, adj, neigh="deg", s2l_neigh=False, adj_limit=10000, rep=""):
        off = np.ascontiguousarray(off, np.int64)
        adj = np.ascontiguousarray(adj, np.int32)
        return cls(ref_lib().ref_open_csr(len(off) - 1, off, adj, neigh.encode(), int(s2l_neigh),
                                          adj_limit, rep.encode()))

    def run(self, order="deg", s2l=False, micro=True, workers=1):
        ref_lib().ref_run(self.h, order.encode(), int(s2l), int(micro), workers)
        return self

    def run_sample(self, ids, order="deg", s2l=False, micro=True, workers=1):
        ids = np.ascontiguousarray(ids, np.int64)
        ref_lib().ref_run_ids(self.h, order.encode(), int(s2l), ids, len(ids), int(micro), workers)
        return self

    def time_sample(self, stride, order="deg", s2l=False, workers=1):
        sec = ctypes.c_double()
        k = ref_lib().ref_run_sample(self.h, order.encode(), int(s2l), workers, stride, ctypes.byref(sec))
        return k, sec.value

    @property
    def n(self):
        return ref_lib().ref_n(self.h)

    @property
    def m(self):
        return ref_lib().ref_m(self.h)

    @property
    def max_core(self):
        return ref_lib().ref_max_core(self.h)

    @property
    def r(self):
        return ref_lib().ref_r(self.h)

    def totals(self):
        t = np.zeros(17, np.uint64)
        ref_lib().ref_totals(self.h, t)
        return t

    def micro(self):
        m = ref_lib().ref_n_ord(self.h)
        src = np.zeros(m + 1, np.int64)
        dst = np.zeros(m + 1, np.int64)
        cols = np.zeros((m + 1) * 8, np.uint64)
        ref_lib().ref_micro(self.h, src, dst, cols)
        return src[:m], dst[:m], cols[: 8 * m].reshape(m, 8)

    def csr(self):
        off = np.zeros(self.n + 1, np.int64)
        adj = np.zeros(2 * self.m + 1, np.int32)
        ref_lib().ref_csr(self.h, off, adj)
        return off, adj[: off[-1]]

    def __del__(self):
        if getattr(self, "h", None):
            ref_lib().ref_close(self.h)
            self.h = None
