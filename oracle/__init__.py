"""CPU oracle for the SSTGraph hot path -- TEST INFRASTRUCTURE.

Loads two CPU libraries through ctypes:

* ``_build/libsst_oracle.so``: the C restatement in ``sst_oracle.c``
  (storage semantics, generators, BFS/PR/CC/BC/TC).  Builds anywhere.
* ``_ref/libsstref.so``: the reference's own ``SparseMatrixV<true>`` /
  ``TinySetV`` / ``rMat`` compiled from the reference headers plus the
  stand-in headers in ``shim/`` (only where the reference tree exists).

Only tests, the smoke check and the CPU-baseline leg of bench.py use this
package; the product (``sstgraph_gb300``) never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libsst_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsstref.so")

_u32p = ctypes.c_void_p
_lib = None
_ref = None


def build(ref: bool = False) -> None:
    """Compile the oracle (and, if asked and possible, the reference build)."""
    targets = ["all"]
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE] + targets, check=True)


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        vp, u32, u64, dbl, i32 = (ctypes.c_void_p, ctypes.c_uint32,
                                  ctypes.c_uint64, ctypes.c_double, ctypes.c_int)
        sig = {
            "sst_o_mix64": (u64, [u64]),
            "sst_o_draw": (u64, [u64, u64, u64]),
            "sst_o_ref_hash64": (u64, [u64]),
            "sst_o_ref_hash32": (u32, [u32]),
            "sst_o_rmat": (None, [u32, dbl, dbl, dbl, u64, u64, u64, vp]),
            "sst_o_er": (None, [u32, u64, u64, u64, vp]),
            "sst_o_ref_rmat_stream": (None, [u32, dbl, dbl, dbl, u64, u64, vp]),
            "sst_o_new": (vp, [u32]),
            "sst_o_new2": (vp, [u32, u32]),
            "sst_o_free": (None, [vp]),
            "sst_o_insert_batch": (None, [vp, vp, u64]),
            "sst_o_remove_batch": (None, [vp, vp, u64]),
            "sst_o_M": (u64, [vp]),
            "sst_o_degree": (u32, [vp, u32]),
            "sst_o_has": (i32, [vp, u32, u32]),
            "sst_o_degrees": (None, [vp, vp]),
            "sst_o_to_csr": (None, [vp, vp, vp]),
            "sst_o_common_neighbors": (u64, [vp, u32, u32, i32]),
            "sst_o_touch_all_sum": (u64, [vp]),
            "sst_o_sample_edges": (None, [vp, u64, u64, u64, vp]),
            "sst_o_bfs": (None, [vp, u32, vp]),
            "sst_o_pagerank": (None, [vp, u32, dbl, vp]),
            "sst_o_cc": (None, [vp, vp]),
            "sst_o_bc": (None, [vp, u32, vp]),
            "sst_o_tc": (u64, [vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _pairs(edges) -> np.ndarray:
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.uint32).reshape(-1, 2))
    return e


# ---------------------------------------------------------------- generators
def rmat(scale, count, a=0.57, b=0.19, c=0.19, seed=1, first=0) -> np.ndarray:
    out = np.empty((count, 2), np.uint32)
    lib().sst_o_rmat(scale, a, b, c, seed, first, count, _ptr(out))
    return out


def er(n, count, seed=4, first=0) -> np.ndarray:
    out = np.empty((count, 2), np.uint32)
    lib().sst_o_er(n, seed, first, count, _ptr(out))
    return out


def ref_rmat_stream(nn, count, a=0.5, b=0.1, c=0.1, first=0) -> np.ndarray:
    out = np.empty((count, 2), np.uint32)
    lib().sst_o_ref_rmat_stream(nn, a, b, c, first, count, _ptr(out))
    return out


def symmetrize(edges) -> np.ndarray:
    e = _pairs(edges)
    return np.concatenate([e, e[:, ::-1]], axis=0).copy()


# --------------------------------------------------------------------- graph
class OracleGraph:
    """Restated SparseMatrixV<true>: per-row sorted sets of uint32 columns."""

    def __init__(self, n: int, width: int | None = None):
        self.n = int(n)
        self.width = self.n if width is None else int(width)
        self._h = lib().sst_o_new2(self.n, self.width)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().sst_o_free(h)
            self._h = None

    def insert_batch(self, edges):
        e = _pairs(edges)
        lib().sst_o_insert_batch(self._h, _ptr(e), e.shape[0])

    def remove_batch(self, edges):
        e = _pairs(edges)
        lib().sst_o_remove_batch(self._h, _ptr(e), e.shape[0])

    def M(self) -> int:
        return int(lib().sst_o_M(self._h))

    def getDegree(self, v) -> int:
        return int(lib().sst_o_degree(self._h, v))

    def has(self, r, c) -> bool:
        return bool(lib().sst_o_has(self._h, r, c))

    def degrees(self) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        lib().sst_o_degrees(self._h, _ptr(out))
        return out

    def csr(self):
        off = np.empty(self.n + 1, np.uint64)
        cols = np.empty(max(self.M(), 1), np.uint32)
        lib().sst_o_to_csr(self._h, _ptr(off), _ptr(cols))
        return off, cols[: int(off[-1])]

    def common_neighbors(self, a, b, early_end=False) -> int:
        return int(lib().sst_o_common_neighbors(self._h, a, b, int(early_end)))

    def touch_all_sum(self) -> int:
        return int(lib().sst_o_touch_all_sum(self._h))

    def sample_edges(self, count, seed, first=0) -> np.ndarray:
        out = np.empty((count, 2), np.uint32)
        lib().sst_o_sample_edges(self._h, seed, first, count, _ptr(out))
        return out

    def bfs(self, src) -> np.ndarray:
        out = np.empty(self.n, np.int32)
        lib().sst_o_bfs(self._h, src, _ptr(out))
        return out

    def pagerank(self, iters=10, damping=0.85) -> np.ndarray:
        out = np.empty(self.n, np.float64)
        lib().sst_o_pagerank(self._h, iters, damping, _ptr(out))
        return out

    def cc(self) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        lib().sst_o_cc(self._h, _ptr(out))
        return out

    def bc(self, src) -> np.ndarray:
        out = np.empty(self.n, np.float64)
        lib().sst_o_bc(self._h, src, _ptr(out))
        return out

    def tc(self, per_vertex=False):
        if per_vertex:
            pv = np.empty(self.n, np.uint64)
            t = lib().sst_o_tc(self._h, _ptr(pv))
            return int(t), pv
        return int(lib().sst_o_tc(self._h, None))


# ----------------------------------------------------- the reference's build
def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    """The reference's own storage code (oracle/_ref); raises if not built."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError(REF_SO)
        L = ctypes.CDLL(REF_SO)
        vp, u32, u64, dbl, i32 = (ctypes.c_void_p, ctypes.c_uint32,
                                  ctypes.c_uint64, ctypes.c_double, ctypes.c_int)
        sig = {
            "ref_graph_new": (vp, [u32]),
            "ref_graph_free": (None, [vp]),
            "ref_insert_batch": (None, [vp, vp, u64]),
            "ref_remove_batch": (None, [vp, vp, u64]),
            "ref_insert": (None, [vp, u32, u32]),
            "ref_remove": (None, [vp, u32, u32]),
            "ref_has": (i32, [vp, u32, u32]),
            "ref_degree": (u32, [vp, u32]),
            "ref_M": (u64, [vp]),
            "ref_common_neighbors": (u64, [vp, u32, u32, i32]),
            "ref_touch_all_sum": (u64, [vp]),
            "ref_to_csr": (None, [vp, vp, vp]),
            "ref_degree_order_map": (None, [vp, vp]),
            "ref_rewrite_graph": (vp, [vp, vp]),
            "ref_set_new": (vp, [u32]),
            "ref_set_free": (None, [vp]),
            "ref_set_insert": (None, [vp, u32]),
            "ref_set_remove": (None, [vp, u32]),
            "ref_set_has": (i32, [vp, u32]),
            "ref_set_n": (u64, [vp]),
            "ref_set_to_array": (u64, [vp, vp]),
            "ref_hash64": (u64, [u64]),
            "ref_hash32": (u32, [u32]),
            "ref_rmat_stream": (None, [u32, dbl, dbl, dbl, u64, vp]),
            "ref_random_data": (None, [u64, u32, u32, vp]),
            "ref_load_mtx": (u64, [ctypes.c_char_p, ctypes.POINTER(u32),
                                   ctypes.POINTER(vp)]),
            "ref_free": (None, [vp]),
            "ref_tinyset_thresholds": (None, [u64, vp]),
            "ref_wgraph_new": (vp, [u32]),
            "ref_wgraph_free": (None, [vp]),
            "ref_winsert_batch": (None, [vp, vp, vp, u64]),
            "ref_wremove_each": (None, [vp, vp, u64]),
            "ref_wM": (u64, [vp]),
            "ref_wvalue": (u32, [vp, u32, u32]),
            "ref_wto_csr": (None, [vp, vp, vp, vp]),
            "ref_tinyset_width": (u32, [u64, vp, u64]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _ref = L
    return _ref


class RefGraph:
    """The reference SparseMatrixV<true> (compiled reference code)."""

    def __init__(self, n: int):
        self.n = int(n)
        self._h = ref().ref_graph_new(self.n)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            ref().ref_graph_free(h)
            self._h = None

    def insert_batch(self, edges):
        e = _pairs(edges)
        ref().ref_insert_batch(self._h, _ptr(e), e.shape[0])

    def remove_batch(self, edges):
        e = _pairs(edges)
        ref().ref_remove_batch(self._h, _ptr(e), e.shape[0])

    def M(self) -> int:
        return int(ref().ref_M(self._h))

    def has(self, r, c) -> bool:
        return bool(ref().ref_has(self._h, r, c))

    def getDegree(self, v) -> int:
        return int(ref().ref_degree(self._h, v))

    def csr(self):
        off = np.empty(self.n + 1, np.uint64)
        cols = np.empty(max(self.M(), 1), np.uint32)
        ref().ref_to_csr(self._h, _ptr(off), _ptr(cols))
        return off, cols[: int(off[-1])]

    def common_neighbors(self, a, b, early_end=False) -> int:
        return int(ref().ref_common_neighbors(self._h, a, b, int(early_end)))

    def touch_all_sum(self) -> int:
        return int(ref().ref_touch_all_sum(self._h))

    def degree_order_map(self) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        ref().ref_degree_order_map(self._h, _ptr(out))
        return out

    def rewrite_graph(self, label_map) -> "RefGraph":
        m = np.ascontiguousarray(label_map, np.uint32)
        g = RefGraph.__new__(RefGraph)
        g.n = self.n
        g._h = ref().ref_rewrite_graph(self._h, _ptr(m))
        return g


class RefWGraph:
    """The reference SparseMatrixV<true, uint32_t> (compiled reference code):
    insert_batch with a value per pair; removes one edge at a time (the
    reference's weighted remove_batch does not compile)."""

    def __init__(self, n: int):
        self.n = int(n)
        self._h = ref().ref_wgraph_new(self.n)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            ref().ref_wgraph_free(h)
            self._h = None

    def insert_batch(self, edges, values):
        e = _pairs(edges)
        v = np.ascontiguousarray(np.asarray(values, np.uint32).reshape(-1))
        ref().ref_winsert_batch(self._h, _ptr(e), _ptr(v), e.shape[0])

    def remove_each(self, edges):
        e = _pairs(edges)
        ref().ref_wremove_each(self._h, _ptr(e), e.shape[0])

    def M(self) -> int:
        return int(ref().ref_wM(self._h))

    def value(self, r, c) -> int:
        return int(ref().ref_wvalue(self._h, r, c))

    def csr_values(self):
        m = self.M()
        off = np.empty(self.n + 1, np.uint64)
        cols = np.empty(max(m, 1), np.uint32)
        vals = np.empty(max(m, 1), np.uint32)
        ref().ref_wto_csr(self._h, _ptr(off), _ptr(cols), _ptr(vals))
        k = int(off[-1])
        return off, cols[:k], vals[:k]


def degree_order_map(degrees) -> np.ndarray:
    """Restated degree_order_map (SparseMatrix.hpp:737-752): rank of each
    vertex when ordered by (degree, id) descending."""
    d = np.asarray(degrees, np.int64)
    ids = np.arange(len(d), dtype=np.int64)
    order = np.lexsort((-ids, -d))
    out = np.empty(len(d), np.uint32)
    out[order] = np.arange(len(d), dtype=np.uint32)
    return out


def relabel(edges, label_map) -> np.ndarray:
    e = _pairs(edges)
    return np.ascontiguousarray(np.asarray(label_map, np.uint32)[e])


def ref_random_data(n, max_val, seed=0) -> np.ndarray:
    out = np.empty(n, np.uint32)
    ref().ref_random_data(n, max_val, seed, _ptr(out))
    return out


def ref_load_mtx(path):
    rows = ctypes.c_uint32(0)
    p = ctypes.c_void_p(0)
    m = ref().ref_load_mtx(path.encode(), ctypes.byref(rows), ctypes.byref(p))
    arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint32)),
                                shape=(m * 2,)).copy().reshape(-1, 2)
    ref().ref_free(p)
    return int(rows.value), arr
