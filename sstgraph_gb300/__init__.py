"""sstgraph_gb300 -- GB300-native dynamic graph (SSTGraph's hot path).

Python mirror of the reference's graph interface over the C ABI in
include/sstgraph.h (libsstgraph_gb300.so, built in-tree by build.py).  Names
follow the reference: ``SparseMatrixV`` (include/SSTGraph/SparseMatrix.hpp)
with ``insert_batch`` / ``remove_batch`` / ``has`` / ``getDegree`` / ``M`` /
``map_neighbors`` / ``common_neighbors`` / ``touch_all_sum``, and the
EdgeMapVertexMap entry points the reference drivers call (``BFS``, ``PR_S``,
``CC``, ``BC``, ``TC``, ``TouchAll``; internal/test.hpp:476-618).

Every call runs on the GPU.  There is no CPU fallback: if the library is
missing or no GPU is usable, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libsstgraph_gb300.so")

HOST_PTR = 0
DEVICE_PTR = 1
SEMI_SORTED = 2

_STATUS = {0: "ok", -1: "invalid argument", -2: "out of device memory",
           -3: "HBM budget exceeded", -4: "device wait timed out",
           -5: "CUDA device error", -6: "invalid state"}


class SSTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status


class sst_config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int),
                ("hbm_budget_bytes", ctypes.c_uint64),
                ("initial_slots", ctypes.c_uint64),
                ("upper_root", ctypes.c_float),
                ("lower_root", ctypes.c_float),
                ("grow_fill", ctypes.c_float),
                ("keep_self_loops", ctypes.c_uint32),
                ("weighted", ctypes.c_uint32)]


class sst_tuning(ctypes.Structure):
    _fields_ = [("chunk_leaves", ctypes.c_uint32), ("pr_lanes", ctypes.c_uint32),
                ("bfs_alpha", ctypes.c_uint32), ("pr_ms", ctypes.c_float),
                ("bfs_ms", ctypes.c_float), ("pr_hot", ctypes.c_uint32)]


class sst_server_config(ctypes.Structure):
    _fields_ = [("query_slots", ctypes.c_uint32),
                ("hbm_budget_bytes", ctypes.c_uint64),
                ("max_coalesce", ctypes.c_uint32)]


class sst_request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("pairs", ctypes.c_void_p),
                ("n", ctypes.c_uint64), ("src", ctypes.c_uint32),
                ("iters", ctypes.c_uint32), ("damping", ctypes.c_double),
                ("out", ctypes.c_void_p)]


class sst_request_info(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("epoch", ctypes.c_uint64),
                ("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double)]


REQ_INSERT, REQ_REMOVE, REQ_BFS, REQ_PAGERANK, REQ_TC_VERTICES = 1, 2, 3, 4, 5

# name -> (restype, argtypes); mirrors include/sstgraph.h
_vp, _u32, _u64, _i32, _dbl = (ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64,
                               ctypes.c_int32, ctypes.c_double)
SIGNATURES = {
    "sst_graph_create": (_i32, [_u32, _u32, ctypes.POINTER(sst_config), ctypes.POINTER(_vp)]),
    "sst_graph_destroy": (_i32, [_vp]),
    "sst_graph_clone": (_i32, [_vp, ctypes.POINTER(_vp)]),
    "sst_set_stream": (_i32, [_vp, _vp]),
    "sst_set_plan_graphs": (_i32, [_vp, ctypes.c_int]),
    "sst_sync": (_i32, [_vp]),
    "sst_last_error_message": (ctypes.c_char_p, []),
    "sst_status_string": (ctypes.c_char_p, [_i32]),
    "sst_insert_batch": (_i32, [_vp, _vp, _u64, _u32, ctypes.POINTER(_u64)]),
    "sst_remove_batch": (_i32, [_vp, _vp, _u64, _u32, ctypes.POINTER(_u64)]),
    "sst_update_batches": (_i32, [_vp, _vp, _vp, _vp, _u32, _u32, ctypes.POINTER(_u64)]),
    "sst_insert": (_i32, [_vp, _u32, _u32]),
    "sst_remove": (_i32, [_vp, _u32, _u32]),
    "sst_build_from_csr": (_i32, [_vp, _vp, _vp, _u32]),
    "sst_has_batch": (_i32, [_vp, _vp, _u64, _vp, _u32]),
    "sst_has": (_i32, [_vp, _u32, _u32, ctypes.POINTER(ctypes.c_int)]),
    "sst_num_nodes": (_i32, [_vp, ctypes.POINTER(_u64)]),
    "sst_get_rows": (_i32, [_vp, ctypes.POINTER(_u32)]),
    "sst_get_cols": (_i32, [_vp, ctypes.POINTER(_u32)]),
    "sst_M": (_i32, [_vp, ctypes.POINTER(_u64)]),
    "sst_degrees": (_i32, [_vp, _vp, _u32]),
    "sst_get_degree": (_i32, [_vp, _u32, ctypes.POINTER(_u32)]),
    "sst_neighbors": (_i32, [_vp, _u32, _vp, _u64, ctypes.POINTER(_u64)]),
    "sst_to_csr": (_i32, [_vp, _vp, _vp, _u32]),
    "sst_insert_batch_weighted": (_i32, [_vp, _vp, _vp, _u64, _u32, ctypes.POINTER(_u64)]),
    "sst_values_batch": (_i32, [_vp, _vp, _u64, _vp, _vp, _u32]),
    "sst_to_csr_values": (_i32, [_vp, _vp, _vp, _vp, _u32]),
    "sst_bf": (_i32, [_vp, _u32, _vp, _u32]),
    "sst_common_neighbors_batch": (_i32, [_vp, _vp, _u64, ctypes.c_int, _vp, _u32]),
    "sst_touch_all_sum": (_i32, [_vp, ctypes.POINTER(_u64)]),
    "sst_memory_size": (_i32, [_vp, ctypes.POINTER(_u64)]),
    "sst_release_scratch": (_i32, [_vp]),
    "sst_sample_edges": (_i32, [_vp, _u64, _u64, _u64, _vp, _u32]),
    "sst_degree_order_map": (_i32, [_vp, _vp, _u32]),
    "sst_rewrite_graph": (_i32, [_vp, _vp, _u32, ctypes.POINTER(_vp)]),
    "sst_bfs": (_i32, [_vp, _u32, _vp, _vp, _u32]),
    "sst_pagerank": (_i32, [_vp, _u32, _dbl, _vp, _u32]),
    "sst_cc": (_i32, [_vp, _vp, _u32]),
    "sst_bc": (_i32, [_vp, _u32, _vp, _u32]),
    "sst_bfs_multi": (_i32, [_vp, _vp, _u32, _vp, _u32]),
    "sst_autotune": (_i32, [_vp, ctypes.POINTER(sst_tuning)]),
    "sst_read_graph_file": (_i32, [ctypes.c_char_p, ctypes.POINTER(_u32),
                                   ctypes.POINTER(_u64), ctypes.POINTER(_vp)]),
    "sst_free": (None, [_vp]),
    "sst_load_graph_file": (_i32, [ctypes.c_char_p, ctypes.POINTER(sst_config),
                                   ctypes.POINTER(_vp)]),
    "sst_get_tuning": (_i32, [_vp, ctypes.POINTER(sst_tuning)]),
    "sst_set_tuning": (_i32, [_vp, ctypes.POINTER(sst_tuning)]),
    "sst_bc_multi": (_i32, [_vp, _vp, _u32, _vp, _u32]),
    "sst_tc": (_i32, [_vp, ctypes.POINTER(_u64), _vp, _u32]),
    "sst_touch_all": (_i32, [_vp, ctypes.POINTER(_u64)]),
    "sst_gen_rmat": (_i32, [_u32, _dbl, _dbl, _dbl, _u64, _u64, _u64, _vp, _u32]),
    "sst_gen_er": (_i32, [_u32, _u64, _u64, _u64, _vp, _u32]),
    "sst_gen_ref_rmat": (_i32, [_u32, _dbl, _dbl, _dbl, _u64, _u64, _vp, _u32]),
    "sst_kernel_launches": (_u64, []),
    "sst_set_scan_lookback_polls": (_i32, [_u32, ctypes.POINTER(_u32)]),
    "sst_raw_state": (_i32, [_vp, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_u64)]),
    "sst_pagerank_noalloc": (_i32, [_vp, _u32, _dbl, _vp]),
    "sst_tc_vertices": (_i32, [_vp, _vp, _u64, _vp, _u32]),
    "sst_server_create": (_i32, [_vp, ctypes.POINTER(sst_server_config), ctypes.POINTER(_vp)]),
    "sst_server_slots": (_i32, [_vp, ctypes.POINTER(_u32)]),
    "sst_server_submit": (_i32, [_vp, ctypes.POINTER(sst_request), ctypes.POINTER(_u64)]),
    "sst_server_wait": (_i32, [_vp, _u64, _u32, ctypes.POINTER(sst_request_info)]),
    "sst_server_stats": (_i32, [_vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64),
                                ctypes.POINTER(_u64)]),
    "sst_server_destroy": (_i32, [_vp]),
    "sst_compact_widths": (_i32, [_u64, _vp]),
    "sst_compact_create": (_i32, [_vp, ctypes.POINTER(_vp)]),
    "sst_compact_destroy": (_i32, [_vp]),
    "sst_compact_info": (_i32, [_vp, ctypes.POINTER(_u64), ctypes.POINTER(_u64),
                                ctypes.POINTER(_u64), _vp]),
    "sst_compact_to_csr": (_i32, [_vp, _vp, _vp, _u32]),
    "sst_compact_has_batch": (_i32, [_vp, _vp, _u64, _vp, _u32]),
    "sst_compact_pagerank": (_i32, [_vp, _u32, _dbl, _vp, _u32]),
    "sst_compact_bfs": (_i32, [_vp, _u32, _vp, _u32]),
    "sst_compact_cc": (_i32, [_vp, _vp, _u32]),
    "sst_compact_tc": (_i32, [_vp, ctypes.POINTER(_u64), _vp, _u32]),
    "sst_compact_bc": (_i32, [_vp, _u32, _vp, _u32]),
    "sst_compact_sync": (_i32, [_vp]),
    "sst_compact_set_stream": (_i32, [_vp, _vp]),
    "sst_profile_start": (_i32, [ctypes.c_char_p]),
    "sst_profile_collect": (_i32, [ctypes.c_char_p, _u64]),
}


def profile_start(kernel_filter: str | None = None):
    """Bracket kernel launches with CUDA events (all, or those whose name
    contains kernel_filter) until profile_collect()."""
    _check(lib().sst_profile_start(kernel_filter.encode() if kernel_filter else None))


def profile_collect() -> dict:
    """Per-kernel {name: {"launches": L, "ms": T}} since profile_start()."""
    import json
    buf = ctypes.create_string_buffer(1 << 20)
    _check(lib().sst_profile_collect(buf, len(buf)))
    return json.loads(buf.value.decode())

_lib = None


def lib():
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check(status: int):
    if status != 0:
        raise SSTError(status, lib().sst_last_error_message().decode())


def _ptr(a):
    """ctypes pointer of a numpy array or a torch tensor (host or device)."""
    if isinstance(a, np.ndarray):
        return ctypes.c_void_p(a.ctypes.data), HOST_PTR
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr()), (DEVICE_PTR if a.is_cuda else HOST_PTR)
    raise TypeError(f"unsupported array type {type(a)}")


def _pairs(edges):
    if hasattr(edges, "data_ptr"):
        assert edges.is_contiguous()
        return edges, edges.numel() // 2
    e = np.ascontiguousarray(np.asarray(edges, dtype=np.uint32).reshape(-1, 2))
    return e, e.shape[0]


def set_scan_lookback_polls(polls: int) -> int:
    """Polls of a predecessor's status in the single-pass scans before a
    tile reduces the inputs itself (0: every tile does); returns the previous
    setting.  Results do not depend on it."""
    old = ctypes.c_uint32()
    _check(lib().sst_set_scan_lookback_polls(int(polls), ctypes.byref(old)))
    return old.value


def kernel_launches() -> int:
    return int(lib().sst_kernel_launches())


class SparseMatrixV:
    """Device-resident SparseMatrixV<true> (binary CSR, uint32 ids).

    Reference: include/SSTGraph/SparseMatrix.hpp.  Arrays may be numpy (host)
    or torch CUDA tensors (device); results come back in the same place.
    """

    def __init__(self, height: int, width: int | None = None, *, device: int = 0,
                 hbm_budget_bytes: int = 0, initial_slots: int = 0,
                 upper_root: float = 0.0, lower_root: float = 0.0,
                 grow_fill: float = 0.0, keep_self_loops: bool = False,
                 weighted: bool = False, _handle=None):
        self._h = None
        if _handle is not None:
            self._h = _handle
        else:
            cfg = sst_config(device, hbm_budget_bytes, initial_slots,
                             upper_root, lower_root, grow_fill,
                             1 if keep_self_loops else 0, 1 if weighted else 0)
            h = ctypes.c_void_p()
            _check(lib().sst_graph_create(height, height if width is None else width,
                                          ctypes.byref(cfg), ctypes.byref(h)))
            self._h = h
        r = ctypes.c_uint32()
        _check(lib().sst_get_rows(self._h, ctypes.byref(r)))
        self.rows = r.value
        _check(lib().sst_get_cols(self._h, ctypes.byref(r)))
        self.cols = r.value

    def close(self):
        if self._h:
            lib().sst_graph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def copy(self) -> "SparseMatrixV":
        h = ctypes.c_void_p()
        _check(lib().sst_graph_clone(self._h, ctypes.byref(h)))
        return SparseMatrixV(0, _handle=h)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None):
        _check(lib().sst_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))

    def set_plan_graphs(self, enable):
        """Replay small batches' planning launches as CUDA graphs (True /
        1, default), launch every kernel directly (False / 0), or launch the
        kernels a replay runs directly (2: for per-kernel timing); results
        are the same."""
        mode = enable if isinstance(enable, int) and not isinstance(enable, bool) else (1 if enable else 0)
        _check(lib().sst_set_plan_graphs(self._h, mode))

    def sync(self):
        _check(lib().sst_sync(self._h))

    # -- updates ------------------------------------------------------------
    def insert_batch(self, edges, semi_sorted: bool = False) -> int:
        """Insert (row, col) pairs; returns the count of pairs out of range."""
        e, n = _pairs(edges)
        p, flags = _ptr(e)
        bad = ctypes.c_uint64()
        _check(lib().sst_insert_batch(self._h, p, n, flags | (SEMI_SORTED if semi_sorted else 0),
                                      ctypes.byref(bad)))
        return bad.value

    def remove_batch(self, edges, semi_sorted: bool = False) -> int:
        e, n = _pairs(edges)
        p, flags = _ptr(e)
        bad = ctypes.c_uint64()
        _check(lib().sst_remove_batch(self._h, p, n, flags | (SEMI_SORTED if semi_sorted else 0),
                                      ctypes.byref(bad)))
        return bad.value

    def update_batches(self, batches, ops=None) -> int:
        """Apply a sequence of batches as one pipeline pass.

        batches: list of (k, 2) pair arrays (or one concatenated array with
        `offsets`); ops: per batch 1 = insert, 0 = remove (default: insert).
        """
        if isinstance(batches, tuple) and len(batches) == 2:
            pairs, offsets = batches
        else:
            sizes = [len(b) for b in batches]
            offsets = np.zeros(len(batches) + 1, np.uint64)
            offsets[1:] = np.cumsum(sizes)
            if batches and hasattr(batches[0], "data_ptr"):
                import torch
                pairs = torch.cat(list(batches)).contiguous()
                offsets = torch.from_numpy(offsets.astype(np.int64)).to(pairs.device)
            else:
                pairs = np.ascontiguousarray(np.concatenate(
                    [np.asarray(b, np.uint32).reshape(-1, 2) for b in batches]))
        nb = len(offsets) - 1
        if ops is None:
            ops = [1] * nb
        p, flags = _ptr(pairs)
        if flags == DEVICE_PTR:
            import torch
            ops_t = torch.as_tensor(np.asarray(ops, np.uint8), device=pairs.device)
            po, _ = _ptr(offsets)
            pops, _ = _ptr(ops_t)
        else:
            offsets = np.ascontiguousarray(offsets, np.uint64)
            ops_a = np.ascontiguousarray(np.asarray(ops, np.uint8))
            po, pops = ctypes.c_void_p(offsets.ctypes.data), ctypes.c_void_p(ops_a.ctypes.data)
        bad = ctypes.c_uint64()
        _check(lib().sst_update_batches(self._h, p, po, pops, nb, flags, ctypes.byref(bad)))
        return bad.value

    def insert(self, row: int, col: int):
        _check(lib().sst_insert(self._h, row, col))

    def remove(self, row: int, col: int):
        _check(lib().sst_remove(self._h, row, col))

    def build_from_csr(self, offsets, cols):
        offsets = np.ascontiguousarray(offsets, dtype=np.uint64) if isinstance(offsets, np.ndarray) else offsets
        cols = np.ascontiguousarray(cols, dtype=np.uint32) if isinstance(cols, np.ndarray) else cols
        po, flags = _ptr(offsets)
        pc, _ = _ptr(cols)
        _check(lib().sst_build_from_csr(self._h, po, pc, flags))

    # -- queries ------------------------------------------------------------
    def has(self, row: int, col: int) -> bool:
        r = ctypes.c_int()
        _check(lib().sst_has(self._h, row, col, ctypes.byref(r)))
        return bool(r.value)

    def has_batch(self, edges, out=None):
        e, n = _pairs(edges)
        p, flags = _ptr(e)
        if out is None:
            if flags == DEVICE_PTR:
                import torch
                out = torch.empty(n, dtype=torch.uint8, device=e.device)
            else:
                out = np.empty(n, np.uint8)
        po, _ = _ptr(out)
        _check(lib().sst_has_batch(self._h, p, n, po, flags))
        return out

    def num_nodes(self) -> int:
        return self.rows

    def get_rows(self) -> int:
        return self.rows

    def get_cols(self) -> int:
        return self.cols

    def M(self) -> int:
        r = ctypes.c_uint64()
        _check(lib().sst_M(self._h, ctypes.byref(r)))
        return r.value

    def getDegree(self, v: int) -> int:
        r = ctypes.c_uint32()
        _check(lib().sst_get_degree(self._h, v, ctypes.byref(r)))
        return r.value

    def degrees(self, out=None):
        if out is None:
            out = np.empty(self.rows, np.uint32)
        p, flags = _ptr(out)
        _check(lib().sst_degrees(self._h, p, flags))
        return out

    def neighbors(self, v: int) -> np.ndarray:
        d = self.getDegree(v)
        out = np.empty(max(d, 1), np.uint32)
        full = ctypes.c_uint64()
        _check(lib().sst_neighbors(self._h, v, ctypes.c_void_p(out.ctypes.data), d,
                                   ctypes.byref(full)))
        return out[:d]

    def map_neighbors(self, v: int, f):
        """Host-callback map over v's neighbours in ascending order
        (SparseMatrix.hpp:218-253): f(src, dst) returning True stops early."""
        for x in self.neighbors(v):
            if f(v, int(x)):
                return

    def csr(self):
        m = self.M()
        off = np.empty(self.rows + 1, np.uint64)
        cols = np.empty(max(m, 1), np.uint32)
        _check(lib().sst_to_csr(self._h, ctypes.c_void_p(off.ctypes.data),
                                ctypes.c_void_p(cols.ctypes.data), HOST_PTR))
        return off, cols[:m]

    def insert_batch_weighted(self, edges, values) -> int:
        """Insert (row, col) pairs with one uint32 value each (weighted
        graphs); a present edge takes the new value, the last of equal pairs
        wins.  Returns the count of pairs out of range."""
        e, n = _pairs(edges)
        p, flags = _ptr(e)
        if flags == DEVICE_PTR:
            v = values.contiguous()
        else:
            v = np.ascontiguousarray(np.asarray(values).astype(np.uint32).reshape(-1))
        assert (v.numel() if hasattr(v, "numel") else v.size) == n
        pv, _ = _ptr(v)
        bad = ctypes.c_uint64()
        _check(lib().sst_insert_batch_weighted(self._h, p, pv, n, flags, ctypes.byref(bad)))
        return bad.value

    def values(self, edges):
        """(values, found) of (row, col) pairs on a weighted graph (host)."""
        e = np.ascontiguousarray(np.asarray(edges, np.uint32).reshape(-1, 2))
        n = e.shape[0]
        vals = np.empty(max(n, 1), np.uint32)
        found = np.empty(max(n, 1), np.uint8)
        _check(lib().sst_values_batch(self._h, ctypes.c_void_p(e.ctypes.data), n,
                                      ctypes.c_void_p(vals.ctypes.data),
                                      ctypes.c_void_p(found.ctypes.data), HOST_PTR))
        return vals[:n], found[:n].astype(bool)

    def csr_values(self):
        """(offsets, cols, values) of a weighted graph (host)."""
        m = self.M()
        off = np.empty(self.rows + 1, np.uint64)
        cols = np.empty(max(m, 1), np.uint32)
        vals = np.empty(max(m, 1), np.uint32)
        _check(lib().sst_to_csr_values(self._h, ctypes.c_void_p(off.ctypes.data),
                                       ctypes.c_void_p(cols.ctypes.data),
                                       ctypes.c_void_p(vals.ctypes.data), HOST_PTR))
        return off, cols[:m], vals[:m]

    def common_neighbors(self, a: int, b: int, early_end: bool = False) -> int:
        return int(self.common_neighbors_batch(np.array([[a, b]], np.uint32), early_end)[0])

    def common_neighbors_batch(self, pairs, early_end: bool = False):
        e, n = _pairs(pairs)
        p, flags = _ptr(e)
        if flags == DEVICE_PTR:
            import torch
            out = torch.empty(n, dtype=torch.int64, device=e.device)
        else:
            out = np.empty(n, np.uint64)
        po, _ = _ptr(out)
        _check(lib().sst_common_neighbors_batch(self._h, p, n, int(early_end), po, flags))
        return out

    def touch_all_sum(self) -> int:
        r = ctypes.c_uint64()
        _check(lib().sst_touch_all_sum(self._h, ctypes.byref(r)))
        return r.value

    def get_memory_size(self) -> int:
        r = ctypes.c_uint64()
        _check(lib().sst_memory_size(self._h, ctypes.byref(r)))
        return r.value

    def release_scratch(self):
        """Free the scratch the graph keeps between calls (update, staging,
        traversal buffers); it is allocated again when needed."""
        _check(lib().sst_release_scratch(self._h))

    def raw_state(self):
        """(base, cap, deg, slots, lcnt): the device layout, for checks."""
        n = self.rows
        base = np.empty(max(n, 1), np.uint64)
        cap = np.empty(max(n, 1), np.uint32)
        deg = np.empty(max(n, 1), np.uint32)
        ns = ctypes.c_uint64(0)
        _check(lib().sst_raw_state(self._h, None, None, None, None, None, ctypes.byref(ns)))
        used = ns.value
        slots = np.empty(max(used, 32), np.uint32)
        lcnt = np.empty(max(used // 32, 1), np.uint8)
        ns = ctypes.c_uint64(used)
        _check(lib().sst_raw_state(self._h, ctypes.c_void_p(base.ctypes.data),
                                   ctypes.c_void_p(cap.ctypes.data),
                                   ctypes.c_void_p(deg.ctypes.data),
                                   ctypes.c_void_p(slots.ctypes.data),
                                   ctypes.c_void_p(lcnt.ctypes.data), ctypes.byref(ns)))
        return base[:n], cap[:n], deg[:n], slots[:used], lcnt[:used // 32]

    def degree_order_map(self, out=None):
        """new label of each vertex: its rank by (degree, id) descending"""
        if out is None:
            out = np.empty(self.rows, np.uint32)
        p, flags = _ptr(out)
        _check(lib().sst_degree_order_map(self._h, p, flags))
        return out

    def rewrite_graph(self, new_label_map) -> "SparseMatrixV":
        m = new_label_map
        if isinstance(m, np.ndarray):
            m = np.ascontiguousarray(m, np.uint32)
        p, flags = _ptr(m)
        h = ctypes.c_void_p()
        _check(lib().sst_rewrite_graph(self._h, p, flags, ctypes.byref(h)))
        return SparseMatrixV(0, _handle=h)

    def sample_edges(self, count: int, seed: int, first: int = 0, out=None):
        if out is None:
            out = np.empty((count, 2), np.uint32)
        p, flags = _ptr(out)
        _check(lib().sst_sample_edges(self._h, seed, first, count, p, flags))
        return out


# ---- EdgeMapVertexMap entry points (internal/test.hpp:476-618) ------------
def _out(g, dtype, out, torch_dtype=None):
    if out is None:
        return np.empty(g.rows, dtype)
    return out


def BFS(g: SparseMatrixV, src: int, depths: bool = False, parents=None, out=None):
    """Parents (parent[src] = src, -1 unreached) as the reference returns;
    with depths=True the BFS depths instead (-1 unreached)."""
    buf = _out(g, np.int32, out)
    p, flags = _ptr(buf)
    if depths:
        _check(lib().sst_bfs(g.handle, src, None, p, flags))
    else:
        _check(lib().sst_bfs(g.handle, src, p, None, flags))
    return buf


def BFS_both(g: SparseMatrixV, src: int):
    par = np.empty(g.rows, np.int32)
    dep = np.empty(g.rows, np.int32)
    _check(lib().sst_bfs(g.handle, src, ctypes.c_void_p(par.ctypes.data),
                         ctypes.c_void_p(dep.ctypes.data), HOST_PTR))
    return par, dep


def PR_S(g: SparseMatrixV, iters: int = 10, damping: float = 0.85, out=None):
    buf = _out(g, np.float64, out)
    p, flags = _ptr(buf)
    _check(lib().sst_pagerank(g.handle, iters, damping, p, flags))
    return buf


def BF(g: SparseMatrixV, src: int, out=None):
    """Shortest-path lengths from src over the edge values of a weighted
    graph (int32, unreachable = 2^31-1), as the reference drivers' BF."""
    buf = _out(g, np.int32, out)
    p, flags = _ptr(buf)
    _check(lib().sst_bf(g.handle, src, p, flags))
    return buf


def CC(g: SparseMatrixV, out=None):
    buf = _out(g, np.uint32, out)
    p, flags = _ptr(buf)
    _check(lib().sst_cc(g.handle, p, flags))
    return buf


def BC(g: SparseMatrixV, src: int, out=None):
    buf = _out(g, np.float64, out)
    p, flags = _ptr(buf)
    _check(lib().sst_bc(g.handle, src, p, flags))
    return buf


class TinySetV:
    """One sorted set of uint32 elements in [0, max_el) on the device: the
    reference's binary TinySetV (include/SSTGraph/TinySet.hpp:27-73) as one
    row of a device graph that keeps (0, 0)."""

    def __init__(self, max_el: int, **kw):
        self._g = SparseMatrixV(1, max(int(max_el), 1), keep_self_loops=True, **kw)

    def _pairs(self, els):
        if hasattr(els, "data_ptr"):
            import torch
            e = els.to(torch.int32).reshape(-1)
            return torch.stack([torch.zeros_like(e), e], 1).contiguous()
        e = np.asarray(els, np.uint32).reshape(-1)
        return np.stack([np.zeros_like(e), e], 1)

    def _check_range(self, els):
        e = np.asarray(els.cpu() if hasattr(els, "cpu") else els, np.int64).reshape(-1)
        if e.size and (e.min() < 0 or e.max() >= self._g.cols):
            raise SSTError(-1, "element out of range for this set")

    def has(self, e: int) -> bool:
        return self._g.has(0, int(e)) if 0 <= int(e) < self._g.cols else False

    def value(self, e: int) -> bool:
        return self.has(e)

    def insert(self, e: int):
        self._check_range([e])
        self._g.insert(0, int(e))

    def remove(self, e: int):
        if 0 <= int(e) < self._g.cols:
            self._g.remove(0, int(e))

    def insert_batch(self, els):
        self._check_range(els)
        self._g.insert_batch(self._pairs(els))

    def remove_batch(self, els):
        self._g.remove_batch(self._pairs(els))

    def get_n(self) -> int:
        return self._g.M()

    def get_size(self) -> int:
        return self._g.get_memory_size()

    def map(self, f, no_early_exit: bool = True):
        """f(element) in ascending order; without no_early_exit a true return
        stops the walk (TinySet_small.hpp:303-319)."""
        for x in self._g.neighbors(0):
            r = f(int(x))
            if not no_early_exit and r:
                return

    def elements(self) -> np.ndarray:
        return self._g.neighbors(0)

    def close(self):
        self._g.close()


def compact_widths(max_el: int):
    """get_thresholds (TinySet_small.hpp:227-263) for rows over max_el
    columns: rows with fewer than t[0] ids keep 4-byte keys, fewer than t[1]
    3-byte, fewer than t[2] 2-byte, the rest 1-byte."""
    t = np.zeros(3, np.uint32)
    _check(lib().sst_compact_widths(int(max_el), ctypes.c_void_p(t.ctypes.data)))
    return [int(x) for x in t]


class CompactGraph:
    """Read-only byte-width snapshot of a SparseMatrixV: each row keeps the
    low B bytes of its ids, bucketed by the high part, as the reference's
    TinySetV_small rows do (TinySet_small.hpp:204-293,852-881)."""

    def __init__(self, g: SparseMatrixV):
        h = ctypes.c_void_p()
        _check(lib().sst_compact_create(g.handle, ctypes.byref(h)))
        self._h = h
        self.rows = g.rows

    def close(self):
        if getattr(self, "_h", None):
            lib().sst_compact_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self) -> dict:
        sb, db, m = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        pw = np.zeros(4, np.uint64)
        _check(lib().sst_compact_info(self._h, ctypes.byref(sb), ctypes.byref(db),
                                      ctypes.byref(m), ctypes.c_void_p(pw.ctypes.data)))
        return {"storage_bytes": sb.value, "device_bytes": db.value, "edges": m.value,
                "rows_per_width": {i + 1: int(pw[i]) for i in range(4)}}

    def csr(self):
        m = self.info()["edges"]
        off = np.empty(self.rows + 1, np.uint64)
        cols = np.empty(max(m, 1), np.uint32)
        _check(lib().sst_compact_to_csr(self._h, ctypes.c_void_p(off.ctypes.data),
                                        ctypes.c_void_p(cols.ctypes.data), HOST_PTR))
        return off, cols[:m]

    def has_batch(self, edges, out=None):
        e, n = _pairs(edges)
        p, flags = _ptr(e)
        if out is None:
            if flags == DEVICE_PTR:
                import torch
                out = torch.empty(n, dtype=torch.uint8, device=e.device)
            else:
                out = np.empty(n, np.uint8)
        po, _ = _ptr(out)
        _check(lib().sst_compact_has_batch(self._h, p, n, po, flags))
        return out

    def pagerank(self, iters: int = 10, damping: float = 0.85, out=None):
        buf = np.empty(self.rows, np.float64) if out is None else out
        p, flags = _ptr(buf)
        _check(lib().sst_compact_pagerank(self._h, iters, damping, p, flags))
        return buf

    def bfs(self, src: int, out=None):
        """BFS depths from src (-1 unreached), as BFS(g, src, depths=True)."""
        buf = np.empty(self.rows, np.int32) if out is None else out
        p, flags = _ptr(buf)
        _check(lib().sst_compact_bfs(self._h, int(src), p, flags))
        return buf

    def cc(self, out=None):
        """Component labels (the component's smallest id), as CC(g)."""
        buf = np.empty(self.rows, np.uint32) if out is None else out
        p, flags = _ptr(buf)
        _check(lib().sst_compact_cc(self._h, p, flags))
        return buf

    def bc(self, src: int, out=None):
        """Single-source dependency scores, as BC(g, src) (within 1e-9)."""
        buf = np.empty(self.rows, np.float64) if out is None else out
        p, flags = _ptr(buf)
        _check(lib().sst_compact_bc(self._h, int(src), p, flags))
        return buf

    def tc(self, per_vertex: bool = False):
        """Triangle count (and per-vertex counts), as TC(g)."""
        total = ctypes.c_uint64()
        if per_vertex:
            pv = np.empty(self.rows, np.uint64)
            _check(lib().sst_compact_tc(self._h, ctypes.byref(total),
                                        ctypes.c_void_p(pv.ctypes.data), HOST_PTR))
            return total.value, pv
        _check(lib().sst_compact_tc(self._h, ctypes.byref(total), None, HOST_PTR))
        return total.value

    def sync(self):
        _check(lib().sst_compact_sync(self._h))

    def set_stream(self, stream_ptr: int | None):
        _check(lib().sst_compact_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)))


def read_graph_file(path: str):
    """(rows, pairs) of a .mtx / .adj file as the reference's readers give
    them (internal/helpers.hpp:379-657): pairs is an (n, 2) uint32 array."""
    rows, cnt, p = ctypes.c_uint32(), ctypes.c_uint64(), ctypes.c_void_p()
    _check(lib().sst_read_graph_file(os.fsencode(path), ctypes.byref(rows),
                                     ctypes.byref(cnt), ctypes.byref(p)))
    try:
        n = cnt.value
        buf = (ctypes.c_uint32 * max(2 * n, 1)).from_address(p.value)
        pairs = np.frombuffer(buf, np.uint32, 2 * n).reshape(n, 2).copy()
    finally:
        lib().sst_free(p)
    return rows.value, pairs


def load_graph_file(path: str, device: int = 0) -> "SparseMatrixV":
    """Device graph built from a .mtx / .adj file (sst_load_graph_file)."""
    cfg = sst_config(device, 0, 0, 0.0, 0.0, 0.0, 0)
    h = ctypes.c_void_p()
    _check(lib().sst_load_graph_file(os.fsencode(path), ctypes.byref(cfg), ctypes.byref(h)))
    return SparseMatrixV(0, _handle=h)


def _tuning_dict(t):
    return {"chunk_leaves": t.chunk_leaves, "pr_lanes": t.pr_lanes,
            "bfs_alpha": t.bfs_alpha, "pr_hot": t.pr_hot, "pr_ms": t.pr_ms,
            "bfs_ms": t.bfs_ms}


def autotune(g: SparseMatrixV) -> dict:
    """Time the traversal knobs on g and keep the fastest (sst_autotune)."""
    t = sst_tuning()
    _check(lib().sst_autotune(g.handle, ctypes.byref(t)))
    return _tuning_dict(t)


def get_tuning(g: SparseMatrixV) -> dict:
    t = sst_tuning()
    _check(lib().sst_get_tuning(g.handle, ctypes.byref(t)))
    return _tuning_dict(t)


def set_tuning(g: SparseMatrixV, chunk_leaves=32, pr_lanes=8, bfs_alpha=20, pr_hot=0):
    t = sst_tuning(chunk_leaves, pr_lanes, bfs_alpha, 0.0, 0.0, pr_hot)
    _check(lib().sst_set_tuning(g.handle, ctypes.byref(t)))


def _sources(srcs, flags, like):
    """Source ids where the call's flags say the arrays are (host or the
    output tensor's device)."""
    if hasattr(srcs, "data_ptr"):
        if flags == DEVICE_PTR and srcs.is_cuda:
            srcs = srcs.contiguous()
            return srcs, ctypes.c_void_p(srcs.data_ptr())
        srcs = srcs.cpu().numpy()
    a = np.ascontiguousarray(np.asarray(srcs).astype(np.uint32).ravel())
    if flags == DEVICE_PTR:
        import torch
        t = torch.from_numpy(a.view(np.int32)).to(like.device)
        return t, ctypes.c_void_p(t.data_ptr())
    return a, ctypes.c_void_p(a.ctypes.data)


def _count(srcs):
    return int(srcs.numel()) if hasattr(srcs, "numel") else int(np.asarray(srcs).size)


def BFS_multi(g: SparseMatrixV, srcs, out=None):
    """Depths from each of k <= 64 sources in one traversal: (k, rows)
    int32, row i for srcs[i], -1 unreached."""
    k = _count(srcs)
    if out is None:
        out = np.empty((k, g.rows), np.int32)
    p, flags = _ptr(out)
    keep, sp = _sources(srcs, flags, out)
    _check(lib().sst_bfs_multi(g.handle, sp, k, p, flags))
    return out


def BC_multi(g: SparseMatrixV, srcs, out=None):
    """BC(g, s) for each of k <= 64 sources, every launch covering all of
    them: (k, rows) float64, row i equal to BC(g, srcs[i])."""
    k = _count(srcs)
    if out is None:
        out = np.empty((k, g.rows), np.float64)
    p, flags = _ptr(out)
    keep, sp = _sources(srcs, flags, out)
    _check(lib().sst_bc_multi(g.handle, sp, k, p, flags))
    return out


def TC(g: SparseMatrixV, per_vertex: bool = False):
    total = ctypes.c_uint64()
    if per_vertex:
        pv = np.empty(g.rows, np.uint64)
        _check(lib().sst_tc(g.handle, ctypes.byref(total), ctypes.c_void_p(pv.ctypes.data), HOST_PTR))
        return total.value, pv
    _check(lib().sst_tc(g.handle, ctypes.byref(total), None, HOST_PTR))
    return total.value


def TC_vertices(g: SparseMatrixV, vertices) -> np.ndarray:
    """triangles containing each listed vertex"""
    v = np.ascontiguousarray(vertices, np.uint32)
    out = np.empty(len(v), np.uint64)
    _check(lib().sst_tc_vertices(g.handle, ctypes.c_void_p(v.ctypes.data), len(v),
                                 ctypes.c_void_p(out.ctypes.data), HOST_PTR))
    return out


class Server:
    """Serving loop over a device-resident graph (include/sstgraph.h,
    sst_server_*): submit updates and queries, wait for results."""

    def __init__(self, g: SparseMatrixV, query_slots: int = 2,
                 hbm_budget_bytes: int = 0, max_coalesce: int = 0):
        self.g = g
        cfg = sst_server_config(query_slots, hbm_budget_bytes, max_coalesce)
        h = ctypes.c_void_p()
        _check(lib().sst_server_create(g.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}
        s = ctypes.c_uint32()
        _check(lib().sst_server_slots(h, ctypes.byref(s)))
        self.slots = s.value

    def _submit(self, req, keep):
        t = ctypes.c_uint64()
        _check(lib().sst_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = keep
        return t.value

    def insert(self, pairs) -> int:
        p = np.ascontiguousarray(np.asarray(pairs, np.uint32).reshape(-1, 2))
        return self._submit(sst_request(REQ_INSERT, p.ctypes.data, len(p), 0, 0, 0.0, None), (p, None))

    def remove(self, pairs) -> int:
        p = np.ascontiguousarray(np.asarray(pairs, np.uint32).reshape(-1, 2))
        return self._submit(sst_request(REQ_REMOVE, p.ctypes.data, len(p), 0, 0, 0.0, None), (p, None))

    def bfs(self, src) -> int:
        out = np.empty(self.g.rows, np.int32)
        return self._submit(sst_request(REQ_BFS, None, 0, src, 0, 0.0, out.ctypes.data), (None, out))

    def pagerank(self, iters=5, damping=0.85) -> int:
        out = np.empty(self.g.rows, np.float64)
        return self._submit(sst_request(REQ_PAGERANK, None, 0, 0, iters, damping,
                                        out.ctypes.data), (None, out))

    def tc_vertices(self, vertices) -> int:
        v = np.ascontiguousarray(vertices, np.uint32)
        out = np.empty(len(v), np.uint64)
        return self._submit(sst_request(REQ_TC_VERTICES, v.ctypes.data, len(v), 0, 0, 0.0,
                                        out.ctypes.data), (v, out))

    def wait(self, ticket, timeout_ms=600000):
        """-> (result array or None, info dict)"""
        info = sst_request_info()
        st = lib().sst_server_wait(self._h, ticket, timeout_ms, ctypes.byref(info))
        keep = self._keep.pop(ticket, (None, None))
        _check(st)
        return keep[1], {"epoch": info.epoch, "queue_ms": info.queue_ms,
                         "run_ms": info.run_ms, "total_ms": info.total_ms}

    def stats(self):
        e, p, u = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().sst_server_stats(self._h, ctypes.byref(e), ctypes.byref(p), ctypes.byref(u)))
        return {"epoch": e.value, "passes": p.value, "update_edges": u.value}

    def close(self):
        if self._h:
            lib().sst_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def TouchAll(g: SparseMatrixV) -> int:
    r = ctypes.c_uint64()
    _check(lib().sst_touch_all(g.handle, ctypes.byref(r)))
    return r.value


# ---- device generators ------------------------------------------------------
def gen_rmat(scale, count, a=0.57, b=0.19, c=0.19, seed=1, first=0, out=None):
    if out is None:
        out = np.empty((count, 2), np.uint32)
    p, flags = _ptr(out)
    _check(lib().sst_gen_rmat(scale, a, b, c, seed, first, count, p, flags))
    return out


def gen_er(n, count, seed=4, first=0, out=None):
    if out is None:
        out = np.empty((count, 2), np.uint32)
    p, flags = _ptr(out)
    _check(lib().sst_gen_er(n, seed, first, count, p, flags))
    return out


def gen_ref_rmat(nn, count, a=0.5, b=0.1, c=0.1, first=0, out=None):
    if out is None:
        out = np.empty((count, 2), np.uint32)
    p, flags = _ptr(out)
    _check(lib().sst_gen_ref_rmat(nn, a, b, c, first, count, p, flags))
    return out
