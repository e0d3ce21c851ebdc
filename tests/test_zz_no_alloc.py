"""PageRank entry point that allocates nothing (sst_pagerank_noalloc).

Callers that cannot allocate -- a serving loop under a fixed HBM budget, or
a host program whose other GPU streams would stall on the device-wide
synchronisation of cudaMalloc / cudaFree -- use this variant: its scratch
is a fixed array inside the library.  The test calls it through the C ABI
twice in a row (the second call must not see the first call's leftovers)
and compares each result with sst_pagerank, within the PageRank tolerance
of the other tests (1e-9 relative L-inf).  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL = 1e-9


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_noalloc_matches_pagerank_twice(sg):
    import torch
    n = 1 << 15
    pairs = oracle.symmetrize(oracle.rmat(15, 16 * n, seed=1))
    g = sg.SparseMatrixV(n)
    g.insert_batch(pairs)
    ref = sg.PR_S(g, 10)
    o = oracle.OracleGraph(n)
    o.insert_batch(pairs)
    want = o.pagerank(10)
    L = sg.lib()
    outs = [torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
            for _ in range(2)]
    torch.cuda.synchronize()
    free = []
    for call in range(2):
        free.append(torch.cuda.mem_get_info()[0])
        st = L.sst_pagerank_noalloc(g.handle, 10, 0.85, ctypes.c_void_p(outs[call].data_ptr()))
        assert st == 0, L.sst_last_error_message().decode()
        g.sync()
        got = outs[call].cpu().numpy()
        assert relerr(got, ref) <= REL, f"call {call} vs sst_pagerank"
        assert relerr(got, want) <= REL, f"call {call} vs the oracle"
    # after the first call (which may load the kernels), a call leaves the
    # device's free memory exactly as it found it
    assert torch.cuda.mem_get_info()[0] == free[1]
    # a smaller graph after a larger one: the shared array is re-initialised
    h = sg.SparseMatrixV(1000)
    h.insert_batch(oracle.symmetrize(oracle.er(1000, 3000, seed=2)))
    out = torch.empty(1000, dtype=torch.float64, device="cuda")
    assert L.sst_pagerank_noalloc(h.handle, 20, 0.85, ctypes.c_void_p(out.data_ptr())) == 0
    h.sync()
    assert relerr(out.cpu().numpy(), sg.PR_S(h, 20)) <= REL


def test_noalloc_rejects_oversized_graph(sg):
    import torch
    g = sg.SparseMatrixV((1 << 18) + 1)
    out = torch.empty((1 << 18) + 1, dtype=torch.float64, device="cuda")
    L = sg.lib()
    st = L.sst_pagerank_noalloc(g.handle, 5, 0.85, ctypes.c_void_p(out.data_ptr()))
    assert st == -1
    assert b"262144" in L.sst_last_error_message()


def test_noalloc_rejects_non_square_graph(sg):
    import torch
    g = sg.SparseMatrixV(8, 1 << 20)
    g.insert_batch(np.array([[1, (1 << 20) - 1]], dtype=np.uint32))
    out = torch.empty(8, dtype=torch.float64, device="cuda")
    L = sg.lib()
    st = L.sst_pagerank_noalloc(g.handle, 5, 0.85, ctypes.c_void_p(out.data_ptr()))
    assert st == -1
    assert b"rows as columns" in L.sst_last_error_message()
