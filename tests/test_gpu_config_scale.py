"""Parity at the benchmark configurations' own sizes, device vs the CPU
oracle on the same seeded inputs.

* Static analytics (RMAT scale 22, 8 * 2^22 generated edges, seed 3,
  symmetrised; Erdos-Renyi with 2^22 vertices and average degree 16,
  seed 4): BFS depths from three sources, the CC labelling and triangle
  counts (total and per vertex) bit-exact; PageRank (20 iterations) and BC
  from vertex 0 within 1e-9 relative L-inf.  The reference drivers run these
  algorithms at internal/test.hpp:848-958.
* Multi-source traversals on the RMAT scale-24 base graph (seed 5): all 64
  BFS rows bit-exact and all 16 BC rows within 1e-9, sources drawn
  uniformly.
* Dynamic updates on the same scale-24 graph: insert batches of 1e2 .. 1e7
  RMAT edges (seed 6) of which 5% are edges already present, each followed
  by a delete batch of as many edges sampled uniformly from the graph; the
  whole CSR equal after every batch (internal/test.hpp:636-689 drives the
  reference's batches the same way).

The oracle's serial algorithms run one source per thread (ctypes releases
the GIL), so the multi-source rows finish in seconds.
"""
import concurrent.futures as cf

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL = 1e-9
RMAT = dict(a=0.57, b=0.19, c=0.19)


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def pool():
    return cf.ThreadPoolExecutor(max_workers=16)


def same_csr(g, o):
    assert g.M() == o.M()
    og, cg = g.csr()
    oo, co = o.csr()
    assert np.array_equal(og, oo)
    assert np.array_equal(cg, co)


def build_pair(sg, n, pairs):
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(pairs)
    o.insert_batch(pairs)
    return g, o


# ------------------------------------------------------- static analytics
def static_graphs():
    n = 1 << 22
    yield "rmat22", n, lambda: oracle.symmetrize(oracle.rmat(22, 8 * n, seed=3, **RMAT))
    yield "er22", n, lambda: oracle.symmetrize(oracle.er(n, 8 * n, seed=4))


@pytest.fixture(scope="module", params=[x[0] for x in static_graphs()])
def static_pair(request, sg):
    name, n, make = next(x for x in static_graphs() if x[0] == request.param)
    g, o = build_pair(sg, n, make())
    yield name, g, o
    g.close()
    del o


def test_static_structure(sg, static_pair):
    _, g, o = static_pair
    same_csr(g, o)


def test_static_bfs_three_sources(sg, static_pair):
    _, g, o = static_pair
    deg = o.degrees()
    srcs = [0, int(np.argmax(deg)), int(np.nonzero(deg)[0][len(np.nonzero(deg)[0]) // 2])]
    with pool() as ex:
        want = list(ex.map(o.bfs, srcs))
    for s, w in zip(srcs, want):
        assert np.array_equal(sg.BFS(g, s, depths=True), w), s


def test_static_cc(sg, static_pair):
    _, g, o = static_pair
    assert np.array_equal(sg.CC(g), o.cc())


def test_static_tc(sg, static_pair):
    _, g, o = static_pair
    t, pv = sg.TC(g, per_vertex=True)
    te, pve = o.tc(per_vertex=True)
    assert t == te
    assert np.array_equal(pv, pve)
    assert sg.TC(g) == te  # the count-only kernel


def test_static_pagerank_20(sg, static_pair):
    _, g, o = static_pair
    assert relerr(sg.PR_S(g, 20), o.pagerank(20)) <= REL


def test_static_bc(sg, static_pair):
    _, g, o = static_pair
    assert relerr(sg.BC(g, 0), o.bc(0)) <= REL


# ----------------------------------------------- scale-24 base graph (C3/C4)
@pytest.fixture(scope="module")
def base24(sg):
    n = 1 << 24
    g, o = build_pair(sg, n, oracle.symmetrize(oracle.rmat(24, 8 * n, seed=5, **RMAT)))
    yield n, g, o
    g.close()
    del o


def test_multi_source_rows_64_bfs_16_bc(sg, base24):
    """Runs before the update stream below, on the symmetric base graph."""
    n, g, o = base24
    rng = np.random.default_rng(17)
    srcs = rng.integers(0, n, 64).astype(np.uint32)
    got = sg.BFS_multi(g, srcs)
    with pool() as ex:
        want = list(ex.map(lambda s: o.bfs(int(s)), srcs))
    for i, w in enumerate(want):
        assert np.array_equal(got[i], w), (i, int(srcs[i]))
    del got, want
    bsrc = rng.integers(0, n, 16).astype(np.uint32)
    got = sg.BC_multi(g, bsrc)
    with pool() as ex:
        want = list(ex.map(lambda s: o.bc(int(s)), bsrc))
    for i, w in enumerate(want):
        assert relerr(got[i], w) <= REL, (i, int(bsrc[i]))


def test_hub_source_bc_and_snapshot(sg, base24):
    """BC and BFS from vertex 0 (the largest RMAT hub) on the scale-24
    graph and on its byte-width snapshot against the oracle; runs before
    the update stream below, on the symmetric base graph."""
    n, g, o = base24
    want_bc, want_d = o.bc(0), o.bfs(0)
    scale = max(np.max(np.abs(want_bc)), 1e-300)
    assert np.max(np.abs(sg.BC(g, 0) - want_bc)) / scale <= REL
    assert np.array_equal(sg.BFS(g, 0, depths=True), want_d)
    c = sg.CompactGraph(g)
    try:
        assert np.array_equal(c.bfs(0), want_d)
        assert np.max(np.abs(c.bc(0) - want_bc)) / scale <= REL
    finally:
        c.close()


def test_update_stream_1e2_to_1e7(sg, base24):
    """Each insert batch: 95% new RMAT edges and 5% sampled existing edges;
    each delete batch: as many sampled existing edges; the CSR after every
    batch equals the oracle's.  The device's sampler draws the same edges as
    the oracle's from the same graph."""
    n, g, o = base24
    first = 0
    for k, b in enumerate([10 ** e for e in range(2, 8)]):
        dup = b // 20
        ins = np.concatenate([oracle.rmat(24, b - dup, seed=6, first=first, **RMAT),
                              o.sample_edges(dup, seed=8, first=first)])
        first += b
        g.insert_batch(ins)
        o.insert_batch(ins)
        same_csr(g, o)
        rem = o.sample_edges(b, seed=7, first=first)
        assert np.array_equal(g.sample_edges(b, seed=7, first=first), rem), b
        g.remove_batch(rem)
        o.remove_batch(rem)
        same_csr(g, o)
