"""Device BFS / PageRank / CC / BC / TC vs the CPU oracle.
Depths, CC labels and triangle counts bit-exact; PR and BC within 1e-9
relative (L-inf over the vector, normalised by its largest entry)."""
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


def graphs():
    n = 1 << 13
    yield "rmat13", n, oracle.symmetrize(oracle.rmat(13, 16 * n, seed=1))
    yield "er", 5000, oracle.symmetrize(oracle.er(5000, 5000 * 4, seed=4))
    yield "star+isolated", 50, np.array([[0, i] for i in range(1, 30)] + [[i, 0] for i in range(1, 30)], np.uint32)


@pytest.fixture(scope="module", params=[x[0] for x in graphs()])
def pair(request, sg):
    name, n, edges = next(x for x in graphs() if x[0] == request.param)
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(edges)
    o.insert_batch(edges)
    return g, o


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_bfs(sg, pair):
    g, o = pair
    for src in (0, 1, g.rows - 1):
        par, dep = sg.BFS_both(g, src)
        exp = o.bfs(src)
        assert np.array_equal(dep, exp)
        # parents: a neighbour one level up
        assert par[src] == src
        for v in np.nonzero(exp > 0)[0][:2000]:
            p = par[v]
            assert exp[p] == exp[v] - 1 and o.has(int(v), int(p))
        assert np.all(par[exp < 0] == -1)


def test_pagerank(sg, pair):
    g, o = pair
    for iters in (1, 10, 20):
        assert relerr(sg.PR_S(g, iters), o.pagerank(iters)) <= REL


def test_cc(sg, pair):
    g, o = pair
    assert np.array_equal(sg.CC(g), o.cc())


def test_bc(sg, pair):
    g, o = pair
    for src in (0, 3):
        assert relerr(sg.BC(g, src), o.bc(src)) <= REL


def test_tc(sg, pair):
    g, o = pair
    t, pv = sg.TC(g, per_vertex=True)
    te, pve = o.tc(per_vertex=True)
    assert t == te
    assert np.array_equal(pv, pve)
    assert sg.TC(g) == te  # the count-only kernel


def test_tc_lists_longer_than_the_set(sg):
    """A vertex whose list of higher-ranked neighbours outgrows the
    shared-memory set (more than 1024 entries) is counted by binary search:
    a clique of 1030 vertices, each also tied to a hub of larger degree, so
    clique vertex i keeps the 1029 - i clique vertices above it and the
    hub."""
    k, n = 1030, 1030 + 1 + 1200
    hub = k
    rows, cols = np.triu_indices(k, 1)
    e = [np.stack([rows, cols], 1), np.stack([np.full(k, hub), np.arange(k)], 1),
         np.stack([np.full(1200, hub), np.arange(k + 1, n)], 1)]
    pairs = oracle.symmetrize(np.concatenate(e).astype(np.uint32))
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(pairs)
    o.insert_batch(pairs)
    t, pv = sg.TC(g, per_vertex=True)
    te, pve = o.tc(per_vertex=True)
    assert t == te and sg.TC(g) == te
    assert np.array_equal(pv, pve)
    g.close()


def test_traversals_refuse_non_square_graph(sg):
    """A graph with more columns than rows would send column ids past the
    traversals' per-vertex arrays: every traversal refuses it on the host,
    before any launch, with SST_EINVAL."""
    g = sg.SparseMatrixV(8, 1 << 20)
    g.insert_batch(np.array([[1, (1 << 20) - 1], [2, 3]], dtype=np.uint32))
    calls = [
        ("BFS", lambda: sg.BFS(g, 1, depths=True)),
        ("PR_S", lambda: sg.PR_S(g, 5)),
        ("CC", lambda: sg.CC(g)),
        ("BC", lambda: sg.BC(g, 1)),
        ("TC", lambda: sg.TC(g, per_vertex=True)),
        ("BFS_multi", lambda: sg.BFS_multi(g, [1, 2])),
        ("BC_multi", lambda: sg.BC_multi(g, [1, 2])),
        ("TC_vertices", lambda: sg.TC_vertices(g, [1, 2])),
        ("autotune", lambda: sg.autotune(g)),
        ("CompactGraph.pagerank", lambda: sg.CompactGraph(g).pagerank(5)),
        ("Server", lambda: sg.Server(g)),
    ]
    for name, call in calls:
        with pytest.raises(sg.SSTError) as e:
            call()
        assert e.value.status == -1, name
        assert "rows as columns" in str(e.value), name
    # the graph itself is still usable
    assert g.has(1, (1 << 20) - 1) and g.M() == 2
