"""The CPU oracle's algorithm definitions against independent
implementations: networkx (BFS depths, components, triangles, PageRank at
convergence, Brandes dependencies from networkx's shortest-path DAG) and a
numpy restatement of the fixed-iteration PageRank.  The reference's
algorithm library (EdgeMapVertexMap) is absent, so these pin the definitions
the oracle states in sst_oracle.c."""
import os

import numpy as np
import pytest

import oracle

nx = pytest.importorskip("networkx")

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def graphs():
    d = np.load(os.path.join(GOLD, "examples_mtx.npz"))
    yield "star", int(d["star_rows"]), d["star_edges"]
    yield "johnson8-2-4", int(d["johnson8_2_4_rows"]), d["johnson8_2_4_edges"]
    yield "rmat10", 1 << 10, oracle.symmetrize(oracle.rmat(10, 8 << 10, seed=1))
    yield "er", 800, oracle.symmetrize(oracle.er(800, 1200, seed=4))


@pytest.fixture(params=[x[0] for x in graphs()])
def case(request):
    name, n, e = next(x for x in graphs() if x[0] == request.param)
    o = oracle.OracleGraph(n)
    o.insert_batch(e)
    G = nx.Graph()
    G.add_nodes_from(range(n))
    off, cols = o.csr()
    for v in range(n):
        for w in cols[off[v]:off[v + 1]]:
            G.add_edge(v, int(w))
    return o, G, n


def test_bfs_depths(case):
    o, G, n = case
    for src in (0, n // 2):
        exp = np.full(n, -1, np.int32)
        for v, d in nx.single_source_shortest_path_length(G, src).items():
            exp[v] = d
        assert np.array_equal(o.bfs(src), exp)


def test_components(case):
    o, G, n = case
    exp = np.empty(n, np.uint32)
    for comp in nx.connected_components(G):
        exp[list(comp)] = min(comp)
    assert np.array_equal(o.cc(), exp)


def test_triangles(case):
    o, G, n = case
    tri = nx.triangles(G)
    exp = np.array([tri[v] for v in range(n)], np.uint64)
    total, pv = o.tc(per_vertex=True)
    assert total == sum(tri.values()) // 3
    assert np.array_equal(pv, exp)


def pr_numpy(o, n, iters, d=0.85):
    off, cols = o.csr()
    deg = np.diff(off).astype(np.float64)
    r = np.full(n, 1.0 / n)
    src = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
    for _ in range(iters):
        c = np.where(deg > 0, r / np.maximum(deg, 1), 0.0)
        s = np.zeros(n)
        np.add.at(s, src, c[cols])
        r = (1 - d) / n + d * s
    return r


def test_pagerank_definition(case):
    o, G, n = case
    for it in (1, 10, 20):
        a, b = o.pagerank(it), pr_numpy(o, n, it)
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    # no vertex without edges: the fixed point is networkx's PageRank
    if min(dict(G.degree()).values()) > 0 and nx.is_connected(G):
        ref = nx.pagerank(G, alpha=0.85, tol=1e-15, max_iter=2000)
        exp = np.array([ref[v] for v in range(n)])
        assert np.max(np.abs(o.pagerank(300) - exp)) <= 1e-9 * np.max(exp)


def test_bc_dependencies(case):
    o, G, n = case
    from networkx.algorithms.centrality.betweenness import (
        _single_source_shortest_path_basic,
    )
    for src in (0, 1):
        S, P, sigma, _ = _single_source_shortest_path_basic(G, src)
        delta = dict.fromkeys(S, 0.0)
        for w in reversed(S):
            for v in P[w]:
                delta[v] += sigma[v] / sigma[w] * (1.0 + delta[w])
        exp = np.zeros(n)
        for v, x in delta.items():
            exp[v] = x
        got = o.bc(src)
        assert np.max(np.abs(got - exp)) <= 1e-9 * max(1.0, np.max(np.abs(exp)))
