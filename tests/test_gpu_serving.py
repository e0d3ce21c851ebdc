"""Serving loop: a mixed stream of update and query requests served
concurrently (updates coalesced per writer pass, queries on snapshots in
several slots).  Each query's result must equal the same query run alone on
the graph after exactly the update requests its snapshot covers (its epoch):
bit-exact for BFS depths and triangle counts, PageRank within 1e-9."""
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def test_results_same_alone_and_in_the_mix(sg):
    scale = 12
    n = 1 << scale
    base = oracle.symmetrize(oracle.rmat(scale, 8 * n, seed=21))
    rng = np.random.default_rng(5)
    g = sg.SparseMatrixV(n)
    g.insert_batch(base)
    srv = sg.Server(g, query_slots=3)
    assert srv.slots == 3

    updates = []       # (kind, pairs) in submission order
    queries = []       # (ticket, kind, arg)
    tickets = []
    inserted = []
    for wave in range(8):
        for _ in range(4):
            if inserted and rng.random() < 0.35:
                # removals keep the graph symmetric: the traversals pull over
                # out-lists, which are the in-lists only on a symmetric graph
                src = np.concatenate(inserted)
                p = oracle.symmetrize(src[rng.integers(0, len(src), int(rng.integers(1, 500)))])
                updates.append(("remove", p))
                tickets.append(("u", srv.remove(p)))
            else:
                k = int(rng.integers(1, 3000))
                p = oracle.symmetrize(oracle.rmat(scale, k, seed=22, first=len(updates) * 5000))
                inserted.append(p)
                updates.append(("insert", p))
                tickets.append(("u", srv.insert(p)))
        for _ in range(3):
            kind = ["bfs", "pr", "tc"][int(rng.integers(0, 3))]
            if kind == "bfs":
                src = int(rng.integers(0, n))
                t = srv.bfs(src)
            elif kind == "pr":
                src = None
                t = srv.pagerank(5)
            else:
                src = rng.integers(0, n, 200).astype(np.uint32)
                t = srv.tc_vertices(src)
            queries.append((t, kind, src))
        time.sleep(0.002)

    results = {}
    for kind, t in tickets:
        srv.wait(t)
    for t, kind, arg in queries:
        results[t] = srv.wait(t)
    stats = srv.stats()
    srv.close()
    assert stats["epoch"] == len(updates)

    # the live graph holds all updates, in order
    o = oracle.OracleGraph(n)
    o.insert_batch(base)
    for kind, p in updates:
        (o.insert_batch if kind == "insert" else o.remove_batch)(p)
    assert np.array_equal(g.csr()[1], o.csr()[1])

    epochs = sorted({results[t][1]["epoch"] for t, _, _ in queries})
    alone = {}
    h = sg.SparseMatrixV(n)
    h.insert_batch(base)
    applied = 0
    for ep in epochs:
        while applied < ep:
            kind, p = updates[applied]
            (h.insert_batch if kind == "insert" else h.remove_batch)(p)
            applied += 1
        for t, kind, arg in queries:
            if results[t][1]["epoch"] != ep:
                continue
            if kind == "bfs":
                alone[t] = sg.BFS(h, arg, depths=True)
            elif kind == "pr":
                alone[t] = sg.PR_S(h, 5)
            else:
                alone[t] = sg.TC_vertices(h, arg)
    for t, kind, arg in queries:
        got = results[t][0]
        if kind == "pr":
            assert np.max(np.abs(got - alone[t])) <= 1e-9 * np.max(np.abs(alone[t]))
        else:
            assert np.array_equal(got, alone[t]), (kind, results[t][1])
    assert len(epochs) >= 2  # queries saw different prefixes of the stream


def test_tc_vertices_matches_oracle(sg):
    n = 1 << 11
    e = oracle.symmetrize(oracle.rmat(11, 8 * n, seed=3))
    g = sg.SparseMatrixV(n)
    g.insert_batch(e)
    o = oracle.OracleGraph(n)
    o.insert_batch(e)
    _, pv = o.tc(per_vertex=True)
    vs = np.arange(n, dtype=np.uint32)
    assert np.array_equal(sg.TC_vertices(g, vs), pv)


def test_budget_limits_slots(sg):
    n = 1 << 12
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(oracle.rmat(12, 8 * n, seed=4)))
    big = g.get_memory_size()  # the live graph, update scratch included
    # a slot costs one snapshot (vertex table, slab, traversal buffers):
    # admission grows with the budget and stops at the request
    counts = []
    for extra in (big // 8, big // 2, 2 * big, 64 * big):
        try:
            srv = sg.Server(g, query_slots=8, hbm_budget_bytes=big + extra)
        except sg.SSTError:  # room for no snapshot at all
            counts.append(0)
            continue
        counts.append(srv.slots)
        srv.close()
    assert counts == sorted(counts) and counts[-1] == 8 and counts[0] < 8
    assert all(0 <= c <= 8 for c in counts)
    with pytest.raises(sg.SSTError):  # no room for one snapshot
        sg.Server(g, query_slots=2, hbm_budget_bytes=big + 1024)
