"""Byte-width snapshot (sst_compact_*) against the graph it was taken from
and the layout restatement (oracle/compact.py): the decoded CSR bit-exact,
rows per key width and storage bytes as the restatement predicts,
membership answers equal, PageRank equal bit for bit to the PMA
PageRank (the same fixed-point arithmetic over the same rows), and, on
symmetric graphs, BFS depths, CC labels and triangle counts equal to the
graph's and the oracle's and BC within 1e-9 relative of the oracle's."""
import numpy as np
import pytest

import oracle
from oracle import compact as oc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def rows_at(rng, n, sizes):
    """(row, col) pairs: row r gets sizes[r] distinct columns below n, the
    largest id among them for the odd rows."""
    out = []
    for r, k in sizes.items():
        cols = rng.choice(n, size=k, replace=False).astype(np.uint32)
        if r % 2:
            cols[0] = n - 1
        out.append(np.stack([np.full(k, r, np.uint32), cols], 1))
    return np.concatenate(out)


def check_snapshot(sg, g, n):
    c = sg.CompactGraph(g)
    try:
        off, cols = c.csr()
        goff, gcols = g.csr()
        assert np.array_equal(off, goff) and np.array_equal(cols, gcols)
        deg = g.degrees()
        info = c.info()
        assert info["edges"] == g.M()
        assert info["rows_per_width"] == oc.rows_per_width(deg, n)
        assert info["storage_bytes"] == oc.storage_bytes(deg, n)
        rng = np.random.default_rng(5)
        m = len(gcols)
        rows = np.repeat(np.arange(n, dtype=np.uint32), np.diff(goff).astype(np.int64))
        pick = rng.integers(0, max(m, 1), min(m, 20000)) if m else np.zeros(0, np.int64)
        q = [np.stack([rows[pick], gcols[pick]], 1) if m else np.zeros((0, 2), np.uint32),
             rng.integers(0, n, (20000, 2)).astype(np.uint32),
             np.array([[0, n - 1], [1, n - 1], [n - 1, 0], [n, 0], [0, n],
                       [1, 0xFFFFFFFF]], np.uint32)]
        q = np.concatenate(q).astype(np.uint32)
        assert np.array_equal(c.has_batch(q), g.has_batch(q))
        for iters in (1, 10):
            a, b = c.pagerank(iters), sg.PR_S(g, iters)
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), iters
        return info
    finally:
        c.close()


def test_every_width_and_directory(sg):
    # 2^20 columns: 4-byte keys below 4 ids, 3-byte below 256, 2-byte (16
    # buckets) below 65,536, 1-byte (4,096 buckets) from there
    n = 1 << 20
    assert oc.widths(n) == [4, 256, 65536]
    rng = np.random.default_rng(1)
    sizes = {1: 70000, 2: 65536, 3: 65535, 4: 256, 5: 255, 6: 4, 7: 3, 8: 1,
             9: 5000, 11: 300}
    hubs = rows_at(rng, n, sizes)
    rand = rng.integers(0, n, (300000, 2)).astype(np.uint32)
    g = sg.SparseMatrixV(n)
    g.insert_batch(np.concatenate([hubs, rand]))
    info = check_snapshot(sg, g, n)
    assert all(info["rows_per_width"][b] > 0 for b in (1, 2, 3, 4))
    g.close()


def test_rmat_symmetric(sg):
    # scale 16: 2-byte keys from 4 ids, 1-byte (256 buckets) from 4,096
    n = 1 << 16
    e = oracle.symmetrize(oracle.rmat(16, 16 * n, seed=1))
    g = sg.SparseMatrixV(n)
    g.insert_batch(e)
    info = check_snapshot(sg, g, n)
    assert info["storage_bytes"] < g.get_memory_size()
    g.close()


def test_empty_tiny_and_after_updates(sg):
    g = sg.SparseMatrixV(1000)
    check_snapshot(sg, g, 1000)
    g.insert_batch(np.array([[3, 999]], np.uint32))
    check_snapshot(sg, g, 1000)
    g.insert_batch(oracle.symmetrize(oracle.rmat(10, 8000, seed=4)))
    g.remove_batch(oracle.symmetrize(oracle.rmat(10, 2000, seed=4)))
    check_snapshot(sg, g, 1000)
    g.close()


def test_snapshot_is_independent_of_later_updates(sg):
    n = 4096
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(oracle.rmat(12, 30000, seed=6)))
    before = g.csr()
    c = sg.CompactGraph(g)
    g.insert_batch(oracle.symmetrize(oracle.rmat(12, 30000, seed=7)))
    off, cols = c.csr()
    assert np.array_equal(off, before[0]) and np.array_equal(cols, before[1])
    c.close()
    g.close()


def test_device_arrays(sg):
    torch = pytest.importorskip("torch")
    n = 1 << 12
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(oracle.rmat(12, 20000, seed=8)))
    c = sg.CompactGraph(g)
    q = torch.randint(0, n, (5000, 2), dtype=torch.int32, device="cuda")
    assert torch.equal(c.has_batch(q).cpu(), g.has_batch(q).cpu())
    pr = torch.empty(n, dtype=torch.float64, device="cuda")
    c.pagerank(10, out=pr)
    assert np.array_equal(pr.cpu().numpy().view(np.uint64),
                          sg.PR_S(g, 10).view(np.uint64))
    c.close()
    g.close()


def test_weighted_graph_refused(sg):
    g = sg.SparseMatrixV(8, weighted=True)
    with pytest.raises(sg.SSTError):
        sg.CompactGraph(g)
    g.close()


def check_traversals(sg, g, n, srcs):
    """BFS, CC, BC and TC on the snapshot = on the live graph = the oracle."""
    off, cols = g.csr()
    o = oracle.OracleGraph(n)
    rows = np.repeat(np.arange(n, dtype=np.uint32), np.diff(off).astype(np.int64))
    o.insert_batch(np.stack([rows, cols], 1))
    c = sg.CompactGraph(g)
    try:
        for s in srcs:
            want = o.bfs(int(s))
            assert np.array_equal(c.bfs(int(s)), want), s
            assert np.array_equal(sg.BFS(g, int(s), depths=True), want), s
        want = o.cc()
        assert np.array_equal(c.cc(), want)
        assert np.array_equal(sg.CC(g), want)
        for src in srcs[:3]:
            want = o.bc(int(src))
            err = np.max(np.abs(c.bc(int(src)) - want)) / max(np.max(np.abs(want)), 1e-300)
            assert err <= 1e-9, src
        t, pv = o.tc(per_vertex=True)
        ct, cpv = c.tc(per_vertex=True)
        assert ct == t and c.tc() == t
        assert np.array_equal(cpv, pv)
    finally:
        c.close()


def test_traversals_rmat(sg):
    n = 1 << 16
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(oracle.rmat(16, 16 * n, seed=1)))
    deg = g.degrees()
    check_traversals(sg, g, n, [0, int(np.argmax(deg)), int(np.nonzero(deg)[0][-1]), 12345])
    g.close()


def test_traversals_every_width_symmetric(sg):
    """Rows of every key width with bucket directories (2^20 columns), made
    symmetric; several components."""
    n = 1 << 20
    rng = np.random.default_rng(3)
    sizes = {1: 70000, 2: 65536, 3: 300, 4: 256, 5: 4, 6: 3, 9: 5000}
    hubs = rows_at(rng, n, sizes)
    rand = rng.integers(0, n, (200000, 2)).astype(np.uint32)
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(np.concatenate([hubs, rand])))
    info = check_snapshot(sg, g, n)
    assert all(info["rows_per_width"][b] > 0 for b in (1, 2, 3, 4))
    check_traversals(sg, g, n, [1, 2, 9, 5, int(rand[0, 0]), n - 1])
    g.close()


def test_traversals_device_arrays_and_refusal(sg):
    torch = pytest.importorskip("torch")
    n = 1 << 12
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(oracle.rmat(12, 20000, seed=8)))
    c = sg.CompactGraph(g)
    d = torch.empty(n, dtype=torch.int32, device="cuda")
    c.bfs(7, out=d)
    assert np.array_equal(d.cpu().numpy(), sg.BFS(g, 7, depths=True))
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    c.cc(out=lab)
    assert np.array_equal(lab.cpu().numpy().view(np.uint32), sg.CC(g))
    with pytest.raises(sg.SSTError):
        c.bfs(n)
    c.close()
    g.close()
    w = sg.SparseMatrixV(8, 1 << 20)
    w.insert_batch(np.array([[1, 5]], np.uint32))
    cw = sg.CompactGraph(w)
    for call in (lambda: cw.bfs(1), lambda: cw.cc(), lambda: cw.bc(1), lambda: cw.tc()):
        with pytest.raises(sg.SSTError) as e:
            call()
        assert "rows as columns" in str(e.value)
    cw.close()
    w.close()
