"""Device batch updates vs the CPU oracle: neighbour sets bit-exact after
every batch (reference semantics: SparseMatrix.hpp:556-718)."""
import numpy as np
import pytest

import oracle
from pma_check import check

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def same(g, o, structure=True):
    og, cg = g.csr()
    oo, co = o.csr()
    if structure and g.rows <= 5000:
        errs = check(g, (oo, co))
        assert not errs, errs[:5]
    assert g.M() == o.M()
    assert np.array_equal(og, oo)
    assert np.array_equal(cg, co)
    assert np.array_equal(g.degrees(), o.degrees())


def test_empty_and_tiny(sg):
    g = sg.SparseMatrixV(10)
    o = oracle.OracleGraph(10)
    g.insert_batch(np.zeros((0, 2), np.uint32))
    same(g, o)
    for e in ([[1, 2]], [[1, 2], [1, 2], [2, 2], [3, 1]], [[9, 0], [0, 9]]):
        g.insert_batch(e)
        o.insert_batch(e)
        same(g, o)
    g.remove_batch([[1, 2], [5, 5], [3, 1], [3, 1]])
    o.remove_batch([[1, 2], [5, 5], [3, 1], [3, 1]])
    same(g, o)
    assert g.has(9, 0) and not g.has(1, 2)


@pytest.mark.parametrize("b", [2, 1024, 1025, 2048, 2049, 4096, 4097, 100000,
                               262144, 262145, 400000, 1048576, 1048577])
def test_batch_sizes_across_sort_forms(sg, b):
    """Batch sizes on both sides of each form of the key sort: one CTA
    (up to 2048 keys), one launch a pass over tiles of 1024 keys (up to 2^18
    keys) or of 4096 keys (up to 256 tiles), and the scanned form; each
    batch holds a hub row (skewed high digits) and repeated pairs, and half
    of it is removed again."""
    n = 1 << 14
    rng = np.random.default_rng(b)
    e = rng.integers(0, n, (b, 2)).astype(np.uint32)
    e[: b // 8, 0] = 5
    e[b - b // 10:] = e[: b // 10]
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(e)
    o.insert_batch(e)
    same(g, o, structure=False)
    g.remove_batch(e[::2])
    o.remove_batch(e[::2])
    same(g, o, structure=False)
    g.close()


def test_invalid_ids_skipped(sg):
    g = sg.SparseMatrixV(8)
    bad = g.insert_batch([[1, 2], [8, 1], [1, 100], [3, 4]])
    assert bad == 2
    assert g.M() == 2


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_random_batches(sg, seed):
    rng = np.random.default_rng(seed)
    n = 3000
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    for it in range(12):
        b = int(rng.integers(1, 30000))
        e = rng.integers(0, n, size=(b, 2)).astype(np.uint32)
        e[: b // 2, 0] %= 7  # hubs
        if it % 3 == 2:
            rem = np.concatenate([e[: b // 2], o.sample_edges(b // 2 + 1, seed=it)])
            g.remove_batch(rem)
            o.remove_batch(rem)
        else:
            g.insert_batch(e)
            o.insert_batch(e)
        same(g, o)


def test_rmat_config1_stream(sg):
    """RMAT scale 16, 16 edges/vertex, symmetrised, then 10 batches of 1e4."""
    n = 1 << 16
    base = oracle.symmetrize(oracle.rmat(16, 16 * n, seed=1))
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(base)
    o.insert_batch(base)
    same(g, o)
    for i in range(10):
        b = oracle.rmat(16, 10000, seed=2, first=i * 10000)
        g.insert_batch(b)
        o.insert_batch(b)
        same(g, o)


def test_grow_and_shrink_hub(sg):
    n = 1 << 15
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    cols = np.arange(1, n, dtype=np.uint32)
    e = np.stack([np.zeros_like(cols), cols], 1)
    for part in np.array_split(e, 7):
        g.insert_batch(part)
        o.insert_batch(part)
        same(g, o)
    for part in np.array_split(e[::-1].copy(), 5):
        g.remove_batch(part)
        o.remove_batch(part)
        same(g, o)
    assert g.M() == 0


def test_has_batch(sg):
    n = 1 << 12
    base = oracle.symmetrize(oracle.rmat(12, 8 * n, seed=5))
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(base)
    o.insert_batch(base)
    q = np.concatenate([base[:5000], oracle.rmat(12, 5000, seed=9)])
    got = g.has_batch(q)
    exp = np.array([o.has(int(a), int(b)) for a, b in q], np.uint8)
    assert np.array_equal(got, exp)
    assert g.has(int(base[0, 0]), int(base[0, 1]))


def test_neighbors_and_sample(sg):
    n = 1 << 12
    base = oracle.symmetrize(oracle.rmat(12, 8 * n, seed=6))
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(base)
    o.insert_batch(base)
    off, cols = o.csr()
    for v in [0, 1, 2, 17, n - 1]:
        assert np.array_equal(g.neighbors(v), cols[off[v]:off[v + 1]])
    assert np.array_equal(g.sample_edges(1000, seed=11), o.sample_edges(1000, seed=11))
    assert g.touch_all_sum() == o.touch_all_sum()
    pairs = oracle.rmat(12, 500, seed=12)
    for early in (False, True):
        got = g.common_neighbors_batch(pairs, early)
        exp = [o.common_neighbors(int(a), int(b), early) for a, b in pairs]
        assert list(got) == exp


def test_generators_match_oracle(sg):
    assert np.array_equal(sg.gen_rmat(14, 50000, seed=3, first=77), oracle.rmat(14, 50000, seed=3, first=77))
    assert np.array_equal(sg.gen_er(1000003, 50000, seed=4), oracle.er(1000003, 50000, seed=4))
    assert np.array_equal(sg.gen_ref_rmat(1 << 15, 50000), oracle.ref_rmat_stream(1 << 15, 50000))


def test_pinned_host_inputs(sg):
    """Pinned host pairs (read by the key build in place) and pageable ones
    (copied first) give the same graph as the oracle."""
    torch = pytest.importorskip("torch")
    n = 1 << 12
    rng = np.random.default_rng(21)
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    for i, b in enumerate([1, 1000, 70000, 300000, 5000]):
        e = rng.integers(0, n, (b, 2)).astype(np.uint32)
        pinned = torch.from_numpy(e.view(np.int32)).pin_memory()
        if i % 2:
            g.remove_batch(pinned)
            o.remove_batch(e)
            g.insert_batch(e[: b // 2])
            o.insert_batch(e[: b // 2])
        else:
            g.insert_batch(pinned)
            o.insert_batch(e)
        same(g, o, structure=False)
    w = sg.SparseMatrixV(n, weighted=True)
    e = rng.integers(0, n, (4000, 2)).astype(np.uint32)
    v = rng.integers(0, 1000, 4000).astype(np.uint32)
    w.insert_batch_weighted(torch.from_numpy(e.view(np.int32)).pin_memory(),
                            torch.from_numpy(v.view(np.int32)).pin_memory())
    vals, found = w.values(e)
    last = {}
    for (r, c), x in zip(e.tolist(), v.tolist()):
        if r != c:
            last[(r, c)] = x
    exp = np.array([last.get((r, c), 0) for r, c in e.tolist()], np.uint32)
    ok = np.array([(r, c) in last for r, c in e.tolist()])
    assert np.array_equal(found, ok) and np.array_equal(vals[ok], exp[ok])
    g.close()
    w.close()


def test_pairs_only_4_byte_aligned(sg):
    """Pair arrays at a 4-byte (not 8-byte) aligned address, device and
    pinned host, take the key build's two-loads-a-pair form: same graph as
    the oracle, and the same invalid-pair counts."""
    torch = pytest.importorskip("torch")
    n = 1 << 12
    rng = np.random.default_rng(33)
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    for i, b in enumerate([3, 2000, 150000]):
        e = rng.integers(0, n, (b, 2)).astype(np.uint32)
        e[:5, 1] = n + 7  # out of range: counted, skipped
        buf = torch.empty(2 * b + 1, dtype=torch.int32, device="cuda")
        buf[1:].copy_(torch.from_numpy(e.view(np.int32).reshape(-1)))
        dev = buf[1:]
        assert dev.data_ptr() % 8 == 4
        hbuf = torch.empty(2 * b + 1, dtype=torch.int32).pin_memory()
        hbuf[1:].copy_(torch.from_numpy(e.view(np.int32).reshape(-1)))
        host = hbuf[1:]
        assert host.data_ptr() % 8 == 4
        assert g.insert_batch(dev if i % 2 == 0 else host) == min(5, b)
        o.insert_batch(e[e[:, 1] < n])  # the oracle gets the valid pairs
        same(g, o, structure=False)
        half = np.ascontiguousarray(e[: b // 2])
        hb = torch.empty(2 * len(half) + 1, dtype=torch.int32, device="cuda")
        hb[1:].copy_(torch.from_numpy(half.view(np.int32).reshape(-1)))
        g.remove_batch(hb[1:])
        o.remove_batch(half[half[:, 1] < n])
        same(g, o, structure=False)
    g.close()


@pytest.mark.parametrize("polls", [0, 1])
def test_scan_lookback_fallback(sg, polls):
    """The single-pass scans' bounded wait: with a poll limit of 0 every
    tile after the first stops waiting at once and reduces its
    predecessors' inputs itself (1: after one look at the flag).  Update
    batches launched directly (so their scans take the single-pass form)
    must still match the oracle, after inserts and removes."""
    n = 1 << 16
    base = oracle.symmetrize(oracle.rmat(16, 8 * n, seed=11))
    g = sg.SparseMatrixV(n)
    g.set_plan_graphs(False)
    o = oracle.OracleGraph(n)
    g.insert_batch(base)
    o.insert_batch(base)
    old = sg.set_scan_lookback_polls(polls)
    try:
        sg.profile_start("k_scan_lb")
        for i, b in enumerate((30000, 200000, 1000000)):
            e = oracle.rmat(16, b, seed=100 + i)
            g.insert_batch(e)
            o.insert_batch(e)
            same(g, o, structure=False)
            r = o.sample_edges(b // 2, seed=200 + i)
            g.remove_batch(r)
            o.remove_batch(r)
            same(g, o, structure=False)
        prof = sg.profile_collect()
    finally:
        sg.set_scan_lookback_polls(old)
    assert sum(v["launches"] for k, v in prof.items() if "k_scan_lb" in k) > 0, prof
    assert sg.set_scan_lookback_polls(old) == old


def test_release_scratch_after_bulk_load(sg):
    """A large batch grows the update scratch; sst_release_scratch gives it
    back (the memory size falls to about the storage), and the graph keeps
    working: updates, traversals and tuning after the release match the
    oracle."""
    n = 1 << 16
    base = oracle.symmetrize(oracle.rmat(16, 16 * n, seed=21))
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(base)
    o.insert_batch(base)
    sg.set_tuning(g, chunk_leaves=16, pr_lanes=4, bfs_alpha=10)
    sg.PR_S(g, 3)
    grown = g.get_memory_size()
    g.release_scratch()
    trimmed = g.get_memory_size()
    # the 2M-pair load's scratch is hundreds of bytes a pair, the storage
    # about 6 bytes an edge
    assert 4 * trimmed < grown, (trimmed, grown)
    assert sg.get_tuning(g)["chunk_leaves"] == 16
    # symmetric updates keep the graph a valid traversal input
    e = oracle.symmetrize(oracle.rmat(16, 50000, seed=22))
    g.insert_batch(e)
    o.insert_batch(e)
    same(g, o, structure=False)
    g.release_scratch()
    r = oracle.symmetrize(o.sample_edges(20000, seed=23))
    g.remove_batch(r)
    o.remove_batch(r)
    same(g, o, structure=False)
    g.release_scratch()
    assert np.array_equal(sg.CC(g), o.cc())
