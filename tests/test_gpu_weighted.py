"""Weighted graphs (sst_config.weighted) against the weighted oracle:
values bit-exact after every batch -- including present edges overwritten,
equal pairs in one batch (last wins), leaf merges, window rebalances and
resizes of a growing hub row, deletes that shrink rows -- the PMA invariants
of the ids, copies carrying values, Bellman-Ford distances bit-exact, and
the operations a weighted graph refuses."""
import numpy as np
import pytest

import pma_check
from oracle.weighted import INF32, WeightedOracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def same(g, o):
    off, cols, vals = g.csr_values()
    eo, ec, ev = o.csr_values()
    assert np.array_equal(off, eo)
    assert np.array_equal(cols, ec)
    assert np.array_equal(vals, ev)


@pytest.mark.parametrize("seed", [1, 2])
def test_random_weighted_stream(sg, seed):
    rng = np.random.default_rng(seed)
    n = 1500
    g = sg.SparseMatrixV(n, weighted=True)
    o = WeightedOracle(n)
    for step in range(14):
        k = int(rng.integers(1, 6000))
        p = rng.integers(0, n, (k, 2)).astype(np.uint32)
        if step % 4 == 3:
            # a hub row grows past several capacity classes
            p[: k // 2, 0] = 7
        v = rng.integers(0, 1 << 31, k).astype(np.uint32)
        if step % 3 == 2 and step:
            off, cols, _ = o.csr_values()
            rows = np.repeat(np.arange(n), np.diff(off).astype(np.int64))
            pick = rng.integers(0, len(cols), min(len(cols), 3000))
            rm = np.stack([rows[pick], cols[pick]], 1).astype(np.uint32)
            g.remove_batch(rm)
            o.remove_batch(rm)
        else:
            g.insert_batch_weighted(p, v)
            o.insert_batch(p, v)
        same(g, o)
        assert pma_check.check(g) == []
    q = rng.integers(0, n, (500, 2)).astype(np.uint32)
    vals, found = g.values(q)
    for (a, b), val, f in zip(q.tolist(), vals.tolist(), found.tolist()):
        exp = o.value(a, b)
        assert f == (exp is not None)
        assert val == (exp if exp is not None else 0)
    c = g.copy()
    same(c, o)
    c.close()
    g.close()


@pytest.mark.parametrize("b", [1024, 1025, 4097, 262144, 262145])
def test_last_value_wins_across_sort_forms(sg, b):
    """Repeated pairs with different values in one batch, at sizes on both
    sides of each form of the key-value sort: the sort is stable, so the
    last value of each pair is the one stored."""
    n = 1 << 13
    rng = np.random.default_rng(b)
    p = rng.integers(0, n, (b, 2)).astype(np.uint32)
    p[: b // 8, 0] = 3
    p[b - b // 5:] = p[: b // 5]
    v = rng.integers(0, 1 << 31, b).astype(np.uint32)
    g = sg.SparseMatrixV(n, weighted=True)
    o = WeightedOracle(n)
    g.insert_batch_weighted(p, v)
    o.insert_batch(p, v)
    same(g, o)
    g.close()


def test_overwrite_and_duplicates_in_one_batch(sg):
    g = sg.SparseMatrixV(10, weighted=True)
    g.insert_batch_weighted(np.array([[1, 2], [1, 3], [1, 2]], np.uint32), [5, 6, 7])
    vals, found = g.values(np.array([[1, 2], [1, 3], [1, 4]], np.uint32))
    assert vals.tolist() == [7, 6, 0] and found.tolist() == [True, True, False]
    g.insert_batch_weighted(np.array([[1, 3]], np.uint32), [11])
    assert g.values(np.array([[1, 3]], np.uint32))[0].tolist() == [11]
    g.insert_batch(np.array([[1, 5]], np.uint32))  # plain insert: value 1
    assert g.values(np.array([[1, 5]], np.uint32))[0].tolist() == [1]
    assert g.M() == 3
    g.close()


def test_bellman_ford(sg):
    rng = np.random.default_rng(9)
    n = 2000
    g = sg.SparseMatrixV(n, weighted=True)
    o = WeightedOracle(n)
    p = rng.integers(0, n, (12000, 2)).astype(np.uint32)
    v = rng.integers(0, 5000, 12000).astype(np.uint32)
    g.insert_batch_weighted(p, v)
    o.insert_batch(p, v)
    for src in (0, 17, 1999):
        assert np.array_equal(sg.BF(g, src), o.bf(src)), src
    # an isolated source reaches only itself
    iso = int(np.setdiff1d(np.arange(n), p[:, 0])[0])
    d = sg.BF(g, iso)
    assert d[iso] == 0 and np.all(np.delete(d, iso) == INF32)
    g.close()


def test_weighted_refusals(sg):
    g = sg.SparseMatrixV(8, weighted=True)
    u = sg.SparseMatrixV(8)
    with pytest.raises(sg.SSTError):
        u.insert_batch_weighted(np.array([[1, 2]], np.uint32), [3])
    with pytest.raises(sg.SSTError):
        sg.BF(u, 0)
    with pytest.raises(sg.SSTError):
        g.update_batches([np.array([[1, 2]], np.uint32)])
    with pytest.raises(sg.SSTError):
        sg.BF(g, 8)
    g.close()
    u.close()


def test_device_matches_reference_weighted_stream(sg):
    """The device replays the stream the reference's own
    SparseMatrixV<true, uint32_t> wrote (tests/golden/weighted_stream.npz):
    CSR and values equal to the reference's after every batch."""
    from weighted_golden import replay
    g = replay(lambda n: sg.SparseMatrixV(n, weighted=True),
               lambda g, p, v: g.insert_batch_weighted(p, v),
               lambda g, p: g.remove_batch(p))
    g.close()
