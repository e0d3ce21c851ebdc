"""The weighted-graph oracle against independent checks: value semantics on
hand-made batches, and its Bellman-Ford against scipy's Dijkstra (equal for
non-negative lengths)."""
import numpy as np
import pytest

from oracle.weighted import INF32, WeightedOracle


def test_value_semantics():
    o = WeightedOracle(5)
    o.insert_batch([[0, 1], [0, 1], [1, 2], [2, 2], [7, 1]], [5, 9, 3, 4, 1])
    assert o.value(0, 1) == 9  # last of equal pairs wins
    assert o.value(2, 2) is None  # self-loop skipped
    o.insert_batch([[0, 1]], [2])  # a present edge takes the new value
    assert o.value(0, 1) == 2
    o.remove_batch([[0, 1], [3, 4]])
    assert o.value(0, 1) is None
    off, cols, vals = o.csr_values()
    assert off.tolist() == [0, 0, 1, 1, 1, 1]
    assert cols.tolist() == [2] and vals.tolist() == [3]


def test_bf_matches_dijkstra():
    sp = pytest.importorskip("scipy.sparse")
    csgraph = pytest.importorskip("scipy.sparse.csgraph")
    rng = np.random.default_rng(2)
    n = 300
    pairs = rng.integers(0, n, (2500, 2))
    vals = rng.integers(0, 1000, 2500)
    o = WeightedOracle(n)
    o.insert_batch(pairs, vals)
    off, cols, w = o.csr_values()
    # zero lengths are dropped by the sparse matrix: shift all lengths by one
    # in both computations so the comparison stays exact
    o2 = WeightedOracle(n)
    o2.insert_batch(pairs, vals + 1)
    off2, cols2, w2 = o2.csr_values()
    a = sp.csr_matrix((w2.astype(np.float64), cols2.astype(np.int64),
                       off2.astype(np.int64)), shape=(n, n))
    for src in (0, 5, 123):
        exp = csgraph.dijkstra(a, directed=True, indices=src)
        got = o2.bf(src)
        exp32 = np.where(np.isinf(exp), INF32, exp).astype(np.int64)
        assert np.array_equal(got.astype(np.int64), exp32)


def test_oracle_matches_reference_weighted_stream():
    """The restatement replays the reference's weighted stream (values of
    present edges overwritten, removes) with the reference's CSR and values
    after every batch."""
    from weighted_golden import replay
    replay(WeightedOracle, lambda g, p, v: g.insert_batch(p, v),
           lambda g, p: g.remove_batch(p))
