"""Batched form: many uneven insert/remove batches in one pipeline pass
(sst_update_batches) must leave the graph exactly as applying them one after
another does (the CPU oracle, and the plain per-batch device path)."""
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


def stream(n, seed, count, rng):
    """uneven batches; removes draw from earlier inserts so they hit edges
    that exist, and later batches re-insert some removed edges"""
    batches, ops = [], []
    pool = []
    for i in range(count):
        size = int(min(20000, max(1, rng.lognormal(np.log(300), 1.5))))
        if i % 3 == 2 and pool:
            src = np.concatenate(pool)
            b = src[rng.integers(0, len(src), size)]
            ops.append(0)
        else:
            b = oracle.rmat(int(np.log2(n)), size, seed=seed, first=i * 100000)
            if i % 5 == 4 and pool:  # re-insert some earlier edges
                src = np.concatenate(pool)
                b = np.concatenate([b, src[rng.integers(0, len(src), size // 4 + 1)]])
            pool.append(b)
            ops.append(1)
        batches.append(np.ascontiguousarray(b, np.uint32))
    return batches, ops


@pytest.mark.parametrize("seed", [1, 2])
def test_batched_equals_sequential(sg, seed):
    n = 1 << 12
    rng = np.random.default_rng(seed)
    base = oracle.symmetrize(oracle.rmat(12, 8 * n, seed=seed + 10))
    batches, ops = stream(n, seed, 60, rng)
    batches[3] = np.concatenate([batches[3], [[5, 5], [n + 3, 1], [7, n]]]).astype(np.uint32)

    o = oracle.OracleGraph(n)
    o.insert_batch(base)
    for b, op in zip(batches, ops):
        (o.insert_batch if op else o.remove_batch)(b)

    g = sg.SparseMatrixV(n)
    g.insert_batch(base)
    bad = g.update_batches(batches, ops)
    assert bad == 2
    og, cg = g.csr()
    oo, co = o.csr()
    assert np.array_equal(og, oo) and np.array_equal(cg, co)
    assert not check(g, (oo, co))

    p = sg.SparseMatrixV(n)
    p.insert_batch(base)
    for b, op in zip(batches, ops):
        (p.insert_batch if op else p.remove_batch)(b)
    op_, cp = p.csr()
    assert np.array_equal(op_, og) and np.array_equal(cp, cg)


def test_batched_device_pointers(sg):
    import torch
    n = 1 << 10
    rng = np.random.default_rng(7)
    batches, ops = stream(n, 3, 20, rng)
    o = oracle.OracleGraph(n)
    for b, op in zip(batches, ops):
        (o.insert_batch if op else o.remove_batch)(b)
    g = sg.SparseMatrixV(n)
    g.update_batches([torch.from_numpy(b.astype(np.int32)).cuda() for b in batches], ops)
    g.sync()
    og, cg = g.csr()
    oo, co = o.csr()
    assert np.array_equal(og, oo) and np.array_equal(cg, co)


def test_batched_single_and_empty(sg):
    g = sg.SparseMatrixV(16)
    assert g.update_batches([np.zeros((0, 2), np.uint32)], [1]) == 0
    g.update_batches([np.array([[1, 2], [2, 1]], np.uint32), np.array([[1, 2]], np.uint32)], [1, 0])
    assert g.M() == 1 and g.has(2, 1) and not g.has(1, 2)
