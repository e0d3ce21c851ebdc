"""The device path against golden fixtures made by the reference's own code
(tests/golden/make_golden.py): bit-exact neighbour sets after every batch,
common_neighbors, has, touch_all_sum, the reference's rMat stream and the
reference .mtx loader's graphs."""
import hashlib
import os

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def load(name):
    return np.load(os.path.join(GOLD, name))


def digest(off, cols):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(cols, np.uint32).tobytes())
    return h.hexdigest()


def test_reference_rmat_stream_on_device(sg):
    d = load("ref_rmat_stream.npz")
    got = sg.gen_ref_rmat(int(d["nn"]), d["pairs"].shape[0])
    assert np.array_equal(got, d["pairs"])


def test_known_answer_sets(sg):
    d = load("known_answer.npz")
    for b in (1, 2, 3, 4):
        vals = d[f"in_{b}"]
        row = 1 if 1 not in set(vals.tolist()) else 0
        g = sg.SparseMatrixV(2, 0xFFFFFFFE)
        g.insert_batch(np.stack([np.full_like(vals, row), vals], 1))
        assert np.array_equal(g.neighbors(row), d[f"full_{b}"])
        h = vals[: len(vals) // 2]
        g.remove_batch(np.stack([np.full_like(h, row), h], 1))
        assert np.array_equal(g.neighbors(row), d[f"half_{b}"])
        g.close()


def test_rmat16_stream_digests(sg):
    d = load("rmat16_stream.npz")
    n = 1 << int(d["scale"])
    base = oracle.symmetrize(oracle.rmat(16, 16 * n, seed=1))
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)  # draws the same removal samples
    g.insert_batch(base)
    o.insert_batch(base)
    got = [digest(*g.csr())]
    assert np.array_equal(g.degrees(), d["deg_base"])
    for i in range(10):
        b = oracle.rmat(16, 10000, seed=2, first=i * 10000)
        g.insert_batch(b)
        o.insert_batch(b)
        got.append(digest(*g.csr()))
    for i in range(5):
        rem = o.sample_edges(20000, seed=3, first=i * 20000)
        # the device sampler draws the same edges from the same graph
        assert np.array_equal(g.sample_edges(20000, seed=3, first=i * 20000), rem)
        g.remove_batch(rem)
        o.remove_batch(rem)
        got.append(digest(*g.csr()))
    assert got == list(d["digests"])
    assert list(np.asarray([g.M()])) == [int(d["M"][-1])]
    assert np.array_equal(g.degrees(), d["deg_final"])
    assert g.touch_all_sum() == int(d["touch_all_sum"])
    pairs = d["cn_pairs"]
    assert list(g.common_neighbors_batch(pairs, False)) == list(d["cn_full"])
    assert list(g.common_neighbors_batch(pairs, True)) == list(d["cn_early"])
    assert np.array_equal(g.has_batch(d["has_q"]), d["has_ans"])


def test_degree_order_relabel(sg):
    d = load("degree_order.npz")
    n = 1 << 16
    g = sg.SparseMatrixV(n)
    g.insert_batch(oracle.symmetrize(oracle.rmat(16, 16 * n, seed=1)))
    m = g.degree_order_map()
    assert np.array_equal(m, d["map"])
    r = g.rewrite_graph(m)
    assert digest(*r.csr()) == str(d["digest"])
    assert r.touch_all_sum() == int(d["touch_all_sum"])
    # PageRank on the relabelled graph is the same vector, permuted
    pr = sg.PR_S(g, 10)
    prr = sg.PR_S(r, 10)
    assert np.max(np.abs(prr[m] - pr)) <= 1e-12 * np.max(pr)


def test_examples_mtx(sg):
    d = load("examples_mtx.npz")
    for key in ("star", "johnson8_2_4"):
        g = sg.SparseMatrixV(int(d[f"{key}_rows"]))
        g.insert_batch(d[f"{key}_edges"])
        off, cols = g.csr()
        assert np.array_equal(off, d[f"{key}_off"])
        assert np.array_equal(cols, d[f"{key}_cols"])
