"""The TinySetV facade (one device row that keeps element 0 of row 0) against
a Python set, after the reference's Tinyset_test.cpp: random inserts below
max, membership, removes, ordered map, early exit, and batch inserts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


@pytest.mark.parametrize("max_el,count", [(1, 1), (100, 80), (1 << 20, 20000)])
def test_add_has_remove(sg, max_el, count):
    rng = np.random.default_rng(max_el)
    ts = sg.TinySetV(max_el)
    model = set()
    vals = rng.integers(0, max_el, count)
    for v in vals[: min(count, 300)]:
        ts.insert(int(v))
        model.add(int(v))
    ts.insert_batch(vals.astype(np.uint32))
    model.update(int(v) for v in vals)
    assert ts.get_n() == len(model)
    probe = np.unique(np.concatenate([vals, rng.integers(0, max_el, 500)]))
    for v in probe[:2000]:
        assert ts.has(int(v)) == (int(v) in model)
    assert np.array_equal(ts.elements(), np.array(sorted(model), np.uint32))
    drop = vals[: count // 2]
    for v in drop[:200]:
        ts.remove(int(v))
        model.discard(int(v))
    ts.remove_batch(drop.astype(np.uint32))
    model.difference_update(int(v) for v in drop)
    assert ts.get_n() == len(model)
    assert np.array_equal(ts.elements(), np.array(sorted(model), np.uint32))
    ts.close()


def test_zero_map_and_range(sg):
    ts = sg.TinySetV(1000)
    ts.insert_batch(np.array([0, 5, 3, 999, 5], np.uint32))
    assert ts.has(0) and ts.has(999) and not ts.has(1)
    seen = []
    ts.map(seen.append)
    assert seen == [0, 3, 5, 999]
    first = []
    ts.map(lambda e: first.append(e) or e >= 3, no_early_exit=False)
    assert first == [0, 3]
    with pytest.raises(sg.SSTError):
        ts.insert(1000)
    assert not ts.has(5000)
    ts.close()
