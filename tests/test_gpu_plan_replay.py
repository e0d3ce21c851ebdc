"""Update batches up to 2^20 pairs replay their planning launches (sort to
plan readback) from a captured CUDA graph, sized by the batch's size class
(b rounded up to m * 2^k, m in 4..7) and working on the device-side count.
The replayed form must give the same graph as the directly launched form
(sst_set_plan_graphs off) and as the oracle: on cache hits with new contents, on new device buffers, after
repacks that move the slab, past the cache's capacity and under the kernel
profiler."""
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


def equal(a, b):
    oa, ca = a.csr()
    ob, cb = b.csr()
    return a.M() == b.M() and np.array_equal(oa, ob) and np.array_equal(ca, cb)


def batches(rng, n, sizes, o):
    for i, b in enumerate(sizes):
        e = rng.integers(0, n, size=(b, 2)).astype(np.uint32)
        e[: b // 3, 0] %= 5  # hubs
        if i % 4 == 3:
            yield "remove", np.concatenate([e[: b // 2], o.sample_edges(b - b // 2, seed=i)])
        else:
            yield "insert", e


def run(sg, n, sizes, seed, **kw):
    rng = np.random.default_rng(seed)
    a = sg.SparseMatrixV(n, **kw)
    d = sg.SparseMatrixV(n, **kw)
    d.set_plan_graphs(False)
    o = oracle.OracleGraph(n)
    for op, e in batches(rng, n, sizes, o):
        getattr(a, op + "_batch")(e)
        getattr(d, op + "_batch")(e)
        getattr(o, op + "_batch")(e)
        assert equal(a, d)
        assert equal(a, o)
    a.close()
    d.close()


def test_same_size_new_contents(sg):
    run(sg, 5000, [1000] * 6 + [7, 7, 7, 1, 1, 4096, 4096, 4097], seed=1)


def test_sizes_sharing_a_class(sg):
    # 897..1024 share one launch size, as do 65..80 and 4097..5120
    run(sg, 5000, [1024, 897, 1000, 1023, 897, 65, 80, 77, 66, 5120, 4097, 4500, 5000],
        seed=8)


def test_across_sort_forms(sg):
    # one CTA sort, single-launch passes and the largest replayed size
    run(sg, 1 << 16, [2048, 2049, 30000, 30000, (1 << 18) - 1, 1 << 18, (1 << 18) + 1,
                      (1 << 20) - 1, 1 << 20, (1 << 20) + 1], seed=2)


def test_repacks_move_the_slab(sg):
    # a slab with little room repacks often: each repack is a new layout
    run(sg, 3000, [2500] * 16, seed=3, initial_slots=64)


def test_more_sizes_than_cached(sg):
    # every size class (64 .. 2^20: 57 of them, one more than the cache
    # holds), one size below each class's bound, then the first ones again
    classes = [64] + [m << k for k in range(4, 18) for m in (5, 6, 7, 8)]
    assert len(classes) == 57 and classes[-1] == 1 << 20
    sizes = [c - 1 - (c >> 4) for c in classes]
    run(sg, 4000, sizes + sizes[:8], seed=4)


def test_new_device_buffers(sg):
    torch = pytest.importorskip("torch")
    n = 1 << 12
    a = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    gen = torch.Generator().manual_seed(5)
    for i in range(6):
        e = torch.randint(0, n, (3000, 2), generator=gen, dtype=torch.int32)
        dev = e.cuda()
        if i % 3 == 2:
            a.remove_batch(dev)
            o.remove_batch(e.numpy().astype(np.uint32))
        else:
            a.insert_batch(dev)
            o.insert_batch(e.numpy().astype(np.uint32))
        del dev
        assert equal(a, o)
    a.close()


def test_batched_form_next_to_replay(sg):
    # the batched form's passes (keys presorted) launch directly, between
    # replayed single batches
    n = 2000
    rng = np.random.default_rng(6)
    a = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    ins = rng.integers(0, n, size=(4000, 2)).astype(np.uint32)
    rem = ins[::3].copy()
    a.update_batches([ins, rem], [1, 0])
    o.insert_batch(ins)
    o.remove_batch(rem)
    assert equal(a, o)
    a.insert_batch(ins[:1000])
    o.insert_batch(ins[:1000])
    assert equal(a, o)
    a.close()


def test_under_the_profiler(sg):
    # replays are timed as one entry; kernels launched directly still are
    sg.profile_start()
    try:
        run(sg, 3000, [1500, 1500, 1500, 1500], seed=7)
    finally:
        prof = sg.profile_collect()
    assert prof["update_plan_graph"]["launches"] == 4  # the replaying graph's
    assert "k_make_keys_packed" in prof


def test_direct_launch_of_replay_forms(sg):
    """Mode 2 launches the kernels a replay runs one by one (same size
    classes; single-pass scans tagged from the device epoch, which a
    one-thread kernel advances per sequence): same graph as the replayed
    form and the oracle."""
    n = 1 << 14
    rng = np.random.default_rng(9)
    a = sg.SparseMatrixV(n)
    d = sg.SparseMatrixV(n)
    d.set_plan_graphs(2)
    o = oracle.OracleGraph(n)
    seen = set()
    for op, e in batches(rng, n, [1000, 30000, 200000, 1 << 20, 5000, 4096], o):
        getattr(a, op + "_batch")(e)
        getattr(o, op + "_batch")(e)
        sg.profile_start()
        getattr(d, op + "_batch")(e)
        d.sync()
        seen |= set(sg.profile_collect())
        assert equal(a, d)
        assert equal(a, o)
    # the sequence advances the device epoch its scans take their tags from
    assert "k_scan_epoch_bump" in seen, sorted(seen)
    assert any("k_scan_lb" in k for k in seen), sorted(seen)
    assert any("k_scatter" in k for k in seen), sorted(seen)
    assert "update_plan_graph" not in seen
    a.close()
    d.close()
