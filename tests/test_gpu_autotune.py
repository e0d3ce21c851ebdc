"""The autotuner and the knobs it turns: every setting gives the same
results (PageRank bit-exact -- its sums are exact integers -- BFS depths and
multi-source rows bit-exact), the tuner returns settings from its search
space, and out-of-range settings are refused."""
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


@pytest.fixture(scope="module")
def pair(sg):
    n = 1 << 13
    e = oracle.symmetrize(oracle.rmat(13, 16 * n, seed=1))
    g = sg.SparseMatrixV(n)
    g.insert_batch(e)
    o = oracle.OracleGraph(n)
    o.insert_batch(e)
    return g, o


def test_every_setting_same_result(sg, pair):
    g, o = pair
    ref_pr = None
    exp_bfs = o.bfs(3)
    srcs = np.array([3, 77, 4000, 8191], np.uint32)
    exp_multi = np.stack([o.bfs(int(s)) for s in srcs])
    for cl in (1, 4, 8, 16, 32):
        for lanes in (4, 8, 16):
            for alpha, hot in ((1, 0), (20, 4096), (1000, 24576)):
                sg.set_tuning(g, chunk_leaves=cl, pr_lanes=lanes, bfs_alpha=alpha,
                              pr_hot=hot)
                assert sg.get_tuning(g)["chunk_leaves"] == cl
                pr = sg.PR_S(g, 7)
                if ref_pr is None:
                    ref_pr = pr
                    exp = o.pagerank(7)
                    assert np.max(np.abs(pr - exp)) <= 1e-9 * np.max(np.abs(exp))
                assert np.array_equal(pr, ref_pr), (cl, lanes, alpha, hot)
                assert np.array_equal(sg.BFS(g, 3, depths=True), exp_bfs)
                assert np.array_equal(sg.BFS_multi(g, srcs), exp_multi)
    sg.set_tuning(g)


def test_autotune_picks_from_space(sg, pair):
    g, o = pair
    t = sg.autotune(g)
    assert t["chunk_leaves"] in (8, 16, 32)
    assert t["pr_lanes"] in (4, 8, 16)
    assert t["bfs_alpha"] in (5, 10, 20, 40, 80)
    assert t["pr_hot"] in (0, 2048, 4096, 8192)
    assert t["pr_ms"] > 0 and t["bfs_ms"] > 0
    assert sg.get_tuning(g)["bfs_alpha"] == t["bfs_alpha"]
    exp = o.pagerank(10)
    assert np.max(np.abs(sg.PR_S(g, 10) - exp)) <= 1e-9 * np.max(np.abs(exp))
    sg.set_tuning(g)


def test_bad_settings_refused(sg, pair):
    g, _ = pair
    for kw in ({"chunk_leaves": 0}, {"chunk_leaves": 33}, {"pr_lanes": 5},
               {"bfs_alpha": 0}, {"pr_hot": 24577}):
        with pytest.raises(sg.SSTError):
            sg.set_tuning(g, **kw)
