"""Multi-source BFS and BC (k <= 64 sources per call) against the per-source
oracle and the single-source device paths: depths bit-exact, BC bit-exact
to sst_bc of each source (same arithmetic order) and within 1e-9 relative
of the oracle."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

REL = 1e-9


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def graphs():
    n = 1 << 13
    yield "rmat13", n, oracle.symmetrize(oracle.rmat(13, 16 * n, seed=1))
    yield "er", 5000, oracle.symmetrize(oracle.er(5000, 5000 * 4, seed=4))
    # a star, an isolated tail and a long path: many levels, unreachable rows
    path = [[i, i + 1] for i in range(40, 399)]
    star = [[0, i] for i in range(1, 30)]
    yield "star+path", 420, oracle.symmetrize(np.array(star + path, np.uint32))


@pytest.fixture(scope="module", params=[x[0] for x in graphs()])
def pair(request, sg):
    name, n, edges = next(x for x in graphs() if x[0] == request.param)
    g = sg.SparseMatrixV(n)
    o = oracle.OracleGraph(n)
    g.insert_batch(edges)
    o.insert_batch(edges)
    return g, o


def sources(n, k, seed):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, n, k).astype(np.uint32)
    if k > 3:
        s[1] = s[0]  # a repeated source
        s[2] = n - 1
    return s


@pytest.mark.parametrize("k", [1, 5, 64])
def test_bfs_multi_matches_oracle(sg, pair, k):
    g, o = pair
    srcs = sources(g.rows, k, seed=k)
    dep = sg.BFS_multi(g, srcs)
    assert dep.shape == (k, g.rows)
    for i, s in enumerate(srcs):
        assert np.array_equal(dep[i], o.bfs(int(s))), (i, int(s))


@pytest.mark.parametrize("k", [1, 16])
def test_bc_multi_matches_single_and_oracle(sg, pair, k):
    g, o = pair
    srcs = sources(g.rows, k, seed=100 + k)
    out = sg.BC_multi(g, srcs)
    assert out.shape == (k, g.rows)
    for i, s in enumerate(srcs):
        one = sg.BC(g, int(s))
        assert np.array_equal(out[i], one), (i, int(s))
        exp = o.bc(int(s))
        assert np.max(np.abs(out[i] - exp)) <= REL * max(np.max(np.abs(exp)), 1e-300)


def test_multi_device_buffers(sg, pair):
    torch = pytest.importorskip("torch")
    g, o = pair
    srcs = torch.tensor(sources(g.rows, 8, seed=7).astype(np.int64), dtype=torch.int32,
                        device="cuda")
    out = torch.empty((8, g.rows), dtype=torch.int32, device="cuda")
    sg.BFS_multi(g, srcs, out=out)
    host = out.cpu().numpy()
    for i, s in enumerate(srcs.cpu().numpy()):
        assert np.array_equal(host[i], o.bfs(int(s)))


def test_multi_argument_errors(sg, pair):
    g, _ = pair
    with pytest.raises(sg.SSTError):
        sg.BFS_multi(g, np.zeros(65, np.uint32))
    with pytest.raises(sg.SSTError):
        sg.BFS_multi(g, np.array([0, g.rows], np.uint32))
    with pytest.raises(sg.SSTError):
        sg.BC_multi(g, np.array([g.rows + 5], np.uint32))
    assert sg.BFS_multi(g, np.zeros(0, np.uint32)).shape == (0, g.rows)
