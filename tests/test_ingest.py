"""Graph file ingest (sst_read_graph_file / sst_load_graph_file): the
reference readers' behaviour (internal/helpers.hpp:379-657) on written
files, errors instead of exits, the reference's own example files against
the golden fixtures made with its loader (when the reference tree is here),
and (GPU) the built graph against the oracle."""
import os

import numpy as np
import pytest

import oracle

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
REF_EXAMPLES = "/root/reference/examples"


@pytest.fixture(scope="module")
def sg():
    import __graft_entry__ as ge
    ge.build()
    import sstgraph_gb300
    return sstgraph_gb300


def write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_mtx_pattern_symmetrised_in_file_order(sg, tmp_path):
    f = write(tmp_path, "a.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n"
              "% a comment\n%another\n4 4 3\n2 1\n3 1\n4 3\n")
    rows, pairs = sg.read_graph_file(f)
    assert rows == 4
    assert pairs.tolist() == [[1, 0], [0, 1], [2, 0], [0, 2], [3, 2], [2, 3]]


def test_mtx_values_ignored(sg, tmp_path):
    f = write(tmp_path, "b.mtx", "%%MatrixMarket matrix coordinate real general\n"
              "3 3 2\n1 2 0.5\n3 3 7\n")
    rows, pairs = sg.read_graph_file(f)
    assert rows == 3 and pairs.tolist() == [[0, 1], [1, 0], [2, 2], [2, 2]]


def test_adj_plain_and_weighted(sg, tmp_path):
    f = write(tmp_path, "c.adj", "AdjacencyGraph\n3\n4\n0\n2\n3\n1\n2\n0\n0\n")
    rows, pairs = sg.read_graph_file(f)
    assert rows == 3 and pairs.tolist() == [[0, 1], [0, 2], [1, 0], [2, 0]]
    f = write(tmp_path, "d.adj.shuf", "WeightedAdjacencyGraph\n2\n2\n0 1\n1 0\n5 6\n")
    rows, pairs = sg.read_graph_file(f)
    assert rows == 2 and pairs.tolist() == [[0, 1], [1, 0]]


@pytest.mark.parametrize("name,text", [
    ("e.mtx", "%%MatrixMarket matrix array real general\n2 2 1\n1 1 1\n"),
    ("f.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n3 3 2\n1 2\n"),
    ("g.mtx", "%%MatrixMarket matrix coordinate pattern general\n3 4 1\n1 2\n"),
    ("h.mtx", "%%MatrixMarket matrix coordinate pattern general\n3 3 1\n0 2\n"),
    ("i.mtx", "no header\n"),
    ("j.adj", "AdjacencyGraph\n2\n2\n0\n1\n1\n"),
    ("k.adj", "AdjacencyGraph\n2\n1\n0\n1\n5\n"),
    ("l.txt", "AdjacencyGraph\n1\n1\n0\n0\n"),
])
def test_malformed_files_are_errors(sg, tmp_path, name, text):
    with pytest.raises(sg.SSTError):
        sg.read_graph_file(write(tmp_path, name, text))


def test_missing_file_is_an_error(sg, tmp_path):
    with pytest.raises(sg.SSTError):
        sg.read_graph_file(str(tmp_path / "absent.mtx"))


@pytest.mark.skipif(not os.path.isdir(REF_EXAMPLES), reason="reference tree not present")
def test_reference_examples_match_the_reference_loader(sg):
    d = np.load(os.path.join(GOLD, "examples_mtx.npz"))
    for stem, key in (("star", "star"), ("johnson8-2-4", "johnson8_2_4")):
        rows, pairs = sg.read_graph_file(os.path.join(REF_EXAMPLES, stem + ".mtx"))
        assert rows == int(d[key + "_rows"])
        assert np.array_equal(pairs, d[key + "_edges"])


@pytest.mark.gpu
def test_loaded_graph_matches_oracle(sg, tmp_path):
    rng = np.random.default_rng(3)
    n = 300
    e = rng.integers(1, n + 1, (2000, 2))
    body = "".join(f"{a} {b}\n" for a, b in e)
    f = write(tmp_path, "r.mtx",
              f"%%MatrixMarket matrix coordinate pattern symmetric\n{n} {n} {len(e)}\n{body}")
    rows, pairs = sg.read_graph_file(f)
    g = sg.load_graph_file(f)
    o = oracle.OracleGraph(rows)
    o.insert_batch(pairs)
    off, cols = g.csr()
    eoff, ecols = o.csr()
    assert g.rows == n and np.array_equal(off, eoff) and np.array_equal(cols, ecols)
    g.close()
