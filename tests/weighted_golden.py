"""Replay of tests/golden/weighted_stream.npz (written by the reference's own
SparseMatrixV<true, uint32_t>, see make_golden.py) on any weighted graph
with insert_batch(pairs, values), remove_batch(pairs) and csr_values()."""
import hashlib
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                    "weighted_stream.npz")


def digest(off, cols, vals):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(cols, np.uint32).tobytes())
    h.update(np.ascontiguousarray(vals, np.uint32).tobytes())
    return h.hexdigest()


def replay(make_graph, insert, remove):
    """Builds the fixture's graph and applies its batches; after every batch
    checks the CSR with values against the reference's digest.  Returns the
    final (off, cols, vals) and the fixture."""
    d = np.load(PATH)
    n = 1 << int(d["scale"])
    g = make_graph(n)
    insert(g, d["base"], d["base_val"])
    steps = [str(x) for x in d["steps"]]
    k = 0

    def check(tag):
        nonlocal k
        assert steps[k] == tag
        got = g.csr_values()
        assert len(got[1]) == int(d["M"][k]), tag
        assert digest(*got) == str(d["digests"][k]), tag
        k += 1
        return got

    got = check("base")
    for i in range(6):
        insert(g, d[f"ins_{i}"], d[f"insval_{i}"])
        got = check(f"i{i}")
        if f"rem_{i}" in d:
            remove(g, d[f"rem_{i}"])
            got = check(f"r{i}")
    assert k == len(steps)
    for a, b in zip(got, (d["off_final"], d["cols_final"], d["vals_final"])):
        assert np.array_equal(a, b)
    return g
