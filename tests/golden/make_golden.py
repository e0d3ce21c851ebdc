"""Generate the golden fixtures in this directory from the reference's own
code (oracle/_ref/libsstref.so: SparseMatrixV<true>, TinySetV, rMat,
create_random_data and the .mtx loader compiled from the reference headers).

Run in a checkout that has the reference tree (the reference is not shipped
with this repository):

    python -c "import oracle; oracle.build(ref=True)"
    python tests/golden/make_golden.py [path/to/reference]

Fixtures (all small, npz):
  ref_rmat_stream.npz   rMat(2^15, hash64(0), .5, .1, .1) edges 0..19999
                        (internal/rmat_util.h:82-131, internal/test.hpp:645-654)
  known_answer.npz      create_random_data(10000, max, seed 0) for the four
                        key widths of PMA_test.cpp:15-84, the sorted set a
                        TinySetV holds after inserting them, and after
                        removing the first half
  rmat16_stream.npz     scale-16 RMAT base graph (16 edges/vertex, seed 1,
                        symmetrised) built with SparseMatrixV::insert_batch,
                        then 10 insert batches of 1e4 RMAT edges (seed 2) and
                        5 remove batches of sampled edges: degrees and a
                        sha256 of the CSR after every batch, touch_all_sum,
                        common_neighbors on sampled pairs, has() on queries
  degree_order.npz      degree_order_map() of that base graph and a sha256 of
                        rewrite_graph(map)'s CSR (SparseMatrix.hpp:737-766)
  examples_mtx.npz      examples/*.mtx through the reference loader
                        (helpers.hpp:379-529): symmetrised edge lists and the
                        CSR of the graph built from them
  tinyset_widths.npz    TinySetV_small::get_thresholds(max_el) for a range of
                        column counts (TinySet_small.hpp:227-263), and the key
                        width get_b() of a reference set after inserting k
                        distinct ids, for k on both sides of each threshold
  weighted_stream.npz   SparseMatrixV<true, uint32_t> (internal/test.hpp:714):
                        a weighted RMAT scale-10 base graph, then 6 batches of
                        weighted inserts (a fifth of each re-inserts present
                        edges with new values: PMA.hpp:1137-1145) with removes
                        of sampled edges after every second one; the batches
                        and a sha256 of the CSR with its values after every
                        batch (the last one in full).  No
                        pair repeats inside a batch: the reference's batch
                        sort (SparseMatrix.hpp:489-494) does not define which
                        of equal pairs wins.  Removes go through the
                        single-edge remove (the weighted remove_batch does not
                        compile in the reference)

`--only tinyset_widths` / `--only weighted_stream` writes that fixture alone.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402


def csr_digest(off, cols):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(cols, np.uint32).tobytes())
    return h.hexdigest()


TINYSET_MAX_ELS = [1, 2, 100, 255, 256, 257, 1024, 65535, 65536, 65537,
                   1 << 20, 3000000, 1 << 24, (1 << 24) + 1, 1 << 25, 1 << 30,
                   0xFFFFFFFF]


def tinyset_widths():
    import ctypes
    R = oracle.ref()
    th = np.zeros((len(TINYSET_MAX_ELS), 3), np.uint32)
    for i, mx in enumerate(TINYSET_MAX_ELS):
        t = np.zeros(3, np.uint32)
        R.ref_tinyset_thresholds(mx, ctypes.c_void_p(t.ctypes.data))
        th[i] = t
    # widths of real reference sets: k distinct ids below max_el (seed 7)
    rng = np.random.default_rng(7)
    rows = []
    for mx in (1 << 10, 1 << 16, 1 << 20, 1 << 24):
        t = np.zeros(3, np.uint32)
        R.ref_tinyset_thresholds(mx, ctypes.c_void_p(t.ctypes.data))
        ks = {1, 2, 3}
        for x in t.tolist():
            for k in (x - 1, x, x + 1):
                if 1 <= k <= min(mx, 1 << 21):
                    ks.add(k)
        for k in sorted(ks):
            els = rng.choice(mx, size=k, replace=False).astype(np.uint32)
            b = R.ref_tinyset_width(mx, ctypes.c_void_p(els.ctypes.data), k)
            rows.append((mx, k, b))
    w = np.array(rows, np.uint64)
    np.savez_compressed(os.path.join(HERE, "tinyset_widths.npz"),
                        max_el=np.array(TINYSET_MAX_ELS, np.uint64), thresholds=th,
                        width_max_el=w[:, 0], width_count=w[:, 1], width=w[:, 2])


def wcsr_digest(off, cols, vals):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(off, np.uint64).tobytes())
    h.update(np.ascontiguousarray(cols, np.uint32).tobytes())
    h.update(np.ascontiguousarray(vals, np.uint32).tobytes())
    return h.hexdigest()


def weighted_stream():
    scale, n = 10, 1 << 10
    rng = np.random.default_rng(12)
    g = oracle.RefWGraph(n)

    def unique_pairs(e):
        _, idx = np.unique(e[:, 0].astype(np.int64) * n + e[:, 1], return_index=True)
        return np.ascontiguousarray(e[np.sort(idx)])

    base = unique_pairs(oracle.symmetrize(oracle.rmat(scale, 8 * n, seed=31)))
    bval = rng.integers(1, 1 << 20, len(base)).astype(np.uint32)
    g.insert_batch(base, bval)
    out = {"scale": np.uint32(scale), "base": base, "base_val": bval}
    steps, digests, ms = [], [], []

    def snap(tag):
        off, cols, vals = g.csr_values()
        digests.append(wcsr_digest(off, cols, vals))
        ms.append(len(cols))
        steps.append(tag)
        out["off_final"], out["cols_final"], out["vals_final"] = off, cols, vals
        return off, cols

    off, cols = snap("base")
    for i in range(6):
        new = oracle.rmat(scale, 600, seed=32, first=i * 600)
        rows = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
        pick = rng.choice(len(cols), 150, replace=False)
        old = np.stack([rows[pick], cols[pick]], 1).astype(np.uint32)
        ins = unique_pairs(np.concatenate([new, old]))
        val = rng.integers(1, 1 << 20, len(ins)).astype(np.uint32)
        g.insert_batch(ins, val)
        out[f"ins_{i}"] = ins
        out[f"insval_{i}"] = val
        off, cols = snap(f"i{i}")
        if i % 2 == 1:
            rows = np.repeat(np.arange(n), np.diff(off.astype(np.int64)))
            pick = rng.choice(len(cols), 120, replace=False)
            rem = np.stack([rows[pick], cols[pick]], 1).astype(np.uint32)
            g.remove_each(rem)
            out[f"rem_{i}"] = rem
            off, cols = snap(f"r{i}")
    out["steps"] = np.array(steps)
    out["digests"] = np.array(digests)
    out["M"] = np.array(ms, np.uint64)
    np.savez_compressed(os.path.join(HERE, "weighted_stream.npz"), **out)


def main(ref_root):
    R = oracle.ref()
    # --- reference batch stream
    out = np.empty((20000, 2), np.uint32)
    R.ref_rmat_stream(1 << 15, 0.5, 0.1, 0.1, 20000, oracle._ptr(out))
    np.savez_compressed(os.path.join(HERE, "ref_rmat_stream.npz"), nn=1 << 15, pairs=out)

    # --- known-answer sets (PMA_test.cpp:15-84 inputs)
    ka = {}
    for b in (1, 2, 3, 4):
        mx = 0xFFFFFFFF if b == 4 else (1 << (8 * b))
        n = min(mx - 1, 10000)
        vals = oracle.ref_random_data(n, mx, 0)
        s = R.ref_set_new(0xFFFFFFFE)
        for v in vals.tolist():
            R.ref_set_insert(s, v)
        full = np.empty(int(R.ref_set_n(s)), np.uint32)
        R.ref_set_to_array(s, oracle._ptr(full))
        for v in vals[: n // 2].tolist():
            R.ref_set_remove(s, v)
        half = np.empty(int(R.ref_set_n(s)), np.uint32)
        R.ref_set_to_array(s, oracle._ptr(half))
        R.ref_set_free(s)
        ka[f"in_{b}"] = vals
        ka[f"full_{b}"] = full
        ka[f"half_{b}"] = half
    np.savez_compressed(os.path.join(HERE, "known_answer.npz"), **ka)

    # --- scale-16 RMAT stream through SparseMatrixV
    scale, n = 16, 1 << 16
    base = oracle.symmetrize(oracle.rmat(scale, 16 * n, seed=1))
    g = oracle.RefGraph(n)
    g.insert_batch(base)
    digests, ms, degs = [], [], []

    def snap():
        off, cols = g.csr()
        digests.append(csr_digest(off, cols))
        ms.append(g.M())
        degs.append(np.diff(off).astype(np.uint32))
        return off, cols

    snap()
    for i in range(10):
        g.insert_batch(oracle.rmat(scale, 10000, seed=2, first=i * 10000))
        snap()
    o = oracle.OracleGraph(n)  # only to draw existing edges to remove
    o.insert_batch(base)
    for i in range(10):
        o.insert_batch(oracle.rmat(scale, 10000, seed=2, first=i * 10000))
    for i in range(5):
        rem = o.sample_edges(20000, seed=3, first=i * 20000)
        g.remove_batch(rem)
        o.remove_batch(rem)
        snap()
    off, cols = g.csr()
    pairs = oracle.rmat(scale, 4000, seed=9)
    cn_full = np.array([g.common_neighbors(int(a), int(b), False) for a, b in pairs], np.uint64)
    cn_early = np.array([g.common_neighbors(int(a), int(b), True) for a, b in pairs], np.uint64)
    q = np.concatenate([o.sample_edges(3000, seed=10), oracle.rmat(scale, 3000, seed=11)])
    has = np.array([g.has(int(a), int(b)) for a, b in q], np.uint8)
    np.savez_compressed(
        os.path.join(HERE, "rmat16_stream.npz"), scale=scale, digests=np.array(digests),
        M=np.array(ms, np.uint64), deg_final=degs[-1], deg_base=degs[0],
        touch_all_sum=np.uint64(g.touch_all_sum()), cn_pairs=pairs, cn_full=cn_full,
        cn_early=cn_early, has_q=q, has_ans=has)

    # --- degree-ordered relabelling of the scale-16 base graph
    #     (SparseMatrix.hpp:737-766)
    g0 = oracle.RefGraph(n)
    g0.insert_batch(base)
    dmap = g0.degree_order_map()
    rg = g0.rewrite_graph(dmap)
    roff, rcols = rg.csr()
    np.savez_compressed(os.path.join(HERE, "degree_order.npz"), map=dmap,
                        digest=np.array(csr_digest(roff, rcols)),
                        touch_all_sum=np.uint64(rg.touch_all_sum()))

    # --- bundled examples through the reference loader
    ex = {}
    for name in ("star", "johnson8-2-4"):
        rows, edges = oracle.ref_load_mtx(os.path.join(ref_root, "examples", name + ".mtx"))
        eg = oracle.RefGraph(rows)
        eg.insert_batch(edges)
        off, cols = eg.csr()
        key = name.replace("-", "_")
        ex[f"{key}_rows"] = np.uint32(rows)
        ex[f"{key}_edges"] = edges
        ex[f"{key}_off"] = off
        ex[f"{key}_cols"] = cols
    np.savez_compressed(os.path.join(HERE, "examples_mtx.npz"), **ex)
    tinyset_widths()
    weighted_stream()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if "--only" in sys.argv and sys.argv[-1] == "tinyset_widths":
        tinyset_widths()
    elif "--only" in sys.argv and sys.argv[-1] == "weighted_stream":
        weighted_stream()
    else:
        main(args[0] if args else "/root/reference")
