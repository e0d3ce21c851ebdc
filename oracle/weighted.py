"""Weighted-graph oracle -- TEST INFRASTRUCTURE (only tests use it).

A Python restatement, for test sizes, of the reference's weighted binary CSR
(``SparseMatrixV<true, uint32_t>``):

* per-row maps col -> value; an insert of a present edge takes the new value
  (``PMA.hpp:1137-1145``: "update its value if needed"), and of equal pairs in
  one batch the last wins (the reference sorts the batch by row, stably, then
  inserts row by row in order, ``SparseMatrix.hpp:556-643``);
* self-loops are skipped on insert (``SparseMatrix.hpp:570,602``); removing
  an absent edge is a no-op;
* ``bf(src)``: single-source shortest-path lengths over the values as edge
  lengths, the quantity the drivers' ``BF(g, src)`` computes
  (``internal/test.hpp:611-634``); Bellman-Ford rounds written from the
  definition (relax every out-edge of every vertex until nothing changes),
  unreachable = 2^31 - 1, lengths saturate there.
"""
from __future__ import annotations

import numpy as np

INF32 = 0x7FFFFFFF


class WeightedOracle:
    def __init__(self, n: int):
        self.n = int(n)
        self.rows = [dict() for _ in range(self.n)]

    def insert_batch(self, pairs, values=None):
        p = np.asarray(pairs, np.int64).reshape(-1, 2)
        v = np.ones(len(p), np.int64) if values is None else np.asarray(values, np.int64)
        for (a, b), w in zip(p.tolist(), v.tolist()):
            if a >= self.n or b >= self.n or a == b:
                continue
            self.rows[a][b] = w

    def remove_batch(self, pairs):
        for a, b in np.asarray(pairs, np.int64).reshape(-1, 2).tolist():
            if a < self.n:
                self.rows[a].pop(b, None)

    def csr_values(self):
        off = np.zeros(self.n + 1, np.uint64)
        cols, vals = [], []
        for v in range(self.n):
            ks = sorted(self.rows[v])
            cols.extend(ks)
            vals.extend(self.rows[v][k] for k in ks)
            off[v + 1] = off[v] + len(ks)
        return off, np.array(cols, np.uint32), np.array(vals, np.uint32)

    def value(self, a, b):
        return self.rows[a].get(b)

    def bf(self, src: int) -> np.ndarray:
        dist = [None] * self.n
        dist[src] = 0
        changed = True
        rounds = 0
        while changed:
            changed = False
            rounds += 1
            assert rounds <= self.n + 1
            for u in range(self.n):
                du = dist[u]
                if du is None:
                    continue
                for v, w in self.rows[u].items():
                    nd = du + w
                    if dist[v] is None or nd < dist[v]:
                        dist[v] = nd
                        changed = True
        return np.array([INF32 if d is None else min(d, INF32) for d in dist], np.int32)
