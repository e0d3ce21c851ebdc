"""Structural invariants of the device PMA layout, checked on the host from
sstgraph_gb300.SparseMatrixV.raw_state():

* cap is 0 or a power of two; deg <= cap; cap > 0 exactly when deg > 0
* a segment starts on a multiple of min(cap, 32) and lies inside the slab
* one-leaf segment (cap <= 32): deg sorted ids packed left, EMPTY after
* multi-leaf segment: each leaf holds lcnt >= 1 ids packed left, EMPTY
  after, leaf counts sum to deg, ids strictly ascending across leaves
* live segments do not overlap
"""
import numpy as np

EMPTY = 0xFFFFFFFF


def check(g, expect_csr=None):
    base, cap, deg, slots, lcnt = g.raw_state()
    n = g.rows
    errors = []
    spans = []
    rows = []
    for v in range(n):
        c, d, b = int(cap[v]), int(deg[v]), int(base[v])
        if c & (c - 1):
            errors.append(f"v{v}: cap {c} not a power of two")
            continue
        if (c == 0) != (d == 0) or d > c:
            errors.append(f"v{v}: cap {c} deg {d}")
            continue
        if c == 0:
            rows.append(np.zeros(0, np.uint32))
            continue
        if b % min(c, 32) or b + c > len(slots):
            errors.append(f"v{v}: base {b} cap {c} slab {len(slots)}")
            continue
        spans.append((b, b + c, v))
        seg = slots[b:b + c]
        if c <= 32:
            vals = seg[:d]
            if np.any(seg[d:] != EMPTY):
                errors.append(f"v{v}: non-empty tail")
        else:
            cnts = lcnt[b // 32: (b + c) // 32].astype(np.int64)
            if np.any(cnts < 1) or np.any(cnts > 32):
                errors.append(f"v{v}: leaf counts {cnts.min()}..{cnts.max()}")
            if cnts.sum() != d:
                errors.append(f"v{v}: leaf counts sum {cnts.sum()} != deg {d}")
            leaves = seg.reshape(-1, 32)
            parts = []
            for li, k in enumerate(cnts):
                k = int(min(max(k, 0), 32))
                parts.append(leaves[li, :k])
                if np.any(leaves[li, k:] != EMPTY):
                    errors.append(f"v{v}: leaf {li} non-empty tail")
            vals = np.concatenate(parts) if parts else np.zeros(0, np.uint32)
        if np.any(vals == EMPTY) or np.any(np.diff(vals.astype(np.int64)) <= 0):
            errors.append(f"v{v}: ids not strictly ascending")
        rows.append(vals)
        if len(errors) > 20:
            break
    spans.sort()
    for (b0, e0, v0), (b1, e1, v1) in zip(spans, spans[1:]):
        if b1 < e0:
            errors.append(f"segments of v{v0} and v{v1} overlap")
            break
    if expect_csr is not None and not errors:
        off, cols = expect_csr
        for v in range(n):
            if not np.array_equal(rows[v], cols[off[v]:off[v + 1]]):
                errors.append(f"v{v}: neighbours differ from the oracle")
                if len(errors) > 10:
                    break
    return errors
