"""Byte-width row layout of the reference's TinySetV_small, restated for
the tests (test infrastructure only).

* widths(max_el): get_thresholds (TinySet_small.hpp:227-263) -- the element
  counts at which a row's keys shrink from 4 to 3, 2 and 1 bytes, from the
  reference's memory model: count*b*2 bytes of keys plus, when the row needs
  more than one bucket, 12 bytes per bucket header
  (sizeof(PMA<sized_uint<4>>), PMA.hpp:170-175; find_best_b_for_given_
  element_count, TinySet_small.hpp:265-293).
* width_of(count, t): find_b_for_el_count (TinySet_small.hpp:204-214).
* bucket_count(max_el, b): calc_pma_count (TinySet_small.hpp:216-224);
  bucket of an id = id >> 8b (which_pma, TinySet_small.hpp:852-860).
* storage_bytes(degrees, max_el): bytes of the device snapshot that keeps
  every row in this layout: deg*b per row, plus 4*(buckets+1)+3 for the
  bucket directory of a multi-bucket row, plus the index (8 bytes of offset
  per row and one more, 4 bytes of length per row).

Pinned against the reference's own get_thresholds / get_b() by the fixture
tests/golden/tinyset_widths.npz (tests/golden/make_golden.py).
"""
from __future__ import annotations

import numpy as np

BUCKET_HEADER_BYTES = 12


def bucket_count(max_el: int, b: int) -> int:
    c = max(1, max_el >> (8 * b))
    if (c << (8 * b)) < max_el:
        c += 1
    return c


def _best_width(count: int, max_el: int) -> int:
    best, best_mem = None, None
    for b in (4, 3, 2, 1):
        pmas = bucket_count(max_el, b)
        mem = count * b * 2 + (0 if pmas == 1 else pmas * BUCKET_HEADER_BYTES)
        if best is None or mem < best_mem:
            best, best_mem = b, mem
    return best


def widths(max_el: int) -> list[int]:
    t24, t16, t8, cur = 2, 0, 0, 32
    c = 2
    while c < 0xFFFFFFFF // 2:
        b = _best_width(c, max_el)
        if b < cur:
            cur = b
            if b == 3:
                t24 = c * 2
            elif b == 2:
                t16 = c * 2
            elif b == 1:
                t8 = c * 2
        c *= 2
    if t16 <= t24:
        t16 = t24 * 2
    if t8 <= t16:
        t8 = t16 * 2
    return [t24, t16, t8]


def width_of(count: int, t) -> int:
    return 4 if count < t[0] else 3 if count < t[1] else 2 if count < t[2] else 1


def row_bytes(count: int, max_el: int, t) -> int:
    b = width_of(count, t)
    nb = bucket_count(max_el, b)
    return count * b + (4 * (nb + 1) + 3 if nb > 1 else 0)


def storage_bytes(degrees, max_el: int) -> int:
    t = widths(max_el)
    deg = np.asarray(degrees, np.int64)
    total = 0
    for d in np.unique(deg):
        total += int((deg == d).sum()) * row_bytes(int(d), max_el, t)
    return total + 8 * (len(deg) + 1) + 4 * len(deg)


def rows_per_width(degrees, max_el: int) -> dict:
    t = widths(max_el)
    out = {1: 0, 2: 0, 3: 0, 4: 0}
    for d, k in zip(*np.unique(np.asarray(degrees, np.int64), return_counts=True)):
        out[width_of(int(d), t)] += int(k)
    return out
