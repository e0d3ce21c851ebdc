"""Key widths of the byte-width row layout (TinySetV_small) on the host: the
oracle's restatement and the library's sst_compact_widths against the
reference's own get_thresholds and get_b() (tests/golden/tinyset_widths.npz,
made by tests/golden/make_golden.py from the compiled reference)."""
import os

import numpy as np

from oracle import compact as oc

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                    "tinyset_widths.npz")


def test_oracle_thresholds_match_reference():
    d = np.load(GOLD)
    for mx, t in zip(d["max_el"].tolist(), d["thresholds"].tolist()):
        assert oc.widths(mx) == t, mx


def test_oracle_widths_match_reference_sets():
    d = np.load(GOLD)
    for mx, k, b in zip(d["width_max_el"].tolist(), d["width_count"].tolist(),
                        d["width"].tolist()):
        assert oc.width_of(k, oc.widths(mx)) == b, (mx, k)


def test_library_thresholds_match_reference():
    import sstgraph_gb300 as sg  # host function: no device needed
    d = np.load(GOLD)
    for mx, t in zip(d["max_el"].tolist(), d["thresholds"].tolist()):
        assert sg.compact_widths(mx) == t, mx


def test_published_thresholds_at_the_bench_shapes():
    # RMAT scale 24 rows: 3-byte keys from 4 ids, 2-byte from 4096 (256
    # buckets), 1-byte from 1,048,576 (65,536 buckets); scale 16: 2-byte
    # keys from 4 ids
    assert oc.widths(1 << 24) == [4, 4096, 1 << 20]
    assert oc.bucket_count(1 << 24, 2) == 256 and oc.bucket_count(1 << 24, 1) == 65536
    assert oc.width_of(4, oc.widths(1 << 16)) == 2
