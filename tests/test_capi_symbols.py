"""The C-ABI library builds, loads without a GPU and exports every entry
point include/sstgraph.h declares (no compute calls)."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "sstgraph.h")).read()
    return sorted(set(re.findall(r"SST_API[^;(]*?\b(sst_\w+)\s*\(", src)))


def test_library_exports_header():
    from sstgraph_gb300 import build
    build.build()
    lib = ctypes.CDLL(build.LIB)
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    import sstgraph_gb300
    assert set(declared()) == set(sstgraph_gb300.SIGNATURES)


def test_no_device_means_error_not_fallback():
    import torch
    if torch.cuda.is_available():
        return
    import sstgraph_gb300 as sg
    try:
        sg.SparseMatrixV(10)
    except sg.SSTError as e:
        assert e.status == -5
    else:
        raise AssertionError("graph creation must fail without a GPU")
