"""Calibrate the CPU baseline: the reference's own storage code against the
oracle port on the same update workload -- TEST INFRASTRUCTURE.

The GPU host cannot build the reference (its sources are not shipped
there), so the timed CPU arm of the benchmark is the C restatement in
sst_oracle.c.  This script, run where the reference tree is present, times
both on the same workload shape as the benchmark (RMAT base graph seed 5,
8 * 2^scale generated edges, symmetrised; insert batches of 95% new RMAT
edges seed 6 plus 5% existing edges, each followed by an equal-size delete
of sampled existing edges) and reports the reference's throughput as a
multiple of the port's, so the benchmark's ratio against the port can be
read against SSTGraph's own packed-memory-array code
(SparseMatrix.hpp:556-718 over PMA.hpp:1084-1363).

    python oracle/calibrate_ref.py [--scale 20] [--reps 2]

Both run with all host threads (OpenMP; the reference through the
ParallelTools stand-in in oracle/shim).  Prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402

RMAT = dict(a=0.57, b=0.19, c=0.19)
SIZES = [1000, 10000, 100000, 1000000]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args()
    oracle.build(ref=True)
    if not oracle.ref_available():
        print(json.dumps({"unavailable": "reference build (oracle/_ref) missing"}))
        return
    n = 1 << a.scale
    base = oracle.symmetrize(oracle.rmat(a.scale, 8 * n, seed=5, **RMAT))
    out = {"scale": a.scale, "threads": os.cpu_count(), "base_pairs": int(len(base)),
           "sizes": SIZES, "reps": a.reps}
    graphs = {}
    for name, cls in (("port", oracle.OracleGraph), ("reference", oracle.RefGraph)):
        t0 = time.perf_counter()
        g = cls(n)
        g.insert_batch(base)
        out[f"{name}_build_s"] = time.perf_counter() - t0
        graphs[name] = g
    # one stream of batches, drawn from the port (its sampler), applied to both
    first = 0
    t_ins = {"port": 0.0, "reference": 0.0}
    t_rem = {"port": 0.0, "reference": 0.0}
    edges = 0
    for rep in range(a.reps):
        for b in SIZES:
            dup = b // 20
            ins = np.concatenate([oracle.rmat(a.scale, b - dup, seed=6, first=first, **RMAT),
                                  graphs["port"].sample_edges(dup, seed=8, first=first)])
            rem = graphs["port"].sample_edges(b, seed=7, first=first + b)
            first += 2 * b
            edges += b
            for name, g in graphs.items():
                t0 = time.perf_counter()
                g.insert_batch(ins)
                t_ins[name] += time.perf_counter() - t0
                t0 = time.perf_counter()
                g.remove_batch(rem)
                t_rem[name] += time.perf_counter() - t0
    po, pc = graphs["port"].csr()
    ro, rc = graphs["reference"].csr()
    out["same_graph"] = bool(np.array_equal(po, ro) and np.array_equal(pc, rc))
    for name in graphs:
        out[f"{name}_insert_edges_per_s"] = edges / t_ins[name]
        out[f"{name}_remove_edges_per_s"] = edges / t_rem[name]
    out["reference_over_port_insert"] = t_ins["port"] / t_ins["reference"]
    out["reference_over_port_remove"] = t_rem["port"] / t_rem["reference"]
    print(json.dumps(out))


if __name__ == "__main__":
    main()
