"""Benchmark: SSTGraph's dynamic-graph hot path on one GB300.

Workload (default): RMAT scale-24 base graph (2^24 vertices, 8*2^24 generated
edges from stream seed 5, a/b/c/d = .57/.19/.19/.05, symmetrised -> ~268M
directed edges), then a stream of update batches whose sizes cycle through
1e3, 1e4, 1e5, 1e6 edges: each insert batch is 95% new RMAT edges (seed 6)
and 5% edges sampled from the graph (existing-edge duplicates), each followed
by an equal-size delete batch of edges sampled uniformly from the base graph.

One step = one insert batch + its delete batch.  `value` = inserted edges/s
(input batch size / insert time, as the reference reports,
internal/test.hpp:681-683) with batches resident in HBM; `e2e` = steps of
the same sizes with fresh batches through the C ABI from pinned host buffers
(host->device copy inside the timed call).  PageRank (FP64 pull, 10 iterations) and BFS from vertex 0 on
the updated graph are reported alongside, each with its HBM roofline.

--impl reference times the CPU implementation of the same path (the oracle
port in oracle/, all host threads) on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZES = [1000, 10000, 100000, 1000000]
RMAT = dict(a=0.57, b=0.19, c=0.19)


def strict(x):
    """The value with every non-finite float replaced by None (the printed
    lines are strict JSON)."""
    if isinstance(x, float) and not math.isfinite(x):
        return None
    if isinstance(x, dict):
        return {k: strict(v) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [strict(v) for v in x]
    return x


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def args_parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=24)
    ap.add_argument("--warmup", type=int, default=4)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=int, default=24)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle replay of the bench graph's batches")
    ap.add_argument("--pr-iters", type=int, default=10)
    ap.add_argument("--profile-batch", type=int, default=1000000,
                    help="--only insert-profile: pairs in the profiled batch")
    ap.add_argument("--profile-op", default="insert", choices=["insert", "remove"],
                    help="--only insert-profile: the profiled batch's operation")
    ap.add_argument("--algo", default="tc", choices=["bfs", "pagerank", "cc", "bc", "tc"],
                    help="--only algo-profile: the algorithm profiled")
    ap.add_argument("--graph", default="rmat", choices=["rmat", "er"],
                    help="--only algo-profile: RMAT (seed 3) or Erdos-Renyi (seed 4), "
                         "8 * 2^scale generated edges, symmetrised")
    ap.add_argument("--batched-batches", type=int, default=512)
    ap.add_argument("--serve-requests", type=int, default=400)
    # offered load of the serving latency run (requests/s): below the
    # measured capacity at scale 25, so the latencies are not queueing alone
    ap.add_argument("--serve-rate", type=float, default=150.0)
    ap.add_argument("--serve-scale", type=int, default=25)
    ap.add_argument("--only", default="all",
                    choices=["all", "updates", "pagerank", "bfs", "batched", "serving",
                             "multi", "compact", "extras", "static", "insert-profile",
                             "algo-profile"],
                    help="one part of the run (profiling cases): the update steps "
                         "alone, or one traversal on the base graph")
    return ap.parse_args()


def dist_init(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


class Clocks:
    """nvidia-smi sampler running across the timed region."""

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"sst_clocks_{os.getpid()}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev),
                 "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        # the timed region can be shorter than the sampling period: start it
        # only once the sampler is producing, and stop the sampler only after
        # it has taken one more sample
        self.lines0 = self._wait_lines(1)
        return self

    def _wait_lines(self, at_least, limit_s=3.0):
        t0 = time.time()
        while self.proc and time.time() - t0 < limit_s:
            self.f.flush()
            try:
                k = sum(1 for _ in open(self.path))
            except OSError:
                k = 0
            if k >= at_least:
                return k
            time.sleep(0.02)
        return 0

    def __exit__(self, *a):
        if self.proc:
            self._wait_lines(self.lines0 + 1)
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, val in zip(names, f[3:7]):
                if val.lower() == "active":
                    reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- workload
def batch_plan(steps, warmup):
    return [SIZES[i % len(SIZES)] for i in range(warmup + steps)]


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def run_cpu(scale, plan, label):
    """Oracle port on the host cores: build the base graph, then time
    insert / remove of each planned batch.  Returns (edges/s, details)."""
    import numpy as np

    import oracle
    oracle.build()
    n = 1 << scale
    t0 = time.time()
    base = oracle.symmetrize(oracle.rmat(scale, 8 * n, seed=5, **RMAT))
    o = oracle.OracleGraph(n)
    o.insert_batch(base)
    del base
    build_s = time.time() - t0
    ins_t = rem_t = 0.0
    ins_e = 0
    first = 0
    for i, b in enumerate(plan):
        k_new = b - b // 20
        ins = np.concatenate([oracle.rmat(scale, k_new, seed=6, first=first, **RMAT),
                              o.sample_edges(b // 20, seed=8, first=first)])
        first += b
        t = time.perf_counter()
        o.insert_batch(ins)
        ins_t += time.perf_counter() - t
        ins_e += b
        rem = o.sample_edges(b, seed=7, first=first)
        t = time.perf_counter()
        o.remove_batch(rem)
        rem_t += time.perf_counter() - t
    return ins_e / ins_t, {"build_s": round(build_s, 2), "insert_s": ins_t,
                           "remove_s": rem_t, "edges": ins_e,
                           "sample": label}


def check_parity(g, scale, applied):
    """Replay the bench graph's history on the oracle port (host threads):
    the scale-`scale` base graph, then every update batch in the order it
    was applied; compare the device graph's whole CSR with the oracle's."""
    import hashlib

    import numpy as np

    import oracle
    oracle.build()
    n = 1 << scale
    t0 = time.time()
    base = oracle.symmetrize(oracle.rmat(scale, 8 * n, seed=5, **RMAT))
    o = oracle.OracleGraph(n)
    o.insert_batch(base)
    del base
    for op, x in applied:
        getattr(o, op + "_batch")(x)
    off_o, col_o = o.csr()
    off_g, col_g = g.csr()
    equal = bool(o.M() == g.M() and np.array_equal(off_o, off_g) and
                 np.array_equal(col_o, col_g))
    digest = hashlib.sha256(off_g.tobytes())
    digest.update(col_g.tobytes())
    return {"equal": equal, "edges": int(g.M()), "batches_replayed": len(applied),
            "csr_sha256": digest.hexdigest(), "oracle_s": round(time.time() - t0, 2),
            "check": "whole CSR (offsets and columns) of the device graph after the "
                     "timed, end-to-end and kernel-pass batches = the oracle port's "
                     "after replaying the same base graph and batches"}


def reference_arm(a):
    rank, world = dist_init(a.gpus)
    if rank != 0:
        return
    plan = batch_plan(a.steps, a.warmup)[a.warmup:]
    v, det = run_cpu(a.scale, plan, f"all {len(plan)} timed batches ({sum(plan)} edges) "
                     f"of the workload on the scale-{a.scale} base graph")
    cores = cpu_threads()
    line = {
        "impl": "reference", "metric": "batch-insert edges/s", "value": v,
        "unit": "edges/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * (det["insert_s"] + det["remove_s"]) / max(len(plan), 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u32", "data": "synthetic RMAT (seeded)",
        "config": workload_config(a),
        "cpu_baseline": {"value": v, "unit": "edges/s", "cores": cores, "kind": "port",
                         "sample": det["sample"]},
        "e2e": {"value": v, "unit": "edges/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "detail": det,
        "note": "reference storage code cannot be built on the GPU host (its "
                "sources are not shipped there); the C restatement in oracle/ is timed",
    }
    print(json.dumps(strict(line), allow_nan=False))


def workload_config(a):
    n = 1 << a.scale
    return {"workload": f"dynamic updates on RMAT scale-{a.scale}",
            "vertices": n, "base_generated_edges": 8 * n, "symmetrised": True,
            "rmat_abcd": [0.57, 0.19, 0.19, 0.05], "seeds": {"base": 5, "insert": 6,
                                                             "delete": 7, "dup": 8},
            "batch_sizes": SIZES, "dup_fraction": 0.05,
            "step": "insert batch + equal-size delete batch",
            "l2": "flushed (256 MiB write) between timed steps",
            "parallelism": "replicas" if a.gpus > 1 else "single GPU"}


def insert_profile(a):
    """One update batch for a profiler: the scale-`scale` RMAT base graph
    (seed 5, symmetrised), a warm-up batch of `profile_batch` pairs (it
    grows the scratch and captures the planning graph), then one more such
    batch between cudaProfilerStart and cudaProfilerStop, so
    `ncu --profile-from-start off` sees that batch's launches alone.
    Inserts are RMAT pairs (seed 6); with --profile-op remove the batches
    are existing edges sampled from the graph (seed 7)."""
    import torch

    import sstgraph_gb300 as sg
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    n = 1 << a.scale
    g = sg.SparseMatrixV(n, initial_slots=int(3.2 * 16 * n))
    g.set_stream(stream.cuda_stream)
    b = a.profile_batch
    with torch.cuda.stream(stream):
        x = torch.empty((8 * n, 2), dtype=torch.int32, device="cuda")
        sg.gen_rmat(a.scale, 8 * n, seed=5, out=x, **RMAT)
        g.insert_batch(x)
        g.insert_batch(x.flip(1).contiguous())
        del x
        ys = [torch.empty((b, 2), dtype=torch.int32, device="cuda") for _ in range(2)]
        for i, y in enumerate(ys):
            sg.gen_rmat(a.scale, b, seed=6, first=i * b, out=y, **RMAT)
    torch.cuda.synchronize()
    op = g.insert_batch
    if a.profile_op == "remove":
        op = g.remove_batch
        for i, y in enumerate(ys):
            g.sample_edges(b, seed=7, first=i * b, out=y)
        torch.cuda.synchronize()
    op(ys[0])
    torch.cuda.synchronize()
    e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
    torch.cuda.profiler.start()
    e0.record(stream)
    op(ys[1])
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"only": "insert-profile", "op": a.profile_op, "scale": a.scale,
                      "batch": b, "edges": g.M(), "batch_us": e0.elapsed_time(e1) * 1e3}))
    g.close()


def algo_profile(a):
    """One call of one algorithm for a profiler: the static-analytics graph
    (RMAT seed 3 or Erdos-Renyi seed 4, 8 * 2^scale generated edges,
    symmetrised), one warm-up call, then one call between cudaProfilerStart
    and cudaProfilerStop."""
    import torch

    import sstgraph_gb300 as sg
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    n = 1 << a.scale
    g = sg.SparseMatrixV(n)
    g.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        x = torch.empty((8 * n, 2), dtype=torch.int32, device="cuda")
        if a.graph == "rmat":
            sg.gen_rmat(a.scale, 8 * n, seed=3, out=x, **RMAT)
        else:
            sg.gen_er(n, 8 * n, seed=4, out=x)
        g.insert_batch(x)
        g.insert_batch(x.flip(1).contiguous())
        del x
    torch.cuda.synchronize()
    g.release_scratch()
    sg.autotune(g)
    out = {"pagerank": torch.empty(n, dtype=torch.float64, device="cuda"),
           "bc": torch.empty(n, dtype=torch.float64, device="cuda")}
    d = torch.empty(n, dtype=torch.int32, device="cuda")
    run = {"bfs": lambda: sg.BFS(g, 0, depths=True, out=d),
           "pagerank": lambda: sg.PR_S(g, 20, out=out["pagerank"]),
           "cc": lambda: sg.CC(g, out=d),
           "bc": lambda: sg.BC(g, 0, out=out["bc"]),
           "tc": lambda: sg.TC(g)}[a.algo]
    run()
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    torch.cuda.profiler.start()
    run()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    print(json.dumps({"only": "algo-profile", "algo": a.algo, "graph": a.graph,
                      "scale": a.scale, "edges": g.M(), "best_ms": best}))
    g.close()


def main():
    a = args_parse()
    if a.impl == "reference":
        return reference_arm(a)
    if a.only == "insert-profile":
        return insert_profile(a)
    if a.only == "algo-profile":
        return algo_profile(a)
    import numpy as np
    import torch

    import sstgraph_gb300 as sg
    rank, world = dist_init(a.gpus)
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    sg.lib()
    stream = torch.cuda.Stream()
    n = 1 << a.scale
    hbm_peak, peak_kind = peaks()

    # ---- base graph (setup, untimed)
    g = sg.SparseMatrixV(n, device=dev, initial_slots=int(3.2 * 16 * n))
    g.set_stream(stream.cuda_stream)
    chunk = 1 << 25
    total = 8 * n
    t0 = time.time()
    with torch.cuda.stream(stream):
        buf = torch.empty((chunk, 2), dtype=torch.int32, device="cuda")
        for first in range(0, total, chunk):
            k = min(chunk, total - first)
            sg.gen_rmat(a.scale, k, seed=5, first=first, out=buf[:k], **RMAT)
            g.insert_batch(buf[:k])
            g.insert_batch(buf[:k].flip(1).contiguous())
        del buf
    torch.cuda.synchronize()
    build_s = time.time() - t0
    m0 = g.M()

    def measure_pagerank(gg=None):
        gg = gg or g
        m = gg.M()
        with torch.cuda.stream(stream):
            out = torch.empty(n, dtype=torch.float64, device="cuda")
            sg.PR_S(gg, 1, out=out)  # warm: work lists
        torch.cuda.synchronize()
        prt = {}
        for it in (a.pr_iters, 2 * a.pr_iters):
            best = 1e30
            for _ in range(3):
                with torch.cuda.stream(stream):
                    pr_flush.fill_(it)
                s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s0.record(stream)
                sg.PR_S(gg, it, out=out)
                s1.record(stream)
                s1.synchronize()
                best = min(best, s0.elapsed_time(s1) / 1e3)
            prt[it] = best
        t_iter = (prt[2 * a.pr_iters] - prt[a.pr_iters]) / a.pr_iters
        pr_bytes = 4 * m + 24 * n
        pr_gbs = pr_bytes / t_iter / 1e9
        sg.profile_start()
        sg.PR_S(gg, a.pr_iters, out=out)
        torch.cuda.synchronize()
        pr_prof = sg.profile_collect()
        pagerank = {"gteps": m / t_iter / 1e9, "ms_per_iter": t_iter * 1e3,
                    "algorithmic_bytes_per_iter": pr_bytes,
                    "roofline": {"bound": "hbm", "achieved": pr_gbs, "peak": hbm_peak,
                                 "unit": "GB/s", "frac": pr_gbs / hbm_peak,
                                 "peak_kind": peak_kind, "traffic": None,
                                 "kernels": "one iteration = k_pr_small + k_pr_chunks + k_pr_fix"},
                    "kernels": pr_prof}
        return pagerank

    def measure_compact():
        """Byte-width snapshot of the bench graph (sst_compact_*): build time,
        storage against the live PMA graph, and PageRank read from the
        compressed rows (bit-equal to sst_pagerank) against the PMA PageRank."""
        m = g.M()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        c = sg.CompactGraph(g)
        build_s = time.perf_counter() - t0
        c.set_stream(stream.cuda_stream)
        info = c.info()
        out = torch.empty(n, dtype=torch.float64, device="cuda")
        c.pagerank(1, out=out)
        torch.cuda.synchronize()
        prt = {}
        for it in (a.pr_iters, 2 * a.pr_iters):
            best = 1e30
            for _ in range(3):
                with torch.cuda.stream(stream):
                    pr_flush.fill_(it)
                s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s0.record(stream)
                c.pagerank(it, out=out)
                s1.record(stream)
                s1.synchronize()
                best = min(best, s0.elapsed_time(s1) / 1e3)
            prt[it] = best
        t_iter = (prt[2 * a.pr_iters] - prt[a.pr_iters]) / a.pr_iters
        ref = torch.empty(n, dtype=torch.float64, device="cuda")
        with torch.cuda.stream(stream):
            sg.PR_S(g, a.pr_iters, out=ref)
            c.pagerank(a.pr_iters, out=out)
        torch.cuda.synchronize()
        equal = bool(torch.equal(out.view(torch.int64), ref.view(torch.int64)))
        sg.profile_start()
        c.pagerank(a.pr_iters, out=out)
        torch.cuda.synchronize()
        cprof = sg.profile_collect()
        sg.profile_start()
        sg.PR_S(g, a.pr_iters, out=ref)
        torch.cuda.synchronize()
        pprof = sg.profile_collect()
        # the other traversals on the snapshot beside the live graph's
        trav = {}

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            r = fn()
            s1.record(stream)
            s1.synchronize()
            return s0.elapsed_time(s1), r

        d1 = torch.empty(n, dtype=torch.int32, device="cuda")
        d2 = torch.empty(n, dtype=torch.int32, device="cuda")
        for name, on_snap, on_live, same in (
                ("bfs", lambda: c.bfs(0, out=d1), lambda: sg.BFS(g, 0, depths=True, out=d2),
                 lambda: bool(torch.equal(d1, d2))),
                ("cc", lambda: c.cc(out=d1), lambda: sg.CC(g, out=d2),
                 lambda: bool(torch.equal(d1, d2)))):
            ms_s, _ = timed(on_snap)
            ms_l, _ = timed(on_live)
            trav[name] = {"snapshot_ms": ms_s, "graph_ms": ms_l, "equal": same()}
        b1 = torch.empty(n, dtype=torch.float64, device="cuda")
        b2 = torch.empty(n, dtype=torch.float64, device="cuda")
        ms_s, _ = timed(lambda: c.bc(0, out=b1))
        ms_l, _ = timed(lambda: sg.BC(g, 0, out=b2))
        # after the update stream the graph is directed (inserts are not
        # symmetrised), where BC is not defined: the difference is reported,
        # not judged (BC parity is tested on symmetric graphs)
        # (a directed graph can leave vertices with no shortest-path count
        # under the symmetric formulation: their values are not finite, and
        # are counted, not compared)
        fin = torch.isfinite(b1) & torch.isfinite(b2)
        nfin = int((~fin).sum().item())
        diff = (b1 - b2)[fin].abs().max().item() if nfin < n else 0.0
        scale = b2[fin].abs().max().item() if nfin < n else 0.0
        trav["bc"] = {"snapshot_ms": ms_s, "graph_ms": ms_l,
                      "max_rel_diff_on_directed_graph": diff / max(scale, 1e-300),
                      "nonfinite_entries": nfin,
                      "nonfinite_in_same_places":
                          bool(torch.equal(torch.isfinite(b1), torch.isfinite(b2)))}
        ms_s, t_s = timed(lambda: c.tc())
        ms_l, t_l = timed(lambda: sg.TC(g))
        trav["tc"] = {"snapshot_ms": ms_s, "graph_ms": ms_l, "equal": t_s == t_l}
        del d1, d2, b1, b2
        # the live graph's storage: vertex table (base, cap, deg) and the
        # slab's used slots with their leaf counts
        nslots = ctypes.c_uint64()
        sg.lib().sst_raw_state(g.handle, None, None, None, None, None, ctypes.byref(nslots))
        pma_storage = 16 * n + 4 * nslots.value + nslots.value // 32
        c.close()
        return {"build_s": build_s, "edges": m,
                "storage_bytes": info["storage_bytes"],
                "bytes_per_edge": info["storage_bytes"] / max(m, 1),
                "pma_storage_bytes": pma_storage,
                "pma_bytes_per_edge": pma_storage / max(m, 1),
                "graph_device_bytes": g.get_memory_size(),
                "rows_per_width": info["rows_per_width"],
                "pagerank_ms_per_iter": t_iter * 1e3,
                "pagerank_bytes_per_iter": info["storage_bytes"] + 24 * n,
                "pagerank_equal_to_pma": equal,
                "traversals": trav,
                "kernels": cprof, "pma_kernels": pprof}

    def measure_bfs():
        m = g.M()
        dep = torch.empty(n, dtype=torch.int32, device="cuda")
        sg.BFS(g, 0, depths=True, out=dep)
        torch.cuda.synchronize()
        bt = 1e30
        for _ in range(3):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            sg.BFS(g, 0, depths=True, out=dep)
            s1.record(stream)
            s1.synchronize()
            bt = min(bt, s0.elapsed_time(s1) / 1e3)
        degs = torch.from_numpy(g.degrees().astype(np.int64))
        reached = (dep.cpu() >= 0)
        m_r = int(degs[reached].sum())
        sg.profile_start()
        sg.BFS(g, 0, depths=True, out=dep)
        torch.cuda.synchronize()
        bfs = {"gteps": m_r / bt / 1e9, "ms": bt * 1e3, "reached": int(reached.sum()),
               "edges_reached": m_r,
               "roofline": {"bound": "hbm", "achieved": (4 * m_r + 12 * n) / bt / 1e9,
                            "peak": hbm_peak, "unit": "GB/s",
                            "frac": (4 * m_r + 12 * n) / bt / 1e9 / hbm_peak},
               "kernels": sg.profile_collect()}
        return bfs

    def measure_extras():
        """The rows beside the update path: parse and device build of a .mtx
        file (sst_read_graph_file, sst_load_graph_file) and Bellman-Ford
        (sst_bf) on a weighted RMAT graph."""
        res = {}
        # ingest: RMAT scale 18, 16 generated edges per vertex, one line each
        sc, per = 18, 16
        nn = 1 << sc
        k = per * nn
        x = torch.empty((k, 2), dtype=torch.int32, device="cuda")
        with torch.cuda.stream(stream):
            sg.gen_rmat(sc, k, seed=21, out=x, **RMAT)
        torch.cuda.synchronize()
        e = (x.cpu().numpy().astype(np.int64) + 1).astype(str)  # 1-based ids
        body = "\n".join(np.char.add(np.char.add(e[:, 0], " "), e[:, 1]).tolist())
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, f"rmat{sc}.mtx")
            with open(path, "w") as f:
                f.write(f"%%MatrixMarket matrix coordinate pattern symmetric\n{nn} {nn} {k}\n")
                f.write(body + "\n")
            size = os.path.getsize(path)
            t0 = time.perf_counter()
            rows, pairs = sg.read_graph_file(path)
            t_read = time.perf_counter() - t0
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gl = sg.load_graph_file(path, device=dev)
            gl.sync()
            t_load = time.perf_counter() - t0
            m_l = gl.M()
            gl.close()
        res["ingest"] = {"file": f"RMAT scale {sc}, {k} lines (.mtx, symmetric)",
                         "file_bytes": size, "pairs": int(len(pairs)),
                         "read_s": t_read, "read_mb_per_s": size / t_read / 1e6,
                         "load_s": t_load, "stored_edges": m_l,
                         "load_edges_per_s": m_l / t_load,
                         "note": "read: parse to host pairs; load: parse, then the "
                                 "device bulk build"}
        # Bellman-Ford: RMAT scale 22, 16 edges per vertex, values 1..255
        sc = 22
        nn = 1 << sc
        k = 16 * nn
        gw = sg.SparseMatrixV(nn, device=dev, weighted=True)
        gw.set_stream(stream.cuda_stream)
        gen = torch.Generator(device="cuda").manual_seed(22)
        with torch.cuda.stream(stream):
            x = torch.empty((k, 2), dtype=torch.int32, device="cuda")
            sg.gen_rmat(sc, k, seed=22, out=x, **RMAT)
            v = torch.randint(1, 256, (k,), dtype=torch.int32, device="cuda", generator=gen)
            gw.insert_batch_weighted(x, v)
            out = torch.empty(nn, dtype=torch.int32, device="cuda")
            sg.BF(gw, 0, out=out)
        torch.cuda.synchronize()
        bt = 1e30
        for _ in range(3):
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            sg.BF(gw, 0, out=out)
            s1.record(stream)
            s1.synchronize()
            bt = min(bt, s0.elapsed_time(s1) / 1e3)
        reached = int((out < 2 ** 31 - 1).sum().item())
        res["bellman_ford"] = {"graph": f"weighted RMAT scale {sc}, {k} generated edges, "
                                        "values 1..255", "edges": gw.M(), "ms": bt * 1e3,
                               "reached": reached, "edges_per_s": gw.M() / bt}
        gw.close()
        return res

    def measure_static():
        """Static analytics at scale (RMAT scale 22, 8 * 2^22 generated edges,
        seed 3; Erdos-Renyi, 2^22 vertices, average degree 16, seed 4; both
        symmetrised): BFS from 0, PageRank 20 iterations, CC, BC from 0 and
        TC on the device (best of 3 after a warm-up, CUDA events), each with
        its HBM roofline from its algorithmic bytes, beside the oracle port
        on all host threads (one warm-up, then one timed run) on the same
        graph, whose results are checked against the device's (depths, CC
        labels and triangle counts equal; PageRank and BC within 1e-9)."""
        import oracle
        oracle.build()
        out = {}
        nn = 1 << 22
        specs = [("rmat22", lambda x, first, k: sg.gen_rmat(22, k, seed=3, first=first,
                                                             out=x, **RMAT),
                  lambda: oracle.rmat(22, 8 * nn, seed=3, **RMAT)),
                 ("er22", lambda x, first, k: sg.gen_er(nn, k, seed=4, first=first, out=x),
                  lambda: oracle.er(nn, 8 * nn, seed=4))]
        for name, dev_gen, cpu_gen in specs:
            gg = sg.SparseMatrixV(nn, device=dev)
            gg.set_stream(stream.cuda_stream)
            total, ch = 8 * nn, 1 << 24
            with torch.cuda.stream(stream):
                x = torch.empty((ch, 2), dtype=torch.int32, device="cuda")
                for first in range(0, total, ch):
                    k = min(ch, total - first)
                    dev_gen(x[:k], first, k)
                    gg.insert_batch(x[:k])
                    gg.insert_batch(x[:k].flip(1).contiguous())
                del x
            torch.cuda.synchronize()
            m = gg.M()
            tuning = sg.autotune(gg)
            off, cols = gg.csr()
            deg = np.diff(off.astype(np.int64))
            rows = np.repeat(np.arange(nn, dtype=np.int64), deg)
            # TC reads: every stored id once (orientation), the oriented
            # lists N+ written and read back into the per-u sets, and every
            # entry of N+(v) for each oriented edge (u, v) probed once;
            # the orientation keeps an edge at its lower (degree, id) rank
            c64 = cols.astype(np.int64)
            rank_r = deg[rows] * nn + rows
            rank_c = deg[c64] * nn + c64
            up = rank_c > rank_r
            dplus = np.bincount(rows[up], minlength=nn).astype(np.int64)
            m_plus = int(up.sum())
            probes = int(dplus[c64[up]].sum())
            tc_bytes = 4 * m + 8 * m_plus + 4 * probes
            del off, cols, rows, c64, rank_r, rank_c, up, dplus
            dep = torch.empty(nn, dtype=torch.int32, device="cuda")
            pr = torch.empty(nn, dtype=torch.float64, device="cuda")
            lab = torch.empty(nn, dtype=torch.int32, device="cuda")
            bc = torch.empty(nn, dtype=torch.float64, device="cuda")
            tcv = {}
            runs = {"bfs": lambda: sg.BFS(gg, 0, depths=True, out=dep),
                    "pagerank20": lambda: sg.PR_S(gg, 20, out=pr),
                    "cc": lambda: sg.CC(gg, out=lab),
                    "bc": lambda: sg.BC(gg, 0, out=bc),
                    "tc": lambda: tcv.__setitem__("t", sg.TC(gg))}
            gpu = {}
            for alg, fn in runs.items():
                fn()
                torch.cuda.synchronize()
                best = 1e30
                for _ in range(3):
                    with torch.cuda.stream(stream):
                        pr_flush.fill_(1)
                    s0, s1 = (torch.cuda.Event(enable_timing=True) for _ in range(2))
                    s0.record(stream)
                    fn()
                    s1.record(stream)
                    s1.synchronize()
                    best = min(best, s0.elapsed_time(s1) / 1e3)
                gpu[alg] = best
            d_dep = dep.cpu().numpy()
            m_r = int(deg[d_dep >= 0].sum())
            byts = {"bfs": 4 * m_r + 12 * nn, "pagerank20": 20 * (4 * m + 24 * nn),
                    "cc": 4 * m + 8 * nn, "bc": 8 * m_r + 28 * nn,
                    "tc": tc_bytes}
            res = {"vertices": nn, "edges": m, "tuning": tuning, "bfs_edges_reached": m_r,
                   "triangles": tcv["t"], "algorithms": {}}
            # the oracle port on the same graph, all host threads
            pairs = oracle.symmetrize(cpu_gen())
            t0 = time.perf_counter()
            o = oracle.OracleGraph(nn)
            o.insert_batch(pairs)
            res["cpu_build_s"] = time.perf_counter() - t0
            del pairs
            cpu_fn = {"bfs": lambda: o.bfs(0), "pagerank20": lambda: o.pagerank(20),
                      "cc": o.cc, "bc": lambda: o.bc(0), "tc": o.tc}
            cpu, cres = {}, {}
            for alg, fn in cpu_fn.items():
                if alg != "tc":
                    fn()
                t0 = time.perf_counter()
                cres[alg] = fn()
                cpu[alg] = time.perf_counter() - t0
            dev_res = {"bfs": d_dep, "pagerank20": pr.cpu().numpy(), "cc": lab.cpu().numpy(),
                       "bc": bc.cpu().numpy(), "tc": tcv["t"]}

            def agree(alg):
                a, b = dev_res[alg], cres[alg]
                if alg in ("pagerank20", "bc"):
                    return bool(np.max(np.abs(a - b)) <= 1e-9 * max(np.max(np.abs(b)), 1e-300))
                if alg == "cc":
                    return bool(np.array_equal(a.view(np.uint32), b))
                return bool(np.array_equal(a, b))
            for alg in runs:
                gbs = byts[alg] / gpu[alg] / 1e9
                r = {"gpu_ms": 1e3 * gpu[alg], "cpu_ms": 1e3 * cpu[alg],
                     "speedup": cpu[alg] / gpu[alg], "algorithmic_bytes": byts[alg],
                     "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm_peak,
                                  "unit": "GB/s", "frac": gbs / hbm_peak},
                     "matches_oracle": agree(alg)}
                if alg == "bfs":
                    r["gteps"] = m_r / gpu[alg] / 1e9
                if alg == "pagerank20":
                    r["gteps"] = 20 * m / gpu[alg] / 1e9
                res["algorithms"][alg] = r
            res["cpu_cores"] = cpu_threads()
            out[name] = res
            del o
            gg.close()
        out["bytes"] = {"bfs": "4 m_r + 12 n", "pagerank20": "20 (4 m + 24 n)",
                        "cc": "4 m + 8 n (one pass over the edges and labels)",
                        "bc": "8 m_r + 28 n",
                        "tc": "sum over (u, v), v < u of 4 (d<(u) + d<(v)) + 4 m"}
        return out

    def measure_multi():
        """64-source BFS and 16-source BC (uniform sources) in one call each,
        against the same sources run one call per source."""
        rng = np.random.default_rng(17)
        res = {}
        for kind, k in (("bfs", 64), ("bc", 16)):
            srcs = rng.integers(0, n, k).astype(np.uint32)
            dt = torch.int32 if kind == "bfs" else torch.float64
            out = torch.empty((k, n), dtype=dt, device="cuda")
            one = torch.empty(n, dtype=dt, device="cuda")
            multi_fn = sg.BFS_multi if kind == "bfs" else sg.BC_multi

            def single(s):
                if kind == "bfs":
                    sg.BFS(g, int(s), depths=True, out=one)
                else:
                    sg.BC(g, int(s), out=one)
            multi_fn(g, srcs, out=out)  # warm
            torch.cuda.synchronize()
            t = {}
            for form in ("multi", "single"):
                s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s0.record(stream)
                if form == "multi":
                    multi_fn(g, srcs, out=out)
                else:
                    for sidx in srcs:
                        single(sidx)
                s1.record(stream)
                s1.synchronize()
                t[form] = s0.elapsed_time(s1) / 1e3
            # spot check: the last source's row equals its single-source result
            single(srcs[-1])
            torch.cuda.synchronize()
            same = bool(torch.equal(out[k - 1], one))
            res[kind] = {"sources": k, "multi_ms": 1e3 * t["multi"],
                         "single_ms": 1e3 * t["single"],
                         "speedup": t["single"] / t["multi"], "last_row_equal": same}
            del out
        return res

    def measure_batched(reps=3):
        """The batched-form configuration: 512 update batches with log-normal
        sizes (floor(exp(N(ln 1e4, 1.5))), capped at 1e7, no lower clip);
        every fourth batch removes edges sampled from the graph, the others
        insert RMAT edges.  The same stream is applied to device copies of
        the graph in two forms: one insert_batch / remove_batch call per
        batch (plain) and one update_batches call for the whole stream
        (batched).  Each copy first takes a disjoint warm-up stream of the
        same sizes in the same form (untimed: scratch grown, kernels loaded),
        so the timed stream measures the steady state; median of `reps`
        copies per form.  The two forms' final graphs are compared whole
        (CSR)."""
        rng = np.random.default_rng(11)
        sizes = np.minimum(np.floor(np.exp(rng.normal(np.log(1e4), 1.5, a.batched_batches))),
                           1e7).astype(np.int64)
        sizes = np.maximum(sizes, 1)
        ops = [0 if i % 4 == 3 else 1 for i in range(len(sizes))]

        def stream_of(first):
            out = []
            with torch.cuda.stream(stream):
                for sz, op in zip(sizes.tolist(), ops):
                    x = torch.empty((sz, 2), dtype=torch.int32, device="cuda")
                    if op:
                        sg.gen_rmat(a.scale, sz, seed=12, first=first, out=x, **RMAT)
                    else:
                        g.sample_edges(sz, seed=14, first=first, out=x)
                    first += sz
                    out.append(x)
            return out

        total_e = int(sizes.sum())
        warm, bl = stream_of(0), stream_of(total_e)
        torch.cuda.synchronize()
        res = {}
        csr = {}
        for form in ("plain", "batched"):
            times, checks = [], []
            for rep in range(reps):
                gc = g.copy()
                gc.set_stream(stream.cuda_stream)
                if form == "plain":
                    for x, op in zip(warm, ops):
                        (gc.insert_batch if op else gc.remove_batch)(x)
                else:
                    gc.update_batches(warm, ops)
                torch.cuda.synchronize()
                s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s0.record(stream)
                if form == "plain":
                    for x, op in zip(bl, ops):
                        (gc.insert_batch if op else gc.remove_batch)(x)
                else:
                    gc.update_batches(bl, ops)
                s1.record(stream)
                s1.synchronize()
                times.append(s0.elapsed_time(s1) / 1e3)
                checks.append([gc.M(), gc.touch_all_sum()])
                if rep == 0:
                    csr[form] = gc.csr()
                gc.close()
            t = float(np.median(times))
            res[form] = {"edges_per_s": total_e / t, "s": t, "check": checks[0],
                         "same_each_rep": all(c == checks[0] for c in checks)}
        same = (res["plain"]["check"] == res["batched"]["check"] and
                res["plain"]["same_each_rep"] and res["batched"]["same_each_rep"] and
                all(np.array_equal(x, y) for x, y in zip(csr["plain"], csr["batched"])))
        del csr
        return {"batches": len(bl), "edges": total_e, "reps": reps,
                "removes": int(len(ops) - sum(ops)),
                "sizes": {"min": int(sizes.min()), "median": int(np.median(sizes)),
                          "mean": float(sizes.mean()), "max": int(sizes.max())},
                "plain_edges_per_s": res["plain"]["edges_per_s"],
                "batched_edges_per_s": res["batched"]["edges_per_s"],
                "plain_s": res["plain"]["s"], "batched_s": res["batched"]["s"],
                "speedup": res["batched"]["edges_per_s"] / res["plain"]["edges_per_s"],
                "same_graph": same,
                "check": "whole CSR, M and touch_all_sum of both forms' final graphs"}

    def measure_serving():
        """The serving configuration: an RMAT scale-`serve_scale` graph (8 * n
        generated edges, seed 7, symmetrised) held on the device, its bulk-
        load scratch released, served under a 60 GB HBM budget.  Requests:
        70% update batches (log-normal sizes, median 1e3, sigma 1, at most
        1e5; 30% of them remove edges sampled from the graph, the rest insert
        RMAT edges), 30% queries split evenly between single-source BFS, a
        5-iteration PageRank refresh and per-vertex triangle counts of 1e4
        random vertices.  Two runs: Poisson arrivals at `serve_rate`/s for
        latency (completion - arrival), then every request of a second stream
        offered at once (load above capacity) for the sustained rates."""
        sc = a.serve_scale
        nn = 1 << sc
        gs = sg.SparseMatrixV(nn, device=dev, initial_slots=int(3.2 * 16 * nn))
        gs.set_stream(stream.cuda_stream)
        total, ch = 8 * nn, 1 << 25
        t0 = time.time()
        with torch.cuda.stream(stream):
            x = torch.empty((ch, 2), dtype=torch.int32, device="cuda")
            for first in range(0, total, ch):
                k = min(ch, total - first)
                sg.gen_rmat(sc, k, seed=7, first=first, out=x[:k], **RMAT)
                gs.insert_batch(x[:k])
                gs.insert_batch(x[:k].flip(1).contiguous())
            del x
        torch.cuda.synchronize()
        build_s = time.time() - t0
        mem_loaded = gs.get_memory_size()
        gs.release_scratch()
        mem_trimmed = gs.get_memory_size()
        rng = np.random.default_rng(31)
        first = [0]

        def make_requests(count):
            reqs = []
            for _ in range(count):
                r = rng.random()
                if r < 0.7:
                    sz = int(min(1e5, max(1, rng.lognormal(np.log(1e3), 1.0))))
                    if rng.random() < 0.3:
                        reqs.append(("remove", gs.sample_edges(sz, seed=15, first=first[0])))
                    else:
                        reqs.append(("insert", sg.gen_rmat(sc, sz, seed=13, first=first[0],
                                                           **RMAT)))
                    first[0] += sz
                elif r < 0.8:
                    reqs.append(("bfs", int(rng.integers(0, nn))))
                elif r < 0.9:
                    reqs.append(("pagerank", 5))
                else:
                    reqs.append(("tc", rng.integers(0, nn, 10000).astype(np.uint32)))
            return reqs

        def run(srv, reqs, arrive):
            tickets = []
            t0 = time.perf_counter()
            for (kind, arg), at in zip(reqs, arrive):
                if at is not None:
                    now = time.perf_counter()
                    if t0 + at > now:
                        time.sleep(t0 + at - now)
                if kind == "insert":
                    t = srv.insert(arg)
                elif kind == "remove":
                    t = srv.remove(arg)
                elif kind == "bfs":
                    t = srv.bfs(arg)
                elif kind == "pagerank":
                    t = srv.pagerank(arg)
                else:
                    t = srv.tc_vertices(arg)
                tickets.append((kind, t, arg, time.perf_counter() - t0))
            lat = {}
            upd_edges = queries = 0
            upd_end = qry_end = 0.0  # completion of the last update / query
            for kind, t, arg, at in tickets:
                _, info = srv.wait(t)
                lat.setdefault(kind, []).append(info["total_ms"])
                end = at + info["total_ms"] / 1e3
                if kind in ("insert", "remove"):
                    upd_edges += len(arg)
                    upd_end = max(upd_end, end)
                else:
                    queries += 1
                    qry_end = max(qry_end, end)
            wall = time.perf_counter() - t0
            allv = [x for v in lat.values() for x in v]
            return {"requests": len(reqs), "wall_s": wall,
                    "p50_ms": float(np.percentile(allv, 50)),
                    "p99_ms": float(np.percentile(allv, 99)),
                    "by_kind": {k: {"n": len(v), "p50_ms": float(np.percentile(v, 50)),
                                    "p99_ms": float(np.percentile(v, 99))}
                                for k, v in lat.items()},
                    "update_edges": upd_edges, "updates_done_s": upd_end,
                    "update_edges_per_s": upd_edges / max(upd_end, 1e-9),
                    "queries": queries, "queries_done_s": qry_end,
                    "queries_per_s": queries / max(qry_end, 1e-9)}

        lat_reqs = make_requests(a.serve_requests)
        sat_reqs = make_requests(2 * a.serve_requests)
        srv = sg.Server(gs, query_slots=4, hbm_budget_bytes=60 << 30)
        slots = srv.slots
        gaps = rng.exponential(1.0 / a.serve_rate, len(lat_reqs))
        latency = run(srv, lat_reqs, np.cumsum(gaps).tolist())
        latency["rate_per_s"] = a.serve_rate
        sat = run(srv, sat_reqs, [None] * len(sat_reqs))
        sat["offered"] = "all requests submitted at once (offered load above capacity)"
        st = srv.stats()
        srv.close()
        out = {"scale": sc, "vertices": nn, "edges": gs.M(), "build_s": build_s,
               "graph_bytes_after_load": mem_loaded, "graph_bytes_trimmed": mem_trimmed,
               "hbm_budget_bytes": 60 << 30, "slots": slots,
               "p50_ms": latency["p50_ms"], "p99_ms": latency["p99_ms"],
               "sustained_update_edges_per_s": sat["update_edges_per_s"],
               "latency_run": latency, "saturation_run": sat,
               "writer_passes": st["passes"]}
        gs.close()
        return out

    if a.only not in ("all", "updates"):
        pr_flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")
        res = {"only": a.only, "scale": a.scale, "edges": m0}
        if a.only == "pagerank":
            res["pagerank"] = measure_pagerank()
        elif a.only == "serving":
            res["serving"] = measure_serving()
        elif a.only == "batched":
            res["batched"] = measure_batched()
        elif a.only == "multi":
            res["multi_source"] = measure_multi()
        elif a.only == "extras":
            res["extras"] = measure_extras()
        elif a.only == "compact":
            res["compact"] = measure_compact()
        elif a.only == "static":
            res["static_analytics"] = measure_static()
        else:
            res["bfs"] = measure_bfs()
        g.close()
        print(json.dumps(strict(res), allow_nan=False))
        return

    # ---- batches: inserts are 95% new RMAT edges and 5% sampled existing
    # edges, removes are sampled existing edges (sampled from the graph as it
    # is when the batches are made)
    plan = batch_plan(a.steps, a.warmup)

    def make_batches(first, host, sizes=None):
        ins, rem = [], []
        with torch.cuda.stream(stream):
            for b in (plan if sizes is None else sizes):
                k_new = b - b // 20
                x = torch.empty((b, 2), dtype=torch.int32, device="cuda")
                sg.gen_rmat(a.scale, k_new, seed=6, first=first, out=x[:k_new], **RMAT)
                g.sample_edges(b // 20, seed=8, first=first, out=x[k_new:])
                r = torch.empty((b, 2), dtype=torch.int32, device="cuda")
                g.sample_edges(b, seed=7, first=first, out=r)
                first += b
                ins.append(x.cpu().pin_memory() if host else x)
                rem.append(r.cpu().pin_memory() if host else r)
        torch.cuda.synchronize()
        return ins, rem, first

    # every batch applied to g, in order, as host arrays: the oracle replays
    # them after the timed region to check the final graph (parity)
    applied = []

    def record(ins, rem, lo, hi):
        for i in range(lo, hi):
            for op, x in (("insert", ins[i]), ("remove", rem[i])):
                applied.append((op, x.cpu().numpy().view(np.uint32).reshape(-1, 2).copy()))

    ins_d, rem_d, next_first = make_batches(0, host=False)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.int32, device="cuda")
    pr_flush = flush

    per_size = {}  # batch size -> [insert s, remove s, steps] of timed steps

    def run_steps(lo, hi, ins, rem, sizes=None):
        ti = tr = 0.0
        edges = 0
        for i in range(lo, hi):
            with torch.cuda.stream(stream):
                flush.fill_(i)
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record(stream)
            g.insert_batch(ins[i])
            e1.record(stream)
            g.remove_batch(rem[i])
            e2.record(stream)
            e2.synchronize()
            a_, b_ = e0.elapsed_time(e1) / 1e3, e1.elapsed_time(e2) / 1e3
            ti += a_
            tr += b_
            edges += plan[i]
            if sizes is not None:
                ps = sizes.setdefault(plan[i], [0.0, 0.0, 0])
                ps[0] += a_
                ps[1] += b_
                ps[2] += 1
        return ti, tr, edges

    # ---- warmup + timed (device-resident batches).  Batches up to 2^20
    # pairs replay their planning launches from CUDA graphs (captured in the
    # warm-up, one per batch size class and operation), inside which kernels
    # cannot be timed one by one, so the timed region runs without the
    # kernel profiler; per-kernel times come from a pass after it (below).
    run_steps(0, a.warmup, ins_d, rem_d)
    record(ins_d, rem_d, 0, a.warmup + a.steps)
    barrier(world)
    torch.cuda.synchronize()
    l0 = sg.kernel_launches()
    with Clocks(dev) as clk:
        ti, tr, edges = run_steps(a.warmup, a.warmup + a.steps, ins_d, rem_d, per_size)
    torch.cuda.synchronize()
    launches = sg.kernel_launches() - l0
    barrier(world)
    clocks = clk.summary()
    ti = max_over_ranks(ti, world)
    tr = max_over_ranks(tr, world)
    value = world * edges / ti
    ms_per_step = 1e3 * (ti + tr) / a.steps

    # ---- e2e: steps of the same sizes through host (pinned) buffers, with
    # fresh batches (the device pass's edges are already in the graph)
    del ins_d, rem_d
    ins_h, rem_h, next_first = make_batches(next_first, host=True)
    record(ins_h, rem_h, 0, a.warmup + a.steps)
    run_steps(0, a.warmup, ins_h, rem_h)
    eti, etr, eedges = run_steps(a.warmup, a.warmup + a.steps, ins_h, rem_h)
    e2e = {"value": world * eedges / max_over_ranks(eti, world), "unit": "edges/s",
           "h2d_bytes_per_step": int(8 * sum(plan[a.warmup:]) * 2 / a.steps),
           "d2h_bytes_per_step": 16,
           "note": "insert+remove via sst_insert_batch/sst_remove_batch on pinned host "
                   "pairs; each call returns the invalid-pair count (8 B) to the host"}
    del ins_h, rem_h

    # ---- kernel times: one step of each batch size on fresh batches, the
    # kernels a replay runs launched one by one (same size classes and scan
    # forms as the timed region: sst_set_plan_graphs mode 2) and bracketed
    # by events
    ins_p, rem_p, next_first = make_batches(next_first, host=False, sizes=SIZES)
    record(ins_p, rem_p, 0, len(SIZES))
    g.set_plan_graphs(2)
    sg.profile_start()
    run_steps(0, len(SIZES), ins_p, rem_p)
    torch.cuda.synchronize()
    prof_all = sg.profile_collect()
    g.set_plan_graphs(True)
    prof = prof_all
    del ins_p, rem_p

    # ---- parity at full size: the oracle port replays the base graph and
    # every batch above; the device graph's CSR must equal its CSR
    parity = None
    if rank == 0 and not a.no_parity:
        parity = check_parity(g, a.scale, applied)
    del applied

    batched = pagerank = bfs = serving = multi = compact = extras = static = None
    if a.only == "all":
        batched = measure_batched()
        t0 = time.time()
        tuning = sg.autotune(g)
        tuning["tune_s"] = time.time() - t0
        pagerank = measure_pagerank()
        pagerank["tuning"] = tuning
        # the reference's degree-ordered mode (internal/test.hpp:460-467):
        # relabel by degree, run on the relabelled copy, map results back
        t0 = time.time()
        dmap = torch.empty(n, dtype=torch.int32, device="cuda")
        g.degree_order_map(out=dmap)
        gr = g.rewrite_graph(dmap)
        gr.set_stream(stream.cuda_stream)
        torch.cuda.synchronize()
        relabel_s = time.time() - t0
        tuning_deg = sg.autotune(gr)
        pr_deg = measure_pagerank(gr)
        pr_deg["tuning"] = tuning_deg
        o1 = torch.empty(n, dtype=torch.float64, device="cuda")
        o2 = torch.empty(n, dtype=torch.float64, device="cuda")
        sg.PR_S(g, a.pr_iters, out=o1)
        sg.PR_S(gr, a.pr_iters, out=o2)
        torch.cuda.synchronize()
        pr_deg["same_result_after_relabel"] = bool(
            (o2[dmap.long()] - o1).abs().max().item() <= 1e-12 * o1.abs().max().item())
        pr_deg["relabel_s"] = relabel_s
        pagerank["degree_ordered"] = pr_deg
        gr.close()
        bfs = measure_bfs()
        multi = measure_multi()
        compact = measure_compact()
        extras = measure_extras()
        if rank == 0 and not a.no_cpu_baseline:
            static = measure_static()
        serving = measure_serving()


    # ---- roofline of the update step's dominant kernel
    upd_kernels = {"kernel_pass": prof_all,
                   "note": "one step of each batch size on fresh batches after the timed "
                           "region; the kernels the timed region replays (same forms) "
                           "launched one by one and event-timed"}
    roofline = update_roofline(prof, prof_all, hbm_peak, peak_kind)
    # the whole step against the same peak: 28 B per input pair (read 8 B,
    # one sort write + read 16 B, write 4 B) over insert + delete time
    step_pairs = 2 * sum(plan[a.warmup:]) / a.steps
    step_gbs = 28 * step_pairs / (ms_per_step / 1e3) / 1e9
    roofline["whole_step"] = {"pairs_per_step": step_pairs, "bytes_per_pair": 28,
                              "achieved": step_gbs, "frac": step_gbs / hbm_peak}

    # ---- CPU baseline (bounded sample, rank 0 only)
    cpu = None
    if rank == 0 and not a.no_cpu_baseline and a.only == "all":
        sample = SIZES
        v, det = run_cpu(a.scale, sample,
                         f"one insert+delete batch of each size {SIZES} on the "
                         f"scale-{a.scale} base graph (base graph build untimed)")
        cpu = {"value": v, "unit": "edges/s", "cores": cpu_threads(), "kind": "port",
               "sample": det["sample"], "detail": det}

    g.close()
    if rank != 0:
        return
    line = {
        "metric": "batch-insert edges/s", "value": value, "unit": "edges/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32",
        "data": "synthetic RMAT (seeded device generator; no dataset)",
        "config": workload_config(a),
        "roofline": roofline,
        "parity": parity,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clocks,
        "remove_edges_per_s": world * edges / tr,
        "per_batch_size": {str(b): {"insert_us": 1e6 * v[0] / v[2], "remove_us": 1e6 * v[1] / v[2],
                                    "steps": v[2]} for b, v in sorted(per_size.items())},
        "base_graph": {"edges": m0, "build_s": round(build_s, 2)},
        "batched_form": batched,
        "pagerank": pagerank,
        "bfs": bfs,
        "multi_source": multi,
        "compact_snapshot": compact,
        "ingest_and_weighted": extras,
        "static_analytics": static,
        "serving": serving,
        "update_kernels": upd_kernels,
    }
    print(json.dumps(strict(line), allow_nan=False))


# DRAM bytes (read + write) per launch from one ncu capture of one 1e6-pair
# insert (profiles/scan_scatter_locate_1e6_insert_rmat21.md): the host-sized
# single-pass scans read their input once and their writes stay in L2
# (mean over the five of the planning sequence); a one-sweep scatter pass
# over 1e6 keys reads the keys once; the leaf search reads ~5.6 random
# sectors a key.
NCU_TRAFFIC = {"(k_scan_lb<T, Op, Epi>)": 6.75e6, "(k_scatter_os<false, 16>)": 8.30e6,
               "k_locate": 1.92e8}


def update_roofline(prof, prof_all, hbm_peak, peak_kind):
    """Roofline of the update step's dominant kernel from its live event
    timings in the kernel pass after the timed region (one step of each
    batch size, the kernels the timed region runs launched one by one), with
    its share there.

    Algorithmic bytes are declared by each launch site at its launch size
    (what the kernel must read and write, independent of caching):
      radix histogram pass   8 B per key + 4 B per block-digit counter
      radix scatter pass     16 B per key (24 B with values) + counters
      one-CTA sort           16 B per key (24 B with values)
      scan                   2 x element size per element
    achieved = declared bytes / event time, summed over the timed launches.
    """
    # the profiler names a kernel's forms apart (template instances, scans
    # over a device-side count): group them by kernel function, as the ncu
    # launch-list summary in profiles/ does
    def func(nm):
        return nm.strip("()").split("<")[0].split(",")[0].strip()

    groups = {}
    for nm, v in prof.items():
        g = groups.setdefault(func(nm), {"launches": 0, "ms": 0.0, "forms": []})
        g["launches"] += v["launches"]
        g["ms"] += v["ms"]
        g["forms"].append(nm)
    total_ms = sum(v["ms"] for v in prof_all.values())

    def roofline_of(base, grp):
        # achieved: the launches whose algorithmic bytes are declared (a scan
        # over a device-side count declares none: its launch size overstates
        # its work)
        decl = [prof[nm] for nm in grp["forms"] if prof[nm].get("bytes", 0)]
        traffic = [NCU_TRAFFIC[nm] for nm in grp["forms"] if nm in NCU_TRAFFIC]
        r = {"bound": "hbm", "kernel": base, "launches": grp["launches"],
             "ms_total": grp["ms"], "share_of_step_kernel_time": grp["ms"] / total_ms,
             "forms": grp["forms"],
             "peak": hbm_peak, "unit": "GB/s", "peak_kind": peak_kind,
             "traffic": traffic[0] if traffic else None,
             "traffic_basis": "DRAM read + write per launch in one 1e6-pair insert (ncu); "
                              "the kernel pass's launches span all four batch sizes"}
        if decl:
            byts = sum(v["bytes"] for v in decl)
            ms = sum(v["ms"] for v in decl)
            nl = sum(v["launches"] for v in decl)
            ach = byts / (ms / 1e3) / 1e9
            r.update({"achieved": ach, "frac": ach / hbm_peak,
                      "algorithmic_bytes_per_launch": byts / nl,
                      "avg_launch_us": 1e3 * ms / nl,
                      "declared_launches": nl})
        else:
            r.update({"achieved": None, "frac": None})
        return r

    ranked = sorted(groups.items(), key=lambda kv: -kv[1]["ms"])
    out = roofline_of(*ranked[0])
    # the next group too: the two largest are within a few points of each
    # other, and which one leads depends on how launches are timed (here
    # each launch is bracketed by events, so many small launches weigh a
    # little more than in ncu's serialised launch list)
    if len(ranked) > 1:
        nxt = roofline_of(*ranked[1])
        out["runner_up"] = {k: nxt[k] for k in ("kernel", "launches", "ms_total",
                                                 "share_of_step_kernel_time", "achieved",
                                                 "frac", "traffic")
                            if k in nxt}
    return out


if __name__ == "__main__":
    main()
