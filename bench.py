"""Benchmark of the per-round graph operator on one GB300 (replicas for N>1).

Workload (one step): connected components on the symmetrised graph and
weighted SSSP (uint32 weights in [1,255], source 0) on the directed graph,
both seeded RMAT scale 22 (4.19M vertices, edge factor 16, a/b/c/d =
0.57/0.19/0.19/0.05, self-loops and duplicates removed), laid out as 1
compute + 3 memory partitions (edge-balanced contiguous ranges) in HBM with
bitvector-compacted sync.  Every step runs both algorithms to convergence
from init().  The graphs are synthetic (no dataset is involved).

value: Graph500-style GTEPS = (E_cc + E_sssp) / step time, inputs resident in
HBM, CUDA events on the ctx streams.  e2e: the same through the C ABI with
host buffers: every step uploads the partitioned CSR (pinned host memory),
runs, and reads the results back.

`--impl reference` times the reference algorithm on the host cores: the
reference project cannot be built (its Galois/MPI dependencies are absent),
so the arm runs the oracle's restatement of its round protocol with all host
threads ("kind": "port").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "GTEPS (PR/CC/SSSP, RMAT-24) & % HBM roofline; learned+batched vs plain GPU"
SCALE, EF, NUM_MEMORY = 22, 16, 3
RMAT_ABC = (0.57, 0.19, 0.19)
# DRAM bytes (read + write) per edge of k_push_lbs in its ncu capture (CC
# round 0 on RMAT-21, every vertex active): 249.9 MB for the 50.2 M edges of
# non-hub rows.
DRAM_BYTES_PER_PUSH_EDGE = 249.9e6 / 50.2e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-pagerank", action="store_true")
    ap.add_argument("--pr-scale", type=int, default=24)
    ap.add_argument("--batch", action="store_true", help="run the batched workload (default at N=1)")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-graphs", type=int, default=512)
    ap.add_argument("--batch-sources", type=int, default=64)
    ap.add_argument("--policy", choices=["fixed", "learned"], default="fixed",
                    help="round policy of the headline runs (the other one is timed beside it when the model "
                         "file is present)")
    ap.add_argument("--kernel-run-pr", action="store_true",
                    help="only run PageRank (Jacobi pull, RMAT-{pr-scale}) for warmup + steps iterations and print a "
                         "short summary: the target of per-kernel profilers")
    ap.add_argument("--ingest-run", action="store_true",
                    help="only build the partition layouts of the workload's graphs on the GPU "
                         "(grd_ingest, warmup + steps times each), for profiling")
    ap.add_argument("--kernel-run", action="store_true",
                    help="only run the workload's steps with the rounds driven from the host (plain kernel "
                         "launches, no CUDA graphs) and print a short summary: the target of per-kernel profilers")
    return ap.parse_args()


def bench_batch(g, args, local) -> dict:
    """Batched workload: (1) 512 graphs (log-uniform scale 10..18, ef in
    {4,8,16,32}, half RMAT / half ER) each running CC and 20-iteration
    PageRank; (2) 64 SSSP sources on one RMAT-20 graph (w in [1,255]).
    Plain = one ctx per graph (per source), run one after another with the
    fixed schedule; batched = one disjoint union per algorithm, schedule
    picked by the autotuner, one device-driven launch per algorithm."""
    import numpy as np
    from grudon_gb300 import autotune
    from grudon_gb300 import batch as B
    t_gen = time.perf_counter()
    spec = B.batch_spec(args.batch_graphs)
    sym = [B.make_graph(s, symmetrize=True) for s in spec]
    dirg = [B.make_graph(s) for s in spec]
    t_gen = time.perf_counter() - t_gen
    E1 = sum(x.num_edges for x in sym) + 20 * sum(x.num_edges for x in dirg)
    _, _, plain_s = B.run_plain_graphs(sym, dirg, 20, local)
    Uc, Up = B.Union(sym), B.Union(dirg)
    tune_cc = autotune.tune(Uc.graph, g.GRD_CC, lambda c: c.init(), device=local, reps=2)
    best = tune_cc.best
    part = Uc.graph.partition_edge_balanced(best.num_memory) if best.num_memory > 1 else None
    model = load_policy_model()
    pol = g.GRD_POLICY_LEARNED if model is not None else g.GRD_POLICY_FIXED
    ctx_c = g.Context(Uc.graph, part, best.num_memory, local)
    ctx_c.set_algo(g.GRD_CC, policy=pol, **best.params())
    ctx_c.set_policy(model)
    part = Up.graph.partition_edge_balanced(best.num_memory) if best.num_memory > 1 else None
    ctx_p = g.Context(Up.graph, part, best.num_memory, local)
    ctx_p.set_algo(g.GRD_PR_PULL, max_rounds=20, tolerance=0.0)
    for c in (ctx_c, ctx_p):  # warm-up
        c.init()
        c.run()
    reps = 3
    t0 = time.perf_counter()
    for _ in range(reps):
        for c in (ctx_c, ctx_p):
            c.init()
            c.run()
    ctx_c.synchronize()
    batched_s = (time.perf_counter() - t0) / reps
    ctx_c.close()
    ctx_p.close()
    part1 = {"graphs": len(spec), "vertices": int(Uc.sizes.sum()), "edges_cc": Uc.graph.num_edges,
             "edges_pr": Up.graph.num_edges, "generate_s": t_gen,
             "plain_s": plain_s, "batched_s": batched_s, "speedup": plain_s / batched_s,
             "batched_gteps": E1 / batched_s / 1e9, "plain_gteps": E1 / plain_s / 1e9,
             "autotuned": best.__dict__, "tune_table_ms": [round(r["ms"], 3) for r in tune_cc.table]}

    # (2) multi-source SSSP
    G = g.Graph.rmat(20, 16, weighted=True)
    rng = np.random.default_rng(0x53535350)
    sources = rng.integers(0, G.num_vertices, args.batch_sources)
    c1 = g.Context(G, None, 1, local)
    c1.set_algo(g.GRD_SSSP_W)
    c1.init()
    c1.run()
    t0 = time.perf_counter()
    for s in sources:
        c1.set_algo(g.GRD_SSSP_W, source=int(s))
        c1.init()
        c1.run()
    c1.synchronize()
    plain2 = time.perf_counter() - t0
    c1.close()
    U = B.Union([G] * len(sources))
    c2 = g.Context(U.graph, None, 1, local)
    c2.set_algo(g.GRD_SSSP_W, policy=pol)
    c2.set_policy(model)
    srcs = U.bases + sources
    c2.init_sources(srcs)
    c2.run()
    t0 = time.perf_counter()
    for _ in range(reps):
        c2.init_sources(srcs)
        st = c2.run()
    c2.synchronize()
    batched2 = (time.perf_counter() - t0) / reps
    c2.close()
    E2 = len(sources) * G.num_edges
    part2 = {"sources": len(sources), "graph": "RMAT-20 ef16 w in [1,255]", "plain_s": plain2,
             "batched_s": batched2, "speedup": plain2 / batched2, "rounds": st["rounds"],
             "batched_gteps": E2 / batched2 / 1e9, "plain_gteps": E2 / plain2 / 1e9}
    total_plain, total_batched = plain_s + plain2, batched_s + batched2
    return {"part1_graphs": part1, "part2_sssp_sources": part2,
            "end_to_end_speedup": total_plain / total_batched,
            "policy": "learned" if model is not None else "fixed",
            "note": "plain: one ctx per graph (per source) with the fixed per-round rule; batched: one union per "
                    "algorithm, autotuned schedule and the learned round policy (CC, SSSP; PageRank is Jacobi "
                    "pull); timings exclude layout build"}


def bench_pagerank(g, args, local, hbm_peak, barrier, ws) -> dict:
    """PageRank, RMAT-24 (ef16), 1C+3M: Jacobi with FP32 Kahan sums and an FP64
    residual, until L1 residual / V < 1e-7 or 100 iterations."""
    threads = max(1, (os.cpu_count() or 1) // ws)
    a, b, c = RMAT_ABC
    G = g.Graph.rmat(args.pr_scale, EF, a, b, c, seed=g.rmat_seed(args.pr_scale, EF), threads=threads)
    part = G.partition_edge_balanced(NUM_MEMORY)
    ctx = g.Context(G, part, num_memory=NUM_MEMORY, device=local)
    ctx.set_algo(g.GRD_PR_PULL, max_rounds=100, tolerance=1e-7)
    ctx.init()
    ctx.run()  # warm-up
    ctx.set_profiling(True)
    reps = 2
    stats = []
    barrier()
    t0 = time.perf_counter()
    for _ in range(reps):
        ctx.init()
        stats.append(ctx.run())
    barrier()
    dt = (time.perf_counter() - t0) / reps
    st = stats[-1]
    it = st["rounds"]
    pull_ms = sum(s["stage_ms"][1] for s in stats) / reps
    rounds_ms = sum(s["stage_ms"][4] for s in stats) / reps
    S = sum(ctx.layout_info(p)[0] + ctx.layout_info(p)[1] for p in range(NUM_MEMORY))
    # pull edge-map bytes per iteration: in_off + partial writes + dirty bits
    # over the slots, index + contribution gather per in-edge
    alg = it * (S * 8 + S / 8 + G.num_edges * 8)
    ach = alg / (pull_ms / 1e3) / 1e9 if pull_ms else 0.0
    ranks = ctx.read_ranks()
    ctx.close()
    return {
        "workload": f"PageRank Jacobi (FP32 Kahan, FP64 residual), RMAT-{args.pr_scale} ef{EF}, 1C+{NUM_MEMORY}M, "
                    "stop at L1 residual/V < 1e-7 or 100 iterations",
        "num_vertices": G.num_vertices, "num_edges": G.num_edges, "iterations": it,
        "converged": st["converged"], "last_residual_per_vertex": st["last_residual"],
        "seconds_per_run": dt, "gteps": G.num_edges * it / dt / 1e9,
        "ms_per_iteration": rounds_ms / max(it, 1),
        "roofline": {"bound": "hbm", "kernel": "pull edge-map (k_pull_pr + k_pull_hub)", "achieved": ach,
                     "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak, "traffic": None},
        "_graph": G, "_ranks": ranks,
    }


def bench_ingest(g, args, G_cc, G_ss, p_cc, p_ss, local, barrier, dev) -> dict:
    """Partition layout of both graphs built on the host (layout.cpp, all
    host threads) and on the GPU (grd_ingest: the CSR uploaded from host
    memory, then proxies, translation slots and the relabelled CSR built by
    kernels); then the headline steps end to end from the host CSR: ingest,
    run both algorithms, read the results."""
    from grudon_gb300.replicas import job_throughput
    t0 = time.perf_counter()
    for G, p in ((G_cc, p_cc), (G_ss, p_ss)):
        g.layout_preview(G, p, NUM_MEMORY, 0)
    host_ms = (time.perf_counter() - t0) * 1e3
    dctx = [g.Context(G, p, num_memory=NUM_MEMORY, device=local, device_layout=True)
            for G, p in ((G_cc, p_cc), (G_ss, p_ss))]
    try:
        best = None
        for _ in range(3):
            barrier()
            t0 = time.perf_counter()
            nbytes = sum(c.ingest(G, p) for c, G, p in zip(dctx, (G_cc, G_ss), (p_cc, p_ss)))
            barrier()
            dt = (time.perf_counter() - t0) * 1e3
            best = dt if best is None else min(best, dt)
        for c, a in zip(dctx, (g.GRD_CC, g.GRD_SSSP_W)):
            c.set_algo(a)
        E = G_cc.num_edges + G_ss.num_edges
        for c in dctx:  # warm the loop graphs
            c.init()
            c.run()
        barrier()
        t0 = time.perf_counter()
        (cc, ss), graphs = dctx, ((G_cc, p_cc), (G_ss, p_ss))
        # every step ingests both CSRs and reads both results back; each
        # ingest overlaps the other graph's queued run
        cc.ingest(*graphs[0])
        for k in range(args.steps):
            cc.init()
            cc.run(wait=False)
            ss.ingest(*graphs[1])
            cc.wait()
            cc.read_props()
            ss.init()
            ss.run(wait=False)
            if k + 1 < args.steps:
                cc.ingest(*graphs[0])
            ss.wait()
            ss.read_props()
        barrier()
        thr, _, _ = job_throughput(args.steps * E, time.perf_counter() - t0, dev)
    finally:
        for c in dctx:
            c.close()
    return {"host_layout_ms": host_ms, "device_layout_ms": best, "speedup": host_ms / best,
            "device_h2d_bytes": nbytes, "host_threads": os.cpu_count(),
            "e2e_from_host_csr": {"value": thr / 1e9, "unit": "GTEPS",
                                  "note": "per step: CSR upload + device layout build + both runs + results read, "
                                          "each graph's ingest overlapping the other's run"}}


def pr_fp64_check(pr: dict, cpu: dict) -> None:
    """FP64 Jacobi on the host for the same iteration count (CPU-baseline
    leg): reports its time and the GPU's max relative error against it."""
    import numpy as np
    from oracle import ffi as O
    G = pr["_graph"]
    t0 = time.perf_counter()
    ref, it, _ = O.pr_jacobi_fp64_mt(G.row_offsets, G.col_indices, iters=pr["iterations"])
    secs = time.perf_counter() - t0
    got = pr["_ranks"].astype(np.float64)
    both0 = (got == 0) & (ref == 0)
    rel = np.where(both0, 0.0, np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300))
    pr["max_rel_err_vs_fp64"] = float(rel.max())
    cpu["pagerank_fp64"] = {"seconds": secs, "iterations": it, "threads": os.cpu_count(),
                            "gteps": G.num_edges * it / secs / 1e9,
                            "kind": "FP64 Jacobi restatement (oracle), all host threads"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 20 ms (the timed region
    of a default run lasts well under a second)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_policy_model():
    """The shipped learned round-policy model, or None."""
    from grudon_gb300 import policy as P
    return P.load_model() if P.MODEL_FILE.exists() else None


def make_graphs(scale: int, threads: int):
    import grudon_gb300 as g
    a, b, c = RMAT_ABC
    seed = g.rmat_seed(scale, EF)
    G_cc = g.Graph.rmat(scale, EF, a, b, c, seed=seed, symmetrize=True, threads=threads)
    G_ss = g.Graph.rmat(scale, EF, a, b, c, seed=seed, weighted=True, threads=threads)
    return seed, G_cc, G_ss


def cpu_baseline(G_cc, G_ss, p_cc, p_ss, steps: int = 1) -> dict:
    """The oracle's restated round protocol, all host threads, run() only."""
    from oracle import ffi as O
    threads = os.cpu_count() or 1
    L_cc = O.Layout(G_cc.row_offsets, G_cc.col_indices, mirror=p_cc, num_memory=NUM_MEMORY)
    L_ss = O.Layout(G_ss.row_offsets, G_ss.col_indices, G_ss.weights, mirror=p_ss, num_memory=NUM_MEMORY)
    t_total = 0.0
    for _ in range(steps):
        t0 = time.perf_counter()
        L_cc.run(O.ORC_CC, threads=threads)
        L_ss.run(O.ORC_SSSP_W, threads=threads)
        t_total += time.perf_counter() - t0
    E = G_cc.num_edges + G_ss.num_edges
    return {"value": steps * E / t_total / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
            "seconds": t_total,
            "sample": f"{steps} full step(s): CC + weighted SSSP to convergence on the same RMAT-{SCALE} graphs, "
                      f"1C+{NUM_MEMORY}M, oracle restatement of the reference round protocol (reference "
                      f"unbuildable: Galois/MPI absent), {threads} host threads"}


def bench_reference_cpu_case(g, local) -> dict:
    """The reference's own CPU-runnable case: plain (delta-push) PageRank,
    damping 0.85, 20 iterations, seeded RMAT-16 ef16, 1 compute + 1 memory
    partition.  The whole run on the GPU (one device-loop launch, init
    excluded) beside the oracle restatement on all host threads (run()
    only), medians."""
    import numpy as np
    import torch
    from oracle import ffi as O
    G = g.Graph.rmat(16, EF, seed=g.rmat_seed(16, EF))
    with g.Context(G, None, num_memory=1, device=local) as ctx:
        ctx.set_algo(g.GRD_PR_DELTA, max_rounds=20)
        ts = []
        for k in range(13):
            ctx.init()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st = ctx.run()
            if k >= 3:
                ts.append(time.perf_counter() - t0)
        ranks = ctx.read_ranks()
    L = O.Layout(G.row_offsets, G.col_indices, num_memory=1)
    threads = os.cpu_count() or 1
    cs = []
    for _ in range(3):
        t0 = time.perf_counter()
        ref = L.run(O.ORC_PR_DELTA, max_rounds=20, threads=threads)
        cs.append(time.perf_counter() - t0)
    gpu_ms, cpu_ms = 1e3 * statistics.median(ts), 1e3 * statistics.median(cs)
    return {"workload": "PageRank delta push, damping 0.85, 20 iterations, RMAT-16 ef16, 1C+1M",
            "num_edges": G.num_edges, "rounds": st["rounds"], "gpu_ms": gpu_ms, "cpu_ms": cpu_ms,
            "cpu_threads": threads, "speedup": cpu_ms / gpu_ms,
            "max_abs_rank_diff": float(np.abs(ranks - ref["ranks"]).max())}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    seed, G_cc, G_ss = make_graphs(args.scale, 0)
    p_cc = G_cc.partition_edge_balanced(NUM_MEMORY)
    p_ss = G_ss.partition_edge_balanced(NUM_MEMORY)
    from oracle import ffi as O
    threads = os.cpu_count() or 1
    L_cc = O.Layout(G_cc.row_offsets, G_cc.col_indices, mirror=p_cc, num_memory=NUM_MEMORY)
    L_ss = O.Layout(G_ss.row_offsets, G_ss.col_indices, G_ss.weights, mirror=p_ss, num_memory=NUM_MEMORY)
    for _ in range(args.warmup):
        L_cc.run(O.ORC_CC, threads=threads)
        L_ss.run(O.ORC_SSSP_W, threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        L_cc.run(O.ORC_CC, threads=threads)
        L_ss.run(O.ORC_SSSP_W, threads=threads)
    dt = time.perf_counter() - t0
    E = G_cc.num_edges + G_ss.num_edges
    value = args.steps * E / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": workload_config(args.scale, seed, G_cc, G_ss),
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"each step: CC + weighted SSSP to convergence (full workload), "
                                   f"{threads} host threads; reference itself unbuildable (Galois/MPI absent)"},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(scale, seed, G_cc, G_ss) -> dict:
    return {
        "workload": f"CC (symmetrised) + weighted SSSP (w in [1,255], source 0) to convergence, RMAT-{scale} "
                    f"ef{EF} a/b/c/d .57/.19/.19/.05, 1 compute + {NUM_MEMORY} memory partitions, bitvector or list "
                    f"sync and push or pull chosen per round",
        "scale": scale, "edge_factor": EF, "seed": seed, "num_vertices": G_cc.num_vertices,
        "E_cc_symmetrised": G_cc.num_edges, "E_sssp": G_ss.num_edges,
        "partitions": f"1C+{NUM_MEMORY}M edge-balanced contiguous",
        "l2": "inputs larger than L2 (CSR indices 0.27-0.5 GB > 129 MB), no flush",
        "streams": "CC then SSSP within a step, each on its own ctx stream",
    }


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    ws, rank, local = dist_env()
    import numpy as np
    import torch
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import grudon_gb300 as g

    threads = max(1, (os.cpu_count() or 1) // ws)
    if args.kernel_run_pr:
        a, b, c = RMAT_ABC
        G = g.Graph.rmat(args.pr_scale, EF, a, b, c, seed=g.rmat_seed(args.pr_scale, EF), threads=threads)
        with g.Context(G, G.partition_edge_balanced(NUM_MEMORY), num_memory=NUM_MEMORY, device=local) as ctx:
            ctx.set_algo(g.GRD_PR_PULL, max_rounds=args.warmup + args.steps, tolerance=0.0)
            ctx.init()
            st = ctx.run()
        if rank == 0:
            print(json.dumps({"kernel_run_pr": True, "scale": args.pr_scale, "iterations": st["rounds"],
                              "edges": G.num_edges}), flush=True)
        return
    seed, G_cc, G_ss = make_graphs(args.scale, threads)
    p_cc = G_cc.partition_edge_balanced(NUM_MEMORY)
    p_ss = G_ss.partition_edge_balanced(NUM_MEMORY)
    if args.ingest_run:
        for G, p in ((G_cc, p_cc), (G_ss, p_ss)):
            with g.Context(G, p, num_memory=NUM_MEMORY, device=local, device_layout=True) as c:
                for _ in range(args.warmup + args.steps):
                    c.ingest(G, p)
        if rank == 0:
            print(json.dumps({"ingest_run": True, "scale": args.scale,
                              "builds_per_graph": 1 + args.warmup + args.steps}), flush=True)
        return
    ctx_cc = g.Context(G_cc, p_cc, num_memory=NUM_MEMORY, device=local)
    ctx_ss = g.Context(G_ss, p_ss, num_memory=NUM_MEMORY, device=local)
    model = load_policy_model()

    def set_policy(policy, offload=g.GRD_OFFLOAD_NDP):
        for c, a in ((ctx_cc, g.GRD_CC), (ctx_ss, g.GRD_SSSP_W)):
            c.set_algo(a, policy=policy, offload=offload)
            c.set_policy(model if policy == g.GRD_POLICY_LEARNED else None)

    # The headline runs the library's default schedule, the fixed threshold
    # rule (push only: no in-edge view), unless --policy learned.  The shipped
    # learned policy, when its model file is present, is timed next to it.
    policy = g.GRD_POLICY_LEARNED if (args.policy == "learned" and model is not None) else g.GRD_POLICY_FIXED
    set_policy(g.GRD_POLICY_FIXED)
    E = G_cc.num_edges + G_ss.num_edges
    slots = {id(c): sum(sum(c.layout_info(p)[:2]) for p in range(NUM_MEMORY)) for c in (ctx_cc, ctx_ss)}

    def step(host_loop=False):
        """Both algorithms to convergence, one after the other (run
        concurrently on their two streams they were slower: their full-wave
        push kernels compete for the SMs and L2)."""
        out = []
        for c in (ctx_cc, ctx_ss):
            c.init()
            out.append(c.run(host_loop=host_loop))
        return out

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    if args.kernel_run:
        set_policy(policy)
        for _ in range(args.warmup + args.steps):
            sts = step(host_loop=True)
        barrier()
        if rank == 0:
            print(json.dumps({"kernel_run": True, "workload": workload_config(args.scale, seed, G_cc, G_ss)["workload"],
                              "policy": "learned" if policy == g.GRD_POLICY_LEARNED else "fixed",
                              "rounds": [st["rounds"] for st in sts],
                              "launches_per_step": sum(st["kernel_launches"] for st in sts)}), flush=True)
        ctx_cc.close()
        ctx_ss.close()
        return

    s_cc = torch.cuda.ExternalStream(ctx_cc.stream())
    s_ss = torch.cuda.ExternalStream(ctx_ss.stream())
    from grudon_gb300.replicas import job_throughput
    dev = torch.device("cuda", local) if ws > 1 else None

    def timed():
        """W warm-up steps, then K timed steps: every step runs both
        algorithms to convergence, each as one device-driven CUDA-graph
        launch; CUDA events on the ctx streams."""
        for _ in range(args.warmup):
            step()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        ev0.record(s_cc)
        agg = {"edges": 0, "launches": 0, "rounds": [], "device_loop": [], "push_rounds": 0, "pull_rounds": 0}
        for _ in range(args.steps):
            for st in step():
                agg["edges"] += st["edges_scanned"]
                agg["launches"] += st["kernel_launches"]
                agg["rounds"].append(st["rounds"])
                agg["device_loop"].append(st["device_loop"])
                agg["push_rounds"] += st["push_rounds"]
                agg["pull_rounds"] += st["pull_rounds"]
        ev1.record(s_ss)
        barrier()
        thr, secs, _ = job_throughput(args.steps * E, ev0.elapsed_time(ev1) / 1e3, dev)
        return thr / 1e9, secs * 1e3, agg

    def summary(v, ms, a):
        return {"value": v, "ms_per_step": ms / args.steps, "rounds_per_step": a["rounds"][:2],
                "push_rounds_per_step": a["push_rounds"] / args.steps,
                "pull_rounds_per_step": a["pull_rounds"] / args.steps, "gpu_launches": a["launches"]}

    clocks = ClockSampler(local)
    clocks.start()
    runs = {}
    if policy == g.GRD_POLICY_LEARNED:  # the plain method first (before the in-edge view exists)
        runs["fixed"] = summary(*timed())
        set_policy(policy)
    value, dt_ms, agg = timed()
    clk = clocks.stop()
    runs["learned" if policy == g.GRD_POLICY_LEARNED else "fixed"] = summary(value, dt_ms, agg)

    # Stage timing for the roofline: the same steps driven from the host with
    # CUDA events around every stage of every round (same kernels, same
    # per-round choices).
    for c in (ctx_cc, ctx_ss):
        c.set_profiling(True)
    prof = {"edge_map_ms": 0.0, "fwd_ms": 0.0, "bwd_ms": 0.0, "update_ms": 0.0, "rounds_ms": 0.0, "alg_bytes": 0.0,
            "push_rounds": 0, "pull_rounds": 0, "lbs_ms": 0.0, "lbs_bytes": 0.0, "lbs_launches": 0,
            "lbs_edges": 0}
    for _ in range(args.steps):
        for st, c, weighted, Eg in zip(step(host_loop=True), (ctx_cc, ctx_ss), (False, True),
                                        (G_cc.num_edges, G_ss.num_edges)):
            for i, k in enumerate(("fwd_ms", "edge_map_ms", "bwd_ms", "update_ms", "rounds_ms")):
                prof[k] += st["stage_ms"][i]
            wb = 4 if weighted else 0
            push_edges = st["edges_scanned"] - st["pull_rounds"] * Eg
            S = slots[id(c)]
            prof["alg_bytes"] += (st["push_actives"] * 12 + push_edges * (12 + wb) +
                                  st["pull_rounds"] * (Eg * (8 + wb) + S * 8 + S / 8))
            prof["push_rounds"] += st["push_rounds"]
            prof["pull_rounds"] += st["pull_rounds"]
            # the load-balanced push kernel alone, by the push round's
            # algorithmic bytes: DP/RB/SV of each active (12), then per edge
            # its column index (4), weight (4, weighted) and the destination's
            # read-modify-write (8)
            prof["lbs_ms"] += st["lbs_ms"]
            prof["lbs_launches"] += st["lbs_launches"]
            prof["lbs_edges"] += st["lbs_edges"]
            prof["lbs_bytes"] += st["lbs_actives"] * 12 + st["lbs_edges"] * (12 + wb)
    for c in (ctx_cc, ctx_ss):
        c.set_profiling(False)

    # Host->device bandwidth of the layout upload alone (both graphs, best of 3).
    up_s = []
    for _ in range(3):
        barrier()
        t0 = time.perf_counter()
        up_bytes = sum(c.upload() for c in (ctx_cc, ctx_ss))
        barrier()
        up_s.append(time.perf_counter() - t0)
    upload_gbs = up_bytes / min(up_s) / 1e9

    # End to end through the C ABI with host buffers.  Results are read into
    # pinned host arrays allocated once, as a serving loop keeps them.
    res_cc = torch.empty(G_cc.num_vertices, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    res_ss = torch.empty(G_ss.num_vertices, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    barrier()
    h2d = 0
    t0 = time.perf_counter()
    # Every step copies both graphs' layouts and reads both results back.  The
    # copies are pipelined with the runs: CC's copy has the link to itself,
    # SSSP's follows it and overlaps CC's run, and once CC's result is read
    # the next step's CC copy overlaps SSSP's run.
    # Runs and reads are queued (run(wait=False), read_props(wait=False)) and
    # ordered by stream events: CC's run waits for SSSP's previous run, SSSP's
    # for CC's, so the two never share the GPU, and the host waits only on
    # work already finished, queuing each run before the GPU reaches it.
    up_done, cc_done, ss_done = torch.cuda.Event(), torch.cuda.Event(), torch.cuda.Event()
    h2d += ctx_cc.upload()
    for k in range(args.steps):
        up_done.record(s_cc)
        s_ss.wait_event(up_done)
        h2d += ctx_ss.upload()
        ctx_cc.wait()  # CC's previous run; its stream then holds only this step's copy
        if k:
            s_cc.wait_event(ss_done)
        ctx_cc.init()
        ctx_cc.run(wait=False)
        ctx_cc.read_props(out=res_cc, wait=False)
        cc_done.record(s_cc)
        if k + 1 < args.steps:
            h2d += ctx_cc.upload()
        ctx_ss.wait()
        s_ss.wait_event(cc_done)
        ctx_ss.init()
        ctx_ss.run(wait=False)
        ctx_ss.read_props(out=res_ss, wait=False)
        ss_done.record(s_ss)
    ctx_cc.wait()
    ctx_ss.wait()
    barrier()
    e2e_thr, _, _ = job_throughput(args.steps * E, time.perf_counter() - t0, dev)
    # the queued reads delivered the final results (checked outside the timed region)
    if not (np.array_equal(res_cc, ctx_cc.read_props()) and np.array_equal(res_ss, ctx_ss.read_props())):
        raise RuntimeError("queued result reads differ from a blocking read")
    e2e = {"value": e2e_thr / 1e9, "unit": "GTEPS",
           "h2d_bytes_per_step": h2d // args.steps,
           "d2h_bytes_per_step": 4 * (G_cc.num_vertices + G_ss.num_vertices),
           "upload_alone_gbs": upload_gbs}
    ingest = bench_ingest(g, args, G_cc, G_ss, p_cc, p_ss, local, barrier, dev)

    # The other schedule on the same contexts; the learned one must leave
    # every result bit-identical.
    results_identical = None
    if model is not None:
        if "learned" not in runs:
            set_policy(g.GRD_POLICY_LEARNED)
            runs["learned"] = summary(*timed())
        outs = []
        for pol in (g.GRD_POLICY_FIXED, g.GRD_POLICY_LEARNED):
            set_policy(pol)
            outs.append([(c.init(), c.run(), c.read_props())[2] for c in (ctx_cc, ctx_ss)])
        results_identical = all(bool((a == b).all()) for a, b in zip(*outs))

    # The reference's offload engine (NDPEngine: NO_OFFLOAD rounds, the
    # compute partition pushing over the shipped adjacency, when the frontier
    # holds at most V/20 vertices) against the all-NDP_OFFLOAD schedule it
    # hard-codes, both with the fixed rule, timed back to back on the same
    # contexts; results must be bit-identical.
    set_policy(g.GRD_POLICY_FIXED)
    ndp_run = summary(*timed())
    base_props = [(c.init(), c.run(), c.read_props())[2] for c in (ctx_cc, ctx_ss)]
    set_policy(g.GRD_POLICY_FIXED, g.GRD_OFFLOAD_ENGINE)
    eng_run = summary(*timed())
    sts = [(c.init(), c.run())[1] for c in (ctx_cc, ctx_ss)]
    off_props = [c.read_props() for c in (ctx_cc, ctx_ss)]
    offload = {"ndp": ndp_run,
               "engine": eng_run | {"no_offload_rounds_per_step": [st["no_offload_rounds"] for st in sts]},
               "engine_speedup_vs_ndp": eng_run["value"] / ndp_run["value"],
               "results_bit_identical": all(bool((a == b).all()) for a, b in zip(base_props, off_props))}
    set_policy(policy)

    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    stage_ach = prof["alg_bytes"] / (prof["edge_map_ms"] / 1e3) / 1e9 if prof["edge_map_ms"] > 0 else 0.0
    nl = max(prof["lbs_launches"], 1)
    lbs_ach = prof["lbs_bytes"] / (prof["lbs_ms"] / 1e3) / 1e9 if prof["lbs_ms"] > 0 else 0.0
    roofline = {"bound": "hbm", "kernel": "k_push_lbs (load-balanced push edge-map)",
                "achieved": lbs_ach, "peak": hbm_peak, "unit": "GB/s", "frac": lbs_ach / hbm_peak,
                "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                # DRAM bytes per edge of the kernel in its ncu capture, times
                # this run's average edges per launch
                "traffic": DRAM_BYTES_PER_PUSH_EDGE * prof["lbs_edges"] / nl,
                "alg_bytes_per_launch": prof["lbs_bytes"] / nl, "avg_launch_ms": prof["lbs_ms"] / nl,
                "launches": prof["lbs_launches"],
                "edge_map_stage": {"achieved": stage_ach, "frac": stage_ach / hbm_peak,
                                   "kernels": "k_deg_* (list rounds), k_push_lbs, k_hub_push, k_diff_dirty (push) or k_pull* (pull)",
                                   "share_of_rounds": prof["edge_map_ms"] / prof["rounds_ms"]
                                   if prof["rounds_ms"] else None},
                "push_rounds_per_step": prof["push_rounds"] / args.steps,
                "pull_rounds_per_step": prof["pull_rounds"] / args.steps,
                "stage_ms_per_step": {k: prof[k] / args.steps for k in
                                      ("fwd_ms", "edge_map_ms", "bwd_ms", "update_ms", "rounds_ms")}}
    pr = None
    if not args.no_pagerank:
        pr = bench_pagerank(g, args, local, hbm_peak, barrier, ws)
    batch = bench_batch(g, args, local) if (args.batch or (ws == 1 and not args.no_batch)) else None
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": workload_config(args.scale, seed, G_cc, G_ss) | {"parallelism": f"replicas x{ws}"},
            "e2e": e2e, "gpu_launches": agg["launches"], "roofline": roofline, "clocks": clk,
            "rounds_per_step": agg["rounds"][:2], "device_loop": all(agg["device_loop"]),
            "edges_scanned_gteps": ws * agg["edges"] / (dt_ms / 1e3) / 1e9,
            "policy": {"headline": "learned" if policy == g.GRD_POLICY_LEARNED else "fixed",
                       "model": "grudon_gb300/policy_model.json" if model is not None else None,
                       **runs,
                       "learned_speedup_vs_fixed": (runs["learned"]["value"] / runs["fixed"]["value"])
                       if "learned" in runs else None,
                       "results_bit_identical": results_identical},
            "offload": offload,
        }
        if ws == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(G_cc, G_ss, p_cc, p_ss)
            line["reference_cpu_case"] = bench_reference_cpu_case(g, local)
            if pr is not None:
                pr_fp64_check(pr, line["cpu_baseline"])
        if pr is not None:
            pr.pop("_graph", None)
            pr.pop("_ranks", None)
            line["pagerank_rmat24"] = pr
        if batch is not None:
            line["batch"] = batch
        line["ingest"] = ingest
        print(json.dumps(line), flush=True)
    ctx_cc.close()
    ctx_ss.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
