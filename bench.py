"""Benchmark of the per-round graph operator on one GB300 (replicas for N>1).

Workload (one step, the PR/CC/SSSP RMAT-24 metric): on seeded RMAT scale 24
(16.8M vertices, edge factor 16, a/b/c/d = 0.57/0.19/0.19/0.05, self-loops
and duplicates removed), laid out as 1 compute + 3 memory partitions
(edge-balanced contiguous ranges) in HBM with bitvector-compacted sync:
  * connected components on the symmetrised graph, to convergence;
  * weighted SSSP (uint32 weights in [1,255], source 0) on the directed
    graph, to convergence;
  * PageRank (Jacobi, damping 0.85, FP32 ranks with Kahan-compensated sums,
    FP64 residual) on the directed graph until the L1 residual / V < 1e-7 or
    100 iterations.
The graphs are synthetic (no dataset is involved).

value: Graph500-style GTEPS = (E_cc + E_sssp + iterations * E_pr) / step time,
inputs resident in HBM, CUDA events on the ctx streams.  e2e: the same
through the C ABI with host buffers: every step uploads the three partitioned
layouts from pinned host memory, runs, and reads the results back.

`--impl reference` times the reference algorithm on the host cores.  The
reference project cannot be built (its Galois/MPI dependencies are absent),
so the arm runs the oracle's restatement of its round protocol (CC, SSSP) and
of the PageRank workload's Jacobi iteration with all host threads ("kind":
"port"), on graphs made by the oracle's own generator: it loads no library of
the product.
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
SCALE, EF, NUM_MEMORY = 24, 16, 3
RMAT_ABC = (0.57, 0.19, 0.19)
PR_MAX_ITERS, PR_TOL = 100, 1e-7
# DRAM bytes (read + write) per in-edge of k_pr_pull in its ncu capture
# (PageRank RMAT-22, 65.2 M in-edges): 292.0 MB per launch.
DRAM_BYTES_PER_PULL_EDGE = 292.0e6 / 65.24e6
# ... and of k_push_lbs (CC round 0 on RMAT-21): 251.0 MB for 50.2 M edges.
DRAM_BYTES_PER_PUSH_EDGE = 251.0e6 / 50.2e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline, e2e and parity only (no batch, policy, offload, ingest or RMAT-22 legs)")
    ap.add_argument("--batch", action="store_true", help="run the batched workload (default at N=1)")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--batch-graphs", type=int, default=512)
    ap.add_argument("--batch-sources", type=int, default=64)
    ap.add_argument("--policy", choices=["fixed", "learned"], default="fixed",
                    help="round policy of the CC/SSSP runs of the headline (the other one is timed beside it when "
                         "the model file is present)")
    ap.add_argument("--kernel-run", action="store_true",
                    help="only run the workload's steps with the rounds driven from the host (plain kernel "
                         "launches, no CUDA graphs) and print a short summary: the target of per-kernel profilers")
    ap.add_argument("--kernel-run-pr", action="store_true",
                    help="only run PageRank (RMAT-{scale}) for warmup + steps iterations from the host: the "
                         "target of per-kernel profilers")
    ap.add_argument("--ingest-run", action="store_true",
                    help="only build the three contexts' partition layouts on the GPU (RMAT-{scale}) and "
                         "re-ingest each warmup + steps times: the target of per-kernel profilers")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def csr_checksum(ro, col, w=None) -> str:
    """Order-sensitive 64-bit digest of a CSR (hex): both arms state which
    graphs they ran in their config."""
    import numpy as np
    m = np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        acc = np.uint64(len(ro) - 1) * m
        for arr in (ro, col, w):
            if arr is None:
                continue
            a = np.ascontiguousarray(arr).astype(np.uint64, copy=False)
            idx = np.arange(1, len(a) + 1, dtype=np.uint64)
            acc = acc * np.uint64(31) + np.sum((a + np.uint64(1)) * (idx * m | np.uint64(1)), dtype=np.uint64)
    return f"{int(acc):016x}"


def workload_config(scale, seed, V, E_cc, E_dir, ck_cc, ck_dir, ws) -> dict:
    return {
        "workload": f"one step = CC (symmetrised) + weighted SSSP (w in [1,255], source 0) + PageRank (Jacobi, "
                    f"FP32 Kahan sums, FP64 residual, until L1 residual/V < {PR_TOL:g} or {PR_MAX_ITERS} "
                    f"iterations), RMAT-{scale} ef{EF} a/b/c/d .57/.19/.19/.05, 1 compute + {NUM_MEMORY} memory "
                    f"partitions with bitvector-compacted sync",
        "scale": scale, "edge_factor": EF, "seed": seed, "num_vertices": V,
        "E_cc_symmetrised": E_cc, "E_directed": E_dir,
        "csr_checksum": {"symmetrised": ck_cc, "directed_weighted": ck_dir},
        "partitions": f"1C+{NUM_MEMORY}M edge-balanced contiguous",
        "units": "GTEPS = (E_cc + E_sssp + pagerank_iterations * E_pr) / step time",
        "l2": "inputs larger than L2 (CSR indices 1-2 GB > 129 MB), no flush",
        "parallelism": f"replicas x{ws}",
    }


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 20 ms during the timed
    region."""

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


def hbm_peak() -> tuple[float, str]:
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
        if "hbm_gbs" in peaks:
            return float(peaks["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# --------------------------------------------------------------- GPU arm --
def load_policy_model():
    """The shipped learned round-policy model, or None."""
    from grudon_gb300 import policy as P
    return P.load_model() if P.MODEL_FILE.exists() else None


class Workload:
    """The three contexts of one step: CC on the symmetrised graph, weighted
    SSSP and PageRank on the directed graph (each its own partitioned layout
    in HBM, each on its own stream)."""

    def __init__(self, g, scale, threads, local):
        a, b, c = RMAT_ABC
        self.g = g
        self.seed = g.rmat_seed(scale, EF)
        self.G_cc = g.Graph.rmat(scale, EF, a, b, c, seed=self.seed, symmetrize=True, threads=threads)
        self.G_d = g.Graph.rmat(scale, EF, a, b, c, seed=self.seed, weighted=True, threads=threads)
        self.p_cc = self.G_cc.partition_edge_balanced(NUM_MEMORY)
        self.p_d = self.G_d.partition_edge_balanced(NUM_MEMORY)
        # PageRank reads no weights: its context holds the directed CSR alone
        self.G_pr = g.Graph.from_csr(self.G_d.row_offsets, self.G_d.col_indices)
        self.cc = g.Context(self.G_cc, self.p_cc, num_memory=NUM_MEMORY, device=local)
        self.ss = g.Context(self.G_d, self.p_d, num_memory=NUM_MEMORY, device=local)
        self.pr = g.Context(self.G_pr, self.p_d, num_memory=NUM_MEMORY, device=local)
        self.pr.set_algo(g.GRD_PR_PULL, max_rounds=PR_MAX_ITERS, tolerance=PR_TOL)
        self.ctxs = (self.cc, self.ss, self.pr)
        self.E_cc, self.E_d = self.G_cc.num_edges, self.G_d.num_edges
        self.V = self.G_cc.num_vertices

    def set_policy(self, policy, model=None, offload=None):
        g = self.g
        off = g.GRD_OFFLOAD_NDP if offload is None else offload
        for c, a in ((self.cc, g.GRD_CC), (self.ss, g.GRD_SSSP_W)):
            c.set_algo(a, policy=policy, offload=off)
            c.set_policy(model if policy == g.GRD_POLICY_LEARNED else None)

    def units(self, sts) -> float:
        return self.E_cc + self.E_d + sts[2]["rounds"] * self.E_d

    def close(self):
        for c in self.ctxs:
            c.close()


def timed_steps(W, args, barrier, streams, which=(0, 1, 2)):
    """W warm-up steps, then K timed steps: every step runs the contexts in
    `which` to convergence from init(), each as one device-driven CUDA-graph
    launch.  CUDA events on the ctx streams bracket the step and each run."""
    import torch
    ctxs = [W.ctxs[i] for i in which]
    strm = [streams[i] for i in which]

    def step():
        out = []
        for c in ctxs:
            c.init()
            out.append(c.run())
        return out

    for _ in range(args.warmup):
        step()
    per = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(len(ctxs) * args.steps)]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    agg = {"units": 0.0, "edges": 0, "launches": 0, "rounds": [], "pr_iterations": [], "device_loop": True,
           "push_rounds": 0, "pull_rounds": 0}
    barrier()
    ev0.record(strm[0])
    k = 0
    for _ in range(args.steps):
        sts = []
        for c, s in zip(ctxs, strm):
            per[k][0].record(s)
            c.init()
            st = c.run()
            per[k][1].record(s)
            k += 1
            sts.append(st)
        for st in sts:
            agg["edges"] += st["edges_scanned"]
            agg["launches"] += st["kernel_launches"]
            agg["device_loop"] = agg["device_loop"] and bool(st["device_loop"])
            agg["push_rounds"] += st["push_rounds"]
            agg["pull_rounds"] += st["pull_rounds"]
        agg["rounds"].append([st["rounds"] for st in sts])
        if which == (0, 1, 2):
            agg["units"] += W.units(sts)
            agg["pr_iterations"].append(sts[2]["rounds"])
        else:
            agg["units"] += sum((W.E_cc, W.E_d, W.E_d)[i] * (1 if i < 2 else st["rounds"])
                                for i, st in zip(which, sts))
    ev1.record(strm[-1])
    barrier()
    secs = ev0.elapsed_time(ev1) / 1e3
    per_ms = [[0.0] * args.steps for _ in ctxs]
    for j in range(len(ctxs) * args.steps):
        per_ms[j % len(ctxs)][j // len(ctxs)] = per[j][0].elapsed_time(per[j][1])
    agg["ctx_ms"] = [statistics.median(x) for x in per_ms]
    return secs, agg


def profile_pass(W):
    """The same step with the rounds driven from the host and CUDA events
    around every stage and around the two edge-map kernels (the
    load-balanced push of CC/SSSP, the edge-balanced pull of PageRank)."""
    out = {}
    for c in W.ctxs:
        c.set_profiling(True)
    try:
        for name, c in zip(("cc", "sssp", "pagerank"), W.ctxs):
            c.init()
            out[name] = c.run(host_loop=True)
    finally:
        for c in W.ctxs:
            c.set_profiling(False)
    return out


def roofline_of(W, prof, pr_run_ms, peak, peak_src):
    """k_pr_pull (the dominant kernel: the PageRank edge-map) by the pull
    round's algorithmic bytes, the whole PageRank iteration by its
    algorithmic bytes, and the load-balanced push of CC/SSSP."""
    p = prof["pagerank"]
    S = sum(sum(W.pr.layout_info(i)[:2]) for i in range(NUM_MEMORY))
    V, E = W.V, W.E_d
    # pull round over every slot: offsets, partial write, per in-edge its
    # index and the source value gathered, the frontier bitmap
    pull_bytes = (S + 1) * 4 + S * 4 + E * 8 + V / 8
    nl = max(p["pull_launches"], 1)
    pull_ms = p["pull_ms"] / nl
    ach = pull_bytes / (pull_ms / 1e3) / 1e9 if pull_ms > 0 else 0.0
    it = max(p["rounds"], 1)
    iter_bytes = V * 16 + E * 8  # per iteration: offset, contribution read, rank and contribution writes; index + gather per edge
    iter_ms = pr_run_ms / it
    iter_ach = iter_bytes / (iter_ms / 1e3) / 1e9
    push = {}
    lbs_ms = sum(prof[k]["lbs_ms"] for k in ("cc", "sssp"))
    lbs_n = max(sum(prof[k]["lbs_launches"] for k in ("cc", "sssp")), 1)
    lbs_bytes = sum(prof[k]["lbs_actives"] * 12 + prof[k]["lbs_edges"] * (12 + (4 if k == "sssp" else 0))
                    for k in ("cc", "sssp"))
    lbs_edges = sum(prof[k]["lbs_edges"] for k in ("cc", "sssp"))
    if lbs_ms > 0:
        a = lbs_bytes / (lbs_ms / 1e3) / 1e9
        push = {"kernel": "k_push_lbs (load-balanced push edge-map of CC/SSSP)", "achieved": a, "frac": a / peak,
                "alg_bytes_per_launch": lbs_bytes / lbs_n, "avg_launch_ms": lbs_ms / lbs_n, "launches": lbs_n,
                "traffic": DRAM_BYTES_PER_PUSH_EDGE * lbs_edges / lbs_n}
    return {
        "bound": "hbm", "kernel": "k_pr_pull (edge-balanced PageRank pull edge-map)",
        "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "peak_source": peak_src,
        # DRAM bytes per in-edge of the kernel's ncu capture times this graph's in-edges
        "traffic": DRAM_BYTES_PER_PULL_EDGE * E,
        "alg_bytes_per_launch": pull_bytes, "avg_launch_ms": pull_ms, "launches": p["pull_launches"],
        "pagerank_iteration": {"alg_bytes": iter_bytes, "ms": iter_ms, "achieved": iter_ach,
                               "frac": iter_ach / peak,
                               "kernels": "k_pr_pull, k_pr_fix, k_pr_update, k_pr_round_end"},
        "push_edge_map": push,
        "stage_ms": {k: prof[k]["stage_ms"] for k in prof},
    }


def e2e_pass(W, args, barrier, streams, dev):
    """End to end through the C ABI with host buffers: every step copies the
    three layouts from pinned host memory and reads the three results back
    into pinned host arrays.  Copies are pipelined with the runs, one step
    ahead: once a step's three runs are queued, the next step's layouts are
    queued on each context's own stream, so CC's and SSSP's copies overlap
    the long PageRank run and PageRank's copy (queued behind its own run)
    overlaps the next CC and SSSP runs.  Runs and reads are queued
    (run(wait=False), read(wait=False)) and ordered by stream events so that
    the three runs never share the GPU."""
    import numpy as np
    import torch
    from grudon_gb300.replicas import job_throughput
    V = W.V
    res = [torch.empty(V, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
           torch.empty(V, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32),
           torch.empty(V, dtype=torch.float32, pin_memory=True).numpy()]

    def read(i, c, wait):
        return c.read_ranks(out=res[i], wait=wait) if i == 2 else c.read_props(out=res[i], wait=wait)

    run_done = [torch.cuda.Event() for _ in range(3)]
    n = len(W.ctxs)
    # the three uploads alone, one after another (link bandwidth)
    barrier()
    t0 = time.perf_counter()
    up_bytes = sum(c.upload() for c in W.ctxs)
    barrier()
    upload_alone_gbs = up_bytes / (time.perf_counter() - t0) / 1e9
    barrier()
    t0 = time.perf_counter()
    marks = []
    h2d = sum(c.upload() for c in W.ctxs)  # the first step's layouts
    for k in range(args.steps):
        marks.append(time.perf_counter())
        for i, c in enumerate(W.ctxs):
            c.wait()
            c.init()  # set-up after this context's upload; may overlap the previous context's run
            if k or i:
                streams[i].wait_event(run_done[(i - 1) % n])
            c.run(wait=False)
            read(i, c, False)
            run_done[i].record(streams[i])
        if k + 1 < args.steps:  # the next step's layouts, each behind its own context's run and read
            h2d += sum(c.upload() for c in W.ctxs)
    sts = [c.wait() for c in W.ctxs]
    barrier()
    secs = time.perf_counter() - t0
    units = args.steps * W.units(sts)  # every step runs the same graphs from init()
    thr, _, _ = job_throughput(units, secs, dev)
    for i, c in enumerate(W.ctxs):  # the queued reads delivered the final results
        got = res[i].copy()
        if not np.array_equal(got, c.read_ranks() if i == 2 else c.read_props()):
            raise RuntimeError("queued result reads differ from a blocking read")
    marks.append(t0 + secs)
    gaps = [1e3 * (b - a) for a, b in zip(marks, marks[1:])]
    return {"value": thr / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": h2d // args.steps,
            "d2h_bytes_per_step": 4 * 3 * V, "upload_alone_gbs": upload_alone_gbs,
            "host_ms_per_step": {"first": gaps[0], "median_rest": statistics.median(gaps[1:]) if len(gaps) > 1
                                 else None, "max": max(gaps)}}


def parity_and_cpu(W, gpu_out, pr_iters, threads):
    """Outside the timed region: the oracle's restated round protocol (CC,
    weighted SSSP) and the restated FP32-Kahan Jacobi PageRank on the same
    graphs, all host threads, timed as the CPU baseline (one full step); the
    GPU results against them (CC/SSSP bit-exact, rounds equal), the
    reference's verify() invariants on the device, and the PageRank ranks
    against FP64 Jacobi for the same iteration count (max relative error
    <= 1e-5)."""
    import numpy as np
    from oracle import ffi as O
    G_cc, G_d = W.G_cc, W.G_d
    L_cc = O.Layout(G_cc.row_offsets, G_cc.col_indices, mirror=W.p_cc, num_memory=NUM_MEMORY)
    L_ss = O.Layout(G_d.row_offsets, G_d.col_indices, G_d.weights, mirror=W.p_d, num_memory=NUM_MEMORY)
    t0 = time.perf_counter()
    r_cc = L_cc.run(O.ORC_CC, threads=threads)
    t_cc = time.perf_counter() - t0
    t0 = time.perf_counter()
    r_ss = L_ss.run(O.ORC_SSSP_W, threads=threads)
    t_ss = time.perf_counter() - t0
    P = O.PrJacobi(G_d.row_offsets, G_d.col_indices, threads=threads)
    P.init()
    t0 = time.perf_counter()
    it, _ = P.iterate(pr_iters)
    t_pr = time.perf_counter() - t0
    cpu_ranks = P.ranks()
    ref64, it64, _ = O.pr_jacobi_fp64_mt(G_d.row_offsets, G_d.col_indices, iters=pr_iters, threads=threads)

    def rel(got):
        got = got.astype(np.float64)
        both0 = (got == 0) & (ref64 == 0)
        return float(np.where(both0, 0.0, np.abs(got - ref64) / np.maximum(np.abs(ref64), 1e-300)).max())

    cc_ok = bool(np.array_equal(gpu_out["cc"], r_cc["props"]))
    ss_ok = bool(np.array_equal(gpu_out["sssp"], r_ss["props"]))
    pr_err = rel(gpu_out["pagerank"])
    parity = {
        "cc": "bit-exact" if cc_ok else "MISMATCH", "cc_rounds_equal": gpu_out["rounds"][0] == r_cc["stats"]["rounds"],
        "sssp": "bit-exact" if ss_ok else "MISMATCH",
        "sssp_rounds_equal": gpu_out["rounds"][1] == r_ss["stats"]["rounds"],
        "verify_errors": gpu_out["verify"],
        "pagerank": {"max_rel_err_vs_fp64": pr_err, "bound": 1e-5, "iterations": pr_iters,
                     "cpu_fp32_kahan_max_rel_err_vs_fp64": rel(cpu_ranks)},
        "graphs": f"the benchmark's RMAT-{W.G_cc.num_vertices.bit_length() - 1} graphs",
    }
    parity["ok"] = bool(cc_ok and ss_ok and parity["cc_rounds_equal"] and parity["sssp_rounds_equal"] and
                        not any(gpu_out["verify"].values()) and pr_err <= 1e-5)
    units = W.E_cc + W.E_d + pr_iters * W.E_d
    cpu = {"value": units / (t_cc + t_ss + t_pr) / 1e9, "unit": "GTEPS", "cores": threads, "kind": "port",
           "seconds": t_cc + t_ss + t_pr, "seconds_cc_sssp_pagerank": [t_cc, t_ss, t_pr],
           "sample": f"one full step on the same graphs: CC + weighted SSSP to convergence (the oracle's "
                     f"restatement of the reference round protocol, 1C+{NUM_MEMORY}M) and {pr_iters} PageRank "
                     f"Jacobi iterations (FP32 Kahan, FP64 residual), {threads} host threads; the reference "
                     f"itself is unbuildable (Galois/MPI absent)"}
    return parity, cpu


def bench_rmat22(g, args, local, barrier, threads):
    """Config 2 of the workload definition, kept beside the headline: plain
    CC + weighted SSSP on RMAT-22, 1C+3M, device-driven loops."""
    import torch
    a, b, c = RMAT_ABC
    seed = g.rmat_seed(22, EF)
    G_cc = g.Graph.rmat(22, EF, a, b, c, seed=seed, symmetrize=True, threads=threads)
    G_d = g.Graph.rmat(22, EF, a, b, c, seed=seed, weighted=True, threads=threads)
    cc = g.Context(G_cc, G_cc.partition_edge_balanced(NUM_MEMORY), num_memory=NUM_MEMORY, device=local)
    ss = g.Context(G_d, G_d.partition_edge_balanced(NUM_MEMORY), num_memory=NUM_MEMORY, device=local)
    cc.set_algo(g.GRD_CC)
    ss.set_algo(g.GRD_SSSP_W)
    try:
        for _ in range(3):
            for x in (cc, ss):
                x.init()
                x.run()
        s0, s1 = torch.cuda.ExternalStream(cc.stream()), torch.cuda.ExternalStream(ss.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n = 10
        barrier()
        e0.record(s0)
        for _ in range(n):
            for x in (cc, ss):
                x.init()
                x.run()
        e1.record(s1)
        barrier()
        ms = e0.elapsed_time(e1) / n
    finally:
        cc.close()
        ss.close()
    return {"workload": "CC (symmetrised) + weighted SSSP to convergence, RMAT-22 ef16, 1C+3M",
            "value": (G_cc.num_edges + G_d.num_edges) / (ms / 1e3) / 1e9, "unit": "GTEPS", "ms_per_step": ms,
            "E_cc_symmetrised": G_cc.num_edges, "E_sssp": G_d.num_edges}


def bench_policy_offload(g, W, args, barrier, streams):
    """CC + SSSP of the headline under the other schedules, timed on the same
    contexts: the shipped learned round policy, and the reference's NDPEngine
    offload rule; each must leave every result bit-identical."""
    model = load_policy_model()
    out = {}
    W.set_policy(g.GRD_POLICY_FIXED)
    base_s, base = timed_steps(W, args, barrier, streams, which=(0, 1))
    base_props = [(c.init(), c.run(), c.read_props())[2] for c in (W.cc, W.ss)]
    out["fixed"] = {"value": base["units"] / base_s / 1e9, "ms_per_step": base_s * 1e3 / args.steps,
                    "rounds": base["rounds"][0], "push_rounds_per_step": base["push_rounds"] / args.steps,
                    "pull_rounds_per_step": base["pull_rounds"] / args.steps}
    if model is not None:
        W.set_policy(g.GRD_POLICY_LEARNED, model)
        s, a = timed_steps(W, args, barrier, streams, which=(0, 1))
        props = [(c.init(), c.run(), c.read_props())[2] for c in (W.cc, W.ss)]
        out["learned"] = {"value": a["units"] / s / 1e9, "ms_per_step": s * 1e3 / args.steps,
                          "rounds": a["rounds"][0], "push_rounds_per_step": a["push_rounds"] / args.steps,
                          "pull_rounds_per_step": a["pull_rounds"] / args.steps,
                          "results_bit_identical": all(bool((x == y).all()) for x, y in zip(base_props, props))}
        out["learned_speedup_vs_fixed"] = out["learned"]["value"] / out["fixed"]["value"]
    if model is not None:
        out["held_out"] = policy_held_out(g, model)
    W.set_policy(g.GRD_POLICY_FIXED, offload=g.GRD_OFFLOAD_ENGINE)
    s, a = timed_steps(W, args, barrier, streams, which=(0, 1))
    sts = [(c.init(), c.run())[1] for c in (W.cc, W.ss)]
    props = [c.read_props() for c in (W.cc, W.ss)]
    W.set_policy(g.GRD_POLICY_FIXED)
    offload = {"ndp": out["fixed"]["value"], "engine": a["units"] / s / 1e9,
               "engine_speedup_vs_ndp": (a["units"] / s / 1e9) / out["fixed"]["value"],
               "no_offload_rounds_per_step": [st["no_offload_rounds"] for st in sts],
               "results_bit_identical": all(bool((x == y).all()) for x, y in zip(base_props, props))}
    return {"cc_sssp": out, "model": "grudon_gb300/policy_model.json" if model is not None else None}, offload


def policy_leg(g, model, G, algo, max_rounds=None, reps=2) -> dict:
    """The fixed rule against the shipped model on one graph that no model
    was trained on: 1C+3M, device-driven runs, best of `reps`; the results
    (labels, distances or ranks) must be bit-identical."""
    import numpy as np
    import torch
    res, outs = {}, []
    kw = {} if max_rounds is None else {"max_rounds": max_rounds}
    with g.Context(G, G.partition_edge_balanced(NUM_MEMORY), NUM_MEMORY) as ctx:
        s = torch.cuda.ExternalStream(ctx.stream())
        for name, pol in (("fixed", g.GRD_POLICY_FIXED), ("learned", g.GRD_POLICY_LEARNED)):
            ctx.set_algo(algo, policy=pol, **kw)
            ctx.set_policy(model if pol == g.GRD_POLICY_LEARNED else None)
            best, st = float("inf"), None
            for _ in range(reps):
                ctx.init()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                st = ctx.run()
                e1.record(s)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            outs.append(ctx.read_ranks() if algo == g.GRD_PR_DELTA else ctx.read_props())
            res[name] = {"ms": best, "rounds": st["rounds"], "push_rounds": st["push_rounds"],
                         "pull_rounds": st["pull_rounds"]}
    res["learned_speedup_vs_fixed"] = res["fixed"]["ms"] / res["learned"]["ms"]
    res["results_bit_identical"] = bool(np.array_equal(outs[0], outs[1]))
    return res


def policy_held_out(g, model) -> dict:
    """The learned policy on two held-out workloads: CC on a 3000 x 3000 grid
    (weights in [1,255], 1000 rounds) and delta PageRank (the reference's own
    algorithm, which the fixed rule runs push-only) on the benchmark's
    RMAT-22 directed graph."""
    a, b, c = RMAT_ABC
    out = {"grid3000_cc": policy_leg(g, model, g.Graph.grid(3000, seed=3000), g.GRD_CC, max_rounds=1000)}
    G = g.Graph.rmat(22, EF, a, b, c, seed=g.rmat_seed(22, EF))
    out["rmat22_pr_delta"] = policy_leg(g, model, G, g.GRD_PR_DELTA)
    return out


def bench_ingest(g, W, args, local, barrier, dev) -> dict:
    """The partition layout of the three contexts built on the host
    (layout.cpp, all host threads) and on the GPU (grd_ingest: the CSR
    uploaded from host memory, then proxies, translation slots, the relabelled
    CSR and, for PageRank, the in-edge view built by kernels)."""
    graphs = ((W.G_cc, W.p_cc), (W.G_d, W.p_d), (W.G_pr, W.p_d))
    t0 = time.perf_counter()
    for G, p in graphs[:2]:
        g.layout_preview(G, p, NUM_MEMORY, 0)
    host_ms = (time.perf_counter() - t0) * 1e3
    dctx = [g.Context(G, p, num_memory=NUM_MEMORY, device=local, device_layout=True) for G, p in graphs]
    try:
        dctx[2].set_algo(g.GRD_PR_PULL, max_rounds=PR_MAX_ITERS, tolerance=PR_TOL)  # builds its in-edge view
        best = None
        for _ in range(3):
            barrier()
            t0 = time.perf_counter()
            nbytes = sum(c.ingest(G, p) for c, (G, p) in zip(dctx, graphs))
            barrier()
            dt = (time.perf_counter() - t0) * 1e3
            best = dt if best is None else min(best, dt)
    finally:
        for c in dctx:
            c.close()
    return {"host_layout_ms_cc_sssp": host_ms, "device_layout_ms_all_three": best, "device_h2d_bytes": nbytes,
            "host_threads": os.cpu_count(),
            "note": "device: CSR upload from pageable host memory + layout build of the three contexts (PageRank's "
                    "in-edge view included); host: layout.cpp for the CC and SSSP graphs"}


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
    lab_seq, rk_seq, plain_s = B.run_plain_graphs(sym, dirg, 20, local)
    lab_con, rk_con, plain_con_s = B.run_plain_graphs(sym, dirg, 20, local, concurrent=True)
    plain_same = all(bool(np.array_equal(a, b)) for a, b in zip(lab_seq + rk_seq, lab_con + rk_con))
    Uc, Up = B.Union(sym), B.Union(dirg)
    reps = 3

    def time_union(cc_kw, cc_policy, model_, num_memory):
        """One union per algorithm: CC with the given schedule and policy, 20
        PageRank iterations; seconds per (CC + PageRank) pass, best of reps."""
        pc = Uc.graph.partition_edge_balanced(num_memory) if num_memory > 1 else None
        pp = Up.graph.partition_edge_balanced(num_memory) if num_memory > 1 else None
        with g.Context(Uc.graph, pc, num_memory, local) as cc_, g.Context(Up.graph, pp, num_memory, local) as pr_:
            cc_.set_algo(g.GRD_CC, policy=cc_policy, **cc_kw)
            cc_.set_policy(model_)
            pr_.set_algo(g.GRD_PR_PULL, max_rounds=20, tolerance=0.0)
            best_ = float("inf")
            for k in range(reps + 1):
                t0_ = time.perf_counter()
                for c_ in (cc_, pr_):
                    c_.init()
                    c_.run()
                cc_.synchronize()
                if k:
                    best_ = min(best_, time.perf_counter() - t0_)
            return best_, cc_.read_props()

    # batching alone: the unions with the library defaults and the fixed rule
    union_fixed_s, props_fixed = time_union({}, g.GRD_POLICY_FIXED, None, 1)
    tune_cc = autotune.tune(Uc.graph, g.GRD_CC, lambda c: c.init(), device=local, reps=2)
    best = tune_cc.best
    model = load_policy_model()
    pol = g.GRD_POLICY_LEARNED if model is not None else g.GRD_POLICY_FIXED
    # + the autotuned schedule, then + the learned round policy
    union_tuned_s, _ = time_union(best.params(), g.GRD_POLICY_FIXED, None, best.num_memory)
    batched_s, props_learned = time_union(best.params(), pol, model, best.num_memory)
    part1 = {"graphs": len(spec), "vertices": int(Uc.sizes.sum()), "edges_cc": Uc.graph.num_edges,
             "edges_pr": Up.graph.num_edges, "generate_s": t_gen,
             "plain_s": plain_s, "batched_s": batched_s, "speedup": plain_s / batched_s,
             "plain_concurrent_s": plain_con_s, "speedup_vs_concurrent_plain": plain_con_s / batched_s,
             "plain_concurrent_results_identical": plain_same,
             "union_fixed_s": union_fixed_s, "union_tuned_s": union_tuned_s,
             "speedup_batching": plain_s / union_fixed_s, "speedup_autotune": union_fixed_s / union_tuned_s,
             "speedup_learned_policy": union_tuned_s / batched_s,
             "results_bit_identical": bool(np.array_equal(props_fixed, props_learned)),
             "batched_gteps": E1 / batched_s / 1e9, "plain_gteps": E1 / plain_s / 1e9,
             "autotuned": best.__dict__, "tune_table_ms": [round(r["ms"], 3) for r in tune_cc.table]}

    # (2) multi-source SSSP: per-source runs against one grd_sssp_multi call
    # (64 distance lanes per vertex over the one resident CSR)
    G = g.Graph.rmat(20, 16, weighted=True)
    rng = np.random.default_rng(0x53535350)
    sources = rng.integers(0, G.num_vertices, args.batch_sources)
    c1 = g.Context(G, None, 1, local)
    c1.set_algo(g.GRD_SSSP_W)
    c1.init()
    c1.run()
    single = []
    t0 = time.perf_counter()
    for s in sources:
        c1.set_algo(g.GRD_SSSP_W, source=int(s))
        c1.init()
        c1.run()
        single.append(c1.read_props())
    c1.synchronize()
    plain2 = time.perf_counter() - t0
    c1.set_algo(g.GRD_SSSP_W)
    c1.init()
    dist, st = c1.sssp_multi(sources)  # warm-up (first call allocates)
    ts = []
    for _ in range(reps):
        c1.init()
        t0 = time.perf_counter()
        dist, st = c1.sssp_multi(sources)
        ts.append(time.perf_counter() - t0)
    batched2 = min(ts)
    identical = all(bool(np.array_equal(dist[i], single[i])) for i in range(len(sources)))
    c1.close()
    E2 = len(sources) * G.num_edges
    part2 = {"sources": len(sources), "graph": "RMAT-20 ef16 w in [1,255]", "plain_s": plain2,
             "batched_s": batched2, "speedup": plain2 / batched2, "rounds": st["rounds"],
             "batched_gteps": E2 / batched2 / 1e9, "plain_gteps": E2 / plain2 / 1e9,
             "method": "grd_sssp_multi: 64 distance lanes per vertex over one CSR (the graph held once in HBM); "
                       "batched time includes reading the 64 x V distances back",
             "bit_identical_to_single_source_runs": identical}
    total_plain, total_batched = plain_s + plain2, batched_s + batched2
    return {"part1_graphs": part1, "part2_sssp_sources": part2,
            "end_to_end_speedup": total_plain / total_batched,
            "shares": "part 1 splits into batching (plain -> one union per algorithm, library defaults, fixed "
                      "rule), the autotuned schedule and the learned policy; part 2's gain is the shared CSR",
            "policy": "learned" if model is not None else "fixed",
            "note": "plain: one ctx per graph (per source) with the fixed per-round rule, run one after another; "
                    "part 1 also times the same contexts with all runs queued at once (plain_concurrent_s); "
                    "batched: part 1 one "
                    "union per algorithm, autotuned schedule and the learned round policy (CC; PageRank is "
                    "Jacobi pull), part 2 one multi-source call; timings exclude layout build"}


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


def kernel_run(g, args, local, rank, threads):
    """Host-driven steps only (plain launches), for per-kernel profilers."""
    W = Workload(g, args.scale, threads, local)
    try:
        W.set_policy(g.GRD_POLICY_FIXED)
        for _ in range(args.warmup + args.steps):
            sts = [(c.init(), c.run(host_loop=True))[1] for c in W.ctxs]
        if rank == 0:
            print(json.dumps({"kernel_run": True, "scale": args.scale, "rounds": [st["rounds"] for st in sts],
                              "launches_per_step": sum(st["kernel_launches"] for st in sts)}), flush=True)
    finally:
        W.close()


def ingest_run(g, args, local, rank, threads):
    """Device-layout contexts for the workload's three graphs (CC symmetrised,
    SSSP weighted, PageRank with its in-edge view), each re-ingested
    warmup + steps times."""
    a, b, c = RMAT_ABC
    seed = g.rmat_seed(args.scale, EF)
    G_cc = g.Graph.rmat(args.scale, EF, a, b, c, seed=seed, symmetrize=True, threads=threads)
    G_d = g.Graph.rmat(args.scale, EF, a, b, c, seed=seed, weighted=True, threads=threads)
    G_pr = g.Graph.from_csr(G_d.row_offsets, G_d.col_indices)
    graphs = ((G_cc, G_cc.partition_edge_balanced(NUM_MEMORY)), (G_d, G_d.partition_edge_balanced(NUM_MEMORY)),
              (G_pr, G_d.partition_edge_balanced(NUM_MEMORY)))
    ctxs = [g.Context(G, p, num_memory=NUM_MEMORY, device=local, device_layout=True) for G, p in graphs]
    try:
        ctxs[2].set_algo(g.GRD_PR_PULL)  # builds its in-edge view
        h2d = 0
        for _ in range(args.warmup + args.steps):
            h2d = sum(ctx.ingest(G, p) for ctx, (G, p) in zip(ctxs, graphs))
        for ctx in ctxs:
            ctx.synchronize()
    finally:
        for ctx in ctxs:
            ctx.close()
    if rank == 0:
        print(json.dumps({"ingest_run": True, "scale": args.scale, "h2d_bytes_per_ingest": h2d}), flush=True)


def kernel_run_pr(g, args, local, rank, threads):
    a, b, c = RMAT_ABC
    G = g.Graph.rmat(args.scale, EF, a, b, c, seed=g.rmat_seed(args.scale, EF), threads=threads)
    with g.Context(G, G.partition_edge_balanced(NUM_MEMORY), num_memory=NUM_MEMORY, device=local) as ctx:
        ctx.set_algo(g.GRD_PR_PULL, max_rounds=args.warmup + args.steps, tolerance=0.0)
        ctx.init()
        st = ctx.run(host_loop=True)
    if rank == 0:
        print(json.dumps({"kernel_run_pr": True, "scale": args.scale, "iterations": st["rounds"],
                          "edges": G.num_edges}), flush=True)


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
    from grudon_gb300.replicas import job_throughput

    threads = max(1, (os.cpu_count() or 1) // ws)
    if args.kernel_run_pr:
        kernel_run_pr(g, args, local, rank, threads)
        return
    if args.ingest_run:
        ingest_run(g, args, local, rank, threads)
        return
    if args.kernel_run:
        kernel_run(g, args, local, rank, threads)
        return

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    dev = torch.device("cuda", local) if ws > 1 else None
    peak, peak_src = hbm_peak()
    W = Workload(g, args.scale, threads, local)
    model = load_policy_model()
    learned = args.policy == "learned" and model is not None
    W.set_policy(g.GRD_POLICY_LEARNED if learned else g.GRD_POLICY_FIXED, model)
    streams = [torch.cuda.ExternalStream(c.stream()) for c in W.ctxs]

    clocks = ClockSampler(local)
    clocks.start()
    secs, agg = timed_steps(W, args, barrier, streams)
    clk = clocks.stop()
    thr, secs_max, _ = job_throughput(agg["units"], secs, dev)
    value = thr / 1e9

    prof = profile_pass(W)
    roofline = roofline_of(W, prof, agg["ctx_ms"][2], peak, peak_src)
    gpu_out = {"cc": W.cc.read_props(), "sssp": W.ss.read_props(), "pagerank": W.pr.read_ranks(),
               "rounds": agg["rounds"][-1]}
    gpu_out["verify"] = {"cc": W.cc.verify()["errors"], "sssp": W.ss.verify()["errors"]}
    e2e = e2e_pass(W, args, barrier, streams, dev)

    extras = {}
    if not args.no_extras:
        extras["policy"], extras["offload"] = bench_policy_offload(g, W, args, barrier, streams)
        extras["ingest"] = bench_ingest(g, W, args, local, barrier, dev)
    line = {
        "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs_max * 1e3 / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32", "data": "synthetic",
        "config": workload_config(args.scale, W.seed, W.V, W.E_cc, W.E_d,
                                  csr_checksum(W.G_cc.row_offsets, W.G_cc.col_indices),
                                  csr_checksum(W.G_d.row_offsets, W.G_d.col_indices, W.G_d.weights), ws),
        "e2e": e2e, "gpu_launches": agg["launches"], "roofline": roofline, "clocks": clk,
        "per_algorithm": {
            name: {"ms": agg["ctx_ms"][i], "gteps": units / (agg["ctx_ms"][i] / 1e3) / 1e9}
            for i, (name, units) in enumerate((("cc", W.E_cc), ("sssp", W.E_d),
                                               ("pagerank", W.E_d * agg["pr_iterations"][-1])))},
        "rounds_per_step": agg["rounds"][-1], "pagerank_iterations": agg["pr_iterations"][-1],
        "device_loop": agg["device_loop"], "policy_headline": "learned" if learned else "fixed",
        "edges_scanned_gteps": ws * agg["edges"] / secs_max / 1e9,
    }
    failed = False
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        parity, cpu = parity_and_cpu(W, gpu_out, agg["pr_iterations"][-1], os.cpu_count() or 1)
        line["parity"] = parity
        line["cpu_baseline"] = cpu
        failed = not parity["ok"]
    W.close()
    if not args.no_extras:
        extras["config2_rmat22"] = bench_rmat22(g, args, local, barrier, threads)
        if rank == 0 and ws == 1:
            extras["reference_cpu_case"] = bench_reference_cpu_case(g, local)
        if args.batch or (ws == 1 and not args.no_batch):
            extras["batch"] = bench_batch(g, args, local)
    line.update(extras)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    if failed:
        sys.exit("parity check failed on the benchmark graphs")


# --------------------------------------------------------- reference arm --
def run_reference(args):
    """The reference algorithm on the host cores (the oracle's restatement,
    all threads), on graphs built by the oracle's generator (no product
    library is loaded).  Each step is a bounded sample: the steps take turns
    over CC to convergence, SSSP to convergence and 4 PageRank iterations;
    the value is the full step's units over the full step's estimated time
    (mean CC time + mean SSSP time + iterations x mean iteration time)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import ffi as O
    threads = os.cpu_count() or 1
    a, b, c = RMAT_ABC
    seed = O.rmat_seed(args.scale, EF)
    ro_s, col_s, _ = O.gen_rmat(args.scale, EF, a, b, c, seed, symmetrize=True, threads=threads)
    ro_d, col_d, w_d = O.gen_rmat(args.scale, EF, a, b, c, seed, weighted=True, threads=threads)
    p_s, p_d = O.partition_edge_balanced(ro_s, NUM_MEMORY), O.partition_edge_balanced(ro_d, NUM_MEMORY)
    V, E_cc, E_d = len(ro_s) - 1, len(col_s), len(col_d)
    config = workload_config(args.scale, seed, V, E_cc, E_d, csr_checksum(ro_s, col_s),
                             csr_checksum(ro_d, col_d, w_d), ws)
    L_cc = O.Layout(ro_s, col_s, mirror=p_s, num_memory=NUM_MEMORY)
    L_ss = O.Layout(ro_d, col_d, w_d, mirror=p_d, num_memory=NUM_MEMORY)
    P = O.PrJacobi(ro_d, col_d, threads=threads)
    # the PageRank step's iteration count under its own stop rule
    P.init()
    iters, _ = P.iterate(PR_MAX_ITERS, PR_TOL)
    P.init()
    times = {0: [], 1: [], 2: []}
    sample_iters = 4

    def sample(k):
        kind = k % 3
        t0 = time.perf_counter()
        if kind == 0:
            L_cc.run(O.ORC_CC, threads=threads)
        elif kind == 1:
            L_ss.run(O.ORC_SSSP_W, threads=threads)
        else:
            P.iterate(sample_iters)
        return kind, time.perf_counter() - t0

    for k in range(args.warmup):
        sample(k)
    for k in range(args.steps):
        kind, dt = sample(k)
        times[kind].append(dt / (sample_iters if kind == 2 else 1))
    for kind in (0, 1, 2):  # every part sampled at least once
        if not times[kind]:
            times[kind].append(sample(kind)[1] / (sample_iters if kind == 2 else 1))
    step_s = statistics.mean(times[0]) + statistics.mean(times[1]) + iters * statistics.mean(times[2])
    units = E_cc + E_d + iters * E_d
    value = units / step_s / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GTEPS", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32", "data": "synthetic", "config": config,
        "cpu_baseline": {"value": value, "unit": "GTEPS", "cores": threads, "kind": "port",
                         "sample": f"steps take turns over CC to convergence, weighted SSSP to convergence and "
                                   f"{sample_iters} PageRank iterations (oracle restatements, {threads} host "
                                   f"threads); value = full step units / (mean CC + mean SSSP + {iters} x mean "
                                   f"iteration time); samples per part: {[len(times[k]) for k in (0, 1, 2)]}; "
                                   f"reference itself unbuildable (Galois/MPI absent)"},
        "e2e": {"value": value, "unit": "GTEPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "pagerank_iterations": iters,
        "seconds_cc_sssp_iteration": [statistics.mean(times[k]) for k in (0, 1, 2)],
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
