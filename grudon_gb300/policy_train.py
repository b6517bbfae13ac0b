"""Trains the learned round policy on the GPU and writes the model file.

Training graphs: RMAT scale 18-22 with quadrant a in [0.45, 0.65]
(b = c = (1 - a - 0.05) / 2, d = 0.05) and 2D 4-neighbour grids 512^2 -
4096^2 with uint32 weights in [1, 255].  For each graph and algorithm (CC on
the symmetrised graph, weighted SSSP and delta PageRank on the directed one)
the plain method runs once per forced round mode; the per-round timings are
the targets (grudon_gb300.policy.collect).  Held-out evaluation (--held-out):
RMAT-24 (a = 0.57, a value not trained on: CC, weighted SSSP, delta
PageRank) and a 3000^2 grid (a size and seed not trained on: CC, weighted
SSSP), offline (measured per-round table) and online (device-loop runs,
learned vs fixed rule, results compared bit for bit).

    python -m grudon_gb300.policy_train --out grudon_gb300/policy_model.json \
        --report policy_report.json [--held-out] [--quick]
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

import grudon_gb300 as g
from grudon_gb300 import policy as P

ER_D = 0.05


def rmat(scale: int, a: float, sym: bool, weighted: bool, ef: int = 16) -> g.Graph:
    b = (1.0 - a - ER_D) / 2.0
    seed = g.rmat_seed(scale, ef) ^ int(round(a * 1000)) << 32
    return g.Graph.rmat(scale, ef, a, b, b, seed=seed, symmetrize=sym, weighted=weighted)


def training_tables(scales, avals, grids, reps: int, log=print):
    tabs = []
    for s in scales:
        for a in avals:
            t0 = time.time()
            Gs = rmat(s, a, True, False)
            tabs.append(P.collect(Gs, g.GRD_CC, f"cc-rmat{s}-a{a:.2f}", reps=reps))
            del Gs
            Gd = rmat(s, a, False, True)
            tabs.append(P.collect(Gd, g.GRD_SSSP_W, f"sssp-rmat{s}-a{a:.2f}", reps=reps))
            tabs.append(P.collect(Gd, g.GRD_PR_DELTA, f"pr-rmat{s}-a{a:.2f}", reps=reps))
            del Gd
            log(f"rmat{s} a={a:.2f}: {time.time() - t0:.1f}s")
    for k in grids:
        t0 = time.time()
        Gg = g.Graph.grid(k, seed=k)
        stride = max(1, k // 256)  # grids run up to the round cap: subsample
        tabs.append(P.collect(Gg, g.GRD_SSSP_W, f"sssp-grid{k}", reps=reps, stride=stride))
        tabs.append(P.collect(Gg, g.GRD_CC, f"cc-grid{k}", reps=reps, stride=stride))
        del Gg
        log(f"grid{k}: {time.time() - t0:.1f}s")
    return tabs


def summarize(tabs, model) -> dict:
    out, tot = {}, {"chosen_ms": 0.0, "fixed_ms": 0.0, "best_ms": 0.0}
    for t in tabs:
        r = P.table_totals(t, P.choose(model, t))
        r["rounds"] = len(t.x)
        out[t.name] = {k: round(v, 4) if isinstance(v, float) else v for k, v in r.items()}
        for k in tot:
            tot[k] += r[k]
    tot["gain_vs_fixed"] = tot["fixed_ms"] / max(tot["chosen_ms"], 1e-12)
    return {"tables": out, "total": tot}


def online(G: g.Graph, algo: int, model, name: str, reps: int = 3) -> dict:
    """Device-loop runs with the fixed rule and with the model: best time of
    `reps`, and the results compared bit for bit (CC/SSSP)."""
    import torch
    part = G.partition_edge_balanced(3)
    res = {}
    with g.Context(G, part, 3) as ctx:
        outs = {}
        for pol in (g.GRD_POLICY_FIXED, g.GRD_POLICY_LEARNED):
            ctx.set_algo(algo, policy=pol, direction=g.GRD_DIR_AUTO)
            ctx.set_policy(model if pol == g.GRD_POLICY_LEARNED else None)
            s = torch.cuda.ExternalStream(ctx.stream())
            best = float("inf")
            st = None
            for _ in range(reps + 1):
                ctx.init()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                st = ctx.run()
                e1.record(s)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            outs[pol] = ctx.read_props() if algo != g.GRD_PR_DELTA else ctx.read_ranks()
            res["learned" if pol else "fixed"] = {"ms": best, "rounds": st["rounds"], "push_rounds": st["push_rounds"],
                                                   "pull_rounds": st["pull_rounds"]}
        res["bit_identical"] = bool(np.array_equal(outs[0], outs[1]))
    res["speedup"] = res["fixed"]["ms"] / res["learned"]["ms"]
    return res


def held_out(model, reps: int, quick: bool, log=print) -> dict:
    s, k = (16, 200) if quick else (24, 3000)
    out = {"offline": {}, "online": {}}
    tabs = []
    t0 = time.time()
    Gs = rmat(s, 0.57, True, False)
    tabs.append(P.collect(Gs, g.GRD_CC, f"cc-rmat{s}", reps=reps))
    out["online"][f"cc-rmat{s}"] = online(Gs, g.GRD_CC, model, f"cc-rmat{s}")
    del Gs
    Gd = rmat(s, 0.57, False, True)
    tabs.append(P.collect(Gd, g.GRD_SSSP_W, f"sssp-rmat{s}", reps=reps))
    out["online"][f"sssp-rmat{s}"] = online(Gd, g.GRD_SSSP_W, model, f"sssp-rmat{s}")
    tabs.append(P.collect(Gd, g.GRD_PR_DELTA, f"pr-rmat{s}", reps=reps))
    out["online"][f"pr-rmat{s}"] = online(Gd, g.GRD_PR_DELTA, model, f"pr-rmat{s}")
    del Gd
    log(f"held-out rmat{s}: {time.time() - t0:.1f}s")
    t0 = time.time()
    Gg = g.Graph.grid(k, seed=k)
    tabs.append(P.collect(Gg, g.GRD_SSSP_W, f"sssp-grid{k}", reps=reps, stride=max(1, k // 256)))
    out["online"][f"sssp-grid{k}"] = online(Gg, g.GRD_SSSP_W, model, f"sssp-grid{k}")
    tabs.append(P.collect(Gg, g.GRD_CC, f"cc-grid{k}", reps=reps, stride=max(1, k // 256)))
    out["online"][f"cc-grid{k}"] = online(Gg, g.GRD_CC, model, f"cc-grid{k}")
    del Gg
    log(f"held-out grid{k}: {time.time() - t0:.1f}s")
    out["offline"] = summarize(tabs, model)
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", default=str(P.MODEL_FILE))
    ap.add_argument("--report", default="")
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--held-out", action="store_true")
    ap.add_argument("--quick", action="store_true", help="small graphs (smoke test of the pipeline)")
    args = ap.parse_args(argv)
    log = lambda m: print(m, file=sys.stderr, flush=True)
    if args.quick:
        scales, avals, grids = (12, 13), (0.45, 0.65), (64, 128)
    else:
        scales, avals, grids = (18, 19, 20, 21, 22), (0.45, 0.55, 0.65), (512, 1024, 2048, 4096)
    t0 = time.time()
    tabs = training_tables(scales, avals, grids, args.reps, log)
    x, y, mask = P.stack(tabs)
    log(f"training samples: {len(x)} ({time.time() - t0:.1f}s to collect)")
    t1 = time.time()
    model, curve = P.train(x, y, mask, steps=args.steps, lr=args.lr, seed=args.seed)
    log(f"trained {args.steps} steps in {time.time() - t1:.2f}s: loss {curve[0]:.4f} -> {curve[-1]:.4f}")
    report = {"samples": int(len(x)), "steps": args.steps, "lr": args.lr, "seed": args.seed,
              "loss_first": float(curve[0]), "loss_last": float(curve[-1]),
              "train_graphs": {"rmat_scales": list(scales), "rmat_a": list(avals), "grids": list(grids)},
              "in_sample": summarize(tabs, model)}
    meta = {k: report[k] for k in ("samples", "steps", "lr", "seed", "loss_first", "loss_last", "train_graphs")}
    meta["in_sample_gain_vs_fixed"] = report["in_sample"]["total"]["gain_vs_fixed"]
    P.save_model(model, args.out, meta)
    if args.held_out:
        report["held_out"] = held_out(model, args.reps, args.quick, log)
    if args.report:
        with open(args.report, "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps({"in_sample_total": report["in_sample"]["total"],
                      "held_out_total": report.get("held_out", {}).get("offline", {}).get("total"),
                      "held_out_online": report.get("held_out", {}).get("online")}, indent=1))
    return 0


if __name__ == "__main__":
    sys.exit(main())
