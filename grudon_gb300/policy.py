"""Learned round policy: training data from the plain method's own per-round
timings, GPU training, and model files.

Every round of CC and SSSP computes the same values, dirty sets and frontier
in each of the four round modes (push / pull x bitvector / list), so running
the algorithm once per forced mode yields, for every round, the measured time
of all four modes on the same state.  Those times (log2 ms) are the MLP's
regression targets; its inputs are the frontier shape entering the round
(grd_policy_features).  At run time the round takes the mode with the smallest
prediction (GRD_POLICY_LEARNED), which never changes CC/SSSP results.
"""
from __future__ import annotations

import ctypes as C
import json
import math
from dataclasses import dataclass, field
from pathlib import Path
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

from . import _ffi
from . import (GRD_CC, GRD_DIR_PULL, GRD_DIR_PUSH, GRD_FMT_BITVEC, GRD_FMT_LIST, GRD_PR_DELTA, GRD_SSSP_HOP,
               GRD_SSSP_W, Context, GrdError, Graph, lib)

MODEL_FILE = Path(__file__).resolve().parent / "policy_model.json"
NIN, NHID, NOUT = _ffi.GRD_POLICY_IN, _ffi.GRD_POLICY_HID, _ffi.GRD_POLICY_OUT
# (direction, frontier format) forcing each round mode, in mode order.
FORCED = [(GRD_DIR_PUSH, GRD_FMT_BITVEC), (GRD_DIR_PUSH, GRD_FMT_LIST), (GRD_DIR_PULL, GRD_FMT_BITVEC),
          (GRD_DIR_PULL, GRD_FMT_LIST)]
ALL_MODES = 0xF
# A frontier this small runs push + list in one CTA without inference (the
# device rule, K_TINY_ACTIVE / K_TINY_EDGES).
TINY_ACTIVE, TINY_EDGES = 2048, 16384


def _f32p(a: np.ndarray):
    return a.ctypes.data_as(_ffi.f32p)


def _check(rc: int) -> None:
    if rc != 0:
        raise GrdError(rc, lib().grd_policy_error().decode())


# ------------------------------------------------------------------ models --
def model_to_dict(m: _ffi.grd_policy_model) -> dict:
    return {f: list(getattr(m, f)) for f, _ in _ffi.grd_policy_model._fields_}


def model_from_dict(d: dict) -> _ffi.grd_policy_model:
    m = _ffi.grd_policy_model()
    d = dict(d)
    d.setdefault("lo", [-1e30] * NIN)  # files without a training range: no clamping
    d.setdefault("hi", [1e30] * NIN)
    for f, t in _ffi.grd_policy_model._fields_:
        arr = getattr(m, f)
        vals = d[f]
        if len(vals) != len(arr):
            raise ValueError(f"model field {f}: {len(vals)} values, expected {len(arr)}")
        for i, v in enumerate(vals):
            arr[i] = v
    return m


def save_model(m: _ffi.grd_policy_model, path, meta: Optional[dict] = None) -> None:
    Path(path).write_text(json.dumps({"model": model_to_dict(m), "meta": meta or {}}, indent=None))


def load_model(path=MODEL_FILE) -> _ffi.grd_policy_model:
    return model_from_dict(json.loads(Path(path).read_text())["model"])


def load_meta(path=MODEL_FILE) -> dict:
    return json.loads(Path(path).read_text()).get("meta", {})


def model_arrays(m: _ffi.grd_policy_model) -> Dict[str, np.ndarray]:
    """float64 views: weights decoded from fp16, [out][in] matrices."""
    def half(a, shape):
        return np.frombuffer(bytes(a), dtype=np.uint16).view(np.float16).astype(np.float64).reshape(shape)
    return {"mean": np.array(m.mean, dtype=np.float64), "scale": np.array(m.scale, dtype=np.float64),
            "w1": half(m.w1, (NHID, NIN)), "b1": np.array(m.b1, dtype=np.float64),
            "w2": half(m.w2, (NHID, NHID)), "b2": np.array(m.b2, dtype=np.float64),
            "w3": half(m.w3, (NOUT, NHID)), "b3": np.array(m.b3, dtype=np.float64),
            "lo": np.array(m.lo, dtype=np.float64), "hi": np.array(m.hi, dtype=np.float64)}


# ---------------------------------------------------------------- features --
def features(frontier, frontier_edges, unvisited, max_degree, rounds, num_vertices: int, num_edges: int) -> np.ndarray:
    f = [np.ascontiguousarray(np.asarray(a, dtype=np.uint64)) for a in (frontier, frontier_edges, unvisited,
                                                                         max_degree)]
    r = np.ascontiguousarray(np.asarray(rounds, dtype=np.uint32))
    n = len(r)
    out = np.zeros((n, NIN), dtype=np.float32)
    _check(lib().grd_policy_features(*(a.ctypes.data_as(_ffi.u64p) for a in f), r.ctypes.data_as(_ffi.u32p),
                                     num_vertices, num_edges, n, _f32p(out)))
    return out


def log_features(log: Sequence[dict], num_vertices: int, num_edges: int) -> np.ndarray:
    return features([r["frontier_in"] for r in log], [r["frontier_edges_in"] for r in log],
                    [r["unvisited_in"] for r in log], [r["max_degree_in"] for r in log],
                    [r["round"] for r in log], num_vertices, num_edges)


# ------------------------------------------------------- training data ------
@dataclass
class RoundTable:
    """Per-round features and measured time (ms) of each forced mode."""
    name: str
    algo: int
    x: np.ndarray            # [n, 8] raw features
    ms: np.ndarray           # [n, 4] round time per mode (NaN: not measured)
    fixed_mode: np.ndarray   # [n] mode the fixed rule chose
    tiny: np.ndarray         # [n] the frontier fits one CTA (mode fixed: push + list)
    info: dict = field(default_factory=dict)

    def targets(self) -> Tuple[np.ndarray, np.ndarray]:
        """log2 round times relative to the mean over the measured modes of
        the same round (only the ordering of the modes matters)."""
        ok = np.isfinite(self.ms) & (self.ms > 0)
        lg = np.where(ok, np.log2(np.where(ok, self.ms, 1.0)), 0.0)
        mean = lg.sum(axis=1, keepdims=True) / np.maximum(ok.sum(axis=1, keepdims=True), 1)
        y = np.where(ok, lg - mean, 0.0).astype(np.float32)
        return y, ok.astype(np.uint8)


def _profiled_run(ctx: Context, algo: int, init, reps: int, **kw) -> List[dict]:
    """Per-round log of the best of `reps` profiled runs (element-wise min of
    the round times; the trajectory is the same in every run)."""
    best = None
    for _ in range(reps):
        ctx.set_algo(algo, **kw)
        init(ctx)
        ctx.run(host_loop=True)
        log = ctx.round_log()
        if best is None:
            best = log
        else:
            if len(log) != len(best):
                if algo != GRD_PR_DELTA:
                    raise RuntimeError("round count changed between identical runs")
                # float atomics: delta PageRank may end a round sooner or later
                n = min(len(log), len(best))
                best, log = best[:n], log[:n]
            for a, b in zip(best, log):
                a["ms"] = [min(u, v) for u, v in zip(a["ms"], b["ms"])]
    return best


def collect(graph: Graph, algo: int, name: str = "", num_memory: int = 3, reps: int = 2, max_rounds: int = 1000,
            source: int = 0, stride: int = 1) -> RoundTable:
    """Runs `algo` once per forced round mode (profiled host loop, each round
    one graph launch) and tabulates the round times.  CC/SSSP trajectories
    are identical in every mode; delta PageRank's are compared by round index
    over the common prefix."""
    part = graph.partition_edge_balanced(num_memory) if num_memory > 1 else None
    init = (lambda c: c.init())
    kw = dict(max_rounds=max_rounds, source=source)
    with Context(graph, part, num_memory) as ctx:
        ctx.set_profiling(True)
        # the fixed rule first: before a forced pull builds the in-edge view
        # it only pushes, as the plain method does
        fixed = _profiled_run(ctx, algo, init, 1, **kw)
        logs = []
        for d, f in FORCED:
            logs.append(_profiled_run(ctx, algo, init, reps, direction=d, frontier_format=f, **kw))
    n = min(len(l) for l in logs)
    if algo != GRD_PR_DELTA:
        if any(len(l) != n for l in logs) or len(fixed) != n:
            raise RuntimeError(f"{name}: round counts differ between modes")
        for l in logs[1:]:
            for a, b in zip(logs[0], l):
                if a["frontier_in"] != b["frontier_in"] or a["frontier_edges_in"] != b["frontier_edges_in"]:
                    raise RuntimeError(f"{name}: trajectories differ between modes")
    n = min(n, len(fixed))
    idx = np.arange(0, n, max(1, stride))
    base = logs[0]
    x = log_features([base[i] for i in idx], graph.num_vertices, graph.num_edges)
    ms = np.array([[logs[m][i]["ms"][4] for m in range(NOUT)] for i in idx], dtype=np.float64)
    fm = np.array([fixed[i]["mode"] for i in idx], dtype=np.int32)
    tiny = np.array([base[i]["frontier_in"] <= TINY_ACTIVE and base[i]["frontier_edges_in"] <= TINY_EDGES
                     for i in idx], dtype=bool)
    return RoundTable(name, algo, x, ms, fm, tiny, {"rounds": n, "V": graph.num_vertices, "E": graph.num_edges})


def stack(tables: Iterable[RoundTable]) -> Tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Training arrays of the rounds the model decides (not the tiny ones)."""
    xs, ys, ms = [], [], []
    for t in tables:
        y, m = t.targets()
        keep = ~t.tiny
        xs.append(t.x[keep])
        ys.append(y[keep])
        ms.append(m[keep])
    return (np.ascontiguousarray(np.concatenate(xs), dtype=np.float32),
            np.ascontiguousarray(np.concatenate(ys), dtype=np.float32),
            np.ascontiguousarray(np.concatenate(ms), dtype=np.uint8))


# --------------------------------------------------------------- GPU calls --
def train(x: np.ndarray, y: np.ndarray, mask: np.ndarray, steps: int = 3000, lr: float = 3e-3,
          weight_decay: float = 1e-4, seed: int = 1, device: int = 0):
    """GPU training; returns (model, loss curve)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    cfg = _ffi.grd_policy_train_cfg(steps, lr, weight_decay, seed, device)
    m = _ffi.grd_policy_model()
    curve = np.zeros(steps, dtype=np.float32)
    _check(lib().grd_policy_train(_f32p(x), _f32p(y), mask.ctypes.data_as(_ffi.u8p), len(x), C.byref(cfg),
                                  C.byref(m), _f32p(curve)))
    return m, curve


def grad(model, x: np.ndarray, y: np.ndarray, mask: np.ndarray, device: int = 0) -> Tuple[float, np.ndarray]:
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.ascontiguousarray(y, dtype=np.float32)
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    loss = C.c_float()
    g = np.zeros(_ffi.GRD_POLICY_NPARAM, dtype=np.float32)
    _check(lib().grd_policy_grad(C.byref(model), _f32p(x), _f32p(y), mask.ctypes.data_as(_ffi.u8p), len(x), device,
                                 C.byref(loss), _f32p(g)))
    return float(loss.value), g


def predict(model, x: np.ndarray, allowed: int = ALL_MODES, device: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.zeros((len(x), NOUT), dtype=np.float32)
    ch = np.zeros(len(x), dtype=np.int32)
    _check(lib().grd_policy_predict(C.byref(model), _f32p(x), len(x), allowed, device, _f32p(out),
                                    ch.ctypes.data_as(C.POINTER(C.c_int32))))
    return out, ch


# -------------------------------------------------------------- evaluation --
MARGIN = 0.1  # = P_MARGIN of the device rule (log2 units)


def fixed_rule_mode(frontier, frontier_edges, num_slots: int, num_edges: int, dense_div: int = 8) -> np.ndarray:
    """The plain method's choice (fixed rule without the in-edge view)."""
    f = np.asarray(frontier, dtype=np.float64)
    fe = np.asarray(frontier_edges, dtype=np.float64)
    lst = (f * dense_div < num_slots) & (fe * dense_div < num_edges)
    return np.where(lst, 1, 0).astype(np.int32)


def decide(out: np.ndarray, fallback: np.ndarray, tiny: np.ndarray, allowed: int = ALL_MODES) -> np.ndarray:
    """The device rule: the fastest predicted allowed mode when it beats the
    fallback's prediction by more than MARGIN, else the fallback; push + list
    for tiny frontiers."""
    o = np.where([(allowed >> m) & 1 for m in range(NOUT)], out, np.inf)
    best = np.argmin(o, axis=1)
    rows = np.arange(len(out))
    ch = np.where(o[rows, best] + MARGIN < out[rows, fallback], best, fallback)
    return np.where(tiny, 1, ch).astype(np.int32)


def choose(model, t: RoundTable, allowed: int = ALL_MODES) -> np.ndarray:
    """The learned policy's mode for every round of a table, as the device
    applies it."""
    out, _ = predict(model, t.x, allowed)
    return decide(out, t.fixed_mode, t.tiny, allowed)


def table_totals(t: RoundTable, choice: np.ndarray) -> dict:
    """Measured time of the rounds under a per-round choice, next to the
    fixed rule, each forced mode and the per-round best."""
    ms = np.where(np.isfinite(t.ms), t.ms, np.inf)
    rows = np.arange(len(ms))
    out = {"chosen_ms": float(ms[rows, choice].sum()), "fixed_ms": float(ms[rows, t.fixed_mode].sum()),
           "best_ms": float(ms.min(axis=1).sum())}
    for m in range(NOUT):
        out[f"mode{m}_ms"] = float(ms[:, m].sum())
    return out
