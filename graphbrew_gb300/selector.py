"""Learned replacement for the algorithm-14 frozen selector.

The reference's deployable rule (``ShouldUseAllKernelLowReuseRule``,
``bench/include/graphbrew/reorder/reorder_adaptive.h:302-333``, applied by
``SelectAllKernelLowReuseRule``, ``:335-385``) picks the FastLeiden-Gorder8
recipe when

    supported kernel and reuse <= 2 and N >= 1000 and wsr <= 3.2 and
    ((cv <= 2.68 and (avg_degree <= 60 or wsr <= 0.82)) or cv > 8)

on Tier-0 sampled features, and otherwise its fallback arm (Rabbit Order, or
DBG "5" where Rabbit is not built).  Here every arm runs on the GPU: the
features come from ``gbgpu_tier0_features``, the working-set ratio is taken
against the GPU's L2 (the kernels run there), and a float32 MLP
(features -> 64 -> 64 -> 3) trained by the library's own forward/backward
kernels predicts the log10 end-to-end time (mapping + reuse x kernel) of
three arms: GraphBrew algorithm 12, DBG, and the original order.  The frozen
rule stays as the fallback (inputs outside the training range) and as the
judge the learned selector is evaluated against.

Command line (GPU):

    python -m graphbrew_gb300.selector collect --first 0 --count 2200 --out records.npz
    python -m graphbrew_gb300.selector train --data records.npz --out model.npz
    python -m graphbrew_gb300.selector evaluate --data records.npz --model model.npz
    python -m graphbrew_gb300.selector export --model model.npz --out model.gbsel

The exported file drives ``-o 14:_:_:_:learned-mlp:best-endtoend:<reuse>``
through the C ABI (``gbgpu_select_arm``) and ``gbconvert -M model.gbsel``.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

from . import DEFAULT_RECIPE, Context

ARMS = ("gb12", "dbg", "original")
KERNELS = ("pr", "bfs", "cc")
REUSES = (1, 2)
FAMILIES = ("rmat", "urand", "grid", "planted")
TIER0_KEYS = ("num_nodes", "num_edges", "avg_degree", "degree_cv", "internal_density", "hub_concentration",
              "packing_factor", "normalized_edge_span", "window_neighbor_overlap")
FEATURE_NAMES = ("log10_nodes", "log10_edges", "avg_degree", "degree_cv", "hub_concentration",
                 "normalized_edge_span", "window_neighbor_overlap", "property_wsr",
                 "kernel_pr", "kernel_bfs", "kernel_cc", "reuse")
TRAIN_SEEDS = range(0, 2000)
HELDOUT_SEEDS = range(2000, 2200)
GB300_L2_BYTES = 126 * 1024 * 1024


def modeled_property_bytes(kernel: str, n: int) -> int:
    """ModeledPropertyBytes (reorder_types.h:1226-1258) for PR, BFS and CC."""
    bitmap = (n + 7) // 8
    if kernel == "pr":
        return n * 2 * 4
    if kernel == "bfs":
        return n * 2 * 4 + 2 * bitmap
    if kernel == "cc":
        return n * 4 + bitmap
    raise ValueError(kernel)


def working_set_ratio(tier0, kernel: str, cache_bytes: int) -> float:
    return modeled_property_bytes(kernel, int(tier0[0])) / float(cache_bytes)


def frozen_rule(tier0, kernel: str, reuse: float, cache_bytes: int) -> str:
    """ShouldUseAllKernelLowReuseRule: algorithm 12 or the fallback arm (DBG)."""
    wsr = working_set_ratio(tier0, kernel, cache_bytes)
    n, avg, cv = tier0[0], tier0[2], tier0[3]
    use = (reuse <= 2.0 and n >= 1000 and wsr <= 3.2 and
           ((cv <= 2.68 and (avg <= 60.0 or wsr <= 0.82)) or cv > 8.0))
    return "gb12" if use else "dbg"


def feature_vector(tier0, kernel: str, reuse: float, cache_bytes: int) -> np.ndarray:
    return np.array([
        math.log10(tier0[0] + 1.0), math.log10(tier0[1] + 1.0), tier0[2], tier0[3], tier0[5], tier0[7],
        tier0[8], working_set_ratio(tier0, kernel, cache_bytes),
        float(kernel == "pr"), float(kernel == "bfs"), float(kernel == "cc"), float(reuse)], dtype=np.float64)


# ---------------------------------------------------------------------------
# Graphs and measurements (GPU)
# ---------------------------------------------------------------------------
def random_graph(seed: int, device="cuda", scale_range=(14, 20)):
    """Seeded synthetic graph of the training distribution: RMAT, uniform,
    grid or planted partition, 2^14 .. 2^20 vertices."""
    from . import graphgen as gg
    rng = np.random.default_rng(seed)
    fam = FAMILIES[seed % 4]
    scale = int(rng.integers(scale_range[0], scale_range[1] + 1))
    if fam == "rmat":
        rp, col = gg.rmat(scale, int(rng.integers(4, 33)), seed=seed, device=device)
    elif fam == "urand":
        rp, col = gg.uniform(scale, int(rng.integers(2, 17)), seed=seed, device=device)
    elif fam == "grid":
        rows = 1 << (scale // 2)
        rp, col = gg.grid(rows, (1 << scale) // rows, float(rng.uniform(0.0, 0.2)), seed=seed, device=device)
    else:
        rp, col, _ = gg.planted_partition(1 << scale, int(rng.integers(4, 65)), int(rng.integers(4, 33)),
                                          float(rng.uniform(0.02, 0.3)), seed=seed, device=device)
    return fam, scale, rp, col


def _kernel_ms(ctx: Context, rp, col, kernel: str, source: int) -> float:
    if kernel == "pr":
        return ctx.pagerank(rp, col, max_iters=20, epsilon=1e-4)[2]
    if kernel == "bfs":
        return ctx.bfs(rp, col, source)[1]
    return ctx.connected_components(rp, col)[1]


def measure_graph(ctx: Context, rp, col, recipe: str = DEFAULT_RECIPE, repeats: int = 2):
    """(tier0[9], map_ms[3], kernel_ms[3 arms][3 kernels]) for one graph."""
    import torch
    n = rp.numel() - 1
    deg = rp[1:] - rp[:-1]
    src0 = int(torch.argmax(deg).item()) if n else 0
    tier0 = ctx.tier0_features(rp, col)
    map_ms = np.zeros(3)
    # Algorithm 12: mapping + validation + relabel, the builder's lifecycle.
    ids, orp, ocol, st = ctx.map_and_relabel(rp, col, recipe)
    map_ms[0] = st["total_ms"]
    graphs = [(orp, ocol, int(ids[src0].item()))]
    # DBG: mapping + relabel.
    dids, dbg_ms = ctx.dbg_mapping(rp, col)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    drp, dcol, _ = ctx.relabel_by_mapping(rp, col, dids)
    e1.record()
    e1.synchronize()
    map_ms[1] = dbg_ms + e0.elapsed_time(e1)
    graphs.append((drp, dcol, int(dids[src0].item())))
    graphs.append((rp, col, src0))
    kms = np.zeros((3, 3))
    for a, (grp, gcol, src) in enumerate(graphs):
        for k, kern in enumerate(KERNELS):
            kms[a, k] = min(_kernel_ms(ctx, grp, gcol, kern, src) for _ in range(repeats))
    return np.asarray(tier0, dtype=np.float64), map_ms, kms


def collect(ctx: Context, seeds, log=None, checkpoint=None):
    """Measure every seed's graph; `checkpoint(records)` is called every 100
    graphs with what has been measured so far."""
    import torch
    recs = {"seed": [], "family": [], "scale": [], "tier0": [], "map_ms": [], "kernel_ms": []}
    l2 = np.int64(torch.cuda.get_device_properties(0).L2_cache_size)

    def snapshot():
        out = {k: np.asarray(v) for k, v in recs.items()}
        out["l2_bytes"] = l2
        return out
    t0 = time.time()
    for i, seed in enumerate(seeds):
        fam, scale, rp, col = random_graph(seed)
        tier0, map_ms, kms = measure_graph(ctx, rp, col)
        for k, v in (("seed", seed), ("family", FAMILIES.index(fam)), ("scale", scale), ("tier0", tier0),
                     ("map_ms", map_ms), ("kernel_ms", kms)):
            recs[k].append(v)
        if (i + 1) % 100 == 0:
            if log:
                log(f"{i + 1} graphs, {time.time() - t0:.0f} s")
            if checkpoint:
                checkpoint(snapshot())
    return snapshot()


# ---------------------------------------------------------------------------
# Dataset rows, model, evaluation
# ---------------------------------------------------------------------------
def end_to_end_ms(map_ms, kernel_ms, arm: int, kernel: int, reuse: int) -> float:
    return float(map_ms[arm] + reuse * kernel_ms[arm, kernel])


def dataset_rows(data, mask, cache_bytes=GB300_L2_BYTES):
    """X [rows x 12], T [rows x 3] = log10 end-to-end ms of each arm, and the
    (graph index, kernel, reuse) of every row."""
    X, T, meta = [], [], []
    for g in np.nonzero(mask)[0]:
        for k, kern in enumerate(KERNELS):
            for r in REUSES:
                X.append(feature_vector(data["tier0"][g], kern, r, cache_bytes))
                T.append([math.log10(max(1e-3, end_to_end_ms(data["map_ms"][g], data["kernel_ms"][g], a, k, r)))
                          for a in range(3)])
                meta.append((g, k, r))
    return np.array(X), np.array(T), meta


def init_params(ctx: Context, in_dim: int, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    h, o = 64, 3
    parts = [rng.normal(0, math.sqrt(2.0 / in_dim), (in_dim, h)), np.zeros(h),
             rng.normal(0, math.sqrt(2.0 / h), (h, h)), np.zeros(h),
             rng.normal(0, math.sqrt(1.0 / h), (h, o)), np.zeros(o)]
    p = np.concatenate([x.ravel() for x in parts]).astype(np.float32)
    assert p.size == ctx.mlp_param_count(in_dim)
    return p


class LearnedSelector:
    """Standardised features -> MLP -> arm with the smallest predicted time;
    the frozen rule where the features leave the training range."""

    def __init__(self, params, mean, std, lo, hi, cache_bytes=GB300_L2_BYTES):
        self.params, self.mean, self.std, self.lo, self.hi = params, mean, std, lo, hi
        self.cache_bytes = cache_bytes
        self.train_loss = None

    @classmethod
    def train(cls, ctx: Context, X, T, epochs=300, batch=128, lr=2e-3, seed=0, cache_bytes=GB300_L2_BYTES):
        mean, std = X.mean(0), X.std(0) + 1e-9
        params = init_params(ctx, X.shape[1], seed)
        params, loss = ctx.mlp_train(params, (X - mean) / std, T, epochs=epochs, batch=batch, lr=lr, seed=seed)
        sel = cls(params, mean, std, X.min(0), X.max(0), cache_bytes)
        sel.train_loss = loss
        return sel

    def in_range(self, x) -> bool:
        span = self.hi - self.lo
        return bool(np.all(x >= self.lo - 0.25 * span) and np.all(x <= self.hi + 0.25 * span))

    def predict(self, ctx: Context, X) -> np.ndarray:
        return ctx.mlp_forward(self.params, (np.atleast_2d(X) - self.mean) / self.std)

    def choose(self, ctx: Context, tier0, kernel: str, reuse: int):
        x = feature_vector(tier0, kernel, reuse, self.cache_bytes)
        if not self.in_range(x):
            return frozen_rule(tier0, kernel, reuse, self.cache_bytes), "frozen-rule-fallback"
        return ARMS[int(np.argmin(self.predict(ctx, x)[0]))], "learned-mlp"

    def save_binary(self, path):
        """The model file gbgpu_selector_model_load reads (include/gbgpu.h):
        magic, sizes, cache bytes, float32 parameters, float64 mean / std / lo / hi."""
        import struct
        in_dim = int(len(self.mean))
        with open(path, "wb") as f:
            f.write(b"GBSEL01\0")
            f.write(struct.pack("<4i", in_dim, 64, 3, 0))
            f.write(struct.pack("<q", int(self.cache_bytes)))
            f.write(np.ascontiguousarray(self.params, dtype="<f4").tobytes())
            for v in (self.mean, self.std, self.lo, self.hi):
                f.write(np.ascontiguousarray(v, dtype="<f8").tobytes())

    def save(self, path):
        np.savez(path, params=self.params, mean=self.mean, std=self.std, lo=self.lo, hi=self.hi,
                 cache_bytes=self.cache_bytes)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        return cls(d["params"], d["mean"], d["std"], d["lo"], d["hi"], int(d["cache_bytes"]))


def evaluate(ctx: Context, selector: LearnedSelector, data, mask) -> dict:
    """Realised end-to-end time of the learned and the frozen choices over
    every (graph, kernel, reuse) row of the masked graphs."""
    out = {"rows": 0, "learned_ms": 0.0, "frozen_ms": 0.0, "best_ms": 0.0, "fallbacks": 0,
           "learned_better": 0, "frozen_better": 0, "learned_arms": {a: 0 for a in ARMS}}
    for g in np.nonzero(mask)[0]:
        t0, mm, km = data["tier0"][g], data["map_ms"][g], data["kernel_ms"][g]
        for k, kern in enumerate(KERNELS):
            for r in REUSES:
                arm, how = selector.choose(ctx, t0, kern, r)
                farm = frozen_rule(t0, kern, r, selector.cache_bytes)
                lt = end_to_end_ms(mm, km, ARMS.index(arm), k, r)
                ft = end_to_end_ms(mm, km, ARMS.index(farm), k, r)
                out["rows"] += 1
                out["learned_ms"] += lt
                out["frozen_ms"] += ft
                out["best_ms"] += min(end_to_end_ms(mm, km, a, k, r) for a in range(3))
                out["fallbacks"] += how != "learned-mlp"
                out["learned_better"] += lt < ft
                out["frozen_better"] += ft < lt
                out["learned_arms"][arm] += 1
    out["learned_over_frozen"] = out["learned_ms"] / out["frozen_ms"] if out["frozen_ms"] else None
    return out


def split_masks(data):
    seeds = data["seed"]
    return (seeds >= TRAIN_SEEDS.start) & (seeds < TRAIN_SEEDS.stop), \
        (seeds >= HELDOUT_SEEDS.start) & (seeds < HELDOUT_SEEDS.stop)


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m graphbrew_gb300.selector")
    sub = ap.add_subparsers(dest="cmd", required=True)
    c = sub.add_parser("collect")
    c.add_argument("--first", type=int, default=0)
    c.add_argument("--count", type=int, default=2200)
    c.add_argument("--out", required=True)
    t = sub.add_parser("train")
    t.add_argument("--data", required=True)
    t.add_argument("--out", required=True)
    t.add_argument("--epochs", type=int, default=300)
    e = sub.add_parser("evaluate")
    e.add_argument("--data", required=True)
    e.add_argument("--model", required=True)
    x = sub.add_parser("export")
    x.add_argument("--model", required=True)
    x.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    if a.cmd == "export":
        LearnedSelector.load(a.model).save_binary(a.out)
        return
    ctx = Context(0)
    if a.cmd == "collect":
        data = collect(ctx, range(a.first, a.first + a.count), log=lambda m: print(m, file=sys.stderr),
                       checkpoint=lambda d: np.savez_compressed(a.out, **d))
        np.savez_compressed(a.out, **data)
        print(json.dumps({"graphs": int(len(data["seed"]))}))
    elif a.cmd == "train":
        data = dict(np.load(a.data))
        train_mask, _ = split_masks(data)
        cache = int(data.get("l2_bytes", GB300_L2_BYTES))
        X, T, _ = dataset_rows(data, train_mask, cache)
        sel = LearnedSelector.train(ctx, X, T, epochs=a.epochs, cache_bytes=cache)
        sel.save(a.out)
        print(json.dumps({"rows": int(len(X)), "train_loss": sel.train_loss}))
    else:
        data = dict(np.load(a.data))
        _, held = split_masks(data)
        sel = LearnedSelector.load(a.model)
        print(json.dumps(evaluate(ctx, sel, data, held)))


if __name__ == "__main__":
    main()
