"""The selector's arms timed on the reference's CPU path, beside the GPU path.

MEASUREMENT INFRASTRUCTURE (oracle side): it runs the oracle's CPU kernels,
which the product never does.  Algorithm 14 (bench/include/graphbrew/reorder/
reorder_adaptive.h:335-385, 517-715) picks, per graph and benchmark kernel,
the arm with the smallest map + reuse x kernel time.  On the reference's own
path every arm runs on the host: the algorithm-12 mapping (here the oracle's
OpenMP cd_parallel restatement, the same CPU stand-in as bench.py's reference
arm), DBG, relabelling, and GAPBS's OpenMP PageRank / BFS / CC
(oracle/gb_kernels_cpu.c).  This script times those arms on the host's cores
for the held-out graphs of the selector's dataset and reports, over every
(graph, kernel, reuse) row:

  * the reference CPU path with its frozen rule (cache = the host's LLC);
  * the best CPU arm per row;
  * the GPU path with the frozen rule and with the learned MLP (the GPU
    times are the dataset's own, measured by ``python -m
    graphbrew_gb300.selector collect``), and the best GPU arm.

    python oracle/selector_cpu_path.py --out selector_cpu_path.json [--count 200]

Needs a GPU (the graphs are regenerated on it and the learned model runs its
forward kernel there).
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import pyoracle as po  # noqa: E402
from graphbrew_gb300 import selector as S  # noqa: E402

DATA = os.path.join(ROOT, "graphbrew_gb300", "data")


def host_llc_bytes(default=32 << 20):
    """Largest cache of cpu0 from sysfs (the reference's rule measures its
    working set against the machine's last-level cache)."""
    best = 0
    base = "/sys/devices/system/cpu/cpu0/cache"
    try:
        for d in os.listdir(base):
            p = os.path.join(base, d, "size")
            if os.path.exists(p):
                s = open(p).read().strip()
                mult = {"K": 1 << 10, "M": 1 << 20, "G": 1 << 30}.get(s[-1], 1)
                best = max(best, int(s[:-1] if s[-1] in "KMG" else s) * mult)
    except OSError:
        pass
    return best or default


def cpu_arms(rp, col, threads, repeats=2):
    """(map_ms[3], kernel_ms[3 arms][3 kernels]) on the host cores."""
    n = len(rp) - 1
    src0 = int(np.argmax(np.diff(rp))) if n else 0
    map_ms = np.zeros(3)
    t0 = time.perf_counter()
    res = po.auto_resolution(rp, col)
    ids, _, _, _ = po.map_graph(rp, col, res, parallel=True, threads=threads)
    t1 = time.perf_counter()
    grp, gcol = po.relabel(rp, col, ids, threads=threads)
    t2 = time.perf_counter()
    map_ms[0] = (t2 - t0) * 1e3
    dids, dms = po.dbg_cpu(rp, col, threads=threads)
    t3 = time.perf_counter()
    drp, dcol = po.relabel(rp, col, dids, threads=threads)
    map_ms[1] = dms + (time.perf_counter() - t3) * 1e3
    graphs = [(grp, gcol, int(ids[src0])), (drp, dcol, int(dids[src0])), (rp, col, src0)]
    kms = np.zeros((3, 3))
    for a, (g_rp, g_col, src) in enumerate(graphs):
        kms[a, 0] = min(po.pagerank_cpu(g_rp, g_col, 20, 1e-4, threads)[2] for _ in range(repeats))
        kms[a, 1] = min(po.bfs_cpu(g_rp, g_col, src, threads)[1] for _ in range(repeats))
        kms[a, 2] = min(po.cc_cpu(g_rp, g_col, threads)[1] for _ in range(repeats))
    return map_ms, kms, (t1 - t0) * 1e3


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--records", default=os.path.join(DATA, "selector_records.npz"))
    ap.add_argument("--model", default=os.path.join(DATA, "selector_mlp.npz"))
    ap.add_argument("--count", type=int, default=200)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    po.build()
    threads = a.threads or (os.cpu_count() or 1)
    data = dict(np.load(a.records))
    _, held = S.split_masks(data)
    idx = np.nonzero(held)[0][: a.count]
    gpu_cache = int(data.get("l2_bytes", S.GB300_L2_BYTES))
    cpu_cache = host_llc_bytes()
    ctx = S.Context(0)
    sel = S.LearnedSelector.load(a.model)
    tot = {k: 0.0 for k in ("cpu_frozen", "cpu_best", "gpu_frozen", "gpu_learned", "gpu_best")}
    rows, per_graph, t_start = 0, [], time.time()
    for gi in idx:
        seed = int(data["seed"][gi])
        fam, scale, rp_d, col_d = S.random_graph(seed)
        rp, col = rp_d.cpu().numpy(), col_d.cpu().numpy()
        cmap, ckm, leiden_ms = cpu_arms(rp, col, threads)
        t0, gmap, gkm = data["tier0"][gi], data["map_ms"][gi], data["kernel_ms"][gi]
        for k, kern in enumerate(S.KERNELS):
            for r in S.REUSES:
                cpu = [S.end_to_end_ms(cmap, ckm, arm, k, r) for arm in range(3)]
                gpu = [S.end_to_end_ms(gmap, gkm, arm, k, r) for arm in range(3)]
                tot["cpu_frozen"] += cpu[S.ARMS.index(S.frozen_rule(t0, kern, r, cpu_cache))]
                tot["cpu_best"] += min(cpu)
                tot["gpu_frozen"] += gpu[S.ARMS.index(S.frozen_rule(t0, kern, r, gpu_cache))]
                tot["gpu_learned"] += gpu[S.ARMS.index(sel.choose(ctx, t0, kern, r)[0])]
                tot["gpu_best"] += min(gpu)
                rows += 1
        per_graph.append({"seed": seed, "family": fam, "scale": scale, "vertices": len(rp) - 1,
                          "entries": len(col), "cpu_map_ms": cmap.round(3).tolist(),
                          "cpu_kernel_ms": ckm.round(3).tolist(), "gpu_map_ms": np.round(gmap, 3).tolist()})
        print(f"{len(per_graph)} graphs, {time.time() - t_start:.0f} s", file=sys.stderr, flush=True)
    out = {"rows": rows, "graphs": len(per_graph), "host_threads": threads, "host_llc_bytes": cpu_cache,
           "gpu_l2_bytes": gpu_cache, "totals_ms": tot,
           "ratios": {"cpu_frozen_over_gpu_learned": tot["cpu_frozen"] / tot["gpu_learned"],
                      "gpu_frozen_over_gpu_learned": tot["gpu_frozen"] / tot["gpu_learned"],
                      "cpu_best_over_gpu_learned": tot["cpu_best"] / tot["gpu_learned"]},
           "per_graph": per_graph}
    with open(a.out, "w") as f:
        json.dump(out, f)
    print(json.dumps({k: v for k, v in out.items() if k != "per_graph"}))


if __name__ == "__main__":
    main()
