"""Benchmark: algorithm-12 mapping construction (FastLeiden-Gorder8) on one GB300.

Workload: GAPBS's own RMAT graph for ``converter -g 22 -s`` (scale 22, degree
16, a/b/c = 0.57/0.19/0.19, seed kRandSeed; generator.h:101-164 and the
builder's squish), rebuilt here by the library's GAPBS generator: 4,194,302
vertices, 128,311,450 directed int32 entries.  Recipe
``-o 12:leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_parallel:
sgmb4096:gordf5000:norefine:2:2``.  One step = the builder's mapping
lifecycle: GraphBrew core (Leiden + COMPOSE) + permutation validation + CSR
relabel ("Reorder End-to-End Time", builder.h:881-892).

metric  Medges/s = directed CSR entries / end-to-end mapping seconds.
value   device-resident graph, CUDA events on the library's stream.
e2e     same metric through the public C ABI with host (pinned) buffers:
        the CSR copied in and the permutation plus relabelled CSR copied out
        inside every step.  ``e2e_pageable`` is the same with pageable buffers
        (what a GAPBS caller's pvector memory is).
parity  outside the timed region: the timed permutation's "Mapping
        Fingerprint" and the relabelled CSR's checksums against the
        reference's values on the same graph (tests/golden/gapbs_pins.json).

``--impl reference`` times the CPU restatement of the reference's path (the
oracle, OpenMP on every host core) on the same graph; the reference's own
sources are not present on the GPU host, so it cannot be compiled there.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RECIPE = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_parallel:"
          "sgmb4096:gordf5000:norefine:2:2")
METRIC = "GPU reorder Medges/s vs host CPU; map+kernel time, learned vs frozen rule"
SCALE = 22
EDGE_FACTOR = 16
CPU_BASELINE_RUNS = 5
# Local-moving DRAM traffic per mapping of GAPBS -g 22 (ncu, warm L2):
# 6.445 GB read + 3.341 GB written by the round kernels.
LOCAL_MOVE_DRAM_BYTES_G22 = 9.787e9
PINS_PATH = os.path.join(ROOT, "tests", "golden", "gapbs_pins.json")


def load_pins(scale):
    """The reference's answers on GAPBS -g <scale> (None if not pinned)."""
    try:
        with open(PINS_PATH) as f:
            return json.load(f)["rmat"].get(str(scale))
    except (OSError, KeyError, ValueError):
        return None


def workload_name(scale):
    return f"gapbs_rmat{scale}_ef{EDGE_FACTOR}_fastleiden_gorder8"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--scale", type=int, default=SCALE)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--engine", default="auto", choices=["auto", "exact", "async"],
                    help="local-moving engine for cd_parallel: the library default (serial-order at every "
                         "size), serial-order, or asynchronous")
    a = ap.parse_args()
    if a.engine == "exact":
        os.environ["GBGPU_EXACT_MAX_VERTICES"] = str(1 << 62)
    elif a.engine == "async":
        os.environ["GBGPU_EXACT_MAX_VERTICES"] = "0"
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def host_cores():
    return os.cpu_count() or 1


# ---------------------------------------------------------------------------
# CPU legs (oracle restatement of the reference path)
# ---------------------------------------------------------------------------
def cpu_mapping_seconds(rp, col, threads):
    """One end-to-end mapping on the host cores: Leiden (cd_parallel, OpenMP),
    COMPOSE, validation, relabel.  Returns (seconds, new_ids)."""
    import pyoracle as po
    ar = po.auto_resolution(rp, col)
    t0 = time.perf_counter()
    ids, _, _, _ = po.map_graph(rp, col, ar, parallel=True, threads=threads)
    rc = po.validate_permutation(ids)
    po.relabel(rp, col, ids, threads=threads)
    t1 = time.perf_counter()
    assert rc == 0
    return t1 - t0, ids


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as po
    po.build()
    threads = host_cores()
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    # The same graph as the GPU arm, at the requested scale: every step is one
    # full mapping + validation + relabel of it.
    rp, col = po.gapbs_graph(args.scale, EDGE_FACTOR)
    nnz = len(col)
    for _ in range(args.warmup):
        cpu_mapping_seconds(rp, col, threads)
    times = [cpu_mapping_seconds(rp, col, threads)[0] for _ in range(args.steps)]
    total = sum(times)
    value = nnz * len(times) / total / 1e6
    sample = (f"GAPBS -g {args.scale} graph ({nnz} directed entries), one full mapping+validation+relabel per "
              f"step, {len(times)} steps, median {statistics.median(times):.2f} s")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Medges/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / len(times) * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic (GAPBS RMAT generator, kRandSeed)",
        "config": {"workload": workload_name(args.scale), "recipe": "12:" + RECIPE,
                   "scale": args.scale, "edge_factor": EDGE_FACTOR, "vertices": len(rp) - 1,
                   "directed_entries": nnz},
        "cpu_baseline": {"value": value, "unit": "Medges/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "Medges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def relabel_bytes(n, nnz):
    # read col + gather new_ids + write out_col (4 B each per entry),
    # inverse map and row offsets (per vertex: read old offsets 16 B,
    # inverse 4 B, write new offsets 8 B, scan read+write 16 B).
    return 12 * nnz + 44 * n


def local_move_bytes(n, nnz):
    # One local-moving sweep: col 4 B + neighbour community 4 B + affected-flag
    # write 1 B per entry; offsets 8 B, vertex state 4 + 8 + 8 + 1 B per vertex.
    return 9 * nnz + 29 * n + 8


def aggregate_bytes(n, nnz):
    # col + community gather per entry, inter-community keys written and
    # sorted (upper bound: every entry), weights / remap / renumber per vertex.
    return 8 * nnz + 12 * nnz + 24 * n


def compose_bytes(n, nnz):
    # grouping and placement ~48 B per vertex, BFS / Gorder gathers 12 B per entry.
    return 48 * n + 12 * nnz


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    import numpy as np
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from graphbrew_gb300 import build as gbuild
    gbuild.build()
    import graphbrew_gb300 as gb
    from graphbrew_gb300 import graphgen as gg

    # Every rank maps its own replica (the path does not shard; no collective).
    rp, col = gg.gapbs(args.scale, EDGE_FACTOR, device="cuda")
    n, nnz = rp.numel() - 1, col.numel()
    ctx = gb.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

    def step():
        ids, orp, ocol, st = ctx.map_and_relabel(rp, col, RECIPE)
        return ids, orp, ocol, st

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    stats = []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        ids, orp, ocol, st = step()
        stats.append(st)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if world > 1:
        dist.barrier()
    ms_total = ev0.elapsed_time(ev1)
    if world > 1:
        t = torch.tensor([ms_total], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_total = float(t.item())
    ms_step = ms_total / args.steps
    value = nnz * world * args.steps / (ms_total / 1e3) / 1e6

    # Correctness of what was timed (outside the timed region): a valid
    # permutation, and -- where the reference's answer on this graph is
    # pinned -- the same permutation and relabelled CSR as the reference's.
    assert ctx.validate_permutation(ids) == 0
    pin = load_pins(args.scale)
    fp = gb.mapping_fingerprint(ids)
    parity = {"fingerprint": fp, "relabel_row_ptr": gg.checksum(orp), "relabel_col": gg.checksum(ocol)}
    if pin is not None:
        same = (fp == pin["fingerprint_cd_serial"] and parity["relabel_row_ptr"] == pin["relabel_row_ptr"]
                and parity["relabel_col"] == pin["relabel_col"])
        parity.update({"reference_fingerprint": pin["fingerprint_cd_serial"],
                       "graph_matches_reference": gg.checksum(rp) == pin["row_ptr"] and gg.checksum(col) == pin["col"],
                       "result": "bit-exact" if same else "mismatch",
                       "against": "reference cd_serial mapping + RelabelByMapping on the same graph"})
    else:
        parity["result"] = "unpinned at this scale"

    def host_e2e(pinned):
        """Median-free whole-step timing through the C ABI with host buffers."""
        if pinned:
            h_rp, h_col = rp.cpu().pin_memory(), col.cpu().pin_memory()
            h_ids = torch.empty(n, dtype=torch.int32).pin_memory()
            h_orp = torch.empty(n + 1, dtype=torch.int64).pin_memory()
            h_ocol = torch.empty(nnz, dtype=torch.int32).pin_memory()
        else:
            h_rp, h_col = rp.cpu(), col.cpu()
            h_ids = torch.empty(n, dtype=torch.int32)
            h_orp = torch.empty(n + 1, dtype=torch.int64)
            h_ocol = torch.empty(nnz, dtype=torch.int32)
        lib = gb.library()
        opts = RECIPE.encode()

        def host_step():
            s = gb.GbgpuStats()
            rc = lib.gbgpu_map_and_relabel(ctx.handle, h_rp.data_ptr(), h_col.data_ptr(), n, nnz, opts, -1.0,
                                           h_ids.data_ptr(), h_orp.data_ptr(), h_ocol.data_ptr(),
                                           gb.C.byref(s), 0)
            assert rc == 0, lib.gbgpu_last_error(ctx.handle)
            return s

        for _ in range(max(3, args.warmup)):
            host_step()
        t0 = time.perf_counter()
        host_stats, marks = [], [t0]
        for _ in range(args.steps):
            host_stats.append(host_step())
            marks.append(time.perf_counter())
        t1 = marks[-1]
        assert gb.mapping_fingerprint(h_ids.numpy()) == fp
        e2e_s = (t1 - t0) / args.steps
        return {"value": nnz * world / e2e_s / 1e6, "unit": "Medges/s",
                "h2d_bytes_per_step": 8 * (n + 1) + 4 * nnz,
                "d2h_bytes_per_step": 4 * n + 8 * (n + 1) + 4 * nnz,
                "ms_per_step": e2e_s * 1e3, "host_buffers": "pinned" if pinned else "pageable",
                "step_wall_ms": [round((b - a) * 1e3, 2) for a, b in zip(marks, marks[1:])],
                "step_device_ms": [round(float(x.total_ms), 2) for x in host_stats],
                "step_h2d_ms": [round(float(x.h2d_ms), 2) for x in host_stats],
                "step_relabel_ms": [round(float(x.relabel_ms), 2) for x in host_stats],
                "step_local_move_ms": [round(float(x.local_move_ms), 2) for x in host_stats],
                "h2d_ms": float(np.median([x.h2d_ms for x in host_stats])),
                "d2h_ms": float(np.median([x.d2h_ms for x in host_stats])),
                "call_device_ms": float(np.median([x.total_ms for x in host_stats])),
                "call_stages_ms": {k: float(np.median([getattr(x, k) for x in host_stats]))
                                   for k in ("local_move_ms", "aggregate_ms", "compose_ms", "relabel_ms")}}

    # End to end through the C ABI with host buffers (pinned, then pageable).
    e2e = e2e_pageable = None
    if not args.no_e2e:
        e2e = host_e2e(True)
        e2e_pageable = host_e2e(False)

    # Stage split and the roofline of the dominant stage.  The serial-order
    # local moving is a chain of short dependent rounds (latency-bound by
    # construction); the streaming stages are reported beside it.
    def avg(key):
        return sum(s[key] for s in stats) / len(stats)
    stage_ms = {k: avg(k) for k in ("leiden_ms", "local_move_ms", "aggregate_ms", "compose_ms", "intra_ms",
                                    "validate_ms", "relabel_ms", "total_ms")}
    iters = avg("iterations")
    peak, peak_kind = load_peaks()
    stage_bytes = {"local_move": local_move_bytes(n, nnz) * iters, "aggregate": aggregate_bytes(n, nnz),
                   "compose": compose_bytes(n, nnz), "relabel": relabel_bytes(n, nnz)}
    stages = {}
    for k, b in stage_bytes.items():
        ms = stage_ms[k + "_ms"]
        ach = b / (ms / 1e3) / 1e9 if ms > 0 else 0.0
        stages[k] = {"ms": ms, "algorithmic_bytes": b, "achieved_gbs": ach, "frac": ach / peak}
    dom = max(stages, key=lambda k: stages[k]["ms"])
    # DRAM bytes (read + write) of the stage's kernels per mapping, from one
    # ncu capture of this workload (profiles/launches_dram_gapbs22.md); only
    # the GAPBS -g 22 workload was captured.
    traffic = extra = None
    if dom == "local_move" and args.scale == 22:
        traffic = LOCAL_MOVE_DRAM_BYTES_G22
        extra = {"per": "mapping: the stage's kernel launches summed, like achieved",
                 "ratio_to_algorithmic": LOCAL_MOVE_DRAM_BYTES_G22 / stage_bytes[dom],
                 "source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, warm L2, one full-size capture"}
    roofline = {"bound": "hbm", "kernel": dom + " (stage: its kernels' launches per mapping)",
                "achieved": stages[dom]["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": stages[dom]["frac"], "peak_source": peak_kind, "traffic": traffic, "traffic_detail": extra,
                "algorithmic_bytes_per_launch": stage_bytes[dom], "stages": stages,
                "local_move_rounds": avg("local_move_rounds"),
                "note": "serial-order local moving is bound by the latency of its dependent rounds, not by HBM"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as po
        po.build()
        threads = host_cores()
        h_rp, h_col = rp.cpu().numpy(), col.cpu().numpy()
        secs = sorted(cpu_mapping_seconds(h_rp, h_col, threads)[0] for _ in range(CPU_BASELINE_RUNS))
        med = statistics.median(secs)
        cpu = {"value": nnz / med / 1e6, "unit": "Medges/s", "cores": threads, "kind": "port",
               "sample": f"median of {CPU_BASELINE_RUNS} full mappings+validation+relabel of the same GAPBS "
                         f"-g {args.scale} graph (OpenMP cd_parallel restatement; runs "
                         + ", ".join(f"{x:.2f}" for x in secs) + " s)"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Medges/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32",
            "data": "synthetic (GAPBS RMAT generator, kRandSeed; edge list on the host, squished on the device)",
            "config": {"workload": workload_name(args.scale),
                       "recipe": "12:" + RECIPE, "scale": args.scale, "edge_factor": EDGE_FACTOR,
                       "vertices": n, "directed_entries": nnz, "parallelism": f"replicas{world}",
                       "local_move_engine": args.engine,
                       "l2": "inputs larger than L2 (CSR 0.55 GB vs 129 MB L2)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "e2e_pageable": e2e_pageable,
            "parity": parity,
            "clocks": clocks,
            "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
            "stages_ms": stage_ms,
            "mapping": {"passes": stats[-1]["passes"], "iterations": stats[-1]["iterations"],
                        "communities": stats[-1]["communities"],
                        "largest_community": stats[-1]["largest_community"],
                        "bfs_levels": stats[-1]["bfs_levels"], "isolated": stats[-1]["isolated"],
                        "gorder_communities": stats[-1]["gorder_communities"],
                        "fallback_communities": stats[-1]["fallback_communities"]},
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
