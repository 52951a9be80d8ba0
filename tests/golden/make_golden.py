"""Regenerate the golden fixtures from the GraphBrew reference.

Run in a container where the GraphBrew sources are mounted and the reference
harness is built (``make -C oracle ref``):

    python tests/golden/make_golden.py

It writes
  * ``mapping_cases.npz``: small graphs (the reference's own test edge lists,
    graphs from the reference's own generator, seeded project graphs) with the
    reference's outputs on them: automatic resolution, cd_serial membership,
    orderCompose on that membership for several recipes, the end-to-end
    mapping, RelabelByMapping's CSR and org ids, and parallel-mode modularity
    samples;
  * ``parser_cases.json``: option strings with the reference's effective-config
    JSON or exception text;
  * ``manifest.json``: per-case scalars (fingerprints, counts, resolutions).

The fixtures are what the tests compare against where the reference itself
cannot run (the GPU machine).
"""
from __future__ import annotations

import json
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from graphbrew_gb300 import graphgen as gg  # noqa: E402

GRAPHBREW_SRC = os.environ.get("GRAPHBREW_SRC", "/root/reference")

SERIAL = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:"
          "sgmb4096:gordf5000:norefine:2:2")
PARALLEL = SERIAL.replace("cd_serial", "cd_parallel")
# orderCompose variants checked on the cd_serial membership.
COMPOSE_RECIPES = {
    "gorder8_f5000": SERIAL,
    "gorder8_f64": SERIAL.replace("gordf5000", "gordf64"),
    "gorder5_f16": SERIAL.replace("gw8", "gw5").replace("gordf5000", "gordf16"),
    "bfs_sizeasc": "leiden:compose:sg_none:comm_size_asc:intra_bfs:cd_serial:norefine:2:2",
    "bfs_degdesc": "leiden:compose:sg_none:comm_degree_desc:intra_bfs:cd_serial:norefine:2:2",
    "gorder8_identity": "leiden:compose:sg_none:comm_identity:intra_gorder:gw8:gordf32:cd_serial:norefine:2:2",
}


def el_graph(name):
    path = os.path.join(GRAPHBREW_SRC, "scripts", "test", "data", name + ".el")
    edges = [tuple(int(x) for x in line.split()[:2]) for line in open(path) if line.strip()]
    n = max(max(u, v) for u, v in edges) + 1
    rp, col = gg.from_edges(n, edges)
    return rp.numpy(), col.numpy()


def graphs():
    out = {}
    for name in ["tiny", "star", "path", "dangling", "disconnected", "isolated"]:
        out["el_" + name] = el_graph(name)
    out["gapbs_g10"] = po.ref_gapbs_graph(10)
    out["gapbs_u10"] = po.ref_gapbs_graph(10, 16, uniform=True)
    rp, col = gg.rmat(12, 16, seed=12)
    out["rmat12"] = (rp.numpy(), col.numpy())
    rp, col = gg.uniform(11, 8, seed=11)
    out["urand11"] = (rp.numpy(), col.numpy())
    rp, col = gg.grid(40, 50, seed=4)
    out["grid40x50"] = (rp.numpy(), col.numpy())
    rp, col, _ = gg.planted_partition(20000, 16, seed=5)
    out["planted20k"] = (rp.numpy(), col.numpy())
    return out


def parser_cases():
    corpus = json.load(open(os.path.join(GRAPHBREW_SRC, "bench", "tests", "data",
                                         "graphbrew_novelty_parser_cases.json")))["cases"]
    cases = [":".join(c["tokens"]) for c in corpus]
    cases += [SERIAL, PARALLEL, "leiden", "", "rabbit", "hubcluster",
              "leiden:compose:sg_super_rabbit:comm_identity:intra_gorder:gw8",
              "leiden:8:0.75:3:2:auto", "hrab:gvecsr:0.75", "leiden:1.5x", "leiden:compose:sgmb0",
              "quality", "dynamic_0.5", "leiden:dynamic", "10:2", "leiden:10:2:3", "gord12:gordf100",
              "leiden:0x1p-1", "leiden:compose:gw101", "sgres0.5", "hubx0.5", "leiden:final7",
              "leiden:depth3:sub:auto"]
    toks = ["leiden", "compose", "sg_none", "sg_super_rcm", "comm_size_desc", "comm_degree", "s2_identity",
            "intra_gorder", "intra_bfs", "intra_rcm", "gw8", "gw0", "gw5", "cd_parallel", "cd_serial",
            "sgmb4096", "sgmb1", "gordf5000", "gordf0", "norefine", "2", "3", "10", "0.7", "1e0", "auto", "0",
            "dynamic", "hrab", "tqr", "rabbit", "graphbrew", "final8", "depth2", "sub3", "subauto", "hubx",
            "hubx1.5", "gord", "gord8", "sgres2", "gamma0.1", "hsort", "rcm", "bfs_intra", "cd_full",
            "cd_louvain", "cd_lp", "cd_gve", "refine0", "refine3", "totalm", "halfm", "gvecsr", "quality",
            "verify", "capacity_runs", "capl2k4", "capllck16", "capv8", "intra_gorder_faithful",
            "refine_2swap", "merge", "lazyupdate", "bogus", "", "1.5", "-1", "0x10"]
    rng = random.Random(1)
    for _ in range(600):
        k = rng.randint(0, 8)
        first = rng.choice(["leiden", "leiden", "rabbit", "hubcluster", "compose", "", "quality", "cd_parallel"])
        cases.append(":".join([first] + [rng.choice(toks) for _ in range(k)]))
    out = []
    for c in cases:
        for ar in (0.6649478123456789, 1.0):
            rc, text = po.ref_effective_config(c, ar)
            out.append({"options": c, "auto_resolution": ar, "ok": rc == 0, "text": text})
    return out


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    arrays = {}
    manifest = {"serial_recipe": SERIAL, "parallel_recipe": PARALLEL, "compose_recipes": COMPOSE_RECIPES,
                "cases": {}}
    for name, (rp, col) in graphs().items():
        rp = np.ascontiguousarray(rp, dtype=np.int64)
        col = np.ascontiguousarray(col, dtype=np.int32)
        n = len(rp) - 1
        ref = po.load_reference()
        ar = ref.ref_auto_resolution(n, rp, col)
        memb, summary = po.ref_leiden(rp, col, SERIAL, ar, threads=1)
        full = po.ref_generate_mapping(rp, col, SERIAL, ar, threads=1)
        out_rp, out_col, org = po.ref_relabel(rp, col, full)
        arrays[f"{name}/row_ptr"] = rp
        arrays[f"{name}/col"] = col
        arrays[f"{name}/membership_serial"] = memb
        arrays[f"{name}/new_ids_serial"] = full
        arrays[f"{name}/relabel_row_ptr"] = out_rp
        arrays[f"{name}/relabel_col"] = out_col
        arrays[f"{name}/relabel_org_ids"] = org
        case = {"n": n, "nnz": int(len(col)), "auto_resolution": ar,
                "serial_summary": [int(x) for x in summary],
                "serial_fingerprint": po.fingerprint(full), "compose": {}}
        for key, recipe in COMPOSE_RECIPES.items():
            ids, gst = po.ref_compose(rp, col, memb, recipe, ar, threads=1)
            arrays[f"{name}/compose_{key}"] = ids
            case["compose"][key] = {"gorder_stats": [int(x) for x in gst], "fingerprint": po.fingerprint(ids)}
        qs = []
        for t in range(3):
            mpar, _ = po.ref_leiden(rp, col, PARALLEL, ar, threads=4)
            qs.append(ref.ref_modularity(n, rp, col, mpar, 1.0))
        case["parallel_modularity_samples"] = qs
        case["serial_modularity"] = ref.ref_modularity(n, rp, col, memb, 1.0)
        manifest["cases"][name] = case
        print(name, n, len(col), case["serial_fingerprint"], flush=True)
    # Gorder known-answer test of the reference's own suite (K4, window 5).
    k4 = [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]
    rp = np.array([0, 3, 6, 9, 12], dtype=np.int64)
    col = np.array([v for row in k4 for v in row], dtype=np.int32)
    lids = np.zeros(4, dtype=np.int32)
    po.load_reference().ref_gorder_kat(4, rp, col, 5, lids)
    manifest["gorder_kat_k4_w5"] = [int(x) for x in lids]
    np.savez_compressed(os.path.join(HERE, "mapping_cases.npz"), **arrays)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)
    with open(os.path.join(HERE, "parser_cases.json"), "w") as f:
        json.dump(parser_cases(), f, indent=0)


if __name__ == "__main__":
    main()
