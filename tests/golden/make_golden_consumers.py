"""Golden outputs of the selector's inputs, from the GraphBrew reference.

Run where the reference harness is built (``make -C oracle ref``):

    python tests/golden/make_golden_consumers.py

It writes ``consumer_cases.npz`` and ``consumer_manifest.json`` with, per graph,
GenerateDBGMapping's forward map (bench/include/graphbrew/reorder/
reorder_hub.h:267-342) and ComputeTier0SampledGraphFeatures' nine values
(bench/include/graphbrew/reorder/reorder_types.h:6066-6186), both computed by
the reference code itself:

  * every graph of ``mapping_cases.npz`` (full DBG maps stored);
  * seeded generator graphs large enough that the Tier-0 sample exceeds its
    1024-vertex floor (only the generator arguments, the DBG map's FNV-1a
    fingerprint and the features are stored; the tests regenerate the graph).
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from graphbrew_gb300 import graphgen as gg  # noqa: E402

# (name, generator, kwargs): regenerated identically by graphgen in the tests.
GENERATED = [
    ("rmat21_e8", "rmat", {"scale": 21, "edge_factor": 8, "seed": 3}),
    ("urand20_e8", "uniform", {"scale": 20, "edge_factor": 8, "seed": 4}),
    ("rmat18_e16", "rmat", {"scale": 18, "edge_factor": 16, "seed": 5}),
    ("grid1100", "grid", {"rows": 1100, "cols": 1100, "drop": 0.1, "seed": 6}),
]


def generate(kind, kw):
    if kind == "rmat":
        return gg.rmat(kw["scale"], kw["edge_factor"], seed=kw["seed"])
    if kind == "uniform":
        return gg.uniform(kw["scale"], kw["edge_factor"], seed=kw["seed"])
    if kind == "grid":
        return gg.grid(kw["rows"], kw["cols"], kw["drop"], seed=kw["seed"])
    raise ValueError(kind)


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    cases = np.load(os.path.join(HERE, "mapping_cases.npz"))
    names = sorted({k.split("/")[0] for k in cases.files})
    arrays, manifest = {}, {"small": {}, "generated": {}}
    for name in names:
        rp, col = cases[f"{name}/row_ptr"], cases[f"{name}/col"]
        arrays[f"{name}/dbg_ids"] = po.ref_dbg_mapping(rp, col)
        manifest["small"][name] = {"tier0": list(po.ref_tier0_features(rp, col).values())}
    for name, kind, kw in GENERATED:
        rp, col = generate(kind, kw)
        rp, col = rp.numpy(), col.numpy()
        ids = po.ref_dbg_mapping(rp, col)
        manifest["generated"][name] = {
            "kind": kind, "kwargs": kw, "n": int(len(rp) - 1), "nnz": int(len(col)),
            "dbg_fingerprint": po.fingerprint(ids),
            "tier0": list(po.ref_tier0_features(rp, col).values()),
        }
        print(name, len(rp) - 1, len(col))
    np.savez_compressed(os.path.join(HERE, "consumer_cases.npz"), **arrays)
    with open(os.path.join(HERE, "consumer_manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)


if __name__ == "__main__":
    main()
