"""Golden outputs of orderCompose with a super-graph order, from the reference.

Run where the reference harness is built (``make -C oracle ref``):

    python tests/golden/make_golden_super.py

sg_super_rcm (bench/include/graphbrew/reorder/reorder_graphbrew.h:4990-5090,
5726-5871), sg_super_rabbit (:5495-5715) and sg_hilbert (:6421-6459) give
stage1Perm, which the community
order keeps for equal keys (:6460-6462).  The reference builds the
super-graph in per-thread std::unordered_maps, so only its one-thread result
is reproducible; the harness runs it with one OpenMP thread.
``super_cases.npz`` holds the forward map for

    leiden:compose:<super order>:<community order>:intra_bfs:cd_serial:norefine:2:2

on every graph of ``mapping_cases.npz`` (cd_serial membership) and the
seeded generator graphs of ``make_golden_sorted.py`` (membership stored),
with size-desc and identity community orders.
``super_pins.json`` holds the SHA-256 of the forward map (int32,
little-endian) with both community orders on RMAT scale 18 and 19 graphs
(``graphgen.rmat(s, 16, seed)``, membership from the oracle's serial Leiden)
and on a 4096 x 4096 grid whose largest community's pair weight reaches 2^24.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from graphbrew_gb300 import graphgen as gg  # noqa: E402
from make_golden_sorted import generator_graphs  # noqa: E402

SUPER = {"super-rcm": "sg_super_rcm", "super-rabbit": "sg_super_rabbit", "hilbert": "sg_hilbert"}
COMM = {"size-desc": "comm_size_desc", "identity": "comm_identity"}
BIG = {"rmat18_s11": (18, 11), "rmat19_s12": (19, 12), "grid4096_bands": None}


def recipe(sup, comm="size-desc"):
    return f"leiden:compose:{SUPER[sup]}:{COMM[comm]}:intra_bfs:cd_serial:norefine:2:2"


def big_graph(name):
    if BIG[name] is None:
        # A 4096 x 4096 grid: rows 0..2047 in community 0 (about 2^25
        # entries inside, so its pair weight stops at 2^24 and the float
        # degree sums round in the reference's order), the other rows in
        # bands of 37 rows.
        rp, col = gg.grid(4096, 4096, 0.0, seed=1)
        rp, col = rp.numpy(), col.numpy()
        row = np.arange(len(rp) - 1) // 4096
        return rp, col, np.where(row < 2048, 0, 1 + (row - 2048) // 37).astype(np.uint32)
    scale, seed = BIG[name]
    rp, col = gg.rmat(scale, 16, seed=seed)
    rp, col = rp.numpy(), col.numpy()
    memb, _ = po.leiden(rp, col, po.auto_resolution(rp, col))
    return rp, col, memb


def digest(ids):
    return hashlib.sha256(np.ascontiguousarray(ids, dtype="<i4").tobytes()).hexdigest()


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    cases = np.load(os.path.join(HERE, "mapping_cases.npz"))
    names = sorted({k.split("/")[0] for k in cases.files})
    graphs = [(nm, cases[f"{nm}/row_ptr"], cases[f"{nm}/col"], cases[f"{nm}/membership_serial"]) for nm in names]
    out = {}
    for nm, (rp, col) in generator_graphs().items():
        memb, _ = po.leiden(rp, col, po.auto_resolution(rp, col))
        out[f"{nm}/membership"] = memb
        graphs.append((nm, rp, col, memb))
    for nm, rp, col, memb in graphs:
        for sup in SUPER:
            for comm in COMM:
                out[f"{nm}/{sup}/{comm}"] = po.ref_compose(rp, col, memb, recipe(sup, comm), 1.0, threads=1)[0]
    np.savez_compressed(os.path.join(HERE, "super_cases.npz"), **out)
    pins = {}
    for nm in BIG:
        rp, col, memb = big_graph(nm)
        pins[nm] = {sup: {comm: digest(po.ref_compose(rp, col, memb, recipe(sup, comm), 1.0, threads=1)[0])
                          for comm in COMM} for sup in SUPER}
    with open(os.path.join(HERE, "super_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)


if __name__ == "__main__":
    main()
