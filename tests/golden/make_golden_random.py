"""Golden outputs of orderCompose with intra_random, from the reference.

Run where the reference harness is built (``make -C oracle ref``):

    python tests/golden/make_golden_random.py

intra_random (bench/include/graphbrew/reorder/reorder_graphbrew.h:6825-6845)
shuffles each community with a std::mt19937 seeded 0xDEADBEEF ^ community id
through std::uniform_int_distribution.  ``random_cases.npz`` holds the
reference's forward map for

    leiden:compose:sg_none:<community order>:intra_random:cd_serial:norefine:2:2

on every graph of ``mapping_cases.npz`` (its cd_serial membership) and on the
seeded generator graphs of ``make_golden_sorted.py`` (membership stored), with
size-desc and degree-desc community orders.  ``random_pins.json`` holds the
SHA-256 of the reference's forward map (int32, little-endian) on two
synthetic cases whose communities are large enough for the distribution to
reject draws (about size^2 / 2^34 of them per community): a 512 x 512 grid
with every vertex in community 0, and a 1024 x 1024 grid in three
communities 5, 6, 7 (vertex v in 5 + v mod 3).
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

COMM = {"size-desc": "comm_size_desc", "degree-desc": "comm_degree_desc"}


def recipe(comm="size-desc"):
    return f"leiden:compose:sg_none:{COMM[comm]}:intra_random:cd_serial:norefine:2:2"


def big_cases():
    """(name, row_ptr, col, membership) of the pinned synthetic cases."""
    rp, col = gg.grid(512, 512, 0.0, seed=1)
    yield "grid512_one", rp.numpy(), col.numpy(), np.zeros(512 * 512, dtype=np.uint32)
    rp, col = gg.grid(1024, 1024, 0.0, seed=1)
    n = 1024 * 1024
    yield "grid1024_three", rp.numpy(), col.numpy(), (np.arange(n) % 3 + 5).astype(np.uint32)


def digest(ids):
    return hashlib.sha256(np.ascontiguousarray(ids, dtype="<i4").tobytes()).hexdigest()


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    cases = np.load(os.path.join(HERE, "mapping_cases.npz"))
    names = sorted({k.split("/")[0] for k in cases.files})
    out = {}
    for name in names:
        rp, col = cases[f"{name}/row_ptr"], cases[f"{name}/col"]
        memb = cases[f"{name}/membership_serial"]
        for comm in COMM:
            out[f"{name}/{comm}"] = po.ref_compose(rp, col, memb, recipe(comm), 1.0)[0]
    for name, (rp, col) in generator_graphs().items():
        memb, _ = po.leiden(rp, col, po.auto_resolution(rp, col))
        out[f"{name}/membership"] = memb
        for comm in COMM:
            out[f"{name}/{comm}"] = po.ref_compose(rp, col, memb, recipe(comm), 1.0)[0]
    np.savez_compressed(os.path.join(HERE, "random_cases.npz"), **out)
    pins = {name: {"vertices": len(rp) - 1, "sha256": digest(po.ref_compose(rp, col, memb, recipe(), 1.0)[0])}
            for name, rp, col, memb in big_cases()}
    with open(os.path.join(HERE, "random_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)


if __name__ == "__main__":
    main()
