"""Golden outputs of GraphBrew-Leiden with refinement, from the reference.

Run where the reference harness is built (``make -C oracle ref``):

    python tests/golden/make_golden_refine.py

For every graph of ``mapping_cases.npz`` and three seeded generator graphs
(regenerated by the tests, not stored), ``refine_cases.npz`` holds, for

    leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:sgmb4096:gordf5000:refine0:2:2

the reference's auto resolution, final membership (runGraphBrew with the
refinement phase of bench/include/graphbrew/reorder/reorder_graphbrew.h:7330-7392
in pass 0) and forward map (generateGraphBrewMapping).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from graphbrew_gb300 import graphgen as gg  # noqa: E402

REFINE = "leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:sgmb4096:gordf5000:refine0:2:2"


def generator_graphs():
    gen = {"rmat13_s21": gg.rmat(13, 16, seed=21), "rmat15_s22": gg.rmat(15, 12, seed=22),
           "grid80x90": gg.grid(80, 90, 0.1, seed=23)}
    return {k: (rp.numpy(), col.numpy()) for k, (rp, col) in gen.items()}


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    cases = np.load(os.path.join(HERE, "mapping_cases.npz"))
    graphs = {n: (cases[f"{n}/row_ptr"], cases[f"{n}/col"]) for n in sorted({k.split("/")[0] for k in cases.files})}
    graphs.update(generator_graphs())
    out = {}
    for name, (rp, col) in graphs.items():
        ar = po.auto_resolution(rp, col)   # pinned to the reference's in test_oracle_golden.py
        memb, _ = po.ref_leiden(rp, col, REFINE, ar)
        out[f"{name}/auto_resolution"] = np.float64(ar)
        out[f"{name}/membership"] = memb
        out[f"{name}/new_ids"] = po.ref_generate_mapping(rp, col, REFINE, ar)
    np.savez_compressed(os.path.join(HERE, "refine_cases.npz"), **out)


if __name__ == "__main__":
    main()
