"""Golden outputs of orderCompose with the sorted intra orders, from the reference.

Run where the reference harness is built (``make -C oracle ref``):

    python tests/golden/make_golden_sorted.py

For every graph of ``mapping_cases.npz`` (with its cd_serial membership) and
four seeded generator graphs (regenerated by the tests; membership from the
oracle's serial Leiden, stored), ``sorted_cases.npz`` holds the reference's forward map for

    leiden:compose:sg_none:<community order>:<intra order>:cd_serial:norefine:2:2

with the intra orders HubSort, DegreeAsc, Hub2, Alternate, BoundaryLast and
CoreOrder (bench/include/graphbrew/reorder/reorder_graphbrew.h:6759-6955).
Their std::sort leaves ties in libstdc++'s introsort order, which these
fixtures record.
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

ORDERS = {"hubsort": "intra_hubsort", "degree-asc": "intra_deg_asc", "hub2": "intra_hub2",
          "alternate": "intra_alternate", "boundary-last": "intra_boundary_last", "core": "intra_core"}


def generator_graphs():
    """The seeded generator graphs (regenerated by the tests, not stored)."""
    gen = {"rmat12_s3": gg.rmat(12, 16, seed=3), "rmat14_s4": gg.rmat(14, 16, seed=4),
           "grid60x70": gg.grid(60, 70, 0.1, seed=5), "rmat15_s9": gg.rmat(15, 8, seed=9)}
    return {k: (rp.numpy(), col.numpy()) for k, (rp, col) in gen.items()}


def recipe(intra_token, comm="comm_size_desc"):
    return f"leiden:compose:sg_none:{comm}:{intra_token}:cd_serial:norefine:2:2"


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    cases = np.load(os.path.join(HERE, "mapping_cases.npz"))
    names = sorted({k.split("/")[0] for k in cases.files})
    out = {}
    for name in names:
        rp, col = cases[f"{name}/row_ptr"], cases[f"{name}/col"]
        memb = cases[f"{name}/membership_serial"]
        for key, tok in ORDERS.items():
            out[f"{name}/{key}"] = po.ref_compose(rp, col, memb, recipe(tok), 1.0)[0]
    for name, (rp, col) in generator_graphs().items():
        memb, _ = po.leiden(rp, col, po.auto_resolution(rp, col))
        out[f"{name}/membership"] = memb
        for key, tok in ORDERS.items():
            out[f"{name}/{key}"] = po.ref_compose(rp, col, memb, recipe(tok), 1.0)[0]
        # A community order other than size-desc, once per generator graph.
        out[f"{name}/hubsort_degdesc"] = po.ref_compose(rp, col, memb, recipe("intra_hubsort", "comm_degree_desc"),
                                                        1.0)[0]
    np.savez_compressed(os.path.join(HERE, "sorted_cases.npz"), **out)


if __name__ == "__main__":
    main()
