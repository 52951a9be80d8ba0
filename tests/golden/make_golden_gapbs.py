"""Pin GAPBS's synthetic graphs and the reference's answers on them.

Run where the GraphBrew sources are mounted and the reference harness is built
(``make -C oracle ref``):

    python tests/golden/make_golden_gapbs.py

For ``converter -g <scale> -s`` (RMAT) and ``-u <scale> -s`` (uniform) it builds
the graph with the reference's own generator and builder
(``po.ref_gapbs_graph``: bench/include/external/gapbs/generator.h and
builder.h, through oracle/ref_harness.cc) and records its size and the
checksums of its CSR arrays (``graphgen.checksum``).  For the RMAT scales in
``MAPPED`` it also runs the reference's ``generateGraphBrewMapping`` with the
cd_serial recipe (deterministic; the GPU's cd_parallel runs the same serial
order) and records the "Mapping Fingerprint" and the checksums of
``RelabelByMapping``'s CSR.  Output: ``gapbs_pins.json``.

The cd_serial fingerprints of ``-g 16/20/22`` were also measured with the
reference's own ``converter`` binary (9b52c0603aacbbdb, 1bb16f3ac238f77f,
91a0f15d18ec743d); the harness must agree with them, which this script checks.
"""
from __future__ import annotations

import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import pyoracle as po  # noqa: E402
from graphbrew_gb300 import graphgen as gg  # noqa: E402

SERIAL = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:"
          "sgmb4096:gordf5000:norefine:2:2")
RMAT_SCALES = [10, 12, 14, 16, 18, 20, 22]
UNIFORM_SCALES = [10, 14, 18, 20]
MAPPED = [16, 20, 22]
CONVERTER = {16: "9b52c0603aacbbdb", 20: "1bb16f3ac238f77f", 22: "91a0f15d18ec743d"}


def ck(a):
    return gg.checksum(torch.from_numpy(np.ascontiguousarray(a)))


def main():
    if po.load_reference() is None:
        sys.exit("reference harness not built (make -C oracle ref)")
    threads = os.cpu_count() or 1
    out = {"source": "reference generator + builder + generateGraphBrewMapping via oracle/ref_harness.cc",
           "recipe_serial": "12:" + SERIAL, "rmat": {}, "uniform": {}}
    for kind, scales in (("rmat", RMAT_SCALES), ("uniform", UNIFORM_SCALES)):
        for s in scales:
            t0 = time.time()
            rp, col = po.ref_gapbs_graph(s, 16, uniform=(kind == "uniform"))
            rec = {"n": int(len(rp) - 1), "nnz": int(len(col)), "row_ptr": ck(rp), "col": ck(col)}
            if kind == "rmat" and s in MAPPED:
                ar = po.load_reference().ref_auto_resolution(len(rp) - 1, rp, col)
                ids = po.ref_generate_mapping(rp, col, SERIAL, ar, threads=threads)
                fp = po.fingerprint(ids)
                assert fp == CONVERTER[s], (s, fp, CONVERTER[s])
                orp, ocol, _ = po.ref_relabel(rp, col, ids)
                rec.update({"auto_resolution": ar, "fingerprint_cd_serial": fp,
                            "relabel_row_ptr": ck(orp), "relabel_col": ck(ocol)})
            out[kind][str(s)] = rec
            print(kind, s, rec, f"{time.time() - t0:.1f}s", flush=True)
    with open(os.path.join(HERE, "gapbs_pins.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
