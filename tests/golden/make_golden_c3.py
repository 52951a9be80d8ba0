"""Pin the full-size weak-structure graphs (uniform 2^23, degree 16; grid
4096 x 4096 with 5 % of edges deleted) to the oracle's serial-order mapping.

    python tests/golden/make_golden_c3.py

The graphs come from graphbrew_gb300.graphgen (seeded, device-independent);
the oracle (oracle/gb_oracle.c, pinned against the reference on the golden
graphs and on GAPBS -g 16/20/22) maps them with the cd_serial recipe.  Output
``c3_pins.json``: graph checksums, the oracle's automatic resolution, the
mapping's fingerprint and the relabelled CSR's checksums.  The GPU's
cd_parallel on the uniform graph runs the same serial order, and cd_serial on
the grid does.
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

SEED = 27491095


def ck(a):
    return gg.checksum(torch.from_numpy(np.ascontiguousarray(a)))


def main():
    out = {}
    for name, make in (("urand23", lambda: gg.uniform(23, 16, seed=SEED)),
                       ("grid4096", lambda: gg.grid(4096, 4096, 0.05, seed=SEED))):
        t0 = time.time()
        rp_t, col_t = make()
        rp, col = rp_t.numpy(), col_t.numpy()
        del rp_t, col_t
        ar = po.auto_resolution(rp, col)
        ids, _, _, _ = po.map_graph(rp, col, ar, parallel=False)
        orp, ocol = po.relabel(rp, col, ids)
        out[name] = {"n": int(len(rp) - 1), "nnz": int(len(col)), "row_ptr": ck(rp), "col": ck(col),
                     "auto_resolution": ar, "fingerprint_cd_serial": po.fingerprint(ids),
                     "relabel_row_ptr": ck(orp), "relabel_col": ck(ocol)}
        print(name, out[name], f"{time.time() - t0:.1f}s", flush=True)
    with open(os.path.join(HERE, "c3_pins.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
