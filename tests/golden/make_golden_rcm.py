"""Golden outputs of orderCompose with intra-community RCM and RCM++, from the reference.

Run where the reference harness is built (``make -C oracle ref``):

    python tests/golden/make_golden_rcm.py

For every graph of ``mapping_cases.npz`` (with its cd_serial membership) and
three seeded generator graphs (membership from the oracle's serial Leiden,
stored), ``rcm_cases.npz`` holds the reference's forward map for

    leiden:compose:sg_none:comm_size_desc:intra_rcm:cd_serial:norefine:2:2

i.e. intraRCM (bench/include/graphbrew/reorder/reorder_graphbrew.h:4000-4134)
applied to every community, and the same with ``intra_rcmpp`` (intraRCMpp,
:4154-4342) as ``<name>/rcmpp_ids``.
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

RCM = "leiden:compose:sg_none:comm_size_desc:intra_rcm:cd_serial:norefine:2:2"
RCMPP = RCM.replace("intra_rcm", "intra_rcmpp")


def main():
    if po.load_reference() is None:
        raise SystemExit("reference harness not built: make -C oracle ref")
    cases = np.load(os.path.join(HERE, "mapping_cases.npz"))
    names = sorted({k.split("/")[0] for k in cases.files})
    out = {}
    for name in names:
        rp, col = cases[f"{name}/row_ptr"], cases[f"{name}/col"]
        memb = cases[f"{name}/membership_serial"]
        out[f"{name}/rcm_ids"] = po.ref_compose(rp, col, memb, RCM, 1.0)[0]
        out[f"{name}/rcmpp_ids"] = po.ref_compose(rp, col, memb, RCMPP, 1.0)[0]
    gen = {"rmat12_s3": gg.rmat(12, 16, seed=3), "rmat14_s4": gg.rmat(14, 16, seed=4),
           "grid60x70": gg.grid(60, 70, 0.1, seed=5)}
    for name, (rp, col) in gen.items():
        rp, col = rp.numpy(), col.numpy()
        memb, _ = po.leiden(rp, col, po.auto_resolution(rp, col))
        out[f"{name}/row_ptr"] = rp
        out[f"{name}/col"] = col
        out[f"{name}/membership"] = memb
        out[f"{name}/rcm_ids"] = po.ref_compose(rp, col, memb, RCM, 1.0)[0]
        out[f"{name}/rcmpp_ids"] = po.ref_compose(rp, col, memb, RCMPP, 1.0)[0]
    np.savez_compressed(os.path.join(HERE, "rcm_cases.npz"), **out)


if __name__ == "__main__":
    main()
