"""Leiden with refinement on the GPU (refine0: localMovingPhase<true> after
pass 0's local moving, reorder_graphbrew.h:7330-7392), bit for bit against
the reference's memberships and forward maps, and against the oracle on
larger graphs (the serial-order engine gives cd_serial semantics)."""
import os
import sys

import numpy as np
import pytest
import torch

import pyoracle as po
import graphbrew_gb300 as gb
from graphbrew_gb300 import graphgen as gg
from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
from make_golden_refine import REFINE, generator_graphs  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = np.load(os.path.join(GOLDEN, "refine_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def gen_graphs():
    return generator_graphs()


@pytest.mark.parametrize("name", NAMES)
def test_refine_against_reference(ctx, name, golden_arrays, gen_graphs):
    if name in gen_graphs:
        rp, col = gen_graphs[name]
    else:
        rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
    ar = float(CASES[f"{name}/auto_resolution"])
    memb, _ = ctx.run_graphbrew(rp, col, REFINE, ar)
    np.testing.assert_array_equal(np.asarray(memb).view(np.uint32), CASES[f"{name}/membership"])
    ids, _ = ctx.generate_mapping(rp, col, REFINE, ar)
    np.testing.assert_array_equal(ids, CASES[f"{name}/new_ids"])


@pytest.mark.parametrize("scale", [16, 18])
def test_refine_rmat_against_oracle(ctx, scale):
    rp_t, col_t = gg.rmat(scale, 16, seed=300 + scale, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    recipe = REFINE.replace("cd_serial", "cd_parallel")
    ids, st = ctx.generate_mapping(rp_t, col_t, recipe, ar)
    memb, _ = po.leiden(rp, col, ar, refine_depth=0)
    ids_orc, _ = po.compose(rp, col, memb)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)


@pytest.mark.parametrize("graph", ["rmat17", "grid512"])
@pytest.mark.parametrize("split_min", ["4096", "200"])
@pytest.mark.parametrize("refine", [False, True])
def test_batched_super_move_against_oracle(ctx, monkeypatch, refine, split_min, graph):
    """The super-move's batched launches (used above one cluster's size;
    forced here) give the cluster kernel's memberships: lanes for super-nodes
    up to 8 neighbours, warps up to 128, a CTA each above, and above
    split_min neighbours several CTAs per super-node (edge segments into one
    table, table segments selecting, the last one reducing).  The grid's
    super-nodes are mostly of the lane kind, RMAT's of all kinds."""
    monkeypatch.setenv("GBGPU_SUPER_CLUSTER_MAX_EDGES", "0")
    monkeypatch.setenv("GBGPU_SUPER_SPLIT_MIN", split_min)
    if graph == "rmat17":
        rp_t, col_t = gg.rmat(17, 16, seed=400, device="cuda")
    else:
        rp_t, col_t = gg.grid(512, 512, 0.05, seed=401, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    recipe = REFINE if refine else REFINE.replace("refine0", "norefine")
    memb, st = ctx.run_graphbrew(rp_t, col_t, recipe, ar)
    assert st["super_move_ctas"] == 0
    want, _ = po.leiden(rp, col, ar, refine_depth=0 if refine else None)
    np.testing.assert_array_equal(memb.cpu().numpy().view(np.uint32), want)
