"""Super-graph orders on the GPU (sg_super_rcm, sg_super_rabbit, sg_hilbert;
reorder_graphbrew.h:4990-5090, 5495-5871, 6395-6462): the per-community
std::unordered_map simulations, the George-Liu / Cuthill-McKee BFS, the
Rabbit merge chain and the Hilbert keys give the reference's one-thread
permutation bit for bit, given the same membership; on the RMAT-18/19 and
grid pins and through the whole mapping against the oracle."""
import json
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
from make_golden_super import BIG, COMM, SUPER, big_graph, digest, recipe  # noqa: E402
from make_golden_sorted import generator_graphs  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = np.load(os.path.join(GOLDEN, "super_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})
with open(os.path.join(GOLDEN, "super_pins.json")) as f:
    PINS = json.load(f)


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("sup", sorted(SUPER))
def test_super_against_reference(ctx, sup, golden_arrays):
    gen = generator_graphs()
    for name in NAMES:
        if name in gen:
            rp, col = gen[name]
            memb = CASES[f"{name}/membership"]
        else:
            rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
            memb = golden_arrays[f"{name}/membership_serial"]
        for comm in COMM:
            ids, _ = ctx.order_compose(rp, col, memb, recipe(sup, comm))
            np.testing.assert_array_equal(ids, CASES[f"{name}/{sup}/{comm}"], err_msg=f"{name} {comm}")


@pytest.mark.parametrize("name", sorted(BIG))
def test_super_pinned(ctx, name):
    rp, col, memb = big_graph(name)
    for sup in SUPER:
        for comm in COMM:
            ids, _ = ctx.order_compose(rp, col, memb, recipe(sup, comm))
            assert digest(ids) == PINS[name][sup][comm], (sup, comm)


def test_super_rabbit_saturated_weights_against_oracle(ctx):
    """RMAT-20 with its own mapping's membership: the giant community holds
    more than 2^24 entries, so its pair weight stops at 2^24 and the float
    sums of the Rabbit merge chain round in the reference's order."""
    rp_t, col_t = gg.rmat(20, 16, seed=81, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, _ = ctx.run_graphbrew(rp_t, col_t, recipe("super-rabbit"), ar)
    memb = memb.cpu().numpy().view(np.uint32)
    src = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    same = memb[src] == memb[col]
    assert np.bincount(memb[src][same]).max() > (1 << 24)
    for sup in ("super-rabbit", "super-rcm"):
        ids, _ = ctx.order_compose(rp, col, memb, recipe(sup))
        ids_orc, _ = po.compose(rp, col, memb, "size-desc", "bfs", super_order=sup)
        np.testing.assert_array_equal(ids, ids_orc, err_msg=sup)


@pytest.mark.parametrize("sup", sorted(SUPER))
def test_super_mapping_against_oracle(ctx, sup):
    rp_t, col_t = gg.rmat(17, 16, seed=79, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    rec = f"leiden:compose:{SUPER[sup]}:comm_size_desc:intra_gorder:gw8:cd_serial:sgmb4096:gordf5000:norefine:2:2"
    ids, _ = ctx.generate_mapping(rp_t, col_t, rec, ar)
    memb, _ = po.leiden(rp, col, ar)
    ids_orc, _ = po.compose(rp, col, memb, "size-desc", "gorder", super_order=sup)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)


@pytest.mark.parametrize("layout", ["many-mid-maps", "one-huge-map"])
def test_super_map_tiers_against_oracle(ctx, layout):
    """Memberships that put communities' maps in every size tier of the map
    simulations: 1,500 random communities of a uniform graph (maps of tens to
    hundreds of keys: the warp tier and the shared-memory CTA tier), and half
    the graph in community 0 beside 30,000 small ones (community 0's map has
    about 24,000 keys, more than a CTA's shared memory holds: the global
    tier)."""
    rp_t, col_t = gg.uniform(16, 16, seed=82, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    n = len(rp) - 1
    h = (np.arange(n, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)) >> np.uint64(40)
    if layout == "many-mid-maps":
        memb = (h % np.uint64(1500)).astype(np.uint32)
    else:
        memb = np.where(np.arange(n) < n // 2, 0, 1 + h % np.uint64(30000)).astype(np.uint32)
    for sup in ("super-rcm", "super-rabbit"):
        ids, _ = ctx.order_compose(rp, col, memb, recipe(sup))
        ids_orc, _ = po.compose(rp, col, memb, "size-desc", "bfs", super_order=sup)
        np.testing.assert_array_equal(ids, ids_orc, err_msg=sup)


def test_super_rabbit_arena_growth(ctx, monkeypatch):
    """With no room beyond the initial lists the merge chain stops at the
    first aggregated list that does not fit, the arena grows and the chain
    resumes there: the permutation is unchanged (the RMAT-18 pin)."""
    monkeypatch.setenv("GBGPU_RABBIT_ARENA_SLACK", "1")
    rp, col, memb = big_graph("rmat18_s11")
    ids, _ = ctx.order_compose(rp, col, memb, recipe("super-rabbit"))
    assert digest(ids) == PINS["rmat18_s11"]["super-rabbit"]["size-desc"]
