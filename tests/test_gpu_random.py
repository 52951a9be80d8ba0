"""intra_random on the GPU (reorder_graphbrew.h:6825-6845): the warp-per-
community MT19937 draws and the reservation rounds of the swaps give the
reference's permutation bit for bit, given the same membership; on the
large-community pins (rejected draws included) and through the whole
mapping against the oracle."""
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
from make_golden_random import COMM, big_cases, digest, recipe  # noqa: E402
from make_golden_sorted import generator_graphs  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = np.load(os.path.join(GOLDEN, "random_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})
with open(os.path.join(GOLDEN, "random_pins.json")) as f:
    PINS = json.load(f)


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("comm", sorted(COMM))
def test_random_against_reference(ctx, comm, golden_arrays):
    gen = generator_graphs()
    for name in NAMES:
        if name in gen:
            rp, col = gen[name]
            memb = CASES[f"{name}/membership"]
        else:
            rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
            memb = golden_arrays[f"{name}/membership_serial"]
        ids, _ = ctx.order_compose(rp, col, memb, recipe(comm))
        np.testing.assert_array_equal(ids, CASES[f"{name}/{comm}"], err_msg=name)


def test_random_large_communities_pinned(ctx):
    for name, rp, col, memb in big_cases():
        ids, _ = ctx.order_compose(rp, col, memb, recipe())
        assert digest(ids) == PINS[name]["sha256"], name


def test_random_mapping_against_oracle(ctx):
    rp_t, col_t = gg.rmat(17, 16, seed=78, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    ids, _ = ctx.generate_mapping(rp_t, col_t, recipe(), ar)
    memb, _ = po.leiden(rp, col, ar, super_move_batch=1)   # the recipe has no sgmb token
    ids_orc, _ = po.compose(rp, col, memb, "size-desc", "random")
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)
