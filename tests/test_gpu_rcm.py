"""Intra-community reverse Cuthill-McKee on the GPU (intraRCM,
reorder_graphbrew.h:4000-4134, and intraRCMpp, :4154-4342) against the
reference's outputs, bit for bit, given the same membership; and against the
oracle on larger graphs."""
import os

import numpy as np
import pytest
import torch

import pyoracle as po
import graphbrew_gb300 as gb
from graphbrew_gb300 import graphgen as gg
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RCM = "leiden:compose:sg_none:comm_size_desc:intra_rcm:cd_serial:norefine:2:2"
RECIPES = {"rcm": RCM, "rcmpp": RCM.replace("intra_rcm", "intra_rcmpp")}
RCM_CASES = np.load(os.path.join(GOLDEN, "rcm_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in RCM_CASES.files})


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("order", ["rcm", "rcmpp"])
@pytest.mark.parametrize("name", NAMES)
def test_rcm_against_reference(ctx, name, order, golden_arrays):
    if f"{name}/row_ptr" in RCM_CASES.files:
        rp, col, memb = RCM_CASES[f"{name}/row_ptr"], RCM_CASES[f"{name}/col"], RCM_CASES[f"{name}/membership"]
    else:
        rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
        memb = golden_arrays[f"{name}/membership_serial"]
    ids, st = ctx.order_compose(rp, col, memb, RECIPES[order])
    np.testing.assert_array_equal(ids, RCM_CASES[f"{name}/{order}_ids"])


@pytest.mark.parametrize("order", ["rcm", "rcmpp"])
@pytest.mark.parametrize("kind", ["rmat18", "grid"])
def test_rcm_mapping_against_oracle(ctx, kind, order):
    if kind == "rmat18":
        rp_t, col_t = gg.rmat(18, 16, seed=41, device="cuda")
    else:
        rp_t, col_t = gg.grid(300, 300, 0.08, seed=42, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    ids, _ = ctx.generate_mapping(rp_t, col_t, RECIPES[order], ar)
    m_orc, _ = po.leiden(rp, col, ar, super_move_batch=1)   # the recipe has no sgmb token
    ids_orc, _ = po.compose(rp, col, m_orc, "size-desc", order)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)
