"""Sorted intra orders on the GPU (HubSort, DegreeAsc, Hub2, Alternate,
BoundaryLast, CoreOrder; reorder_graphbrew.h:6759-6955) against the
reference's outputs bit for bit, given the same membership, and against the
oracle on larger graphs -- including a community whose degrees drive
libstdc++'s introsort into its heap-sort fallback."""
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
from make_golden_sorted import ORDERS, generator_graphs  # noqa: E402
from test_oracle_sorted import _Adversary, _introsort_with  # noqa: E402

pytestmark = pytest.mark.gpu

CASES = np.load(os.path.join(GOLDEN, "sorted_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})


def recipe(order, comm="comm_size_desc"):
    return f"leiden:compose:sg_none:{comm}:{ORDERS[order]}:cd_serial:norefine:2:2"


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def gen_graphs():
    return generator_graphs()


@pytest.mark.parametrize("order", sorted(ORDERS))
def test_sorted_against_reference(ctx, order, golden_arrays, gen_graphs):
    for name in NAMES:
        if name in gen_graphs:
            rp, col = gen_graphs[name]
            memb = CASES[f"{name}/membership"]
        else:
            rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
            memb = golden_arrays[f"{name}/membership_serial"]
        ids, _ = ctx.order_compose(rp, col, memb, recipe(order))
        np.testing.assert_array_equal(ids, CASES[f"{name}/{order}"], err_msg=name)
        if order == "hubsort" and f"{name}/hubsort_degdesc" in CASES.files:
            ids, _ = ctx.order_compose(rp, col, memb, recipe(order, "comm_degree_desc"))
            np.testing.assert_array_equal(ids, CASES[f"{name}/hubsort_degdesc"], err_msg=name)


@pytest.mark.parametrize("order", sorted(ORDERS))
def test_sorted_mapping_against_oracle(ctx, order):
    rp_t, col_t = gg.rmat(17, 16, seed=77, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    ids, _ = ctx.generate_mapping(rp_t, col_t, recipe(order), ar)
    memb, _ = po.leiden(rp, col, ar, super_move_batch=1)   # the recipe has no sgmb token
    ids_orc, _ = po.compose(rp, col, memb, "size-desc", order)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)


def _adversarial_hub_graph(n):
    """Community 0 = vertices 0..n-1 with degrees chosen so that HubSort's
    keys are McIlroy's adversarial values; their neighbours are padding
    vertices in community 1."""
    adv = _Adversary(n)
    _introsort_with(list(range(n)), adv.less, adv)
    assert adv.depth_hits > 0
    val = np.array(adv.val, dtype=np.int64)
    deg = (n + 2) - val                   # larger value -> smaller degree -> larger ~deg key
    pad = int(deg.max())
    nv = n + pad
    rows = [[] for _ in range(nv)]
    for i in range(n):
        for j in range(int(deg[i])):
            rows[i].append(n + j)
            rows[n + j].append(i)
    rp = np.zeros(nv + 1, dtype=np.int64)
    rp[1:] = np.cumsum([len(r) for r in rows])
    col = np.concatenate([np.sort(np.array(r, dtype=np.int32)) for r in rows])
    memb = np.zeros(nv, dtype=np.uint32)
    memb[n:] = 1
    return rp, col, memb


@pytest.mark.parametrize("order", ["hubsort", "alternate"])
def test_sorted_heap_fallback_against_oracle(ctx, order):
    rp, col, memb = _adversarial_hub_graph(700)
    ids, _ = ctx.order_compose(rp, col, memb, recipe(order))
    ids_orc, _ = po.compose(rp, col, memb, "size-desc", order)
    np.testing.assert_array_equal(ids, ids_orc)
    # The community's order is the toolchain's std::sort of its vertices.
    key = (0xFFFFFFFF - np.diff(rp)).astype(np.uint64)
    want = po.std_sort(np.arange(700, dtype=np.uint32), key)
    if order == "hubsort":
        base = ids[:700].min()
        np.testing.assert_array_equal(np.argsort(ids[:700] - base), want)


def _hub_core_graph(seed):
    """Two communities over 30,000 vertices; about ten hubs of 4,500-12,000
    neighbours in each (rows of the peel's CTA tier, 513-8,192 entries, and of
    its whole-grid tier above), a dense core of 60 vertices, and random
    background edges, so that long rows enter the peel's frontiers both from
    the level scans and from decrements."""
    rng = np.random.default_rng(seed)
    n = 30000
    memb = (rng.random(n) < 0.5).astype(np.uint32)
    src, dst = [], []
    hubs = rng.choice(n, 20, replace=False)
    for h in hubs:
        d = int(rng.integers(4500, 12000))
        nb = rng.choice(n, d, replace=False)
        src.append(np.full(d, h))
        dst.append(nb)
    core = rng.choice(n, 60, replace=False)
    cs, cd = np.meshgrid(core, core)
    src.append(cs.ravel())
    dst.append(cd.ravel())
    e = rng.integers(0, n, size=(150000, 2))
    src.append(e[:, 0])
    dst.append(e[:, 1])
    s_ = np.concatenate(src + dst)
    d_ = np.concatenate(dst + src)
    keep = s_ != d_
    key = np.unique(s_[keep].astype(np.int64) * n + d_[keep])
    rows, cols = key // n, (key % n).astype(np.int32)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp), cols, memb


@pytest.mark.parametrize("seed", [1, 2])
def test_core_order_heavy_rows_against_oracle(ctx, seed):
    rp, col, memb = _hub_core_graph(seed)
    deg = np.diff(rp)
    assert ((deg > 512) & (deg <= 8192)).sum() >= 5 and (deg > 8192).sum() >= 5
    ids, _ = ctx.order_compose(rp, col, memb, recipe("core"))
    ids_orc, _ = po.compose(rp, col, memb, "size-desc", "core")
    np.testing.assert_array_equal(ids, ids_orc)
