"""The oracle's Leiden refinement (refine0: refinement phase in pass 0,
reorder_graphbrew.h:7330-7392 with localMovingPhase<true>) against the
reference's memberships and forward maps (``tests/golden/refine_cases.npz``,
made by ``make_golden_refine.py``)."""
import os
import sys

import numpy as np
import pytest

import pyoracle as po
from conftest import GOLDEN

sys.path.insert(0, GOLDEN)
from make_golden_refine import generator_graphs  # noqa: E402

CASES = np.load(os.path.join(GOLDEN, "refine_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})


@pytest.fixture(scope="module")
def gen_graphs():
    return generator_graphs()


def _graph(name, golden_arrays, gen_graphs):
    if name in gen_graphs:
        return gen_graphs[name]
    return golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]


@pytest.mark.parametrize("name", NAMES)
def test_refine_membership_and_mapping(name, golden_arrays, gen_graphs):
    rp, col = _graph(name, golden_arrays, gen_graphs)
    ar = float(CASES[f"{name}/auto_resolution"])
    assert ar == po.auto_resolution(rp, col)
    memb, _ = po.leiden(rp, col, ar, refine_depth=0)
    np.testing.assert_array_equal(memb, CASES[f"{name}/membership"])
    ids, _ = po.compose(rp, col, memb)
    np.testing.assert_array_equal(ids, CASES[f"{name}/new_ids"])


def test_refinement_changes_the_result_somewhere(golden_arrays, gen_graphs):
    changed = 0
    for name in NAMES:
        rp, col = _graph(name, golden_arrays, gen_graphs)
        ar = float(CASES[f"{name}/auto_resolution"])
        plain, _ = po.leiden(rp, col, ar)
        changed += not np.array_equal(plain, CASES[f"{name}/membership"])
    assert changed >= 5
