"""The oracle's intraRCM and intraRCMpp restatements against the reference's outputs (CPU)."""
import os

import numpy as np
import pytest

import pyoracle as po
from conftest import GOLDEN

RCM_CASES = np.load(os.path.join(GOLDEN, "rcm_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in RCM_CASES.files})


@pytest.mark.parametrize("order", ["rcm", "rcmpp"])
@pytest.mark.parametrize("name", NAMES)
def test_rcm_compose(name, order, golden_arrays):
    if f"{name}/row_ptr" in RCM_CASES.files:
        rp, col, memb = RCM_CASES[f"{name}/row_ptr"], RCM_CASES[f"{name}/col"], RCM_CASES[f"{name}/membership"]
    else:
        rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
        memb = golden_arrays[f"{name}/membership_serial"]
    ids, _ = po.compose(rp, col, memb, "size-desc", order)
    np.testing.assert_array_equal(ids, RCM_CASES[f"{name}/{order}_ids"])


def test_rcmpp_differs_from_rcm_somewhere():
    differ = [n for n in NAMES if not np.array_equal(RCM_CASES[f"{n}/rcm_ids"], RCM_CASES[f"{n}/rcmpp_ids"])]
    assert len(differ) >= 5
