"""intra_random in the oracle, pinned twice.

* The restatement of std::mt19937 + libstdc++'s uniform_int_distribution
  (orc_random_draws) against the toolchain's own, draw for draw, on sizes up
  to 2^22 (about a thousand rejected draws).
* orderCompose with intra_random against the reference's outputs
  (``tests/golden/random_cases.npz`` and the SHA-256 pins of
  ``random_pins.json``, made by ``make_golden_random.py``).
"""
import json
import os
import sys

import numpy as np
import pytest

import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from make_golden_random import COMM, big_cases, digest  # noqa: E402
from make_golden_sorted import generator_graphs  # noqa: E402

CASES = np.load(os.path.join(HERE, "golden", "random_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})
with open(os.path.join(HERE, "golden", "random_pins.json")) as f:
    PINS = json.load(f)


@pytest.mark.parametrize("seed,count", [(0xDEADBEEF, 0), (0xDEADBEEF, 1), (0xDEADBEEF, 2), (0xDEADBEEF ^ 7, 625),
                                        (0xDEADBEEF ^ 123, 100000), (1, 1 << 22)])
def test_draws_match_toolchain(seed, count):
    np.testing.assert_array_equal(po.random_draws(seed, count), po.std_shuffle_draws(seed, count))


def test_compose_random_against_reference(golden_arrays):
    gen = generator_graphs()
    for name in NAMES:
        if name in gen:
            rp, col = gen[name]
            memb = CASES[f"{name}/membership"]
        else:
            rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
            memb = golden_arrays[f"{name}/membership_serial"]
        for comm in COMM:
            ids, _ = po.compose(rp, col, memb, comm, "random")
            np.testing.assert_array_equal(ids, CASES[f"{name}/{comm}"], err_msg=f"{name} {comm}")


def test_compose_random_large_communities_pinned():
    for name, rp, col, memb in big_cases():
        ids, _ = po.compose(rp, col, memb, "size-desc", "random")
        assert digest(ids) == PINS[name]["sha256"], name
