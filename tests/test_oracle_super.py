"""Super-graph orders in the oracle (sg_super_rcm, sg_hilbert), pinned twice.

* The restatement of libstdc++'s std::unordered_map iteration order
  (orc_umap_order: insertion at a bucket's front or the list's front, rehash
  by the same rules) against the toolchain's own container on random key
  sequences across many rehashes, and its growth table against the
  container's bucket_count().
* orderCompose with each super-graph order against the reference's
  one-thread outputs (``tests/golden/super_cases.npz`` and the SHA-256 pins
  of ``super_pins.json``, made by ``make_golden_super.py``).
"""
import json
import os
import sys

import numpy as np
import pytest

import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from make_golden_super import BIG, COMM, SUPER, big_graph, digest  # noqa: E402
from make_golden_sorted import generator_graphs  # noqa: E402

CASES = np.load(os.path.join(HERE, "golden", "super_cases.npz"))
NAMES = sorted({k.split("/")[0] for k in CASES.files})
with open(os.path.join(HERE, "golden", "super_pins.json")) as f:
    PINS = json.load(f)
GROWTH = [13, 29, 59, 127, 257, 541, 1109, 2357, 5087, 10273, 20753, 42043, 85229, 172933, 351061, 712697]


def _key_sequences(seed, count):
    rng = np.random.default_rng(seed)
    for t in range(count):
        k = int(rng.integers(0, 60)) if t % 3 == 0 else int(rng.integers(0, 4000))
        if t % 40 == 0:
            k = int(rng.integers(20000, 200000))
        hi = [64, 6000, 1 << 20, 1 << 32][t % 4]
        keys = rng.permutation(np.unique(rng.integers(0, hi, size=k, dtype=np.uint64)).astype(np.uint32))
        yield keys


def test_umap_order_matches_toolchain():
    for keys in _key_sequences(3, 160):
        np.testing.assert_array_equal(po.umap_order(keys), po.std_umap_order(keys))


def test_umap_growth_table_matches_toolchain():
    assert po.std_umap_bucket_count(1) == GROWTH[0]
    for a, b in zip(GROWTH, GROWTH[1:]):
        assert po.std_umap_bucket_count(a) == a
        assert po.std_umap_bucket_count(a + 1) == b


def _graphs(golden_arrays):
    gen = generator_graphs()
    for name in NAMES:
        if name in gen:
            rp, col = gen[name]
            memb = CASES[f"{name}/membership"]
        else:
            rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
            memb = golden_arrays[f"{name}/membership_serial"]
        yield name, rp, col, memb


@pytest.mark.parametrize("sup", sorted(SUPER))
def test_compose_super_against_reference(golden_arrays, sup):
    for name, rp, col, memb in _graphs(golden_arrays):
        for comm in COMM:
            ids, _ = po.compose(rp, col, memb, comm, "bfs", super_order=sup)
            np.testing.assert_array_equal(ids, CASES[f"{name}/{sup}/{comm}"], err_msg=f"{name} {comm}")


@pytest.mark.parametrize("name", sorted(BIG))
def test_compose_super_pinned(name):
    rp, col, memb = big_graph(name)
    for sup in SUPER:
        for comm in COMM:
            ids, _ = po.compose(rp, col, memb, comm, "bfs", super_order=sup)
            assert digest(ids) == PINS[name][sup][comm], (sup, comm)
