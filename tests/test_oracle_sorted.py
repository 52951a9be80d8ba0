"""Sorted intra orders in the oracle, pinned twice.

* The restatement of libstdc++'s std::sort (whose tie order the reference's
  HubSort / DegreeAsc / Hub2 / Alternate / BoundaryLast / CoreOrder inherit)
  against the toolchain's own std::sort, element for element, on random,
  tie-heavy, presorted and adversarial inputs -- the adversarial ones drive the
  introsort into its heap-sort fallback.
* orderCompose with each of those orders against the reference's outputs
  (``tests/golden/sorted_cases.npz``, made by ``make_golden_sorted.py``).
"""
import os
import sys

import numpy as np
import pytest

import pyoracle as po

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

from make_golden_sorted import ORDERS, generator_graphs  # noqa: E402


def _inputs(seed, count):
    rng = np.random.default_rng(seed)
    for t in range(count):
        n = int(rng.integers(0, 40)) if t % 3 == 0 else int(rng.integers(0, 3000))
        distinct = int(rng.integers(1, 6)) if t % 2 else 1 << 40
        key = rng.integers(0, distinct, size=max(n, 1)).astype(np.uint64)
        if t % 5 == 0:
            key = np.sort(key)
        elif t % 7 == 0:
            key = np.sort(key)[::-1].copy()
        elems = rng.permutation(n).astype(np.uint32) if t % 4 == 0 else np.arange(n, dtype=np.uint32)
        yield elems, key


def test_sort_restatement_matches_std_sort():
    for elems, key in _inputs(0, 1500):
        np.testing.assert_array_equal(po.libstdcxx_sort(elems, key), po.std_sort(elems, key))


def test_heap_sort_restatement_matches_std_partial_sort():
    for elems, key in _inputs(1, 600):
        np.testing.assert_array_equal(po.libstdcxx_heap_sort(elems, key), po.std_heap_sort(elems, key))


class _Adversary:
    """McIlroy's "antiqsort" adversary: values are fixed lazily, so that the
    pivot candidates end up low; on the values it leaves, a median-of-three
    quicksort goes quadratic and introsort hits its depth limit."""

    def __init__(self, n):
        self.gas = n
        self.val = [n] * n
        self.solid = 0
        self.candidate = -1
        self.depth_hits = 0

    def less(self, x, y):
        if self.val[x] == self.gas and self.val[y] == self.gas:
            self._freeze(x if x == self.candidate else y)
        if self.val[x] == self.gas:
            self.candidate = x
        elif self.val[y] == self.gas:
            self.candidate = y
        return self.val[x] < self.val[y]

    def _freeze(self, i):
        self.val[i] = self.solid
        self.solid += 1


def _introsort_with(a, less, adv):
    """The same introsort skeleton as the restatement, over a comparator
    callback; only used to drive the adversary (heap sort and the final
    insertion sort compare too, but the input is fixed by then)."""

    def median_to_first(r, x, y, z):
        if less(a[x], a[y]):
            if less(a[y], a[z]):
                a[r], a[y] = a[y], a[r]
            elif less(a[x], a[z]):
                a[r], a[z] = a[z], a[r]
            else:
                a[r], a[x] = a[x], a[r]
        elif less(a[x], a[z]):
            a[r], a[x] = a[x], a[r]
        elif less(a[y], a[z]):
            a[r], a[z] = a[z], a[r]
        else:
            a[r], a[y] = a[y], a[r]

    def partition(first, last, pivot):
        while True:
            while less(a[first], a[pivot]):
                first += 1
            last -= 1
            while less(a[pivot], a[last]):
                last -= 1
            if not first < last:
                return first
            a[first], a[last] = a[last], a[first]
            first += 1

    def loop(first, last, depth):
        while last - first > 16:
            if depth == 0:
                adv.depth_hits += 1
                return
            depth -= 1
            mid = first + (last - first) // 2
            median_to_first(first, first + 1, mid, last - 1)
            cut = partition(first + 1, last, first)
            loop(cut, last, depth)
            last = cut

    n = len(a)
    if n:
        loop(0, n, 2 * (n.bit_length() - 1))


@pytest.mark.parametrize("n", [200, 1000, 4099])
def test_sort_restatement_on_adversarial_input(n):
    adv = _Adversary(n)
    _introsort_with(list(range(n)), adv.less, adv)
    assert adv.depth_hits > 0, "the adversary should exhaust the depth limit"
    key = np.array(adv.val, dtype=np.uint64)
    elems = np.arange(n, dtype=np.uint32)
    ours = po.libstdcxx_sort(elems, key)
    np.testing.assert_array_equal(ours, po.std_sort(elems, key))
    assert np.all(np.diff(key[ours].astype(np.int64)) >= 0)


@pytest.fixture(scope="module")
def sorted_golden():
    return np.load(os.path.join(HERE, "golden", "sorted_cases.npz"))


def _graphs(sorted_golden, mapping_golden):
    names = sorted({k.split("/")[0] for k in sorted_golden.files})
    gen = generator_graphs()
    for name in names:
        if name in gen:
            rp, col = gen[name]
            memb = sorted_golden[f"{name}/membership"]
        else:
            rp, col = mapping_golden[f"{name}/row_ptr"], mapping_golden[f"{name}/col"]
            memb = mapping_golden[f"{name}/membership_serial"]
        yield name, rp, col, memb


@pytest.mark.parametrize("order", sorted(ORDERS))
def test_oracle_sorted_intra_matches_reference(order, sorted_golden, golden_arrays):
    checked = 0
    for name, rp, col, memb in _graphs(sorted_golden, golden_arrays):
        ids, _ = po.compose(rp, col, memb, "size-desc", order)
        np.testing.assert_array_equal(ids, sorted_golden[f"{name}/{order}"], err_msg=name)
        checked += 1
        if order == "hubsort" and f"{name}/hubsort_degdesc" in sorted_golden.files:
            ids, _ = po.compose(rp, col, memb, "degree-desc", "hubsort")
            np.testing.assert_array_equal(ids, sorted_golden[f"{name}/hubsort_degdesc"], err_msg=name)
    assert checked >= 16
