"""The CPU oracle against the reference's outputs stored in tests/golden.

These pin the oracle before it is trusted as the checker of the CUDA path:
cd_serial community detection, orderCompose for several recipes, the end-to-end
mapping (with its FNV fingerprint), RelabelByMapping, and the reference's own
Gorder known-answer test (bench/tests/test_graphbrew_config.cc:974-1000).
"""
import numpy as np
import pytest

import pyoracle as po
from conftest import case_names

RECIPE_ARGS = {
    "gorder8_f5000": dict(community_order="size-desc", intra_order="gorder", gorder_window=8, gorder_fallback=5000),
    "gorder8_f64": dict(community_order="size-desc", intra_order="gorder", gorder_window=8, gorder_fallback=64),
    "gorder5_f16": dict(community_order="size-desc", intra_order="gorder", gorder_window=5, gorder_fallback=16),
    "bfs_sizeasc": dict(community_order="size-asc", intra_order="bfs", gorder_window=5, gorder_fallback=0),
    "bfs_degdesc": dict(community_order="degree-desc", intra_order="bfs", gorder_window=5, gorder_fallback=0),
    "gorder8_identity": dict(community_order="identity", intra_order="gorder", gorder_window=8, gorder_fallback=32),
}


def graph(g, name):
    return g[f"{name}/row_ptr"], g[f"{name}/col"]


@pytest.mark.parametrize("name", case_names())
def test_auto_resolution(name, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    # The reference sums the degree variance with an OpenMP reduction; the
    # oracle sums serially, so only the last bits may differ.
    assert po.auto_resolution(rp, col) == pytest.approx(manifest["cases"][name]["auto_resolution"], rel=1e-12)


@pytest.mark.parametrize("name", case_names())
def test_serial_leiden_membership(name, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    case = manifest["cases"][name]
    memb, st = po.leiden(rp, col, case["auto_resolution"])
    np.testing.assert_array_equal(memb, golden_arrays[f"{name}/membership_serial"])
    assert [st.passes, st.iterations, st.communities] == case["serial_summary"]


@pytest.mark.parametrize("name", case_names())
@pytest.mark.parametrize("recipe", sorted(RECIPE_ARGS))
def test_compose_given_membership(name, recipe, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    memb = golden_arrays[f"{name}/membership_serial"]
    ids, st = po.compose(rp, col, memb, **RECIPE_ARGS[recipe])
    np.testing.assert_array_equal(ids, golden_arrays[f"{name}/compose_{recipe}"])
    gst = manifest["cases"][name]["compose"][recipe]["gorder_stats"]
    if RECIPE_ARGS[recipe]["intra_order"] == "gorder":
        assert [st.gorder_communities, st.gorder_vertices, st.gorder_max_community,
                st.fallback_communities, st.fallback_vertices] == gst


@pytest.mark.parametrize("name", case_names())
def test_end_to_end_serial_mapping(name, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    case = manifest["cases"][name]
    ids, _, _, _ = po.map_graph(rp, col, case["auto_resolution"])
    np.testing.assert_array_equal(ids, golden_arrays[f"{name}/new_ids_serial"])
    assert po.fingerprint(ids) == case["serial_fingerprint"]
    assert po.validate_permutation(ids) == 0


@pytest.mark.parametrize("name", case_names())
def test_relabel(name, golden_arrays):
    rp, col = graph(golden_arrays, name)
    ids = golden_arrays[f"{name}/new_ids_serial"]
    orp, ocol = po.relabel(rp, col, ids)
    np.testing.assert_array_equal(orp, golden_arrays[f"{name}/relabel_row_ptr"])
    np.testing.assert_array_equal(ocol, golden_arrays[f"{name}/relabel_col"])


def test_gorder_known_answer(manifest):
    # K4, window 5: the reference's own test expects local ids {0, 3, 2, 1}.
    rp = np.array([0, 3, 6, 9, 12], dtype=np.int64)
    col = np.array([1, 2, 3, 0, 2, 3, 0, 1, 3, 0, 1, 2], dtype=np.int32)
    ids, _ = po.compose(rp, col, np.zeros(4, dtype=np.uint32), "size-desc", "gorder", 5, 0)
    assert list(ids) == manifest["gorder_kat_k4_w5"] == [0, 3, 2, 1]


def test_validate_permutation_cases():
    assert po.validate_permutation(np.array([2, 0, 1], dtype=np.int32)) == 0
    assert po.validate_permutation(np.array([2, 3, 1], dtype=np.int32)) == 1
    assert po.validate_permutation(np.array([2, 2, 1], dtype=np.int32)) == 2
    # first failure in index order decides
    assert po.validate_permutation(np.array([0, 0, 5], dtype=np.int32)) == 2
    assert po.validate_permutation(np.array([5, 0, 0], dtype=np.int32)) == 1
    assert po.validate_permutation(np.array([], dtype=np.int32)) == 0


def test_fingerprint_empty_and_identity():
    assert po.fingerprint(np.array([], dtype=np.int32)) == "%016x" % 1469598103934665603
    a = po.fingerprint(np.arange(10, dtype=np.int32))
    b = po.fingerprint(np.arange(10, dtype=np.int32)[::-1].copy())
    assert a != b
