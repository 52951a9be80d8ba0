"""The oracle against the reference itself, run live.

Skipped where the reference harness (oracle/_ref/libgbref.so) was not built:
it compiles from the GraphBrew headers, which only the development container
has.  The committed golden fixtures cover the same ground everywhere else.
"""
import numpy as np
import pytest

import pyoracle as po
from graphbrew_gb300 import graphgen as gg

pytestmark = pytest.mark.skipif(po.load_reference() is None, reason="reference harness not built here")

SERIAL = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:"
          "sgmb4096:gordf5000:norefine:2:2")


def _check(rp, col, fallback=5000):
    rp, col = np.ascontiguousarray(rp), np.ascontiguousarray(col)
    ar = po.load_reference().ref_auto_resolution(len(rp) - 1, rp, col)
    recipe = SERIAL.replace("gordf5000", f"gordf{fallback}")
    ref_ids = po.ref_generate_mapping(rp, col, recipe, ar)
    ids, _, _, _ = po.map_graph(rp, col, ar, gorder_fallback=fallback)
    np.testing.assert_array_equal(ids, ref_ids)
    orp, ocol = po.relabel(rp, col, ids)
    rrp, rcol, _ = po.ref_relabel(rp, col, ids)
    np.testing.assert_array_equal(orp, rrp)
    np.testing.assert_array_equal(ocol, rcol)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_rmat_seeds(seed):
    rp, col = gg.rmat(11, 16, seed=seed)
    _check(rp.numpy(), col.numpy(), fallback=200)


@pytest.mark.parametrize("seed", [7, 8])
def test_planted_and_grid(seed):
    rp, col, _ = gg.planted_partition(6000, 8, seed=seed)
    _check(rp.numpy(), col.numpy(), fallback=300)
    rp, col = gg.grid(30 + seed, 41, seed=seed)
    _check(rp.numpy(), col.numpy(), fallback=50)


def test_gapbs_g16_serial_fingerprint():
    # Measured with the reference's converter (-g 16, cd_serial, 1 and 8 threads).
    rp, col = po.ref_gapbs_graph(16)
    ar = po.load_reference().ref_auto_resolution(len(rp) - 1, rp, col)
    ids, _, _, cst = po.map_graph(rp, col, ar)
    assert po.fingerprint(ids) == "9b52c0603aacbbdb"
    assert cst.fallback_communities == 1  # one community above 5000 -> BFS


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_super_orders_and_random_intra_live(seed):
    """sg_super_rcm / sg_super_rabbit / sg_hilbert and intra_random against
    the reference run live with one thread, on random memberships (from a
    few large communities to many small ones), community orders size-desc
    and identity."""
    rng = np.random.default_rng(seed)
    rp, col = gg.rmat(12 + seed % 3, 12, seed=seed)
    rp, col = rp.numpy(), col.numpy()
    n = len(rp) - 1
    k = [3, 40, 900][seed % 3]
    memb = rng.integers(0, k, size=n).astype(np.uint32)
    memb[rng.random(n) < 0.3] = 0   # one community far larger than the rest
    for sup, tok in (("super-rcm", "sg_super_rcm"), ("super-rabbit", "sg_super_rabbit"), ("hilbert", "sg_hilbert")):
        for comm, ctok in (("size-desc", "comm_size_desc"), ("identity", "comm_identity")):
            opts = f"leiden:compose:{tok}:{ctok}:intra_bfs:cd_serial:norefine:2:2"
            ref = po.ref_compose(rp, col, memb, opts, 1.0, threads=1)[0]
            ids, _ = po.compose(rp, col, memb, comm, "bfs", super_order=sup)
            np.testing.assert_array_equal(ids, ref, err_msg=f"{sup} {comm}")
    opts = "leiden:compose:sg_none:comm_size_desc:intra_random:cd_serial:norefine:2:2"
    ids, _ = po.compose(rp, col, memb, "size-desc", "random")
    np.testing.assert_array_equal(ids, po.ref_compose(rp, col, memb, opts, 1.0, threads=1)[0])
