"""GAPBS's own synthetic graphs and the reference's answers on them.

``graphgen.gapbs`` must build exactly the graph the reference's converter
builds for ``-g <scale>`` / ``-u <scale>`` (generator.h:101-164, builder.h
squish), and the oracle must map GAPBS ``-g 16 / 20 / 22`` to the permutation
whose "Mapping Fingerprint" the reference's converter printed with the
cd_serial recipe (9b52c0603aacbbdb, 1bb16f3ac238f77f, 91a0f15d18ec743d).
The values come from ``tests/golden/make_golden_gapbs.py`` (reference harness);
these tests need only the committed pins, so they also run where the
reference is absent.
"""
import json
import os

import numpy as np
import pytest
import torch

import pyoracle as po
from graphbrew_gb300 import graphgen as gg

HERE = os.path.dirname(os.path.abspath(__file__))
PINS = json.load(open(os.path.join(HERE, "golden", "gapbs_pins.json")))


def _ck(a):
    return gg.checksum(torch.from_numpy(np.ascontiguousarray(a)))


@pytest.mark.parametrize("kind,scale", [("rmat", s) for s in (10, 12, 14, 16, 18, 20)] +
                         [("uniform", s) for s in (10, 14, 18, 20)])
def test_generator_builds_the_reference_graph(kind, scale):
    rp, col = gg.gapbs(scale, 16, uniform=(kind == "uniform"))
    pin = PINS[kind][str(scale)]
    assert rp.numel() - 1 == pin["n"] and col.numel() == pin["nnz"]
    assert gg.checksum(rp) == pin["row_ptr"] and gg.checksum(col) == pin["col"]


@pytest.mark.parametrize("kind,scale", [("rmat", 12), ("uniform", 14), ("rmat", 20)])
def test_oracle_side_builder_builds_the_reference_graph(kind, scale):
    rp, col = po.gapbs_graph(scale, 16, uniform=(kind == "uniform"))
    pin = PINS[kind][str(scale)]
    assert _ck(rp) == pin["row_ptr"] and _ck(col) == pin["col"]


@pytest.mark.skipif(po.load_reference() is None, reason="reference harness not built here")
@pytest.mark.parametrize("kind,scale", [("rmat", 11), ("uniform", 12), ("rmat", 17)])
def test_generator_equals_reference_builder_live(kind, scale):
    rp, col = gg.gapbs(scale, 8 if scale == 11 else 16, uniform=(kind == "uniform"))
    rrp, rcol = po.ref_gapbs_graph(scale, 8 if scale == 11 else 16, uniform=(kind == "uniform"))
    np.testing.assert_array_equal(rp.numpy(), rrp)
    np.testing.assert_array_equal(col.numpy(), rcol)


def test_edge_count_rejects_bad_arguments():
    from graphbrew_gb300 import library
    assert library().gbgpu_gapbs_edge_count(31, 16) == -1
    assert library().gbgpu_gapbs_edge_count(4, -1) == -1
    assert library().gbgpu_gapbs_edge_count(4, 16) == 256


@pytest.mark.parametrize("scale", [16, 20, 22])
def test_oracle_maps_gapbs_rmat_to_the_reference_fingerprint(scale):
    """The headline graph (-g 22) included: the oracle's cd_serial mapping and
    relabelled CSR are the reference's, by fingerprint and checksums."""
    pin = PINS["rmat"][str(scale)]
    rp, col = po.gapbs_graph(scale, 16)
    # The reference's resolution sums degrees in OpenMP reduction order; the
    # oracle's agrees to 1e-12 relative, and the mapping uses the reference's.
    assert po.auto_resolution(rp, col) == pytest.approx(pin["auto_resolution"], rel=1e-12)
    ids, _, _, _ = po.map_graph(rp, col, pin["auto_resolution"], parallel=False, threads=0)
    assert po.fingerprint(ids) == pin["fingerprint_cd_serial"]
    orp, ocol = po.relabel(rp, col, ids)
    assert _ck(orp) == pin["relabel_row_ptr"] and _ck(ocol) == pin["relabel_col"]
