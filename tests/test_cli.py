"""gbconvert: the GAPBS converter lifecycle on the mapping path.

CPU: the native generators equal graphbrew_gb300.graphgen graph for graph,
and the .sg writer round-trips.  GPU: a cd_serial run's .lo labels and
"Mapping Fingerprint" equal the oracle's mapping on the same graph.
"""
import os
import subprocess

import numpy as np
import pytest

import pyoracle as po
from graphbrew_gb300 import graphgen as gg
from conftest import ROOT

CLI = os.path.join(ROOT, "graphbrew_gb300", "gbconvert")
SERIAL = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:"
          "sgmb4096:gordf5000:norefine:2:2")


def read_sg(path):
    b = open(path, "rb").read()
    ne = int(np.frombuffer(b[1:9], np.int64)[0])
    n = int(np.frombuffer(b[9:17], np.int64)[0])
    o = 17
    rp = np.frombuffer(b[o:o + 8 * (n + 1)], np.int64)
    o += 8 * (n + 1)
    col = np.frombuffer(b[o:o + 4 * ne], np.int32)
    o += 4 * ne
    org = np.frombuffer(b[o:o + 4 * n], np.int32)
    return rp, col, org


@pytest.fixture(scope="module")
def cli():
    if not os.path.exists(CLI):
        from graphbrew_gb300 import build
        build.build()
    return CLI


@pytest.mark.parametrize("flag,scale,deg,seed", [("-g", 11, 8, 3), ("-u", 10, 8, 11)])
def test_native_generators_match(cli, tmp_path, flag, scale, deg, seed):
    out = tmp_path / "g.sg"
    subprocess.run([cli, flag, str(scale), "-k", str(deg), "-r", str(seed), "-b", str(out)], check=True,
                   capture_output=True)
    rp, col, org = read_sg(out)
    ref = gg.rmat(scale, deg, seed=seed) if flag == "-g" else gg.uniform(scale, deg, seed=seed)
    np.testing.assert_array_equal(rp, ref[0].numpy())
    np.testing.assert_array_equal(col, ref[1].numpy())
    np.testing.assert_array_equal(org, np.arange(len(rp) - 1, dtype=np.int32))


def test_el_input_and_sg_roundtrip(cli, tmp_path):
    el = tmp_path / "t.el"
    el.write_text("0 1\n1 2\n2 3\n3 0\n0 2\n4 4\n")
    sg = tmp_path / "t.sg"
    subprocess.run([cli, "-f", str(el), "-s", "-b", str(sg)], check=True, capture_output=True)
    rp, col, _ = read_sg(sg)
    exp_rp, exp_col = gg.from_edges(5, [(0, 1), (1, 2), (2, 3), (3, 0), (0, 2), (4, 4)])
    np.testing.assert_array_equal(rp, exp_rp.numpy())
    np.testing.assert_array_equal(col, exp_col.numpy())
    sg2 = tmp_path / "t2.sg"
    subprocess.run([cli, "-f", str(sg), "-b", str(sg2)], check=True, capture_output=True)
    assert open(sg, "rb").read() == open(sg2, "rb").read()


@pytest.mark.gpu
def test_cli_serial_mapping_lifecycle(cli, tmp_path):
    lo = tmp_path / "map.lo"
    r = subprocess.run([cli, "-g", "12", "-k", "16", "-r", "12", "-o", "12:" + SERIAL, "-q", str(lo)],
                       check=True, capture_output=True, text=True)
    rp, col = gg.rmat(12, 16, seed=12)
    rp, col = rp.numpy(), col.numpy()
    # The CLI computes the automatic resolution on the device; the oracle runs
    # with the exact value it printed in its effective config.
    import json
    line = next(l for l in r.stdout.splitlines() if l.startswith("GraphBrew Effective Config: "))
    res = json.loads(line[len("GraphBrew Effective Config: "):])["resolution"]
    assert res == pytest.approx(po.auto_resolution(rp, col), rel=1e-12)
    ids, _, _, _ = po.map_graph(rp, col, res)
    labels = np.array([int(x) for x in lo.read_text().split()], dtype=np.int32)
    org = np.empty_like(ids)
    org[ids] = np.arange(len(ids), dtype=np.int32)
    np.testing.assert_array_equal(labels, org)
    assert f"Mapping Fingerprint: {po.fingerprint(ids)}" in r.stdout
    for label in ("Reorder Core Time", "Reorder Validation Time", "Reorder Apply Time", "Reorder End-to-End Time"):
        assert label + ":" in r.stdout


@pytest.mark.parametrize("flag,scale", [("-g", 12), ("-u", 11)])
def test_gapbs_generator_without_seed(cli, tmp_path, flag, scale):
    """Without -r, -g/-u build GAPBS's own graph (the converter's)."""
    out = tmp_path / "g.sg"
    subprocess.run([cli, flag, str(scale), "-b", str(out)], check=True, capture_output=True)
    rp, col, _ = read_sg(out)
    erp, ecol = po.gapbs_graph(scale, 16, uniform=(flag == "-u"))
    np.testing.assert_array_equal(rp, erp)
    np.testing.assert_array_equal(col, ecol)


@pytest.mark.gpu
def test_cli_gapbs_g16_prints_the_converters_fingerprint(cli):
    """`gbconvert -g 16 -s -o 12:<cd_serial recipe>` prints the fingerprint the
    reference's `converter` printed for the same command (9b52c0603aacbbdb)."""
    r = subprocess.run([cli, "-g", "16", "-s", "-o", "12:" + SERIAL], check=True, capture_output=True, text=True)
    assert "Mapping Fingerprint: 9b52c0603aacbbdb" in r.stdout
