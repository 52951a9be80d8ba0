"""The oracle's restatements of the selector's inputs, pinned (CPU).

DBG and the Tier-0 features are checked against the reference's own outputs
(``golden/consumer_cases.npz``, made by ``golden/make_golden_consumers.py``
from the reference code); BFS and connected components against scipy's
independent graph routines; PageRank against its fixed-point equation.
"""
import json
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.csgraph as csg

import pyoracle as po
from graphbrew_gb300 import graphgen as gg
from conftest import GOLDEN, case_names


@pytest.fixture(scope="module")
def consumer():
    with open(os.path.join(GOLDEN, "consumer_manifest.json")) as f:
        man = json.load(f)
    return man, np.load(os.path.join(GOLDEN, "consumer_cases.npz"))


def generate(kind, kw):
    if kind == "rmat":
        return gg.rmat(kw["scale"], kw["edge_factor"], seed=kw["seed"])
    if kind == "uniform":
        return gg.uniform(kw["scale"], kw["edge_factor"], seed=kw["seed"])
    return gg.grid(kw["rows"], kw["cols"], kw["drop"], seed=kw["seed"])


def check_tier0(got: dict, want: list):
    vals = list(got.values())
    # Degree statistics and hub terms are summed in the reference's order: exact.
    assert vals[:7] == want[:7], (vals, want)
    np.testing.assert_allclose(vals[7], want[7], rtol=1e-12, atol=0)
    assert vals[8] == want[8]


@pytest.mark.parametrize("name", case_names())
def test_dbg_small(name, golden_arrays, consumer):
    rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
    np.testing.assert_array_equal(po.dbg_mapping(rp, col), consumer[1][f"{name}/dbg_ids"])


@pytest.mark.parametrize("name", case_names())
def test_tier0_small(name, golden_arrays, consumer):
    rp, col = golden_arrays[f"{name}/row_ptr"], golden_arrays[f"{name}/col"]
    check_tier0(po.tier0_features(rp, col), consumer[0]["small"][name]["tier0"])


@pytest.mark.parametrize("name", ["rmat18_e16", "grid1100", "urand20_e8"])
def test_generated(name, consumer):
    case = consumer[0]["generated"][name]
    rp, col = generate(case["kind"], case["kwargs"])
    rp, col = rp.numpy(), col.numpy()
    assert (len(rp) - 1, len(col)) == (case["n"], case["nnz"])
    assert po.fingerprint(po.dbg_mapping(rp, col)) == case["dbg_fingerprint"]
    check_tier0(po.tier0_features(rp, col), case["tier0"])


def _scipy_graph(rp, col):
    n = len(rp) - 1
    return sp.csr_matrix((np.ones(len(col)), col, rp), shape=(n, n))


@pytest.mark.parametrize("seed", [1, 2])
def test_bfs_and_cc_against_scipy(seed):
    # A graph with several components and isolated vertices.
    rp, col, _ = gg.planted_partition(3000, 6, degree=3, mixing=0.0, seed=seed)
    rp, col = rp.numpy(), col.numpy()
    A = _scipy_graph(rp, col)
    src = int(np.argmax(np.diff(rp)))
    dist = csg.shortest_path(A, unweighted=True, indices=src)
    want = np.where(np.isinf(dist), -1, dist).astype(np.int32)
    np.testing.assert_array_equal(po.bfs_depths(rp, col, src), want)
    ncomp, lab = csg.connected_components(A, directed=False)
    first = np.full(ncomp, len(rp), dtype=np.int64)
    np.minimum.at(first, lab, np.arange(len(rp) - 1))
    np.testing.assert_array_equal(po.cc_min_labels(rp, col), first[lab].astype(np.int32))
    assert ncomp > 1


def test_pagerank_fixed_point():
    rp, col = gg.rmat(10, 8, seed=9)
    rp, col = rp.numpy(), col.numpy()
    s = po.pagerank(rp, col, max_iters=500, epsilon=1e-14)
    n = len(rp) - 1
    deg = np.diff(rp).astype(np.float64)
    contrib = np.where(deg > 0, s / np.maximum(deg, 1), 0.0)
    inc = np.bincount(np.repeat(np.arange(n), np.diff(rp)), weights=contrib[col], minlength=n)
    np.testing.assert_allclose(s, 0.15 / n + 0.85 * inc, rtol=1e-10, atol=1e-15)


# ---- the OpenMP CPU kernels used to time the selector's arms on the host ----
@pytest.mark.parametrize("kind", ["planted", "rmat", "grid"])
def test_cpu_kernels_against_scipy(kind):
    if kind == "planted":
        rp, col, _ = gg.planted_partition(20000, 8, degree=4, mixing=0.01, seed=3)
    elif kind == "rmat":
        rp, col = gg.rmat(15, 8, seed=4)
    else:
        rp, col = gg.grid(150, 160, 0.1, seed=5)
    rp, col = rp.numpy(), col.numpy()
    A = _scipy_graph(rp, col)
    src = int(np.argmax(np.diff(rp)))
    dist = csg.shortest_path(A, unweighted=True, indices=src)
    want = np.where(np.isinf(dist), -1, dist).astype(np.int32)
    for threads in (1, 4):
        got, ms = po.bfs_cpu(rp, col, src, threads=threads)
        np.testing.assert_array_equal(got, want)
        assert ms >= 0
        comp, _ = po.cc_cpu(rp, col, threads=threads)
        _, labels = csg.connected_components(A, directed=False)
        # same partition: component ids map one to one
        pairs = set(zip(comp.tolist(), labels.tolist()))
        assert len(pairs) == len(set(comp.tolist())) == len(set(labels.tolist()))
    ids, _ = po.dbg_cpu(rp, col, threads=4)
    np.testing.assert_array_equal(ids, po.dbg_mapping(rp, col))


def test_cpu_pagerank_matches_fixed_point():
    rp, col = gg.rmat(14, 8, seed=6)
    rp, col = rp.numpy(), col.numpy()
    ref = po.pagerank(rp, col, max_iters=200, epsilon=1e-12)
    got, iters, ms = po.pagerank_cpu(rp, col, max_iters=200, epsilon=1e-9, threads=4)
    assert iters < 200 and ms >= 0
    # float32 scores, Gauss-Seidel sweeps: the same fixed point to float accuracy
    np.testing.assert_allclose(got, ref, rtol=2e-3, atol=1e-9)
