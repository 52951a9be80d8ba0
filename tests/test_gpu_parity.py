"""CUDA path against the oracle and the reference's golden outputs (GB300).

Integer work is bit-exact: orderCompose (placement, Gorder, BFS fallback),
RelabelByMapping, validation and the fingerprint must equal the reference's
outputs on the same membership.  Community detection in cd_parallel mode is
nondeterministic in the reference itself, so it is judged by invariants
(a valid membership whose community totals match, a valid permutation) and
by modularity against the reference's own run-to-run spread.
"""
import numpy as np
import pytest
import torch

import pyoracle as po
import graphbrew_gb300 as gb
from graphbrew_gb300 import graphgen as gg
from conftest import case_names

pytestmark = pytest.mark.gpu

SERIAL = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_serial:"
          "sgmb4096:gordf5000:norefine:2:2")
PARALLEL = SERIAL.replace("cd_serial", "cd_parallel")


@pytest.fixture(scope="module")
def ctx():
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    c = gb.Context(0)
    yield c
    c.close()


def graph(g, name):
    return g[f"{name}/row_ptr"], g[f"{name}/col"]


def to_dev(*arrays):
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


@pytest.mark.parametrize("name", case_names())
def test_compose_bit_exact(ctx, name, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    memb = golden_arrays[f"{name}/membership_serial"]
    for key, recipe in manifest["compose_recipes"].items():
        ids, st = ctx.order_compose(rp, col, memb, recipe)
        np.testing.assert_array_equal(ids, golden_arrays[f"{name}/compose_{key}"], err_msg=f"{name}/{key}")
        if "intra_gorder" in recipe:
            gst = manifest["cases"][name]["compose"][key]["gorder_stats"]
            assert [st["gorder_communities"], st["gorder_vertices"], st["gorder_max_community"],
                    st["fallback_communities"], st["fallback_vertices"]] == gst


@pytest.mark.parametrize("name", case_names())
def test_compose_device_pointers(ctx, name, golden_arrays):
    rp, col = graph(golden_arrays, name)
    memb = golden_arrays[f"{name}/membership_serial"].astype(np.int32)
    drp, dcol, dmemb = to_dev(rp, col, memb)
    ids, _ = ctx.order_compose(drp, dcol, dmemb, SERIAL)
    assert ids.is_cuda
    np.testing.assert_array_equal(ids.cpu().numpy(), golden_arrays[f"{name}/compose_gorder8_f5000"])


@pytest.mark.parametrize("name", case_names())
def test_relabel_bit_exact(ctx, name, golden_arrays):
    rp, col = graph(golden_arrays, name)
    ids = golden_arrays[f"{name}/new_ids_serial"]
    orp, ocol, org = ctx.relabel_by_mapping(rp, col, ids)
    np.testing.assert_array_equal(orp, golden_arrays[f"{name}/relabel_row_ptr"])
    np.testing.assert_array_equal(ocol, golden_arrays[f"{name}/relabel_col"])
    np.testing.assert_array_equal(org, golden_arrays[f"{name}/relabel_org_ids"])


def test_validate_permutation(ctx):
    assert ctx.validate_permutation(np.array([2, 0, 1], dtype=np.int32)) == 0
    assert ctx.validate_permutation(np.array([2, 3, 1], dtype=np.int32)) == 1
    assert ctx.validate_permutation(np.array([2, 2, 1], dtype=np.int32)) == 2
    assert ctx.validate_permutation(np.array([0, 0, 5], dtype=np.int32)) == 2
    assert ctx.validate_permutation(np.array([5, 0, 0], dtype=np.int32)) == 1
    assert ctx.validate_permutation(np.array([-1, 0, 1], dtype=np.int32)) == 1
    assert ctx.validate_permutation(np.array([], dtype=np.int32)) == 0
    big = np.random.default_rng(0).permutation(1 << 20).astype(np.int32)
    assert ctx.validate_permutation(torch.from_numpy(big).cuda()) == 0
    big[12345] = big[777]
    assert ctx.validate_permutation(big) == 2


def test_relabel_every_row_class(ctx):
    """Rows on both sides of each relabel class boundary (thread 16, warp 256,
    256-thread CTA 2,048, 1,024-thread CTA 16,384, global sort above)."""
    rng = np.random.default_rng(11)
    n = 60000
    src, dst = [], []
    for hub, d in enumerate([16, 17, 256, 257, 2048, 2049, 16384, 16385, 30000, 5000, 700]):
        nb = rng.choice(np.arange(20, n), d, replace=False)
        src.append(np.full(d, hub))
        dst.append(nb)
    e = rng.integers(20, n, size=(200000, 2))
    src.append(e[:, 0])
    dst.append(e[:, 1])
    s_ = np.concatenate(src + dst)
    d_ = np.concatenate(dst + src)
    keep = s_ != d_
    key = np.unique(s_[keep].astype(np.int64) * n + d_[keep])
    rows, cols = key // n, (key % n).astype(np.int32)
    rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rp, rows + 1, 1)
    rp = np.cumsum(rp)
    deg = np.diff(rp)
    for d in (16, 17, 256, 257, 2048, 2049, 16384, 16385):
        assert d in set(deg[:11].tolist())
    ids = rng.permutation(n).astype(np.int32)
    orp, ocol, _ = ctx.relabel_by_mapping(rp, cols, ids)
    erp, ecol = po.relabel(rp, cols, ids)
    np.testing.assert_array_equal(orp, erp)
    np.testing.assert_array_equal(ocol, ecol)


def test_relabel_rejects_non_permutation(ctx):
    rp = np.array([0, 1, 2], dtype=np.int64)
    col = np.array([1, 0], dtype=np.int32)
    with pytest.raises(RuntimeError, match="duplicate"):
        ctx.relabel_by_mapping(rp, col, np.array([0, 0], dtype=np.int32))


def _chunked_graph():
    """Valid squished CSR whose rows cross the input check's 4096-entry
    chunks, with runs of empty rows and a row that starts exactly on a chunk
    boundary after a row ending in a larger id."""
    rng = np.random.default_rng(7)
    n = 50000
    deg = rng.integers(0, 40, n)
    deg[100:5000] = 0
    deg[7] = 9000
    rp = np.zeros(n + 1, dtype=np.int64)
    rp[1:] = np.cumsum(deg)
    # Move degree so that some row begins at entry 4096 * 3.
    k = int(np.searchsorted(rp, 4096 * 3))
    shift = 4096 * 3 - int(rp[k - 1])
    deg[k - 1] = shift
    rp[1:] = np.cumsum(deg)
    col = np.concatenate([np.sort(rng.choice(n, int(d), replace=False)) for d in deg]).astype(np.int32)
    return rp, col, k - 1


def test_input_check_accepts_and_rejects(ctx):
    rp, col, row = _chunked_graph()
    assert 4096 * 3 in set(rp.tolist())
    ctx.connected_components(rp, col)
    dcol = torch.from_numpy(col).cuda()
    ctx.connected_components(torch.from_numpy(rp).cuda(), dcol)
    # One descending pair inside a row, right across a chunk boundary.
    assert 4096 * 5 not in set(rp.tolist())
    bad = col.copy()
    bad[4096 * 5] = bad[4096 * 5 - 1]
    with pytest.raises(ValueError, match="sorted ascending"):
        ctx.connected_components(rp, bad)
    bad = col.copy()
    bad[-1] = len(rp) - 1
    with pytest.raises(ValueError, match="out of range"):
        ctx.connected_components(rp, bad)
    bad = col.copy()
    bad[4096 * 2 + 5] = -3
    with pytest.raises(ValueError, match="out of range"):
        ctx.connected_components(rp, bad)
    small = np.array([0, 2, 3, 4], dtype=np.int64)
    with pytest.raises(ValueError, match="sorted ascending"):
        ctx.connected_components(small, np.array([2, 1, 0, 0], dtype=np.int32))
    with pytest.raises(ValueError, match="sorted ascending"):
        ctx.connected_components(small, np.array([1, 1, 0, 0], dtype=np.int32))
    with pytest.raises(ValueError, match="row offsets"):
        ctx.connected_components(np.array([0, 3, 1, 4], dtype=np.int64), np.array([0, 1, 2, 0], dtype=np.int32))
    with pytest.raises(ValueError, match="row offsets"):
        ctx.connected_components(np.array([1, 2, 3, 4], dtype=np.int64), np.array([1, 2, 0, 0], dtype=np.int32))


@pytest.mark.parametrize("name", case_names())
def test_auto_resolution(ctx, name, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    assert ctx.auto_resolution(rp, col) == pytest.approx(manifest["cases"][name]["auto_resolution"], rel=1e-12)


@pytest.mark.parametrize("name", case_names())
def test_serial_leiden_bit_exact(ctx, name, manifest, golden_arrays):
    """cd_serial community detection equals the reference's, id for id."""
    rp, col = graph(golden_arrays, name)
    case = manifest["cases"][name]
    memb, st = ctx.run_graphbrew(rp, col, SERIAL, case["auto_resolution"])
    np.testing.assert_array_equal(memb, golden_arrays[f"{name}/membership_serial"])
    assert [st["passes"], st["iterations"], st["communities"]] == case["serial_summary"]


@pytest.mark.parametrize("name", case_names())
def test_serial_mapping_bit_exact(ctx, name, manifest, golden_arrays):
    """The whole cd_serial mapping equals the reference's (and its fingerprint)."""
    rp, col = graph(golden_arrays, name)
    case = manifest["cases"][name]
    ids, _ = ctx.generate_mapping(rp, col, SERIAL, case["auto_resolution"])
    np.testing.assert_array_equal(ids, golden_arrays[f"{name}/new_ids_serial"])
    assert gb.mapping_fingerprint(ids) == case["serial_fingerprint"]


@pytest.mark.parametrize("scale,window", [(14, 8192), (16, 32768), (16, 1024), (18, 4096), (20, 8192),
                                          (20, 32768), (18, 65536)])
def test_serial_engine_against_oracle(ctx, scale, window, monkeypatch):
    """Serial-order engine at larger sizes and window settings: bit-exact."""
    monkeypatch.setenv("GBGPU_EXACT_WINDOW", str(window))
    rp_t, col_t = gg.rmat(scale, 16, seed=200 + scale, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, st = ctx.run_graphbrew(rp_t, col_t, SERIAL, ar)
    m_orc, ost = po.leiden(rp, col, ar)
    np.testing.assert_array_equal(memb.cpu().numpy().view(np.uint32), m_orc)
    assert [st["passes"], st["iterations"]] == [ost.passes, ost.iterations]
    ids, _ = ctx.generate_mapping(rp_t, col_t, SERIAL, ar)
    ids_orc, _ = po.compose(rp, col, m_orc)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)


def test_serial_engine_host_driven_rounds(ctx, monkeypatch):
    """Rounds enqueued from the host (no device-side loop): same membership."""
    monkeypatch.setenv("GBGPU_EXACT_GRAPH", "0")
    rp_t, col_t = gg.rmat(16, 16, seed=216, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, st = ctx.run_graphbrew(rp_t, col_t, SERIAL, ar)
    m_orc, _ = po.leiden(rp, col, ar)
    np.testing.assert_array_equal(memb.cpu().numpy().view(np.uint32), m_orc)
    assert st["local_move_rounds"] > 0


def test_parallel_recipe_is_serial_order(ctx):
    """cd_parallel runs the serial-order engine: same membership as cd_serial
    and as the oracle's serial sweep, on a graph with multi-segment hubs."""
    rp_t, col_t = gg.rmat(19, 16, seed=77, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    assert np.diff(rp).max() > 4 * 4096
    ar = po.auto_resolution(rp, col)
    m_par, _ = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    m_ser, _ = ctx.run_graphbrew(rp_t, col_t, SERIAL, ar)
    np.testing.assert_array_equal(m_par.cpu().numpy(), m_ser.cpu().numpy())
    m_orc, _ = po.leiden(rp, col, ar)
    np.testing.assert_array_equal(m_par.cpu().numpy().view(np.uint32), m_orc)


@pytest.mark.parametrize("family", ["urand", "grid"])
def test_weak_structure_graphs_bit_exact(ctx, family):
    """Uniform-random and grid graphs (weak community structure, long BFS
    chains): the whole mapping equals the oracle's serial-order result."""
    if family == "urand":
        rp_t, col_t = gg.uniform(17, 16, seed=31, device="cuda")
    else:
        rp_t, col_t = gg.grid(400, 400, 0.05, seed=32, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, st = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    m_orc, ost = po.leiden(rp, col, ar)
    np.testing.assert_array_equal(memb.cpu().numpy().view(np.uint32), m_orc)
    ids, _ = ctx.generate_mapping(rp_t, col_t, PARALLEL, ar)
    ids_orc, _ = po.compose(rp, col, m_orc)
    np.testing.assert_array_equal(ids.cpu().numpy(), ids_orc)


@pytest.mark.parametrize("family", ["urand23", "grid4096"])
def test_full_size_weak_structure_graphs(ctx, family):
    """The full-size uniform (2^23 vertices, degree 16) and 4096 x 4096 grid
    graphs: a valid permutation, relabelled CSR with the same entry count."""
    if family == "urand23":
        rp_t, col_t = gg.uniform(23, 16, seed=27491095, device="cuda")
    else:
        rp_t, col_t = gg.grid(4096, 4096, 0.05, seed=27491095, device="cuda")
    ids, orp, ocol, st = ctx.map_and_relabel(rp_t, col_t, PARALLEL)
    assert ctx.validate_permutation(ids) == 0
    assert int(orp[-1].item()) == col_t.numel() and ocol.numel() == col_t.numel()
    assert st["passes"] <= 2 and st["communities"] > 1
    del ids, orp, ocol
    # Quality floor at full size (resolution 1): on the grid cd_parallel runs
    # the racy stream mode, so its result varies from run to run; the oracle's
    # restatement of the reference's cd_parallel reaches 0.50 there (8 and 16
    # threads), the serial order 0.536.  Uniform: the serial order gives 0.047.
    memb, _ = ctx.run_graphbrew(rp_t, col_t, PARALLEL)
    q = po.modularity(rp_t.cpu().numpy(), col_t.cpu().numpy(), memb.cpu().numpy().view(np.uint32), 1.0)
    assert q >= (0.49 if family == "grid4096" else 0.045), (family, q)


def test_async_engine_quality(ctx, monkeypatch):
    """The asynchronous cd_parallel engine stays close to the serial result."""
    monkeypatch.setenv("GBGPU_EXACT_MAX_VERTICES", "0")
    rp_t, col_t = gg.rmat(17, 16, seed=5, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, _ = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    q = po.modularity(rp, col, memb.cpu().numpy().view(np.uint32), 1.0)
    m_ser, _ = po.leiden(rp, col, ar)
    q_ser = po.modularity(rp, col, m_ser, 1.0)
    assert q >= q_ser - 0.02, (q, q_ser)
    ids, _ = ctx.generate_mapping(rp_t, col_t, PARALLEL, ar)
    assert ctx.validate_permutation(ids) == 0


def test_async_single_stream_is_serial(ctx, monkeypatch):
    """Stream mode with one stream sweeps every vertex in id order with each
    move visible to the next: on a graph without hubs that is the serial
    sweep (cd_serial, reorder_graphbrew.h:7330-7392), bit for bit."""
    monkeypatch.setenv("GBGPU_EXACT_MAX_VERTICES", "0")
    monkeypatch.setenv("GBGPU_ASYNC_STREAMS", "1")
    rp_t, col_t = gg.grid(96, 96, 0.05, seed=11, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, _ = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    want, _ = po.leiden(rp, col, ar)
    np.testing.assert_array_equal(memb.cpu().numpy().view(np.uint32), want)


@pytest.mark.parametrize("streams", ["304", "1216"])
def test_async_streams_quality_on_grid(ctx, monkeypatch, streams):
    """Stream mode (each warp sweeps its own block in order) keeps the serial
    sweep's modularity on high-locality graphs, where chunk mode loses it,
    while each block spans about a grid row or more (862 and 216 vertices
    here, rows of 512)."""
    monkeypatch.setenv("GBGPU_EXACT_MAX_VERTICES", "0")
    monkeypatch.setenv("GBGPU_ASYNC_STREAMS", streams)
    rp_t, col_t = gg.grid(512, 512, 0.05, seed=12, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    memb, _ = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    m = memb.cpu().numpy().view(np.uint32)
    _check_membership(rp, col, m)
    q = po.modularity(rp, col, m, 1.0)
    m_ser, _ = po.leiden(rp, col, ar)
    q_ser = po.modularity(rp, col, m_ser, 1.0)
    assert q >= q_ser - 0.01, (q, q_ser)
    ids, _ = ctx.generate_mapping(rp_t, col_t, PARALLEL, ar)
    assert ctx.validate_permutation(ids) == 0


def test_auto_stream_mode_on_high_locality_graphs(ctx, monkeypatch):
    """cd_parallel picks the stream mode on large graphs whose neighbours sit
    at nearby ids (a 1024 x 1024 grid) and keeps the serial order's
    modularity; GBGPU_ASYNC_AUTO=0 keeps the serial-order engine, bit for
    bit; RMAT (no id locality) keeps it by itself."""
    rp_t, col_t = gg.grid(1024, 1024, 0.05, seed=13, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    ar = po.auto_resolution(rp, col)
    m_ser, _ = po.leiden(rp, col, ar)
    q_ser = po.modularity(rp, col, m_ser, 1.0)
    memb, st = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    assert st["local_move_streams"] >= 1216
    m = memb.cpu().numpy().view(np.uint32)
    _check_membership(rp, col, m)
    q = po.modularity(rp, col, m, 1.0)
    assert q >= q_ser - 0.01, (q, q_ser)
    ids, st = ctx.generate_mapping(rp_t, col_t, PARALLEL, ar)
    assert ctx.validate_permutation(ids) == 0
    monkeypatch.setenv("GBGPU_ASYNC_AUTO", "0")
    memb, st = ctx.run_graphbrew(rp_t, col_t, PARALLEL, ar)
    assert st["local_move_streams"] == 0
    np.testing.assert_array_equal(memb.cpu().numpy().view(np.uint32), m_ser)
    monkeypatch.delenv("GBGPU_ASYNC_AUTO")
    rp_t, col_t = gg.rmat(20, 16, seed=14, device="cuda")
    _, st = ctx.run_graphbrew(rp_t, col_t, PARALLEL)
    assert st["local_move_streams"] == 0


def _check_membership(rp, col, memb):
    n = len(rp) - 1
    assert memb.shape == (n,)
    assert (memb.astype(np.int64) < n).all()


@pytest.mark.parametrize("name", case_names())
def test_parallel_leiden_and_mapping(ctx, name, manifest, golden_arrays):
    rp, col = graph(golden_arrays, name)
    case = manifest["cases"][name]
    ar = case["auto_resolution"]
    memb, st = ctx.run_graphbrew(rp, col, PARALLEL, ar)
    _check_membership(rp, col, memb)
    assert st["passes"] <= 2
    q = po.modularity(rp, col, memb, 1.0)
    ref_q = case["parallel_modularity_samples"] + [case["serial_modularity"]]
    # The reference's own parallel runs spread widely on some graphs; the GPU
    # result must not fall meaningfully below the worst of them.
    assert q >= min(ref_q) - 0.02, (q, ref_q)
    # Given the GPU membership, COMPOSE is exact against the oracle.
    ids_gpu, _ = ctx.order_compose(rp, col, memb, PARALLEL)
    ids_orc, _ = po.compose(rp, col, memb)
    np.testing.assert_array_equal(ids_gpu, ids_orc)
    ids, st2 = ctx.generate_mapping(rp, col, PARALLEL, ar)
    assert po.validate_permutation(ids) == 0


@pytest.mark.parametrize("scale,fallback", [(14, 5000), (16, 5000), (16, 300), (18, 5000)])
def test_seeded_rmat_against_oracle(ctx, scale, fallback):
    rp_t, col_t = gg.rmat(scale, 16, seed=100 + scale, device="cuda")
    rp, col = rp_t.cpu().numpy(), col_t.cpu().numpy()
    recipe = PARALLEL.replace("gordf5000", f"gordf{fallback}")
    ar = po.auto_resolution(rp, col)
    memb, st = ctx.run_graphbrew(rp_t, col_t, recipe, ar)
    memb = memb.cpu().numpy().view(np.uint32)
    _check_membership(rp, col, memb)
    ids_gpu, cst = ctx.order_compose(rp_t, col_t, torch.from_numpy(memb.view(np.int32)).cuda(), recipe)
    ids_orc, ost = po.compose(rp, col, memb, gorder_fallback=fallback)
    np.testing.assert_array_equal(ids_gpu.cpu().numpy(), ids_orc)
    assert cst["fallback_communities"] == ost.fallback_communities
    orp, ocol, _ = ctx.relabel_by_mapping(rp_t, col_t, ids_gpu)
    erp, ecol = po.relabel(rp, col, ids_orc)
    np.testing.assert_array_equal(orp.cpu().numpy(), erp)
    np.testing.assert_array_equal(ocol.cpu().numpy(), ecol)
    q_gpu = po.modularity(rp, col, memb, 1.0)
    m_ser, _ = po.leiden(rp, col, ar)
    q_ser = po.modularity(rp, col, m_ser, 1.0)
    assert q_gpu >= q_ser - 0.03, (q_gpu, q_ser)


def test_edge_cases(ctx):
    # empty graph
    ids, _ = ctx.generate_mapping(np.zeros(1, dtype=np.int64), np.zeros(0, dtype=np.int32), PARALLEL, 1.0)
    assert len(ids) == 0
    # all isolated
    ids, _ = ctx.generate_mapping(np.zeros(6, dtype=np.int64), np.zeros(0, dtype=np.int32), PARALLEL, 1.0)
    assert list(ids) == [0, 1, 2, 3, 4]
    # one edge + isolated tail
    rp, col = gg.from_edges(4, [(1, 2)])
    ids, _ = ctx.generate_mapping(rp.numpy(), col.numpy(), PARALLEL, 1.0)
    memb, _ = ctx.run_graphbrew(rp.numpy(), col.numpy(), PARALLEL, 1.0)
    np.testing.assert_array_equal(ids, po.compose(rp.numpy(), col.numpy(), memb)[0])


@pytest.mark.parametrize("hub_degree", [40, 700, 3000, 20000, 70000])
def test_hub_vertices(ctx, hub_degree):
    # A star plus a ring: exercises register, shared-table and global-table
    # accumulation, the CTA row sort and the long-row radix sort.
    n = hub_degree + 1
    edges = [(0, i) for i in range(1, n)] + [(i, i + 1) for i in range(1, n - 1)]
    rp_t, col_t = gg.from_edges(n, edges)
    rp, col = rp_t.numpy(), col_t.numpy()
    memb, _ = ctx.run_graphbrew(rp, col, PARALLEL, 1.0)
    ids_gpu, _ = ctx.order_compose(rp, col, memb, PARALLEL.replace("gordf5000", "gordf100"))
    ids_orc, _ = po.compose(rp, col, memb, gorder_fallback=100)
    np.testing.assert_array_equal(ids_gpu, ids_orc)
    orp, ocol, _ = ctx.relabel_by_mapping(rp, col, ids_orc)
    erp, ecol = po.relabel(rp, col, ids_orc)
    np.testing.assert_array_equal(orp, erp)
    np.testing.assert_array_equal(ocol, ecol)


def test_large_community_gorder_paths(ctx):
    # Communities of 20..6000 vertices: thread, shared-memory and global
    # UnitHeap variants, against the oracle.
    rp_t, col_t, planted = gg.planted_partition(60000, 12, degree=10, mixing=0.02, seed=9)
    rp, col = rp_t.numpy(), col_t.numpy()
    memb = planted.numpy().astype(np.uint32)
    for fallback in (8000, 100000):
        recipe = PARALLEL.replace("gordf5000", f"gordf{fallback}")
        ids_gpu, st = ctx.order_compose(rp, col, memb, recipe)
        ids_orc, ost = po.compose(rp, col, memb, gorder_fallback=fallback)
        np.testing.assert_array_equal(ids_gpu, ids_orc)
        assert st["gorder_max_community"] == ost.gorder_max_community


def test_unsupported_and_bad_options(ctx):
    rp, col = gg.from_edges(3, [(0, 1), (1, 2)])
    with pytest.raises(NotImplementedError):
        ctx.generate_mapping(rp.numpy(), col.numpy(), "leiden", 1.0)  # LAYER ordering
    with pytest.raises(ValueError):
        ctx.generate_mapping(rp.numpy(), col.numpy(), "leiden:compose:sgmb0", 1.0)
    with pytest.raises(ValueError):
        ctx.generate_mapping(np.array([0, 5], dtype=np.int64), np.zeros(1, dtype=np.int32), PARALLEL, 1.0)


def test_graph_generator_cpu_gpu_identical():
    a = gg.rmat(12, 8, seed=3)
    b = gg.rmat(12, 8, seed=3, device="cuda")
    assert torch.equal(a[0], b[0].cpu()) and torch.equal(a[1], b[1].cpu())


def test_map_and_relabel_lifecycle(ctx, golden_arrays):
    rp, col = graph(golden_arrays, "rmat12")
    ids, orp, ocol, st = ctx.map_and_relabel(rp, col, PARALLEL)
    assert po.validate_permutation(ids) == 0
    erp, ecol = po.relabel(rp, col, ids)
    np.testing.assert_array_equal(orp, erp)
    np.testing.assert_array_equal(ocol, ecol)
    assert st["total_ms"] > 0 and st["kernel_launches"] > 0


@pytest.mark.parametrize("M,R", [
    (64155273.0, 1.0),            # RMAT scale 22 (directed entries / 2), resolution 1
    (64155273.0, 0.6969314931),   # ... and a fractional resolution like the automatic one
    (1.0, 1.0), (7.0, 3.25), (1234567.0, 0.1),
    (2.0 ** 40 + 12345.0, 1.5),   # totals near 2^41
    (3.9e15, 0.75),               # 2 M M far above 2^53
])
def test_delta_reciprocal_form_equals_division(ctx, M, R):
    """The kernels' deltaModularity (double-double reciprocals, exact FMA
    remainder, midpoint test) equals the two full divisions bit for bit; the
    same call also checks bare quotients over exponents -200..200."""
    assert ctx.selfcheck_delta(M, R, count=1 << 22, seed=int(M) % 1000 + 7) == 0


def test_map_and_relabel_into_pinned_host_buffers(ctx):
    """Host buffers through the C ABI: a page-locked out_col is written by the
    relabel kernels directly, a pageable one through a copy; both give the
    device-resident call's permutation and relabelled CSR."""
    rp, col = gg.rmat(16, 12, seed=21)
    want_ids, want_rp, want_col, _ = ctx.map_and_relabel(rp.cuda(), col.cuda(), SERIAL)
    want = (want_ids.cpu().numpy(), want_rp.cpu().numpy(), want_col.cpu().numpy())
    n, nnz = rp.numel() - 1, col.numel()
    h_rp, h_col = rp.pin_memory(), col.pin_memory()
    for pinned in (True, False):
        ids = torch.empty(n, dtype=torch.int32)
        orp = torch.empty(n + 1, dtype=torch.int64)
        ocol = torch.empty(nnz, dtype=torch.int32)
        if pinned:
            ids, orp, ocol = ids.pin_memory(), orp.pin_memory(), ocol.pin_memory()
        st = gb.GbgpuStats()
        rc = gb.library().gbgpu_map_and_relabel(ctx.handle, h_rp.data_ptr(), h_col.data_ptr(), n, nnz,
                                                SERIAL.encode(), -1.0, ids.data_ptr(), orp.data_ptr(),
                                                ocol.data_ptr(), gb.C.byref(st), 0)
        assert rc == 0
        for got, exp in zip((ids.numpy(), orp.numpy(), ocol.numpy()), want):
            np.testing.assert_array_equal(got, exp)
