"""ctypes bindings for the CPU oracle (and, where it was built, the reference harness).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py``.  The product package never imports it.

``load()`` returns the plain-C oracle (``_build/libgborc.so``, built by
``make`` in this directory).  ``load_reference()`` returns the harness over the
GraphBrew reference headers (``_ref/libgbref.so``) or ``None`` where it was not
built (it needs the reference sources, which only the development container
has).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libgborc.so")
REF_SO = os.path.join(HERE, "_ref", "libgbref.so")

_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")

# Algorithm-12 defaults (reorder_types.h:213-226) for the GVE-style path.
DEFAULT_TOLERANCE = 1e-2
DEFAULT_AGGREGATION_TOLERANCE = 0.8
DEFAULT_TOLERANCE_DROP = 10.0

COMM_ORDERS = {"size-desc": 0, "size-asc": 1, "degree-desc": 2, "degree-asc": 3, "identity": 6}
INTRA_ORDERS = {"bfs": 0, "rcm": 1, "rcmpp": 2, "gorder": 4, "hubsort": 6, "degree-asc": 7, "hub2": 8, "alternate": 9,
                "random": 10, "boundary-last": 11, "core": 12}
_u64p = np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS")
STDSORT_SO = os.path.join(HERE, "_build", "libstdsort.so")


class Graph(C.Structure):
    _fields_ = [("n", C.c_int64), ("row_ptr", C.c_void_p), ("col", C.c_void_p)]


class LeidenCfg(C.Structure):
    _fields_ = [("resolution", C.c_double), ("tolerance", C.c_double),
                ("aggregation_tolerance", C.c_double), ("tolerance_drop", C.c_double),
                ("max_iterations", C.c_int), ("max_passes", C.c_int),
                ("total_edges_m", C.c_int), ("super_move_batch", C.c_int),
                ("parallel", C.c_int), ("threads", C.c_int), ("refine", C.c_int),
                ("refine_depth", C.c_int)]


class LeidenStats(C.Structure):
    _fields_ = [("passes", C.c_int), ("iterations", C.c_int),
                ("pass_iterations", C.c_int * 16), ("pass0_communities", C.c_int64),
                ("aggregated_communities", C.c_int64), ("super_move_iterations", C.c_int),
                ("super_moves", C.c_int64), ("communities", C.c_int64),
                ("local_move_seconds", C.c_double), ("aggregate_seconds", C.c_double)]


class ComposeCfg(C.Structure):
    _fields_ = [("community_order", C.c_int), ("intra_order", C.c_int),
                ("gorder_window", C.c_int), ("gorder_fallback", C.c_int),
                ("threads", C.c_int), ("super_order", C.c_int), ("super_gamma", C.c_float)]


SUPER_ORDERS = {"none": 0, "super-rabbit": 1, "super-rcm": 2, "hilbert": 4}


class ComposeStats(C.Structure):
    _fields_ = [("num_communities", C.c_int64), ("isolated", C.c_int64),
                ("gorder_communities", C.c_int64), ("gorder_vertices", C.c_int64),
                ("gorder_max_community", C.c_int64), ("fallback_communities", C.c_int64),
                ("fallback_vertices", C.c_int64), ("largest_community", C.c_int64)]


def build() -> str:
    """Compile the plain-C oracle and the CPU-side GAPBS graph builder (seconds)."""
    subprocess.run(["make", "-s", "-C", HERE, "_build/libgborc.so", "_build/libgbgapbs.so"], check=True)
    return ORACLE_SO


GAPBS_SO = os.path.join(HERE, "_build", "libgbgapbs.so")


def gapbs_graph(scale, degree=16, uniform=False):
    """GAPBS's graph for ``-g/-u <scale> -k <degree> -s`` built on the host
    (oracle/gapbs_graph.cc): (row_ptr int64, col int32) numpy arrays."""
    if not os.path.exists(GAPBS_SO):
        build()
    lib = C.CDLL(GAPBS_SO)
    lib.orc_gapbs_build.restype = C.c_int64
    lib.orc_gapbs_build.argtypes = [C.c_int, C.c_int, C.c_int]
    lib.orc_gapbs_nnz.restype = C.c_int64
    lib.orc_gapbs_copy.argtypes = [_i64p, _i32p]
    n = lib.orc_gapbs_build(scale, degree, int(bool(uniform)))
    rp = np.zeros(n + 1, dtype=np.int64)
    cl = np.zeros(lib.orc_gapbs_nnz(), dtype=np.int32)
    lib.orc_gapbs_copy(rp, cl)
    return rp, cl


_lib = None
_ref = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        lib = C.CDLL(ORACLE_SO)
        lib.orc_auto_resolution.restype = C.c_double
        lib.orc_auto_resolution.argtypes = [C.POINTER(Graph)]
        lib.orc_leiden.argtypes = [C.POINTER(Graph), C.POINTER(LeidenCfg), _u32p, C.POINTER(LeidenStats)]
        lib.orc_compose.argtypes = [C.POINTER(Graph), _u32p, C.POINTER(ComposeCfg), _i32p, C.POINTER(ComposeStats)]
        lib.orc_validate_permutation.argtypes = [_i32p, C.c_int64]
        lib.orc_fingerprint.restype = C.c_uint64
        lib.orc_fingerprint.argtypes = [_i32p, C.c_int64]
        lib.orc_relabel.argtypes = [C.POINTER(Graph), _i32p, _i64p, _i32p, C.c_int]
        lib.orc_modularity.restype = C.c_double
        lib.orc_modularity.argtypes = [C.POINTER(Graph), _u32p, C.c_double]
        lib.orc_max_threads.restype = C.c_int
        lib.orc_libstdcxx_sort.argtypes = [_u32p, C.c_int64, _u64p]
        lib.orc_libstdcxx_heap_sort.argtypes = [_u32p, C.c_int64, _u64p]
        lib.orc_random_draws.argtypes = [C.c_uint32, C.c_int64, _u32p]
        lib.orc_umap_order.argtypes = [_u32p, C.c_int64, _u32p]
        lib.orc_super_stage1.argtypes = [C.POINTER(Graph), _u32p, C.c_int, C.c_float, _u32p]
        lib.orc_pagerank_gs.restype = C.c_double
        lib.orc_pagerank_gs.argtypes = [C.POINTER(Graph), C.c_int, C.c_double, _f32p, C.c_int,
                                        C.POINTER(C.c_int)]
        lib.orc_bfs_do.restype = C.c_double
        lib.orc_bfs_do.argtypes = [C.POINTER(Graph), C.c_int64, _i32p, C.c_int]
        lib.orc_cc_afforest.restype = C.c_double
        lib.orc_cc_afforest.argtypes = [C.POINTER(Graph), _i32p, C.c_int]
        lib.orc_dbg_cpu.restype = C.c_double
        lib.orc_dbg_cpu.argtypes = [C.POINTER(Graph), _i32p, C.c_int]
        _lib = lib
    return _lib


def libstdcxx_sort(elems, key):
    """The oracle's restatement of libstdc++ std::sort: elems (uint32 ids)
    sorted by key[elem] ascending, ties left where introsort leaves them."""
    e = np.array(elems, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint64)
    if load().orc_libstdcxx_sort(e, len(e), k) != 0:
        raise RuntimeError("orc_libstdcxx_sort failed")
    return e


def libstdcxx_heap_sort(elems, key):
    """The restatement's depth-limit fallback (heap sort) alone."""
    e = np.array(elems, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint64)
    if load().orc_libstdcxx_heap_sort(e, len(e), k) != 0:
        raise RuntimeError("orc_libstdcxx_heap_sort failed")
    return e


def _stdsort_lib():
    if not os.path.exists(STDSORT_SO):
        subprocess.run(["make", "-s", "-C", HERE, "_build/libstdsort.so"], check=True)
    lib = C.CDLL(STDSORT_SO)
    lib.pin_std_sort.argtypes = [_u32p, C.c_int64, _u64p]
    lib.pin_std_heap_sort.argtypes = [_u32p, C.c_int64, _u64p]
    lib.pin_std_shuffle_draws.argtypes = [C.c_uint32, C.c_int64, _u32p]
    lib.pin_umap_order.argtypes = [_u32p, C.c_int64, _u32p]
    lib.pin_umap_bucket_count.restype = C.c_int64
    lib.pin_umap_bucket_count.argtypes = [C.c_int64]
    return lib


def std_sort(elems, key):
    """The toolchain's own std::sort with the same comparator (pin)."""
    e = np.array(elems, dtype=np.uint32)
    _stdsort_lib().pin_std_sort(e, len(e), np.ascontiguousarray(key, dtype=np.uint64))
    return e


def random_draws(seed, count):
    """The oracle's intra_random swap indices: out[j], j = count-1 .. 1."""
    out = np.zeros(max(count, 1), dtype=np.uint32)
    if load().orc_random_draws(seed, count, out) != 0:
        raise RuntimeError("orc_random_draws failed")
    return out[:count]


def std_shuffle_draws(seed, count):
    """The same indices from the toolchain's std::mt19937 and
    std::uniform_int_distribution<size_t> (pin)."""
    out = np.zeros(max(count, 1), dtype=np.uint32)
    _stdsort_lib().pin_std_shuffle_draws(seed, count, out)
    return out[:count]


def umap_order(keys):
    """The oracle's libstdc++ unordered_map iteration order for distinct
    keys inserted in order."""
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    out = np.zeros(max(len(k), 1), dtype=np.uint32)
    if load().orc_umap_order(k, len(k), out) != 0:
        raise RuntimeError("orc_umap_order failed")
    return out[:len(k)]


def super_stage1(row_ptr, col, membership, super_order, gamma=0.1):
    """stage1Perm of a super-graph order ("super-rcm" / "super-rabbit" /
    "hilbert")."""
    g, keep = _as_graph(row_ptr, col)
    memb = np.ascontiguousarray(membership, dtype=np.uint32)
    out = np.zeros(int(memb.max()) + 1 if len(memb) else 1, dtype=np.uint32)
    if load().orc_super_stage1(C.byref(g), memb, SUPER_ORDERS[super_order], gamma, out) != 0:
        raise RuntimeError("orc_super_stage1 failed")
    return out


def std_umap_order(keys):
    """The same from the toolchain's std::unordered_map (pin)."""
    k = np.ascontiguousarray(keys, dtype=np.uint32)
    out = np.zeros(max(len(k), 1), dtype=np.uint32)
    _stdsort_lib().pin_umap_order(k, len(k), out)
    return out[:len(k)]


def std_umap_bucket_count(count):
    """bucket_count() of the toolchain's std::unordered_map after count
    distinct insertions (pin of the growth table)."""
    return int(_stdsort_lib().pin_umap_bucket_count(count))


def std_heap_sort(elems, key):
    """The toolchain's std::partial_sort over the whole range (pin)."""
    e = np.array(elems, dtype=np.uint32)
    _stdsort_lib().pin_std_heap_sort(e, len(e), np.ascontiguousarray(key, dtype=np.uint64))
    return e


def load_reference():
    """The reference harness, or None where it was not built here."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        lib = C.CDLL(REF_SO)
        lib.ref_auto_resolution.restype = C.c_double
        lib.ref_auto_resolution.argtypes = [C.c_int64, _i64p, _i32p]
        lib.ref_effective_config_json.argtypes = [C.c_char_p, C.c_double, C.c_char_p, C.c_size_t]
        lib.ref_run_graphbrew.argtypes = [C.c_int64, _i64p, _i32p, C.c_char_p, C.c_double, _u32p,
                                          _i64p, C.c_int, C.c_char_p, C.c_size_t]
        lib.ref_order_compose.argtypes = [C.c_int64, _i64p, _i32p, _u32p, C.c_char_p, C.c_double,
                                          _i32p, _i64p, C.c_int, C.c_char_p, C.c_size_t]
        lib.ref_generate_mapping.argtypes = [C.c_int64, _i64p, _i32p, C.c_char_p, C.c_double, _i32p,
                                             C.c_int, C.c_char_p, C.c_size_t]
        lib.ref_relabel.argtypes = [C.c_int64, _i64p, _i32p, _i32p, _i64p, _i32p, _i32p, C.c_int]
        lib.ref_modularity.restype = C.c_double
        lib.ref_modularity.argtypes = [C.c_int64, _i64p, _i32p, _u32p, C.c_double]
        lib.ref_gorder_kat.argtypes = [C.c_int64, _i64p, _i32p, C.c_int, _i32p]
        lib.ref_gapbs_generate.restype = C.c_int64
        lib.ref_gapbs_generate.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int64), C.c_int]
        lib.ref_last_graph_copy.argtypes = [_i64p, _i32p]
        lib.ref_set_threads.argtypes = [C.c_int]
        lib.ref_dbg_mapping.argtypes = [C.c_int64, _i64p, _i32p, _i32p]
        lib.ref_tier0_features.argtypes = [C.c_int64, _i64p, _i32p, C.POINTER(C.c_double)]
        _ref = lib
    return _ref


def _as_graph(row_ptr, col):
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    col = np.ascontiguousarray(col, dtype=np.int32)
    g = Graph(len(row_ptr) - 1, row_ptr.ctypes.data, col.ctypes.data)
    return g, (row_ptr, col)


# --------------------------------------------------------------------------
# Oracle API
# --------------------------------------------------------------------------

def auto_resolution(row_ptr, col) -> float:
    g, keep = _as_graph(row_ptr, col)
    return load().orc_auto_resolution(C.byref(g))


def leiden(row_ptr, col, resolution, max_iterations=2, max_passes=2, super_move_batch=4096,
           parallel=False, threads=0, total_edges_m=True, refine_depth=None):
    """refine_depth: None = norefine; k = refine<k> (refinement in passes 0..k,
    -1 in every pass)."""
    g, keep = _as_graph(row_ptr, col)
    cfg = LeidenCfg(resolution, DEFAULT_TOLERANCE, DEFAULT_AGGREGATION_TOLERANCE,
                    DEFAULT_TOLERANCE_DROP, max_iterations, max_passes, int(total_edges_m),
                    super_move_batch, int(parallel), threads, int(refine_depth is not None),
                    -1 if refine_depth is None else int(refine_depth))
    memb = np.zeros(g.n, dtype=np.uint32)
    st = LeidenStats()
    rc = load().orc_leiden(C.byref(g), C.byref(cfg), memb, C.byref(st))
    if rc != 0:
        raise RuntimeError(f"orc_leiden failed: {rc}")
    return memb, st


def compose(row_ptr, col, membership, community_order="size-desc", intra_order="gorder",
            gorder_window=8, gorder_fallback=5000, threads=0, super_order="none", super_gamma=0.1):
    g, keep = _as_graph(row_ptr, col)
    cfg = ComposeCfg(COMM_ORDERS[community_order], INTRA_ORDERS[intra_order], gorder_window,
                     gorder_fallback, threads, SUPER_ORDERS[super_order], super_gamma)
    memb = np.ascontiguousarray(membership, dtype=np.uint32)
    out = np.zeros(g.n, dtype=np.int32)
    st = ComposeStats()
    rc = load().orc_compose(C.byref(g), memb, C.byref(cfg), out, C.byref(st))
    if rc != 0:
        raise RuntimeError(f"orc_compose failed: {rc}")
    return out, st


def validate_permutation(new_ids) -> int:
    ids = np.ascontiguousarray(new_ids, dtype=np.int32)
    return load().orc_validate_permutation(ids, len(ids))


def fingerprint(new_ids) -> str:
    ids = np.ascontiguousarray(new_ids, dtype=np.int32)
    return "%016x" % load().orc_fingerprint(ids, len(ids))


def relabel(row_ptr, col, new_ids, threads=0):
    g, keep = _as_graph(row_ptr, col)
    ids = np.ascontiguousarray(new_ids, dtype=np.int32)
    out_rp = np.zeros(g.n + 1, dtype=np.int64)
    out_col = np.zeros(len(keep[1]), dtype=np.int32)
    rc = load().orc_relabel(C.byref(g), ids, out_rp, out_col, threads)
    if rc != 0:
        raise RuntimeError(f"orc_relabel failed: {rc}")
    return out_rp, out_col


def modularity(row_ptr, col, membership, resolution=1.0) -> float:
    g, keep = _as_graph(row_ptr, col)
    return load().orc_modularity(C.byref(g), np.ascontiguousarray(membership, dtype=np.uint32),
                                 resolution)


def map_graph(row_ptr, col, resolution, parallel=False, threads=0, max_iterations=2,
              max_passes=2, super_move_batch=4096, gorder_window=8, gorder_fallback=5000,
              intra_order="gorder", community_order="size-desc"):
    """The whole FastLeiden-Gorder8 recipe: Leiden, then COMPOSE."""
    memb, lst = leiden(row_ptr, col, resolution, max_iterations, max_passes, super_move_batch,
                       parallel, threads)
    ids, cst = compose(row_ptr, col, memb, community_order, intra_order, gorder_window,
                       gorder_fallback, 0 if parallel else 1)
    return ids, memb, lst, cst


# --------------------------------------------------------------------------
# Reference harness API (development container only)
# --------------------------------------------------------------------------

def ref_effective_config(opts: str, auto_res: float):
    buf = C.create_string_buffer(8192)
    rc = load_reference().ref_effective_config_json(opts.encode(), auto_res, buf, len(buf))
    return rc, buf.value.decode()


def ref_leiden(row_ptr, col, opts, auto_res, threads=1):
    ref = load_reference()
    ref.ref_set_threads(threads)
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    memb = np.zeros(len(rp) - 1, dtype=np.uint32)
    summ = np.zeros(3, dtype=np.int64)
    err = C.create_string_buffer(1024)
    rc = ref.ref_run_graphbrew(len(rp) - 1, rp, cl, opts.encode(), auto_res, memb, summ, 1, err, 1024)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return memb, summ


def ref_compose(row_ptr, col, membership, opts, auto_res, threads=1):
    ref = load_reference()
    ref.ref_set_threads(threads)
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    ids = np.zeros(len(rp) - 1, dtype=np.int32)
    st = np.zeros(5, dtype=np.int64)
    err = C.create_string_buffer(1024)
    rc = ref.ref_order_compose(len(rp) - 1, rp, cl, np.ascontiguousarray(membership, dtype=np.uint32),
                               opts.encode(), auto_res, ids, st, 1, err, 1024)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return ids, st


def ref_generate_mapping(row_ptr, col, opts, auto_res, threads=1):
    ref = load_reference()
    ref.ref_set_threads(threads)
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    ids = np.zeros(len(rp) - 1, dtype=np.int32)
    err = C.create_string_buffer(1024)
    rc = ref.ref_generate_mapping(len(rp) - 1, rp, cl, opts.encode(), auto_res, ids, 1, err, 1024)
    if rc != 0:
        raise RuntimeError(err.value.decode())
    return ids


def ref_relabel(row_ptr, col, new_ids):
    ref = load_reference()
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    out_rp = np.zeros(len(rp), dtype=np.int64)
    out_col = np.zeros(len(cl), dtype=np.int32)
    org = np.zeros(len(rp) - 1, dtype=np.int32)
    ref.ref_relabel(len(rp) - 1, rp, cl, np.ascontiguousarray(new_ids, dtype=np.int32), out_rp, out_col, org, 1)
    return out_rp, out_col, org


def ref_gapbs_graph(scale, degree=16, uniform=False):
    ref = load_reference()
    nnz = C.c_int64(0)
    n = ref.ref_gapbs_generate(scale, degree, int(uniform), C.byref(nnz), 1)
    rp = np.zeros(n + 1, dtype=np.int64)
    cl = np.zeros(nnz.value, dtype=np.int32)
    ref.ref_last_graph_copy(rp, cl)
    return rp, cl


def ref_dbg_mapping(row_ptr, col):
    ref = load_reference()
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    out = np.zeros(len(rp) - 1, dtype=np.int32)
    ref.ref_dbg_mapping(len(rp) - 1, rp, cl, out)
    return out


def ref_tier0_features(row_ptr, col):
    ref = load_reference()
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    out = (C.c_double * 9)()
    ref.ref_tier0_features(len(rp) - 1, rp, cl, out)
    return dict(zip(TIER0_KEYS, list(out)))


TIER0_KEYS = ("num_nodes", "num_edges", "avg_degree", "degree_cv", "internal_density", "hub_concentration",
              "packing_factor", "normalized_edge_span", "window_neighbor_overlap")


# --------------------------------------------------------------------------
# Timed consumers, the DBG arm, Tier-0 features and the MLP (numpy restatements)
# --------------------------------------------------------------------------

def dbg_mapping(row_ptr, col):
    """GenerateDBGMapping (bench/include/graphbrew/reorder/reorder_hub.h:267-342):
    8 degree buckets (avg/2, avg, 2avg, ..., 32avg, inf), highest bucket first,
    vertex-id order inside a bucket."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    n = len(rp) - 1
    if n == 0:
        return np.zeros(0, dtype=np.int32)
    deg = np.diff(rp).astype(np.uint64)
    avg = np.uint64((rp[-1]) // n)
    th = [avg // np.uint64(2), avg, avg * np.uint64(2), avg * np.uint64(4), avg * np.uint64(8),
          avg * np.uint64(16), avg * np.uint64(32)]
    bucket = np.full(n, 7, dtype=np.int64)
    for j in range(6, -1, -1):
        bucket[deg <= th[j]] = j
    order = np.argsort(7 - bucket, kind="stable")
    ids = np.empty(n, dtype=np.int32)
    ids[order] = np.arange(n, dtype=np.int32)
    return ids


# ---- the reference's CPU benchmark kernels (OpenMP; for timing arms) ----
def pagerank_cpu(row_ptr, col, max_iters=20, epsilon=1e-4, threads=0):
    """PageRank pull, Gauss-Seidel (bench/src/pr.cc:40-90): (scores, iterations, ms)."""
    g, keep = _as_graph(row_ptr, col)
    out = np.zeros(g.n, dtype=np.float32)
    it = C.c_int()
    ms = load().orc_pagerank_gs(C.byref(g), int(max_iters), float(epsilon), out, int(threads), C.byref(it))
    return out, it.value, ms


def bfs_cpu(row_ptr, col, source, threads=0):
    """Direction-optimizing BFS (bench/src/bfs.cc): (depths, ms)."""
    g, keep = _as_graph(row_ptr, col)
    out = np.zeros(g.n, dtype=np.int32)
    ms = load().orc_bfs_do(C.byref(g), int(source), out, int(threads))
    return out, ms


def cc_cpu(row_ptr, col, threads=0):
    """Afforest connected components (bench/src/cc.cc): (component ids, ms)."""
    g, keep = _as_graph(row_ptr, col)
    out = np.zeros(g.n, dtype=np.int32)
    ms = load().orc_cc_afforest(C.byref(g), out, int(threads))
    return out, ms


def dbg_cpu(row_ptr, col, threads=0):
    """GenerateDBGMapping on the host cores: (new ids, ms)."""
    g, keep = _as_graph(row_ptr, col)
    out = np.zeros(g.n, dtype=np.int32)
    ms = load().orc_dbg_cpu(C.byref(g), out, int(threads))
    return out, ms


def bfs_depths(row_ptr, col, source):
    """BFS depth of every vertex from source (-1 unreached)."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    cl = np.asarray(col)
    n = len(rp) - 1
    depth = np.full(n, -1, dtype=np.int32)
    depth[source] = 0
    frontier = [source]
    level = 0
    while frontier:
        nxt = []
        for u in frontier:
            for v in cl[rp[u]:rp[u + 1]]:
                if depth[v] < 0:
                    depth[v] = level + 1
                    nxt.append(int(v))
        frontier = nxt
        level += 1
    return depth


def cc_min_labels(row_ptr, col):
    """Connected components labelled by their smallest vertex id."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    cl = np.asarray(col)
    n = len(rp) - 1
    parent = np.arange(n)

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x
    for u in range(n):
        for v in cl[rp[u]:rp[u + 1]]:
            a, b = find(u), find(int(v))
            if a != b:
                parent[max(a, b)] = min(a, b)
    return np.array([find(x) for x in range(n)], dtype=np.int32)


def pagerank(row_ptr, col, max_iters=20, epsilon=1e-4, damp=0.85):
    """Pull PageRank (bench/src/pr.cc:40-90) as Jacobi sweeps in float64."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    cl = np.asarray(col, dtype=np.int64)
    n = len(rp) - 1
    deg = np.diff(rp).astype(np.float64)
    score = np.full(n, 1.0 / n)
    src = np.repeat(np.arange(n), np.diff(rp))
    for _ in range(max_iters):
        contrib = np.where(deg > 0, score / np.maximum(deg, 1), 0.0)
        incoming = np.bincount(src, weights=contrib[cl], minlength=n)
        new = (1.0 - damp) / n + damp * incoming
        err = np.abs(new - score).sum()
        score = new
        if err < epsilon:
            break
    return score


def tier0_features(row_ptr, col):
    """ComputeTier0SampledGraphFeatures (reorder_types.h:6066-6186) with sample seed 0."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    cl = np.asarray(col, dtype=np.int64)
    n = len(rp) - 1
    s = max(1024, min(int(np.sqrt(float(n))), 8192))
    s = min(s, n)
    nodes = [((2 * i + 1) * n) // (2 * s) for i in range(s)]
    degs = [int(rp[v + 1] - rp[v]) for v in nodes]
    dsum = 0.0
    for d in degs:
        dsum += d
    avg = dsum / s
    var = 0.0
    for d in degs:
        var += (d - avg) * (d - avg)
    variance = var / (s - 1) if s > 1 else 0.0
    cv = np.sqrt(variance) / avg if avg > 0 else 0.0
    pairs = sorted(zip(degs, nodes), key=lambda p: (-p[0], p[1]))
    hub_count = max(1, s // 10)
    hsum = 0.0
    for d, _ in pairs[:hub_count]:
        hsum += d
    hubs = [v for _, v in pairs[:hub_count]]
    lines = {v // 8 for v in hubs}
    span, edges, window = 0.0, 0, 0
    den = float(max(1, n - 1))
    for _, v in pairs:
        for d in cl[rp[v]:rp[v + 1]]:
            span += abs(int(d) - v) / den
            edges += 1
            window += abs(int(d) // 8 - v // 8) <= 1
    return {"num_nodes": float(n), "num_edges": float(rp[-1]), "avg_degree": avg, "degree_cv": cv,
            "internal_density": avg / (n - 1) if n > 1 else 0.0,
            "hub_concentration": hsum / dsum if dsum > 0 else 0.0,
            "packing_factor": len(hubs) / len(lines) if lines else 0.0,
            "normalized_edge_span": span / edges if edges else 0.0,
            "window_neighbor_overlap": window / edges if edges else 0.0}


def mlp_unpack(params, in_dim, hidden=64, out=3):
    p = np.asarray(params, dtype=np.float64)
    shapes = [(in_dim, hidden), (hidden,), (hidden, hidden), (hidden,), (hidden, out), (out,)]
    res, o = [], 0
    for sh in shapes:
        k = int(np.prod(sh))
        res.append(p[o:o + k].reshape(sh))
        o += k
    return res


def mlp_loss_grad(params, X, T):
    """float64 forward/backward of the in -> 64 -> 64 -> 3 ReLU MLP under mean squared error."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    W1, b1, W2, b2, W3, b3 = mlp_unpack(params, X.shape[1])
    H1 = np.maximum(X @ W1 + b1, 0)
    H2 = np.maximum(H1 @ W2 + b2, 0)
    Y = H2 @ W3 + b3
    B, O = Y.shape
    loss = ((Y - T) ** 2).sum() / (B * O)
    dY = 2 * (Y - T) / (B * O)
    gW3, gb3 = H2.T @ dY, dY.sum(0)
    dH2 = (dY @ W3.T) * (H2 > 0)
    gW2, gb2 = H1.T @ dH2, dH2.sum(0)
    dH1 = (dH2 @ W2.T) * (H1 > 0)
    gW1, gb1 = X.T @ dH1, dH1.sum(0)
    grad = np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])
    return loss, grad, Y
