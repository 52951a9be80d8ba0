"""GB300-native GraphBrew algorithm-12 mapping construction.

Python mirror of the reference's mapping-path interface over the C ABI in
``include/gbgpu.h`` (libgbgpu.so, built in-tree by ``graphbrew_gb300.build``):

==============================  ==================================================
this package                    GraphBrew reference
==============================  ==================================================
``parse_graphbrew_config``      ``parseGraphBrewCliConfig`` + effective-config JSON
                                (reorder_graphbrew_parser.h:714-912)
``generate_mapping``            ``generateGraphBrewMapping`` (reorder_graphbrew.h:7836)
``run_graphbrew``               ``runGraphBrew`` (reorder_graphbrew.h:7238)
``order_compose``               ``orderCompose`` (reorder_graphbrew.h:6286)
``validate_permutation``        ``ValidatePermutationOrThrow`` (builder.h:2042)
``mapping_fingerprint``         ``MappingFingerprint`` (builder.h:1398)
``relabel_by_mapping``          ``RelabelByMapping`` (builder.h:1046)
``auto_resolution``             ``computeAutoResolution`` (reorder_types.h:2743)
==============================  ==================================================

Arrays may be numpy arrays (host; copied in and out inside the call) or CUDA
torch tensors (device-resident; no copies).  Errors raise the exception type
the reference throws: ``ValueError`` for std::invalid_argument (bad options or
graphs), ``RuntimeError`` for std::runtime_error (validation failures and CUDA
errors), ``OverflowError`` for std::overflow_error, ``NotImplementedError`` for
options that are valid in the grammar but not on the GPU path.  There is no CPU
fallback: importing the package fails if libgbgpu.so is missing.
"""
from __future__ import annotations

import ctypes as C
import json
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgbgpu.so")

DEFAULT_RECIPE = ("leiden:compose:sg_none:comm_size_desc:intra_gorder:gw8:cd_parallel:"
                  "sgmb4096:gordf5000:norefine:2:2")

OK, E_INVALID, E_UNSUPPORTED, E_CUDA, E_NOMEM, E_NOT_PERMUTATION, E_PARSE, E_OVERFLOW, E_TIMEOUT = range(9)
DEVICE_POINTERS = 0x1
QUIET = 0x2


class GbgpuConfig(C.Structure):
    _fields_ = [("resolution", C.c_double), ("tolerance", C.c_double),
                ("aggregation_tolerance", C.c_double), ("tolerance_drop", C.c_double),
                ("max_iterations", C.c_int32), ("max_passes", C.c_int32),
                ("total_edges_m", C.c_int32), ("gve_aggregation", C.c_int32),
                ("use_refinement", C.c_int32), ("refinement_depth", C.c_int32),
                ("deterministic", C.c_int32), ("super_move_batch", C.c_int32),
                ("ordering", C.c_int32), ("super_graph_order", C.c_int32),
                ("community_order", C.c_int32), ("intra_order", C.c_int32),
                ("refinement_pass", C.c_int32), ("gorder_window", C.c_int32),
                ("gorder_fallback", C.c_int32), ("algorithm", C.c_int32)]


class GbgpuGraph(C.Structure):
    _fields_ = [("row_ptr", C.c_void_p), ("col", C.c_void_p), ("n", C.c_int64), ("nnz", C.c_int64),
                ("new_ids_out", C.c_void_p)]


class GbgpuSchedule(C.Structure):
    _fields_ = [("streams", C.c_int32), ("order", C.c_int32), ("exact_window", C.c_int64)]


class GbgpuStats(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("leiden_ms", C.c_double), ("local_move_ms", C.c_double),
                ("aggregate_ms", C.c_double), ("compose_ms", C.c_double), ("intra_ms", C.c_double),
                ("validate_ms", C.c_double), ("relabel_ms", C.c_double), ("h2d_ms", C.c_double),
                ("d2h_ms", C.c_double), ("passes", C.c_int32), ("iterations", C.c_int32),
                ("super_move_iterations", C.c_int32), ("super_move_ctas", C.c_int32),
                ("super_moves", C.c_int64), ("pass0_communities", C.c_int64),
                ("aggregated_communities", C.c_int64), ("communities", C.c_int64),
                ("num_communities", C.c_int64), ("isolated", C.c_int64),
                ("gorder_communities", C.c_int64), ("gorder_vertices", C.c_int64),
                ("gorder_max_community", C.c_int64), ("fallback_communities", C.c_int64),
                ("fallback_vertices", C.c_int64), ("largest_community", C.c_int64),
                ("bfs_levels", C.c_int64), ("kernel_launches", C.c_int64), ("resolution", C.c_double),
                ("local_move_rounds", C.c_int64), ("local_move_evaluations", C.c_int64),
                ("local_move_streams", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class GbgpuSelectionPolicy(C.Structure):
    _fields_ = [("model", C.c_int32), ("criterion", C.c_int32), ("reuse", C.c_double),
                ("reuse_explicit", C.c_int32)]


class GbgpuSelectorModel(C.Structure):
    _fields_ = [("in_dim", C.c_int32), ("params", C.c_void_p), ("mean", C.c_void_p), ("std", C.c_void_p),
                ("lo", C.c_void_p), ("hi", C.c_void_p), ("cache_bytes", C.c_int64)]


class GbgpuSelection(C.Structure):
    _fields_ = [("policy", GbgpuSelectionPolicy), ("arm", C.c_int32), ("applied", C.c_char * 160),
                ("reason", C.c_char * 48), ("features", C.c_double * 9), ("property_bytes", C.c_int64),
                ("cache_bytes", C.c_int64), ("property_wsr", C.c_double), ("predicted_log10_ms", C.c_float * 3)]

    def as_dict(self):
        return {"model": self.policy.model, "criterion": self.policy.criterion, "reuse": self.policy.reuse,
                "arm": self.arm, "applied": self.applied.decode(), "reason": self.reason.decode(),
                "features": list(self.features), "property_bytes": self.property_bytes,
                "cache_bytes": self.cache_bytes, "property_wsr": self.property_wsr,
                "predicted_log10_ms": list(self.predicted_log10_ms)}


KERNELS = {"generic": 0, "pr": 1, "bfs": 2, "cc": 3, "sssp": 4, "bc": 5, "tc": 6, "pr_spmv": 7, "cc_sv": 8}
SELECTOR_MODEL_PATH = os.path.join(_HERE, "data", "selector_mlp.gbsel")

# Every entry point declared in include/gbgpu.h, with its ctypes signature.
_P = C.c_void_p
SIGNATURES = {
    "gbgpu_ctx_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int]),
    "gbgpu_ctx_destroy": (None, [_P]),
    "gbgpu_last_error": (C.c_char_p, [_P]),
    "gbgpu_set_stream": (C.c_int, [_P, _P]),
    "gbgpu_synchronize": (C.c_int, [_P]),
    "gbgpu_parse_config": (C.c_int, [C.c_char_p, C.c_double, C.POINTER(GbgpuConfig), C.c_char_p, C.c_size_t]),
    "gbgpu_auto_resolution": (C.c_int, [_P, _P, C.c_int64, C.c_int64, C.c_uint32, C.POINTER(C.c_double)]),
    "gbgpu_generate_mapping": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.c_char_p, C.c_double, _P,
                                         C.POINTER(GbgpuStats), C.c_uint32]),
    "gbgpu_leiden": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.c_char_p, C.c_double, _P,
                               C.POINTER(GbgpuStats), C.c_uint32]),
    "gbgpu_compose": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _P, C.c_char_p, _P,
                                C.POINTER(GbgpuStats), C.c_uint32]),
    "gbgpu_validate_permutation": (C.c_int, [_P, _P, C.c_int64, C.c_uint32, C.POINTER(C.c_int32)]),
    "gbgpu_relabel_csr": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _P, _P, _P, _P, C.c_uint32]),
    "gbgpu_map_and_relabel": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.c_char_p, C.c_double, _P, _P, _P,
                                        C.POINTER(GbgpuStats), C.c_uint32]),
    "gbgpu_validate_permutation_noalloc": (C.c_int, [_P, _P, C.c_int64, C.POINTER(C.c_int32)]),
    "gbgpu_fingerprint": (C.c_uint64, [_P, C.c_int64]),
    "gbgpu_selfcheck_delta": (C.c_int, [_P, C.c_double, C.c_double, C.c_int64, C.c_uint64,
                                        C.POINTER(C.c_int64)]),
    "gbgpu_gapbs_edge_count": (C.c_int64, [C.c_int32, C.c_int32]),
    "gbgpu_gapbs_edge_list": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, _P, _P, C.c_int32]),
    "gbgpu_version": (C.c_char_p, []),
    "gbgpu_parse_selection_policy": (C.c_int, [C.c_char_p, C.POINTER(GbgpuSelectionPolicy), C.c_char_p,
                                               C.c_size_t]),
    "gbgpu_selection_model_name": (C.c_char_p, [C.c_int32]),
    "gbgpu_selection_criterion_name": (C.c_char_p, [C.c_int32]),
    "gbgpu_apply_selection_rule": (C.c_int, [C.c_int32, _P, C.c_double, C.c_int32, C.c_double,
                                             C.POINTER(GbgpuSelection)]),
    "gbgpu_modeled_property_bytes": (C.c_int64, [C.c_int32, C.c_int64, C.c_int64]),
    "gbgpu_selector_model_load": (C.c_int, [C.c_char_p, C.POINTER(C.POINTER(GbgpuSelectorModel))]),
    "gbgpu_selector_model_free": (None, [C.POINTER(GbgpuSelectorModel)]),
    "gbgpu_select_arm": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.c_char_p, C.c_int32,
                                   C.POINTER(GbgpuSelectorModel), C.POINTER(GbgpuSelection), C.c_uint32]),
    "gbgpu_generate_mappings_batched": (C.c_int, [_P, C.POINTER(GbgpuGraph), C.c_int32, C.c_char_p,
                                                  C.POINTER(GbgpuSchedule), _P, C.POINTER(C.c_double), C.c_uint32]),
    "gbgpu_pagerank": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.c_int32, C.c_double, _P,
                                 C.POINTER(C.c_int32), C.POINTER(C.c_double), C.c_uint32]),
    "gbgpu_bfs": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.c_int64, _P, C.POINTER(C.c_double), C.c_uint32]),
    "gbgpu_connected_components": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _P, C.POINTER(C.c_double),
                                             C.c_uint32]),
    "gbgpu_dbg_mapping": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, _P, C.POINTER(C.c_double), C.c_uint32]),
    "gbgpu_tier0_features": (C.c_int, [_P, _P, _P, C.c_int64, C.c_int64, C.POINTER(C.c_double), C.c_uint32]),
    "gbgpu_mlp_param_count": (C.c_int, [C.c_int32]),
    "gbgpu_mlp_forward": (C.c_int, [_P, _P, _P, C.c_int32, C.c_int32, _P, C.c_uint32]),
    "gbgpu_mlp_gradient": (C.c_int, [_P, _P, _P, _P, C.c_int32, C.c_int32, _P, C.POINTER(C.c_float),
                                     C.c_uint32]),
    "gbgpu_mlp_train": (C.c_int, [_P, _P, _P, _P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_float,
                                  C.c_uint64, C.POINTER(C.c_float), C.c_uint32]),
}

_lib = None


def library():
    """Load libgbgpu.so (in-tree); raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m graphbrew_gb300.build` "
                "(the mapping path has no CPU fallback)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _raise(status: int, message: str):
    if status in (E_INVALID, E_PARSE):
        raise ValueError(message)
    if status == E_UNSUPPORTED:
        raise NotImplementedError(message)
    if status == E_OVERFLOW:
        raise OverflowError(message)
    if status == E_NOMEM:
        raise MemoryError(message)
    raise RuntimeError(message)


def parse_graphbrew_config(options, auto_resolution: float = 1.0):
    """Parse "-o 12:" tokens; returns (config dict, effective-config JSON text)."""
    opts = options if isinstance(options, str) else ":".join(options)
    cfg = GbgpuConfig()
    buf = C.create_string_buffer(16384)
    rc = library().gbgpu_parse_config(opts.encode(), float(auto_resolution), C.byref(cfg), buf, len(buf))
    text = buf.value.decode()
    if rc != OK:
        _raise(rc, text)
    return {k: getattr(cfg, k) for k, _ in cfg._fields_}, text


def mapping_fingerprint(new_ids) -> str:
    ids = np.ascontiguousarray(_to_numpy(new_ids), dtype=np.int32)
    return "%016x" % library().gbgpu_fingerprint(ids.ctypes.data, len(ids))


def _to_numpy(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().numpy()
    except ImportError:
        pass
    return np.asarray(a)


def _is_cuda(a) -> bool:
    try:
        import torch
        return isinstance(a, torch.Tensor) and a.is_cuda
    except ImportError:
        return False


class Context:
    """One GPU context: a CUDA stream and a stream-ordered memory pool."""

    def __init__(self, device: int = -1):
        h = C.c_void_p()
        rc = library().gbgpu_ctx_create(C.byref(h), device)
        if rc != OK:
            _raise(rc, f"gbgpu_ctx_create failed with status {rc}")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            library().gbgpu_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, rc):
        if rc != OK:
            _raise(rc, library().gbgpu_last_error(self._h).decode())

    def set_stream(self, stream_ptr: int | None):
        self._check(library().gbgpu_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def synchronize(self):
        self._check(library().gbgpu_synchronize(self._h))

    # -- argument marshalling ------------------------------------------------
    def _graph_args(self, row_ptr, col):
        dev = _is_cuda(row_ptr)
        if dev != _is_cuda(col):
            raise ValueError("row_ptr and col must both be host arrays or both CUDA tensors")
        if dev:
            import torch
            if row_ptr.dtype != torch.int64 or col.dtype != torch.int32:
                raise ValueError("row_ptr must be int64 and col int32")
            row_ptr, col = row_ptr.contiguous(), col.contiguous()
            self._follow_torch_stream(row_ptr)
            return row_ptr, col, row_ptr.data_ptr(), col.data_ptr(), row_ptr.numel() - 1, col.numel(), True
        rp = np.ascontiguousarray(_to_numpy(row_ptr), dtype=np.int64)
        cl = np.ascontiguousarray(_to_numpy(col), dtype=np.int32)
        return rp, cl, rp.ctypes.data, cl.ctypes.data if len(cl) else 0, len(rp) - 1, len(cl), False

    def _follow_torch_stream(self, t):
        """Device-tensor calls run on torch's current stream of the tensor's
        device, so they are ordered after the kernels that produced the inputs
        and before whatever consumes the outputs."""
        import torch
        st = torch.cuda.current_stream(t.device)
        if st.cuda_stream == 0:
            # The legacy default stream has no handle to order against the
            # context's non-blocking stream: wait for it instead.
            st.synchronize()
            self.set_stream(None)
        else:
            self.set_stream(st.cuda_stream)

    @staticmethod
    def _out(n, dtype, dev, like=None):
        if dev:
            import torch
            tdt = {np.int32: torch.int32, np.uint32: torch.int32, np.int64: torch.int64}[dtype]
            t = torch.empty(max(n, 0), dtype=tdt, device=like.device)
            return t, t.data_ptr()
        a = np.zeros(max(n, 0), dtype=dtype)
        return a, a.ctypes.data if n else 0

    # -- entry points ----------------------------------------------------------
    def auto_resolution(self, row_ptr, col) -> float:
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        out = C.c_double()
        self._check(library().gbgpu_auto_resolution(self._h, prp, n, nnz, DEVICE_POINTERS if dev else 0,
                                                      C.byref(out)))
        return out.value

    def generate_mapping(self, row_ptr, col, options=DEFAULT_RECIPE, auto_resolution=None):
        """Forward map old id -> new id (int32), and the call's statistics."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        out, pout = self._out(n, np.int32, dev, rp)
        st = GbgpuStats()
        ar = -1.0 if auto_resolution is None else float(auto_resolution)
        opts = options if isinstance(options, str) else ":".join(options)
        self._check(library().gbgpu_generate_mapping(self._h, prp, pcl, n, nnz, opts.encode(), ar, pout,
                                                       C.byref(st), DEVICE_POINTERS if dev else 0))
        return out, st.as_dict()

    def run_graphbrew(self, row_ptr, col, options=DEFAULT_RECIPE, resolution=None):
        """Community detection only: membership (uint32) and statistics."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        out, pout = self._out(n, np.uint32, dev, rp)
        st = GbgpuStats()
        ar = -1.0 if resolution is None else float(resolution)
        opts = options if isinstance(options, str) else ":".join(options)
        self._check(library().gbgpu_leiden(self._h, prp, pcl, n, nnz, opts.encode(), ar, pout, C.byref(st),
                                             DEVICE_POINTERS if dev else 0))
        return out, st.as_dict()

    def order_compose(self, row_ptr, col, membership, options=DEFAULT_RECIPE):
        """COMPOSE stage only, from a membership vector."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        if dev:
            import torch
            memb = membership.contiguous()
            if memb.dtype not in (torch.int32, torch.uint32):
                memb = memb.to(torch.int32)
            pm = memb.data_ptr()
        else:
            memb = np.ascontiguousarray(_to_numpy(membership), dtype=np.uint32)
            pm = memb.ctypes.data if n else 0
        out, pout = self._out(n, np.int32, dev, rp)
        st = GbgpuStats()
        opts = options if isinstance(options, str) else ":".join(options)
        self._check(library().gbgpu_compose(self._h, prp, pcl, n, nnz, pm, opts.encode(), pout, C.byref(st),
                                              DEVICE_POINTERS if dev else 0))
        return out, st.as_dict()

    def validate_permutation(self, new_ids) -> int:
        """0 valid, 1 out-of-range id, 2 duplicate id."""
        dev = _is_cuda(new_ids)
        if dev:
            ids = new_ids.contiguous()
            self._follow_torch_stream(ids)
            p, n = ids.data_ptr(), ids.numel()
        else:
            ids = np.ascontiguousarray(_to_numpy(new_ids), dtype=np.int32)
            p, n = (ids.ctypes.data if len(ids) else 0), len(ids)
        res = C.c_int32()
        self._check(library().gbgpu_validate_permutation(self._h, p, n, DEVICE_POINTERS if dev else 0,
                                                           C.byref(res)))
        return res.value

    def relabel_by_mapping(self, row_ptr, col, new_ids):
        """Rebuilt CSR under new_ids and the new -> old map (org ids)."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        if dev:
            ids = new_ids.contiguous()
            pid = ids.data_ptr()
        else:
            ids = np.ascontiguousarray(_to_numpy(new_ids), dtype=np.int32)
            pid = ids.ctypes.data if n else 0
        orp, porp = self._out(n + 1, np.int64, dev, rp)
        ocol, pocol = self._out(nnz, np.int32, dev, rp)
        org, porg = self._out(n, np.int32, dev, rp)
        self._check(library().gbgpu_relabel_csr(self._h, prp, pcl, n, nnz, pid, porp, pocol, porg,
                                                  DEVICE_POINTERS if dev else 0))
        return orp, ocol, org

    def map_and_relabel(self, row_ptr, col, options=DEFAULT_RECIPE, auto_resolution=None, relabel=True):
        """The builder's mapping lifecycle on one resident graph: mapping,
        validation, relabel.  Returns (new_ids, out_row_ptr, out_col, stats)."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        ids, pids = self._out(n, np.int32, dev, rp)
        orp, porp = self._out(n + 1, np.int64, dev, rp) if relabel else (None, 0)
        ocol, pocol = self._out(nnz, np.int32, dev, rp) if relabel else (None, 0)
        st = GbgpuStats()
        ar = -1.0 if auto_resolution is None else float(auto_resolution)
        opts = options if isinstance(options, str) else ":".join(options)
        self._check(library().gbgpu_map_and_relabel(self._h, prp, pcl, n, nnz, opts.encode(), ar, pids, porp,
                                                       pocol, C.byref(st), DEVICE_POINTERS if dev else 0))
        return ids, orp, ocol, st.as_dict()

    def generate_mappings_batched(self, graphs, options=DEFAULT_RECIPE, streams=4, order=1, exact_window=0):
        """Map many graphs (list of (row_ptr, col) torch CUDA tensor pairs)
        concurrently.  Returns (list of new_ids tensors, list of stats dicts,
        wall ms)."""
        import torch
        count = len(graphs)
        arr = (GbgpuGraph * max(1, count))()
        outs, keep = [], []
        for i, (rp, col) in enumerate(graphs):
            if not (_is_cuda(rp) and _is_cuda(col)):
                raise ValueError("batched mapping takes CUDA tensors")
            rp, col = rp.contiguous(), col.contiguous()
            keep.append((rp, col))
            n = rp.numel() - 1
            ids = torch.empty(max(n, 0), dtype=torch.int32, device=rp.device)
            outs.append(ids)
            arr[i] = GbgpuGraph(rp.data_ptr(), col.data_ptr(), n, col.numel(), ids.data_ptr() if n else 0)
        if keep:
            torch.cuda.current_stream(keep[0][0].device).synchronize()
        sts = (GbgpuStats * max(1, count))()
        sched = GbgpuSchedule(int(streams), int(order), int(exact_window))
        wall = C.c_double()
        opts = options if isinstance(options, str) else ":".join(options)
        self._check(library().gbgpu_generate_mappings_batched(self._h, arr, count, opts.encode(), C.byref(sched),
                                                                C.cast(sts, C.c_void_p), C.byref(wall),
                                                                DEVICE_POINTERS))
        return outs, [sts[i].as_dict() for i in range(count)], wall.value

    # -- consumers timed after a mapping, DBG arm, selector ---------------------
    def _vertex_out(self, fn, row_ptr, col, dtype, *extra):
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        out, pout = self._out(n, dtype, dev, rp)
        ms = C.c_double()
        self._check(fn(self._h, prp, pcl, n, nnz, *extra, pout, C.byref(ms), DEVICE_POINTERS if dev else 0))
        return out, ms.value

    def selfcheck_delta(self, M, R, count=1 << 22, seed=1):
        """Results of the reciprocal-based deltaModularity that differ from
        full double divisions, over `count` seeded inputs (0 expected)."""
        bad = C.c_int64()
        self._check(library().gbgpu_selfcheck_delta(self._h, float(M), float(R), int(count), int(seed),
                                                    C.byref(bad)))
        return bad.value

    def pagerank(self, row_ptr, col, max_iters=20, epsilon=1e-4):
        """PageRank scores (float32), sweeps run, kernel ms."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        if dev:
            import torch
            out = torch.empty(n, dtype=torch.float32, device=rp.device)
            pout = out.data_ptr()
        else:
            out = np.zeros(n, dtype=np.float32)
            pout = out.ctypes.data if n else 0
        it, ms = C.c_int32(), C.c_double()
        self._check(library().gbgpu_pagerank(self._h, prp, pcl, n, nnz, int(max_iters), float(epsilon), pout,
                                               C.byref(it), C.byref(ms), DEVICE_POINTERS if dev else 0))
        return out, it.value, ms.value

    def bfs(self, row_ptr, col, source=0):
        """BFS depth per vertex (-1 unreached) and kernel ms."""
        return self._vertex_out(library().gbgpu_bfs, row_ptr, col, np.int32, C.c_int64(int(source)))

    def connected_components(self, row_ptr, col):
        """Smallest vertex id of each vertex's component, and kernel ms."""
        return self._vertex_out(library().gbgpu_connected_components, row_ptr, col, np.int32)

    def dbg_mapping(self, row_ptr, col):
        """DBG forward map (algorithm 5) and kernel ms."""
        return self._vertex_out(library().gbgpu_dbg_mapping, row_ptr, col, np.int32)

    def tier0_features(self, row_ptr, col) -> np.ndarray:
        """The nine Tier-0 sampled features (float64, host)."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        out = (C.c_double * 9)()
        self._check(library().gbgpu_tier0_features(self._h, prp, pcl, n, nnz, out, DEVICE_POINTERS if dev else 0))
        return np.array(out[:], dtype=np.float64)

    @staticmethod
    def mlp_param_count(in_dim: int) -> int:
        return library().gbgpu_mlp_param_count(int(in_dim))

    @staticmethod
    def _f32(a):
        return np.ascontiguousarray(_to_numpy(a), dtype=np.float32)

    def mlp_forward(self, params, X):
        p, x = self._f32(params), self._f32(X)
        rows, in_dim = x.shape
        y = np.zeros((rows, 3), dtype=np.float32)
        self._check(library().gbgpu_mlp_forward(self._h, p.ctypes.data, x.ctypes.data, rows, in_dim,
                                                  y.ctypes.data, 0))
        return y

    def select_arm(self, row_ptr, col, options, kernel="pr", model=None):
        """Algorithm 14 on one graph: ``options`` are the fields after "14:"
        (e.g. "_:_:_:learned-mlp:best-endtoend:1"), ``kernel`` the benchmark
        kind, ``model`` a SelectorModel (needed by learned-mlp).  Returns the
        selection as a dict (arm 12 / 5 / 0, recipe, reason, features)."""
        rp, cl, prp, pcl, n, nnz, dev = self._graph_args(row_ptr, col)
        out = GbgpuSelection()
        mp = model.ptr if model is not None else None
        self._check(library().gbgpu_select_arm(self._h, prp, pcl, n, nnz, options.encode(), KERNELS[kernel], mp,
                                                 C.byref(out), DEVICE_POINTERS if dev else 0))
        return out.as_dict()

    def mlp_gradient(self, params, X, T):
        """(gradient packed like params, mean squared error)."""
        p, x, t = self._f32(params), self._f32(X), self._f32(T)
        rows, in_dim = x.shape
        g = np.zeros_like(p)
        loss = C.c_float()
        self._check(library().gbgpu_mlp_gradient(self._h, p.ctypes.data, x.ctypes.data, t.ctypes.data, rows,
                                                   in_dim, g.ctypes.data, C.byref(loss), 0))
        return g, loss.value

    def mlp_train(self, params, X, T, epochs=200, batch=64, lr=1e-3, seed=0):
        """Adam on the GPU; returns (new params, last epoch's mean loss)."""
        p, x, t = self._f32(params).copy(), self._f32(X), self._f32(T)
        rows, in_dim = x.shape
        loss = C.c_float()
        self._check(library().gbgpu_mlp_train(self._h, p.ctypes.data, x.ctypes.data, t.ctypes.data, rows, in_dim,
                                                int(epochs), int(batch), float(lr), int(seed), C.byref(loss), 0))
        return p, loss.value


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context()
    return _default_ctx


class SelectorModel:
    """A learned selector loaded by the C ABI (gbgpu_selector_model_load)."""

    def __init__(self, path=SELECTOR_MODEL_PATH):
        self.ptr = C.POINTER(GbgpuSelectorModel)()
        rc = library().gbgpu_selector_model_load(path.encode(), C.byref(self.ptr))
        if rc != OK:
            _raise(rc, f"cannot load selector model {path}")

    def close(self):
        if self.ptr:
            library().gbgpu_selector_model_free(self.ptr)
            self.ptr = C.POINTER(GbgpuSelectorModel)()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def parse_selection_policy(options: str) -> dict:
    """ParseDeployableSelectionPolicy on the fields after "14:"; raises
    ValueError with the reference's exception text."""
    pol = GbgpuSelectionPolicy()
    err = C.create_string_buffer(512)
    rc = library().gbgpu_parse_selection_policy(options.encode(), C.byref(pol), err, 512)
    if rc != OK:
        _raise(rc, err.value.decode())
    return {"model": pol.model, "criterion": pol.criterion, "reuse": pol.reuse, "explicit": pol.reuse_explicit}


def generate_mapping(row_ptr, col, options=DEFAULT_RECIPE, auto_resolution=None):
    return default_context().generate_mapping(row_ptr, col, options, auto_resolution)[0]


def relabel_by_mapping(row_ptr, col, new_ids):
    return default_context().relabel_by_mapping(row_ptr, col, new_ids)


def validate_permutation(new_ids) -> int:
    return default_context().validate_permutation(new_ids)


def version() -> str:
    return library().gbgpu_version().decode()


def effective_config(options, auto_resolution: float = 1.0) -> dict:
    """The effective-config JSON as a dict."""
    return json.loads(parse_graphbrew_config(options, auto_resolution)[1])
