"""Seeded synthetic graph generators producing squished undirected CSR graphs.

These build the inputs of the mapping path (the GAPBS builder's job in the
reference: ``bench/include/external/gapbs/generator.h:101-164`` generates the
edge list and ``builder.h:254-312`` symmetrizes, sorts, de-duplicates and drops
self-loops).

``gapbs`` is the reference's own graph: the edge list of ``converter -g/-u``
drawn by the library's host generator (``gbgpu_gapbs_edge_list``: per-block
``std::mt19937`` seeded with kRandSeed + block, ``std::shuffle`` id
permutation), then squished here with the builder's vertex count (largest id
+ 1).  The other generators are the project's seeded families: every random
draw is a counter-based SplitMix64 hash of ``(seed, stream, index)`` so the
same graph comes out of any device and any block partition.  Their RMAT
quadrant rule (A/B/C = 0.57/0.19/0.19 compared on 32-bit draws) follows
``generator.h:124-146``.

All functions take a ``device`` so bench-sized graphs are built in HBM; the
arithmetic is plain 64-bit integer work and gives identical graphs on CPU and
GPU.  Output: ``(row_ptr int64[n+1], col int32[nnz])`` with every row sorted
ascending and free of duplicates and self-loops.
"""
from __future__ import annotations

import math

import torch

_MASK64 = (1 << 64) - 1


def _s64(c: int) -> int:
    """Two's-complement int64 view of an unsigned 64-bit constant."""
    c &= _MASK64
    return c - (1 << 64) if c >= (1 << 63) else c


def _srl(x: torch.Tensor, k: int) -> torch.Tensor:
    """Logical right shift of an int64 tensor holding unsigned bits."""
    return (x >> k) & ((1 << (64 - k)) - 1)


_G = _s64(0x9E3779B97F4A7C15)
_M1 = _s64(0xBF58476D1CE4E5B9)
_M2 = _s64(0x94D049BB133111EB)


def mix64(x: torch.Tensor) -> torch.Tensor:
    """SplitMix64 finalizer (Steele, Lea & Flood 2014) on int64 bit patterns."""
    x = x + _G
    x = (x ^ _srl(x, 30)) * _M1
    x = (x ^ _srl(x, 27)) * _M2
    return x ^ _srl(x, 31)


def draw64(seed: int, stream: int, index: torch.Tensor) -> torch.Tensor:
    """64 random bits for each counter in ``index`` (int64 tensor)."""
    base = mix64(torch.tensor([_s64(seed * 0x100000001B3 + stream * 0x9E3779B1)],
                              dtype=torch.int64, device=index.device))
    return mix64(index ^ base)


def checksum(t: torch.Tensor) -> str:
    """Position-dependent 64-bit checksum of an integer array (on its own
    device): the wrapping sum over i of mix64(i * golden + t[i]), as 16 hex
    digits.  Equal arrays give equal sums; used to pin large CSR arrays against
    committed values without storing them."""
    x = t.reshape(-1).to(torch.int64)
    idx = torch.arange(x.numel(), dtype=torch.int64, device=x.device)
    total = int(mix64(idx * _G + x).sum().item())
    return "%016x" % (total & _MASK64)


def _permutation(n: int, seed: int, device) -> torch.Tensor:
    """A seeded permutation of 0..n-1 (rank of each id under a hash key)."""
    ids = torch.arange(n, dtype=torch.int64, device=device)
    key = draw64(seed, 2, ids)
    order = torch.sort(key, stable=True).indices
    perm = torch.empty_like(ids)
    perm[order] = ids
    return perm


def squish(src: torch.Tensor, dst: torch.Tensor, n: int):
    """Symmetrize, drop self-loops, sort rows and de-duplicate (builder.h:254-312)."""
    keep = src != dst
    src, dst = src[keep], dst[keep]
    a = torch.cat([src, dst])
    b = torch.cat([dst, src])
    del src, dst
    key = a * n + b
    del a, b
    key = torch.unique(key, sorted=True)
    u = torch.div(key, n, rounding_mode="floor")
    v = key - u * n
    del key
    counts = torch.bincount(u, minlength=n)
    row_ptr = torch.zeros(n + 1, dtype=torch.int64, device=u.device)
    row_ptr[1:] = torch.cumsum(counts, 0)
    return row_ptr, v.to(torch.int32)


def gapbs(scale: int, degree: int = 16, uniform: bool = False, device="cpu", threads: int = 0):
    """The graph GAPBS builds for ``-g <scale> -k <degree> -s`` (RMAT) or
    ``-u <scale> -k <degree> -s`` (uniform): same edge list, vertex count =
    largest id + 1 (builder.h:469-470), symmetrized and squished."""
    import numpy as np

    from graphbrew_gb300 import library
    lib = library()
    m = lib.gbgpu_gapbs_edge_count(scale, degree)
    if m < 0:
        raise ValueError(f"GAPBS generator: bad scale {scale} or degree {degree}")
    src = np.empty(max(m, 1), dtype=np.int32)
    dst = np.empty(max(m, 1), dtype=np.int32)
    rc = lib.gbgpu_gapbs_edge_list(scale, degree, int(bool(uniform)), src.ctypes.data, dst.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError(f"gbgpu_gapbs_edge_list failed with status {rc}")
    src, dst = src[:m], dst[:m]
    n = int(max(int(src.max()), int(dst.max())) + 1) if m > 0 else 0
    s = torch.from_numpy(src).to(device=device, dtype=torch.int64)
    d = torch.from_numpy(dst).to(device=device, dtype=torch.int64)
    del src, dst
    return squish(s, d, n)


def rmat(scale: int, edge_factor: int = 16, seed: int = 27491095, device="cpu",
         a: float = 0.57, b: float = 0.19, c: float = 0.19, permute: bool = True):
    """RMAT / Kronecker graph with 2^scale vertices and edge_factor * 2^scale edges."""
    n = 1 << scale
    m = n * edge_factor
    umax = 0xFFFFFFFF
    A, B, C = int(a * umax), int(b * umax), int(c * umax)
    e = torch.arange(m, dtype=torch.int64, device=device)
    src = torch.zeros(m, dtype=torch.int64, device=device)
    dst = torch.zeros(m, dtype=torch.int64, device=device)
    words = (scale + 1) // 2
    for j in range(words):
        r64 = draw64(seed, 1, e * words + j)
        for half in range(2):
            depth = 2 * j + half
            if depth >= scale:
                break
            r = (r64 & 0xFFFFFFFF) if half == 0 else _srl(r64, 32)
            src = src << 1
            dst = dst << 1
            top = r < (A + B)
            dst = dst + (top & (r > A)).to(torch.int64)
            bottom = ~top
            src = src + bottom.to(torch.int64)
            dst = dst + (bottom & (r > (A + B + C))).to(torch.int64)
        del r64
    del e
    if permute:
        perm = _permutation(n, seed, device)
        src, dst = perm[src], perm[dst]
    return squish(src, dst, n)


def uniform(log_n: int, degree: int = 16, seed: int = 27491095, device="cpu"):
    """Uniform-random graph with 2^log_n vertices and degree * 2^log_n edge draws
    (the count GAPBS draws for ``-u <log_n> -k <degree>``, generator.h:69-73)."""
    n = 1 << log_n
    m = n * degree
    e = torch.arange(m, dtype=torch.int64, device=device)
    src = _srl(draw64(seed, 3, 2 * e), 1) % n
    dst = _srl(draw64(seed, 3, 2 * e + 1), 1) % n
    del e
    return squish(src, dst, n)


def grid(rows: int, cols: int, delete_fraction: float = 0.05, seed: int = 27491095,
         device="cpu"):
    """4-neighbour rows x cols grid with a seeded fraction of edges deleted."""
    n = rows * cols
    r = torch.arange(rows, dtype=torch.int64, device=device)
    cidx = torch.arange(cols, dtype=torch.int64, device=device)
    rr, cc = torch.meshgrid(r, cidx, indexing="ij")
    v = (rr * cols + cc).reshape(-1)
    right_ok = (cc < cols - 1).reshape(-1)
    down_ok = (rr < rows - 1).reshape(-1)
    src = torch.cat([v[right_ok], v[down_ok]])
    dst = torch.cat([v[right_ok] + 1, v[down_ok] + cols])
    idx = torch.arange(src.numel(), dtype=torch.int64, device=device)
    threshold = int(math.ceil(delete_fraction * (1 << 32)))
    keep = _srl(draw64(seed, 4, idx), 32) >= threshold
    return squish(src[keep], dst[keep], n)


def planted_partition(n: int, communities: int, degree: int = 16, mixing: float = 0.1,
                      zipf_s: float = 1.2, seed: int = 27491095, device="cpu"):
    """Planted-partition graph: Zipf(s)-sized communities, a ``mixing`` fraction
    of edge endpoints drawn from the whole graph, ids shuffled.

    Returns ``(row_ptr, col, planted)`` where ``planted[v]`` is v's community.
    """
    k = max(1, min(communities, n))
    w = torch.tensor([1.0 / (i + 1) ** zipf_s for i in range(k)], dtype=torch.float64)
    sizes = torch.floor(w / w.sum() * n).to(torch.int64)
    sizes = torch.clamp(sizes, min=1)
    sizes[0] += n - int(sizes.sum())
    starts = torch.zeros(k + 1, dtype=torch.int64)
    starts[1:] = torch.cumsum(sizes, 0)
    starts = starts.to(device)
    sizes = sizes.to(device)
    block_of = torch.repeat_interleave(torch.arange(k, device=device), sizes)
    m = n * degree // 2
    e = torch.arange(m, dtype=torch.int64, device=device)
    u = _srl(draw64(seed, 5, 3 * e), 1) % n
    cu = block_of[u]
    inside = _srl(draw64(seed, 5, 3 * e + 1), 11).to(torch.float64) * (1.0 / (1 << 53)) >= mixing
    r2 = _srl(draw64(seed, 5, 3 * e + 2), 1)
    v_in = starts[cu] + r2 % sizes[cu]
    v_out = r2 % n
    v = torch.where(inside, v_in, v_out)
    perm = _permutation(n, seed, device)
    row_ptr, col = squish(perm[u], perm[v], n)
    planted = torch.empty(n, dtype=torch.int64, device=device)
    planted[perm] = block_of
    return row_ptr, col, planted


def from_edges(n: int, edges, device="cpu"):
    """CSR from an iterable of (u, v) pairs (symmetrized and squished)."""
    if len(edges) == 0:
        return torch.zeros(n + 1, dtype=torch.int64, device=device), torch.zeros(0, dtype=torch.int32, device=device)
    t = torch.tensor(edges, dtype=torch.int64, device=device)
    return squish(t[:, 0], t[:, 1], n)
