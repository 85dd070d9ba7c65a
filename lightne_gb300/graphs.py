"""Seeded synthetic graphs and the ``AdjacencyGraph`` text format.

The reference reads undirected graphs as Ligra ``AdjacencyGraph`` text
(``ligra/graph_io.h:185-250``): the header token, ``n``, ``m`` (the number of
*directed* CSR entries, i.e. twice the undirected edge count), ``n`` offsets
and ``m`` neighbour ids, whitespace separated.  Neighbour order matters: the
random walk picks ``nbrs[off[u] + (rand % deg(u))]``
(``LightNE/PathEmbed.h:37-49``), so every generator here emits each row
sorted ascending and the file keeps that order.

Graphs are returned as ``(offsets int64[n+1], nbrs int32[2m])``: symmetric, no
self loops, no duplicate edges.
"""
from __future__ import annotations

import os
import struct

import numpy as np

__all__ = [
    "chung_lu",
    "rmat",
    "sbm",
    "csr_from_edges",
    "write_adjacency_graph",
    "read_adjacency_graph",
    "write_csr_bin",
    "read_csr_bin",
    "path_graph",
    "star_graph",
    "complete_graph",
]


def csr_from_edges(n: int, lo: np.ndarray, hi: np.ndarray):
    """Symmetric CSR from undirected edges (lo < hi, unique), rows sorted."""
    lo = np.asarray(lo, dtype=np.int64)
    hi = np.asarray(hi, dtype=np.int64)
    src = np.concatenate([lo, hi])
    dst = np.concatenate([hi, lo])
    order = np.lexsort((dst, src))
    src = src[order]
    dst = dst[order]
    deg = np.bincount(src, minlength=n).astype(np.int64)
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(deg, out=off[1:])
    return off, dst.astype(np.int32)


def _unique_edges_in_order(keys: np.ndarray) -> np.ndarray:
    """Unique values of ``keys`` in order of first appearance."""
    _, first = np.unique(keys, return_index=True)
    first.sort()
    return keys[first]


def chung_lu(n: int, m: int, exponent: float = 2.1, seed: int = 1):
    """Chung-Lu power-law graph with exactly ``m`` undirected edges.

    Vertex ``i`` has weight ``(i+1)^(-1/(exponent-1))``.  Endpoint pairs are
    drawn independently in proportion to the weights (numpy PCG64 seeded with
    ``seed``); self loops are dropped and duplicates removed, and the first
    ``m`` distinct edges in draw order are kept.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    w = np.power(np.arange(1, n + 1, dtype=np.float64), -1.0 / (exponent - 1.0))
    cdf = np.cumsum(w)
    cdf /= cdf[-1]
    have = np.zeros(0, dtype=np.int64)
    batch = max(1 << 16, int(m * 1.5))
    while have.size < m:
        a = np.searchsorted(cdf, rng.random(batch), side="right")
        b = np.searchsorted(cdf, rng.random(batch), side="right")
        a = np.minimum(a, n - 1)
        b = np.minimum(b, n - 1)
        keep = a != b
        lo = np.minimum(a[keep], b[keep])
        hi = np.maximum(a[keep], b[keep])
        keys = np.concatenate([have, lo * n + hi])
        have = _unique_edges_in_order(keys)
        batch = max(1 << 16, int((m - have.size) * 3) + 1024)
    have = have[:m]
    return csr_from_edges(n, have // n, have % n)


def rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
         c: float = 0.19, seed: int = 3):
    """R-MAT graph on 2^scale vertices, edge_factor * 2^scale draws,
    symmetrised, deduplicated, self loops removed."""
    n = 1 << scale
    draws = edge_factor * n
    rng = np.random.Generator(np.random.PCG64(seed))
    src = np.zeros(draws, dtype=np.int64)
    dst = np.zeros(draws, dtype=np.int64)
    chunk = 1 << 24
    for s in range(0, draws, chunk):
        e = min(draws, s + chunk)
        k = e - s
        u = np.zeros(k, dtype=np.int64)
        v = np.zeros(k, dtype=np.int64)
        for bit in range(scale):
            r = rng.random(k)
            right = (r >= a) & (r < a + b) | (r >= a + b + c)
            down = r >= a + b
            u |= down.astype(np.int64) << bit
            v |= right.astype(np.int64) << bit
        src[s:e] = u
        dst[s:e] = v
    keep = src != dst
    lo = np.minimum(src[keep], dst[keep])
    hi = np.maximum(src[keep], dst[keep])
    keys = np.unique(lo * n + hi)
    return csr_from_edges(n, keys // n, keys % n)


def sbm(n: int, blocks: int = 50, mean_degree: float = 24.0, ratio: float = 20.0,
        seed: int = 6):
    """Stochastic block model, equal blocks, p_in/p_out = ratio, expected
    mean degree ``mean_degree``.  Edges are drawn per block pair with a
    binomial count and uniform endpoints, then deduplicated.  Returns
    ``(offsets, nbrs, labels)``."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bs = n // blocks
    sizes = np.full(blocks, bs, dtype=np.int64)
    sizes[: n - bs * blocks] += 1
    starts = np.zeros(blocks + 1, dtype=np.int64)
    np.cumsum(sizes, out=starts[1:])
    # mean degree = p_in*(bs-1) + p_out*(n-bs); p_in = ratio * p_out
    p_out = mean_degree / (ratio * (bs - 1) + (n - bs))
    p_in = ratio * p_out
    los, his = [], []
    for i in range(blocks):
        for j in range(i, blocks):
            if i == j:
                pairs = sizes[i] * (sizes[i] - 1) // 2
                p = p_in
            else:
                pairs = sizes[i] * sizes[j]
                p = p_out
            cnt = rng.binomial(int(pairs), p)
            u = starts[i] + rng.integers(0, sizes[i], cnt)
            v = starts[j] + rng.integers(0, sizes[j], cnt)
            keep = u != v
            los.append(np.minimum(u[keep], v[keep]))
            his.append(np.maximum(u[keep], v[keep]))
    lo = np.concatenate(los)
    hi = np.concatenate(his)
    keys = np.unique(lo * n + hi)
    labels = np.repeat(np.arange(blocks, dtype=np.int32), sizes)
    off, nbrs = csr_from_edges(n, keys // n, keys % n)
    return off, nbrs, labels


def path_graph(n: int):
    i = np.arange(n - 1, dtype=np.int64)
    return csr_from_edges(n, i, i + 1)


def star_graph(n: int):
    i = np.arange(1, n, dtype=np.int64)
    return csr_from_edges(n, np.zeros_like(i), i)


def complete_graph(n: int):
    lo, hi = np.triu_indices(n, 1)
    return csr_from_edges(n, lo, hi)


def write_adjacency_graph(path: str, off: np.ndarray, nbrs: np.ndarray) -> None:
    """Write Ligra ``AdjacencyGraph`` text (offsets without the final entry)."""
    n = off.size - 1
    with open(path, "w") as f:
        f.write("AdjacencyGraph\n%d\n%d\n" % (n, nbrs.size))
        f.write("\n".join(map(str, off[:-1].tolist())))
        f.write("\n")
        if nbrs.size:
            f.write("\n".join(map(str, nbrs.tolist())))
            f.write("\n")


def read_adjacency_graph(path: str):
    """Parse ``AdjacencyGraph`` text, as ``ligra/graph_io.h:185-230`` does:
    whitespace tokens, the header, then n offsets and m targets; the final
    offset is set to m."""
    with open(path, "rb") as f:
        toks = f.read().split()
    if not toks or toks[0] != b"AdjacencyGraph":
        raise ValueError("%s: not an AdjacencyGraph file" % path)
    n = int(toks[1])
    m = int(toks[2])
    if len(toks) != n + m + 3:
        raise ValueError("%s: expected %d tokens, found %d" % (path, n + m + 3, len(toks)))
    arr = np.array(toks[3:], dtype=np.int64)
    off = np.empty(n + 1, dtype=np.int64)
    off[:n] = arr[:n]
    off[n] = m
    return off, arr[n:].astype(np.int32)


_ADJ_MAGIC = b"LNEADJ01"


def write_adjacency_binary(path: str, off: np.ndarray, nbrs: np.ndarray) -> None:
    """Binary AdjacencyGraph, read by the LightNE command line without text
    parsing: magic, int64 n, int64 m, int64 offsets[n+1], int32 targets[m]
    (little endian)."""
    off = np.ascontiguousarray(off, dtype=np.int64)
    with open(path, "wb") as f:
        f.write(_ADJ_MAGIC)
        f.write(struct.pack("<qq", off.size - 1, int(nbrs.size)))
        f.write(off.astype("<i8").tobytes())
        f.write(np.ascontiguousarray(nbrs, dtype="<i4").tobytes())


def read_adjacency_binary(path: str):
    with open(path, "rb") as f:
        if f.read(8) != _ADJ_MAGIC:
            raise ValueError("%s: not an LNEADJ01 file" % path)
        n, m = struct.unpack("<qq", f.read(16))
        off = np.frombuffer(f.read(8 * (n + 1)), dtype="<i8").astype(np.int64)
        nbrs = np.frombuffer(f.read(4 * m), dtype="<i4").astype(np.int32)
    if off[0] != 0 or off[-1] != m:
        raise ValueError("%s: offsets do not span the targets" % path)
    return off, nbrs


_CSR_MAGIC = b"LNECSR01"


def write_csr_bin(path: str, row_ptr, col, val) -> None:
    """Canonical CSR file: magic, int64 n, int64 nnz, int64 row_ptr[n+1],
    int32 col[nnz], float32 val[nnz]."""
    row_ptr = np.ascontiguousarray(row_ptr, dtype=np.int64)
    with open(path, "wb") as f:
        f.write(_CSR_MAGIC)
        f.write(struct.pack("<qq", row_ptr.size - 1, int(row_ptr[-1])))
        f.write(row_ptr.tobytes())
        f.write(np.ascontiguousarray(col, dtype=np.int32).tobytes())
        f.write(np.ascontiguousarray(val, dtype=np.float32).tobytes())


def read_csr_bin(path: str):
    with open(path, "rb") as f:
        if f.read(8) != _CSR_MAGIC:
            raise ValueError("%s: not an LNECSR01 file" % path)
        n, nnz = struct.unpack("<qq", f.read(16))
        row_ptr = np.frombuffer(f.read(8 * (n + 1)), dtype=np.int64).copy()
        col = np.frombuffer(f.read(4 * nnz), dtype=np.int32).copy()
        val = np.frombuffer(f.read(4 * nnz), dtype=np.float32).copy()
    return row_ptr, col, val


def graph_cache_path(name: str) -> str:
    root = os.environ.get("LNE_GRAPH_CACHE", os.path.join(os.path.dirname(__file__), "..", "_build", "graphs"))
    os.makedirs(root, exist_ok=True)
    return os.path.join(root, name)
