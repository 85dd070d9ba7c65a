"""Convert an edge list or a .mat adjacency matrix to the AdjacencyGraph file
the LightNE command line reads, as text (the reference's format) or as the
binary AdjacencyGraph (LNEADJ01) that loads without text parsing.

The reference's converter is LightNE's util/x2adj.py (load_edgelist,
x2adjcencygraph): an edge list (.edge/.txt/.csv, one "u v" pair per line,
'#' comments) or a .mat file's "network" matrix becomes a symmetric,
self-loop-free, unweighted CSR with sorted neighbour lists.  The same rules
are applied here; ``--relabel`` maps the ids seen to 0..n-1 in order of
first appearance (``--idmap`` writes "original new" lines).

    python -m lightne_gb300.x2adj --file g.edge --output g.adj [--make-sym]
                                  [--relabel --idmap ids.txt] [--binary]
"""
from __future__ import annotations

import argparse
import pathlib
import sys

import numpy as np

from . import graphs


def load_edgelist(path: str, relabel: bool = False, make_sym: bool = False):
    """(n, lo, hi) of the undirected edges of an edge list: ids as integers,
    relabelled to 0..n-1 by first appearance when ``relabel``."""
    rows = []
    with open(path) as f:
        for line in f:
            line = line.strip()
            if not line or line.startswith("#"):
                continue
            parts = line.replace(",", " ").split()
            rows.append((int(parts[0]), int(parts[1])))
    data = np.array(rows, dtype=np.int64).reshape(-1, 2)
    ids = None
    if relabel:
        flat = data.reshape(-1)
        uniq, first = np.unique(flat, return_index=True)
        order = np.argsort(first, kind="stable")
        ids = uniq[order]
        remap = np.empty(uniq.size, dtype=np.int64)
        remap[order] = np.arange(uniq.size)
        data = remap[np.searchsorted(uniq, flat)].reshape(-1, 2)
        n = uniq.size
    else:
        n = int(data.max()) + 1 if data.size else 0
    u, v = data[:, 0], data[:, 1]
    if not make_sym:
        # the input must already list both directions; keep each pair once
        fwd = set(zip(u.tolist(), v.tolist()))
        missing = [(a, b) for a, b in fwd if (b, a) not in fwd and a != b]
        if missing:
            raise ValueError("%s: input is not symmetric (e.g. %s without its reverse); use --make-sym"
                             % (path, missing[0]))
    keep = u != v
    lo = np.minimum(u[keep], v[keep])
    hi = np.maximum(u[keep], v[keep])
    return n, lo, hi, ids


def load_mat(path: str, variable: str = "network"):
    """(n, lo, hi) of a symmetric .mat adjacency matrix (nonzeros as edges,
    the diagonal dropped)."""
    import scipy.io
    import scipy.sparse as sp
    A = sp.coo_matrix(scipy.io.loadmat(path)[variable])
    if A.shape[0] != A.shape[1]:
        raise ValueError("%s: the matrix is not square" % path)
    S = sp.csr_matrix(A)
    if (abs(S - S.T) > 1e-10).nnz:
        raise ValueError("%s: the matrix is not symmetric" % path)
    keep = (A.row != A.col) & (A.data != 0)
    lo = np.minimum(A.row[keep], A.col[keep]).astype(np.int64)
    hi = np.maximum(A.row[keep], A.col[keep]).astype(np.int64)
    return A.shape[0], lo, hi


def convert(path: str, output: str, make_sym: bool = False, relabel: bool = False, idmap: str | None = None,
            binary: bool = False):
    suffix = pathlib.Path(path).suffix
    ids = None
    if suffix == ".mat":
        n, lo, hi = load_mat(path)
    elif suffix in (".edge", ".txt", ".csv"):
        n, lo, hi, ids = load_edgelist(path, relabel=relabel, make_sym=make_sym)
    else:
        raise NotImplementedError("%s: unknown input type %r" % (path, suffix))
    keys = np.unique(lo * max(n, 1) + hi)
    off, nbrs = graphs.csr_from_edges(n, keys // max(n, 1), keys % max(n, 1))
    if binary:
        graphs.write_adjacency_binary(output, off, nbrs)
    else:
        graphs.write_adjacency_graph(output, off, nbrs)
    if idmap and ids is not None:
        with open(idmap, "w") as f:
            for new, orig in enumerate(ids.tolist()):
                f.write("%d %d\n" % (orig, new))
    return off, nbrs


def main(argv=None):
    ap = argparse.ArgumentParser("to AdjacencyGraph")
    ap.add_argument("--file", required=True, help="edge list (.edge/.txt/.csv) or .mat")
    ap.add_argument("--output", required=True)
    ap.add_argument("--make-sym", action="store_true", help="add the reverse of every edge")
    ap.add_argument("--relabel", action="store_true", help="map ids to 0..n-1 by first appearance")
    ap.add_argument("--idmap", help="with --relabel: write 'original new' id pairs here")
    ap.add_argument("--binary", action="store_true", help="write the binary AdjacencyGraph (LNEADJ01)")
    a = ap.parse_args(argv)
    off, nbrs = convert(a.file, a.output, a.make_sym, a.relabel, a.idmap, a.binary)
    print("wrote %s: n=%d, %d directed edges" % (a.output, off.size - 1, nbrs.size), file=sys.stderr)


if __name__ == "__main__":
    main()
