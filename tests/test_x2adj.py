"""The AdjacencyGraph converter (lightne_gb300.x2adj, the role of LightNE's
util/x2adj.py) and the binary AdjacencyGraph format: edge lists with and
without --make-sym, relabelling, .mat input, text and binary outputs read
back to the same arrays."""
import os

import numpy as np
import pytest
import scipy.io
import scipy.sparse as sp

from lightne_gb300 import graphs, x2adj


def _write_edges(path, pairs):
    with open(path, "w") as f:
        f.write("# a comment\n")
        for u, v in pairs:
            f.write("%d %d\n" % (u, v))


def test_edgelist_make_sym_text_and_binary(tmp_path):
    pairs = [(0, 1), (1, 2), (2, 0), (3, 3), (1, 0), (4, 2)]
    src = tmp_path / "g.edge"
    _write_edges(src, pairs)
    off, nbrs = x2adj.convert(str(src), str(tmp_path / "g.adj"), make_sym=True)
    toff, tnbrs = graphs.read_adjacency_graph(str(tmp_path / "g.adj"))
    assert np.array_equal(off, toff) and np.array_equal(nbrs, tnbrs)
    # expected: symmetric, no self loop, sorted neighbours, duplicates merged
    A = sp.csr_matrix((np.ones(nbrs.size), nbrs, off), shape=(5, 5))
    assert (A != A.T).nnz == 0 and A.diagonal().sum() == 0
    assert nbrs.tolist() == [1, 2, 0, 2, 0, 1, 4, 2]
    x2adj.convert(str(src), str(tmp_path / "g.bin"), make_sym=True, binary=True)
    boff, bnbrs = graphs.read_adjacency_binary(str(tmp_path / "g.bin"))
    assert np.array_equal(off, boff) and np.array_equal(nbrs, bnbrs)
    assert os.path.getsize(tmp_path / "g.bin") == 24 + 8 * 6 + 4 * 8


def test_edgelist_must_be_symmetric_without_make_sym(tmp_path):
    src = tmp_path / "g.txt"
    _write_edges(src, [(0, 1), (1, 2), (2, 1)])
    with pytest.raises(ValueError, match="not symmetric"):
        x2adj.convert(str(src), str(tmp_path / "g.adj"))
    _write_edges(src, [(0, 1), (1, 0)])
    off, nbrs = x2adj.convert(str(src), str(tmp_path / "g.adj"))
    assert nbrs.tolist() == [1, 0]


def test_relabel_and_idmap(tmp_path):
    src = tmp_path / "g.csv"
    _write_edges(src, [(100, 7), (7, 55), (55, 100)])
    off, nbrs = x2adj.convert(str(src), str(tmp_path / "g.adj"), make_sym=True, relabel=True,
                              idmap=str(tmp_path / "ids.txt"))
    assert off.size - 1 == 3
    ids = [tuple(map(int, l.split())) for l in open(tmp_path / "ids.txt")]
    assert ids == [(100, 0), (7, 1), (55, 2)]


def test_mat_input(tmp_path):
    off0, nbrs0 = graphs.chung_lu(200, 800, 2.1, seed=3)
    A = sp.csr_matrix((np.ones(nbrs0.size), nbrs0, off0), shape=(200, 200))
    scipy.io.savemat(tmp_path / "g.mat", {"network": A})
    off, nbrs = x2adj.convert(str(tmp_path / "g.mat"), str(tmp_path / "g.adj"))
    assert np.array_equal(off, off0) and np.array_equal(nbrs, nbrs0)


def test_binary_rejects_bad_files(tmp_path):
    p = tmp_path / "bad.bin"
    p.write_bytes(b"LNEADJ01" + b"\x00" * 8)
    with pytest.raises(Exception):
        graphs.read_adjacency_binary(str(p))
