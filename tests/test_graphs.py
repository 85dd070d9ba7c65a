"""Synthetic graph generators and the AdjacencyGraph format."""
import os
import tempfile

import numpy as np

from lightne_gb300 import graphs


def check_symmetric_simple(off, nbrs):
    n = off.size - 1
    src = np.repeat(np.arange(n), np.diff(off))
    assert (src != nbrs).all(), "self loop"
    for u in range(min(n, 200)):
        row = nbrs[off[u]:off[u + 1]]
        assert (np.diff(row) > 0).all(), "row not strictly ascending"
    fwd = set(zip(src.tolist(), nbrs.tolist()))
    assert all((v, u) in fwd for u, v in list(fwd)[:5000])


def test_chung_lu_exact_edge_count():
    off, nbrs = graphs.chung_lu(1000, 5000, 2.1, seed=3)
    assert off.size == 1001 and nbrs.size == 10000
    check_symmetric_simple(off, nbrs)
    off2, nbrs2 = graphs.chung_lu(1000, 5000, 2.1, seed=3)
    assert np.array_equal(off, off2) and np.array_equal(nbrs, nbrs2)


def test_rmat_and_sbm_small():
    off, nbrs = graphs.rmat(10, 8, seed=3)
    assert off.size == 1025
    check_symmetric_simple(off, nbrs)
    off, nbrs, lab = graphs.sbm(2000, blocks=10, mean_degree=12, ratio=20, seed=6)
    check_symmetric_simple(off, nbrs)
    deg = np.diff(off).mean()
    assert 9 < deg < 15
    src = np.repeat(np.arange(2000), np.diff(off))
    same = (lab[src] == lab[nbrs]).mean()
    assert same > 0.4  # p_in/p_out = 20 with 10 blocks: ~2/3 of edges inside a block


def test_adjacency_graph_roundtrip():
    off, nbrs = graphs.chung_lu(300, 1000, 2.1, seed=1)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "g.adj")
        graphs.write_adjacency_graph(p, off, nbrs)
        txt = open(p).read().split()
        assert txt[0] == "AdjacencyGraph" and int(txt[1]) == 300 and int(txt[2]) == 2000
        off2, nbrs2 = graphs.read_adjacency_graph(p)
        assert np.array_equal(off, off2) and np.array_equal(nbrs, nbrs2)
        rp = np.array([0, 2, 3], dtype=np.int64)
        graphs.write_csr_bin(os.path.join(td, "m.csr"), rp, np.array([0, 1, 1], np.int32),
                             np.array([1, 2, 3], np.float32))
        a, b, c = graphs.read_csr_bin(os.path.join(td, "m.csr"))
        assert np.array_equal(a, rp) and b.tolist() == [0, 1, 1] and c.tolist() == [1, 2, 3]
