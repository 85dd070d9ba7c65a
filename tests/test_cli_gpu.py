"""The drop-in LightNE command line (lightne_gb300/bin/LightNE): same flags,
AdjacencyGraph input, raw float32 -ne_out / -pro_out outputs and log lines
as the reference binary (LightNE/LightNE.cc)."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT
from lightne_gb300 import graphs
from lightne_gb300.api import Graph, chebyshev_expansion, generate_trunc_log_matrix_v2, get_embedding_dense, randsvd

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "lightne_gb300", "bin", "LightNE")


def test_cli_matches_library(ctx, lib):
    off, nbrs = graphs.chung_lu(2000, 16000, 2.1, seed=30)
    with tempfile.TemporaryDirectory() as td:
        gpath = os.path.join(td, "g.adj")
        graphs.write_adjacency_graph(gpath, off, nbrs)
        ne, pro = os.path.join(td, "g.ne"), os.path.join(td, "g.pro")
        r = subprocess.run([EXE, "-walklen", "10", "-rounds", "1", "-s", "-m", "-ne_out", ne, "-pro_out", pro,
                            "-ne_method", "netsmf", "-rank", "40", "-dim", "32", "-order", "10", "-analyze", "1",
                            "-sample", "0", "-upper", "0", "-tablesz", "2000000", "-sample_ratio", "1.5",
                            "-seed", "12", gpath], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        assert "### n: 2000" in r.stdout and "### Running Time:" in r.stdout
        assert "###  -rank = 40" in r.stdout
        e_cli = np.fromfile(ne, dtype=np.float32).reshape(2000, 32)
        p_cli = np.fromfile(pro, dtype=np.float32).reshape(2000, 32)
    g = Graph.from_numpy(ctx, off, nbrs)
    csr, _ = generate_trunc_log_matrix_v2(ctx, g, 12, walk_len=10, table_size=2_000_000, sample_ratio=1.5)
    emb, _, _ = randsvd(ctx, csr, 40, 32, seed=777)
    y, _ = chebyshev_expansion(ctx, g, emb, 32, order=10)
    pro_lib, _ = get_embedding_dense(ctx, y, 32)
    assert np.array_equal(e_cli, emb.cpu().numpy())
    assert np.array_equal(p_cli, pro_lib.cpu().numpy())
    norms = np.linalg.norm(p_cli, axis=1)
    live = norms > 1e-5  # isolated vertices keep a zero row, as in the reference
    assert live.sum() > 1500
    np.testing.assert_allclose(norms[live], 1.0, rtol=1e-5)
    csr.free()
    g.free()


def test_cli_table_full_and_bad_input():
    off, nbrs = graphs.chung_lu(500, 4000, 2.1, seed=31)
    with tempfile.TemporaryDirectory() as td:
        gpath = os.path.join(td, "g.adj")
        graphs.write_adjacency_graph(gpath, off, nbrs)
        r = subprocess.run([EXE, "-rounds", "1", "-s", "-tablesz", "10", "-mem_ratio", "0", "-seed", "1", gpath],
                           capture_output=True, text=True, timeout=120)
        assert r.returncode == 3 and "looping forever" in r.stdout
        bad = os.path.join(td, "bad.adj")
        open(bad, "w").write("NotAGraph\n1\n0\n0\n")
        r = subprocess.run([EXE, "-s", bad], capture_output=True, text=True, timeout=60)
        assert r.returncode != 0 and "AdjacencyGraph" in r.stderr


def test_cli_binary_input_matches_text():
    """The binary AdjacencyGraph (lightne_gb300.x2adj --binary) gives the same
    run as the text file."""
    off, nbrs = graphs.chung_lu(1500, 9000, 2.1, seed=33)
    outs = []
    with tempfile.TemporaryDirectory() as td:
        for kind in ("text", "binary"):
            gpath = os.path.join(td, "g." + kind)
            if kind == "text":
                graphs.write_adjacency_graph(gpath, off, nbrs)
            else:
                graphs.write_adjacency_binary(gpath, off, nbrs)
            ne = os.path.join(td, kind + ".ne")
            r = subprocess.run([EXE, "-rounds", "1", "-s", "-ne_out", ne, "-rank", "24", "-dim", "16",
                                "-tablesz", "1000000", "-seed", "5", gpath], capture_output=True, text=True,
                               timeout=300)
            assert r.returncode == 0, r.stderr
            assert "### n: 1500" in r.stdout
            outs.append(np.fromfile(ne, dtype=np.float32))
    assert np.array_equal(outs[0], outs[1])
