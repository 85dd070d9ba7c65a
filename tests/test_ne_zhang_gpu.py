"""-ne_method ne_zhang_et_al (LightNE/PathEmbed.h:410-463): the 1-hop log
matrix on the device against its FP64 restatement (structure identical,
values within one float ulp: the FP64 sums may round differently in the
last bit), the embedding (randsvd with normalised rows) against the FP64
oracle on the same sketch, and the command line against the library."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT
from lightne_gb300 import graphs
from lightne_gb300.api import Graph, gaussian, ne_zhang_matrix, randsvd
from oracle import linalg_oracle as lo

pytestmark = pytest.mark.gpu

EXE = os.path.join(ROOT, "lightne_gb300", "bin", "LightNE")


@pytest.fixture(scope="module")
def graph(ctx):
    off, nbrs = graphs.chung_lu(3000, 30000, 2.1, seed=41)
    g = Graph.from_numpy(ctx, off, nbrs)
    yield g, off, nbrs
    g.free()


def test_matrix_matches_restatement(ctx, graph):
    g, off, nbrs = graph
    M = ne_zhang_matrix(ctx, g)
    rp, col, val = M.download()
    ref = lo.ne_zhang_matrix(off, nbrs)
    assert np.array_equal(rp, ref.indptr) and np.array_equal(col, ref.indices)
    ulp = np.spacing(np.abs(ref.data).astype(np.float32))
    assert (np.abs(val - ref.data) <= ulp).all()
    assert (val == ref.data).mean() > 0.999
    M.free()


def test_embedding_matches_fp64(ctx, graph):
    g, off, nbrs = graph
    M = ne_zhang_matrix(ctx, g)
    rp, col, val = M.download()
    import scipy.sparse as sp
    A = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(off.size - 1, off.size - 1))
    rank, dim = 48, 32
    emb, S, _ = randsvd(ctx, M, rank, dim, normalize=True, seed=777)
    om = gaussian(ctx, 777, 0, A.shape[0], rank).double().cpu().numpy()
    P = gaussian(ctx, 777, 1, rank, rank).double().cpu().numpy()
    ref, Sref = lo.randsvd(A, om, P, dim, normalize=True)
    err = lo.procrustes_rel_error(emb.double().cpu().numpy(), ref)
    assert err < 1e-4, err
    assert lo.rel_sv_error(S[:dim], Sref[:dim]) < 1e-4
    M.free()


def test_cli_ne_zhang(ctx, graph):
    g, off, nbrs = graph
    with tempfile.TemporaryDirectory() as td:
        gpath = os.path.join(td, "g.adj")
        graphs.write_adjacency_graph(gpath, off, nbrs)
        ne = os.path.join(td, "g.ne")
        r = subprocess.run([EXE, "-rounds", "1", "-s", "-ne_out", ne, "-ne_method", "ne_zhang_et_al", "-rank", "40",
                            "-dim", "32", gpath], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        assert "###  -ne_method = ne_zhang_et_al" in r.stdout
        e_cli = np.fromfile(ne, dtype=np.float32).reshape(off.size - 1, 32)
    M = ne_zhang_matrix(ctx, g)
    emb, _, _ = randsvd(ctx, M, 40, 32, normalize=True, seed=777)
    assert np.array_equal(e_cli, emb.cpu().numpy())
    M.free()
