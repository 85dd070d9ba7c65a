"""Pins the oracle (oracle/sparsify_port.c) to the reference: the canonical
CSR of the reference's own sparsifier (tests/golden/sparsify_*.npz, made by
tests/golden/make_golden.py from the compiled reference code) must be
reproduced exactly."""
import glob
import json
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from oracle import port

CASES = sorted(glob.glob(os.path.join(GOLDEN, "sparsify_*.npz")))


def load_case(path):
    z = np.load(path)
    prm = json.loads(str(z["params"]))
    return z["offsets"], z["nbrs"], prm, (z["row_ptr"], z["col"], z["val"])


def run_port(off, nbrs, prm, nthreads=0):
    return port.sparsify(off, nbrs, prm["seed"], walk_len=prm["walk_len"], tablesz=prm["tablesz"],
                         negative=prm["negative"], sample=prm["sample"], sample_ratio=prm["sample_ratio"],
                         mem_ratio=prm["mem_ratio"], upper=prm["upper"], nthreads=nthreads)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[9:-4] for c in CASES])
def test_port_matches_reference_golden(path):
    off, nbrs, prm, (rp, col, val) = load_case(path)
    (rp2, col2, val2), st = run_port(off, nbrs, prm)
    assert np.array_equal(rp, rp2)
    assert np.array_equal(col, col2)
    if prm["sample"] == 0:
        assert np.array_equal(val.view(np.uint32), val2.view(np.uint32))
    else:
        # weights are sums of doubles in thread order: equal up to rounding
        np.testing.assert_allclose(val2, val, rtol=1e-6, atol=0)


def test_port_single_vs_many_threads_identical():
    off, nbrs, prm, _ = load_case(os.path.join(GOLDEN, "sparsify_chunglu1000_T3.npz"))
    a, _ = run_port(off, nbrs, prm, nthreads=1)
    b, _ = run_port(off, nbrs, prm, nthreads=4)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8))


def test_port_params_match_reference_formula():
    # M = T*n*ln(n)*ratio, 1/lambda = M/m_dir, capacity = 2^ceil(log2(2*max(T n ln n mem, tablesz)))
    p = port.params(10312, 667966, 10, 13_000_000, np.float32(70.095396).item(), 1.0)
    assert p["capacity"] == 2 ** 25
    assert p["exp_rv_rounded"] == 100
    assert 0.0 < p["frac"] < 1.0


REF_BIN = os.path.join(ROOT, "oracle", "_ref", "ref_sparsify")


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="reference build (oracle/_ref) not present")
def test_port_matches_live_reference_midsize():
    from lightne_gb300 import graphs
    off, nbrs = graphs.chung_lu(2000, 20000, 2.1, seed=5)
    prm = dict(seed=2024, walk_len=10, tablesz=3_000_000, negative=1, sample=0, sample_ratio=1.5,
               mem_ratio=1.0, upper=0)
    with tempfile.TemporaryDirectory() as td:
        g = os.path.join(td, "g.adj")
        o = os.path.join(td, "g.csr")
        graphs.write_adjacency_graph(g, off, nbrs)
        subprocess.run([REF_BIN, g, o, "2024", "10", "3000000", "1", "0", "1.5", "1.0", "0"], check=True,
                       stdout=subprocess.DEVNULL)
        rp, col, val = graphs.read_csr_bin(o)
    (rp2, col2, val2), _ = run_port(off, nbrs, prm)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
    assert np.array_equal(val.view(np.uint32), val2.view(np.uint32))


def test_port_table_full_status():
    off, nbrs, prm, _ = load_case(os.path.join(GOLDEN, "sparsify_chunglu300.npz"))
    # mem_ratio 0 and tablesz 1: capacity 2 slots, far fewer than the distinct pairs
    with pytest.raises(RuntimeError, match="status 3"):
        port.sparsify(off, nbrs, 1, walk_len=10, tablesz=1, mem_ratio=0.0, sample_ratio=1.0)


@pytest.mark.skipif(not os.path.exists(REF_BIN), reason="reference build (oracle/_ref) not present")
def test_port_matches_live_reference_property():
    """Property check: on random small graphs and parameters (-sample 0),
    the port's CSR is the reference's, bit for bit."""
    hypothesis = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")
    from lightne_gb300 import graphs

    @hypothesis.settings(max_examples=60, deadline=None, derandomize=True)
    @hypothesis.given(n=st.integers(10, 300), deg=st.integers(1, 4), exp=st.sampled_from([2.1, 2.5, 3.0]),
                      gseed=st.integers(0, 10 ** 6), seed=st.integers(0, 2 ** 63 - 1),
                      walk_len=st.integers(1, 12), negative=st.integers(1, 5), upper=st.integers(0, 1),
                      ratio=st.floats(0.2, 3.0))
    def check(n, deg, exp, gseed, seed, walk_len, negative, upper, ratio):
        m = min(n * deg, n * (n - 1) // 4)
        off, nbrs = graphs.chung_lu(n, m, exp, seed=gseed)
        if off[-1] == 0:
            return
        compared.append(int(off[-1]))
        ratio = float(np.float32(ratio))
        tablesz = 4 * walk_len * n * 10
        prm = dict(seed=seed, walk_len=walk_len, tablesz=tablesz, negative=negative, sample=0,
                   sample_ratio=ratio, mem_ratio=1.0, upper=upper)
        with tempfile.TemporaryDirectory() as td:
            g = os.path.join(td, "g.adj")
            o = os.path.join(td, "g.csr")
            graphs.write_adjacency_graph(g, off, nbrs)
            subprocess.run([REF_BIN, g, o, str(seed), str(walk_len), str(tablesz), str(negative), "0", repr(ratio),
                            "1.0", str(upper)], check=True, stdout=subprocess.DEVNULL)
            rp, col, val = graphs.read_csr_bin(o)
        (rp2, col2, val2), _ = run_port(off, nbrs, prm)
        assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
        assert np.array_equal(val.view(np.uint32), val2.view(np.uint32))

    compared = []
    check()
    assert len(compared) >= 45, compared
