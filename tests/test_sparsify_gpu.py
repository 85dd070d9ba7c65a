"""Parity of the device sparsifier (lne_sparsify through the C ABI) with the
reference: the reference's own CSR for small graphs (tests/golden), and the
oracle port (pinned to the reference) at config-1 size.  Bit-exact for
-sample 0: row_ptr, col and the float bits of every value."""
import glob
import json
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN
from lightne_gb300 import graphs
from lightne_gb300._lib import LNE_ERR_INVALID, LNE_ERR_TABLE_FULL, LneError
from lightne_gb300.api import Graph, generate_trunc_log_matrix_v2
from oracle import port

pytestmark = pytest.mark.gpu

CASES = sorted(glob.glob(os.path.join(GOLDEN, "sparsify_*.npz")))


def device_sparsify(ctx, off, nbrs, prm):
    g = Graph.from_numpy(ctx, off, nbrs)
    csr, st = generate_trunc_log_matrix_v2(ctx, g, prm["seed"], walk_len=prm["walk_len"], upper=prm["upper"],
                                           sample=prm["sample"], table_size=prm["tablesz"],
                                           negative=prm["negative"], sample_ratio=prm["sample_ratio"],
                                           mem_ratio=prm["mem_ratio"])
    out = csr.download()
    csr.free()
    g.free()
    return out, st


def assert_csr_equal(a, b, exact=True):
    assert np.array_equal(a[0], b[0]), "row_ptr differs"
    assert np.array_equal(a[1], b[1]), "col differs"
    if exact:
        diff = np.flatnonzero(a[2].view(np.uint32) != b[2].view(np.uint32))
        assert diff.size == 0, "values differ at %s: %s vs %s" % (diff[:5], a[2][diff[:5]], b[2][diff[:5]])
    else:
        np.testing.assert_allclose(a[2], b[2], rtol=1e-6, atol=0)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[9:-4] for c in CASES])
def test_device_matches_reference_golden(ctx, path):
    z = np.load(path)
    prm = json.loads(str(z["params"]))
    got, st = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
    assert_csr_equal(got, (z["row_ptr"], z["col"], z["val"]), exact=prm["sample"] == 0)
    assert st["nnz"] == z["row_ptr"][-1]


# Aggregation of the samples: the sliced shared-memory count (default), the
# pair table in HBM (slots = 0), a single 64-slot slice that overflows and
# reruns through the pair table, and forced slice counts.
AGGREGATION = {"table": (0, -1), "overflow64": (64, 0), "bits1": (256, 1), "bits9": (8192, 9)}


@pytest.mark.parametrize("mode", sorted(AGGREGATION))
def test_aggregation_paths_match_reference_golden(ctx, mode):
    slots, bits = AGGREGATION[mode]
    ctx.set_sparsify_slices(slots, bits)
    try:
        for path in CASES:
            z = np.load(path)
            prm = json.loads(str(z["params"]))
            if prm["sample"] != 0:
                continue
            got, st = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
            assert_csr_equal(got, (z["row_ptr"], z["col"], z["val"]))
            if mode == "table":
                assert st["sliced"] == 0
            elif mode == "overflow64":  # one slice of 64 slots
                assert st["sliced"] == (1 if st["distinct"] <= 64 else 0), (path, st["distinct"])
            elif mode == "bits1":  # two slices of 256 slots
                if st["distinct"] > 512:
                    assert st["sliced"] == 0
            else:
                assert st["sliced"] == 1
    finally:
        ctx.set_sparsify_slices()


def test_default_aggregation_is_sliced_for_counts(ctx):
    z = np.load(os.path.join(GOLDEN, "sparsify_chunglu300.npz"))
    prm = json.loads(str(z["params"]))
    _, st = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
    assert st["sliced"] == 1
    z = np.load(os.path.join(GOLDEN, "sparsify_chunglu300_sample1.npz"))
    prm = json.loads(str(z["params"]))
    _, st = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
    assert st["sliced"] == 0  # weights (-sample 1) always go through the pair table


def test_device_matches_oracle_config1(ctx):
    # config 1: Chung-Lu n=10,312, m=333,983, T=10, samples = 20*T*m (ratio as float)
    off, nbrs = graphs.chung_lu(10312, 333983, 2.1, seed=1)
    ratio = float(np.float32(70.095396))
    prm = dict(seed=1, walk_len=10, tablesz=13_500_000, negative=1, sample=0, sample_ratio=ratio, mem_ratio=1.0,
               upper=0)
    got, st = device_sparsify(ctx, off, nbrs, prm)
    assert st["sliced"] == 1
    ref, pst = port.sparsify(off, nbrs, 1, walk_len=10, tablesz=13_500_000, sample_ratio=ratio)
    assert st["samples_emitted"] == pst["samples"]
    assert st["distinct"] == pst["distinct"]
    assert st["m_exact"] == pst["M_exact"] and st["factor"] == pst["factor"]
    assert_csr_equal(got, ref)
    # the same matrix through the pair table in HBM
    ctx.set_sparsify_slices(0)
    try:
        got2, st2 = device_sparsify(ctx, off, nbrs, prm)
    finally:
        ctx.set_sparsify_slices()
    assert st2["sliced"] == 0 and st2["distinct"] == st["distinct"]
    assert_csr_equal(got2, ref)


def test_row_sort_tiers_match_reference_golden(ctx):
    """The hash-range rounds on every golden case with the rows of more than
    32 entries sorted through the column bitmap, in windows of 2048 columns
    (several windows where the graph has more vertices)."""
    ctx.set_sparsify_batch(4096)
    ctx.set_sparsify_rounds(1, 32)
    ctx.set_row_sort_window(2048)
    try:
        for path in CASES:
            z = np.load(path)
            prm = json.loads(str(z["params"]))
            if prm["sample"] != 0:
                continue
            got, _ = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
            assert_csr_equal(got, (z["row_ptr"], z["col"], z["val"]))
    finally:
        ctx.set_sparsify_rounds()
        ctx.set_row_sort_window()
        ctx.set_sparsify_batch(0)


def test_row_sort_windows_match_oracle_config1(ctx):
    """Config 1 through the rounds (n = 10,312: six bitmap windows of 2048
    columns; rows of more than 32 entries through the bitmap) against the
    port."""
    off, nbrs = graphs.chung_lu(10312, 333983, 2.1, seed=1)
    ratio = float(np.float32(70.095396))
    prm = dict(seed=1, walk_len=10, tablesz=13_500_000, negative=1, sample=0, sample_ratio=ratio, mem_ratio=1.0,
               upper=0)
    ctx.set_sparsify_batch(1 << 22)
    ctx.set_sparsify_rounds(1, 32)
    ctx.set_row_sort_window(2048)
    try:
        got, st = device_sparsify(ctx, off, nbrs, prm)
    finally:
        ctx.set_sparsify_rounds()
        ctx.set_row_sort_window()
        ctx.set_sparsify_batch(0)
    assert st["sliced"] == 2
    ref, _ = port.sparsify(off, nbrs, 1, walk_len=10, tablesz=13_500_000, sample_ratio=ratio)
    assert_csr_equal(got, ref)


def test_device_matches_oracle_config2(ctx):
    """Config 2 at full size: Chung-Lu n=1,138,499, m=2,990,443, T=10,
    samples = 100 * m (ratio 1.883551 as a float): 299M samples, 351M CSR
    entries, bit for bit against the port (about half a minute of host
    time on 16 cores)."""
    off, nbrs = graphs.chung_lu(1138499, 2990443, 2.1, seed=2)
    ratio = float(np.float32(1.883551))
    prm = dict(seed=2, walk_len=10, tablesz=200_000_000, negative=1, sample=0, sample_ratio=ratio, mem_ratio=1.0,
               upper=0)
    got, st = device_sparsify(ctx, off, nbrs, prm)
    assert st["sliced"] == 1
    assert st["nnz"] == 350_893_437
    ref, pst = port.sparsify(off, nbrs, 2, walk_len=10, tablesz=200_000_000, sample_ratio=ratio)
    assert st["samples_emitted"] == pst["samples"] == 299_044_249
    assert st["distinct"] == pst["distinct"]
    assert st["m_exact"] == pst["M_exact"] and st["factor"] == pst["factor"]
    assert_csr_equal(got, ref)


def test_device_matches_oracle_midsize_variants(ctx):
    off, nbrs = graphs.chung_lu(5000, 40000, 2.1, seed=9)
    for prm in [dict(seed=77, walk_len=5, tablesz=2_000_000, negative=3, sample=0, sample_ratio=0.8,
                     mem_ratio=1.0, upper=1),
                dict(seed=2 ** 63 + 11, walk_len=10, tablesz=2_000_000, negative=1, sample=0, sample_ratio=1.3,
                     mem_ratio=1.0, upper=0)]:
        got, _ = device_sparsify(ctx, off, nbrs, prm)
        ref, _ = port.sparsify(off, nbrs, prm["seed"], walk_len=prm["walk_len"], tablesz=prm["tablesz"],
                               negative=prm["negative"], sample_ratio=prm["sample_ratio"], upper=prm["upper"])
        assert_csr_equal(got, ref)


def test_device_matches_oracle_random_small_cases(ctx):
    """Seeded random small graphs and parameters (-sample 0): the device CSR
    (sliced aggregation by default) is the port's, bit for bit."""
    rng = np.random.default_rng(2026)
    for case in range(12):
        n = int(rng.integers(10, 400))
        m = min(n * int(rng.integers(1, 5)), n * (n - 1) // 4)
        off, nbrs = graphs.chung_lu(n, m, float(rng.choice([2.1, 2.5, 3.0])), seed=int(rng.integers(0, 10 ** 6)))
        if off[-1] == 0:
            continue
        walk_len = int(rng.integers(1, 13))
        prm = dict(seed=int(rng.integers(0, 2 ** 63 - 1)), walk_len=walk_len, tablesz=40 * walk_len * n,
                   negative=int(rng.integers(1, 6)), sample=0, sample_ratio=float(np.float32(rng.uniform(0.2, 3.0))),
                   mem_ratio=1.0, upper=int(rng.integers(0, 2)))
        got, st = device_sparsify(ctx, off, nbrs, prm)
        ref, _ = port.sparsify(off, nbrs, prm["seed"], walk_len=walk_len, tablesz=prm["tablesz"],
                               negative=prm["negative"], sample_ratio=prm["sample_ratio"], upper=prm["upper"])
        assert st["sliced"] == 1, case
        assert_csr_equal(got, ref)


def test_batched_samples_match_reference_golden(ctx):
    """Sample buffers of a few thousand keys: the edge range is walked in
    batches, each added to the pair table in turn (the path of runs above
    2^30 samples); the CSR is still the reference's."""
    ctx.set_sparsify_batch(4096)
    try:
        for path in CASES:
            z = np.load(path)
            prm = json.loads(str(z["params"]))
            got, st = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
            assert_csr_equal(got, (z["row_ptr"], z["col"], z["val"]), exact=prm["sample"] == 0)
            if st["samples_emitted"] > 4096:
                assert st["sliced"] == 0
    finally:
        ctx.set_sparsify_batch(0)


def test_rounds_match_reference_golden(ctx):
    """The hash-range rounds (the counts path above one batch when the pair
    table does not fit), forced with 4096-sample batches, so that a case
    runs up to hundreds of rounds; rows above 64 entries are sorted through
    the column bitmap.  The CSR is the reference's."""
    ctx.set_sparsify_batch(4096)
    ctx.set_sparsify_rounds(1, 64)
    try:
        for path in CASES:
            z = np.load(path)
            prm = json.loads(str(z["params"]))
            if prm["sample"] != 0:
                continue
            got, st = device_sparsify(ctx, z["offsets"], z["nbrs"], prm)
            assert_csr_equal(got, (z["row_ptr"], z["col"], z["val"]))
            if st["samples_emitted"] > 4096:
                assert st["sliced"] == 2, path
    finally:
        ctx.set_sparsify_rounds()
        ctx.set_sparsify_batch(0)


def test_rounds_match_oracle_config1(ctx):
    """Config 1 (26.75M entries) through 32 rounds of 2^22-sample batches,
    against the port."""
    off, nbrs = graphs.chung_lu(10312, 333983, 2.1, seed=1)
    ratio = float(np.float32(70.095396))
    prm = dict(seed=1, walk_len=10, tablesz=13_500_000, negative=1, sample=0, sample_ratio=ratio, mem_ratio=1.0,
               upper=0)
    ctx.set_sparsify_batch(1 << 22)
    ctx.set_sparsify_rounds(1, 0)
    try:
        got, st = device_sparsify(ctx, off, nbrs, prm)
    finally:
        ctx.set_sparsify_rounds()
        ctx.set_sparsify_batch(0)
    assert st["sliced"] == 2
    ref, pst = port.sparsify(off, nbrs, 1, walk_len=10, tablesz=13_500_000, sample_ratio=ratio)
    assert st["samples_emitted"] == pst["samples"] and st["distinct"] == pst["distinct"]
    assert st["m_exact"] == pst["M_exact"] and st["factor"] == pst["factor"]
    assert_csr_equal(got, ref)


def test_device_is_deterministic(ctx):
    off, nbrs = graphs.chung_lu(3000, 30000, 2.1, seed=4)
    prm = dict(seed=5, walk_len=10, tablesz=2_000_000, negative=1, sample=0, sample_ratio=1.0, mem_ratio=1.0,
               upper=0)
    a, _ = device_sparsify(ctx, off, nbrs, prm)
    b, _ = device_sparsify(ctx, off, nbrs, prm)
    assert_csr_equal(a, b)


def test_table_full_is_a_status_and_context_survives(ctx):
    off, nbrs = graphs.chung_lu(2000, 20000, 2.1, seed=2)
    prm = dict(seed=1, walk_len=10, tablesz=1000, negative=1, sample=0, sample_ratio=1.0, mem_ratio=0.0,
               upper=0)
    with pytest.raises(LneError) as ei:
        device_sparsify(ctx, off, nbrs, prm)
    assert ei.value.status == LNE_ERR_TABLE_FULL
    # the same context keeps working
    prm.update(tablesz=2_000_000, mem_ratio=1.0)
    got, _ = device_sparsify(ctx, off, nbrs, prm)
    assert got[0][-1] > 0
    # the rounds path reports the same status
    prm.update(tablesz=1000, mem_ratio=0.0)
    ctx.set_sparsify_batch(4096)
    ctx.set_sparsify_rounds(1, 0)
    try:
        with pytest.raises(LneError) as ei:
            device_sparsify(ctx, off, nbrs, prm)
        assert ei.value.status == LNE_ERR_TABLE_FULL
    finally:
        ctx.set_sparsify_rounds()
        ctx.set_sparsify_batch(0)


def test_invalid_graph_rejected(ctx):
    off = np.array([0, 1, 2], dtype=np.int64)
    nbrs = np.array([1, 5], dtype=np.int32)  # 5 is out of range
    with pytest.raises(LneError) as ei:
        Graph.from_numpy(ctx, off, nbrs)
    assert ei.value.status == LNE_ERR_INVALID
    with pytest.raises(LneError):
        Graph.from_numpy(ctx, np.array([0, 2, 1], dtype=np.int64), np.array([1, 0], dtype=np.int32))


def test_trunc_log_hard_cases(ctx, lib):
    cases = json.load(open(os.path.join(GOLDEN, "trunclog_log.json")))["cases"]
    x = np.array([struct.unpack("<d", struct.pack("<Q", int(c[0], 16)))[0] for c in cases])
    glibc = np.array([struct.unpack("<d", struct.pack("<Q", int(c[1], 16)))[0] for c in cases])
    cr = np.array([struct.unpack("<d", struct.pack("<Q", int(c[2], 16)))[0] for c in cases])
    out = np.empty_like(x)
    import ctypes
    rc = lib.lne_trunc_log_values(ctx.handle, ctypes.c_void_p(x.ctypes.data), x.size,
                                  ctypes.c_void_p(out.ctypes.data))
    assert rc == 0
    assert np.array_equal(out.view(np.uint64), cr.view(np.uint64))
    # against glibc: equal floats wherever glibc itself is correctly rounded
    ok = glibc.view(np.uint64) == cr.view(np.uint64)
    assert ok.mean() > 0.99
    assert np.array_equal(out[ok].astype(np.float32).view(np.uint32), glibc[ok].astype(np.float32).view(np.uint32))


def test_hub_rows_use_merge_passes(ctx):
    # a star plus a sparse Chung-Lu part: the hub's row of M has far more
    # than 16384 entries, so it is sorted in segments and merged
    from lightne_gb300.graphs import csr_from_edges
    n = 60000
    leaves = np.arange(1, n, dtype=np.int64)
    o2, n2 = graphs.chung_lu(n, 30000, 2.1, seed=8)
    src = np.repeat(np.arange(n), np.diff(o2))
    keep = src < n2
    lo = np.concatenate([np.zeros(n - 1, np.int64), src[keep]])
    hi = np.concatenate([leaves, n2[keep].astype(np.int64)])
    key = np.unique(lo * n + hi)
    off, nbrs = csr_from_edges(n, key // n, key % n)
    prm = dict(seed=31, walk_len=3, tablesz=3_000_000, negative=1, sample=0, sample_ratio=0.6, mem_ratio=1.0,
               upper=0)
    got, st = device_sparsify(ctx, off, nbrs, prm)
    rl = np.diff(got[0])
    assert rl.max() > 2 * 16384, rl.max()
    ref, _ = port.sparsify(off, nbrs, 31, walk_len=3, tablesz=3_000_000, sample_ratio=0.6)
    assert_csr_equal(got, ref)
