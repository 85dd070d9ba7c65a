"""Regenerates the golden fixtures in this directory from the REFERENCE itself.

Run where the reference sources are checked out, naming their root:

    python tests/golden/make_golden.py --ref <reference checkout>

It builds the reference's own sparsifier and generator code with
oracle/Makefile (`make ref`, outputs under oracle/_ref/), runs them on small
seeded graphs, and writes:

  sparsify_<case>.npz   graph (offsets, nbrs), parameters, and the
                        reference's canonical CSR (row_ptr, col, val)
  propagate_<case>.npz  graph, input embedding a, parameters, and the outputs
                        of the reference's own chebyshev_expansion
                        (oracle/ref_propagate_harness.cc): a - conv, the
                        (A + I)(a - conv) product, the returned embedding
  randsvd_<case>.npz    parameters, sketch seed, and the singular values and
                        embedding of the reference's own MKLRedSVD::run +
                        compute_u_sigma_root (oracle/ref_randsvd_harness.cc)
                        on a golden sparsifier matrix, with the Gaussian
                        sketches Omega, P drawn by numpy from the seed
  rng_streams.json      pbbs::random known-answer streams and map_uint64_t
  trunclog_log.json     glibc log values at inputs whose float rounding is
                        close to a tie (the hard cases of the trunc-log value)

The fixtures are small so that they can be committed; the GPU tests and the
oracle tests read them without the reference tree.
"""
from __future__ import annotations

import argparse
import json
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from lightne_gb300 import graphs  # noqa: E402

# name: (graph builder, params)
CASES = {
    "chunglu300": (lambda: graphs.chung_lu(300, 2000, 2.1, seed=11),
                   dict(seed=1, walk_len=10, tablesz=200000, negative=1, sample=0, sample_ratio=1.0,
                        mem_ratio=1.0, upper=0)),
    "chunglu300_frac": (lambda: graphs.chung_lu(300, 2000, 2.1, seed=11),
                        dict(seed=7, walk_len=10, tablesz=200000, negative=1, sample=0, sample_ratio=0.37,
                             mem_ratio=1.0, upper=0)),
    "chunglu300_upper_neg5": (lambda: graphs.chung_lu(300, 2000, 2.1, seed=11),
                              dict(seed=99, walk_len=6, tablesz=200000, negative=5, sample=0,
                                   sample_ratio=1.0, mem_ratio=1.0, upper=1)),
    "chunglu1000_T3": (lambda: graphs.chung_lu(1000, 6000, 2.1, seed=12),
                       dict(seed=123456789, walk_len=3, tablesz=400000, negative=1, sample=0,
                            sample_ratio=0.5, mem_ratio=1.0, upper=0)),
    "path40": (lambda: graphs.path_graph(40),
               dict(seed=5, walk_len=10, tablesz=0, negative=1, sample=0, sample_ratio=3.0, mem_ratio=1.0,
                    upper=0)),
    "star30": (lambda: graphs.star_graph(30),
               dict(seed=6, walk_len=4, tablesz=0, negative=1, sample=0, sample_ratio=2.0, mem_ratio=1.0,
                    upper=0)),
    "complete10_T1": (lambda: graphs.complete_graph(10),
                      dict(seed=8, walk_len=1, tablesz=0, negative=1, sample=0, sample_ratio=5.0,
                           mem_ratio=1.0, upper=0)),
    "chunglu300_sample1": (lambda: graphs.chung_lu(300, 2000, 2.1, seed=11),
                           dict(seed=3, walk_len=10, tablesz=200000, negative=1, sample=1,
                                sample_ratio=1.0, mem_ratio=1.0, upper=0)),
    "single_edge": (lambda: graphs.csr_from_edges(2, np.array([0]), np.array([1])),
                    dict(seed=21, walk_len=10, tablesz=0, negative=1, sample=0, sample_ratio=8.0,
                         mem_ratio=1.0, upper=0)),
    "chunglu500_T20_neg2": (lambda: graphs.chung_lu(500, 3000, 2.1, seed=13),
                            dict(seed=2 ** 62 + 17, walk_len=20, tablesz=500000, negative=2, sample=0,
                                 sample_ratio=0.9, mem_ratio=1.0, upper=0)),
    "hubs2000": (lambda: graphs.chung_lu(2000, 8000, 2.02, seed=14),
                 dict(seed=31337, walk_len=8, tablesz=0, negative=1, sample=0, sample_ratio=1.2,
                      mem_ratio=1.0, upper=0)),
    "rmat10": (lambda: graphs.rmat(10, 8, seed=15),
               dict(seed=4242, walk_len=10, tablesz=0, negative=1, sample=0, sample_ratio=1.0,
                    mem_ratio=1.0, upper=0)),
}

# name: (graph builder, dim, order, mu, s, input seed) for the propagation
PROP_CASES = {
    "chunglu800_K10": (lambda: graphs.chung_lu(800, 6000, 2.1, seed=16), 16, 10, 0.2, 0.5, 1),
    "chunglu400_K3_mu05_s1": (lambda: graphs.chung_lu(400, 2500, 2.1, seed=17), 8, 3, 0.5, 1.0, 2),
    "star2500_K10": (lambda: graphs.star_graph(2500), 8, 10, 0.2, 0.5, 3),
    "path300_K2": (lambda: graphs.path_graph(300), 8, 2, 0.2, 0.5, 4),
    "rmat10_K10": (lambda: graphs.rmat(10, 8, seed=15), 16, 10, 0.2, 0.5, 5),
}

RNG_CASES = [(0, 0, 12), (1, 0, 8), (12345, (17 << 32) | 4, 16), (2 ** 63 + 5, 2 ** 40 + 3, 8),
             (time_seed := 1733240000, (1 << 32) | 2, 8)]


def run_ref_sparsify(ref_dir: str, off, nbrs, prm: dict):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_sparsify")
    with tempfile.TemporaryDirectory() as td:
        gpath = os.path.join(td, "g.adj")
        opath = os.path.join(td, "g.csr")
        graphs.write_adjacency_graph(gpath, off, nbrs)
        args = [exe, gpath, opath, str(prm["seed"]), str(prm["walk_len"]), str(prm["tablesz"]),
                str(prm["negative"]), str(prm["sample"]), repr(prm["sample_ratio"]),
                repr(prm["mem_ratio"]), str(prm["upper"])]
        env = dict(os.environ, NUM_THREADS="4")
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, env=env)
        return graphs.read_csr_bin(opath)


# name: (sparsifier golden case, rank, dim, normalize, sketch seed)
SVD_CASES = {
    "chunglu1000_T3_r24": ("chunglu1000_T3", 24, 16, 0, 1),
    "hubs2000_r40_norm": ("hubs2000", 40, 32, 1, 2),
    "rmat10_r32": ("rmat10", 32, 24, 0, 3),
}


def svd_sketches(n, rank, seed):
    """Omega (n x rank) then P (rank x rank), float32 N(0,1) from numpy's
    seeded generator (platform independent)."""
    rng = np.random.default_rng(seed)
    return (rng.standard_normal((n, rank)).astype(np.float32), rng.standard_normal((rank, rank)).astype(np.float32))


def run_ref_randsvd(rp, col, val, omega, P, rank, dim, normalize):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_randsvd")
    with tempfile.TemporaryDirectory() as td:
        cpath, opath, ppath, out = (os.path.join(td, x) for x in ("a.csr", "o.f32", "p.f32", "out.bin"))
        graphs.write_csr_bin(cpath, rp, col, val)
        omega.tofile(opath)
        P.tofile(ppath)
        subprocess.run([exe, cpath, opath, ppath, out, str(rank), str(dim), str(normalize)], check=True,
                       stdout=subprocess.DEVNULL, env=dict(os.environ, NUM_THREADS="4"))
        raw = open(out, "rb").read()
    assert raw[:8] == b"LNESVD01"
    n, r, d = (int(x) for x in np.frombuffer(raw[8:32], dtype=np.int64))
    S = np.frombuffer(raw[32:32 + 4 * r], dtype=np.float32).copy()
    o = 32 + 4 * r + 4 * n * r
    emb = np.frombuffer(raw[o:o + 4 * n * d], dtype=np.float32).reshape(n, d).copy()
    return S, emb


def make_randsvd_fixtures():
    for name, (case, rank, dim, normalize, seed) in SVD_CASES.items():
        z = np.load(os.path.join(HERE, "sparsify_%s.npz" % case))
        rp, col, val = z["row_ptr"], z["col"], z["val"]
        omega, P = svd_sketches(rp.size - 1, rank, seed)
        S, emb = run_ref_randsvd(rp, col, val, omega, P, rank, dim, normalize)
        np.savez_compressed(os.path.join(HERE, "randsvd_%s.npz" % name), S=S, emb=emb,
                            params=json.dumps(dict(matrix=case, rank=rank, dim=dim, normalize=normalize,
                                                   sketch_seed=seed)))
        print("%-24s n=%d rank=%d dim=%d" % (name, rp.size - 1, rank, dim))


def run_ref_propagate(off, nbrs, a, order, mu, s_):
    """The reference's chebyshev_expansion on (graph, a): returns a - conv,
    (A + I)(a - conv) and the embedding, each n x dim float32."""
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_propagate")
    with tempfile.TemporaryDirectory() as td:
        gpath, apath, opath = (os.path.join(td, x) for x in ("g.adj", "a.f32", "out.bin"))
        graphs.write_adjacency_graph(gpath, off, nbrs)
        np.ascontiguousarray(a, dtype=np.float32).tofile(apath)
        subprocess.run([exe, gpath, apath, opath, str(a.shape[1]), str(order), repr(mu), repr(s_)], check=True,
                       stdout=subprocess.DEVNULL, env=dict(os.environ, NUM_THREADS="4"))
        raw = open(opath, "rb").read()
    assert raw[:8] == b"LNEPRP01"
    n, d = (int(x) for x in np.frombuffer(raw[8:24], dtype=np.int64))
    m = np.frombuffer(raw[24:], dtype=np.float32).reshape(3, n, d)
    return m[0].copy(), m[1].copy(), m[2].copy()


def make_propagation_fixtures():
    for name, (mk, dim, order, mu, s_, aseed) in PROP_CASES.items():
        off, nbrs = mk()
        a = np.random.default_rng(aseed).standard_normal((off.size - 1, dim)).astype(np.float32)
        a_out, y, emb = run_ref_propagate(off, nbrs, a, order, mu, s_)
        np.savez_compressed(os.path.join(HERE, "propagate_%s.npz" % name), offsets=off, nbrs=nbrs, a=a,
                            a_out=a_out, y=y, emb=emb,
                            params=json.dumps(dict(dim=dim, order=order, mu=mu, s=s_)))
        print("%-24s n=%d m_dir=%d dim=%d K=%d" % (name, off.size - 1, nbrs.size, dim, order))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="root of the reference checkout (read only)")
    ap.add_argument("--only", nargs="*", help="regenerate only these sparsifier cases (and nothing else)")
    ap.add_argument("--propagation-only", action="store_true",
                    help="regenerate only the propagation and randomized-SVD fixtures")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + args.ref], check=True)
    if args.propagation_only:
        make_propagation_fixtures()
        make_randsvd_fixtures()
        return
    for name, (mk, prm) in CASES.items():
        if args.only and name not in args.only:
            continue
        off, nbrs = mk()
        rp, col, val = run_ref_sparsify(args.ref, off, nbrs, prm)
        np.savez_compressed(os.path.join(HERE, "sparsify_%s.npz" % name), offsets=off, nbrs=nbrs,
                            row_ptr=rp, col=col, val=val, params=json.dumps(prm))
        print("%-24s n=%d m_dir=%d nnz=%d" % (name, off.size - 1, nbrs.size, rp[-1]))
    if args.only:
        return
    make_propagation_fixtures()
    make_randsvd_fixtures()
    streams = []
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_rng")
    for seed, idx, cnt in RNG_CASES:
        out = subprocess.run([exe, str(seed), str(idx), str(cnt)], check=True, capture_output=True,
                             text=True).stdout.split("\n")
        rows = [ln.split() for ln in out[1:] if ln.strip()]
        streams.append({"seed": str(seed), "fork": str(idx), "forked_rand0": out[0].strip(),
                        "rand": [r[0] for r in rows], "next_rand0": [r[1] for r in rows],
                        "map_uint64": [r[2] for r in rows]})
    with open(os.path.join(HERE, "rng_streams.json"), "w") as f:
        json.dump(streams, f, indent=1)
    # glibc log at inputs near float-rounding ties (see lne_math.cuh)
    import math

    import mpmath
    mpmath.mp.prec = 256
    hard = []
    rng = np.random.default_rng(2024)
    targets = rng.uniform(0.01, 25.0, 4000)
    for t in targets:
        yb = struct.unpack("<Q", struct.pack("<d", float(t)))[0]
        yb = (yb & ~((1 << 29) - 1)) | (1 << 28)  # a double exactly halfway between two floats
        y = struct.unpack("<d", struct.pack("<Q", yb))[0]
        x = math.exp(y)
        xb = struct.unpack("<Q", struct.pack("<d", x))[0]
        for dx in range(-3, 4):
            xx = struct.unpack("<d", struct.pack("<Q", xb + dx))[0]
            lg = math.log(xx)
            lb = struct.unpack("<Q", struct.pack("<d", lg))[0]
            low = lb & ((1 << 29) - 1)
            if abs(low - (1 << 28)) <= 4 and len(hard) < 1500:
                cr = float(mpmath.log(mpmath.mpf(xx)))
                crb = struct.unpack("<Q", struct.pack("<d", cr))[0]
                hard.append(["%016x" % (xb + dx), "%016x" % lb, "%016x" % crb])
    with open(os.path.join(HERE, "trunclog_log.json"), "w") as f:
        json.dump({"note": "x, glibc log(x), correctly rounded log(x) (mpmath, 256 bits), as IEEE-754 "
                           "hex; the rounding of log(x) to float is within 4 ulp of a tie",
                   "cases": hard}, f, indent=0)
    print("rng cases", len(streams), "log hard cases", len(hard))


if __name__ == "__main__":
    main()
