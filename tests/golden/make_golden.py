"""Regenerates the golden fixtures in this directory from the REFERENCE itself.

Run in a checkout that has the reference sources (default /root/reference):

    python tests/golden/make_golden.py [--ref /root/reference]

It builds the reference's own sparsifier and generator code with
oracle/Makefile (`make ref`, outputs under oracle/_ref/), runs them on small
seeded graphs, and writes:

  sparsify_<case>.npz   graph (offsets, nbrs), parameters, and the
                        reference's canonical CSR (row_ptr, col, val)
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    ap.add_argument("--only", nargs="*", help="regenerate only these sparsifier cases (and nothing else)")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + args.ref], check=True)
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
