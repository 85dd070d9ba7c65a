"""Host build of lightne_gb300/csrc/lne_math.cuh (the same source the
kernels use): the double-double log behind the exact trunc-log value, and
the hash, against the golden hard cases (glibc and correctly rounded log)."""
import json
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

SRC = r'''
#include "lne_math.cuh"
#include <cstdio>
int main() {
  unsigned long long b;
  while (scanf("%llx", &b) == 1) {
    double x; __builtin_memcpy(&x, &b, 8);
    lne::dd r = lne::log_dd(x);
    double y = r.hi + r.lo;
    unsigned long long yb; __builtin_memcpy(&yb, &y, 8);
    printf("%016llx %d %016llx %016llx\n", yb, (int)lne::float_rounding_is_close(y),
           (unsigned long long)lne::hash64_2(b), (unsigned long long)lne::hash64_2_inv(b));
  }
}
'''


@pytest.fixture(scope="module")
def prog():
    td = tempfile.mkdtemp()
    src = os.path.join(td, "t.cc")
    exe = os.path.join(td, "t")
    open(src, "w").write(SRC)
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "lightne_gb300", "csrc"), src,
                    "-o", exe, "-lm"], check=True)
    return exe


def run(exe, xs_hex):
    out = subprocess.run([exe], input="\n".join(xs_hex), capture_output=True, text=True, check=True).stdout
    return [ln.split() for ln in out.strip().split("\n")]


def f64(h):
    return struct.unpack("<d", struct.pack("<Q", int(h, 16)))[0]


def test_log_dd_is_correctly_rounded_on_hard_cases(prog):
    cases = json.load(open(os.path.join(GOLDEN, "trunclog_log.json")))["cases"]
    assert len(cases) > 500
    rows = run(prog, [c[0] for c in cases])
    bad = [(c, r) for c, r in zip(cases, rows) if r[0] != c[2]]
    assert not bad, bad[:3]
    # every case is inside the window that routes to the slow path
    assert all(r[1] == "1" for r in rows)


def test_log_dd_random_inputs_match_glibc_float(prog):
    rng = np.random.default_rng(7)
    xs = rng.uniform(1.0, 5e6, 20000)
    hexes = ["%016x" % struct.unpack("<Q", struct.pack("<d", float(x)))[0] for x in xs]
    rows = run(prog, hexes)
    mism = 0
    for x, r in zip(xs, rows):
        mism += np.float32(f64(r[0])) != np.float32(np.log(x))
    assert mism == 0


def test_hash_matches_oracle(prog):
    from oracle import port
    xs = ["%016x" % v for v in [0, 1, 2, 12345, 2 ** 63, 2 ** 64 - 1]]
    rows = run(prog, xs)
    for x, r in zip(xs, rows):
        assert int(r[2], 16) == port.hash64_2(int(x, 16))


def test_hash_inverse_round_trips(prog):
    from oracle import port
    rng = np.random.default_rng(11)
    vals = [0, 1, 2 ** 63, 2 ** 64 - 1] + [int(v) for v in rng.integers(0, 2 ** 63, 2000, dtype=np.int64)]
    rows = run(prog, ["%016x" % v for v in vals])
    for v, r in zip(vals, rows):
        assert port.hash64_2(int(r[3], 16)) == v
    # the sliced aggregation uses the all-ones word as its empty marker: its
    # preimage is not a pair key (lo <= hi) of any graph with int32 vertex ids
    pre = int(run(prog, ["%016x" % (2 ** 64 - 1)])[0][3], 16)
    assert (pre & 0xffffffff) >= 2 ** 31 or (pre >> 32) >= 2 ** 31


GM_SRC = r'''
#include "lne_math.cuh"
#include <cstdio>
int main() {
  unsigned long long x; unsigned d;
  while (scanf("%llx %x", &x, &d) == 2)
    printf("%u\n", lne::gm_mod(x, d, lne::gm_magic(d)));
}
'''


def test_gm_mod_matches_64bit_remainder():
    td = tempfile.mkdtemp()
    src, exe = os.path.join(td, "g.cc"), os.path.join(td, "g")
    open(src, "w").write(GM_SRC)
    subprocess.run(["g++", "-O2", "-I", os.path.join(ROOT, "lightne_gb300", "csrc"), src, "-o", exe], check=True)
    rng = np.random.default_rng(5)
    ds = [1, 2, 3, 7, 10, 64, 65, 2 ** 31 - 1, 2 ** 31, 2 ** 31 + 1, 2 ** 32 - 1] + \
        [int(v) for v in rng.integers(1, 2 ** 32, 300)] + [int(v) for v in rng.integers(1, 5000, 300)]
    cases = []
    for d in ds:
        for x in [0, 1, d - 1, d, 2 ** 64 - 1, 2 ** 63] + [int(v) for v in rng.integers(0, 2 ** 63, 20)] + \
                [int(v) * 2 + 1 for v in rng.integers(2 ** 62, 2 ** 63, 5)]:
            cases.append((x % 2 ** 64, d))
    inp = "\n".join("%x %x" % (x, d) for x, d in cases)
    out = subprocess.run([exe], input=inp, capture_output=True, text=True, check=True).stdout.split()
    bad = [(x, d, int(o)) for (x, d), o in zip(cases, out) if int(o) != x % d]
    assert not bad, bad[:5]
