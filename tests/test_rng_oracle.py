"""The oracle's counter-based generator against known-answer streams of the
reference's own pbbs::random / hash64_2 / map_uint64_t (tests/golden)."""
import json
import os

from conftest import GOLDEN
from oracle import port

MASK = (1 << 64) - 1


def h(x):
    return port.hash64_2(x & MASK)


def test_streams_match_reference():
    streams = json.load(open(os.path.join(GOLDEN, "rng_streams.json")))
    assert streams
    for s in streams:
        seed, idx = int(s["seed"]), int(s["fork"])
        state = h(h((idx + seed) & MASK))  # fork(i) = h(h(i + state))
        assert h(state) == int(s["forked_rand0"])
        for r, nxt, mp in zip(s["rand"], s["next_rand0"], s["map_uint64"]):
            assert h(state) == int(r)
            state = h(h(state))  # next() = h(h(state))
            assert h(state) == int(nxt)
            assert port.lib().lne_port_map_uint64(int(r)) == float(mp)


def test_hash_fixed_points():
    # splitmix64 finaliser: h(0) == 0 and it is a bijection on a few samples
    assert h(0) == 0
    vals = {h(i) for i in range(1000)}
    assert len(vals) == 1000
