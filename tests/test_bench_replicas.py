"""The bench's multi-GPU path runs independent replicas (the pipeline has no
data-path exchange on one graph): ranks meet at barriers, the step time is
the max over ranks and the throughput is all ranks' units over that time.
Checked with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

from conftest import ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank), LNE_BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    ms = 100.0 + 25.0 * r  # rank 1 is the slower replica
    mx = bench.allmax(w, ms)
    out[r] = (w, mx, bench.replica_value(1000, w, mx))
    bench.barrier(w)
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_replicas_max_time_and_total_throughput():
    ws = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(ws, _free_port(), out), nprocs=ws, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for w, mx, val in res.values():
        assert w == 2
        assert mx == 125.0
        assert val == pytest.approx(2 * 1000 / 0.125)


def test_single_process_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.allmax(1, 3.5) == 3.5
    assert bench.replica_value(10, 1, 500.0) == pytest.approx(20.0)
