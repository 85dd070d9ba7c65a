"""Benchmark of the LightNE hot path on one GB300 (driver contract).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2|c1]

Workload (default c2): seeded Chung-Lu power-law graph (exponent 2.1) with
n = 1,138,499 vertices and m = 2,990,443 undirected edges, T = 10, b = 1,
samples = 100 * m = 299,044,300 (-sample_ratio 1.883551 as a float), -sample 0.
A step is one pass of the NetSMF sparsifier over the graph: path sampling
into the pair table, trunc-log, canonical CSR.  `value` is samples per
second with the graph resident in HBM; `e2e` is the same metric through the
C ABI with host buffers (graph upload, sparsifier, CSR download every step).

Under torchrun (N > 1) every rank runs an independent replica of the
workload (no data-path collective: the sparsifier does not exchange data);
`value` is the total over ranks divided by the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (n, m, exponent, seed, walk_len, sample_ratio, tablesz)
    "c1": dict(n=10312, m=333983, seed=1, walk_len=10, sample_ratio=70.095396, tablesz=13_500_000,
               label="chung-lu n=10312 m=333983 T=10 b=1 samples=20*T*m"),
    "c2": dict(n=1138499, m=2990443, seed=2, walk_len=10, sample_ratio=1.883551, tablesz=200_000_000,
               label="chung-lu n=1138499 m=2990443 T=10 b=1 samples=100*m"),
}
METRIC = "embed secs, samples/s, SpMM HBM GB/s: BF16 vs FP32 GPU form at fixed FP64 error"


def load_graph(name):
    from lightne_gb300 import graphs
    w = WORKLOADS[name]
    path = graphs.graph_cache_path("%s_chunglu_%d_%d_s%d.npz" % (name, w["n"], w["m"], w["seed"]))
    if os.path.exists(path):
        z = np.load(path)
        return z["off"], z["nbrs"]
    off, nbrs = graphs.chung_lu(w["n"], w["m"], 2.1, seed=w["seed"])
    np.savez(path, off=off, nbrs=nbrs)
    return off, nbrs


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("LNE_BENCH_GLOO") is None else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, ws, rank):
    """CPU arm: the oracle port of the reference sparsifier (the reference's
    own code cannot be compiled on the benchmark host), all host threads,
    each step a bounded slice of the workload's directed edges."""
    if rank != 0:
        return
    from oracle import port
    off, nbrs = load_graph(args.workload)
    w = WORKLOADS[args.workload]
    ratio = float(np.float32(w["sample_ratio"]))
    frac = 0.25
    e_end = int(nbrs.size * frac)
    cores = os.cpu_count()
    secs = []
    got = 0
    for i in range(args.warmup + args.steps):
        n_s, sec = port.sample_range(off, nbrs, w["seed"], 0, e_end, walk_len=w["walk_len"], tablesz=w["tablesz"],
                                     sample_ratio=ratio, nthreads=cores)
        if i >= args.warmup:
            secs.append(sec)
            got = n_s
    per = float(np.mean(secs))
    val = got / per
    sample = "sampler+pair-table over the first %.0f%% of directed edges (%d samples/step)" % (frac * 100, got)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "samples/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
        "config": {"workload": w["label"], "stage": "sparsifier"},
        "cpu_baseline": {"value": val, "unit": "samples/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def cpu_baseline(off, nbrs, w):
    from oracle import port
    ratio = float(np.float32(w["sample_ratio"]))
    frac = 0.25
    e_end = int(nbrs.size * frac)
    cores = os.cpu_count()
    got, sec = port.sample_range(off, nbrs, w["seed"], 0, e_end, walk_len=w["walk_len"], tablesz=w["tablesz"],
                                 sample_ratio=ratio, nthreads=cores)
    return {"value": got / sec, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": "sampler+pair-table, first %.0f%% of directed edges (%d samples, %.1f s)" % (frac * 100, got,
                                                                                                sec)}


def run_ours(args, ws, rank, local):
    import torch

    from lightne_gb300 import _lib
    from lightne_gb300.api import Context, Graph, generate_trunc_log_matrix_v2
    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    ratio = float(np.float32(w["sample_ratio"]))
    off, nbrs = load_graph(args.workload)
    stream = torch.cuda.current_stream()
    ctx = Context(local, stream=stream.cuda_stream)
    d_off = torch.from_numpy(off).cuda()
    d_nbrs = torch.from_numpy(nbrs).cuda()
    g = Graph.from_device(ctx, off.size - 1, d_off.data_ptr(), d_nbrs.data_ptr(), int(off[-1]))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    seed = w["seed"] + rank

    def step():
        csr, st = generate_trunc_log_matrix_v2(ctx, g, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                               sample_ratio=ratio)
        csr.free()
        return st

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    stats = []
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (outside the step events)
            ev[i][0].record(stream)
            stats.append(step())
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    ms = allmax(ws, ms)
    samples = stats[-1]["samples_emitted"]
    value = samples * ws / (ms / 1e3)
    ms_sample = float(np.mean([s["ms_sample"] for s in stats]))

    # e2e through the C ABI with host (pinned) buffers: upload + sparsify + download
    off_p = torch.from_numpy(off).pin_memory().numpy()
    nbrs_p = torch.from_numpy(nbrs).pin_memory().numpy()
    e2e_t = []
    d2h = 0
    for i in range(max(1, min(args.steps, 3)) + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gg = Graph.from_numpy(ctx, off_p, nbrs_p)
        csr, st = generate_trunc_log_matrix_v2(ctx, gg, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                               sample_ratio=ratio)
        rp, col, val = csr.download()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        csr.free()
        gg.free()
        d2h = rp.nbytes + col.nbytes + val.nbytes
        if i > 0:
            e2e_t.append(t1 - t0)
    e2e_s = allmax(ws, float(np.mean(e2e_t)))
    h2d = off.nbytes + nbrs.nbytes

    if rank == 0:
        hbm, kind = peaks()
        bytes_per_sample = 70.0  # 54 B of walk gathers + 16 B slot touch at T=10
        achieved = samples * bytes_per_sample / (ms_sample / 1e3) / 1e9
        line = {
            "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded Chung-Lu; no dataset)",
            "config": {"workload": w["label"], "stage": "sparsifier (sampler, pair table, trunc-log, CSR)",
                       "samples_per_step": samples, "nnz": stats[-1]["nnz"], "distinct": stats[-1]["distinct"],
                       "capacity": stats[-1]["capacity"], "l2": "512 MiB flush between timed steps",
                       "ms_sample": ms_sample, "ms_trunclog": float(np.mean([s["ms_trunclog"] for s in stats])),
                       "ms_csr": float(np.mean([s["ms_csr"] for s in stats]))},
            "e2e": {"value": samples * ws / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s},
            "gpu_launches": int(stats[-1]["kernel_launches"]) * args.steps,
            "roofline": {"kernel": "k_sample (sampler + pair-table insert)", "bound": "hbm",
                         "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "peak_kind": kind, "bytes_model": "70 B/sample", "traffic": None},
            "clocks": clk.summary(),
        }
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(off, nbrs, w)
        print(json.dumps(line))
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        from lightne_gb300 import build
        if rank == 0:
            build.build()
        barrier(ws)
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
