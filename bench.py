"""Benchmark of the LightNE embedding pipeline on one GB300 (driver contract).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2|c1] [--accuracy]

Workload (default c2): seeded Chung-Lu power-law graph (exponent 2.1) with
n = 1,138,499 vertices and m = 2,990,443 undirected edges, T = 10, b = 1,
samples = 100 * m (-sample_ratio 1.883551 as a float), -sample 0, rank 138
(d = 128 + 10 oversampling), dim 128, order 10, mu = 0.2, s = 0.5.
A step is one full embedding: NetSMF sparsifier (path sampling into the pair
table, trunc-log, canonical CSR), randomized SVD and U sqrt(S), spectral
propagation, dense SVD embedding.  `value` is samples per second of the
whole pipeline (samples / step time) with the graph resident in HBM, for
the BF16 form (BF16 SpMM operands, FP32 accumulation); the FP32 form is
timed in the same run and reported beside it.  `e2e` is the same metric
through the C ABI with host buffers: graph upload, pipeline, embedding
download every step.  --accuracy additionally measures both forms against
the FP64 oracle (minutes of host time).

Under torchrun (N > 1) every rank runs an independent replica of the
workload: the pipeline has no data-path exchange on one graph; `value` is
the total over ranks divided by the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import warnings

import numpy as np

warnings.filterwarnings("ignore", message="Sparse CSR tensor support")
ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c1": dict(n=10312, m=333983, seed=1, walk_len=10, sample_ratio=70.095396, tablesz=13_500_000, rank=138,
               dim=128, order=10,
               label="chung-lu n=10312 m=333983 T=10 b=1 samples=20*T*m rank=138 dim=128 K=10"),
    "c2": dict(n=1138499, m=2990443, seed=2, walk_len=10, sample_ratio=1.883551, tablesz=200_000_000, rank=138,
               dim=128, order=10,
               label="chung-lu n=1138499 m=2990443 T=10 b=1 samples=100*m rank=138 dim=128 K=10"),
}
METRIC = "embed secs, samples/s, SpMM HBM GB/s: BF16 vs FP32 GPU form at fixed FP64 error"
SVD_SEED = 777


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

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in self.rows) if v is not None]
        mx = [v for v in (num(r[2]) for r in self.rows) if v is not None]
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


# ---------------------------------------------------------------------------
# CPU side (the oracle port of the reference, timed on the host cores)
# ---------------------------------------------------------------------------
def cpu_sparsify(off, nbrs, w):
    """The C port of the sparsifier on the full workload, all host threads:
    returns the CSR and its stats (sampling and CSR seconds)."""
    from oracle import cpu_pipeline, port
    cores = cpu_pipeline.set_threads()
    ratio = float(np.float32(w["sample_ratio"]))
    return port.sparsify(off, nbrs, w["seed"], walk_len=w["walk_len"], tablesz=w["tablesz"], sample_ratio=ratio,
                         nthreads=cores)


def cpu_pipeline_seconds(off, nbrs, w, sp=None, edge_frac=None):
    """Seconds of the reference pipeline on this host's cores: the C port of
    the sparsifier (the full run in `sp`, or, with edge_frac, the sampler
    over that fraction of the edges scaled to all samples plus the full
    run's CSR time), and the dense stages on a bounded sample scaled by
    operation count (oracle/cpu_pipeline.py)."""
    from oracle import cpu_pipeline, port
    cores = cpu_pipeline.set_threads()
    if sp is None:
        sp = cpu_sparsify(off, nbrs, w)
    (rp, col, val), st = sp
    t_sample, t_csr = st["sec_sample"], st["sec_csr"]
    if edge_frac is not None:
        ratio = float(np.float32(w["sample_ratio"]))
        got, sec = port.sample_range(off, nbrs, w["seed"], 0, int(nbrs.size * edge_frac), walk_len=w["walk_len"],
                                     tablesz=w["tablesz"], sample_ratio=ratio, nthreads=cores)
        t_sample = sec * st["samples"] / max(got, 1)
    dense = cpu_pipeline.dense_stage_seconds(rp, col, val, off, nbrs, rank=w["rank"], dim=w["dim"],
                                             order=w["order"])
    total = t_sample + t_csr + dense["randsvd"] + dense["propagate"] + dense["dense_embed"]
    return {"total": total, "sampler": t_sample, "csr": t_csr, "randsvd": dense["randsvd"],
            "propagate": dense["propagate"], "dense_embed": dense["dense_embed"], "samples": st["samples"],
            "cores": cores, "spmm_sample_rows": dense["spmm_sample_rows"], "edge_frac": edge_frac}


def cpu_sample_text(c):
    samp = ("sampler over the first %.0f%% of directed edges scaled to all samples" % (100 * c["edge_frac"])
            if c["edge_frac"] else "full sparsifier run")
    return ("C port of the sparsifier (%s: %.1f s sampling, %.1f s CSR); randomized SVD, propagation and dense "
            "SVD in torch FP32 on %d threads, SpMM timed over a 5%% row sample (%d rows) and scaled by nnz, "
            "QR/GEMM/SVD timed once and scaled by count"
            % (samp, c["sampler"], c["csr"], c["cores"], c["spmm_sample_rows"]))


def run_reference(args, ws, rank):
    """CPU arm: the oracle port of the reference (the reference's own code
    does not build on the benchmark host), every host thread.  One full
    sparsifier run sets up the matrix; each step then times a bounded sample
    (sampler over a quarter of the edges, dense stages on a row sample)."""
    if rank != 0:
        return
    off, nbrs = load_graph(args.workload)
    w = WORKLOADS[args.workload]
    sp = cpu_sparsify(off, nbrs, w)
    secs = []
    c = None
    for i in range(args.warmup + args.steps):
        c = cpu_pipeline_seconds(off, nbrs, w, sp=sp, edge_frac=0.25)
        if i >= args.warmup:
            secs.append(c["total"])
    per = float(np.mean(secs))
    val = c["samples"] / per
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "samples/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded Chung-Lu; no dataset)",
        "config": {"workload": w["label"], "stages_s": {k: c[k] for k in ("sampler", "csr", "randsvd",
                                                                           "propagate", "dense_embed")}},
        "cpu_baseline": {"value": val, "unit": "samples/s", "cores": c["cores"], "kind": "port",
                         "sample": cpu_sample_text(c)},
        "e2e": {"value": val, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def pipeline_step(ctx, g, w, precision, seed):
    from lightne_gb300.api import chebyshev_expansion, generate_trunc_log_matrix_v2, get_embedding_dense, randsvd
    ratio = float(np.float32(w["sample_ratio"]))
    csr, s1 = generate_trunc_log_matrix_v2(ctx, g, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                           sample_ratio=ratio)
    emb, S, s2 = randsvd(ctx, csr, w["rank"], w["dim"], precision=precision, seed=SVD_SEED)
    y, s3 = chebyshev_expansion(ctx, g, emb, w["dim"], order=w["order"], precision=precision)
    out, S2 = get_embedding_dense(ctx, y, w["dim"])
    nnz = csr.nnz
    csr.free()
    return out, emb, {"sparsify": s1, "randsvd": s2, "propagate": s3, "nnz": nnz}


def time_form(ctx, g, w, precision, seed, steps, warmup, stream, flush):
    import torch
    for _ in range(warmup):
        pipeline_step(ctx, g, w, precision, seed)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stats = []
    out = None
    for i in range(steps):
        flush.zero_()  # L2 flush between timed steps (outside the step events)
        ev[i][0].record(stream)
        out, emb, st = pipeline_step(ctx, g, w, precision, seed)
        ev[i][1].record(stream)
        stats.append(st)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    return ms, stats, out, emb


def launches_of(st):
    return (st["sparsify"]["kernel_launches"] + st["randsvd"]["kernel_launches"] +
            st["propagate"]["kernel_launches"] + 12)  # dense embed: QR3 (12 incl. gram/chol), gram, jacobi, gemm...


def run_ours(args, ws, rank, local):
    import torch

    from lightne_gb300.api import Context, Graph
    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    off, nbrs = load_graph(args.workload)
    stream = torch.cuda.current_stream()
    ctx = Context(local, stream=stream.cuda_stream)
    d_off = torch.from_numpy(off).cuda()
    d_nbrs = torch.from_numpy(nbrs).cuda()
    g = Graph.from_device(ctx, off.size - 1, d_off.data_ptr(), d_nbrs.data_ptr(), int(off[-1]))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    seed = w["seed"] + rank
    barrier(ws)
    with ClockSampler(local) as clk:
        ms_bf, st_bf, out_bf, emb_bf = time_form(ctx, g, w, "bf16", seed, args.steps, args.warmup, stream, flush)
        if args.quick:
            ms_fp, st_fp = ms_bf, st_bf
        else:
            ms_fp, st_fp, out_fp, emb_fp = time_form(ctx, g, w, "fp32", seed, args.steps, args.warmup, stream,
                                                     flush)
    barrier(ws)
    if args.quick:
        if rank == 0:
            print(json.dumps({"quick": True, "ms_per_step_bf16": ms_bf, "stages": st_bf[-1]}))
        ctx.close()
        return
    ms_bf = allmax(ws, ms_bf)
    ms_fp = allmax(ws, ms_fp)
    samples = st_bf[-1]["sparsify"]["samples_emitted"]
    value = samples * ws / (ms_bf / 1e3)

    # e2e through the C ABI with host (pinned) buffers: upload, pipeline, download
    off_p = torch.from_numpy(off).pin_memory().numpy()
    nbrs_p = torch.from_numpy(nbrs).pin_memory().numpy()
    e2e_t = []
    host_out = torch.empty(off.size - 1, w["dim"], dtype=torch.float32).pin_memory()
    for i in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gg = Graph.from_numpy(ctx, off_p, nbrs_p)
        out, _, _ = pipeline_step(ctx, gg, w, "bf16", seed)
        host_out.copy_(out)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        gg.free()
        if i > 0:
            e2e_t.append(t1 - t0)
    e2e_s = allmax(ws, float(np.mean(e2e_t)))
    h2d = off.nbytes + nbrs.nbytes
    d2h = host_out.numel() * 4

    if rank == 0:
        hbm, kind = peaks()
        s_last = st_bf[-1]
        n = off.size - 1
        nnz = s_last["nnz"]
        ld = (w["rank"] + 7) // 8 * 8

        def spmm_gbs(st, sx):
            ms = float(np.mean([x["randsvd"]["ms_spmm2"] for x in st]))
            comp = 8 * (n + 1) + 8 * nnz + n * ld * sx + n * ld * 4
            gath = 8 * (n + 1) + 8 * nnz + nnz * ld * sx + n * ld * 4
            return ms, comp / (ms / 1e3) / 1e9, gath / (ms / 1e3) / 1e9

        ms_spmm_bf, comp_bf, gath_bf = spmm_gbs(st_bf, 2)
        ms_spmm_fp, comp_fp, gath_fp = spmm_gbs(st_fp, 4)
        ms_sample = float(np.mean([x["sparsify"]["ms_sample"] for x in st_bf]))
        sampler_gbs = samples * 70.0 / (ms_sample / 1e3) / 1e9
        stage = lambda st, a, b: float(np.mean([x[a][b] for x in st]))  # noqa: E731
        # the largest single kernel: the sampler (one launch) or the SVD SpMM
        if ms_sample >= ms_spmm_bf:
            roof = {"kernel": "k_sample (path sampler + pair-table insert)", "bound": "hbm",
                    "achieved": sampler_gbs, "bytes_model": "70 B/sample (54 B walk gathers + 16 B slot)",
                    "ms_per_launch": ms_sample}
        else:
            roof = {"kernel": "k_spmm (B = A Q, BF16 operand)", "bound": "hbm", "achieved": comp_bf,
                    "bytes_model": "compulsory: 8(n+1) + 8 nnz + n ld 2 + n ld 4", "ms_per_launch": ms_spmm_bf}
        roof.update({"peak": hbm, "unit": "GB/s", "frac": roof["achieved"] / hbm, "peak_kind": kind,
                     "traffic": None})
        line = {
            "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_bf, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 SpMM operands, fp32 accumulate (int64 sparsifier)",
            "data": "synthetic (seeded Chung-Lu; no dataset)",
            "config": {
                "workload": w["label"], "samples_per_step": samples, "nnz": nnz,
                "l2": "512 MiB flush between timed steps",
                "embed_secs_bf16": ms_bf / 1e3, "embed_secs_fp32": ms_fp / 1e3,
                "fp32_form_value": samples * ws / (ms_fp / 1e3), "bf16_over_fp32_speedup": ms_fp / ms_bf,
                "stages_ms_bf16": {
                    "sample": ms_sample, "trunclog": stage(st_bf, "sparsify", "ms_trunclog"),
                    "csr": stage(st_bf, "sparsify", "ms_csr"), "randsvd": stage(st_bf, "randsvd", "ms_total"),
                    "propagate": stage(st_bf, "propagate", "ms_total")},
                "stages_ms_fp32": {
                    "randsvd": stage(st_fp, "randsvd", "ms_total"), "propagate": stage(st_fp, "propagate",
                                                                                       "ms_total")},
                "spmm_svd_bf16": {"ms": ms_spmm_bf, "GB/s_compulsory": comp_bf, "GB/s_gather": gath_bf},
                "spmm_svd_fp32": {"ms": ms_spmm_fp, "GB/s_compulsory": comp_fp, "GB/s_gather": gath_fp},
                "sampler_GB/s": sampler_gbs,
            },
            "e2e": {"value": samples * ws / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s},
            "gpu_launches": int(launches_of(s_last)) * args.steps,
            "roofline": roof,
            "clocks": clk.summary(),
        }
        if args.accuracy:
            line["accuracy"] = accuracy(ctx, g, w, seed, off, nbrs)
        if not args.no_cpu_baseline:
            c = cpu_pipeline_seconds(off, nbrs, w)
            line["cpu_baseline"] = {"value": c["samples"] / c["total"], "unit": "samples/s", "cores": c["cores"],
                                    "kind": "port", "sample": cpu_sample_text(c), "seconds": c["total"]}
        print(json.dumps(line))
    ctx.close()


def accuracy(ctx, g, w, seed, off, nbrs):
    """Both forms against the FP64 oracle on this workload (minutes of host
    time): randomized SVD singular values, subspace angle and embedding
    error after Procrustes, propagation output error, final embedding."""
    import scipy.sparse as sp
    import torch

    from lightne_gb300.api import chebyshev_expansion, gaussian, generate_trunc_log_matrix_v2, randsvd
    from oracle import linalg_oracle as lo
    ratio = float(np.float32(w["sample_ratio"]))
    csr, _ = generate_trunc_log_matrix_v2(ctx, g, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                          sample_ratio=ratio)
    rp, col, val = csr.download()
    n = off.size - 1
    A = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(n, n))
    res = {}
    # both forms share one (BF16-representable) sketch, so one FP64 run serves both
    P = gaussian(ctx, SVD_SEED, 1, w["rank"], w["rank"]).double().cpu().numpy()
    om = gaussian(ctx, SVD_SEED, 0, n, w["rank"]).double().cpu().numpy()
    t0 = time.perf_counter()
    ref, Sref = lo.randsvd(A, om, P, w["dim"])
    yref, _ = lo.propagate(off, nbrs, ref.astype(np.float32), order=w["order"])
    res["oracle_seconds"] = time.perf_counter() - t0
    for form in ("fp32", "bf16"):
        emb, S, _ = randsvd(ctx, csr, w["rank"], w["dim"], precision=form, seed=SVD_SEED)
        e = emb.double().cpu().numpy()
        # propagate the oracle's embedding so that the stage error is isolated
        y, _ = chebyshev_expansion(ctx, g, ref.astype(np.float32), w["dim"], order=w["order"], precision=form)
        yy = y.double().cpu().numpy()
        res[form] = {
            "svd_singular_values_max_rel": lo.rel_sv_error(S[:w["dim"]], Sref[:w["dim"]]),
            "svd_subspace_max_angle_rad": lo.max_principal_angle(e, ref),
            "svd_embedding_rel_frobenius_procrustes": lo.procrustes_rel_error(e, ref),
            "propagation_rel_frobenius": float(np.linalg.norm(yy - yref) / np.linalg.norm(yref)),
        }
    csr.free()
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--accuracy", action="store_true")
    ap.add_argument("--quick", action="store_true", help="BF16 form only, no e2e / CPU legs (for profiling)")
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
