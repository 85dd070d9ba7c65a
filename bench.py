"""Benchmark of the LightNE embedding pipeline on one GB300 (driver contract).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload c2|c1|c3|c5] [--no-accuracy] [--no-cpu-baseline]
                    [--micro gram|gemm|spmm|spmm16|spmm8|prop] [--quick]

Workload (default c2): seeded Chung-Lu power-law graph (exponent 2.1) with
n = 1,138,499 vertices and m = 2,990,443 undirected edges, T = 10, b = 1,
samples = 100 * m (-sample_ratio 1.883551 as a float), -sample 0, rank 138
(d = 128 + 10 oversampling), dim 128, order 10, mu = 0.2, s = 0.5.
A step is one full embedding: NetSMF sparsifier (path sampling, pair
aggregation, trunc-log, canonical CSR), randomized SVD and U sqrt(S), spectral
propagation, dense SVD embedding.  `value` is samples per second of the
whole pipeline (samples / step time) with the graph resident in HBM, for
the FP16 form (FP16 SpMM operands, FP32 accumulation); the BF16 and FP32
forms are timed in the same run and reported beside it.  `e2e` is the same
metric through the C ABI with host buffers: graph upload, pipeline,
embedding download every step.  After the timed region, every form is
measured against the FP64 oracle (stage errors and the final embedding's,
with the 1e-3 gate), and the CPU port of the reference runs one whole
embedding on the host cores (`cpu_baseline`), whose sparse matrix is
compared bit for bit with the device's (`parity`).

Under torchrun (N > 1) every rank runs an independent replica of the
workload: the pipeline has no data-path exchange on one graph; `value` is
the total over ranks divided by the max time over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
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
    """Max of x over the ranks (a CUDA tensor under NCCL, a CPU one under gloo)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, ws, max_ms):
    """Whole-job throughput of ws independent replicas: the units all ranks
    processed over the slowest rank's time."""
    return units_per_rank * ws / (max_ms / 1e3)


# ---------------------------------------------------------------------------
# CPU side (the oracle port of the reference, timed on the host cores)
# ---------------------------------------------------------------------------
def cpu_pipeline_run(off, nbrs, w, seed):
    """One whole embedding of the workload by the CPU port of the reference
    pipeline (oracle/cpu_pipeline.py), every host thread, nothing scaled.
    Returns (pipeline, seconds)."""
    from oracle import cpu_pipeline
    pipe = cpu_pipeline.Pipeline(off, nbrs, w, seed)
    cpu_pipeline.warmup(off, nbrs, w, seed, pipe.cores, 2)
    secs = pipe.run()
    return pipe, secs


def cpu_sample_text(pipe, secs, steps=None):
    st = pipe.stage_s
    head = ("one whole embedding, every unit run once in order" if steps is None else
            "one whole embedding cut into %d steps of consecutive work units (the steps together run the "
            "pipeline once, in order)" % steps)
    return ("%s: C port of the sparsifier (%.1f s: sampler + pair table + trunc-log + CSR), randomized SVD "
            "(%.1f s), propagation (%.1f s) and dense SVD (%.1f s) in FP32 with row-parallel C CSR products "
            "and torch-CPU QR/GEMM/SVD on %d threads; %.1f s in total, nothing scaled"
            % (head, st.get("sparsify", 0.0), st.get("randsvd", 0.0), st.get("propagate", 0.0),
               st.get("dense_embed", 0.0), pipe.cores, secs))


def run_reference(args, ws, rank):
    """CPU arm: the oracle port of the reference pipeline (the reference's own
    code does not build on the benchmark host: it needs MKL), every host
    thread.  The K timed steps are K consecutive groups of the pipeline's
    work units, so together they run one whole embedding exactly once; the
    warm-up steps run sampler chunks in a throwaway table."""
    if rank != 0:
        return
    from oracle import cpu_pipeline
    off, nbrs = load_graph(args.workload)
    w = WORKLOADS[args.workload]
    pipe = cpu_pipeline.Pipeline(off, nbrs, w, w["seed"])
    cpu_pipeline.warmup(off, nbrs, w, w["seed"], pipe.cores, args.warmup)
    cuts = cpu_pipeline.step_groups(len(pipe.units), args.steps)
    secs = [pipe.run(cuts[i], cuts[i + 1]) for i in range(len(cuts) - 1)]
    total = float(np.sum(secs))
    val = pipe.samples / total
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": val, "unit": "samples/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / len(secs) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (seeded Chung-Lu; no dataset)",
        "config": {"workload": w["label"], "pipeline_seconds": total, "steps_timed": len(secs),
                   "units": len(pipe.units), "stages_s": dict(pipe.stage_s), "samples": pipe.samples},
        "cpu_baseline": {"value": val, "unit": "samples/s", "cores": pipe.cores, "kind": "port",
                         "sample": cpu_sample_text(pipe, total, len(secs))},
        "e2e": {"value": val, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------
def pipeline_step(ctx, g, w, precision, seed):
    from lightne_gb300.api import chebyshev_expansion, generate_trunc_log_matrix_v2, get_embedding_dense, randsvd
    # the 16-bit forms run one FP64 Jacobi sweep after the FP32 ones in both
    # core SVDs; the FP32 form sweeps in FP64 until they converge
    ctx.set_core_svd_fp64(1 if precision == "fp32" else 0)
    ratio = float(np.float32(w["sample_ratio"]))
    csr, s1 = generate_trunc_log_matrix_v2(ctx, g, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                           sample_ratio=ratio)
    emb, S, s2 = randsvd(ctx, csr, w["rank"], w["dim"], precision=precision, seed=SVD_SEED)
    y, s3 = chebyshev_expansion(ctx, g, emb, w["dim"], order=w["order"], precision=precision)
    out, S2 = get_embedding_dense(ctx, y, w["dim"])
    nnz = csr.nnz
    csr.free()
    return out, emb, {"sparsify": s1, "randsvd": s2, "propagate": s3, "nnz": nnz}


def launch_count(ctx):
    import ctypes

    from lightne_gb300 import _lib
    v = ctypes.c_int64()
    _lib.check(_lib.load().lne_ctx_launch_count(ctx.handle, ctypes.byref(v)))
    return v.value


def time_form(ctx, g, w, precision, seed, steps, warmup, stream, flush):
    """Mean ms per step of one form (CUDA events on the context's stream, L2
    flushed between steps) and the library's kernel launches in the timed
    steps."""
    import torch
    for _ in range(warmup):
        pipeline_step(ctx, g, w, precision, seed)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    stats = []
    out = emb = None
    launches = 0
    for i in range(steps):
        flush.zero_()  # L2 flush between timed steps (outside the step events)
        c0 = launch_count(ctx)
        ev[i][0].record(stream)
        out, emb, st = pipeline_step(ctx, g, w, precision, seed)
        ev[i][1].record(stream)
        launches += launch_count(ctx) - c0
        stats.append(st)
    torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    return ms, stats, out, emb, launches


class _DevArray:
    """A device buffer of the library seen by torch without a copy."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3}


def plain_fp32_step(ctx, g, w, seed, A_struct, lib):
    """The plain FP32 GPU form: the same sparsifier, then the reference's
    dense stages as unfused library calls on the GPU (cuSPARSE SpMM through
    torch.sparse, cuSOLVER QR and SVD, cuBLAS GEMMs, one elementwise kernel
    per axpy): MKLRedSVD::run (mklredsvd.cc:93-403), compute_u_sigma_root
    (PathEmbed.h:371-408), chebyshev_expansion (SpectralPropagation.h:45-221)
    and get_embedding_dense (SpectralPropagation.h:16-43)."""
    import ctypes

    import torch

    from lightne_gb300.api import generate_trunc_log_matrix_v2
    ratio = float(np.float32(w["sample_ratio"]))
    csr, _ = generate_trunc_log_matrix_v2(ctx, g, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                          sample_ratio=ratio)
    n, nnz, r, d = csr.n, csr.nnz, w["rank"], w["dim"]
    rp, cp, vp = csr.device_ptrs()
    crow = torch.as_tensor(_DevArray(rp, (n + 1,), "<i8"), device="cuda").to(torch.int32)
    col = torch.as_tensor(_DevArray(cp, (nnz,), "<i4"), device="cuda")
    val = torch.as_tensor(_DevArray(vp, (nnz,), "<f4"), device="cuda")
    A = torch.sparse_csr_tensor(crow, col, val, size=(n, n))
    omega = torch.empty(n, r, dtype=torch.float32, device="cuda")
    _lib_check(lib.lne_gaussian(ctx.handle, SVD_SEED, 0, n, r, ctypes.c_void_p(omega.data_ptr()), r))
    P = torch.empty(r, r, dtype=torch.float32, device="cuda")
    _lib_check(lib.lne_gaussian(ctx.handle, SVD_SEED, 1, r, r, ctypes.c_void_p(P.data_ptr()), r))
    Y = A @ omega
    Q = torch.linalg.qr(Y).Q
    B = A @ Q
    Z = torch.linalg.qr(B @ P).Q
    C = Z.T @ B
    U, S, _ = torch.linalg.svd(C)
    emb = Z @ (U[:, :d] * torch.sqrt(S[:d]))
    # propagation: M = (I - D~^-1 (A + I)) - mu I on the graph, recursion
    # with one SpMM and separate axpys per half-step
    crow_m, col_m, dt = A_struct
    mu, sp = 0.2, 0.5
    inv = 1.0 / dt
    vals = torch.empty(col_m.numel(), dtype=torch.float32, device="cuda")
    vals.copy_(torch.repeat_interleave(-inv, (crow_m[1:] - crow_m[:-1]).long()))
    vals[crow_m[:-1].long()] = 1.0 - mu - inv
    M = torch.sparse_csr_tensor(crow_m, col_m, vals, size=(n, n))
    coef = [float(x) for x in chebyshev_coef(w["order"], sp)]
    a = emb
    T0 = a
    T1 = 0.5 * (M @ (M @ a)) - a
    conv = coef[0] * T0 + coef[1] * T1
    for k in range(2, w["order"]):
        T2 = M @ (M @ T1) - 2.0 * T1 - T0
        conv = conv + coef[k] * T2
        T0, T1 = T1, T2
    a = a - conv
    ones = torch.ones(col_m.numel(), dtype=torch.float32, device="cuda")
    AI = torch.sparse_csr_tensor(crow_m, col_m, ones, size=(n, n))
    y = AI @ a
    Uy, Sy, _ = torch.linalg.svd(y, full_matrices=False)
    out = Uy * torch.sqrt(Sy)
    out = out / torch.clamp(out.norm(dim=1, keepdim=True), min=1e-30)
    csr.free()
    return out


def chebyshev_coef(order, s):
    from lightne_gb300.api import chebyshev_coefficients
    return chebyshev_coefficients(order, s)


def _lib_check(rc):
    from lightne_gb300 import _lib
    _lib.check(rc)


def _lib_load():
    from lightne_gb300 import _lib
    return _lib.load()


def plain_struct(off, nbrs):
    """CSR structure of A + I with the self loop first in every row (the
    operator's layout, SpectralPropagation.h:51-75) and d~ = degree + 1."""
    import torch
    n = off.size - 1
    deg = np.diff(off)
    crow = (off + np.arange(n + 1)).astype(np.int32)
    col = np.empty(crow[-1], dtype=np.int32)
    col[crow[:-1]] = np.arange(n, dtype=np.int32)
    mask = np.ones(crow[-1], dtype=bool)
    mask[crow[:-1]] = False
    col[mask] = nbrs
    return (torch.from_numpy(crow).cuda(), torch.from_numpy(col).cuda(),
            torch.from_numpy((deg + 1).astype(np.float32)).cuda())


def time_plain(ctx, g, w, seed, off, nbrs, steps, warmup, stream, flush):
    import torch

    from lightne_gb300 import _lib
    lib = _lib.load()
    st = plain_struct(off, nbrs)
    for _ in range(warmup):
        plain_fp32_step(ctx, g, w, seed, st, lib)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        plain_fp32_step(ctx, g, w, seed, st, lib)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return float(np.mean(times))


def profiled_traffic(name):
    """dram__bytes_read.sum + dram__bytes_write.sum per launch, from the line
    `traffic_bytes_per_launch: N` of a committed ncu summary in profiles/."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            return int(line.split(":")[1])
    return None


# The forms timed on the GPU: FP16 (the headline: 16-bit SpMM operands that
# meet the 1e-3 FP64 error gate), BF16 (the form as first specified: 16-bit
# operands with 8 significant bits), FP32 (the plain form).
FORMS = ("fp16", "bf16", "fp32")
HEADLINE = "fp16"
ERROR_GATE = 1e-3


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
    forms = (args.form or HEADLINE,) if args.quick else FORMS
    barrier(ws)
    res = {}
    with ClockSampler(local) as clk:
        for form in forms:
            res[form] = time_form(ctx, g, w, form, seed, args.steps, args.warmup, stream, flush)
    barrier(ws)
    if args.quick:
        if rank == 0:
            f0 = forms[0]
            print(json.dumps({"quick": True, "form": f0, "ms_per_step": res[f0][0], "stages": res[f0][1][-1],
                              "gpu_launches_per_step": res[f0][4] / args.steps}))
        ctx.close()
        return
    ms = {f: allmax(ws, res[f][0]) for f in forms}
    st_h = res[HEADLINE][1]
    samples = st_h[-1]["sparsify"]["samples_emitted"]
    value = replica_value(samples, ws, ms[HEADLINE])

    # e2e through the C ABI with host (pinned) buffers: upload, pipeline, download
    off_p = torch.from_numpy(off).pin_memory().numpy()
    nbrs_p = torch.from_numpy(nbrs).pin_memory().numpy()
    e2e_t, parts = [], []
    host_out = torch.empty(off.size - 1, w["dim"], dtype=torch.float32).pin_memory()
    for i in range(4):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gg = Graph.from_numpy(ctx, off_p, nbrs_p)  # host -> device copies and the graph build (synchronises)
        ta = time.perf_counter()
        out, _, _ = pipeline_step(ctx, gg, w, HEADLINE, seed)
        torch.cuda.synchronize()
        tb = time.perf_counter()
        # the embedding to the host through the C ABI (lne_copy_to_host)
        _lib_check(_lib_load().lne_copy_to_host(ctx.handle, ctypes.c_void_p(host_out.data_ptr()),
                                                ctypes.c_void_p(out.data_ptr()), out.numel() * 4))
        t1 = time.perf_counter()
        gg.free()
        if i > 0:
            e2e_t.append(t1 - t0)
            parts.append((ta - t0, tb - ta, t1 - tb))
    e2e_s = allmax(ws, float(np.mean(e2e_t)))
    e2e_parts = {k: float(np.mean([p_[j] for p_ in parts])) for j, k in enumerate(("upload_s", "pipeline_s",
                                                                                     "download_s"))}
    h2d = off.nbytes + nbrs.nbytes
    d2h = host_out.numel() * 4
    ms_plain = None
    if rank == 0 and not args.no_plain:
        ms_plain = time_plain(ctx, g, w, seed, off, nbrs, max(1, min(args.steps, 2)), 1, stream, flush)

    if rank == 0:
        hbm, kind = peaks()
        n = off.size - 1
        nnz = st_h[-1]["nnz"]
        ld = (w["rank"] + 7) // 8 * 8
        sx = {"fp32": 4, "bf16": 2, "fp16": 2}

        def spmm_gbs(form):
            ms_ = float(np.mean([x["randsvd"]["ms_spmm2"] for x in res[form][1]]))
            comp = 8 * (n + 1) + 8 * nnz + n * ld * sx[form] + n * ld * 4
            gath = 8 * (n + 1) + 8 * nnz + nnz * ld * sx[form] + n * ld * 4
            return {"ms": ms_, "GB/s_compulsory": comp / (ms_ / 1e3) / 1e9, "GB/s_gather": gath / (ms_ / 1e3) / 1e9,
                    "bytes_compulsory": comp}

        stage = lambda form, a, b: float(np.mean([x[a][b] for x in res[form][1]]))  # noqa: E731
        ms_sample = stage(HEADLINE, "sparsify", "ms_sample")
        sampler_gbs = samples * 70.0 / (ms_sample / 1e3) / 1e9
        # The roofline kernel: the randomized SVD's SpMM B = A Q (one lne_spmm
        # call per step: the main column slab, the tail slab from its dense
        # copy, the long-row chunk sums), timed by the library's CUDA events on
        # the launching stream.  Its DRAM traffic per call comes from the
        # committed ncu capture of the same call at this workload.
        sp_h = spmm_gbs(HEADLINE)
        traffic = profiled_traffic("spmm_fp16_c2.md") if args.workload == "c2" else None
        roof = {"kernel": "k_spmm<__half> (B = A Q, FP16 copy of 2^12 Q, n x %d: the main column slab, the "
                          "tail slab and the long-row chunk sums of one lne_spmm call)" % ld,
                "bound": "hbm", "achieved": sp_h["GB/s_compulsory"],
                "bytes_model": "compulsory 8(n+1) + 8 nnz + n ld 2 (Q) + n ld 4 (B) = %d B per call"
                               % sp_h["bytes_compulsory"],
                "ms_per_launch": sp_h["ms"], "achieved_gather_model": sp_h["GB/s_gather"],
                "peak": hbm, "unit": "GB/s", "frac": sp_h["GB/s_compulsory"] / hbm, "peak_kind": kind,
                "traffic": traffic,
                "traffic_GB/s": None if traffic is None else traffic / (sp_h["ms"] / 1e3) / 1e9}
        forms_cfg = {}
        for form in forms:
            forms_cfg[form] = {
                "embed_secs": ms[form] / 1e3, "samples_per_s": replica_value(samples, ws, ms[form]),
                "stages_ms": {"sample": stage(form, "sparsify", "ms_sample"),
                              "trunclog": stage(form, "sparsify", "ms_trunclog"),
                              "csr": stage(form, "sparsify", "ms_csr"),
                              "randsvd": stage(form, "randsvd", "ms_total"),
                              "propagate": stage(form, "propagate", "ms_total")},
                "spmm_B_AQ": spmm_gbs(form),
            }
        line = {
            "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms[HEADLINE], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp16 SpMM operands, fp32 accumulate (int64 sparsifier)",
            "data": "synthetic (seeded Chung-Lu; no dataset)",
            "config": {
                "workload": w["label"], "samples_per_step": samples, "nnz": nnz, "form": HEADLINE,
                "l2": "512 MiB flush between timed steps",
                "forms": forms_cfg,
                "fp16_over_fp32_speedup": ms["fp32"] / ms["fp16"],
                "bf16_over_fp32_speedup": ms["fp32"] / ms["bf16"],
                "sampler_GB/s": sampler_gbs,
                "plain_fp32_gpu": None if ms_plain is None else {
                    "embed_secs": ms_plain / 1e3, "fp16_form_speedup": ms_plain / ms[HEADLINE],
                    "form": "same sparsifier; dense stages as unfused cuSPARSE/cuSOLVER/cuBLAS calls via torch, "
                            "FP32"},
            },
            "e2e": {"value": samples * ws / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "seconds_per_step": e2e_s, "breakdown": e2e_parts},
            "gpu_launches": int(res[HEADLINE][4]),
            "roofline": roof,
            "clocks": clk.summary(),
        }
        csr_dev = None
        if not args.no_accuracy or not args.no_cpu_baseline:
            csr_dev = device_csr(ctx, g, w, seed)
        if not args.no_accuracy:
            line["accuracy"] = accuracy(ctx, g, w, off, nbrs, csr_dev, forms)
        if not args.no_cpu_baseline:
            pipe, secs = cpu_pipeline_run(off, nbrs, w, seed)
            line["cpu_baseline"] = {"value": pipe.samples / secs, "unit": "samples/s", "cores": pipe.cores,
                                    "kind": "port", "sample": cpu_sample_text(pipe, secs), "seconds": secs}
            rp, col, val = csr_dev
            prp, pcol, pval = pipe.csr
            line["parity"] = {
                "csr_bit_exact": bool(np.array_equal(rp, prp) and np.array_equal(col, pcol) and
                                      np.array_equal(val.view(np.uint32), pval.view(np.uint32))),
                "nnz": int(rp[-1]), "nnz_port": int(prp[-1]),
                "against": "the C port of the reference sparsifier (oracle/sparsify_port.c, pinned to the "
                           "reference's own generate_trunc_log_matrix_v2 by tests/golden), same seed"}
        print(json.dumps(line))
    ctx.close()


def device_csr(ctx, g, w, seed):
    """The device sparsifier's CSR of this workload, downloaded."""
    from lightne_gb300.api import generate_trunc_log_matrix_v2
    csr, _ = generate_trunc_log_matrix_v2(ctx, g, seed, walk_len=w["walk_len"], table_size=w["tablesz"],
                                          sample_ratio=float(np.float32(w["sample_ratio"])))
    out = csr.download()
    csr.free()
    return out


def run_micro(args, local):
    """One C-ABI call timed alone at the workload's sizes (CUDA events on the
    context's stream, 512 MiB L2 flush before every launch): the Gram
    (lne_gram, A = B, n x rank), the tall update GEMM (lne_gemm_tall,
    n x rank times rank x rank), the randomized SVD's SpMM B = A Q
    (lne_spmm, FP32 Q, n x ld), its sketch product Y = A Omega from the FP8
    copy (spmm8) or the whole spectral propagation (prop:
    lne_propagate, BF16 form, n x dim, order K on the graph; its bytes model
    is the compulsory traffic of its 2K - 1 SpMM half-steps and recursion
    streams).  Prints ms per launch and the bytes model."""
    import ctypes

    import torch

    from lightne_gb300 import _lib
    from lightne_gb300.api import Context, Graph, generate_trunc_log_matrix_v2
    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    ctx = Context(local, stream=stream.cuda_stream)
    n = w["n"]
    r = w["rank"]
    ld = (r + 7) // 8 * 8
    vp = ctypes.c_void_p
    X = torch.empty((n, ld), dtype=torch.float32, device="cuda")
    _lib.check(lib.lne_gaussian(ctx.handle, 1, 7, n, ld, vp(X.data_ptr()), ld))
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    csr = None
    if args.micro == "gram":
        G = torch.empty((r, r), dtype=torch.float64, device="cuda")
        call = lambda: lib.lne_gram(ctx.handle, vp(X.data_ptr()), ld, r, vp(X.data_ptr()), ld, r, n,  # noqa: E731
                                    vp(G.data_ptr()))
        model = n * ld * 4
        bytes_text = "n ld 4 (A read once)"
    elif args.micro == "gemm":
        W = torch.randn((r, r), dtype=torch.float32, device="cuda")
        Out = torch.empty((n, ld), dtype=torch.float32, device="cuda")
        call = lambda: lib.lne_gemm_tall(ctx.handle, vp(X.data_ptr()), ld, r, vp(W.data_ptr()), r, n,  # noqa: E731
                                         vp(Out.data_ptr()), ld)
        model = 2 * n * ld * 4
        bytes_text = "2 n ld 4 (In read, Out written)"
    elif args.micro == "prop":
        from lightne_gb300.api import PropagateParams
        off, nbrs = load_graph(args.workload)
        g = Graph.from_numpy(ctx, off, nbrs)
        d, K = w["dim"], w["order"]
        del X
        A0 = torch.randn((n, d), dtype=torch.float32, device="cuda", generator=torch.Generator("cuda").manual_seed(4))
        Yp = torch.empty_like(A0)
        prm = _lib.PropagateParams(dim=d, order=K, precision=_lib.LNE_PREC_BF16, mu=0.2, s=0.5)
        call = lambda: lib.lne_propagate(ctx.handle, g.handle, ctypes.byref(prm), vp(A0.data_ptr()),  # noqa: E731
                                         vp(Yp.data_ptr()), vp(0), None)
        m_dir = int(off[-1])
        # per SpMM (2K - 1 of them): vertex records (16 n) and neighbours
        # (4 m_dir) once, the BF16 operand once (2 n d), its FP32 result
        # written once (4 n d); the fused recursion streams are not counted
        model = (2 * K - 1) * (16 * n + 4 * m_dir + 6 * n * d)
        bytes_text = "(2K-1) (16 n + 4 m_dir + 2 n d + 4 n d): graph, BF16 operand once, FP32 result"
    else:
        off, nbrs = load_graph(args.workload)
        g = Graph.from_numpy(ctx, off, nbrs)
        csr, _ = generate_trunc_log_matrix_v2(ctx, g, w["seed"], walk_len=w["walk_len"], table_size=w["tablesz"],
                                              sample_ratio=float(np.float32(w["sample_ratio"])))
        g.free()
        Y = torch.empty((n, ld), dtype=torch.float32, device="cuda")
        if args.micro == "spmm16":
            # B = A Q of the FP16 form: an FP16 copy of 2^12 Q
            Xh = (X * 4096.0).to(torch.float16)
            del X
            call = lambda: lib.lne_spmm(ctx.handle, csr.handle, _lib.LNE_PREC_FP16,  # noqa: E731
                                        vp(Xh.data_ptr()), ld, ld, 1.0 / 4096.0, 0.0, vp(Y.data_ptr()), ld)
            model = 8 * (n + 1) + 8 * csr.nnz + n * ld * 2 + n * ld * 4
            bytes_text = "8(n+1) + 8 nnz + n ld 2 + n ld 4 (CSR, FP16 Q once, B written)"
        elif args.micro == "spmm8":
            # the sketch product Y = A Omega of the BF16 form: Omega's values
            # are e4m3-representable, so its FP8 copy is exact
            ldq = (r + 15) // 16 * 16
            om = torch.zeros((n, ldq), dtype=torch.float32, device="cuda")
            _lib.check(lib.lne_gaussian(ctx.handle, SVD_SEED, 0, n, r, vp(om.data_ptr()), ldq))
            Xq = om.to(torch.float8_e4m3fn)
            del om, X
            call = lambda: lib.lne_spmm(ctx.handle, csr.handle, _lib.LNE_PREC_FP8,  # noqa: E731
                                        vp(Xq.data_ptr()), ldq, ld, 1.0, 0.0, vp(Y.data_ptr()), ld)
            model = 8 * (n + 1) + 8 * csr.nnz + n * ldq + n * ld * 4
            bytes_text = "8(n+1) + 8 nnz + n ldq + n ld 4 (CSR, FP8 Omega once, Y written)"
        else:
            call = lambda: lib.lne_spmm(ctx.handle, csr.handle, 0, vp(X.data_ptr()), ld, ld, 1.0, 0.0,  # noqa: E731
                                        vp(Y.data_ptr()), ld)
            model = 8 * (n + 1) + 8 * csr.nnz + 2 * n * ld * 4
            bytes_text = "8(n+1) + 8 nnz + 2 n ld 4 (CSR, Q once, B written)"
    for panel_mb in [float(x) for x in str(args.panel_mb).split(",")]:
        _lib.check(lib.lne_ctx_set_spmm_panel_bytes(ctx.handle, int(panel_mb * (1 << 20))))
        for _ in range(args.warmup):
            _lib.check(call())
        torch.cuda.synchronize()
        times = []
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            _lib.check(call())
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        ms = float(np.mean(times))
        hbm, kind = peaks()
        print(json.dumps({"micro": args.micro, "panel_mb": panel_mb, "workload": w["label"], "n": n, "rank": r,
                          "ld": ld, "nnz": csr.nnz if csr else None, "ms_per_launch": ms, "bytes_model": bytes_text,
                          "bytes": model, "GB/s": model / (ms / 1e3) / 1e9, "peak_GB/s": hbm, "peak_kind": kind,
                          "frac": model / (ms / 1e3) / 1e9 / hbm}))
    if csr:
        csr.free()
    if args.micro == "prop":
        g.free()
    ctx.close()


SCALE_RUNS = {
    "c3": dict(kind="rmat", scale=22, edge_factor=16, seed=3, walk_len=10, per_edge=100, tablesz=4_250_000_000,
               rank=138, dim=128, order=10,
               label="R-MAT (0.57, 0.19, 0.19, 0.05) scale 22 edge factor 16 symmetrised dedup, T=10, "
                     "samples=10*T*m, rank 138, dim 128, K=10"),
    "c5": dict(kind="sbm", n=1 << 23, blocks=50, degree=24.0, ratio=20.0, seed=6, walk_len=10, per_edge=100,
               tablesz=8_500_000_000, rank=138, dim=128, order=10, adam_steps=20,
               label="SBM n=2^23, 50 equal blocks, mean degree 24, p_in/p_out=20, T=10, samples=10*T*m (a pair "
                     "table of 2^34 slots, 275 GB, does not fit: hash-range rounds), rank 138, dim 128, K=10, "
                     "20 Adam steps"),
}


def csr_checksum(csr):
    """Order-sensitive checksum of a device CSR (row_ptr, col, float bits),
    in 2^28-entry chunks (int64 sums wrap)."""
    import torch
    rp, cp, vp = csr.device_ptrs()
    n, nnz = csr.n, csr.nnz
    rpt = torch.as_tensor(_DevArray(rp, (n + 1,), "<i8"), device="cuda")
    colt = torch.as_tensor(_DevArray(cp, (nnz,), "<i4"), device="cuda")
    valt = torch.as_tensor(_DevArray(vp, (nnz,), "<i4"), device="cuda")
    mono = bool((rpt[1:] >= rpt[:-1]).all().item()) and int(rpt[-1].item()) == nnz
    h = int((rpt * 1000003).sum().item())
    step = 1 << 28
    for a in range(0, nnz, step):
        b = min(nnz, a + step)
        idx = torch.arange(a, b, device="cuda", dtype=torch.int64)
        h += int((colt[a:b].long() * 2654435761 + valt[a:b].long() * 40503 + idx).sum().item())
        h &= (1 << 63) - 1
    return h, mono


def run_scale(args, local):
    """Configs 3 and 5 at full size (not the headline line): the sparsifier
    twice (same CSR checksum: determinism at size), both SVD and propagation
    forms, BF16 vs FP32 embedding distance; config 5 then learns (mu, s)
    and a softmax classifier on the planted blocks with 20 Adam steps
    through the propagation adjoint (10% seeded training split)."""
    import math

    import torch

    from lightne_gb300 import graphs
    from lightne_gb300.api import (ChebyshevPropagation, Context, Graph, chebyshev_expansion,
                                   generate_trunc_log_matrix_v2, get_embedding_dense, randsvd)
    from oracle import linalg_oracle as lo
    torch.cuda.set_device(local)
    w = SCALE_RUNS[args.workload]
    t0 = time.time()
    labels = None
    if w["kind"] == "rmat":
        off, nbrs = graphs.rmat(w["scale"], w["edge_factor"], seed=w["seed"])
    else:
        off, nbrs, labels = graphs.sbm(w["n"], w["blocks"], w["degree"], w["ratio"], seed=w["seed"])
    gen_s = time.time() - t0
    n, m = off.size - 1, nbrs.size // 2
    ratio = float(np.float32(w["per_edge"] * m / (w["walk_len"] * n * math.log(n))))
    stream = torch.cuda.current_stream()
    ctx = Context(local, stream=stream.cuda_stream)
    g = Graph.from_numpy(ctx, off, nbrs)
    out = {"workload": w["label"], "n": n, "m": m, "sample_ratio_float": ratio, "graph_gen_s": gen_s,
           "device_free_gb_before_sparsify": torch.cuda.mem_get_info()[0] / 1e9}
    sums = []
    csr = None
    for rep in range(2):
        if csr is not None:
            csr.free()
        torch.cuda.synchronize()
        t = time.time()
        csr, st = generate_trunc_log_matrix_v2(ctx, g, w["seed"], walk_len=w["walk_len"], table_size=w["tablesz"],
                                               sample_ratio=ratio)
        torch.cuda.synchronize()
        out["sparsify_s"] = time.time() - t
        sums.append(csr_checksum(csr))
    out["sparsify"] = {k: st[k] for k in ("samples_emitted", "distinct", "nnz_upper", "nnz", "capacity",
                                          "ms_sample", "ms_trunclog", "ms_csr", "sliced")}
    out["csr_row_ptr_ok"] = sums[0][1]
    out["deterministic"] = sums[0][0] == sums[1][0]
    embs = {}
    for prec in FORMS:
        torch.cuda.synchronize()
        t = time.time()
        emb, S, s2 = randsvd(ctx, csr, w["rank"], w["dim"], precision=prec, seed=SVD_SEED)
        y, s3 = chebyshev_expansion(ctx, g, emb, w["dim"], order=w["order"], precision=prec)
        pro, _ = get_embedding_dense(ctx, y, w["dim"])
        torch.cuda.synchronize()
        out["dense_s_" + prec] = time.time() - t
        out["randsvd_ms_" + prec] = s2["ms_total"]
        out["propagate_ms_" + prec] = s3["ms_total"]
        embs[prec] = (emb, pro)
        del y
    csr.free()
    e32, p32 = (x.double().cpu().numpy() for x in embs["fp32"])
    for prec in ("fp16", "bf16"):
        e16, p16 = (x.double().cpu().numpy() for x in embs[prec])
        out[prec + "_vs_fp32_svd_procrustes"] = lo.procrustes_rel_error(e16, e32)
        out[prec + "_vs_fp32_final_procrustes"] = lo.procrustes_rel_error(p16, p32)
        del e16, p16
    del p32
    if w["kind"] == "rmat":
        # The propagation and dense-SVD stages against the FP64 host oracle,
        # on one common input (the FP32 form's SVD embedding): the FP64
        # randomized SVD of this matrix (7.4e9 entries) is out of reach on
        # the host, the propagation (133M graph entries) is not.
        t = time.time()
        a32 = e32.astype(np.float32)
        del e32
        yref, _ = lo.propagate(off, nbrs, a32, order=w["order"])
        fin_ref, _ = lo.dense_embed(yref)
        fp64 = {"oracle_seconds": None, "input": "the FP32 form's SVD embedding"}
        for prec in FORMS:
            y, _ = chebyshev_expansion(ctx, g, a32, w["dim"], order=w["order"], precision=prec)
            yy = y.double().cpu().numpy()
            fin, _ = get_embedding_dense(ctx, y, w["dim"])
            del y
            fp64[prec] = {"propagation_rel_frobenius": float(np.linalg.norm(yy - yref) / np.linalg.norm(yref)),
                          "propagation_then_dense_svd_procrustes":
                              lo.procrustes_rel_error(fin.double().cpu().numpy(), fin_ref)}
            del yy, fin
        dense, _ = get_embedding_dense(ctx, yref.astype(np.float32), w["dim"])
        fp64["dense_svd_alone_procrustes"] = lo.procrustes_rel_error(dense.double().cpu().numpy(), fin_ref)
        fp64["oracle_seconds"] = time.time() - t
        out["fp64_stages"] = fp64
        del yref, fin_ref, dense
    if labels is not None:
        emb = embs[HEADLINE][0]
        del embs
        rng = np.random.default_rng(w["seed"])
        perm = rng.permutation(n)
        tr = torch.from_numpy(perm[: n // 10]).cuda()
        te = torch.from_numpy(perm[n // 10:]).cuda()
        yl = torch.from_numpy(labels.astype(np.int64)).cuda()
        # the softmax classifier is first fitted on the features of the
        # initial (mu, s) (the propagation is fixed, so this needs no
        # adjoint); the 20 Adam steps then move (mu, s) and the classifier
        # together, the filter's gradients coming from the adjoint
        with torch.no_grad():
            y0 = chebyshev_expansion(ctx, g, emb, w["dim"], order=w["order"], mu=0.2, s=0.5, precision=HEADLINE)[0]
            z0 = (y0 / y0.norm(dim=1, keepdim=True).clamp_min(1e-12))[tr]
        del y0
        W = torch.zeros(w["dim"], w["blocks"], device="cuda", requires_grad=True)
        b = torch.zeros(w["blocks"], device="cuda", requires_grad=True)
        fit = torch.optim.Adam([W, b], lr=0.1)
        for _ in range(300):
            fit.zero_grad()
            torch.nn.functional.cross_entropy(z0 @ W + b, yl[tr]).backward()
            fit.step()
        del z0
        mu = torch.tensor(0.2, device="cuda", requires_grad=True)
        sp_ = torch.tensor(0.5, device="cuda", requires_grad=True)
        opt = torch.optim.Adam([{"params": [mu, sp_], "lr": 0.02}, {"params": [W, b], "lr": 0.02}])
        hist = []
        torch.cuda.synchronize()
        t = time.time()
        for step in range(w["adam_steps"] + 1):
            y = ChebyshevPropagation(emb, mu, sp_, ctx, g, w["order"], HEADLINE)
            z = y / y.norm(dim=1, keepdim=True).clamp_min(1e-12)
            loss = torch.nn.functional.cross_entropy(z[tr] @ W + b, yl[tr])
            if step in (0, w["adam_steps"] // 2, w["adam_steps"]):
                with torch.no_grad():
                    acc = ((z[te] @ W + b).argmax(1) == yl[te]).float().mean().item()
                hist.append({"step": step, "loss": loss.item(), "test_acc": acc, "mu": mu.item(), "s": sp_.item()})
            if step == w["adam_steps"]:
                break
            opt.zero_grad()
            loss.backward()
            opt.step()
            del y, z
        torch.cuda.synchronize()
        out["adam"] = {"seconds": time.time() - t, "trace": hist}
    print(json.dumps({"scale_run": args.workload, **out}))
    g.free()
    ctx.close()


def accuracy(ctx, g, w, off, nbrs, csr_host, forms):
    """Every form against the FP64 oracle on this workload (oracle/linalg_oracle.py,
    same sketches): randomized SVD singular values, subspace angle and
    embedding error after Procrustes; the propagation stage alone (each form
    propagates the oracle's embedding); and the final embedding of the whole
    chain (randomized SVD, propagation, dense SVD: the form's own chain
    against the FP64 chain), after Procrustes."""
    import scipy.sparse as sp

    from lightne_gb300.api import CSR, chebyshev_expansion, gaussian, get_embedding_dense, randsvd
    from oracle import linalg_oracle as lo
    rp, col, val = csr_host
    n = off.size - 1
    A = sp.csr_matrix((val.astype(np.float64), col, rp), shape=(n, n))
    res = {"gate": ERROR_GATE}
    # every form shares the sketches, so one FP64 run serves all of them
    P = gaussian(ctx, SVD_SEED, 1, w["rank"], w["rank"]).double().cpu().numpy()
    om = gaussian(ctx, SVD_SEED, 0, n, w["rank"]).double().cpu().numpy()
    t0 = time.perf_counter()
    ref, Sref = lo.randsvd(A, om, P, w["dim"])
    del om
    ref32 = ref.astype(np.float32)
    yiso, _ = lo.propagate(off, nbrs, ref32, order=w["order"])
    ychain, _ = lo.propagate(off, nbrs, ref, order=w["order"])
    fin_ref, _ = lo.dense_embed(ychain)
    del ychain
    res["oracle_seconds"] = time.perf_counter() - t0
    import torch
    d_rp, d_col, d_val = (torch.from_numpy(a).cuda() for a in (rp, col, val))
    csr = CSR.wrap_device(ctx, n, int(rp[-1]), d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr())
    for form in forms:
        ctx.set_core_svd_fp64(1 if form == "fp32" else 0)  # as in pipeline_step
        emb, S, _ = randsvd(ctx, csr, w["rank"], w["dim"], precision=form, seed=SVD_SEED)
        e = emb.double().cpu().numpy()
        y, _ = chebyshev_expansion(ctx, g, ref32, w["dim"], order=w["order"], precision=form)
        yy = y.double().cpu().numpy()
        del y
        yc, _ = chebyshev_expansion(ctx, g, emb, w["dim"], order=w["order"], precision=form)
        fin, _ = get_embedding_dense(ctx, yc, w["dim"])
        del yc
        final = lo.procrustes_rel_error(fin.double().cpu().numpy(), fin_ref)
        res[form] = {
            "svd_singular_values_max_rel": lo.rel_sv_error(S[:w["dim"]], Sref[:w["dim"]]),
            "svd_subspace_max_angle_rad": lo.max_principal_angle(e, ref),
            "svd_embedding_rel_frobenius_procrustes": lo.procrustes_rel_error(e, ref),
            "propagation_rel_frobenius": float(np.linalg.norm(yy - yiso) / np.linalg.norm(yiso)),
            "final_embedding_rel_frobenius_procrustes": final,
            "meets_gate": bool(final <= ERROR_GATE),
        }
    csr.free()
    del d_rp, d_col, d_val
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS) + sorted(SCALE_RUNS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 oracle errors of every form")
    ap.add_argument("--quick", action="store_true", help="headline form only, no e2e / CPU legs (for profiling)")
    ap.add_argument("--form", choices=list(FORMS), help="--quick: the form to time (default: the headline form)")
    ap.add_argument("--micro", choices=["gram", "gemm", "spmm", "spmm16", "spmm8", "prop"],
                    help="time one C-ABI call alone (for profiling)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP32 GPU form (library calls) leg")
    ap.add_argument("--panel-mb", default="0",
                    help="--micro: comma-separated SpMM column-panel budgets in MiB, each timed in turn (0: no "
                         "panels; negative: two panels, the lowest ids up to the budget, then the rest)")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        from lightne_gb300 import build
        if rank == 0:
            build.build()
        barrier(ws)
        if args.micro:
            run_micro(args, local)
        elif args.workload in SCALE_RUNS:
            run_scale(args, local)
        else:
            run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
