#!/usr/bin/env python3
"""Benchmark of the MESSI likelihood hot path on GB300.

One step = one structure-integrated likelihood evaluation (what every NLopt
objective and every MCMC proposal of the reference runs,
src/FARCE.jl:2322-2345): unpaired column likelihoods, pair likelihoods of
every column pair within the span limit mixed over 45 categories (16-state
pruning for the 36 with lambda != 1; the 9 with lambda = 1 are the product of
the unpaired columns, as in the reference's CPU path, src/FARCE.jl:1891-1901),
gap masking and the banded KH99 inside pass to Z.  Workload: seeded synthetic
alignment of 64 sequences x 1,000 nt, max pair span 500 (374,750 pairs).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` is site-pair likelihoods/s with the alignment
resident in HBM (CUDA events on the library's stream, L2 flushed between
steps); ``e2e`` runs the reference-facing call chain (felsensteincuda ->
maskgapped -> computeinsideKH99, src/MESSI.jl:305-311) with host buffers.
``--impl reference`` times the FP64 CPU restatement of the reference's CPU
path (oracle/) on this host's cores.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "site-pair likelihoods/s"
UNIT = "pairs/s"
WORKLOAD = "c2"
WORKLOAD_TEXT = {"c2": "c2: 64 seqs x 1,000 nt, max pair span 500",
                 "c2p": "c2p: 64 seqs x 600 nt, max pair span 300",
                 "c4": "c4: 30 seqs x 9,000 nt, max pair span 800",
                 "c4p": "c4p: 8 seqs x 9,000 nt, max pair span 800",
                 "c1": "c1: 16 seqs x 120 nt, all pairs"}
BYTES_PER_UPDATE = 212  # algorithmic bytes of one node update (2 child rows + exps + indices in, 1 row out)
# DRAM bytes (read + write) per node update of the pruning kernel from one ncu
# capture of the c2-shaped profiling case, averaged over two interior-level
# launches (profiles/prune_msg_kernel_c2p.md); scaled by updates per launch.
TRAFFIC_BYTES_PER_UPDATE = 118.3


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms",
                                          "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # the sampler is live before the timed region starts; samples
            # taken before it (the first one) are left out of the summary
            t0 = time.perf_counter()
            while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        self.start = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in (self.lines[self.start:] or self.lines):
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x, ws):
    """Largest value of x over the ranks (the whole job takes as long as its
    slowest rank).  Works on the NCCL (GPU tensor) and gloo (CPU) backends."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    if dist.get_backend() == "nccl":
        t = torch.tensor([float(x)], dtype=torch.float64, device=f"cuda:{torch.cuda.current_device()}")
    else:
        t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, steps, max_ms, ws):
    """Units processed by all ranks per second of the slowest rank (weak
    scaling: every rank evaluates its own replica)."""
    return ws * units_per_rank * steps / (max_ms / 1e3)


def workload_config(workload, npairs, ws):
    """The `config` object both arms print (identical, so the two lines
    describe the same workload)."""
    return {"workload": WORKLOAD_TEXT[workload] + ", 45 categories (3 x 3 site rates x 5 lambda; the 9 with "
                        "lambda = 1 are the product of two unpaired columns, as in the reference's CPU path), "
                        "synthetic from seed, 5% gaps",
            "pairs_per_step": npairs,
            "step": "unpaired columns + pair pruning + gap mask + inside pass -> Z",
            "l2": "GPU arm: L2 flushed between steps (256 MB write outside the timed events); CPU arm: host "
                  "caches not flushed",
            "parallelism": f"replicas x{ws}"}


def make_params(s, count, seed):
    """`count` parameter vectors around the workload's generating vector (the
    moves an MCMC chain makes); discretised on the host like getparams."""
    import numpy as np

    from messi_gb300 import model as M
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        p = s.params15.copy()
        p[0:3] = np.clip(p[0:3] * np.exp(rng.normal(0, 0.02, 3)), 1.0, 50.0)
        p[3:9] = p[3:9] * np.exp(rng.normal(0, 0.02, 6))
        out.append(M.getparams(p, s.dataset.branchlengths))
    return out


def fp64_step(s, nthreads, rows=None):
    """One evaluation by the FP64 CPU restatement of the reference's CPU path
    (oracle/): unpaired columns, pair pruning of every pair in the band (the
    lambda = 1 categories as the product of the unpaired columns, as
    src/FARCE.jl:1891-1901 does), maskgapped!, and the dense inside pass
    (computeinsideparallel, src/InsideOutsideAlgorithm.jl:682-749).  rows =
    (x0, x1) restricts the pairs to a block of alignment rows (a warm-up
    sample).  Returns (seconds, Z, u, masked pair matrix, pairs evaluated)."""
    import numpy as np

    from oracle import c_oracle as co
    from oracle import model_ref as mr
    ds = s.dataset
    t0 = time.perf_counter()
    rp = mr.getparams(s.params15, ds.branchlengths)
    P, pi16, logw, _, l1, s1, s2 = mr.pair_categories(rp)
    u, ubs = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
    p, _ = co.pair_matrix(ds.children, ds.seqindex, ds.masks, P, pi16, logw, s.W, rows=rows, nthreads=nthreads,
                          lambda1_cat=l1, u_by_site=ubs, site1=s1, site2=s2)
    pm = co.maskgapped(p, ds.gapfrequency, 1.0)
    Z = float(co.inside(u, pm, 1.0, nthreads=nthreads)[0, 0, ds.numcols - 1])
    dt = time.perf_counter() - t0
    npairs = int(np.isfinite(p[np.triu_indices(ds.numcols, 1)]).sum())
    return dt, Z, u, pm, npairs


def parity_against_fp64(ctx, s, h, Z_ref, u_ref, pm_ref):
    """Errors of the timed GPU path against the FP64 chain on the same
    workload and parameters (outside the timed region): Z of
    messi_likelihood, every pair log-likelihood, and the base-pairing
    posteriors of the GPU chain (messi_posteriors on the GPU's scores) against
    those of the FP64 chain (banded FP64 inside/outside/posteriors on the
    FP64 scores; equal to the dense chain, which the CPU tests pin)."""
    import numpy as np

    from messi_gb300 import api
    from messi_gb300 import model as M
    from oracle import c_oracle as co
    ds = s.dataset
    prm = M.getparams(s.params15, ds.branchlengths)
    m = api.ModelArgs(prm)
    gf = np.ascontiguousarray(ds.gapfrequency, np.float64)
    import ctypes
    Zc = ctypes.c_double()
    ctx.check(ctx.lib.messi_likelihood(ctx.handle, h.handle, ctypes.byref(m.struct),
                                       gf.ctypes.data_as(ctypes.c_void_p), 1.0, ctypes.byref(Zc), None),
              "messi_likelihood")
    u = api.computeunpairedlikelihoods(ds, prm, ctx=ctx)
    mat, _ = api.felsensteincuda(ds, prm, None, s.W, ctx=ctx)
    api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
    fin = np.isfinite(pm_ref)
    same_pattern = bool(np.array_equal(fin, np.isfinite(mat)))
    pair_err = float((np.abs(mat[fin] - pm_ref[fin]) / np.maximum(np.abs(pm_ref[fin]), 1.0)).max())
    _, single, pair = api.computeposteriors(u, mat, maxspan=s.W, ctx=ctx)
    _, s_ref, up_ref, lo_ref = co.posteriors_banded(u_ref, pm_ref, s.W)
    up, lo = co.band_of(pair, s.W)
    post_err = max(float(np.abs(single - s_ref).max()), float(np.abs(up - up_ref).max()),
                   float(np.abs(lo - lo_ref).max()))
    return {"rel_loglik_err": abs(Zc.value - Z_ref) / abs(Z_ref), "Z": Zc.value, "Z_fp64": Z_ref,
            "max_pair_loglik_rel_err": pair_err, "pair_pattern_equal": same_pattern,
            "max_unpaired_rel_err": float(np.max(np.abs(u - u_ref) / np.abs(u_ref))),
            "max_posterior_err": post_err,
            "against": "FP64 CPU chain (oracle/) on the same workload and parameters: unpaired, all pairs, "
                       "maskgapped, dense inside; posteriors from the FP64 scores"}


def reference_gpu_rate(s, npairs):
    """Pairs/s of the reference's kernels (src/cuda/felsenstein.cu, inside.cu,
    compiled unmodified for sm_103a) replaying its launch sequence on the same
    workload: pair pruning for all 45 categories + the inside pass."""
    try:
        from oracle import c_oracle as co
        from oracle import model_ref as mr
        from oracle import ref_kernels as rk
        if not rk.available():
            return {"unavailable": "reference cubins not built (make -C oracle ref)"}
        ds = s.dataset
        rp = mr.getparams(s.params15, ds.branchlengths)
        P, pi16, logw, *_ = mr.pair_categories(rp)
        plan = rk.index_plan(ds.children, ds.seqindex, ds.masks, s.W)
        u, _ = mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
        tp, ti = {}, {}
        t0 = time.perf_counter()
        mr.unpaired_loglik(ds.tree_arrays(), ds.masks, rp)
        t_unp = 1e3 * (time.perf_counter() - t0)
        p = rk.pair_matrix(ds.children, ds.seqindex, ds.masks, P, pi16, logw, s.W, plan=plan, timing=tp)
        p = co.maskgapped(p, ds.gapfrequency, 1.0)
        Zr, _ = rk.inside(u, p, timing=ti)
        total = tp["ms"] + ti["ms"] + t_unp
        return {"value": npairs / (total / 1e3), "unit": UNIT, "kind": "reference",
                "impl": "the reference's CUDA kernels (src/cuda/felsenstein.cu, inside.cu) compiled unmodified "
                        "for sm_103a, its Julia launch sequence replayed (oracle/ref_kernels.py), on this GPU; "
                        "unpaired columns on the host in FP64 as the reference does",
                "same_workload": True, "pairs_ms": tp["ms"], "inside_ms": ti["ms"], "unpaired_ms": t_unp,
                "ms_per_step": total, "Z": Zr,
                "ours_vs_this": None}
    except Exception as exc:  # the reference path is a reported baseline only
        return {"unavailable": f"{type(exc).__name__}: {exc}"[:200]}


def total_pairs(L, W):
    return sum(min(W, L - 1 - x) for x in range(L))


def run_reference(args):
    """The reference arm: the reference's path cannot run here (Julia is
    absent), so its FP64 CPU restatement (oracle/, kind "port") evaluates the
    full workload on every host core, one whole evaluation per timed step.
    Warm-up is one small sample (a block of rows) whatever --warmup says:
    CPU code has no JIT or caches worth warming, and full warm-up steps
    would only lengthen the run."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from messi_gb300 import synth
    s = synth.make_workload(args.workload, seed=1)
    L, W = s.dataset.numcols, s.W
    npairs = total_pairs(L, W)
    nthreads = os.cpu_count() or 1
    fp64_step(s, nthreads, rows=(0, 8))
    times = []
    Z = None
    for k in range(args.steps):
        dt, Z, _, _, n = fp64_step(s, nthreads)
        assert n == npairs, (n, npairs)
        times.append(dt)
    value = npairs * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic",
        "config": workload_config(args.workload, npairs, ws),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"the full workload every step ({npairs} pairs, unpaired columns, gap mask, "
                                   f"dense inside pass); warm-up: one 8-row block of pairs"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "Z": Z,
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    from messi_gb300 import api, synth

    s = synth.make_workload(args.workload, seed=1 + rank)
    ds = s.dataset
    L, W = ds.numcols, s.W
    npairs = total_pairs(L, W)
    params = make_params(s, args.warmup + args.steps, seed=rank)
    ctx = api.get_context(local)
    h = ctx.dataset(ds, W)
    stats = h.stats()
    margs = [api.ModelArgs(p) for p in params]
    gf = np.ascontiguousarray(ds.gapfrequency, np.float64)

    import ctypes
    Zc = ctypes.c_double()

    def step(m):
        ctx.check(ctx.lib.messi_likelihood(ctx.handle, h.handle, ctypes.byref(m.struct),
                                           gf.ctypes.data_as(ctypes.c_void_p), 1.0, ctypes.byref(Zc), None),
                  "messi_likelihood")
        return ctx.last_launches()

    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    for k in range(args.warmup):
        flush.zero_()  # the flush kernel's first launch loads its module: keep that out of the timed loop
        torch.cuda.synchronize()
        step(margs[k])
    # further untimed steps until launch-shape autotuning has finished and the
    # step replays its captured graph (the first evaluations of a dataset time
    # candidate shapes; the graph is captured once the shapes are fixed)
    r0 = ctx.graph_replays()
    for k in range(32):
        if ctx.graph_replays() > r0 + 1:
            break
        flush.zero_()
        torch.cuda.synchronize()
        step(margs[k % len(margs)])
    shapes = ctx.launch_shapes()
    if args.profile_only:
        # minimal launch sequence for profilers: the timed steps only
        for k in range(args.steps):
            step(margs[args.warmup + k])
        torch.cuda.synchronize()
        print(json.dumps({"profile_only": args.workload, "steps": args.steps, "Z": Zc.value}), flush=True)
        return

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- timed region: K steps, L2 flushed between steps (outside the events)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches = 0
    barrier()
    torch.cuda.synchronize()
    t_flush = t_call = 0.0
    replays0 = ctx.graph_replays()
    with Clocks(local) as clk:
        t_wall = time.perf_counter()
        for k in range(args.steps):
            a = time.perf_counter()
            flush.zero_()
            torch.cuda.synchronize()
            b = time.perf_counter()
            ev[k][0].record(stream)
            launches += step(margs[args.warmup + k])
            ev[k][1].record(stream)
            c = time.perf_counter()
            t_flush += b - a
            t_call += c - b
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
    replays = ctx.graph_replays() - replays0
    barrier()
    per = [a.elapsed_time(b) for a, b in ev]
    ms = max_over_ranks(sum(per), ws)
    ms_per_step = ms / args.steps
    value = whole_job_rate(npairs, args.steps, ms, ws)
    # host wall clock of the timed loop: the L2 flush and its synchronise
    # (outside the events) and the messi_likelihood call, which returns after
    # its stream synchronise (host staging + device work + Z read-back)
    wall = {"ms_per_step": 1e3 * t_wall / args.steps, "flush_ms_per_step": 1e3 * t_flush / args.steps,
            "call_ms_per_step": 1e3 * t_call / args.steps}

    # ---- kernel-level timing pass (event pairs around each pruning launch)
    ctx.profile(True)
    nprof = min(args.steps, 5)
    for k in range(nprof):
        flush.zero_()
        torch.cuda.synchronize()
        step(margs[args.warmup + k])
    p_ms, p_n, p_units = ctx.profile_read(0)
    i_ms, i_n, i_cells = ctx.profile_read(1)
    s_ms, s_n, s_cells = ctx.profile_read(2)
    ctx.profile(False)
    peak, peak_kind = measured_peaks()
    achieved = (p_units * BYTES_PER_UPDATE / 1e9) / (p_ms / 1e3) if p_ms > 0 else None
    units_per_launch = p_units / p_n if p_n else None
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
        "frac": (achieved / peak) if achieved else None,
        "traffic": (TRAFFIC_BYTES_PER_UPDATE * units_per_launch) if (TRAFFIC_BYTES_PER_UPDATE and units_per_launch)
        else None,
        "kernel": "prune_msg_kernel", "peak_source": f"{peak_kind} hbm_gbs",
        "bytes_per_unit": BYTES_PER_UPDATE, "unit_name": "node update (pair x category x internal node)",
        "units_per_launch": units_per_launch, "launches": p_n, "avg_launch_ms": p_ms / p_n if p_n else None,
        "kernel_ms_per_step": p_ms / nprof,
    }
    inside_ms = (i_ms + s_ms) / nprof
    band_cells = sum(L - d for d in range(W + 1)) + max(0, L - 1 - W)

    # ---- e2e: the reference-facing call chain with host buffers
    ne2e = min(args.steps, 5)
    t_e2e = []
    # warm-up: the pairs-only and inside-only entry points are workloads of
    # their own for the launch-shape autotuner, whose first calls time
    # candidate shapes
    for k in range(max(args.warmup, 5)):
        prm = params[k % len(params)]
        u = api.computeunpairedlikelihoods(ds, prm, ctx=ctx)
        mat, _ = api.felsensteincuda(ds, prm, None, W, ctx=ctx)
        api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
        api.computeinsideKH99(u, mat, ctx=ctx)
    for k in range(ne2e):
        prm = params[args.warmup + k]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u = api.computeunpairedlikelihoods(ds, prm, ctx=ctx)
        mat, _ = api.felsensteincuda(ds, prm, None, W, ctx=ctx)
        api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
        api.computeinsideKH99(u, mat, ctx=ctx)
        t_e2e.append(time.perf_counter() - t0)
    # staged model uploads (eigensystems, branch lengths, pi16, weights, lambda
    # indices, unpaired eigensystems, pi4, site weights): one per call
    Cp = api.ModelArgs(params[0]).pruned_categories()
    unpaired_bytes = (ds.numnodes + 3 * (4 + 16 + 4) + 4 + 3) * 8
    pair_bytes = Cp * ((16 + 256 + 16) * 8 + 16 * 4 + 8 + 4)
    h2d = 2 * unpaired_bytes + pair_bytes + L * L * 8 + L * 8
    d2h = L * 8 + L * L * 8 + 8
    e2e_value = whole_job_rate(npairs, 1, 1e3 * max_over_ranks(statistics.mean(t_e2e), ws), ws)

    # ---- CPU baseline and parity (rank 0, single process): one full FP64
    # evaluation of the same workload, whose outputs also check the GPU path
    cpu = parity = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        t_full, Z_ref, u_ref, pm_ref, n_cpu = fp64_step(s, nthreads)
        cpu = {"value": n_cpu / t_full, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"one full evaluation ({n_cpu} pairs, unpaired columns, gap mask, dense inside pass; "
                         f"{t_full:.1f} s)"}
        parity = parity_against_fp64(ctx, s, h, Z_ref, u_ref, pm_ref)

    # ---- second baseline: the reference's own CUDA kernels on this GPU
    refgpu = None
    if rank == 0 and ws == 1 and not args.no_reference_gpu:
        refgpu = reference_gpu_rate(s, npairs)
        if refgpu.get("value"):
            refgpu["ours_vs_this"] = {"value": value / refgpu["value"], "e2e": e2e_value / refgpu["value"]}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32", "data": "synthetic",
        "config": workload_config(args.workload, npairs, ws),
        "plan": stats,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "chain": "computeunpairedlikelihoods + felsensteincuda + maskgapped + computeinsideKH99"},
        "gpu_launches": launches,
        "graph_replays_in_timed_steps": replays,
        "launch_shapes": shapes,
        "roofline": roofline,
        "inside": {"cells_per_s": band_cells / (inside_ms / 1e3) if inside_ms > 0 else None,
                   "band_cells": band_cells, "full_triangle_cells": L * (L + 1) // 2,
                   "ms_per_pass": inside_ms, "wavefront_ms": i_ms / nprof, "suffix_ms": s_ms / nprof,
                   "launches_per_pass": (i_n + s_n) / nprof},
        "wall": wall,
        "clocks": clk.summary(),
        "parity": parity,
        "cpu_baseline": cpu,
        "baseline_gpu": refgpu,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_mcmc(args):
    """Config 5: plain move-8 random walk vs the learned mixture proposal on
    the c2 alignment, each for --mcmc-iters iterations (first third burn-in;
    the learned proposal trains during burn-in and is frozen after)."""
    import numpy as np

    from messi_gb300 import mcmc, synth
    s = synth.make_workload(args.workload, seed=1)
    ds = s.dataset
    n = args.mcmc_iters
    burn = n // 3
    theta0 = mcmc.theta_from_p15(s.params15)
    out = {}
    means = {}
    for kind in ("plain", "learned"):
        tgt = mcmc.Target(ds, s.params15[11:14], s.W)
        learned = mcmc.LearnedProposal(mcmc.alignment_summaries(ds), seed=3) if kind == "learned" else None
        res = mcmc.run_chain(tgt, theta0, n, burn, proposal=kind, seed=11, learned=learned,
                             fit_every=max(25, burn // 10), fit_steps=150)
        Z = np.array([mcmc.to_z(t) for t in res.samples])
        ess = np.array([mcmc.ess(Z[:, k]) for k in range(mcmc.NFREE)])
        se = np.array([mcmc.mcse(res.samples[:, k]) for k in range(mcmc.NFREE)])
        out[kind] = {"ess_per_s": (ess / res.seconds).tolist(), "ess": ess.tolist(), "seconds": res.seconds,
                     "median_ess_per_s": float(np.median(ess / res.seconds)),
                     "min_ess_per_s": float(np.min(ess / res.seconds)), "accept": res.accept,
                     "likelihood_evals": res.evals, "gpu_launches": tgt.launches, **res.extra}
        means[kind] = (res.samples.mean(axis=0), se)
    (mp, sp), (ml, sl) = means["plain"], means["learned"]
    z = np.abs(mp - ml) / np.sqrt(sp ** 2 + sl ** 2)
    ratio = out["learned"]["median_ess_per_s"] / out["plain"]["median_ess_per_s"]
    per_param = (np.array(out["learned"]["ess_per_s"]) / np.array(out["plain"]["ess_per_s"])).tolist()
    line = {"metric": "MCMC ESS/s learned vs plain proposal", "value": ratio, "unit": "x (median over parameters)",
            "higher_is_better": True, "n_gpus": 1, "iterations": n, "burnin": burn, "data": "synthetic",
            "config": {"workload": WORKLOAD_TEXT[args.workload] + ", 45 categories", "parameters": list(mcmc.FREE)},
            "plain": out["plain"], "learned": out["learned"],
            "per_parameter_ratio": per_param, "min_per_parameter_ratio": float(min(per_param)),
            "worst_parameter_ratio": out["learned"]["min_ess_per_s"] / out["plain"]["min_ess_per_s"],
            "posterior_mean_agreement_z": z.tolist(), "max_z": float(z.max()),
            "within_2_mcse": bool(np.all(z <= 2.0 * math.sqrt(2.0)))}
    print(json.dumps(line), flush=True)


def run_batch(args):
    """Batched evaluation (config 3: many alignments, W = L - 1 each): one
    messi_batch_likelihood per step against the same alignments evaluated one
    messi_likelihood call at a time.  Prints its own JSON line."""
    import ctypes

    import numpy as np
    import torch

    from messi_gb300 import api, synth
    from messi_gb300 import model as M

    t0 = time.perf_counter()
    wl = synth.make_batch(args.batch, seed=1)
    t_synth = time.perf_counter() - t0
    datasets = [w.dataset for w in wl]
    params = [M.getparams(w.params15, w.dataset.branchlengths) for w in wl]
    npairs = sum(total_pairs(d.numcols, d.numcols - 1) for d in datasets)
    ctx = api.get_context(0)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", 0))
    t0 = time.perf_counter()
    b = api.Batch(datasets, ctx=ctx)
    t_plan = time.perf_counter() - t0
    st = b.stats()
    for _ in range(args.warmup):
        Z = b.likelihood(params)
    if args.profile_only:
        # minimal launch sequence for profilers: the timed steps only
        for _ in range(args.steps):
            Z = b.likelihood(params)
        torch.cuda.synchronize()
        print(json.dumps({"profile_only": args.batch, "steps": args.steps, "Z0": float(Z[0])}), flush=True)
        return
    # until autotuning has finished and the batch step replays its graph
    r0 = ctx.graph_replays()
    for _ in range(16):
        if ctx.graph_replays() > r0 + 1:
            break
        Z = b.likelihood(params)
    shapes = ctx.launch_shapes()
    replays0 = ctx.graph_replays()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches = 0
    wall = 0.0
    with Clocks(0) as clk:
        for k in range(args.steps):
            torch.cuda.synchronize()
            t_host = time.perf_counter()
            ev[k][0].record(stream)
            Z = b.likelihood(params)
            ev[k][1].record(stream)
            torch.cuda.synchronize()
            wall += time.perf_counter() - t_host
            launches += ctx.last_launches()
    batch_replays = ctx.graph_replays() - replays0
    ms_batch = sum(a.elapsed_time(c) for a, c in ev) / args.steps
    wall_batch = 1e3 * wall / args.steps
    ctx.profile(True)
    b.likelihood(params)
    p_ms, _, p_units = ctx.profile_read(0)
    i_ms, _, i_cells = ctx.profile_read(1)
    ctx.profile(False)
    b.close()
    # the same alignments one call at a time (plans built outside the timing),
    # on a context with the default launch shapes and each call's graph
    # captured before the timed call, the best case for single calls
    os.environ["MESSI_AUTOTUNE"] = "0"
    ctx = api.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream(), device=torch.device("cuda", 0))
    seq_ms = 0.0
    seq_wall = 0.0
    seq_launches = 0
    Zs = np.empty(len(datasets))
    Zc = ctypes.c_double()
    for k, (d, p) in enumerate(zip(datasets, params)):
        h = api.DatasetHandle(ctx, d, d.numcols - 1)
        m = api.ModelArgs(p)
        gf = np.ascontiguousarray(d.gapfrequency, np.float64)

        def one():
            ctx.check(ctx.lib.messi_likelihood(ctx.handle, h.handle, ctypes.byref(m.struct),
                                               gf.ctypes.data_as(ctypes.c_void_p), 1.0, ctypes.byref(Zc), None),
                      "messi_likelihood")
        one()
        one()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t_host = time.perf_counter()
        e0.record(stream)
        one()
        e1.record(stream)
        torch.cuda.synchronize()
        seq_wall += 1e3 * (time.perf_counter() - t_host)
        seq_ms += e0.elapsed_time(e1)
        seq_launches += ctx.last_launches()
        Zs[k] = Zc.value
        h.close()
    rel = float(np.max(np.abs(Z - Zs) / np.abs(Zs)))
    line = {"metric": METRIC, "value": npairs / (ms_batch / 1e3), "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batch, "higher_is_better": True, "dtype": "fp32/fp64",
            "data": "synthetic",
            "config": {"workload": f"{args.batch}: {len(datasets)} alignments, W = L - 1 each",
                       "pairs": npairs, "columns": int(sum(d.numcols for d in datasets)),
                       "sequences": int(sum(d.numseqs for d in datasets))},
            "wall_ms_per_step": wall_batch,
            "sequential": {"value": npairs / (seq_ms / 1e3), "ms_per_step": seq_ms, "wall_ms_per_step": seq_wall,
                           "gpu_launches": seq_launches},
            "speedup_vs_sequential": seq_ms / ms_batch, "wall_speedup_vs_sequential": seq_wall / wall_batch,
            "gpu_launches": launches // max(1, args.steps),
            "graph_replays_in_timed_steps": batch_replays, "launch_shapes": shapes,
            "max_rel_diff_vs_sequential": rel, "plan_seconds": t_plan, "synth_seconds": t_synth, "stats": st,
            "kernels": {"prune_ms": p_ms, "prune_updates": p_units, "inside_ms": i_ms, "inside_cells": i_cells,
                        "prune_GBps_algorithmic": (p_units * BYTES_PER_UPDATE / 1e9) / (p_ms / 1e3) if p_ms else None},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def run_structures(args):
    """Structure outputs on the c2 alignment: posterior decoding (ours vs the
    reference's posteriordecoding kernel replayed on the same GPU), the
    device-resident consensus chain, stochastic sampling and the
    fixed-structure likelihood.  Prints its own JSON line (wall times of the
    host-facing calls, medians over --steps)."""
    import numpy as np
    import torch

    from messi_gb300 import api, synth
    from messi_gb300 import model as M
    s = synth.make_workload(args.workload, seed=1)
    ds = s.dataset
    L, W = ds.numcols, s.W
    prm = M.getparams(s.params15, ds.branchlengths)
    ctx = api.get_context(0)
    u = api.computeunpairedlikelihoods(ds, prm, ctx=ctx)
    mat, _ = api.felsensteincuda(ds, prm, None, W, ctx=ctx)
    api.maskgapped(mat, ds.gapfrequency, 1.0, -np.inf)
    _, single, pair = api.computeposteriors(u, mat, ctx=ctx)
    paired1 = np.where(s.paired >= 0, s.paired + 1, 0)

    def timed(fn, n):
        out, ts = None, []
        for k in range(args.warmup + n):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = fn()
            torch.cuda.synchronize()
            if k >= args.warmup:
                ts.append(1e3 * (time.perf_counter() - t0))
        return out, statistics.median(ts)

    nsamp = 1000
    (e, sm), t_dec = timed(lambda: api.computeposteriordecodingcuda(single, pair, 2.0, ctx=ctx), args.steps)
    cons, t_cons = timed(lambda: api.consensusstructure(u, mat, ctx=ctx), args.steps)
    post, t_post = timed(lambda: api.computeposteriors(u, mat, ctx=ctx), args.steps)
    # device time of the posterior chain's passes (CUDA events around each launch)
    ctx.profile(True)
    api.computeposteriors(u, mat, ctx=ctx)
    post_kernels = {name: ctx.profile_read(k)[0] for k, name in ((1, "inside_wavefront_ms"), (2, "inside_suffix_ms"),
                                                                 (3, "outside_wavefront_ms"))}
    ctx.profile(False)
    (S, pri), t_samp = timed(lambda: api.samplestructures(u, mat, nsamp, seed=3, ctx=ctx), args.steps)
    fx, t_fix = timed(lambda: api._structure_call(ds, prm, paired1, ctx), args.steps)
    band, t_band = timed(lambda: api.computestructureintegratedlikelihood(ds, prm, W, ctx=ctx), args.steps)
    ref = None
    try:
        from oracle import ref_kernels as rk
        if rk.available():
            (er, sr), t_ref = timed(lambda: rk.posterior_decoding(single, pair, 2.0), max(1, min(args.steps, 3)))
            ref = {"ms": t_ref, "bit_identical_e": bool(np.array_equal(e, er.astype(np.float64))),
                   "bit_identical_s": bool(np.array_equal(sm, sr)),
                   "kind": "reference posteriordecoding kernel (src/cuda/inside.cu) compiled unmodified, one "
                           "launch per span as src/InsideCUDA.jl:202-204"}
    except Exception as exc:
        ref = {"unavailable": f"{type(exc).__name__}: {exc}"[:200]}
    npairs_struct = int(np.count_nonzero(paired1) // 2)
    line = {"metric": "structure outputs (ms per call)", "workload": WORKLOAD_TEXT[args.workload],
            "steps": args.steps, "warmup": args.warmup,
            "posterior_decoding_ms": t_dec, "decoding_cells": L * (L - 1) // 2,
            "reference_decoding": ref,
            "posteriors_ms": t_post, "posterior_chain_kernels": post_kernels, "consensus_chain_ms": t_cons,
            "consensus_pairs": int(np.count_nonzero(cons) // 2),
            "sampling_ms": t_samp, "structures_per_s": nsamp / (t_samp / 1e3), "samples": nsamp,
            "fixed_structure_ms": t_fix, "fixed_structure_pairs": npairs_struct,
            "band_likelihood_ms": t_band}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 100 for the bench line and the reference arm, about 1 s of "
                         "timed work; 5 with --structures, 3 with --batch)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--mcmc", action="store_true", help="run the MCMC comparison (config 5) instead")
    ap.add_argument("--mcmc-iters", type=int, default=20000)
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(WORKLOAD_TEXT))
    ap.add_argument("--structures", action="store_true",
                    help="time the structure outputs (decoding, consensus, sampling, fixed structure)")
    ap.add_argument("--batch", choices=["c3", "c3s"], default=None,
                    help="time the batched evaluation of a batch workload instead (own JSON line)")
    ap.add_argument("--profile-only", action="store_true",
                    help="run warm-up + timed steps only (for ncu), print a short line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.steps is None:
        args.steps = 3 if args.batch else (5 if args.structures or args.impl == "reference" else 100)
    if args.mcmc:
        run_mcmc(args)
    elif args.batch:
        run_batch(args)
    elif args.structures:
        run_structures(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
