#!/usr/bin/env python3
"""Benchmark of the particle-isosurface path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one frame reconstructed: 1,000,000 particles in (the dam-break
column + spray workload, r = 0.01, seeded synthetic) -> triangle mesh out:
hash grid, anisotropy, normals, octree with field sampling, dual-cell
extraction.  `value` is frames/s with the particles already in HBM (pi_frame_reset
+ pi_run on a resident frame); `e2e` is frames/s through pi_reconstruct with
pinned host buffers (particles host->device and the mesh device->host inside
the timed region).  Steps are timed with CUDA events on the library stream;
between steps a 512 MiB buffer is written to flush L2.

Multi-GPU: the path runs one frame per GPU with no exchange, so N ranks run
N independent replicas (weak scaling); rank 0 prints the whole-job value.

--impl reference times the reference algorithm on the host cores: the CPU
oracle (a restatement of the reference's OpenMP code, built with the
reference's -O3 -fopenmp) on a bounded sample of the same frame: the hash
grid, anisotropy and normal stages run in full, and the octree/extraction
time is the frame's field-evaluation count divided by the oracle's measured
evaluation rate (the oracle's tree bookkeeping and serial mesh dedupe are not
counted, which favours the CPU).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "field evals/s & frames/s at 1M particles; p50/p99 frame latency; err vs FP64"
UNIT = "frames/s"
WORKLOAD = "dam_break column+spray, 1,000,000 particles, r=0.01, seed 2"
# Nominal flops per candidate pair of one field evaluation (3 sub, 9 FMA, norm,
# scale, sqrt, spline, accumulate; FMA counted as 2).
FLOPS_PER_PAIR = 38
# Field evaluations (octree samples, leaf values, bisection steps) of this
# frame, counted by a full oracle run of it (oracle/pi_oracle.cpp counters).
ORACLE_FIELD_EVALS = 147191991
ORACLE_PAIRS = 7205138892
# dram__bytes_read.sum + dram__bytes_write.sum of the field-evaluation launches
# of one 1M-particle frame (k_q_eval_thread x2, k_q_eval), one ncu capture
# (--metrics dram__bytes_read.sum,dram__bytes_write.sum -k regex:k_q_eval -c 3)
FIELD_DRAM_BYTES_PER_FRAME = 380755200


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", "--particles", dest="n", type=int, default=1_000_000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample-evals", type=int, default=200_000)
    p.add_argument("--qef", action="store_true", help="with --single: per-leaf QEF vertices on")
    p.add_argument("--samples-per-lane", type=int, default=0, choices=[0, 1, 2, 4],
                   help="with --single: fix the chunked evaluation's samples per lane (0 = timed choice)")
    p.add_argument("--single", action="store_true",
                   help="reconstruct one frame once and print its counters (for profiler captures)")
    p.add_argument("--workload", choices=["dam_break_1m", "batch64", "serving", "stress", "grid"], default="dam_break_1m",
                   help="dam_break_1m: the metric's frame (default); batch64: 64 mixed frames batched vs one at "
                        "a time; serving: Poisson stream through the request loop; stress: sheets and filaments")
    p.add_argument("--frames", type=int, default=64, help="frames of the batch64 workload")
    p.add_argument("--requests", type=int, default=120, help="requests of the serving workload")
    p.add_argument("--max-n", type=int, default=4_000_000, help="largest serving request")
    p.add_argument("--rate", type=float, default=20.0, help="serving arrival rate (requests/s)")
    p.add_argument("--slots", type=int, default=8)
    return p.parse_args()


def batch64(a):
    """64 independent frames (1-6 spheres/slabs, 50k-2M particles): one at a
    time on one stream versus all submitted to the request loop."""
    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    from particleisosurface_gb300 import synth
    B.build()
    frames = synth.batch_frames(a.frames)
    total_n = sum(fr.n for fr in frames)
    ctx = N.Context(0)
    # warm-up
    for fr in frames[:2]:
        f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
        f.close()
    t0 = time.perf_counter()
    for fr in frames:
        f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
        f.mesh()
        f.close()
    t_seq = time.perf_counter() - t0
    ctx.close()
    # device-resident form: the 64 frames stay uploaded; one at a time on one
    # context versus spread over `slots` contexts (own streams) driven by as
    # many host threads (the C calls release the GIL).  Frames go to the
    # contexts largest first, each to the least-loaded one (by particles), so
    # that the threads finish together.
    import threading
    ctxs = [N.Context(0) for _ in range(a.slots)]
    load = [0] * a.slots
    owner = [0] * len(frames)
    for k in sorted(range(len(frames)), key=lambda k: -frames[k].n):
        owner[k] = min(range(a.slots), key=lambda s: load[s])
        load[owner[k]] += frames[k].n
    res = [N.Frame(ctxs[owner[k]], N.default_params(fr.radius)).upload(fr.xyz) for k, fr in enumerate(frames)]
    for f in res[:2]:
        f.reset().run()
    t0 = time.perf_counter()
    for f in res:
        f.reset().run()  # returns once the frame is done
    t_res_seq = time.perf_counter() - t0

    def work(k):
        for f in sorted((res[j] for j in range(len(res)) if owner[j] == k), key=lambda f: -f.n):
            f.reset().run()

    t0 = time.perf_counter()
    ths = [threading.Thread(target=work, args=(k,)) for k in range(a.slots)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    t_res_con = time.perf_counter() - t0
    for f in res:
        f.close()
    for c in ctxs:
        c.close()

    srv = N.Server(0, slots=a.slots, budget_bytes=0)
    for fr in frames[:2]:
        srv.result(srv.submit(fr.xyz, N.default_params(fr.radius)))
    # a batch job: submitted largest first (the request loop admits in order)
    t0 = time.perf_counter()
    tickets = [srv.submit(fr.xyz, N.default_params(fr.radius)) for fr in sorted(frames, key=lambda fr: -fr.n)]
    lat = [srv.result(t)[2] for t in tickets]
    t_bat = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    print(json.dumps({
        "metric": METRIC, "workload": "batch64", "value": len(frames) / t_bat, "unit": UNIT,
        "one_at_a_time_frames_per_s": len(frames) / t_seq, "speedup_vs_one_at_a_time": t_seq / t_bat,
        "resident": {"one_at_a_time_frames_per_s": len(frames) / t_res_seq,
                     "concurrent_frames_per_s": len(frames) / t_res_con,
                     "speedup": t_res_seq / t_res_con,
                     "timing": "host wall clock around pi_run on device-resident frames (pi_run returns when "
                               "its frame is done)"},
        "frames": len(frames), "particles_total": total_n, "slots": a.slots, "max_in_flight": st["max_in_flight"],
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "timing": "host wall clock, host buffers in and out (upload, run, mesh download)",
        "data": "synthetic (seeded unions of spheres and slabs)"}))


def grid(a):
    """UniformGrid (the reference's dense-grid mode) on the 1M-particle frame:
    the field on the lattice of spacing r over the particles' box.  value =
    lattice points per second with the particles resident and the lattice
    written to device memory; e2e = the same through pi_grid_sample into a
    pinned host buffer (device-to-host copy of the values inside the region)."""
    import ctypes as C

    import torch

    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    B.build()
    fr = make_frame(a.n)
    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    f.hashgrid().aniso().normals()
    dims, box, npts = f.grid_dims()
    stream = torch.cuda.ExternalStream(N.lib().pi_ctx_stream(ctx.h), device=0)
    d_out = torch.empty(npts, device="cuda", dtype=torch.float32)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(a.warmup):
        f.grid_sample_device(d_out.data_ptr(), npts)
    ctx.profile(True)
    ctx.kernel_time()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    clocks = Clocks(0)
    torch.cuda.synchronize()
    clocks.start()
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
        ev[k][0].record(stream)
        f.grid_sample_device(d_out.data_ptr(), npts)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    kt = ctx.kernel_time()
    ctx.profile(False)
    ms = float(np.mean([s0.elapsed_time(e1) for s0, e1 in ev]))
    info = f.info()
    host = torch.empty(npts, dtype=torch.float32).pin_memory()
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
        ev2[k][0].record(stream)
        N.check(N.lib().pi_grid_sample(f.h, C.cast(host.data_ptr(), C.POINTER(C.c_float)), npts))
        ev2[k][1].record(stream)
    torch.cuda.synchronize()
    e2e_ms = float(np.mean([s0.elapsed_time(e1) for s0, e1 in ev2]))
    vals = host.numpy()
    pairs = info["grid_pairs"]
    achieved = pairs * FLOPS_PER_PAIR / (kt["ms"] / a.steps / 1000.0) / 1e12
    peak = fp32_gemm_tflops(torch)
    line = {
        "metric": METRIC, "workload": "grid", "value": npts / (ms / 1000.0), "unit": "lattice points/s",
        "ms_per_step": ms, "steps": a.steps, "warmup": a.warmup, "higher_is_better": True,
        "config": {"workload": WORKLOAD + "; UniformGrid lattice, spacing r", "dims": [int(d) for d in dims],
                   "points": int(npts), "l2": "512 MiB buffer written between steps"},
        "candidate_pairs_per_step": pairs, "kernel_ms_per_step": kt["ms"] / a.steps,
        "e2e": {"value": npts / (e2e_ms / 1000.0), "unit": "lattice points/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 4 * int(npts)},
        "roofline": {"kernel": "k_grid_eval", "bound": "fp32", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak,
                     "peak_source": "measured in this run: cuBLAS FP32 GEMM 8192^3, TF32 off"},
        "clocks": ck, "values_min_max": [float(vals.min()), float(vals.max())],
        "data": "synthetic (seeded dam-break column + spray)"}
    if not a.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import pyoracle as O
        O.build()
        nthreads = os.cpu_count() or 1
        O.set_threads(nthreads)
        o = O.OracleFrame(fr.xyz, fr.radius)
        for s in (1, 2, 3):
            o.stage(s)
        rng = np.random.default_rng(7)
        m = min(a.cpu_sample_evals, int(npts))
        pick = rng.choice(int(npts), m, replace=False)
        zz, yy, xx = np.unravel_index(pick, (int(dims[2]), int(dims[1]), int(dims[0])))
        f32 = np.float32

        def coord(ax, i):
            st = f32(int(dims[ax]) - 1)
            return (f32(st - i.astype(f32)) / st) * box[2 * ax] + (i.astype(f32) / st) * box[2 * ax + 1]

        pts = np.stack([coord(0, xx), coord(1, yy), coord(2, zz)], -1).astype(np.float32)
        t0 = time.perf_counter()
        o.eval(pts)
        te = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": m / te, "unit": "lattice points/s", "cores": nthreads, "kind": "port",
                                "sample": "oracle SingleEval at %d random lattice points of the same grid" % m}
    print(json.dumps(line))
    f.close()
    ctx.close()


def serving(a):
    """Poisson stream of frame requests (sequences advected by swirl plus
    gravity) replayed in real time into the request loop."""
    import threading

    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    from particleisosurface_gb300 import synth
    B.build()
    reqs = synth.serving_requests(count=a.requests, n_max=a.max_n, rate_hz=a.rate)
    base = {}
    xyzs = []
    for r in reqs:
        key = r["seq"]
        if key not in base:
            fr = synth.mixed_frame(r["seed"], r["n"], r["radius"])
            base[key] = (fr.xyz64, fr.scale)
        p, sc = base[key]
        if r["step"]:
            p = synth.advect(p, r["w"], synth.SERVE_G, (r["step"] - 1) * synth.SERVE_DT, synth.SERVE_DT, steps=1,
                             scale=sc)
        base[key] = (p, sc)
        xyzs.append(np.ascontiguousarray(p.astype(np.float32)))
    srv = N.Server(0, slots=a.slots, budget_bytes=0)
    srv.result(srv.submit(xyzs[0], N.default_params(reqs[0]["radius"])))  # warm-up
    tickets = [None] * len(reqs)
    results = [None] * len(reqs)

    def collector():
        for i in range(len(reqs)):
            while tickets[i] is None:
                time.sleep(0.0005)
            results[i] = srv.result(tickets[i])[2:]

    th = threading.Thread(target=collector)
    th.start()
    t0 = time.perf_counter()
    for i, r in enumerate(reqs):
        wait = r["t"] - (time.perf_counter() - t0)
        if wait > 0:
            time.sleep(wait)
        tickets[i] = srv.submit(xyzs[i], N.default_params(r["radius"]))
    th.join()
    t_all = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    lat = np.array([x[0] for x in results])
    print(json.dumps({
        "metric": METRIC, "workload": "serving", "value": len(reqs) / t_all, "unit": UNIT,
        "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
        "requests": len(reqs), "arrival_rate_hz": a.rate, "n_range": [10000, a.max_n],
        "particles_total": int(sum(x.shape[0] for x in xyzs)), "slots": a.slots,
        "max_in_flight": st["max_in_flight"], "wall_s": t_all,
        "data": "synthetic (seeded sequences advected by swirl plus gravity)"}))


def stress(a):
    """Sheets and filaments: FP32/FP64 eigen split, errors against the FP64 oracle."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O

    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    from particleisosurface_gb300 import synth
    B.build()
    O.build()
    fr = synth.sheets_and_filaments(n=500_000)
    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz)
    f.run()
    f.reset()
    t0 = time.perf_counter()
    f.run()
    sec = time.perf_counter() - t0
    info = f.info()
    o64 = O.OracleFrame(fr.xyz, fr.radius, flags=O.FP64)
    for s in (1, 2, 3):
        o64.stage(s)
    xm, G, det = o64.aniso()
    gG = f.dump(N.DUMP_G)
    flags = f.dump(N.DUMP_FP64_FLAGS).astype(bool)
    eG = np.abs(gG - G).reshape(len(G), -1).max(1)
    rng = np.random.default_rng(3)
    pts = (fr.xyz[rng.choice(fr.n, 20000)] + rng.normal(0, 1.5 * fr.radius, (20000, 3))).astype(np.float32)
    ms = info["max_scalar"]
    ef = np.abs(f.eval(pts) - o64.eval(pts)) / ms
    print(json.dumps({
        "metric": METRIC, "workload": "stress", "value": 1.0 / sec, "unit": UNIT,
        "particles": fr.n, "fp64_eigen_particles": int(info["fp64_eigen"]),
        "fp32_eigen_particles": int(fr.n - info["fp64_eigen"]),
        "G_err_vs_fp64": {"max_fp64_path": float(eG[flags].max()) if flags.any() else None,
                          "max_fp32_path": float(eG[~flags].max()) if (~flags).any() else None,
                          "rms": float(np.sqrt(np.mean(eG ** 2)))},
        "field_err_vs_fp64_over_maxscalar": {"max": float(ef.max()), "rms": float(np.sqrt(np.mean(ef ** 2)))},
        "nodes": info["num_nodes"], "vertices": info["num_vertices"],
        "data": "synthetic (seeded sheets on planes and saddles, Bezier filaments)"}))
    f.close()
    ctx.close()


def single(a):
    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    B.build()
    fr = make_frame(a.n)
    ctx = N.Context(0)
    ctx.tune(a.samples_per_lane)
    p = N.default_params(fr.radius)
    p.qef = 1 if a.qef else 0
    f = N.Frame(ctx, p).upload(fr.xyz).run()
    info = f.info()
    print(json.dumps({k: info[k] for k in ("num_nodes", "num_vertices", "num_triangles", "field_evals",
                                           "candidate_pairs", "stage_ms", "qef_accepted")}))
    f.close()
    ctx.close()


def fp32_gemm_tflops(torch, n=8192, reps=5):
    """Measured FP32 denominator: cuBLAS SGEMM n^3 with TF32 off (FFMA pipe),
    best of `reps`, CUDA events."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, device="cuda", dtype=torch.float32)
        b = torch.randn(n, n, device="cuda", dtype=torch.float32)
        torch.matmul(a, b)
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        del a, b
        return 2.0 * n ** 3 / (best / 1000.0) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def rank_max(x, world):
    """Max of a per-rank number over all ranks (timings: the slowest rank sets
    the step time).  Host-side gloo collective; frames never leave their GPU."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        """Starts the sampler and returns once its first sample is written, so
        that nvidia-smi's own start-up (process, NVML) lies before the timed
        region rather than inside its first steps."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.time()
        while time.time() - t0 < 1.5 and self.proc.poll() is None:
            if os.path.getsize(self.tmp.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = [r.split(",") for r in open(self.tmp.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.tmp.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        load = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": float(np.median(load)) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_frame(n):
    from particleisosurface_gb300 import synth
    return synth.dam_break(n=n, seed=2)


def cpu_sample(fr, field_evals, sample_evals, nthreads):
    """Bounded CPU measurement of one frame with the oracle (see module doc).
    Returns (seconds per frame, evals/s, detail)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle as O
    O.build()
    O.set_threads(nthreads)
    o = O.OracleFrame(fr.xyz, fr.radius)
    t0 = time.perf_counter()
    for s in (1, 2, 3):
        o.stage(s)
    t13 = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    idx = rng.choice(fr.n, sample_evals)
    pts = (fr.xyz[idx] + rng.normal(0, 1.5 * fr.radius, (sample_evals, 3))).astype(np.float32)
    t0 = time.perf_counter()
    o.eval(pts)
    te = time.perf_counter() - t0
    rate = sample_evals / te
    o.close()
    sec = t13 + field_evals / rate
    return sec, rate, {"stages_1_3_s": round(t13, 3), "eval_sample_s": round(te, 3)}


def reference_arm(a):
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        if rank != 0:
            dist.barrier()
            dist.destroy_process_group()
            return
    fr = make_frame(a.n)
    nthreads = os.cpu_count() or 1
    times = []
    for k in range(a.warmup + a.steps):
        sec, rate, det = cpu_sample(fr, ORACLE_FIELD_EVALS * a.n // 1_000_000, a.cpu_sample_evals, nthreads)
        if k >= a.warmup:
            times.append(sec)
    ms = 1000.0 * float(np.mean(times))
    value = 1000.0 / ms
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "frames_per_step": 1},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "oracle stages 1-3 on the full frame + %d field evals; octree/extraction = "
                                   "%d evals / measured rate" % (a.cpu_sample_evals, ORACLE_FIELD_EVALS)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "field_evals_per_s": rate, "p50_ms": 1000 * float(np.percentile(times, 50)),
        "p99_ms": 1000 * float(np.percentile(times, 99)),
    }
    print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def ours(a):
    import torch

    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    B.build()
    torch.cuda.set_device(local)
    fr = make_frame(a.n)
    ctx = N.Context(local)
    params = N.default_params(fr.radius)
    stream = torch.cuda.ExternalStream(N.lib().pi_ctx_stream(ctx.h), device=local)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # ---- device-resident frames: value ----
    f = N.Frame(ctx, params).upload(fr.xyz)
    for _ in range(a.warmup):
        f.reset().run()
    info = f.info()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    launches0 = ctx.stats()["launches"]
    ctx.profile(True)
    ctx.kernel_time()  # reset
    clocks = Clocks(local)
    barrier()
    clocks.start()
    t_wall = time.perf_counter()
    step_launches = 0
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
        l0 = ctx.stats()["launches"]
        ev[k][0].record(stream)
        f.reset().run()
        ev[k][1].record(stream)
        step_launches += ctx.stats()["launches"] - l0
    barrier()
    t_wall = time.perf_counter() - t_wall
    ck = clocks.stop()
    kt = ctx.kernel_time()
    ctx.profile(False)
    step_ms = [s.elapsed_time(e) for s, e in ev]
    info = f.info()
    ms = rank_max(float(np.mean(step_ms)), world)

    # ---- the same frame with the per-leaf FP64 QEF solve switched on ----
    pq = N.default_params(fr.radius)
    pq.qef = 1
    fq = N.Frame(ctx, pq).upload(fr.xyz)
    for _ in range(a.warmup):
        fq.reset().run()
    evq = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    barrier()
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
        evq[k][0].record(stream)
        fq.reset().run()
        evq[k][1].record(stream)
    barrier()
    qef_ms = rank_max(float(np.mean([s.elapsed_time(e) for s, e in evq])), world)
    qinfo = fq.info()
    fq.close()

    # ---- end to end through the C ABI with pinned host buffers: e2e ----
    xyz_h = torch.from_numpy(fr.xyz).pin_memory()
    mv = int(info["num_vertices"] * 1.5) + 1024
    mt = int(info["num_triangles"] * 1.5) + 1024
    v_h = torch.empty((mv, 3), dtype=torch.float32).pin_memory()
    t_h = torch.empty((mt, 3), dtype=torch.int32).pin_memory()
    import ctypes as C
    nv, nt = C.c_int64(), C.c_int64()

    def e2e_step():
        N.check(N.lib().pi_reconstruct(
            ctx.h, C.byref(params), C.cast(xyz_h.data_ptr(), C.POINTER(C.c_float)), fr.n,
            C.cast(v_h.data_ptr(), C.POINTER(C.c_float)), mv, C.cast(t_h.data_ptr(), C.POINTER(C.c_int32)), mt,
            C.byref(nv), C.byref(nt)))

    for _ in range(max(1, a.warmup)):
        e2e_step()
    ev2 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    barrier()
    for k in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(k & 0xff)
        ev2[k][0].record(stream)
        e2e_step()
        ev2[k][1].record(stream)
    barrier()
    e2e_ms = rank_max(float(np.mean([s.elapsed_time(e) for s, e in ev2])), world)

    if rank == 0:
        evals = info["field_evals"]
        line = {
            "metric": METRIC, "value": world * 1000.0 / ms, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam-break column + spray)",
            "config": {"workload": WORKLOAD, "frames_per_step_per_gpu": 1, "parallelism": "replicas",
                       "l2": "512 MiB buffer written between steps", "depth_max": info["depth_max"],
                       "nodes": info["num_nodes"], "vertices": info["num_vertices"],
                       "triangles": info["num_triangles"],
                       "samples_per_lane": dict(zip(["leaf_level", "level_above"], ctx.tuning()))},
            "field_evals_per_s": world * evals / (ms / 1000.0),
            "field_evals_per_frame": evals,
            "candidate_pairs_per_frame": info["candidate_pairs"],
            "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
            "stage_ms": dict(zip(["upload", "hash", "aniso", "normals", "octree", "qef", "extract", "download"],
                                 [round(x, 3) for x in info["stage_ms"]])),
            "wall_s_timed": t_wall,
            "gpu_launches": int(step_launches),
            "e2e": {"value": world * 1000.0 / e2e_ms, "unit": UNIT, "h2d_bytes_per_step": 12 * fr.n,
                    "d2h_bytes_per_step": 12 * int(nv.value) + 12 * int(nt.value)},
            "clocks": ck,
            "qef_on": {"ms_per_step": qef_ms, "frames_per_s": world * 1000.0 / qef_ms,
                       "field_evals_per_frame": qinfo["field_evals"],
                       "candidate_pairs_per_frame": qinfo["candidate_pairs"],
                       "qef_vertices_accepted": qinfo["qef_accepted"]},
        }
        # dominant kernel: field evaluation at octree samples (k_q_eval)
        if kt["ms"] > 0 and kt["launches"] > 0:
            achieved = kt["pairs"] * FLOPS_PER_PAIR / (kt["ms"] / 1000.0) / 1e12
            sm_mhz = ck.get("sm_max_mhz") or 2070.0
            nominal = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
            peak = fp32_gemm_tflops(torch)
            line["roofline"] = {"kernel": "k_q_eval_thread + k_q_eval (field evaluation at octree samples)",
                                "bound": "fp32",
                                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                                "traffic": FIELD_DRAM_BYTES_PER_FRAME if fr.n == 1_000_000 else None,
                                "traffic_per": "frame (the same launches), one ncu capture of "
                                               "dram__bytes_read.sum + dram__bytes_write.sum",
                                "peak_source": "measured in this run: cuBLAS FP32 GEMM 8192^3, TF32 off, best of 5 "
                                               "(MEASURED_PEAKS.json has HBM and bf16 figures only)",
                                "nominal_fp32_peak": nominal, "frac_of_nominal": achieved / nominal,
                                "kernel_ms_per_step": kt["ms"] / a.steps,
                                "launches_per_step": kt["launches"] / a.steps}
        if not a.no_cpu_baseline and world == 1:
            nthreads = os.cpu_count() or 1
            oracle_evals = ORACLE_FIELD_EVALS * fr.n // 1_000_000
            sec, rate, det = cpu_sample(fr, oracle_evals, a.cpu_sample_evals, nthreads)
            line["cpu_baseline"] = {"value": 1.0 / sec, "unit": UNIT, "cores": nthreads, "kind": "port",
                                    "sample": "oracle stages 1-3 on the full frame + %d field evals; "
                                              "octree/extraction = %d evals (the oracle's count on this frame) "
                                              "/ measured rate" % (a.cpu_sample_evals, oracle_evals),
                                    "field_evals_per_s": rate, **det}
        print(json.dumps(line))
    f.close()
    ctx.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main():
    a = parse()
    if a.workload != "dam_break_1m" and a.impl == "ours":
        {"batch64": batch64, "serving": serving, "stress": stress, "grid": grid}[a.workload](a)
    elif a.single:
        single(a)
    elif a.impl == "reference":
        reference_arm(a)
    else:
        ours(a)


if __name__ == "__main__":
    main()
