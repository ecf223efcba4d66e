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


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--n", type=int, default=1_000_000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample-evals", type=int, default=200_000)
    p.add_argument("--single", action="store_true",
                   help="reconstruct one frame once and print its counters (for profiler captures)")
    return p.parse_args()


def single(a):
    from particleisosurface_gb300 import _native as N
    from particleisosurface_gb300 import build as B
    B.build()
    fr = make_frame(a.n)
    ctx = N.Context(0)
    f = N.Frame(ctx, N.default_params(fr.radius)).upload(fr.xyz).run()
    info = f.info()
    print(json.dumps({k: info[k] for k in ("num_nodes", "num_vertices", "num_triangles", "field_evals",
                                           "candidate_pairs", "stage_ms")}))
    f.close()
    ctx.close()


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
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

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
    ms = float(np.mean(step_ms))
    if world > 1:
        t = torch.tensor([ms], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())

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
    e2e_ms = float(np.mean([s.elapsed_time(e) for s, e in ev2]))
    if world > 1:
        t = torch.tensor([e2e_ms], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())

    if rank == 0:
        evals = info["field_evals"]
        line = {
            "metric": METRIC, "value": world * 1000.0 / ms, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam-break column + spray)",
            "config": {"workload": WORKLOAD, "frames_per_step_per_gpu": 1, "parallelism": "replicas",
                       "l2": "512 MiB buffer written between steps", "depth_max": info["depth_max"],
                       "nodes": info["num_nodes"], "vertices": info["num_vertices"],
                       "triangles": info["num_triangles"]},
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
        }
        # dominant kernel: field evaluation at octree samples (k_sample)
        if kt["ms"] > 0 and kt["launches"] > 0:
            achieved = kt["pairs"] * FLOPS_PER_PAIR / (kt["ms"] / 1000.0) / 1e12
            sm_mhz = ck.get("sm_max_mhz") or 2070.0
            peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
            line["roofline"] = {"kernel": "k_sample (field evaluation at octree samples)", "bound": "fp32",
                                "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                                "traffic": None,
                                "peak_source": "nominal FP32: 152 SMs x 128 lanes x 2 flop x max SM clock "
                                               "(MEASURED_PEAKS.json has no FP32 figure)",
                                "kernel_ms_per_step": kt["ms"] / a.steps,
                                "launches_per_step": kt["launches"] / a.steps}
        if not a.no_cpu_baseline and world == 1:
            nthreads = os.cpu_count() or 1
            sec, rate, det = cpu_sample(fr, evals, a.cpu_sample_evals, nthreads)
            line["cpu_baseline"] = {"value": 1.0 / sec, "unit": UNIT, "cores": nthreads, "kind": "port",
                                    "sample": "oracle stages 1-3 on the full frame + %d field evals; "
                                              "octree/extraction = %d evals / measured rate" % (a.cpu_sample_evals,
                                                                                              evals),
                                    "field_evals_per_s": rate, **det}
        print(json.dumps(line))
    f.close()
    ctx.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


def main():
    a = parse()
    if a.single:
        single(a)
    elif a.impl == "reference":
        reference_arm(a)
    else:
        ours(a)


if __name__ == "__main__":
    main()
