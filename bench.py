"""Benchmark: particle-steps/s of the interval push on one GB300.

Workload (the scale configuration): a 1024 x 2048 compact field on stretched
y edges (dy proportional to 1 + 4 (y/2)^2 over [-2, 2], x uniform on [-1, 1]),
Harris sheet plus 8 magnetic islands (psi = 0.1 cos(4 pi x) exp(-y^2/0.04)),
two frames with seeded 1 % multiplicative noise; a particle population
injected uniformly over the domain (p = p0, times spread over the first
interval) and pushed across consecutive MHD intervals.  One step = one
``kpt_push_interval`` over the whole population (Parker transport; the mixed
precision path is the headline, the plain FP64 push is measured beside it).

Timing: CUDA events on the library's stream around exactly K steps after W
warm-up steps; the tables (2 x 135 MB mixed, 2 x 270 MB FP64) exceed the
129 MB L2, so no flush is needed between steps.  ``e2e`` is the same metric
through the C ABI with host buffers: every step uploads the particle state
from pinned host memory, pushes and downloads it.

``--impl reference`` times the CPU baseline: the oracle restatement of the
reference push (bit-identical to the reference's own code on the same
inputs), OpenMP on all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

fields = importlib.import_module("kokkos-particletransport_gb300.fields")

NX, NY = 1024, 2048
SEED = 114514
START_FRAME = 100
METRIC = "particle-steps/s, 1 GB300: mixed+surrogate vs plain FP64 at <=1% spectrum error"
BYTES_PER_STEP = {"f64": 1024, "mixed": 512}  # 2 frames x 4 corners x 16 comps x 8|4 B


def make_workload():
    ye = fields.stretched_edges(NY, -2.0, 2.0, strength=4.0)
    f0 = fields.harris_field(NX, NY, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=1)
    f1 = fields.harris_field(NX, NY, y_edges=ye, island_amplitude=0.1, noise=0.01, seed=2)
    return f0, f1


def settings_dict(kpt):
    s = kpt.default_settings(kperp_over_kpara=0.05, split_ratio=1.2)
    return s


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as stream:
            data = json.load(stream)
        return float(data["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                         text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": smax or None, "reasons": sorted(reasons), "samples": len(sm)}


def run_gpu(args):
    import torch
    kpt = importlib.import_module("kokkos-particletransport_gb300")
    f0, f1 = make_workload()
    settings = settings_dict(kpt)
    ctx = kpt.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    n = args.particles
    results = {}
    for label, precision in (("mixed", kpt.PRECISION_MIXED), ("f64", kpt.PRECISION_F64)):
        lower = ctx.field(f0, kpt.TABLE_PARKER16, precision)
        upper = ctx.field(f1, kpt.TABLE_PARKER16, precision)
        parts = ctx.particles(n)
        ctx.inject(parts, lower, settings, n, START_FRAME, SEED)
        start = parts.download()
        frame = START_FRAME
        for _ in range(args.warmup):
            if args.sort_tile > 0:
                ctx.sort(parts, lower, args.sort_tile, args.sort_tile)
            ctx.push_interval(parts, lower, upper, settings, frame, SEED)
            frame += 1
        torch.cuda.synchronize()
        begin = torch.cuda.Event(enable_timing=True)
        end = torch.cuda.Event(enable_timing=True)
        kernel_ms = []
        steps = 0
        with ClockSampler() as clocks:
            begin.record(stream)
            for _ in range(args.steps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                if args.sort_tile > 0:
                    ctx.sort(parts, lower, args.sort_tile, args.sort_tile)
                e0.record(stream)
                stats = ctx.push_interval(parts, lower, upper, settings, frame, SEED)
                e1.record(stream)
                steps += stats.particle_steps
                frame += 1
                e1.synchronize()
                kernel_ms.append(e0.elapsed_time(e1))
            end.record(stream)
            end.synchronize()
        total_ms = begin.elapsed_time(end)
        # e2e: through the C ABI with host buffers (H2D upload, push, D2H download)
        host = {k: v.copy() for k, v in start.items()}
        e2e_steps = 0
        t0 = time.perf_counter()
        for k in range(args.steps):
            parts.upload(host, n)
            if args.sort_tile > 0:
                ctx.sort(parts, lower, args.sort_tile, args.sort_tile)
            stats = ctx.push_interval(parts, lower, upper, settings, START_FRAME + k, SEED)
            host = parts.download(n)
            e2e_steps += stats.particle_steps
        e2e_s = time.perf_counter() - t0
        results[label] = dict(total_ms=total_ms, kernel_ms=kernel_ms, steps=steps,
                              clocks=clocks.summary(), e2e_steps=e2e_steps, e2e_s=e2e_s,
                              state_bytes=n * (7 * 8 + 2 * 4))
        for obj in (lower, upper, parts):
            obj.close()
    ctx.close()
    return results


def run_focused(args):
    """Focused transport with the slab-QLT closure on the same field: one
    interval push of the population per step, FP64 and mixed."""
    import torch
    kpt = importlib.import_module("kokkos-particletransport_gb300")
    f0, f1 = make_workload()
    settings = kpt.default_settings(kperp_over_kpara=0.05, focused=1, closure=kpt.CLOSURE_QLT)
    ctx = kpt.Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    out = {}
    for label, precision in (("mixed", kpt.PRECISION_MIXED), ("f64", kpt.PRECISION_F64)):
        n = args.focused_particles
        lower = ctx.field(f0, kpt.TABLE_FOCUSED21, precision)
        upper = ctx.field(f1, kpt.TABLE_FOCUSED21, precision)
        parts = ctx.particles(n)
        ctx.inject(parts, lower, settings, n, START_FRAME, SEED)
        start = parts.download()
        # warm-up: one interval on a copy of the population
        ctx.sort(parts, lower, 16, 16)
        ctx.push_interval(parts, lower, upper, settings, START_FRAME, SEED)
        parts.upload(start, n)
        ctx.sort(parts, lower, 16, 16)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        stats = ctx.push_interval(parts, lower, upper, settings, START_FRAME, SEED)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[label] = {"value": stats.particle_steps / (ms / 1e3), "ms": ms,
                      "particle_steps": int(stats.particle_steps), "particles": n}
        for obj in (lower, upper, parts):
            obj.close()
    ctx.close()
    out["speedup_mixed_over_f64"] = out["mixed"]["value"] / out["f64"]["value"]
    return out


def cpu_baseline(particles: int, steps: int = 1):
    """Oracle restatement (OpenMP, all host threads) on a bounded sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    binding = importlib.import_module("binding")
    kpt = importlib.import_module("kokkos-particletransport_gb300")
    f0, f1 = make_workload()
    oracle = binding.Oracle()
    params = binding.default_params(kperp_over_kpara=0.05, split_ratio=1.2)
    grid = oracle.grid(f0.x_edges, f0.y_edges)
    lo, up = oracle.table(f0), oracle.table(f1)
    parts = binding.empty_particles(particles)
    oracle.inject(grid, params, START_FRAME * 0.1, START_FRAME, SEED, particles, 0, particles,
                  parts)
    threads = os.cpu_count() or 1
    total_steps = 0
    t0 = time.perf_counter()
    for k in range(steps):
        frame = START_FRAME + k
        s = oracle.push(grid, lo, up, params, frame * params["mhd_dt"], frame, SEED, particles,
                        parts, threads=threads)
        total_steps += int(s.sum())
    elapsed = time.perf_counter() - t0
    oracle.free_grid(grid)
    del kpt
    return total_steps / elapsed, threads, elapsed, total_steps


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=5)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    parser.add_argument("--particles", type=int, default=1 << 20)
    parser.add_argument("--cpu-particles", type=int, default=1 << 15)
    parser.add_argument("--focused-particles", type=int, default=1 << 16,
                        help="population of the focused/QLT leg (0 skips it)")
    parser.add_argument("--sort-tile", type=int, default=16,
                        help="cell-sort tile (cells) before each push; 0 disables")
    args = parser.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    config = {"workload": f"parker push, {NX}x{NY} stretched-y Harris+islands field, "
                          f"{args.particles} particles, consecutive intervals",
              "nx": NX, "ny": NY, "particles": args.particles, "transport": "parker",
              "l2": "tables larger than L2 (no flush)", "sort_tile": args.sort_tile}
    if args.impl == "reference":
        if rank != 0:
            return
        value, threads, elapsed, total = cpu_baseline(args.cpu_particles, max(1, args.steps))
        line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "impl": "reference",
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": dict(config,
                                                                    particles=args.cpu_particles),
                "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads,
                                 "kind": "port",
                                 "sample": f"{args.cpu_particles} particles x {args.steps} "
                                           f"intervals ({total} particle-steps, {elapsed:.1f} s)"},
                "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    results = run_gpu(args)
    focused = run_focused(args) if args.focused_particles > 0 else None
    peak, peak_kind = read_peaks()
    mixed, f64 = results["mixed"], results["f64"]
    value = mixed["steps"] / (mixed["total_ms"] / 1e3)
    f64_value = f64["steps"] / (f64["total_ms"] / 1e3)
    kernel_s = np.mean(mixed["kernel_ms"]) / 1e3
    steps_per_launch = mixed["steps"] / args.steps
    achieved = steps_per_launch * BYTES_PER_STEP["mixed"] / kernel_s / 1e9
    cpu_value, cpu_threads, cpu_elapsed, cpu_total = cpu_baseline(args.cpu_particles, 1)
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mixed["total_ms"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
        "data": "synthetic", "config": config,
        "plain_f64": {"value": f64_value, "ms_per_step": f64["total_ms"] / args.steps,
                      "speedup_mixed_over_f64": value / f64_value},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None,
                     "model": "512 B per particle-step (2 frames x 4 corners x 16 f32)",
                     "peak_kind": peak_kind},
        "cpu_baseline": {"value": cpu_value, "unit": "particle-steps/s", "cores": cpu_threads,
                         "kind": "port",
                         "sample": f"{args.cpu_particles} particles x 1 interval "
                                   f"({cpu_total} particle-steps, {cpu_elapsed:.1f} s)"},
        "e2e": {"value": mixed["e2e_steps"] / mixed["e2e_s"], "unit": "particle-steps/s",
                "h2d_bytes_per_step": mixed["state_bytes"],
                "d2h_bytes_per_step": mixed["state_bytes"]},
        # per timed step: the push, plus 3 cell-sort kernels when sorting
        "focused_qlt": focused,
        "gpu_launches": args.steps * (1 + (3 if args.sort_tile > 0 else 0)),
        "clocks": mixed["clocks"],
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
