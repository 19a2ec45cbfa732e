"""Speed of the C restatement (oracle/kpt_oracle.c, the CPU baseline the
bench times) against the reference's own driver code on the Kokkos-API shim
(oracle/_ref), on identical workloads and the same host cores.

Test infrastructure: run where the reference build exists (oracle/_ref), e.g.

    OMP_PROC_BIND=spread OMP_PLACES=threads python oracle/time_port_vs_reference.py

Workloads (the reference driver's own physics; both codes draw the same keyed
noise, so they execute the same substeps and the restatement's step count
applies to both):
  parker_c1     256x512 uniform Harris field, 25,600 particles injected in
                |y| < 0.2, kperp/kpara 0.05, 100 fixed steps per interval
  focused_c1    the same field and particles, focused transport with the
                driver's reduced pitch-angle closure, 100 fixed steps
  parker_adaptive  the same, Parker with the driver's adaptive dt
Prints one JSON object: per workload the particle-steps, each code's push
seconds (best of `--repeats`) and the restatement/reference speed ratio.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import binding  # noqa: E402

fields = __import__("importlib").import_module("kokkos-particletransport_gb300.fields")


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--repeats", type=int, default=3)
    parser.add_argument("--particles", type=int, default=25600)
    args = parser.parse_args()
    threads = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    # both on the C library's pow, as the bench's CPU baseline and a real
    # Kokkos host build are
    oracle = binding.Oracle(libm_pow=True)
    ref = binding.ReferenceHarness(libm_pow=True)
    field = fields.harris_field(256, 512)
    frame, seed, n = 0, 114514, args.particles
    out = {"threads": threads, "cpu": platform_cpu(), "particles": n, "workloads": {}}
    with tempfile.TemporaryDirectory() as field_dir:
        for f in (frame, frame + 1):
            fields.write_compact_field(fields.field_file_path(field_dir, f), field)
        grid = oracle.grid(field.x_edges, field.y_edges)
        cases = {
            "parker_c1": dict(kperp_over_kpara=0.05, dt_min_rel=1e-2, dt_max_rel=1e-2),
            "focused_c1": dict(kperp_over_kpara=0.05, focused=1, dt_min_rel=1e-2,
                               dt_max_rel=1e-2),
            "parker_adaptive": dict(kperp_over_kpara=0.05),
        }
        for name, overrides in cases.items():
            params = binding.default_params(**overrides)
            focused = bool(params["focused"])
            start = binding.empty_particles(n)
            count = oracle.inject(grid, params, frame * params["mhd_dt"], frame, seed, n, 0, n,
                                  start, band=(-0.2, 0.2))
            lo, up = oracle.table(field, focused), oracle.table(field, focused)
            port_s, ref_s, steps = [], [], 0
            for _ in range(args.repeats):
                a = {k: v.copy() for k, v in start.items()}
                t0 = time.perf_counter()
                per = oracle.push(grid, lo, up, params, frame * params["mhd_dt"], frame, seed,
                                  count, a, threads=threads)
                port_s.append(time.perf_counter() - t0)
                steps = int(per.sum())
                b = {k: v.copy() for k, v in start.items()}
                ref.push(field_dir, params, seed, frame, n, count, b)
                ref_s.append(ref.last_move_seconds())
                same = all(np.array_equal(a[k][:count], b[k][:count]) for k in a)
            out["workloads"][name] = {
                "particle_steps": steps, "port_s": min(port_s), "reference_s": min(ref_s),
                "port_particle_steps_per_s": steps / min(port_s),
                "reference_particle_steps_per_s": steps / min(ref_s),
                "port_over_reference_speed": min(ref_s) / min(port_s),
                "identical_results": bool(same)}
        oracle.free_grid(grid)
    print(json.dumps(out, indent=1))


def platform_cpu() -> str:
    try:
        with open("/proc/cpuinfo") as stream:
            for line in stream:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


if __name__ == "__main__":
    main()
