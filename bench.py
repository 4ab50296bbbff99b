#!/usr/bin/env python
"""Time-step throughput of the GB300 engine on the 128x128x64 multi-material lattice.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision fp64|fp32c]

Workload (seeded, synthetic; no public dataset exists for this path): 128x128x64 grid, Bernoulli
0.85 fill (largest 6-connected component kept: ~0.89 M voxels, ~2.25 M links), 4 bilinear
materials (E log-uniform 1e5..1e7 Pa, rho 1000..3000, nu 0.3), gravity and floor, 1 cm voxels,
dt = recommendedTimeStep() at t = 0, then fixed.  A bench step is one doTimeStep.

value  voxel-steps/s with the scene resident on the GPU: K steps timed with CUDA events on the
       engine stream (first to last kernel), max over ranks.  The state (~1 GB) exceeds L2, so no
       flush is needed between steps.
e2e    the same metric through the public C facade per step: upload every voxel's temperature from
       pinned host memory (vx_set_temperatures), doTimeStep, read every position back into pinned
       memory (vx_read_positions); host wall clock.
N > 1  replicas only: each rank simulates its own copy (the lattice does not shard without a halo
       exchange); value = all ranks' voxel-steps / max time.
--impl reference  times the reference's CPU time step (the oracle restatement, C-library math,
       OpenMP on all host cores, as the reference's USE_OMP build) on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "voxel-steps/s at 1M voxels (128x128x64 multi-material lattice)"
UNIT = "voxel-steps/s"


def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class _Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _peak_hbm():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic(kernel: str, n_voxels: int, n_links: int):
    """DRAM bytes per launch from the committed ncu capture (profiles/traffic.json), scaled by
    the units one launch processes; None when no capture is committed."""
    try:
        t = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))[kernel]
        return t["bytes_per_voxel"] * n_voxels + t["bytes_per_link"] * n_links
    except Exception:
        return None


def build_lattice(sim_factory):
    from voxelyze_gb300 import scenes as S

    sc = S.lattice(128, 128, 64)
    sim = sim_factory(sc.voxel_size)
    S.apply(sc, sim)
    return sc, sim


def cpu_oracle_rate(sc, threads: int, budget_s: float, steps_cap: int | None = None):
    """Voxel-steps/s of the oracle (C-library math, `threads` OpenMP threads) on `sc`."""
    from voxelyze_gb300 import facade as F, scenes as S

    lib = C.CDLL(os.path.join(ROOT, "oracle", "_build", "libvxoracle.so"))
    lib.vxo_set_math(0)
    sim = F.Sim(lib, "vxo", sc.voxel_size)
    S.apply(sc, sim)
    lib.vxo_set_threads(C.c_void_p(sim.h), threads)
    dt = sim.recommended_time_step()
    sim.do_time_step(dt)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        sim.do_time_step(dt)
        n += 1
        el = time.perf_counter() - t0
        if el >= budget_s or (steps_cap and n >= steps_cap):
            break
    return sim.voxel_count() * n / el, n, el


def run_reference(args, world, rank):
    if rank != 0:
        return
    from voxelyze_gb300 import scenes as S

    sc = S.lattice(128, 128, 64)
    cores = os.cpu_count() or 1
    # warmup and timed steps, each one doTimeStep of the full lattice on all host cores
    rate_w, _, _ = cpu_oracle_rate(sc, cores, 0.0, steps_cap=max(1, args.warmup))
    rate, n, el = cpu_oracle_rate(sc, cores, 0.0, steps_cap=max(1, args.steps))
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": n,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "lattice 128x128x64, fill 0.85, 4 bilinear materials, nu 0.3, gravity+floor",
                       "voxels": sc.n_voxels, "precision": "fp64 CPU, C-library math"},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{n} doTimeStep calls of the full 128x128x64 lattice"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args, world, rank, local):
    import voxelyze_gb300 as vg

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    lib = vg.library()
    sc, sim = build_lattice(vg.Sim)
    nv, nl = sim.voxel_count(), sim.link_count()
    if args.precision == "fp32c":
        if lib.vx_set_precision(C.c_void_p(sim.h), 1) != 0:
            raise RuntimeError("FP32C precision not available")
    dt = sim.recommended_time_step()
    h = C.c_void_p(sim.h)
    lib.vx_step_timing.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    if sim.do_time_steps(args.warmup, dt) != args.warmup:
        raise RuntimeError("warm-up diverged")

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    # ---- device-timed throughput (CUDA events on the engine stream) -------------------------
    lib.vx_enable_timing(h, 1)
    barrier()
    with _Clocks(local) as clk:
        done = sim.do_time_steps(args.steps, dt)
    barrier()
    lib.vx_enable_timing(h, 0)
    if done != args.steps:
        raise RuntimeError(f"diverged after {done} steps")
    tm = (C.c_float * 4)()
    lib.vx_step_timing(h, tm)
    batch_ms, link_ms, col_ms, vox_ms = [float(x) for x in tm]
    # per-step time over the timed region: first kernel to last, plus one step's own length
    total_ms = batch_ms * args.steps / max(args.steps - 1, 1) if args.steps > 1 else link_ms + col_ms + vox_ms
    if world > 1:
        import torch
        import torch.distributed as dist

        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * nv * args.steps / (total_ms / 1e3)

    # ---- end to end through the public C facade ----------------------------------------------
    import torch

    temps = torch.zeros(nv, dtype=torch.float32, pin_memory=True)
    pos = torch.empty(3 * nv, dtype=torch.float64, pin_memory=True)
    lib.vx_set_temperatures.argtypes = [C.c_void_p, C.c_void_p]
    lib.vx_read_positions.argtypes = [C.c_void_p, C.c_void_p]
    e2e_steps = max(3, min(args.steps, 50))
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        if lib.vx_set_temperatures(h, temps.data_ptr()) != 0:
            raise RuntimeError("vx_set_temperatures failed")
        if lib.vx_do_time_step(h, C.c_float(dt)) != 1:
            raise RuntimeError("e2e step diverged")
        if lib.vx_read_positions(h, pos.data_ptr()) != 0:
            raise RuntimeError("vx_read_positions failed")
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_value = world * nv * e2e_steps / e2e_s

    # ---- roofline of the dominant pass -----------------------------------------------------
    from voxelyze_gb300 import roofline as R

    b = R.fp64_bytes(nv, nl, poisson=True)
    kernel = "link" if link_ms >= vox_ms else "voxel"
    k_ms = link_ms if kernel == "link" else vox_ms
    achieved = b[kernel] / (k_ms / 1e3) / 1e9
    peak, peak_kind = _peak_hbm()
    roof = {"bound": "hbm", "kernel": f"k_{kernel} (FP64 {kernel} pass)", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": b[kernel], "ms_per_launch": k_ms,
            "traffic": _traffic(f"k_{kernel}_fp64", nv, nl),
            "note": "FP64 pass: bound by the FP64 pipe on GB300, not by HBM"}

    # ---- CPU baseline: the oracle on the host cores, bounded sample ----------------------------
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        rate, n, el = cpu_oracle_rate(sc, cores, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{n} doTimeStep calls of the full lattice in {el:.1f} s (OpenMP, C-library math)"}

    launches_per_step = 3  # Poisson pre-pass, link pass, voxel pass
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic",
            "config": {"workload": "lattice 128x128x64, fill 0.85, 4 bilinear materials, nu 0.3, gravity+floor, 1 cm",
                       "voxels": nv, "links": nl, "precision": args.precision, "parallelism": f"replicas x{world}",
                       "l2": "state ~1 GB > 129 MB L2, no flush", "dt": dt,
                       "per_pass_ms": {"link": link_ms, "collide": col_ms, "voxel": vox_ms}},
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 4 * nv, "d2h_bytes_per_step": 24 * nv,
                    "steps": e2e_steps},
            "clocks": clk.summary(), "gpu_launches": launches_per_step * args.steps}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32c"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    world, rank, local = _dist()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
