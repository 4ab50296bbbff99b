#!/usr/bin/env python
"""Time-step throughput of the GB300 engine on the 128x128x64 multi-material lattice.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--precision fp32c|fp64]
                    [--workload lattice|cantilever|porous|population]

Workload (seeded, synthetic; no public dataset exists for this path): 128x128x64 grid, Bernoulli
0.85 fill (largest 6-connected component kept: ~0.89 M voxels, ~2.25 M links), 4 bilinear
materials (E log-uniform 1e5..1e7 Pa, rho 1000..3000, nu 0.3), gravity and floor, 1 cm voxels,
dt = recommendedTimeStep() at t = 0, then fixed.  A bench step is one doTimeStep.  --workload
selects the other seeded scenes (40x8x8 cantilever; 64^3 porous body with collisions; 4,096
independent bodies with in-step CTE actuation, whose CPU baseline steps the first 64 bodies).

value  voxel-steps/s of the FP32-compensated path (--precision, default fp32c) with the scene
       resident on the GPU: K steps timed with CUDA events on the engine stream (first to last
       kernel), max over ranks.  The FP64 path is timed the same way in the same run and reported
       beside it, with the FP32C position error against it (the FP64 path is bit-identical to the
       FP64 oracle).  The state (0.6-1 GB) exceeds L2, so no flush is needed between steps.
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
import threading
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
    """SM clock and clock-event (throttle) reasons sampled during the timed region: NVML through
    ctypes every ~2 ms (read-only queries), else ``nvidia-smi -lms 200``."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # nvmlClocksEventReason bits
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
            0x80: "hw_power_brake_slowdown"}

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.f = None
        self.p = None
        self.nvml = None
        self.samples = []
        self.stop = threading.Event()
        self.th = None

    def _nvml_open(self):
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = C.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.gpu), C.byref(h)) != 0:
                return None
            fn = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
            return lib, h, fn
        except (OSError, AttributeError):
            return None

    def _poll(self):
        lib, h, reasons_fn = self.nvml
        mhz, mx, mask = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self.stop.is_set():
            if (lib.nvmlDeviceGetClockInfo(h, 1, C.byref(mhz)) == 0 and
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 and reasons_fn(h, C.byref(mask)) == 0):
                self.samples.append((float(mhz.value), float(mx.value), int(mask.value)))
            time.sleep(0.002)

    def __enter__(self):
        self.nvml = self._nvml_open()
        if self.nvml:
            self.th = threading.Thread(target=self._poll, daemon=True)
            self.th.start()
            return self
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.th:
            self.stop.set()
            self.th.join()
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        if self.nvml:
            for mhz, m, mask in self.samples:
                sm.append(mhz)
                mx = max(mx, m)
                for bit, name in self.BITS.items():
                    if mask & bit:
                        reasons.add(name)
            src = "nvml"
        else:
            src = "nvidia-smi"
            if self.f:
                self.f.flush()
                self.f.seek(0)
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
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no clock samples"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm),
                "source": src}


def _peak_hbm():
    try:
        return float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


DIMS = (128, 128, 64)


class Workload:
    """One seeded synthetic scene of the benchmark set; ``scene()`` builds the full case and
    ``cpu_sample()`` the bounded sample the CPU baseline steps (the full scene unless stated)."""

    def __init__(self, name, metric, desc, scene, cpu_sample=None, actuation=None, sample_desc=None, horizon=1000):
        self.name, self.metric, self.desc = name, metric, desc
        self.scene = scene
        self.horizon = horizon                # steps over which the FP32C error is reported
        self.cpu_sample = cpu_sample or scene
        self.actuation = actuation            # (amplitude, frequency) of in-step CTE actuation
        self.sample_desc = sample_desc


def workloads():
    from voxelyze_gb300 import scenes as S

    d = DIMS
    return {
        "lattice": Workload(
            "lattice", "voxel-steps/s at 1M voxels (128x128x64 multi-material lattice)",
            "lattice %dx%dx%d, fill 0.85, 4 bilinear materials, nu 0.3, gravity+floor, 1 cm" % d,
            lambda: S.lattice(*DIMS)),
        "cantilever": Workload(
            "cantilever", "voxel-steps/s (40x8x8 cantilever)",
            "cantilever 40x8x8, 5 mm, E 1 MPa, x=0 face fixed, -1 N per tip voxel", lambda: S.cantilever(40, 8, 8),
            horizon=10000),
        "porous": Workload(
            "porous", "voxel-steps/s (64^3 porous body, collisions)",
            "porous 64^3 (sigma 3, void 0.4), nu 0.35, dropped 2 voxels onto the floor, gravity, collisions, "
            "friction 1.0/0.5", lambda: S.porous(64), horizon=5000),
        "population": Workload(
            "population", "voxel-steps/s (4,096 independent bodies)",
            "4,096 bodies, sides 4..24, occupancy 0.6, passive/active CTE materials, floor+gravity, friction "
            "1.0/0.5, ambient temperature 0.1 sin(2 pi 2 t) applied inside every step",
            lambda: S.population(4096), cpu_sample=lambda: S.population(64), actuation=(0.1, 2.0),
            sample_desc="the first 64 bodies of the same generator"),
    }


def build_scene(sim_factory, sc):
    from voxelyze_gb300 import scenes as S

    sim = sim_factory(sc.voxel_size)
    S.apply(sc, sim)
    return sim


def cpu_oracle_rate(sc, threads: int, budget_s: float, steps_cap: int | None = None, actuation=None):
    """Voxel-steps/s of the oracle (C-library math, `threads` OpenMP threads) on `sc`, over exactly
    `steps_cap` steps if given, else over as many steps as fit in `budget_s` seconds; with
    `actuation` = (amplitude, frequency), setAmbientTemperature(a sin(2 pi f t), true) before each
    step, as the reference's user loop would call it."""
    import math

    from voxelyze_gb300 import facade as F, scenes as S

    lib = C.CDLL(os.path.join(ROOT, "oracle", "_build", "libvxoracle.so"))
    lib.vxo_set_math(0)
    sim = F.Sim(lib, "vxo", sc.voxel_size)
    S.apply(sc, sim)
    lib.vxo_set_threads(C.c_void_p(sim.h), threads)
    dt = sim.recommended_time_step()

    def step(k):
        if actuation:
            sim.set_ambient_temperature(float(actuation[0] * math.sin(2 * math.pi * actuation[1] * k * dt)), True)
        sim.do_time_step(dt)

    step(0)  # warm
    n, t0 = 0, time.perf_counter()
    while True:
        step(n + 1)
        n += 1
        el = time.perf_counter() - t0
        if (n >= steps_cap) if steps_cap else (el >= budget_s):
            break
    return sim.voxel_count() * n / el, n, el


def run_reference(args, world, rank):
    if rank != 0:
        return
    W = workloads()[args.workload]
    sc = W.cpu_sample()
    cores = os.cpu_count() or 1
    # warmup and timed steps, each one doTimeStep of the sample on all host cores
    cpu_oracle_rate(sc, cores, 0.0, steps_cap=max(1, args.warmup), actuation=W.actuation)
    rate, n, el = cpu_oracle_rate(sc, cores, 0.0, steps_cap=max(1, args.steps), actuation=W.actuation)
    sample = f"{n} doTimeStep calls of the {'full ' if W.sample_desc is None else ''}{W.name}"
    if W.sample_desc:
        sample += f" ({W.sample_desc}, {sc.n_voxels} voxels)"
    line = {"metric": W.metric, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": n,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / n, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": W.desc, "voxels": sc.n_voxels, "precision": "fp64 CPU, C-library math"},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def _timed(lib, sim, steps, dt, local, barrier):
    """K steps as they normally run (CUDA-graph replay), timed by one CUDA event pair on the engine
    stream around the batch; then K more steps with per-pass events (no graphs) for the per-kernel
    split.  Returns both and the clocks sampled during the first."""
    h = C.c_void_p(sim.h)
    tm = (C.c_float * 4)()
    cnt = (C.c_longlong * 8)()
    lib.vx_counters(h, cnt, 8)
    launches0 = cnt[6]
    lib.vx_enable_timing(h, 2)
    barrier()
    with _Clocks(local) as clk:
        done = sim.do_time_steps(steps, dt)
    barrier()
    if done != steps:
        raise RuntimeError(f"diverged after {done} steps")
    lib.vx_step_timing(h, tm)
    total_ms = float(tm[0])
    lib.vx_counters(h, cnt, 8)
    launches = int(cnt[6] - launches0)
    lib.vx_enable_timing(h, 1)
    if sim.do_time_steps(steps, dt) != steps:
        raise RuntimeError("diverged in the per-pass timing run")
    lib.vx_enable_timing(h, 0)
    lib.vx_step_timing(h, tm)
    _, link_ms, col_ms, vox_ms = [float(x) for x in tm]
    return {"total_ms": total_ms, "link_ms": link_ms, "collide_ms": col_ms, "voxel_ms": vox_ms, "clocks": clk.summary(),
            "launches": launches}


def run_ours(args, world, rank, local):
    import voxelyze_gb300 as vg
    from voxelyze_gb300 import facade as F, roofline as R

    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    from voxelyze_gb300.replicas import aggregate_rate, barrier

    W = workloads()[args.workload]
    lib = vg.library()
    lib.vx_step_timing.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
    sc = W.scene()
    sim64 = build_scene(vg.Sim, sc)
    sim32 = build_scene(vg.Sim, sc)
    F.Engine(sim32).set_precision(1)
    if W.actuation:
        for sim in (sim64, sim32):
            F.Engine(sim).set_actuation(F.ACT_UNIFORM, *W.actuation)
    nv, nl = sim64.voxel_count(), sim64.link_count()
    dt = sim64.recommended_time_step()
    sim32.recommended_time_step()
    # launch shapes, link-pass variant and graph length from the engine's autotuner (it restores the
    # state it stepped); untimed
    launch = {}
    for name, sim in (("fp64", sim64), ("fp32c", sim32)):
        E = F.Engine(sim)
        if not args.no_autotune:
            E.autotune(16, dt)
        blk = E.launch()
        launch[name] = {"block_link": blk[0], "block_voxel": blk[1], "graph_chunk": blk[2],
                        "link_pipeline": E.link_pipeline(), "link_split": E.link_split(),
                        "body_batch_voxels": E.body_batches()[0], "autotuned": not args.no_autotune}
    for sim in (sim64, sim32):
        if sim.do_time_steps(args.warmup, dt) != args.warmup:
            raise RuntimeError("warm-up diverged")
    head = sim32 if args.precision == "fp32c" else sim64
    other = sim64 if head is sim32 else sim32
    t_head = _timed(lib, head, args.steps, dt, local, barrier)
    t_other = _timed(lib, other, args.steps, dt, local, barrier)
    for t in (t_head, t_other):
        t["value"], _, secs = aggregate_rate(nv * args.steps, t["total_ms"] / 1e3)
        t["total_ms"] = 1e3 * secs

    # FP32C error against the FP64 path (bit-identical to the FP64 oracle), both run on to the
    # workload's horizon (1,000 steps for the lattice; the population stops at 1,000 of its 10,000)
    done = args.warmup + 2 * args.steps
    if not args.quick_error:
        more = max(0, W.horizon - done)
        for sim in (sim64, sim32):
            if more and sim.do_time_steps(more, dt) != more:
                raise RuntimeError("diverged on the way to the error horizon")
        done += more
    p64 = sim64.voxel_state()["pos"]
    p32 = sim32.voxel_state()["pos"]
    disp = p64 - sc.xyz * sc.voxel_size
    err = {"steps": done,
           "rel_pos": float(np.abs(p32 - p64).max() / np.abs(p64).max()),
           "rel_disp": float(np.abs(p32 - p64).max() / max(np.abs(disp).max(), 1e-30))}
    extra = {}
    if sc.body is not None:  # per-body centre-of-mass displacement (both precisions agree)
        off = np.concatenate([[0], np.cumsum(np.bincount(sc.body))]).astype(np.int32)
        com0 = np.stack([np.bincount(sc.body, weights=sc.xyz[:, k] * sc.voxel_size) for k in range(3)], 1)
        com0 /= np.bincount(sc.body)[:, None]
        c32, c64 = F.Engine(sim32).body_com(off), F.Engine(sim64).body_com(off)
        d32 = c32 - com0
        extra["body_com_displacement"] = {"bodies": int(len(off) - 1), "mean_dx": float(d32[:, 0].mean()),
                                          "mean_dz": float(d32[:, 2].mean()),
                                          "max_abs_fp32c_minus_fp64": float(np.abs(c32 - c64).max())}

    # ---- end to end through the public C facade ----------------------------------------------
    import torch

    h = C.c_void_p(head.h)
    if W.actuation:
        F.Engine(head).set_actuation(F.ACT_OFF)  # the host sends the temperatures instead
    temps = torch.zeros(nv, dtype=torch.float32, pin_memory=True)
    # each step's positions land in one of two pinned buffers; the copy of step k runs while step
    # k + 1 computes (vx_read_positions_async), and the clock stops after the last copy has landed
    pos = [torch.empty(3 * nv, dtype=torch.float64, pin_memory=True) for _ in range(2)]
    # raw pinned addresses (the facade binding declares typed pointers for numpy callers)
    set_temps = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)(("vx_set_temperatures", lib))
    read_pos = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)(("vx_read_positions_async", lib))
    e2e_steps = max(3, min(args.steps, 50))

    def e2e_step(k):
        if set_temps(h, temps.data_ptr()) != 0:
            raise RuntimeError("vx_set_temperatures failed")
        if lib.vx_do_time_step(h, C.c_float(dt)) != 1:
            raise RuntimeError("e2e step diverged")
        if read_pos(h, pos[k % 2].data_ptr()) != 0:
            raise RuntimeError("vx_read_positions_async failed")

    for k in range(3):  # untimed: the first single step captures its graph, the first read allocates
        e2e_step(k)
    if lib.vx_read_wait(h) != 0:
        raise RuntimeError("vx_read_wait failed")
    barrier()
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        e2e_step(k)
    if lib.vx_read_wait(h) != 0:
        raise RuntimeError("vx_read_wait failed")
    e2e_value, _, _ = aggregate_rate(nv * e2e_steps, time.perf_counter() - t0)
    barrier()
    # the last overlapped read against a synchronous one (outside the timed region)
    check = np.zeros(3 * nv, np.float64)
    if lib.vx_read_positions(h, check.ctypes.data_as(C.POINTER(C.c_double))) != 0 or \
            not np.array_equal(check, pos[(e2e_steps - 1) % 2].numpy()):
        raise RuntimeError("the overlapped position read differs from a synchronous read")

    # ---- roofline of the dominant pass of the headline precision ------------------------------
    fp32 = head is sim32
    poisson = any(m.nu != 0 for m in sc.materials)
    if fp32:  # links outside the small-angle branch also move their angle1v (counted after the run)
        large = int(nl - np.count_nonzero(head.link_state()["smallAngle"])) if nl else 0
        b = R.fp32c_bytes(nv, nl, poisson=poisson, large_angle_links=large)
    else:
        large = None
        b = R.fp64_bytes(nv, nl, poisson=poisson)
    kernel = "link" if t_head["link_ms"] >= t_head["voxel_ms"] else "voxel"
    k_ms = t_head[f"{kernel}_ms"]
    achieved = b[kernel] / (k_ms / 1e3) / 1e9
    peak, peak_kind = _peak_hbm()
    kname = f"k_{kernel}{'32' if fp32 else ''}"
    label = f"k_poisson + {kname}" if (kernel == "link" and not fp32 and poisson) else kname
    traffic = R.measured_traffic(f"{'fp32c' if fp32 else 'fp64'}_{kernel}", nv, nl) \
        if args.workload == "lattice" else None
    roof = {"bound": "hbm", "kernel": f"{label} ({'FP32C' if fp32 else 'FP64'} {kernel} pass)", "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": b[kernel], "ms_per_launch": k_ms, "traffic": traffic,
            "step_bytes": b["step"], "step_frac": b["step"] / (t_head["total_ms"] / args.steps / 1e3) / 1e9 / peak,
            "large_angle_links": large,
            # both passes of the step against the same peak (CUDA events around each pass)
            "per_kernel": [{"kernel": f"k_{k}{'32' if fp32 else ''}", "algorithmic_bytes_per_launch": b[k],
                            "ms_per_launch": t_head[f"{k}_ms"],
                            "achieved": b[k] / (t_head[f"{k}_ms"] / 1e3) / 1e9,
                            "frac": b[k] / (t_head[f"{k}_ms"] / 1e3) / 1e9 / peak}
                           for k in ("link", "voxel") if t_head[f"{k}_ms"] > 0]}

    # FP64 path against the FP64 pipe: its link pass issues double operations, not bytes, at the
    # rate that bounds it.  Instructions per link counted by ncu on the same generator (roofline.py),
    # peak measured here by vxg_probe_fp64_rate.
    o64 = t_other if fp32 else t_head
    fp64_roof = None
    fma_s, probe_ms = C.c_double(0), C.c_float(0)
    lib.vxg_probe_fp64_rate.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_float)]
    if lib.vxg_probe_fp64_rate(0, 4096, C.byref(fma_s), C.byref(probe_ms)) == 0 and fma_s.value > 0:
        f = R.fp64_ops(nv, nl, poisson=poisson)
        if f is not None and o64["link_ms"] > 0:
            ach = f["link_flops"] / (o64["link_ms"] / 1e3) / 1e9
            ach_i = f["link_pipe_inst"] / (o64["link_ms"] / 1e3) / 1e9
            peak_flops = 2 * fma_s.value / 1e9
            peak_inst = fma_s.value / 32 / 1e9  # warp instructions
            fp64_roof = {"bound": "fp64", "kernel": "k_link (FP64 link pass)", "achieved": ach, "peak": peak_flops,
                         "unit": "GFLOP/s", "frac": ach / peak_flops,
                         "pipe_inst_per_s": {"achieved": 1e9 * ach_i, "peak": 1e9 * peak_inst,
                                             "frac": ach_i / peak_inst},
                         "flops_per_launch": f["link_flops"], "ms_per_launch": o64["link_ms"],
                         "peak_source": "measured: vxg_probe_fp64_rate (fma.rn.f64 chains on every SM, "
                                        "%.3f ms best of 5)" % probe_ms.value,
                         "counts": "ncu instruction counts per link, roofline.FP64_OPS"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        cs = W.cpu_sample()
        rate, n, el = cpu_oracle_rate(cs, cores, args.cpu_seconds, actuation=W.actuation)
        what = "the full scene" if W.sample_desc is None else f"{W.sample_desc}, {cs.n_voxels} voxels"
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"{n} doTimeStep calls of {what} in {el:.1f} s (OpenMP, C-library math)"}
        # the serial build beside it (the reference's default build has no OpenMP)
        srate, sn, sel = cpu_oracle_rate(cs, 1, max(2.0, args.cpu_seconds / 3), actuation=W.actuation)
        cpu["serial"] = {"value": srate, "unit": UNIT, "cores": 1,
                         "sample": f"{sn} doTimeStep calls of {what} in {sel:.1f} s (one thread)"}

    o = t_other
    line = {"metric": W.metric, "value": t_head["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_head["total_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if fp32 else "f64", "data": "synthetic",
            "config": {"workload": W.desc, "voxels": nv, "links": nl, "precision": args.precision,
                       "parallelism": f"replicas x{world}",
                       "l2": "state > 129 MB L2, no flush" if nv >= 500000 else
                             "state partly L2-resident (small scene), no flush",
                       "dt": dt,
                       "per_pass_ms": {"link": t_head["link_ms"], "collide": t_head["collide_ms"],
                                       "voxel": t_head["voxel_ms"]},
                       "other_precision": {"precision": "fp64" if fp32 else "fp32c", "value": o["value"],
                                           "ms_per_step": o["total_ms"] / args.steps,
                                           "per_pass_ms": {"link": o["link_ms"], "collide": o["collide_ms"],
                                                           "voxel": o["voxel_ms"]}},
                       "launch": launch,
                       "fp32c_over_fp64": (t_head["value"] / o["value"]) if fp32 else (o["value"] / t_head["value"]),
                       "fp32c_error_vs_fp64": err, **extra},
            "roofline": roof, "roofline_fp64": fp64_roof, "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 4 * nv, "d2h_bytes_per_step": 24 * nv,
                    "steps": e2e_steps,
                    "path": "vx_set_temperatures (pinned) + vx_do_time_step + vx_read_positions_async (two pinned "
                            "buffers; step k's copy overlaps step k+1), vx_read_wait before the clock stops"},
            "clocks": t_head["clocks"], "gpu_launches": t_head["launches"]}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def run_adjoint(args, world, rank, local):
    """The gradient workload (256 bodies of 16^3 cells): reverse-mode gradient of the per-body
    centre-of-mass x after 2,000 steps with
    respect to every voxel's E, density and actuation phase (FP64 path, checkpoints every 100
    steps), timed; then checked against central differences on 64 random parameters."""
    import voxelyze_gb300 as vg
    from voxelyze_gb300 import gradcheck as G, scenes as S

    if rank != 0:
        return
    lib = vg.library()
    nsteps, K = 2000, 100
    sc = S.graded_population(256, 16, 0.7)
    off = G.body_offsets(sc)
    rng = np.random.default_rng(7)
    bodies = rng.choice(len(off) - 1, size=64, replace=False)
    pick = [(int(b), int(rng.integers(off[b], off[b + 1])), "E" if i % 2 == 0 else "phase")
            for i, b in enumerate(bodies)]
    ad, obj, t_adj, dt, dec = G.adjoint(lib, sc, nsteps, K, pick)
    rows = G.differences(lib, sc, pick, nsteps, dt, ad, 1e-3, 1e-2)
    # the same parameters with the plain run's contact and friction decisions replayed, wider steps,
    # Richardson-extrapolated
    frozen = G.differences(lib, sc, pick, nsteps, dt, ad, 1.6e-2, 0.16, decisions=dec)
    fe = np.array([r["richardson_error"] for r in frozen])
    # the same comparison as vectors, per kind: |ad - fd| over |fd| in the 2-norm and in the max-norm
    by_kind = {}
    for kind in ("E", "phase"):
        idx = [i for i, p in enumerate(pick) if p[2] == kind]
        a = np.array([frozen[i]["adjoint"] for i in idx])
        f = np.array([frozen[i]["richardson"] for i in idx])
        by_kind[kind] = {"parameters": len(idx), "rel_l2": float(np.linalg.norm(a - f) / np.linalg.norm(f)),
                         "rel_max": float(np.abs(a - f).max() / np.abs(f).max())}
    # the four worst parameters: their frozen-decision differences at four step sizes, to show
    # whether the differences themselves have settled to the adjoint's precision
    worst = sorted(range(len(frozen)), key=lambda i: -frozen[i]["richardson_error"])[:4]
    wpick = [pick[i] for i in worst]
    seq = [G.central_differences(lib, sc, wpick, nsteps, dt, off, 1.6e-2 / 2 ** k, 0.16 / 2 ** k, 0.1, 2.0, dec)
           for k in range(4)]
    worst_rows = [{"kind": wpick[j][2], "adjoint": float(frozen[i]["adjoint"]),
                   "richardson_error": float(frozen[i]["richardson_error"]),
                   "fd_h_h2_h4_h8": [float(seq[k][j]) for k in range(4)]} for j, i in enumerate(worst)]
    sim, _ = G.build(lib, sc, sc.phase, 0.1, 2.0)
    sim.recommended_time_step()
    t0 = time.perf_counter()
    sim.do_time_steps(nsteps, dt)
    t_fwd = time.perf_counter() - t0
    nv = sim.voxel_count()
    d = np.array([r["distance"] for r in rows if r["smooth"]])
    cpu = None
    if not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        sample = S.graded_population(4, 16, 0.7)
        rate, n, el = cpu_oracle_rate(sample, cores, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"forward doTimeStep of 4 bodies ({sample.n_voxels} voxels), {n} steps in {el:.1f} s; "
                         "the reference has no gradient: finite differences cost 2 such runs per parameter"}
    line = {"metric": "adjoint voxel-steps/s (256 bodies of 16^3, d centre-of-mass x / d per-voxel E, rho, phase)",
            "value": nv * nsteps / t_adj, "unit": UNIT, "n_gpus": 1, "steps": nsteps, "warmup": 0,
            "ms_per_step": 1e3 * t_adj / nsteps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "256 bodies of 16^3 cells (occupancy 0.7), one material per voxel, E log-uniform "
                                   "3e5..3e6 Pa, CTE 0.01, per-voxel phase, floor+friction+gravity, 2,000 steps, "
                                   "checkpoint every 100", "voxels": nv,
                       "forward_voxel_steps_per_s": nv * nsteps / t_fwd, "adjoint_over_forward_time": t_adj / t_fwd,
                       "gradient_check": {"parameters": len(rows), "smooth": int(len(d)),
                                          "fd_steps": "1e-3 relative (E), 1e-2 rad (phase), and a quarter of each",
                                          "distance_median": float(np.median(d)),
                                          "distance_p90": float(np.percentile(d, 90)),
                                          "distance_max": float(d.max()),
                                          "within_1e-4": float(np.mean(d <= 1e-4))},
                       "gradient_check_frozen_decisions": {
                           "parameters": len(frozen),
                           "fd_steps": "1.6e-2 relative (E), 0.16 rad (phase), and a quarter of each, with the "
                                       "plain run's floor-contact and static-friction decisions replayed; "
                                       "Richardson-extrapolated",
                           "error_median": float(np.median(fe)), "error_p90": float(np.percentile(fe, 90)),
                           "error_max": float(fe.max()), "within_1e-4": float(np.mean(fe <= 1e-4)),
                           "within_1e-3": float(np.mean(fe <= 1e-3)),
                           "as_vectors": by_kind, "worst": worst_rows}},
            "cpu_baseline": cpu, "timing": "host wall clock around vxg_adjoint_com_x (synchronous)"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32c", choices=["fp64", "fp32c"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the engine's default launch shapes")
    ap.add_argument("--quick-error", action="store_true",
                    help="report the FP32C error where the timed steps end, not at the workload's horizon")
    ap.add_argument("--dims", default="128,128,64", help="lattice size (smaller cases for profiling)")
    ap.add_argument("--workload", default="lattice",
                    choices=["lattice", "cantilever", "porous", "population", "adjoint"],
                    help="lattice (the headline), cantilever, porous (collisions), population (4,096 bodies), "
                         "adjoint (256 bodies, gradients checked against finite differences)")
    args = ap.parse_args()
    global DIMS
    DIMS = tuple(int(x) for x in args.dims.split(","))
    world, rank, local = _dist()
    if args.workload == "adjoint":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the reference has no gradient of the time step"}))
        else:
            run_adjoint(args, world, rank, local)
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
