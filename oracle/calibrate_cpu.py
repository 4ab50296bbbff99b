"""Times the oracle's CPU time step against the reference's own USE_OMP build on the same scene.

Test infrastructure: bench.py's CPU baseline and its reference arm time the oracle (the reference's
sources are not on the GPU host), so this script, run where the reference build exists
(oracle/_ref, made by oracle/build_ref.sh), records how the two compare on this machine's cores.

    python oracle/calibrate_cpu.py [--dims 128,128,64] [--steps 20]

Both run the bench's lattice generator with C-library math; the oracle with one OpenMP thread per
core (vxo_set_threads), the reference with OMP_NUM_THREADS set to the same count before it loads.
The single-thread rates of the oracle and of the reference's serial build are timed beside them.
Prints one Markdown table row per build.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _rate(lib, prefix, sc, steps, threads=None):
    from voxelyze_gb300 import facade as F, scenes as S

    sim = F.Sim(lib, prefix, sc.voxel_size)
    S.apply(sc, sim)
    if threads is not None:
        lib.vxo_set_threads(C.c_void_p(sim.h), threads)
    dt = sim.recommended_time_step()
    sim.do_time_steps(2, dt)  # warm
    t0 = time.perf_counter()
    assert sim.do_time_steps(steps, dt) == steps
    el = time.perf_counter() - t0
    return sc.n_voxels * steps / el, el


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--dims", default="128,128,64")
    ap.add_argument("--steps", type=int, default=20)
    args = ap.parse_args()
    cores = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(cores)  # read by the reference's OpenMP runtime at load
    from voxelyze_gb300 import scenes as S

    sc = S.lattice(*(int(x) for x in args.dims.split(",")))
    oracle = C.CDLL(os.path.join(ROOT, "oracle", "_build", "libvxoracle.so"))
    oracle.vxo_set_math(0)
    oracle.vxo_set_threads.argtypes = [C.c_void_p, C.c_int]
    ref_omp = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvxref_omp.so"))
    ref = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvxref.so"))
    rows = [("oracle (vx_oracle.cpp, -O2, OpenMP)", cores, *_rate(oracle, "vxo", sc, args.steps, cores)),
            ("reference USE_OMP build (-O3 -fopenmp -DUSE_OMP)", cores, *_rate(ref_omp, "vxr", sc, args.steps)),
            ("oracle, one thread", 1, *_rate(oracle, "vxo", sc, max(2, args.steps // 4), 1)),
            ("reference serial build (-O3)", 1, *_rate(ref, "vxr", sc, max(2, args.steps // 4)))]
    print(f"lattice {args.dims} ({sc.n_voxels} voxels), {cores} host cores")
    print("| build | threads | voxel-steps/s | seconds |")
    print("|---|---:|---:|---:|")
    for name, th, rate, el in rows:
        print(f"| {name} | {th} | {rate:.3e} | {el:.1f} |")


if __name__ == "__main__":
    main()
