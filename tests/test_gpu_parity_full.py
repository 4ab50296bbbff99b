"""FP64 GPU path against the oracle at the benchmark configurations' full sizes and horizons.

* Multi-material lattice 128x128x64 (0.89 M voxels, 2.25 M links), 1,000 steps: bit-identical to
  the oracle in its correctly rounded mode at steps 250, 500 and 1,000; against the oracle with the
  C library's sin/cos/acos (the reference's own arithmetic) every position and orientation within
  1e-10 relative.
* Porous 64^3 body with collisions (157,219 voxels), dropped onto the floor: the collision pair list
  identical to the oracle's at every rebuild, and the whole state at checkpoints; the same generator
  at 32^3 bit-identical over the full 5,000-step horizon.
* 64 bodies of the 4,096-body population (the generator's first 64, sides 4..24, in-step CTE
  actuation, floor and friction), 10,000 steps: bit-identical at four checkpoints.
* Cantilever 40x8x8: the error against the C-library oracle at 1,000 and 10,000 steps, reported.

The oracle runs with one OpenMP thread per host core (its threaded step is bit-identical to its
serial step).  Reference behaviour followed: src/Voxelyze.cpp:251-284 (doTimeStep), :670-750
(collisions).
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np
import pytest

from conftest import make_sim, max_rel_pos_err, state_diff
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu

THREADS = max(1, os.cpu_count() or 1)
TWO_PI = 2.0 * 3.141592653589793


def _sim_pair(product_lib, oracle_lib, sc):
    g = make_sim(product_lib, "vx", sc)
    o = make_sim(oracle_lib, "vxo", sc)
    oracle_lib.vxo_set_threads(C.c_void_p(o.h), THREADS)
    return g, o


def _orient_err(a, b):
    return float(np.abs(a.voxel_state()["orient"] - b.voxel_state()["orient"]).max())


def test_lattice_full_size_full_horizon(product_lib, oracle_lib):
    sc = S.lattice(128, 128, 64)
    oracle_lib.vxo_set_math(1)
    try:
        g, o = _sim_pair(product_lib, oracle_lib, sc)
        dt = o.recommended_time_step()
        assert g.recommended_time_step() == dt
        t0 = time.perf_counter()
        done = 0
        for upto in (250, 500, 1000):
            n = upto - done
            assert g.do_time_steps(n, dt) == o.do_time_steps(n, dt) == n
            done = upto
            assert state_diff(g, o) == [], f"state differs after {done} steps"
        t_cr = time.perf_counter() - t0
    finally:
        oracle_lib.vxo_set_math(0)
    del o
    c = make_sim(oracle_lib, "vxo", sc)  # C-library math (mode 0)
    oracle_lib.vxo_set_threads(C.c_void_p(c.h), THREADS)
    t0 = time.perf_counter()
    assert c.do_time_steps(1000, dt) == 1000
    err_pos, err_q = max_rel_pos_err(g, c), _orient_err(g, c)
    print(f"lattice 128x128x64, 1000 steps: bit-identical to the correctly rounded oracle ({t_cr:.0f} s); "
          f"against the C-library oracle max rel position error {err_pos:.3e}, max orientation "
          f"difference {err_q:.3e} ({time.perf_counter() - t0:.0f} s)")
    assert err_pos <= 1e-10 and err_q <= 1e-10


def _pairs_at_rebuilds(product_lib, oracle_lib, sc, steps, check_every):
    oracle_lib.vxo_set_math(1)
    try:
        g, o = _sim_pair(product_lib, oracle_lib, sc)
        dt = o.recommended_time_step()
        assert g.recommended_time_step() == dt
        cnt = (C.c_longlong * 8)()
        rebuilds = compared = 0
        max_pairs = 0
        for s in range(1, steps + 1):
            assert g.do_time_step(dt) and o.do_time_step(dt)
            product_lib.vx_counters(C.c_void_p(g.h), cnt, 8)
            if cnt[4] != rebuilds:  # VXG_C_REBUILDS: the GPU rebuilt its pair list in this step
                rebuilds = cnt[4]
                pg, po = g.collisions(), o.collisions()
                assert np.array_equal(pg, po), f"pair list differs at the rebuild in step {s}"
                compared += 1
                max_pairs = max(max_pairs, len(pg))
            if s % check_every == 0 or s == steps:
                assert state_diff(g, o) == [], f"state differs after {s} steps"
        return rebuilds, compared, max_pairs, g
    finally:
        oracle_lib.vxo_set_math(0)


def test_porous_full_size_full_horizon(product_lib, oracle_lib):
    """The porous 64^3 collision body at full size over its 5,000-step horizon: every rebuild (the body falls, its surface
    voxels drift past the watch distance, it lands) compared pair for pair, the state every 500."""
    rebuilds, compared, max_pairs, g = _pairs_at_rebuilds(product_lib, oracle_lib, S.porous(64), 5000, 500)
    zmin = float(g.voxel_state()["pos"][:, 2].min())
    print(f"porous 64^3: {compared} rebuilds compared over 5000 steps, up to {max_pairs} pairs, lowest z {zmin:.4f}")
    assert compared >= 2 and compared == rebuilds


def test_porous_reduced_full_horizon(product_lib, oracle_lib):
    """The porous collision generator at 32^3 over the full 5,000-step horizon: the drop, the impact and the
    contacts; pair lists at every rebuild and the state every 500 steps."""
    rebuilds, compared, max_pairs, g = _pairs_at_rebuilds(product_lib, oracle_lib, S.porous(32), 5000, 500)
    zmin = float(g.voxel_state()["pos"][:, 2].min())
    print(f"porous 32^3: {compared} rebuilds over 5000 steps, up to {max_pairs} pairs, lowest z {zmin:.4f}")
    assert compared >= 2 and max_pairs > 0


def _cr_sin(lib, x: float) -> float:
    xi = np.array([x], np.float64)
    yo = np.zeros(1, np.float64)
    lib.vxo_crmath_eval(0, 1, xi.ctypes.data_as(C.c_void_p), yo.ctypes.data_as(C.c_void_p), None)
    return float(yo[0])


def test_population_sample_full_horizon(product_lib, oracle_lib):
    """The first 64 bodies of the 4,096-body population, 10,000 steps with the ambient temperature
    0.1 sin(2 pi 2 t) set before every step (the GPU applies it inside the step)."""
    sc = S.population(64)
    oracle_lib.vxo_set_math(1)
    try:
        g, o = _sim_pair(product_lib, oracle_lib, sc)
        dt = o.recommended_time_step()
        assert g.recommended_time_step() == dt
        F.Engine(g).set_actuation(F.ACT_UNIFORM, 0.1, 2.0)
        done = 0
        for upto in (2500, 5000, 7500, 10000):
            assert g.do_time_steps(upto - done, dt) == upto - done
            for _ in range(upto - done):
                t = float(o.current_time())
                o.set_ambient_temperature(float(np.float32(0.1 * _cr_sin(oracle_lib, TWO_PI * 2.0 * t))), True)
                assert o.do_time_step(dt)
            done = upto
            assert state_diff(g, o) == [], f"state differs after {done} steps"
    finally:
        oracle_lib.vxo_set_math(0)


def test_cantilever_error_against_c_library(product_lib, oracle_lib):
    """The 40x8x8 cantilever against the reference's own arithmetic (C-library sin/cos/acos): the error at 1,000
    and 10,000 steps, reported (the GPU is bit-identical to the correctly rounded oracle over the
    whole horizon, test_gpu_parity.py)."""
    oracle_lib.vxo_set_math(0)
    sc = S.cantilever(40, 8, 8)
    g = make_sim(product_lib, "vx", sc)
    o = make_sim(oracle_lib, "vxo", sc)
    dt = o.recommended_time_step()
    out = {}
    done = 0
    for upto in (1000, 10000):
        assert g.do_time_steps(upto - done, dt) == o.do_time_steps(upto - done, dt) == upto - done
        done = upto
        out[upto] = (max_rel_pos_err(g, o), _orient_err(g, o))
    print("cantilever 40x8x8 vs C-library oracle: " +
          ", ".join(f"{k} steps: rel pos {v[0]:.3e}, orient {v[1]:.3e}" for k, v in out.items()))
    assert all(np.isfinite(v[0]) for v in out.values())
