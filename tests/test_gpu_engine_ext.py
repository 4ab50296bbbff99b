"""Engine extensions on the GPU: per-step actuation inside the step, body centres of mass, device
snapshots, launch shapes and the autotuner.

Actuation is checked bit for bit against the oracle driven the reference's way - the temperature
set by setAmbientTemperature(T, true) / CVX_Voxel::setTemperature before every doTimeStep
(Voxelyze.cpp:585-594, VX_Voxel.cpp:108-114), T = amplitude * sin(2 pi frequency t + phase) with
t = currentTime() at the step start, the sine correctly rounded as on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import make_sim, state_diff
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu

TWO_PI = 2.0 * 3.141592653589793


@pytest.fixture()
def cr_oracle(oracle_lib):
    oracle_lib.vxo_set_math(1)
    yield oracle_lib
    oracle_lib.vxo_set_math(0)


def _cr_sin(lib, x: float) -> float:
    xi = np.array([x], np.float64)
    yo = np.zeros(1, np.float64)
    lib.vxo_crmath_eval(0, 1, xi.ctypes.data_as(C.c_void_p), yo.ctypes.data_as(C.c_void_p), None)
    return float(yo[0])


def _oracle_actuated_steps(o, lib, n, dt, amp, freq, phase=None):
    for _ in range(n):
        t = float(o.current_time())
        if phase is None:
            temp = float(np.float32(amp * _cr_sin(lib, TWO_PI * freq * t)))
            o.set_ambient_temperature(temp, True)
        else:
            for v in range(o.voxel_count()):
                temp = float(np.float32(amp * _cr_sin(lib, TWO_PI * freq * t + float(phase[v]))))
                o.set_temperature(v, temp)
        assert o.do_time_step(dt)


def test_uniform_actuation_matches_reference_loop(product_lib, cr_oracle):
    sc = S.population(4, 3, 5)
    g = make_sim(product_lib, "vx", sc)
    o = make_sim(cr_oracle, "vxo", sc)
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    E = F.Engine(g)
    E.set_actuation(F.ACT_UNIFORM, 0.2, 40.0)
    for n in (1, 70, 130):  # single step, chunk-graph run (64-step graphs) with a remainder
        assert g.do_time_steps(n, dt) == n
        _oracle_actuated_steps(o, cr_oracle, n, dt, 0.2, 40.0)
        assert state_diff(g, o) == [], f"after {n}-step batch"


def test_per_voxel_actuation_matches_reference_loop(product_lib, cr_oracle):
    sc = S.population(3, 3, 4)
    g = make_sim(product_lib, "vx", sc)
    o = make_sim(cr_oracle, "vxo", sc)
    dt = o.recommended_time_step()
    g.recommended_time_step()
    rng = np.random.default_rng(5)
    phase = rng.uniform(0, 2 * np.pi, g.voxel_count()).astype(np.float32)
    F.Engine(g).set_actuation(F.ACT_PER_VOXEL, 0.15, 25.0, phase)
    assert g.do_time_steps(90, dt) == 90
    _oracle_actuated_steps(o, cr_oracle, 90, dt, 0.15, 25.0, phase)
    assert state_diff(g, o) == []


def test_actuation_temperatures_at_scale(product_lib):
    """FP64 per-voxel actuation on ~1.5 million voxels for 6 steps: every temperature equals
    (float)(amplitude * sin(2 pi f t + phase)) with the C library's sine (numpy), so the fast sine
    with its rounding test and the correctly rounded fallback give the reference's floats."""
    sc = S.population(1024, 3, 24, seed=4)
    g = make_sim(product_lib, "vx", sc)
    dt = g.recommended_time_step()
    rng = np.random.default_rng(9)
    phase = rng.uniform(0, 2 * np.pi, g.voxel_count()).astype(np.float32)
    amp, freq = 0.15, 25.0
    F.Engine(g).set_actuation(F.ACT_PER_VOXEL, amp, freq, phase)
    t = np.float32(0.0)
    for _ in range(6):
        assert g.do_time_steps(1, dt) == 1
        temp = g.voxel_state()["temp"].astype(np.float32)
        arg = 2.0 * 3.141592653589793 * freq * np.float64(t) + phase.astype(np.float64)
        want = (amp * np.sin(arg)).astype(np.float32)
        assert np.array_equal(temp, want), int((temp != want).sum())
        t = np.float32(t + np.float32(dt))
    print(f"{g.voxel_count()} voxels x 6 steps of actuation temperatures equal the C library's")


def test_actuation_fp32c_tracks_fp64(product_lib):
    sc = S.population(8, 3, 6)
    for m in sc.materials:
        m.mu_static = m.mu_kinetic = 0.0
    a = make_sim(product_lib, "vx", sc)
    b = make_sim(product_lib, "vx", sc)
    Eb = F.Engine(b)
    Eb.set_precision(1)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    for e in (F.Engine(a), Eb):
        e.set_actuation(F.ACT_UNIFORM, 0.1, 20.0)
    assert a.do_time_steps(400, dt) == 400
    assert b.do_time_steps(400, dt) == 400
    pa, pb = a.voxel_state()["pos"], b.voxel_state()["pos"]
    rel = float(np.abs(pa - pb).max() / np.abs(pa).max())
    print(f"population 8 bodies, in-step actuation, 400 steps: FP32C rel pos err {rel:.3e}")
    assert rel <= 1e-6
    assert np.allclose(a.voxel_state()["temp"], b.voxel_state()["temp"], atol=1e-6)


@pytest.mark.parametrize("precision", [0, 1])
def test_body_com(product_lib, precision):
    sc = S.population(6, 3, 5)
    g = make_sim(product_lib, "vx", sc)
    E = F.Engine(g)
    E.set_precision(precision)
    g.do_time_steps(150, g.recommended_time_step())
    body = sc.body
    order = np.argsort(body, kind="stable")
    assert np.array_equal(order, np.arange(len(body))), "population bodies are contiguous voxel ranges"
    off = np.concatenate([[0], np.cumsum(np.bincount(body))]).astype(np.int32)
    com = E.body_com(off)
    st = g.voxel_state()
    mass = np.array([np.float32(sc.materials[m].rho * sc.voxel_size ** 3) for m in sc.mats], np.float64)
    for b in range(len(off) - 1):
        sl = slice(off[b], off[b + 1])
        want = (st["pos"][sl] * mass[sl, None]).sum(0) / mass[sl].sum()
        assert np.allclose(com[b], want, rtol=1e-6, atol=1e-9), (b, com[b], want)


def test_snapshot_restore_replays_exactly(product_lib):
    sc = S.porous(12, sigma=1.5)
    g = make_sim(product_lib, "vx", sc)
    E = F.Engine(g)
    dt = g.recommended_time_step()
    g.do_time_steps(40, dt)
    E.snapshot(3)
    g.do_time_steps(80, dt)
    first = g.voxel_state()["raw_d"].copy(), g.link_state()["raw_d"].copy(), g.collisions().copy(), g.current_time()
    E.restore(3)
    g.do_time_steps(80, dt)
    second = g.voxel_state()["raw_d"], g.link_state()["raw_d"], g.collisions(), g.current_time()
    for x, y in zip(first, second):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("shape", [(64, 512, 8), (512, 64, 2), (128, 128, 256)])
def test_launch_shapes_do_not_change_results(product_lib, shape):
    sc = S.lattice(14, 12, 8)
    a = make_sim(product_lib, "vx", sc)
    b = make_sim(product_lib, "vx", sc)
    F.Engine(b).set_launch(*shape)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    assert a.do_time_steps(300, dt) == b.do_time_steps(300, dt) == 300
    assert state_diff(a, b) == []


def test_autotune_leaves_state_unchanged(product_lib):
    sc = S.lattice(24, 24, 12)
    a = make_sim(product_lib, "vx", sc)
    b = make_sim(product_lib, "vx", sc)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    a.do_time_steps(20, dt)
    b.do_time_steps(20, dt)
    best = F.Engine(b).autotune(8, dt)
    assert best[0] in (64, 128, 256, 512) and best[1] in (64, 128, 256, 512) and best[2] % 2 == 0
    assert state_diff(a, b) == []
    assert a.do_time_steps(100, dt) == b.do_time_steps(100, dt) == 100
    assert state_diff(a, b) == []
