"""Host edits between steps, the reference's way: per-voxel CVX_Voxel::setTemperature
and CVX_External setters called between doTimeStep calls (src/VX_Voxel.cpp:108-114,
include/VX_External.h:39-90).  While the device holds the newer state the product queues the
temperatures and applies them on the device before the next step or host read, and uploads only
the externals table when existing externals change.  Checked bit for bit against the oracle
driven by the same calls, in both orders of edits and reads.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import make_sim, state_diff
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture()
def cr_oracle(oracle_lib):
    oracle_lib.vxo_set_math(1)
    yield oracle_lib
    oracle_lib.vxo_set_math(0)


def _pair(product_lib, oracle, sc):
    return make_sim(product_lib, "vx", sc), make_sim(oracle, "vxo", sc)


@pytest.mark.parametrize("precision", [0, 1])
def test_per_voxel_temperature_every_step(product_lib, cr_oracle, precision):
    """Every voxel's temperature set through setTemperature before each step (a phase-shifted
    CTE actuation), with a temperature read in the middle of the run: FP64 identical to the
    oracle bit for bit; FP32C with the same temperatures and positions within 1e-6."""
    sc = S.population(6, 3, 6)
    g, o = _pair(product_lib, cr_oracle, sc)
    F.Engine(g).set_precision(precision)
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == pytest.approx(dt, rel=0 if precision == 0 else 1e-6)
    rng = np.random.default_rng(3)
    phase = rng.uniform(0, 2 * np.pi, g.voxel_count())
    nv = g.voxel_count()
    for k in range(40):
        temps = (0.1 * np.sin(2 * np.pi * 2.0 * k * dt + phase)).astype(np.float32)
        for v in range(nv):
            g.set_temperature(v, float(temps[v]))
            o.set_temperature(v, float(temps[v]))
        if k == 20:  # a host read between the edits and the step applies them first
            assert g.voxel_state()["temp"][5] == temps[5]
        assert g.do_time_step(dt) and o.do_time_step(dt)
    if precision == 0:
        assert state_diff(g, o) == []
    else:
        pa, pb = g.voxel_state()["pos"], o.voxel_state()["pos"]
        assert np.abs(pa - pb).max() / np.abs(pb).max() <= 1e-6
        assert np.array_equal(g.voxel_state()["temp"], o.voxel_state()["temp"])


def test_external_edits_every_step(product_lib, cr_oracle):
    """Forces and moments of existing externals changed before every step (the externals-table
    upload), then a new external and a prescribed displacement mid-run (the full table path)."""
    sc = S.cantilever(10, 3, 3, voxel_size=0.005, tip_force=-0.01)
    g, o = _pair(product_lib, cr_oracle, sc)
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    tip = [int(v) for v in sc.force_idx]
    for k in range(60):
        for s in (g, o):
            for j, v in enumerate(tip):
                s.set_force(v, 0.001 * np.sin(0.1 * k + j), 0.0, -0.01 * (1 + 0.5 * np.cos(0.05 * k)))
                s.set_moment(v, 0.0, 1e-5 * k, 0.0)
            if k == 30:
                s.set_force(40, 0.0, 0.002, 0.0)              # voxel 40 had no external
                s.set_displacement(1, F.Z_TRANSLATE, 1e-4)    # voxel 1 is fixed: prescribe a shift
        assert g.do_time_step(dt) and o.do_time_step(dt)
    assert state_diff(g, o) == []


def test_queued_temperatures_around_ambient_temperature(product_lib, cr_oracle):
    """Queued per-voxel temperatures, then setAmbientTemperature(T, true) (applied on the device),
    then more queued ones and a new external: every edit lands in call order."""
    sc = S.population(4, 3, 5)
    g, o = _pair(product_lib, cr_oracle, sc)
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    for s in (g, o):
        assert s.do_time_steps(10, dt) == 10
        for v in range(0, s.voxel_count(), 3):
            s.set_temperature(v, 0.05)
        assert s.do_time_steps(5, dt) == 5
        for v in range(0, s.voxel_count(), 2):
            s.set_temperature(v, -0.03)
        s.set_ambient_temperature(0.02, True)
        for v in range(1, s.voxel_count(), 4):
            s.set_temperature(v, 0.07)
        s.set_force(3, 0.0, 0.0, -0.001)
        assert s.do_time_steps(10, dt) == 10
    assert state_diff(g, o) == []


@pytest.mark.parametrize("batch", [1, 7])
def test_fp32c_temperatures_rest_lengths_in_the_link_pass(product_lib, batch):
    """FP32C: the rest lengths of temperatures set with vx_set_temperatures are recomputed by the
    next step's link pass when that step is launched on its own (batch 1), and by a rest-length pass
    otherwise (a captured batch of 7), always as CVX_Voxel::setTemperature leaves them
    (src/VX_Voxel.cpp:108-114, src/VX_Link.cpp:137-140).  Against a twin whose rest lengths are read
    back (which brings them up to date) before every batch, the whole state is identical bit for
    bit after every batch; a Poisson-ratio lattice covers the Poisson branch of the link pass."""
    import ctypes as C

    from conftest import state_diff

    sc = S.lattice(14, 10, 8)
    a = make_sim(product_lib, "vx", sc)
    b = make_sim(product_lib, "vx", sc)
    for s in (a, b):
        F.Engine(s).set_precision(1)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    st = product_lib.vx_set_temperatures
    st.argtypes = [C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(11)
    nv = a.voxel_count()
    for k in range(6):
        temps = np.ascontiguousarray(rng.uniform(-0.5, 0.5, nv).astype(np.float32))
        for s in (a, b):
            assert st(C.c_void_p(s.h), temps.ctypes.data) == 0
        b.link_state()  # reads the rest lengths: the separate rest-length pass runs first
        assert a.do_time_steps(batch, dt) == b.do_time_steps(batch, dt) == batch
        assert state_diff(a, b) == [], f"after batch {k}"
