"""Degenerate scenes on the GPU against the oracle: no voxels, one voxel (no links, so the dt comes
from recommendedTimeStep's per-voxel fallback, src/Voxelyze.cpp:302-307), two voxels, and a scene
emptied by removing its voxels; in both precisions, batched and single steps."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import state_diff
from voxelyze_gb300 import facade as F

pytestmark = pytest.mark.gpu


@pytest.fixture()
def cr_oracle(oracle_lib):
    oracle_lib.vxo_set_math(1)
    yield oracle_lib
    oracle_lib.vxo_set_math(0)


def _both(product_lib, oracle, voxels, precision=0, gravity=True):
    out = []
    for lib, pre in ((product_lib, "vx"), (oracle, "vxo")):
        s = F.Sim(lib, pre, 0.01)
        m = s.add_material(1e6, 1000.0)
        if gravity:
            s.set_gravity(1.0)
            s.enable_floor(True)
        for xyz in voxels:
            s.set_voxel(m, *xyz)
        if pre == "vx":
            F.Engine(s).set_precision(precision)
        out.append(s)
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_empty_scene(product_lib, cr_oracle, precision):
    g, o = _both(product_lib, cr_oracle, [], precision)
    assert g.recommended_time_step() == o.recommended_time_step() == 0.0
    assert g.do_time_step(-1.0) and o.do_time_step(-1.0)
    assert g.do_time_steps(10, 1e-4) == o.do_time_steps(10, 1e-4) == 10
    assert g.voxel_count() == 0 and g.link_count() == 0


@pytest.mark.parametrize("precision", [0, 1])
def test_single_voxel_falls_to_the_floor(product_lib, cr_oracle, precision):
    g, o = _both(product_lib, cr_oracle, [(0, 0, 1)], precision)  # 1 cm up: lands after ~900 steps
    dt = o.recommended_time_step()
    assert dt > 0 and g.recommended_time_step() == pytest.approx(dt, rel=0 if precision == 0 else 1e-6)
    for _ in range(3):
        assert g.do_time_steps(500, dt) == o.do_time_steps(500, dt) == 500
        assert g.do_time_step(-1.0) and o.do_time_step(-1.0)
    if precision == 0:
        assert state_diff(g, o) == []
    else:  # FP32C: its own recommended dt (FP32) in the single steps, FP32 floor contact
        pa, pb = g.voxel_state()["pos"], o.voxel_state()["pos"]
        err = np.abs(pa - pb).max()
        print(f"single voxel FP32C (bouncing on the floor, z = {pb[0, 2]:.4e} m): position error {err:.3e} m")
        assert err <= 1e-4 * 0.01  # of the 1 cm fall


def test_two_voxels_then_emptied(product_lib, cr_oracle):
    g, o = _both(product_lib, cr_oracle, [(0, 0, 0), (1, 0, 0)], 0, gravity=False)
    for s in (g, o):
        s.set_fixed_all(0)
        s.set_force(1, 0.0, 0.0, -0.01)
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    assert g.do_time_steps(300, dt) == o.do_time_steps(300, dt) == 300
    assert state_diff(g, o) == []
    for s in (g, o):
        s.remove_voxel(0, 0, 0)
        s.remove_voxel(1, 0, 0)
    assert g.voxel_count() == 0 and g.link_count() == 0
    assert g.do_time_steps(5, dt) == o.do_time_steps(5, dt) == 5
