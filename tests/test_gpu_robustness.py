"""Bad input and injected faults become error returns, or the reference's own behaviour, never a
device fault.

* Index fields uploaded through the engine ABI (include/vxg.h) are checked on the device before the
  first kernel that dereferences them: an out-of-range link endpoint, voxel link or material makes
  the step return an error naming the field, nothing runs, and the scene steps again once the field
  is corrected.
* A NaN external force injected on the host propagates exactly as in the reference (its divergence
  test, strain > 100, is false for NaN, src/Voxelyze.cpp:263-269): the same voxels turn NaN, and the
  others stay bit-identical to the oracle.
* Repeated runs are bit-identical (the gathers sum in a fixed order, without atomics), also with
  collisions and in FP32C.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import make_sim, state_diff
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu

VXG_F_VOXEL_MATERIAL, VXG_F_VOXEL_LINKS, VXG_F_LINK_VOXELS = 0, 2, 12


@pytest.fixture
def cr_oracle(oracle_lib):
    """The oracle with correctly rounded sin/cos/acos, as the GPU's FP64 path."""
    oracle_lib.vxo_set_math(1)
    yield oracle_lib
    oracle_lib.vxo_set_math(0)


def _engine(lib, sim):
    lib.vx_engine.restype = C.c_void_p
    lib.vx_engine.argtypes = [C.c_void_p]
    e = lib.vx_engine(C.c_void_p(sim.h))
    assert e
    lib.vxg_set_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong]
    lib.vxg_get_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong]
    lib.vxg_last_error.restype = C.c_char_p
    lib.vxg_last_error.argtypes = [C.c_void_p]
    return e


@pytest.mark.parametrize("field,comps,bad,name", [
    (VXG_F_LINK_VOXELS, 2, lambda a, nv, nl: a.__setitem__(nl + 5, nv), "link voxel"),
    (VXG_F_VOXEL_LINKS, 6, lambda a, nv, nl: a.__setitem__(3 * nv + 2, nl + 7), "voxel link"),
    (VXG_F_VOXEL_MATERIAL, 1, lambda a, nv, nl: a.__setitem__(nv - 1, 99), "voxel material"),
])
@pytest.mark.parametrize("precision", [0, 1])
def test_index_out_of_range_is_an_error(product_lib, field, comps, bad, name, precision):
    sim = make_sim(product_lib, "vx", S.lattice(6, 5, 4))
    F.Engine(sim).set_precision(precision)
    dt = sim.recommended_time_step()
    assert sim.do_time_steps(10, dt) == 10
    before = sim.voxel_state()["pos"].copy()
    e = _engine(product_lib, sim)
    nv, nl = sim.voxel_count(), sim.link_count()
    n = comps * (nl if field == VXG_F_LINK_VOXELS else nv)
    good = np.zeros(n, np.int32)
    assert product_lib.vxg_get_field(e, field, good.ctypes.data, n) == 0
    broken = good.copy()
    bad(broken, nv, nl)
    assert product_lib.vxg_set_field(e, field, broken.ctypes.data, n) == 0
    assert sim.do_time_steps(10, dt) < 0
    msg = product_lib.vxg_last_error(e).decode()
    assert "index out of range" in msg and name in msg, msg
    assert product_lib.vxg_set_field(e, field, good.ctypes.data, n) == 0
    assert np.array_equal(sim.voxel_state()["pos"], before)  # nothing ran
    assert sim.do_time_steps(10, dt) == 10


def test_nan_force_propagates_like_the_reference(product_lib, cr_oracle):
    """A NaN vertical force on one voxel: one more voxel layer turns NaN each step, through the
    links, in both libraries; the rest stay bit-identical.  A NaN horizontal force on a voxel that
    rests on the floor never enters the state at all: the static-friction test (force^2 > (mu N)^2,
    src/VX_Voxel.cpp:283-291) is false for NaN, so the latch holds and zeroes the motion."""
    sc = S.lattice(6, 5, 4)
    g, o = make_sim(product_lib, "vx", sc), make_sim(cr_oracle, "vxo", sc)
    for s in (g, o):
        s.set_force(7, 0.0, 0.0, float("nan"))
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    for _ in range(4):
        assert g.do_time_steps(1, dt) == o.do_time_steps(1, dt) == 1
        pg, po = g.voxel_state()["pos"], o.voxel_state()["pos"]
        nan_g, nan_o = np.isnan(pg), np.isnan(po)
        assert nan_g.any() and not nan_g.all()
        assert np.array_equal(nan_g, nan_o)
        assert np.array_equal(pg[~nan_g], po[~nan_o])
    h, q = make_sim(product_lib, "vx", sc), make_sim(cr_oracle, "vxo", sc)
    for s in (h, q):
        s.set_force(7, float("nan"), 0.0, 0.0)
    assert h.do_time_steps(60, dt) == q.do_time_steps(60, dt) == 60
    assert not np.isnan(h.voxel_state()["pos"]).any()
    assert state_diff(h, q) == []


@pytest.mark.parametrize("precision", [0, 1])
def test_repeat_runs_are_bit_identical(product_lib, precision):
    sc = S.porous(20, sigma=1.5)  # floor, friction and collisions
    runs = []
    for _ in range(2):
        s = make_sim(product_lib, "vx", sc)
        F.Engine(s).set_precision(precision)
        dt = s.recommended_time_step()
        assert s.do_time_steps(300, dt) == 300
        runs.append(s)
    assert state_diff(*runs) == []
    assert np.array_equal(runs[0].collisions(), runs[1].collisions())


@pytest.mark.parametrize("precision", [0, 1])
def test_shrunk_externals_table_rechecks_indices(product_lib, precision):
    """A table re-uploaded with fewer entries (here the externals, emptied through the engine ABI)
    keeps its allocation but not its old count: a voxel still naming an external that is gone makes
    the next step an index error instead of a read of the stale entry."""
    sim = make_sim(product_lib, "vx", S.cantilever(6, 2, 2, voxel_size=0.005, tip_force=-0.01))
    F.Engine(sim).set_precision(precision)
    assert sim.do_time_steps(5, -1.0) == 5
    e = _engine(product_lib, sim)
    product_lib.vxg_set_externals.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    assert product_lib.vxg_set_externals(e, None, 0) == 0
    assert sim.do_time_steps(5, -1.0) < 0
    msg = product_lib.vxg_last_error(e).decode()
    assert "index out of range" in msg and "voxel external" in msg, msg


def test_state_info_extremes_start_like_the_reference(product_lib):
    """stateInfo starts MIN at FLT_MAX and MAX at -FLT_MAX (src/Voxelyze.cpp:755-756): with every
    voxel's momentum infinite, VELOCITY MIN stays FLT_MAX and MAX is infinite, on the device as on
    the host."""
    sim = make_sim(product_lib, "vx", S.lattice(6, 5, 4))
    assert sim.do_time_steps(2, sim.recommended_time_step()) == 2
    e = _engine(product_lib, sim)
    nv = sim.voxel_count()
    VXG_F_LINMOM = 5
    mom = np.full(3 * nv, np.inf)
    assert product_lib.vxg_set_field(e, VXG_F_LINMOM, mom.ctypes.data, 3 * nv) == 0
    dev = product_lib.vx_state_info_device
    dev.restype = C.c_float
    dev.argtypes = [C.c_void_p, C.c_int, C.c_int]
    flt_max = float(np.finfo(np.float32).max)
    assert dev(C.c_void_p(sim.h), F.VELOCITY, F.MIN) == flt_max
    assert dev(C.c_void_p(sim.h), F.VELOCITY, F.MAX) == np.inf
    assert sim.state_info(F.VELOCITY, F.MIN) == flt_max
    assert sim.state_info(F.VELOCITY, F.MAX) == np.inf
