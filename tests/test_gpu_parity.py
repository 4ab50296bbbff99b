"""GPU FP64 path against the oracle, bit for bit.

The oracle runs in its correctly-rounded mode (vxo_set_math(1)): sin/cos/acos are then the same
correctly rounded values the GPU computes, and every other operation is the reference's own IEEE
arithmetic, so the whole state (positions, momenta, orientations, link pose, forces, strains,
flags) must be identical after any number of steps.  Against the C-library oracle (the reference's
exact arithmetic) the two can differ only where glibc's sin/cos/acos is not correctly rounded;
those runs report the error and the engine's count of such near-midpoint evaluations.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import make_sim, max_rel_pos_err, state_diff
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu


@pytest.fixture()
def cr_oracle(oracle_lib):
    oracle_lib.vxo_set_math(1)
    yield oracle_lib
    oracle_lib.vxo_set_math(0)


def _pair(product_lib, oracle_lib, scene, threads=1):
    g = make_sim(product_lib, "vx", scene)
    o = make_sim(oracle_lib, "vxo", scene)
    if threads > 1:
        oracle_lib.vxo_set_threads(C.c_void_p(o.h), threads)
    return g, o


def _run_exact(g, o, steps, chunk, dt):
    done = 0
    while done < steps:
        n = min(chunk, steps - done)
        assert g.do_time_steps(n, dt) == o.do_time_steps(n, dt)
        done += n
        assert state_diff(g, o) == [], f"state differs after {done} steps"


def test_recommended_dt(product_lib, cr_oracle):
    for sc in (S.cantilever(), S.lattice(10, 10, 6), S.porous(12, sigma=1.0), S.population(4, 3, 5)):
        g, o = _pair(product_lib, cr_oracle, sc)
        assert g.recommended_time_step() == o.recommended_time_step()
        assert state_diff(g, o) == []


def test_cantilever_small(product_lib, cr_oracle):
    g, o = _pair(product_lib, cr_oracle, S.cantilever(8, 3, 3, voxel_size=0.005, tip_force=-0.05))
    _run_exact(g, o, 600, 150, o.recommended_time_step())


def test_cantilever_full_horizon(product_lib, cr_oracle):
    """40x8x8 cantilever, -1 N per tip voxel, dt = recommendedTimeStep, 10,000 steps."""
    g, o = _pair(product_lib, cr_oracle, S.cantilever())
    dt = o.recommended_time_step()
    _run_exact(g, o, 10000, 2500, dt)


def test_large_angle_branch(product_lib, cr_oracle):
    """20 voxels in a row, E = 10 kPa, a small tip load: links cross into and out of the
    large-angle branch all through 2,000 steps (acos/sin/cos, src/VX_Link.cpp:92-110)."""
    g, o = _pair(product_lib, cr_oracle, S.cantilever(20, 1, 1, E=1e4, tip_force=-0.02))
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    large = 0
    for n in (250, 250, 250, 250, 1000):
        assert g.do_time_steps(n, dt) == o.do_time_steps(n, dt) == n
        assert state_diff(g, o) == []
        large += int((g.link_state()["smallAngle"] == 0).sum())
    assert large > 0


def test_single_steps_equal_batched(product_lib, cr_oracle):
    sc = S.cantilever(10, 3, 2, voxel_size=0.005, tip_force=-0.02)
    a = make_sim(product_lib, "vx", sc)
    b = make_sim(product_lib, "vx", sc)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    for _ in range(60):
        assert a.do_time_step(dt)
    assert b.do_time_steps(60, dt) == 60
    assert state_diff(a, b) == []


def test_lattice_poisson_bilinear_floor(product_lib, cr_oracle):
    g, o = _pair(product_lib, cr_oracle, S.lattice(16, 16, 8))
    _run_exact(g, o, 300, 100, o.recommended_time_step())


def test_lattice_recommended_dt_every_step(product_lib, cr_oracle):
    g, o = _pair(product_lib, cr_oracle, S.lattice(10, 8, 6, seed=7))
    _run_exact(g, o, 60, 20, -1.0)
    assert g.current_time() == o.current_time()


def test_population_temperature_and_reset(product_lib, cr_oracle):
    g, o = _pair(product_lib, cr_oracle, S.population(8, 3, 7))
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    _run_exact(g, o, 100, 50, dt)
    for t in (0.05, -0.03, 0.1):
        g.set_ambient_temperature(t, True)
        o.set_ambient_temperature(t, True)
        _run_exact(g, o, 40, 40, dt)
    g.reset_time()
    o.reset_time()
    assert state_diff(g, o) == []
    _run_exact(g, o, 60, 30, dt)


def _custom(s):
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.1)
    s.material_set(m, F.PROP_POISSON, 0.3)
    m2 = s.add_material(3e6, 1.5e3)
    s.set_model(m2, [0.01, 0.05, 0.2], [3e4, 8e4, 1.2e5])
    s.material_set(m2, F.PROP_CTE, 0.01)
    for i in range(6):
        for j in range(3):
            for k in range(2):
                v = s.set_voxel(m if (i + j) % 2 else m2, i, j, k)
                if i == 0:
                    s.set_fixed(v, F.X_TRANSLATE | F.Z_TRANSLATE | F.X_ROTATE)
                if i == 5:
                    s.set_displacement(v, F.Y_ROTATE, 0.2)
                    s.set_moment(v, 1e-4, 0, 2e-4)
                    s.set_force(v, 0.05, 0.02, -0.1)
    s.set_gravity(0.5)
    s.enable_floor(True)
    s.set_temperature(3, 2.0)


def test_partial_fixes_rotation_data_model(product_lib, cr_oracle):
    g = F.Sim(product_lib, "vx", 0.002)
    o = F.Sim(cr_oracle, "vxo", 0.002)
    _custom(g)
    _custom(o)
    assert state_diff(g, o) == []
    for _ in range(5):
        assert g.do_time_steps(100, -1.0) == o.do_time_steps(100, -1.0)
        assert state_diff(g, o) == []
    for info in range(10):
        for t in range(4):
            a, b = g.state_info(info, t), o.state_info(info, t)
            assert a == b or (np.isnan(a) and np.isnan(b)), (info, t, a, b)


def test_divergence_stops_like_the_reference(product_lib, cr_oracle):
    """A force far too large for the step: doTimeStep returns false at the same step, with the
    link state advanced and the voxels not (Voxelyze.cpp:263-269)."""
    sc = S.cantilever(4, 1, 1, voxel_size=0.001, tip_force=5e3)
    g, o = _pair(product_lib, cr_oracle, sc)
    dt = o.recommended_time_step() * 4
    ng = g.do_time_steps(200, dt)
    no = o.do_time_steps(200, dt)
    assert ng == no < 200
    assert state_diff(g, o) == []
    assert g.do_time_step(dt) == o.do_time_step(dt)
    assert state_diff(g, o) == []


def test_collisions_pairs_and_state(product_lib, cr_oracle):
    sc = S.porous(16, sigma=1.5)
    g, o = _pair(product_lib, cr_oracle, sc)
    dt = o.recommended_time_step()
    for _ in range(3):
        assert g.do_time_steps(100, dt) == o.do_time_steps(100, dt)
        assert np.array_equal(g.collisions(), o.collisions())
        assert state_diff(g, o) == []


def test_against_c_library_oracle_reports_error(product_lib, oracle_lib):
    """The reference's own arithmetic (C-library sin/cos/acos): bit-identical unless the
    C library's rounding differs from the correctly rounded value; the error is reported."""
    oracle_lib.vxo_set_math(0)
    g, o = _pair(product_lib, oracle_lib, S.lattice(12, 12, 8))
    dt = o.recommended_time_step()
    g.do_time_steps(200, dt)
    o.do_time_steps(200, dt)
    err = max_rel_pos_err(g, o)
    cnt = (C.c_longlong * 8)()
    product_lib.vx_counters(C.c_void_p(g.h), cnt, 8)
    print(f"lattice 12x12x8, 200 steps: max rel pos err vs C-library oracle {err:.3e}, "
          f"transcendental evals {cnt[0]}, near-midpoint {cnt[2]}")
    assert err <= 1e-10


@pytest.mark.parametrize("dims", [(128, 128, 64)])
def test_large_lattice_full_size(product_lib, cr_oracle, dims):
    """The 128x128x64 multi-material lattice (~0.9 M voxels, ~2.25 M links): bit-identical to the
    threaded oracle for a few steps, then 1,000 GPU steps stay finite and on the floor."""
    sc = S.lattice(*dims)
    g, o = _pair(product_lib, cr_oracle, sc, threads=16)
    dt = o.recommended_time_step()
    assert g.recommended_time_step() == dt
    _run_exact(g, o, 4, 2, dt)
    assert g.do_time_steps(996, dt) == 996
    pos = g.voxel_state()["pos"]
    assert np.all(np.isfinite(pos))
    assert pos[:, 2].min() > -0.5 * sc.voxel_size


def test_state_info_device_reduction(product_lib, cr_oracle):
    """vxg_reduce (CVoxelyze::stateInfoDevice): MIN and MAX equal the reference's serial float
    reduction exactly; TOTAL and AVERAGE accumulate in double, within 1e-5 of it."""
    sc = S.lattice(20, 16, 10)
    g, o = _pair(product_lib, cr_oracle, sc)
    dt = o.recommended_time_step()
    g.do_time_steps(120, dt)
    o.do_time_steps(120, dt)
    f = product_lib.vx_state_info_device
    f.restype = C.c_float
    f.argtypes = [C.c_void_p, C.c_int, C.c_int]
    for info in (F.DISPLACEMENT, F.VELOCITY, F.KINETIC_ENERGY, F.ANGULAR_VELOCITY, F.ENG_STRESS, F.ENG_STRAIN,
                 F.STRAIN_ENERGY, F.MASS):
        for t in (F.MIN, F.MAX, F.TOTAL, F.AVERAGE):
            dev = f(C.c_void_p(g.h), info, t)
            ref = o.state_info(info, t)
            if t in (F.MIN, F.MAX):
                assert dev == ref, (info, t, dev, ref)
            else:
                assert abs(dev - ref) <= 1e-5 * max(abs(ref), 1e-30), (info, t, dev, ref)
