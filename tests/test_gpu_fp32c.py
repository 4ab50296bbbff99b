"""FP32-compensated path (precision mode 1) against the FP64 path.

The FP64 GPU path is bit-identical to the oracle (test_gpu_parity.py), so its positions stand in
for the FP64 oracle here.  Errors are stated as
    max |pos_fp32c - pos_fp64| / max |pos_fp64|        (relative position error)
    max |pos_fp32c - pos_fp64| / max |disp_fp64|       (relative to the largest displacement)
and each test states its tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import make_sim
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu


def _pair(product_lib, scene):
    a = make_sim(product_lib, "vx", scene)
    b = make_sim(product_lib, "vx", scene)
    assert product_lib.vx_set_precision(__import__("ctypes").c_void_p(b.h), 1) == 0
    return a, b


def _errors(a, b, scene):
    pa, pb = a.voxel_state()["pos"], b.voxel_state()["pos"]
    disp = pa - scene.xyz * scene.voxel_size
    d = np.abs(pa - pb)
    return float(d.max() / np.abs(pa).max()), float(d.max() / max(np.abs(disp).max(), 1e-30))


def test_lattice_1000_steps(product_lib):
    """The 128x128x64 multi-material lattice, 1,000 steps: relative position error <= 1e-5."""
    sc = S.lattice(128, 128, 64)
    a, b = _pair(product_lib, sc)
    dt = a.recommended_time_step()
    assert b.recommended_time_step() == pytest.approx(dt, rel=1e-6)
    assert a.do_time_steps(1000, dt) == 1000
    assert b.do_time_steps(1000, dt) == 1000
    rel_pos, rel_disp = _errors(a, b, sc)
    print(f"lattice 128x128x64, 1000 steps: rel pos err {rel_pos:.3e}, rel disp err {rel_disp:.3e}")
    assert rel_pos <= 1e-5
    assert rel_disp <= 1e-3


def test_small_lattice_poisson_dt_every_step(product_lib):
    sc = S.lattice(16, 16, 8)
    a, b = _pair(product_lib, sc)
    assert a.do_time_steps(300, -1.0) == 300
    assert b.do_time_steps(300, -1.0) == 300
    rel_pos, rel_disp = _errors(a, b, sc)
    print(f"lattice 16x16x8, dt every step, 300 steps: rel pos err {rel_pos:.3e}, rel disp err {rel_disp:.3e}")
    assert rel_pos <= 1e-5
    assert rel_disp <= 1e-3


@pytest.mark.parametrize("friction", [False, True])
def test_population_with_temperature(product_lib, friction):
    """Bodies on the floor with CTE actuation.  Without friction FP32C tracks FP64 closely.  With
    friction, the static-friction latch compares the horizontal force against mu * N while the
    normal force N is still ~0 at first contact (VX_Voxel.cpp:285-291); FP32 rounding noise flips
    that ill-conditioned test for some voxels, which then slide, so the bound is looser."""
    sc = S.population(16, 4, 10)
    if not friction:
        for m in sc.materials:
            m.mu_static = m.mu_kinetic = 0.0
    a, b = _pair(product_lib, sc)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    for k in range(10):
        t = 0.1 * np.sin(2 * np.pi * 2 * k * 50 * dt)
        a.set_ambient_temperature(float(t), True)
        b.set_ambient_temperature(float(t), True)
        assert a.do_time_steps(50, dt) == 50
        assert b.do_time_steps(50, dt) == 50
    rel_pos, rel_disp = _errors(a, b, sc)
    print(f"population 16 bodies, CTE actuation, friction={friction}, 500 steps: "
          f"rel pos err {rel_pos:.3e}, rel disp err {rel_disp:.3e}")
    if friction:
        assert rel_pos <= 1e-3
    else:
        assert rel_pos <= 1e-6
        assert rel_disp <= 1e-3


def test_friction_error_is_the_scene_conditioning(product_lib):
    """The friction population's FP32C error is the conditioning of the scene, not of FP32C: two
    FP64 runs whose only difference is one ulp in every initial voxel position (nextafter towards
    +inf) drift apart by an amount of the same order as FP32C drifts from FP64 over the same 500
    steps.  The static-friction latch compares the horizontal force with mu * N while N is ~0 at
    first contact (src/VX_Voxel.cpp:285-291), so any rounding difference can flip it for a voxel,
    which then slides."""
    import ctypes as C

    sc = S.population(16, 4, 10)
    a, b = _pair(product_lib, sc)
    c = make_sim(product_lib, "vx", sc)
    product_lib.vx_engine.restype = C.c_void_p
    product_lib.vx_engine.argtypes = [C.c_void_p]
    product_lib.vxg_set_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_longlong]
    pos = c.voxel_state()["pos"]
    bumped = np.ascontiguousarray(np.nextafter(pos, np.inf).T).ravel()  # component-major
    VXG_F_POS = 4
    assert product_lib.vxg_set_field(product_lib.vx_engine(C.c_void_p(c.h)), VXG_F_POS, bumped.ctypes.data,
                                     bumped.size) == 0
    dt = a.recommended_time_step()
    for s in (b, c):
        s.recommended_time_step()
    for k in range(10):
        t = float(0.1 * np.sin(2 * np.pi * 2 * k * 50 * dt))
        for s in (a, b, c):
            s.set_ambient_temperature(t, True)
            assert s.do_time_steps(50, dt) == 50
    _, d32 = _errors(a, b, sc)
    _, d64 = _errors(a, c, sc)
    print(f"population 16 bodies with friction, 500 steps: FP32C vs FP64 {d32:.3e}, FP64 with one ulp "
          f"moved in every initial position vs FP64 {d64:.3e} (relative to the largest displacement)")
    assert d64 > 0.0
    assert d64 >= 0.1 * d32


def test_cantilever_small_deflection(product_lib):
    """Static-like cantilever (small load): FP32C converges to the same deflection."""
    sc = S.cantilever(20, 4, 4, voxel_size=0.005, tip_force=-0.01)
    a, b = _pair(product_lib, sc)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    assert a.do_time_steps(3000, dt) == 3000
    assert b.do_time_steps(3000, dt) == 3000
    rel_pos, rel_disp = _errors(a, b, sc)
    print(f"cantilever 20x4x4, 3000 steps: rel pos err {rel_pos:.3e}, rel disp err {rel_disp:.3e}")
    assert rel_pos <= 1e-5
    assert rel_disp <= 2e-4


def test_fp32c_state_roundtrip_and_reset(product_lib):
    sc = S.lattice(8, 8, 4)
    a, b = _pair(product_lib, sc)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    b.do_time_steps(100, dt)
    b.reset_time()
    a.reset_time()
    st_a, st_b = a.voxel_state(), b.voxel_state()
    assert np.array_equal(st_a["pos"], st_b["pos"])
    assert b.do_time_steps(50, dt) == 50
    assert np.all(np.isfinite(b.voxel_state()["pos"]))


def _fp32c(product_lib, scene, blocks_per_sm, split=True):
    s = make_sim(product_lib, "vx", scene)
    E = F.Engine(s)
    E.set_precision(1)
    E.set_link_pipeline(blocks_per_sm)
    E.set_link_split(split)
    assert E.link_pipeline() == blocks_per_sm and E.link_split() == split
    return s


@pytest.mark.parametrize("scene", ["lattice_poisson", "cantilever", "population_actuated", "graded", "floppy"])
@pytest.mark.parametrize("variant", ["pipelined_all", "pipelined_1", "general"])
def test_link_pass_variants_are_bit_identical(product_lib, scene, variant):
    """The FP32C link-pass variants against the split pass (a small-angle kernel, then the general
    kernel over the links it deferred): every state array identical bit for bit after each batch.
    Variants: the pipelined pass (cp.async staging, resident grid; one block per SM makes every
    block walk many tiles, both halves of the double buffer) and the general one-thread-per-link
    pass (the default).  The scenes cover Poisson's ratio != 0 with bilinear materials, a fixed cantilever,
    in-step CTE actuation with floor and friction, and one material per voxel.  The floppy beam (20
    voxels in a row, E = 10 kPa) moves links into and out of the large-angle branch all through the
    run, so the split pass defers links every step: the pipelined pass always reads each link's
    stored angle1v, the small-angle kernel takes it as zero, so identical states also check that
    the stored angle1v of a small-angle link is zero."""
    from conftest import state_diff

    blocks_per_sm = {"pipelined_all": -1, "pipelined_1": 1, "general": 0}[variant]

    sc = {"lattice_poisson": lambda: S.lattice(40, 36, 20),
          "cantilever": lambda: S.cantilever(40, 8, 8),
          "population_actuated": lambda: S.population(24, 4, 12),
          "graded": lambda: S.graded_population(6, 10),
          "floppy": lambda: S.cantilever(20, 1, 1, E=1e4, tip_force=-0.02)}[scene]()
    a = _fp32c(product_lib, sc, 0)
    b = _fp32c(product_lib, sc, blocks_per_sm, split=variant != "general")
    dt = a.recommended_time_step()
    assert b.recommended_time_step() == dt
    if scene in ("population_actuated", "graded"):
        for s in (a, b):
            F.Engine(s).set_actuation(F.ACT_UNIFORM, 0.1, 2.0)
    n, batches = (250, 8) if scene == "floppy" else (70, 3)
    large = 0
    for _ in range(batches):
        assert a.do_time_steps(n, dt) == b.do_time_steps(n, dt) == n
        assert state_diff(a, b) == []
        large += int((a.link_state()["smallAngle"] == 0).sum())
    if scene == "floppy":
        assert large > 0


def _dynamic_state(s):
    v, l = s.voxel_state(), s.link_state()
    return [v["raw_d"], v["temp"], v["staticFriction"], l["raw_d"], l["raw_f"], l["raw_i"]]


@pytest.mark.parametrize("edit", [False, True])
def test_fused_poisson_cache_matches_prepass(product_lib, edit):
    """FP32C with nu = 0.3: the voxel pass filling each Poisson-strain cache for the next step
    (default) against a pre-pass filling it before every link pass.  Positions, momenta,
    orientations, temperatures and every link-state array are identical bit for bit after each
    batch.  With `edit`, between batches forces on the x-max face change (their x component decides
    the tension terms of CVX_Voxel::strain, src/VX_Voxel.cpp:313-318) and the x = 0 face gets
    fixed: the caches filled ahead of time must be refilled from the edited externals."""
    sc = S.lattice(24, 20, 12)
    a = _fp32c(product_lib, sc, 0)
    b = _fp32c(product_lib, sc, 0)
    F.Engine(b).set_poisson_fusion(False)
    dt = a.recommended_time_step()
    assert b.recommended_time_step() == dt
    xmax = np.flatnonzero(sc.xyz[:, 0] == sc.xyz[:, 0].max())
    x0 = np.flatnonzero(sc.xyz[:, 0] == 0)
    for k in range(4):
        if edit:
            for s in (a, b):
                for v in xmax:
                    s.set_force(int(v), 0.02 * (k - 1), 0.0, -0.01 * k)
                if k == 2:
                    for v in x0:
                        s.set_fixed_all(int(v))
        assert a.do_time_steps(40, dt) == b.do_time_steps(40, dt) == 40
        for x, y in zip(_dynamic_state(a), _dynamic_state(b)):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("friction", [False, True])
def test_collisions_fp32c_tracks_fp64(product_lib, friction):
    """The porous collision scene (the 64^3 collision body's generator at 20^3) dropped onto the floor with
    collisions on: FP32C against FP64.  Both start from the same lattice, so the first pair list
    is the same set; the contact forces are FP32 in FP32C (offsets from lattice offsets plus
    displacement differences).  Without friction FP32C tracks FP64 closely; with friction the
    static-friction latch at first floor contact (src/VX_Voxel.cpp:285-291) is ill-conditioned, so
    the bound is looser."""
    sc = S.porous(20, sigma=1.5, z_offset=0)  # on the floor from the start
    if not friction:
        for m in sc.materials:
            m.mu_static = m.mu_kinetic = 0.0
    a, b = _pair(product_lib, sc)
    dt = a.recommended_time_step()
    assert b.recommended_time_step() == pytest.approx(dt, rel=1e-6)
    assert a.do_time_steps(1, dt) == b.do_time_steps(1, dt) == 1
    pa, pb = a.collisions(), b.collisions()
    assert len(pa) > 0 and np.array_equal(pa, pb)
    for _ in range(6):
        assert a.do_time_steps(100, dt) == b.do_time_steps(100, dt) == 100
    rel_pos, rel_disp = _errors(a, b, sc)
    na, nb = len(a.collisions()), len(b.collisions())
    print(f"porous 20^3 with collisions, friction={friction}, 601 steps: rel pos err {rel_pos:.3e}, "
          f"rel disp err {rel_disp:.3e}, pairs FP64 {na} FP32C {nb}")
    assert abs(na - nb) <= max(2, na // 100)
    if friction:
        assert rel_pos <= 1e-3
    else:
        assert rel_pos <= 1e-5


def test_positions_into_pinned_memory(product_lib):
    """Reading FP32C positions into pinned host memory converts them on the device straight into
    that buffer; the values equal the staged read (pageable destination) bit for bit."""
    import ctypes as C

    import torch

    sc = S.lattice(24, 20, 10)
    s = _fp32c(product_lib, sc, 0)
    dt = s.recommended_time_step()
    read = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)(("vx_read_positions", product_lib))
    for _ in range(3):
        assert s.do_time_steps(25, dt) == 25
        pinned = torch.empty(3 * s.voxel_count(), dtype=torch.float64, pin_memory=True)
        assert read(s.h, pinned.data_ptr()) == 0
        staged = np.zeros(3 * s.voxel_count(), np.float64)
        assert read(s.h, staged.ctypes.data) == 0
        assert np.array_equal(pinned.numpy(), staged)
        assert np.array_equal(staged.reshape(3, -1).T, s.voxel_state()["pos"])


@pytest.mark.parametrize("precision", [0, 1])
def test_async_position_reads(product_lib, precision):
    """vx_read_positions_async: each step's positions are staged on the device and copied while the
    next steps run; after vx_read_wait every buffer holds exactly what a synchronous read after
    that step returned (a second simulator stepping alongside), for pinned and pageable buffers,
    for more reads in flight than staging buffers, and across a change of the scene's size."""
    import torch

    sc = S.lattice(24, 20, 10)
    a, b = (make_sim(product_lib, "vx", sc) for _ in range(2))
    for s in (a, b):
        F.Engine(s).set_precision(precision)
    Eb = F.Engine(b)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    n = 3 * a.voxel_count()
    bufs = [torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() if k % 3 else np.zeros(n)
            for k in range(7)]
    want = []
    for k in range(7):
        assert a.do_time_steps(3, dt) == b.do_time_steps(3, dt) == 3
        want.append(F.Engine(a).read_positions().T.reshape(-1).copy())
        Eb.read_positions_async(bufs[k])
    Eb.read_wait()
    for k in range(7):
        assert np.array_equal(bufs[k], want[k]), f"read {k}"
    nv = b.voxel_count()
    b.set_voxel(0, 40, 40, 0)
    assert b.voxel_count() == nv + 1
    out = np.zeros(3 * b.voxel_count())
    assert b.do_time_steps(2, dt) == 2
    Eb.read_positions_async(out)
    Eb.read_wait()
    assert np.array_equal(out, Eb.read_positions().T.reshape(-1))


@pytest.mark.parametrize("precision", [0, 1])
def test_temperatures_from_pinned_memory(product_lib, precision):
    """vx_set_temperatures from pinned host memory is read by a kernel (16-byte loads where the
    buffer is aligned, single floats where not) instead of a copy: the same state bit for bit as
    temperatures from pageable memory, on a voxel count that is not a multiple of four."""
    import ctypes as C

    import torch

    from conftest import state_diff

    sc = S.lattice(13, 11, 7)
    sims = [make_sim(product_lib, "vx", sc) for _ in range(3)]
    for s in sims:
        F.Engine(s).set_precision(precision)
    nv = sims[0].voxel_count()
    assert nv % 4 != 0
    set_t = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)(("vx_set_temperatures", product_lib))
    rng = np.random.default_rng(5)
    dt = sims[0].recommended_time_step()
    for s in sims[1:]:
        s.recommended_time_step()
    pinned = torch.empty(nv + 1, dtype=torch.float32, pin_memory=True)
    for _ in range(4):
        t = rng.uniform(-20, 20, nv).astype(np.float32)
        pinned[:nv] = torch.from_numpy(t)
        assert set_t(sims[0].h, t.ctypes.data) == 0
        assert set_t(sims[1].h, pinned.data_ptr()) == 0
        pinned[1:] = torch.from_numpy(t)
        assert set_t(sims[2].h, pinned.data_ptr() + 4) == 0  # 4 bytes past a 16-byte boundary
        for s in sims:
            assert s.do_time_steps(3, dt) == 3
    assert state_diff(sims[0], sims[1]) == []
    assert state_diff(sims[0], sims[2]) == []


def _launches(lib, sim):
    import ctypes as C

    cnt = (C.c_longlong * 8)()
    assert lib.vx_counters(C.c_void_p(sim.h), cnt, 8) == 0
    return int(cnt[6])


def _bodies_scene(kind):
    """300 small bodies (3 to 6 cells a side) on the floor with friction, two materials (one with
    CTE); 'poisson': both materials with nu = 0.3 (the Poisson cache filled by the voxel phase)."""
    sc = S.population(300, 3, 6, seed=11)
    if kind == "poisson":
        for m in sc.materials:
            m.nu = 0.3
    return sc


def _packed_groups(sizes, target):
    """Groups of consecutive bodies of these voxel counts, each up to `target` voxels (a larger
    body alone): the packing vxg_set_body_batches describes."""
    groups, cur = 0, 0
    for n in sizes:
        if cur and cur + n > target:
            groups, cur = groups + 1, 0
        cur += n
    return groups + 1


@pytest.mark.parametrize("kind", ["plain", "uniform_actuation", "phase_actuation", "poisson"])
def test_body_batches_are_bit_identical(product_lib, kind):
    """vxg_set_body_batches: each batch in one persistent launch whose CTAs take groups of bodies
    through every step (actuation, links, voxels, block barriers), against the default two passes
    per step replayed from CUDA graphs; every state array identical bit for bit after batches of
    1, 50 and 130 steps, and the time.  The body batch is checked to have run (three launches per
    batch) with one group per body (voxels per group 1: 300 groups) and with consecutive bodies
    packed up to 100 voxels to a group (196 groups, more than the SMs)."""
    from conftest import state_diff

    sc = _bodies_scene(kind)
    for target in (1, 100):
        a, b = (make_sim(product_lib, "vx", sc) for _ in range(2))
        for s in (a, b):
            E = F.Engine(s)
            E.set_precision(1)
            if kind == "uniform_actuation":
                E.set_actuation(F.ACT_UNIFORM, 0.2, 3.0)
            elif kind == "phase_actuation":
                ph = np.random.default_rng(3).uniform(0, 2 * np.pi, sc.n_voxels).astype(np.float32)
                E.set_actuation(F.ACT_PER_VOXEL, 0.2, 3.0, ph)
        Eb = F.Engine(b)
        Eb.set_body_batches(target)
        per_group, groups = Eb.body_batches()
        assert per_group == target
        assert groups == _packed_groups(np.bincount(sc.body), target)
        dt = a.recommended_time_step()
        assert b.recommended_time_step() == dt
        for n in (1, 50, 130):
            l0 = _launches(product_lib, b)
            assert a.do_time_steps(n, dt) == b.do_time_steps(n, dt) == n
            if n > 1:  # the body kernel, its closing kernel and the control words' read
                assert _launches(product_lib, b) - l0 == 3, "the body batch did not run"
            assert state_diff(a, b) == [], f"after a batch of {n} (voxels per group {target})"
        assert a.current_time() == b.current_time()


def test_body_batch_divergence_is_rolled_back(product_lib):
    """One body pulled by a force far too large for it (src/Voxelyze.cpp:263-269): the body batch
    in which its links diverge is put back and run again as passes, which stop at the same step as
    the passes of a second simulator, with every other body at that step too (links advanced,
    voxels not); one more batch after it matches as well."""
    from conftest import state_diff

    sc = _bodies_scene("plain")
    sc.force_idx = np.array([int(np.flatnonzero(sc.body == 7)[0])])
    sc.force_val = np.array([[3e4, 0.0, 1e4]], np.float32)
    a, b = (make_sim(product_lib, "vx", sc) for _ in range(2))
    for s in (a, b):
        F.Engine(s).set_precision(1)
    F.Engine(b).set_body_batches(1)
    dt = a.recommended_time_step()
    b.recommended_time_step()
    assert a.do_time_steps(1, dt) == b.do_time_steps(1, dt) == 1
    na, nb = a.do_time_steps(200, dt), b.do_time_steps(200, dt)
    assert 1 <= na == nb < 200
    assert state_diff(a, b) == []
    assert a.current_time() == b.current_time()
    assert a.do_time_steps(3, dt) == b.do_time_steps(3, dt)
    assert state_diff(a, b) == []


def test_body_batches_need_separate_bodies(product_lib):
    """A single connected lattice is one piece: no group per SM, so batches run as passes."""
    sc = S.lattice(20, 16, 10)
    b = make_sim(product_lib, "vx", sc)
    E = F.Engine(b)
    E.set_precision(1)
    E.set_body_batches(1)
    assert E.body_batches() == (1, 1)
    dt = b.recommended_time_step()
    l0 = _launches(product_lib, b)
    assert b.do_time_steps(10, dt) == 10
    assert _launches(product_lib, b) - l0 > 3
