"""Known-answer physics tests of the reference (test/tVoxelyze.h), restated as functions that
build a scene on any simulator behind the facade and return what the reference test asserts on.

Each function takes ``mk(voxel_size) -> Sim`` and returns a dict of results plus ``sims`` (the
simulators built, for bit-level comparison between backends).  Expected values and tolerances are
the reference test's own; the two stale constants noted in the reference suite
(poissonsSmall, deformableMaterialPossions) are asserted against the reference build instead.
"""
from __future__ import annotations

import numpy as np

from voxelyze_gb300 import facade as F

TX, TY, TZ, RX, RY, RZ = range(6)
DIRS = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]


def dofmask(tx, ty, tz, rx, ry, rz):
    return (tx * F.X_TRANSLATE) | (ty * F.Y_TRANSLATE) | (tz * F.Z_TRANSLATE) | (rx * F.X_ROTATE) | \
        (ry * F.Y_ROTATE) | (rz * F.Z_ROTATE)


def rotation_vector(q):
    """Quat3D::ToRotationVector (Quat3D.h:117-122) on a (w, x, y, z) row."""
    w, x, y, z = (float(v) for v in q)
    if w >= 1.0 or w <= -1.0:
        return np.zeros(3)
    sl = 1.0 - w * w
    if sl < 2.4e-3:
        return np.array([x, y, z]) * 2.0 * np.sqrt((2 - 2 * w) / sl)
    return np.array([x, y, z]) * 2.0 * np.arccos(w) / np.sqrt(sl)


def two_vox(mk, v1_fixed, d, force, moment, dof, max_steps, expected, what):
    """test2Vox harness (tVoxelyze.h:63-113): steps until 10 consecutive samples match."""
    sz = 0.001
    s = mk(sz)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.2)
    off = DIRS[d]
    v1 = s.set_voxel(m, 0, 0, 0)
    if v1_fixed:
        s.set_fixed_all(v1)
    else:
        s.set_force(v1, -force[0], -force[1], -force[2])
        s.set_moment(v1, -moment[0], -moment[1], -moment[2])
        s.set_fixed(v1, dof)
    v2 = s.set_voxel(m, *off)
    s.set_force(v2, *force)
    s.set_moment(v2, *moment)
    s.set_fixed(v2, dof)
    ts = s.recommended_time_step()
    conv = 0
    k = 0
    for k in range(max_steps):
        s.do_time_step(ts)
        st = s.voxel_state()
        if what < 3:
            data = st["pos"][v2][what] - off[what] * sz
        else:
            data = rotation_vector(st["orient"][v2])[what - 3]
        if abs(data - expected) < abs(expected) * 1e-5 or np.float32(data) == np.float32(expected):
            conv += 1
        else:
            conv = 0
        if conv == 10:
            break
    return {"steps": k, "sims": [s]}


F3 = np.float32
FPX, FNX, FPY, FNY, FPZ, FNZ = (1e-3, 0, 0), (-1e-3, 0, 0), (0, 1e-3, 0), (0, -1e-3, 0), (0, 0, 1e-3), (0, 0, -1e-3)
MPX, MNX, MPY, MPZ = (1e-9, 0, 0), (-1e-9, 0, 0), (0, 1e-9, 0), (0, 0, 1e-9)
Z3 = (0, 0, 0)

# (v1_fixed, dir, force, moment, dof, max_steps, expected, what, bound) from tVoxelyze.h:143-252
TWO_VOX_CASES = [
    (True, 0, FPX, Z3, dofmask(0, 1, 1, 1, 1, 1), 1000, 1e-6, TX, 150),
    (True, 0, FNY, Z3, dofmask(1, 0, 1, 1, 1, 1), 1000, -1e-6, TY, 150),
    (True, 0, FPZ, Z3, dofmask(1, 1, 0, 1, 1, 1), 1000, 1e-6, TZ, 150),
    (True, 3, FPY, Z3, dofmask(1, 0, 1, 1, 1, 1), 1000, 1e-6, TY, 150),
    (True, 5, FPX, Z3, dofmask(0, 1, 1, 1, 1, 1), 1000, 1e-6, TX, 150),
    (True, 0, Z3, MNX, dofmask(1, 1, 1, 0, 1, 1), 1000, -1.2e-5, RX, 200),
    (True, 0, Z3, MPY, dofmask(1, 1, 1, 1, 0, 1), 1000, 3e-6, RY, 200),
    (True, 2, Z3, MPX, dofmask(1, 1, 1, 0, 1, 1), 1000, 3e-6, RX, 200),
    (True, 4, Z3, MPZ, dofmask(1, 1, 1, 1, 1, 0), 1000, 1.2e-5, RZ, 200),
    (True, 0, Z3, MPY, dofmask(1, 1, 0, 1, 0, 1), 1000, -6e-9, TZ, 300),
    (True, 0, FPY, Z3, dofmask(1, 0, 1, 1, 1, 0), 1000, 6e-3, RZ, 300),
    (False, 0, FPX, Z3, dofmask(0, 1, 1, 1, 1, 1), 1000, 5e-7, TX, 100),
    (False, 2, FPY, Z3, dofmask(1, 0, 1, 1, 1, 1), 1000, 5e-7, TY, 100),
    (False, 5, FPZ, Z3, dofmask(1, 1, 0, 1, 1, 1), 1000, 5e-7, TZ, 100),
    (False, 0, Z3, MPX, dofmask(1, 1, 1, 0, 1, 1), 1000, 6e-6, RX, 150),
    (False, 1, Z3, MPY, dofmask(1, 1, 1, 1, 0, 1), 1000, 6e-6, RY, 150),
    (False, 4, Z3, MPZ, dofmask(1, 1, 1, 1, 1, 0), 1000, 6e-6, RZ, 150),
]


def internal_damping(mk):  # tVoxelyze.h:261-286
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    v1 = s.set_voxel(m, 0, 0, 0)
    s.set_force(v1, 1e-6, 1e-6, 1e-6)
    for d in DIRS:
        s.set_fixed_all(s.set_voxel(m, *d))
    ts = s.recommended_time_step()
    s.do_time_steps(100, ts)
    return {"y": s.voxel_state()["pos"][v1][1], "sims": [s]}


def global_damping(mk):  # tVoxelyze.h:288-338
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 1.0)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 0.0)
    v1 = s.set_voxel(m, 0, 0, 0)
    s.set_force(v1, 1e-6, 1e-6, 1e-6)
    for d in DIRS:
        s.set_fixed_all(s.set_voxel(m, *d))
    ts = s.recommended_time_step()
    s.do_time_steps(100, ts)
    p1 = s.voxel_state()["pos"][v1].copy()
    s2 = mk(0.001)
    m2 = s2.add_material(1e6, 1e3)
    s2.material_set(m2, F.PROP_ZETA_GLOBAL, 0.25)
    s2.material_set(m2, F.PROP_ZETA_INTERNAL, 0.0)
    s2.set_fixed_all(s2.set_voxel(m2, 0, 0, 0))
    v22 = s2.set_voxel(m2, 1, 0, 0)
    s2.set_force(v22, 1e-6, 1e-6, 1e-6)
    ts = s2.recommended_time_step()
    s2.do_time_steps(300, ts)
    return {"p1": p1, "y2": s2.voxel_state()["pos"][v22][1], "sims": [s, s2]}


def combined_damping(mk):  # tVoxelyze.h:340-379
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    for i in range(4):
        for j in range(3):
            for k in range(3):
                v = s.set_voxel(m, i, j, k)
                if i == 0:
                    s.set_fixed_all(v)
                elif i == 3:
                    s.set_force(v, 0, 0, 1e-6)
    out = []
    for i in range(2):
        s.material_set(m, F.PROP_ZETA_GLOBAL, np.float32(0.05) + np.float32(0.05) * i)
        ts = s.recommended_time_step()
        s.reset_time()
        s.do_time_steps(1000, ts)
        out.append(s.voxel_state()["pos"][s.voxel_index(3, 0, 0)][2])
    return {"z": out, "sims": [s]}


def frequency(mk):  # tVoxelyze.h:415-443
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 0.0)
    v1 = s.set_voxel(m, 0, 0, 0)
    v2 = s.set_voxel(m, 1, 0, 0)
    s.set_fixed_all(v1)
    s.set_fixed(v2, dofmask(0, 1, 1, 1, 1, 1))
    s.set_force(v2, 1e-3, 0, 0)
    ts = np.float32(s.recommended_time_step() / np.float32(10))
    data = []
    for _ in range(1000):
        s.do_time_step(ts)
        data.append(s.voxel_state()["pos"][v2][0] - 0.001001)
    zc = []
    for i in range(1, len(data)):
        if (data[i - 1] <= 0 < data[i]) or (data[i - 1] >= 0 > data[i]):
            zc.append(ts * ((i - 1) + data[i - 1] / (data[i - 1] - data[i])))
    period = float(np.mean(np.diff(zc)) * 2) if len(zc) > 1 else -1.0
    return {"period": period, "sims": [s]}


def large_deformation_damping(mk):  # tVoxelyze.h:445-470
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.2)
    v1 = s.set_voxel(m, 0, 0, 0)
    v2 = s.set_voxel(m, 1, 0, 0)
    ts = s.recommended_time_step()
    s.set_fixed_all(v1)
    s.set_force(v2, -0.2, 0.0, 0.2)
    s.do_time_steps(200, ts)
    return {"z": s.voxel_state()["pos"][v2][2], "sims": [s]}


def multi_simple2(mk):  # tVoxelyze.h:649-684
    s = mk(0.001)
    m1 = s.add_material(1e6, 1e3)
    m2 = s.add_material(1e9, 1e3)
    for m in (m1, m2):
        s.material_set(m, F.PROP_ZETA_GLOBAL, 0.01)
        s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    for i in range(8):
        v = s.set_voxel(m1 if (i // 2) % 2 == 0 else m2, i, 0, 0)
        if i == 0:
            s.set_fixed_all(v)
        if i == 7:
            s.set_force(v, 1e-3, 0, 0)
    ts = s.recommended_time_step()
    s.do_time_steps(10000, ts)
    return {"x": s.voxel_state()["pos"][s.voxel_index(7, 0, 0)][0] - 0.007, "sims": [s]}


def poissons_large(mk):  # tVoxelyze.h:715-768
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_POISSON, 0.3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.2)
    for i in range(9):
        for j in range(2):
            for k in range(2):
                v = s.set_voxel(m, i, j, k)
                if i == 0:
                    s.set_fixed_all(v)
                if i == 8:
                    s.set_displacement_all(v, (float(np.float32(1e-3)), 0.0, 0.0))
    ts = s.recommended_time_step()
    s.do_time_steps(300, ts)
    # strain of the middle voxel from its corner offset (tVoxelyze.h:752-757), and the x reaction
    # the four displaced voxels need against the stress sigma_x over the voxel's deformed cross
    # section (:759-768), all in float as the reference computes them
    f32 = np.float32
    mid = s.voxel_index(4, 0, 0)
    size = f32(2) * s.corner_offset(mid, 7)
    strain = (size - f32(0.001)) / f32(0.001)
    mu = f32(0.3)
    e_hat = f32(1e6) / ((f32(1) - f32(2) * mu) * (f32(1) + mu))
    sigma_x = e_hat * ((f32(1) - mu) * strain[0] + mu * (strain[1] + strain[2]))
    size2 = s.corner_offset(mid, 7) - s.corner_offset(mid, 0)
    f_x = sigma_x * f32(4) * size2[1] * size2[2]
    total = f32(0)
    for j in range(2):
        for k in range(2):
            total = total + s.external_force(s.voxel_index(8, j, k))[0]
    return {"x": s.voxel_state()["pos"][mid][0] - 0.004, "strain": strain, "reaction_x": float(total),
            "stress_force_x": float(f_x), "sims": [s]}


def poissons_small(mk):  # tVoxelyze.h:689-711
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.material_set(m, F.PROP_POISSON, 0.3)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.3)
    for i in range(3):
        v = s.set_voxel(m, i, 0, 0)
        if i == 0:
            s.set_fixed_all(v)
        if i == 2:
            s.set_force(v, 1e-3, 0, 0)
    ts = s.recommended_time_step()
    s.do_time_steps(200, ts)
    return {"x": s.voxel_state()["pos"][2][0] - 0.002, "sims": [s]}


def deformable_material(mk):  # tVoxelyze.h:845-891
    s = mk(0.001)
    m = s.add_material(1e6, 1e3)
    s.set_model_bilinear(m, 1e6, 5e5, 1e5)
    s.material_set(m, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.2)
    for i in range(5):
        for j in range(3):
            for k in range(3):
                v = s.set_voxel(m, i, j, k)
                if i == 0:
                    s.set_fixed_all(v)
                if i == 4:
                    s.set_force(v, 0.2, 0.0, 0.0)
    ts = s.recommended_time_step()
    s.do_time_steps(400, ts)
    for j in range(3):
        for k in range(3):
            s.set_force(s.voxel_index(4, j, k), 0.0, 0.0, 0.0)
    s.do_time_steps(250, ts)
    return {"x": s.voxel_state()["pos"][s.voxel_index(4, 1, 1)][0] - 0.004, "sims": [s]}


def temperature(mk):  # tVoxelyze.h:989-1032
    s = mk(0.001)
    m1 = s.add_material(1e6, 1e3)
    s.material_set(m1, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m1, F.PROP_ZETA_GLOBAL, 0.15)
    s.material_set(m1, F.PROP_CTE, 0.01)
    m2 = s.add_material(1e7, 1e3)
    s.material_set(m2, F.PROP_ZETA_INTERNAL, 1.0)
    s.material_set(m2, F.PROP_ZETA_GLOBAL, 0.15)
    for i in range(3):
        a = s.set_voxel(m1, i, 0, 0)
        b = s.set_voxel(m2, i, 0, 1)
        if i == 0:
            s.set_fixed_all(a)
            s.set_fixed_all(b)
    s.set_ambient_temperature(5, True)
    ts = s.recommended_time_step()
    s.do_time_steps(500, ts)
    z1 = s.voxel_state()["pos"][s.voxel_index(2, 0, 0)][2]
    s.reset_time()
    s.set_ambient_temperature(-5, True)
    s.do_time_steps(500, ts)
    z2 = s.voxel_state()["pos"][s.voxel_index(2, 0, 0)][2]
    return {"z1": z1, "z2": z2, "sims": [s]}


def static_friction(mk):  # tVoxelyze.h:1034-1110
    """Six cases on one voxel resting on the floor: a horizontal force just below and just above
    mu_s times the normal force, at 1 g, at 2 g, and at 1 g with mu_s = 2 (in that order, on the
    same simulator, with resetTime between cases as the reference test does)."""
    vsize, density = 0.001, 1e3
    s = mk(vsize)
    s.enable_floor(True)
    s.set_gravity(1.0)
    m = s.add_material(1e6, density)
    normal = float(np.float32(density * vsize ** 3 * 9.80665))
    v = s.set_voxel(m, 0, 0, 0)
    s.material_set(m, F.PROP_MU_STATIC, 1.0)
    s.material_set(m, F.PROP_MU_KINETIC, 0.1)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 1.0)
    ts = s.recommended_time_step()
    xs = []
    for gravity, mu_s, factors in ((1.0, None, (0.9, 1.1)), (2.0, None, (1.9, 2.1)), (1.0, 2.0, (1.9, 2.1))):
        if gravity != 1.0 or mu_s is not None:
            s.set_gravity(gravity)
        if mu_s is not None:
            s.material_set(m, F.PROP_MU_STATIC, mu_s)
        for factor in factors:
            s.do_time_steps(50, ts)
            s.set_force(v, float(np.float32(factor) * np.float32(normal)), 0.0, 0.0)
            s.do_time_steps(10, ts)
            xs.append(s.voxel_state()["pos"][v][0])
            s.set_force(v, 0.0, 0.0, 0.0)
            s.reset_time()
    return {"x_below": xs[0::2], "x_above": xs[1::2], "sims": [s]}


def collisions(mk):  # tVoxelyze.h:1169-1197
    s = mk(0.001)
    s.enable_floor(True)
    s.set_gravity(1.0)
    m = s.add_material(1e6, 1e6)
    s.material_set(m, F.PROP_ZETA_GLOBAL, 0.0)
    v1 = s.set_voxel(m, 0, 0, 0)
    s.set_fixed_all(v1)
    v2 = s.set_voxel(m, 0, 0, 2)
    s.enable_collisions(True)
    ts = s.recommended_time_step()
    s.do_time_steps(150, ts)
    return {"z": s.voxel_state()["pos"][v2][2], "sims": [s]}


def float_eq(a, b, ulps=4):
    """gtest's EXPECT_FLOAT_EQ: the two values as floats are within 4 ulps."""
    def key(x):
        i = int(np.array(np.float32(x)).view(np.int32))
        return i if i >= 0 else -(i & 0x7FFFFFFF)
    return abs(key(a) - key(b)) <= ulps


def check_expectations(name, r):
    """The reference test's assertions for each KAT."""
    if name == "internal_damping":
        assert float_eq(r["y"], np.float32(1e-9) / np.float32(6))
    elif name == "global_damping":
        assert all(float_eq(p, np.float32(1e-9) / np.float32(6)) for p in r["p1"])
        assert float_eq(r["y2"], 4e-9)
    elif name == "combined_damping":
        for z in r["z"]:
            assert abs(1.742e-8 - z) <= 1e-10
    elif name == "frequency":
        expected = 2 * 3.1415926 / np.sqrt(1e9)
        assert abs(expected - r["period"]) <= expected / 1000
    elif name == "large_deformation_damping":
        assert abs(9.5587e-4 - r["z"]) <= 1e-7
    elif name == "multi_simple2":
        assert abs(3.5035e-6 - float(np.float32(r["x"]))) <= 1e-10
    elif name == "poissons_large":
        assert abs(5e-4 - float(np.float32(r["x"]))) <= 1e-7
        assert abs(1.306e-1 - r["strain"][0]) <= 1e-3
        assert abs(-4.048e-2 - r["strain"][1]) <= 1e-5
        assert abs(-4.048e-2 - r["strain"][2]) <= 1e-5
        assert abs(r["reaction_x"] - r["stress_force_x"]) <= 0.01
    elif name == "deformable_material":
        assert abs(4e-4 - float(np.float32(r["x"]))) <= 1e-7
    elif name == "temperature":
        assert abs(2.55e-5 - r["z1"]) <= 1e-8
        assert abs(-2.591e-5 - r["z2"]) <= 1e-8
    elif name == "static_friction":
        assert len(r["x_below"]) == len(r["x_above"]) == 3
        assert all(x == 0.0 for x in r["x_below"])
        assert all(x != 0.0 for x in r["x_above"])
    elif name == "collisions":
        assert r["z"] > 0.001


KATS = {
    "internal_damping": internal_damping,
    "global_damping": global_damping,
    "combined_damping": combined_damping,
    "frequency": frequency,
    "large_deformation_damping": large_deformation_damping,
    "multi_simple2": multi_simple2,
    "poissons_small": poissons_small,
    "poissons_large": poissons_large,
    "deformable_material": deformable_material,
    "temperature": temperature,
    "static_friction": static_friction,
    "collisions": collisions,
}
