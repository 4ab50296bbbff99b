"""Central differences of the body centre-of-mass objective (the gradient workload's) taken with
the REFERENCE build, as a fixture.

The objective is a body's mass-weighted centre-of-mass x after `nsteps` steps, with each voxel's
temperature set before every step to amplitude * sin(2 pi frequency t + phase[v]) through
CVX_Voxel::setTemperature (src/VX_Voxel.cpp:108-114; t = currentTime, the sine the C library's),
one material per voxel, floor, friction and gravity (the differentiation configuration on one small
body).  The reference library compiled from its own sources (oracle/_ref/libvxref.so, made by
oracle/build_ref.sh) takes the steps; its sources exist only where the fixture is generated, so the
GPU test that checks the adjoint against these differences reads the committed fixture.

For each picked parameter (a voxel's Young's modulus, density or phase) two central differences are
taken, at step h and h/4 (E and density 1.6e-2 relative, phase 0.04 rad), with the perturbed values
held as the reference holds them (E and density as floats) and those realised floats in the
denominators; (16 D(h/4) - D(h)) / 15 (Richardson) removes their h^2 truncation.  The reference's
floor contact and static-friction latch are branches: a perturbed run can take another branch
somewhere in the body, which the differences then measure; smaller phase steps make that rarer.

    python tests/golden/make_adjoint_ref_fd.py      # writes tests/golden/adjoint_ref_fd.npz
"""
from __future__ import annotations

import ctypes as C
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from voxelyze_gb300 import facade as F, scenes as S  # noqa: E402

NSTEPS = 400
AMPLITUDE, FREQUENCY = 0.1, 2.0
E_STEP, RHO_STEP, PHASE_STEP = 1.6e-2, 1.6e-2, 0.04


def scene():
    """One body of 6^3 cells at occupancy 0.7 (largest component), the differentiation
    configuration's materials and actuation."""
    return S.graded_population(n_bodies=1, side=6, occupancy=0.7, seed=21)


def mass_of(rho, s):  # CVX_MaterialVoxel::updateDerived, src/VX_MaterialVoxel.cpp:61-62
    return np.float32((s * s * s) * float(np.float32(rho)))


def com_x(lib, sc, E, rho, phase, dt):
    """Centre-of-mass x after NSTEPS reference steps of the actuated scene."""
    sim = F.Sim(lib, "vxr", sc.voxel_size)
    for k in range(len(E)):
        m = sim.add_material(float(E[k]), float(rho[k]))
        mt = sc.materials[k]
        sim.material_set(m, F.PROP_CTE, mt.cte)
        sim.material_set(m, F.PROP_MU_STATIC, mt.mu_static)
        sim.material_set(m, F.PROP_MU_KINETIC, mt.mu_kinetic)
    sim.set_gravity(sc.gravity)
    sim.enable_floor(True)
    sim.set_voxels(sc.mats, sc.xyz)
    set_t = sim.f["voxel_set_temperature"]
    n = len(E)
    ph = [float(p) for p in phase]
    for _ in range(NSTEPS):
        t = float(sim.current_time())
        base = 2.0 * 3.141592653589793 * FREQUENCY * t
        for v in range(n):
            set_t(sim.h, v, float(np.float32(AMPLITUDE * math.sin(base + ph[v]))))
        assert sim.do_time_step(dt)
    x = sim.voxel_state()["pos"][:, 0]
    m = np.array([mass_of(r, sc.voxel_size) for r in rho], np.float64)
    return float((m * x).sum() / m.sum())


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvxref.so"))
    sc = scene()
    n = sc.n_voxels
    E0 = np.array([m.E for m in sc.materials], np.float32)
    rho0 = np.array([m.rho for m in sc.materials], np.float32)
    ph0 = sc.phase.astype(np.float32)
    probe = F.Sim(lib, "vxr", sc.voxel_size)
    S.apply(sc, probe)
    dt = probe.recommended_time_step()
    base = com_x(lib, sc, E0, rho0, ph0, dt)
    rng = np.random.default_rng(7)
    voxels = rng.choice(n, size=24, replace=False)
    picks = [(int(v), "E") for v in voxels[:10]] + [(int(v), "phase") for v in voxels[10:20]] + \
            [(int(v), "rho") for v in voxels[20:]]
    rows = []
    for v, kind in picks:
        d = []
        for scale in (1.0, 0.25):
            vals, objs = [], []
            for sign in (+1, -1):
                E, rho, ph = E0.copy(), rho0.copy(), ph0.copy()
                if kind == "E":
                    E[v] = np.float32(E0[v] * (1 + sign * E_STEP * scale)); vals.append(float(E[v]))
                elif kind == "rho":
                    rho[v] = np.float32(rho0[v] * (1 + sign * RHO_STEP * scale)); vals.append(float(rho[v]))
                else:
                    ph[v] = np.float32(ph0[v] + sign * PHASE_STEP * scale); vals.append(float(ph[v]))
                objs.append(com_x(lib, sc, E, rho, ph, dt))
            d.append((objs[0] - objs[1]) / (vals[0] - vals[1]))
        rows.append((d[0], d[1], (16.0 * d[1] - d[0]) / 15.0))
        print(f"voxel {v:4d} {kind:5s}: D(h) {d[0]: .6e}  D(h/4) {d[1]: .6e}  Richardson {rows[-1][2]: .6e}")
    out = os.path.join(HERE, "adjoint_ref_fd.npz")
    np.savez_compressed(out, xyz=sc.xyz, E=E0, rho=rho0, phase=ph0, dt=np.float32(dt), nsteps=NSTEPS,
                        amplitude=AMPLITUDE, frequency=FREQUENCY, objective=base,
                        pick_voxel=np.array([p[0] for p in picks], np.int32),
                        pick_kind=np.array([p[1] for p in picks]),
                        fd=np.array(rows, np.float64))
    print(f"{n} voxels, {NSTEPS} steps, dt {dt:.6e}, objective {base:.12e} -> {out}")


if __name__ == "__main__":
    main()
