"""Adjoint gradients of the body centre-of-mass objective against central finite differences.

Scenes are multi-body scenes with one material per voxel and per-voxel actuation phases (the
temperature of voxel v before each step is amplitude * sin(2 pi frequency t + phase[v])), as
``scenes.graded_population`` builds them.  The objective is the sum over bodies of the mass-weighted
centre-of-mass x after ``nsteps`` steps (``vxg_adjoint_com_x``).  Bodies are independent, so one
voxel per body can be perturbed in the same run and each body's centre of mass gives that voxel's
difference quotient.  Denominators use the float values the materials and phases actually hold:
the reference stores E as a float and rounds (1 + temperature * CTE) and the stresses to float, so a
relative step much below ~1e-4 measures that rounding rather than the derivative.
"""
from __future__ import annotations

import copy

import numpy as np

from . import facade as F
from . import scenes as S


def body_offsets(scene) -> np.ndarray:
    return np.concatenate([[0], np.cumsum(np.bincount(scene.body))]).astype(np.int32)


def build(lib, scene, phase, amplitude: float, frequency: float):
    """A product-library simulator of ``scene`` with per-voxel actuation; returns (sim, engine)."""
    sim = F.Sim(lib, "vx", scene.voxel_size)
    S.apply(scene, sim)
    eng = F.Engine(sim)
    eng.set_actuation(F.ACT_PER_VOXEL, amplitude, frequency, phase)
    return sim, eng


def body_com_x(lib, scene, phase, nsteps: int, dt: float, off, amplitude: float, frequency: float) -> np.ndarray:
    sim, eng = build(lib, scene, phase, amplitude, frequency)
    sim.recommended_time_step()
    if sim.do_time_steps(nsteps, dt) != nsteps:
        raise RuntimeError("the run diverged")
    return eng.body_com(off)[:, 0]


def central_differences(lib, scene, pick, nsteps, dt, off, rel_step, phase_step, amplitude, frequency):
    """d(body centre-of-mass x)/d(parameter) for each (body, voxel, kind) in ``pick`` (kind "E",
    "rho" or "phase"; at most one voxel per body), by central differences."""
    coms, vals = [], []
    for sign in (+1, -1):
        s2 = copy.deepcopy(scene)
        ph = scene.phase.copy()
        realized = []
        for _, v, kind in pick:
            if kind == "E":
                s2.materials[v].E = float(np.float32(scene.materials[v].E * (1 + sign * rel_step)))
                realized.append(s2.materials[v].E)
            elif kind == "rho":
                s2.materials[v].rho = float(np.float32(scene.materials[v].rho * (1 + sign * rel_step)))
                realized.append(s2.materials[v].rho)
            else:
                ph[v] = np.float32(ph[v] + sign * phase_step)
                realized.append(float(ph[v]))
        coms.append(body_com_x(lib, s2, ph, nsteps, dt, off, amplitude, frequency))
        vals.append(realized)
    return np.array([(coms[0][b] - coms[1][b]) / (vals[0][i] - vals[1][i]) for i, (b, _, _) in enumerate(pick)])


def compare(adjoint, fd_h, fd_h4, smooth_spread: float = 0.1):
    """Per parameter: the adjoint's distance to the interval spanned by the differences at steps h
    and h/4, relative to the largest of the three magnitudes, and whether the two differences agree
    within ``smooth_spread`` (where they do not, a friction latch or contact decision changed
    between the perturbed runs: the objective is not smooth at that scale and the difference
    crosses a branch the adjoint does not follow)."""
    out = []
    for ad, f1, f2 in zip(adjoint, fd_h, fd_h4):
        scale = max(abs(f1), abs(f2), abs(ad), 1e-300)
        lo, hi = min(f1, f2), max(f1, f2)
        out.append({"adjoint": float(ad), "fd_h": float(f1), "fd_h4": float(f2),
                    "smooth": abs(f1 - f2) <= smooth_spread * scale,
                    "distance": max(lo - ad, ad - hi, 0.0) / scale})
    return out


def check(lib, scene, nsteps: int, checkpoint_every: int, pick, rel_step: float, phase_step: float,
          amplitude: float = 0.1, frequency: float = 2.0):
    """Adjoint of the run against central differences at steps h and h/4 for the parameters in
    ``pick``; returns (rows as in ``compare``, objective, adjoint seconds, dt)."""
    import time

    off = body_offsets(scene)
    sim, eng = build(lib, scene, scene.phase, amplitude, frequency)
    dt = sim.recommended_time_step()
    t0 = time.perf_counter()
    obj, gE, gR, gP = eng.adjoint_com_x(nsteps, dt, off, checkpoint_every=checkpoint_every)
    t_adj = time.perf_counter() - t0
    if not np.array_equal(obj, body_com_x(lib, scene, scene.phase, nsteps, dt, off, amplitude, frequency)):
        raise AssertionError("the differentiated run differs from the plain run")
    grads = {"E": gE, "rho": gR, "phase": gP}
    ad = [grads[kind][v] for _, v, kind in pick]
    fd1 = central_differences(lib, scene, pick, nsteps, dt, off, rel_step, phase_step, amplitude, frequency)
    fd2 = central_differences(lib, scene, pick, nsteps, dt, off, rel_step / 4, phase_step / 4, amplitude, frequency)
    return compare(ad, fd1, fd2), obj, t_adj, dt
