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


def body_com_x(lib, scene, phase, nsteps: int, dt: float, off, amplitude: float, frequency: float,
               decisions=None, record: bool = False):
    """Per-body centre-of-mass x after the run.  ``record``: also return the run's floor-contact
    and static-friction decisions (vxg_set_decisions); ``decisions``: take those branches instead of
    deciding (a perturbed run that follows a recorded one)."""
    sim, eng = build(lib, scene, phase, amplitude, frequency)
    sim.recommended_time_step()
    if record:
        eng.set_decisions(1, nsteps)
    elif decisions is not None:
        eng.set_decisions(2, nsteps)
        eng.put_decisions(decisions)
    if sim.do_time_steps(nsteps, dt) != nsteps:
        raise RuntimeError("the run diverged")
    com = eng.body_com(off)[:, 0]
    return (com, eng.decisions(nsteps)) if record else com


def central_differences(lib, scene, pick, nsteps, dt, off, rel_step, phase_step, amplitude, frequency,
                        decisions=None):
    """d(body centre-of-mass x)/d(parameter) for each (body, voxel, kind) in ``pick`` (kind "E",
    "rho" or "phase"; at most one voxel per body), by central differences; with ``decisions`` both
    perturbed runs take the recorded run's contact and friction branches."""
    coms, vals = [], []
    for sign in (+1, -1):
        s2 = copy.deepcopy(scene)
        ph = scene.phase.copy()
        realized = []
        for _, v, kind in pick:
            if kind == "E":
                m = s2.materials[v]
                m.E = float(np.float32(scene.materials[v].E * (1 + sign * rel_step)))
                if m.model is not None and m.model[0] == "linear":  # setModelLinear(E, failure stress)
                    m.model = ("linear", m.E) + tuple(m.model[2:])
                realized.append(m.E)
            elif kind == "rho":
                s2.materials[v].rho = float(np.float32(scene.materials[v].rho * (1 + sign * rel_step)))
                realized.append(s2.materials[v].rho)
            else:
                ph[v] = np.float32(ph[v] + sign * phase_step)
                realized.append(float(ph[v]))
        coms.append(body_com_x(lib, s2, ph, nsteps, dt, off, amplitude, frequency, decisions=decisions))
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
        # Richardson extrapolation of the two central differences: their O(h^2) truncation
        # cancels, (16 D(h/4) - D(h)) / 15
        rich = (16.0 * f2 - f1) / 15.0
        out.append({"adjoint": float(ad), "fd_h": float(f1), "fd_h4": float(f2),
                    "smooth": abs(f1 - f2) <= smooth_spread * scale,
                    "distance": max(lo - ad, ad - hi, 0.0) / scale,
                    "richardson": float(rich), "richardson_error": abs(rich - ad) / max(abs(ad), 1e-300)})
    return out


def adjoint(lib, scene, nsteps: int, checkpoint_every: int, pick, amplitude: float = 0.1, frequency: float = 2.0):
    """The adjoint gradients of the parameters in ``pick``; returns (their values, objective,
    adjoint seconds, dt, the plain run's branch decisions).  The plain run, stepped separately with
    its decisions recorded, must reproduce the differentiated run's objective bit for bit."""
    import time

    off = body_offsets(scene)
    sim, eng = build(lib, scene, scene.phase, amplitude, frequency)
    dt = sim.recommended_time_step()
    t0 = time.perf_counter()
    obj, gE, gR, gP = eng.adjoint_com_x(nsteps, dt, off, checkpoint_every=checkpoint_every)
    t_adj = time.perf_counter() - t0
    base, dec = body_com_x(lib, scene, scene.phase, nsteps, dt, off, amplitude, frequency, record=True)
    if not np.array_equal(obj, base):
        raise AssertionError("the differentiated run differs from the plain run")
    grads = {"E": gE, "rho": gR, "phase": gP}
    return [grads[kind][v] for _, v, kind in pick], obj, t_adj, dt, dec


def differences(lib, scene, pick, nsteps: int, dt: float, ad, rel_step: float, phase_step: float,
                amplitude: float = 0.1, frequency: float = 2.0, decisions=None):
    """``compare`` rows of the adjoint values ``ad`` against central differences at steps h and
    h/4; with ``decisions`` (the plain run's) the perturbed runs follow its branches."""
    off = body_offsets(scene)
    fd1 = central_differences(lib, scene, pick, nsteps, dt, off, rel_step, phase_step, amplitude, frequency,
                              decisions)
    fd2 = central_differences(lib, scene, pick, nsteps, dt, off, rel_step / 4, phase_step / 4, amplitude,
                              frequency, decisions)
    return compare(ad, fd1, fd2)


def check(lib, scene, nsteps: int, checkpoint_every: int, pick, rel_step: float, phase_step: float,
          amplitude: float = 0.1, frequency: float = 2.0, frozen: bool = False):
    """Adjoint of the run against central differences at steps h and h/4 for the parameters in
    ``pick``; returns (rows as in ``compare``, objective, adjoint seconds, dt).  ``frozen``: the
    perturbed runs replay the unperturbed run's floor-contact and static-friction decisions, so the
    differences measure the derivative along the branches the adjoint follows; decisions flipping
    elsewhere in a body no longer enter them."""
    ad, obj, t_adj, dt, dec = adjoint(lib, scene, nsteps, checkpoint_every, pick, amplitude, frequency)
    if frozen and not np.array_equal(obj, body_com_x(lib, scene, scene.phase, nsteps, dt, body_offsets(scene),
                                                     amplitude, frequency, decisions=dec)):
        raise AssertionError("replaying a run's own decisions changes it")
    rows = differences(lib, scene, pick, nsteps, dt, ad, rel_step, phase_step, amplitude, frequency,
                       dec if frozen else None)
    return rows, obj, t_adj, dt
