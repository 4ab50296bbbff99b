"""Adjoint of the FP64 time step (vxg_adjoint_com_x) against central finite differences.

Scene: bodies with one material per voxel (E log-uniform in [3e5, 3e6] Pa, density 1000, CTE 0.01,
friction 1.0/0.5), floor and gravity, per-voxel actuation phase (temperature 0.1 sin(2 pi 2 t +
phase) every step).  Objective: the sum over bodies of the mass-weighted centre-of-mass x after the
run.  Bodies are independent, so one voxel per body is perturbed in the same run and each body's
centre of mass gives that voxel's difference quotient; denominators use the float values the
materials and phases actually hold.  Steps are 1e-3 relative for E and density and 1e-2 rad for the
phase (and a quarter of each): the reference's arithmetic rounds (1 + temperature * CTE) and the
stresses to float, so much smaller steps measure that rounding rather than the derivative.
"""
from __future__ import annotations

import copy

import numpy as np
import pytest

from conftest import make_sim
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu

AMP, FREQ = 0.1, 2.0


def _offsets(sc):
    return np.concatenate([[0], np.cumsum(np.bincount(sc.body))]).astype(np.int32)


def _build(product_lib, sc, phase):
    g = make_sim(product_lib, "vx", sc)
    eng = F.Engine(g)
    eng.set_actuation(F.ACT_PER_VOXEL, AMP, FREQ, phase)
    return g, eng


def _run_com(product_lib, sc, phase, nsteps, dt, off):
    g, eng = _build(product_lib, sc, phase)
    g.recommended_time_step()
    assert g.do_time_steps(nsteps, dt) == nsteps
    return eng.body_com(off)[:, 0]


def _fd(product_lib, sc, pick, nsteps, dt, off, rel_step, phase_step):
    """Central differences of every body's centre-of-mass x, one perturbed voxel per body."""
    coms, vals = [], []
    for sign in (+1, -1):
        s2 = copy.deepcopy(sc)
        ph = sc.phase.copy()
        realized = []
        for b, v, kind in pick:
            if kind == "E":
                s2.materials[v].E = float(np.float32(sc.materials[v].E * (1 + sign * rel_step)))
                realized.append(s2.materials[v].E)
            elif kind == "rho":
                s2.materials[v].rho = float(np.float32(sc.materials[v].rho * (1 + sign * rel_step)))
                realized.append(s2.materials[v].rho)
            else:
                ph[v] = np.float32(ph[v] + sign * phase_step)
                realized.append(float(ph[v]))
        coms.append(_run_com(product_lib, s2, ph, nsteps, dt, off))
        vals.append(realized)
    return np.array([(coms[0][b] - coms[1][b]) / (vals[0][i] - vals[1][i]) for i, (b, v, kind) in enumerate(pick)])


def _fd_check(product_lib, sc, nsteps, K, rel_step, phase_step, tol, seed=0, min_smooth=0.6):
    """Adjoint against central differences at two steps, h and h/4.  Where the two differences
    disagree by more than 10 % the objective is not smooth at that scale (a friction latch or contact
    decision changed between the perturbed runs, so the difference crosses a branch the adjoint does
    not follow); those parameters are reported and left out.  For every other parameter the adjoint
    must lie within tol (relative) of the interval spanned by the two differences, whose spread is
    the differences' own rounding noise."""
    off = _offsets(sc)
    nb = len(off) - 1
    g, eng = _build(product_lib, sc, sc.phase)
    dt = g.recommended_time_step()
    obj, gE, gR, gP = eng.adjoint_com_x(nsteps, dt, off, checkpoint_every=K)
    # the differentiated run is the plain run
    assert np.array_equal(obj, _run_com(product_lib, sc, sc.phase, nsteps, dt, off))
    rng = np.random.default_rng(seed)
    kinds = ["E", "rho", "phase"]
    pick = [(b, int(rng.integers(off[b], off[b + 1])), kinds[b % 3]) for b in range(nb)]
    fd1 = _fd(product_lib, sc, pick, nsteps, dt, off, rel_step, phase_step)
    fd2 = _fd(product_lib, sc, pick, nsteps, dt, off, rel_step / 4, phase_step / 4)
    errs = []
    for i, (b, v, kind) in enumerate(pick):
        ad = {"E": gE, "rho": gR, "phase": gP}[kind][v]
        scale = max(abs(fd1[i]), abs(fd2[i]), abs(ad), 1e-300)
        smooth = abs(fd1[i] - fd2[i]) <= 0.1 * scale
        lo, hi = min(fd1[i], fd2[i]), max(fd1[i], fd2[i])
        err = max(lo - ad, ad - hi, 0.0) / scale
        if smooth:
            errs.append(err)
        print("body %3d voxel %5d d/d%-5s fd(h) % .6e fd(h/4) % .6e adjoint % .6e dist %.2e%s"
              % (b, v, kind, fd1[i], fd2[i], ad, err, "" if smooth else "  (crosses a branch: left out)"))
    print(f"{len(errs)} of {len(pick)} parameters smooth; adjoint distance to the differences: "
          f"worst {max(errs):.3e}, median {float(np.median(errs)):.3e} ({nsteps} steps, checkpoint every {K})")
    assert len(errs) >= min_smooth * len(pick)
    assert max(errs) <= tol


def test_adjoint_small_population(product_lib):
    """6 bodies of 5^3 cells, 300 steps, checkpoints every 64 steps (five recomputed segments)."""
    sc = S.graded_population(6, 5, 0.7, seed=11)
    _fd_check(product_lib, sc, nsteps=300, K=64, rel_step=1e-3, phase_step=1e-2, tol=2e-3)


def test_adjoint_longer_horizon_more_bodies(product_lib):
    """12 bodies of 8^3 cells, 1,000 steps, checkpoints every 100."""
    sc = S.graded_population(12, 8, 0.7, seed=12)
    _fd_check(product_lib, sc, nsteps=1000, K=100, rel_step=1e-3, phase_step=1e-2, tol=2e-3, seed=1)


def test_adjoint_rejects_out_of_scope(product_lib):
    sc = S.graded_population(2, 4, 0.7, seed=3)
    sc.materials[0].nu = 0.3
    g, eng = _build(product_lib, sc, sc.phase)
    dt = g.recommended_time_step()
    with pytest.raises(RuntimeError, match="Poisson"):
        eng.adjoint_com_x(10, dt, _offsets(sc), checkpoint_every=5)
