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

import numpy as np
import pytest

from voxelyze_gb300 import gradcheck as G, scenes as S

pytestmark = pytest.mark.gpu

AMP, FREQ = 0.1, 2.0


def _fd_check(product_lib, sc, nsteps, K, rel_step, phase_step, tol, seed=0, min_smooth=0.6):
    """Adjoint against central differences at two steps, h and h/4 (voxelyze_gb300.gradcheck), one
    parameter per body cycling through E, density and phase.  Parameters whose two differences
    disagree by more than 10 % cross a branch and are reported and left out; every other adjoint
    must lie within tol (relative) of the interval spanned by the two differences, whose spread is
    the differences' own rounding noise."""
    off = G.body_offsets(sc)
    rng = np.random.default_rng(seed)
    kinds = ["E", "rho", "phase"]
    pick = [(b, int(rng.integers(off[b], off[b + 1])), kinds[b % 3]) for b in range(len(off) - 1)]
    rows, _, _, _ = G.check(product_lib, sc, nsteps, K, pick, rel_step, phase_step, AMP, FREQ)
    errs = []
    for (b, v, kind), r in zip(pick, rows):
        if r["smooth"]:
            errs.append(r["distance"])
        print("body %3d voxel %5d d/d%-5s fd(h) % .6e fd(h/4) % .6e adjoint % .6e dist %.2e%s"
              % (b, v, kind, r["fd_h"], r["fd_h4"], r["adjoint"], r["distance"],
                 "" if r["smooth"] else "  (crosses a branch: left out)"))
    print(f"{len(errs)} of {len(pick)} parameters smooth; adjoint distance to the differences: "
          f"worst {max(errs):.3e}, median {float(np.median(errs)):.3e} ({nsteps} steps, checkpoint every {K})")
    assert len(errs) >= min_smooth * len(pick)
    assert max(errs) <= tol
    return errs


def test_adjoint_small_population(product_lib):
    """6 bodies of 5^3 cells, 300 steps, checkpoints every 64 steps (five recomputed segments)."""
    sc = S.graded_population(6, 5, 0.7, seed=11)
    _fd_check(product_lib, sc, nsteps=300, K=64, rel_step=1e-3, phase_step=1e-2, tol=2e-3)


def test_adjoint_longer_horizon_more_bodies(product_lib):
    """12 bodies of 8^3 cells, 1,000 steps, checkpoints every 100."""
    sc = S.graded_population(12, 8, 0.7, seed=12)
    _fd_check(product_lib, sc, nsteps=1000, K=100, rel_step=1e-3, phase_step=1e-2, tol=2e-3, seed=1)


def test_adjoint_gradient_workload_horizon(product_lib):
    """The gradient workload's bodies and horizon on a quarter of its 256 bodies: 64 bodies of 16^3 cells
    (occupancy 0.7), 2,000 steps with floor, friction and gravity, checkpoints every 100 steps; E
    and phase of one voxel in each of 32 bodies.  Over this horizon contact and friction decisions
    make some differences non-smooth at any usable step, so the bound is on the median distance
    (1e-4) and the 90th percentile (1e-2) of the smooth ones."""
    sc = S.graded_population(64, 16, 0.7)
    off = G.body_offsets(sc)
    rng = np.random.default_rng(7)
    bodies = rng.choice(64, size=32, replace=False)
    pick = [(int(b), int(rng.integers(off[b], off[b + 1])), "E" if i % 2 == 0 else "phase")
            for i, b in enumerate(bodies)]
    rows, _, t_adj, _ = G.check(product_lib, sc, 2000, 100, pick, 1e-3, 1e-2, AMP, FREQ)
    d = np.array([r["distance"] for r in rows if r["smooth"]])
    print(f"2,000-step gradient horizon, {sc.n_voxels} voxels: adjoint {t_adj:.1f} s; {len(d)} of "
          f"{len(rows)} smooth; distance median {np.median(d):.2e}, 90th pct {np.percentile(d, 90):.2e}, "
          f"max {d.max():.2e}; within 1e-4: {np.mean(d <= 1e-4):.2f}")
    assert len(d) >= 0.75 * len(rows)
    assert np.median(d) <= 1e-4
    assert np.percentile(d, 90) <= 1e-2


def test_adjoint_against_frozen_decision_differences(product_lib):
    """12 bodies of 8^3 cells, 1,000 steps.  The perturbed runs replay the unperturbed run's
    floor-contact and static-friction decisions (vxg_set_decisions), so the differences measure the
    derivative along the branches the adjoint follows, and the O(h^2) truncation of the two central
    differences (h = 1.6e-2 relative for E and density, 0.16 rad for phases, and a quarter of each)
    is removed by Richardson extrapolation.  Every parameter then agrees with the adjoint; the
    remaining error is the differences' own noise from the float roundings of the reference's
    arithmetic (replaying a run's own decisions reproduces it bit for bit, checked first)."""
    sc = S.graded_population(12, 8, 0.7, seed=12)
    off = G.body_offsets(sc)
    rng = np.random.default_rng(1)
    kinds = ["E", "rho", "phase"]
    pick = [(b, int(rng.integers(off[b], off[b + 1])), kinds[b % 3]) for b in range(len(off) - 1)]
    rows, _, _, _ = G.check(product_lib, sc, 1000, 100, pick, 1.6e-2, 0.16, AMP, FREQ, frozen=True)
    err = np.array([r["richardson_error"] for r in rows])
    for (b, v, kind), r in zip(pick, rows):
        print("body %3d voxel %5d d/d%-5s adjoint % .6e extrapolated % .6e error %.2e"
              % (b, v, kind, r["adjoint"], r["richardson"], r["richardson_error"]))
    print(f"frozen decisions: error median {np.median(err):.2e}, max {err.max():.2e}")
    assert np.median(err) <= 1e-4
    assert err.max() <= 5e-4


def test_adjoint_with_partial_fixes(product_lib):
    """Externals that fix some degrees of freedom (CVX_External::setFixed, the fixes at the end of
    CVX_Voxel::timeStep): in each of 12 bodies of 8^3 cells three voxels are fixed in z
    translation, in x and y rotation, and in x translation with z rotation (the last through the
    rotation vector of the new orientation).  Frozen-decision central differences with Richardson
    extrapolation, 600 steps: the adjoint agrees with them as without fixes, per parameter (median)
    and as a gradient vector per kind."""
    sc = S.graded_population(12, 8, 0.7, seed=12)
    off = G.body_offsets(sc)
    rng = np.random.default_rng(2)
    idx, mask = [], []
    for b in range(len(off) - 1):
        vs = rng.choice(np.arange(off[b], off[b + 1]), 3, replace=False)
        idx += [int(x) for x in vs]
        mask += [4, 8 | 16, 1 | 32]
    sc.fixed_idx = np.array(idx, np.int64)
    sc.fixed_mask = np.array(mask, np.int64)
    kinds = ["E", "rho", "phase"]
    pick = [(b, int(rng.integers(off[b], off[b + 1])), kinds[b % 3]) for b in range(len(off) - 1)]
    rows, _, _, _ = G.check(product_lib, sc, 600, 100, pick, 1.6e-2, 0.16, AMP, FREQ, frozen=True)
    err = np.array([r["richardson_error"] for r in rows])
    for (b, v, kind), r in zip(pick, rows):
        print("body %3d voxel %5d d/d%-5s adjoint % .6e extrapolated % .6e error %.2e"
              % (b, v, kind, r["adjoint"], r["richardson"], r["richardson_error"]))
    print(f"partial fixes, frozen decisions: error median {np.median(err):.2e}, max {err.max():.2e}")
    assert np.median(err) <= 1e-4
    # per kind as a gradient vector, in the 2-norm and the max-norm (the smallest gradients sit in
    # the differences' float-rounding noise, so their own relative error says little)
    for kind in kinds:
        ad = np.array([r["adjoint"] for (b, v, k), r in zip(pick, rows) if k == kind])
        fd = np.array([r["richardson"] for (b, v, k), r in zip(pick, rows) if k == kind])
        two = np.linalg.norm(ad - fd) / np.linalg.norm(fd)
        inf = np.abs(ad - fd).max() / np.abs(fd).max()
        print(f"d/d{kind}: vector error {two:.2e} (2-norm), {inf:.2e} (max-norm)")
        assert two <= 1e-4 and inf <= 1e-4


def test_adjoint_with_poisson_ratio(product_lib):
    """Poisson's ratio 0.3 for every voxel (CVX_Link::updateTransverseInfo and CVX_Voxel::strain
    (true)): each link's stress takes the transverse strain sum and its axial force the transverse
    area of its two voxels, whose Poisson strains the pre-pass recomputes from the previous step's
    link strains and the links' strain ratios (E of one end over E of the other); the adjoint
    carries both back.  The bending cantilevers (no floor, so no contact decisions), 200 steps.
    The reference rounds powf(1 + sum, -nu) - 1 to float, which quantises the Poisson strains and
    makes the differences ragged: where the two differences (4e-3 relative and 0.04 rad, and a
    quarter of each) agree within 1 %, the adjoint lies within 1e-3 of the interval they span."""
    sc = _beams()
    for m in sc.materials:
        m.nu = 0.3
    off = G.body_offsets(sc)
    rng = np.random.default_rng(3)
    kinds = ["E", "rho", "phase"]
    free = lambda b: [v for v in range(off[b], off[b + 1]) if sc.xyz[v, 0] > 0]
    pick = [(b, int(rng.choice(free(b))), kinds[b % 3]) for b in range(len(off) - 1)]
    rows, _, _, _ = G.check(product_lib, sc, 200, 50, pick, 4e-3, 0.04, AMP, FREQ, frozen=True)
    for (b, v, kind), r in zip(pick, rows):
        print("body %3d voxel %5d d/d%-5s adjoint % .6e D(h) % .6e D(h/4) % .6e distance %.2e"
              % (b, v, kind, r["adjoint"], r["fd_h"], r["fd_h4"], r["distance"]))
    smooth = [abs(r["fd_h"] - r["fd_h4"]) <= 1e-2 * max(abs(r["fd_h"]), abs(r["fd_h4"])) for r in rows]
    print(f"{sum(smooth)} of {len(rows)} parameters with agreeing differences")
    assert sum(smooth) >= 5 and {k for (b, v, k), s in zip(pick, smooth) if s} == set(kinds)
    assert max(r["distance"] for r, s in zip(rows, smooth) if s) <= 1e-3


def _beams(n=8, length=12, E_range=(1e4, 3e4), seed=7, tip=-0.05, fail_strain=None):
    """n soft cantilevers of length x 2 x 2 cells (one material per voxel, E log-uniform in E_range,
    density 1000, CTE 0.01), fixed at x = 0, each of the four tip voxels pulled down by `tip` N,
    gravity, no floor; per-voxel phases.  They bend far enough for links near the root to take
    orientLink's large-angle branch.  fail_strain: a linear material with that failure strain
    (CVX_Material::setModelLinear's failure stress over E)."""
    rng = np.random.default_rng(seed)
    xyz, body = [], []
    for b in range(n):
        for x in range(length):
            for y in range(2):
                for z in range(2):
                    xyz.append((x, 4 * b + y, 20 + z))
                    body.append(b)
    xyz = np.array(xyz, np.int32)
    nv = len(xyz)
    lo, hi = np.log10(E_range[0]), np.log10(E_range[1])
    Es = (10.0 ** rng.uniform(lo, hi, nv)).astype(np.float32)
    mats = [S.Material(E=float(e), rho=1e3, cte=0.01,
                       model=None if fail_strain is None else ("linear", float(e), float(e) * fail_strain)) for e in Es]
    sc = S.Scene(0.01, mats, np.arange(nv, dtype=np.int32), xyz, gravity=1.0, floor=False,
                 body=np.array(body, np.int32), name="beams")
    sc.fixed_all = np.flatnonzero(xyz[:, 0] == 0)
    sc.force_idx = np.flatnonzero(xyz[:, 0] == length - 1)
    sc.force_val = np.tile(np.array([[0.0, 0.0, tip]], np.float32), (len(sc.force_idx), 1))
    sc.phase = rng.uniform(0.0, 2.0 * np.pi, nv).astype(np.float32)
    return sc


def test_adjoint_through_large_angle_links(product_lib):
    """Soft cantilevers pulled at the tip bend until links near the root take orientLink's
    large-angle branch (VX_Link.cpp:77-119: the frame from FromAngleToPosX, the angle1 rotation of
    the negative end's forces).  The adjoint differentiates both branches.  Central differences
    over 200 steps (no floor, so no contact decisions) at steps of 4e-3 relative (E, density) and
    0.04 rad (phase) and a quarter of each: where a perturbed run moves a link's switch between the
    branches to another step the two differences disagree, and such parameters are reported and
    left out; every other parameter, of every kind, agrees with the adjoint to 1e-3 after Richardson
    extrapolation."""
    sc = _beams()
    off = G.body_offsets(sc)
    sim, _ = G.build(product_lib, sc, sc.phase, AMP, FREQ)
    dt = sim.recommended_time_step()
    assert sim.do_time_steps(200, dt) == 200
    large = int(np.count_nonzero(sim.link_state()["smallAngle"] == 0))
    print(f"links in the large-angle branch after 200 steps: {large} of {sim.link_count()}")
    assert large > 0
    rng = np.random.default_rng(3)
    kinds = ["E", "rho", "phase"]
    free = lambda b: [v for v in range(off[b], off[b + 1]) if sc.xyz[v, 0] > 0]
    pick = [(b, int(rng.choice(free(b))), kinds[b % 3]) for b in range(len(off) - 1)]
    rows, _, _, _ = G.check(product_lib, sc, 200, 50, pick, 4e-3, 0.04, AMP, FREQ, frozen=True)
    err = np.array([r["richardson_error"] for r in rows])
    for (b, v, kind), r in zip(pick, rows):
        print("body %3d voxel %5d d/d%-5s adjoint % .6e D(h) % .6e D(h/4) % .6e extrapolated % .6e error %.2e"
              % (b, v, kind, r["adjoint"], r["fd_h"], r["fd_h4"], r["richardson"], r["richardson_error"]))
    print(f"large-angle beams: error median {np.median(err):.2e}, max {err.max():.2e}")
    smooth = [abs(r["fd_h"] - r["fd_h4"]) <= 1e-2 * max(abs(r["fd_h"]), abs(r["fd_h4"])) for r in rows]
    print(f"{sum(smooth)} of {len(rows)} parameters with agreeing differences")
    assert sum(smooth) >= 6 and {k for (b, v, k), s in zip(pick, smooth) if s} == set(kinds)
    assert max(e for e, s in zip(err, smooth) if s) <= 1e-3


def test_adjoint_through_failing_links(product_lib):
    """Linear materials with a failure strain (CVX_Link::isFailed: once a link's largest strain
    passes it, it applies no force): the bending cantilevers with a failure strain of 0.05, so that
    links near the roots fail during the 200 steps.  The adjoint follows each link's failure as the
    forward run took it (the taped largest strain); central differences as for the large-angle
    test, with parameters whose perturbed runs fail a link at another step reported and left out."""
    sc = _beams(fail_strain=0.05)
    off = G.body_offsets(sc)
    sim, _ = G.build(product_lib, sc, sc.phase, AMP, FREQ)
    dt = sim.recommended_time_step()
    assert sim.do_time_steps(200, dt) == 200
    failed = int(np.count_nonzero(sim.link_state()["maxStrain"] > 0.05))
    print(f"failed links after 200 steps: {failed} of {sim.link_count()}")
    assert failed > 0
    rng = np.random.default_rng(4)
    kinds = ["E", "rho", "phase"]
    free = lambda b: [v for v in range(off[b], off[b + 1]) if sc.xyz[v, 0] > 0]
    pick = [(b, int(rng.choice(free(b))), kinds[b % 3]) for b in range(len(off) - 1)]
    rows, _, _, _ = G.check(product_lib, sc, 200, 50, pick, 4e-3, 0.04, AMP, FREQ, frozen=True)
    err = np.array([r["richardson_error"] for r in rows])
    for (b, v, kind), r in zip(pick, rows):
        print("body %3d voxel %5d d/d%-5s adjoint % .6e D(h) % .6e D(h/4) % .6e extrapolated % .6e error %.2e"
              % (b, v, kind, r["adjoint"], r["fd_h"], r["fd_h4"], r["richardson"], r["richardson_error"]))
    smooth = [abs(r["fd_h"] - r["fd_h4"]) <= 1e-2 * max(abs(r["fd_h"]), abs(r["fd_h4"])) for r in rows]
    print(f"{sum(smooth)} of {len(rows)} parameters with agreeing differences")
    assert sum(smooth) >= 5 and {k for (b, v, k), s in zip(pick, smooth) if s} == set(kinds)
    assert max(e for e, s in zip(err, smooth) if s) <= 1e-3


def test_decision_replay_follows_the_recorded_branches(product_lib):
    """Replaying a run's own decisions reproduces it bit for bit; a perturbed scene, left to decide
    for itself, takes other branches (which replay holds to the recorded ones)."""
    sc = S.graded_population(4, 6, 0.7, seed=5)
    off = G.body_offsets(sc)
    g, _ = G.build(product_lib, sc, sc.phase, AMP, FREQ)
    dt = g.recommended_time_step()
    base, dec = G.body_com_x(product_lib, sc, sc.phase, 400, dt, off, AMP, FREQ, record=True)
    assert dec.shape == (400, sc.n_voxels) and (dec & 1).any() and (dec & 2).any()
    assert np.array_equal(G.body_com_x(product_lib, sc, sc.phase, 400, dt, off, AMP, FREQ, decisions=dec), base)
    ph = (sc.phase + np.float32(0.5)).astype(np.float32)
    _, own = G.body_com_x(product_lib, sc, ph, 400, dt, off, AMP, FREQ, record=True)
    assert not np.array_equal(own, dec)


def test_adjoint_refuses_while_decisions_are_recorded(product_lib):
    sc = S.graded_population(2, 4, 0.7, seed=3)
    g, eng = G.build(product_lib, sc, sc.phase, AMP, FREQ)
    dt = g.recommended_time_step()
    eng.set_decisions(1, 5)
    with pytest.raises(RuntimeError, match="decisions"):
        eng.adjoint_com_x(10, dt, G.body_offsets(sc), checkpoint_every=5)
    eng.set_decisions(0)
    eng.adjoint_com_x(10, dt, G.body_offsets(sc), checkpoint_every=5)


def test_adjoint_rejects_out_of_scope(product_lib):
    sc = S.graded_population(2, 4, 0.7, seed=3)
    sc.materials[0].nu = 0.3
    g, eng = G.build(product_lib, sc, sc.phase, AMP, FREQ)
    dt = g.recommended_time_step()
    with pytest.raises(RuntimeError, match="Poisson"):
        eng.adjoint_com_x(10, dt, G.body_offsets(sc), checkpoint_every=5)
