"""The adjoint against finite differences of the reference itself, and through torch.autograd.

* tests/golden/adjoint_ref_fd.npz holds central differences of a body's centre-of-mass x after
  400 steps taken with the reference library compiled from its own sources (one 155-voxel body,
  one material per voxel, per-voxel actuation phase, floor, friction, gravity; made by
  tests/golden/make_adjoint_ref_fd.py).  The GPU adjoint of the same run (FP64 path) is compared
  with their Richardson extrapolation for every parameter whose two differences (steps h and h/4)
  agree within 1 %; where they do not, a floor-contact or static-friction decision somewhere in the
  body flipped between the perturbed runs (the reference cannot replay a run's decisions), and the
  difference measures that jump, not the derivative along the branches the adjoint follows.
* voxelyze_gb300.autograd.AdjointComX: J.backward() returns the adjoint's gradient, and
  torch.autograd.gradcheck (central differences in float64 through the same Function) agrees
  with it on E, density and phase multipliers of a few voxels; the Function evaluates J with the
  unperturbed run's floor-contact and static-friction decisions replayed, so the differences
  follow the branches the adjoint differentiates along.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu


def _fixture_scene(fx):
    n = len(fx["E"])
    mats = [S.Material(E=float(fx["E"][k]), rho=float(fx["rho"][k]), cte=0.01, mu_static=1.0, mu_kinetic=0.5)
            for k in range(n)]
    sc = S.Scene(0.01, mats, np.arange(n, dtype=np.int32), fx["xyz"].astype(np.int32), gravity=1.0, floor=True,
                 body=np.zeros(n, np.int32))
    sc.phase = fx["phase"].astype(np.float32)
    return sc


def test_adjoint_against_reference_differences(product_lib):
    fx = dict(np.load(os.path.join(ROOT, "tests", "golden", "adjoint_ref_fd.npz")))
    sc = _fixture_scene(fx)
    sim = F.Sim(product_lib, "vx", sc.voxel_size)
    S.apply(sc, sim)
    eng = F.Engine(sim)
    eng.set_actuation(F.ACT_PER_VOXEL, float(fx["amplitude"]), float(fx["frequency"]), sc.phase)
    dt = sim.recommended_time_step()
    assert np.float32(dt) == fx["dt"]
    obj, gE, gR, gP = eng.adjoint_com_x(int(fx["nsteps"]), dt, np.array([0, sc.n_voxels], np.int32))
    rel_obj = abs(obj[0] - float(fx["objective"])) / abs(float(fx["objective"]))
    grads = {"E": gE, "rho": gR, "phase": gP}
    rows = []
    for v, kind, (d1, d2, rich) in zip(fx["pick_voxel"], fx["pick_kind"], fx["fd"]):
        ad = grads[str(kind)][int(v)]
        smooth = abs(d1 - d2) <= 0.01 * max(abs(d1), abs(d2))
        rows.append((int(v), str(kind), ad, rich, abs(ad - rich) / abs(rich), smooth))
    for r in rows:
        print("voxel %4d %-5s adjoint % .6e  reference FD (Richardson) % .6e  rel. diff %.2e %s"
              % (r[0], r[1], r[2], r[3], r[4], "" if r[5] else "(differences disagree: branch crossed)"))
    print(f"objective: GPU {obj[0]:.15e}, reference {float(fx['objective']):.15e} (rel. {rel_obj:.2e})")
    assert rel_obj <= 1e-9
    smooth = [r for r in rows if r[5]]
    assert len(smooth) >= 10 and {r[1] for r in smooth} == {"E", "rho", "phase"}
    assert max(r[4] for r in smooth) <= 2e-3


def test_autograd_function(product_lib):
    torch = pytest.importorskip("torch")
    from voxelyze_gb300.autograd import AdjointComX, ComXObjective

    sc = S.graded_population(n_bodies=2, side=5, occupancy=0.7, seed=33)
    objective = ComXObjective(product_lib, sc, nsteps=300, checkpoint_every=50, freeze_decisions=True)
    E0, R0, P0 = (torch.tensor(a, dtype=torch.float64) for a in objective.initial())
    E, R, P = (t.clone().requires_grad_(True) for t in (E0, R0, P0))
    J = AdjointComX.apply(E, R, P, objective)
    J.backward()
    ref_J, gE, gR, gP = objective.run(*(t.numpy() for t in (E0, R0, P0)))
    assert J.item() == ref_J
    assert np.array_equal(E.grad.numpy(), gE) and np.array_equal(R.grad.numpy(), gR)
    assert np.array_equal(P.grad.numpy(), gP)

    # gradcheck on per-voxel multipliers of three voxels' E, density and phase offsets: central
    # differences in float64 through the same Function (steps large enough to stay above the
    # float rounding of E and density, small enough for the h^2 truncation to stay below rtol)
    rng = np.random.default_rng(3)
    vox = torch.tensor(rng.choice(sc.n_voxels, size=3, replace=False))

    def f(x):
        Ex = E0.clone().index_put((vox,), E0[vox] * x[0:3])
        Rx = R0.clone().index_put((vox,), R0[vox] * x[3:6])
        Px = P0.clone().index_put((vox,), P0[vox] + x[6:9])
        return AdjointComX.apply(Ex, Rx, Px, objective)

    x0 = torch.tensor([1.0] * 6 + [0.0] * 3, dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(f, (x0,), eps=4e-3, atol=1e-10, rtol=5e-3)
