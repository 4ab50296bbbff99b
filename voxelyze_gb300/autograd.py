"""A torch.autograd.Function over the adjoint C ABI (vx_adjoint_com_x), for checking gradients.

The objective is J(E, rho, phase) = the sum over bodies of each body's mass-weighted centre-of-mass
x after ``nsteps`` FP64 steps of a scene with one material per voxel and per-voxel actuation
(temperature = amplitude * sin(2 pi frequency t + phase[v]) inside every step).  ``forward`` builds
the scene with the given per-voxel Young's moduli, densities and phases (E and density rounded to
float, as CVX_Material holds them), runs the differentiated run and keeps dJ/dE, dJ/drho and
dJ/dphase; ``backward`` scales them by the incoming gradient.  The time step is fixed once, from
the unperturbed scene, so perturbed evaluations step the same dt.

This module exists so that torch.autograd.gradcheck and finite differences taken through the same
call can check the hand-written adjoint kernels.  It is not on the time-step path and nothing else
in the package imports it.
"""
from __future__ import annotations

import copy

import numpy as np
import torch

from . import facade as F
from . import scenes as S


class ComXObjective:
    """The run that ``AdjointComX`` differentiates: topology, actuation and horizon of one
    multi-body scene whose per-voxel parameters are the inputs."""

    def __init__(self, lib, scene, nsteps: int, checkpoint_every: int = 100, amplitude: float = 0.1,
                 frequency: float = 2.0, dt: float | None = None, freeze_decisions: bool = False):
        if scene.body is None or len(scene.materials) != scene.n_voxels:
            raise ValueError("needs a multi-body scene with one material per voxel")
        self.lib, self.scene = lib, scene
        self.nsteps, self.checkpoint_every = nsteps, checkpoint_every
        self.amplitude, self.frequency = amplitude, frequency
        self.offsets = np.concatenate([[0], np.cumsum(np.bincount(scene.body))]).astype(np.int32)
        if dt is None:
            sim, _ = self._build(*self.initial())
            dt = sim.recommended_time_step()
        self.dt = float(dt)
        # freeze_decisions: J is evaluated with the floor-contact and static-friction decisions of
        # the run at the scene's own parameters replayed (vxg_set_decisions), so that values at
        # perturbed parameters follow the branches the adjoint differentiates along
        self.decisions = None
        if freeze_decisions:
            sim, eng = self._build(*self.initial())
            sim.recommended_time_step()
            eng.set_decisions(1, nsteps)
            if sim.do_time_steps(nsteps, self.dt) != nsteps:
                raise RuntimeError("the run diverged")
            self.decisions = eng.decisions(nsteps)

    def initial(self):
        """The scene's own (E, rho, phase) as float64 arrays."""
        sc = self.scene
        return (np.array([m.E for m in sc.materials], np.float64), np.array([m.rho for m in sc.materials], np.float64),
                np.asarray(sc.phase, np.float64))

    def _build(self, E, rho, phase):
        sc = copy.copy(self.scene)
        sc.materials = [copy.copy(m) for m in self.scene.materials]
        for k, m in enumerate(sc.materials):
            m.E = float(np.float32(E[k]))
            m.rho = float(np.float32(rho[k]))
        sim = F.Sim(self.lib, "vx", sc.voxel_size)
        S.apply(sc, sim)
        eng = F.Engine(sim)
        eng.set_actuation(F.ACT_PER_VOXEL, self.amplitude, self.frequency, np.asarray(phase, np.float32))
        return sim, eng

    def run(self, E, rho, phase):
        """(J, dJ/dE, dJ/drho, dJ/dphase) at these per-voxel parameters."""
        sim, eng = self._build(E, rho, phase)
        sim.recommended_time_step()  # the reference's first call also refreshes link state
        obj, gE, gR, gP = eng.adjoint_com_x(self.nsteps, self.dt, self.offsets, checkpoint_every=self.checkpoint_every)
        J = float(obj.sum())
        if self.decisions is not None:  # the value along the recorded branches
            sim, eng = self._build(E, rho, phase)
            sim.recommended_time_step()
            eng.set_decisions(2, self.nsteps)
            eng.put_decisions(self.decisions)
            if sim.do_time_steps(self.nsteps, self.dt) != self.nsteps:
                raise RuntimeError("the run diverged")
            J = float(eng.body_com(self.offsets)[:, 0].sum())
        return J, gE, gR, gP


class AdjointComX(torch.autograd.Function):
    """J = AdjointComX.apply(E, rho, phase, objective) with E, rho, phase float64 tensors of one
    value per voxel; J is a float64 scalar whose gradient comes from the adjoint kernels."""

    @staticmethod
    def forward(ctx, E, rho, phase, objective: ComXObjective):
        J, gE, gR, gP = objective.run(E.detach().cpu().double().numpy(), rho.detach().cpu().double().numpy(),
                                      phase.detach().cpu().double().numpy())
        ctx.save_for_backward(torch.from_numpy(gE), torch.from_numpy(gR), torch.from_numpy(gP))
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        gE, gR, gP = ctx.saved_tensors
        return grad * gE, grad * gR, grad * gP, None
