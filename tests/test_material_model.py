"""CVX_Material::stress and modulus (src/VX_Material.cpp:165-226) of the product's host library,
which derives the material tables the GPU reads, against the reference build and the oracle, bit
for bit, on seeded random linear, bilinear and data-table models with failure points, at strains
around each model point, with and without a transverse strain sum (Poisson's ratio)."""
from __future__ import annotations

import numpy as np
import pytest

from voxelyze_gb300 import facade as F


def _models(sim, rng):
    mats = []
    for k in range(12):
        E = float(np.float32(10 ** rng.uniform(4, 7)))
        m = sim.add_material(E, 1000.0)
        if k % 2:
            sim.material_set(m, F.PROP_POISSON, float(np.float32(rng.uniform(0.05, 0.45))))
        kind = k % 3
        if kind == 0:
            sim.set_model_linear(m, E, float(np.float32(E * rng.uniform(0.01, 0.2))) if rng.random() < 0.5 else -1.0)
        elif kind == 1:
            ys = float(np.float32(E * rng.uniform(0.005, 0.05)))
            fs = float(np.float32(ys * rng.uniform(1.5, 4))) if rng.random() < 0.5 else -1.0
            sim.set_model_bilinear(m, E, float(np.float32(E * rng.uniform(0.05, 0.5))), ys, fs)
        else:
            n = int(rng.integers(3, 7))
            strain = np.concatenate([[0.0], np.sort(rng.uniform(0.002, 0.3, n - 1))]).astype(np.float32)
            slope = E * np.concatenate([[1.0], rng.uniform(0.05, 0.9, n - 2)])
            stress = np.concatenate([[0.0], np.cumsum(np.diff(strain) * slope)]).astype(np.float32)
            sim.set_model(m, strain, stress)
        mats.append(m)
    return mats


def _strains(rng):
    base = np.concatenate([np.linspace(-0.4, 0.4, 161), rng.uniform(-0.35, 0.35, 200), [0.0, 1e-7, -1e-7]])
    return base.astype(np.float32)


@pytest.mark.parametrize("seed", range(4))
def test_stress_and_modulus_match_reference_build(product_lib, ref_lib, oracle_lib, seed):
    sims = [F.Sim(product_lib, "vx", 0.01), F.Sim(ref_lib, "vxr", 0.01), F.Sim(oracle_lib, "vxo", 0.01)]
    mats = [_models(s, np.random.default_rng(seed)) for s in sims]
    strains = _strains(np.random.default_rng(100 + seed))
    tss_values = (0.0, 0.003, -0.002)
    for k in range(len(mats[0])):
        for force_linear in (False, True):
            for tss in tss_values:
                got = [np.array([s.material_stress(ms[k], float(e), tss, force_linear) for e in strains], np.float32)
                       for s, ms in zip(sims, mats)]
                assert np.array_equal(got[0].view(np.uint32), got[1].view(np.uint32)), (k, force_linear, tss)
                assert np.array_equal(got[2].view(np.uint32), got[1].view(np.uint32)), (k, force_linear, tss)
        mod = [np.array([s.material_modulus(ms[k], float(e)) for e in strains], np.float32) for s, ms in zip(sims, mats)]
        assert np.array_equal(mod[0].view(np.uint32), mod[1].view(np.uint32)), k
        assert np.array_equal(mod[2].view(np.uint32), mod[1].view(np.uint32)), k
