"""Per-voxel and per-link queries (CVX_Voxel::externalForce/externalMoment, cornerOffset/
cornerPosition, force/moment, isYielded/isFailed, pressure; CVX_Link::strainEnergy/isYielded/
isFailed; src/VX_Voxel.cpp:92-159, include/VX_Voxel.h:79-130, src/VX_Link.cpp:127-135, 251-257).

The scene is a 10x3x3 beam of a bilinear material with a failure stress, Poisson's ratio 0.3 and
a CTE: the x=0 face fixed, a tip load that yields and then fails links, one voxel fixed only in z
translation and x rotation (so its external force mixes the applied and the reaction components),
one voxel with an applied moment, and one heated slice (its corner offsets scale with the base
size).  Every query of every voxel and link is compared at four checkpoints.  On the CPU the
oracle's restatement must equal the reference build exactly; on the GPU (FP64 path) the product
must equal the oracle in its correctly rounded mode exactly.
"""
from __future__ import annotations

import numpy as np
import pytest

from voxelyze_gb300 import facade as F, scenes as S


def build(sim):
    sc = S.cantilever(10, 3, 3, voxel_size=0.01, E=1e6, tip_force=-4.0)
    sc.materials[0].model = ("bilinear", 1e6, 2e5, 2e4, 6e4)
    sc.materials[0].nu = 0.3
    sc.materials[0].cte = 0.01
    S.apply(sc, sim)
    sim.f["external_set_fixed"](sim.h, sim.voxel_index(5, 0, 0), F.Z_TRANSLATE | F.X_ROTATE)
    sim.f["external_set_moment"](sim.h, sim.voxel_index(7, 2, 2), 0.0, 0.02, 0.0)
    for y in range(3):
        for z in range(3):
            sim.f["voxel_set_temperature"](sim.h, sim.voxel_index(3, y, z), 0.5)
    return sim


def compare(a, b, checkpoints=4, steps=150):
    dt = a.recommended_time_step()
    assert b.recommended_time_step() == dt
    seen = {"yielded": 0, "failed": 0}
    for k in range(checkpoints):
        assert a.do_time_steps(steps, dt) == b.do_time_steps(steps, dt)
        qa, qb = a.queries(), b.queries()
        bad = [n for n in qa if not np.array_equal(qa[n], qb[n])]
        assert bad == [], f"queries differ after {(k + 1) * steps} steps: {bad}"
        seen["yielded"] = max(seen["yielded"], int(qa["voxel_yielded"].sum()))
        seen["failed"] = max(seen["failed"], int(qa["link_failed"].sum()))
    # the run covers the yielded and the failed branches of every query
    assert seen["yielded"] > 0 and seen["failed"] > 0, seen
    return qa


def test_queries_oracle_equal_reference(oracle_lib, ref_lib):
    oracle_lib.vxo_set_math(0)
    compare(build(F.Sim(oracle_lib, "vxo", 0.01)), build(F.Sim(ref_lib, "vxr", 0.01)))


def test_query_arguments_are_checked(oracle_lib):
    s = build(F.Sim(oracle_lib, "vxo", 0.01))
    with pytest.raises(IndexError):
        s.corner_offset(0, 8)
    with pytest.raises(IndexError):
        s.external_force(s.voxel_count())
    assert s.f["link_is_failed"](s.h, s.link_count()) == -1
    # a voxel without an external answers zero
    assert np.array_equal(s.external_force(s.voxel_index(1, 1, 1)), np.zeros(3, np.float32))


@pytest.mark.gpu
def test_queries_gpu_equal_oracle(product_lib, oracle_lib):
    oracle_lib.vxo_set_math(1)
    try:
        compare(build(F.Sim(product_lib, "vx", 0.01)), build(F.Sim(oracle_lib, "vxo", 0.01)))
    finally:
        oracle_lib.vxo_set_math(0)


@pytest.mark.gpu
def test_queries_fp32c_track_fp64(product_lib):
    """FP32C: the same queries read from the FP32C state stay close to the FP64 path's (the
    positions to 1e-6 relative, the reactions to 1e-3 of their largest magnitude) over the first
    checkpoint, before links fail."""
    a = build(F.Sim(product_lib, "vx", 0.01))
    b = build(F.Sim(product_lib, "vx", 0.01))
    F.Engine(b).set_precision(1)
    dt = a.recommended_time_step()
    assert a.do_time_steps(100, dt) == b.do_time_steps(100, dt) == 100
    qa, qb = a.queries(), b.queries()
    cp = qa["corner_position"]
    assert np.abs(qb["corner_position"] - cp).max() <= 1e-6 * np.abs(cp).max()
    ef = qa["external_force"]
    assert np.abs(qb["external_force"] - ef).max() <= 1e-3 * np.abs(ef).max()
    assert np.array_equal(qa["voxel_failed"], qb["voxel_failed"])
