"""Topology edits between steps: setVoxel over an existing voxel (material
replacement), setVoxel(NULL) (removal), replaceMaterial, removeMaterial and setVoxelSize
(src/Voxelyze.cpp:384-498, 541-575, 643-668).  Each edit renumbers voxels or links the way the
reference's lists do (removal shifts later entries down; a replaced voxel's links move to the end
of the link list, voxels visited z, then y, then x by replaceMaterial), and the state after every
block of steps must match bit for bit: the oracle against the reference build on the host, the GPU
against the oracle.

The sequence avoids what the reference itself cannot do: its replaceMaterial and removeMaterial
walk the bounding box and dereference empty cells (so both run on a full box, removeMaterial on a
material without voxels, since removing any empties cells it then visits), and its removeVoxel
erases from the voxel list while iterating (so the last voxel of the list is never removed).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import state_diff
from voxelyze_gb300 import facade as F


def build(lib, prefix):
    s = F.Sim(lib, prefix, 0.01)
    m0 = s.add_material(1e6, 1000.0)
    m1 = s.add_material(3e6, 1500.0)
    s.material_set(m1, F.PROP_POISSON, 0.3)
    for z in range(3):
        for y in range(4):
            for x in range(6):
                s.set_voxel(m0 if x < 3 else m1, x, y, z)
    for v in range(s.voxel_count()):
        if v % 6 == 0:
            s.set_fixed_all(v)
        elif v % 6 == 5:
            s.set_force(v, 0.0, 0.02, -0.05)
    return s


def edit_blocks(s):
    """Yields after each block of steps; the edits between blocks are the same for every library."""
    dt = s.recommended_time_step()
    assert dt > 0
    m2 = s.add_material(5e5, 800.0)
    assert s.do_time_steps(40, dt) == 40
    yield "initial"
    assert s.replace_material(1, m2)                 # full box: every cell occupied
    assert s.do_time_steps(40, dt) == 40
    yield "replaceMaterial"
    m3 = s.add_material(2e6, 900.0)
    assert s.remove_material(m3)                      # a material without voxels, full box
    assert s.do_time_steps(20, dt) == 20
    yield "removeMaterial"
    s.set_voxel(0, 4, 2, 1)                           # material replacement of one voxel
    for x, y, z in ((2, 1, 1), (3, 2, 0), (1, 3, 2)):
        s.remove_voxel(x, y, z)
    assert s.do_time_steps(40, dt) == 40
    yield "replace + remove voxels"
    s.set_voxel(m2, 2, 1, 1)                          # a removed site filled again (list end)
    s.set_voxel_size(0.012)
    dt = s.recommended_time_step()
    assert s.do_time_steps(40, dt) == 40
    yield "re-add + setVoxelSize"


def run_pair(a, b):
    ga, gb = edit_blocks(a), edit_blocks(b)
    for name in ga:
        assert next(gb) == name
        assert a.voxel_count() == b.voxel_count() and a.link_count() == b.link_count(), name
        assert state_diff(a, b) == [], name


def test_oracle_matches_reference_build(oracle_lib, ref_lib):
    oracle_lib.vxo_set_math(0)  # the C library's sin/cos/acos, as the reference build
    run_pair(build(oracle_lib, "vxo"), build(ref_lib, "vxr"))


@pytest.mark.gpu
def test_gpu_matches_oracle(product_lib, oracle_lib):
    oracle_lib.vxo_set_math(1)
    try:
        run_pair(build(product_lib, "vx"), build(oracle_lib, "vxo"))
    finally:
        oracle_lib.vxo_set_math(0)


def test_remove_material_with_voxels(product_lib, oracle_lib):
    """removeMaterial on a material in use (the reference cannot: it dereferences the cells it has
    emptied): its voxels and links go, later material indices move down; host only."""
    sims = [build(product_lib, "vx"), build(oracle_lib, "vxo")]
    for s in sims:
        n = s.voxel_count()
        assert s.remove_material(0)
        assert s.voxel_count() == n // 2
    a, b = sims
    assert a.link_count() == b.link_count()
    la, lb = a.link_state(), b.link_state()
    assert np.array_equal(la["vneg"], lb["vneg"]) and np.array_equal(la["vpos"], lb["vpos"])
