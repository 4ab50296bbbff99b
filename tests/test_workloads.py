"""The seeded workloads bench.py measures, pinned by their sizes (no GPU): the 128x128x64 lattice
(fill 0.85, largest 6-connected component) has 890,860 voxels and 2,247,152 links, counted here as
the face-adjacent occupied pairs, the links setVoxel creates (src/Voxelyze.cpp:406-457)."""
from __future__ import annotations

import numpy as np

from voxelyze_gb300 import scenes as S


def _links(xyz):
    occ = np.zeros(tuple(xyz.max(axis=0) + 2), bool)
    occ[tuple(xyz.T)] = True
    return int((occ[1:] & occ[:-1]).sum() + (occ[:, 1:] & occ[:, :-1]).sum() + (occ[:, :, 1:] & occ[:, :, :-1]).sum())


def test_headline_lattice_size():
    sc = S.lattice(128, 128, 64)
    assert sc.n_voxels == 890_860
    assert _links(sc.xyz) == 2_247_152
    assert len(sc.materials) == 4 and all(m.nu == 0.3 for m in sc.materials)


def test_cantilever_size():
    sc = S.cantilever(40, 8, 8)
    assert sc.n_voxels == 2_560
    assert _links(sc.xyz) == 6_976
