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


def _pieces(xyz):
    """Starts of the runs of the voxel order that no link crosses: the cut rule of the engine's
    body batches (a difference array over each link's end indices)."""
    n = len(xyz)
    index = {tuple(p): i for i, p in enumerate(xyz)}
    cover = np.zeros(n + 1, np.int64)
    for i, p in enumerate(xyz):
        for d in ((1, 0, 0), (0, 1, 0), (0, 0, 1)):
            j = index.get((p[0] + d[0], p[1] + d[1], p[2] + d[2]))
            if j is not None:
                a, b = min(i, j), max(i, j)
                cover[a] += 1
                cover[b] -= 1
    run = np.cumsum(cover[:n])
    return np.concatenate([[0], np.flatnonzero(run[:-1] == 0) + 1])


def test_population_bodies_are_pieces():
    """Body batches need each body to be a run of the voxel order that no link crosses: the
    population generator adds body after body with gaps between them, and each body is one
    connected component, so its pieces are exactly its bodies."""
    sc = S.population(64)
    starts = _pieces(sc.xyz)
    offsets = np.concatenate([[0], np.cumsum(np.bincount(sc.body))])[:-1]
    assert np.array_equal(starts, offsets)
