"""Deformed mesh (CVX_MeshRender, src/VX_MeshRender.cpp): topology against the reference build on
the host; vertex positions and normals, computed on the GPU, against the reference's mesh of the
same undeformed-but-heated scene (committed fixture) and against a direct evaluation of the
reference's formulas from the simulator's own state after stepping.

The direct evaluation follows CVX_Voxel::cornerPosition / cornerOffset (src/VX_Voxel.cpp:141-159)
and Quat3D::RotateVec3D's float-vector form (include/Quat3D.h:179-186) operation by operation in
numpy float32 / float64, so the comparison is bit for bit.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT, make_sim
from voxelyze_gb300 import facade as F, scenes as S

GOLDEN = os.path.join(ROOT, "tests", "golden", "mesh_ref.npz")
f32, f64 = np.float32, np.float64

SCENES = {
    "lattice": lambda: S.lattice(8, 6, 4),
    "porous": lambda: S.porous(10, sigma=1.2),
    "population": lambda: S.population(5, 3, 6),
}


def heated_scene():
    """A small two-material body with a temperature per voxel (CTE 0.01 on one material), so the
    corner offsets differ voxel by voxel before any step: the fixture scene."""
    return S.population(3, 3, 5, seed=9)


def heat(sim, n):
    for v in range(n):
        sim.set_temperature(v, float(f32(0.3 * np.sin(0.7 * v))))


@pytest.mark.parametrize("name", list(SCENES))
def test_topology_matches_reference(product_lib, ref_lib, name):
    """Quads (vertex order included), quad voxels and edges in the reference's order (host only)."""
    sc = SCENES[name]()
    out = []
    for lib, pre in ((product_lib, "vx"), (ref_lib, "vxr")):
        sim = make_sim(lib, pre, sc)
        sim.mesh_generate()  # the product's first update needs a GPU; the topology does not
        out.append(sim.mesh())
    a, b = out
    assert a["vertices"].shape == b["vertices"].shape
    assert np.array_equal(a["quads"], b["quads"])
    assert np.array_equal(a["lines"], b["lines"])


def _voxel_links(ls, nv):
    lk = np.full((nv, 6), -1, np.int64)
    for l, (vn, vp, ax) in enumerate(zip(ls["vneg"], ls["vpos"], ls["axis"])):
        lk[vn, 2 * ax] = l
        lk[vp, 2 * ax + 1] = l
    return lk


def expected_mesh(sim, sc, mesh):
    """Vertices and normals from the simulator's state by the reference's formulas."""
    vs, ls = sim.voxel_state(), sim.link_state()
    nv = sim.voxel_count()
    pos, q, temp = vs["pos"], vs["orient"], vs["temp"].astype(f32)
    mats = sc.materials
    E = np.array([f32(mats[m].E) for m in sc.mats], f32)
    cte = np.array([f32(mats[m].cte) for m in sc.mats], f32)
    size = f64(sc.voxel_size)
    lk = _voxel_links(ls, nv)
    strain = ls["strain"].astype(f32)
    ratio = (E[ls["vpos"]] / E[ls["vneg"]]).astype(f32)
    verts = np.zeros_like(mesh["vertices"])
    corner_cache = {}

    def corner(v, c):
        key = (v, c)
        if key in corner_cache:
            return corner_cache[key]
        fT = f32(1) + temp[v] * cte[v]
        off = np.zeros(3, f32)
        for i in range(3):
            pos_link = bool(c & (1 << (2 - i)))
            l = lk[v, 2 * i + (0 if pos_link else 1)]
            st = f64(1.0 if pos_link else -1.0)
            if l >= 0:
                s, r = strain[l], ratio[l]
                half = (f32(2) * s * r) / (f32(1) + r) if pos_link else (f32(2) * s) / (f32(1) + r)
                st = f64((f32(1) + half) * f32(1 if pos_link else -1))
            off[i] = f32((f64(0.5) * (f64(fT) * size)) * st)
        w, x, y, z = q[v]
        fx, fy, fz = off
        tw = f32(fx * x + fy * y + fz * z)
        tx = f32(fx * w - fy * z + fz * y)
        ty = f32(fx * z + fy * w - fz * x)
        tz = f32(-fx * y + fy * x + fz * w)
        out = np.array([f32(pos[v, 0]) + f32(w * tx + x * tw + y * tz - z * ty),
                        f32(pos[v, 1]) + f32(w * ty - x * tz + y * tw + z * tx),
                        f32(pos[v, 2]) + f32(w * tz + x * ty - y * tx + z * tw)], f32)
        corner_cache[key] = out
        return out

    index = {tuple(map(int, p)): k for k, p in enumerate(sc.xyz)}
    for i, (gx, gy, gz) in enumerate(mesh["lattice"]):
        acc = np.zeros(3, f32)
        n = 0
        for j in range(8):
            key = (gx - (1 if j & 4 else 0), gy - (1 if j & 2 else 0), gz - (1 if j & 1 else 0))
            v = index.get(key)
            if v is None:
                continue
            acc = acc + corner(v, j)
            n += 1
        verts[i] = acc * (f32(1) / f32(n))
    v = verts[mesh["quads"]]
    a, b = v[:, 1] - v[:, 0], v[:, 3] - v[:, 0]
    nrm = np.stack([a[:, 1] * b[:, 2] - a[:, 2] * b[:, 1], a[:, 2] * b[:, 0] - a[:, 0] * b[:, 2],
                    a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]], 1).astype(f32)
    length = np.sqrt((nrm[:, 0] * nrm[:, 0] + nrm[:, 1] * nrm[:, 1]) + nrm[:, 2] * nrm[:, 2]).astype(f32)
    nrm = np.where(length[:, None] > 0, nrm / np.where(length > 0, length, 1)[:, None], nrm).astype(f32)
    return verts, nrm


# corners of the exposed face in each link direction (X+, X-, Y+, Y-, Z+, Z-) in quad vertex order;
# corner bits are x << 2 | y << 1 | z (CVX_Voxel::voxelCorner)
FACE_CORNERS = [[4, 6, 7, 5], [0, 1, 3, 2], [2, 3, 7, 6], [0, 4, 5, 1], [1, 5, 7, 3], [0, 2, 6, 4]]
DIRS = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]


def vertex_corners(sc):
    """Lattice corner of each mesh vertex, numbered as CVX_MeshRender::generateMesh numbers them
    (first appearance over voxels in list order, exposed faces in direction order)."""
    occupied = {tuple(map(int, p)) for p in sc.xyz}
    seen, corners = {}, []
    for p in sc.xyz:
        x, y, z = map(int, p)
        for d, (dx, dy, dz) in enumerate(DIRS):
            if (x + dx, y + dy, z + dz) in occupied:
                continue
            for c in FACE_CORNERS[d]:
                key = (x + ((c >> 2) & 1), y + ((c >> 1) & 1), z + (c & 1))
                if key not in seen:
                    seen[key] = len(corners)
                    corners.append(key)
    return np.array(corners, np.int64)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name", ["lattice", "population"])
def test_vertices_and_normals_follow_the_state(product_lib, name, precision):
    """After 150 steps (gravity, floor; population with CTE actuation), the GPU mesh equals the
    reference's formulas evaluated on the simulator's own state, bit for bit."""
    sc = SCENES[name]()
    sim = make_sim(product_lib, "vx", sc)
    F.Engine(sim).set_precision(precision)
    dt = sim.recommended_time_step()
    assert dt > 0
    if name == "population":
        F.Engine(sim).set_actuation(F.ACT_UNIFORM, 0.1, 2.0)
    assert sim.do_time_steps(150, dt) == 150
    assert sim.mesh_generate()
    m = sim.mesh()
    m["lattice"] = vertex_corners(sc)
    assert len(m["lattice"]) == len(m["vertices"])
    verts, nrm = expected_mesh(sim, sc, m)
    assert np.array_equal(m["vertices"], verts)
    assert np.array_equal(m["normals"], nrm)


@pytest.mark.gpu
def test_heated_scene_matches_reference_fixture(product_lib, tmp_path):
    """The reference's own mesh (vertices, normals, colours, OBJ file) of a scene with a
    temperature per voxel, before any step: the GPU mesh is identical."""
    g = np.load(GOLDEN)
    sc = heated_scene()
    sim = make_sim(product_lib, "vx", sc)
    heat(sim, sim.voxel_count())
    assert sim.mesh_generate()
    for coloring in (F.MESH_MATERIAL, F.MESH_FAILURE, F.MESH_STATE_INFO):
        assert sim.mesh_update(coloring, F.DISPLACEMENT if coloring != F.MESH_STATE_INFO else F.KINETIC_ENERGY)
        m = sim.mesh()  # (at rest the state-info colours are 0/0: NaN in both)
        assert np.array_equal(m["colors"], g[f"colors{coloring}"], equal_nan=True)
    for k in ("vertices", "normals", "quads", "lines"):
        assert np.array_equal(m[k], g[k]), k
    assert sim.mesh_save_obj(str(tmp_path / "m.obj"))
    assert open(tmp_path / "m.obj").read() == str(g["obj"])
