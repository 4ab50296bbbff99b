"""Seeded synthetic scenes for the time-step workloads.

No public benchmark or dataset exists for the time-step path; every workload is synthetic and
seeded.  Each generator returns a :class:`Scene` (materials, voxel list in insertion order,
externals, globals) that :func:`apply` pushes through the facade calls of any simulator.  Voxel
insertion order is fixed (z outer, y, x inner), and it fixes the voxel and link indexing of the
reference (Voxelyze.cpp:439-461, 508-539).

Workloads (sizes as stated; the largest connected component is kept where a fill is random):
  cantilever      40x8x8 solid, 5 mm, E=1 MPa, rho=1000, x=0 face fixed, -1 N z on each x=39 voxel
  lattice         128x128x64 Bernoulli(0.85), 4 bilinear materials, nu=0.3, gravity + floor, 1 cm
  porous          64^3 Gaussian-smoothed noise at 0.4 void, nu=0.35, friction, collisions, 1 cm
  population      many small bodies (sides 4..24, occupancy 0.6), passive/active CTE materials
  phase_bodies    bodies of 16^3 at occupancy 0.7 with per-voxel stiffness and actuation phase
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import facade as F


@dataclass
class Material:
    E: float = 1e6
    rho: float = 1e3
    model: Optional[tuple] = None  # ("bilinear", E, Ep, sigma_y, sigma_f) | ("linear", E, sigma_f) | ("data", strain, stress)
    nu: float = 0.0
    cte: float = 0.0
    mu_static: float = 0.0
    mu_kinetic: float = 0.0
    zeta_internal: float = 1.0
    zeta_global: float = 0.0
    zeta_collision: float = 0.0


@dataclass
class Scene:
    voxel_size: float
    materials: list
    mats: np.ndarray          # (N,) material index per voxel, insertion order
    xyz: np.ndarray           # (N,3) lattice index per voxel
    fixed_all: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))   # voxel indices
    fixed_idx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))   # partial fixes:
    fixed_mask: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))  # dofComponent bits
    force_idx: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    force_val: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.float32))
    gravity: float = 0.0
    floor: bool = False
    collisions: bool = False
    body: Optional[np.ndarray] = None   # (N,) body id per voxel for multi-body scenes
    name: str = ""

    @property
    def n_voxels(self) -> int:
        return int(len(self.mats))


def apply(scene: Scene, sim: "F.Sim") -> None:
    """Push ``scene`` through the facade of ``sim`` in a fixed call order."""
    for m in scene.materials:
        k = sim.add_material(m.E, m.rho)
        if m.model is not None:
            kind = m.model[0]
            if kind == "bilinear":
                sim.set_model_bilinear(k, *m.model[1:])
            elif kind == "linear":
                sim.set_model_linear(k, *m.model[1:])
            elif kind == "data":
                sim.set_model(k, m.model[1], m.model[2])
        if m.nu != 0.0:
            sim.material_set(k, F.PROP_POISSON, m.nu)
        if m.cte != 0.0:
            sim.material_set(k, F.PROP_CTE, m.cte)
        if m.mu_static != 0.0:
            sim.material_set(k, F.PROP_MU_STATIC, m.mu_static)
        if m.mu_kinetic != 0.0:
            sim.material_set(k, F.PROP_MU_KINETIC, m.mu_kinetic)
        if m.zeta_internal != 1.0:
            sim.material_set(k, F.PROP_ZETA_INTERNAL, m.zeta_internal)
        if m.zeta_global != 0.0:
            sim.material_set(k, F.PROP_ZETA_GLOBAL, m.zeta_global)
        if m.zeta_collision != 0.0:
            sim.material_set(k, F.PROP_ZETA_COLLISION, m.zeta_collision)
    if scene.gravity != 0.0:
        sim.set_gravity(scene.gravity)
    if scene.floor:
        sim.enable_floor(True)
    if scene.collisions:
        sim.enable_collisions(True)
    sim.set_voxels(scene.mats, scene.xyz)
    for v in scene.fixed_all:
        sim.set_fixed_all(int(v), True)
    for v, mask in zip(scene.fixed_idx, scene.fixed_mask):
        sim.set_fixed(int(v), int(mask))
    for v, f in zip(scene.force_idx, scene.force_val):
        sim.set_force(int(v), float(f[0]), float(f[1]), float(f[2]))


# ---------------------------------------------------------------------------------------------
def _ordered(occ: np.ndarray, offset=(0, 0, 0)) -> np.ndarray:
    """Lattice indices of the occupied cells of ``occ[x,y,z]`` in z-outer, y, x-inner order."""
    x, y, z = np.nonzero(occ)
    order = np.lexsort((x, y, z))
    xyz = np.stack([x[order], y[order], z[order]], axis=1).astype(np.int32)
    return xyz + np.asarray(offset, np.int32)


def largest_component(occ: np.ndarray) -> np.ndarray:
    """Keep the largest 6-connected component of a boolean grid."""
    from scipy import ndimage

    lab, n = ndimage.label(occ)
    if n <= 1:
        return occ.copy()
    sizes = np.bincount(lab.ravel())
    sizes[0] = 0
    return lab == int(np.argmax(sizes))


def cantilever(nx=40, ny=8, nz=8, voxel_size=0.005, E=1e6, rho=1e3, tip_force=-1.0) -> Scene:
    occ = np.ones((nx, ny, nz), bool)
    xyz = _ordered(occ)
    mats = np.zeros(len(xyz), np.int32)
    fixed = np.nonzero(xyz[:, 0] == 0)[0]
    tip = np.nonzero(xyz[:, 0] == nx - 1)[0]
    fv = np.zeros((len(tip), 3), np.float32)
    fv[:, 2] = tip_force
    return Scene(voxel_size, [Material(E=E, rho=rho)], mats, xyz, fixed_all=fixed, force_idx=tip,
                 force_val=fv, name=f"cantilever_{nx}x{ny}x{nz}")


def lattice(nx=128, ny=128, nz=64, fill=0.85, n_materials=4, seed=2, voxel_size=0.01, nu=0.3) -> Scene:
    rng = np.random.default_rng(seed)
    occ = largest_component(rng.random((nx, ny, nz)) < fill)
    mats_def = []
    for _ in range(n_materials):
        E = float(np.float32(10.0 ** rng.uniform(5.0, 7.0)))
        rho = float(np.float32(rng.uniform(1000.0, 3000.0)))
        mats_def.append(Material(E=E, rho=rho, model=("bilinear", E, 0.2 * E, 0.05 * E, -1.0), nu=nu))
    xyz = _ordered(occ)
    mats = rng.integers(0, n_materials, len(xyz)).astype(np.int32)
    return Scene(voxel_size, mats_def, mats, xyz, gravity=1.0, floor=True,
                 name=f"lattice_{nx}x{ny}x{nz}")


def porous(n=64, sigma=3.0, void=0.4, seed=3, voxel_size=0.01, z_offset=2, collisions=True) -> Scene:
    from scipy import ndimage

    rng = np.random.default_rng(seed)
    field_ = ndimage.gaussian_filter(rng.random((n, n, n)), sigma=sigma, mode="wrap")
    occ = largest_component(field_ > np.quantile(field_, void))
    m = Material(E=5e5, rho=1200.0, nu=0.35, mu_static=1.0, mu_kinetic=0.5)
    xyz = _ordered(occ, offset=(0, 0, z_offset))
    return Scene(voxel_size, [m], np.zeros(len(xyz), np.int32), xyz, gravity=1.0, floor=True,
                 collisions=collisions, name=f"porous_{n}")


def population(n_bodies=4096, side_lo=4, side_hi=24, occupancy=0.6, seed=4, voxel_size=0.01,
               gap=2) -> Scene:
    """Independent bodies laid out on a 2-D grid of cells with ``gap`` empty cells between them,
    so no link joins two bodies.  Per voxel: passive (CTE 0) or active (CTE 0.01) material."""
    rng = np.random.default_rng(seed)
    passive = Material(E=1e6, rho=1e3, mu_static=1.0, mu_kinetic=0.5)
    active = Material(E=1e6, rho=1e3, cte=0.01, mu_static=1.0, mu_kinetic=0.5)
    cols = int(np.ceil(np.sqrt(n_bodies)))
    pitch = side_hi + gap
    xyzs, mats, body = [], [], []
    for b in range(n_bodies):
        sx, sy, sz = rng.integers(side_lo, side_hi + 1, 3)
        occ = largest_component(rng.random((sx, sy, sz)) < occupancy)
        ox, oy = (b % cols) * pitch, (b // cols) * pitch
        xyz = _ordered(occ, offset=(ox, oy, 0))
        xyzs.append(xyz)
        mats.append(rng.integers(0, 2, len(xyz)).astype(np.int32))
        body.append(np.full(len(xyz), b, np.int32))
    return Scene(voxel_size, [passive, active], np.concatenate(mats), np.concatenate(xyzs),
                 gravity=1.0, floor=True, body=np.concatenate(body), name=f"population_{n_bodies}")


def graded_population(n_bodies=256, side=16, occupancy=0.7, seed=5, voxel_size=0.01, gap=2,
                      E_range=(3e5, 3e6)) -> Scene:
    """Bodies of side^3 cells (occupancy, largest component kept) on a 2-D grid, one material per
    voxel with Young's modulus log-uniform in E_range, density 1000, CTE 0.01, friction 1.0/0.5;
    floor and gravity.  ``phase`` (per-voxel actuation phase, uniform in [0, 2 pi)) is attached to
    the returned scene."""
    rng = np.random.default_rng(seed)
    cols = int(np.ceil(np.sqrt(n_bodies)))
    pitch = side + gap
    xyzs, body = [], []
    for b in range(n_bodies):
        occ = largest_component(rng.random((side, side, side)) < occupancy)
        ox, oy = (b % cols) * pitch, (b // cols) * pitch
        xyz = _ordered(occ, offset=(ox, oy, 0))
        xyzs.append(xyz)
        body.append(np.full(len(xyz), b, np.int32))
    xyz = np.concatenate(xyzs)
    n = len(xyz)
    lo, hi = np.log10(E_range[0]), np.log10(E_range[1])
    E = (10.0 ** rng.uniform(lo, hi, n)).astype(np.float32)
    mats = [Material(E=float(e), rho=1e3, cte=0.01, mu_static=1.0, mu_kinetic=0.5) for e in E]
    sc = Scene(voxel_size, mats, np.arange(n, dtype=np.int32), xyz, gravity=1.0, floor=True,
               body=np.concatenate(body), name=f"graded_population_{n_bodies}x{side}")
    sc.phase = rng.uniform(0.0, 2.0 * np.pi, n).astype(np.float32)
    return sc
