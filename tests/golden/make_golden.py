"""Generates the golden fixtures in this directory from the REFERENCE library compiled from its own
sources (oracle/build_ref.sh -> oracle/_ref/libvxref.so).  Run here, where the reference tree
exists:  python tests/golden/make_golden.py        (all fixtures)
         python tests/golden/make_golden.py json   (the scene file and mesh only)

Each fixture holds the reference's full state after a known number of steps of one scene, either
in full (small scenes) or as SHA-256 digests of the state bytes plus a sample of voxels (larger
scenes), together with the platform it was generated on (the C library's sin/cos/acos/powf enter
the bits).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import platform
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from voxelyze_gb300 import facade as F, scenes as S  # noqa: E402


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def snapshot(sim, full: bool, sample=None):
    v, l = sim.voxel_state(), sim.link_state()
    out = {"voxel_d": digest(v["raw_d"]), "voxel_f": digest(v["raw_f"]), "voxel_i": digest(v["raw_i"]),
           "link_d": digest(l["raw_d"]), "link_f": digest(l["raw_f"]), "link_i": digest(l["raw_i"][:, :5])}
    arrays = {}
    if full:
        arrays = {"voxel_d": v["raw_d"], "link_d": l["raw_d"], "link_f": l["raw_f"]}
    elif sample is not None:
        arrays = {"voxel_d_sample": v["raw_d"][sample]}
    return out, arrays


SCENES = {
    # name: (scene factory, steps per checkpoint, checkpoints, dt mode, full arrays)
    "cantilever_40x8x8": (lambda: S.cantilever(), 500, 2, "recommended", False),
    "cantilever_8x3x3": (lambda: S.cantilever(8, 3, 3, voxel_size=0.005, tip_force=-0.05), 200, 2, "recommended", True),
    "lattice_16x16x8": (lambda: S.lattice(16, 16, 8), 100, 2, "recommended", False),
    "lattice_8x8x6_dt_every_step": (lambda: S.lattice(8, 8, 6), 20, 2, "every_step", False),
    "porous_16_collisions": (lambda: S.porous(16, sigma=1.5), 100, 2, "recommended", False),
    "population_8": (lambda: S.population(8, 3, 7), 100, 1, "recommended", False),
}


def save_scene_json(lib):
    """scene_ref.vxl.json: CVoxelyze::saveJSON of the scene test_scene_json.build_scene makes."""
    from test_scene_json import build_scene

    sim = build_scene(lib, "vxr")
    assert sim.save_json(os.path.join(HERE, "scene_ref.vxl.json"))


def save_mesh(lib):
    """mesh_ref.npz: the reference CVX_MeshRender of test_mesh.heated_scene with test_mesh.heat
    applied: vertices, normals, quads, edges, the quad colours of each colouring, the OBJ text."""
    from test_mesh import heat, heated_scene

    sc = heated_scene()
    sim = F.Sim(lib, "vxr", sc.voxel_size)
    S.apply(sc, sim)
    heat(sim, sim.voxel_count())
    sim.mesh_generate()
    out = {}
    for coloring in (F.MESH_MATERIAL, F.MESH_FAILURE, F.MESH_STATE_INFO):
        sim.mesh_update(coloring, F.DISPLACEMENT if coloring != F.MESH_STATE_INFO else F.KINETIC_ENERGY)
        out[f"colors{coloring}"] = sim.mesh()["colors"]
    m = sim.mesh()
    for k in ("vertices", "normals", "quads", "lines"):
        out[k] = m[k]
    obj = os.path.join(HERE, "_mesh.obj")
    sim.mesh_save_obj(obj)
    out["obj"] = np.array(open(obj).read())
    os.remove(obj)
    np.savez_compressed(os.path.join(HERE, "mesh_ref.npz"), **out)


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvxref.so"))
    save_scene_json(lib)
    save_mesh(lib)
    if sys.argv[1:] in (["json"], ["mesh"]):
        return
    meta = {"platform": platform.machine(), "libc": platform.libc_ver()[1], "scenes": {}}
    for name, (mk, steps, cps, mode, full) in SCENES.items():
        sc = mk()
        sim = F.Sim(lib, "vxr", sc.voxel_size)
        S.apply(sc, sim)
        dt = sim.recommended_time_step()
        use = -1.0 if mode == "every_step" else dt
        rng = np.random.default_rng(0)
        sample = np.sort(rng.choice(sim.voxel_count(), size=min(64, sim.voxel_count()), replace=False))
        entry = {"steps": steps, "dt": float(dt), "dt_mode": mode, "n_voxels": sim.voxel_count(),
                 "n_links": sim.link_count(), "checkpoints": [], "sample": sample.tolist()}
        arrays = {}
        for k in range(cps):
            n = sim.do_time_steps(steps, use)
            assert n == steps, (name, n)
            snap, arr = snapshot(sim, full, sample)
            if name.startswith("porous"):
                pairs = sim.collisions()
                snap["pairs"] = digest(pairs.astype(np.int32))
                snap["n_pairs"] = int(len(pairs))
            snap["time"] = float(sim.current_time())
            entry["checkpoints"].append(snap)
            for key, a in arr.items():
                arrays[f"cp{k}_{key}"] = a
        if arrays:
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
        meta["scenes"][name] = entry
        print(name, entry["n_voxels"], entry["n_links"])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main()
