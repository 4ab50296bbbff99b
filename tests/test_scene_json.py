"""*.vxl.json scene files (CVoxelyze::loadJSON / saveJSON, src/Voxelyze.cpp:61-241) against the
reference build.

The product writes the reference's layout (keys, order, indentation) and the shortest decimal form
of each double that reads back to it; the reference's rapidjson writer sometimes picks another
17-digit form of the same double.  So files are compared as text with every number replaced by a
placeholder, and the numbers are compared as the doubles they read back to.  Both libraries load
each other's files into scenes that save to the same document.  These tests run on the host only
(scene building, no time step): where the reference build is absent the committed fixture written
by it (tests/golden/scene_ref.vxl.json, tests/golden/make_golden.py) stands in.
"""
from __future__ import annotations

import json
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from voxelyze_gb300 import facade as F, scenes as S

NUM = re.compile(r"-?\d+(?:\.\d+)?(?:[eE][+-]?\d+)?")
GOLDEN = os.path.join(ROOT, "tests", "golden", "scene_ref.vxl.json")


def build_scene(lib, prefix):
    """A scene exercising every key the writer emits except data-model materials (which the
    reference cannot read back): two linear materials with Poisson's ratio, CTE, friction, damping,
    a failure strain and a name; gravity, floor, ambient temperature; externals with fixed DOFs,
    prescribed translation and rotation, forces and moments, one shared by several voxels."""
    sc = S.cantilever(6, 3, 2)
    sim = F.Sim(lib, prefix, sc.voxel_size)
    S.apply(sc, sim)
    k = sim.add_material(2.5e6, 1200.0)
    sim.material_set(k, F.PROP_POISSON, 0.3)
    sim.material_set(k, F.PROP_CTE, 0.01)
    sim.material_set(k, F.PROP_MU_STATIC, 0.8)
    sim.material_set(k, F.PROP_MU_KINETIC, 0.4)
    sim.material_set(k, F.PROP_ZETA_GLOBAL, 0.05)
    sim.set_model_linear(k, 2.5e6, 3.0e5)
    for x in range(6, 9):
        sim.set_voxel(k, x, 0, 0)
    sim.set_gravity(1.0)
    sim.enable_floor(True)
    sim.set_ambient_temperature(0.25, False)
    sim.set_moment(3, 0.1, -0.2, 1e-7)
    sim.set_displacement(5, F.Z_TRANSLATE, 0.001)
    sim.set_displacement(7, F.X_ROTATE, 0.02)
    sim.set_force(9, 0.0, 0.5, -1.25)
    return sim


def split(text):
    """(layout with numbers replaced, list of numbers as doubles)"""
    return NUM.sub("#", text), [float(x) for x in NUM.findall(text)]


def save(sim, path):
    assert sim.save_json(str(path))
    return open(path).read()


def test_product_file_is_valid_json_with_the_reference_keys(product_lib, tmp_path):
    text = save(build_scene(product_lib, "vx"), tmp_path / "p.vxl.json")
    doc = json.loads(text)
    assert list(doc)[:5] == ["voxelSize", "relativeAmbientTemperature", "gravityAcceleration", "floorEnabled",
                             "materials"]
    assert len(doc["voxels"]) % 4 == 0 and len(doc["materials"]) == 2
    assert {tuple(e["voxelIndices"][:1]) for e in doc["externals"]}


def test_save_matches_reference_build(product_lib, ref_lib, tmp_path):
    ours = save(build_scene(product_lib, "vx"), tmp_path / "p.vxl.json")
    ref = save(build_scene(ref_lib, "vxr"), tmp_path / "r.vxl.json")
    lo, no = split(ours)
    lr, nr = split(ref)
    assert lo == lr                      # same keys, order, layout, integers and literals
    assert no == nr                      # every number reads back to the same double
    differing = sum(a != b for a, b in zip(NUM.findall(ours), NUM.findall(ref)))
    print(f"{len(no)} numbers, {differing} written with another 17-digit form of the same double")


def test_each_loads_the_others_file(product_lib, ref_lib, tmp_path):
    ours = save(build_scene(product_lib, "vx"), tmp_path / "p.vxl.json")
    ref = save(build_scene(ref_lib, "vxr"), tmp_path / "r.vxl.json")
    # the product reads the reference's file; the reference reads the product's
    p2 = F.Sim(product_lib, "vx", 0.001)
    assert p2.load_json(str(tmp_path / "r.vxl.json"))
    r2 = F.Sim(ref_lib, "vxr", 0.001)
    assert r2.load_json(str(tmp_path / "p.vxl.json"))
    again_p = save(p2, tmp_path / "p2.vxl.json")
    again_r = save(r2, tmp_path / "r2.vxl.json")
    # neither reader restores gravity, floor or ambient temperature (the reference reads only the
    # voxel size, materials, voxels and externals), so compare what the files carry over
    for a, b in ((again_p, ref), (again_r, ours), (again_p, again_r)):
        da, db = json.loads(a), json.loads(b)
        for key in ("voxelSize", "materials", "voxels", "externals"):
            assert da[key] == db[key], key
    assert p2.voxel_count() == r2.voxel_count() and p2.link_count() == r2.link_count()


def test_golden_reference_file_round_trips(product_lib, tmp_path):
    """The committed file written by the reference build loads and saves back to the same document
    (the reference's own writer does not restore what its reader skips, so those keys go)."""
    sim = F.Sim(product_lib, "vx", 0.001)
    assert sim.load_json(GOLDEN)
    again = json.loads(save(sim, tmp_path / "g.vxl.json"))
    gold = json.load(open(GOLDEN))
    for key in ("voxelSize", "materials", "voxels", "externals"):
        assert again[key] == gold[key], key
    assert sim.voxel_count() == len(gold["voxels"]) // 4


def test_kind_rules_and_bad_files(product_lib, tmp_path):
    """Keys whose value has another kind than the reference tests for are skipped (an integer
    literal is not a double); an unparsable file loads as an empty document; a missing file fails."""
    p = tmp_path / "k.vxl.json"
    p.write_text('{"voxelSize": 0.01, "materials": [{"youngsModulus": 5000000, "density": 500.0}, '
                 '{"youngsModulus": 2.0e6, "density": 700, "red": 3, "poissonsRatio": 0.25}], '
                 '"voxels": [0, 0, 0, 0, 1, 0, 0, 1]}')
    sim = F.Sim(product_lib, "vx", 0.001)
    assert sim.load_json(str(p))
    d = json.loads(save(sim, tmp_path / "k2.vxl.json"))
    assert d["voxelSize"] == 0.01 and sim.voxel_count() == 2 and sim.link_count() == 1
    m0, m1 = d["materials"]
    assert m0["youngsModulus"] == 1.0 and "density" not in m0      # the model key was skipped
    assert m1["youngsModulus"] == 2.0e6 and "density" not in m1 and m1["red"] == 3
    assert m1["poissonsRatio"] == pytest.approx(0.25)
    bad = tmp_path / "bad.vxl.json"
    bad.write_text('{"voxelSize": 0.01, "materials": [')
    assert sim.load_json(str(bad)) and sim.voxel_count() == 0
    assert not sim.load_json(str(tmp_path / "missing.vxl.json"))


@pytest.mark.gpu
def test_loaded_scene_steps_like_the_built_one(product_lib, tmp_path):
    """A scene saved and loaded back steps bit-identically to the scene built through the API (the
    file carries everything the step uses except the globals the reader skips, set again here)."""
    from conftest import state_diff

    a = build_scene(product_lib, "vx")
    save(a, tmp_path / "s.vxl.json")
    b = F.Sim(product_lib, "vx", 0.001)
    assert b.load_json(str(tmp_path / "s.vxl.json"))
    b.set_gravity(1.0)
    b.enable_floor(True)
    b.set_ambient_temperature(0.25, False)
    dt = a.recommended_time_step()
    assert dt > 0 and b.recommended_time_step() == dt
    assert a.do_time_steps(200, dt) == b.do_time_steps(200, dt) == 200
    assert state_diff(a, b) == []
    assert np.array_equal(a.voxel_state()["pos"], b.voxel_state()["pos"])


def test_cpp_scene_file_calls(product_lib, tmp_path):
    """saveJSON, the JSON constructor and loadJSON from C++ against include/ (host only)."""
    import subprocess

    src = os.path.join(ROOT, "tests", "cpp", "json_example.cpp")
    libdir = os.path.join(ROOT, "voxelyze_gb300", "_build")
    exe = str(tmp_path / "json_example")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-L", libdir,
                    "-lvoxelyze_gb300", f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    out = subprocess.run([exe, str(tmp_path / "a.vxl.json"), str(tmp_path / "b.vxl.json")], check=True,
                         capture_output=True, text=True).stdout.split()
    got = dict(zip(out[::2], out[1::2]))
    assert got == {"voxels": "3", "links": "2", "materials": "1", "nu": "0.3", "loaded": "1", "same": "1"}


def _random_scene(lib, prefix, seed):
    """Seeded random scene: 1-4 linear materials with random E, density, Poisson's ratio, CTE,
    friction and damping; a random occupancy of a small box with a random material per voxel;
    random externals (fixed DOFs, prescribed translations and rotations, forces, moments)."""
    rng = np.random.default_rng(seed)
    sim = F.Sim(lib, prefix, float(rng.choice([0.001, 0.005, 0.01])))
    mats = []
    for _ in range(int(rng.integers(1, 5))):
        E, rho = float(10 ** rng.uniform(4, 7)), float(rng.uniform(500, 3000))
        m = sim.add_material(E, rho)
        if rng.random() < 0.5:
            sim.material_set(m, F.PROP_POISSON, float(rng.uniform(0, 0.45)))
        sim.material_set(m, F.PROP_CTE, float(rng.uniform(0, 0.02)))
        sim.material_set(m, F.PROP_MU_STATIC, float(rng.uniform(0, 1)))
        sim.material_set(m, F.PROP_MU_KINETIC, float(rng.uniform(0, 0.5)))
        sim.material_set(m, F.PROP_ZETA_GLOBAL, float(rng.uniform(0, 0.2)))
        if rng.random() < 0.3:
            sim.set_model_linear(m, E, float(rng.uniform(0.05, 0.5)))
        mats.append(m)
    n = 0
    for z in range(3):
        for y in range(4):
            for x in range(5):
                if rng.random() < 0.6:
                    sim.set_voxel(mats[int(rng.integers(len(mats)))], x, y, z)
                    n += 1
    for v in rng.choice(n, size=min(n, 6), replace=False) if n else []:
        v = int(v)
        kind = int(rng.integers(4))
        if kind == 0:
            sim.set_fixed(v, int(rng.integers(1, 64)))
        elif kind == 1:
            sim.set_force(v, *(float(x) for x in rng.normal(0, 1, 3)))
        elif kind == 2:
            sim.set_moment(v, *(float(x) for x in rng.normal(0, 1e-3, 3)))
        else:
            sim.set_displacement(v, int(rng.choice([F.X_TRANSLATE, F.Y_TRANSLATE, F.Z_TRANSLATE])),
                                 float(rng.normal(0, 1e-3)))
    return sim


def _within_one_ulp(a, b):
    """Equal JSON values, numbers allowed to differ by one ulp."""
    if isinstance(a, dict):
        return isinstance(b, dict) and a.keys() == b.keys() and all(_within_one_ulp(a[k], b[k]) for k in a)
    if isinstance(a, list):
        return isinstance(b, list) and len(a) == len(b) and all(_within_one_ulp(x, y) for x, y in zip(a, b))
    if isinstance(a, float) and isinstance(b, float):
        return a == b or np.nextafter(a, b) == b
    return a == b


@pytest.mark.parametrize("seed", range(24))
def test_random_scenes_match_reference_build(product_lib, ref_lib, tmp_path, seed):
    """Seeded random scenes save to the reference build's document (layout, and every number as a
    double), and each library loads the other's file back to the same scene.  This library reads
    every number correctly rounded; the reference's reader (rapidjson's default number parsing)
    reads some 17-digit numbers one ulp off, so in that direction numbers may differ by one ulp."""
    ours = save(_random_scene(product_lib, "vx", seed), tmp_path / "p.vxl.json")
    ref = save(_random_scene(ref_lib, "vxr", seed), tmp_path / "r.vxl.json")
    lo, no = split(ours)
    lr, nr = split(ref)
    assert lo == lr
    assert no == nr
    p2 = F.Sim(product_lib, "vx", 0.001)
    r2 = F.Sim(ref_lib, "vxr", 0.001)
    assert p2.load_json(str(tmp_path / "r.vxl.json")) and r2.load_json(str(tmp_path / "p.vxl.json"))
    da = json.loads(save(p2, tmp_path / "p2.vxl.json"))  # ours reading the reference's file
    db = json.loads(save(r2, tmp_path / "r2.vxl.json"))  # the reference reading ours
    orig = json.loads(ours)
    for key in ("voxelSize", "materials", "voxels", "externals"):
        assert da[key] == orig[key], key                  # exact
        assert _within_one_ulp(db[key], orig[key]), key
    assert p2.voxel_count() == r2.voxel_count() and p2.link_count() == r2.link_count()
