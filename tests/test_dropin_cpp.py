"""The drop-in C++ API: the reference README example compiled against include/ and linked with the
product library (compile check on CPU; run and compare with the oracle on the GPU)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from voxelyze_gb300 import facade as F

SRC = os.path.join(ROOT, "tests", "cpp", "dropin_example.cpp")
LIBDIR = os.path.join(ROOT, "voxelyze_gb300", "_build")


def _compile(tmp_path):
    exe = str(tmp_path / "dropin_example")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), SRC,
                    "-L", LIBDIR, "-lvoxelyze_gb300", f"-Wl,-rpath,{LIBDIR}", "-o", exe], check=True)
    return exe


def test_readme_example_compiles_and_links(product_lib, tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_readme_example_runs_like_the_oracle(product_lib, oracle_lib, tmp_path):
    exe = _compile(tmp_path)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines()
    rows = np.array([[float(x) for x in line.split()[1:]] for line in out[:3]])
    oracle_lib.vxo_set_math(1)
    s = F.Sim(oracle_lib, "vxo", 0.005)
    m = s.add_material(1000000, 1000)
    v1, _, v3 = s.set_voxel(m, 0, 0, 0), s.set_voxel(m, 1, 0, 0), s.set_voxel(m, 2, 0, 0)
    s.set_fixed_all(v1)
    s.set_force(v3, 0, 0, -1)
    for _ in range(100):
        s.do_time_step(-1.0)
    st = s.voxel_state()
    ref = np.concatenate([st["pos"], st["orient"]], axis=1)
    assert np.array_equal(rows, ref)
    assert out[3].startswith(f"links {s.link_count()}")
