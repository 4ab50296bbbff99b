"""Host-side check of the hand-written step adjoint (voxelyze_gb300/csrc/vx_adjoint.cuh), compiled
with g++: its forward recomputation matches vx64::link_update / vx64::voxel_update bit for bit on
random inputs, and its derivatives match central differences of that forward output by output
(worst relative error, floored at 1e-4 of each output's largest gradient component, below 2e-3).
Large-angle links (both frame formulas of orientLink, strains of 0.1-0.6): the difference nearest
the adjoint among six steps, floored at 1e-3 of each output's largest component, below 5e-3.
Links with Poisson's ratio 0.3 also take their ends' Poisson strains as inputs and give the axial
strain as an output; a voxel's Poisson strains (CVX_Voxel::strain(true)) are checked against
differences of vx64::poisson_strain_links with respect to its links' strains, below 2e-3."""
from __future__ import annotations

import os
import subprocess

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "adjoint_check.cpp")


def test_adjoint_against_finite_differences_on_cpu(tmp_path):
    exe = str(tmp_path / "adjoint_check")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "voxelyze_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"), SRC, "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    print(out.stdout)
    assert out.returncode == 0, out.stdout
    res = {}
    for line in out.stdout.splitlines():
        p = line.split()
        res[p[0]] = [float(x) for x in p[1:]]
    assert res["link_forward_mismatch"][0] == 0
    assert res["voxel_forward_mismatch"][0] == 0
    assert res["link"][1] > 10000 and res["link"][0] < 2e-3
    assert res["link_large"][2] >= 100 and res["link_large"][0] < 5e-3
    assert res["poisson"][1] > 1000 and res["poisson"][0] < 2e-3
    assert res["voxel"][1] > 10000 and res["voxel"][0] < 2e-3
