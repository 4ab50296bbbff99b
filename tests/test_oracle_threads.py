"""The oracle's OpenMP run (the CPU baseline's configuration) gives the same bits as its serial
run: the Poisson-strain cache is filled by a serial-equivalent pre-pass, and every gather sums in
a fixed order (no GPU)."""
from __future__ import annotations

import ctypes as C

import pytest

from conftest import make_sim, state_diff
from voxelyze_gb300 import scenes as S


@pytest.mark.parametrize("name,mk", [
    ("lattice_poisson", lambda: S.lattice(10, 10, 6)),
    ("porous_collisions", lambda: S.porous(12, sigma=1.2)),
    ("population", lambda: S.population(6, 3, 6)),
])
def test_openmp_run_equals_serial_run(oracle_lib, name, mk):
    oracle_lib.vxo_set_math(0)
    sc = mk()
    a, b = make_sim(oracle_lib, "vxo", sc), make_sim(oracle_lib, "vxo", sc)
    oracle_lib.vxo_set_threads(C.c_void_p(b.h), 8)
    dt = a.recommended_time_step()
    assert b.recommended_time_step() == dt
    for n in (40, 80):
        assert a.do_time_steps(n, dt) == b.do_time_steps(n, dt) == n
        assert state_diff(a, b) == []
