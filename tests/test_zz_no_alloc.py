"""vx_state_info_into: the stateInfo reduction written to caller device memory through a fixed
scratch array, checked against vx_state_info_device (the allocating reduction) on the same state.

MIN and MAX must be identical; TOTAL and AVERAGE are double sums over a different partition of the
elements, so they agree to a relative 1e-6.  Each comparison is made on two calls in a row (the
second finds the scratch counter left at zero by the first).  The output buffer is allocated here
by the test; the entry point itself allocates nothing.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import make_sim
from voxelyze_gb300 import facade as F, scenes as S

pytestmark = pytest.mark.gpu

INFOS = (F.DISPLACEMENT, F.VELOCITY, F.KINETIC_ENERGY, F.ANGULAR_DISPLACEMENT, F.ANGULAR_VELOCITY,
         F.ENG_STRESS, F.ENG_STRAIN, F.STRAIN_ENERGY, F.MASS)
TYPES = (F.MIN, F.MAX, F.TOTAL, F.AVERAGE)


def _bind(lib):
    into = lib.vx_state_info_into
    into.restype = C.c_int
    into.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_char_p)]
    dev = lib.vx_state_info_device
    dev.restype = C.c_float
    dev.argtypes = [C.c_void_p, C.c_int, C.c_int]
    return into, dev


def _check_scene(lib, sim, torch):
    into, dev = _bind(lib)
    out = torch.full((len(INFOS), len(TYPES)), float("nan"), device="cuda", dtype=torch.float32)
    for call in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        for a, info in enumerate(INFOS):
            for b, t in enumerate(TYPES):
                why = C.c_char_p()
                rc = into(C.c_void_p(sim.h), info, t, C.c_void_p(out[a, b].data_ptr()), C.byref(why))
                assert rc == 0, (info, t, why.value)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        for a, info in enumerate(INFOS):
            for b, t in enumerate(TYPES):
                ref = dev(C.c_void_p(sim.h), info, t)
                if t in (F.MIN, F.MAX):
                    assert got[a, b] == np.float32(ref), (call, info, t, got[a, b], ref)
                else:
                    assert abs(float(got[a, b]) - ref) <= 1e-6 * max(abs(ref), 1e-30), (call, info, t, got[a, b], ref)


@pytest.mark.parametrize("precision", [0, 1])
def test_matches_allocating_reduction(product_lib, precision):
    torch = pytest.importorskip("torch")
    sc = S.lattice(24, 20, 12)
    g = make_sim(product_lib, "vx", sc)
    if precision:
        assert product_lib.vx_set_precision(C.c_void_p(g.h), 1) == 0
    dt = g.recommended_time_step()
    assert g.do_time_steps(150, dt) == 150
    _check_scene(product_lib, g, torch)
    assert g.do_time_steps(50, dt) == 50  # state moved on: same agreement
    _check_scene(product_lib, g, torch)


def test_rejections_leave_output_untouched(product_lib):
    torch = pytest.importorskip("torch")
    into, _ = _bind(product_lib)
    g = make_sim(product_lib, "vx", S.cantilever(6, 2, 2, voxel_size=0.005, tip_force=-0.01))
    out = torch.full((1,), 7.0, device="cuda", dtype=torch.float32)
    why = C.c_char_p()
    # host edits not yet uploaded are refused (uploading could allocate)
    assert into(C.c_void_p(g.h), F.MASS, F.TOTAL, C.c_void_p(out.data_ptr()), C.byref(why)) != 0
    assert b"not on the device" in why.value
    g.do_time_steps(5, -1.0)
    assert into(C.c_void_p(g.h), F.PRESSURE, F.TOTAL, C.c_void_p(out.data_ptr()), C.byref(why)) != 0
    assert b"PRESSURE" in why.value
    assert into(C.c_void_p(g.h), F.MASS, 9, C.c_void_p(out.data_ptr()), C.byref(why)) != 0
    torch.cuda.synchronize()
    assert out.item() == 7.0


def test_counts_beyond_the_scratch_are_refused(product_lib):
    """160x160x80 lattice: ~1.7 M voxels (reduced), ~4.4 M links (more than 4,194,304: refused)."""
    torch = pytest.importorskip("torch")
    into, dev = _bind(product_lib)
    g = make_sim(product_lib, "vx", S.lattice(160, 160, 80))
    assert g.voxel_count() <= 4194304 < g.link_count()
    g.do_time_steps(2, g.recommended_time_step())
    out = torch.full((2,), 7.0, device="cuda", dtype=torch.float32)
    why = C.c_char_p()
    rc = into(C.c_void_p(g.h), F.ENG_STRAIN, F.MAX, C.c_void_p(out[0].data_ptr()), C.byref(why))
    assert rc != 0 and b"4,194,304" in why.value
    assert into(C.c_void_p(g.h), F.MASS, F.TOTAL, C.c_void_p(out[1].data_ptr()), C.byref(why)) == 0, why.value
    torch.cuda.synchronize()
    assert out[0].item() == 7.0
    ref = dev(C.c_void_p(g.h), F.MASS, F.TOTAL)
    assert abs(out[1].item() - ref) <= 1e-6 * ref
