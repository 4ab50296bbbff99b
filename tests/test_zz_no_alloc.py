"""vx_state_info_into: the stateInfo reduction written to caller device memory through a fixed
scratch array, for callers that may not allocate.  Checked against vx_state_info_device (the
allocating reduction) on the same state, and its MIN and MAX against the host stateInfo, which
follows the reference's loop (src/Voxelyze.cpp:752-800).

MIN and MAX must be identical; TOTAL and AVERAGE are double sums over a different partition of the
elements, so they agree to a relative 1e-6.  Each comparison is made on two calls in a row (the
second finds the scratch counter left at zero by the first).  The output buffer is allocated here
by the test; the entry point itself allocates nothing, which one test checks by issuing a call while
its stream is captured in global mode: an allocation or a synchronisation inside the call would make
that capture fail.
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
    host = lib.vx_state_info
    host.restype = C.c_float
    host.argtypes = [C.c_void_p, C.c_int, C.c_int]
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
                    h = np.float32(host(C.c_void_p(sim.h), info, t))
                    if info == F.ANGULAR_DISPLACEMENT:
                        # the host takes the C library's acos, the device a correctly rounded one:
                        # their doubles can differ by one ulp, which after the float cast is at most
                        # one float ulp
                        assert abs(got[a, b] - h) <= np.spacing(h), (call, info, t, got[a, b], h)
                    else:
                        assert got[a, b] == h, (call, info, t, got[a, b], h)
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


def _cuda_driver():
    import ctypes.util

    name = ctypes.util.find_library("cuda") or "libcuda.so.1"
    cu = C.CDLL(name)
    cu.cuStreamBeginCapture_v2.argtypes = [C.c_void_p, C.c_int]
    cu.cuStreamEndCapture.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    cu.cuGraphInstantiateWithFlags.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_ulonglong]
    cu.cuGraphLaunch.argtypes = [C.c_void_p, C.c_void_p]
    cu.cuStreamSynchronize.argtypes = [C.c_void_p]
    cu.cuGraphExecDestroy.argtypes = [C.c_void_p]
    cu.cuGraphDestroy.argtypes = [C.c_void_p]
    return cu


@pytest.mark.parametrize("precision", [0, 1])
def test_no_allocation_or_synchronisation_inside_the_call(product_lib, precision):
    """After a first call (which looks the scratch up), a second call is issued while the
    simulation's stream is captured in global mode.  Global mode refuses allocations and
    synchronisations while the capture is open, so a call that made one would fail or leave the
    capture invalidated.  The captured work is then run once and its value compared with a plain
    call's.  In FP32C the state is stepped between the calls, so the call has state fields to
    convert."""
    torch = pytest.importorskip("torch")
    into, dev = _bind(product_lib)
    cu = _cuda_driver()
    product_lib.vx_engine.restype = C.c_void_p
    product_lib.vx_engine.argtypes = [C.c_void_p]
    product_lib.vxg_stream.restype = C.c_void_p
    product_lib.vxg_stream.argtypes = [C.c_void_p]
    g = make_sim(product_lib, "vx", S.lattice(12, 10, 8))
    if precision:
        assert product_lib.vx_set_precision(C.c_void_p(g.h), 1) == 0
    dt = g.recommended_time_step()
    assert g.do_time_steps(40, dt) == 40
    out = torch.full((2,), float("nan"), device="cuda", dtype=torch.float32)
    torch.cuda.synchronize()
    why = C.c_char_p()
    assert into(C.c_void_p(g.h), F.KINETIC_ENERGY, F.MAX, C.c_void_p(out[0].data_ptr()), C.byref(why)) == 0, why.value
    assert g.do_time_steps(10, dt) == 10
    stream = product_lib.vxg_stream(product_lib.vx_engine(C.c_void_p(g.h)))
    assert stream
    p1 = C.c_void_p(out[1].data_ptr())  # nothing of torch runs while the capture is open
    torch.cuda.synchronize()
    assert cu.cuStreamBeginCapture_v2(C.c_void_p(stream), 0) == 0  # 0: CU_STREAM_CAPTURE_MODE_GLOBAL
    rc = into(C.c_void_p(g.h), F.KINETIC_ENERGY, F.MAX, p1, C.byref(why))
    graph = C.c_void_p()
    end = cu.cuStreamEndCapture(C.c_void_p(stream), C.byref(graph))
    assert rc == 0, why.value
    assert end == 0, f"capture invalidated (CUresult {end}): the call allocated or synchronised"
    exe = C.c_void_p()
    assert cu.cuGraphInstantiateWithFlags(C.byref(exe), graph, 0) == 0
    assert cu.cuGraphLaunch(exe, C.c_void_p(stream)) == 0
    assert cu.cuStreamSynchronize(C.c_void_p(stream)) == 0
    cu.cuGraphExecDestroy(exe)
    cu.cuGraphDestroy(graph)
    ref = dev(C.c_void_p(g.h), F.KINETIC_ENERGY, F.MAX)
    assert out[1].item() == np.float32(ref)
