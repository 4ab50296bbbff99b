"""The correctly rounded sin/cos/acos the FP64 GPU path uses (voxelyze_gb300/csrc/vx_crmath.h),
checked on the host against 256-bit arithmetic on the argument ranges the time step produces, plus
edge points.  The same header compiles into the device code; tests/test_gpu_parity.py checks the
device evaluation against this host evaluation bit for bit."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

mp = pytest.importorskip("mpmath")
from mpmath.libmp.libmpf import to_float  # noqa: E402


def _eval(lib, fn, x):
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    f = np.zeros(len(x), np.int32)
    lib.vxo_crmath_eval(fn, len(x), x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p),
                        f.ctypes.data_as(C.c_void_p))
    return y, f


def _inputs(fn, n, seed):
    rng = np.random.default_rng(seed)
    if fn in (0, 1):  # half angles from FromRotationVector / FromAngleToPosX: [0, pi]
        x = np.concatenate([rng.uniform(0, 3.2, n // 2), 10 ** rng.uniform(-9, 0, n // 4),
                            rng.uniform(1.55, 1.59, n // 4), [0.0, 1e-300, np.pi / 2, np.pi, 3.0]])
    else:  # acos of quaternion w and normalised components: [-1, 1]
        x = np.concatenate([rng.uniform(-1, 1, n // 2), 1 - 10 ** rng.uniform(-15, -1, n // 4),
                            -1 + 10 ** rng.uniform(-15, -1, n // 4), [-1.0, 1.0, 0.0, 0.5, -0.5, 0.999, -0.999]])
    return x


@pytest.mark.parametrize("fn,name", [(0, "sin"), (1, "cos"), (2, "acos")])
def test_correctly_rounded(oracle_lib, fn, name):
    mp.mp.prec = 256
    x = _inputs(fn, 6000, 10 + fn)
    y, flags = _eval(oracle_lib, fn, x)
    ref = {0: mp.sin, 1: mp.cos, 2: mp.acos}[fn]
    bad = [float(xi) for xi, yi in zip(x, y) if to_float(ref(mp.mpf(float(xi)))._mpf_, rnd="n") != yi]
    assert bad == []
    assert int((flags & 1).sum()) == 0  # no uncertified rounding on these inputs
