"""GB300-native time-step engine for Voxelyze scenes.

The product is the shared library built from ``voxelyze_gb300/csrc`` (sm_103a CUDA kernels, the
``vxg_*`` engine C ABI, and the drop-in ``CVoxelyze`` C++ API with its ``vx_*`` C facade).  This
package only locates and loads it; :mod:`voxelyze_gb300.facade` binds the facade and
:mod:`voxelyze_gb300.scenes` generates the seeded workloads.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvoxelyze_gb300.so")
_LIB = None


def library() -> C.CDLL:
    """Load the product library.  Raises if it has not been built: there is no fallback path."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"{LIB_PATH} is missing; build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        _LIB = C.CDLL(LIB_PATH)
    return _LIB


def Sim(voxel_size: float = 0.001):
    """A drop-in ``CVoxelyze`` instance on the GPU, driven through the ``vx_*`` facade."""
    from .facade import Sim as _Sim

    return _Sim(library(), "vx", voxel_size)
