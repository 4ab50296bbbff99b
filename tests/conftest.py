"""Shared fixtures.  CPU tests use the oracle (and the reference build where present); tests marked
``gpu`` drive the product library on cuda:0 and fail if it cannot run there."""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

ORACLE_SO = os.path.join(ROOT, "oracle", "_build", "libvxoracle.so")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libvxref.so")
PRODUCT_SO = os.path.join(ROOT, "voxelyze_gb300", "_build", "libvoxelyze_gb300.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _ensure_built():
    if not (os.path.exists(ORACLE_SO) and os.path.exists(PRODUCT_SO)):
        import __graft_entry__

        __graft_entry__.build()


@pytest.fixture(scope="session")
def oracle_lib():
    _ensure_built()
    lib = ctypes.CDLL(ORACLE_SO)
    lib.vxo_set_math.argtypes = [ctypes.c_int]
    lib.vxo_set_threads.argtypes = [ctypes.c_void_p, ctypes.c_int]
    return lib


@pytest.fixture(scope="session")
def ref_lib():
    if not os.path.exists(REF_SO):
        pytest.skip("reference build (oracle/_ref) not present on this machine")
    return ctypes.CDLL(REF_SO)


@pytest.fixture(scope="session")
def product_lib():
    _ensure_built()
    import voxelyze_gb300

    return voxelyze_gb300.library()


def make_sim(lib, prefix, scene):
    from voxelyze_gb300 import facade as F, scenes as S

    sim = F.Sim(lib, prefix, scene.voxel_size)
    S.apply(scene, sim)
    return sim


def state_diff(a, b):
    """Names of the state arrays in which two simulators differ (bit for bit)."""
    va, vb = a.voxel_state(), b.voxel_state()
    la, lb = a.link_state(), b.link_state()
    bad = []
    for k in ("raw_d", "raw_f", "raw_i"):
        if not np.array_equal(va[k], vb[k]):
            bad.append("voxel." + k)
        A, B = la[k], lb[k]
        if k == "raw_i":  # the last column is the link-material id, numbered per simulator
            A, B = A[:, :5], B[:, :5]
        if not np.array_equal(A, B):
            bad.append("link." + k)
    return bad


def max_rel_pos_err(a, b):
    pa, pb = a.voxel_state()["pos"], b.voxel_state()["pos"]
    return float(np.max(np.abs(pa - pb)) / max(np.max(np.abs(pb)), 1e-30))
