"""The product library loads without a GPU and exports every entry point its public C headers
declare (include/vxg.h, include/vx_capi.h).  No compute call is made here."""
from __future__ import annotations

import os
import re

from conftest import ROOT


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b((?:vxg|vx)_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_headers_declare_entry_points():
    assert "vxg_step" in _declared("vxg.h")
    assert "vx_do_time_step" in _declared("vx_capi.h")


def test_library_exports_all_declared_symbols(product_lib):
    missing = []
    for h in ("vxg.h", "vx_capi.h"):
        for name in _declared(h):
            try:
                getattr(product_lib, name)
            except AttributeError:
                missing.append(name)
    assert missing == []


def test_product_does_not_link_the_oracle(product_lib):
    path = product_lib._name
    deps = open("/proc/self/maps").read()
    assert "libvxoracle" not in os.path.basename(path)
    assert os.path.exists(path) and deps  # loaded in-tree


def test_python_binding_uses_declared_entry_points(product_lib):
    """Every vx_* function voxelyze_gb300.facade binds is declared in include/vx_capi.h."""
    from voxelyze_gb300 import facade as F

    declared = set(_declared("vx_capi.h"))
    bound = {f"vx_{k}" for d in (F._SIGS, F._OPT_SIGS, F._EXT_SIGS) for k in d}
    assert sorted(bound - declared) == []
