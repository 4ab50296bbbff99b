"""Host logic of the gradient check (voxelyze_gb300/gradcheck.py), no GPU: the comparison of an
adjoint with two central differences, and the Richardson extrapolation that removes their O(h^2)
truncation."""
from __future__ import annotations

import numpy as np

from voxelyze_gb300 import gradcheck as G


def _central(f, x, h):
    return (f(x + h) - f(x - h)) / (2 * h)


def test_richardson_removes_the_truncation_of_a_sinusoid():
    """d/dphi of a sin(w t + phi): central differences at 0.16 and 0.04 rad are off by h^2/6
    (4.3e-3 and 2.7e-4 relative); the extrapolation agrees to rounding."""
    a, w, t = 0.1, 2 * np.pi * 2.0, 0.37
    f = lambda phi: a * np.sin(w * t + phi)
    phis = np.linspace(0.1, 6.0, 25)
    exact = a * np.cos(w * t + phis)
    d1 = np.array([_central(f, p, 0.16) for p in phis])
    d2 = np.array([_central(f, p, 0.04) for p in phis])
    rows = G.compare(exact, d1, d2)
    rel1 = np.abs(d1 - exact) / np.abs(exact)
    assert np.allclose(rel1, 0.16 ** 2 / 6, rtol=2e-3)
    err = np.array([r["richardson_error"] for r in rows])
    assert err.max() < 1e-6
    assert all(r["smooth"] for r in rows)


def test_distance_to_the_interval_and_branch_crossings():
    rows = G.compare([1.0, 1.0, 2.0], [0.98, 1.2, 1.0], [1.02, 1.15, 3.0])
    assert rows[0]["distance"] == 0.0                       # inside [0.98, 1.02]
    assert abs(rows[1]["distance"] - 0.15 / 1.2) < 1e-12    # below [1.15, 1.2]
    assert rows[0]["smooth"] and rows[1]["smooth"]          # within 10 % of each other
    assert not rows[2]["smooth"]                            # 1.0 vs 3.0: a branch was crossed
