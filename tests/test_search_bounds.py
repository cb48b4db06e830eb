"""CPU checks of the float bounds behind the GPU search and the far-field tiles.

* The search's float fast accept implies the reference predicate, and its
  float cell range covers every cell the double range covered: a C
  restatement of those formulas (tests/search_bounds.c) on seeded adversarial
  cases (thin shell |dr| ~ hh, periodic edges, six box sizes).
* The far-field tiles' interpolation error: 8 Chebyshev nodes on a tile whose
  half-width is at most 0.2 of the distance to the pole of the 1/V^(2r) wing
  terms.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fast_accept_and_cell_range(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "search_bounds")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "search_bounds.c"), "-lm"], check=True)
    r = subprocess.run([exe, "1000000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "fast_accept bad=0" in r.stdout and "cell_range bad=0" in r.stdout


def _cheb_rel_err(t, m, n):
    k = np.arange(m)
    x = np.cos((2 * k + 1) * np.pi / (2 * m))
    lam = np.array([1.0 / np.prod([x[i] - x[j] for j in range(m) if j != i]) for i in range(m)])
    s = np.linspace(-1, 1, 4001)
    d = s[:, None] - x[None, :]
    d[d == 0] = 1e-300
    L = (lam / d) / np.sum(lam / d, axis=1, keepdims=True)
    f = lambda v: (1 + t * v) ** (-n)
    return np.max(np.abs(L @ f(x) - f(s)) / np.abs(f(s)))


def test_tile_interpolation_error():
    # tile half-width 32 pixels, nearest pixel edge >= 128 pixels from the line centre
    t = 32.0 / (128.0 + 32.0)
    assert _cheb_rel_err(t, 8, 2) < 3e-7      # the dominant 1/V^2 term
    assert _cheb_rel_err(t, 8, 4) < 7e-6      # 1/V^4, a few percent of the wing there
