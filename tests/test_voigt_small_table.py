"""The small-damping Voigt form of the FP32 deposit (fsg_voigt.cuh,
voigt_small32) from the generated table (voigt_table.h, FSG_KTAB_INIT),
evaluated here in float64 with the device's interval and cubic, against
scipy's Faddeeva function: H within 6e-7 relative for a <= 2e-3 on [0, 16),
and the derivative form of the backward kernel against central differences
of wofz."""
import os
import re

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(HERE, "..", "fake_spectra_gb300", "csrc", "voigt_table.h")


def _ktab():
    text = open(HEADER).read()
    body = text[text.index("#define FSG_KTAB_INIT"):]
    body = body[:body.index("}\n")]
    rows = re.findall(r"\{([^{}]*)\}", body)
    tab = np.array([[float.fromhex(v.strip().rstrip("f")) for v in r.split(",")] for r in rows])
    assert tab.shape == (160, 4)
    return tab.astype(np.float32).astype(np.float64)   # the device holds floats


def _small(x, a, tab):
    j = np.minimum(np.floor(10 * x).astype(int), 159)
    t = 10 * x - j
    c = tab[j]
    k = c[:, 0] + t * (c[:, 1] + t * (c[:, 2] + t * c[:, 3]))
    dk = 10 * (c[:, 1] + t * (2 * c[:, 2] + t * 3 * c[:, 3]))
    e = np.exp(-x * x)
    g = 1 + a * a * (1 - 2 * x * x)
    h = e * g + a * k
    dhdx = -2 * x * e * (g + 2 * a * a) + a * dk
    dhda = 2 * a * e * (1 - 2 * x * x) + k
    return h, dhdx, dhda


def test_small_damping_form_against_wofz():
    wofz = pytest.importorskip("scipy.special").wofz
    tab = _ktab()
    x = np.linspace(0.0, 15.9, 200001)
    for a in (0.0, 1e-5, 3e-4, 1e-3, 2e-3):
        h, _, _ = _small(x, a, tab)
        want = wofz(x + 1j * a).real
        rel = np.abs(h - want) / want
        assert rel.max() < 6e-7, (a, rel.max(), x[rel.argmax()])


def test_small_damping_derivatives():
    wofz = pytest.importorskip("scipy.special").wofz
    tab = _ktab()
    x = np.linspace(0.05, 15.85, 20001)
    a = 1e-3
    _, dhdx, dhda = _small(x, a, tab)
    ex, ea = 1e-5, 1e-7
    fx = (wofz(x + ex + 1j * a).real - wofz(x - ex + 1j * a).real) / (2 * ex)
    fa = (wofz(x + 1j * (a + ea)).real - wofz(x + 1j * (a - ea)).real) / (2 * ea)
    # relative to the scale of each derivative (they cross zero)
    assert np.abs(dhdx - fx).max() < 2e-4 * np.abs(fx).max()
    assert np.abs(dhda - fa).max() < 2e-4 * np.abs(fa).max()
