"""The C oracle against golden outputs of the reference itself (tests/golden/,
produced by tests/golden/make_golden.py from the unmodified reference build).
These run everywhere, including machines without the reference checkout."""
import numpy as np
import pytest

from conftest import golden
from fake_spectra_gb300 import synth

# The reference is built with -ffast-math; the oracle is not.  Observed
# differences: tau <= 3e-14, colden <= 2e-12 relative.
RTOL_TAU = 1e-12
RTOL_COLDEN = 1e-11


def close(o, r, rtol):
    d = np.abs(o - r)
    bad = d > rtol * np.abs(r) + 1e-300
    assert not bad.any(), "max rel diff %.3e" % (d / np.maximum(np.abs(r), 1e-300)).max()


def test_pairs_edges(port):
    e = golden("edges.npz")
    off, part, dr2 = port.near_particles(e["pos"], e["hh"], e["axis"], e["cofm"], float(e["box"]))
    assert np.array_equal(off, e["off"])
    assert np.array_equal(part, e["part"])
    assert np.array_equal(dr2.view(np.int64), e["dr2"].view(np.int64))


def test_pairs_config0_slice(port):
    c = golden("config0_slice.npz")
    off, part, dr2 = port.near_particles(c["pos"], c["hh"], c["axis"], c["cofm"], float(c["box"]))
    assert np.array_equal(off, c["off"]) and np.array_equal(part, c["part"])
    assert np.array_equal(dr2.view(np.int64), c["dr2"].view(np.int64))


@pytest.mark.parametrize("kernel", [0, 1, 3])
@pytest.mark.parametrize("compute_tau", [0, 1])
def test_edges_spectra(port, kernel, compute_tau):
    e = golden("edges.npz")
    t = synth.LYA
    o = port.particle_interpolate(compute_tau, int(e["nbins"]), kernel, float(e["box"]),
                                  float(e["velfac"]), 0.25, t.lambda_cm, t.gamma, t.fosc,
                                  t.amumass, 1e-7, e["pos"], e["vel"], e["dens"], e["temp"],
                                  e["hh"], e["axis"], e["cofm"])
    r = e["%s_k%d" % ("tau" if compute_tau else "colden", kernel)]
    close(o, r, RTOL_TAU if compute_tau else RTOL_COLDEN)


@pytest.mark.parametrize("tr", [synth.LYA, synth.LYB, synth.CIV], ids=lambda t: t.name)
@pytest.mark.parametrize("compute_tau", [0, 1])
def test_config0_slice_spectra(port, tr, compute_tau):
    c = golden("config0_slice.npz")
    o = port.particle_interpolate(compute_tau, int(c["nbins"]), 1, float(c["box"]),
                                  float(c["velfac"]), float(c["atime"]), tr.lambda_cm, tr.gamma,
                                  tr.fosc, tr.amumass, 1e-7, c["pos"], c["vel"], c["dens"],
                                  c["temp"], c["hh"], c["axis"], c["cofm"])
    r = c["%s_%s" % ("tau" if compute_tau else "colden", tr.name)]
    close(o, r, RTOL_TAU if compute_tau else RTOL_COLDEN)


def test_voigt_vs_reference_faddeeva(port):
    v = golden("voigt.npz")
    H = np.array([port.voigt(x, y) for x, y in zip(v["u"], v["a"])])
    rel = np.abs(H - v["H"]) / np.abs(v["H"])
    assert rel.max() < 5e-14


def test_voigt_vs_scipy(port):
    wofz = pytest.importorskip("scipy.special").wofz
    rng = np.random.default_rng(2)
    u = np.concatenate([rng.uniform(-9, 9, 400), rng.uniform(-500, 500, 100)])
    a = 10 ** rng.uniform(-7, 0.8, u.size)
    H = np.array([port.voigt(x, y) for x, y in zip(u, a)])
    ref = wofz(u + 1j * a).real
    assert (np.abs(H - ref) / ref).max() < 1e-12


def test_voigt_continued_fraction_levels(port):
    # the continued fraction's level count steps down with |z| (|z| >= 7): just
    # above each step, over the quadrant and next to the real axis
    wofz = pytest.importorskip("scipy.special").wofz
    rng = np.random.default_rng(3)
    for r in (7.0, 8.0, 10.0, 12.0, 15.0, 20.0, 30.0, 50.0, 100.0, 1e4):
        th = np.concatenate([rng.uniform(0, np.pi / 2, 200), [1e-9, 1e-4, np.pi / 2 - 1e-9]])
        rr = r * (1 + 1e-9)
        u, a = rr * np.cos(th), np.maximum(rr * np.sin(th), 1e-12)
        H = np.array([port.voigt(x, y) for x, y in zip(u, a)])
        ref = wofz(u + 1j * a).real
        assert (np.abs(H - ref) / np.abs(ref)).max() < 1e-13, r


def test_oracle_threads_deterministic(port):
    c = golden("config0_slice.npz")
    t = synth.LYA
    args = (1, int(c["nbins"]), 1, float(c["box"]), float(c["velfac"]), float(c["atime"]),
            t.lambda_cm, t.gamma, t.fosc, t.amumass, 1e-7, c["pos"], c["vel"], c["dens"],
            c["temp"], c["hh"], c["axis"], c["cofm"])
    n0 = port.get_threads()
    try:
        port.set_threads(1)
        a = port.particle_interpolate(*args)
        port.set_threads(4)
        b = port.particle_interpolate(*args)
    finally:
        port.set_threads(n0)
    assert np.array_equal(a, b)
