"""Synthetic workload generators: sizes and conventions of the benchmark configs."""
import numpy as np

from fake_spectra_gb300 import synth


def test_cosmology():
    atime, rscale, velfac = synth.cosmology()
    assert atime == 0.25
    assert abs(velfac - 0.111524) < 1e-5


def test_config0():
    w = synth.config0()
    assert w.npart == 32 ** 3 and w.nlos == 64 and w.nbins == 111
    assert w.pos.dtype == np.float32 and w.cofm.dtype == np.float64 and w.axis.dtype == np.int32
    assert (w.axis == 1).all()
    assert (w.pos >= 0).all() and (w.pos < w.box).all()
    assert abs(float(np.mean(w.hh.astype(np.float64) ** -3 * (2 * w.box / 32) ** 3)) - 1.0) < 0.1
    w2 = synth.config0()
    assert np.array_equal(w.pos, w2.pos) and np.array_equal(w.dens["HI"], w2.dens["HI"])


def test_small_variants():
    w = synth.config1(nside=32)
    assert w.nbins == 6691 and w.nlos == 3600 and (w.axis == 3).all()
    assert np.allclose(np.unique(w.cofm[:, 0]), np.arange(60) * 1000.0)
    w = synth.config2(nside=16)
    assert set(w.dens) == {"HI", "CIV"} and len(w.transitions) == 3
    w = synth.config3(nside=32, nlos=300)
    assert w.nbins == 11152
    assert list(np.bincount(w.axis)[1:]) == [100, 100, 100]
    w = synth.config4(nside=16, nlos=64)
    assert w.nbins == 1115


def test_config3_axis_split():
    counts = [32768 // 3 + (1 if i < 32768 - 3 * (32768 // 3) else 0) for i in range(3)]
    assert counts == [10923, 10923, 10922]
