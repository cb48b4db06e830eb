"""`_near_lines` (py_module.cpp:25-99): the particles within their smoothing
length of any sightline, against the reference's pair lists (golden fixtures
made by the reference build) and the oracle."""
import numpy as np
import pytest

from conftest import golden
from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


def _expected(off, part):
    return np.unique(np.asarray(part[:off[-1]], dtype=np.int64)).astype(np.int32)


@pytest.mark.parametrize("fixture", ["index_testcpp.npz", "edges.npz", "config0_slice.npz"])
def test_near_lines_golden(fsg, fixture):
    from fake_spectra_gb300._spectra_priv import _near_lines
    g = golden(fixture)
    got = _near_lines(float(g["box"]), g["pos"].astype(np.float32), g["hh"].astype(np.float32),
                      g["axis"].astype(np.int32), g["cofm"].astype(np.float64))
    assert got.dtype == np.int32
    np.testing.assert_array_equal(got, _expected(g["off"], g["part"]))


def test_near_lines_config0_and_device(fsg, ctx, port):
    import torch
    from fake_spectra_gb300 import interp
    from fake_spectra_gb300._spectra_priv import _near_lines
    w = synth.config0()
    off, part, _ = port.near_particles(w.pos, w.hh, w.axis, w.cofm, w.box)
    want = _expected(off, part)
    got = _near_lines(w.box, w.pos, w.hh, w.axis, w.cofm)
    np.testing.assert_array_equal(got, want)
    dev = interp.near_lines_device(ctx, w.box, torch.from_numpy(w.pos).cuda(),
                                   torch.from_numpy(w.hh).cuda(), w.axis, w.cofm)
    np.testing.assert_array_equal(dev.cpu().numpy(), want)


def test_near_lines_degenerate_smoothing(fsg, port):
    """NaN, +-inf, zero and negative smoothing lengths and out-of-box positions
    resolve as the reference's predicate does (per-particle oracle)."""
    from fake_spectra_gb300._spectra_priv import _near_lines
    rng = np.random.default_rng(7)
    box = 1000.0
    n = 4000
    pos = rng.uniform(0, box, size=(n, 3)).astype(np.float32)
    hh = rng.uniform(1, 60, size=n).astype(np.float32)
    hh[:50] = np.nan
    hh[50:100] = np.inf
    hh[100:150] = -np.inf
    hh[150:200] = 0.0
    hh[200:250] = -5.0
    pos[250:300] += np.float32(box)          # outside the box
    pos[300:350] -= np.float32(box)
    pos[350:360, 0] = np.nan
    axis = rng.integers(1, 4, size=40).astype(np.int32)
    cofm = rng.uniform(0, box, size=(40, 3))
    got = _near_lines(box, pos, hh, axis, cofm)
    want = [i for i in range(n) if port.near_lines(cofm, axis, box, pos[i], hh[i])]
    np.testing.assert_array_equal(got, np.asarray(want, dtype=np.int32))


def test_near_lines_empty(fsg):
    from fake_spectra_gb300._spectra_priv import _near_lines
    pos = np.zeros((0, 3), np.float32)
    assert _near_lines(10.0, pos, np.zeros(0, np.float32), np.array([1], np.int32),
                       np.zeros((1, 3))).shape == (0,)
    pos = np.ones((5, 3), np.float32)
    got = _near_lines(10.0, pos, np.ones(5, np.float32), np.zeros(0, np.int32),
                      np.zeros((0, 3)))
    assert got.shape == (0,) and got.dtype == np.int32
