"""Voronoi-mesh kernel (kernel 2) on the GPU: the cell segments along each
sightline (IndexTable::assign_cells) and the arepo deposit branches, against
the reference's outputs (tests/golden/voronoi.npz) and the oracle."""
import numpy as np
import pytest

from conftest import golden
from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


def _gpu(g, t, ct, precision="fp64", nbins=None):
    from fake_spectra_gb300._spectra_priv import _Particle_Interpolate
    return _Particle_Interpolate(ct, int(nbins or g["nbins"]), 2, float(g["box"]),
                                 float(g["velfac"]), 0.25, t.lambda_cm, t.gamma, t.fosc,
                                 t.amumass, 1e-7, g["pos"], g["vel"], g["dens"], g["temp"],
                                 g["hh"], g["axis"], g["cofm"], precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_voronoi_matches_reference_outputs(fsg, precision):
    g = golden("voronoi.npz")
    for t in (synth.LYA, synth.CIV):
        np.testing.assert_allclose(_gpu(g, t, 1, precision), g["tau_" + t.name], rtol=1e-11,
                                   atol=5e-7 * 1e-7)
        np.testing.assert_allclose(_gpu(g, t, 0, precision), g["colden_" + t.name], rtol=1e-11,
                                   atol=0)


def test_voronoi_random_against_oracle(fsg, port):
    rng = np.random.default_rng(4)
    box = 2000.0
    n = 6000
    g = dict(pos=rng.uniform(0, box, (n, 3)).astype(np.float32),
             vel=(40 * rng.standard_normal((n, 3))).astype(np.float32),
             dens=(rng.lognormal(0, 1, n) * 1e11).astype(np.float32),
             temp=(1e4 * rng.lognormal(0, 0.3, n)).astype(np.float32),
             hh=(90.0 * rng.lognormal(0, 0.2, n)).astype(np.float32),
             axis=rng.integers(1, 4, 20).astype(np.int32),
             cofm=rng.uniform(0, box, (20, 3)), box=box, velfac=synth.cosmology()[2])
    nbins = int(box * g["velfac"])
    for ct in (0, 1):
        want = port.particle_interpolate(ct, nbins, 2, box, g["velfac"], 0.25,
                                         synth.LYA.lambda_cm, synth.LYA.gamma, synth.LYA.fosc,
                                         synth.LYA.amumass, 1e-7, g["pos"], g["vel"], g["dens"],
                                         g["temp"], g["hh"], g["axis"], g["cofm"])
        got = _gpu(g, synth.LYA, ct, nbins=nbins)
        assert (want != 0).sum() > 100
        np.testing.assert_allclose(got, want, rtol=1e-11, atol=1e-14 * np.abs(want).max())
