"""The oracle's Voronoi path (kernel 2: assign_cells, index_table.cpp:152-223,
and the arepo branches of absorption.cpp) against the reference build's
outputs stored in tests/golden/voronoi.npz."""
import numpy as np

from conftest import golden
from fake_spectra_gb300 import synth


def _call(impl, g, t, ct):
    return impl.particle_interpolate(ct, int(g["nbins"]), 2, float(g["box"]), float(g["velfac"]),
                                     0.25, t.lambda_cm, t.gamma, t.fosc, t.amumass, 1e-7,
                                     g["pos"], g["vel"], g["dens"], g["temp"], g["hh"], g["axis"],
                                     g["cofm"])


def test_voronoi_oracle_matches_reference_outputs(impls):
    g = golden("voronoi.npz")
    for impl in impls:
        for t in (synth.LYA, synth.CIV):
            np.testing.assert_allclose(_call(impl, g, t, 1), g["tau_" + t.name], rtol=1e-12,
                                       atol=1e-300)
            np.testing.assert_allclose(_call(impl, g, t, 0), g["colden_" + t.name], rtol=1e-13,
                                       atol=0)


def test_voronoi_fixture_has_a_wrapping_cell(port):
    g = golden("voronoi.npz")
    box = float(g["box"])
    off, part, _ = port.near_particles(g["pos"], g["hh"], g["axis"], g["cofm"], box)
    seg = port.assign_cells(g["pos"], part[off[0]:off[1]], int(g["axis"][0]), g["cofm"][0], box)
    lo, hi = seg[0::2], seg[1::2]
    live = hi < 2 * box
    assert live.any()
    # the first cell wraps: it starts past box/2 and ends past the box
    assert ((lo > box / 2) & (hi > box) & (hi < 2 * box)).any()
    # cells tile the sightline once
    assert abs((hi[live] - lo[live]).sum() - box) < 1e-3 * box
