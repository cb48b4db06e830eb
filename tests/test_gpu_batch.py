"""Batched form: several lines and both quantities in one call (one search, one
CUDA graph) give exactly what the single-line calls give."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_equals_single_calls(ctx, precision):
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config2(nside=24)
    sub = np.arange(0, w.nlos, 113)
    w.axis, w.cofm = w.axis[sub], w.cofm[sub]
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pos, vel, temp, hh = T(w.pos), T(w.vel), T(w.temp), T(w.hh)
    dens = {k: T(v) for k, v in w.dens.items()}
    lines = [(t, dens[t.species], True, t.name != "lyb") for t in w.transitions]
    for rep in range(2):    # second call reuses the instantiated graph
        outs = I.spectra_batch_device(ctx, w.nbins, w.kernel, w.box, w.velfac, w.atime,
                                      w.tautail, pos, vel, temp, hh, w.axis, w.cofm, lines,
                                      precision=precision)
        for (t, d, want_tau, want_col), (tau, col) in zip(lines, outs):
            for ct, got in ((1, tau), (0, col)):
                if got is None:
                    continue
                args = w.call_args(t, ct)
                ref = I.particle_interpolate_device(ctx, *args[:11], pos, vel, d, temp, hh,
                                                    args[16], args[17], precision=precision)
                assert torch.equal(got, ref), (t.name, ct, rep)
