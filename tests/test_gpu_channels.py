"""Weighted column densities in one pass (fsg_colden_channels_device): every
channel equals the single-channel compute_tau=0 interpolation bit for bit, in
both forms, with the accumulators in shared memory and in global memory, and
with a channel whose sightlines go to the non-finite fallback."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


def _weights(w):
    # the weights of Spectra.get_velocity / get_temp / get_dens_weighted_density
    rng = np.random.default_rng(11)
    d = w.dens["HI"]
    return [d, d * w.vel[:, 0], d * w.vel[:, 1], d * w.vel[:, 2], d * w.temp,
            d * rng.lognormal(0, 1, size=d.shape).astype(np.float32)]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("nbins", [111, 3000])
def test_channels_equal_single_calls(ctx, precision, nbins):
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    pos, vel, temp, hh = T(w.pos), T(w.vel), T(w.temp), T(w.hh)
    dens = [T(x) for x in _weights(w)]
    if nbins == 3000:
        dens = dens + dens[:2]    # 8 channels: accumulators do not fit in shared memory
    outs = I.colden_channels_device(ctx, nbins, w.kernel, w.box, w.velfac, pos, hh, w.axis,
                                    w.cofm, dens, precision=precision)
    assert len(outs) == len(dens)
    for c, d in enumerate(dens):
        args = list(w.call_args(synth.LYA, 0))
        args[1] = nbins
        ref = I.particle_interpolate_device(ctx, *args[:11], pos, vel, d, temp, hh, w.axis,
                                            w.cofm, precision=precision)
        assert torch.equal(outs[c], ref), c


def test_channels_nonfinite_fallback(ctx, port):
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    pos, vel, temp, hh = T(w.pos), T(w.vel), T(w.temp), T(w.hh)
    d0 = w.dens["HI"].copy()
    d1 = d0.copy()
    off, part, _ = port.near_particles(w.pos, w.hh, w.axis, w.cofm, w.box)
    d1[part[off[3]]] = np.inf    # one particle of sightline 3
    outs = I.colden_channels_device(ctx, w.nbins, w.kernel, w.box, w.velfac, pos, hh, w.axis,
                                    w.cofm, [T(d0), T(d1)], precision="fp32")
    for c, d in enumerate((d0, d1)):
        args = w.call_args(synth.LYA, 0)
        ref = I.particle_interpolate_device(ctx, *args[:11], pos, vel, T(d), temp, hh, w.axis,
                                            w.cofm, precision="fp32")
        a, b = outs[c].cpu().numpy(), ref.cpu().numpy()
        assert np.array_equal(np.isinf(a), np.isinf(b))
        fin = np.isfinite(b)
        np.testing.assert_allclose(a[fin], b[fin], rtol=1e-12, atol=0)
    assert np.isinf(outs[1][3].cpu().numpy()).any()
    assert torch.isfinite(outs[0]).all()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_signed_weights_match_oracle(ctx, port, precision):
    """dens x v_x is negative for about half the particles (the velocity weight of
    Spectra.get_velocity, spectra.py:945-990).  Both the single call and the
    channel kernel are compared with the oracle's column density
    (absorption.cpp:167-210) of the same signed weights.  The error is measured
    against the column density of |weights|, since a signed pixel sum may cancel
    to near zero: 1e-11 of it in the FP64 form, 1e-5 in the FP32 form."""
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    sw = (w.dens["HI"] * w.vel[:, 0]).astype(np.float32)
    assert (sw < 0).mean() > 0.4
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    pos, vel, temp, hh = T(w.pos), T(w.vel), T(w.temp), T(w.hh)
    args = list(w.call_args(synth.LYA, 0))
    args[13] = sw
    want = port.particle_interpolate(*args)
    args[13] = np.abs(sw)
    mag = port.particle_interpolate(*args)
    tol = (1e-11 if precision == "fp64" else 1e-5) * mag
    single = I.particle_interpolate_device(ctx, *args[:11], pos, vel, T(sw), temp, hh, w.axis,
                                           w.cofm, precision=precision).cpu().numpy()
    chans = I.colden_channels_device(ctx, w.nbins, w.kernel, w.box, w.velfac, pos, hh, w.axis,
                                     w.cofm, [T(w.dens["HI"]), T(sw)], precision=precision)
    for got in (single, chans[1].cpu().numpy()):
        assert (want < 0).any() and (want > 0).any()
        err = np.abs(got - want)
        assert (err <= tol).all(), (precision, float((err / np.maximum(mag, 1e-300)).max()))
