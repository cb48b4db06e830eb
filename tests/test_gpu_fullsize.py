"""The full 256^3 workload (16.8M particles, 3600 sightlines x 6691 pixels):
properties that do not depend on size, checked at full size - the FP32 form
against the FP64 form on a sightline subset, bitwise reproducibility, exact
linearity of the column density in the density, and the pair count against
the search-only entry point."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w256():
    import torch
    w = synth.generate_torch(1, device="cuda")
    torch.cuda.synchronize()
    return w


def test_fp32_against_fp64_subset(ctx, w256):
    from fake_spectra_gb300 import interp as I
    w = w256
    lines = np.arange(0, w.nlos, 57)
    for ct in (1, 0):
        a = list(w.call_args(synth.LYA, ct))
        full32 = I.particle_interpolate_device(ctx, *a, precision="fp32").cpu().numpy()[lines]
        a[16], a[17] = w.axis[lines], w.cofm[lines]
        sub64 = I.particle_interpolate_device(ctx, *a, precision="fp64").cpu().numpy()
        if ct:
            assert np.abs(np.exp(-full32) - np.exp(-sub64)).max() <= 1e-4
            big = sub64 >= 1e-3
            assert (np.abs(full32 - sub64)[big] / sub64[big]).max() <= 1e-4
        else:
            nz = sub64 != 0
            assert (np.abs(full32 - sub64)[nz] / np.abs(sub64[nz])).max() <= 1e-5


def test_fp32_reproducible_and_colden_linear(ctx, w256):
    import torch
    from fake_spectra_gb300 import interp as I
    w = w256
    a = list(w.call_args(synth.LYA, 1))
    t1 = I.particle_interpolate_device(ctx, *a, precision="fp32")
    t2 = I.particle_interpolate_device(ctx, *a, precision="fp32")
    assert torch.equal(t1, t2)
    c = list(w.call_args(synth.LYA, 0))
    c1 = I.particle_interpolate_device(ctx, *c, precision="fp32")
    c[13] = c[13] * 2
    c2 = I.particle_interpolate_device(ctx, *c, precision="fp32")
    assert torch.equal(c2, 2 * c1)


def test_pair_count_consistent(ctx, w256):
    from fake_spectra_gb300 import interp as I
    w = w256
    n = I.build_pairs(ctx, w.box, w.pos, w.hh, w.axis, w.cofm)
    I.particle_interpolate_device(ctx, *w.call_args(synth.LYA, 1), precision="fp32")
    assert ctx.stats()["npairs"] == n > 1e6


def test_host_api_large_output(ctx, w256):
    """The host-pointer entry point with a 193 MB output (its fresh NumPy array
    pre-faulted by host threads during the GPU work) equals the device entry
    point."""
    import torch
    from fake_spectra_gb300 import interp as I
    from fake_spectra_gb300._spectra_priv import _Particle_Interpolate
    w = w256
    a = list(w.call_args(synth.LYA, 1))
    dev = I.particle_interpolate_device(ctx, *a, precision="fp32").cpu().numpy()
    h = [x.cpu().numpy() for x in (w.pos, w.vel, w.dens["HI"], w.temp, w.hh)]
    host = _Particle_Interpolate(*a[:11], *h, w.axis, w.cofm, precision="fp32")
    assert host.nbytes >= 64 << 20
    np.testing.assert_array_equal(host, dev)
