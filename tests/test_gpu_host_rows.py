"""The host-pointer entry (fsg_particle_interpolate through the Python drop-in)
deposits in row groups and copies each group's rows out while later groups
compute.  Its output must equal the device entry's bit for bit (the
fixed-point sums do not depend on the launch), for tau and column density,
in both forms.  Rows that the FP64 fallback redoes after their group was
copied (a particle with an infinite density makes its sightlines' sums
non-finite) must arrive too: the fallback adds in the order of the pair
list, which the search fills with atomics, so their finite pixels agree to
rounding (1e-12 relative) and their infinite pixels exactly."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def work():
    # the 128^3 recipe at 64^3 particles with 1024 sightlines: four row groups
    return synth.generate_torch(4, nside=64, device="cuda").to_host()


@pytest.mark.parametrize("precision,compute_tau", [("fp32", 1), ("fp32", 0), ("fp64", 1)])
def test_row_groups_match_device_entry(ctx, work, precision, compute_tau):
    import torch
    from fake_spectra_gb300 import interp as I
    from fake_spectra_gb300._spectra_priv import _Particle_Interpolate
    a = list(work.call_args(synth.LYA, compute_tau))
    assert len(work.axis) >= 256
    got = _Particle_Interpolate(*a, precision=precision)
    d = list(a)
    for k in range(11, 16):
        d[k] = torch.from_numpy(np.ascontiguousarray(a[k])).cuda()
    want = I.particle_interpolate_device(ctx, *d, precision=precision).cpu().numpy()
    assert np.array_equal(got, want)
    assert (got != 0).any(axis=1).mean() > 0.9


def test_row_groups_with_fallback_rows(ctx, work, port):
    import torch
    from fake_spectra_gb300 import interp as I
    from fake_spectra_gb300._spectra_priv import _Particle_Interpolate
    a = list(work.call_args(synth.LYA, 1))
    dens = np.array(a[13], dtype=np.float32, copy=True)
    lines = [5, 700]   # in the first and the third row group
    off, part, _ = port.near_particles(work.pos, work.hh, work.axis[lines], work.cofm[lines],
                                       work.box)
    dens[part[off[0]]] = np.inf
    dens[part[off[1]]] = np.inf
    a[13] = dens
    got = _Particle_Interpolate(*a, precision="fp32")
    d = list(a)
    for k in range(11, 16):
        d[k] = torch.from_numpy(np.ascontiguousarray(a[k])).cuda()
    want = I.particle_interpolate_device(ctx, *d, precision="fp32").cpu().numpy()
    assert np.isinf(want[lines]).any(axis=1).all()
    assert np.array_equal(np.isinf(got), np.isinf(want))
    redone = ~np.isfinite(want).all(axis=1)
    assert np.array_equal(got[~redone], want[~redone])
    fin = np.isfinite(want) & redone[:, None]
    np.testing.assert_allclose(got[fin], want[fin], rtol=1e-12, atol=0)
