"""The entry point that allocates no device memory, checked against the
allocating entry point on the same inputs.

It exists for callers that cannot call cudaMalloc (their host application's
allocator owns the GPU memory, or the call sits in a loop that must not
synchronise the device for an allocation).  This file is collected last so
that a run stopping at its first failure has already run every other test;
it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu

RTOL = 1e-11       # the tolerance of the FP64 parity tests
ATOL_TAU = 5e-7


def _dev(args):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in args[11:16]]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("compute_tau", [1, 0])
def test_noalloc_matches_allocating_entry_point(ctx, precision, compute_tau):
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    args = w.call_args(synth.LYA, compute_tau)
    dev = _dev(args)
    want = I.particle_interpolate_device(ctx, *args[:11], *dev, args[16], args[17],
                                         precision=precision).cpu().numpy()
    out = torch.empty((w.nlos, w.nbins), dtype=torch.float64, device="cuda")
    for _ in range(2):   # two calls in a row: the shared scratch is reused
        out.fill_(-1.0)
        got = I.particle_interpolate_noalloc(*args[:11], *dev, args[16], args[17], out=out,
                                             precision=precision).cpu().numpy()
        atol = ATOL_TAU if compute_tau else 0.0
        assert got.shape == want.shape
        assert np.all(np.abs(got - want) <= RTOL * np.abs(want) + atol)


def test_noalloc_rejects_sizes_beyond_its_limits(fsg):
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    args = list(w.call_args(synth.LYA, 1))
    dev = _dev(args)
    many = 8193
    axis = np.ones(many, np.int32)
    cofm = np.zeros((many, 3))
    with pytest.raises(ValueError, match="no-allocation limit"):
        I.particle_interpolate_noalloc(*args[:11], *dev, axis, cofm,
                                       out=torch.empty((many, w.nbins), dtype=torch.float64,
                                                       device="cuda"))
    args[1] = 1 << 20
    with pytest.raises(ValueError, match="no-allocation limit"):
        I.particle_interpolate_noalloc(*args[:11], *dev, args[16], args[17],
                                       out=torch.empty((w.nlos, 1), dtype=torch.float64,
                                                       device="cuda"))
