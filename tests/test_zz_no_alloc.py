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


@pytest.mark.parametrize("nbins", [0, 3000])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("compute_tau", [1, 0])
def test_noalloc_matches_allocating_entry_point(ctx, precision, compute_tau, nbins):
    """nbins 0: the workload's 111 pixels; 3000 pixels (0.37 km/s) puts far damping
    wings more than 128 pixels from their line centres, so the FP32 form also
    runs its far-field tile path, which shares the tile weight table."""
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    if nbins:
        w.nbins = nbins
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
    """Too many sightlines and too many pixels are rejected before any work."""
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


def test_noalloc_rejects_too_many_pairs_then_recovers(ctx):
    """8192 sightlines through the 32^3 workload make about 11 million pairs,
    beyond the array's ~5.4 million: the call stops after the pair count with
    a ValueError, and the next call (which reuses the same array) is still
    right."""
    import torch
    from fake_spectra_gb300 import interp as I
    w = synth.config0()
    args = list(w.call_args(synth.LYA, 1))
    dev = _dev(args)
    rng = np.random.default_rng(21)
    many = 8192
    axis = np.ones(many, np.int32)
    cofm = rng.uniform(0.0, w.box, size=(many, 3))
    with pytest.raises(ValueError, match="no-allocation limit"):
        I.particle_interpolate_noalloc(*args[:11], *dev, axis, cofm,
                                       out=torch.empty((many, w.nbins), dtype=torch.float64,
                                                       device="cuda"), precision="fp32")
    want = I.particle_interpolate_device(ctx, *args[:11], *dev, args[16], args[17],
                                         precision="fp32").cpu().numpy()
    got = I.particle_interpolate_noalloc(*args[:11], *dev, args[16], args[17],
                                         precision="fp32").cpu().numpy()
    assert np.all(np.abs(got - want) <= RTOL * np.abs(want) + ATOL_TAU)


def test_noalloc_rejects_host_output(fsg):
    """A host pointer where device memory is required is refused before any
    work is queued (checked through the C ABI with cudaPointerGetAttributes)."""
    import ctypes
    import torch
    from fake_spectra_gb300 import _lib
    w = synth.config0()
    args = w.call_args(synth.LYA, 1)
    dev = _dev(args)
    host_out = np.zeros((w.nlos, w.nbins))
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    eb = _lib.errbuf()
    rc = _lib.load().fsg_particle_interpolate_noalloc(
        1, w.nbins, w.kernel, *[float(x) for x in args[3:11]], *[p(t) for t in dev], w.npart,
        w.axis.ctypes.data_as(ctypes.c_void_p), w.cofm.ctypes.data_as(ctypes.c_void_p), w.nlos,
        host_out.ctypes.data_as(ctypes.c_void_p), 1,
        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), eb, 512)
    assert rc == _lib.FSG_ERR_VALUE
    assert b"not device memory" in eb.value
