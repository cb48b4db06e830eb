"""Flux statistics on the GPU, with the interface of the reference module
``fake_spectra.fluxstatistics`` (fluxstatistics.py:1-110).

``mean_flux``, ``flux_pdf`` and ``flux_power`` take optical depths as a NumPy
array or a torch tensor; tensors already on the GPU (the output of
``interp.particle_interpolate_device``) are used in place, NumPy arrays are
copied to the device.  The reductions, the histogram and the batched
real-to-complex transforms run in libfsg (fsg_flux.cu, cuFFT).
"""
import ctypes
import math

import numpy as np

from . import _lib

_CTX = None


def _context():
    global _CTX
    if _CTX is None:
        import torch
        _CTX = _lib.Context(torch.cuda.current_device())
    return _CTX


def _device_tau(tau):
    import torch
    if isinstance(tau, torch.Tensor):
        t = tau.detach()
        if not t.is_cuda:
            t = t.cuda()
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(tau, dtype=np.float64))).cuda()
    return t.to(torch.float64).contiguous()


def _bind(ctx):
    import torch
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)


def obs_mean_tau(redshift):
    """Effective optical depth 0.0023 (1+z)^3.65 (0711.1862; fluxstatistics.py:20-23)."""
    return 0.0023 * (1.0 + redshift) ** 3.65


def mean_flux(tau, mean_flux_desired, tol=1e-5, thresh=1e30):
    """Scale factor s of tau with mean(exp(-s tau)) = mean_flux_desired
    (fluxstatistics.py:25-40): Newton-Raphson on the GPU."""
    t = _device_tau(tau)
    n = int(t.numel())
    if n == 0:
        return 0
    ctx = _context()
    _bind(ctx)
    out = ctypes.c_double(0.0)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_mean_flux_scale_device(ctx.handle, ctypes.c_void_p(t.data_ptr()), n,
                                                float(mean_flux_desired), float(tol),
                                                float(thresh), ctypes.byref(out), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out.value


def _mean_of_flux(t, scale):
    ctx = _context()
    _bind(ctx)
    out = ctypes.c_double(0.0)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_mean_flux_device(ctx.handle, ctypes.c_void_p(t.data_ptr()),
                                          int(t.numel()), float(scale), ctypes.byref(out), eb,
                                          512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out.value


def flux_pdf(tau, nbins=20, mean_flux_desired=None):
    """Normalised histogram of the flux exp(-s tau) on nbins equal bins of
    [0, 1] (fluxstatistics.py:42-51): (bin centres, density)."""
    t = _device_tau(tau)
    scale = 1.
    if mean_flux_desired is not None:
        scale = mean_flux(t, mean_flux_desired)
    bins = np.arange(nbins + 1) / (1. * nbins)
    counts = np.zeros(nbins, dtype=np.int64)
    ctx = _context()
    _bind(ctx)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_flux_histogram_device(
        ctx.handle, ctypes.c_void_p(t.data_ptr()), int(t.numel()), float(scale),
        bins.ctypes.data_as(ctypes.c_void_p), int(nbins), counts.ctypes.data_as(ctypes.c_void_p),
        eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    # density as np.histogram(density=True): counts / width / total
    n = counts.astype(np.float64)
    fpdf = n / np.diff(bins) / n.sum()
    cbins = (bins[1:] + bins[:-1]) / 2.
    return cbins, fpdf


def _window_function(k, *, R, dv):
    """Spectrograph response: a Gaussian of FWHM R times the pixel sinc
    (fluxstatistics.py:63-72)."""
    sigma = R / (2 * np.sqrt(2 * np.log(2)))
    return np.exp(-0.5 * (k * sigma) ** 2) * np.sinc(k * dv / 2 / math.pi)


def _flux_power_bins(vmax, npix):
    """k of each rfft mode in s/km for a sightline of length vmax km/s
    (fluxstatistics.py:197-216)."""
    return np.fft.rfftfreq(npix) * (2.0 * math.pi * npix / vmax)


def flux_power(tau, vmax, spec_res=8, mean_flux_desired=None, window=False):
    """Mean 1-D power spectrum of d_F = exp(-s tau) / <F> - 1 along the
    sightlines (fluxstatistics.py:74-110): (k in s/km, power in km/s)."""
    t = _device_tau(tau)
    if t.dim() != 2:
        raise ValueError("tau must have shape (NumLos, npix)")
    nspec, npix = int(t.shape[0]), int(t.shape[1])
    scale = 1.
    if mean_flux_desired is not None:
        scale = mean_flux(t, mean_flux_desired)
    else:
        mean_flux_desired = _mean_of_flux(t, 1.0)
    power = np.zeros(npix // 2 + 1, dtype=np.float64)
    ctx = _context()
    _bind(ctx)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_flux_power_device(ctx.handle, ctypes.c_void_p(t.data_ptr()), nspec, npix,
                                           float(scale), float(mean_flux_desired), float(vmax),
                                           power.ctypes.data_as(ctypes.c_void_p), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    kf = _flux_power_bins(vmax, npix)
    if window and spec_res > 0:
        power /= _window_function(kf, R=spec_res, dv=vmax / npix) ** 2
    return kf, power
