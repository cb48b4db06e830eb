"""CPU restatement (NumPy) of the reference's flux statistics: test
infrastructure only, the checker of fake_spectra_gb300.fluxstatistics.

* mean_flux_scale: get_mean_flux_scale, fake_spectra/py_module.cpp:235-260
  (Newton-Raphson; the same update, clamp and stopping rule).
* flux_pdf: fake_spectra/fluxstatistics.py:42-51 (np.histogram, density).
* flux_power: fake_spectra/fluxstatistics.py:53-110 (per-sightline rfft power,
  averaged, optional window division), bins as fluxstatistics.py:197-216.
"""
import math

import numpy as np


def mean_flux_scale(tau, mean_flux_desired, tol=1e-5, thresh=1e30):
    tau = np.asarray(tau, dtype=np.float64).reshape(-1)
    if tau.size == 0:
        return 0
    used = tau[~(tau > thresh)]
    newscale = 1.0
    while True:
        scale = newscale
        e = np.exp(-scale * used)
        newscale = scale + (e.sum() - mean_flux_desired * used.size) / (e * used).sum()
        if newscale <= 0:
            newscale = 1e-10
        if not abs(newscale - scale) > tol * newscale:
            return newscale


def flux_pdf(tau, nbins=20, mean_flux_desired=None):
    tau = np.asarray(tau, dtype=np.float64)
    scale = 1.0 if mean_flux_desired is None else mean_flux_scale(tau, mean_flux_desired)
    edges = np.arange(nbins + 1) / (1. * nbins)
    counts, _ = np.histogram(np.exp(-scale * tau), bins=edges)
    density = counts / np.diff(edges) / counts.sum()
    return (edges[1:] + edges[:-1]) / 2., density, counts


def power_bins(vmax, npix):
    return np.fft.rfftfreq(npix) * (2.0 * math.pi * npix / vmax)


def window(k, R, dv):
    sigma = R / (2 * np.sqrt(2 * np.log(2)))
    return np.exp(-0.5 * (k * sigma) ** 2) * np.sinc(k * dv / 2 / math.pi)


def flux_power(tau, vmax, spec_res=8, mean_flux_desired=None, use_window=False):
    tau = np.asarray(tau, dtype=np.float64)
    nspec, npix = tau.shape
    if mean_flux_desired is not None:
        scale = mean_flux_scale(tau, mean_flux_desired)
    else:
        scale = 1.0
        mean_flux_desired = np.mean(np.exp(-tau))
    dflux = np.exp(-scale * tau) / mean_flux_desired - 1.
    power = (np.abs(np.fft.rfft(dflux, axis=1)) ** 2 / npix ** 2).sum(axis=0) * vmax / nspec
    k = power_bins(vmax, npix)
    if use_window and spec_res > 0:
        power = power / window(k, spec_res, vmax / npix) ** 2
    return k, power
