"""Flux statistics on the GPU (fsg_flux.cu) against the oracle restatement and
the known answers of the reference's tests (test_statistics.py:8-73)."""
import math

import numpy as np
import pytest

from oracle import fluxstats as fs

pytestmark = pytest.mark.gpu


def _taus(seed=3, nspec=64, npix=1115):
    rng = np.random.default_rng(seed)
    # log-normal optical depths with saturated and empty pixels, as in spectra
    tau = np.exp(rng.normal(0.0, 2.0, size=(nspec, npix)))
    tau[rng.random(tau.shape) < 0.01] = 0.0
    tau[rng.random(tau.shape) < 0.01] = 1e4
    return tau


def test_known_answers_on_gpu(fsg):
    from fake_spectra_gb300 import fluxstatistics as st
    tol = 1e-4
    nn = np.arange(1, 101)
    tau = np.log(nn)
    for s in (1.0, 2.0, 0.5):
        assert abs(st.mean_flux(tau, np.mean(nn ** (-s)), tol) - s) < tol
    cbins, hist = st.flux_pdf(np.log(nn.astype(np.double)), 20)
    expected = np.array([16., 2.2, 0.6, 0.2, 0.2, 0.2, 0.2, 0., 0., 0., 0.2, 0., 0., 0., 0., 0.,
                         0., 0., 0., 0.2])
    assert cbins[0] == 1 / 40. and cbins[-1] == 1. - 1 / 40.
    assert abs(expected.sum() - hist.sum()) < 1e-3
    assert np.all(np.abs(hist[3:] - expected[3:]) < 1e-3)
    assert abs(hist[0] - expected[0]) < 1e-2
    for bb in (200, 201):
        xx = np.linspace(0, 51, bb)
        inn = np.sin(2 * math.pi * xx) + 1.5
        single = np.abs(np.fft.rfft(np.exp(-inn) - 1)) ** 2 / bb ** 2
        k, power = st.flux_power(np.vstack([inn] * 10), vmax=1., spec_res=0.01, window=True)
        power = power / 12.5569
        wind = st._window_function(k[1:], R=0.01, dv=1 / bb)
        assert np.all(np.abs(power[1:] * wind ** 2 - single[1:]) < 0.01 * single[1:])
        assert power[0] < 1e-20


@pytest.mark.parametrize("thresh", [1e30, 50.0])
def test_mean_flux_matches_oracle(fsg, thresh):
    from fake_spectra_gb300 import fluxstatistics as st
    from fake_spectra_gb300._spectra_priv import _rescale_mean_flux
    tau = _taus()
    for mfd in (0.3, 0.7, 0.95):
        want = fs.mean_flux_scale(tau, mfd, 1e-10, thresh)
        got = st.mean_flux(tau, mfd, 1e-10, thresh)
        assert abs(got - want) <= 1e-9 * want
        got2 = _rescale_mean_flux(tau.reshape(-1), mfd, tau.size, 1e-10, thresh)
        assert abs(got2 - want) <= 1e-9 * want


def test_flux_pdf_counts_exact(fsg):
    from fake_spectra_gb300 import fluxstatistics as st
    tau = _taus(5)
    tau[0, :10] = -1.0          # flux above 1: outside the bins
    tau[1, :10] = np.nan        # not counted
    for nbins in (20, 7, 1000):
        _, want_density, counts = fs.flux_pdf(tau, nbins)
        _, got = st.flux_pdf(tau, nbins)
        np.testing.assert_array_equal(got, want_density)
    clean = _taus(6)
    _, want, _ = fs.flux_pdf(clean, 20, mean_flux_desired=0.6)
    _, got = st.flux_pdf(clean, 20, mean_flux_desired=0.6)
    np.testing.assert_allclose(got, want, rtol=1e-12)


@pytest.mark.parametrize("npix", [1115, 200, 201])
def test_flux_power_matches_oracle(fsg, npix):
    from fake_spectra_gb300 import fluxstatistics as st
    tau = _taus(7, nspec=300, npix=npix)
    for mfd, window in ((None, False), (0.65, True)):
        k0, want = fs.flux_power(tau, 1234.5, 8, mfd, window)
        k1, got = st.flux_power(tau, 1234.5, 8, mfd, window)
        np.testing.assert_array_equal(k1, k0)
        np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-14 * np.abs(want).max())


def test_flux_statistics_on_device_tensors(fsg):
    import torch
    from fake_spectra_gb300 import fluxstatistics as st
    tau = _taus(9)
    t = torch.from_numpy(tau).cuda()
    assert st.mean_flux(t, 0.5, 1e-10) == st.mean_flux(tau, 0.5, 1e-10)
    np.testing.assert_array_equal(st.flux_power(t, 100.0)[1], st.flux_power(tau, 100.0)[1])
