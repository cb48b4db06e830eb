"""The oracle's flux statistics against the known answers of the reference's
own tests (fake_spectra/tests/test_statistics.py:8-73), restated."""
import math

import numpy as np

from oracle import fluxstats as fs


def test_mean_flux_known_answers():
    # test_statistics.py:8-19: tau = log n, so mean(n^-s) is hit at scale s
    tol = 1e-4
    nn = np.arange(1, 101)
    tau = np.log(nn)
    for s in (1.0, 2.0, 0.5):
        mf = np.mean(nn ** (-s))
        assert abs(fs.mean_flux_scale(tau, mf, tol) - s) < tol


def test_flux_pdf_known_answers():
    # test_statistics.py:21-36
    nn = np.arange(1, 101, dtype=np.double)
    cbins, hist, _ = fs.flux_pdf(np.log(nn), 20)
    assert cbins[0] == 0. + 1 / 40. and cbins[-1] == 1. - 1. / 40.
    expected = np.array([16., 2.2, 0.6, 0.2, 0.2, 0.2, 0.2, 0., 0., 0., 0.2, 0., 0., 0., 0., 0.,
                         0., 0., 0., 0.2])
    assert abs(expected.sum() - hist.sum()) < 1e-3
    assert np.all(np.abs(hist[3:] - expected[3:]) < 1e-3)
    assert abs(hist[0] - expected[0]) < 1e-2


def test_flux_power_known_answers():
    # test_statistics.py:55-73: a sine optical depth gives one spectral line
    for bb in (200, 201):
        xx = np.linspace(0, 51, bb)
        inn = np.sin(2 * math.pi * xx) + 1.5
        single = np.abs(np.fft.rfft(np.exp(-inn) - 1)) ** 2 / bb ** 2
        taus = np.vstack([inn] * 10)
        k, power = fs.flux_power(taus, vmax=1., spec_res=0.01, use_window=True)
        power = power / 12.5569
        wind = fs.window(k[1:], 0.01, 1 / bb)
        assert np.all(np.abs(power[1:] * wind ** 2 - single[1:]) < 0.01 * single[1:])
        assert power[0] < 1e-20
