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


@pytest.mark.parametrize("npix,nspec", [
    (1115, 300), (200, 300), (201, 300), (11152, 37), (6691, 20), (1, 5), (2, 4), (3, 7),
    (97, 33), (4096, 16), (2 * 3 * 5 * 7 * 11 * 13, 9), (61 * 59, 6), (2 * 67, 11)])
def test_flux_power_matches_oracle(fsg, npix, nspec):
    """Own transforms against numpy's rfft: direct passes (radices 16/8/4/2
    and odd radices up to 63), Bluestein for lengths with a larger prime
    factor (1115 = 5 x 223, 6691 prime, 97, 134 = 2 x 67), odd and even
    sightline counts (an unpaired last sightline)."""
    from fake_spectra_gb300 import fluxstatistics as st
    tau = _taus(7, nspec=nspec, npix=npix)
    vmax = 1.1 * npix + 10.0   # keeps the window function above underflow at every k
    for mfd, window in ((None, False), (0.65, True)):
        k0, want = fs.flux_power(tau, vmax, 8, mfd, window)
        k1, got = st.flux_power(tau, vmax, 8, mfd, window)
        assert np.isfinite(want).all()
        np.testing.assert_array_equal(k1, k0)
        np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-14 * np.abs(want).max())


def test_flux_statistics_on_device_tensors(fsg):
    import torch
    from fake_spectra_gb300 import fluxstatistics as st
    tau = _taus(9)
    t = torch.from_numpy(tau).cuda()
    assert st.mean_flux(t, 0.5, 1e-10) == st.mean_flux(tau, 0.5, 1e-10)
    np.testing.assert_array_equal(st.flux_power(t, 100.0)[1], st.flux_power(tau, 100.0)[1])


def _hist_device(tau, scale, edges):
    """fsg_flux_histogram_device on a device copy of tau with the given edges."""
    import ctypes
    import torch
    from fake_spectra_gb300 import _lib
    from fake_spectra_gb300 import fluxstatistics as st
    t = torch.as_tensor(np.ascontiguousarray(tau, dtype=np.float64).reshape(-1), device="cuda")
    edges = np.ascontiguousarray(edges, dtype=np.float64)
    counts = np.zeros(len(edges) - 1, dtype=np.int64)
    ctx = st._context()
    st._bind(ctx)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_flux_histogram_device(
        ctx.handle, ctypes.c_void_p(t.data_ptr()), int(t.numel()), float(scale),
        edges.ctypes.data_as(ctypes.c_void_p), len(edges) - 1,
        counts.ctypes.data_as(ctypes.c_void_p), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return counts


def _edge_taus(edges, scale, n_random, seed):
    """Optical depths whose flux sits on, or a few ulps either side of, every
    edge, plus the special values and a log-normal bulk."""
    rng = np.random.default_rng(seed)
    with np.errstate(divide="ignore", invalid="ignore"):
        at = -np.log(np.asarray(edges, dtype=np.float64)) / scale
    at = at[np.isfinite(at)]
    near = [at]
    for k in (1, 2, 3, 8, 64):
        near += [at + k * np.spacing(at), at - k * np.spacing(at)]
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-300, -1e-300, 5e-324, 1e4, 746.0,
                        745.0, 700.0, 88.0, 103.0, -1e-17, 1e-17, 1e300])
    bulk = np.exp(rng.normal(0.0, 2.5, size=n_random))
    bulk[rng.random(n_random) < 0.02] = 1e4
    tau = np.concatenate(near + [special, bulk])
    return tau[rng.permutation(len(tau))]


@pytest.mark.parametrize("nb,scale,kind", [
    (20, 1.0, "unit"), (1, 1.0, "unit"), (2, 0.37, "unit"), (256, 1.0, "unit"),
    (257, 1.0, "unit"), (8192, 1.9, "unit"), (40, 0.8, "sqrt"), (33, 1.0, "short"),
    (17, 1.0, "wide"), (5, 0.0, "unit")])
def test_flux_histogram_edges_exact(fsg, nb, scale, kind):
    """Counts equal np.histogram of the device's FP64 flux exp(-scale tau)
    bin for bin, with the flux on and next to every edge, F = 1 at the closed
    top edge, underflow to 0, NaN and +-inf, on both the per-warp (nb <= 256)
    and the per-block histograms, over enough pixels that every warp takes
    many grid-stride trips through its recheck queue.  Against numpy's own
    exponential on the host the counts differ only by pixels whose flux lies
    within two ulps of an edge: the two exponentials are not both correctly
    rounded, so such a pixel can fall on either side."""
    import torch
    u = np.arange(nb + 1) / (1. * nb)
    edges = {"unit": u, "sqrt": np.sqrt(u), "short": 0.05 + 0.85 * u,
             "wide": -0.25 + 1.5 * u}[kind]
    tau = _edge_taus(edges, scale if scale > 0 else 1.0, 3_000_000, nb)
    got = _hist_device(tau, scale, edges)
    f_dev = torch.exp((-scale) * torch.as_tensor(tau, device="cuda")).cpu().numpy()
    want_dev, _ = np.histogram(f_dev, bins=edges)
    np.testing.assert_array_equal(got, want_dev)
    with np.errstate(over="ignore", invalid="ignore"):
        f_host = np.exp(-scale * tau)
    want, _ = np.histogram(f_host, bins=edges)
    ok = np.isfinite(f_host)
    near = np.array([np.count_nonzero(np.abs(f_host[ok] - e) <= 2 * np.spacing(abs(e)))
                     for e in edges])
    assert (np.abs(got - want) <= near[:-1] + near[1:]).all()


def test_flux_histogram_bin_limit(fsg):
    with pytest.raises(ValueError, match="nbins"):
        _hist_device(np.zeros(10), 1.0, np.arange(8194) / 8193.)


def test_flux_exponential_accuracy(fsg):
    """The table-driven FP64 exponential of the mean-flux and power passes
    against CUDA's exp and numpy's: within one ulp on the arguments the passes
    see (-scale tau, from huge to zero) and across the whole double range
    within two ulps of each (each is itself within about one ulp of the true
    value), exact at the special values, subnormal results, overflow."""
    import ctypes
    import torch
    from fake_spectra_gb300 import _lib
    from fake_spectra_gb300 import fluxstatistics as st
    rng = np.random.default_rng(31)
    y = np.concatenate([
        -np.exp(rng.uniform(-40, 7, 2_000_000)),          # -scale tau, tau lognormal-like
        rng.uniform(-745.2, 709.8, 2_000_000),            # the whole finite range
        rng.uniform(-1e-3, 1e-3, 200_000), np.linspace(-709, -707, 20001),
        np.linspace(707, 709.78, 20001), np.linspace(-746, -744, 20001),
        [0.0, -0.0, 1.0, -1.0, np.log(2.0), 709.78, 709.79, -745.13321910194122, -745.14,
         -800.0, 1e300, -1e300, np.inf, -np.inf, np.nan, 5e-324, -5e-324]])
    yd = torch.as_tensor(y, device="cuda")
    out = torch.empty_like(yd)
    ctx = st._context()
    st._bind(ctx)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_flux_exp_device(ctx.handle, ctypes.c_void_p(yd.data_ptr()), len(y),
                                         ctypes.c_void_p(out.data_ptr()), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    got = out.cpu().numpy()
    for name, want in (("cuda", torch.exp(yd).cpu().numpy()), ("numpy", np.exp(y))):
        same_class = (np.isnan(got) == np.isnan(want)) & (np.isinf(got) == np.isinf(want))
        assert same_class.all(), name
        fin = np.isfinite(want) & (want > 0)
        ulps = np.abs(got[fin].view(np.int64) - want[fin].view(np.int64))
        print("\nflux exp vs %s exp: %.4f%% equal, %.4f%% 1 ulp, max %d ulp" % (
            name, 100 * np.mean(ulps == 0), 100 * np.mean(ulps == 1), ulps.max()))
        assert ulps.max() <= 2, (name, int(ulps.max()), y[fin][np.argmax(ulps)])
        zero = np.isfinite(want) & (want == 0)
        assert (got[zero] <= 5e-324).all(), name
    assert got[np.isinf(y) & (y > 0)][0] == np.inf and got[np.isinf(y) & (y < 0)][0] == 0.0
    assert got[y == 0.0].tolist() == [1.0, 1.0]
