"""Known-answer tests of the reference's own unit tests (fake_spectra/test.cpp),
restated as data and run against the CPU oracle (and the reference build where
it exists).  These pin the oracle that the GPU parity tests trust."""
import math

import numpy as np
import pytest

from conftest import golden


def near(x, y, rel=1e-5):
    # FLOATS_NEAR_TO (test.cpp:29-31) / FLOATS_APPROX_NEAR_TO (rel=1e-2, test.cpp:33-35)
    assert math.isfinite(x) and math.isfinite(y)
    assert abs(x - y) <= max(abs(x), abs(y)) * rel, "%r is not close to %r" % (x, y)


def test_sph_cubic_kernel(impls):
    # test.cpp:37-46
    norm = 32. / 4 / math.pi
    for o in impls:
        near(o.sph_cubic_kernel(1) + 1, 1)
        near(o.sph_cubic_kernel(0), norm)
        near(o.sph_cubic_kernel(0.5), 0.25 * norm)
        near(o.sph_cubic_kernel(0.25), 0.71875 * norm)
        near(o.sph_cubic_kernel(0.75), 0.03125 * norm)


def test_sph_cubic_kern_frac(impls):
    # test.cpp:48-79 (integrals evaluated with Mathematica)
    corr = 3 / (4 * math.pi)
    for o in impls:
        f = o.sph_cubic_kern_frac
        near(f(-1, 1, 1, 0, 1), 3 * 2 / math.pi)
        near(f(-3, 10, 1, 0, 1), 3 * 2 / math.pi)
        near(f(-0.15, -0.1, 1, 0, 1), corr * 0.489167, 1e-2)
        near(f(0.05, 0.1, 1, 0.4, 0.774597), corr * 0.051004, 1e-2)
        near(f(0.15, 0.16, 1, 0.8, 0.447214), corr * 0.000167423, 1e-2)
        near(f(-0.05, 0.1, 1, 0.9, 0.316228), corr * 0.00040101, 1e-2)
        near(f(0.3, 1, 1, 0.3, 0.83666), corr * 0.177801, 1e-2)
        assert f(1.5, 2, 1, 0, 1) == 0


VELFAC_TEST = 414.50523718485636 / 1e3 * 0.2 / 0.71
LYA_TEST = (1215.6701e-10, 6.265e8, 0.416400, 1.00794)


def test_compute_colden(impls):
    # test.cpp:82-151
    for o in impls:
        line = LYA_TEST + (VELFAC_TEST, 10000, 1, 1, 1e-5)
        colden = np.zeros(2000)
        nonzero = set()
        o.add_colden_particle(line, colden, 0, 1, 5002.5, 1)
        total = 8 * 3. / (4 * math.pi)
        assert colden[999] == 0
        near(colden[1000], total)
        assert colden[1001] == 0
        nonzero.add(1000)
        total /= 4
        o.add_colden_particle(line, colden, 0, 1 / 8., 1002.5, 2)
        assert colden[199] == 0
        near(colden[200], total)
        assert colden[201] == 0
        nonzero.add(200)
        o.add_colden_particle(line, colden, 0, 10 / 8., 1012.5, 2)
        assert colden[201] == 0
        near(colden[202], 10 * total)
        assert colden[203] == 0
        nonzero.add(202)
        o.add_colden_particle(line, colden, 0, 1 / 8., 1030, 2)
        assert colden[204] == 0
        near(colden[205], total / 2.)
        near(colden[206], total / 2.)
        assert colden[207] == 0
        nonzero |= {205, 206}
        o.add_colden_particle(line, colden, 0, 1 / 8., 10000, 2)
        assert colden[1998] == 0
        near(colden[1999], total / 2.)
        near(colden[0], total / 2.)
        assert colden[1] == 0
        nonzero |= {1999, 0}
        o.add_colden_particle(line, colden, 0.7, 1, 4852.5, 1)
        near(colden[969] + 1, 1)
        near(colden[970], 0.0451531 * 3 / (4 * math.pi), 1e-2)
        assert colden[971] == 0
        nonzero.add(970)
        o.add_colden_particle(line, colden, 1.0, 1, 4802.5, 1)
        near(colden[960] + 1, 1)
        for i in range(2000):
            if i not in nonzero:
                assert colden[i] + i == i


def test_index_table_near_lines(impls):
    # test.cpp:164-248
    d = golden("index_testcpp.npz")
    cofm, axis, box = d["cofm"], d["axis"], float(d["box"])
    for o in impls:
        nl = lambda p, h: o.near_lines(cofm, axis, box, np.array(p, dtype=np.float32), h)
        n = nl([500, 2000, 1000], 1)
        assert n == {6: 0.0}
        n = nl([5000, 2000, 1000], 1)
        assert n == {6: 0.0}
        n = nl([5010, 2010, 990], 20)
        assert n == {6: 10 * 10 + 10 * 10.}
        assert nl([5010, 2010, 990], 10) == {}
        n = nl([4000, 4000, 4000], 1)
        assert n == {0: 0.0, 1: 0.0}
        n = nl([4000, 4000, 4000], 25)
        assert n == {0: 0.0, 1: 0.0, 2: 20 * 20 + 10 * 10., 3: 10 * 10.}
        n = nl([1000, 9999.9, 9999.9], 0.6)
        assert sorted(n) == [4, 5]
        near(n[4], 0.5 * 0.5 + 0.2 * 0.2, 1e-2)
        near(n[5], 0.3 * 0.3 + 0.4 * 0.4, 1e-2)
        n = nl([1000.5, 2000, 501], 1.5)
        assert sorted(n) == [7, 8, 9]
        near(n[7], 0.25, 1e-2)
        near(n[8], 0.25 + 1, 1e-2)
        near(n[9], 1, 1e-2)


def test_index_table_near_particles(impls):
    # test.cpp:250-281, plus exact equality with the reference's pair lists
    d = golden("index_testcpp.npz")
    for o in impls:
        off, part, dr2 = o.near_particles(d["pos"], d["hh"], d["axis"], d["cofm"], float(d["box"]))
        sizes = np.diff(off)
        assert list(sizes) == [1, 1, 1, 2, 1, 2, 3, 1, 1, 1, 0, 0, 0]
        lists = [list(part[off[i]:off[i + 1]]) for i in range(len(sizes))]
        assert lists[0][0] == 3
        assert 3 in lists[3]
        assert 4 in lists[5] and 8 in lists[5]
        assert lists[6] == [0, 1, 2]
        assert lists[8][0] == 5
        assert np.array_equal(off, d["off"]) and np.array_equal(part, d["part"])
        assert np.array_equal(dr2.view(np.int64), d["dr2"].view(np.int64))


def test_profile(impls):
    # test.cpp:284-302
    cases = [(0, 0, 1), (0, 0.1, 0.896457), (0.1, 1e-6, 0.990048), (0.1, 1e-4, 0.989939),
             (15, 1e-6, 2.52441e-9), (15, 1e-4, 2.52441e-7), (20, 1e-7, 1.4158e-10),
             (1, 1e-4, 0.367888), (1.5, 1e-6, 0.1054), (2, 1e-7, 0.0183157),
             (1, 1e-3, 0.367965)]
    for o in impls:
        for u, a, v in cases:
            near(o.voigt(u, a), v)


def test_single_absorber(impls):
    # test.cpp:304-332
    corr = 3 / (4 * math.pi)
    for o in impls:
        bb = 0.128557 * math.sqrt(2e4 / 1)
        t = lambda vdr2, vsm, aa, lo, hi: o.tau_kern_outer(bb, vdr2, vsm, aa, 1, lo, hi)
        near(t(0, 10, 1e-4, 0, 0), corr * 78.0409)
        near(t(0, 10, 1e-4, 5, 5), corr * 72.6216)
        near(t(0, 10, 1e-4, 10, 10), corr * 58.5185)
        near(t(0, 10, 1e-4, 20, 20), corr * 24.6696)
        near(t(0, 2, 1e-4, 5, 5), corr * 14.8203)
        near(t(25, 10, 1e-4, 0, 0), corr * 18.218, 1e-2)
        near(t(25, 10, 1e-4, 5, 5), corr * 16.9436, 1e-2)
        bb = 0.128557 * math.sqrt(2e4 / 16)
        t = lambda vdr2, vsm, aa, lo, hi: o.tau_kern_outer(bb, vdr2, vsm, aa, 1, lo, hi)
        near(t(0, 5, 1e-6, 0, 10), corr * 16.0403, 1e-2)
        near(t(0, 5, 1e-6, -5, 5), corr * 27.1978, 1e-2)


def test_add_tau(impls):
    # test.cpp:339-381
    BOLTZMANN, PROTONMASS = 1.3806504e-16, 1.67262178e-24
    velfac = VELFAC_TEST
    temp, smooth, amp = 2e4, 3, 7.57973e-15
    bb = math.sqrt(2.0 * BOLTZMANN / PROTONMASS) / 1e5 * math.sqrt(temp / 1.00794)
    voigt_fac = 1215.6701e-10 * 6.265e8 / (4. * math.pi) / 1e5
    rscale = 3.085678e21 * 0.25 / 0.7
    line = LYA_TEST + (velfac, 10000, 0.25, 1, 1e-5)
    for o in impls:
        vbin = lambda b, p: 10000 * velfac / 2000 * b - velfac * p
        SA = lambda b, p, dens: (amp * dens / bb * o.tau_kern_outer(
            bb, 0, velfac * smooth, voigt_fac / bb, 1, vbin(b, p), vbin(b + 1, p)) / velfac)
        tau = np.zeros(2000)
        o.add_tau_particle(line, tau, 0, 1e-3 * rscale, 5002.5, 0, temp, smooth)
        near(tau[999], SA(999, 5002.5, 1e-3 * rscale))
        near(tau[1000], SA(1000, 5002.5, 1e-3 * rscale))
        near(tau[1001], tau[999])
        for b in (400, 401, 402):
            near(tau[b], SA(b, 5002.5, 1e-3 * rscale))
        tau[:] = 0
        pecvel = 10000 / 2000 * 3 * velfac
        o.add_tau_particle(line, tau, 0, 1e-3 * rscale, 5002.5, pecvel, temp, smooth)
        near(tau[1002], SA(999, 5002.5, 1e-3 * rscale))
        near(tau[1003], SA(1000, 5002.5, 1e-3 * rscale))
        near(tau[1004], tau[1002])
        tau[:] = 0
        o.add_tau_particle(line, tau, 1, 1, 5002.5, 0, 10000, 1)
        near(tau[1000] + 1, 1)
        near(tau[1501] + 1, 1)


def test_tau_colden_consistency(impls):
    # test.cpp:384-404
    velfac = VELFAC_TEST
    rscale = 3.085678e21 * 0.25 / 0.7
    line = LYA_TEST + (velfac, 10000, 0.25, 1, 1e-5)
    for o in impls:
        tau = np.zeros(2000)
        colden = np.zeros(2000)
        o.add_tau_particle(line, tau, 0, 0.1 * rscale, 5002.5, 0, 2e4, 3)
        o.add_colden_particle(line, colden, 0, 0.1 * rscale, 5002.5, 3)
        near(tau.sum() / colden.sum(), 7.57973e-15 / velfac / 2.81809)
