"""TEST INFRASTRUCTURE: a dense FP64 PyTorch re-implementation of the tau
deposit (absorption.cpp:212-279, singleabs.h:104-167) for gradient checks.

Every pair is evaluated on its full +-nbins/2 pixel range and masked with the
reference's tautail stop rule (the mask carries no gradient, as the window is
held fixed in the backward).  The profile H = Re w(u + i a) and its partial
derivatives come from scipy.special.wofz through a custom autograd function:
dw/dz = -2 z w + 2i/sqrt(pi), so dH/du = Re w', dH/da = -Im w'.  Only the
midpoint rule of tau_kern_outer is implemented: callers use pixels narrower
than b/2 for every particle.
"""
import math

import numpy as np
import torch

PI = math.pi
SIGMA_T = 6.652458558e-25
BOLTZMANN = 1.3806504e-16
PROTONMASS = 1.67262178e-24
LIGHT_KMS = 2.99792458e10 / 1e5


class _VoigtH(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, a):
        from scipy.special import wofz
        z = u.detach().numpy() + 1j * a.detach().numpy()
        w = wofz(z)
        ctx.z = z
        ctx.w = w
        return torch.from_numpy(np.ascontiguousarray(w.real))

    @staticmethod
    def backward(ctx, g):
        dw = -2.0 * ctx.z * ctx.w + 2j / math.sqrt(PI)
        return g * torch.from_numpy(dw.real.copy()), g * torch.from_numpy(-dw.imag.copy())


def cubic_kernel(q):
    norm = 32. / 4 / PI
    out = torch.where(q < 0.5, norm * (1 - 6 * q * q + 6 * q ** 3), norm * 2 * (1 - q) ** 3)
    return torch.where(q >= 1, torch.zeros_like(q), out)


def dense_tau(line, nbins, box, velfac, tautail, nlos, pair_line, pair_dr2, ppos, pvel, dens,
              temp, hh):
    """tau [nlos, nbins] (float64, differentiable in pvel, dens, temp: 1 entry per pair)."""
    lam, gamma, fosc, amumass = line
    sigma_a = math.sqrt(3.0 * PI * SIGMA_T / 8.0) * lam * fosc
    bfac = math.sqrt(2.0 * BOLTZMANN / (amumass * PROTONMASS)) / 1e5
    voigt_fac = gamma * lam / (4. * PI) / 1e5
    vbox = box * velfac
    bintov = vbox / nbins
    btherm = bfac * torch.sqrt(temp)
    vel = velfac * ppos + pvel
    vdr2 = (velfac * pair_dr2) * velfac
    vsmooth = velfac * hh
    vhigh = torch.sqrt(torch.clamp(vsmooth * vsmooth - vdr2, min=0.0))
    deltav = 2. * vhigh / 8
    i = torch.arange(1, 8, dtype=torch.float64)
    vv = i[None, :] * deltav[:, None] - vhigh[:, None]                      # [P, 7]
    w = cubic_kernel(torch.sqrt(vdr2[:, None] + vv * vv) / vsmooth[:, None])
    aa = voigt_fac / btherm
    amp = sigma_a / math.sqrt(PI) * (LIGHT_KMS / btherm)
    zmax = torch.floor(vel.detach() / bintov)
    half = nbins // 2
    k = torch.arange(-half, half, dtype=torch.float64)                      # pixel offsets
    z = zmax[:, None] + k[None, :]                                          # [P, K]
    vlow = z * bintov - vel[:, None]
    # tau_kern_outer: midpoint (np = 1) or trapezoid sub-samples, per pair
    with torch.no_grad():
        half_b = btherm / 2.
        npts = torch.where(bintov < half_b, torch.ones_like(half_b),
                           2 * torch.ceil(bintov / half_b / 2) + 1).to(torch.int64)
    S = torch.zeros(vlow.shape, dtype=torch.float64)
    for n in torch.unique(npts).tolist():
        sel = npts == n
        if n == 1:
            offs, wts = [0.5 * bintov], [1.0]
        else:
            dv = bintov / (n - 1)
            offs = [i * dv for i in range(n)]
            wts = [(0.5 if i in (0, n - 1) else 1.0) / (n - 1) for i in range(n)]
        vl = vlow[sel]
        acc = torch.zeros(vl.shape, dtype=torch.float64)
        for off, wt in zip(offs, wts):
            vouter = vl + off
            u = (vv[sel][:, None, :] - vouter[:, :, None]) / btherm[sel][:, None, None]
            a3 = aa[sel][:, None, None].expand_as(u)
            H = _VoigtH.apply(u.reshape(-1), a3.reshape(-1)).reshape(u.shape)
            acc = acc + wt * (H * w[sel][:, None, :]).sum(-1)
        S = S.index_put((sel.nonzero()[:, 0],), acc)
    tl = (amp * dens)[:, None] * deltav[:, None] * S / velfac
    # stop rule: forward from k = 0, backward from k = -1, each including the
    # first pixel below tautail
    with torch.no_grad():
        below = (tl < tautail)
        fwd = below[:, half:]
        bwd = torch.flip(below[:, :half], dims=[1])
        def keep(b):
            # pixel m kept iff no pixel before m (in walk order) was below tautail
            prior = torch.cumsum(b.to(torch.int64), dim=1) - b.to(torch.int64)
            return prior == 0
        mask = torch.cat([torch.flip(keep(bwd), dims=[1]), keep(fwd)], dim=1)
    contrib = torch.where(mask, tl, torch.zeros_like(tl))
    j = torch.remainder(z, nbins).to(torch.int64)
    tau = torch.zeros(nlos * nbins, dtype=torch.float64)
    tau = tau.index_add(0, (pair_line[:, None] * nbins + j).reshape(-1), contrib.reshape(-1))
    return tau.reshape(nlos, nbins)
