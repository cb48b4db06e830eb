"""torch.autograd access to the tau deposit (tuned FP32 form).

`particle_tau(ctx, line, geometry, pos, vel, dens, temp, hh, axis, cofm)` returns
tau (float64, [nlos, nbins]) differentiable with respect to `dens`, `temp` and
`vel` (the line-of-sight component).  The forward is the FP32 deposit kernel,
the backward the hand-written backward kernel (include/fsg.h,
fsg_tau_backward_reuse_device), which reuses the forward's sightline search
when it is still the context's last one (torch's version counters guard the
saved positions and smoothing lengths) and recomputes the profiles instead of
storing them.  Positions and smoothing lengths are inputs without gradients.
"""
import torch

from . import interp


class _ParticleTau(torch.autograd.Function):
    @staticmethod
    def forward(fctx, ctx, args, pos, vel, dens, temp, hh, axis, cofm):
        tau = interp.particle_interpolate_device(ctx, *args, pos, vel, dens, temp, hh, axis, cofm,
                                                 precision="fp32")
        fctx.ctx = ctx
        fctx.args = args
        fctx.generation = ctx.search_generation()
        fctx.axis = axis
        fctx.cofm = cofm
        fctx.save_for_backward(pos, vel, dens, temp, hh)
        return tau

    @staticmethod
    def backward(fctx, grad_tau):
        pos, vel, dens, temp, hh = fctx.saved_tensors
        gd, gt, gv = interp.tau_backward_device(fctx.ctx, *fctx.args[1:], pos, vel, dens, temp, hh,
                                                fctx.axis, fctx.cofm,
                                                grad_tau.to(torch.float64),
                                                generation=fctx.generation)
        return None, None, None, gv, gd, gt, None, None, None


def particle_tau(ctx, nbins, kernel, box, velfac, atime, lam, gamma, fosc, amumass, tautail,
                 pos, vel, dens, temp, hh, axis, cofm):
    """Differentiable tau (see module docstring)."""
    args = (1, int(nbins), int(kernel), float(box), float(velfac), float(atime), float(lam),
            float(gamma), float(fosc), float(amumass), float(tautail))
    return _ParticleTau.apply(ctx, args, pos, vel, dens, temp, hh, axis, cofm)
