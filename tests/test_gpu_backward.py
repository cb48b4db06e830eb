"""The backward kernel (FP32) against FP64 central differences of the CPU oracle
and against a dense FP64 PyTorch re-implementation with scipy's Faddeeva
function.  Loss: sum (exp(-tau) - F_target)^2."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


def small_workload():
    w = synth.config4(nside=20, nlos=24)
    # keep every pixel narrower than b/2 (midpoint rule, as the dense reference assumes)
    w.temp = np.maximum(w.temp, np.float32(2000.0))
    return w


def gpu_grads(ctx, w, target):
    import torch
    from fake_spectra_gb300.autograd import particle_tau
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pos, vel, dens, temp, hh = T(w.pos), T(w.vel), T(w.dens["HI"]), T(w.temp), T(w.hh)
    vel.requires_grad_(True)
    dens.requires_grad_(True)
    temp.requires_grad_(True)
    t = synth.LYA
    tau = particle_tau(ctx, w.nbins, w.kernel, w.box, w.velfac, w.atime, t.lambda_cm, t.gamma,
                       t.fosc, t.amumass, w.tautail, pos, vel, dens, temp, hh, w.axis, w.cofm)
    loss = ((torch.exp(-tau) - T(target)) ** 2).sum()
    loss.backward()
    return (dens.grad.cpu().numpy().astype(np.float64), temp.grad.cpu().numpy().astype(np.float64),
            vel.grad.cpu().numpy().astype(np.float64))


def oracle_loss(port, w, target, lines, field, ip, value, comp=0):
    args = list(w.call_args(synth.LYA, 1))
    arr = {"dens": 13, "temp": 14, "vel": 12}[field]
    a = args[arr].copy()
    if field == "vel":
        a[ip, comp] = value
    else:
        a[ip] = value
    args[arr] = a
    args[16] = w.axis[lines]
    args[17] = w.cofm[lines]
    tau = port.particle_interpolate(*args)
    return float(((np.exp(-tau) - target[lines]) ** 2).sum())


def test_backward_matches_oracle_finite_differences(ctx, port):
    w = small_workload()
    t = synth.LYA
    base = port.particle_interpolate(*w.call_args(t, 1))
    target = np.exp(-0.7 * base)
    gd, gT, gv = gpu_grads(ctx, w, target)
    off, part, _ = port.near_particles(w.pos, w.hh, w.axis, w.cofm, w.box)
    line_of = np.repeat(np.arange(w.nlos), np.diff(off))
    rng = np.random.default_rng(3)
    cand = np.unique(part)
    checked = 0
    scale = {"dens": np.abs(gd).max(), "temp": np.abs(gT).max(), "vel": np.abs(gv).max()}
    for ip in rng.choice(cand, size=min(40, cand.size), replace=False):
        lines = np.unique(line_of[part == ip])
        for field, g in (("dens", gd[ip]), ("temp", gT[ip]), ("vel", gv[ip, 0])):
            x0 = {"dens": w.dens["HI"][ip], "temp": w.temp[ip], "vel": w.vel[ip, 0]}[field]
            ests = []
            for rel in (2e-6, 8e-6):
                step = max(abs(float(x0)) * rel, 1e-6 if field == "vel" else 1e-30)
                xp, xm = np.float32(x0 + step), np.float32(x0 - step)
                lp = oracle_loss(port, w, target, lines, field, ip, xp)
                lm = oracle_loss(port, w, target, lines, field, ip, xm)
                ests.append((lp - lm) / (float(xp) - float(xm)))
            fd = ests[0]
            if abs(ests[0] - ests[1]) > 0.02 * max(abs(ests[0]), 1e-12 * scale[field]):
                continue   # the step moved a window edge (tautail rule): not differentiable here
            assert abs(g - fd) <= 2e-3 * abs(fd) + 2e-4 * scale[field], (field, ip, g, fd)
            checked += 1
    assert checked >= 60


def test_backward_matches_dense_torch_fp64(ctx, port):
    import torch
    from dense_ref import dense_tau
    w = small_workload()
    lines = np.array([0, 5, 11])
    w.axis, w.cofm = w.axis[lines], w.cofm[lines]
    t = synth.LYA
    target = np.exp(-0.7 * port.particle_interpolate(*w.call_args(t, 1)))
    gd, gT, gv = gpu_grads(ctx, w, target)
    off, part, dr2 = port.near_particles(w.pos, w.hh, w.axis, w.cofm, w.box)
    pl = np.repeat(np.arange(w.nlos), np.diff(off))
    f64 = lambda a: torch.tensor(np.asarray(a, dtype=np.float64))
    dens = f64(w.dens["HI"]).requires_grad_(True)
    temp = f64(w.temp).requires_grad_(True)
    vlos = f64(w.vel[:, 0]).requires_grad_(True)
    pi = torch.from_numpy(part.astype(np.int64))
    tau = dense_tau((t.lambda_cm, t.gamma, t.fosc, t.amumass), w.nbins, w.box, w.velfac,
                    w.tautail, w.nlos, torch.from_numpy(pl), f64(dr2), f64(w.pos[part, 0]),
                    vlos[pi], dens[pi], temp[pi], f64(w.hh[part]))
    loss = ((torch.exp(-tau) - f64(target)) ** 2).sum()
    loss.backward()
    for name, g_gpu, g_ref in (("dens", gd, dens.grad), ("temp", gT, temp.grad),
                               ("vel", gv[:, 0], vlos.grad)):
        g_ref = g_ref.numpy()
        sel = np.unique(part)
        err = np.abs(g_gpu[sel] - g_ref[sel])
        tol = 2e-3 * np.abs(g_ref[sel]) + 2e-4 * np.abs(g_ref[sel]).max()
        assert (err <= tol).all(), (name, err.max(), np.abs(g_ref[sel]).max())
