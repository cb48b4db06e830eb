"""The backward kernel (FP32) against FP64 central differences of the CPU oracle
and against a dense FP64 PyTorch re-implementation with scipy's Faddeeva
function.  Loss: sum (exp(-tau) - F_target)^2.

Two workloads: a quick 20^3 / 24-sightline one in which a fifth of the
particles are cooled so that tau_kern_outer sub-samples their pixels
(singleabs.h:104-126; some so cold that the FP32 form walks them in FP64),
and the 128^3 / 1024-sightline workload at 2 km/s with 256 random particles
and a relative step of 1e-6."""
import numpy as np
import pytest

from fake_spectra_gb300 import synth

pytestmark = pytest.mark.gpu


def small_workload():
    w = synth.config4(nside=20, nlos=24)
    # cool 15% of the particles to 300 K (b/2 = 1.1 km/s < the 2 km/s pixel: three
    # trapezoid sub-samples) and 5% to 20 K (nine sub-samples: the FP32 form's FP64 walk)
    rng = np.random.default_rng(8)
    r = rng.random(w.npart)
    w.temp = np.where(r < 0.15, np.float32(300.0), np.where(r < 0.2, np.float32(20.0), w.temp))
    w.temp = w.temp.astype(np.float32)
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


def _npoints(bfac, temp, bintov):
    """tau_kern_outer's sub-sample count (singleabs.h:113-116) for a float32 temperature."""
    half_b = bfac * np.sqrt(np.float64(temp)) / 2.
    return 1 if bintov < half_b else int(2 * np.ceil(bintov / half_b / 2) + 1)


def test_backward_config4_against_oracle_fd(ctx, port):
    """128^3 particles (L = 20 Mpc/h), 1024 sightlines along axis 1, 2 km/s pixels,
    Ly-a; F_target is the forward output of a second seed.  dL/d(dens), dL/dT and
    dL/d(v_los) of 256 random particles against FP64 central differences of the
    oracle with a relative step of 1e-6.

    tau is a sum over pairs (part_int.cpp:20-51), so moving one particle changes
    only its own pairs' terms: the difference of the loss is evaluated from the
    oracle's per-pair deposit (LineAbsorption::add_tau_particle,
    absorption.cpp:212-279) at x+ and x-, on the oracle's tau of every sightline
    the particle touches, pixel by pixel as e-(expm1(c- - c+))(e+ + e- - 2F).
    A step that moves a window edge (the set of deposited pixels changes, e.g.
    the particle's pixel or the tautail stop pixel) or the sub-sample count is
    not differentiable there; it is skipped and counted.  The recipe's
    temperatures stay above 1800 K, so every pixel takes the midpoint rule here;
    the sub-sampled forms are covered by the quick workload above."""
    import torch
    from fake_spectra_gb300.autograd import particle_tau
    from fake_spectra_gb300 import interp as I
    t = synth.LYA
    w = synth.generate_torch(4, device="cuda")
    wt = synth.generate_torch(4, seed=5, device="cuda")
    ftarget = torch.exp(-I.particle_interpolate_device(ctx, *wt.call_args(t, 1),
                                                       precision="fp32"))
    del wt
    dens = w.dens["HI"].clone().requires_grad_(True)
    temp = w.temp.clone().requires_grad_(True)
    vel = w.vel.clone().requires_grad_(True)
    tau = particle_tau(ctx, w.nbins, w.kernel, w.box, w.velfac, w.atime, t.lambda_cm, t.gamma,
                       t.fosc, t.amumass, w.tautail, w.pos, vel, dens, temp, w.hh, w.axis,
                       w.cofm)
    ((torch.exp(-tau) - ftarget) ** 2).sum().backward()
    gd = dens.grad.cpu().numpy().astype(np.float64)
    gT = temp.grad.cpu().numpy().astype(np.float64)
    gv = vel.grad[:, 0].cpu().numpy().astype(np.float64)
    F = ftarget.cpu().numpy()
    wh = w.to_host()
    off, part, dr2 = port.near_particles(wh.pos, wh.hh, w.axis, w.cofm, w.box)
    line_of = np.repeat(np.arange(w.nlos), np.diff(off))
    rng = np.random.default_rng(44)
    chosen = rng.choice(np.unique(part), size=256, replace=False)
    touched = np.unique(line_of[np.isin(part, chosen)])
    # the oracle's tau of every touched sightline (particles near them, ascending)
    near = np.unique(part[np.isin(line_of, touched)])
    a = list(wh.call_args(t, 1))
    for k in range(11, 16):
        a[k] = a[k][near]
    a[16], a[17] = w.axis[touched], w.cofm[touched]
    base = dict(zip(touched.tolist(), port.particle_interpolate(*a)))
    geom = (t.lambda_cm, t.gamma, t.fosc, t.amumass, w.velfac, w.box, w.atime, w.kernel,
            w.tautail)
    bfac = np.sqrt(2.0 * 1.3806504e-16 / (t.amumass * 1.67262178e-24)) / 1e5
    bintov = w.box * w.velfac / w.nbins

    def contrib(e, ip, dens_, temp_, vlos):
        c = np.zeros(w.nbins)
        port.add_tau_particle(geom, c, dr2[e], dens_, wh.pos[ip, 0], vlos, temp_, wh.hh[ip])
        return c

    grads = {"dens": gd, "temp": gT, "vel": gv}
    scale = {k: np.abs(v[chosen]).max() for k, v in grads.items()}
    errs, skipped, checked = [], 0, 0
    for ip in chosen:
        es = np.nonzero(part == ip)[0]
        x0 = {"dens": wh.dens["HI"][ip], "temp": wh.temp[ip], "vel": wh.vel[ip, 0]}
        for field in ("dens", "temp", "vel"):
            step = abs(float(x0[field])) * 1e-6
            xp, xm = np.float32(x0[field] + step), np.float32(x0[field] - step)
            if field == "temp" and _npoints(bfac, xp, bintov) != _npoints(bfac, xm, bintov):
                skipped += 1
                continue
            dL, edge = 0.0, False
            for e in es:
                vals = {}
                for sgn, x in (("+", xp), ("-", xm)):
                    v = dict(x0)
                    v[field] = x
                    vals[sgn] = contrib(e, ip, v["dens"], v["temp"], v["vel"])
                c0 = contrib(e, ip, x0["dens"], x0["temp"], x0["vel"])
                if not (np.array_equal(vals["+"] != 0, c0 != 0)
                        and np.array_equal(vals["-"] != 0, c0 != 0)):
                    edge = True
                    break
                l = line_of[e]
                rest = base[l] - c0
                tp, tm = rest + vals["+"], rest + vals["-"]
                ep, em = np.exp(-tp), np.exp(-tm)
                dL += float(np.sum(em * np.expm1(vals["-"] - vals["+"]) *
                                   (ep + em - 2.0 * F[l])))
            if edge:
                skipped += 1
                continue
            fd = dL / (float(xp) - float(xm))
            g = grads[field][ip]
            errs.append((field, abs(g - fd) / max(abs(fd), 1e-300)))
            assert abs(g - fd) <= 2e-3 * abs(fd) + 2e-4 * scale[field], (field, ip, g, fd)
            checked += 1
    rel = np.array([e for _, e in errs])
    print("\nconfig-4 gradient check: %d of %d derivatives checked, %d skipped (window edge or "
          "sub-sample count moved by the step); relative error median %.2e, 99th pct %.2e"
          % (checked, 3 * len(chosen), skipped, np.median(rel), np.percentile(rel, 99)))
    assert checked >= 0.9 * 3 * len(chosen)


def test_backward_reuses_the_forward_search(ctx):
    """The autograd backward reuses the forward's sightline search (the
    context's search generation and the search inputs match), and gives the
    gradients of the backward that searches again, up to the order of its
    float atomics.  After another search on the context the reuse entry
    searches again."""
    import torch
    from fake_spectra_gb300 import interp as I
    w = small_workload()
    target = np.exp(-np.full((len(w.axis), w.nbins), 0.3))
    gd, gt, gv = gpu_grads(ctx, w, target)
    assert ctx.stats()["search_reused"] == 1
    T = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    t = synth.LYA
    args = (w.nbins, w.kernel, w.box, w.velfac, w.atime, t.lambda_cm, t.gamma, t.fosc,
            t.amumass, w.tautail)
    pos, vel, dens, temp, hh = T(w.pos), T(w.vel), T(w.dens["HI"]), T(w.temp), T(w.hh)
    tau = I.particle_interpolate_device(ctx, 1, *args, pos, vel, dens, temp, hh, w.axis, w.cofm,
                                        precision="fp32")
    F = torch.exp(-tau)
    grad_tau = -2.0 * (F - T(target)) * F
    gen = ctx.search_generation()
    # an unrelated search on the same context in between: the reuse entry must search again
    I.particle_interpolate_device(ctx, 1, *args, pos + 1.0, vel, dens, temp, hh, w.axis,
                                  w.cofm, precision="fp32")
    r = I.tau_backward_device(ctx, *args, pos, vel, dens, temp, hh, w.axis, w.cofm, grad_tau,
                              generation=gen)
    assert ctx.stats()["search_reused"] == 0
    fresh = I.tau_backward_device(ctx, *args, pos, vel, dens, temp, hh, w.axis, w.cofm, grad_tau)
    for got, want in zip((gd, gt, gv), fresh):
        want = want.cpu().numpy().astype(np.float64)
        np.testing.assert_allclose(got, want, rtol=1e-4, atol=1e-6 * np.abs(want).max())
    for got, want in zip(r, fresh):
        np.testing.assert_allclose(got.cpu().numpy(), want.cpu().numpy(), rtol=1e-4,
                                   atol=1e-6 * float(want.abs().max()))
