"""Device-resident entry points (particle arrays already in HBM as torch tensors).

These are what a batched caller uses: the particle arrays live on the GPU,
the sightline tables (axis, cofm) are small host arrays, and outputs are
float64 device tensors.  Kernels run on torch's current CUDA stream.
"""
import ctypes

import numpy as np

from . import _lib


def _dptr(t, dtype_name, name):
    import torch
    want = {"float32": torch.float32, "float64": torch.float64}[dtype_name]
    if not t.is_cuda:
        raise ValueError("%s must be a CUDA tensor" % name)
    if t.dtype != want:
        raise TypeError("%s must be %s" % (name, dtype_name))
    if not t.is_contiguous():
        raise ValueError("%s must be contiguous" % name)
    return ctypes.c_void_p(t.data_ptr())


def _host_tables(axis, cofm):
    axis = np.ascontiguousarray(np.asarray(axis), dtype=None)
    cofm = np.ascontiguousarray(np.asarray(cofm), dtype=None)
    if axis.dtype != np.int32:
        raise TypeError("Axis must be a 32-bit integer\n")
    if cofm.dtype != np.float64:
        raise TypeError("Sightline positions must have 64-bit float type\n")
    if cofm.ndim != 2 or cofm.shape[1] != 3 or cofm.shape[0] != axis.shape[0]:
        raise ValueError("cofm must have dimensions (np.size(axis),3) \n")
    return axis, cofm


def _bind_stream(ctx):
    import torch
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)


def particle_interpolate_device(ctx, compute_tau, nbins, kernel, box, velfac, atime, lam, gamma,
                                fosc, amumass, tautail, pos, vel, dens, temp, h, axis, cofm,
                                out=None, precision="fp64", threads=0, persistent=-1,
                                count_work=False, far_tiles=True, chunk=0, tune=0, records=-1):
    """`_Particle_Interpolate` on device tensors; returns `out` (nlos, nbins) float64 on device.
    far_tiles=False deposits the far damping wing of the FP32 form pixel by pixel.
    threads/chunk/persistent/records left at 0/0/-1/-1 take the autotuner's
    launch in the FP32 form (tune: 0 cached, 1 time again, -1 library defaults);
    records=1 routes the FP32 optical depth through staged pair records."""
    import torch
    axis, cofm = _host_tables(axis, cofm)
    nlos = int(axis.shape[0])
    npart = int(pos.shape[0])
    if out is None:
        out = torch.empty((nlos, int(nbins)), dtype=torch.float64, device=pos.device)
    args_p = [_dptr(pos, "float32", "pos"),
              _dptr(vel, "float32", "vel") if compute_tau else None,
              _dptr(dens, "float32", "dens"),
              _dptr(temp, "float32", "temp") if compute_tau else None,
              _dptr(h, "float32", "h")]
    _bind_stream(ctx)
    opt = _lib.make_options(precision, threads, persistent, count_work, far_tiles, chunk, tune,
                            records)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_particle_interpolate_device(
        ctx.handle, int(compute_tau), int(nbins), int(kernel), float(box), float(velfac),
        float(atime), float(lam), float(gamma), float(fosc), float(amumass), float(tautail),
        *args_p, npart, axis.ctypes.data_as(ctypes.c_void_p),
        cofm.ctypes.data_as(ctypes.c_void_p), nlos, _dptr(out, "float64", "out"),
        ctypes.byref(opt), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out


def spectra_batch_device(ctx, nbins, kernel, box, velfac, atime, tautail, pos, vel, temp, h,
                         axis, cofm, lines, precision="fp32", threads=0, persistent=-1, chunk=0,
                         tune=0, records=-1):
    """Several absorption lines in one call (one sightline search, one CUDA graph).

    lines: sequence of (transition, dens, want_tau, want_colden) with
    `transition` having lambda_cm/gamma/fosc/amumass and `dens` a float32 device
    tensor.  Returns a list of (tau, colden) float64 device tensors (None where
    not wanted)."""
    import torch
    axis, cofm = _host_tables(axis, cofm)
    nlos = int(axis.shape[0])
    arr = (_lib.Line * max(1, len(lines)))()
    outs = []
    for k, (t, dens, want_tau, want_colden) in enumerate(lines):
        tau = torch.empty((nlos, int(nbins)), dtype=torch.float64, device=pos.device) \
            if want_tau else None
        col = torch.empty((nlos, int(nbins)), dtype=torch.float64, device=pos.device) \
            if want_colden else None
        arr[k].lambda_ = float(t.lambda_cm)
        arr[k].gamma = float(t.gamma)
        arr[k].fosc = float(t.fosc)
        arr[k].amumass = float(t.amumass)
        arr[k].dens = _dptr(dens, "float32", "dens")
        arr[k].tau = _dptr(tau, "float64", "tau") if tau is not None else None
        arr[k].colden = _dptr(col, "float64", "colden") if col is not None else None
        outs.append((tau, col))
    _bind_stream(ctx)
    opt = _lib.make_options(precision, threads, persistent, chunk=chunk, tune=tune,
                            records=records)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_spectra_batch_device(
        ctx.handle, int(nbins), int(kernel), float(box), float(velfac), float(atime),
        float(tautail), _dptr(pos, "float32", "pos"), _dptr(vel, "float32", "vel"),
        _dptr(temp, "float32", "temp"), _dptr(h, "float32", "h"), int(pos.shape[0]),
        axis.ctypes.data_as(ctypes.c_void_p), cofm.ctypes.data_as(ctypes.c_void_p), nlos,
        len(lines), arr, ctypes.byref(opt), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return outs


def tau_backward_device(ctx, nbins, kernel, box, velfac, atime, lam, gamma, fosc, amumass,
                        tautail, pos, vel, dens, temp, h, axis, cofm, grad_tau,
                        generation=None):
    """Gradients (d_dens, d_temp, d_vel) of L from dL/dtau, FP32, new float32 tensors.
    With `generation` (ctx.search_generation() right after the forward call on
    the same pos, h, axis and cofm, whose contents the caller has not changed)
    the forward's sightline search is reused when it is still the context's
    last one."""
    import torch
    axis, cofm = _host_tables(axis, cofm)
    gd = torch.zeros_like(dens)
    gt = torch.zeros_like(temp)
    gv = torch.zeros_like(vel)
    grad_tau = grad_tau.contiguous()
    _bind_stream(ctx)
    eb = _lib.errbuf()
    L = _lib.load()
    tail = (int(nbins), int(kernel), float(box), float(velfac), float(atime), float(lam),
            float(gamma), float(fosc), float(amumass), float(tautail),
            _dptr(pos, "float32", "pos"), _dptr(vel, "float32", "vel"),
            _dptr(dens, "float32", "dens"), _dptr(temp, "float32", "temp"),
            _dptr(h, "float32", "h"), int(pos.shape[0]), axis.ctypes.data_as(ctypes.c_void_p),
            cofm.ctypes.data_as(ctypes.c_void_p), int(axis.shape[0]),
            _dptr(grad_tau, "float64", "grad_tau"), _dptr(gd, "float32", "gd"),
            _dptr(gt, "float32", "gt"), _dptr(gv, "float32", "gv"), eb, 512)
    if generation is None:
        rc = L.fsg_tau_backward_device(ctx.handle, *tail)
    else:
        rc = L.fsg_tau_backward_reuse_device(ctx.handle, int(generation), *tail)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return gd, gt, gv


def near_lines_device(ctx, box, pos, h, axis, cofm):
    """`_near_lines` on device tensors: ascending int32 indices (device tensor) of
    the particles within their smoothing length of any sightline."""
    import torch
    axis, cofm = _host_tables(axis, cofm)
    npart = int(pos.shape[0])
    out = torch.empty(max(npart, 1), dtype=torch.int32, device=pos.device)
    _bind_stream(ctx)
    n = ctypes.c_int64(0)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_near_lines_device(ctx.handle, float(box), _dptr(pos, "float32", "pos"),
                                 _dptr(h, "float32", "h"), npart,
                                 axis.ctypes.data_as(ctypes.c_void_p),
                                 cofm.ctypes.data_as(ctypes.c_void_p), int(axis.shape[0]),
                                 ctypes.c_void_p(out.data_ptr()), ctypes.byref(n), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out[:n.value]


def colden_channels_device(ctx, nbins, kernel, box, velfac, pos, h, axis, cofm, dens,
                           precision="fp64"):
    """Several weighted column densities in one pass: one (nlos, nbins) float64
    device tensor per float32 density tensor in `dens` (at most 8), each equal to
    the compute_tau=0 interpolation with that density."""
    import torch
    axis, cofm = _host_tables(axis, cofm)
    nlos = int(axis.shape[0])
    dens = list(dens)
    outs = [torch.empty((nlos, int(nbins)), dtype=torch.float64, device=pos.device)
            for _ in dens]
    dp = (ctypes.c_void_p * max(len(dens), 1))(*[_dptr(d, "float32", "dens").value
                                                 for d in dens])
    op = (ctypes.c_void_p * max(len(outs), 1))(*[o.data_ptr() for o in outs])
    _bind_stream(ctx)
    opt = _lib.make_options(precision)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_colden_channels_device(ctx.handle, int(nbins), int(kernel), float(box),
                                      float(velfac), _dptr(pos, "float32", "pos"),
                                      _dptr(h, "float32", "h"), int(pos.shape[0]),
                                      axis.ctypes.data_as(ctypes.c_void_p),
                                      cofm.ctypes.data_as(ctypes.c_void_p), nlos, len(dens),
                                      ctypes.cast(dp, ctypes.c_void_p),
                                      ctypes.cast(op, ctypes.c_void_p), ctypes.byref(opt), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return outs


def build_pairs(ctx, box, pos, h, axis, cofm):
    """Sightline-particle search on the device; returns the number of pairs."""
    axis, cofm = _host_tables(axis, cofm)
    _bind_stream(ctx)
    n = ctypes.c_int64(0)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_build_pairs_device(ctx.handle, float(box), _dptr(pos, "float32", "pos"),
                                  _dptr(h, "float32", "h"), int(pos.shape[0]),
                                  axis.ctypes.data_as(ctypes.c_void_p),
                                  cofm.ctypes.data_as(ctypes.c_void_p), int(axis.shape[0]),
                                  ctypes.byref(n), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return int(n.value)


def copy_pairs(ctx, nlos, npairs, sorted=True):
    """Pair lists of the last search as CSR numpy arrays (offsets, part, dr2)."""
    off = np.zeros(nlos + 1, dtype=np.int64)
    part = np.zeros(max(npairs, 1), dtype=np.int32)
    dr2 = np.zeros(max(npairs, 1), dtype=np.float64)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_copy_pairs(ctx.handle, off.ctypes.data_as(ctypes.c_void_p),
                          part.ctypes.data_as(ctypes.c_void_p),
                          dr2.ctypes.data_as(ctypes.c_void_p), int(bool(sorted)), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return off, part[:npairs], dr2[:npairs]


def particle_interpolate_noalloc(compute_tau, nbins, kernel, box, velfac, atime, lam, gamma,
                                 fosc, amumass, tautail, pos, vel, dens, temp, h, axis, cofm,
                                 out=None, precision="fp64"):
    """`_Particle_Interpolate` through the entry point that allocates no device memory.

    For callers that may not call cudaMalloc (their application owns the GPU's
    memory).  Scratch is a fixed 64 MiB array inside the library; limits: at
    most 8192 sightlines, about 5.4 million sightline-particle pairs, and nbins
    within the shared-memory capacity (include/fsg.h gives the figure for each
    form).  The call runs on the device that holds `pos`.  `out` (float64, on
    that device) is the only buffer the caller provides; allocate it up front
    if allocation is not allowed at call time."""
    import torch
    axis, cofm = _host_tables(axis, cofm)
    nlos = int(axis.shape[0])
    # the C side works on the current device: make it the one the data is on
    with torch.cuda.device(pos.device):
        if out is None:
            out = torch.empty((nlos, int(nbins)), dtype=torch.float64, device=pos.device)
        prec = _lib.make_options(precision).precision
        eb = _lib.errbuf()
        L = _lib.load()
        rc = L.fsg_particle_interpolate_noalloc(
            int(compute_tau), int(nbins), int(kernel), float(box), float(velfac), float(atime),
            float(lam), float(gamma), float(fosc), float(amumass), float(tautail),
            _dptr(pos, "float32", "pos"), _dptr(vel, "float32", "vel") if compute_tau else None,
            _dptr(dens, "float32", "dens"),
            _dptr(temp, "float32", "temp") if compute_tau else None,
            _dptr(h, "float32", "h"), int(pos.shape[0]), axis.ctypes.data_as(ctypes.c_void_p),
            cofm.ctypes.data_as(ctypes.c_void_p), nlos, _dptr(out, "float64", "out"), prec,
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out
