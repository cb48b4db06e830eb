"""Drop-in replacement for the reference extension module ``fake_spectra._spectra_priv``.

``_near_lines`` keeps the reference's arguments, checks and result
(py_module.cpp:25-99, Py_near_lines): the ascending int32 indices of the
particles within their smoothing length of any sightline.

``_rescale_mean_flux`` (py_module.cpp:262-282, Py_mean_flux) returns the
Newton-Raphson scale of tau that gives the desired mean flux.

``_Particle_Interpolate`` keeps the reference's positional arguments, argument
checks, exception classes and return value (py_module.cpp:103-233,
Py_Particle_Interpolation): a new float64 array of shape (NumLos, nbins)
holding tau (compute_tau=1) or the column density (compute_tau=0).  The work
runs on the GPU through libfsg's C ABI; there is no CPU path.

Differences from the reference, all for inputs on which the reference has
undefined behaviour: axis values outside {1, 2, 3}, non-finite sightline
positions, pos/vel arrays that are not (Npart, 3), and a non-positive box size
raise ValueError.  The Voronoi-mesh kernel (kernel=2) runs in the FP64 form
whatever precision is asked for, and a cell whose points along a sightline are
not contiguous (where the reference calls exit) raises ValueError.
"""
import ctypes

import numpy as np

from . import _lib

_ATTR_MSG = ("Incorrect arguments: use compute_tau, nbins, boxsize, velfac, atime, lambda, gamma, "
             "fosc, species mass (amu), min. tau,  pos, vel, dens, temp, h, axis, cofm\n")


def _as_int(v):
    # PyArg_ParseTuple "i": integers (or __index__), not floats
    if isinstance(v, (bool, int, np.integer)):
        return int(v)
    if isinstance(v, (float, np.floating)):
        raise AttributeError(_ATTR_MSG)
    try:
        return int(v.__index__())
    except Exception:
        raise AttributeError(_ATTR_MSG) from None


def _as_float(v):
    # "d": floats or integers
    try:
        return float(v)
    except Exception:
        raise AttributeError(_ATTR_MSG) from None


def _to_numpy(a):
    if isinstance(a, np.ndarray):
        return a
    # torch tensors are accepted as well (moved to host memory)
    if hasattr(a, "detach") and hasattr(a, "cpu") and hasattr(a, "numpy"):
        return a.detach().cpu().numpy()
    raise AttributeError(_ATTR_MSG)


def check_arrays(compute_tau, pos, vel, dens, temp, h, axis, cofm):
    """The dtype and shape checks of py_module.cpp:121-151, in the same order."""
    for a in (pos, vel, dens, temp, h):
        if a.dtype != np.float32:
            raise TypeError("One of the data arrays does not have 32-bit float type\n")
    if cofm.dtype != np.float64:
        raise TypeError("Sightline positions must have 64-bit float type\n")
    if axis.dtype != np.int32:
        raise TypeError("Axis must be a 32-bit integer\n")
    npart = pos.shape[0] if pos.ndim >= 1 else 0
    if dens.ndim < 1 or h.ndim < 1 or npart != dens.shape[0] or npart != h.shape[0]:
        raise ValueError(" Dens, pos and h must have the same length\n")
    if cofm.ndim != 2 or axis.ndim < 1 or cofm.shape[0] != axis.shape[0] or cofm.shape[1] != 3:
        raise ValueError("cofm must have dimensions (np.size(axis),3) \n")
    if pos.ndim != 2 or pos.shape[1] != 3:
        raise ValueError("pos must have dimensions (Npart, 3)\n")
    if compute_tau:
        if vel.ndim != 2 or vel.shape[0] != npart or vel.shape[1] != 3:
            raise ValueError("vel must have dimensions (Npart, 3)\n")
        if temp.ndim < 1 or temp.shape[0] != npart:
            raise ValueError("temp must have the same length as dens\n")
    return npart, int(axis.shape[0])


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _Particle_Interpolate(*args, precision="fp64", threads=0, persistent=-1, chunk=0, tune=0,
                          records=-1):
    """tau or colden along every sightline; see the module docstring.  The keyword
    arguments select the form (precision) and the deposit launch (FP32 form:
    left at 0/-1 the autotuner picks it)."""
    if len(args) != 18:
        raise AttributeError(_ATTR_MSG)
    compute_tau, nbins, kernel = (_as_int(v) for v in args[:3])
    box, velfac, atime, lam, gamma, fosc, amumass, tautail = (_as_float(v) for v in args[3:11])
    pos, vel, dens, temp, h, axis, cofm = (_to_numpy(a) for a in args[11:18])
    npart, nlos = check_arrays(compute_tau, pos, vel, dens, temp, h, axis, cofm)
    if nbins < 0:
        raise ValueError("negative dimensions are not allowed")
    pos = np.ascontiguousarray(pos)
    dens = np.ascontiguousarray(dens)
    h = np.ascontiguousarray(h)
    axis = np.ascontiguousarray(axis)
    cofm = np.ascontiguousarray(cofm)
    if compute_tau:
        vel = np.ascontiguousarray(vel)
        temp = np.ascontiguousarray(temp)
    out = np.zeros((nlos, nbins), dtype=np.float64)
    if nlos == 0 or nbins == 0:
        return out
    L = _lib.load()
    opt = _lib.make_options(precision, threads, persistent, chunk=chunk, tune=tune,
                            records=records)
    eb = _lib.errbuf()
    rc = L.fsg_particle_interpolate(int(compute_tau), nbins, kernel, box, velfac, atime, lam,
                                    gamma, fosc, amumass, tautail, _ptr(pos),
                                    _ptr(vel) if compute_tau else None, _ptr(dens),
                                    _ptr(temp) if compute_tau else None, _ptr(h), npart,
                                    _ptr(axis), _ptr(cofm), nlos, _ptr(out), ctypes.byref(opt), eb,
                                    512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out


def _near_lines(*args):
    """Indices of the particles near any sightline; see the module docstring."""
    if len(args) != 5:
        raise TypeError("_near_lines takes (box, pos, hh, axis, cofm)")
    box = _as_float(args[0])
    pos, hh, axis, cofm = (_to_numpy(a) for a in args[1:5])
    # the checks of py_module.cpp:36-54, in the same order and classes
    if cofm.ndim < 2 or axis.ndim < 1:
        raise ValueError("cofm must have dimensions (np.size(axis),3) \n")
    if cofm.shape[0] != axis.shape[0] or cofm.shape[1] != 3:
        raise ValueError("cofm must have dimensions (np.size(axis),3) \n")
    if cofm.dtype != np.float64 or axis.dtype != np.int32:
        raise ValueError("cofm must have 64-bit float type and axis must be a 32-bit integer\n")
    if pos.dtype != np.float32 or hh.dtype != np.float32:
        raise TypeError("pos and h must have 32-bit float type\n")
    npart = pos.shape[0] if pos.ndim >= 1 else 0
    if pos.ndim != 2 or pos.shape[1] != 3:
        raise ValueError("pos must have dimensions (Npart, 3)\n")
    if hh.ndim < 1 or hh.shape[0] < npart:
        raise ValueError("h must have at least Npart entries\n")
    pos = np.ascontiguousarray(pos)
    hh = np.ascontiguousarray(hh)
    axis = np.ascontiguousarray(axis)
    cofm = np.ascontiguousarray(cofm)
    nlos = int(axis.shape[0])
    out = np.empty(max(npart, 1), dtype=np.int32)
    if npart == 0 or nlos == 0:
        return out[:0].copy()
    n = ctypes.c_int64(0)
    eb = _lib.errbuf()
    L = _lib.load()
    rc = L.fsg_near_lines(box, _ptr(pos), _ptr(hh), npart, _ptr(axis), _ptr(cofm), nlos,
                          _ptr(out), ctypes.byref(n), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out[:n.value].copy()


_MF_MSG = ("Incorrect arguments: use tau (array), mean_flux_desired (double), nbins (int), "
           "tol (double), thresh (double)\n")


def _rescale_mean_flux(*args):
    """Scale factor of tau with mean(exp(-scale tau)) = mean_flux_desired."""
    if len(args) != 5 or not isinstance(args[0], np.ndarray):
        raise AttributeError(_MF_MSG)
    tau = args[0]
    try:
        mfd = float(args[1])
        nbins = int(args[2].__index__()) if not isinstance(args[2], (int, np.integer)) \
            else int(args[2])
        tol, thresh = float(args[3]), float(args[4])
    except Exception:
        raise AttributeError(_MF_MSG) from None
    if tau.dtype != np.float64:
        raise TypeError("Optical depth must have 64-bit float type\n")
    tau = np.ascontiguousarray(tau).reshape(-1)
    if nbins < 0 or nbins > tau.size:
        raise ValueError("nbins must be between 0 and the size of tau\n")
    out = ctypes.c_double(0.0)
    eb = _lib.errbuf()
    rc = _lib.load().fsg_rescale_mean_flux(_ptr(tau), nbins, mfd, tol, thresh,
                                           ctypes.byref(out), eb, 512)
    _lib.raise_for(rc, eb.value.decode(errors="replace"))
    return out.value
