"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle.

Two libraries, both used only as checkers (tests/, ``__graft_entry__.smoke()``)
and as the timed CPU baseline in ``bench.py``; the product package never
imports this module.

* ``port()``  -- ``oracle/_build/libfsgoracle.so``, this project's C restatement
  of the reference path (``oracle/fsg_oracle.c``), built by
  ``oracle/build_oracle.sh``.  Available wherever gcc is.
* ``ref()``   -- ``oracle/_ref/libfsref.so``, the reference's own C++ sources
  compiled unmodified (``oracle/build_ref.sh``).  Only exists where the
  reference checkout exists; ``ref()`` returns None elsewhere.

Both expose the same numpy-level helpers through :class:`Oracle`.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libfsgoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfsref.so")

_c_int = ctypes.c_int
_c_ll = ctypes.c_longlong
_c_d = ctypes.c_double
_c_f = ctypes.c_float
_p = ctypes.c_void_p


def build_port(force=False):
    """Compile the C restatement if its library is missing or older than its
    source (or force)."""
    src = os.path.join(HERE, "fsg_oracle.c")
    stale = os.path.exists(PORT_SO) and os.path.getmtime(PORT_SO) < os.path.getmtime(src)
    if force or stale or not os.path.exists(PORT_SO):
        subprocess.check_call(["sh", os.path.join(HERE, "build_oracle.sh")],
                              stdout=subprocess.DEVNULL)
    return PORT_SO


def reference_root():
    """Where the reference checkout is: $FSG_REFERENCE_ROOT, else a directory
    named ``reference`` beside this repository.  Returns None when neither
    holds the reference's ``fake_spectra`` sources."""
    cands = [os.environ.get("FSG_REFERENCE_ROOT"),
             os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isfile(os.path.join(c, "fake_spectra", "part_int.cpp")):
            return c
    return None


def build_ref(reference_root_dir=None, force=False):
    """Compile the unmodified reference sources, when they are present."""
    reference_root_dir = reference_root_dir or reference_root()
    if not reference_root_dir or not os.path.isdir(os.path.join(reference_root_dir,
                                                                "fake_spectra")):
        return None
    if force or not os.path.exists(REF_SO):
        subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh"),
                               reference_root_dir], stdout=subprocess.DEVNULL)
    return REF_SO


def _ptr(a):
    return a.ctypes.data_as(_p)


class Oracle:
    """numpy wrappers over one of the two oracle libraries (prefix fsgo_ or fsr_)."""

    def __init__(self, path, prefix):
        self.path = path
        self.prefix = prefix
        self.lib = ctypes.CDLL(path)
        L = self.lib
        f = self._fn
        f("particle_interpolate").argtypes = [_c_int, _c_int, _c_int] + [_c_d] * 8 + \
            [_p] * 5 + [_c_ll, _p, _p, _c_int, _p] + ([_p] if prefix == "fsgo_" else [])
        f("particle_interpolate").restype = _c_int
        f("near_particles").argtypes = [_p, _p, _c_ll, _p, _p, _c_int, _c_d, _p, _p, _p, _c_ll]
        f("near_particles").restype = _c_ll
        f("near_lines").argtypes = [_p, _p, _c_int, _c_d, _p, _c_f, _p, _p, _c_int]
        f("near_lines").restype = _c_int
        self.has_voigt = hasattr(L, prefix + "voigt") or hasattr(L, prefix + "profile")
        vname = "voigt" if prefix == "fsgo_" else "profile"
        f(vname).argtypes = [_c_d, _c_d]
        f(vname).restype = _c_d
        self._voigt = f(vname)
        for name in ("sph_cubic_kernel", "sph_quintic_kernel"):
            f(name).argtypes = [_c_d]
            f(name).restype = _c_d
        f("tau_kern_outer").argtypes = [_c_d, _c_d, _c_d, _c_d, _c_int, _c_d, _c_d]
        f("tau_kern_outer").restype = _c_d
        tail = [_p] if prefix == "fsgo_" else []
        f("add_tau_particle").argtypes = [_c_d] * 7 + [_c_int, _c_d, _p, _c_int, _c_d] + \
            [_c_f] * 5 + tail
        f("add_tau_particle").restype = None
        f("add_colden_particle").argtypes = [_c_d] * 7 + [_c_int, _c_d, _p, _c_int, _c_d] + \
            [_c_f] * 3
        f("add_colden_particle").restype = None
        if prefix == "fsgo_":
            L.fsgo_set_threads.argtypes = [_c_int]
            L.fsgo_get_threads.restype = _c_int
            L.fsgo_faddeeva.argtypes = [_c_d, _c_d, _p, _p]
            L.fsgo_dawson.argtypes = [_c_d]
            L.fsgo_dawson.restype = _c_d
            L.fsgo_kern_frac.argtypes = [_c_int, _c_d, _c_d, _c_d, _c_d, _c_d]
            L.fsgo_kern_frac.restype = _c_d
            L.fsgo_assign_cells.argtypes = [_p, _p, _c_int, _c_int, _p, _c_d, _p]
            L.fsgo_assign_cells.restype = _c_int
            L.fsgo_particle_interpolate_timed.argtypes = [_c_int, _c_int, _c_int] + \
                [_c_d] * 8 + [_p] * 5 + [_c_ll, _p, _p, _c_int, _p, _p, _p]
            L.fsgo_particle_interpolate_timed.restype = _c_int
            L.fsgo_search_seconds.argtypes = [_p, _p, _c_ll, _p, _p, _c_int, _c_d, _p]
            L.fsgo_search_seconds.restype = _c_d
        else:
            L.fsr_sph_cubic_kern_frac.argtypes = [_c_d] * 5
            L.fsr_sph_cubic_kern_frac.restype = _c_d

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- full call -----------------------------------------------------------
    def particle_interpolate(self, compute_tau, nbins, kernel, box, velfac, atime, lam, gamma,
                             fosc, amumass, tautail, pos, vel, dens, temp, h, axis, cofm,
                             count_evals=False):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        dens = np.ascontiguousarray(dens, dtype=np.float32)
        temp = np.ascontiguousarray(temp, dtype=np.float32)
        h = np.ascontiguousarray(h, dtype=np.float32)
        axis = np.ascontiguousarray(axis, dtype=np.int32)
        cofm = np.ascontiguousarray(cofm, dtype=np.float64)
        nlos = int(axis.shape[0])
        out = np.zeros((nlos, int(nbins)), dtype=np.float64)
        args = [int(compute_tau), int(nbins), int(kernel), float(box), float(velfac),
                float(atime), float(lam), float(gamma), float(fosc), float(amumass),
                float(tautail), _ptr(pos), _ptr(vel), _ptr(dens), _ptr(temp), _ptr(h),
                int(pos.shape[0]), _ptr(axis), _ptr(cofm), nlos, _ptr(out)]
        ev = _c_ll(0)
        if self.prefix == "fsgo_":
            args.append(ctypes.cast(ctypes.byref(ev), _p) if count_evals else None)
        rc = self._fn("particle_interpolate")(*args)
        if rc != 0:
            raise RuntimeError("oracle particle_interpolate failed with %d" % rc)
        if count_evals:
            return out, int(ev.value)
        return out

    def particle_interpolate_timed(self, compute_tau, nbins, kernel, box, velfac, atime, lam,
                                   gamma, fosc, amumass, tautail, pos, vel, dens, temp, h, axis,
                                   cofm):
        """(out, search seconds, per-sightline deposit seconds of one thread); C
        restatement only."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        dens = np.ascontiguousarray(dens, dtype=np.float32)
        temp = np.ascontiguousarray(temp, dtype=np.float32)
        h = np.ascontiguousarray(h, dtype=np.float32)
        axis = np.ascontiguousarray(axis, dtype=np.int32)
        cofm = np.ascontiguousarray(cofm, dtype=np.float64)
        nlos = int(axis.shape[0])
        out = np.zeros((nlos, int(nbins)), dtype=np.float64)
        line_sec = np.zeros(max(nlos, 1), dtype=np.float64)
        ts = _c_d(0.0)
        rc = self.lib.fsgo_particle_interpolate_timed(
            int(compute_tau), int(nbins), int(kernel), float(box), float(velfac), float(atime),
            float(lam), float(gamma), float(fosc), float(amumass), float(tautail), _ptr(pos),
            _ptr(vel), _ptr(dens), _ptr(temp), _ptr(h), int(pos.shape[0]), _ptr(axis),
            _ptr(cofm), nlos, _ptr(out), ctypes.cast(ctypes.byref(ts), _p), _ptr(line_sec))
        if rc != 0:
            raise RuntimeError("oracle particle_interpolate failed with %d" % rc)
        return out, float(ts.value), line_sec[:nlos]

    def search_seconds(self, pos, h, axis, cofm, box):
        """(wall seconds, pairs) of the pair search alone; C restatement only."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        h = np.ascontiguousarray(h, dtype=np.float32)
        axis = np.ascontiguousarray(axis, dtype=np.int32)
        cofm = np.ascontiguousarray(cofm, dtype=np.float64)
        n = _c_ll(0)
        sec = self.lib.fsgo_search_seconds(_ptr(pos), _ptr(h), int(pos.shape[0]), _ptr(axis),
                                           _ptr(cofm), int(axis.shape[0]), float(box),
                                           ctypes.cast(ctypes.byref(n), _p))
        return float(sec), int(n.value)

    # -- pair lists ----------------------------------------------------------
    def near_particles(self, pos, h, axis, cofm, box):
        """CSR pair lists: (offsets[nlos+1], part[int32], dr2[float64])."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        h = np.ascontiguousarray(h, dtype=np.float32)
        axis = np.ascontiguousarray(axis, dtype=np.int32)
        cofm = np.ascontiguousarray(cofm, dtype=np.float64)
        nlos = int(axis.shape[0])
        counts = np.zeros(nlos, dtype=np.int64)
        fn = self._fn("near_particles")
        empty_i = np.zeros(1, dtype=np.int32)
        empty_d = np.zeros(1, dtype=np.float64)
        total = fn(_ptr(pos), _ptr(h), int(pos.shape[0]), _ptr(axis), _ptr(cofm), nlos,
                   float(box), _ptr(counts), _ptr(empty_i), _ptr(empty_d), 0)
        part = np.zeros(max(total, 1), dtype=np.int32)
        dr2 = np.zeros(max(total, 1), dtype=np.float64)
        if total > 0:
            fn(_ptr(pos), _ptr(h), int(pos.shape[0]), _ptr(axis), _ptr(cofm), nlos, float(box),
               _ptr(counts), _ptr(part), _ptr(dr2), total)
        off = np.zeros(nlos + 1, dtype=np.int64)
        np.cumsum(counts, out=off[1:])
        return off, part[:total], dr2[:total]

    def assign_cells(self, pos, part, axis, cofm3, box):
        """Voronoi segments (float32, 2 per cell) of one sightline's cells."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        part = np.ascontiguousarray(part, dtype=np.int32)
        cofm3 = np.ascontiguousarray(cofm3, dtype=np.float64)
        seg = np.zeros(2 * max(len(part), 1), dtype=np.float32)
        rc = self._fn("assign_cells")(_ptr(pos), _ptr(part), int(len(part)), int(axis),
                                      _ptr(cofm3), float(box), _ptr(seg))
        if rc != 0:
            raise RuntimeError("non-contiguous Voronoi cell (the reference exits here)")
        return seg[:2 * len(part)]

    def near_lines(self, cofm, axis, box, pos3, hh, cap=4096):
        cofm = np.ascontiguousarray(cofm, dtype=np.float64)
        axis = np.ascontiguousarray(axis, dtype=np.int32)
        pos3 = np.ascontiguousarray(pos3, dtype=np.float32)
        lines = np.zeros(cap, dtype=np.int32)
        dr2 = np.zeros(cap, dtype=np.float64)
        n = self._fn("near_lines")(_ptr(cofm), _ptr(axis), int(axis.shape[0]), float(box),
                                   _ptr(pos3), float(np.float32(hh)), _ptr(lines), _ptr(dr2), cap)
        return dict(zip(lines[:n].tolist(), dr2[:n].tolist()))

    # -- scalar pieces -------------------------------------------------------
    def voigt(self, u, a):
        return self._voigt(float(u), float(a))

    def sph_cubic_kernel(self, q):
        return self._fn("sph_cubic_kernel")(float(q))

    def sph_quintic_kernel(self, q):
        return self._fn("sph_quintic_kernel")(float(q))

    def sph_cubic_kern_frac(self, zlow, zhigh, smooth, dr2, zrange):
        if self.prefix == "fsgo_":
            return self.lib.fsgo_kern_frac(1, zlow, zhigh, smooth, dr2, zrange)
        return self.lib.fsr_sph_cubic_kern_frac(zlow, zhigh, smooth, dr2, zrange)

    def tau_kern_outer(self, btherm, vdr2, vsmooth, aa, kernel, vlow, vhigh):
        return self._fn("tau_kern_outer")(btherm, vdr2, vsmooth, aa, kernel, vlow, vhigh)

    def add_tau_particle(self, line, tau, dr2, dens, ppos, pvel, temp, smooth):
        """line = (lambda_cm, gamma, fosc, amumass, velfac, box, atime, kernel, tautail)."""
        lam, gamma, fosc, mass, velfac, box, atime, kernel, tautail = line
        args = [lam, gamma, fosc, mass, velfac, box, atime, int(kernel), tautail, _ptr(tau),
                int(tau.shape[0]), float(dr2), dens, ppos, pvel, temp, smooth]
        if self.prefix == "fsgo_":
            args.append(None)
        self._fn("add_tau_particle")(*args)

    def add_colden_particle(self, line, colden, dr2, dens, ppos, smooth):
        lam, gamma, fosc, mass, velfac, box, atime, kernel, tautail = line
        self._fn("add_colden_particle")(lam, gamma, fosc, mass, velfac, box, atime, int(kernel),
                                        tautail, _ptr(colden), int(colden.shape[0]), float(dr2),
                                        dens, ppos, smooth)

    def set_threads(self, n):
        if self.prefix == "fsgo_":
            self.lib.fsgo_set_threads(int(n))

    def get_threads(self):
        if self.prefix == "fsgo_":
            return int(self.lib.fsgo_get_threads())
        return os.cpu_count() or 1


_PORT = None
_REF = None


def port():
    """The C restatement (always available where gcc is)."""
    global _PORT
    if _PORT is None:
        _PORT = Oracle(build_port(), "fsgo_")
    return _PORT


def ref():
    """The unmodified reference build, or None when the reference is absent."""
    global _REF
    if _REF is None:
        path = REF_SO if os.path.exists(REF_SO) else build_ref()
        if path is None or not os.path.exists(path):
            return None
        _REF = Oracle(path, "fsr_")
    return _REF
