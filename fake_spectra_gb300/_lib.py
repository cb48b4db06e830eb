"""ctypes binding of libfsg.so (the C ABI in include/fsg.h).

The library is built in-tree by ``fake_spectra_gb300.build.build()``.  There is
no CPU fallback: if the library is missing, loading raises.
"""
import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libfsg.so")

FSG_OK = 0
FSG_ERR_VALUE = 1
FSG_ERR_TYPE = 2
FSG_ERR_MEMORY = 3
FSG_ERR_CUDA = 4
FSG_ERR_NOT_IMPLEMENTED = 5
FSG_ERR_DEVICE = 6

FSG_PREC_FP64 = 0
FSG_PREC_FP32 = 1

# Names exported by libfsg.so, one per declaration in include/fsg.h.
EXPORTS = (
    "fsg_version",
    "fsg_measure_fma_peak",
    "fsg_context_create",
    "fsg_context_destroy",
    "fsg_context_set_stream",
    "fsg_context_stats",
    "fsg_default_context_stats",
    "fsg_particle_interpolate",
    "fsg_particle_interpolate_device",
    "fsg_spectra_batch_device",
    "fsg_tau_backward_device",
    "fsg_tau_backward_reuse_device",
    "fsg_context_search_generation",
    "fsg_build_pairs_device",
    "fsg_copy_pairs",
    "fsg_particle_interpolate_noalloc",
    "fsg_near_lines",
    "fsg_near_lines_device",
    "fsg_colden_channels_device",
    "fsg_rescale_mean_flux",
    "fsg_mean_flux_scale_device",
    "fsg_mean_flux_device",
    "fsg_flux_exp_device",
    "fsg_flux_histogram_device",
    "fsg_flux_power_device",
    "fsg_tune_cache_file",
    "fsg_tune_cache_lookup",
    "fsg_tune_cache_store",
    "fsg_tune_cache_clear",
)

_c_int = ctypes.c_int
_c_i64 = ctypes.c_int64
_c_i32 = ctypes.c_int32
_c_d = ctypes.c_double
_p = ctypes.c_void_p
_c_size = ctypes.c_size_t


class Options(ctypes.Structure):
    _fields_ = [("precision", _c_int), ("threads", _c_int), ("persistent", _c_int),
                ("count_work", _c_int), ("no_far_tiles", _c_int), ("chunk", _c_int),
                ("tune", _c_int), ("records", _c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("npairs", _c_i64), ("gpu_launches", _c_i64), ("fallback_lines", _c_i32),
                ("reserved", _c_i32), ("ms_search", _c_d), ("ms_deposit", _c_d),
                ("evals_core", _c_i64), ("evals_wing", _c_i64), ("evals_other", _c_i64),
                ("pixels", _c_i64), ("evals_wing_multipole", _c_i64),
                ("samples_wing_path", _c_i64), ("samples_core_path", _c_i64),
                ("samples_mixed_path", _c_i64), ("launch_threads", _c_i32),
                ("launch_chunk", _c_i32), ("launch_persistent", _c_i32),
                ("launch_tuned", _c_i32), ("tune_ran", _c_i32), ("tune_candidates", _c_i32),
                ("tune_sample_lines", _c_i32), ("launch_records", _c_i32),
                ("tune_ms_default", _c_d), ("tune_ms_best", _c_d), ("ms_h2d", _c_d),
                ("ms_d2h", _c_d), ("ms_flux", _c_d), ("search_reused", _c_i32)]


class TuneKey(ctypes.Structure):
    _fields_ = [(n, _c_i32) for n in ("sms", "precision", "compute_tau", "kernel", "nbins_b",
                                      "pairs_med_b", "pairs_p99_b", "lines_b", "damp_b")]


class TuneEntry(ctypes.Structure):
    _fields_ = [("threads", _c_i32), ("chunk", _c_i32), ("persistent", _c_i32),
                ("records", _c_i32), ("candidates", _c_i32), ("sample_lines", _c_i32),
                ("ms_default", _c_d), ("ms_best", _c_d)]


class Line(ctypes.Structure):
    _fields_ = [("lambda_", _c_d), ("gamma", _c_d), ("fosc", _c_d), ("amumass", _c_d),
                ("dens", _p), ("tau", _p), ("colden", _p)]


class FsgError(RuntimeError):
    """A CUDA-side failure reported by libfsg."""


class FsgDeviceError(FsgError):
    """A kernel reported an internal limit (FSG_ERR_DEVICE)."""


def raise_for(code, msg):
    """Map an fsg_status to the exception class the reference raises."""
    if code == FSG_OK:
        return
    text = msg or "fsg error %d" % code
    if code == FSG_ERR_VALUE:
        raise ValueError(text)
    if code == FSG_ERR_TYPE:
        raise TypeError(text)
    if code == FSG_ERR_MEMORY:
        raise MemoryError(text)
    if code == FSG_ERR_NOT_IMPLEMENTED:
        raise NotImplementedError(text)
    if code == FSG_ERR_DEVICE:
        raise FsgDeviceError(text)
    raise FsgError(text)


_lib = None
_lock = threading.Lock()

_INTERP_ARGS = [_c_int, _c_int, _c_int] + [_c_d] * 8 + [_p] * 5 + [_c_i64, _p, _p, _c_i32, _p,
                                                                     _p, _p, _c_size]


def load(path=None):
    """Load libfsg.so (once).  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise ImportError("libfsg.so is not built (%s); run "
                              "fake_spectra_gb300.build.build() on a machine with nvcc" % path)
        L = ctypes.CDLL(path)
        L.fsg_version.restype = ctypes.c_char_p
        L.fsg_measure_fma_peak.argtypes = [_c_int, ctypes.POINTER(_c_d), _p, _c_size]
        L.fsg_context_create.argtypes = [_c_int, ctypes.POINTER(_p), _p, _c_size]
        L.fsg_context_destroy.argtypes = [_p]
        L.fsg_context_destroy.restype = None
        L.fsg_context_set_stream.argtypes = [_p, _p]
        L.fsg_context_stats.argtypes = [_p, ctypes.POINTER(Stats)]
        L.fsg_default_context_stats.argtypes = [ctypes.POINTER(Stats)]
        L.fsg_particle_interpolate.argtypes = _INTERP_ARGS
        L.fsg_particle_interpolate_device.argtypes = [_p] + _INTERP_ARGS
        L.fsg_spectra_batch_device.argtypes = ([_p, _c_int, _c_int] + [_c_d] * 4 + [_p] * 4 +
                                               [_c_i64, _p, _p, _c_i32, _c_int,
                                                ctypes.POINTER(Line), _p, _p, _c_size])
        L.fsg_tau_backward_device.argtypes = ([_p, _c_int, _c_int] + [_c_d] * 8 + [_p] * 5 +
                                              [_c_i64, _p, _p, _c_i32, _p, _p, _p, _p, _p,
                                               _c_size])
        L.fsg_tau_backward_reuse_device.argtypes = ([_p, ctypes.c_uint64, _c_int, _c_int] +
                                                    [_c_d] * 8 + [_p] * 5 +
                                                    [_c_i64, _p, _p, _c_i32, _p, _p, _p, _p,
                                                     _p, _c_size])
        L.fsg_context_search_generation.argtypes = [_p, ctypes.POINTER(ctypes.c_uint64)]
        L.fsg_build_pairs_device.argtypes = [_p, _c_d, _p, _p, _c_i64, _p, _p, _c_i32,
                                             ctypes.POINTER(_c_i64), _p, _c_size]
        L.fsg_copy_pairs.argtypes = [_p, _p, _p, _p, _c_int, _p, _c_size]
        L.fsg_particle_interpolate_noalloc.argtypes = ([_c_int, _c_int, _c_int] + [_c_d] * 8 +
                                                       [_p] * 5 + [_c_i64, _p, _p, _c_i32, _p,
                                                                   _c_int, _p, _p, _c_size])
        L.fsg_near_lines.argtypes = [_c_d, _p, _p, _c_i64, _p, _p, _c_i32, _p,
                                     ctypes.POINTER(_c_i64), _p, _c_size]
        L.fsg_near_lines_device.argtypes = [_p, _c_d, _p, _p, _c_i64, _p, _p, _c_i32, _p,
                                            ctypes.POINTER(_c_i64), _p, _c_size]
        L.fsg_colden_channels_device.argtypes = ([_p, _c_int, _c_int, _c_d, _c_d, _p, _p, _c_i64,
                                                  _p, _p, _c_i32, _c_int, _p, _p, _p, _p,
                                                  _c_size])
        L.fsg_rescale_mean_flux.argtypes = [_p, _c_i64, _c_d, _c_d, _c_d, ctypes.POINTER(_c_d),
                                            _p, _c_size]
        L.fsg_mean_flux_scale_device.argtypes = [_p, _p, _c_i64, _c_d, _c_d, _c_d,
                                                 ctypes.POINTER(_c_d), _p, _c_size]
        L.fsg_mean_flux_device.argtypes = [_p, _p, _c_i64, _c_d, ctypes.POINTER(_c_d), _p,
                                           _c_size]
        L.fsg_flux_exp_device.argtypes = [_p, _p, _c_i64, _p, _p, _c_size]
        L.fsg_flux_histogram_device.argtypes = [_p, _p, _c_i64, _c_d, _p, _c_int, _p, _p,
                                                _c_size]
        L.fsg_flux_power_device.argtypes = [_p, _p, _c_i64, _c_i64, _c_d, _c_d, _c_d, _p, _p,
                                            _c_size]
        L.fsg_tune_cache_file.argtypes = [ctypes.c_char_p, _p, _c_size]
        L.fsg_tune_cache_lookup.argtypes = [ctypes.POINTER(TuneKey), ctypes.POINTER(TuneEntry)]
        L.fsg_tune_cache_store.argtypes = [ctypes.POINTER(TuneKey), ctypes.POINTER(TuneEntry),
                                           _p, _c_size]
        L.fsg_tune_cache_clear.argtypes = []
        L.fsg_tune_cache_clear.restype = None
        _lib = L
        return L


def errbuf():
    return ctypes.create_string_buffer(512)


def make_options(precision="fp64", threads=0, persistent=-1, count_work=False, far_tiles=True,
                 chunk=0, tune=0, records=-1):
    """fsg_options.  threads/chunk 0 and persistent/records -1 leave the launch to
    the autotuner (FP32 form; tune 0 = cached choice, 1 = time again, -1 =
    library defaults) or to the library defaults (FP64 form)."""
    o = Options()
    o.chunk = int(chunk)
    o.records = int(records)
    o.tune = int(tune)
    o.count_work = int(bool(count_work))
    o.no_far_tiles = int(not far_tiles)
    if precision in ("fp64", FSG_PREC_FP64):
        o.precision = FSG_PREC_FP64
    elif precision in ("fp32", FSG_PREC_FP32):
        o.precision = FSG_PREC_FP32
    else:
        raise ValueError("precision must be 'fp64' or 'fp32'")
    o.threads = int(threads)
    o.persistent = int(persistent)
    return o


class Context:
    """An fsg_context: one device, one stream, a cached device workspace."""

    def __init__(self, device=0):
        L = load()
        h = _p()
        eb = errbuf()
        raise_for(L.fsg_context_create(int(device), ctypes.byref(h), eb, 512), eb.value.decode())
        self._h = h
        self._lib = L
        self.device = int(device)

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr):
        """Run on a cudaStream_t handle; 0/None is the CUDA default stream."""
        self._lib.fsg_context_set_stream(self._h, _p(stream_ptr) if stream_ptr else None)

    def stats(self):
        s = Stats()
        self._lib.fsg_context_stats(self._h, ctypes.byref(s))
        return _stats_dict(s)

    def search_generation(self):
        """The context's sightline-search generation (grows with every search)."""
        g = ctypes.c_uint64(0)
        if load().fsg_context_search_generation(self.handle, ctypes.byref(g)) != FSG_OK:
            raise RuntimeError("fsg_context_search_generation failed")
        return int(g.value)

    def close(self):
        if self._h:
            self._lib.fsg_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def default_context_stats():
    """Statistics of the library-owned context behind the host-pointer entry
    points (the last fsg_particle_interpolate call on the current device)."""
    s = Stats()
    L = load()
    if L.fsg_default_context_stats(ctypes.byref(s)) != FSG_OK:
        return None
    return _stats_dict(s)


def _stats_dict(s):
    return {"npairs": int(s.npairs), "gpu_launches": int(s.gpu_launches),
            "fallback_lines": int(s.fallback_lines), "ms_search": float(s.ms_search),
            "ms_deposit": float(s.ms_deposit), "evals_core": int(s.evals_core),
            "evals_wing": int(s.evals_wing), "evals_other": int(s.evals_other),
            "pixels": int(s.pixels), "evals_wing_multipole": int(s.evals_wing_multipole),
            "samples_wing_path": int(s.samples_wing_path),
            "samples_core_path": int(s.samples_core_path),
            "samples_mixed_path": int(s.samples_mixed_path),
            "launch": {"threads": int(s.launch_threads), "chunk": int(s.launch_chunk),
                       "persistent": int(s.launch_persistent),
                       "records": int(s.launch_records), "tuned": bool(s.launch_tuned)},
            "tune": {"ran": bool(s.tune_ran), "candidates": int(s.tune_candidates),
                     "sample_lines": int(s.tune_sample_lines),
                     "ms_default": float(s.tune_ms_default),
                     "ms_best": float(s.tune_ms_best)},
            "ms_h2d": float(s.ms_h2d), "ms_d2h": float(s.ms_d2h), "ms_flux": float(s.ms_flux),
            "search_reused": int(s.search_reused)}


def fma_peak_tflops(precision="fp32"):
    """Peak FMA throughput of the current GPU (TFLOP/s), own microbenchmark."""
    L = load()
    v = _c_d(0.0)
    eb = errbuf()
    prec = FSG_PREC_FP64 if precision in ("fp64", FSG_PREC_FP64) else FSG_PREC_FP32
    raise_for(L.fsg_measure_fma_peak(prec, ctypes.byref(v), eb, 512), eb.value.decode())
    return float(v.value)


def tune_cache_file(path):
    """Name the autotuner's cache file (loaded now, appended to later); None/''
    keeps the cache in the process only."""
    L = load()
    eb = errbuf()
    raise_for(L.fsg_tune_cache_file(path.encode() if path else None, eb, 512),
              eb.value.decode())


def tune_cache_lookup(key):
    """The cached fsg_tune_entry of a TuneKey as a dict, or None."""
    e = TuneEntry()
    if not load().fsg_tune_cache_lookup(ctypes.byref(key), ctypes.byref(e)):
        return None
    return {f: getattr(e, f) for f, _ in TuneEntry._fields_}


def tune_cache_store(key, threads, chunk, persistent, ms_default=0.0, ms_best=0.0,
                     candidates=0, sample_lines=0, records=0):
    e = TuneEntry(threads, chunk, persistent, records, candidates, sample_lines, ms_default,
                  ms_best)
    eb = errbuf()
    raise_for(load().fsg_tune_cache_store(ctypes.byref(key), ctypes.byref(e), eb, 512),
              eb.value.decode())


def tune_cache_clear():
    load().fsg_tune_cache_clear()
