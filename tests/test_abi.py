"""Host-side checks that need no GPU: the C ABI library loads and exports every
entry point declared in include/fsg.h, and the drop-in boundary raises the
reference's exception classes (py_module.cpp:117-151) before any device work."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from fake_spectra_gb300 import build, _lib
    path = build.build()
    return ctypes.CDLL(path)


def header_symbols():
    text = open(os.path.join(ROOT, "include", "fsg.h")).read()
    # declarations: "<type> [*]fsg_name(" at the start of a line
    decl = re.compile(r"^(?:const\s+)?[a-z_0-9]+\s*\*?\s*(fsg_[a-z_0-9]+)\s*\(", re.M)
    return sorted(set(decl.findall(text)))


def test_header_declares_entry_points():
    syms = header_symbols()
    for s in ("fsg_particle_interpolate", "fsg_particle_interpolate_device",
              "fsg_build_pairs_device", "fsg_copy_pairs", "fsg_context_create"):
        assert s in syms


def test_library_exports_header(lib):
    for s in header_symbols():
        assert hasattr(lib, s), "libfsg.so does not export %s" % s


def test_python_binding_covers_header():
    from fake_spectra_gb300 import _lib
    assert sorted(_lib.EXPORTS) == header_symbols()


def test_version(lib):
    lib.fsg_version.restype = ctypes.c_char_p
    assert lib.fsg_version().startswith(b"fsg")


def _args(n=10, nlos=2, nbins=16):
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 100, (n, 3)).astype(np.float32)
    vel = np.zeros((n, 3), np.float32)
    dens = np.ones(n, np.float32)
    temp = np.full(n, 1e4, np.float32)
    h = np.full(n, 5, np.float32)
    axis = np.array([1] * nlos, np.int32)
    cofm = rng.uniform(0, 100, (nlos, 3))
    return [1, nbins, 1, 100.0, 0.1, 0.25, 1215.67e-8, 6.265e8, 0.4164, 1.00794, 1e-7,
            pos, vel, dens, temp, h, axis, cofm]


def call(args):
    from fake_spectra_gb300._spectra_priv import _Particle_Interpolate
    return _Particle_Interpolate(*args)


@pytest.mark.parametrize("i", [11, 12, 13, 14, 15])
def test_float32_type_errors(i):
    a = _args()
    a[i] = a[i].astype(np.float64)
    with pytest.raises(TypeError, match="32-bit float"):
        call(a)


def test_cofm_type_error():
    a = _args()
    a[17] = a[17].astype(np.float32)
    with pytest.raises(TypeError, match="64-bit float"):
        call(a)


def test_axis_type_error():
    a = _args()
    a[16] = a[16].astype(np.int64)
    with pytest.raises(TypeError, match="32-bit integer"):
        call(a)


def test_length_mismatch():
    a = _args()
    a[13] = a[13][:-1]
    with pytest.raises(ValueError, match="same length"):
        call(a)
    a = _args()
    a[15] = a[15][:-1]
    with pytest.raises(ValueError, match="same length"):
        call(a)


def test_cofm_shape():
    a = _args()
    a[16] = a[16][:1]
    with pytest.raises(ValueError, match="cofm must have dimensions"):
        call(a)
    a = _args()
    a[17] = np.zeros((2, 2))
    with pytest.raises(ValueError, match="cofm must have dimensions"):
        call(a)


def test_bad_argument_kinds():
    a = _args()
    a[1] = 16.0          # nbins must be an int, as PyArg_ParseTuple "i" demands
    with pytest.raises(AttributeError):
        call(a)
    a = _args()
    a[11] = a[11].tolist()   # arrays must be arrays
    with pytest.raises(AttributeError):
        call(a)
    with pytest.raises(AttributeError):
        call(_args()[:-1])


def test_axis_out_of_range(lib):
    a = _args()
    a[16] = np.array([1, 4], np.int32)
    with pytest.raises(ValueError, match="axes must be 1, 2 or 3"):
        call(a)


def test_voronoi_rejected_where_unsupported(lib):
    """kernel=2 runs through the interpolation entry points (GPU tests); the
    no-allocation entry point rejects it before touching the device."""
    import ctypes
    from fake_spectra_gb300 import _lib
    a = _args()
    ptr = lambda x: np.ascontiguousarray(x).ctypes.data_as(ctypes.c_void_p)
    out = np.zeros((2, 16))
    eb = _lib.errbuf()
    rc = _lib.load().fsg_particle_interpolate_noalloc(
        1, 16, 2, *[float(v) for v in a[3:11]], ptr(a[11]), ptr(a[12]), ptr(a[13]), ptr(a[14]),
        ptr(a[15]), len(a[11]), ptr(a[16]), ptr(a[17]), len(a[16]), ptr(out), 0, None, eb, 512)
    with pytest.raises(NotImplementedError):
        _lib.raise_for(rc, eb.value.decode())


def test_empty_outputs_need_no_device():
    a = _args(nlos=0)
    a[16] = np.zeros(0, np.int32)
    a[17] = np.zeros((0, 3))
    out = call(a)
    assert out.shape == (0, 16) and out.dtype == np.float64
    a = _args(nbins=0)
    out = call(a)
    assert out.shape == (2, 0)


def test_struct_layouts(tmp_path):
    """The ctypes mirrors of fsg_options, fsg_stats and fsg_line have the C
    header's size and field offsets."""
    import shutil
    import subprocess
    from fake_spectra_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"fsg_options": _lib.Options, "fsg_stats": _lib.Stats, "fsg_line": _lib.Line}
    rename = {"lambda_": "lambda"}
    src = ['#include <stddef.h>', '#include <stdio.h>', '#include "fsg.h"', "int main(void) {"]
    for cname, cls in structs.items():
        src.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in cls._fields_:
            cf = rename.get(f, f)
            src.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, cf))
    src.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), "-o", exe, str(c)], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for f, _ in cls._fields_:
            assert got[(cname, f)] == getattr(cls, f).offset, (cname, f)
