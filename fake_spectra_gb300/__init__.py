"""fake_spectra_gb300: fake_spectra's sightline interpolation (`_Particle_Interpolate`)
as hand-written CUDA for GB300 (sm_103a), behind a C ABI (include/fsg.h).

* ``fake_spectra_gb300._spectra_priv._Particle_Interpolate`` -- the drop-in for
  the reference extension call (numpy in, numpy out).
* ``fake_spectra_gb300.interp`` -- the same work on device-resident tensors.
* ``fake_spectra_gb300.synth`` -- seeded synthetic snapshots for the benchmark
  workloads.
* ``fake_spectra_gb300.build`` -- builds libfsg.so in-tree.
"""
from . import _lib  # noqa: F401

__all__ = ["_lib"]
