"""The argument checks of `_near_lines` (py_module.cpp:36-54) raise the
reference's exception classes before any GPU work."""
import numpy as np
import pytest

from fake_spectra_gb300._spectra_priv import _near_lines

POS = np.zeros((4, 3), np.float32)
HH = np.ones(4, np.float32)
AXIS = np.array([1, 2], np.int32)
COFM = np.zeros((2, 3))


def test_cofm_shape():
    with pytest.raises(ValueError, match="cofm must have dimensions"):
        _near_lines(10.0, POS, HH, AXIS, np.zeros((3, 3)))
    with pytest.raises(ValueError, match="cofm must have dimensions"):
        _near_lines(10.0, POS, HH, AXIS, np.zeros(6))


def test_table_dtypes_are_value_errors():
    with pytest.raises(ValueError, match="64-bit float"):
        _near_lines(10.0, POS, HH, AXIS, COFM.astype(np.float32))
    with pytest.raises(ValueError, match="32-bit integer"):
        _near_lines(10.0, POS, HH, AXIS.astype(np.int64), COFM)


def test_particle_dtypes_are_type_errors():
    with pytest.raises(TypeError, match="32-bit float"):
        _near_lines(10.0, POS.astype(np.float64), HH, AXIS, COFM)
    with pytest.raises(TypeError, match="32-bit float"):
        _near_lines(10.0, POS, HH.astype(np.float64), AXIS, COFM)
