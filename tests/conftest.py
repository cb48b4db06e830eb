import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the libfsg kernels)")


def golden(name):
    with np.load(os.path.join(GOLDEN, name), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def ref():
    import oracle
    r = oracle.ref()
    if r is None:
        pytest.skip("reference sources not available on this machine")
    return r


@pytest.fixture(scope="session")
def impls(port):
    """The C restatement, plus the reference build where it exists."""
    import oracle
    out = [port]
    r = oracle.ref()
    if r is not None:
        out.append(r)
    return out


@pytest.fixture(scope="session")
def fsg():
    """libfsg built and a CUDA device present (gpu tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test collected on a machine without CUDA")
    from fake_spectra_gb300 import build, _lib
    build.build()
    _lib.load()
    return _lib


@pytest.fixture(scope="session")
def ctx(fsg):
    from fake_spectra_gb300 import _lib
    c = _lib.Context(0)
    yield c
    c.close()
