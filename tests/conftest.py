"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs
on the CPU.  The oracle (oracle/) is the checker: tests may call it, the
product never does."""
import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    """The oracle, built; where the reference checkout exists (never on the
    GPU machines) its own sources are built beside it for the pinning tests."""
    import oracle as o
    o.build(ref=True)
    return o


@pytest.fixture(scope="session")
def pkg():
    return importlib.import_module("3dcompactsolver_gb300")


@pytest.fixture(scope="session")
def cases():
    return importlib.import_module("3dcompactsolver_gb300.cases")


@pytest.fixture(scope="session")
def gpu_pkg(pkg):
    """The package with its CUDA library built; fails (never skips) when the
    library cannot be built or loaded on a GPU machine."""
    b = importlib.import_module("3dcompactsolver_gb300.build")
    b.build()
    pkg.lib()
    return pkg


def rel_err(a, b, scale=None):
    """Relative max-norm error max|a-b| / max|b| of one field; `scale`
    replaces max|b| where a field's own maximum is not its natural size."""
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.abs(b).max() if scale is None else scale
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def state_errors(q, qr):
    """Per conserved field relative max-norm errors of q against qr (both
    (5, Nz, Ny, Nx)).  Density and energy are measured against their own
    maxima; the three momenta against the largest momentum component, since a
    component can start at zero (w of the Taylor-Green vortex)."""
    mom = max(float(np.abs(qr[f]).max()) for f in (1, 2, 3))
    return [rel_err(q[f], qr[f], mom if f in (1, 2, 3) else None) for f in range(5)]


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name))
