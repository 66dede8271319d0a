"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device and the in-tree CUDA library;
everything else runs on the CPU (oracle checks, host logic, ABI export checks)."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reflib():
    from oracle import build as ob
    if not ob.ref_available():
        pytest.skip("reference source tree not present (oracle/_ref is built only where it is)")
    from oracle.oracle import RefLib
    return RefLib()


def load_golden(name: str):
    """(meta list, arrays) of a tests/golden/<name>.npz fixture."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"])) if "meta" in z.files else None
    return meta, z


def golden_json(name: str):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def rb():
    """The package with its CUDA library built and loaded (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from randblas_gb300 import build as rbuild
    rbuild.build()
    import randblas_gb300
    randblas_gb300.lib()
    return randblas_gb300


@pytest.fixture(scope="session")
def rb_host():
    """The package with its CUDA library built and loaded, for host-only calls (no GPU)."""
    from randblas_gb300 import build as rbuild
    rbuild.build()
    import randblas_gb300
    randblas_gb300.lib()
    return randblas_gb300
