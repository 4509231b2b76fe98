import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")

# Parity bar of the plain FP64 form against the reference's cpu/ path: normwise relative
# error per conserved variable, max|a - ref| / max|ref| over interior cells.
FP64_TOL = 1e-12
# Mixed-precision form against FP64 after its step count.
MIXED_TOL = 1e-6


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.build(ref=True)
    O.set_threads(os.cpu_count() or 1)
    return O


@pytest.fixture(scope="session")
def cns():
    import cns_nospec_gb300 as C
    from cns_nospec_gb300 import build
    build.build()
    return C


@pytest.fixture(scope="session")
def gpu(cns):
    lib = cns.load()
    rc = lib.cns_set_device(0)
    if rc != 0:
        pytest.fail("GPU test without a usable CUDA device: " + lib.cns_last_error().decode())
    return lib


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def normwise(a, ref, interior_only=True, ng=4):
    """max|a-ref| / max|ref| per trailing-axis variable."""
    if interior_only:
        a = a[ng:-ng, ng:-ng, ng:-ng]
        ref = ref[ng:-ng, ng:-ng, ng:-ng]
    d = np.abs(a - ref).reshape(-1, a.shape[-1]).max(axis=0)
    r = np.abs(ref).reshape(-1, ref.shape[-1]).max(axis=0)
    r = np.where(r == 0, 1.0, r)
    return d / r
