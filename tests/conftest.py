import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (os.path.join(ROOT, "n-body_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


def golden(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


def rel_err_stats(got, ref):
    """Per-body |got - ref| / |ref| over xyz: returns (rms, max)."""
    got = np.asarray(got, np.float64)[:, :3]
    ref = np.asarray(ref, np.float64)[:, :3]
    num = np.linalg.norm(got - ref, axis=1)
    den = np.linalg.norm(ref, axis=1)
    mask = den > 0
    e = num[mask] / den[mask]
    if e.size == 0:
        return 0.0, float(num.max(initial=0.0))
    return float(np.sqrt(np.mean(e * e))), float(e.max())


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build(reference=False)
    return pyoracle


@pytest.fixture(scope="session")
def nb():
    """The CUDA library, built in-tree (no fallback: a failed build fails the test)."""
    import nbody_gb300
    from nbody_gb300 import build as nbuild

    nbuild.build()

    nbody_gb300.lib()
    return nbody_gb300


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
