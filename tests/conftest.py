"""Shared pytest setup: the `gpu` marker, paths to the oracle and the product
library's Python binding, and fixture loading."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", os.path.join("les-model_gb300", "py")):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
GRIDS = ("box12", "aniso16", "tiny7")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def golden_mesh(d):
    import oracle as O
    nx, ny, nz = (int(x) for x in d["mesh"])
    return O.Mesh(nx, ny, nz, *[float(x) for x in d["h"]])


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle as O
    return O.Oracle()


def same(a, b):
    """Bitwise equality up to the sign of zero (NaNs equal)."""
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def maxrel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)
