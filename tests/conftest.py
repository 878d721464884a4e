"""Shared pytest setup: the `gpu` marker, import paths and fixture loading."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ggks-multiselect_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_files():
    """Known-answer and numpy cross-check fixtures (each holds its input)."""
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "kat_*.npz"))
                  + glob.glob(os.path.join(GOLDEN_DIR, "xcheck_*.npz")))


def ref_files():
    """Fixtures holding outputs of the reference itself (the input is
    regenerated from its recipe; tests/golden/ref_inputs.py)."""
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "ref_*.npz")))


def load_golden(path):
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


def bits(a):
    """Bit patterns of an array, for bit-exact comparison (NaN-safe)."""
    a = np.ascontiguousarray(a)
    if a.dtype == np.float32:
        return a.view(np.uint32)
    if a.dtype == np.float64:
        return a.view(np.uint64)
    return a


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle
