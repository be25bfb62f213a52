import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files}
    for k in ("nside_x", "nside_y", "Mx", "My", "P"):
        d[k] = int(d[k])
    for k in ("xi", "Lx", "Ly", "w", "eta"):
        d[k] = float(d[k])
    return d


def relerr(a, b):
    """Normwise relative error max|a-b| / max|b| over finite entries.

    Non-finite entries must sit at the same places in both arrays (the
    reference yields NaN where a target coincides with a periodic image of a
    source in a neighbouring box); otherwise the error is inf.
    """
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return np.inf
    fa, fb = np.isfinite(a), np.isfinite(b)
    if not np.array_equal(fa, fb) or not np.array_equal(np.isnan(a), np.isnan(b)):
        return np.inf
    if not fb.any():
        return 0.0
    den = np.abs(b[fb]).max()
    num = np.abs(a[fb] - b[fb]).max()
    return num / den if den > 0 else num


@pytest.fixture(scope="session")
def golden():
    return load_golden
