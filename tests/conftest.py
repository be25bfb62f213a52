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


def _finite_pair(a, b):
    """(a, b) restricted to their finite entries, or None when the non-finite
    entries do not sit at the same places (the reference yields NaN where a
    target coincides with a periodic image of a source in a neighbouring box,
    and so must the library)."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return None
    fa, fb = np.isfinite(a), np.isfinite(b)
    if not np.array_equal(fa, fb) or not np.array_equal(np.isnan(a), np.isnan(b)):
        return None
    return a[fb], b[fb]


def normwise_err(a, b):
    """max|a-b| / max|b| over finite entries (inf if the non-finite entries differ)."""
    p = _finite_pair(a, b)
    if p is None:
        return np.inf
    a, b = p
    if b.size == 0:
        return 0.0
    den, num = np.abs(b).max(), np.abs(a - b).max()
    return num / den if den > 0 else num


def rms_err(a, b):
    """||a-b||_2 / ||b||_2 over finite entries (inf if the non-finite entries differ).

    The normwise error alone is blind where the stresslet is largest: on
    uniform clouds a few near-singular pairs make max|b| huge, so an error
    spread over typical targets barely registers against it.
    """
    p = _finite_pair(a, b)
    if p is None:
        return np.inf
    a, b = p
    if b.size == 0:
        return 0.0
    den, num = np.sqrt(np.mean(b * b)), np.sqrt(np.mean((a - b) ** 2))
    return num / den if den > 0 else num


def relerr(a, b):
    """Parity error used by every parity assertion: the larger of the
    normwise error max|a-b| / max|b| and the RMS-relative error
    ||a-b|| / ||b||, over finite entries.  Non-finite entries must sit at the
    same places in both arrays; otherwise the error is inf."""
    return max(normwise_err(a, b), rms_err(a, b))


@pytest.fixture(scope="session")
def golden():
    return load_golden
