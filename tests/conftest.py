import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libceed_b200 library")


GOLDEN = os.path.join(ROOT, "tests", "golden")


def relinf(a, b):
    """Relative l-infinity distance max|a-b| / max|b| (the parity measure for FP64 applies)."""
    import numpy as np

    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b)) if b.size else 1.0
    return float(np.max(np.abs(a - b)) / (scale if scale > 0 else 1.0)) if b.size else 0.0
