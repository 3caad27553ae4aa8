import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "sucem-fem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


def golden(name):
    import numpy as np
    return np.load(os.path.join(GOLDEN, name))
