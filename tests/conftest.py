import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


_CACHE = {}


def workload(name, **kw):
    """Seeded synthetic workloads by name (redux_gb300.synth.workload), generated once per
    session."""
    from redux_gb300 import synth
    key = (name, tuple(sorted(kw.items())))
    if key not in _CACHE:
        _CACHE[key] = synth.workload(name, **kw)
    return _CACHE[key]


@pytest.fixture(scope="session")
def w0():
    return workload("plain64")


@pytest.fixture(scope="session")
def w2small():
    # the production geometry (88 x 88, 36 modes, 3 channels) with 4 frames and 2 patches
    return workload("production88", n_patches=2, frames=4)
