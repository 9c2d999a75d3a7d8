"""pytest configuration: the `gpu` marker and shared fixtures.

Tests marked ``gpu`` need a CUDA device (sm_103) and the built library
(``python -c "import __graft_entry__ as g; g.build()"``); everything else
runs on a CPU-only machine.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    import json
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(d, "golden_reference.json")) as f:
        meta = json.load(f)
    data = dict(np.load(os.path.join(d, "golden_reference.npz")))
    return meta, data
