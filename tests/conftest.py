import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    from __graft_entry__ import reference_tree
    pyoracle.build(ref=True, tree=reference_tree())
    return pyoracle


@pytest.fixture(scope="session")
def tx():
    from transientx_gb300 import _build
    _build.build()
    import transientx_gb300
    transientx_gb300.load_library()
    return transientx_gb300


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(ROOT, "tests", "golden")
    return {"boxcar": np.load(os.path.join(d, "boxcar.npz")),
            "cluster": np.load(os.path.join(d, "cluster.npz"))}
