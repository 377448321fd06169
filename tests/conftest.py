"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on a
machine without a GPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    if not os.path.exists(pyoracle.ORACLE_SO):
        pyoracle.build()
    return pyoracle.Oracle()


@pytest.fixture(scope="session")
def reference():
    import pyoracle
    if not pyoracle.reference_available():
        pytest.skip("reference CPU library not built here (reference tree absent)")
    return pyoracle.Reference()


@pytest.fixture(scope="session")
def golden():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    return {n: {k.split("/")[1]: g[k] for k in g.files if k.split("/")[0] == n} for n in names}


@pytest.fixture(scope="session")
def wc():
    import wavecuda_gb300 as wc
    if not os.path.exists(wc.LIB_PATH):
        from wavecuda_gb300 import build
        build.build()
    wc.lib()
    return wc


@pytest.fixture(scope="session")
def gpu(wc):
    if wc.device_count() < 1:
        pytest.fail("GPU test run without a CUDA device")
    return wc
