import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
if str(REPO) not in sys.path:
    sys.path.insert(0, str(REPO))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU and the CUDA library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def reference():
    from oracle import Reference
    ref = Reference.load()
    if ref is None:
        pytest.skip("the reference shaders compiled as C++ are not available here")
    return ref


@pytest.fixture(scope="session")
def cflib():
    """libcfcull.so, built on demand."""
    from hellovulkan_gb300 import build
    build.build()
    from hellovulkan_gb300 import _lib
    return _lib.lib()


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(REPO / "tests" / "golden" / "golden_cases.npz")


@pytest.fixture(scope="session")
def golden_consumers():
    """FrustumCulling.comp and Scene.frag's lookup and lighting outputs made
    by the reference's own shader code (tests/golden/make_golden.py)."""
    import numpy as np
    return np.load(REPO / "tests" / "golden" / "golden_consumers.npz")


@pytest.fixture(scope="session")
def gpu(cflib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a GPU test ran without a visible CUDA device")
    from hellovulkan_gb300.pipelines import Context
    return Context(0)
