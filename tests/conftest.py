import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden" / "reference_golden.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def ref():
    import oracle
    r = oracle.ref()
    if r is None:
        pytest.skip("the reference sources are not available here to build oracle/_ref")
    return r


@pytest.fixture(scope="session")
def pa():
    """The GPU package with its native library built; GPU tests only."""
    from parallelalgorithms_gb300 import build as pabuild
    pabuild.build()
    import parallelalgorithms_gb300 as p
    if not p.lib().pa_device_available():
        pytest.fail("no CUDA device available for a test marked gpu")
    return p


@pytest.fixture(scope="session")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("torch sees no CUDA device for a test marked gpu")
    return torch
