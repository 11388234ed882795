import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA kernels through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build libskyr.so and the CPU oracle once per session (no-op when current)."""
    import __graft_entry__ as g

    g.build()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.set_device(0)
    return torch


@pytest.fixture()
def ctx(cuda):
    from skyrendering_gb300.atmosphere import Context

    c = Context()
    yield c
    c.close()
