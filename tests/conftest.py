import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "simplemoc-kernel_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

# The reference's sources, where mounted (MOC_REFERENCE_SOURCES, else a "reference"
# directory beside this repository): the live pin tests build against them.
REFERENCE_SOURCES = os.environ.get("MOC_REFERENCE_SOURCES") or os.path.join(
    os.path.dirname(ROOT), "reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the libraries and the oracle once per session (incremental)."""
    import mocatt_build
    import oracle

    mocatt_build.build()
    oracle.build(REFERENCE_SOURCES if os.path.isdir(REFERENCE_SOURCES) else None)
    yield


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return torch.device("cuda:0")


@pytest.fixture(scope="session")
def handle(cuda):
    import mocatt

    h = mocatt.Handle(0)
    yield h
    h.close()
