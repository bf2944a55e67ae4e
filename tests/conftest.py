import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def lib():
    """The product library; built in-tree when missing (no fallback exists)."""
    from proteus_gb300 import abi, build

    if not os.path.exists(abi.LIB_PATH):
        build.build()
    return abi.load()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def ctx(lib):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from proteus_gb300 import engine

    c = engine.Context(0, pool_bytes=40 << 30)
    yield c
    c.close()


@pytest.fixture(scope="session")
def golden():
    import json

    with open(os.path.join(ROOT, "tests", "golden", "reference_cases.json")) as f:
        ref = json.load(f)
    with open(os.path.join(ROOT, "tests", "golden", "rjstepwise_cases.json")) as f:
        rj = json.load(f)
    return {"reference": ref, "rjstepwise": rj}
