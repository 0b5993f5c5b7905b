import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle as O

    O.ensure_built(with_ref=True)
    return O.load("oracle")


@pytest.fixture(scope="session")
def ref_lib():
    import oracle as O

    O.ensure_built(with_ref=True)
    lib = O.load("ref")
    if lib is None:
        pytest.skip("reference not compiled here (no reference checkout)")
    return lib


@pytest.fixture(scope="session")
def gpu_lib():
    import lila_gb300

    lila_gb300.build()
    return lila_gb300
