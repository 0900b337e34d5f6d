import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a GB300)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def oracle_port():
    import oracle
    return oracle.Oracle("port")


@pytest.fixture(scope="session")
def oracle_best():
    """The reference-built driver where the reference compiled, else the port."""
    import oracle
    try:
        return oracle.Oracle("reference")
    except Exception:
        return oracle.Oracle("port")


@pytest.fixture(scope="session")
def gb300():
    """Builds (if needed) and loads the CUDA library; fails loudly if absent."""
    import daxtoolkit_gb300
    from daxtoolkit_gb300 import build as b
    b.build()
    daxtoolkit_gb300.capi.lib()
    from daxtoolkit_gb300 import cont
    return cont
