import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long CPU test")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def ref_build():
    """The reference's kernel sources compiled as C++ (development container only)."""
    from oracle import REF_SO, RefBuild, build_ref

    if not REF_SO.exists():
        if build_ref() is None:
            pytest.skip("reference sources not present on this machine")
    return RefBuild()


@pytest.fixture(scope="session")
def gpu_lib():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from libclsph_gb300.gpu import load_library

    return load_library()
