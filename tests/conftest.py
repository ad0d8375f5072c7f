import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(REPO, "lightmetrica-v2_gb300"), os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def repo_dir():
    return REPO


@pytest.fixture(scope="session")
def reference_root():
    """The reference source tree: $LM_REFERENCE_ROOT, else a `reference`
    directory beside the repository (absent on machines without it)."""
    return os.environ.get("LM_REFERENCE_ROOT", os.path.join(os.path.dirname(REPO), "reference"))


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(REPO, "tests", "golden")


@pytest.fixture(scope="session")
def oracle_lib():
    import lmoracle

    lmoracle.build()
    return lmoracle


@pytest.fixture(scope="session")
def gpu_lib():
    """liblmgpu.so, built if needed; GPU tests fail (not skip) if it cannot load."""
    from lmgpu import build as lbuild

    lbuild.build()
    import lmgpu

    lmgpu.lib()
    return lmgpu
