import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs through the C ABI")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc

    orc.build()
    return orc.Oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference's own CPU kernels; only where the reference checkout exists."""
    from oracle import oracle as orc

    src = orc.reference_src()
    if src is None:
        pytest.skip("reference checkout not present (LBM_REFERENCE_DIR)")
    orc.build(src)
    return orc.Reference()


@pytest.fixture(scope="session")
def lib():
    """The solver library, built in-tree if needed (nvcc cross-compiles without a GPU)."""
    from cavityflow_cuda_gb300 import build, load_library

    build.build()
    return load_library()


@pytest.fixture(scope="session")
def gpu(lib):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return lib
