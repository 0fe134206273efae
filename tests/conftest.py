import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")
    config.addinivalue_line("markers", "slow: long-running (large states)")


@pytest.fixture(scope="session")
def engine_lib():
    """The engine's shared library, rebuilt if any source is newer (nvcc cross-compiles without a GPU)."""
    from quantumforge_gb300 import _build, _native

    if _native.lib_path() == _build.LIB:
        _build.build()
    return _native.load()


@pytest.fixture(scope="session")
def backend(engine_lib):
    import torch  # noqa: F401  (torch brings the CUDA driver up first)

    from quantumforge_gb300 import CudaBackend

    b = CudaBackend(0)
    yield b
    b.close()
