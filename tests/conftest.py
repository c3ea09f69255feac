import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def gpu_library():
    """The built CUDA library; GPU tests fail loudly when it is missing."""
    import torch

    from sand_atlas_dem_gb300 import native

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    if not native.LIBRARY.exists():
        native.build()
    return native.load()
