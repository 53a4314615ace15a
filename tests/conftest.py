import pathlib
import sys

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA extension")


@pytest.fixture(scope="session")
def gpu_lib():
    import lambda_gb300 as lg
    lg.build()
    return lg
